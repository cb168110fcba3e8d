// Exact gradient dS/dR of the whole-ring action at level 0 (the "adjoint" of the action
// evaluation), the total action it differentiates, the virial centroid term built on it, and a
// hybrid Monte Carlo path move driven by it.
//
// The action of one species' path, summed over every link b -> b+1 of the ring (level 0):
//   Kinetic        sum_b phi(r_{b+1} - r_b),  phi(d) = sum_c image(d_c) + |d|^2 / (4 lambda tau)
//                  (kinetic_class.h:105-122 with the free-particle splines of free_spline_class.h)
//   HarmonicTrap   cofactor_a sum_b |r_b|^2                                   (trap_class.h:40-62)
//   BarePairAction sum_pairs sum_b tau (V(r_b) + V(r_{b+1})) / 2  (pair_action_class.h:267-302,
//                  bare_pair_action_class.h:98-149; V clamped to the table's grid) plus, with the
//                  Ewald split, tau sum_b sum_k v_k Re(rho_a(k,b) conj(rho_b(k,b))) (x 2 for a != b)
// The reference differentiates only parts of this (kinetic_class.h:125-144 exactly; the pair
// short-range part by central differences with eps = 1e-4, pair_action_class.h:135-155; the trap
// and the Ewald part not at all). Here every term has its analytic derivative:
//   kinetic   dS/dr_b = phi'(r_b - r_{b-1}) - phi'(r_{b+1} - r_b)
//   trap      2 cofactor_a r_b
//   pair      tau sum_q V'(|r_pq|) r_pq / |r_pq|      (zero where the table clamps V flat)
//   Ewald     -2 tau sum_k v_k k Im(conj(rho_other(k,b)) exp(i k.r_b))
// where rho_other is the partner species' density (the own species' for a homologous action).
// The densities and the Ewald sums over k run in double-float (FP32 pairs, ~1e-14 relative) on
// the FP32 pipe; every other term and every total is FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../common/philox.h"
#include "../framework/context.h"
#include "actions.cuh"
#include "phase_dd.cuh"
#include "reduce.cuh"

namespace pimc {
namespace {

/// d/dx of EvalCubic: zero outside the grid, where EvalCubic holds the end value.
__device__ __forceinline__ double EvalCubicDeriv(const CubicTable& t, double x) {
    if (x < t.x0 || x > t.x1) return 0.;
    int i;
    if (t.uniform) {
        i = (int)floor((x - t.x0) * t.inv_dx);
        i = min(max(i, 0), t.n - 2);
    } else {
        int j = (int)floor((x - t.x0) * t.inv_dx);
        j = min(max(j, 0), t.n_bucket - 1);
        i = t.bucket[j];
        while (i < t.n - 2 && __ldg(&t.x[i + 1]) <= x) ++i;
    }
    const Cubic4 c = t.c[i];
    const double u = x - __ldg(&t.x[i]);
    return c.c1 + u * (2. * c.c2 + 3. * u * c.c3);
}

/// Per-bead pair potential V(r) of the primitive action (one half of CalcV's two ends) and dV/dr,
/// with the reference's two clamps (bare_pair_action_class.h:98-111).
__device__ __forceinline__ void PairVBead(const PairDev& pa, double r, double& v, double& dv) {
    const bool in1 = r >= pa.r_v_min && r <= pa.r_v_max;
    const double r1 = fmin(fmax(r, pa.r_v_min), pa.r_v_max);
    if (pa.is_coulomb) {
        v = 1. / r1;
        dv = in1 ? -1. / (r1 * r1) : 0.;
    } else {
        v = EvalCubic(pa.v_r, r1);
        dv = in1 ? EvalCubicDeriv(pa.v_r, r1) : 0.;
    }
    if (pa.use_long_range) {
        const bool in2 = r1 >= pa.r_vl_min && r1 <= pa.r_vl_max;
        const double r2 = fmin(fmax(r1, pa.r_vl_min), pa.r_vl_max);
        v -= EvalCubic(pa.v_long_r, r2);
        if (in1 && in2) dv -= EvalCubicDeriv(pa.v_long_r, r2);
    }
}

__device__ __forceinline__ size_t GIdx(uint32_t b, uint32_t d, uint32_t g, uint32_t np) { return ((size_t)b * 3 + d) * np + g; }

__global__ void KineticGradKernel(const SystemDev sys, const double* __restrict__ pos, const KineticDev k, double* __restrict__ grad) {
    const uint32_t ns = sys.sp_n[k.species], M = sys.M, np = sys.n_pad, off = sys.sp_off[k.species];
    const double i4lt = k.i4lt_level[0];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (uint64_t)ns * M; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(i / ns), g = off + (uint32_t)(i % ns);
        const uint32_t bm = b == 0 ? M - 1 : b - 1, bp = b + 1 == M ? 0 : b + 1;
        for (uint32_t d = 0; d < sys.n_d; ++d) {
            const double x = PosAt(pos, np, b, d, g);
            const double dm = MinImage(x - PosAt(pos, np, bm, d, g), sys.L, sys.iL);
            const double dp = MinImage(PosAt(pos, np, bp, d, g) - x, sys.L, sys.iL);
            double fm = 2. * dm * i4lt, fp = 2. * dp * i4lt;
            if (k.has_images) {
                fm += EvalCubicDeriv(k.image[0], dm);
                fp += EvalCubicDeriv(k.image[0], dp);
            }
            grad[GIdx(b, d, g, np)] += fm - fp;
        }
    }
}

__global__ void TrapGradKernel(const SystemDev sys, const double* __restrict__ pos, const TrapDev t, double* __restrict__ grad) {
    const uint32_t ns = sys.sp_n[t.species], M = sys.M, np = sys.n_pad, off = sys.sp_off[t.species];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (uint64_t)ns * M; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(i / ns), g = off + (uint32_t)(i % ns);
        for (uint32_t d = 0; d < sys.n_d; ++d) grad[GIdx(b, d, g, np)] += 2. * t.cofactor_a * PosAt(pos, np, b, d, g);
    }
}

__device__ __forceinline__ dd SplitDD(double x) {
    const float h = (float)x;
    return dd{h, (float)(x - (double)h)};
}

/// Per-slice densities of every kept species from one position copy, in double-float: one block per
/// (k-range of kRhoDDThreads x kRhoDDKPerThread k-vectors, slice, slot), each thread summing its
/// kRhoDDKPerThread k-vectors over the particles in order, in chunks whose phase rows sit in
/// shared memory (species_class.h:380-403). A wide k-range keeps the phase rows, which every block
/// of a slice forms again, to a few per thread.
constexpr uint32_t kRhoDDChunk = 32;
constexpr uint32_t kRhoDDThreads = 128;
constexpr uint32_t kRhoDDKPerThread = 8;

__global__ void __launch_bounds__(kRhoDDThreads) RhoDDKernel(const SystemDev sys, const double* __restrict__ pos, const int* __restrict__ slot_species,
                                                             const float4* __restrict__ tab256, dd iL, dd two_pi, float4* __restrict__ rho) {
    extern __shared__ ddc rtab[];  // [kRhoDDChunk][3][stride]
    const uint32_t stride = (uint32_t)max(max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const uint32_t b = blockIdx.y, slot = blockIdx.z;
    const uint32_t s = (uint32_t)slot_species[slot], ns = sys.sp_n[s], off = sys.sp_off[s], K = sys.K, np = sys.n_pad, n_d = sys.n_d;
    const uint32_t k0 = blockIdx.x * (kRhoDDThreads * kRhoDDKPerThread) + threadIdx.x;
    int32_t pk[kRhoDDKPerThread];
    ddc acc[kRhoDDKPerThread];
#pragma unroll
    for (uint32_t j = 0; j < kRhoDDKPerThread; ++j) {
        const uint32_t k = k0 + j * kRhoDDThreads;
        pk[j] = k < K ? sys.kidx[k] : 0;
        acc[j] = ddc{DD(0.f), DD(0.f)};
    }
    for (uint32_t p0 = 0; p0 < ns; p0 += kRhoDDChunk) {
        const uint32_t cnt = min(kRhoDDChunk, ns - p0);
        __syncthreads();
        for (uint32_t t = threadIdx.x; t < cnt * 3 * stride; t += blockDim.x) {
            const uint32_t pi = t / (3 * stride), rem = t - pi * 3 * stride, d = rem / stride, n = rem - d * stride;
            if (d < n_d && (int)n <= sys.max_index[d]) rtab[t] = PhaseDD(SplitDD(PosAt(pos, np, b, d, off + p0 + pi)), (int)n, iL, two_pi, tab256);
        }
        __syncthreads();
        for (uint32_t pi = 0; pi < cnt; ++pi)
#pragma unroll
            for (uint32_t j = 0; j < kRhoDDKPerThread; ++j)
                if (k0 + j * kRhoDDThreads < K) acc[j] = CAdd(acc[j], PhaseProductDD(rtab + (size_t)pi * 3 * stride, stride, n_d, pk[j]));
    }
#pragma unroll
    for (uint32_t j = 0; j < kRhoDDKPerThread; ++j) {
        const uint32_t k = k0 + j * kRhoDDThreads;
        if (k < K) rho[((size_t)slot * sys.M + b) * K + k] = Pack(acc[j]);
    }
}

/// Ewald forces: one warp per (slice, particle), lanes over the stored k-vectors in double-float;
/// the particle's per-dimension phase rows sit in shared memory.
__global__ void EwaldGradDDKernel(const SystemDev sys, const double* __restrict__ pos, const PairDev pa, const float4* __restrict__ rho_a,
                                  const float4* __restrict__ rho_b, const float2* __restrict__ vk, const float4* __restrict__ tab256, dd iL, dd two_pi,
                                  double* __restrict__ grad) {
    extern __shared__ ddc etab[];  // [warps][3][stride]
    const uint32_t stride = (uint32_t)max(max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const uint32_t warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    ddc* my = etab + (size_t)w * 3 * stride;
    const uint32_t na = sys.sp_n[pa.sa], nb = sys.sp_n[pa.sb], M = sys.M, np = sys.n_pad, K = sys.K, n_d = sys.n_d;
    const bool hom = pa.sa == pa.sb;
    const uint32_t ng = hom ? na : na + nb;
    for (uint64_t it = (uint64_t)blockIdx.x * warps + w; it < (uint64_t)ng * M; it += (uint64_t)gridDim.x * warps) {
        const uint32_t b = (uint32_t)(it / ng), j = (uint32_t)(it % ng);
        const bool in_a = j < na;
        const uint32_t g = in_a ? sys.sp_off[pa.sa] + j : sys.sp_off[pa.sb] + (j - na);
        const float4* rho = (in_a ? rho_b : rho_a) + (size_t)b * K;
        __syncwarp();
        for (uint32_t t = lane; t < 3 * stride; t += 32) {
            const uint32_t d = t / stride, n = t - d * stride;
            if (d < n_d && (int)n <= sys.max_index[d]) my[t] = PhaseDD(SplitDD(PosAt(pos, np, b, d, g)), (int)n, iL, two_pi, tab256);
        }
        __syncwarp();
        dd acc[3] = {DD(0.f), DD(0.f), DD(0.f)};
        for (uint32_t k = lane; k < K; k += 32) {
            const int32_t pk = sys.kidx[k];
            const ddc e = PhaseProductDD(my, stride, n_d, pk);
            const ddc r = Unpack(rho[k]);
            const float2 v = vk[k];
            const dd f = Mul(dd{v.x, v.y}, Sub(Mul(r.re, e.im), Mul(r.im, e.re)));  // v_k Im(conj(rho) e)
            for (uint32_t d = 0; d < n_d; ++d) acc[d] = Add(acc[d], MulF(f, (float)KIdx(pk, (int)d)));
        }
        for (uint32_t d = 0; d < n_d; ++d) {
            const dd s = WarpSumDD(acc[d]);
            if (lane == 0) grad[GIdx(b, d, g, np)] += -2. * sys.tau * sys.box[d] * ToDouble(s);
        }
    }
}

/// The Ewald force on a bead of species s from every selected long-range pair action is
/// -2 tau box_d sum_k k_d Im(conj(W_s(k)) e^{i k r}) with W_s = sum_a v^a_k rho_{o(a)}(k), o(a) the
/// action's other species (s itself for a homologous action): the actions' terms are linear in the
/// densities, so one pass over k per bead covers them all. One thread per (slice, k) forms W_s.
__global__ void EwaldWeightKernel(const SystemDev sys, const float4* __restrict__ rho, const float2* const* __restrict__ vk, const int* __restrict__ other_slot,
                                  uint32_t n_terms, float4* __restrict__ w) {
    const uint64_t n = (uint64_t)sys.M * sys.K;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)(i % sys.K);
        ddc acc{{0.f, 0.f}, {0.f, 0.f}};
        for (uint32_t a = 0; a < n_terms; ++a) {
            const float2 v = vk[a][k];
            const ddc r = Unpack(rho[(size_t)other_slot[a] * sys.M * sys.K + i]);
            const dd vv{v.x, v.y};
            acc = CAdd(acc, ddc{Mul(vv, r.re), Mul(vv, r.im)});
        }
        w[i] = Pack(acc);
    }
}

/// Ewald forces on the beads of one species from its weight W_s (EwaldWeightKernel): one warp per
/// (slice, particle), lanes over the k-vectors in double-float, the particle's per-dimension phase
/// rows in shared memory.
__global__ void EwaldGradSpeciesKernel(const SystemDev sys, const double* __restrict__ pos, uint32_t species, const float4* __restrict__ w,
                                       const float4* __restrict__ tab256, dd iL, dd two_pi, double* __restrict__ grad) {
    extern __shared__ ddc etab_s[];  // [warps][3][stride]
    const uint32_t stride = (uint32_t)max(max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const uint32_t warps = blockDim.x >> 5, wi = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    ddc* my = etab_s + (size_t)wi * 3 * stride;
    const uint32_t ns = sys.sp_n[species], off = sys.sp_off[species], M = sys.M, np = sys.n_pad, K = sys.K, n_d = sys.n_d;
    for (uint64_t it = (uint64_t)blockIdx.x * warps + wi; it < (uint64_t)ns * M; it += (uint64_t)gridDim.x * warps) {
        const uint32_t b = (uint32_t)(it / ns), g = off + (uint32_t)(it % ns);
        const float4* wb = w + (size_t)b * K;
        __syncwarp();
        for (uint32_t t = lane; t < 3 * stride; t += 32) {
            const uint32_t d = t / stride, n = t - d * stride;
            if (d < n_d && (int)n <= sys.max_index[d]) my[t] = PhaseDD(SplitDD(PosAt(pos, np, b, d, g)), (int)n, iL, two_pi, tab256);
        }
        __syncwarp();
        dd acc[3] = {DD(0.f), DD(0.f), DD(0.f)};
        for (uint32_t k = lane; k < K; k += 32) {
            const int32_t pk = sys.kidx[k];
            const ddc e = PhaseProductDD(my, stride, n_d, pk);
            const ddc r = Unpack(wb[k]);
            const dd f = Sub(Mul(r.re, e.im), Mul(r.im, e.re));  // Im(conj(W) e)
            for (uint32_t d = 0; d < n_d; ++d) acc[d] = Add(acc[d], MulF(f, (float)KIdx(pk, (int)d)));
        }
        for (uint32_t d = 0; d < n_d; ++d) {
            const dd s = WarpSumDD(acc[d]);
            if (lane == 0) grad[GIdx(b, d, g, np)] += -2. * sys.tau * sys.box[d] * ToDouble(s);
        }
    }
}

/// HMC momenta: standard normals for every coordinate of the moving particles, in the path order
/// (moving particle, slice, dimension); normal j is component j % 4 of Philox block 1 + j / 4
/// of the attempt's stream (two Box-Muller pairs per block).
__global__ void HmcMomentaKernel(const SystemDev sys, MoveStream st, const uint32_t* __restrict__ moving, uint32_t n_moving,
                                 double* __restrict__ mom) {
    const uint32_t M = sys.M, np = sys.n_pad, n_d = sys.n_d;
    const uint64_t n = (uint64_t)n_moving * M * n_d;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t d = (uint32_t)(j % n_d), b = (uint32_t)((j / n_d) % M), gi = (uint32_t)(j / ((uint64_t)n_d * M));
        const Philox4 w = st.Block(1u + (uint32_t)(j >> 2));
        float z0, z1;
        const uint32_t c = (uint32_t)(j & 3u);
        if (c < 2) BoxMullerF(w.v[0], w.v[1], z0, z1);
        else BoxMullerF(w.v[2], w.v[3], z0, z1);
        mom[GIdx(b, d, moving[gi], np)] = (double)((c & 1u) ? z1 : z0);
    }
}

__global__ void AxpyKernel(double* __restrict__ y, const double* __restrict__ x, double a, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) y[i] += a * x[i];
}

int Blocks(const Context& c, uint64_t n, int threads) {
    const uint64_t want = (n + threads - 1) / threads;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)c.n_sm * 16));
}

}  // namespace

/// Double-float densities of `pos` (adjoint scratch; the committed densities are untouched), and
/// the double-float tables the adjoint kernels read (phase rows, v_k per long-range action).
const float4* Context::ScratchRho(const double* pos) {
    if (!rho_slots || !sys.K) return nullptr;
    const size_t n = (size_t)rho_slots * sys.M * sys.K;
    if (!rho_scratch_ || rho_scratch_->bytes < n * sizeof(float4)) rho_scratch_.reset(new DeviceBuffer(n * sizeof(float4)));
    if (!phase_tab_) {
        std::vector<float4> t(256);
        PhaseTable256(t.data());
        phase_tab_.reset(new DeviceBuffer(256 * sizeof(float4)));
        CudaCheck(cudaMemcpy(phase_tab_->ptr, t.data(), 256 * sizeof(float4), cudaMemcpyHostToDevice), "phase table");
        adj_vk_.resize(actions.size());
        for (size_t i = 0; i < actions.size(); ++i) {
            if (actions[i].kind != 2 || !sys.pair[actions[i].index].use_long_range) continue;
            const auto& hv = host_vk[actions[i].index];
            std::vector<float2> v(sys.K);
            for (uint32_t k = 0; k < sys.K; ++k) {
                float h, l;
                SplitDouble(hv[k], h, l);
                v[k] = make_float2(h, l);
            }
            adj_vk_[i].reset(new DeviceBuffer(sys.K * sizeof(float2)));
            CudaCheck(cudaMemcpy(adj_vk_[i]->ptr, v.data(), sys.K * sizeof(float2), cudaMemcpyHostToDevice), "v_k table");
        }
    }
    std::vector<int> slot_species(rho_slots, 0);
    for (uint32_t s = 0; s < sys.S; ++s)
        if (sys.sp_rho[s] >= 0) slot_species[sys.sp_rho[s]] = (int)s;
    uint32_t* dss = Parts(rho_slots);
    CudaCheck(cudaMemcpyAsync(dss, slot_species.data(), rho_slots * sizeof(int), cudaMemcpyHostToDevice, stream), "slot upload");
    const uint32_t stride = (uint32_t)std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const size_t smem = (size_t)kRhoDDChunk * 3 * stride * sizeof(ddc);
    CudaCheck(cudaFuncSetAttribute(RhoDDKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute");
    dd iL, two_pi;
    SplitDouble(sys.iL, iL.hi, iL.lo);
    SplitDouble(2. * M_PI, two_pi.hi, two_pi.lo);
    const uint32_t k_per_block = kRhoDDThreads * kRhoDDKPerThread;
    RhoDDKernel<<<dim3((sys.K + k_per_block - 1) / k_per_block, sys.M, rho_slots), kRhoDDThreads, smem, stream>>>(sys, pos, reinterpret_cast<const int*>(dss),
                                                                                     phase_tab_->as<float4>(), iL, two_pi, rho_scratch_->as<float4>());
    CudaCheck(cudaGetLastError(), "rho launch");
    return rho_scratch_->as<float4>();
}

/// Selection: a >= 0 one action, -1 every action, -2 every non-kinetic action.
static bool Selected(const ActionHost& ah, int sel, int i) {
    if (ah.is_importance_weight) return false;
    if (sel >= 0) return sel == i;
    if (sel == -2) return ah.kind != 0;
    return true;
}

/// The whole-ring action and its exact gradient cover Kinetic, HarmonicTrap and BarePairAction.
static void RequireAdjointActions(const Context& c, int sel) {
    if (c.AnyPerm())
        throw PimcError(kErrUnsupported, "the whole-ring action and its gradient assume paths without exchanges");
    for (size_t i = 0; i < c.actions.size(); ++i)
        if (Selected(c.actions[i], sel, (int)i) && c.actions[i].kind == 2 && c.sys.pair[c.actions[i].index].kind != kPairBare)
            throw PimcError(kErrUnsupported, "the whole-ring action and its gradient cover Kinetic, HarmonicTrap and BarePairAction");
}

double Context::TotalActionDev(int a, const double* pos, const float4* rho) {
    RequireAdjointActions(*this, a);
    const uint32_t M = sys.M, np = sys.n_pad, n_d = sys.n_d;
    const double L = sys.L, iL = sys.iL, tau = sys.tau;
    double total = 0.;
    for (size_t i = 0; i < actions.size(); ++i) {
        const ActionHost& ah = actions[i];
        if (!Selected(ah, a, (int)i)) continue;
        double part = 0.;
        if (ah.kind == 0) {
            const KineticDev k = sys.kinetic[ah.index];
            const uint32_t ns = sys.sp_n[k.species], off = sys.sp_off[k.species];
            const double i4lt = k.i4lt_level[0];
            SumItems<1>(*this, (uint64_t)ns * M, [=] __device__(uint64_t it, double* v) {
                const uint32_t b = (uint32_t)(it / ns), g = off + (uint32_t)(it % ns), bp = b + 1 == M ? 0 : b + 1;
                double dr[3];
                for (uint32_t d = 0; d < n_d; ++d) dr[d] = MinImage(PosAt(pos, np, bp, d, g) - PosAt(pos, np, b, d, g), L, iL);
                v[0] = -LogRhoFree(dr, n_d, i4lt, &k.image[0], k.has_images);
            }, &part);
        } else if (ah.kind == 1) {
            const TrapDev t = sys.trap[ah.index];
            const uint32_t ns = sys.sp_n[t.species], off = sys.sp_off[t.species];
            SumItems<1>(*this, (uint64_t)ns * M, [=] __device__(uint64_t it, double* v) {
                const uint32_t b = (uint32_t)(it / ns), g = off + (uint32_t)(it % ns);
                double s = 0.;
                for (uint32_t d = 0; d < n_d; ++d) {
                    const double x = PosAt(pos, np, b, d, g);
                    s += x * x;
                }
                v[0] = t.cofactor_a * s;
            }, &part);
        } else {
            const PairDev pa = sys.pair[ah.index];
            if (pa.is_constant) continue;  // pair_action_class.h:268
            const uint32_t na = sys.sp_n[pa.sa], nb = sys.sp_n[pa.sb], oa = sys.sp_off[pa.sa], ob = sys.sp_off[pa.sb];
            const bool hom = pa.sa == pa.sb;
            // tau V(|d_b|) per pair and slice, d_b the minimum image on that slice: the two half
            // links of CalcU that meet at a bead, with each end's distance taken as its own minimum
            // image (the function the double-float pair-force kernel differentiates).
            SumItems<1>(*this, (uint64_t)na * nb * M, [=] __device__(uint64_t it, double* v) {
                const uint32_t q = (uint32_t)(it % nb);
                const uint64_t r0 = it / nb;
                const uint32_t p = (uint32_t)(r0 % na), b = (uint32_t)(r0 / na);
                v[0] = 0.;
                if (hom && q <= p) return;
                double r2 = 0.;
                for (uint32_t d = 0; d < n_d; ++d) {
                    const double x = MinImage(PosAt(pos, np, b, d, ob + q) - PosAt(pos, np, b, d, oa + p), L, iL);
                    r2 += x * x;
                }
                double vb, dvb;
                PairVBead(pa, sqrt(r2), vb, dvb);
                v[0] = tau * vb;
            }, &part);
            if (pa.use_long_range && rho) {
                const float4* ra = rho + (size_t)sys.sp_rho[pa.sa] * M * sys.K;
                const float4* rb = rho + (size_t)sys.sp_rho[pa.sb] * M * sys.K;
                const uint32_t K = sys.K;
                double lr = 0.;
                SumItems<1>(*this, (uint64_t)M * K, [=] __device__(uint64_t it, double* v) {
                    const float4 x = ra[it], y = rb[it];
                    const double xr = (double)x.x + (double)x.y, xi = (double)x.z + (double)x.w;
                    const double yr = (double)y.x + (double)y.y, yi = (double)y.z + (double)y.w;
                    v[0] = pa.v_long_k[it % K] * (xr * yr + xi * yi);
                }, &lr);
                part += (hom ? 1. : 2.) * tau * lr;
            }
        }
        total += part;
    }
    return total;
}

void Context::GradientDev(int a, const double* pos, const float4* rho, double* grad) {
    RequireAdjointActions(*this, a);
    const size_t n = (size_t)sys.M * 3 * sys.n_pad;
    CudaCheck(cudaMemsetAsync(grad, 0, n * sizeof(double), stream), "grad clear");
    const int th = 256;
    // Several actions selected: the Ewald forces per species in one pass (EwaldWeightKernel).
    const bool fused_ewald = a < 0 && rho && sys.K;
    for (size_t i = 0; i < actions.size(); ++i) {
        const ActionHost& ah = actions[i];
        if (!Selected(ah, a, (int)i)) continue;
        if (ah.kind == 0) {
            const KineticDev k = sys.kinetic[ah.index];
            KineticGradKernel<<<Blocks(*this, (uint64_t)sys.sp_n[k.species] * sys.M, th), th, 0, stream>>>(sys, pos, k, grad);
        } else if (ah.kind == 1) {
            const TrapDev t = sys.trap[ah.index];
            TrapGradKernel<<<Blocks(*this, (uint64_t)sys.sp_n[t.species] * sys.M, th), th, 0, stream>>>(sys, pos, t, grad);
        } else {
            const PairDev pa = sys.pair[ah.index];
            if (pa.is_constant) continue;
            PairGradDD(ah.index, pos, grad);
            if (pa.use_long_range && rho && sys.K && !fused_ewald) {
                const uint64_t ng = (uint64_t)(pa.sa == pa.sb ? sys.sp_n[pa.sa] : sys.sp_n[pa.sa] + sys.sp_n[pa.sb]) * sys.M;
                const float4* ra = rho + (size_t)sys.sp_rho[pa.sa] * sys.M * sys.K;
                const float4* rb = rho + (size_t)sys.sp_rho[pa.sb] * sys.M * sys.K;
                const int stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
                const int warps = 8;
                const size_t smem = (size_t)warps * 3 * stride * sizeof(ddc);
                const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((ng + warps - 1) / warps, (uint64_t)n_sm * 16));
                dd iL, two_pi;
                SplitDouble(sys.iL, iL.hi, iL.lo);
                SplitDouble(2. * M_PI, two_pi.hi, two_pi.lo);
                EwaldGradDDKernel<<<blocks, warps * 32, smem, stream>>>(sys, pos, pa, ra, rb, adj_vk_[i]->as<float2>(), phase_tab_->as<float4>(), iL,
                                                                        two_pi, grad);
            }
        }
        CudaCheck(cudaGetLastError(), "gradient launch");
    }
    if (fused_ewald) {
        const int stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
        const int warps = 8;
        const size_t smem = (size_t)warps * 3 * stride * sizeof(ddc);
        dd iL, two_pi;
        SplitDouble(sys.iL, iL.hi, iL.lo);
        SplitDouble(2. * M_PI, two_pi.hi, two_pi.lo);
        const size_t mk = (size_t)sys.M * sys.K;
        for (uint32_t s = 0; s < sys.S; ++s) {
            // the selected long-range actions acting on species s, each with its other species' densities
            std::vector<const float2*> vks;
            std::vector<int> slots;
            for (size_t i = 0; i < actions.size(); ++i) {
                const ActionHost& ah = actions[i];
                if (!Selected(ah, a, (int)i) || ah.kind != 2) continue;
                const PairDev& pa = sys.pair[ah.index];
                if (pa.is_constant || !pa.use_long_range || (pa.sa != s && pa.sb != s)) continue;
                const uint32_t o = pa.sa == s ? pa.sb : pa.sa;
                vks.push_back(adj_vk_[i]->as<float2>());
                slots.push_back(sys.sp_rho[o]);
            }
            if (vks.empty()) continue;
            if (!ewald_w_ || ewald_w_->bytes < mk * sizeof(float4)) ewald_w_.reset(new DeviceBuffer(mk * sizeof(float4)));
            if (!ewald_terms_) ewald_terms_.reset(new DeviceBuffer(kMaxPair * (sizeof(const float2*) + sizeof(int))));
            if (vks.size() > (size_t)kMaxPair) throw PimcError(kErrUnsupported, "more long-range actions on a species than the fused Ewald gradient takes");
            const float2** dv = reinterpret_cast<const float2**>(ewald_terms_->ptr);
            int* ds = reinterpret_cast<int*>(static_cast<char*>(ewald_terms_->ptr) + kMaxPair * sizeof(const float2*));
            CudaCheck(cudaMemcpyAsync(dv, vks.data(), vks.size() * sizeof(const float2*), cudaMemcpyHostToDevice, stream), "ewald terms");
            CudaCheck(cudaMemcpyAsync(ds, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice, stream), "ewald terms");
            EwaldWeightKernel<<<Blocks(*this, mk, th), th, 0, stream>>>(sys, rho, dv, ds, (uint32_t)vks.size(), ewald_w_->as<float4>());
            const uint64_t nbeads = (uint64_t)sys.sp_n[s] * sys.M;
            const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((nbeads + warps - 1) / warps, (uint64_t)n_sm * 16));
            EwaldGradSpeciesKernel<<<blocks, warps * 32, smem, stream>>>(sys, pos, s, ewald_w_->as<float4>(), phase_tab_->as<float4>(), iL, two_pi, grad);
            CudaCheck(cudaGetLastError(), "ewald gradient launch");
            // (the next species' terms and weight reuse both buffers after these kernels, in stream order)
        }
    }
}

double Context::TotalAction(int a, int mode) {
    EnsureFP64();
    if (a >= (int)actions.size() || a < -1) throw PimcError(kErrArg, "action index out of range");
    const double* pos = mode ? sys.pos_new : sys.pos;
    return TotalActionDev(a, pos, ScratchRho(pos));
}

void Context::ActionGradientPath(int a, int mode, double* host) {
    EnsureFP64();
    if (a >= (int)actions.size() || a < -1) throw PimcError(kErrArg, "action index out of range");
    if (!host) throw PimcError(kErrArg, "null output");
    const double* pos = mode ? sys.pos_new : sys.pos;
    const size_t n = (size_t)sys.M * 3 * sys.n_pad;
    if (!grad_ || grad_->bytes < n * sizeof(double)) grad_.reset(new DeviceBuffer(n * sizeof(double)));
    GradientDev(a, pos, ScratchRho(pos), grad_->as<double>());
    std::vector<double> g(n);
    CudaCheck(cudaMemcpyAsync(g.data(), grad_->ptr, n * sizeof(double), cudaMemcpyDeviceToHost, stream), "gradient download");
    Sync();
    for (uint32_t gi = 0; gi < sys.n_total; ++gi)
        for (uint32_t b = 0; b < sys.M; ++b)
            for (uint32_t d = 0; d < sys.n_d; ++d) host[((size_t)gi * sys.M + b) * sys.n_d + d] = g[((size_t)b * 3 + d) * sys.n_pad + gi];
}

/// Action::GetActionGradient with the exact gradient: the sum of dS_a/dr over the listed
/// particles of the action's species and slices b0 .. b1-1 (level 0 only).
void Context::ActionGradientAdjoint(uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level,
                                    int mode, double* out) {
    if (a >= actions.size()) throw PimcError(kErrArg, "action index out of range");
    if (level != 0) throw PimcError(kErrUnsupported, "the exact gradient is defined at level 0");
    if (b1 < b0) throw PimcError(kErrArg, "b1 < b0");
    std::vector<double> g((size_t)sys.n_total * sys.M * sys.n_d);
    ActionGradientPath((int)a, mode, g.data());
    for (uint32_t d = 0; d < sys.n_d; ++d) out[d] = 0.;
    const auto& sl = actions[a].species_list;
    for (uint32_t i = 0; i < n; ++i) {
        if (sp[i] >= sys.S || p[i] >= sys.sp_n[sp[i]]) throw PimcError(kErrArg, "particle out of range");
        if (std::find(sl.begin(), sl.end(), sp[i]) == sl.end()) continue;
        const uint32_t gi = sys.sp_off[sp[i]] + p[i];
        for (uint32_t b = b0; b < b1; ++b)
            for (uint32_t d = 0; d < sys.n_d; ++d) out[d] += g[((size_t)gi * sys.M + (b % sys.M)) * sys.n_d + d];
    }
}

/// Virial centroid term of energy_class.h:78-94 with the exact gradient of every non-kinetic
/// action (trap and Ewald forces included): sum over the species' particles and slices of
/// dS/dr_{p,b} . (r_{p,b} - r_{p,0}).
double Context::VirialCentroidAdjoint(uint32_t s) {
    EnsureFP64();
    const size_t n = (size_t)sys.M * 3 * sys.n_pad;
    if (!grad_ || grad_->bytes < n * sizeof(double)) grad_.reset(new DeviceBuffer(n * sizeof(double)));
    double* grad = grad_->as<double>();
    GradientDev(-2, sys.pos, ScratchRho(sys.pos), grad);
    const double* pos = sys.pos;
    const uint32_t ns = sys.sp_n[s], off = sys.sp_off[s], M = sys.M, np = sys.n_pad, n_d = sys.n_d;
    const double L = sys.L, iL = sys.iL;
    double total = 0.;
    SumItems<1>(*this, (uint64_t)ns * M, [=] __device__(uint64_t it, double* v) {
        const uint32_t b = (uint32_t)(it / ns), g = off + (uint32_t)(it % ns);
        double s2 = 0.;
        for (uint32_t d = 0; d < n_d; ++d)
            s2 += grad[GIdx(b, d, g, np)] * MinImage(PosAt(pos, np, b, d, g) - PosAt(pos, np, 0, d, g), L, iL);
        v[0] = s2;
    }, &total);
    return total;
}

/// Hybrid Monte Carlo over the whole path of the moving species: momenta P ~ N(0, 1) per
/// coordinate, `hmc_steps` leapfrog steps of size `hmc_step` on H = S(R) + |P|^2 / 2 with the
/// exact gradient, accepted with probability min(1, exp(-dH)) against the same log-uniform draw
/// layout as a bisection level (Philox block 0, word 0).
void Context::HmcAttempts(uint32_t m, uint64_t n_att) {
    MoveHost& mh = moves[m];
    EnsureFP64();
    const size_t n = (size_t)sys.M * 3 * sys.n_pad;
    auto ensure = [&](std::unique_ptr<DeviceBuffer>& b) {
        if (!b || b->bytes < n * sizeof(double)) b.reset(new DeviceBuffer(n * sizeof(double)));
    };
    ensure(grad_);
    ensure(mom_);
    ensure(pos_save_);
    double* grad = grad_->as<double>();
    double* mom = mom_->as<double>();
    double* pos = sys.pos;
    std::vector<uint32_t> moving;
    for (uint32_t s = 0; s < sys.S; ++s)
        if (mh.hmc_species < 0 || (uint32_t)mh.hmc_species == s)
            for (uint32_t p = 0; p < sys.sp_n[s]; ++p) moving.push_back(sys.sp_off[s] + p);
    uint32_t* dmov = Parts(moving.size());
    CudaCheck(cudaMemcpyAsync(dmov, moving.data(), moving.size() * 4, cudaMemcpyHostToDevice, stream), "moving upload");
    const double eps = mh.hmc_step;
    const int th = 256;
    auto kinetic_energy = [&]() {
        double k = 0.;
        SumItems<1>(*this, n, [=] __device__(uint64_t i, double* v) { v[0] = 0.5 * mom[i] * mom[i]; }, &k);
        return k;
    };
    for (uint64_t it = 0; it < n_att; ++it) {
        const MoveStream st{seed, chain, m, mh.attempts};
        CudaCheck(cudaMemsetAsync(mom, 0, n * sizeof(double), stream), "momenta clear");
        const uint64_t nm = (uint64_t)moving.size() * sys.M * sys.n_d;
        HmcMomentaKernel<<<Blocks(*this, nm, th), th, 0, stream>>>(sys, st, dmov, (uint32_t)moving.size(), mom);
        CudaCheck(cudaGetLastError(), "momenta launch");
        CudaCheck(cudaMemcpyAsync(pos_save_->ptr, pos, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "save path");
        const double h0 = TotalActionDev(-1, pos, ScratchRho(pos)) + kinetic_energy();
        // Leapfrog: half kick, (drift, kick) x steps with a half final kick.
        GradientDev(-1, pos, ScratchRho(pos), grad);
        AxpyKernel<<<Blocks(*this, n, th), th, 0, stream>>>(mom, grad, -0.5 * eps, n);
        for (uint32_t s = 0; s < mh.hmc_steps; ++s) {
            AxpyKernel<<<Blocks(*this, n, th), th, 0, stream>>>(pos, mom, eps, n);
            GradientDev(-1, pos, ScratchRho(pos), grad);
            AxpyKernel<<<Blocks(*this, n, th), th, 0, stream>>>(mom, grad, s + 1 == mh.hmc_steps ? -0.5 * eps : -eps, n);
        }
        CudaCheck(cudaGetLastError(), "leapfrog launch");
        const double h1 = TotalActionDev(-1, pos, ScratchRho(pos)) + kinetic_energy();
        const double log_accept = -(h1 - h0);
        const Philox4 w0 = st.Block(0);
        const double logu = (double)LogF(U24(w0.v[0]));
        const bool accept = std::isfinite(log_accept) && !(log_accept < logu);
        if (accept) {
            CudaCheck(cudaMemcpyAsync(sys.pos_new, pos, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "commit");
            InitRhoK();
            mh.block_accept++;
            mh.total_accept++;
        } else {
            CudaCheck(cudaMemcpyAsync(pos, pos_save_->ptr, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "restore");
        }
        mh.attempts++;
        mh.block_attempt++;
        mh.total_level0++;
    }
    Sync();
    fp64_valid = true;
    dd_valid = false;
}

}  // namespace pimc
