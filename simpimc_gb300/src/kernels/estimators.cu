// Action-interface and estimator kernels: GetAction / GetActionGradient for one action on a path
// segment, DActionDBeta, Potential, VirialEnergy, the virial centroid term, the charge-density
// initialisation and the g(r) / S(k) accumulators.
//
// Every scalar result is a deterministic two-pass reduction (fixed per-block tree, then one warp
// over the block partials in block order), so repeated calls on the same state agree bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../framework/context.h"
#include "actions.cuh"
#include "reduce.cuh"

namespace pimc {

namespace {

__device__ __forceinline__ uint32_t BeadLoop(uint32_t b, uint32_t M) { return b >= M ? b - M : b; }

// InitRhoK (species_class.h:380-403): rho(b, k) = sum over particles in index order of the bead
// phases, formed in double-float by the densities kernel of the adjoint (Context::ScratchRho: one
// block per (1024 k-vectors, slice, slot), the particles' phase rows staged in shared memory) and
// rounded to FP64 here.
__global__ void DDToDoubleKernel(const float4* __restrict__ in, double2* __restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = in[i];
        out[i] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
    }
}

__global__ void ProposalRhoKernel(const SystemDev sys, uint32_t species, const uint32_t* __restrict__ parts, uint32_t n_parts,
                                  uint32_t b0, uint32_t skip, double2* __restrict__ out) {
    extern __shared__ double2 tab[];  // [2][3][stride]
    const uint32_t j = blockIdx.x;
    const uint32_t b = BeadLoop(b0 + j * skip, sys.M);
    const int stride = max(max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const double2* committed = sys.rho_k + ((size_t)sys.sp_rho[species] * sys.M + b) * sys.K;
    double2* dst = out + (size_t)j * sys.K;
    for (uint32_t k = threadIdx.x; k < sys.K; k += blockDim.x) dst[k] = committed[k];
    for (uint32_t q = 0; q < n_parts; ++q) {
        const uint32_t g = sys.sp_off[species] + parts[q];
        __syncthreads();
        if (threadIdx.x < 2 * sys.n_d) {
            const uint32_t which = threadIdx.x / sys.n_d, d = threadIdx.x % sys.n_d;
            const double x = PosAt(which ? sys.pos_new : sys.pos, sys.n_pad, b, d, g);
            PhaseRow(x, sys.box[d], sys.max_index[d], tab + ((size_t)which * 3 + d) * stride);
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < sys.K; k += blockDim.x) {
            const int32_t pk = sys.kidx[k];
            const double2 en = PhaseProduct(tab + (size_t)3 * stride, stride, sys.n_d, pk);
            const double2 eo = PhaseProduct(tab, stride, sys.n_d, pk);
            double2 v = dst[k];
            v.x += en.x - eo.x;
            v.y += en.y - eo.y;
            dst[k] = v;
        }
    }
}

// g(r) histogram (pair_correlation_class.h:15-28): shared-memory counts, then global atomics.
// The sign cofactor (pair_correlation_class.h:17) enters as a signed increment of the counts.
__global__ void PairCorrelationKernel(const SystemDev sys, uint32_t sa, uint32_t sb, double r_min, double d_ir, uint32_t n_r,
                                      long long sign, unsigned long long* __restrict__ hist) {
    extern __shared__ unsigned int counts[];
    for (uint32_t i = threadIdx.x; i < n_r; i += blockDim.x) counts[i] = 0u;
    __syncthreads();
    const uint32_t na = sys.sp_n[sa], nb = sys.sp_n[sb];
    const uint64_t n_items = (uint64_t)sys.M * na * nb;
    for (uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; it < n_items; it += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(it / ((uint64_t)na * nb));
        const uint32_t rem = (uint32_t)(it % ((uint64_t)na * nb));
        const uint32_t p = rem / nb, q = rem % nb;
        if (sa == sb && q <= p) continue;
        double ra[3], rb[3];
        LoadBead(sys.pos, sys.n_pad, sys.n_d, b, sys.sp_off[sa] + p, ra);
        LoadBead(sys.pos, sys.n_pad, sys.n_d, b, sys.sp_off[sb] + q, rb);
        const double r = DistMinImage(ra, rb, sys.n_d, sys.L, sys.iL);
        // observable_class.h:56-62; a negative index wraps as the reference's unsigned cast does.
        const uint32_t i = (uint32_t)(long long)rint((r - r_min) * d_ir - 0.5);
        if (i < n_r) atomicAdd(&counts[i], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n_r; i += blockDim.x)
        if (counts[i]) atomicAdd(&hist[i], (unsigned long long)(sign * (long long)counts[i]));
}

// S(k) accumulation (structure_factor_class.h:15-32) in the reference's order: one thread per k
// adds the slice terms one by one into the running sum.
__global__ void StructureFactorKernel(const SystemDev sys, const double* __restrict__ kmag, double k_cut, uint32_t slot_a,
                                      uint32_t slot_b, double cofactor, double* __restrict__ sk) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= sys.K || !(kmag[k] < k_cut)) return;
    const double2* ra = sys.rho_k + (size_t)slot_a * sys.M * sys.K;
    const double2* rb = sys.rho_k + (size_t)slot_b * sys.M * sys.K;
    double acc = sk[k];
    for (uint32_t b = 0; b < sys.M; ++b) {
        const double2 a = ra[(size_t)b * sys.K + k], c = rb[(size_t)b * sys.K + k];
        acc += cofactor * (a.x * c.x + a.y * c.y);
    }
    sk[k] = acc;
}

// IlkkaPairAction::CalcGradientULong of one bead (ilkka_pair_action_class.h:231-249):
// sum_k u_long_k k (Re rho_g Im rho_B - Im rho_g Re rho_B), rho_g = exp(i k . r_g) the bead's own
// density and rho_B species b's density on the slice, x2 for two species. One block per (listed
// particle, slice); out[(i * n_slices + j) * 3 + d].
__global__ void IlkkaLongGradKernel(const SystemDev sys, const double* __restrict__ pos, const double* __restrict__ uk,
                                    const uint32_t* __restrict__ glist, uint32_t n_slices, uint32_t b0, uint32_t skip,
                                    const double2* __restrict__ rho_b, int rho_b_slice_major, double scale, double* __restrict__ out) {
    __shared__ double red[3][32];
    const uint32_t i = blockIdx.x / n_slices, j = blockIdx.x % n_slices;
    const uint32_t b = (b0 + j * skip) % sys.M, g = glist[i];
    double r[3];
    LoadBead(pos, sys.n_pad, sys.n_d, b, g, r);
    double acc[3] = {0., 0., 0.};
    for (uint32_t k = threadIdx.x; k < sys.K; k += blockDim.x) {
        const int32_t pk = sys.kidx[k];
        double kv[3] = {0., 0., 0.}, kr = 0.;
        for (uint32_t d = 0; d < sys.n_d; ++d) {
            kv[d] = KIdx(pk, (int)d) * sys.box[d];
            kr += kv[d] * r[d];
        }
        double sn, cs;
        sincos(kr, &sn, &cs);
        const double2 rb = rho_b_slice_major ? rho_b[(size_t)j * sys.K + k] : rho_b[(size_t)b * sys.K + k];
        const double f = uk[k] * (cs * rb.y - sn * rb.x);
        for (uint32_t d = 0; d < 3; ++d) acc[d] += f * kv[d];
    }
    for (int d = 0; d < 3; ++d) {
        double v = acc[d];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[d][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.;
        for (uint32_t w = 0; w < (blockDim.x + 31) / 32; ++w) v += red[threadIdx.x][w];
        out[(size_t)blockIdx.x * 3 + threadIdx.x] = scale * v;
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------
void Context::ComputeRho(const double* pos, double2* out) {
    if (!rho_slots || !sys.K) return;
    const float4* r = ScratchRho(pos);
    const size_t n = (size_t)rho_slots * sys.M * sys.K;
    DDToDoubleKernel<<<(unsigned)std::min<size_t>((n + 255) / 256, (size_t)n_sm * 16), 256, 0, stream>>>(r, out, n);
    CudaCheck(cudaGetLastError(), "init rho_k launch");
    Sync();
}

void Context::InitRhoK() {
    if (!rho_slots || !sys.K) return;
    ComputeRho(sys.pos, sys.rho_k);
    dd_valid = false;
}

static void SpeciesParticles(const Context& c, uint32_t s, const uint32_t* sp, const uint32_t* p, uint32_t n, std::vector<uint32_t>& out) {
    for (uint32_t i = 0; i < n; ++i)
        if (sp[i] == s) {
            if (p[i] >= c.sys.sp_n[s]) throw PimcError(kErrArg, "particle index out of range");
            out.push_back(p[i]);
        }
}

// PairAction::GenerateParticlePairs (pair_action_class.h:62-114).
static void GenPairs(const Context& c, const PairDev& pa, const uint32_t* sp, const uint32_t* p, uint32_t n, std::vector<uint32_t>& pa_list,
                     std::vector<uint32_t>& pb_list, std::vector<uint32_t>& pairs) {
    for (uint32_t i = 0; i < n; ++i) {
        if (sp[i] >= c.sys.S || p[i] >= c.sys.sp_n[sp[i]]) throw PimcError(kErrArg, "particle out of range");
        if (sp[i] == pa.sa) pa_list.push_back(p[i]);
        else if (sp[i] == pa.sb) pb_list.push_back(p[i]);
    }
    if (pa_list.empty() && pb_list.empty()) return;
    std::vector<uint32_t> oa, ob;
    for (uint32_t i = 0; i < c.sys.sp_n[pa.sa]; ++i)
        if (std::find(pa_list.begin(), pa_list.end(), i) == pa_list.end()) oa.push_back(i);
    for (uint32_t i = 0; i < c.sys.sp_n[pa.sb]; ++i)
        if (std::find(pb_list.begin(), pb_list.end(), i) == pb_list.end()) ob.push_back(i);
    auto add = [&](uint32_t x, uint32_t y) {
        pairs.push_back(x);
        pairs.push_back(y);
    };
    if (pa.sa == pa.sb) {
        for (auto x : pa_list)
            for (auto y : oa) add(x, y);
        for (size_t i = 0; i + 1 < pa_list.size(); ++i)
            for (size_t j = i + 1; j < pa_list.size(); ++j) add(pa_list[i], pa_list[j]);
    } else {
        for (auto x : pa_list)
            for (auto y : ob) add(x, y);
        for (auto x : pb_list)
            for (auto y : oa) add(y, x);
        for (auto x : pa_list)
            for (auto y : pb_list) add(x, y);
    }
}

static uint32_t CountLinks(uint32_t b0, uint32_t b1, uint32_t skip, uint32_t M) {
    const uint32_t a0 = b0 % M, end = b1 % M;
    uint32_t a = a0, n = 0;
    while (a != end) {
        a = (a + skip) % M;
        if (++n > M) throw PimcError(kErrArg, "segment end is not reachable at this level");
    }
    return n;
}

// The pair links of slices b0, b0 + skip, ... (ns of them) reach slice b0 + ns skip, and the
// gradient's backward links slice b + M - skip (pair_action_class.h:281-283, 320-322). The reference
// wraps those indices once (bead_loop, species_class.h:101) and reads past its bead array beyond
// 2M; such ranges are refused here.
static void CheckPairSlices(uint32_t b0, uint32_t ns, uint32_t skip, uint32_t M, bool gradient) {
    uint64_t hi = (uint64_t)b0 + (uint64_t)ns * skip;
    if (gradient && ns) hi = std::max<uint64_t>(hi, (uint64_t)b0 + (uint64_t)(ns - 1) * skip + M - skip);
    if (hi >= 2ull * M) throw PimcError(kErrArg, "slice range reaches past one wrap of the ring at this level");
}

double Context::GetAction(uint32_t ai, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level, int mode) {
    EnsureFP64();
    if (ai >= actions.size()) throw PimcError(kErrArg, "action index out of range");
    if (level >= (uint32_t)kMaxLevels) throw PimcError(kErrArg, "level out of range");
    if (b1 < b0 || b0 >= sys.M || b1 - b0 > sys.M) throw PimcError(kErrArg, "slice range out of bounds");
    const ActionHost& ah = actions[ai];
    const double* pos = mode ? sys.pos_new : sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL;
    const uint32_t skip = 1u << level;
    double out = 0.;
    if (ah.kind == 0) {
        const KineticDev k = sys.kinetic[ah.index];
        if (k.image[level].n == 0) throw PimcError(kErrArg, "no kinetic spline for this level");
        std::vector<uint32_t> list;
        SpeciesParticles(*this, k.species, sp, p, n, list);
        const bool exch = !PermIdentity(k.species);
        uint32_t nl;
        if (!exch) {
            nl = CountLinks(b0, b1, skip, M);
        } else {
            // links follow the path permutation at the ring closure (kinetic_class.h:112-119)
            if ((b1 - b0) % skip) throw PimcError(kErrArg, "segment is not a whole number of links at this level");
            nl = (b1 - b0) / skip;
        }
        if (list.empty() || nl == 0) return 0.;
        uint32_t* dl = Parts(list.size());
        for (auto& x : list) x += sys.sp_off[k.species];
        CudaCheck(cudaMemcpyAsync(dl, list.data(), list.size() * 4, cudaMemcpyHostToDevice, stream), "parts upload");
        const uint32_t a0 = b0 % M;
        const double i4 = k.i4lt_level[level];
        const uint32_t* perm = sys.perm;
        const bool whole = b1 - b0 == M;
        SumItems<1>(*this, (uint64_t)list.size() * nl, [=] __device__(uint64_t i, double* v) {
            const uint32_t g = dl[i / nl], j = (uint32_t)(i % nl);
            v[0] = 0.;
            if (exch && whole && perm[g] == g) return;  // the walk's end is its start bead: no links
            const uint32_t q0 = a0 + j * skip, q1 = q0 + skip;
            const uint32_t ga = (exch && q0 >= M) ? perm[g] : g, gn = (exch && q1 >= M) ? perm[g] : g;
            const uint32_t a = q0 % M, nx = q1 % M;
            double dr[3];
            for (uint32_t d = 0; d < n_d; ++d) dr[d] = MinImage(PosAt(pos, np, a, d, ga) - PosAt(pos, np, nx, d, gn), L, iL);
            v[0] = -LogRhoFree(dr, n_d, i4, &k.image[level], k.has_images);
        }, &out);
        return out;
    }
    if (ah.kind == 1) {
        const TrapDev t = sys.trap[ah.index];
        if (level > t.max_level) return 0.;
        bool check = false;
        for (uint32_t i = 0; i < n; ++i) check |= (sp[i] == t.species);
        if (!check) return 0.;
        // trap_class.h:53-58 reads the trap species' bead with every listed particle's index.
        std::vector<uint32_t> list;
        for (uint32_t i = 0; i < n; ++i) {
            if (p[i] >= sys.sp_n[t.species]) throw PimcError(kErrArg, "particle index out of range for the trap species");
            list.push_back(sys.sp_off[t.species] + p[i]);
        }
        const uint32_t ns = b1 > b0 ? (b1 - b0 + skip - 1) / skip : 0;
        if (ns == 0) return 0.;
        uint32_t* dl = Parts(list.size());
        CudaCheck(cudaMemcpyAsync(dl, list.data(), list.size() * 4, cudaMemcpyHostToDevice, stream), "parts upload");
        SumItems<1>(*this, (uint64_t)list.size() * ns, [=] __device__(uint64_t i, double* v) {
            const uint32_t g = dl[i / ns], j = (uint32_t)(i % ns);
            const uint32_t b = BeadLoop(b0 + j * skip, M);
            double s = 0.;
            for (uint32_t d = 0; d < n_d; ++d) {
                const double x = PosAt(pos, np, b, d, g);
                s += x * x;
            }
            v[0] = s;
        }, &out);
        return t.cofactor_a * skip * out;
    }
    // Bare pair action (pair_action_class.h:267-302).
    const PairDev pa = sys.pair[ah.index];
    if (level > pa.max_level || pa.is_constant) return 0.;
    std::vector<uint32_t> la, lb, pairs;
    GenPairs(*this, pa, sp, p, n, la, lb, pairs);
    const uint32_t npairs = (uint32_t)(pairs.size() / 2);
    if (npairs == 0) return 0.;
    const uint32_t ns = (b1 - b0 + skip - 1) / skip;
    CheckPairSlices(b0, ns, skip, M, false);
    uint32_t* dp = Pairs(npairs);
    CudaCheck(cudaMemcpyAsync(dp, pairs.data(), pairs.size() * 4, cudaMemcpyHostToDevice, stream), "pairs upload");
    const uint32_t offa = sys.sp_off[pa.sa], offb = sys.sp_off[pa.sb];
    const double tau = sys.tau;
    double tot = 0.;
    SumItems<1>(*this, (uint64_t)ns * npairs, [=] __device__(uint64_t i, double* v) {
        const uint32_t j = (uint32_t)(i / npairs), q = (uint32_t)(i % npairs);
        const uint32_t bi = BeadLoop(b0 + j * skip, M), bj = BeadLoop(b0 + j * skip + skip, M);
        double A0[3], C0[3], A1[3], C1[3];
        LoadBead(pos, np, n_d, bi, offb + dp[2 * q + 1], A0);
        LoadBead(pos, np, n_d, bi, offa + dp[2 * q], C0);
        LoadBead(pos, np, n_d, bj, offb + dp[2 * q + 1], A1);
        LoadBead(pos, np, n_d, bj, offa + dp[2 * q], C1);
        double r, rp, s;
        DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, s);
        v[0] = PairU(pa, r, rp, s, level, tau);
    }, &tot);
    if (pa.use_long_range) {
        const uint32_t K = sys.K;
        const int stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
        const double2* ra;
        const double2* rb;
        if (mode) {
            double2* tmp = RhoTmp((size_t)2 * ns * K);
            const std::vector<uint32_t>* lists[2] = {&la, &lb};
            const uint32_t spc[2] = {pa.sa, pa.sb};
            // A homologous action has one species: its updated density serves as both factors
            // (species_a and species_b are the same object in pair_action_class.h:294-298).
            const int n_species = pa.sa == pa.sb ? 1 : 2;
            for (int x = 0; x < n_species; ++x) {
                uint32_t* dl = Parts(std::max<size_t>(1, lists[x]->size()));
                if (!lists[x]->empty())
                    CudaCheck(cudaMemcpyAsync(dl, lists[x]->data(), lists[x]->size() * 4, cudaMemcpyHostToDevice, stream), "parts upload");
                ProposalRhoKernel<<<ns, 256, (size_t)2 * 3 * stride * sizeof(double2), stream>>>(sys, spc[x], dl, (uint32_t)lists[x]->size(), b0,
                                                                                               skip, tmp + (size_t)x * ns * K);
                CudaCheck(cudaGetLastError(), "proposal rho launch");
                Sync();  // `Parts` is reused by the next species
            }
            ra = tmp;
            rb = n_species == 1 ? tmp : tmp + (size_t)ns * K;
        } else {
            ra = rb = nullptr;
        }
        const double2* rho = sys.rho_k;
        const int slot_a = sys.sp_rho[pa.sa], slot_b = sys.sp_rho[pa.sb];
        // bare: tau 2^level v_long_k (bare_pair_action_class.h:126-144); Ilkka and David: u_long_k
        // (ilkka_pair_action_class.h:104-122, david_pair_action_class.h:105-123)
        const double* vk = pa.kind != kPairBare ? pa.u_long_k : pa.v_long_k;
        double lr = 0.;
        SumItems<1>(*this, (uint64_t)K * ns, [=] __device__(uint64_t i, double* v) {
            const uint32_t k = (uint32_t)(i / ns), j = (uint32_t)(i % ns);
            double2 a, c;
            if (ra) {
                a = ra[(size_t)j * K + k];
                c = rb[(size_t)j * K + k];
            } else {
                const uint32_t b = BeadLoop(b0 + j * skip, M);
                a = rho[((size_t)slot_a * M + b) * K + k];
                c = rho[((size_t)slot_b * M + b) * K + k];
            }
            v[0] = vk[k] * (a.x * c.x + a.y * c.y);
        }, &lr);
        if (pa.sa != pa.sb) lr *= 2.;
        tot += pa.kind != kPairBare ? lr : skip * sys.tau * lr;
    }
    return tot;
}

void Context::GetActionGradient(uint32_t ai, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level,
                                int mode, double* g) {
    EnsureFP64();
    if (ai >= actions.size()) throw PimcError(kErrArg, "action index out of range");
    if (level >= (uint32_t)kMaxLevels) throw PimcError(kErrArg, "level out of range");
    if (b1 < b0 || b0 >= sys.M || b1 - b0 > sys.M) throw PimcError(kErrArg, "slice range out of bounds");
    for (uint32_t d = 0; d < 3; ++d) g[d] = 0.;
    const ActionHost& ah = actions[ai];
    const double* pos = mode ? sys.pos_new : sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL;
    const uint32_t skip = 1u << level;
    if (ah.kind == 0) {
        // kinetic_class.h:125-144
        const KineticDev k = sys.kinetic[ah.index];
        std::vector<uint32_t> list;
        SpeciesParticles(*this, k.species, sp, p, n, list);
        const bool exch = !PermIdentity(k.species);
        uint32_t nl;
        if (!exch) {
            nl = CountLinks(b0, b1, skip, M);
        } else {
            if ((b1 - b0) % skip) throw PimcError(kErrArg, "segment is not a whole number of links at this level");
            nl = (b1 - b0) / skip;
        }
        if (list.empty() || nl == 0) return;
        for (auto& x : list) x += sys.sp_off[k.species];
        uint32_t* dl = Parts(list.size());
        CudaCheck(cudaMemcpyAsync(dl, list.data(), list.size() * 4, cudaMemcpyHostToDevice, stream), "parts upload");
        const uint32_t a0 = b0 % M;
        const uint32_t* perm = sys.perm;
        const uint32_t* perm_inv = sys.perm_inv;
        const bool whole = b1 - b0 == M;
        double t[3];
        SumItems<3>(*this, (uint64_t)list.size() * nl, [=] __device__(uint64_t i, double* v) {
            const uint32_t gg = dl[i / nl], j = (uint32_t)(i % nl);
            v[0] = v[1] = v[2] = 0.;
            if (exch && whole && perm[gg] == gg) return;
            // GetPrevBead(skip) / GetNextBead(skip) across the ring closure (kinetic_class.h:133-136)
            const int q = (int)(a0 + j * skip), qp = q - (int)skip, qn = q + (int)skip;
            auto lab = [&](int x) -> uint32_t {
                if (!exch) return gg;
                return x < 0 ? perm_inv[gg] : (x >= (int)M ? perm[gg] : gg);
            };
            auto slc = [&](int x) -> uint32_t { return (uint32_t)(((x % (int)M) + (int)M) % (int)M); };
            const uint32_t a = slc(q), nx = slc(qn), pv = slc(qp);
            const uint32_t ga = lab(q), gn = lab(qn), gp = lab(qp);
            for (uint32_t d = 0; d < 3; ++d) {
                if (d >= n_d) {
                    v[d] = 0.;
                    continue;
                }
                const double ra = PosAt(pos, np, a, d, ga);
                const double dprev = MinImage(PosAt(pos, np, pv, d, gp) - ra, L, iL);
                const double dnext = MinImage(ra - PosAt(pos, np, nx, d, gn), L, iL);
                v[d] = -dprev + dnext;
            }
        }, t);
        const double i4 = k.i4lt / skip;
        for (uint32_t d = 0; d < n_d; ++d) g[d] = 2. * i4 * t[d];
        return;
    }
    if (ah.kind == 1) return;  // trap_class.h has no gradient: the base class returns zeros.
    const PairDev pa = sys.pair[ah.index];
    if (level > pa.max_level || pa.is_constant) return;
    std::vector<uint32_t> la, lb, pairs;
    GenPairs(*this, pa, sp, p, n, la, lb, pairs);
    const uint32_t npairs = (uint32_t)(pairs.size() / 2);
    if (npairs == 0) return;
    const uint32_t ns = (b1 - b0 + skip - 1) / skip;
    CheckPairSlices(b0, ns, skip, M, true);
    uint32_t* dp = Pairs(npairs);
    CudaCheck(cudaMemcpyAsync(dp, pairs.data(), pairs.size() * 4, cudaMemcpyHostToDevice, stream), "pairs upload");
    const uint32_t offa = sys.sp_off[pa.sa], offb = sys.sp_off[pa.sb];
    const double tau = sys.tau;
    if (pa.kind == kPairIlkka) {
        // pair_action_class.h:318-334 with IlkkaPairAction's analytic link gradient
        // (ilkka_pair_action_class.h:172-222), links to b + skip and b - skip (+M).
        SumItems<3>(*this, (uint64_t)ns * npairs * 2, [=] __device__(uint64_t i, double* v) {
            const uint32_t link = (uint32_t)(i & 1u);
            const uint64_t ii = i >> 1;
            const uint32_t j = (uint32_t)(ii / npairs), q = (uint32_t)(ii % npairs);
            const uint32_t braw = b0 + j * skip;
            const uint32_t bi = BeadLoop(braw, M);
            const uint32_t bo = link == 0 ? BeadLoop(braw + skip, M) : BeadLoop(braw - skip + M, M);
            double A0[3], C0[3], A1[3], C1[3];
            LoadBead(pos, np, n_d, bi, offb + dp[2 * q + 1], A0);
            LoadBead(pos, np, n_d, bi, offa + dp[2 * q], C0);
            LoadBead(pos, np, n_d, bo, offb + dp[2 * q + 1], A1);
            LoadBead(pos, np, n_d, bo, offa + dp[2 * q], C1);
            IlkkaGradientU(pa, A0, C0, A1, C1, n_d, L, iL, v);
        }, g);
        if (pa.use_long_range && sys.K) {
            // CalcGradientULong once per pair, on the pair's first particle (pair_action_class.h:331-334;
            // ilkka_pair_action_class.h:231-249): the listed first particles with their multiplicity.
            std::vector<uint32_t> firsts(npairs);
            for (uint32_t q = 0; q < npairs; ++q) firsts[q] = offa + pairs[2 * q];
            const double2* rb = sys.rho_k + (size_t)sys.sp_rho[pa.sb] * M * sys.K;
            int slice_major = 0;
            // One scratch block: [NEW-mode densities of species b, ns x K][per (pair, slice) gradients].
            const size_t n_rho = mode ? (size_t)ns * sys.K : 0;
            double2* scratch = RhoTmp(n_rho + ((size_t)npairs * ns * 3 + 1) / 2 + 1);
            double* outg = reinterpret_cast<double*>(scratch + n_rho);
            if (mode) {
                // NEW mode: species b's density with the listed particles at their new positions, as GetAction forms it.
                const int stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
                const std::vector<uint32_t>& lst = pa.sa == pa.sb ? la : lb;
                uint32_t* dl = Parts(std::max<size_t>(1, lst.size()));
                if (!lst.empty()) CudaCheck(cudaMemcpyAsync(dl, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice, stream), "parts upload");
                ProposalRhoKernel<<<ns, 256, (size_t)2 * 3 * stride * sizeof(double2), stream>>>(sys, pa.sb, dl, (uint32_t)lst.size(), b0, skip,
                                                                                               scratch);
                CudaCheck(cudaGetLastError(), "proposal rho launch");
                Sync();  // `Parts` is reused below
                rb = scratch;
                slice_major = 1;
            }
            uint32_t* dg = Parts(firsts.size());
            CudaCheck(cudaMemcpyAsync(dg, firsts.data(), firsts.size() * 4, cudaMemcpyHostToDevice, stream), "parts upload");
            IlkkaLongGradKernel<<<npairs * ns, 256, 0, stream>>>(sys, pos, pa.u_long_k, dg, ns, b0, skip, rb, slice_major,
                                                                pa.sa != pa.sb ? 2. : 1., outg);
            CudaCheck(cudaGetLastError(), "long-range gradient launch");
            std::vector<double> hg((size_t)npairs * ns * 3);
            CudaCheck(cudaMemcpyAsync(hg.data(), outg, hg.size() * sizeof(double), cudaMemcpyDeviceToHost, stream), "read gradient");
            Sync();
            for (uint32_t q = 0; q < npairs; ++q)
                for (uint32_t d = 0; d < n_d; ++d) {
                    double t = 0.;
                    for (uint32_t j = 0; j < ns; ++j) t += hg[((size_t)q * ns + j) * 3 + d];
                    g[d] += t;
                }
        }
        return;
    }
    // pair_action_class.h:135-155 central differences on the first particle's bead, links to
    // b + skip and to b - skip (+M), eps = 1e-4. The Bare action has no long-range gradient.
    SumItems<3>(*this, (uint64_t)ns * npairs * 2, [=] __device__(uint64_t i, double* v) {
        const uint32_t link = (uint32_t)(i & 1u);
        const uint64_t ii = i >> 1;
        const uint32_t j = (uint32_t)(ii / npairs), q = (uint32_t)(ii % npairs);
        const uint32_t braw = b0 + j * skip;
        const uint32_t bi = BeadLoop(braw, M);
        const uint32_t bo = link == 0 ? BeadLoop(braw + skip, M) : BeadLoop(braw - skip + M, M);
        double A0[3], C0[3], A1[3], C1[3];
        LoadBead(pos, np, n_d, bi, offb + dp[2 * q + 1], A0);
        LoadBead(pos, np, n_d, bi, offa + dp[2 * q], C0);
        LoadBead(pos, np, n_d, bo, offb + dp[2 * q + 1], A1);
        LoadBead(pos, np, n_d, bo, offa + dp[2 * q], C1);
        const double eps = 1.e-4;
        for (uint32_t d = 0; d < 3; ++d) {
            if (d >= n_d) {
                v[d] = 0.;
                continue;
            }
            const double c0 = C0[d];
            double r, rp, s;
            C0[d] = c0 + eps;
            DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, s);
            const double f1 = PairU(pa, r, rp, s, level, tau);
            C0[d] = c0 - eps;
            DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, s);
            const double f2 = PairU(pa, r, rp, s, level, tau);
            C0[d] = c0;
            v[d] = (f1 - f2) / (2. * eps);
        }
    }, g);
}

double Context::DActionDBeta(uint32_t ai) {
    EnsureFP64();
    if (ai >= actions.size()) throw PimcError(kErrArg, "action index out of range");
    ActionHost& ah = actions[ai];
    const double* pos = sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL;
    double out = 0.;
    if (ah.kind == 0) {
        // kinetic_class.h:35-45
        const KineticDev k = sys.kinetic[ah.index];
        const uint32_t N = sys.sp_n[k.species], off = sys.sp_off[k.species];
        const uint32_t* perm = sys.perm;
        SumItems<1>(*this, (uint64_t)N * M, [=] __device__(uint64_t i, double* v) {
            const uint32_t g = off + (uint32_t)(i / M), b = (uint32_t)(i % M), bn = (b + 1) % M;
            const uint32_t gn = b + 1 == M ? perm[g] : g;  // GetNextBead(1) across the closure
            double tot = 0., r2 = 0.;
            for (uint32_t d = 0; d < n_d; ++d) {
                const double x = MinImage(PosAt(pos, np, b, d, g) - PosAt(pos, np, bn, d, gn), L, iL);
                if (k.has_images) tot -= EvalCubic(k.d_image_d_tau, x);
                r2 += x * x;
            }
            v[0] = tot - r2 * k.i4ltt;
        }, &out);
        return k.d_action_d_beta_const + out;
    }
    if (ah.kind == 1) {
        const TrapDev t = sys.trap[ah.index];
        const uint32_t N = sys.sp_n[t.species], off = sys.sp_off[t.species];
        SumItems<1>(*this, (uint64_t)N * M, [=] __device__(uint64_t i, double* v) {
            const uint32_t g = off + (uint32_t)(i / M), b = (uint32_t)(i % M);
            double s = 0.;
            for (uint32_t d = 0; d < n_d; ++d) {
                const double x = PosAt(pos, np, b, d, g);
                s += x * x;
            }
            v[0] = s;
        }, &out);
        return t.cofactor_b * out;
    }
    // pair_action_class.h:241-264 with the constant-action cache.
    const PairDev pa = sys.pair[ah.index];
    if (pa.is_constant && !ah.is_first_time) return ah.dUdB_constant;
    const uint32_t na = sys.sp_n[pa.sa], nb = sys.sp_n[pa.sb], offa = sys.sp_off[pa.sa], offb = sys.sp_off[pa.sb];
    const bool hom = pa.sa == pa.sb;
    SumItems<1>(*this, (uint64_t)na * nb * M, [=] __device__(uint64_t i, double* v) {
        const uint32_t b = (uint32_t)(i % M);
        const uint64_t pq = i / M;
        const uint32_t x = (uint32_t)(pq / nb), y = (uint32_t)(pq % nb);
        v[0] = 0.;
        if (hom && y <= x) return;
        const uint32_t bn = (b + 1) % M;
        double A0[3], C0[3], A1[3], C1[3];
        LoadBead(pos, np, n_d, b, offb + y, A0);
        LoadBead(pos, np, n_d, b, offa + x, C0);
        LoadBead(pos, np, n_d, bn, offb + y, A1);
        LoadBead(pos, np, n_d, bn, offa + x, C1);
        double r, rp, s;
        DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, s);
        v[0] = PairdUdBeta(pa, r, rp, s);
    }, &out);
    if (pa.use_long_range) {
        // bare: CalcVLong (bare_pair_action_class.h:126-144); Ilkka and David: CalcdUdBetaLong
        // (ilkka_pair_action_class.h:152-169, david_pair_action_class.h:170-186)
        const bool ilkka = pa.kind != kPairBare;
        const uint32_t K = sys.K;
        const double2* ra = sys.rho_k + (size_t)sys.sp_rho[pa.sa] * M * K;
        const double2* rb = sys.rho_k + (size_t)sys.sp_rho[pa.sb] * M * K;
        const double* vk = ilkka ? pa.du_long_k : pa.v_long_k;
        double lr = 0.;
        SumItems<1>(*this, (uint64_t)K * M, [=] __device__(uint64_t i, double* v) {
            const uint32_t k = (uint32_t)(i / M), b = (uint32_t)(i % M);
            const double2 a = ra[(size_t)b * K + k], c = rb[(size_t)b * K + k];
            v[0] = (a.x * c.x + a.y * c.y) * vk[k];
        }, &lr);
        if (!hom) lr *= 2.;
        out += ilkka ? lr + pa.du_long_k_0 + pa.du_long_r_0 : lr + pa.v_long_k_0 + pa.v_long_r_0;
    }
    if (ah.is_first_time) {
        ah.is_first_time = false;
        ah.dUdB_constant = out;
    }
    return out;
}

double Context::Potential(uint32_t ai) {
    EnsureFP64();
    if (ai >= actions.size()) throw PimcError(kErrArg, "action index out of range");
    ActionHost& ah = actions[ai];
    if (ah.kind != 2) return 0.;  // Kinetic and Trap keep Action::Potential() = 0 (action_class.h:52)
    const PairDev pa = sys.pair[ah.index];
    if (pa.is_constant && !ah.is_first_time) return ah.potential_constant;
    const double* pos = sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL;
    const uint32_t na = sys.sp_n[pa.sa], nb = sys.sp_n[pa.sb], offa = sys.sp_off[pa.sa], offb = sys.sp_off[pa.sb];
    const bool hom = pa.sa == pa.sb;
    double out = 0.;
    SumItems<1>(*this, (uint64_t)na * nb * M, [=] __device__(uint64_t i, double* v) {
        const uint32_t b = (uint32_t)(i % M);
        const uint64_t pq = i / M;
        const uint32_t x = (uint32_t)(pq / nb), y = (uint32_t)(pq % nb);
        v[0] = 0.;
        if (hom && y <= x) return;
        const uint32_t bn = (b + 1) % M;
        double a[3], c[3];
        LoadBead(pos, np, n_d, b, offa + x, a);
        LoadBead(pos, np, n_d, b, offb + y, c);
        const double r = DistMinImage(a, c, n_d, L, iL);
        LoadBead(pos, np, n_d, bn, offa + x, a);
        LoadBead(pos, np, n_d, bn, offb + y, c);
        const double rp = DistMinImage(a, c, n_d, L, iL);
        v[0] = PairV(pa, r, rp);
    }, &out);
    if (pa.use_long_range) {
        const uint32_t K = sys.K;
        const double2* ra = sys.rho_k + (size_t)sys.sp_rho[pa.sa] * M * K;
        const double2* rb = sys.rho_k + (size_t)sys.sp_rho[pa.sb] * M * K;
        const double* vk = pa.v_long_k;
        double lr = 0.;
        SumItems<1>(*this, (uint64_t)K * M, [=] __device__(uint64_t i, double* v) {
            const uint32_t k = (uint32_t)(i / M), b = (uint32_t)(i % M);
            const double2 a = ra[(size_t)b * K + k], c = rb[(size_t)b * K + k];
            v[0] = (a.x * c.x + a.y * c.y) * vk[k];
        }, &lr);
        if (!hom) lr *= 2.;
        out += lr + pa.v_long_k_0 + pa.v_long_r_0;
    }
    if (ah.is_first_time) {
        ah.is_first_time = false;
        ah.potential_constant = out;
    }
    return out;
}

double Context::VirialEnergy(uint32_t ai, double window) {
    EnsureFP64();
    if (ai >= actions.size()) throw PimcError(kErrArg, "action index out of range");
    const ActionHost& ah = actions[ai];
    if (ah.kind != 0) return DActionDBeta(ai);  // action_class.h:40
    // kinetic_class.h:48-102 with each window sum formed directly.
    const KineticDev k = sys.kinetic[ah.index];
    const uint32_t N = sys.sp_n[k.species], off = sys.sp_off[k.species];
    const double* pos = sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL;
    const uint32_t W = window < 1. ? 1u : (uint32_t)std::ceil(window);
    if (W > M && !PermIdentity(k.species)) throw PimcError(kErrArg, "virial window longer than the path of an exchanging species");
    const uint32_t* perm = sys.perm;
    double out = 0.;
    SumItems<1>(*this, (uint64_t)N * M, [=] __device__(uint64_t i, double* v) {
        const uint32_t g = off + (uint32_t)(i / M), b = (uint32_t)(i % M);
        // beads b + w of the path through the ring closure (one crossing: b + W < 2M)
        auto lab = [&](uint32_t x) { return x >= M ? perm[g] : g; };
        double dr1[3] = {0., 0., 0.}, drl[3] = {0., 0., 0.};
        for (uint32_t d = 0; d < n_d; ++d) dr1[d] = MinImage(PosAt(pos, np, (b + 1) % M, d, lab(b + 1)) - PosAt(pos, np, b, d, g), L, iL);
        for (uint32_t w = 0; w < W; ++w) {
            const uint32_t x = b + w, y = b + w + 1;
            for (uint32_t d = 0; d < n_d; ++d) drl[d] += MinImage(PosAt(pos, np, y % M, d, lab(y)) - PosAt(pos, np, x % M, d, lab(x)), L, iL);
        }
        double dot = 0.;
        for (uint32_t d = 0; d < n_d; ++d) dot += drl[d] * dr1[d];
        v[0] = dot;
    }, &out);
    return k.d_action_d_beta_const / window - out * k.i4lt / (window * sys.tau);
}

double Context::VirialCentroid(uint32_t s) {
    EnsureFP64();
    // energy_class.h:81-94: sum over particles and slices of grad S(b, b+1, {p}) . (r_pb - r_p0)
    // for every non-kinetic action; only pair actions have gradients here.
    const double* pos = sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL, tau = sys.tau;
    double total = 0.;
    for (const auto& ah : actions) {
        if (ah.kind != 2 || ah.is_importance_weight) continue;
        const PairDev pa = sys.pair[ah.index];
        if (pa.is_constant) continue;
        if (pa.sa != s && pa.sb != s) continue;
        const uint32_t ns = sys.sp_n[s];
        // Partners: homologous q != p (pair (p, q)); s == sa: q in sb (pair (p, q));
        // s == sb: q in sa (pair (q, p), the gradient is taken on q).
        const bool hom = pa.sa == pa.sb;
        const bool s_is_a = pa.sa == s;
        const uint32_t other = hom ? s : (s_is_a ? pa.sb : pa.sa);
        const uint32_t nq = sys.sp_n[other];
        const uint32_t offs = sys.sp_off[s], offo = sys.sp_off[other];
        double part = 0.;
        SumItems<1>(*this, (uint64_t)ns * M * nq * 2, [=] __device__(uint64_t i, double* v) {
            const uint32_t link = (uint32_t)(i & 1u);
            uint64_t ii = i >> 1;
            const uint32_t q = (uint32_t)(ii % nq);
            ii /= nq;
            const uint32_t b = (uint32_t)(ii % M), pp = (uint32_t)(ii / M);
            v[0] = 0.;
            if (hom && q == pp) return;
            // first (species a) and second (species b) particle of the pair
            const uint32_t ga = (hom || s_is_a) ? offs + pp : offo + q;
            const uint32_t gb = (hom || s_is_a) ? offo + q : offs + pp;
            const uint32_t bo = link == 0 ? (b + 1) % M : (b + M - 1) % M;
            double A0[3], C0[3], A1[3], C1[3];
            LoadBead(pos, np, n_d, b, gb, A0);
            LoadBead(pos, np, n_d, b, ga, C0);
            LoadBead(pos, np, n_d, bo, gb, A1);
            LoadBead(pos, np, n_d, bo, ga, C1);
            double dot = 0.;
            if (pa.kind == kPairIlkka) {
                double gl[3];
                IlkkaGradientU(pa, A0, C0, A1, C1, n_d, L, iL, gl);
                for (uint32_t d = 0; d < n_d; ++d)
                    dot += gl[d] * MinImage(PosAt(pos, np, b, d, offs + pp) - PosAt(pos, np, 0, d, offs + pp), L, iL);
                v[0] = dot;
                return;
            }
            const double eps = 1.e-4;
            for (uint32_t d = 0; d < n_d; ++d) {
                const double c0 = C0[d];
                double r, rp, sd;
                C0[d] = c0 + eps;
                DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, sd);
                const double f1 = PairU(pa, r, rp, sd, 0, tau);
                C0[d] = c0 - eps;
                DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, sd);
                const double f2 = PairU(pa, r, rp, sd, 0, tau);
                C0[d] = c0;
                const double gd = (f1 - f2) / (2. * eps);
                const double dr = MinImage(PosAt(pos, np, b, d, offs + pp) - PosAt(pos, np, 0, d, offs + pp), L, iL);
                dot += gd * dr;
            }
            v[0] = dot;
        }, &part);
        total += part;
        if (pa.kind == kPairIlkka && pa.use_long_range && sys.K) {
            // CalcGradientULong(b, b + 1, first particle) once per pair (pair_action_class.h:331-334):
            // the listed particle itself for every partner when it is species a (or the action is
            // homologous), otherwise every species-a particle once.
            const uint32_t sa = pa.sa, na = sys.sp_n[sa], offa = sys.sp_off[sa];
            std::vector<uint32_t> firsts(na);
            for (uint32_t q = 0; q < na; ++q) firsts[q] = offa + q;
            double2* scratch = RhoTmp(((size_t)na * M * 3 + 1) / 2 + 1);
            double* G = reinterpret_cast<double*>(scratch);
            uint32_t* dg = Parts(na);
            CudaCheck(cudaMemcpyAsync(dg, firsts.data(), na * 4, cudaMemcpyHostToDevice, stream), "parts upload");
            IlkkaLongGradKernel<<<na * M, 256, 0, stream>>>(sys, pos, pa.u_long_k, dg, M, 0, 1,
                                                           sys.rho_k + (size_t)sys.sp_rho[pa.sb] * M * sys.K, 0, hom ? 1. : 2., G);
            CudaCheck(cudaGetLastError(), "long-range gradient launch");
            const bool first_is_s = hom || s_is_a;
            const double mult = hom ? (double)(ns - 1) : (double)sys.sp_n[pa.sb];
            double lrp = 0.;
            SumItems<1>(*this, (uint64_t)ns * M, [=] __device__(uint64_t i, double* v) {
                const uint32_t pp = (uint32_t)(i / M), b = (uint32_t)(i % M);
                double gsum[3] = {0., 0., 0.};
                if (first_is_s) {
                    for (uint32_t d = 0; d < 3; ++d) gsum[d] = mult * G[((size_t)pp * M + b) * 3 + d];
                } else {
                    for (uint32_t q = 0; q < na; ++q)
                        for (uint32_t d = 0; d < 3; ++d) gsum[d] += G[((size_t)q * M + b) * 3 + d];
                }
                double dot = 0.;
                for (uint32_t d = 0; d < n_d; ++d)
                    dot += gsum[d] * MinImage(PosAt(pos, np, b, d, offs + pp) - PosAt(pos, np, 0, d, offs + pp), L, iL);
                v[0] = dot;
            }, &lrp);
            total += lrp;
        }
    }
    return total;
}

void Context::ObservableAccumulate(uint32_t oi) {
    EnsureFP64();
    if (oi >= observables.size()) throw PimcError(kErrArg, "observable index out of range");
    ObservableHost& o = observables[oi];
    if (o.kind == 3 || o.kind == 4) return;  // Time, PathDump: nothing to accumulate
    // Path::GetSign times the importance weight (1: no importance-weight actions), energy_class.h:135-137
    const double cof = PathSign();
    if (o.kind == 5) {  // sign_class.h:12-16
        o.sign_sum += cof;
        o.n_measure++;
        return;
    }
    if (o.kind == 6) {  // permutation_class.h:15-22
        auto c = CycleLengths(o.species);
        for (uint32_t l : c) o.cycles[l - 1] += 1.;
        std::sort(c.begin(), c.end());
        uint32_t sector = (uint32_t)o.partitions.size();
        for (size_t i = 0; i < o.partitions.size(); ++i)
            if (o.partitions[i] == c) sector = (uint32_t)i;
        o.sectors.push_back(sector);
        o.n_measure++;
        return;
    }
    if (o.kind == 0) {
        // energy_class.h:133-161
        if (o.use_thermal) {
            for (size_t i = 0; i < actions.size(); ++i)
                if (!actions[i].is_importance_weight) o.energies[i] += cof * DActionDBeta((uint32_t)i);
        } else if (o.use_virial) {
            double ke = 0.;
            for (size_t i = 0; i < actions.size(); ++i)
                if (actions[i].kind == 0) ke += VirialEnergy((uint32_t)i, (double)o.virial_window);
            for (uint32_t s = 0; s < sys.S; ++s) {
                if (!(sys.sp_lambda[s] > 0.)) continue;
                ke += (o.use_adjoint ? VirialCentroidAdjoint(s) : VirialCentroid(s)) / (2. * sys.tau);
                for (size_t i = 0; i < actions.size(); ++i)
                    if (actions[i].kind == 0)
                        for (uint32_t x : actions[i].species_list)
                            if (x == s) o.energies[i] += cof * ke;
            }
            for (size_t i = 0; i < actions.size(); ++i)
                if (!actions[i].is_importance_weight && actions[i].kind != 0) o.energies[i] += cof * DActionDBeta((uint32_t)i);
        }
        if (o.measure_potential)
            for (size_t i = 0; i < actions.size(); ++i)
                if (!actions[i].is_importance_weight) o.potentials[i] += cof * Potential((uint32_t)i);
    } else if (o.kind == 1) {
        const int blocks = n_sm * 2;
        PairCorrelationKernel<<<blocks, 256, o.n_r * sizeof(unsigned int), stream>>>(sys, o.sa, o.sb, o.r_min, o.d_ir, o.n_r,
                                                                                    (long long)cof, o.hist->as<unsigned long long>());
        CudaCheck(cudaGetLastError(), "g(r) launch");
    } else if (o.kind == 2) {
        if (sys.K) {
            if (!kmag_dev_) {  // |k| of every stored k-vector, uploaded on first use
                kmag_dev_.reset(new DeviceBuffer(sys.K * sizeof(double)));
                CudaCheck(cudaMemcpy(kmag_dev_->ptr, kmags.data(), sys.K * sizeof(double), cudaMemcpyHostToDevice), "kmag upload");
            }
            const double* dk = kmag_dev_->as<double>();
            StructureFactorKernel<<<(sys.K + 255) / 256, 256, 0, stream>>>(sys, dk, o.k_cut, (uint32_t)sys.sp_rho[o.sa], (uint32_t)sys.sp_rho[o.sb],
                                                                           cof, o.sk->as<double>());
            CudaCheck(cudaGetLastError(), "S(k) launch");
        }
    }
    o.n_measure++;
}

std::vector<double> Context::ObservableBlock(uint32_t oi) {
    if (oi >= observables.size()) throw PimcError(kErrArg, "observable index out of range");
    ObservableHost& o = observables[oi];
    std::vector<double> out;
    if (o.kind == 3 || o.kind == 4 || o.n_measure == 0) return out;
    Sync();
    if (o.kind == 5) {  // sign_class.h:34-50
        out.push_back(o.sign_sum / (double)o.n_measure);
        o.sign_sum = 0.;
        o.n_measure = 0;
        return out;
    }
    if (o.kind == 6) {
        // permutation_class.h:76-118: cycle histogram normalised by the number of cycles, then the
        // block's (sector, count) pairs in increasing sector order
        double n_cycles = 0.;
        for (double c : o.cycles) n_cycles += c;
        for (double c : o.cycles) out.push_back(c / n_cycles);
        std::vector<uint32_t> sct = o.sectors;
        std::sort(sct.begin(), sct.end());
        for (size_t i = 0; i < sct.size();) {
            size_t j = i;
            while (j < sct.size() && sct[j] == sct[i]) ++j;
            out.push_back((double)sct[i]);
            out.push_back((double)(j - i));
            i = j;
        }
        std::fill(o.cycles.begin(), o.cycles.end(), 0.);
        o.sectors.clear();
        o.n_measure = 0;
        return out;
    }
    if (o.kind == 0) {
        // energy_class.h:232-253
        const double norm = (double)sys.M * o.n_measure;
        double E = 0.;
        std::vector<double> e(o.energies.size());
        for (size_t i = 0; i < e.size(); ++i) {
            e[i] = o.energies[i] / norm;
            E += e[i];
        }
        out.push_back(E);
        out.insert(out.end(), e.begin(), e.end());
        if (o.measure_potential) {
            double V = 0.;
            std::vector<double> v(o.potentials.size());
            for (size_t i = 0; i < v.size(); ++i) {
                v[i] = o.potentials[i] / norm;
                V += v[i];
            }
            out.push_back(V);
            out.insert(out.end(), v.begin(), v.end());
        }
        std::fill(o.energies.begin(), o.energies.end(), 0.);
        std::fill(o.potentials.begin(), o.potentials.end(), 0.);
    } else if (o.kind == 1) {
        // pair_correlation_class.h:89-123
        std::vector<unsigned long long> h(o.n_r);
        CudaCheck(cudaMemcpy(h.data(), o.hist->ptr, o.n_r * sizeof(unsigned long long), cudaMemcpyDeviceToHost), "read g(r)");
        CudaCheck(cudaMemset(o.hist->ptr, 0, o.n_r * sizeof(unsigned long long)), "reset g(r)");
        const double na = sys.sp_n[o.sa], nb = sys.sp_n[o.sb];
        const double norm = o.sa == o.sb ? 0.5 * o.n_measure * na * (nb - 1) * sys.M / sys.vol : (double)o.n_measure * na * nb * sys.M / sys.vol;
        out.resize(o.n_r);
        for (uint32_t i = 0; i < o.n_r; ++i) {
            const double r1 = o.r_min + i * o.dr;
            const double r2 = (i < o.n_r - 1) ? o.r_min + (i + 1) * o.dr : (2. * r1 - (o.r_min + (i - 1) * o.dr));
            double bin_vol;
            if (sys.n_d == 3) bin_vol = 4. * M_PI / 3. * (r2 * r2 * r2 - r1 * r1 * r1);
            else if (sys.n_d == 2) bin_vol = M_PI * (r2 * r2 - r1 * r1);
            else bin_vol = r2 - r1;
            out[i] = (double)(long long)h[i] / (bin_vol * norm);
        }
    } else if (o.kind == 2) {
        std::vector<double> sk(sys.K);
        if (sys.K) {
            CudaCheck(cudaMemcpy(sk.data(), o.sk->ptr, sys.K * sizeof(double), cudaMemcpyDeviceToHost), "read S(k)");
            CudaCheck(cudaMemset(o.sk->ptr, 0, sys.K * sizeof(double)), "reset S(k)");
        }
        const double norm = (double)o.n_measure * sys.M * sys.sp_n[o.sa] * sys.sp_n[o.sb];
        out.resize(sys.K);
        for (uint32_t k = 0; k < sys.K; ++k) out[k] = sk[k] / norm;
    }
    o.n_measure = 0;
    return out;
}

}  // namespace pimc
