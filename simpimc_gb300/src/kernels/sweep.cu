// The bisection hot path: a persistent cooperative kernel that runs a schedule of Bisect::Attempt
// calls (src/events/moves/single_species_move/bisect/bisect_class.h:39-124) for one chain, with
// the accept/reject commits of bisect_class.h:24-36,127-139, without returning to the host.
//
// Work split of one attempt across the grid (G blocks, all co-resident):
//  * Sampling, the kinetic action and the trap action touch at most 2^n_level beads of one
//    particle. Every block computes them redundantly from the same Philox stream, so every block
//    holds the identical proposal in shared memory and no communication is needed for them.
//  * The pair links of the moved particle (partners x slices) are spread over all threads of the
//    grid; the Ewald k-sum over the segment is split by ownership: block c owns the slices with
//    b mod R == c mod R and the k-vectors of chunk c / R. A block only ever reads and writes the
//    charge densities it owns, so commits need no synchronisation.
//  * Block partial sums are double-buffered in global memory; one bounded grid barrier per level
//    that has grid-wide work; every block then reduces the partials in the same order and takes
//    the same Metropolis decision.
//  * Accepted positions are written by every block (identical values), so each block's later
//    reads see either its own store or an identical one.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../common/philox.h"
#include "../framework/context.h"
#include "actions.cuh"

namespace pimc {

struct SweepArgs {
    SystemDev sys;
    MoveDev moves[kMaxMoves];
    uint64_t attempt_base[kMaxMoves];
    const uint32_t* sched_move;
    const uint64_t* sched_count;
    uint32_t n_entries;
    uint64_t n_rep;
    uint32_t seed, chain;
    uint32_t R, Q;              // ownership: residue classes of slices, chunks of k
    uint32_t seg_cap;           // capacity of the shared segment arrays (beads)
    int32_t tab_stride;         // phase-table row length
    unsigned long long* accepts;  // [2][kMaxMoves]: accepted attempts, attempts reaching level 0
    unsigned long long* bar;
    int* err;
    double* partials;             // [2][gridDim.x]
    uint64_t timeout_ns;
};

namespace {

__device__ __forceinline__ uint32_t Wrap(uint32_t b, uint32_t M) { return b >= M ? b - M : b; }

constexpr int kSweepThreads = 256;

__global__ void __launch_bounds__(kSweepThreads) BisectSweepKernel(const __grid_constant__ SweepArgs a) {
    extern __shared__ double smem[];
    const SystemDev& sys = a.sys;
    const uint32_t n_d = sys.n_d, M = sys.M, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL;
    double* seg_old = smem;                          // [seg_cap][3]
    double* seg_new = seg_old + 3 * a.seg_cap;       // [seg_cap][3]
    double* red = seg_new + 3 * a.seg_cap;           // [32]
    double2* tab = reinterpret_cast<double2*>(red + 32);  // [2][3][tab_stride]
    __shared__ double s_small, s_lsp_old, s_lsp_new, s_total, s_dS;
    __shared__ int s_reject;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t G = gridDim.x, cta = blockIdx.x;
    const uint32_t r_own = cta % a.R, q_own = cta / a.R;
    const bool owns_k = q_own < a.Q;
    const uint32_t k_lo = owns_k ? (uint32_t)(((uint64_t)sys.K * q_own) / a.Q) : 0u;
    const uint32_t k_hi = owns_k ? (uint32_t)(((uint64_t)sys.K * (q_own + 1)) / a.Q) : 0u;
    const int stride = a.tab_stride;

    uint64_t ctr[kMaxMoves];
    for (int m = 0; m < kMaxMoves; ++m) ctr[m] = a.attempt_base[m];
    unsigned long long my_accepts[kMaxMoves], my_reach0[kMaxMoves];
    for (int m = 0; m < kMaxMoves; ++m) my_accepts[m] = my_reach0[m] = 0ull;
    uint64_t nbar = 0;

    for (uint64_t rep = 0; rep < a.n_rep; ++rep) {
        for (uint32_t e = 0; e < a.n_entries; ++e) {
            const uint32_t m = a.sched_move[e];
            const uint64_t count = a.sched_count[e];
            const MoveDev& mv = a.moves[m];
            const uint32_t s = mv.species, B = 1u << mv.n_level;
            const uint32_t g_off = sys.sp_off[s];
            const int slot_s = sys.sp_rho[s];
            for (uint64_t c = 0; c < count; ++c) {
                const MoveStream st{a.seed, a.chain, m, ctr[m]};
                ctr[m] += 1;
                const Philox4 w0 = st.Block(0);
                const uint32_t p = UniformIndex(w0.v[0], sys.sp_n[s]);
                const uint32_t bead0 = UniformIndex(w0.v[1], M);
                const uint32_t g = g_off + p;

                // Segment bead0 .. bead0 + B (wrapping), old and new copies.
                for (uint32_t i = tid; i < (B + 1) * 3; i += blockDim.x) {
                    const uint32_t j = i / 3, d = i % 3;
                    const double v = d < n_d ? PosAt(sys.pos, np, (bead0 + j) % M, d, g) : 0.;
                    seg_old[i] = v;
                    seg_new[i] = v;
                }
                __syncthreads();

                double prev_dS = 0.;
                bool accepted = true;
                uint32_t mid = 0;
                for (int lvl = (int)mv.n_level - 1; lvl >= 0; --lvl) {
                    const uint32_t skip = 1u << lvl;
                    const uint32_t nm = B / (2 * skip);
                    // (1) Sampling, kinetic and trap terms: warp 0 of every block.
                    if (warp == 0) {
                        const double level_tau = sys.tau * skip;
                        const double sigma = sqrt(mv.lambda * level_tau);
                        const double i4s = mv.i4lt_sample[lvl];
                        double lo = 0., ln = 0.;
                        for (uint32_t mm = lane; mm < nm; mm += 32) {
                            const uint32_t ja = mm * 2 * skip, jb = ja + skip, jc = ja + 2 * skip;
                            double dold[3] = {0., 0., 0.}, dnew[3] = {0., 0., 0.};
                            double z[3];
                            BisectNormals(st, mid + mm, z);
                            for (uint32_t d = 0; d < n_d; ++d) {
                                const double ra = seg_old[3 * ja + d], rc = seg_old[3 * jc + d];
                                const double rbar = ra + 0.5 * MinImage(rc - ra, L, iL);
                                dold[d] = MinImage(seg_old[3 * jb + d] - rbar, L, iL);
                                const double na = seg_new[3 * ja + d], nc = seg_new[3 * jc + d];
                                const double nbar = na + 0.5 * MinImage(nc - na, L, iL);
                                dnew[d] = MinImage(0. + sigma * z[d], L, iL);
                                seg_new[3 * jb + d] = nbar + dnew[d];
                            }
                            lo += LogRhoFree(dold, n_d, i4s, &mv.sample_image[lvl], mv.has_images);
                            ln += LogRhoFree(dnew, n_d, i4s, &mv.sample_image[lvl], mv.has_images);
                        }
                        lo = WarpSum(lo);
                        ln = WarpSum(ln);
                        __syncwarp();
                        double small = 0.;
                        // Kinetic action at this level (kinetic_class.h:105-122): links j -> j + skip.
                        for (int ki = 0; ki < mv.n_kinetic; ++ki) {
                            const KineticDev& kd = sys.kinetic[mv.kinetic[ki]];
                            const double i4 = kd.i4lt_level[lvl];
                            for (uint32_t j = lane * skip; j < B; j += 32 * skip) {
                                double dro[3] = {0., 0., 0.}, drn[3] = {0., 0., 0.};
                                for (uint32_t d = 0; d < n_d; ++d) {
                                    dro[d] = MinImage(seg_old[3 * j + d] - seg_old[3 * (j + skip) + d], L, iL);
                                    drn[d] = MinImage(seg_new[3 * j + d] - seg_new[3 * (j + skip) + d], L, iL);
                                }
                                small += -LogRhoFree(drn, n_d, i4, &kd.image[lvl], kd.has_images) +
                                         LogRhoFree(dro, n_d, i4, &kd.image[lvl], kd.has_images);
                            }
                        }
                        // Harmonic trap (trap_class.h:37-61): slices [bead0, bead1) at stride skip.
                        for (int ti = 0; ti < mv.n_trap; ++ti) {
                            const TrapDev& td = sys.trap[mv.trap[ti]];
                            if ((uint32_t)lvl > td.max_level) continue;
                            double acc = 0.;
                            for (uint32_t j = lane * skip; j < B; j += 32 * skip)
                                for (uint32_t d = 0; d < n_d; ++d)
                                    acc += seg_new[3 * j + d] * seg_new[3 * j + d] - seg_old[3 * j + d] * seg_old[3 * j + d];
                            small += td.cofactor_a * skip * acc;
                        }
                        small = WarpSum(small);
                        if (lane == 0) {
                            s_small = small;
                            s_lsp_old = lo;
                            s_lsp_new = ln;
                        }
                    }
                    mid += nm;
                    __syncthreads();

                    // (2) Pair links and Ewald sums: the whole grid.
                    bool grid_work = false;
                    for (int pi = 0; pi < mv.n_pair; ++pi) {
                        const PairDev& pa = sys.pair[mv.pair[pi]];
                        if ((uint32_t)lvl <= pa.max_level && !pa.is_constant && (lvl == 0 || pa.use_long_range)) grid_work = true;
                    }
                    double big = 0.;
                    if (grid_work) {
                        double acc = 0.;
                        const uint64_t gtid = (uint64_t)cta * blockDim.x + tid, gstride = (uint64_t)G * blockDim.x;
                        // Pair links (pair_action_class.h:280-290); CalcU is zero above level 0.
                        if (lvl == 0) {
                            for (int pi = 0; pi < mv.n_pair; ++pi) {
                                const PairDev& pa = sys.pair[mv.pair[pi]];
                                if (pa.is_constant) continue;
                                const bool hom = pa.sa == pa.sb;
                                const uint32_t other = hom ? s : (pa.sa == s ? pa.sb : pa.sa);
                                const uint32_t n_partner = hom ? sys.sp_n[s] - 1 : sys.sp_n[other];
                                const uint64_t n_items = (uint64_t)n_partner * B;
                                const bool moved_is_a = hom || pa.sa == s;
                                for (uint64_t it = gtid; it < n_items; it += gstride) {
                                    const uint32_t jj = (uint32_t)(it % B);
                                    uint32_t qq = (uint32_t)(it / B);
                                    if (hom && qq >= p) ++qq;
                                    const uint32_t gq = sys.sp_off[other] + qq;
                                    const uint32_t bi = (bead0 + jj) % M, bj = (bead0 + jj + 1) % M;
                                    double Q0[3], Q1[3];
                                    LoadBead(sys.pos, np, n_d, bi, gq, Q0);
                                    LoadBead(sys.pos, np, n_d, bj, gq, Q1);
                                    double r, rp, sd, uo, un;
                                    if (moved_is_a) {
                                        DrDrpDrrp(Q0, &seg_old[3 * jj], Q1, &seg_old[3 * (jj + 1)], n_d, L, iL, r, rp, sd);
                                        uo = PairU(pa, r, rp, 0, sys.tau);
                                        DrDrpDrrp(Q0, &seg_new[3 * jj], Q1, &seg_new[3 * (jj + 1)], n_d, L, iL, r, rp, sd);
                                        un = PairU(pa, r, rp, 0, sys.tau);
                                    } else {
                                        DrDrpDrrp(&seg_old[3 * jj], Q0, &seg_old[3 * (jj + 1)], Q1, n_d, L, iL, r, rp, sd);
                                        uo = PairU(pa, r, rp, 0, sys.tau);
                                        DrDrpDrrp(&seg_new[3 * jj], Q0, &seg_new[3 * (jj + 1)], Q1, n_d, L, iL, r, rp, sd);
                                        un = PairU(pa, r, rp, 0, sys.tau);
                                    }
                                    acc += un - uo;
                                }
                            }
                        }
                        // Ewald sums over the owned slices and k-vectors (bare_pair_action_class.h:153-172).
                        bool any_lr = false;
                        for (int pi = 0; pi < mv.n_pair; ++pi) {
                            const PairDev& pa = sys.pair[mv.pair[pi]];
                            if (pa.use_long_range && (uint32_t)lvl <= pa.max_level && !pa.is_constant) any_lr = true;
                        }
                        if (any_lr && owns_k && slot_s >= 0) {
                            double lr = 0.;
                            for (uint32_t jj = skip; jj < B; jj += skip) {
                                const uint32_t b = (bead0 + jj) % M;
                                if (b % a.R != r_own) continue;
                                __syncthreads();
                                if (tid < 2 * (int)n_d) {
                                    const int which = tid / n_d, d = tid % n_d;
                                    const double x = which ? seg_new[3 * jj + d] : seg_old[3 * jj + d];
                                    PhaseRow(x, sys.box[d], sys.max_index[d], tab + ((size_t)which * 3 + d) * stride);
                                }
                                __syncthreads();
                                const double2* rs = sys.rho_k + ((size_t)slot_s * M + b) * sys.K;
                                for (uint32_t k = k_lo + tid; k < k_hi; k += blockDim.x) {
                                    const int32_t pk = sys.kidx[k];
                                    const double2 en = PhaseProduct(tab + 3 * stride, stride, n_d, pk);
                                    const double2 eo = PhaseProduct(tab, stride, n_d, pk);
                                    const double dx = en.x - eo.x, dy = en.y - eo.y;
                                    const double2 rho = rs[k];
                                    for (int pi = 0; pi < mv.n_pair; ++pi) {
                                        const PairDev& pa = sys.pair[mv.pair[pi]];
                                        if (!pa.use_long_range || (uint32_t)lvl > pa.max_level || pa.is_constant) continue;
                                        const double vk = pa.v_long_k[k];
                                        if (pa.sa == pa.sb) {
                                            lr += vk * (dx * (2. * rho.x + dx) + dy * (2. * rho.y + dy));
                                        } else {
                                            const uint32_t o = pa.sa == s ? pa.sb : pa.sa;
                                            const double2 ro = sys.rho_k[((size_t)sys.sp_rho[o] * M + b) * sys.K + k];
                                            lr += 2. * vk * (dx * ro.x + dy * ro.y);
                                        }
                                    }
                                }
                            }
                            acc += skip * sys.tau * lr;
                        }
                        // Grid reduction: block partial -> barrier -> identical ordered sum everywhere.
                        const double bsum = BlockSum(acc, red);
                        ++nbar;
                        if (tid == 0) __stcg(&a.partials[(nbar & 1ull) * G + cta], bsum);
                        if (!GridBarrier(a.bar, nbar, a.err, a.timeout_ns)) return;
                        if (warp == 0) {
                            double t = 0.;
                            for (uint32_t c2 = lane; c2 < G; c2 += 32) t += __ldcg(&a.partials[(nbar & 1ull) * G + c2]);
                            t = WarpSum(t);
                            if (lane == 0) s_total = t;
                        }
                        __syncthreads();
                        big = s_total;
                    }

                    // (3) Metropolis test (bisect_class.h:110-117), identical in every block.
                    if (lvl == 0) my_reach0[m] += 1;
                    if (tid == 0) {
                        const double dS = s_small + big;
                        const double log_sample_ratio = -s_lsp_new + s_lsp_old;
                        const double log_accept = log_sample_ratio - dS + prev_dS;
                        const double u = BisectAcceptUniform(st, B, mv.n_level - 1u - (uint32_t)lvl);
                        int rej = log_accept < log(u) ? 1 : 0;
                        if (!isfinite(log_accept)) {
                            atomicCAS(a.err, 0, kDevErrNonFinite);
                            rej = 2;
                        }
                        s_reject = rej;
                        s_dS = dS;
                    }
                    __syncthreads();
                    const int rej = s_reject;
                    const double dS_level = s_dS;
                    __syncthreads();
                    if (rej == 2) return;
                    if (rej) {
                        accepted = false;
                        break;
                    }
                    prev_dS = dS_level;
                }

                if (accepted) {
                    // bisect_class.h:24-36: commit the resampled beads (both copies).
                    for (uint32_t i = tid; i < (B - 1) * n_d; i += blockDim.x) {
                        const uint32_t j = 1 + i / n_d, d = i % n_d;
                        const size_t idx = ((size_t)((bead0 + j) % M) * 3 + d) * np + g;
                        sys.pos[idx] = seg_new[3 * j + d];
                        sys.pos_new[idx] = seg_new[3 * j + d];
                    }
                    // Per-slice charge densities (species_class.h:406-425 then StoreRhoK): only when a
                    // long-range action of this move updated them.
                    bool any_lr = false;
                    for (int pi = 0; pi < mv.n_pair; ++pi) {
                        const PairDev& pa = sys.pair[mv.pair[pi]];
                        if (pa.use_long_range && !pa.is_constant) any_lr = true;
                    }
                    if (any_lr && owns_k && slot_s >= 0) {
                        for (uint32_t jj = 1; jj < B; ++jj) {
                            const uint32_t b = (bead0 + jj) % M;
                            if (b % a.R != r_own) continue;
                            __syncthreads();
                            if (tid < 2 * (int)n_d) {
                                const int which = tid / n_d, d = tid % n_d;
                                const double x = which ? seg_new[3 * jj + d] : seg_old[3 * jj + d];
                                PhaseRow(x, sys.box[d], sys.max_index[d], tab + ((size_t)which * 3 + d) * stride);
                            }
                            __syncthreads();
                            double2* rs = sys.rho_k + ((size_t)slot_s * M + b) * sys.K;
                            for (uint32_t k = k_lo + tid; k < k_hi; k += blockDim.x) {
                                const int32_t pk = sys.kidx[k];
                                const double2 en = PhaseProduct(tab + 3 * stride, stride, n_d, pk);
                                const double2 eo = PhaseProduct(tab, stride, n_d, pk);
                                double2 v = rs[k];
                                v.x += en.x - eo.x;
                                v.y += en.y - eo.y;
                                rs[k] = v;
                            }
                        }
                    }
                    my_accepts[m] += 1;
                }
                __syncthreads();
            }
        }
    }
    if (cta == 0 && tid == 0)
        for (int m = 0; m < kMaxMoves; ++m)
            {
                a.accepts[m] += my_accepts[m];
                a.accepts[kMaxMoves + m] += my_reach0[m];
            }
}

}  // namespace

// ---------------------------------------------------------------------------------------------

void Context::Sweep(const uint32_t* mv, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep) {
    if (n_entries == 0 || n_rep == 0) return;
    for (uint32_t e = 0; e < n_entries; ++e)
        if (mv[e] >= moves.size()) throw PimcError(kErrArg, "move index out of range");
    static_assert(sizeof(SweepArgs) < 30000, "sweep arguments exceed the kernel parameter space");
    SweepArgs* args = new SweepArgs();
    std::unique_ptr<SweepArgs> guard(args);
    args->sys = sys;
    uint32_t max_level = 1;
    for (size_t m = 0; m < moves.size(); ++m) {
        args->moves[m] = moves[m].dev;
        args->attempt_base[m] = moves[m].attempts;
        max_level = std::max(max_level, moves[m].dev.n_level);
    }
    if (max_level > 10) throw PimcError(kErrUnsupported, "bisection level above 10 in the sweep kernel");
    // Schedule upload (entries then counts).
    std::vector<uint32_t> sm(mv, mv + n_entries);
    std::vector<uint64_t> sc(counts, counts + n_entries);
    if (!sched_) {
        sched_.reset(new DeviceBuffer(1024 * 12));
        accepts_.reset(new DeviceBuffer(2 * kMaxMoves * sizeof(unsigned long long)));
    }
    if (n_entries > 1024) throw PimcError(kErrArg, "schedule longer than 1024 entries");
    uint32_t* dsm = sched_->as<uint32_t>();
    uint64_t* dsc = reinterpret_cast<uint64_t*>(sched_->as<char>() + 4096);
    CudaCheck(cudaMemcpyAsync(dsm, sm.data(), n_entries * 4, cudaMemcpyHostToDevice, stream), "schedule upload");
    CudaCheck(cudaMemcpyAsync(dsc, sc.data(), n_entries * 8, cudaMemcpyHostToDevice, stream), "schedule upload");
    args->sched_move = dsm;
    args->sched_count = dsc;
    args->n_entries = n_entries;
    args->n_rep = n_rep;
    args->seed = seed;
    args->chain = chain;
    args->seg_cap = (1u << max_level) + 1;
    args->tab_stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const size_t smem = (size_t)2 * 3 * args->seg_cap * sizeof(double) + 32 * sizeof(double) + (size_t)2 * 3 * args->tab_stride * sizeof(double2);
    CudaCheck(cudaFuncSetAttribute(BisectSweepKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute");
    int occ = 0;
    CudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, BisectSweepKernel, kSweepThreads, smem), "occupancy");
    if (occ < 1) throw PimcError(kErrCuda, "sweep kernel cannot be resident");
    int G = sweep_grid > 0 ? std::min(sweep_grid, occ * n_sm) : std::min(occ, 2) * n_sm;
    // Ownership of slices: R residue classes (a power of two up to the segment length).
    uint32_t R = 1;
    while (R * 2 <= (1u << max_level) && R * 2 <= (uint32_t)G) R *= 2;
    args->R = R;
    args->Q = std::max<uint32_t>(1, (uint32_t)G / R);
    args->accepts = accepts_->as<unsigned long long>();
    args->bar = Barrier();
    args->err = ErrWord();
    args->partials = Partials((size_t)2 * G);
    args->timeout_ns = timeout_ns;
    CudaCheck(cudaMemsetAsync(accepts_->ptr, 0, 2 * kMaxMoves * sizeof(unsigned long long), stream), "reset accepts");
    CudaCheck(cudaMemsetAsync(Barrier(), 0, sizeof(unsigned long long), stream), "reset barrier");
    void* kargs[] = {args};
    CudaCheck(cudaLaunchCooperativeKernel((void*)BisectSweepKernel, dim3(G), dim3(kSweepThreads), kargs, smem, stream), "sweep launch");
    std::vector<unsigned long long> acc(2 * kMaxMoves);
    CudaCheck(cudaMemcpyAsync(acc.data(), accepts_->ptr, 2 * kMaxMoves * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "read accepts");
    Sync();
    CheckDeviceError();
    // Host bookkeeping of the attempt counters (they define the Philox streams).
    std::vector<uint64_t> per_move(moves.size(), 0);
    for (uint32_t e = 0; e < n_entries; ++e) per_move[mv[e]] += counts[e];
    for (size_t m = 0; m < moves.size(); ++m) {
        const uint64_t n = per_move[m] * n_rep;
        moves[m].attempts += n;
        moves[m].block_attempt += n;
        moves[m].block_accept += acc[m];
        moves[m].total_accept += acc[m];
        moves[m].total_level0 += acc[kMaxMoves + m];
    }
    last_grid_ = G;
}

void Context::MoveAttempts(uint32_t m, uint64_t n) {
    const uint64_t one = n;
    Sweep(&m, &one, 1, 1);
}

// Bisect::Reset (bisect_class.h:142-155) and Move::Write/Reset (move_class.h:296-310).
void Context::WriteBlock() {
    for (size_t i = 0; i < observables.size(); ++i) {
        auto v = ObservableBlock((uint32_t)i);
        if (!v.empty()) blocks[i].push_back(v);
    }
    for (auto& mh : moves) {
        mh.last_ratio = mh.block_attempt ? (double)mh.block_accept / (double)mh.block_attempt : 0.;
        if (!mh.first_block && mh.adaptive && mh.block_attempt > 0) {
            const double ratio = (double)mh.block_accept / (double)mh.block_attempt;
            if (ratio < mh.target_ratio && mh.dev.n_level > 1) mh.dev.n_level--;
            else if ((1u << mh.dev.n_level) < sys.M / 2) mh.dev.n_level++;
        }
        mh.first_block = false;
        mh.block_attempt = 0;
        mh.block_accept = 0;
    }
}

// Loop::DoEvent (loop_class.h:269-274). Consecutive move events are batched into one launch.
void Context::RunNode(const LoopNode& n) {
    // A loop body made only of moves runs as one sweep schedule repeated n_steps times.
    bool only_moves = !n.children.empty();
    for (auto& c : n.children) only_moves &= (c.kind == 1);
    if (only_moves) {
        std::vector<uint32_t> mv;
        std::vector<uint64_t> cnt;
        for (auto& c : n.children) {
            mv.push_back(c.index);
            cnt.push_back(1);
        }
        Sweep(mv.data(), cnt.data(), (uint32_t)mv.size(), n.n_steps);
        return;
    }
    for (uint64_t s = 0; s < n.n_steps; ++s) {
        size_t i = 0;
        while (i < n.children.size()) {
            const LoopNode& c = n.children[i];
            if (c.kind == 1) {
                std::vector<uint32_t> mv;
                std::vector<uint64_t> cnt;
                while (i < n.children.size() && n.children[i].kind == 1) {
                    mv.push_back(n.children[i].index);
                    cnt.push_back(1);
                    ++i;
                }
                Sweep(mv.data(), cnt.data(), (uint32_t)mv.size(), 1);
                continue;
            }
            if (c.kind == 0) RunNode(c);
            else if (c.kind == 2) ObservableAccumulate(c.index);
            else WriteBlock();
            ++i;
        }
    }
}

void Context::Run() { RunNode(main_loop); }

}  // namespace pimc
