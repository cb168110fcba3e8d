// Bisection moves of species whose paths exchange: PermBisectIterative, PermBisectTable and the
// plain Bisect on a species that carries a path permutation
// (src/events/moves/single_species_move/bisect/perm_bisect/perm_bisect_class.h:7-133,
// perm_bisect_iterative_class.h:7-231, perm_bisect_table_class.h:7-240, bisect_class.h:39-139).
//
// Representation. The reference links beads by pointers and relabels them after an accepted
// permutation (AssignParticleLabels, perm_bisect_class.h:47-56), so that between moves every link
// keeps its particle label except at the ring closure. Here that closure is an array: perm[g] is
// the particle whose slice-0 bead follows bead (g, M - 1), perm_inv its inverse. A segment of
// particle p that passes the closure continues on perm[p]. During an attempt the new link of the
// cycle (bead B - 1 of path i to the old end bead of path sigma(i)) is held in shared memory.
//
// Action changes. Kinetic links follow the paths (pointer semantics of kinetic_class.h:105-122).
// The trap and the Ewald part are sums over beads of the label-indexed particle list
// (trap_class.h:37-61, bare_pair_action_class.h:126-144); every moved bead lies on a listed label
// (the particle owning the end bead joins the list when the segment passes the closure), so their
// changes are sums over the moved beads. The short-range pair actions are evaluated link by link
// over the list's labels as PairAction::GetAction does (pair_action_class.h:267-302; the bare
// action's level_tau is tau at level 0 and zero above, bare_pair_action_class.h:146-150), so the
// off-diagonal IlkkaPairAction and DavidPairAction links keep the reference's label pairing across
// the permuted link.
//
// One CTA of kPermThreads runs the attempts of one move in order: the N x N table of free-particle
// weights and the cycle weights in parallel, the cycle selection (iterative walk, or running sum
// and bisection search of the table) on one thread in the reference's order, then per level the
// midpoints, kinetic links, trap beads, pair partners and the moved beads' density changes in
// parallel, with block sums in a fixed order. Random numbers follow the block layout of the
// oracle's PermBisect (seed, chain, move, attempt) streams. No wait spins; every loop is bounded.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../common/philox.h"
#include "../framework/context.h"
#include "actions.cuh"

namespace pimc {

namespace {

constexpr int kPermThreads = 256;
constexpr int kVariantBisect = 0, kVariantIterative = 1, kVariantTable = 2;
constexpr uint32_t kPermMaxPart = 2048;
constexpr uint32_t kCycleCache = 8192;  // table cycle weights kept in shared memory up to this count
constexpr uint32_t kPermChunk = 2048;  // attempts per launch

struct PermArgs {
    SystemDev sys;
    MoveDev mv;
    int variant;
    uint32_t seed, chain, move_index;
    uint64_t attempt0;
    uint32_t n_attempts;
    double epsilon, log_epsilon;
    uint32_t k_part, n_comb, n_types;  // table: cycle c = type c / n_comb over subset c % n_comb
    const uint32_t* combs;             // [n_comb][k_part] particle subsets
    const uint32_t* types;             // [n_types][k_part] permutations of a subset
    double* t;                         // [N][N] free-particle weights
    double* tc;                        // [N][N] iterative: the walk's working copy
    double* cw;                        // [n_cycles] table: cycle weights
    double* ccon;                      // [n_cycles] table: running sums of the kept cycles
    uint32_t* cidx;                    // [n_cycles] table: indices of the kept cycles
    double2* drho;                     // [B][K] moved beads' density change per segment offset
    double* hold;                      // [N][M][3] relabelling buffer
    uint32_t* perm;                    // [n_total]
    uint32_t* perm_inv;                // [n_total]
    unsigned long long* counters;      // accepts, level-0 tests, per cycle length attempts [N], accepts [N]
    int* err;
};

struct PermShared {
    uint32_t n, bead0, p_first, fail;
    double weight, tot0, tot1;
    Philox4 w0;
    double red[3 * (kPermThreads / 32)];
    double qpc, x;
    uint32_t p, cont;
    int decide;
};

// Three block-wide sums at once: warp trees, then every thread adds the warp partials in warp
// order, so all threads hold the same values.
__device__ __forceinline__ void BlockSum3(double& a0, double& a1, double& a2, double* red) {
    a0 = WarpSum(a0);
    a1 = WarpSum(a1);
    a2 = WarpSum(a2);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        red[warp] = a0;
        red[nw + warp] = a1;
        red[2 * nw + warp] = a2;
    }
    __syncthreads();
    double t0 = 0., t1 = 0., t2 = 0.;
    for (int w = 0; w < nw; ++w) {
        t0 += red[w];
        t1 += red[nw + w];
        t2 += red[2 * nw + w];
    }
    a0 = t0;
    a1 = t1;
    a2 = t2;
    __syncthreads();
}

__device__ __forceinline__ void LoadR(const double* __restrict__ pos, uint32_t np, uint32_t n_d, uint32_t b, uint32_t g, double* r) {
#pragma unroll
    for (uint32_t d = 0; d < 3; ++d) r[d] = d < n_d ? pos[((size_t)b * 3 + d) * np + g] : 0.;
}

__device__ __forceinline__ void StoreR(double* __restrict__ pos, uint32_t np, uint32_t n_d, uint32_t b, uint32_t g, const double* r) {
    for (uint32_t d = 0; d < n_d; ++d) pos[((size_t)b * 3 + d) * np + g] = r[d];
}

// The free-particle weight table of the current end map (UpdatePermTable): t[i][j] from the start
// bead of i at bead0 to the end bead of j, the end of a cycle member m being endmap[m].
__device__ void BuildTable(const PermArgs& a, uint32_t bead0, uint32_t B, bool relative, const int* lo_idx, const uint32_t* endmap) {
    const SystemDev& s = a.sys;
    const uint32_t sp = a.mv.species, N = s.sp_n[sp], G0 = s.sp_off[sp], M = s.M, nd = s.n_d, np = s.n_pad;
    const uint32_t tcross = M - bead0, es = (bead0 + B) % M;
    const double i4 = 1. / (4. * a.mv.lambda * s.tau * B);
    const bool copy = a.variant == kVariantIterative;
    auto end_of = [&](uint32_t j) -> uint32_t {
        const int m = lo_idx ? lo_idx[j] : -1;
        if (m >= 0) return endmap[m];
        return B >= tcross ? a.perm[G0 + j] : G0 + j;
    };
    for (uint32_t it = threadIdx.x; it < N * N; it += blockDim.x) {
        const uint32_t i = it / N, j = it % N;
        double ri[3], rj[3];
        LoadR(s.pos, np, nd, bead0, G0 + i, ri);
        LoadR(s.pos, np, nd, es, end_of(j), rj);
        double dij = 0.;
        for (uint32_t d = 0; d < nd; ++d) {
            const double x = MinImage(ri[d] - rj[d], s.L, s.iL);
            dij += x * x;
        }
        double ex;
        if (relative) {
            double rii[3], dii = 0.;
            LoadR(s.pos, np, nd, es, end_of(i), rii);
            for (uint32_t d = 0; d < nd; ++d) {
                const double x = MinImage(ri[d] - rii[d], s.L, s.iL);
                dii += x * x;
            }
            ex = (-dij + dii) * i4;
        } else {
            ex = (-dij) * i4;
        }
        const double v = ex > a.log_epsilon ? exp(ex) : 0.;
        a.t[it] = v;
        if (copy) a.tc[it] = v;
    }
}

// Cycle weights of the table (perm_bisect_table_class.h:15-26) into cw.
__device__ void CycleWeights(const PermArgs& a, uint32_t N, double* cw) {
    const uint32_t n_cycles = a.n_comb * a.n_types, k = a.k_part;
    for (uint32_t c = threadIdx.x; c < n_cycles; c += blockDim.x) {
        const uint32_t* part = a.combs + (size_t)(c % a.n_comb) * k;
        const uint32_t* pm = a.types + (size_t)(c / a.n_comb) * k;
        double w = 1.;
        for (uint32_t i = 0; i < k; ++i) w *= a.t[(size_t)part[i] * N + part[pm[i]]];
        cw[c] = w;
    }
}

__global__ void __launch_bounds__(kPermThreads, 1) PermBisectKernel(const __grid_constant__ PermArgs a) {
    extern __shared__ uint32_t dyn[];
    __shared__ PermShared sh;
    const SystemDev& s = a.sys;
    const MoveDev& mv = a.mv;
    const uint32_t sp = mv.species, N = s.sp_n[sp], G0 = s.sp_off[sp], M = s.M, nd = s.n_d, np = s.n_pad;
    const uint32_t B = 1u << mv.n_level, K = s.K;
    const int slot = s.sp_rho[sp];
    const int stride = max(max(s.max_index[0], s.max_index[1]), s.max_index[2]) + 1;
    // dynamic shared memory: lo_idx[N] (cycle member of a start particle), lpos[N] (place in the
    // particle list), part[N], sigma[N], lab_lo[N], lab_hi[N], end_old[N], end_new[N], lst[2N]
    // (the particle list), then the phase rows 2 x 3 x stride double2.
    int* lo_idx = reinterpret_cast<int*>(dyn);
    int* lpos = lo_idx + N;
    uint32_t* part = reinterpret_cast<uint32_t*>(lpos + N);
    uint32_t* sigma = part + N;
    uint32_t* lab_lo = sigma + N;
    uint32_t* lab_hi = lab_lo + N;
    uint32_t* end_old = lab_hi + N;
    uint32_t* end_new = end_old + N;
    uint32_t* lst = end_new + N;
    // rows of the weight table for the cycle walk [2N], the table's cycle weights [kCycleCache]
    double* row = reinterpret_cast<double*>(reinterpret_cast<uintptr_t>(lst + 2 * N + 1) & ~(uintptr_t)7);
    const uint32_t n_cycles = a.n_comb * a.n_types;
    const bool cw_shared = a.variant == kVariantTable && n_cycles <= kCycleCache;
    double* cws = row + 2 * N;
    double* cw = cw_shared ? cws : a.cw;
    double2* ph = reinterpret_cast<double2*>(reinterpret_cast<uintptr_t>(cws + (cw_shared ? n_cycles : 0) + 1) & ~(uintptr_t)15);
    __shared__ uint32_t s_nlist;
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) lo_idx[i] = lpos[i] = -1;
    const uint32_t base_m = a.variant == kVariantBisect ? 1u : 1u + N;
    const uint32_t base_u = a.variant == kVariantBisect ? 1u + (B - 1u) : base_m + N * (B - 1u);
    __syncthreads();

    for (uint32_t at = 0; at < a.n_attempts; ++at) {
        const MoveStream st{a.seed, a.chain, a.move_index, a.attempt0 + at};
        if (threadIdx.x == 0) {
            const Philox4 w0 = st.Block(0);
            sh.w0 = w0;
            sh.fail = 0;
            if (a.variant == kVariantBisect) {
                sh.p_first = UniformIndex(w0.v[0], N);
                sh.bead0 = UniformIndex(w0.v[1], M);
            } else {
                sh.bead0 = UniformIndex(w0.v[0], M);
                sh.p_first = UniformIndex(w0.v[1], N);
            }
        }
        __syncthreads();
        const uint32_t bead0 = sh.bead0, tcross = M - bead0, es = (bead0 + B) % M;

        // ---- cycle selection ----
        if (a.variant != kVariantBisect) {
            BuildTable(a, bead0, B, a.variant == kVariantTable, nullptr, nullptr);
            __syncthreads();
            if (a.variant == kVariantTable) {
                CycleWeights(a, N, cw);
                __syncthreads();
            }
            if (a.variant == kVariantIterative && threadIdx.x < 32) {
                // perm_bisect_iterative_class.h:32-110 on warp 0: the row of the table is staged in
                // shared memory and its quotients formed by the lanes; lane 0 adds in the
                // reference's order, so the sums and choices are those of the sequential walk.
                const uint32_t lane = threadIdx.x, p0 = sh.p_first;
                double* rt = row;
                double* rc = row + N;
                uint32_t p = p0, n = 0;
                bool ok = false;
                for (uint32_t step = 0; step < N; ++step) {
                    if (lane == 0) part[n] = p;
                    ++n;
                    __syncwarp();
                    for (uint32_t i = lane; i < n; i += 32) a.tc[(size_t)p * N + part[i]] = 0.;
                    __syncwarp();
                    if (lane == 0) a.tc[(size_t)p * N + p0] = a.t[(size_t)p * N + p0];
                    __syncwarp();
                    for (uint32_t i = lane; i < N; i += 32) {
                        rt[i] = a.t[(size_t)p * N + i];
                        rc[i] = a.tc[(size_t)p * N + i];
                    }
                    __syncwarp();
                    if (lane == 0) {
                        double Qp = 0., Qpc = 0.;
                        for (uint32_t i = 0; i < N; ++i) {
                            Qp += rt[i];
                            Qpc += rc[i];
                        }
                        const Philox4 w = st.Block(1u + step);
                        sh.cont = !(Qpc / Qp < Uniform53(w.v[0], w.v[1]));
                        sh.qpc = Qpc;
                        sh.x = Uniform53(w.v[2], w.v[3]);
                    }
                    __syncwarp();
                    if (!sh.cont) break;
                    const double qpc = sh.qpc;
                    for (uint32_t i = lane; i < N; i += 32) rt[i] = rc[i] / qpc;
                    __syncwarp();
                    if (lane == 0) {
                        const double x = sh.x;
                        double tQ = 0.;
                        for (uint32_t i = 0; i < N; ++i) {
                            tQ += rt[i];
                            if (tQ > x) {
                                p = i;
                                break;
                            }
                        }
                        sh.p = p;
                    }
                    __syncwarp();
                    p = sh.p;
                    if (p == p0) {
                        ok = true;
                        break;
                    }
                }
                if (lane == 0) {
                    if (!ok) {
                        sh.n = 0;
                        sh.fail = 1;
                    } else {
                        double w = 1.;
                        for (uint32_t i = 0; i + 1 < n; ++i) w *= a.t[(size_t)part[i] * N + part[i + 1]] / a.t[(size_t)part[i] * N + part[i]];
                        w *= a.t[(size_t)part[n - 1] * N + part[0]] / a.t[(size_t)part[n - 1] * N + part[n - 1]];
                        sh.weight = w;
                        sh.n = n;
                        for (uint32_t i = 0; i < n; ++i) sigma[i] = (i + 1) % n;
                    }
                }
            } else if (a.variant == kVariantTable && threadIdx.x == 0) {
                // perm_bisect_table_class.h:10-28, 105-119
                double total = 0.;
                uint32_t kept = 0;
                for (uint32_t c = 0; c < n_cycles; ++c) {
                    const double w = cw[c];
                    if (w > a.epsilon) {
                        total += w;
                        a.ccon[kept] = total;
                        a.cidx[kept] = c;
                        ++kept;
                    }
                }
                const double x = Uniform53(sh.w0.v[2], sh.w0.v[3]) * total;
                uint32_t kk = 0;
                if (!(x < a.ccon[0])) {
                    uint32_t hi = kept, lo = 0;
                    while (hi - lo > 1) {
                        const uint32_t mid = (hi + lo) >> 1;
                        if (x < a.ccon[mid]) hi = mid;
                        else lo = mid;
                    }
                    kk = min(hi, kept - 1);
                }
                const uint32_t c = a.cidx[kk];
                const uint32_t* cp = a.combs + (size_t)(c % a.n_comb) * a.k_part;
                const uint32_t* pm = a.types + (size_t)(c / a.n_comb) * a.k_part;
                for (uint32_t i = 0; i < a.k_part; ++i) {
                    part[i] = cp[i];
                    sigma[i] = pm[i];
                }
                sh.n = a.k_part;
                sh.weight = cw[c];
                sh.tot0 = total;
            }
        } else if (threadIdx.x == 0) {
            part[0] = sh.p_first;
            sigma[0] = 0;
            sh.n = 1;
            sh.weight = 1.;
        }
        __syncthreads();
        const uint32_t n = sh.n;
        if (n == 0) {  // no cycle selected: the attempt is rejected before any bisection
            __syncthreads();
            continue;
        }
        // ---- the paths of the cycle ----
        for (uint32_t m = threadIdx.x; m < n; m += blockDim.x) {
            const uint32_t g = G0 + part[m];
            lab_lo[m] = g;
            lab_hi[m] = a.perm[g];
            end_old[m] = B < tcross ? g : a.perm[g];
            lo_idx[part[m]] = (int)m;
        }
        __syncthreads();
        for (uint32_t m = threadIdx.x; m < n; m += blockDim.x) end_new[m] = end_old[sigma[m]];
        if (threadIdx.x == 0) {
            // the actions' particle list: the cycle, and the particles owning the end beads when the
            // segment reaches past the closure (perm_bisect_iterative_class.h:141-146, bisect_class.h:61-64)
            uint32_t nl = 0;
            for (uint32_t m = 0; m < n; ++m) {
                lpos[lab_lo[m] - G0] = (int)nl;
                lst[nl++] = lab_lo[m];
            }
            if (B >= tcross)
                for (uint32_t m = 0; m < n; ++m)
                    if (lpos[end_old[m] - G0] < 0) {
                        lpos[end_old[m] - G0] = (int)nl;
                        lst[nl++] = end_old[m];
                    }
            s_nlist = nl;
        }
        __syncthreads();
        const uint32_t nlist = s_nlist;
        auto label = [&](uint32_t m, uint32_t t) -> uint32_t { return t < tcross ? lab_lo[m] : lab_hi[m]; };
        auto slice = [&](uint32_t t) -> uint32_t { return (bead0 + t) % M; };

        bool accepted = true;
        double prev = -log(sh.weight);
        for (int level = (int)mv.n_level - 1; level >= 0; --level) {
            const uint32_t skip = 1u << level, nmid = B >> (level + 1), ngrid = B / skip - 1u;
            const uint32_t off = n * (nmid - 1u);
            const double sigma_l = sqrt(mv.lambda * s.tau * skip);
            double old_lsp = 0., new_lsp = 0., dS = 0.;
            // midpoints (bisect_class.h:74-94 with the OLD-mode end of the cycle path)
            for (uint32_t it = threadIdx.x; it < n * nmid; it += blockDim.x) {
                const uint32_t m = it / nmid, q = it % nmid;
                const uint32_t ta = 2u * skip * q, tb = ta + skip, tcc = ta + 2u * skip;
                double ra[3], rc[3], rb[3], rbar[3], dl[3];
                LoadR(s.pos, np, nd, slice(ta), label(m, ta), ra);
                if (tcc == B) LoadR(s.pos, np, nd, es, end_old[m], rc);
                else LoadR(s.pos, np, nd, slice(tcc), label(m, tcc), rc);
                LoadR(s.pos, np, nd, slice(tb), label(m, tb), rb);
                for (uint32_t d = 0; d < nd; ++d) rbar[d] = ra[d] + 0.5 * MinImage(rc[d] - ra[d], s.L, s.iL);
                for (uint32_t d = 0; d < nd; ++d) dl[d] = MinImage(rb[d] - rbar[d], s.L, s.iL);
                old_lsp += LogRhoFree(dl, nd, mv.i4lt_sample[level], &mv.sample_image[level], mv.has_images);
                float z[3];
                BisectNormals(st, base_m + off + m * nmid + q - 1u, z);
                for (uint32_t d = 0; d < nd; ++d) dl[d] = MinImage(0. + sigma_l * (double)z[d], s.L, s.iL);
                LoadR(s.pos_new, np, nd, slice(ta), label(m, ta), ra);
                if (tcc == B) LoadR(s.pos, np, nd, es, end_new[m], rc);
                else LoadR(s.pos_new, np, nd, slice(tcc), label(m, tcc), rc);
                for (uint32_t d = 0; d < nd; ++d) rbar[d] = ra[d] + 0.5 * MinImage(rc[d] - ra[d], s.L, s.iL);
                for (uint32_t d = 0; d < nd; ++d) rb[d] = rbar[d] + dl[d];
                StoreR(s.pos_new, np, nd, slice(tb), label(m, tb), rb);
                new_lsp += LogRhoFree(dl, nd, mv.i4lt_sample[level], &mv.sample_image[level], mv.has_images);
            }
            __syncthreads();
            // kinetic links along the paths (kinetic_class.h:105-122). A segment of the whole ring
            // (B = M) whose end bead is its start bead has no link in that mode: the walk to
            // GetNextBead(M) stops at once.
            for (int ki = 0; ki < mv.n_kinetic; ++ki) {
                const KineticDev& k = s.kinetic[mv.kinetic[ki]];
                const uint32_t nl = B / skip;
                for (uint32_t it = threadIdx.x; it < n * nl; it += blockDim.x) {
                    const uint32_t m = it / nl, j = it % nl, t0 = j * skip, t1 = t0 + skip;
                    const bool old_empty = B == M && end_old[m] == lab_lo[m], new_empty = B == M && end_new[m] == lab_lo[m];
                    double r0[3], r1[3], dr[3], so = 0., sn = 0.;
                    if (!old_empty) {
                        LoadR(s.pos, np, nd, slice(t0), label(m, t0), r0);
                        if (t1 == B) LoadR(s.pos, np, nd, es, end_old[m], r1);
                        else LoadR(s.pos, np, nd, slice(t1), label(m, t1), r1);
                        for (uint32_t d = 0; d < nd; ++d) dr[d] = MinImage(r0[d] - r1[d], s.L, s.iL);
                        so = -LogRhoFree(dr, nd, k.i4lt_level[level], &k.image[level], k.has_images);
                    }
                    if (!new_empty) {
                        LoadR(s.pos_new, np, nd, slice(t0), label(m, t0), r0);
                        if (t1 == B) LoadR(s.pos, np, nd, es, end_new[m], r1);
                        else LoadR(s.pos_new, np, nd, slice(t1), label(m, t1), r1);
                        for (uint32_t d = 0; d < nd; ++d) dr[d] = MinImage(r0[d] - r1[d], s.L, s.iL);
                        sn = -LogRhoFree(dr, nd, k.i4lt_level[level], &k.image[level], k.has_images);
                    }
                    dS += sn - so;
                }
            }
            // trap beads (trap_class.h:37-61)
            for (int ti = 0; ti < mv.n_trap; ++ti) {
                const TrapDev& tr = s.trap[mv.trap[ti]];
                if ((uint32_t)level > tr.max_level) continue;
                for (uint32_t it = threadIdx.x; it < n * ngrid; it += blockDim.x) {
                    const uint32_t m = it / ngrid, t = (it % ngrid + 1u) * skip;
                    double ro[3], rn[3], so = 0., sn = 0.;
                    LoadR(s.pos, np, nd, slice(t), label(m, t), ro);
                    LoadR(s.pos_new, np, nd, slice(t), label(m, t), rn);
                    for (uint32_t d = 0; d < nd; ++d) {
                        so += ro[d] * ro[d];
                        sn += rn[d] * rn[d];
                    }
                    dS += tr.cofactor_a * skip * (sn - so);
                }
            }
            // bare pair action over the particle list, link by link with the labels' beads
            // (PairAction::GetAction, pair_action_class.h:267-302; GenerateParticlePairs :62-114;
            // Path::DrDrpDrrp, path_class.h:137-150): zero above level 0 (level_tau), and under
            // periodic boundaries r' is the image nearest r, so the link is not a sum over its ends.
            for (int pi = 0; pi < mv.n_pair; ++pi) {
                const PairDev& pa = s.pair[mv.pair[pi]];
                if ((uint32_t)level > pa.max_level || pa.is_constant) continue;
                if (pa.kind == kPairBare && level != 0) continue;
                const bool hom = pa.sa == pa.sb;
                const uint32_t other = hom ? sp : (pa.sa == sp ? pa.sb : pa.sa);
                const uint32_t nq = s.sp_n[other], goff = s.sp_off[other], nlk = B / skip;
                for (uint32_t it = threadIdx.x; it < nlk * nlist * nq; it += blockDim.x) {
                    const uint32_t q = it % nq, rest = it / nq, li = rest % nlist, t = (rest / nlist) * skip;
                    const uint32_t gx = lst[li], gy = goff + q;
                    if (hom) {
                        if (gy == gx) continue;
                        const int ly = lpos[q];
                        if (ly >= 0 && (uint32_t)ly < li) continue;  // a pair within the list: once
                    }
                    const uint32_t b = slice(t), bn = slice(t + skip);
                    double A0[3], C0[3], A1[3], C1[3], r, rp, ss;
                    LoadR(s.pos, np, nd, b, gy, A0);
                    LoadR(s.pos, np, nd, b, gx, C0);
                    LoadR(s.pos, np, nd, bn, gy, A1);
                    LoadR(s.pos, np, nd, bn, gx, C1);
                    DrDrpDrrp(A0, C0, A1, C1, nd, s.L, s.iL, r, rp, ss);
                    const double uo = PairU(pa, r, rp, ss, (uint32_t)level, s.tau);
                    LoadR(s.pos_new, np, nd, b, gy, A0);
                    LoadR(s.pos_new, np, nd, b, gx, C0);
                    LoadR(s.pos_new, np, nd, bn, gy, A1);
                    LoadR(s.pos_new, np, nd, bn, gx, C1);
                    DrDrpDrrp(A0, C0, A1, C1, nd, s.L, s.iL, r, rp, ss);
                    dS += PairU(pa, r, rp, ss, (uint32_t)level, s.tau) - uo;
                }
            }
            // density change of the moved beads at this level's slices (species_class.h:406-425)
            const bool need_rho = slot >= 0 && K > 0;
            if (need_rho) {
                for (uint32_t j = 0; j < ngrid; ++j) {
                    const uint32_t t = (j + 1u) * skip;
                    for (uint32_t m = 0; m < n; ++m) {
                        __syncthreads();
                        if (threadIdx.x < 2u * nd) {
                            const uint32_t which = threadIdx.x / nd, d = threadIdx.x % nd;
                            const double x = (which ? s.pos_new : s.pos)[((size_t)slice(t) * 3 + d) * np + label(m, t)];
                            PhaseRow(x, s.box[d], s.max_index[d], ph + ((size_t)which * 3 + d) * stride);
                        }
                        __syncthreads();
                        for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
                            const int32_t pk = s.kidx[k];
                            const double2 eo = PhaseProduct(ph, stride, nd, pk), en = PhaseProduct(ph + 3 * stride, stride, nd, pk);
                            double2 v = m == 0 ? make_double2(0., 0.) : a.drho[(size_t)t * K + k];
                            v.x += en.x - eo.x;
                            v.y += en.y - eo.y;
                            a.drho[(size_t)t * K + k] = v;
                        }
                    }
                }
                __syncthreads();
                // Ewald part of every pair action touching the species: tau 2^level v_long_k for the
                // bare action (bare_pair_action_class.h:126-144), u_long_k for IlkkaPairAction and
                // DavidPairAction (ilkka_pair_action_class.h:104-122, david_pair_action_class.h:105-123)
                for (int pi = 0; pi < mv.n_pair; ++pi) {
                    const PairDev& pa = s.pair[mv.pair[pi]];
                    if ((uint32_t)level > pa.max_level || pa.is_constant || !pa.use_long_range) continue;
                    const bool hom = pa.sa == pa.sb;
                    const int oslot = hom ? slot : s.sp_rho[pa.sa == sp ? pa.sb : pa.sa];
                    double part_lr = 0.;
                    for (uint32_t it = threadIdx.x; it < ngrid * K; it += blockDim.x) {
                        const uint32_t k = it % K, t = (it / K + 1u) * skip;
                        const double2 ro = s.rho_k[((size_t)slot * M + slice(t)) * K + k];
                        const double2 dv = a.drho[(size_t)t * K + k];
                        const double2 rn = make_double2(ro.x + dv.x, ro.y + dv.y);
                        double dm;
                        if (hom) {
                            dm = (rn.x * rn.x + rn.y * rn.y) - (ro.x * ro.x + ro.y * ro.y);
                        } else {
                            const double2 rb = s.rho_k[((size_t)oslot * M + slice(t)) * K + k];
                            dm = (rn.x * rb.x + rn.y * rb.y) - (ro.x * rb.x + ro.y * rb.y);
                        }
                        part_lr += (pa.kind != kPairBare ? pa.u_long_k[k] : pa.v_long_k[k]) * dm;
                    }
                    dS += (hom ? 1. : 2.) * (pa.kind != kPairBare ? 1. : skip * s.tau) * part_lr;
                }
            }
            // decision (bisect_class.h:103-118)
            BlockSum3(old_lsp, new_lsp, dS, sh.red);
            const double t_old = old_lsp, t_new = new_lsp, t_ds = dS;
            if (threadIdx.x == 0) {
                const double la = -t_new + t_old - t_ds + prev;
                const float lu = LogF(U24(st.Block(base_u + (mv.n_level - 1u - (uint32_t)level)).v[0]));
                int ok = !(la < (double)lu);
                if (!isfinite(la)) {
                    atomicCAS(a.err, 0, kDevErrNonFinite);
                    ok = 0;
                }
                if (ok && level == 0) atomicAdd(&a.counters[1], 1ull);
                sh.decide = ok;
            }
            __syncthreads();
            prev = t_ds;
            if (!sh.decide) {
                accepted = false;
                break;
            }
        }
        // final test of the table (perm_bisect_table_class.h:216-225) with the new end map
        if (accepted && a.variant == kVariantTable && n < N) {
            BuildTable(a, bead0, B, true, lo_idx, end_new);
            __syncthreads();
            CycleWeights(a, N, cw);
            __syncthreads();
            if (threadIdx.x == 0) {
                double total = 0.;
                for (uint32_t c = 0; c < n_cycles; ++c)
                    if (cw[c] > a.epsilon) total += cw[c];
                const Philox4 w = st.Block(base_u + mv.n_level);
                sh.decide = !(sh.tot0 / total < Uniform53(w.v[0], w.v[1]));
            }
            __syncthreads();
            accepted = sh.decide != 0;
        }
        // ---- commit or restore the moved beads ----
        for (uint32_t it = threadIdx.x; it < n * (B - 1u) * nd; it += blockDim.x) {
            const uint32_t d = it % nd, rest = it / nd, m = rest / (B - 1u), t = rest % (B - 1u) + 1u;
            const size_t ix = ((size_t)slice(t) * 3 + d) * np + label(m, t);
            if (accepted) s.pos[ix] = s.pos_new[ix];
            else s.pos_new[ix] = s.pos[ix];
        }
        if (accepted && slot >= 0 && K > 0)
            for (uint32_t it = threadIdx.x; it < (B - 1u) * K; it += blockDim.x) {
                const uint32_t k = it % K, t = it / K + 1u;
                double2* r = &s.rho_k[((size_t)slot * M + slice(t)) * K + k];
                const double2 dv = a.drho[(size_t)t * K + k];
                r->x += dv.x;
                r->y += dv.y;
            }
        __syncthreads();
        // AssignParticleLabels (perm_bisect_class.h:47-56): beads after slice s0 of the paths'
        // labels there move to the label of the path that reaches them.
        bool moved_labels = false;
        for (uint32_t m = 0; m < n; ++m) moved_labels |= sigma[m] != m;
        if (accepted && moved_labels) {
            const uint32_t s0 = slice(B - 1u), ns = M - 1u - s0;
            for (uint32_t it = threadIdx.x; it < n * ns * nd; it += blockDim.x) {
                const uint32_t d = it % nd, rest = it / nd, m = rest / max(ns, 1u), b = s0 + 1u + rest % max(ns, 1u);
                a.hold[((size_t)m * M + b) * 3 + d] = s.pos[((size_t)b * 3 + d) * np + label(sigma[m], B - 1u)];
            }
            __syncthreads();
            for (uint32_t it = threadIdx.x; it < n * ns * nd; it += blockDim.x) {
                const uint32_t d = it % nd, rest = it / nd, m = rest / max(ns, 1u), b = s0 + 1u + rest % max(ns, 1u);
                const size_t ix = ((size_t)b * 3 + d) * np + label(m, B - 1u);
                s.pos[ix] = s.pos_new[ix] = a.hold[((size_t)m * M + b) * 3 + d];
            }
            if (threadIdx.x == 0) {
                // part[] is free now: the closure successors of the labels at s0, read before writing
                for (uint32_t m = 0; m < n; ++m) part[m] = a.perm[label(sigma[m], B - 1u)];
                for (uint32_t m = 0; m < n; ++m) {
                    a.perm[label(m, B - 1u)] = part[m];
                    a.perm_inv[part[m]] = label(m, B - 1u);
                }
            }
        }
        if (threadIdx.x == 0) {
            if (accepted) atomicAdd(&a.counters[0], 1ull);
            if (a.variant != kVariantBisect) {
                atomicAdd(&a.counters[2 + (n - 1)], 1ull);
                if (accepted) atomicAdd(&a.counters[2 + N + (n - 1)], 1ull);
            }
        }
        __syncthreads();
        for (uint32_t m = threadIdx.x; m < n; m += blockDim.x) lo_idx[lab_lo[m] - G0] = -1;
        for (uint32_t i = threadIdx.x; i < nlist; i += blockDim.x) lpos[lst[i] - G0] = -1;
        __syncthreads();
    }
}

}  // namespace

void Context::SyncPermHost() {
    if (perm_host.size() != sys.n_total) perm_host.resize(sys.n_total);
    CudaCheck(cudaMemcpyAsync(perm_host.data(), perm_->ptr, sys.n_total * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "read perm");
    Sync();
}

bool Context::PermIdentity(uint32_t s) const {
    for (uint32_t p = 0; p < sys.sp_n[s]; ++p)
        if (perm_host[sys.sp_off[s] + p] != sys.sp_off[s] + p) return false;
    return true;
}

bool Context::AnyPerm() const {
    for (uint32_t s = 0; s < sys.S; ++s)
        if (!PermIdentity(s)) return true;
    return false;
}

void Context::SetPerm(uint32_t s, const uint32_t* pi) {
    if (s >= sys.S) throw PimcError(kErrArg, "species index out of range");
    const uint32_t N = sys.sp_n[s], G0 = sys.sp_off[s];
    std::vector<char> seen(N, 0);
    for (uint32_t p = 0; p < N; ++p) {
        if (pi[p] >= N || seen[pi[p]]) throw PimcError(kErrArg, "not a permutation of the species' particles");
        seen[pi[p]] = 1;
    }
    for (uint32_t p = 0; p < N; ++p) perm_host[G0 + p] = G0 + pi[p];
    std::vector<uint32_t> inv(sys.n_total);
    for (uint32_t g = 0; g < sys.n_total; ++g) inv[perm_host[g]] = g;
    CudaCheck(cudaMemcpyAsync(perm_->ptr, perm_host.data(), sys.n_total * sizeof(uint32_t), cudaMemcpyHostToDevice, stream), "write perm");
    CudaCheck(cudaMemcpyAsync(perm_inv_->ptr, inv.data(), sys.n_total * sizeof(uint32_t), cudaMemcpyHostToDevice, stream), "write perm");
    Sync();
}

void Context::GetPerm(uint32_t s, uint32_t* out) const {
    if (s >= sys.S) throw PimcError(kErrArg, "species index out of range");
    for (uint32_t p = 0; p < sys.sp_n[s]; ++p) out[p] = perm_host[sys.sp_off[s] + p] - sys.sp_off[s];
}

double Context::PathSign() const {
    // Path::GetSign (path_class.h:169-175): (-1)^(length - 1) per cycle of every fermion species
    int sign = 1;
    for (uint32_t s = 0; s < sys.S; ++s) {
        if (!species_fermi[s]) continue;
        for (uint32_t len : CycleLengths(s))
            if (!(len % 2)) sign = -sign;
    }
    return (double)sign;
}

std::vector<uint32_t> Context::CycleLengths(uint32_t s) const {
    // Species::SetCycleCount (species_class.h:28-45)
    const uint32_t N = sys.sp_n[s], G0 = sys.sp_off[s];
    std::vector<char> seen(N, 0);
    std::vector<uint32_t> out;
    for (uint32_t p = 0; p < N; ++p) {
        if (seen[p]) continue;
        uint32_t len = 0, q = p;
        do {
            seen[q] = 1;
            q = perm_host[G0 + q] - G0;
            ++len;
        } while (q != p && len <= N);
        out.push_back(len);
    }
    return out;
}

bool Context::PermutingSpecies(uint32_t s) const {
    for (const auto& mh : moves)
        if ((mh.kind == 2 || mh.kind == 3) && mh.dev.species == s) return true;
    return !PermIdentity(s);
}

void Context::PermAttempts(uint32_t m, uint64_t n_att) {
    MoveHost& mh = moves[m];
    const uint32_t sp = mh.dev.species, N = sys.sp_n[sp], M = sys.M;
    if (N > kPermMaxPart) throw PimcError(kErrUnsupported, "permuting moves support at most 2048 particles per species");
    if (n_att == 0) return;
    EnsureFP64();
    const uint32_t B = 1u << mh.dev.n_level;
    // scratch
    const size_t n_cycles = (size_t)mh.perm_n_comb * mh.perm_n_types;
    auto ensure = [](std::unique_ptr<DeviceBuffer>& b, size_t bytes) {
        if (!b || b->bytes < bytes) b.reset(new DeviceBuffer(std::max<size_t>(bytes, 16)));
    };
    ensure(perm_t_, (size_t)N * N * sizeof(double) * 2);
    ensure(perm_cyc_, std::max<size_t>(n_cycles, 1) * (2 * sizeof(double) + sizeof(uint32_t)));
    ensure(perm_drho_, (size_t)M * std::max<uint32_t>(sys.K, 1) * sizeof(double2));
    ensure(perm_hold_, (size_t)N * M * 3 * sizeof(double));
    ensure(perm_cnt_, (2 + 2 * (size_t)N) * sizeof(unsigned long long));
    PermArgs a{};
    a.sys = sys;
    a.mv = mh.dev;
    a.variant = mh.kind == 2 ? kVariantIterative : (mh.kind == 3 ? kVariantTable : kVariantBisect);
    a.seed = seed;
    a.chain = chain;
    a.move_index = m;
    a.epsilon = mh.perm_epsilon;
    a.log_epsilon = std::log(mh.perm_epsilon);
    a.k_part = mh.perm_k;
    a.n_comb = mh.perm_n_comb;
    a.n_types = mh.perm_n_types;
    a.combs = mh.perm_combs ? mh.perm_combs->as<uint32_t>() : nullptr;
    a.types = mh.perm_types ? mh.perm_types->as<uint32_t>() : nullptr;
    a.t = perm_t_->as<double>();
    a.tc = a.t + (size_t)N * N;
    a.cw = perm_cyc_->as<double>();
    a.ccon = a.cw + std::max<size_t>(n_cycles, 1);
    a.cidx = reinterpret_cast<uint32_t*>(a.ccon + std::max<size_t>(n_cycles, 1));
    a.drho = perm_drho_->as<double2>();
    a.hold = perm_hold_->as<double>();
    a.perm = perm_->as<uint32_t>();
    a.perm_inv = perm_inv_->as<uint32_t>();
    a.counters = perm_cnt_->as<unsigned long long>();
    a.err = ErrWord();
    const int stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const size_t cyc_smem = (mh.kind == 3 && n_cycles <= kCycleCache) ? n_cycles * sizeof(double) : 0;
    const size_t smem = (size_t)N * 10 * sizeof(uint32_t) + 16 + (size_t)N * 2 * sizeof(double) + cyc_smem + 16 +
                        (size_t)2 * 3 * stride * sizeof(double2);
    CudaCheck(cudaFuncSetAttribute(PermBisectKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "perm smem attribute");
    CudaCheck(cudaMemsetAsync(perm_cnt_->ptr, 0, (2 + 2 * (size_t)N) * sizeof(unsigned long long), stream), "perm counters");
    (void)B;
    for (uint64_t done = 0; done < n_att;) {
        const uint32_t chunk = (uint32_t)std::min<uint64_t>(kPermChunk, n_att - done);
        a.attempt0 = mh.attempts + done;
        a.n_attempts = chunk;
        PermBisectKernel<<<1, kPermThreads, smem, stream>>>(a);
        CudaCheck(cudaGetLastError(), "permuting bisection launch");
        done += chunk;
    }
    std::vector<unsigned long long> cnt(2 + 2 * (size_t)N);
    CudaCheck(cudaMemcpyAsync(cnt.data(), perm_cnt_->ptr, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "read perm counters");
    Sync();
    CheckDeviceError();
    mh.attempts += n_att;
    mh.block_attempt += n_att;
    mh.block_accept += cnt[0];
    mh.total_accept += cnt[0];
    mh.total_level0 += cnt[1];
    if (mh.kind == 2 || mh.kind == 3) {
        for (uint32_t i = 0; i < N; ++i) {
            mh.perm_attempt[i] += cnt[2 + i];
            mh.perm_accept[i] += cnt[2 + N + i];
        }
    }
    dd_valid = false;
    fp64_valid = true;
    SyncPermHost();
}

}  // namespace pimc
