// The bisection hot path: a persistent cooperative kernel that runs a schedule of Bisect::Attempt
// calls (src/events/moves/single_species_move/bisect/bisect_class.h:39-124) for one chain, with
// the accept/reject commits of bisect_class.h:24-36,127-139, without returning to the host.
//
// Arithmetic: double-float (df64.cuh). GB300 issues FP64 at 1/64 of the FP32 rate, so the kernel
// keeps the path, the charge densities and every action term as float pairs (48-bit significand)
// and never touches the FP64 pipe on its critical path. Results agree with the FP64 oracle to
// ~1e-13 relative; the random numbers are exactly specified binary32 transforms (philox.h) that
// the oracle reproduces bit for bit.
//
// One attempt, all co-resident blocks in lock step:
//  1. Every block decodes the same particle/first bead, loads the segment and draws all normals
//     and acceptance logarithms of the attempt in parallel.
//  2. Warp 0 samples every level top-down (the chain of midpoints is inherently sequential);
//     meanwhile other warps build the phase tables of the old positions on this block's slices.
//  3. In parallel: one warp per level reduces that level's sampling log-probabilities, kinetic
//     and trap differences; other warps build the new-position phase tables.
//  4. All threads: pair links of the moved particle (spread over the grid) and the Ewald
//     differences of the owned (slice, k-chunk) cells; block partial -> one bounded grid barrier
//     -> every block sums the partials in the same order.
//  5. Thread 0 replays the reference's per-level Metropolis tests from the precomputed terms
//     (levels below a rejection are discarded), identically in every block.
//  6. On acceptance every block writes the resampled beads (identical values) and updates the
//     charge densities it owns.
// Levels above 0 are computed speculatively: the random numbers of an attempt are indexed per
// bead, so drawing them all up front changes nothing.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../common/philox.h"
#include "../framework/context.h"
#include "actions.cuh"
#include "df64.cuh"
#include "phase_dd.cuh"

namespace pimc {

struct CubicDD {
    const float2* x = nullptr;       // knots (hi, lo)
    const float4* c = nullptr;       // per interval two float4: (c0, c1), (c2, c3) as (hi, lo) pairs
    const int32_t* bucket = nullptr;
    int32_t n = 0, n_bucket = 0, uniform = 0, pad = 0;
    float x0f = 0.f, inv_dxf = 0.f;
    dd x0{0.f, 0.f}, x1{0.f, 0.f};
};

/// Double-float BicubicTable: knots as (hi, lo) pairs, per cell the 16 coefficients as 8 float4 of
/// (hi, lo) pairs in the order of BicubicTable::c.
struct BicubicDD {
    const float2* gx = nullptr;
    const float2* gy = nullptr;
    const int32_t* bx = nullptr;
    const int32_t* by = nullptr;
    const float4* c = nullptr;
    int32_t nx = 0, ny = 0, nbx = 0, nby = 0;
    float x0f = 0.f, inv_dxf = 0.f, y0f = 0.f, inv_dyf = 0.f;
    dd x0{0.f, 0.f}, x1{0.f, 0.f}, y0{0.f, 0.f}, y1{0.f, 0.f};
};

/// Double-float MultiCubic: knots (hi, lo); per interval and component two float4 of (hi, lo)
/// pairs, (c0, c1) and (c2, c3).
struct MultiCubicDD {
    const float2* x = nullptr;
    const int32_t* bucket = nullptr;
    const float4* c = nullptr;
    int32_t n = 0, n_bucket = 0, n_comp = 0, pad = 0;
    float x0f = 0.f, inv_dxf = 0.f;
    dd x0{0.f, 0.f}, x1{0.f, 0.f};
};

struct PairDD {
    uint32_t sa, sb;
    int32_t kind, is_coulomb, use_lr, is_constant, max_level;
    int32_t slot_a, slot_b;
    dd rvmin, rvmax, rvlmin, rvlmax;
    CubicDD v_r, v_long_r;
    const float2* vk;  // [K]: the long-range coefficient the sweep multiplies by tau
    // IlkkaPairAction
    BicubicDD u_xy;
    CubicDD u_long_r;
    dd rumin, rumax;
    // DavidPairAction
    MultiCubicDD u_kj;  // the table of level l from component l * kj_stride
    uint32_t n_order, kj_stride;
};

constexpr int kMoveKinetic = 2;

struct MoveDD {
    uint32_t species, n_level;
    int32_t has_images, n_kin, n_trap, n_pair;
    dd sigma[kMaxLevels], i4s[kMaxLevels];
    CubicDD sample_image[kMaxLevels];
    int32_t kin_has_images[kMoveKinetic];
    dd kin_i4[kMoveKinetic][kMaxLevels];
    CubicDD kin_image[kMoveKinetic][kMaxLevels];
    uint32_t trap_max_level[kMaxTrap];
    dd trap_cofa[kMaxTrap];
    int32_t pair[kMaxPair];
};

struct SweepArgs {
    uint32_t n_d, M, n_pad, K;
    dd L, iL, tau, two_pi;
    uint32_t sp_off[kMaxSpecies], sp_n[kMaxSpecies];
    int32_t max_index[3];
    float2* pos;              // [M][3][n_pad]
    float4* rho;              // [slots][M][K] double-float densities
    float2* rho32;            // [slots][M][K] FP32 densities (FP32 mode)
    const int32_t* kidx;      // [K]
    const float4* phase256;   // exp(2 pi i j / 256), j = 0..255
    const MoveDD* moves;
    const PairDD* pairs;
    uint64_t attempt_base[kMaxMoves];
    const uint32_t* sched_move;
    const uint64_t* sched_count;
    uint32_t n_entries;
    uint64_t n_rep;
    uint32_t seed, chain;
    uint32_t R, Q;            // ownership: slice residue classes, k chunks
    uint32_t seg_cap;         // segment capacity in beads (2^max_level + 1)
    uint32_t tab_stride;      // phase-table row length (max_index + 1)
    uint32_t slices_per_cta;  // owned slices per attempt (segment length / R)
    unsigned long long* counters;  // [2][kMaxMoves]: accepts, attempts reaching level 0
    unsigned long long* bar;
    int* err;
    float2* partials;         // [2][gridDim.x]
    float4* level_out;        // [2][kWaveSlots][kMaxLevels]: (diff, small) of each level from its designated block
    uint64_t timeout_ns;
    unsigned long long* phase_cycles;  // optional [kSweepPhases]: block 0's cycles per phase, summed
    // Concurrent attempts: `wave` groups of `group_ctas` blocks; the schedule flattened per
    // repetition (sched_prefix[e] = attempts before entry e, move_before[e] = attempts of its move
    // before it, per_rep_move[m] = attempts of move m per repetition).
    uint32_t wave, group_ctas;
    uint64_t per_rep;
    uint64_t per_rep_move[kMaxMoves];
    const uint64_t* sched_prefix;
    const uint64_t* move_before;
    // Shared-memory staging (byte offsets into the dynamic shared block).
    uint32_t n_moves, n_pairs;
    uint32_t off_moves, off_pairs, off_phase, off_work;
    uint32_t off_rho_stage, rho_cpt;  // density staging: cells per thread (0: read from global memory)
    uint32_t off_kstage, kstage_n;    // the block's k-chunk of kidx and v_k (0: read from global memory)
    uint32_t n_stage;
    const float2* stage_x[kMaxPair];
    const float4* stage_c[kMaxPair];
    uint32_t stage_n[kMaxPair], stage_off_x[kMaxPair], stage_off_c[kMaxPair];
};

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kDeltaCache = 8;
constexpr uint32_t kMaxOwned = 8;
constexpr uint32_t kWaveSlots = 8;  // most attempts in flight in one round

__device__ __forceinline__ bool CircOverlap(uint32_t s1, uint32_t l1, uint32_t s2, uint32_t l2, uint32_t M) {
    return (s2 + M - s1) % M < l1 || (s1 + M - s2) % M < l2;
}

/// Does attempt j (later in the schedule) read anything attempt i may change? Attempt i changes
/// the beads of its particle and the densities of its inner slices. Attempt j reads its own
/// particle's whole segment and, through its pair links (b, b + 1) for b in [bj, bj + Bj), every
/// particle on every slice of the closed segment: a link at an end slice takes the other
/// particle's bead there, and a pair density u(r, r') does not cancel it between the old and new
/// action. So j conflicts with i whenever i's inner slices meet j's closed segment.
__device__ __forceinline__ bool Conflicts(uint32_t bi, uint32_t Bi, uint32_t bj, uint32_t Bj, uint32_t M) {
    return CircOverlap((bi + 1) % M, Bi - 1, bj, Bj + 1, M);
}

__device__ __forceinline__ dd LoadDD(const float2* p) {
    const float2 v = *p;
    return dd{v.x, v.y};
}

__device__ __forceinline__ dd EvalCubicDD(const CubicDD& t, dd x) {
    x = Min(Max(x, t.x0), t.x1);
    int i;
    if (t.uniform) {
        i = (int)floorf(__fmul_rn(__fsub_rn(x.hi, t.x0f), t.inv_dxf));
        i = min(max(i, 0), t.n - 2);
    } else {
        int j = (int)floorf(__fmul_rn(__fsub_rn(x.hi, t.x0f), t.inv_dxf));
        j = min(max(j, 0), t.n_bucket - 1);
        i = t.bucket[j];
    }
    while (i < t.n - 2 && !Less(x, LoadDD(&t.x[i + 1]))) ++i;
    while (i > 0 && Less(x, LoadDD(&t.x[i]))) --i;
    const float4 a = t.c[2 * i], b = t.c[2 * i + 1];
    const dd u = Sub(x, LoadDD(&t.x[i]));
    const dd v = Add(dd{a.z, a.w}, Mul(u, Add(dd{b.x, b.y}, Mul(u, dd{b.z, b.w}))));
    return Add(dd{a.x, a.y}, Mul(u, v));
}

/// d/dx of EvalCubicDD: zero outside the grid, where EvalCubicDD holds the end value.
__device__ __forceinline__ dd EvalCubicDerivDD(const CubicDD& t, dd x) {
    if (Less(x, t.x0) || Less(t.x1, x)) return DD(0.f);
    int i;
    if (t.uniform) {
        i = (int)floorf(__fmul_rn(__fsub_rn(x.hi, t.x0f), t.inv_dxf));
        i = min(max(i, 0), t.n - 2);
    } else {
        int j = (int)floorf(__fmul_rn(__fsub_rn(x.hi, t.x0f), t.inv_dxf));
        j = min(max(j, 0), t.n_bucket - 1);
        i = t.bucket[j];
    }
    while (i < t.n - 2 && !Less(x, LoadDD(&t.x[i + 1]))) ++i;
    while (i > 0 && Less(x, LoadDD(&t.x[i]))) --i;
    const float4 a = t.c[2 * i], b = t.c[2 * i + 1];
    const dd u = Sub(x, LoadDD(&t.x[i]));
    // c1 + u (2 c2 + 3 u c3)
    return Add(dd{a.z, a.w}, Mul(u, Add(Scale2(dd{b.x, b.y}, 2.f), Mul(u, MulF(dd{b.z, b.w}, 3.f)))));
}

__device__ __forceinline__ dd SplitToDD(double x) {
    const float h = (float)x;
    return dd{h, (float)(x - (double)h)};
}

/// Short-range pair forces of the whole-ring action in double-float (BarePairAction::CalcV's
/// per-bead V(r) with the reference's two clamps, bare_pair_action_class.h:98-111): one thread per
/// (slice, particle of either species), tau V'(r) / r (r_g - r_q) summed over the partners in order.
__global__ void PairGradDDKernel(const SystemDev sys, const double* __restrict__ pos, const PairDD* __restrict__ pdd, uint32_t pair,
                                 double* __restrict__ grad) {
    const PairDD& pa = pdd[pair];
    const uint32_t na = sys.sp_n[pa.sa], nb = sys.sp_n[pa.sb], M = sys.M, np = sys.n_pad, n_d = sys.n_d;
    const bool hom = pa.sa == pa.sb;
    const uint32_t ng = hom ? na : na + nb;
    const dd L = SplitToDD(sys.L), iL = SplitToDD(sys.iL), tau = SplitToDD(sys.tau);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (uint64_t)ng * M; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(i / ng), j = (uint32_t)(i % ng);
        const bool in_a = j < na;
        const uint32_t g = in_a ? sys.sp_off[pa.sa] + j : sys.sp_off[pa.sb] + (j - na);
        const uint32_t q0 = in_a ? sys.sp_off[pa.sb] : sys.sp_off[pa.sa];
        const uint32_t nq = in_a ? nb : na;
        dd rg[3], G[3] = {DD(0.f), DD(0.f), DD(0.f)};
#pragma unroll
        for (uint32_t d = 0; d < 3; ++d) rg[d] = d < n_d ? SplitToDD(PosAt(pos, np, b, d, g)) : DD(0.f);
        for (uint32_t qi = 0; qi < nq; ++qi) {
            const uint32_t q = q0 + qi;
            if (q == g) continue;
            dd dr[3], r2 = DD(0.f);
#pragma unroll
            for (uint32_t d = 0; d < 3; ++d) {
                dr[d] = d < n_d ? MinImageDD(Sub(rg[d], SplitToDD(PosAt(pos, np, b, d, q))), L, iL) : DD(0.f);
                r2 = Add(r2, Sqr(dr[d]));
            }
            if (!(r2.hi > 0.f)) continue;  // coincident beads: no direction (the FP64 form skips r = 0)
            const dd r = Sqrt(r2);
            const bool in1 = !Less(r, pa.rvmin) && !Less(pa.rvmax, r);
            if (!in1) continue;  // V is clamped there: no force from either part
            dd dv = pa.is_coulomb ? Neg(Div(DD(1.f), r2)) : EvalCubicDerivDD(pa.v_r, r);
            if (pa.use_lr && !Less(r, pa.rvlmin) && !Less(pa.rvlmax, r)) dv = Sub(dv, EvalCubicDerivDD(pa.v_long_r, r));
            const dd f = Div(Mul(tau, dv), r);
#pragma unroll
            for (uint32_t d = 0; d < 3; ++d) G[d] = Add(G[d], Mul(f, dr[d]));
        }
#pragma unroll
        for (uint32_t d = 0; d < 3; ++d)
            if (d < n_d) grad[((size_t)b * 3 + d) * np + g] += ToDouble(G[d]);
    }
}

/// Cell of one 2-D table axis holding x (the last knot at or below x, within [0, n - 2]).
__device__ __forceinline__ int GridCellDD(const float2* g, const int32_t* bucket, int n, int nb, float x0f, float inv_dxf, dd x0, dd x1, dd x) {
    const dd xc = Min(Max(x, x0), x1);
    int j = (int)floorf(__fmul_rn(__fsub_rn(xc.hi, x0f), inv_dxf));
    j = min(max(j, 0), nb - 1);
    int i = bucket[j];
    while (i < n - 2 && !Less(xc, LoadDD(&g[i + 1]))) ++i;
    while (i > 0 && Less(xc, LoadDD(&g[i]))) --i;
    return i;
}

/// BicubicTable evaluation in double-float: the cell polynomial at the unclamped arguments.
__device__ __forceinline__ dd EvalBicubicDD(const BicubicDD& t, dd x, dd y) {
    const int i = GridCellDD(t.gx, t.bx, t.nx, t.nbx, t.x0f, t.inv_dxf, t.x0, t.x1, x);
    const int j = GridCellDD(t.gy, t.by, t.ny, t.nby, t.y0f, t.inv_dyf, t.y0, t.y1, y);
    const dd u = Sub(x, LoadDD(&t.gx[i])), v = Sub(y, LoadDD(&t.gy[j]));
    const float4* c = t.c + ((size_t)i * (t.ny - 1) + j) * 8;
    dd acc{0.f, 0.f};
#pragma unroll
    for (int a = 3; a >= 0; --a) {
        const float4 p = c[2 * a], q = c[2 * a + 1];  // (c_a0, c_a1), (c_a2, c_a3)
        const dd row = Add(dd{p.x, p.y}, Mul(v, Add(dd{p.z, p.w}, Mul(v, Add(dd{q.x, q.y}, Mul(v, dd{q.z, q.w}))))));
        acc = a == 3 ? row : Add(row, Mul(u, acc));
    }
    return acc;
}

/// Interval of a MultiCubicDD holding x clamped to the grid, and the offset from its knot.
__device__ __forceinline__ int MultiIntervalDD(const MultiCubicDD& t, dd x, dd& u) {
    x = Min(Max(x, t.x0), t.x1);
    const int i = GridCellDD(t.x, t.bucket, t.n, t.n_bucket, t.x0f, t.inv_dxf, t.x0, t.x1, x);
    u = Sub(x, LoadDD(&t.x[i]));
    return i;
}

__device__ __forceinline__ dd MultiCompDD(const MultiCubicDD& t, int i, dd u, int m) {
    const float4 a = t.c[2 * ((size_t)i * t.n_comp + m)], b = t.c[2 * ((size_t)i * t.n_comp + m) + 1];
    const dd v = Add(dd{a.z, a.w}, Mul(u, Add(dd{b.x, b.y}, Mul(u, dd{b.z, b.w}))));
    return Add(dd{a.x, a.y}, Mul(u, v));
}

/// DavidPairAction::CalcU's off-diagonal expansion at q (david_pair_action_class.h:80-99), with the
/// table whose components start at `base`.
__device__ __forceinline__ dd DavidOffDiagDD(const PairDD& pa, dd q, dd z, dd s, int base) {
    dd uq;
    const int iq = MultiIntervalDD(pa.u_kj, q, uq);
    const dd z2 = Sqr(z), s2 = Sqr(s), is2 = Div(DD(1.f), s2);
    dd s2k = s2, tot{0.f, 0.f};
    for (uint32_t k = 1; k <= pa.n_order; ++k) {
        dd z2j = DD(1.f), cs = s2k;
        for (uint32_t j = 0; j <= k; ++j) {
            tot = Add(tot, Mul(Mul(MultiCompDD(pa.u_kj, iq, uq, base + (int)(k * (k + 1) / 2 + j + 1)), z2j), cs));
            z2j = Mul(z2j, z2);
            cs = Mul(cs, is2);
        }
        s2k = Mul(s2k, s2);
    }
    return tot;
}

/// Sum over dimensions of the image-spline values.
__device__ __forceinline__ dd ImageSum(const CubicDD& t, const dd* dr, uint32_t n_d) {
    dd s{0.f, 0.f};
    for (uint32_t d = 0; d < n_d; ++d) s = Add(s, EvalCubicDD(t, dr[d]));
    return s;
}

/// BarePairAction::CalcV (bare_pair_action_class.h:99-123) in double-float.
__device__ __forceinline__ dd PairVDD(const PairDD& pa, dd r, dd rp) {
    r = Min(Max(r, pa.rvmin), pa.rvmax);
    rp = Min(Max(rp, pa.rvmin), pa.rvmax);
    dd v;
    if (pa.is_coulomb) {
        v = Add(Scale2(Div(DD(1.f), r), 0.5f), Scale2(Div(DD(1.f), rp), 0.5f));
    } else {
        v = Add(Scale2(EvalCubicDD(pa.v_r, r), 0.5f), Scale2(EvalCubicDD(pa.v_r, rp), 0.5f));
    }
    if (pa.use_lr) {
        r = Min(Max(r, pa.rvlmin), pa.rvlmax);
        rp = Min(Max(rp, pa.rvlmin), pa.rvlmax);
        v = Sub(v, Scale2(EvalCubicDD(pa.v_long_r, r), 0.5f));
        v = Sub(v, Scale2(EvalCubicDD(pa.v_long_r, rp), 0.5f));
    }
    return v;
}

/// Path::DrDrpDrrp (path_class.h:137-150) magnitudes |r|, |r'| in double-float.
__device__ __forceinline__ void DrDrpDD(const dd* A0, const dd* C0, const dd* A1, const dd* C1, uint32_t n_d, dd L, dd iL, dd& r,
                                        dd& rp) {
    dd a{0.f, 0.f}, b{0.f, 0.f};
    for (uint32_t d = 0; d < n_d; ++d) {
        const dd rv = MinImageDD(Sub(A0[d], C0[d]), L, iL);
        dd rq = Sub(A1[d], C1[d]);
        const float n = Rint(Mul(Sub(rv, rq), iL));
        if (n != 0.f) rq = Add(rq, MulF(L, n));
        a = Add(a, Sqr(rv));
        b = Add(b, Sqr(rq));
    }
    r = Sqrt(a);
    rp = Sqrt(b);
}

/// FP32 counterpart of PhaseDD: the turn count n x / L is reduced in double-float (so large n x
/// loses no bits), the residue of at most pi/256 is expanded to fifth order in FP32 and rotated by
/// the table entry's leading part.
__device__ __forceinline__ float2 PhaseF(dd x, int n, dd iL, const float4* tab256) {
    if (n == 0) return make_float2(1.f, 0.f);
    dd t = Mul(x, iL);
    t = Sub(t, DD(Rint(t)));
    dd a = MulF(t, (float)n);
    a = Sub(a, DD(Rint(a)));
    const float jf = rintf(__fmul_rn(a.hi, 256.f));
    const dd g = Sub(a, DD(__fmul_rn(jf, 1.f / 256.f)));
    const float eps = __fmul_rn(__fadd_rn(g.hi, g.lo), 6.28318531f);
    const float e2 = __fmul_rn(eps, eps);
    const float sn = __fmaf_rn(__fmul_rn(eps, e2), __fmaf_rn(e2, 1.f / 120.f, -1.f / 6.f), eps);
    const float cs = __fmaf_rn(e2, __fmaf_rn(e2, 1.f / 24.f, -0.5f), 1.f);
    const float4 T = tab256[((int)jf + 256) & 255];  // (re.hi, re.lo, im.hi, im.lo)
    return make_float2(__fsub_rn(__fmul_rn(T.x, cs), __fmul_rn(T.z, sn)), __fadd_rn(__fmul_rn(T.x, sn), __fmul_rn(T.z, cs)));
}

__device__ __forceinline__ float2 CMulF(float2 a, float2 b) {
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

__device__ __forceinline__ float2 PhaseProductF(const float2* tab, uint32_t stride, uint32_t n_d, int32_t packed) {
    float2 f = make_float2(1.f, 0.f);
    for (uint32_t d = 0; d < n_d; ++d) {
        const int n = KIdx(packed, (int)d);
        float2 c = tab[d * stride + (n < 0 ? -n : n)];
        if (n < 0) c.y = -c.y;
        f = d == 0 ? c : CMulF(f, c);
    }
    return f;
}

/// Generation index of the first midpoint of level lvl (levels are sampled from n_level - 1 down).
__device__ __forceinline__ uint32_t LevelFirst(uint32_t nl, int lvl, uint32_t B) {
    uint32_t first = 0;
    for (int l = (int)nl - 1; l > lvl; --l) first += B / (2u << l);
    return first;
}

/// Level sums of one copy of the segment (warp-cooperative; every lane receives the totals):
///   lsp   = sampling log-probability of the copy's midpoints, -i4s |d|^2 - images(d)
///           (free_spline_class.h:76-84 with tau' = tau 2^l / 2, bisect_class.h:85-94);
///   small = kinetic action of the links j -> j + skip (kinetic_class.h:105-122) plus the trap
///           action of slices j at stride skip (trap_class.h:37-61, when lvl <= max_level).
/// A segment spanning the whole ring (B == M) has no kinetic links: the reference walks from the
/// first bead to GetNextBead(B), which is the first bead itself (kinetic_class.h:111-117).
__device__ __forceinline__ void LevelSums(const MoveDD& mv, int lvl, uint32_t B, bool kin_links, const dd* seg, const dd* disp,
                                          uint32_t first, uint32_t n_d, dd L, dd iL, int lane, dd& lsp, dd& small) {
    // Every term is a sum over dimensions (|d|^2 and the image splines), so one lane takes one
    // (item, dimension) pair: the latency of a lane is one dimension's spline evaluation.
    const uint32_t skip = 1u << lvl, nm = B / (2 * skip), nj = (B + skip - 1) / skip;
    dd sp{0.f, 0.f}, sm{0.f, 0.f};
    for (uint32_t i = lane; i < nm * n_d; i += 32) {
        const uint32_t tt = i / n_d, d = i - tt * n_d;
        const dd x = disp[3 * (first + tt) + d];
        dd v = Mul(Sqr(x), mv.i4s[lvl]);
        if (mv.has_images) v = Add(v, EvalCubicDD(mv.sample_image[lvl], x));
        sp = Add(sp, v);
    }
    for (int ki = 0; ki < (kin_links ? mv.n_kin : 0); ++ki)
        for (uint32_t i = lane; i < nj * n_d; i += 32) {
            const uint32_t jt = i / n_d, d = i - jt * n_d, j = jt * skip;
            const dd dr = MinImageDD(Sub(seg[3 * j + d], seg[3 * (j + skip) + d]), L, iL);
            dd v = Mul(Sqr(dr), mv.kin_i4[ki][lvl]);
            if (mv.kin_has_images[ki]) v = Add(v, EvalCubicDD(mv.kin_image[ki][lvl], dr));
            sm = Add(sm, v);
        }
    for (int ti = 0; ti < mv.n_trap; ++ti) {
        if ((uint32_t)lvl > mv.trap_max_level[ti]) continue;
        dd acc{0.f, 0.f};
        for (uint32_t i = lane; i < nj * n_d; i += 32) {
            const uint32_t jt = i / n_d, d = i - jt * n_d;
            acc = Add(acc, Sqr(seg[3 * (jt * skip) + d]));
        }
        sm = Add(sm, MulF(Mul(acc, mv.trap_cofa[ti]), (float)skip));
    }
    WarpSum2DD(sp, sm);
    lsp = Neg(sp);
    small = sm;
}

__device__ __forceinline__ dd ShflXorDD(dd v, int m) {
    return dd{__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
}

/// One radius' share of BarePairAction::CalcV (bare_pair_action_class.h:99-123):
/// 1/(2r) (or v(r)/2 from the table) minus v_long(r)/2, with the reference's clamps.
__device__ __forceinline__ dd PairHalfV(const PairDD& pa, dd r) {
    r = Min(Max(r, pa.rvmin), pa.rvmax);
    dd v = pa.is_coulomb ? Scale2(Div(DD(1.f), r), 0.5f) : Scale2(EvalCubicDD(pa.v_r, r), 0.5f);
    if (pa.use_lr) v = Sub(v, Scale2(EvalCubicDD(pa.v_long_r, Min(Max(r, pa.rvlmin), pa.rvlmax)), 0.5f));
    return v;
}

/// U = tau V of pair link l (level 0) for one copy of the moved particle's segment, evaluated by a
/// quad of lanes: lanes 0-2 take one Cartesian component of Path::DrDrpDrrp (path_class.h:137-150)
/// each, lanes 0 and 1 then take r and r'. Every lane of the warp must call it; the result is
/// returned on lane 0 of the quad (zero elsewhere and for invalid links).
/// With `ext` (the move has an IlkkaPairAction; uniform over the warp) the quad also forms
/// s = |r - r'| (min image), and an Ilkka link is u(q + s/2, q - s/2) from lane 0 minus half the
/// long-range action of r (lane 1) and of r' (lane 2), ilkka_pair_action_class.h:77-101; it is not
/// scaled by tau.
__device__ __forceinline__ dd PairLinkU4(const PairDD* s_pairs, const MoveDD& mv, const uint32_t* link_off, uint32_t l, bool valid, int ql,
                                         uint32_t s, uint32_t p, uint32_t B, uint32_t bead0, uint32_t M, uint32_t np, uint32_t n_d,
                                         const uint32_t* sp_off, const float2* pos, const dd* seg, dd L, dd iL, dd tau, bool ext) {
    dd rv2{0.f, 0.f}, rq2{0.f, 0.f}, ss2{0.f, 0.f};
    int pi = 0;
    if (valid) {
        while (l >= link_off[pi + 1]) ++pi;
        const PairDD& pa = s_pairs[mv.pair[pi]];
        const bool hom = pa.sa == pa.sb;
        const uint32_t other = hom ? s : (pa.sa == s ? pa.sb : pa.sa);
        const uint32_t local = l - link_off[pi];
        const uint32_t jj = local % B;
        uint32_t qq = local / B;
        if (hom && qq >= p) ++qq;
        const uint32_t gq = sp_off[other] + qq;
        if ((uint32_t)ql < n_d) {
            const uint32_t d = ql;
            const dd q0 = LoadDD(&pos[((size_t)((bead0 + jj) % M) * 3 + d) * np + gq]);
            const dd q1 = LoadDD(&pos[((size_t)((bead0 + jj + 1) % M) * 3 + d) * np + gq]);
            const dd m0 = seg[3 * jj + d], m1 = seg[3 * (jj + 1) + d];
            // r = second - first particle; the moved particle is first unless it is species b.
            const bool moved_first = hom || pa.sa == s;
            const dd rv = MinImageDD(moved_first ? Sub(q0, m0) : Sub(m0, q0), L, iL);
            dd rq = moved_first ? Sub(q1, m1) : Sub(m1, q1);
            const float n = Rint(Mul(Sub(rv, rq), iL));
            if (n != 0.f) rq = Add(rq, MulF(L, n));
            rv2 = Sqr(rv);
            rq2 = Sqr(rq);
            if (ext) ss2 = Sqr(MinImageDD(Sub(rv, rq), L, iL));
        }
    }
    rv2 = Add(rv2, ShflXorDD(rv2, 1));
    rv2 = Add(rv2, ShflXorDD(rv2, 2));
    rq2 = Add(rq2, ShflXorDD(rq2, 1));
    rq2 = Add(rq2, ShflXorDD(rq2, 2));
    if (!ext) {
        dd f{0.f, 0.f};
        if (valid && ql < 2) f = PairHalfV(s_pairs[mv.pair[pi]], Sqrt(ql == 0 ? rv2 : rq2));
        f = Add(f, ShflXorDD(f, 1));
        return (valid && ql == 0) ? Mul(tau, f) : dd{0.f, 0.f};
    }
    ss2 = Add(ss2, ShflXorDD(ss2, 1));
    ss2 = Add(ss2, ShflXorDD(ss2, 2));
    dd f{0.f, 0.f};
    bool ilkka = false;
    if (valid) {
        const PairDD& pa = s_pairs[mv.pair[pi]];
        ilkka = pa.kind != kPairBare;  // tables hold the action itself: no tau factor
        if (pa.kind == kPairDavid) {
            // endpoint terms on lanes 0 and 1, the off-diagonal expansion on lane 2 (david_pair_action_class.h:69-102)
            const dd r = Sqrt(rv2), rp = Sqrt(rq2);
            if (ql < 2) {
                dd u;
                const int i = MultiIntervalDD(pa.u_kj, ql == 0 ? r : rp, u);
                f = Scale2(MultiCompDD(pa.u_kj, i, u, 1), 0.5f);
            } else if (ql == 2) {
                const dd sl = Sqrt(ss2), q = Scale2(Add(r, rp), 0.5f);
                if (sl.hi > 0.f && Less(q, pa.u_kj.x1)) f = DavidOffDiagDD(pa, q, Sub(r, rp), sl, 0);
            }
        } else if (!ilkka) {
            if (ql < 2) f = PairHalfV(pa, Sqrt(ql == 0 ? rv2 : rq2));
        } else if (ql == 0) {
            const dd r = Sqrt(rv2), rp = Sqrt(rq2), sl = Sqrt(ss2);
            const dd q = Scale2(Add(r, rp), 0.5f), hs = Scale2(sl, 0.5f);
            f = EvalBicubicDD(pa.u_xy, Add(q, hs), Sub(q, hs));
        } else if (ql < 3 && pa.use_lr) {
            const dd r = Min(Max(Sqrt(ql == 1 ? rv2 : rq2), pa.rumin), pa.rumax);
            f = Neg(Scale2(EvalCubicDD(pa.u_long_r, r), 0.5f));
        }
    }
    f = Add(f, ShflXorDD(f, 1));
    f = Add(f, ShflXorDD(f, 2));
    if (!(valid && ql == 0)) return dd{0.f, 0.f};
    return ilkka ? f : Mul(tau, f);
}

__device__ __forceinline__ void CopyWords(void* dst, const void* src, uint32_t bytes) {
    uint32_t* d = static_cast<uint32_t*>(dst);
    const uint32_t* s = static_cast<const uint32_t*>(src);
    for (uint32_t i = threadIdx.x; i < bytes / 4; i += blockDim.x) d[i] = s[i];
}

/// kF32: FP32 mode. Per-slice densities are FP32 (a.rho32), bead phases are FP32 (PhaseF), and
/// each thread's Ewald differences are summed with a cascaded compensated sum before they join the
/// double-float acceptance pipeline; positions, pair links and level sums stay double-float.
/// A thread's Ewald cells it = tid, tid + T, ... of an attempt's (owned slice, k-chunk) grid, as
/// (slice index, k offset) advanced without a division per cell.
struct CellIter {
    uint32_t si, kk, dq, dr, nk;
    __device__ __forceinline__ CellIter(uint32_t tid, uint32_t T, uint32_t nk_) : nk(nk_ ? nk_ : 1u) {
        si = tid / nk;
        kk = tid - si * nk;
        dq = T / nk;
        dr = T - dq * nk;
    }
    __device__ __forceinline__ void Next() {
        kk += dr;
        si += dq;
        if (kk >= nk) {
            kk -= nk;
            ++si;
        }
    }
};

/// Slice b0 + jj of an M-slice ring (b0 < M, jj < M).
__device__ __forceinline__ uint32_t RingSlice(uint32_t b0, uint32_t jj, uint32_t M) {
    const uint32_t b = b0 + jj;
    return b >= M ? b - M : b;
}

/// Asynchronous global -> shared copies (cp.async), completed by CpAsyncWaitAll of the issuing thread.
__device__ __forceinline__ void CpAsync8(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void CpAsync16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void CpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void CpAsyncWaitAll() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <bool kF32>
__global__ void __launch_bounds__(kThreads, 1) BisectSweepKernel(const __grid_constant__ SweepArgs a) {
    extern __shared__ float4 smem4[];
    const uint32_t n_d = a.n_d, M = a.M, np = a.n_pad, K = a.K;
    const uint32_t cap = a.seg_cap, stride = a.tab_stride;
    // Launch-invariant data staged in shared memory once: move and pair descriptors, the phase
    // table and (when they fit) the long-range spline tables.
    char* sbase = reinterpret_cast<char*>(smem4);
    MoveDD* s_moves = reinterpret_cast<MoveDD*>(sbase + a.off_moves);
    PairDD* s_pairs = reinterpret_cast<PairDD*>(sbase + a.off_pairs);
    float4* s_phase = reinterpret_cast<float4*>(sbase + a.off_phase);
    CopyWords(s_moves, a.moves, a.n_moves * (uint32_t)sizeof(MoveDD));
    CopyWords(s_pairs, a.pairs, a.n_pairs * (uint32_t)sizeof(PairDD));
    CopyWords(s_phase, a.phase256, 256 * (uint32_t)sizeof(float4));
    for (uint32_t j = 0; j < a.n_stage; ++j) {
        CopyWords(sbase + a.stage_off_x[j], a.stage_x[j], a.stage_n[j] * (uint32_t)sizeof(float2));
        CopyWords(sbase + a.stage_off_c[j], a.stage_c[j], 2 * (a.stage_n[j] - 1) * (uint32_t)sizeof(float4));
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (uint32_t i = 0; i < a.n_pairs; ++i)
            for (uint32_t j = 0; j < a.n_stage; ++j) {
                CubicDD* t[3] = {&s_pairs[i].v_long_r, &s_pairs[i].v_r, &s_pairs[i].u_long_r};
                for (CubicDD* c : t)
                    if (c->x == a.stage_x[j]) {
                        c->x = reinterpret_cast<const float2*>(sbase + a.stage_off_x[j]);
                        c->c = reinterpret_cast<const float4*>(sbase + a.stage_off_c[j]);
                    }
            }
    __syncthreads();
    ddc* tab_old = reinterpret_cast<ddc*>(sbase + a.off_work);          // [spc][3][stride]
    ddc* tab_new = tab_old + (size_t)a.slices_per_cta * 3 * stride;       // [spc][3][stride]
    float2* tf_old = reinterpret_cast<float2*>(tab_old);                  // FP32 mode: same rows, float2 entries
    float2* tf_new = reinterpret_cast<float2*>(tab_new);
    dd* seg_old = reinterpret_cast<dd*>(tab_new + (size_t)a.slices_per_cta * 3 * stride);  // [cap][3]
    dd* seg_new = seg_old + 3 * cap;                                      // [cap][3]
    dd* d_old = seg_new + 3 * cap;                                        // [cap][3] sampling displacements
    dd* d_new = d_old + 3 * cap;                                          // [cap][3]
    float* zs = reinterpret_cast<float*>(d_new + 3 * cap);                // [cap][3] normals
    float* logu = zs + 3 * cap;                                           // [kMaxLevels]
    __shared__ dd s_lvl_diff[kMaxLevels], s_lvl_small[kMaxLevels];
    __shared__ dd s_old_lsp[kMaxLevels], s_old_small[kMaxLevels];
    __shared__ dd s_red[kWarps];
    __shared__ dd s_big;
    __shared__ int s_result;
    __shared__ uint32_t s_slice_jj[kMaxOwned];
    __shared__ uint32_t s_n_own;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t G = gridDim.x, cta = blockIdx.x;
    // Group of this block (one attempt per group and round) and its place in the group.
    const uint32_t Gg = a.group_ctas, grp = cta / Gg, lc = cta - grp * Gg;
    const uint32_t r_own = lc % a.R, q_own = lc / a.R;
    const bool owns_k = q_own < a.Q;
    const uint32_t k_lo = owns_k ? (uint32_t)(((uint64_t)K * q_own) / a.Q) : 0u;
    const uint32_t k_hi = owns_k ? (uint32_t)(((uint64_t)K * (q_own + 1)) / a.Q) : 0u;
    // The block's k-chunk of the k-vector indices and of every long-range action's v_k (FP32 mode:
    // the leading float of each), staged once per launch: the chunk is the same in every attempt.
    int32_t* s_kidx = reinterpret_cast<int32_t*>(sbase + a.off_kstage);
    float* s_vkf = reinterpret_cast<float*>(s_kidx + a.kstage_n);    // FP32: [n_pairs][kstage_n]
    float2* s_vkd = reinterpret_cast<float2*>(s_kidx + a.kstage_n);  // double-float: [n_pairs][kstage_n]
    const bool kstaged = a.kstage_n > 0 && k_hi - k_lo <= a.kstage_n;
    if (kstaged) {
        for (uint32_t i = threadIdx.x; i < k_hi - k_lo; i += blockDim.x) s_kidx[i] = a.kidx[k_lo + i];
        for (uint32_t p = 0; p < a.n_pairs; ++p)
            if (s_pairs[p].use_lr && !s_pairs[p].is_constant)
                for (uint32_t i = threadIdx.x; i < k_hi - k_lo; i += blockDim.x) {
                    if constexpr (kF32) s_vkf[(size_t)p * a.kstage_n + i] = s_pairs[p].vk[k_lo + i].x;
                    else s_vkd[(size_t)p * a.kstage_n + i] = s_pairs[p].vk[k_lo + i];
                }
    }
    __syncthreads();
    auto kidx_of = [&](uint32_t k) { return kstaged ? s_kidx[k - k_lo] : a.kidx[k]; };

    uint64_t ctr[kMaxMoves];
    unsigned long long n_acc[kMaxMoves], n_l0[kMaxMoves];
    for (int m = 0; m < kMaxMoves; ++m) {
        ctr[m] = a.attempt_base[m];
        n_acc[m] = n_l0[m] = 0ull;
    }
    uint64_t nbar = 0;
    // Optional phase timing of block 0 (tracing aid; the work done is identical either way).
    const bool timing = a.phase_cycles != nullptr && cta == 0 && tid == 0;
    unsigned long long ph[kSweepTimingSlots] = {0ull};
    long long t_prev = clock64();
    const bool timing_cta = a.phase_cycles != nullptr && cta == 0;
    __shared__ unsigned long long s_role_max[kSweepRoles];
    if (timing_cta && tid < kSweepRoles) s_role_max[tid] = 0ull;
#define PIMC_PHASE(i)                             \
    if (timing) {                                 \
        const long long t_now = clock64();        \
        ph[i] += (unsigned long long)(t_now - t_prev); \
        t_prev = t_now;                           \
    }
#define PIMC_ROLE_BEGIN(v) const long long v = timing_cta ? clock64() : 0ll
#define PIMC_ROLE_END(v, r)                                                                         \
    if (timing_cta && lane == 0) atomicMax(&s_role_max[r], (unsigned long long)(clock64() - v))

    bool abort = false;
    // One bisection attempt of move m with Philox counter actr, by this block's group.
    auto attempt = [&](const uint32_t m, const uint64_t actr) {
            const MoveDD& mv = s_moves[m];
            const uint32_t s = mv.species, nl = mv.n_level, B = 1u << nl;
            const uint32_t g_off = a.sp_off[s];
            bool any_lr = false, grid_work = false, ext_links = false;
            int slot_s = -1, slot_o_first = -1;
            uint32_t n_links = 0;  // pair links of the moved particle over the segment, all pair actions
            uint32_t link_off[kMaxPair + 1];
            for (int pi = 0; pi < mv.n_pair; ++pi) {
                const PairDD& pa = s_pairs[mv.pair[pi]];
                link_off[pi] = n_links;
                if (!pa.is_constant) {
                    grid_work = true;
                    ext_links |= pa.kind != kPairBare;
                    const uint32_t other = pa.sa == pa.sb ? s : (pa.sa == s ? pa.sb : pa.sa);
                    n_links += (pa.sa == pa.sb ? a.sp_n[s] - 1 : a.sp_n[other]) * B;
                }
                if (pa.use_lr && !pa.is_constant) {
                    any_lr = true;
                    slot_s = pa.sa == s ? pa.slot_a : pa.slot_b;
                    if (pa.sa != pa.sb && slot_o_first < 0) slot_o_first = pa.sa == s ? pa.slot_b : pa.slot_a;
                }
            }
            link_off[mv.n_pair] = n_links;
            // Pair link l is evaluated by block l mod Gg of the group, lane quad 127 - (l / Gg) mod
            // 128: links fill the top warps first, which are idle while the sampling chain runs.
            const uint32_t n_quads = blockDim.x / 4;
            const int qlane = tid & 3;
            const uint32_t link_stride = Gg * n_quads;
            const uint32_t link_first = lc + Gg * (n_quads - 1 - (uint32_t)(tid >> 2));
            // Warp-uniform trip count of the link loop (all lanes join the quad shuffles).
            const uint32_t warp_first = lc + Gg * (n_quads - 1 - (uint32_t)((warp * 32 + 31) >> 2));
            const uint32_t link_rounds = warp_first < n_links ? (n_links - warp_first + link_stride - 1) / link_stride : 0u;
            // Designated blocks for the per-level sums when the attempt has a grid phase: the last
            // n_level blocks of the group, one level each (published with the grid barrier).
            const int my_level = (grid_work && lc + nl >= Gg) ? (int)(Gg - 1 - lc) : -1;
            {
                const MoveStream st{a.seed, a.chain, m, actr};
                const Philox4 w0 = st.Block(0);
                const uint32_t p = UniformIndex(w0.v[0], a.sp_n[s]);
                const uint32_t bead0 = UniformIndex(w0.v[1], M);
                const uint32_t g = g_off + p;

                // ---- 1. segment (warps 0-1), normals (warps 2-3), acceptance logarithms (warp 4),
                //         owned slices (warp 5), all in parallel ---------------------------------
                if (warp < 2) {
                    for (uint32_t i = tid; i < (B + 1) * 3; i += 64) {
                        const uint32_t j = i / 3, d = i % 3;
                        dd v{0.f, 0.f};
                        if (d < n_d) v = LoadDD(&a.pos[((size_t)((bead0 + j) % M) * 3 + d) * np + g]);
                        seg_old[i] = v;
                        seg_new[i] = v;
                    }
                } else if (warp < 4) {
                    // two lanes per resampled bead: BisectNormals' two Box-Muller transforms of its
                    // Philox block (z0, z1 from words 0-1 on the even lane, z2 from words 2-3)
                    for (uint32_t j = tid - 64; j < 2 * (B - 1); j += 64) {
                        const uint32_t i = j >> 1;
                        const Philox4 w = st.Block(1u + i);
                        float z0, z1;
                        if ((j & 1u) == 0) {
                            BoxMullerF(w.v[0], w.v[1], z0, z1);
                            zs[3 * i] = z0;
                            zs[3 * i + 1] = z1;
                        } else {
                            BoxMullerF(w.v[2], w.v[3], z0, z1);
                            zs[3 * i + 2] = z0;
                        }
                    }
                } else if (warp == 4) {
                    if (lane < (int)nl) logu[lane] = BisectLogU(st, B, (uint32_t)lane);
                } else if (warp == 5) {
                    uint32_t n = 0;
                    if (owns_k && any_lr)
                        for (uint32_t j0 = 1; j0 < B; j0 += 32) {
                            const uint32_t jj = j0 + lane;
                            const bool mine = jj < B && ((bead0 + jj) % M) % a.R == r_own;
                            const unsigned mask = __ballot_sync(0xffffffffu, mine);
                            if (mine) {
                                const uint32_t slot = n + __popc(mask & ((1u << lane) - 1u));
                                if (slot < kMaxOwned) s_slice_jj[slot] = jj;
                            }
                            n += __popc(mask);
                        }
                    if (lane == 0) s_n_own = n < kMaxOwned ? n : kMaxOwned;
                }
                __syncthreads();
                PIMC_PHASE(0);
                const uint32_t n_own = s_n_own;
                // Prefetch the Ewald cells of this thread's first owned item: the loads overlap with
                // the sampling phases and are consumed in the grid phase.
                const uint32_t nk_own = k_hi - k_lo;
                float4 pre_rho = make_float4(0.f, 0.f, 0.f, 0.f), pre_rho_o = pre_rho;
                // Density staging: every Ewald cell this thread evaluates (cell ci = tid + ci blockDim),
                // the moved species' and the first other species' densities, copied asynchronously into
                // shared memory now and read in the grid phase, so that no cell's load sits on it.
                const bool staged_rho = a.rho_cpt > 0 && n_own * nk_own <= a.rho_cpt * blockDim.x;  // else read global memory
                float2* st_f = reinterpret_cast<float2*>(sbase + a.off_rho_stage);  // FP32: [cpt][blockDim][2]
                float4* st_d = reinterpret_cast<float4*>(sbase + a.off_rho_stage);  // double-float: [cpt][blockDim][2]
                if (staged_rho) {
                    if (any_lr) {
                        uint32_t ci = 0;
                        CellIter cell(tid, blockDim.x, nk_own);
                        for (uint32_t it = tid; it < n_own * nk_own; it += blockDim.x, ++ci, cell.Next()) {
                            const uint32_t k = k_lo + cell.kk;
                            const uint32_t b = RingSlice(bead0, s_slice_jj[cell.si], M);
                            const size_t e = 2 * ((size_t)ci * blockDim.x + tid);
                            if constexpr (kF32) {
                                CpAsync8(st_f + e, &a.rho32[((size_t)slot_s * M + b) * K + k]);
                                if (slot_o_first >= 0) CpAsync8(st_f + e + 1, &a.rho32[((size_t)slot_o_first * M + b) * K + k]);
                            } else {
                                CpAsync16(st_d + e, &a.rho[((size_t)slot_s * M + b) * K + k]);
                                if (slot_o_first >= 0) CpAsync16(st_d + e + 1, &a.rho[((size_t)slot_o_first * M + b) * K + k]);
                            }
                        }
                    }
                    CpAsyncCommit();
                } else if (any_lr && (uint32_t)tid < n_own * nk_own) {
                    const uint32_t k = k_lo + tid % nk_own;
                    const uint32_t b = (bead0 + s_slice_jj[tid / nk_own]) % M;
                    if constexpr (kF32) {
                        const float2 v = a.rho32[((size_t)slot_s * M + b) * K + k];
                        pre_rho = make_float4(v.x, v.y, 0.f, 0.f);
                        if (slot_o_first >= 0) {
                            const float2 w = a.rho32[((size_t)slot_o_first * M + b) * K + k];
                            pre_rho_o = make_float4(w.x, w.y, 0.f, 0.f);
                        }
                    } else {
                        pre_rho = a.rho[((size_t)slot_s * M + b) * K + k];
                        if (slot_o_first >= 0) pre_rho_o = a.rho[((size_t)slot_o_first * M + b) * K + k];
                    }
                }
                dd pair_old{0.f, 0.f};  // stored copy's pair links of this lane's quad (quad lane 0)
                bool old_done = false;
                ddc pre_eo{{0.f, 0.f}, {0.f, 0.f}};
                float2 pre_eo_f = make_float2(0.f, 0.f);
                bool eo_done = false;
                PIMC_ROLE_BEGIN(rt2);
                // Warp roles: level sums run in one warp of a designated block when the attempt has
                // a grid phase (published through the barrier), in one warp per level otherwise.
                const int n_lvl_w = my_level >= 0 ? 1 : (grid_work ? 0 : (int)nl);

                // ---- 2. sampling chain (warp 0) || stored-copy level sums || old phase tables
                //         || stored-copy pair links -------------------------------------------
                const int w_tab2 = 1 + n_lvl_w;
                const int n_tw2 = any_lr ? min((int)(n_own * 3), kWarps - w_tab2 - 1) : 0;
                if (warp == 0) {
                    uint32_t mid = 0;
                    for (int lvl = (int)nl - 1; lvl >= 0; --lvl) {
                        const uint32_t skip = 1u << lvl, nm = B / (2 * skip);
                        const dd sigma = mv.sigma[lvl];
                        for (uint32_t t = lane; t < nm * n_d; t += 32) {
                            const uint32_t mm = t / n_d, d = t % n_d;
                            const uint32_t ja = mm * 2 * skip, jb = ja + skip, jc = ja + 2 * skip;
                            // Path::RBar (path_class.h:124) on the working copy.
                            const dd na = seg_new[3 * ja + d], nc = seg_new[3 * jc + d];
                            const dd nbar2 = Add(na, Scale2(MinImageDD(Sub(nc, na), a.L, a.iL), 0.5f));
                            const dd dn = MinImageDD(MulF(sigma, zs[3 * (mid + mm) + d]), a.L, a.iL);
                            d_new[3 * (mid + mm) + d] = dn;
                            seg_new[3 * jb + d] = Add(nbar2, dn);
                        }
                        mid += nm;
                        __syncwarp();
                    }
                    PIMC_ROLE_END(rt2, 0);
                } else if (warp < w_tab2) {
                    // Everything of the stored copy is known before sampling: its displacements from
                    // the midpoints and its level sums.
                    const int lvl = my_level >= 0 ? my_level : warp - 1;
                    const uint32_t skip = 1u << lvl, nm = B / (2 * skip), first = LevelFirst(nl, lvl, B);
                    for (uint32_t t = lane; t < nm * n_d; t += 32) {
                        const uint32_t mm = t / n_d, d = t % n_d;
                        const uint32_t ja = mm * 2 * skip, jb = ja + skip, jc = ja + 2 * skip;
                        const dd ra = seg_old[3 * ja + d], rc = seg_old[3 * jc + d];
                        const dd rbar = Add(ra, Scale2(MinImageDD(Sub(rc, ra), a.L, a.iL), 0.5f));
                        d_old[3 * (first + mm) + d] = MinImageDD(Sub(seg_old[3 * jb + d], rbar), a.L, a.iL);
                    }
                    __syncwarp();
                    dd lsp, sm;
                    LevelSums(mv, lvl, B, B != M, seg_old, d_old, first, n_d, a.L, a.iL, lane, lsp, sm);
                    if (lane == 0) {
                        s_old_lsp[lvl] = lsp;
                        s_old_small[lvl] = sm;
                    }
                    PIMC_ROLE_END(rt2, 1);
                } else if (warp < w_tab2 + n_tw2) {
                    for (uint32_t task = warp - w_tab2; task < n_own * 3; task += n_tw2) {
                        const uint32_t si = task / 3, d = task % 3;
                        if (d < n_d)
                            for (int n = lane; n <= a.max_index[d]; n += 32)
                                if constexpr (kF32) tf_old[(si * 3 + d) * stride + n] = PhaseF(seg_old[3 * s_slice_jj[si] + d], n, a.iL, s_phase);
                                else tab_old[(si * 3 + d) * stride + n] = PhaseDD(seg_old[3 * s_slice_jj[si] + d], n, a.iL, a.two_pi, s_phase);
                    }
                    PIMC_ROLE_END(rt2, 2);
                } else if (grid_work) {
                    // Pair links of the stored copy (they do not depend on the sampling).
                    for (uint32_t r = 0; r < link_rounds; ++r) {
                        const uint32_t l = link_first + r * link_stride;
                        pair_old = Add(pair_old, PairLinkU4(s_pairs, mv, link_off, l, l < n_links, qlane, s, p, B, bead0, M, np, n_d, a.sp_off,
                                                            a.pos, seg_old, a.L, a.iL, a.tau, ext_links));
                    }
                    old_done = true;
                    PIMC_ROLE_END(rt2, 3);
                }
                __syncthreads();
                PIMC_PHASE(1);
                PIMC_ROLE_BEGIN(rt3);

                // ---- 3. per-level sums of the working copy || new phase tables -------------
                const int n_tw3 = any_lr ? min((int)(n_own * 3), kWarps - n_lvl_w - 1) : 0;
                if (warp < n_lvl_w) {
                    const int lvl = my_level >= 0 ? my_level : warp;
                    dd lsp, sm;
                    LevelSums(mv, lvl, B, B != M, seg_new, d_new, LevelFirst(nl, lvl, B), n_d, a.L, a.iL, lane, lsp, sm);
                    if (lane == 0) {
                        const dd diff = Sub(s_old_lsp[lvl], lsp);   // old log-prob - new log-prob
                        const dd small = Sub(sm, s_old_small[lvl]); // new action - old action
                        if (my_level >= 0) {
                            // published with this attempt's grid barrier (generation nbar + 1)
                            __stcg(&a.level_out[(((nbar + 1) & 1ull) * kWaveSlots + grp) * kMaxLevels + lvl],
                                   make_float4(diff.hi, diff.lo, small.hi, small.lo));
                        } else {
                            s_lvl_diff[lvl] = diff;
                            s_lvl_small[lvl] = small;
                        }
                    }
                    PIMC_ROLE_END(rt3, 4);
                } else {
                    const int w0 = n_lvl_w;
                    const int n_tw = n_tw3;
                    if (warp < w0 + n_tw) {
                        for (uint32_t task = warp - w0; task < n_own * 3; task += n_tw) {
                            const uint32_t si = task / 3, d = task % 3;
                            if (d < n_d)
                                for (int n = lane; n <= a.max_index[d]; n += 32)
                                    if constexpr (kF32) tf_new[(si * 3 + d) * stride + n] = PhaseF(seg_new[3 * s_slice_jj[si] + d], n, a.iL, s_phase);
                                    else tab_new[(si * 3 + d) * stride + n] = PhaseDD(seg_new[3 * s_slice_jj[si] + d], n, a.iL, a.two_pi, s_phase);
                        }
                        PIMC_ROLE_END(rt3, 5);
                    } else if (any_lr && (uint32_t)tid < n_own * nk_own) {
                        // Old-position phase of this thread's first Ewald cell (tables built above).
                        if constexpr (kF32) pre_eo_f = PhaseProductF(tf_old + (size_t)(tid / nk_own) * 3 * stride, stride, n_d, kidx_of(k_lo + tid % nk_own));
                        else pre_eo = PhaseProductDD(tab_old + (size_t)(tid / nk_own) * 3 * stride, stride, n_d, kidx_of(k_lo + tid % nk_own));
                        eo_done = true;
                        PIMC_ROLE_END(rt3, 6);
                    }
                }
                __syncthreads();
                PIMC_PHASE(2);
                PIMC_ROLE_BEGIN(rt4);

                // ---- 4. level-0 grid work: pair links + owned Ewald cells -------------------
                ddc delta_cache[kDeltaCache];
                float2 delta_f[kDeltaCache];
                if (grid_work) {
                    // Pair links (pair_action_class.h:280-290), CalcU = tau V at level 0: the working
                    // copy here; the stored copy was summed during sampling by free warps.
                    dd acc{0.f, 0.f};
                    for (uint32_t r = 0; r < link_rounds; ++r) {
                        const uint32_t l = link_first + r * link_stride;
                        acc = Add(acc, PairLinkU4(s_pairs, mv, link_off, l, l < n_links, qlane, s, p, B, bead0, M, np, n_d, a.sp_off, a.pos,
                                                  seg_new, a.L, a.iL, a.tau, ext_links));
                        if (!old_done)
                            acc = Sub(acc, PairLinkU4(s_pairs, mv, link_off, l, l < n_links, qlane, s, p, B, bead0, M, np, n_d, a.sp_off, a.pos,
                                                      seg_old, a.L, a.iL, a.tau, ext_links));
                    }
                    if (old_done) acc = Sub(acc, pair_old);
                    if (any_lr && kF32) {
                        // FP32 mode: the same cells with FP32 phases and densities; each thread's
                        // terms in a compensated sum, joined to the double-float total once.
                        const uint32_t nk = nk_own;
                        Comp lr32{0.f, 0.f};
                        uint32_t ci = 0;
                        // This cell's densities (the first ones were loaded at the top of the
                        // attempt); the next cell's are requested before this one's arithmetic.
                        float2 rho_nx = make_float2(pre_rho.x, pre_rho.y), ro_nx = make_float2(pre_rho_o.x, pre_rho_o.y);
                        if (staged_rho) CpAsyncWaitAll();
                        CellIter cell(tid, blockDim.x, nk);
                        for (uint32_t it = tid; it < n_own * nk; it += blockDim.x, ++ci, cell.Next()) {
                            const uint32_t si = cell.si, k = k_lo + cell.kk;
                            const uint32_t b = RingSlice(bead0, s_slice_jj[si], M);
                            if (staged_rho) {
                                const float2* e = st_f + 2 * ((size_t)ci * blockDim.x + tid);
                                rho_nx = e[0];
                                ro_nx = e[1];
                            }
                            const float2 rho = rho_nx, ro_first = ro_nx;
                            if (!staged_rho && it + blockDim.x < n_own * nk) {
                                const uint32_t it2 = it + blockDim.x, si2 = it2 / nk, k2 = k_lo + it2 % nk;
                                const uint32_t b2 = (bead0 + s_slice_jj[si2]) % M;
                                rho_nx = a.rho32[((size_t)slot_s * M + b2) * K + k2];
                                if (slot_o_first >= 0) ro_nx = a.rho32[((size_t)slot_o_first * M + b2) * K + k2];
                            }
                            const int32_t pk = kidx_of(k);
                            const float2 en = PhaseProductF(tf_new + (size_t)si * 3 * stride, stride, n_d, pk);
                            const float2 eo = (ci == 0 && eo_done) ? pre_eo_f : PhaseProductF(tf_old + (size_t)si * 3 * stride, stride, n_d, pk);
                            const float2 dl = make_float2(__fsub_rn(en.x, eo.x), __fsub_rn(en.y, eo.y));
                            // the committed value of the cell if the attempt is accepted
                            if (ci < kDeltaCache) delta_f[ci] = make_float2(__fadd_rn(rho.x, dl.x), __fadd_rn(rho.y, dl.y));
                            for (int pi = 0; pi < mv.n_pair; ++pi) {
                                const PairDD& pa = s_pairs[mv.pair[pi]];
                                if (!pa.use_lr || pa.is_constant) continue;
                                const float vk = kstaged ? s_vkf[(size_t)mv.pair[pi] * a.kstage_n + (k - k_lo)] : pa.vk[k].x;
                                if (pa.sa == pa.sb) {
                                    const float t = __fmaf_rn(dl.x, __fmaf_rn(2.f, rho.x, dl.x), __fmul_rn(dl.y, __fmaf_rn(2.f, rho.y, dl.y)));
                                    CompAdd(lr32, __fmul_rn(vk, t));
                                } else {
                                    const int slot_o = pa.sa == s ? pa.slot_b : pa.slot_a;
                                    const float2 ro = slot_o == slot_o_first ? ro_first : a.rho32[((size_t)slot_o * M + b) * K + k];
                                    const float t = __fmaf_rn(dl.x, ro.x, __fmul_rn(dl.y, ro.y));
                                    CompAdd(lr32, __fmul_rn(2.f * vk, t));
                                }
                            }
                        }
                        acc = Add(acc, Mul(a.tau, CompDD(lr32)));
                    } else if (any_lr) {
                        const uint32_t nk = nk_own;
                        dd lr{0.f, 0.f};
                        uint32_t ci = 0;
                        if (staged_rho) CpAsyncWaitAll();
                        CellIter cell(tid, blockDim.x, nk);
                        for (uint32_t it = tid; it < n_own * nk; it += blockDim.x, ++ci, cell.Next()) {
                            const uint32_t si = cell.si, k = k_lo + cell.kk;
                            const uint32_t b = RingSlice(bead0, s_slice_jj[si], M);
                            const int32_t pk = kidx_of(k);
                            const ddc en = PhaseProductDD(tab_new + (size_t)si * 3 * stride, stride, n_d, pk);
                            const ddc eo = (ci == 0 && eo_done) ? pre_eo : PhaseProductDD(tab_old + (size_t)si * 3 * stride, stride, n_d, pk);
                            const ddc dl = CSub(en, eo);
                            const float4* e = st_d + 2 * ((size_t)ci * blockDim.x + tid);
                            const ddc rho = Unpack(staged_rho ? e[0] : (ci == 0 ? pre_rho : a.rho[((size_t)slot_s * M + b) * K + k]));
                            if (ci < kDeltaCache) delta_cache[ci] = CAdd(rho, dl);  // the committed value on acceptance
                            for (int pi = 0; pi < mv.n_pair; ++pi) {
                                const PairDD& pa = s_pairs[mv.pair[pi]];
                                if (!pa.use_lr || pa.is_constant) continue;
                                const float2 vkf = kstaged ? s_vkd[(size_t)mv.pair[pi] * a.kstage_n + (k - k_lo)] : pa.vk[k];
                                const dd vk{vkf.x, vkf.y};
                                if (pa.sa == pa.sb) {
                                    // |rho + D|^2 - |rho|^2 = D.re (2 rho.re + D.re) + D.im (2 rho.im + D.im)
                                    const dd t = Add(Mul(dl.re, Add(Scale2(rho.re, 2.f), dl.re)), Mul(dl.im, Add(Scale2(rho.im, 2.f), dl.im)));
                                    lr = Add(lr, Mul(vk, t));
                                } else {
                                    const int slot_o = pa.sa == s ? pa.slot_b : pa.slot_a;
                                    const ddc ro = Unpack(slot_o == slot_o_first ? (staged_rho ? e[1] : (ci == 0 ? pre_rho_o : a.rho[((size_t)slot_o * M + b) * K + k]))
                                                                                 : a.rho[((size_t)slot_o * M + b) * K + k]);
                                    const dd t = Add(Mul(dl.re, ro.re), Mul(dl.im, ro.im));
                                    lr = Add(lr, Scale2(Mul(vk, t), 2.f));
                                }
                            }
                        }
                        acc = Add(acc, Mul(a.tau, lr));
                    }
                    PIMC_ROLE_END(rt4, 7);
                    // block sum (fixed order) -> partial -> grid barrier -> ordered total
                    ++nbar;
                    const dd v = WarpSumDD(acc);
                    if (lane == 0) s_red[warp] = v;
                    __syncthreads();
                    PIMC_PHASE(3);
                    if (warp == 0) {
                        dd t = lane < kWarps ? s_red[lane] : dd{0.f, 0.f};
                        t = WarpSumDD(t);
                        if (lane == 0) __stcg(&a.partials[(nbar & 1ull) * G + cta], make_float2(t.hi, t.lo));
                    }
                    if (!GridBarrier(a.bar, nbar, a.err, a.timeout_ns)) {
                        abort = true;
                        return;
                    }
                    PIMC_PHASE(4);
                    // The group's partials, one per thread in a single round trip, summed per warp
                    // and then over the warps in order (the same total in every block).
                    const uint32_t n_pw = (Gg + 31) / 32;
                    if ((uint32_t)warp < n_pw) {
                        const uint32_t c2 = (uint32_t)tid;
                        dd t{0.f, 0.f};
                        if (c2 < Gg) {
                            const float2 pv = __ldcg(&a.partials[(nbar & 1ull) * G + grp * Gg + c2]);
                            t = dd{pv.x, pv.y};
                        }
                        t = WarpSumDD(t);
                        if (lane == 0) s_red[warp] = t;
                    } else if ((uint32_t)warp == n_pw && lane < (int)nl) {
                        // level sums from the designated blocks (written before their arrival)
                        const float4 v = __ldcg(&a.level_out[((nbar & 1ull) * kWaveSlots + grp) * kMaxLevels + lane]);
                        s_lvl_diff[lane] = dd{v.x, v.y};
                        s_lvl_small[lane] = dd{v.z, v.w};
                    }
                    __syncthreads();
                    if (warp == 0) {
                        dd t = (uint32_t)lane < n_pw ? s_red[lane] : dd{0.f, 0.f};
                        t = WarpSumDD(t);
                        if (lane == 0) s_big = t;
                    }
                    __syncthreads();
                    PIMC_PHASE(5);
                } else if (tid == 0) {
                    s_big = dd{0.f, 0.f};
                }

                // ---- 5. Metropolis tests of every level (bisect_class.h:110-117) ------------
                // Level l's test reads only its own action change and the one of level l + 1 (the
                // reference's prev_action_change), so lane l evaluates level l and the top-most
                // failing level decides, as the reference's top-down loop would.
                if (warp == 0) {
                    const int lvl = lane;
                    bool fail = false, bad = false;
                    if (lvl < (int)nl) {
                        dd dS = s_lvl_small[lvl];
                        if (lvl == 0) dS = Add(dS, s_big);
                        const dd prev = lvl + 1 < (int)nl ? s_lvl_small[lvl + 1] : dd{0.f, 0.f};
                        const dd log_accept = Add(Sub(s_lvl_diff[lvl], dS), prev);
                        bad = !isfinite(log_accept.hi);
                        fail = bad || Less(log_accept, DD(logu[nl - 1 - lvl]));
                    }
                    const unsigned fm = __ballot_sync(0xffffffffu, fail);
                    const unsigned bm = __ballot_sync(0xffffffffu, bad);
                    if (lane == 0) {
                        int res = 1, top = -1;
                        if (fm) {
                            top = 31 - __clz(fm);
                            res = (bm >> top) & 1u ? 2 : 0;
                            if (res == 2) atomicCAS(a.err, 0, kDevErrNonFinite);
                        }
                        s_result = res | ((top <= 0) ? 4 : 0);  // bit 2: the attempt reached level 0
                    }
                }
                __syncthreads();
                PIMC_PHASE(6);
                const int res = s_result & 3;
                if (res == 2) {
                    abort = true;
                    return;
                }
                if (s_result & 4) n_l0[m] += 1;
                if (!grid_work) {
                    // Every block ran this attempt on the same inputs and commits the same beads;
                    // without a grid phase no barrier has yet kept a fast block's commit from
                    // reaching a slow block that still reads them.
                    ++nbar;
                    if (!GridBarrier(a.bar, nbar, a.err, a.timeout_ns)) {
                        abort = true;
                        return;
                    }
                }

                // ---- 6. commit ---------------------------------------------------------------
                if (res == 1) {
                    for (uint32_t i = tid; i < (B - 1) * n_d; i += blockDim.x) {
                        const uint32_t j = 1 + i / n_d, d = i % n_d;
                        const dd v = seg_new[3 * j + d];
                        a.pos[((size_t)((bead0 + j) % M) * 3 + d) * np + g] = make_float2(v.hi, v.lo);
                    }
                    if (any_lr) {
                        const uint32_t nk = k_hi - k_lo;
                        uint32_t ci = 0;
                        CellIter cell(tid, blockDim.x, nk);
                        for (uint32_t it = tid; it < n_own * nk; it += blockDim.x, ++ci, cell.Next()) {
                            const uint32_t si = cell.si, k = k_lo + cell.kk;
                            const uint32_t b = RingSlice(bead0, s_slice_jj[si], M);
                            // The first kDeltaCache cells of the thread store the value formed in the
                            // grid phase (the cell as loaded there plus the change); later ones re-form it.
                            if constexpr (kF32) {
                                float2* cell = &a.rho32[((size_t)slot_s * M + b) * K + k];
                                if (ci < kDeltaCache) {
                                    *cell = delta_f[ci];
                                } else {
                                    const int32_t pk = kidx_of(k);
                                    const float2 en = PhaseProductF(tf_new + (size_t)si * 3 * stride, stride, n_d, pk);
                                    const float2 eo = PhaseProductF(tf_old + (size_t)si * 3 * stride, stride, n_d, pk);
                                    const float2 dl = make_float2(__fsub_rn(en.x, eo.x), __fsub_rn(en.y, eo.y));
                                    const float2 c0 = staged_rho ? st_f[2 * ((size_t)ci * blockDim.x + tid)] : *cell;
                                    *cell = make_float2(__fadd_rn(c0.x, dl.x), __fadd_rn(c0.y, dl.y));
                                }
                            } else {
                                float4* cell = &a.rho[((size_t)slot_s * M + b) * K + k];
                                if (ci < kDeltaCache) {
                                    *cell = Pack(delta_cache[ci]);
                                } else {
                                    const int32_t pk = kidx_of(k);
                                    const ddc dl = CSub(PhaseProductDD(tab_new + (size_t)si * 3 * stride, stride, n_d, pk),
                                                        PhaseProductDD(tab_old + (size_t)si * 3 * stride, stride, n_d, pk));
                                    *cell = Pack(CAdd(Unpack(staged_rho ? st_d[2 * ((size_t)ci * blockDim.x + tid)] : *cell), dl));
                                }
                            }
                        }
                    }
                    n_acc[m] += 1;
                }
                __syncthreads();
                PIMC_PHASE(7);
                if (timing)
                    for (int r = 0; r < kSweepRoles; ++r) {
                        ph[kSweepPhases + r] += s_role_max[r];
                        s_role_max[r] = 0ull;
                    }
            }
    };

    if (a.wave <= 1) {
        for (uint64_t rep = 0; rep < a.n_rep; ++rep)
            for (uint32_t e = 0; e < a.n_entries; ++e) {
                const uint32_t m = a.sched_move[e];
                for (uint64_t c = 0, count = a.sched_count[e]; c < count; ++c) {
                    attempt(m, ctr[m]);
                    ctr[m] += 1;
                    if (abort) return;
                }
            }
    } else {
        // Rounds of concurrent attempts: the longest prefix of the next `wave` attempts of the
        // schedule in which no attempt reads what an earlier one may change; group j runs attempt
        // j (the sequential chain's result), and a second grid barrier makes every commit visible
        // before the next round reads, unless the next round reads nothing this round changes
        // (its own first barrier then orders these commits before any later round). Idle groups
        // keep the barrier count.
        const uint64_t total = a.n_rep * a.per_rep;
        const uint32_t W = a.wave;  // <= kWaveSlots = 8: lanes 0..2W-1 hold this round's and the next round's candidates
        uint64_t A = 0;
        while (A < total) {
            // Lane x: attempt A + x of the schedule (move, counter, first slice, length) and the
            // mask of the earlier candidates it conflicts with (the same on every warp).
            const uint32_t x = (uint32_t)lane;
            const bool valid = x < 2 * W && A + x < total;
            uint32_t m = 0, bj = 0, Bj = 1;
            uint64_t actr = 0;
            if (valid) {
                const uint64_t xx = A + x, rep = xx / a.per_rep, r = xx - rep * a.per_rep;
                uint32_t lo = 0, hi = a.n_entries;  // the entry holding position r of a repetition
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (a.sched_prefix[mid] <= r) lo = mid;
                    else hi = mid;
                }
                m = a.sched_move[lo];
                actr = a.attempt_base[m] + rep * a.per_rep_move[m] + a.move_before[lo] + (r - a.sched_prefix[lo]);
                const Philox4 w0 = MoveStream{a.seed, a.chain, m, actr}.Block(0);
                bj = UniformIndex(w0.v[1], M);  // the attempt's first slice
                Bj = 1u << s_moves[m].n_level;
            }
            uint32_t cmask = 0;  // bit i: attempt A + i (i < x) changes what attempt A + x reads
            for (uint32_t i = 0; i < 2 * W; ++i) {
                const uint32_t bi = __shfl_sync(0xffffffffu, bj, (int)i), Bi = __shfl_sync(0xffffffffu, Bj, (int)i);
                if (valid && i < x && Conflicts(bi, Bi, bj, Bj, M)) cmask |= 1u << i;
            }
            const uint32_t n_valid = (uint32_t)__popc(__ballot_sync(0xffffffffu, valid));
            // This round: the longest prefix of [0, W) in which no attempt conflicts with an earlier one.
            const unsigned end_r = __ballot_sync(0xffffffffu, valid && x >= 1 && x < W && (cmask & ((1u << x) - 1u)) != 0u);
            const uint32_t w = end_r ? (uint32_t)__ffs(end_r) - 1u : min(W, n_valid);
            // The next round: its prefix from w; the commit barrier is skipped when none of its
            // attempts reads what this round's attempts change.
            const uint32_t below_next = (1u << (w + (x > w ? x - w : 0u))) - 1u;  // candidates w .. x - 1
            const unsigned end_n = __ballot_sync(0xffffffffu, valid && x > w && x < w + W && (cmask & below_next & ~((1u << w) - 1u)) != 0u);
            const uint32_t w_next = end_n ? (uint32_t)__ffs(end_n) - 1u - w : min(W, n_valid - w);
            const unsigned cross = __ballot_sync(0xffffffffu, valid && x >= w && x < w + w_next && (cmask & ((1u << w) - 1u)) != 0u);
            const bool commit_barrier = cross != 0u || w_next == 0u;
            const uint32_t my_m = __shfl_sync(0xffffffffu, m, (int)(grp < w ? grp : 0u));
            const uint64_t my_c = __shfl_sync(0xffffffffu, actr, (int)(grp < w ? grp : 0u));
            if (grp < w) {
                attempt(my_m, my_c);
                if (abort) return;
            } else {
                ++nbar;
                if (!GridBarrier(a.bar, nbar, a.err, a.timeout_ns)) return;
            }
            if (commit_barrier) {
                ++nbar;
                if (!GridBarrier(a.bar, nbar, a.err, a.timeout_ns)) return;
            } else {
                __syncthreads();  // the block's own commits before its next round's reads
            }
            A += w;
        }
    }
#undef PIMC_PHASE
#undef PIMC_ROLE_BEGIN
#undef PIMC_ROLE_END
    if (lc == 0 && tid == 0) {  // each group's first block reports its group's attempts
        for (int m = 0; m < kMaxMoves; ++m) {
            atomicAdd(&a.counters[m], n_acc[m]);
            atomicAdd(&a.counters[kMaxMoves + m], n_l0[m]);
        }
        if (timing)
            for (int i = 0; i < kSweepTimingSlots; ++i) a.phase_cycles[i] += ph[i];
    }
}

// Conversions between the FP64 state and its double-float mirror.
__global__ void ToDDKernel(const double* __restrict__ pos, float2* __restrict__ pos_dd, size_t n_pos, const double2* __restrict__ rho,
                           float4* __restrict__ rho_dd, size_t n_rho) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_pos + n_rho; i += (size_t)gridDim.x * blockDim.x) {
        if (i < n_pos) {
            float h, l;
            SplitDouble(pos[i], h, l);
            pos_dd[i] = make_float2(h, l);
        } else {
            const double2 v = rho[i - n_pos];
            float x0, x1, y0, y1;
            SplitDouble(v.x, x0, x1);
            SplitDouble(v.y, y0, y1);
            rho_dd[i - n_pos] = make_float4(x0, x1, y0, y1);
        }
    }
}

__global__ void FromDDKernel(const float2* __restrict__ pos_dd, double* __restrict__ pos, double* __restrict__ pos_new, size_t n_pos,
                             const float4* __restrict__ rho_dd, double2* __restrict__ rho, size_t n_rho) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_pos + n_rho; i += (size_t)gridDim.x * blockDim.x) {
        if (i < n_pos) {
            const float2 v = pos_dd[i];
            const double x = (double)v.x + (double)v.y;
            pos[i] = x;
            pos_new[i] = x;
        } else {
            const float4 v = rho_dd[i - n_pos];
            rho[i - n_pos] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
        }
    }
}

__global__ void ToF32Kernel(const double2* __restrict__ rho, float2* __restrict__ rho32, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        rho32[i] = make_float2((float)rho[i].x, (float)rho[i].y);
}

__global__ void FromF32Kernel(const float2* __restrict__ rho32, double2* __restrict__ rho, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        rho[i] = make_double2((double)rho32[i].x, (double)rho32[i].y);
}

// FP32 densities from the double-float positions (species_class.h:380-403 in FP32 mode): the sum
// over the species' particles, in particle order, of FP32 bead phases, compensated. One thread
// per k-vector of a 256-wide chunk, one block per (chunk, slice, slot); the phase rows of
// kRho32Chunk particles at a time sit in shared memory.
constexpr uint32_t kRho32Chunk = 64;

__global__ void InitRho32Kernel(const __grid_constant__ SweepArgs a, const int* __restrict__ slot_species) {
    extern __shared__ float2 ftab[];  // [kRho32Chunk][3][stride]
    const uint32_t stride = a.tab_stride, n_d = a.n_d, M = a.M, K = a.K, np = a.n_pad;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, slot = blockIdx.z;
    const uint32_t s = (uint32_t)slot_species[slot];
    const uint32_t ns = a.sp_n[s], off = a.sp_off[s];
    const int32_t pk = k < K ? a.kidx[k] : 0;
    Comp re{0.f, 0.f}, im{0.f, 0.f};
    for (uint32_t p0 = 0; p0 < ns; p0 += kRho32Chunk) {
        const uint32_t cnt = min(kRho32Chunk, ns - p0);
        __syncthreads();
        for (uint32_t t = threadIdx.x; t < cnt * 3 * stride; t += blockDim.x) {
            const uint32_t pi = t / (3 * stride), rem = t - pi * 3 * stride, d = rem / stride, n = rem - d * stride;
            if (d < n_d && (int)n <= a.max_index[d]) {
                const float2 v = a.pos[((size_t)b * 3 + d) * np + off + p0 + pi];
                ftab[t] = PhaseF(dd{v.x, v.y}, (int)n, a.iL, a.phase256);
            }
        }
        __syncthreads();
        if (k < K)
            for (uint32_t pi = 0; pi < cnt; ++pi) {
                const float2 e = PhaseProductF(ftab + (size_t)pi * 3 * stride, stride, n_d, pk);
                CompAdd(re, e.x);
                CompAdd(im, e.y);
            }
    }
    if (k < K) a.rho32[((size_t)slot * M + b) * K + k] = make_float2(__fadd_rn(re.s, re.c), __fadd_rn(im.s, im.c));
}

void Split(double x, dd& out) {
    float h, l;
    SplitDouble(x, h, l);
    out = dd{h, l};
}

/// The 53-bit uniform of two Philox words (philox.h Uniform53) as a float pair, without FP64:
/// u 2^53 = (w0 >> 5) 2^26 + (w1 >> 6); the leading 24 bits exactly, the remaining 29 rounded.
__device__ __forceinline__ void Split53(uint32_t w0, uint32_t w1, dd& u) {
    const uint32_t A = w0 >> 5, Bw = w1 >> 6;
    const float hi = __fmul_rn(__uint2float_rn(A >> 3), 5.9604644775390625e-08f);  // 2^-24
    const unsigned long long R = ((unsigned long long)(A & 7u) << 26) | (unsigned long long)Bw;
    const float lo = __fmul_rn(__ull2float_rn(R), 1.1102230246251565e-16f);  // 2^-53
    u = FastTwoSum(hi, lo);
}

#include "perm_dd.cuh"

}  // namespace

// ---------------------------------------------------------------------------------------------

void Context::EnsureDD() {
    RequirePath();
    if (dd_valid) return;
    const size_t n_pos = (size_t)sys.M * 3 * sys.n_pad;
    const size_t n_rho = (rho_slots && sys.K) ? (size_t)rho_slots * sys.M * sys.K : 0;
    if (!pos_dd_) pos_dd_.reset(new DeviceBuffer(n_pos * sizeof(float2)));
    if (precision == 32) {
        // FP32 mode: the densities are rebuilt from the positions at every sweep call.
        if (!rho32_) rho32_.reset(new DeviceBuffer(std::max<size_t>(n_rho, 1) * sizeof(float2)));
        ToDDKernel<<<n_sm * 4, 256, 0, stream>>>(sys.pos, pos_dd_->as<float2>(), n_pos, sys.rho_k, nullptr, 0);
    } else {
        if (!rho_dd_) rho_dd_.reset(new DeviceBuffer(std::max<size_t>(n_rho, 1) * sizeof(float4)));
        ToDDKernel<<<n_sm * 4, 256, 0, stream>>>(sys.pos, pos_dd_->as<float2>(), n_pos, sys.rho_k, rho_dd_->as<float4>(), n_rho);
    }
    CudaCheck(cudaGetLastError(), "to-dd launch");
    dd_valid = true;
}

void Context::SetPrecision(int bits) {
    if (bits != 32 && bits != 64) throw PimcError(kErrArg, "precision must be 32 or 64");
    if (bits == precision) return;
    EnsureFP64();
    precision = bits;
    dd_valid = false;
}

void PreloadConversionKernels() {
    cudaFuncAttributes fa;
    CudaCheck(cudaFuncGetAttributes(&fa, FromDDKernel), "loading FromDDKernel");
    CudaCheck(cudaFuncGetAttributes(&fa, FromF32Kernel), "loading FromF32Kernel");
}

void Context::EnsureFP64() {
    RequirePath();
    if (fp64_valid) return;
    const size_t n_pos = (size_t)sys.M * 3 * sys.n_pad;
    const size_t n_rho = (rho_slots && sys.K) ? (size_t)rho_slots * sys.M * sys.K : 0;
    if (precision == 32) {
        FromDDKernel<<<n_sm * 4, 256, 0, stream>>>(pos_dd_->as<float2>(), sys.pos, sys.pos_new, n_pos, nullptr, sys.rho_k, 0);
        if (n_rho) FromF32Kernel<<<n_sm * 4, 256, 0, stream>>>(rho32_->as<float2>(), sys.rho_k, n_rho);
    } else {
        FromDDKernel<<<n_sm * 4, 256, 0, stream>>>(pos_dd_->as<float2>(), sys.pos, sys.pos_new, n_pos, rho_dd_->as<float4>(), sys.rho_k, n_rho);
    }
    CudaCheck(cudaGetLastError(), "from-dd launch");
    Sync();
    fp64_valid = true;
}

static CubicDD MakeCubicDD(Context& c, const CubicTable& t, std::vector<std::unique_ptr<DeviceBuffer>>& keep) {
    CubicDD o;
    if (!t.c) return o;
    const Context::HostCubic* h = nullptr;
    for (auto& kv : c.host_cubics)
        if (kv.first == t.c) h = &kv.second;
    if (!h) throw PimcError(kErrState, "spline table without host copy");
    std::vector<float2> x(h->x.size());
    for (size_t i = 0; i < x.size(); ++i) {
        float hi, lo;
        SplitDouble(h->x[i], hi, lo);
        x[i] = make_float2(hi, lo);
    }
    std::vector<float4> cf(2 * h->c.size());
    for (size_t i = 0; i < h->c.size(); ++i) {
        float a0, a1, b0, b1, c0, c1, d0, d1;
        SplitDouble(h->c[i].c0, a0, a1);
        SplitDouble(h->c[i].c1, b0, b1);
        SplitDouble(h->c[i].c2, c0, c1);
        SplitDouble(h->c[i].c3, d0, d1);
        cf[2 * i] = make_float4(a0, a1, b0, b1);
        cf[2 * i + 1] = make_float4(c0, c1, d0, d1);
    }
    keep.emplace_back(new DeviceBuffer(x.size() * sizeof(float2)));
    CudaCheck(cudaMemcpy(keep.back()->ptr, x.data(), x.size() * sizeof(float2), cudaMemcpyHostToDevice), "dd knots");
    o.x = keep.back()->as<float2>();
    keep.emplace_back(new DeviceBuffer(cf.size() * sizeof(float4)));
    CudaCheck(cudaMemcpy(keep.back()->ptr, cf.data(), cf.size() * sizeof(float4), cudaMemcpyHostToDevice), "dd coefficients");
    o.c = keep.back()->as<float4>();
    o.bucket = t.bucket;
    o.n = t.n;
    o.n_bucket = t.n_bucket;
    o.uniform = t.uniform;
    o.x0f = (float)t.x0;
    o.inv_dxf = (float)t.inv_dx;
    // A grid whose spacing is uniform to within a quarter step locates its interval arithmetically
    // (the evaluator's scan corrects the estimate by one either way), skipping the bucket table.
    if (!o.uniform && h->x.size() >= 2) {
        const double step = (h->x.back() - h->x.front()) / (double)(h->x.size() - 1);
        bool near_uniform = step > 0.;
        for (size_t i = 0; near_uniform && i + 1 < h->x.size(); ++i)
            near_uniform = std::fabs((h->x[i + 1] - h->x[i]) - step) <= 0.25 * step;
        if (near_uniform) {
            o.uniform = 1;
            o.inv_dxf = (float)(1. / step);
        }
    }
    Split(t.x0, o.x0);
    Split(t.x1, o.x1);
    return o;
}

static MultiCubicDD MakeMultiCubicDD(Context& c, const MultiCubic& t, std::vector<std::unique_ptr<DeviceBuffer>>& keep) {
    MultiCubicDD o;
    if (!t.c) return o;
    const Context::HostMulti* h = nullptr;
    for (auto& kv : c.host_multis)
        if (kv.first == t.c) h = &kv.second;
    if (!h) throw PimcError(kErrState, "multi-spline table without host copy");
    std::vector<float2> x(h->x.size());
    for (size_t i = 0; i < x.size(); ++i) {
        float hi, lo;
        SplitDouble(h->x[i], hi, lo);
        x[i] = make_float2(hi, lo);
    }
    std::vector<float4> cf(2 * h->c.size());
    for (size_t i = 0; i < h->c.size(); ++i) {
        float a0, a1, b0, b1, c0, c1, d0, d1;
        SplitDouble(h->c[i].c0, a0, a1);
        SplitDouble(h->c[i].c1, b0, b1);
        SplitDouble(h->c[i].c2, c0, c1);
        SplitDouble(h->c[i].c3, d0, d1);
        cf[2 * i] = make_float4(a0, a1, b0, b1);
        cf[2 * i + 1] = make_float4(c0, c1, d0, d1);
    }
    keep.emplace_back(new DeviceBuffer(x.size() * sizeof(float2)));
    CudaCheck(cudaMemcpy(keep.back()->ptr, x.data(), x.size() * sizeof(float2), cudaMemcpyHostToDevice), "dd knots");
    o.x = keep.back()->as<float2>();
    keep.emplace_back(new DeviceBuffer(cf.size() * sizeof(float4)));
    CudaCheck(cudaMemcpy(keep.back()->ptr, cf.data(), cf.size() * sizeof(float4), cudaMemcpyHostToDevice), "dd coefficients");
    o.c = keep.back()->as<float4>();
    o.bucket = t.g.bucket;
    o.n = t.g.n;
    o.n_bucket = t.g.n_bucket;
    o.n_comp = t.n_comp;
    o.x0f = (float)t.g.x0;
    o.inv_dxf = (float)t.g.inv_dx;
    Split(t.g.x0, o.x0);
    Split(t.g.x1, o.x1);
    return o;
}

static BicubicDD MakeBicubicDD(Context& c, const BicubicTable& t, std::vector<std::unique_ptr<DeviceBuffer>>& keep) {
    BicubicDD o;
    if (!t.c) return o;
    const Context::HostBicubic* h = nullptr;
    for (auto& kv : c.host_bicubics)
        if (kv.first == t.c) h = &kv.second;
    if (!h) throw PimcError(kErrState, "2-D spline table without host copy");
    auto knots = [&](const std::vector<double>& x) {
        std::vector<float2> v(x.size());
        for (size_t i = 0; i < x.size(); ++i) {
            float hi, lo;
            SplitDouble(x[i], hi, lo);
            v[i] = make_float2(hi, lo);
        }
        keep.emplace_back(new DeviceBuffer(v.size() * sizeof(float2)));
        CudaCheck(cudaMemcpy(keep.back()->ptr, v.data(), v.size() * sizeof(float2), cudaMemcpyHostToDevice), "dd knots");
        return keep.back()->as<float2>();
    };
    o.gx = knots(h->x);
    o.gy = knots(h->y);
    std::vector<float4> cf(h->c.size() / 2);
    for (size_t i = 0; i + 1 < h->c.size(); i += 2) {
        float a0, a1, b0, b1;
        SplitDouble(h->c[i], a0, a1);
        SplitDouble(h->c[i + 1], b0, b1);
        cf[i / 2] = make_float4(a0, a1, b0, b1);
    }
    keep.emplace_back(new DeviceBuffer(cf.size() * sizeof(float4)));
    CudaCheck(cudaMemcpy(keep.back()->ptr, cf.data(), cf.size() * sizeof(float4), cudaMemcpyHostToDevice), "dd 2-D coefficients");
    o.c = keep.back()->as<float4>();
    o.bx = t.gx.bucket;
    o.by = t.gy.bucket;
    o.nx = t.gx.n;
    o.ny = t.gy.n;
    o.nbx = t.gx.n_bucket;
    o.nby = t.gy.n_bucket;
    o.x0f = (float)t.gx.x0;
    o.inv_dxf = (float)t.gx.inv_dx;
    o.y0f = (float)t.gy.x0;
    o.inv_dyf = (float)t.gy.inv_dx;
    Split(t.gx.x0, o.x0);
    Split(t.gx.x1, o.x1);
    Split(t.gy.x0, o.y0);
    Split(t.gy.x1, o.y1);
    return o;
}

void Context::BuildSweepTables() {
    if (sweep_tables_built_) return;
    std::vector<float4> tab(256);
    for (int j = 0; j < 256; ++j) {
        const double th = 2. * M_PI * j / 256.;
        float a0, a1, b0, b1;
        SplitDouble(std::cos(th), a0, a1);
        SplitDouble(std::sin(th), b0, b1);
        tab[j] = make_float4(a0, a1, b0, b1);
    }
    sweep_tables_.reset(new DeviceBuffer(sizeof(float4) * 256 + sizeof(PairDD) * kMaxPair));
    CudaCheck(cudaMemcpy(sweep_tables_->ptr, tab.data(), sizeof(float4) * 256, cudaMemcpyHostToDevice), "phase table");
    std::vector<PairDD> pd(kMaxPair);
    // Identical tables (one file read by several pair actions) share one device copy.
    std::vector<std::pair<const HostCubic*, CubicDD>> made;
    auto make = [&](const CubicTable& t) -> CubicDD {
        const HostCubic* h = nullptr;
        for (auto& kv : host_cubics)
            if (kv.first == t.c) h = &kv.second;
        for (auto& mk : made)
            if (h && mk.first->x == h->x && mk.first->c.size() == h->c.size() &&
                std::memcmp(mk.first->c.data(), h->c.data(), h->c.size() * sizeof(Cubic4)) == 0)
                return mk.second;
        CubicDD o = MakeCubicDD(*this, t, keep_);
        if (h) made.push_back({h, o});
        return o;
    };
    for (int i = 0; i < sys.n_pair; ++i) {
        const PairDev& p = sys.pair[i];
        PairDD& q = pd[i];
        q.sa = p.sa;
        q.sb = p.sb;
        q.kind = p.kind;
        q.is_coulomb = p.is_coulomb;
        q.use_lr = p.use_long_range;
        q.is_constant = p.is_constant;
        q.max_level = (int32_t)p.max_level;
        q.slot_a = sys.sp_rho[p.sa];
        q.slot_b = sys.sp_rho[p.sb];
        Split(p.r_v_min, q.rvmin);
        Split(p.r_v_max, q.rvmax);
        Split(p.r_vl_min, q.rvlmin);
        Split(p.r_vl_max, q.rvlmax);
        q.v_r = make(p.v_r);
        q.v_long_r = p.use_long_range ? make(p.v_long_r) : CubicDD();
        q.u_xy = BicubicDD();
        q.u_long_r = CubicDD();
        q.rumin = q.rumax = dd{0.f, 0.f};
        q.u_kj = MultiCubicDD();
        q.n_order = p.n_order;
        q.kj_stride = p.kj_stride;
        if (p.kind == kPairDavid) q.u_kj = MakeMultiCubicDD(*this, p.u_kj, keep_);
        if (p.kind == kPairIlkka) {
            q.u_xy = MakeBicubicDD(*this, p.u_xy, keep_);
            if (p.use_long_range) q.u_long_r = make(p.u_long_r);
            Split(p.r_u_min, q.rumin);
            Split(p.r_u_max, q.rumax);
        }
        q.vk = nullptr;
        if (p.use_long_range) {
            std::vector<float2> vk(sys.K);
            for (uint32_t k = 0; k < sys.K; ++k) {
                float hi, lo;
                SplitDouble(host_vk[i][k], hi, lo);
                vk[k] = make_float2(hi, lo);
            }
            keep_.emplace_back(new DeviceBuffer(sys.K * sizeof(float2)));
            CudaCheck(cudaMemcpy(keep_.back()->ptr, vk.data(), sys.K * sizeof(float2), cudaMemcpyHostToDevice), "dd vk");
            q.vk = keep_.back()->as<float2>();
        }
    }
    CudaCheck(cudaMemcpy(sweep_tables_->as<char>() + sizeof(float4) * 256, pd.data(), sizeof(PairDD) * kMaxPair, cudaMemcpyHostToDevice),
              "pair descriptors");
    // Tables worth staging in shared memory: the pair actions' spline tables, once each.
    stage_tables_.clear();
    for (int i = 0; i < sys.n_pair; ++i) {
        const bool bare = pd[i].kind == kPairBare, ilkka = pd[i].kind == kPairIlkka;
        const CubicDD* ts[3] = {&pd[i].v_long_r, &pd[i].v_r, &pd[i].u_long_r};
        const bool used[3] = {bare && pd[i].use_lr != 0, bare && pd[i].is_coulomb == 0, ilkka && pd[i].use_lr != 0};
        for (int j = 0; j < 3; ++j) {
            if (!used[j] || !ts[j]->x) continue;
            bool seen = false;
            for (auto& st : stage_tables_) seen |= (st.x == ts[j]->x);
            if (!seen) stage_tables_.push_back(StageTable{ts[j]->x, ts[j]->c, (uint32_t)ts[j]->n});
        }
    }
    // Double-float sampling/kinetic spline tables are built per move (they depend on n_images).
    sweep_tables_built_ = true;
}

// Double-float move descriptors of every move (sampling and kinetic tables per level, trap
// cofactors, pair indices) in the sweep's descriptor buffer, rebuilt when a level changes
// (adaptive bisection between blocks). Returns the buffer: [kMaxMoves] MoveDD, then the schedule
// and counters the sweep kernel uses.
void Context::PairGradDD(uint32_t pair, const double* pos, double* grad) {
    BuildSweepTables();
    const PairDD* pdd = reinterpret_cast<const PairDD*>(sweep_tables_->as<char>() + sizeof(float4) * 256);
    const PairDev& pa = sys.pair[pair];
    const uint64_t ng = (uint64_t)(pa.sa == pa.sb ? sys.sp_n[pa.sa] : sys.sp_n[pa.sa] + sys.sp_n[pa.sb]) * sys.M;
    const int th = 128;
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((ng + th - 1) / th, (uint64_t)n_sm * 32));
    PairGradDDKernel<<<blocks, th, 0, stream>>>(sys, pos, pdd, pair, grad);
    CudaCheck(cudaGetLastError(), "pair gradient launch");
}

void* Context::MoveDescriptors() {
    BuildSweepTables();
    for (size_t m = 0; m < moves.size(); ++m)
        if (moves[m].dev.n_kinetic > kMoveKinetic) throw PimcError(kErrUnsupported, "more than two kinetic actions on one species");
    std::vector<uint32_t> levels(moves.size());
    for (size_t m = 0; m < moves.size(); ++m) levels[m] = moves[m].dev.n_level;
    if (!sweep_desc_) sweep_desc_.reset(new DeviceBuffer(sizeof(MoveDD) * kMaxMoves + 4096 + 8192 + 2 * kMaxMoves * 8));
    MoveDD* dmoves = sweep_desc_->as<MoveDD>();
    if (levels != desc_levels_) {
        std::vector<MoveDD> md(kMaxMoves, MoveDD{});
        for (size_t m = 0; m < moves.size(); ++m) {
            const MoveDev& d = moves[m].dev;
            MoveDD& o = md[m];
            o.species = d.species;
            o.n_level = d.n_level;
            o.has_images = d.has_images;
            for (uint32_t l = 0; l < d.n_level; ++l) {
                Split(std::sqrt(d.lambda * (sys.tau * (1u << l))), o.sigma[l]);
                Split(d.i4lt_sample[l], o.i4s[l]);
                o.sample_image[l] = d.has_images ? MakeCubicDD(*this, d.sample_image[l], keep_) : CubicDD();
            }
            o.n_kin = d.n_kinetic;
            for (int i = 0; i < d.n_kinetic; ++i) {
                const KineticDev& k = sys.kinetic[d.kinetic[i]];
                o.kin_has_images[i] = k.has_images;
                for (uint32_t l = 0; l < d.n_level; ++l) {
                    if (k.image[l].n == 0) throw PimcError(kErrInput, "kinetic spline missing for a bisection level");
                    Split(k.i4lt_level[l], o.kin_i4[i][l]);
                    o.kin_image[i][l] = k.has_images ? MakeCubicDD(*this, k.image[l], keep_) : CubicDD();
                }
            }
            o.n_trap = d.n_trap;
            for (int i = 0; i < d.n_trap; ++i) {
                o.trap_max_level[i] = sys.trap[d.trap[i]].max_level;
                Split(sys.trap[d.trap[i]].cofactor_a, o.trap_cofa[i]);
            }
            o.n_pair = d.n_pair;
            for (int i = 0; i < d.n_pair; ++i) o.pair[i] = d.pair[i];
        }
        CudaCheck(cudaMemcpyAsync(dmoves, md.data(), sizeof(MoveDD) * kMaxMoves, cudaMemcpyHostToDevice, stream), "move descriptors");
        Sync();
        desc_levels_ = levels;
    }
    return sweep_desc_->ptr;
}

// Whether a Bisect move has pair terms above level 0: a pair action with max_level > 0 whose CalcU
// is non-zero there (pair_action_class.h:267-291), i.e. the table actions (Ilkka, David); the bare
// CalcU is zero above level 0, and Ewald parts above level 0 are refused (RequireLevelZeroDensities).
// The sweep kernel forms pair terms at level 0 only, so such moves run on the permutation kernel's
// plain variant.
bool Context::LevelPairTerms(uint32_t m) const {
    const MoveDev& d = moves[m].dev;
    if (moves[m].kind != 0 || d.n_level < 2) return false;
    for (int i = 0; i < d.n_pair; ++i) {
        const PairDev& p = sys.pair[d.pair[i]];
        if (p.max_level > 0 && !p.is_constant && p.kind != kPairBare) return true;
    }
    return false;
}

// A long-range pair action with max_level > 0 in a move of more than one level is refused. There the
// reference updates the densities once per attempt, at the first level that reaches the action and on
// that level's slices only, and then latches them (need_update_rho_k_, pair_action_class.h:293-298,
// species_class.h:406-425, marked FIXME). The densities then drift from the positions through the
// per-bead stores, which this layout does not keep.
void Context::RequireLevelZeroDensities(uint32_t m) const {
    const MoveDev& d = moves[m].dev;
    if (moves[m].kind == 1 || d.n_level < 2) return;
    for (int i = 0; i < d.n_pair; ++i) {
        const PairDev& p = sys.pair[d.pair[i]];
        if (p.use_long_range && p.max_level > 0 && !p.is_constant)
            throw PimcError(kErrUnsupported, "long-range pair action with max_level > 0 (the reference latches its densities above level 0)");
    }
}

// Every block arrives once at generation 1 of a fresh counter and waits for generation 2, which no
// block reaches: the wait ends only by its time limit (or the iteration cap) and sets the error word.
__global__ void WaitLimitKernel(unsigned long long* ctr, int* err, uint64_t timeout_ns, unsigned long long* waited) {
    const uint64_t t0 = GlobalTimerNs();
    GridBarrier(ctr, 2, err, timeout_ns);
    if (threadIdx.x == 0) atomicMax(waited, (unsigned long long)(GlobalTimerNs() - t0));
}

void Context::CheckWaitLimit(uint64_t timeout_ns, uint64_t* waited_ns) {
    if (timeout_ns > 10000000000ull) throw PimcError(kErrArg, "wait limit above 10 s");
    unsigned long long* w = reinterpret_cast<unsigned long long*>(Result());
    CudaCheck(cudaMemsetAsync(Barrier(), 0, sizeof(unsigned long long), stream), "reset barrier");
    CudaCheck(cudaMemsetAsync(w, 0, sizeof(unsigned long long), stream), "reset wait");
    WaitLimitKernel<<<2, 32, 0, stream>>>(Barrier(), ErrWord(), timeout_ns, w);
    CudaCheck(cudaGetLastError(), "wait-limit launch");
    unsigned long long h = 0;
    CudaCheck(cudaMemcpyAsync(&h, w, sizeof(h), cudaMemcpyDeviceToHost, stream), "read wait");
    Sync();
    if (waited_ns) *waited_ns = h;
    CheckDeviceError(false);
}

void Context::Sweep(const uint32_t* mv, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep) {
    if (n_entries == 0 || n_rep == 0) return;
    RequirePath();
    if (n_entries > 1024) throw PimcError(kErrArg, "schedule longer than 1024 entries");
    for (uint32_t e = 0; e < n_entries; ++e) {
        if (mv[e] >= moves.size()) throw PimcError(kErrArg, "move index out of range");
        RequireLevelZeroDensities(mv[e]);
    }
    bool own_launches = false;
    auto on_perm_kernel = [&](uint32_t m) {
        return moves[m].kind == 2 || moves[m].kind == 3 ||
               (moves[m].kind == 0 && (PermutingSpecies(moves[m].dev.species) || LevelPairTerms(m)));
    };
    for (uint32_t e = 0; e < n_entries; ++e) own_launches |= moves[mv[e]].kind == 1 || on_perm_kernel(mv[e]);
    bool all_perm = true;
    for (uint32_t e = 0; e < n_entries; ++e) all_perm &= on_perm_kernel(mv[e]);
    if (all_perm) {  // every entry on the permutation kernel: enqueue them all, wait once
        PermPrepare(mv, n_entries);
        try {
            for (uint64_t r = 0; r < n_rep; ++r)
                for (uint32_t e = 0; e < n_entries; ++e) PermEnqueue(mv[e], counts[e]);
        } catch (...) {
            PermFinish();
            throw;
        }
        PermFinish();
        return;
    }
    if (own_launches) {  // HMC and exchanging species run their own launches, entry by entry
        for (uint64_t r = 0; r < n_rep; ++r)
            for (uint32_t e = 0; e < n_entries; ++e) {
                if (moves[mv[e]].kind == 1) {
                    HmcAttempts(mv[e], counts[e]);
                } else if (on_perm_kernel(mv[e])) {
                    PermAttempts(mv[e], counts[e]);
                } else {
                    const uint64_t c1 = counts[e];
                    Sweep(&mv[e], &c1, 1, 1);
                }
            }
        return;
    }
    BuildSweepTables();
    uint32_t max_level = 1;
    for (size_t m = 0; m < moves.size(); ++m) {
        const MoveDev& d = moves[m].dev;
        if (d.n_level > 8) throw PimcError(kErrUnsupported, "bisection level above 8 in the sweep kernel");
        max_level = std::max(max_level, d.n_level);
    }
    for (uint32_t e = 0; e < n_entries; ++e)
        if (LevelPairTerms(mv[e])) throw PimcError(kErrState, "pair terms above level 0 in the sweep kernel");
    char* base = static_cast<char*>(MoveDescriptors());
    MoveDD* dmoves = reinterpret_cast<MoveDD*>(base);
    uint32_t* dsm = reinterpret_cast<uint32_t*>(base + sizeof(MoveDD) * kMaxMoves);
    uint64_t* dsc = reinterpret_cast<uint64_t*>(base + sizeof(MoveDD) * kMaxMoves + 4096);
    unsigned long long* dcount = reinterpret_cast<unsigned long long*>(base + sizeof(MoveDD) * kMaxMoves + 4096 + 8192);

    CudaCheck(cudaMemcpyAsync(dsm, mv, n_entries * 4, cudaMemcpyHostToDevice, stream), "schedule");
    CudaCheck(cudaMemcpyAsync(dsc, counts, n_entries * 8, cudaMemcpyHostToDevice, stream), "schedule");
    CudaCheck(cudaMemsetAsync(dcount, 0, 2 * kMaxMoves * 8, stream), "counters");
    EnsureDD();

    SweepArgs* args = new SweepArgs();
    std::unique_ptr<SweepArgs> guard(args);
    args->n_d = sys.n_d;
    args->M = sys.M;
    args->n_pad = sys.n_pad;
    args->K = sys.K;
    Split(sys.L, args->L);
    Split(sys.iL, args->iL);
    Split(sys.tau, args->tau);
    Split(2. * M_PI, args->two_pi);
    for (int s = 0; s < kMaxSpecies; ++s) {
        args->sp_off[s] = sys.sp_off[s];
        args->sp_n[s] = sys.sp_n[s];
    }
    for (int d = 0; d < 3; ++d) args->max_index[d] = sys.max_index[d];
    args->pos = pos_dd_->as<float2>();
    args->rho = precision == 32 ? nullptr : rho_dd_->as<float4>();
    args->rho32 = precision == 32 ? rho32_->as<float2>() : nullptr;
    args->kidx = sys.kidx;
    args->phase256 = sweep_tables_->as<float4>();
    args->moves = dmoves;
    args->pairs = reinterpret_cast<const PairDD*>(sweep_tables_->as<char>() + sizeof(float4) * 256);
    for (size_t m = 0; m < moves.size(); ++m) args->attempt_base[m] = moves[m].attempts;
    args->sched_move = dsm;
    args->sched_count = dsc;
    args->n_entries = n_entries;
    args->n_rep = n_rep;
    args->seed = seed;
    args->chain = chain;
    args->seg_cap = (1u << max_level) + 1;
    args->tab_stride = (uint32_t)std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;

    // Concurrent attempts need every scheduled move to have a grid phase (a non-constant pair
    // action) and segments of at most half the ring; otherwise one attempt at a time. Automatic:
    // three groups when an attempt's density work is small (66-electron gas, 16 slices x 3.6k
    // k-vectors: 9.1 us per attempt against 9.7 with two groups and 11.2 with one), one when it
    // fills the grid (1024 electrons, 16 x 25k: two and four groups were slower).
    uint32_t wave = sweep_wave > 0 ? (uint32_t)std::min(sweep_wave, (int)kWaveSlots)
                                   : ((uint64_t(1) << max_level) * sys.K <= (uint64_t(1) << 17) ? 3u : 1u);
    for (uint32_t e = 0; e < n_entries; ++e) {
        const MoveDev& d = moves[mv[e]].dev;
        bool gw = false;
        for (int i = 0; i < d.n_pair; ++i) gw |= !sys.pair[d.pair[i]].is_constant;
        if (!gw || (2u << d.n_level) > sys.M) wave = 1;
    }
    const int G0 = sweep_grid > 0 ? sweep_grid : n_sm;
    const uint32_t Gg = (uint32_t)G0 / wave;
    const int G = (int)(Gg * wave);
    if (Gg < max_level + 1) throw PimcError(kErrArg, "sweep grid (per concurrent attempt) smaller than the bisection level count");
    if (Gg + 32 > (uint32_t)kThreads) throw PimcError(kErrArg, "sweep grid per concurrent attempt above 480 blocks (one partial per thread)");
    uint32_t R = 1;
    while (R * 2 <= (1u << max_level) && R * 2 <= Gg) R *= 2;
    const uint32_t spc = std::max<uint32_t>(1, (1u << max_level) / R);
    if (spc > kMaxOwned) throw PimcError(kErrUnsupported, "too few blocks for the segment length");
    args->R = R;
    args->Q = std::max<uint32_t>(1, Gg / R);
    args->slices_per_cta = spc;
    args->wave = wave;
    args->group_ctas = Gg;
    {
        // The schedule flattened per repetition, for the rounds' attempt lookup.
        std::vector<uint64_t> pre(n_entries + 1, 0), before(n_entries, 0);
        std::vector<uint64_t> per_move(kMaxMoves, 0);
        for (uint32_t e = 0; e < n_entries; ++e) {
            pre[e + 1] = pre[e] + counts[e];
            before[e] = per_move[mv[e]];
            per_move[mv[e]] += counts[e];
        }
        args->per_rep = pre[n_entries];
        for (int m = 0; m < kMaxMoves; ++m) args->per_rep_move[m] = per_move[m];
        if (!sched_wave_) sched_wave_.reset(new DeviceBuffer(2 * 1025 * sizeof(uint64_t)));
        uint64_t* dw = sched_wave_->as<uint64_t>();
        CudaCheck(cudaMemcpyAsync(dw, pre.data(), pre.size() * 8, cudaMemcpyHostToDevice, stream), "schedule prefix");
        CudaCheck(cudaMemcpyAsync(dw + 1025, before.data(), before.size() * 8, cudaMemcpyHostToDevice, stream), "schedule prefix");
        args->sched_prefix = dw;
        args->move_before = dw + 1025;
    }
    // Shared layout: [move descriptors][pair descriptors][phase table][staged splines][work area].
    auto align16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    const size_t work0 = align16((size_t)2 * spc * 3 * args->tab_stride * sizeof(ddc) + (size_t)4 * 3 * args->seg_cap * sizeof(dd) +
                                 (size_t)3 * args->seg_cap * sizeof(float) + kMaxLevels * sizeof(float));
    // Density staging: the cells a thread evaluates in one attempt, for both species read (owned
    // slices per attempt at most spc + 1 when M is not a multiple of R, k-chunk ceil(K / Q)).
    {
        const uint32_t own_max = std::min<uint32_t>(kMaxOwned, sys.M % R == 0 ? spc : spc + 1);
        const uint64_t cells = (uint64_t)own_max * ((sys.K + args->Q - 1) / args->Q);
        const uint32_t cpt = sys.K && rho_slots ? (uint32_t)((cells + kThreads - 1) / kThreads) : 0u;
        const size_t bytes = (size_t)cpt * kThreads * 2 * (precision == 32 ? sizeof(float2) : sizeof(float4));
        args->rho_cpt = bytes <= (size_t)112 * 1024 ? cpt : 0u;  // larger k-chunks read global memory
    }
    const size_t rho_stage = (size_t)args->rho_cpt * kThreads * 2 * (precision == 32 ? sizeof(float2) : sizeof(float4));
    // The block's k-chunk of kidx and of every pair action's v_k, when some action has a long range.
    {
        bool any_long = false;
        for (int i = 0; i < sys.n_pair; ++i) any_long |= sys.pair[i].use_long_range && !sys.pair[i].is_constant;
        const uint32_t n_chunk = sys.K ? (uint32_t)((sys.K + args->Q - 1) / args->Q + 1) & ~1u : 0u;  // even: keeps v_k 8-byte aligned
        const size_t kbytes = (size_t)n_chunk * (sizeof(int32_t) + (size_t)sys.n_pair * (precision == 32 ? sizeof(float) : sizeof(float2)));
        args->kstage_n = (any_long && kbytes <= (size_t)64 * 1024 && work0 + rho_stage + align16(kbytes) <= (size_t)190 * 1024) ? n_chunk : 0u;
    }
    const size_t kstage = args->kstage_n ? align16((size_t)args->kstage_n * (sizeof(int32_t) + (size_t)sys.n_pair *
                                                                                (precision == 32 ? sizeof(float) : sizeof(float2))))
                                         : 0;
    const size_t work = work0 + rho_stage + kstage;
    size_t off = 0;
    args->n_moves = (uint32_t)moves.size();
    args->n_pairs = (uint32_t)sys.n_pair;
    args->off_moves = (uint32_t)off;
    off = align16(off + moves.size() * sizeof(MoveDD));
    args->off_pairs = (uint32_t)off;
    off = align16(off + (size_t)sys.n_pair * sizeof(PairDD));
    args->off_phase = (uint32_t)off;
    off += 256 * sizeof(float4);
    const size_t smem_cap = 200 * 1024;
    args->n_stage = 0;
    for (const auto& st : stage_tables_) {
        const size_t bx = align16((size_t)st.n * sizeof(float2)), bc = (size_t)2 * (st.n - 1) * sizeof(float4);
        if (off + bx + bc + work > smem_cap || args->n_stage >= (uint32_t)kMaxPair) continue;  // stays in global memory
        const uint32_t j = args->n_stage++;
        args->stage_x[j] = static_cast<const float2*>(st.x);
        args->stage_c[j] = static_cast<const float4*>(st.c);
        args->stage_n[j] = st.n;
        args->stage_off_x[j] = (uint32_t)off;
        args->stage_off_c[j] = (uint32_t)(off + bx);
        off = align16(off + bx + bc);
    }
    args->off_work = (uint32_t)off;
    args->off_rho_stage = (uint32_t)(off + work0);
    args->off_kstage = (uint32_t)(off + work0 + rho_stage);
    const size_t smem = off + work;
    const void* kfn = precision == 32 ? (const void*)BisectSweepKernel<true> : (const void*)BisectSweepKernel<false>;
    CudaCheck(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute");
    int occ = 0;
    CudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, kThreads, smem), "occupancy");
    if (occ < 1) throw PimcError(kErrCuda, "sweep kernel cannot be resident");
    if (G > occ * n_sm) throw PimcError(kErrArg, "sweep grid larger than the co-resident limit");
    args->counters = dcount;
    args->bar = Barrier();
    args->err = ErrWord();
    double* scratch = Partials((size_t)2 * G + 4 * kWaveSlots * kMaxLevels);
    args->partials = reinterpret_cast<float2*>(scratch);
    args->level_out = reinterpret_cast<float4*>(scratch + (size_t)2 * G);
    args->timeout_ns = timeout_ns;
    args->phase_cycles = nullptr;
    if (phase_timing) {
        if (!phase_buf) phase_buf.reset(new DeviceBuffer(kSweepTimingSlots * sizeof(unsigned long long)));
        args->phase_cycles = phase_buf->as<unsigned long long>();
    }
    if (precision == 32 && rho_slots && sys.K) {
        // FP32 densities rebuilt from the positions, which bounds the drift of their FP32 updates.
        std::vector<int> slot_species(rho_slots, 0);
        for (uint32_t sp = 0; sp < sys.S; ++sp)
            if (sys.sp_rho[sp] >= 0) slot_species[sys.sp_rho[sp]] = (int)sp;
        uint32_t* dss = Parts(rho_slots);
        CudaCheck(cudaMemcpyAsync(dss, slot_species.data(), rho_slots * sizeof(int), cudaMemcpyHostToDevice, stream), "slot upload");
        const size_t rsm = (size_t)kRho32Chunk * 3 * args->tab_stride * sizeof(float2);
        CudaCheck(cudaFuncSetAttribute(InitRho32Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm), "smem attribute");
        InitRho32Kernel<<<dim3((sys.K + 255) / 256, sys.M, rho_slots), 256, rsm, stream>>>(*args, reinterpret_cast<const int*>(dss));
        CudaCheck(cudaGetLastError(), "rho32 launch");
    }
    CudaCheck(cudaMemsetAsync(Barrier(), 0, sizeof(unsigned long long), stream), "reset barrier");
    void* kargs[] = {args};
    CudaCheck(cudaLaunchCooperativeKernel(kfn, dim3(G), dim3(kThreads), kargs, smem, stream), "sweep launch");
    fp64_valid = false;
    std::vector<unsigned long long> cnt(2 * kMaxMoves);
    CudaCheck(cudaMemcpyAsync(cnt.data(), dcount, 2 * kMaxMoves * 8, cudaMemcpyDeviceToHost, stream), "read counters");
    Sync();
    CheckDeviceError();
    std::vector<uint64_t> per_move(moves.size(), 0);
    for (uint32_t e = 0; e < n_entries; ++e) per_move[mv[e]] += counts[e];
    for (size_t m = 0; m < moves.size(); ++m) {
        const uint64_t n = per_move[m] * n_rep;
        moves[m].attempts += n;
        moves[m].block_attempt += n;
        moves[m].block_accept += cnt[m];
        moves[m].total_accept += cnt[m];
        moves[m].total_level0 += cnt[kMaxMoves + m];
    }
    last_grid_ = G;
}

// The dynamic shared memory limit of the permutation kernels: the device's opt-in maximum less
// their static part, set once per device to the same value from every context and thread (a
// per-launch value would race between host threads driving different contexts).
static int PermSmemOptin(int device) {
    int v = 0;
    CudaCheck(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "shared memory limit");
    cudaFuncAttributes fa, fb;
    CudaCheck(cudaFuncGetAttributes(&fa, PermBisectKernelDD), "perm kernel attributes");
    CudaCheck(cudaFuncGetAttributes(&fb, PermChainsKernelDD), "perm kernel attributes");
    v -= (int)std::max(fa.sharedSizeBytes, fb.sharedSizeBytes);
    CudaCheck(cudaFuncSetAttribute(PermBisectKernelDD, cudaFuncAttributeMaxDynamicSharedMemorySize, v), "perm smem attribute");
    CudaCheck(cudaFuncSetAttribute(PermChainsKernelDD, cudaFuncAttributeMaxDynamicSharedMemorySize, v), "perm smem attribute");
    return v;
}

// Attempts of a permuting move, or of the plain bisection of an exchanging species, on the
// double-float permutation kernel (perm_dd.cuh): one CTA runs them in order, in launches of at
// most 2048 attempts.
void Context::PermAttempts(uint32_t m, uint64_t n_att) {
    PermDensities();
    PermEnqueue(m, n_att);
    PermFinish();
}

// Launches the attempts on the context's stream without waiting; the move's counters accumulate
// on the device until PermFinish reads them.
void Context::PermEnqueue(uint32_t m, uint64_t n_att) {
    if (n_att == 0) return;
    PermArgsDD a;
    size_t smem = 0;
    PermArgs(m, &a, &smem);
    static int smem_optin[64] = {0};
    int& optin = smem_optin[device & 63];
    if (!optin) optin = PermSmemOptin(device);
    if (smem > (size_t)optin) throw PimcError(kErrUnsupported, "permutation kernel shared memory above the device limit");
    for (uint64_t done = 0; done < n_att;) {
        const uint32_t chunk = (uint32_t)std::min<uint64_t>(2048, n_att - done);
        a.attempt0 = moves[m].attempts + done;
        a.n_attempts = chunk;
        PermBisectKernelDD<<<1, kPermThreads, smem, stream>>>(a);
        CudaCheck(cudaGetLastError(), "permuting bisection launch");
        done += chunk;
    }
    moves[m].attempts += n_att;
    moves[m].block_attempt += n_att;
    perm_pending_ |= 1u << m;
    fp64_valid = false;
}

// The permutation kernel's arguments for move m (attempt0 / n_attempts left to the caller), with
// its scratch sized, and the dynamic shared memory a launch needs.
void Context::PermArgs(uint32_t m, void* out, size_t* smem_out) {
    PermArgsDD& a = *static_cast<PermArgsDD*>(out);
    MoveHost& mh = moves[m];
    const uint32_t sp = mh.dev.species, N = sys.sp_n[sp], M = sys.M;
    if (N > kPermMaxPart)
        throw PimcError(kErrUnsupported, "the permutation kernel (exchanges; pair terms above level 0) takes species of at most 512 particles");
    const uint32_t B = 1u << mh.dev.n_level;
    MoveDD* dmoves = static_cast<MoveDD*>(MoveDescriptors());
    EnsureDD();
    const size_t n_cycles = (size_t)mh.perm_n_comb * mh.perm_n_types, nc = std::max<size_t>(n_cycles, 1);
    auto ensure = [](std::unique_ptr<DeviceBuffer>& b, size_t bytes) {
        if (!b || b->bytes < bytes) b.reset(new DeviceBuffer(std::max<size_t>(bytes, 16)));
    };
    ensure(perm_t_, (size_t)N * N * sizeof(float2) * 3);  // [2][N][N] tables (when not shared) and the exponents
    ensure(perm_segold_, (size_t)N * (B + 1) * 3 * sizeof(float2));
    ensure(perm_cyc_, nc * (3 * sizeof(float2) + sizeof(uint32_t)));
    ensure(perm_prop_, (size_t)N * (B + 1) * 3 * sizeof(float2));
    ensure(perm_drho_, (size_t)(B + 1) * std::max<uint32_t>(sys.K, 1) * sizeof(float4));
    ensure(perm_hold_, (size_t)N * M * 3 * sizeof(float2));
    const size_t cnt_stride = 2 + 2 * (size_t)kPermMaxPart;
    if (!perm_cnt_) {
        perm_cnt_.reset(new DeviceBuffer(kMaxMoves * cnt_stride * sizeof(unsigned long long)));
        CudaCheck(cudaMemsetAsync(perm_cnt_->ptr, 0, perm_cnt_->bytes, stream), "perm counters");
    }
    a = PermArgsDD{};
    a.n_d = sys.n_d;
    a.M = M;
    a.n_pad = sys.n_pad;
    a.K = sys.K;
    Split(sys.L, a.L);
    Split(sys.iL, a.iL);
    Split(sys.tau, a.tau);
    Split(2. * M_PI, a.two_pi);
    Split(std::log(2.), a.ln2);
    Split(1. / (4. * mh.dev.lambda * sys.tau * B), a.i4B);  // i_4_lambda_tau_n_bisect_beads (bisect_class.h:182)
    Split(mh.perm_epsilon, a.eps);
    a.log_eps = (float)std::log(mh.perm_epsilon);
    for (int s = 0; s < kMaxSpecies; ++s) {
        a.sp_off[s] = sys.sp_off[s];
        a.sp_n[s] = sys.sp_n[s];
        a.sp_rho[s] = sys.sp_rho[s];
    }
    for (int d = 0; d < 3; ++d) a.max_index[d] = sys.max_index[d];
    a.pos = pos_dd_->as<float2>();
    a.rho = (rho_slots && sys.K && precision != 32) ? rho_dd_->as<float4>() : nullptr;
    a.rho32 = (rho_slots && sys.K && precision == 32) ? rho32_->as<float2>() : nullptr;
    a.kidx = sys.kidx;
    a.phase256 = sweep_tables_->as<float4>();
    a.mv = dmoves + m;
    a.pairs = reinterpret_cast<const PairDD*>(sweep_tables_->as<char>() + sizeof(float4) * 256);
    a.variant = mh.kind == 2 ? kPermVariantIterative : (mh.kind == 3 ? kPermVariantTable : kPermVariantBisect);
    a.seed = seed;
    a.chain = chain;
    a.move_index = m;
    a.k_part = mh.perm_k;
    a.n_comb = mh.perm_n_comb;
    a.n_types = mh.perm_n_types;
    a.combs = mh.perm_combs ? mh.perm_combs->as<uint32_t>() : nullptr;
    a.types = mh.perm_types ? mh.perm_types->as<uint32_t>() : nullptr;
    a.tg = perm_t_->as<float2>();
    a.ex = a.tg + (size_t)2 * N * N;
    a.seg_old_g = perm_segold_->as<float2>();
    a.cw = perm_cyc_->as<float2>();
    a.cwl = a.cw + nc;
    a.ccon = a.cwl + nc;
    a.cidx = reinterpret_cast<uint32_t*>(a.ccon + nc);
    a.prop = perm_prop_->as<float2>();
    a.drho = perm_drho_->as<float4>();
    a.hold = perm_hold_->as<float2>();
    a.perm = perm_->as<uint32_t>();
    a.perm_inv = perm_inv_->as<uint32_t>();
    a.counters = perm_cnt_->as<unsigned long long>() + m * cnt_stride;
    a.err = ErrWord();
    const size_t stride = (size_t)std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const uint32_t cyc_shared = (mh.kind == 3 && n_cycles <= kPermCycleCache) ? (uint32_t)n_cycles : 0u;
    *smem_out = PermLayout(N, cyc_shared, mh.kind == 2 && N <= kPermTabShared, (uint32_t)stride, PermSegCap(a.variant, N, a.k_part, B),
                           PermZCap(a.variant, N, a.k_part, B))
                    .total;
}

// FP32 mode: the FP32 per-slice densities formed from the positions before the permutation kernel
// runs, as every sweep-kernel call forms them (the kernel then updates them attempt by attempt).
void Context::PermDensities() {
    if (precision != 32 || !rho_slots || !sys.K) return;
    EnsureDD();
    BuildSweepTables();
    SweepArgs a{};
    a.n_d = sys.n_d;
    a.M = sys.M;
    a.n_pad = sys.n_pad;
    a.K = sys.K;
    Split(sys.iL, a.iL);
    for (int s = 0; s < kMaxSpecies; ++s) {
        a.sp_off[s] = sys.sp_off[s];
        a.sp_n[s] = sys.sp_n[s];
    }
    for (int d = 0; d < 3; ++d) a.max_index[d] = sys.max_index[d];
    a.pos = pos_dd_->as<float2>();
    a.rho32 = rho32_->as<float2>();
    a.kidx = sys.kidx;
    a.phase256 = sweep_tables_->as<float4>();
    a.tab_stride = (uint32_t)std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    std::vector<int> slot_species(rho_slots, 0);
    for (uint32_t sp = 0; sp < sys.S; ++sp)
        if (sys.sp_rho[sp] >= 0) slot_species[sys.sp_rho[sp]] = (int)sp;
    uint32_t* dss = Parts(rho_slots);
    CudaCheck(cudaMemcpyAsync(dss, slot_species.data(), rho_slots * sizeof(int), cudaMemcpyHostToDevice, stream), "slot upload");
    const size_t rsm = (size_t)kRho32Chunk * 3 * a.tab_stride * sizeof(float2);
    CudaCheck(cudaFuncSetAttribute(InitRho32Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm), "smem attribute");
    InitRho32Kernel<<<dim3((sys.K + 255) / 256, sys.M, rho_slots), 256, rsm, stream>>>(a, reinterpret_cast<const int*>(dss));
    CudaCheck(cudaGetLastError(), "rho32 launch");
}

// Sizes the permutation kernel's scratch for every move of a schedule before any launch (a later
// move's larger scratch must not replace buffers an earlier launch still uses).
void Context::PermPrepare(const uint32_t* mv, uint32_t n_entries) {
    PermDensities();
    for (uint32_t e = 0; e < n_entries; ++e) {
        PermArgsDD a;
        size_t smem;
        PermArgs(mv[e], &a, &smem);
    }
}

void SweepChains(const std::vector<Context*>& cs, const uint32_t* mv, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep) {
    if (cs.empty() || n_entries == 0 || n_rep == 0) return;
    bool all_perm = true;
    for (size_t i = 0; i < cs.size(); ++i)
        for (size_t j = 0; j < i; ++j)
            if (cs[i] == cs[j]) throw PimcError(kErrArg, "a chain appears twice");
    for (Context* c : cs) {
        if (c->device != cs[0]->device) throw PimcError(kErrArg, "chains on different devices");
        if (c->moves.size() != cs[0]->moves.size()) throw PimcError(kErrArg, "chains with different move lists");
        for (uint32_t e = 0; e < n_entries; ++e) {
            if (mv[e] >= c->moves.size()) throw PimcError(kErrArg, "move index out of range");
            c->RequireLevelZeroDensities(mv[e]);
            const MoveHost& mh = c->moves[mv[e]];
            // every bisection and permuting move fits the one-CTA kernel (its plain variant replays the
            // sweep kernel's draws, in either density precision); HMC and species above kPermMaxPart do not
            const uint32_t sp = mh.dev.species;
            all_perm &= (mh.kind == 0 || mh.kind == 2 || mh.kind == 3) && c->sys.sp_n[sp] <= kPermMaxPart;
            if (counts[e] > (1ull << 31)) throw PimcError(kErrArg, "more than 2^31 attempts in one schedule entry");
        }
    }
    if (!all_perm) {  // chains whose schedules use other kernels: one after another
        for (Context* c : cs) c->Sweep(mv, counts, n_entries, n_rep);
        return;
    }
    const size_t nc = cs.size();
    std::vector<PermArgsDD> args(nc * n_entries);
    std::vector<uint64_t> stride(nc * n_entries);
    size_t smem = 0;
    for (size_t ci = 0; ci < nc; ++ci) {
        Context& c = *cs[ci];
        c.PermFinish();
        c.PermPrepare(mv, n_entries);
        std::vector<uint64_t> per_rep(c.moves.size(), 0), before(c.moves.size(), 0);
        for (uint32_t e = 0; e < n_entries; ++e) per_rep[mv[e]] += counts[e];
        for (uint32_t e = 0; e < n_entries; ++e) {
            size_t sm = 0;
            PermArgsDD& a = args[ci * n_entries + e];
            c.PermArgs(mv[e], &a, &sm);
            smem = std::max(smem, sm);
            a.attempt0 = c.moves[mv[e]].attempts + before[mv[e]];
            a.n_attempts = (uint32_t)counts[e];
            before[mv[e]] += counts[e];
            stride[ci * n_entries + e] = per_rep[mv[e]];
        }
        c.Sync();  // the double-float copies each context prepared on its own stream
    }
    Context& c0 = *cs[0];
    static int smem_optin[64] = {0};
    int& optin = smem_optin[c0.device & 63];
    if (!optin) optin = PermSmemOptin(c0.device);
    if (smem > (size_t)optin) throw PimcError(kErrUnsupported, "permutation kernel shared memory above the device limit");
    DeviceBuffer dargs(args.size() * sizeof(PermArgsDD) + stride.size() * sizeof(uint64_t));
    // The counters change only once nothing can refuse the launch any more.
    for (Context* cp : cs) {
        for (uint32_t e = 0; e < n_entries; ++e) {
            MoveHost& mh = cp->moves[mv[e]];
            mh.attempts += counts[e] * n_rep;
            mh.block_attempt += counts[e] * n_rep;
            cp->perm_pending_ |= 1u << mv[e];
        }
        cp->fp64_valid = false;
    }
    CudaCheck(cudaMemcpyAsync(dargs.ptr, args.data(), args.size() * sizeof(PermArgsDD), cudaMemcpyHostToDevice, c0.stream), "chain arguments");
    uint64_t* dstride = reinterpret_cast<uint64_t*>(dargs.as<char>() + args.size() * sizeof(PermArgsDD));
    CudaCheck(cudaMemcpyAsync(dstride, stride.data(), stride.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, c0.stream), "chain arguments");
    PermChainsKernelDD<<<(unsigned)nc, kPermChainThreads, smem, c0.stream>>>(dargs.as<PermArgsDD>(), dstride, n_entries, n_rep);
    CudaCheck(cudaGetLastError(), "chains launch");
    c0.Sync();
    for (Context* c : cs) c->PermFinish();
}

// Waits for the enqueued permutation launches, folds their device counters into the moves'
// counters and refreshes the host copy of the path permutation.
void Context::PermFinish() {
    if (!perm_pending_) return;
    const size_t cnt_stride = 2 + 2 * (size_t)kPermMaxPart;
    std::vector<unsigned long long> cnt(kMaxMoves * cnt_stride);
    CudaCheck(cudaMemcpyAsync(cnt.data(), perm_cnt_->ptr, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream),
              "read perm counters");
    CudaCheck(cudaMemsetAsync(perm_cnt_->ptr, 0, perm_cnt_->bytes, stream), "perm counters");
    SyncPermHost();  // synchronises the stream
    const uint32_t pending = perm_pending_;
    perm_pending_ = 0;
    CheckDeviceError();
    for (uint32_t m = 0; m < moves.size(); ++m) {
        if (!(pending & (1u << m))) continue;
        MoveHost& mh = moves[m];
        const unsigned long long* c = cnt.data() + m * cnt_stride;
        const uint32_t N = sys.sp_n[mh.dev.species];
        mh.block_accept += c[0];
        mh.total_accept += c[0];
        mh.total_level0 += c[1];
        if (mh.kind == 2 || mh.kind == 3)
            for (uint32_t i = 0; i < N; ++i) {
                mh.perm_attempt[i] += c[2 + i];
                mh.perm_accept[i] += c[2 + N + i];
            }
    }
}

void Context::MoveAttempts(uint32_t m, uint64_t n) {
    const uint64_t one = n;
    Sweep(&m, &one, 1, 1);
}

// Bisect::Reset (bisect_class.h:142-155) and Move::Write/Reset (move_class.h:80-94); PathDump::Write
// (path_dump_class.h:28-66) on every skip-th call.
void Context::WriteBlock() {
    std::vector<double> host;
    for (size_t i = 0; i < observables.size(); ++i) {
        ObservableHost& o = observables[i];
        if (o.kind == 4) {
            if (o.n_write_calls % o.skip == 0) {
                if (host.empty()) {
                    host.resize((size_t)sys.n_total * sys.M * sys.n_d);
                    GetPath(0, host.data());  // [n_total][M][n_d]
                }
                for (uint32_t sp = 0; sp < sys.S; ++sp) {
                    // cube (n_d, n_bead, n_part) column-major: the same order as the host layout
                    const size_t n = (size_t)sys.sp_n[sp] * sys.M * sys.n_d, off = (size_t)sys.sp_off[sp] * sys.M * sys.n_d;
                    o.dumps[sp].emplace_back(host.begin() + off, host.begin() + off + n);
                    // (prev, next) particle of each path at the ring closure (path_dump_class.h:42-47)
                    std::vector<double> pm(2 * (size_t)sys.sp_n[sp]);
                    const uint32_t G0 = sys.sp_off[sp];
                    for (uint32_t p = 0; p < sys.sp_n[sp]; ++p) {
                        pm[2 * p + 1] = (double)(perm_host[G0 + p] - G0);
                        pm[2 * (perm_host[G0 + p] - G0)] = (double)p;
                    }
                    o.dump_perms[sp].push_back(pm);
                }
            }
            o.n_write_calls++;
            continue;
        }
        auto v = ObservableBlock((uint32_t)i);
        if (!v.empty()) blocks[i].push_back(v);
    }
    for (auto& mh : moves) {
        mh.out_attempt.push_back((double)mh.block_attempt);
        mh.out_accept.push_back((double)mh.block_accept);
        mh.out_ratio.push_back(mh.block_attempt ? (double)mh.block_accept / (double)mh.block_attempt : 0.);
        mh.out_level.push_back((double)mh.dev.n_level);
        mh.last_ratio = mh.block_attempt ? (double)mh.block_accept / (double)mh.block_attempt : 0.;
        if (!mh.first_block && mh.adaptive && mh.block_attempt > 0) {
            const double ratio = (double)mh.block_accept / (double)mh.block_attempt;
            if (ratio < mh.target_ratio && mh.dev.n_level > 1) mh.dev.n_level--;
            else if ((1u << mh.dev.n_level) < sys.M / 2) mh.dev.n_level++;
        }
        mh.first_block = false;
        mh.block_attempt = 0;
        mh.block_accept = 0;
        if (mh.kind == 2 || mh.kind == 3) {  // perm_bisect_class.h:119-132
            mh.out_perm_attempt.emplace_back(mh.perm_attempt.begin(), mh.perm_attempt.end());
            mh.out_perm_accept.emplace_back(mh.perm_accept.begin(), mh.perm_accept.end());
            std::fill(mh.perm_attempt.begin(), mh.perm_attempt.end(), 0);
            std::fill(mh.perm_accept.begin(), mh.perm_accept.end(), 0);
        }
    }
}

// Loop::DoEvent (loop_class.h:55-60). Consecutive move events run as one launch.
void Context::RunNode(const LoopNode& n) {
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
