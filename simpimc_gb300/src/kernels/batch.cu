// Batched independent chains: one thread block per chain, bisection sweeps and the thermal
// energy estimator for trapped / bare-Coulomb systems in FP32 with double-float sums.
//
// Algorithm per attempt (the reference's Bisect::Attempt, src/events/moves/single_species_move/
// bisect/bisect_class.h:39-124, with its actions Kinetic kinetic_class.h:105-122, HarmonicTrap
// trap_class.h:40-62 and BarePairAction bare_pair_action_class.h:133-149 / pair_action_class.h:
// 267-302): draw particle and first bead; resample the 2^l - 1 inner beads level by level from
// the free-particle distribution; at every level compare the level's action difference plus the
// sampling ratio (minus the previous level's action difference) with a log-uniform draw; accept
// the segment only if every level passes. The draws come from the same counter-based stream as
// the single-chain path, so a chain replays the FP64 path's Markov chain up to FP32 rounding.
//
// Work split inside a chain's warp group (G warps, T = 32 G lanes):
//   warp 0   draws the normals / uniforms, loads the moved particle's segment, samples the new
//            beads (lanes 0-2, one per dimension), evaluates the old-path sampling, kinetic and
//            trap sums (lanes 3-5), and takes every level decision;
//   all      evaluate the pair differences of the moved particle against the others on the
//            segment's inner slices (items (slice, other particle), coalesced float4 loads of the
//            other particles issued at the top of the attempt), reduce them in double-float.
// Pair terms are zero above level 0 (the primitive action's `1 >> level` factor,
// bare_pair_action_class.h:147), so upper levels are decided before the pair work and a rejection
// there skips it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <ctime>
#include <numeric>

#include <cooperative_groups.h>

#include "../../../include/simpimc_gb300.h"
#include "../common/philox.h"
#include "../framework/batch.h"
#include "../framework/input.h"
#include "../framework/table_io.h"
#include "df64.cuh"

namespace pimc {
namespace {

struct BatchArgs {
    float4* pos;
    const ChainDev* chains;
    const uint32_t* order;
    uint64_t* attempts;  // per chain: attempt counter of its Bisect move
    uint64_t* accepts;
    double* series;      // [chain][series_cap][kBatchSeriesComponents]
    uint64_t* n_meas;    // per chain
    double* last;        // [chain][kBatchSeriesComponents]: latest measurement
    int* err;
    uint64_t* rounds;    // per chain: scheduling rounds of the sweep kernel (one per attempt at wave 1)
    const uint2* cluster_tasks;  // sweep launched as clusters of two blocks: the chains of cluster j's
                                 // blocks (x == y: one chain split over both); null: block -> order[]
    uint32_t series_cap;
};

constexpr uint32_t kMaxB = 1u << kBatchMaxLevels;  // 32
constexpr uint32_t kPrefetch = 4;                  // pair items loaded ahead per lane

/// Barrier over the chain's warp group (named barrier 1; a warp-level barrier for one warp).
__device__ __forceinline__ void GroupSync(uint32_t n_warps) {
    if (n_warps == 1) __syncwarp();
    else asm volatile("bar.sync 1, %0;" ::"r"(n_warps * 32u) : "memory");
}

__device__ __forceinline__ float MinImg(float d, int pbc, float L, float iL) {
    return pbc ? __fsub_rn(d, __fmul_rn(L, rintf(__fmul_rn(d, iL)))) : d;
}

/// Exact i / d for i * d < 2^32 with m = ceil(2^32 / d) (d >= 2: for d = 1 the multiplier 2^32
/// has no 32-bit form; FastDivD handles both).
__device__ __forceinline__ uint32_t FastDiv(uint32_t i, uint32_t m) { return __umulhi(i, m); }
__device__ __forceinline__ uint32_t FastDivD(uint32_t i, uint32_t d, uint32_t m) { return d == 1u ? i : __umulhi(i, m); }

__device__ __forceinline__ dd AddSq(dd acc, float x) { return Add(acc, TwoProd(x, x)); }

__device__ __forceinline__ dd ShflDownDD(dd v, int o) {
    return dd{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

/// Butterfly reduction over the lanes whose xor distance is below 2^log2_width; every lane of a
/// group receives the same total (TwoSum and FP32 addition are commutative).
__device__ __forceinline__ Comp CompWarpSum(Comp v, int width) {
    for (int o = width >> 1; o > 0; o >>= 1) {
        const Comp w{__shfl_xor_sync(0xffffffffu, v.s, o), __shfl_xor_sync(0xffffffffu, v.c, o)};
        v = CompMerge(v, w);
    }
    return v;
}

__device__ __forceinline__ float Sq3(float x, float y, float z) { return __fmaf_rn(x, x, __fmaf_rn(y, y, __fmul_rn(z, z))); }

__device__ __forceinline__ uint32_t Wrap(uint32_t s, uint32_t M) { return s >= M ? s - M : s; }  // s < 2M

template <bool kPbc>
__device__ __forceinline__ float Img(float d, float L, float iL) {
    if constexpr (kPbc) return __fsub_rn(d, __fmul_rn(L, rintf(__fmul_rn(d, iL))));
    else return d;
}

// Paired FP32 arithmetic (sub/mul/fma.rn.f32x2): each half rounds as the scalar operation does,
// so a pair of (old, new) terms costs one instruction and keeps the scalar results.
__device__ __forceinline__ unsigned long long Pk2(float2 v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
__device__ __forceinline__ float2 Un2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ float2 Sub2(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(Pk2(a)), "l"(Pk2(b)));
    return Un2(r);
}
__device__ __forceinline__ float2 Mul2(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(Pk2(a)), "l"(Pk2(b)));
    return Un2(r);
}
__device__ __forceinline__ float2 Fma2(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(Pk2(a)), "l"(Pk2(b)), "l"(Pk2(c)));
    return Un2(r);
}
/// Img on both halves: d - L rint(d / L) with the scalar version's roundings.
template <bool kPbc>
__device__ __forceinline__ float2 Img2(float2 d, float L, float iL) {
    if constexpr (kPbc) {
        const float2 t = Mul2(d, make_float2(iL, iL));
        return Sub2(d, Mul2(make_float2(L, L), make_float2(rintf(t.x), rintf(t.y))));
    } else {
        return d;
    }
}
__device__ __forceinline__ float2 Sq3x2(float2 x, float2 y, float2 z) { return Fma2(x, x, Fma2(y, y, Mul2(z, z))); }

constexpr uint32_t kItems = 4;  // pair items per lane kept in registers (more are loaded in the loop)

/// A chain's beads during a sweep: the global float4 block [M][n_pad] (slice-major, x y z 0), or,
/// when kStaged, three coordinate planes [M][N] in shared memory filled at the start of the
/// launch and written back at its end.
template <bool kStaged>
struct PathView {
    float4* g;
    float* s;
    uint32_t n_pad, n, plane;
    __device__ __forceinline__ float3 Load(uint32_t b, uint32_t q) const {
        if constexpr (kStaged) {
            const uint32_t i = b * n + q;
            return make_float3(s[i], s[plane + i], s[2 * plane + i]);
        } else {
            const float4 v = g[(size_t)b * n_pad + q];
            return make_float3(v.x, v.y, v.z);
        }
    }
    __device__ __forceinline__ void Store(uint32_t b, uint32_t q, float x, float y, float z) const {
        if constexpr (kStaged) {
            const uint32_t i = b * n + q;
            s[i] = x;
            s[plane + i] = y;
            s[2 * plane + i] = z;
        } else {
            g[(size_t)b * n_pad + q] = make_float4(x, y, z, 0.f);
        }
    }
};

/// Draws of one attempt (particle, first bead, normals, log-uniforms; philox.h stream layout) into
/// shared buffers, by one warp; with `seg` also the moved particle's segment as it is now.
__device__ __forceinline__ uint2 DrawAttempt(const MoveStream& st, uint32_t lane, uint32_t N, uint32_t M, uint32_t B, uint32_t NL, uint32_t n_pad,
                                             const float4* __restrict__ pos, float* z, float* logu, float4* seg, uint32_t* pb) {
    const Philox4 w0 = st.Block(0);
    const uint32_t p = UniformIndex(w0.v[0], N), b0 = UniformIndex(w0.v[1], M);
    if (seg) {
        if (lane <= B) seg[lane] = pos[(size_t)Wrap(b0 + lane, M) * n_pad + p];
        if (B == 32 && lane == 0) seg[32] = pos[(size_t)Wrap(b0 + 32u, M) * n_pad + p];
    }
    if (lane == 0) {
        pb[0] = p;
        pb[1] = b0;
    }
    // Two lanes per resampled bead (BisectNormals' two Box-Muller transforms of its Philox block:
    // z0, z1 from words 0-1 on the even lane, z2 from words 2-3 on the odd one), one per level's
    // log-uniform: the draw's latency is one transform's.
    for (uint32_t j = lane; j < 2 * (B - 1) + NL; j += 32) {
        if (j < 2 * (B - 1)) {
            const uint32_t i = j >> 1;
            const Philox4 w = st.Block(1u + i);
            float z0, z1;
            if ((j & 1u) == 0) {
                BoxMullerF(w.v[0], w.v[1], z0, z1);
                z[3 * i] = z0;
                z[3 * i + 1] = z1;
            } else {
                BoxMullerF(w.v[2], w.v[3], z0, z1);
                z[3 * i + 2] = z0;
            }
        } else {
            const uint32_t li = j - 2 * (B - 1);  // 0 = top level
            logu[NL - 1 - li] = BisectLogU(st, B, li);
        }
    }
    return make_uint2(p, b0);
}

/// Warp work of one attempt (bisect_class.h:39-124 above level 0): lane k enters with bead k of
/// the old segment (every lane also holds the last bead B in e*), samples the new beads level by
/// level in registers (bead k = 2^l (2m + 1) from beads k -+ 2^l by shuffles), writes both segment
/// copies for the pair work, forms each level's sampling, kinetic and trap terms (the link's far
/// bead from those copies), reduces them with compensated butterflies over the B lanes that hold
/// terms (all levels in step, so their latencies overlap), and tests every level above 0, lane l
/// deciding level l. Returns with the new bead in n*.
template <bool kPbc, uint32_t NL>
__device__ __forceinline__ void LeaderPhaseL(const ChainDev& c, uint32_t lane, uint32_t M, float ox, float oy, float oz, float ex, float ey,
                                             float ez, const float* zb, const float* logu, float2* s_on, dd* base0_out,
                                             int* upper_out, float& nx, float& ny, float& nz, bool& upper_reg, dd& base0_reg) {
    constexpr uint32_t B = 1u << NL;
    const float L = c.L, iL = c.iL;
    const bool kin_links = B != M;  // whole-ring segment: no kinetic links (kinetic_class.h:111-117)
    const bool inner = lane >= 1 && lane < B;
    const uint32_t lk = lane == 0 ? 31u : (uint32_t)(__ffs(lane) - 1);  // level of bead `lane`
    // An inner bead is drawn once, on its own level: its scaled normal displacement.
    float gx = 0.f, gy = 0.f, gz = 0.f;
    if (inner) {
        const uint32_t zi = 3 * ((B >> (lk + 1)) - 1u + (lane >> (lk + 1)));
        const float sg = c.sigma[lk];
        gx = Img<kPbc>(__fmul_rn(sg, zb[zi]), L, iL);
        gy = Img<kPbc>(__fmul_rn(sg, zb[zi + 1]), L, iL);
        gz = Img<kPbc>(__fmul_rn(sg, zb[zi + 2]), L, iL);
    }
    nx = ox;
    ny = oy;
    nz = oz;
#pragma unroll
    for (int li = (int)NL - 1; li >= 0; --li) {
        const uint32_t skip = 1u << li;
        const bool mine = inner && lk == (uint32_t)li;
        const uint32_t sa = mine ? lane - skip : lane, sc = mine ? lane + skip : lane;
        const float ax = __shfl_sync(0xffffffffu, nx, sa & 31u), ay = __shfl_sync(0xffffffffu, ny, sa & 31u),
                    az = __shfl_sync(0xffffffffu, nz, sa & 31u);
        float cx = __shfl_sync(0xffffffffu, nx, sc & 31u), cy = __shfl_sync(0xffffffffu, ny, sc & 31u),
              cz = __shfl_sync(0xffffffffu, nz, sc & 31u);
        if (sc == 32u) {
            cx = ex;
            cy = ey;
            cz = ez;
        }
        if (mine) {
            nx = __fadd_rn(__fadd_rn(ax, __fmul_rn(0.5f, Img<kPbc>(__fsub_rn(cx, ax), L, iL))), gx);
            ny = __fadd_rn(__fadd_rn(ay, __fmul_rn(0.5f, Img<kPbc>(__fsub_rn(cy, ay), L, iL))), gy);
            nz = __fadd_rn(__fadd_rn(az, __fmul_rn(0.5f, Img<kPbc>(__fsub_rn(cz, az), L, iL))), gz);
        }
    }
    const float dn2 = inner ? Sq3(gx, gy, gz) : 0.f;
    // Segment copies for the pair work and for the links below (bead 32 of a 32-bead segment is e).
    if (lane <= B) {
        s_on[3 * lane] = make_float2(ox, nx);
        s_on[3 * lane + 1] = make_float2(oy, ny);
        s_on[3 * lane + 2] = make_float2(oz, nz);
    }
    if (B == 32 && lane == 0) {
        s_on[96] = make_float2(ex, ex);
        s_on[97] = make_float2(ey, ey);
        s_on[98] = make_float2(ez, ez);
    }
    // Old sampling displacement of bead `lane` on its level.
    float samp = 0.f;
    {
        const uint32_t skip = inner ? (1u << lk) : 0u;
        const uint32_t sa = inner ? lane - skip : lane, sc = inner ? lane + skip : lane;
        const float ax = __shfl_sync(0xffffffffu, ox, sa & 31u), ay = __shfl_sync(0xffffffffu, oy, sa & 31u),
                    az = __shfl_sync(0xffffffffu, oz, sa & 31u);
        float cx = __shfl_sync(0xffffffffu, ox, sc & 31u), cy = __shfl_sync(0xffffffffu, oy, sc & 31u),
              cz = __shfl_sync(0xffffffffu, oz, sc & 31u);
        if (sc == 32u) {
            cx = ex;
            cy = ey;
            cz = ez;
        }
        if (inner) {
            const float bx = __fadd_rn(ax, __fmul_rn(0.5f, Img<kPbc>(__fsub_rn(cx, ax), L, iL)));
            const float by = __fadd_rn(ay, __fmul_rn(0.5f, Img<kPbc>(__fsub_rn(cy, ay), L, iL)));
            const float bz = __fadd_rn(az, __fmul_rn(0.5f, Img<kPbc>(__fsub_rn(cz, az), L, iL)));
            const float do2 = Sq3(Img<kPbc>(__fsub_rn(ox, bx), L, iL), Img<kPbc>(__fsub_rn(oy, by), L, iL), Img<kPbc>(__fsub_rn(oz, bz), L, iL));
            samp = __fmul_rn(c.i4lt_sample[lk], __fsub_rn(dn2, do2));  // log sample ratio term
        }
    }
    __syncwarp();
    // Per level l and lane k (a multiple of 2^l): the action change of link k -> k + 2^l
    // (kinetic) and slice k (trap); the level's totals come from one compensated butterfly each
    // for  D_l = sum of action changes  and  R_l = sampling ratio - D_l.
    Comp Dl[NL + 1], Rl[NL];
    Dl[NL] = Comp{0.f, 0.f};
    const float2 t2 = Sq3x2(make_float2(ox, nx), make_float2(oy, ny), make_float2(oz, nz));  // |r|^2 old, new
#pragma unroll
    for (uint32_t li = 0; li < NL; ++li) {
        float dterm = 0.f;
        const uint32_t skip = 1u << li;
        if (lane < B && (lane & (skip - 1u)) == 0u) {
            const float2* cf = s_on + 3 * (lane + skip);  // far bead of the link, (old, new)
            if (kin_links) {
                const float2 k2 = Sq3x2(Img2<kPbc>(Sub2(make_float2(ox, nx), cf[0]), L, iL), Img2<kPbc>(Sub2(make_float2(oy, ny), cf[1]), L, iL),
                                        Img2<kPbc>(Sub2(make_float2(oz, nz), cf[2]), L, iL));
                dterm = __fmul_rn(c.i4lt_level[li], __fsub_rn(k2.y, k2.x));
            }
            if (c.has_trap && (int)li <= c.trap_max_level)
                dterm = __fadd_rn(dterm, __fmul_rn(__fmul_rn(c.trap_cofa, (float)skip), __fsub_rn(t2.y, t2.x)));
        }
        Dl[li] = Comp{dterm, 0.f};
        Rl[li] = Comp{__fsub_rn(inner && lk == li ? samp : 0.f, dterm), 0.f};
    }
    // Every term sits on a lane below B, so a butterfly over B lanes gives those lanes the totals
    // (the wider one would only merge zeros, which leave a compensated pair unchanged).
#pragma unroll
    for (uint32_t o = B >> 1; o > 0; o >>= 1) {
#pragma unroll
        for (uint32_t li = 0; li < NL; ++li) {
            const Comp dw{__shfl_xor_sync(0xffffffffu, Dl[li].s, o), __shfl_xor_sync(0xffffffffu, Dl[li].c, o)};
            const Comp rw{__shfl_xor_sync(0xffffffffu, Rl[li].s, o), __shfl_xor_sync(0xffffffffu, Rl[li].c, o)};
            Dl[li] = CompMerge(Dl[li], dw);
            Rl[li] = CompMerge(Rl[li], rw);
        }
    }
    // Level l passes if  R_l + D_{l+1} >= log u_l  (bisect_class.h:110-121); lane l tests level l
    // and lane 0 keeps level 0's value for the pair test.
    Comp rs = Rl[0], dn = Dl[1];
#pragma unroll
    for (uint32_t li = 1; li < NL; ++li)
        if (lane == li) {
            rs = Rl[li];
            dn = Dl[li + 1];
        }
    dd la = CompDD(rs);
    if (lane + 1 < NL) la = Add(la, CompDD(dn));
    if (!isfinite(la.hi)) la.hi = -INFINITY;
    const bool fail = lane >= 1 && lane < NL && Less(la, DD(logu[lane]));
    const unsigned fails = __ballot_sync(0xffffffffu, fail);
    // The leader warp keeps both results in registers (lane 0's base0 is level 0's); the shared
    // copies serve the group's other warps.
    upper_reg = fails == 0u;
    base0_reg = la;
    if (lane == 0) {
        *upper_out = fails == 0u;
        *base0_out = la;
    }
}

template <bool kPbc>
__device__ __forceinline__ void LeaderPhase(const ChainDev& c, uint32_t lane, uint32_t NL, uint32_t M, float ox, float oy, float oz, float ex,
                                            float ey, float ez, const float* zb, const float* logu, float2* s_on, dd* base0_out,
                                            int* upper_out, float& nx, float& ny, float& nz, bool& upper_reg, dd& base0_reg) {
    switch (NL) {
        case 1: LeaderPhaseL<kPbc, 1>(c, lane, M, ox, oy, oz, ex, ey, ez, zb, logu, s_on, base0_out, upper_out, nx, ny, nz, upper_reg, base0_reg); break;
        case 2: LeaderPhaseL<kPbc, 2>(c, lane, M, ox, oy, oz, ex, ey, ez, zb, logu, s_on, base0_out, upper_out, nx, ny, nz, upper_reg, base0_reg); break;
        case 3: LeaderPhaseL<kPbc, 3>(c, lane, M, ox, oy, oz, ex, ey, ez, zb, logu, s_on, base0_out, upper_out, nx, ny, nz, upper_reg, base0_reg); break;
        case 4: LeaderPhaseL<kPbc, 4>(c, lane, M, ox, oy, oz, ex, ey, ez, zb, logu, s_on, base0_out, upper_out, nx, ny, nz, upper_reg, base0_reg); break;
        default: LeaderPhaseL<kPbc, 5>(c, lane, M, ox, oy, oz, ex, ey, ez, zb, logu, s_on, base0_out, upper_out, nx, ny, nz, upper_reg, base0_reg); break;
    }
}

/// Pair items of one attempt: (inner slice k in 1..B-1) x (other particle q), item i -> k = i /
/// (N-1); this lane's first kItems items (attempt-independent decomposition in it_k / it_q,
/// beads already in pre[]) and any further ones at stride T. Returns the lane's compensated sum
/// of 1/r_new - 1/r_old (clamped to the table's grid).
template <bool kPbc, bool kStaged>
__device__ __forceinline__ Comp PairPhase(const ChainDev& c, uint32_t t, uint32_t T, uint32_t n_items, uint32_t magic, uint32_t nm1, uint32_t p,
                                          uint32_t b0, uint32_t M, const PathView<kStaged>& path, const uint32_t* it_k, const float3* pre,
                                          const float2* s_on, uint32_t partner_major_nk) {
    const float L = c.L, iL = c.iL, r2_min = c.r2_min, r2_max = c.r2_max;
    Comp acc_u{0.f, 0.f};
    auto item = [&](uint32_t k, float3 rq) {
        const float2* on = s_on + 3 * (k + 1);  // inner bead k + 1, (old, new)
        const float2 r2 = Sq3x2(Img2<kPbc>(Sub2(on[0], make_float2(rq.x, rq.x)), L, iL), Img2<kPbc>(Sub2(on[1], make_float2(rq.y, rq.y)), L, iL),
                                Img2<kPbc>(Sub2(on[2], make_float2(rq.z, rq.z)), L, iL));
        const float r2o = fminf(fmaxf(r2.x, r2_min), r2_max);
        const float r2n = fminf(fmaxf(r2.y, r2_min), r2_max);
        CompAdd(acc_u, __fsub_rn(rsqrtf(r2n), rsqrtf(r2o)));
    };
    if constexpr (kStaged) {  // beads in shared memory: no prefetch, loads batched by the unrolled loop
        const uint32_t nk = partner_major_nk;  // inner slices (0: items flattened)
        if (nk) {
            // lane = partner particle, inner slices in a loop: no index division per item
            for (uint32_t qi = t; qi < nm1; qi += T) {
                const uint32_t q = qi + (qi >= p ? 1u : 0u);
                uint32_t b = Wrap(b0 + 1u, M);
#pragma unroll 4
                for (uint32_t k = 0; k < nk; ++k) {
                    item(k, path.Load(b, q));
                    b = b + 1u == M ? 0u : b + 1u;
                }
            }
        } else {
#pragma unroll 4
            for (uint32_t i = t; i < n_items; i += T) {
                const uint32_t k = FastDivD(i, nm1, magic), qq = i - k * nm1;
                item(k, path.Load(Wrap(b0 + 1u + k, M), qq + (qq >= p ? 1u : 0u)));
            }
        }
    } else {
#pragma unroll
        for (uint32_t j = 0; j < kItems; ++j)
            if (t + j * T < n_items) item(it_k[j], pre[j]);
        for (uint32_t i = t + kItems * T; i < n_items; i += T) {
            const uint32_t k = FastDivD(i, nm1, magic), qq = i - k * nm1;
            item(k, path.Load(Wrap(b0 + 1u + k, M), qq + (qq >= p ? 1u : 0u)));
        }
    }
    return acc_u;
}

/// Level-0 test: pair action difference tau * sum (1/r_new - 1/r_old) over inner slices (each
/// inner slice closes two links with weight 1/2; the segment ends cancel) joins the level's
/// double-float total. Lane 0 decides (the G warp partials merged over the smallest power-of-two
/// lane group that holds them) and every lane of the calling warp gets its answer.
__device__ __forceinline__ bool Level0Accepts(const ChainDev& c, uint32_t lane, uint32_t G, const Comp* part, bool has_items, dd base0, float logu0) {
    dd u = DD(0.f);
    if (has_items) {
        int width = 1;
        while (width < (int)G) width <<= 1;
        u = CompDD(CompWarpSum(lane < G ? part[lane] : Comp{0.f, 0.f}, width));
    }
    dd la0 = Sub(base0, MulF(u, c.tau));
    if (!isfinite(la0.hi)) la0.hi = -INFINITY;
    return __shfl_sync(0xffffffffu, (int)!Less(la0, DD(logu0)), 0) != 0;
}

struct SweepShared {
    ChainDev c;
    float z[2][3 * (kMaxB - 1)];
    float logu[2][kBatchMaxLevels];
    float4 seg[2][kMaxB + 1];
    uint32_t pb[2][2];
    float2 on_[3 * (kMaxB + 1)];  // the attempt's segment, (old, new) per coordinate
    Comp part[kBatchMaxWarps];
    dd base0;  // level-0 log acceptance without the pair term
    int upper_ok;
};

/// One attempt at a time (warp 0 leads; warp 1 draws the next attempt and loads its segment,
/// which is patched from warp 0's registers when both attempts move the same particle).
template <bool kPbc>
__device__ __forceinline__ void SweepChain(SweepShared& sh, BatchArgs a, uint32_t ci, uint32_t G, uint64_t n_sweeps, uint64_t n_attempts) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t T = G * 32u, t = threadIdx.x;
    const ChainDev& c = sh.c;
    const uint32_t N = c.n_part, M = c.n_bead, NL = c.n_level, B = 1u << NL, n_pad = c.n_pad;
    float4* __restrict__ pos = a.pos + c.pos_off;
    const PathView<false> gpath{pos, nullptr, n_pad, N, 0u};

    const uint32_t nm1 = N > 1 ? N - 1 : 1;
    const uint32_t n_items = c.has_pair && N > 1 ? (N - 1) * (B - 1) : 0u;
    const uint32_t magic = (uint32_t)((0x100000000ull + nm1 - 1) / nm1);
    uint32_t it_k[kItems], it_q[kItems];
#pragma unroll
    for (uint32_t j = 0; j < kItems; ++j) {
        const uint32_t i = t + j * T;
        it_k[j] = FastDivD(i, nm1, magic);
        it_q[j] = i - it_k[j] * nm1;
    }

    uint64_t att = a.attempts[ci], acc = a.accepts[ci];
    const uint64_t n_att = n_sweeps ? n_sweeps * c.attempts_per_sweep : n_attempts;
    const bool ahead = G >= 2;
    if (ahead && warp == 1 && n_att > 0)
        DrawAttempt(MoveStream{c.seed, c.chain_id, c.move, att}, lane, N, M, B, NL, n_pad, pos, sh.z[att & 1], sh.logu[att & 1], sh.seg[att & 1],
                    sh.pb[att & 1]);
    GroupSync(G);

    float nx = 0.f, ny = 0.f, nz = 0.f;  // warp 0, lane k: new position of bead k of the last attempt
    bool lead_upper = false;             // warp 0: the upper levels passed (and lane 0's level-0 base)
    dd lead_base0 = DD(0.f);
    uint32_t p_prev = 0xffffffffu, b0_prev = 0;
    bool acc_prev = false;
    for (uint64_t it = 0; it < n_att; ++it, ++att) {
        const uint32_t buf = (uint32_t)(att & 1);
        if (!ahead) {
            DrawAttempt(MoveStream{c.seed, c.chain_id, c.move, att}, lane, N, M, B, NL, n_pad, pos, sh.z[buf], sh.logu[buf], sh.seg[buf], sh.pb[buf]);
            __syncwarp();
        }
        const uint32_t p = sh.pb[buf][0], b0 = sh.pb[buf][1];

        float3 pre[kItems];
#pragma unroll
        for (uint32_t j = 0; j < kItems; ++j)
            if (t + j * T < n_items) pre[j] = gpath.Load(Wrap(b0 + 1u + it_k[j], M), it_q[j] + (it_q[j] >= p ? 1u : 0u));

        if (warp == 0) {
            const float4 sv = sh.seg[buf][lane <= B ? lane : B];
            const float4 se = sh.seg[buf][B];
            float ox = sv.x, oy = sv.y, oz = sv.z, ex = se.x, ey = se.y, ez = se.z;
            if (ahead && acc_prev && p == p_prev) {
                // Beads of this segment inside the last accepted segment: take the committed values.
                const uint32_t off = Wrap(Wrap(b0 + (lane <= B ? lane : B), M) + M - b0_prev, M);
                const uint32_t off_e = Wrap(Wrap(b0 + B, M) + M - b0_prev, M);
                const bool in = off >= 1 && off < B, in_e = off_e >= 1 && off_e < B;
                const float px = __shfl_sync(0xffffffffu, nx, in ? off : 0), py = __shfl_sync(0xffffffffu, ny, in ? off : 0),
                            pz = __shfl_sync(0xffffffffu, nz, in ? off : 0);
                const float qx = __shfl_sync(0xffffffffu, nx, in_e ? off_e : 0), qy = __shfl_sync(0xffffffffu, ny, in_e ? off_e : 0),
                            qz = __shfl_sync(0xffffffffu, nz, in_e ? off_e : 0);
                if (in) {
                    ox = px;
                    oy = py;
                    oz = pz;
                }
                if (in_e) {
                    ex = qx;
                    ey = qy;
                    ez = qz;
                }
            }
            LeaderPhase<kPbc>(c, lane, NL, M, ox, oy, oz, ex, ey, ez, sh.z[buf], sh.logu[buf], sh.on_, &sh.base0, &sh.upper_ok,
                              nx, ny, nz, lead_upper, lead_base0);
        } else if (ahead && warp == 1 && it + 1 < n_att) {
            DrawAttempt(MoveStream{c.seed, c.chain_id, c.move, att + 1}, lane, N, M, B, NL, n_pad, pos, sh.z[buf ^ 1u], sh.logu[buf ^ 1u],
                        sh.seg[buf ^ 1u], sh.pb[buf ^ 1u]);
        }
        GroupSync(G);
        const bool upper_ok = warp == 0 ? lead_upper : sh.upper_ok != 0;

        if (upper_ok && n_items) {
            const Comp u = CompWarpSum(PairPhase<kPbc, false>(c, t, T, n_items, magic, nm1, p, b0, M, gpath, it_k, pre, sh.on_, 0u), 32);
            if (lane == 0) sh.part[warp] = u;
        }
        GroupSync(G);

        if (warp == 0) {
            const bool accepted = upper_ok && Level0Accepts(c, lane, G, sh.part, n_items != 0, lead_base0, sh.logu[buf][0]);
            if (accepted && lane >= 1 && lane < B) pos[(size_t)Wrap(b0 + lane, M) * n_pad + p] = make_float4(nx, ny, nz, 0.f);
            acc += accepted ? 1u : 0u;
            acc_prev = accepted;
            p_prev = p;
            b0_prev = b0;
        }
        GroupSync(G);
    }
    if (t == 0) {
        a.rounds[ci] += att - a.attempts[ci];
        a.attempts[ci] = att;
        a.accepts[ci] = acc;
    }
}

// ---------------------------------------------------------------------------------------------
// Several attempts of one chain at a time. Two attempts commute when neither reads what the other
// writes: different particles whose inner slices are disjoint (an attempt's pair terms read the
// other particles only at its inner slices), or the same particle with each attempt's whole
// segment clear of the other's inner slices. A scoreboard keeps the next kWindow drawn attempts;
// each carries a mask of the attempts before it (up to kWindow - 1 back) that it does not commute
// with. A round runs the first W attempts of the window, in attempt order, that commute with every
// earlier attempt not yet run, one per sub-group of warps; they commit disjoint beads. Every
// attempt therefore reads what it reads in the sequential chain, and the result is the sequential
// chain's: the same accept decisions and the same path.

constexpr uint32_t kWindow = 32;          // attempts the scheduler considers per round (one lane each)
constexpr uint32_t kRing = 2 * kWindow;   // drawn attempts, slot = attempt mod kRing
static_assert((kRing & (kRing - 1)) == 0, "the drawn-attempt ring is indexed by a mask");
static_assert(kMaxWave <= kWindow && kWindow <= 32, "a round's attempts come from the window; one lane per window entry");

/// A ring slot's normals (3 (B - 1) floats) and log-uniforms (n_level floats) live in dynamic
/// shared memory after the staged path.
__host__ __device__ constexpr size_t RingBytes(uint32_t B, uint32_t n_level) { return (size_t)kRing * (3 * (B - 1) + n_level) * sizeof(float); }

struct WaveRing {
    float* z;   // [kRing][3 (B - 1)]
    float* lu;  // [kRing][n_level]
    uint32_t zs, ls;
    __device__ __forceinline__ float* Z(uint32_t slot) const { return z + slot * zs; }
    __device__ __forceinline__ float* LU(uint32_t slot) const { return lu + slot * ls; }
};

struct WaveShared {
    ChainDev c;
    uint32_t pb[kRing][2];
    uint32_t dep[kRing];  // bit d: the attempt does not commute with the one d before it
    float2 on_[kMaxWave][3 * (kMaxB + 1)];
    Comp part[kMaxWave][kBatchMaxWarps];
    dd base0[kMaxWave];
    int upper_ok[kMaxWave];
    unsigned int accepts;
};

__device__ __forceinline__ bool CircOverlap(uint32_t s1, uint32_t l1, uint32_t s2, uint32_t l2, uint32_t M) {
    return Wrap(s2 + M - s1, M) < l1 || Wrap(s1 + M - s2, M) < l2;
}

/// Does either attempt read what the other writes? (Inner slices [b+1, b+B-1] are written; the
/// segment [b, b+B] of the moved particle and the inner slices of every particle are read.)
__device__ __forceinline__ bool Interact(uint32_t pi, uint32_t bi, uint32_t pj, uint32_t bj, uint32_t B, uint32_t M) {
    const uint32_t si = Wrap(bi + 1u, M), sj = Wrap(bj + 1u, M);
    if (pi == pj) return B + 1 > M || CircOverlap(si, B - 1, bj, B + 1, M) || CircOverlap(sj, B - 1, bi, B + 1, M);
    return CircOverlap(si, B - 1, sj, B - 1, M);
}

/// DrawAttempt for attempt y into ring slot `sl`, plus its scoreboard mask: lane d (1 <= d <
/// kWindow) recomputes the particle and first bead of attempt y - d from its stream (block 0).
__device__ __forceinline__ void DrawScored(WaveShared& sh, const WaveRing& ring, uint64_t y, uint32_t lane, uint32_t N, uint32_t M, uint32_t B,
                                           uint32_t NL, uint32_t n_pad, const float4* __restrict__ pos) {
    const ChainDev& c = sh.c;
    const uint32_t sl = (uint32_t)y & (kRing - 1u);
    const Philox4 w0 = MoveStream{c.seed, c.chain_id, c.move, y}.Block(0);
    bool hit = false;
    if (lane >= 1 && lane < kWindow && y >= lane) {
        const Philox4 w = MoveStream{c.seed, c.chain_id, c.move, y - lane}.Block(0);
        hit = Interact(UniformIndex(w.v[0], N), UniformIndex(w.v[1], M), UniformIndex(w0.v[0], N), UniformIndex(w0.v[1], M), B, M);
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) sh.dep[sl] = m;
    DrawAttempt(MoveStream{c.seed, c.chain_id, c.move, y}, lane, N, M, B, NL, n_pad, pos, ring.Z(sl), ring.LU(sl), nullptr, sh.pb[sl]);
}

__device__ __forceinline__ void SubSync(uint32_t id, uint32_t n_warps) {
    if (n_warps == 1) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n_warps * 32u) : "memory");
}

/// Barrier over the two blocks of a cluster (release/acquire: each block's shared-memory writes,
/// local and remote, are visible to both after it).
__device__ __forceinline__ void ClusterPairSync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

/// kSplit: the chain runs on both blocks of a two-block cluster (crank = this block's rank). Both
/// hold the staged path and the same scoreboard; a round takes the first 2W eligible attempts and
/// block r runs those of rank r, r + 2, ...; an accepted attempt writes its beads into both blocks'
/// planes, and a cluster barrier closes each round.
template <bool kPbc, bool kStaged, bool kSplit>
__device__ __forceinline__ void SweepChainW(WaveShared& sh, float* stage, BatchArgs a, uint32_t ci, uint64_t n_sweeps, uint64_t n_attempts,
                                            uint32_t crank) {
    static_assert(!kSplit || kStaged, "a split chain is staged in both blocks");
    const ChainDev& c = sh.c;
    const uint32_t W = c.n_wave, Gs = c.sub_warps, G = W * Gs;
    constexpr uint32_t kMask = kRing - 1;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    // Warp w belongs to sub-group w mod W: the leaders (warps 0..W-1), whose phases are the
    // serial part of a round, sit on different SM sub-partitions.
    const uint32_t sg = warp % W, ws = warp / W, Ts = Gs * 32u, ts = ws * 32u + lane;
    const uint32_t N = c.n_part, M = c.n_bead, NL = c.n_level, B = 1u << NL, n_pad = c.n_pad;
    float4* __restrict__ pos = a.pos + c.pos_off;
    const uint32_t draw_warp = Gs >= 2 ? 1u : 0u;
    const PathView<kStaged> path{pos, stage, n_pad, N, N * M};
    if constexpr (kStaged)  // the path into shared memory (visible after the prologue's barrier)
        for (uint32_t i = threadIdx.x; i < N * M; i += G * 32u) {
            const uint32_t b = i / N, q = i - b * N;
            const float4 v = pos[(size_t)b * n_pad + q];
            stage[i] = v.x;
            stage[N * M + i] = v.y;
            stage[2 * N * M + i] = v.z;
        }
    float* const ring_base = stage + (kStaged ? 3 * N * M : 0u);
    const WaveRing ring{ring_base, ring_base + kRing * 3 * (B - 1), 3 * (B - 1), NL};
    float* peer_stage = stage;  // the other block's planes at the same offset (distributed shared memory)
    if constexpr (kSplit) peer_stage = cooperative_groups::this_cluster().map_shared_rank(stage, crank ^ 1u);
    const PathView<kStaged> peer{pos, peer_stage, n_pad, N, N * M};

    const uint32_t nm1 = N > 1 ? N - 1 : 1;
    const uint32_t n_items = c.has_pair && N > 1 ? (N - 1) * (B - 1) : 0u;
    const uint32_t magic = (uint32_t)((0x100000000ull + nm1 - 1) / nm1);
    uint32_t it_k[kItems], it_q[kItems];
#pragma unroll
    for (uint32_t j = 0; j < kItems; ++j) {
        const uint32_t i = ts + j * Ts;
        it_k[j] = FastDivD(i, nm1, magic);
        it_q[j] = i - it_k[j] * nm1;
    }
    // Staged paths with enough partners for the group's lanes: partner-major pair loop, whose
    // per-lane item count (ceil(nm1 / Ts) (B - 1)) is within 5/4 of the flattened loop's.
    const uint32_t pmk = (kStaged && n_items && (nm1 + Ts - 1) / Ts * (B - 1) * 4u <= (n_items + Ts - 1) / Ts * 5u) ? B - 1 : 0u;

    uint64_t H = a.attempts[ci];  // the first attempt not yet run
    const uint64_t end = H + (n_sweeps ? n_sweeps * c.attempts_per_sweep : n_attempts);
    uint64_t U = ~0ull;           // bit i: attempt H + i not yet run (bits kWindow.. stay set)
    uint64_t n_rounds = 0;
    if (threadIdx.x == 0) sh.accepts = 0;
    // Prologue: the first window's draws, attempt H + x by sub-group x mod W.
    if (ws == draw_warp)
        for (uint64_t y = H + sg; y < end && y < H + kWindow; y += W) DrawScored(sh, ring, y, lane, N, M, B, NL, n_pad, pos);
    if constexpr (kSplit) ClusterPairSync();  // both blocks staged before either commits into the other
    else SubSync(15, G);
    constexpr uint32_t kWays = kSplit ? 2u : 1u;  // blocks sharing the chain's rounds

    while (H < end) {
        // The round's attempts: the first W of the window that commute with every earlier attempt
        // not yet run (the same on every lane of every warp; attempt H always qualifies).
        bool ok = false;
        if (lane < kWindow && H + lane < end && ((U >> lane) & 1u)) {
            const uint32_t dep = sh.dep[(uint32_t)(H + lane) & kMask];
            ok = ((__brev(dep) >> (31u - lane)) & (uint32_t)U) == 0u;  // bit lane - d <- bit d of dep
        }
        const unsigned elig = __ballot_sync(0xffffffffu, ok);
        const uint32_t rank = __popc(elig & ((1u << lane) - 1u));  // eligible attempts before this lane's
        const unsigned sel = __ballot_sync(0xffffffffu, ok && rank < kWays * W);
        const unsigned mine = __ballot_sync(0xffffffffu, ok && rank == kWays * sg + crank);
        const uint64_t U_next = U & ~(uint64_t)sel;
        const uint32_t adv = (uint32_t)__ffsll((long long)U_next) - 1u;  // attempts at the head that are now run (<= kWindow)
        if (mine) {
            const uint32_t pos_in_window = (uint32_t)__ffs(mine) - 1u;
            const uint64_t y = H + pos_in_window;
            const uint32_t slot = (uint32_t)y & kMask;
            const uint32_t p = sh.pb[slot][0], b0 = sh.pb[slot][1];
            float3 pre[kItems];
            if constexpr (!kStaged) {  // global beads: the first items' partners in flight during the leader
#pragma unroll
                for (uint32_t j = 0; j < kItems; ++j)
                    if (ts + j * Ts < n_items) pre[j] = path.Load(Wrap(b0 + 1u + it_k[j], M), it_q[j] + (it_q[j] >= p ? 1u : 0u));
            }
            float nx = 0.f, ny = 0.f, nz = 0.f;
            bool lead_upper = false;
            dd lead_base0 = DD(0.f);
            if (ws == 0) {
                const float3 sv = path.Load(Wrap(b0 + (lane <= B ? lane : B), M), p);
                const float3 se = path.Load(Wrap(b0 + B, M), p);
                LeaderPhase<kPbc>(c, lane, NL, M, sv.x, sv.y, sv.z, se.x, se.y, se.z, ring.Z(slot), ring.LU(slot), sh.on_[sg],
                                  &sh.base0[sg], &sh.upper_ok[sg], nx, ny, nz, lead_upper, lead_base0);
            }
            // Draws that refill the window behind the head's advance (their slots are not in use).
            if (ws == draw_warp) {
                if (draw_warp == 0) __syncwarp();
                for (uint64_t yd = H + kWindow + sg; yd < H + kWindow + adv && yd < end; yd += W) DrawScored(sh, ring, yd, lane, N, M, B, NL, n_pad, pos);
            }
            SubSync(1 + sg, Gs);
            const bool upper_ok = ws == 0 ? lead_upper : sh.upper_ok[sg] != 0;
            if (upper_ok && n_items) {
                const Comp u = CompWarpSum(PairPhase<kPbc, kStaged>(c, ts, Ts, n_items, magic, nm1, p, b0, M, path, it_k, pre, sh.on_[sg], pmk), 32);
                if (lane == 0) sh.part[sg][ws] = u;
            }
            SubSync(1 + sg, Gs);
            if (ws == 0) {
                const bool accepted = upper_ok && Level0Accepts(c, lane, Gs, sh.part[sg], n_items != 0, lead_base0, ring.LU(slot)[0]);
                if (accepted && lane >= 1 && lane < B) {
                    path.Store(Wrap(b0 + lane, M), p, nx, ny, nz);
                    if constexpr (kSplit) peer.Store(Wrap(b0 + lane, M), p, nx, ny, nz);
                }
                if (accepted && lane == 0) atomicAdd(&sh.accepts, 1u);
            }
        } else if (ws == draw_warp) {
            for (uint64_t yd = H + kWindow + sg; yd < H + kWindow + adv && yd < end; yd += W) DrawScored(sh, ring, yd, lane, N, M, B, NL, n_pad, pos);
        }
        if constexpr (kSplit) ClusterPairSync();  // both blocks' commits, local and remote, before the next round
        else SubSync(15, G);
        ++n_rounds;
        U = adv ? (U_next >> adv) | (~0ull << (64u - adv)) : U_next;
        H += adv;
    }
    if constexpr (kStaged)  // every round ended with a block (cluster) barrier: all commits are visible
        if (crank == 0)     // a split chain's two copies are identical
            for (uint32_t i = threadIdx.x; i < N * M; i += G * 32u) {
                const uint32_t b = i / N, q = i - b * N;
                pos[(size_t)b * n_pad + q] = make_float4(stage[i], stage[N * M + i], stage[2 * N * M + i], 0.f);
            }
    if (threadIdx.x == 0) {
        if (kSplit) {
            atomicAdd(reinterpret_cast<unsigned long long*>(&a.accepts[ci]), (unsigned long long)sh.accepts);
        } else {
            a.accepts[ci] += sh.accepts;
        }
        if (crank == 0) {
            a.attempts[ci] = H;
            a.rounds[ci] += n_rounds;
        }
    }
}

union BatchShared {
    SweepShared one;
    WaveShared wave;
};

__global__ void __launch_bounds__(kBatchMaxWarps * 32) BatchSweepKernel(BatchArgs a, uint64_t n_sweeps, uint64_t n_attempts) {
    uint32_t ci, crank = 0;
    bool split = false;
    if (a.cluster_tasks) {  // clusters of two blocks: cluster j runs tasks[j]
        const uint2 task = a.cluster_tasks[blockIdx.x >> 1];
        crank = blockIdx.x & 1u;  // the block's rank in its cluster
        split = task.x == task.y;
        ci = crank ? task.y : task.x;
        if (ci == 0xffffffffu) return;  // the last cluster's second block when the chain count is odd
    } else {
        ci = a.order[blockIdx.x];
    }
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t G = a.chains[ci].n_warps;
    if (warp >= G) return;  // a split chain uses every warp of the block (no early exit before its cluster barriers)
    __shared__ BatchShared sh;
    extern __shared__ float4 batch_stage[];  // staged path planes (chains with `staged` set)
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(a.chains + ci);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&sh.one.c);
        for (uint32_t i = threadIdx.x; i < sizeof(ChainDev) / 4; i += G * 32u) dst[i] = src[i];
    }
    GroupSync(G);
    if (sh.one.c.n_wave > 1) {
        float* stage = reinterpret_cast<float*>(batch_stage);
        if (split) {  // the host splits only staged chains with a wave
            if (sh.one.c.pbc) SweepChainW<true, true, true>(sh.wave, stage, a, ci, n_sweeps, n_attempts, crank);
            else SweepChainW<false, true, true>(sh.wave, stage, a, ci, n_sweeps, n_attempts, crank);
        } else if (sh.one.c.staged) {
            if (sh.one.c.pbc) SweepChainW<true, true, false>(sh.wave, stage, a, ci, n_sweeps, n_attempts, 0);
            else SweepChainW<false, true, false>(sh.wave, stage, a, ci, n_sweeps, n_attempts, 0);
        } else {
            if (sh.one.c.pbc) SweepChainW<true, false, false>(sh.wave, stage, a, ci, n_sweeps, n_attempts, 0);
            else SweepChainW<false, false, false>(sh.wave, stage, a, ci, n_sweeps, n_attempts, 0);
        }
    } else {
        if (sh.one.c.pbc) SweepChain<true>(sh.one, a, ci, G, n_sweeps, n_attempts);
        else SweepChain<false>(sh.one, a, ci, G, n_sweeps, n_attempts);
    }
}

/// Thermal energy estimator (Energy::Accumulate with use_thermal, energy_class.h:36-58): the sum of
/// the actions' DActionDBeta divided by M, per action:
///   Kinetic       N M D / (2 tau) - sum_{p,b} |r_{b+1} - r_b|^2 / (4 lambda tau^2)  kinetic_class.h:35-45
///   HarmonicTrap  cofactor_b sum_{p,b} r^2                                         trap_class.h:20-35
///   Coulomb       sum_{p<q} sum_b (1/r_b + 1/r_{b+1}) / 2                          pair_action_class.h:241-264
/// A chain's slices are split into tasks of kEnergySlices; one block per task stages the task's
/// slices (and the next one) in shared memory, forms the task's three sums, and one warp per chain
/// adds its tasks' sums in task order (deterministic).
constexpr uint32_t kEnergySlices = 8;
constexpr uint32_t kEnergyThreads = 256;

struct EnergyTask {
    uint32_t chain, b0, nb, pad;
};

__global__ void __launch_bounds__(kEnergyThreads) BatchEnergyPartKernel(BatchArgs a, const EnergyTask* __restrict__ tasks, float2* __restrict__ part) {
    const EnergyTask tk = tasks[blockIdx.x];
    const ChainDev& c = a.chains[tk.chain];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t T = blockDim.x, t = threadIdx.x;
    const uint32_t N = c.n_part, M = c.n_bead, n_pad = c.n_pad;
    const int pbc = c.pbc;
    const float L = c.L, iL = c.iL;
    const float4* __restrict__ pos = a.pos + c.pos_off;
    __shared__ dd s_red[3][kEnergyThreads / 32];
    extern __shared__ float4 s_pos[];  // slices b0 .. b0 + nb of the task, [slot][N]
    // i / N by FastDiv (i N < 2^32 here); a divisor of 1 has no 32-bit multiplier
    const uint32_t mN = (uint32_t)((0x100000000ull + N - 1) / N);
    auto div_n = [&](uint32_t i) { return FastDivD(i, N, mN); };
    for (uint32_t i = t; i < N * (tk.nb + 1); i += T) {
        const uint32_t slot = div_n(i), pp = i - slot * N;
        s_pos[i] = pos[(size_t)((tk.b0 + slot) % M) * n_pad + pp];
    }
    __syncthreads();

    dd kin = DD(0.f), trap = DD(0.f), pair = DD(0.f);
    for (uint32_t i = t; i < N * tk.nb; i += T) {
        const uint32_t bb = div_n(i), pp = i - bb * N;
        const float4 r = s_pos[bb * N + pp];
        const float4 r1 = s_pos[(bb + 1) * N + pp];
        // |r_{b+1} - r_b|^2 with exact differences (TwoSum) and products (TwoProd).
        dd dx = TwoSum(r1.x, -r.x), dy = TwoSum(r1.y, -r.y), dz = TwoSum(r1.z, -r.z);
        if (pbc) {
            dx = Sub(dx, DD(__fmul_rn(L, rintf(__fmul_rn(dx.hi, iL)))));
            dy = Sub(dy, DD(__fmul_rn(L, rintf(__fmul_rn(dy.hi, iL)))));
            dz = Sub(dz, DD(__fmul_rn(L, rintf(__fmul_rn(dz.hi, iL)))));
        }
        kin = Add(kin, Add(Add(Sqr(dx), Sqr(dy)), Sqr(dz)));
        trap = AddSq(AddSq(AddSq(trap, r.x), r.y), r.z);
    }
    if (c.has_pair && N > 1) {
        // Unordered pairs of one slice: (p, p + o mod N) for o = 1 .. (N-1)/2, plus o = N/2 for
        // p < N/2 when N is even; items (slice of the task, pair) spread evenly over the block.
        const uint32_t half = (N - 1) / 2, n_main = N * half;
        const uint32_t n_pairs = N * (N - 1) / 2;
        const uint32_t mP = (uint32_t)((0x100000000ull + n_pairs - 1) / n_pairs);
        Comp acc{0.f, 0.f};
        const bool fast = n_pairs > 1 && (uint64_t)n_pairs * tk.nb * n_pairs < (1ull << 32);  // FastDiv exact below 2^32
        for (uint32_t i = t; i < n_pairs * tk.nb; i += T) {
            const uint32_t bb = fast ? FastDiv(i, mP) : i / n_pairs, j = i - bb * n_pairs;
            const float4* row = s_pos + bb * N;
            uint32_t pp, o;
            if (j < n_main) {
                o = 1 + div_n(j);
                pp = j - (o - 1) * N;
            } else {
                pp = j - n_main;
                o = N / 2;
            }
            uint32_t q = pp + o;
            if (q >= N) q -= N;
            const float4 r = row[pp], s = row[q];
            const float x = MinImg(__fsub_rn(r.x, s.x), pbc, L, iL);
            const float y = MinImg(__fsub_rn(r.y, s.y), pbc, L, iL);
            const float z = MinImg(__fsub_rn(r.z, s.z), pbc, L, iL);
            float r2 = __fmaf_rn(x, x, __fmaf_rn(y, y, __fmul_rn(z, z)));
            r2 = fminf(fmaxf(r2, c.r2_min), c.r2_max);
            CompAdd(acc, rsqrtf(r2));
        }
        pair = CompDD(acc);
    }
    kin = WarpSumDD(kin);
    trap = WarpSumDD(trap);
    pair = WarpSumDD(pair);
    if (lane == 0) {
        s_red[0][warp] = kin;
        s_red[1][warp] = trap;
        s_red[2][warp] = pair;
    }
    __syncthreads();
    if (warp == 0) {
        dd v[3];
        for (int q = 0; q < 3; ++q) v[q] = WarpSumDD(lane < T / 32 ? s_red[q][lane] : DD(0.f));
        if (lane == 0)
            for (int q = 0; q < 3; ++q) part[(size_t)blockIdx.x * 3 + q] = make_float2(v[q].hi, v[q].lo);
    }
}

/// One warp per chain: its tasks' sums in task order, then E and its parts (FP64) into the
/// series and the latest-measurement record.
/// One warp per chain of order positions [i0, i1): its tasks [first_task[i], first_task[i + 1]) are
/// summed in task order.
__global__ void BatchEnergyFinishKernel(BatchArgs a, const uint32_t* __restrict__ first_task, const float2* __restrict__ part, uint32_t i0,
                                        uint32_t i1) {
    const uint32_t i = i0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
    if (i >= i1) return;
    const uint32_t ci = a.order[i];
    const ChainDev& c = a.chains[ci];
    const uint32_t t0 = first_task[i], t1 = first_task[i + 1];
    dd s[3] = {DD(0.f), DD(0.f), DD(0.f)};
    for (uint32_t t = t0 + lane; t < t1; t += 32)
        for (int q = 0; q < 3; ++q) {
            const float2 v = part[(size_t)t * 3 + q];
            s[q] = Add(s[q], dd{v.x, v.y});
        }
    for (int q = 0; q < 3; ++q) s[q] = WarpSumDD(s[q]);
    if (lane != 0) return;
    const double inv_m = 1.0 / (double)c.n_bead;
    const double e_kin = (c.kin_const - c.i4ltt * ToDouble(s[0])) * inv_m;
    const double e_trap = c.has_trap ? c.trap_cofb * ToDouble(s[1]) * inv_m : 0.;
    const double e_pair = ToDouble(s[2]) * inv_m;
    const uint64_t n = a.n_meas[ci];
    if (!isfinite(e_kin + e_trap + e_pair)) atomicOr(a.err, kDevErrNonFinite);
    double* last = a.last + (size_t)ci * kBatchSeriesComponents;
    last[0] = e_kin + e_trap + e_pair;
    last[1] = e_kin;
    last[2] = e_trap;
    last[3] = e_pair;
    if (n < a.series_cap) {
        double* out = a.series + ((size_t)ci * a.series_cap + n) * kBatchSeriesComponents;
        out[0] = e_kin + e_trap + e_pair;
        out[1] = e_kin;
        out[2] = e_trap;
        out[3] = e_pair;
    }
    a.n_meas[ci] = n + 1;
}

// ---------------------------------------------------------------------------------------------
// Hybrid Monte Carlo on every chain (the library's whole-path HMC move; no reference counterpart).
// Each chain runs on a cluster of k thread blocks (k = 1, 2, 4 or 8, the same for the launch): block
// r of the cluster owns slices [r M / k, (r + 1) M / k). Per attempt: momenta P ~ N(0, 1) per
// coordinate from the attempt's counter-based stream (normal j of the path-ordered coordinates
// (p, b, d) is component j % 4 of Philox block 1 + j / 4, as the single-chain move draws them);
// leapfrog on H = S(R) + |P|^2 / 2 with the exact gradient of the whole-ring action at level 0
//   S = sum_{p,b} |r_{b+1} - r_b|^2 / (4 lambda tau)        (Kinetic, n_images 0)
//     + cofactor_a sum_{p,b} r^2                           (HarmonicTrap)
//     + tau sum_b sum_{p<q} V(|r_p - r_q|), V = 1/r clamped to the table's r range (BarePairAction);
// then acceptance with probability min(1, exp(-dH)) against the log-uniform of block 0, word 0.
// A block keeps its slices and one halo slice on each side in shared memory as three FP32 planes
// [nb + 2][N], and its beads' momenta as three planes [nb][N]; after every drift the halos are read
// from the neighbouring blocks' shared memory (distributed shared memory, between two cluster
// barriers). Forces and leapfrog updates are FP32 (each thread owns fixed beads); both energies are
// sums of exact differences and products in double-float, reduced over the cluster in block order,
// and dH is formed in FP64, so the decision sees the trajectory's energy change to ~1e-6 absolute.
constexpr uint32_t kHmcThreads = 512;

struct HmcArgs {
    uint64_t* att;  // per chain: HMC attempts (the move's Philox attempt counter)
    uint64_t* acc;
    uint32_t n_attempts;
};

/// Block-wide double-float sums of four quantities (fixed tree; every thread receives them).
__device__ __forceinline__ void BlockSum4DD(dd v[4], dd (*s_red)[kHmcThreads / 32]) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, nw = blockDim.x >> 5;
    for (int q = 0; q < 4; ++q) v[q] = WarpSumDD(v[q]);
    __syncthreads();
    if (lane == 0)
        for (int q = 0; q < 4; ++q) s_red[q][warp] = v[q];
    __syncthreads();
    for (int q = 0; q < 4; ++q) v[q] = WarpSumDD(lane < nw ? s_red[q][lane] : DD(0.f));
}

/// The block's beads: three coordinate planes of rows [nb + 2][N2] (row 0 and row nb + 1 are the
/// neighbouring blocks' edge slices; N2 = N rounded up to even so that partner pairs load as float2).
struct HmcRows {
    float* x;
    float* y;
    float* z;
    uint32_t N, N2;
};

/// Kinetic and trap gradient dS/dr (FP32) of bead (row, p), row >= 1, and, with kEnergy, its share
/// of S: the link to the next slice and its trap term.
template <bool kPbc, bool kEnergy>
__device__ __forceinline__ float3 HmcBeadTerms(const ChainDev& c, const HmcRows& R, uint32_t i, float i4, float cofa, dd& e_kin, dd& e_trap) {
    const uint32_t ip = i - R.N2, in_ = i + R.N2;
    const float x = R.x[i], y = R.y[i], z = R.z[i];
    const float xp = R.x[ip], yp = R.y[ip], zp = R.z[ip], xn = R.x[in_], yn = R.y[in_], zn = R.z[in_];
    // links (b-1 -> b) and (b -> b+1): d/dr_b of |r_{b+1} - r_b|^2 i4 summed = 2 i4 (d_{b-1} - d_b)
    const float dpx = Img<kPbc>(__fsub_rn(x, xp), c.L, c.iL), dpy = Img<kPbc>(__fsub_rn(y, yp), c.L, c.iL),
                dpz = Img<kPbc>(__fsub_rn(z, zp), c.L, c.iL);
    const float dnx = Img<kPbc>(__fsub_rn(xn, x), c.L, c.iL), dny = Img<kPbc>(__fsub_rn(yn, y), c.L, c.iL),
                dnz = Img<kPbc>(__fsub_rn(zn, z), c.L, c.iL);
    const float k2 = 2.f * i4;
    float3 g = make_float3(__fmul_rn(k2, __fsub_rn(dpx, dnx)), __fmul_rn(k2, __fsub_rn(dpy, dny)), __fmul_rn(k2, __fsub_rn(dpz, dnz)));
    if (c.has_trap) {
        const float t2 = 2.f * cofa;
        g.x = __fmaf_rn(t2, x, g.x);
        g.y = __fmaf_rn(t2, y, g.y);
        g.z = __fmaf_rn(t2, z, g.z);
    }
    if constexpr (kEnergy) {
        dd ex = TwoSum(xn, -x), ey = TwoSum(yn, -y), ez = TwoSum(zn, -z);
        if (kPbc) {
            ex = Sub(ex, DD(__fmul_rn(c.L, rintf(__fmul_rn(ex.hi, c.iL)))));
            ey = Sub(ey, DD(__fmul_rn(c.L, rintf(__fmul_rn(ey.hi, c.iL)))));
            ez = Sub(ez, DD(__fmul_rn(c.L, rintf(__fmul_rn(ez.hi, c.iL)))));
        }
        e_kin = Add(e_kin, Add(Add(Sqr(ex), Sqr(ey)), Sqr(ez)));
        e_trap = AddSq(AddSq(AddSq(e_trap, x), y), z);
    }
    return g;
}

/// Pair force on bead (row, p): sum over q of V'(r)/r (r_p - r_q), V = 1/r clamped to the table's
/// range, so V' = -1/r^2 inside it and 0 where clamped (q = p: r = 0 is below the range, whose lower
/// end is positive). Partners go two at a time (q, q + 1) in f32x2 arithmetic, each half rounding
/// as the scalar form does; the even and odd partners' sums are added at the end (an odd N's last
/// partner joins the odd sum). With kEnergy also the sum over q != p of V(r).
template <bool kPbc, bool kEnergy>
__device__ __forceinline__ float3 HmcPairForce(const ChainDev& c, const HmcRows& R, uint32_t row0, uint32_t p, Comp& e_pair) {
    const float* __restrict__ rx = R.x + row0;
    const float* __restrict__ ry = R.y + row0;
    const float* __restrict__ rz = R.z + row0;
    const float x = rx[p], y = ry[p], z = rz[p];
    const float2 X = make_float2(x, x), Y = make_float2(y, y), Z = make_float2(z, z);
    const float r2lo = c.r2_min, r2hi = c.r2_max;
    const uint32_t N = R.N, Ne = N & ~1u;
    float2 fx = make_float2(0.f, 0.f), fy = fx, fz = fx;
#pragma unroll 2
    for (uint32_t q = 0; q < Ne; q += 2) {
        const float2 bx = *reinterpret_cast<const float2*>(rx + q);
        const float2 by = *reinterpret_cast<const float2*>(ry + q);
        const float2 bz = *reinterpret_cast<const float2*>(rz + q);
        const float2 ux = Img2<kPbc>(Sub2(X, bx), c.L, c.iL);
        const float2 uy = Img2<kPbc>(Sub2(Y, by), c.L, c.iL);
        const float2 uz = Img2<kPbc>(Sub2(Z, bz), c.L, c.iL);
        const float2 r2 = Sq3x2(ux, uy, uz);
        const float c0 = fminf(fmaxf(r2.x, r2lo), r2hi), c1 = fminf(fmaxf(r2.y, r2lo), r2hi);
        const float2 inv = make_float2(rsqrtf(c0), rsqrtf(c1));
        if constexpr (kEnergy) {
            CompAdd(e_pair, q == p ? 0.f : inv.x);
            CompAdd(e_pair, q + 1 == p ? 0.f : inv.y);
        }
        float2 f = Mul2(Mul2(inv, inv), inv);
        f.x = c0 == r2.x ? f.x : 0.f;
        f.y = c1 == r2.y ? f.y : 0.f;
        fx = Fma2(f, ux, fx);
        fy = Fma2(f, uy, fy);
        fz = Fma2(f, uz, fz);
    }
    if (N & 1u) {
        const uint32_t q = N - 1;
        const float ux = Img<kPbc>(__fsub_rn(x, rx[q]), c.L, c.iL), uy = Img<kPbc>(__fsub_rn(y, ry[q]), c.L, c.iL),
                    uz = Img<kPbc>(__fsub_rn(z, rz[q]), c.L, c.iL);
        const float r2 = Sq3(ux, uy, uz);
        const float cq = fminf(fmaxf(r2, r2lo), r2hi);
        const float inv = rsqrtf(cq);
        if constexpr (kEnergy) CompAdd(e_pair, q == p ? 0.f : inv);
        const float f = cq == r2 ? __fmul_rn(__fmul_rn(inv, inv), inv) : 0.f;
        fx.y = __fmaf_rn(f, ux, fx.y);
        fy.y = __fmaf_rn(f, uy, fy.y);
        fz.y = __fmaf_rn(f, uz, fz.y);
    }
    return make_float3(__fadd_rn(fx.x, fx.y), __fadd_rn(fy.x, fy.y), __fadd_rn(fz.x, fz.y));
}

/// One kick P -= f dS/dR for the block's beads; with kEnergy also the block's shares of S and
/// |P|^2 (before the kick when `p2_before`, after it when `p2_after`).
template <bool kPbc, bool kEnergy>
__device__ __forceinline__ void HmcKick(const ChainDev& c, const HmcRows& R, float* px, float* py, float* pz, uint32_t E, float f, bool p2_before,
                                        bool p2_after, dd& ek, dd& et, Comp& cp, dd& em) {
    const float i4 = c.i4lt_level[0], cofa = c.trap_cofa, tau = c.tau;
    const uint32_t N = R.N, N2 = R.N2;
    for (uint32_t i = threadIdx.x; i < E; i += blockDim.x) {
        const uint32_t lb = i / N, p = i - lb * N;
        const uint32_t row0 = (lb + 1) * N2;
        float3 g = HmcBeadTerms<kPbc, kEnergy>(c, R, row0 + p, i4, cofa, ek, et);
        if (c.has_pair) {
            const float3 fp = HmcPairForce<kPbc, kEnergy>(c, R, row0, p, cp);
            g.x = __fmaf_rn(-tau, fp.x, g.x);
            g.y = __fmaf_rn(-tau, fp.y, g.y);
            g.z = __fmaf_rn(-tau, fp.z, g.z);
        }
        float mx = px[i], my = py[i], mz = pz[i];
        if (kEnergy && p2_before) em = AddSq(AddSq(AddSq(em, mx), my), mz);  // |P|^2 before the first kick
        mx = __fmaf_rn(-f, g.x, mx);
        my = __fmaf_rn(-f, g.y, my);
        mz = __fmaf_rn(-f, g.z, mz);
        if (kEnergy && p2_after) em = AddSq(AddSq(AddSq(em, mx), my), mz);  // |P|^2 after the last kick
        px[i] = mx;
        py[i] = my;
        pz[i] = mz;
    }
}

struct HmcShared {
    dd red[4][kHmcThreads / 32];
    dd part[4];   // this block's energy sums, read by the whole cluster
    int accept;
};

/// Halo rows 0 and nb + 1 from the neighbouring blocks' last and first own rows (the ring wraps).
__device__ __forceinline__ void HmcHalos(cooperative_groups::cluster_group& cl, const HmcRows& R, uint32_t nb) {
    const uint32_t k = cl.num_blocks(), r = cl.block_rank(), N = R.N, N2 = R.N2;
    float* planes[3] = {R.x, R.y, R.z};
    for (uint32_t i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const uint32_t d = i / N, p = i - d * N;
        float* mine = planes[d];
        const float* left = cl.map_shared_rank(mine, (r + k - 1) % k);
        const float* right = cl.map_shared_rank(mine, (r + 1) % k);
        mine[p] = left[nb * N2 + p];
        mine[(nb + 1) * N2 + p] = right[N2 + p];
    }
}

template <bool kPbc>
__device__ void HmcChain(const BatchArgs& a, const HmcArgs& h, const ChainDev& c, uint32_t ci, float* smem, HmcShared& sh) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t k = cl.num_blocks(), r = cl.block_rank();
    const uint32_t N = c.n_part, M = c.n_bead, n_pad = c.n_pad, N2 = N + (N & 1u);
    const uint32_t nb = M / k, b_lo = r * nb, E = nb * N, RW = (nb + 2) * N2;
    const HmcRows R{smem, smem + RW, smem + 2 * RW, N, N2};
    float* px = smem + 3 * RW;
    float* py = px + E;
    float* pz = py + E;
    const uint32_t t = threadIdx.x, T = blockDim.x;
    float4* pos = a.pos + c.pos_off;
    const float cofa = c.trap_cofa, eps = c.hmc_eps;
    const double i4d = 1. / (4. * (double)c.lambda * (double)c.tau), taud = (double)c.tau;
    uint64_t att = h.att[ci], acc = 0;
    for (uint32_t it = 0; it < h.n_attempts; ++it, ++att) {
        const MoveStream st{c.seed, c.chain_id, c.hmc_move, att};
        // own slices from the committed path (this block wrote them last); momenta from the stream
        for (uint32_t i = t; i < E; i += T) {
            const uint32_t lb = i / N, p = i - lb * N, b = b_lo + lb, ri = (lb + 1) * N2 + p;
            const float4 v = pos[(size_t)b * n_pad + p];
            R.x[ri] = v.x;
            R.y[ri] = v.y;
            R.z[ri] = v.z;
            float z3[3];
            const uint32_t j0 = (p * M + b) * 3u;
            for (uint32_t d = 0; d < 3; ++d) {
                const uint32_t j = j0 + d;
                const Philox4 w = st.Block(1u + (j >> 2));
                float z0, z1;
                if ((j & 3u) < 2u) BoxMullerF(w.v[0], w.v[1], z0, z1);
                else BoxMullerF(w.v[2], w.v[3], z0, z1);
                z3[d] = (j & 1u) ? z1 : z0;
            }
            px[i] = z3[0];
            py[i] = z3[1];
            pz[i] = z3[2];
        }
        cl.sync();
        HmcHalos(cl, R, nb);
        cl.sync();
        double h_start = 0., h_end = 0.;
        const uint32_t n_steps = c.hmc_steps;
        for (uint32_t s = 0; s <= n_steps; ++s) {
            // gradient at the current R; energy at the start (s = 0) and the end (s = n_steps)
            const bool with_energy = s == 0 || s == n_steps;
            const float f = with_energy ? 0.5f * eps : eps;
            dd ek = DD(0.f), et = DD(0.f), em = DD(0.f);
            Comp cp{0.f, 0.f};
            if (with_energy) HmcKick<kPbc, true>(c, R, px, py, pz, E, f, s == 0, s == n_steps, ek, et, cp, em);
            else HmcKick<kPbc, false>(c, R, px, py, pz, E, f, false, false, ek, et, cp, em);
            if (with_energy) {
                dd v[4] = {ek, et, CompDD(cp), em};
                BlockSum4DD(v, sh.red);
                if (t == 0)
                    for (int q = 0; q < 4; ++q) sh.part[q] = v[q];
                cl.sync();
                if (t == 0) {
                    dd tot[4] = {DD(0.f), DD(0.f), DD(0.f), DD(0.f)};
                    for (uint32_t rr = 0; rr < k; ++rr) {  // block order: the same sum in every block
                        const dd* pr = cl.map_shared_rank(sh.part, rr);
                        for (int q = 0; q < 4; ++q) tot[q] = Add(tot[q], pr[q]);
                    }
                    const double hv = i4d * ToDouble(tot[0]) + (c.has_trap ? (double)cofa * ToDouble(tot[1]) : 0.) +
                                      0.5 * taud * ToDouble(tot[2]) + 0.5 * ToDouble(tot[3]);
                    if (s == 0) h_start = hv;
                    else h_end = hv;
                }
            }
            __syncthreads();  // every gradient read of R is done
            if (s == n_steps) break;
            for (uint32_t i = t; i < E; i += T) {  // drift
                const uint32_t lb = i / N, ri = (lb + 1) * N2 + (i - lb * N);
                R.x[ri] = __fmaf_rn(eps, px[i], R.x[ri]);
                R.y[ri] = __fmaf_rn(eps, py[i], R.y[ri]);
                R.z[ri] = __fmaf_rn(eps, pz[i], R.z[ri]);
            }
            cl.sync();  // every block drifted its slices
            HmcHalos(cl, R, nb);
            cl.sync();  // every block read its halos before the next drift
        }
        if (t == 0) {
            const double log_accept = -(h_end - h_start);
            const double logu = (double)LogF(U24(st.Block(0).v[0]));
            sh.accept = (isfinite(log_accept) && !(log_accept < logu)) ? 1 : 0;
        }
        __syncthreads();
        if (sh.accept) {
            for (uint32_t i = t; i < E; i += T) {
                const uint32_t lb = i / N, p = i - lb * N, ri = (lb + 1) * N2 + p;
                pos[(size_t)(b_lo + lb) * n_pad + p] = make_float4(R.x[ri], R.y[ri], R.z[ri], 0.f);
            }
            ++acc;
        }
        cl.sync();  // no block reads its part of a later attempt's sums before every block used these
    }
    if (t == 0 && r == 0) {
        h.att[ci] = att;
        h.acc[ci] += acc;
    }
}

__global__ void __launch_bounds__(kHmcThreads, 2) BatchHmcKernel(BatchArgs a, HmcArgs h) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t ci = a.order[blockIdx.x / cl.num_blocks()];
    const ChainDev& c = a.chains[ci];
    if (c.hmc_eps == 0.f) return;  // the chain has no HMC move (every block of its cluster returns)
    __shared__ HmcShared sh;
    extern __shared__ float4 hmc_stage[];
    float* smem = reinterpret_cast<float*>(hmc_stage);
    if (c.pbc) HmcChain<true>(a, h, c, ci, smem, sh);
    else HmcChain<false>(a, h, c, ci, smem, sh);
}

/// Host layout (every chain's [n_part][n_bead][3] doubles, concatenated) to the device float4
/// layout, one block per chain; a non-finite coordinate sets kDevErrNonFinite and is not stored.
__global__ void HostLayoutToPosKernel(const double* __restrict__ src, const ChainDev* __restrict__ chains, const uint64_t* __restrict__ path_off,
                                      float4* __restrict__ pos, int* err) {
    const ChainDev& c = chains[blockIdx.x];
    const double* in = src + path_off[blockIdx.x];
    float4* out = pos + c.pos_off;
    for (uint32_t i = threadIdx.x; i < c.n_part * c.n_bead; i += blockDim.x) {
        const uint32_t p = i / c.n_bead, b = i - p * c.n_bead;
        const double x = in[3 * (size_t)i], y = in[3 * (size_t)i + 1], z = in[3 * (size_t)i + 2];
        if (!isfinite(x) || !isfinite(y) || !isfinite(z)) {
            atomicOr(err, kDevErrNonFinite);
            continue;
        }
        out[(size_t)b * c.n_pad + p] = make_float4((float)x, (float)y, (float)z, 0.f);
    }
}

__global__ void PosToHostLayoutKernel(const float4* __restrict__ pos, const ChainDev* __restrict__ chains, const uint64_t* __restrict__ path_off,
                                      double* __restrict__ dst) {
    const ChainDev& c = chains[blockIdx.x];
    double* out = dst + path_off[blockIdx.x];
    const float4* in = pos + c.pos_off;
    for (uint32_t i = threadIdx.x; i < c.n_part * c.n_bead; i += blockDim.x) {
        const uint32_t p = i / c.n_bead, b = i - p * c.n_bead;
        const float4 r = in[(size_t)b * c.n_pad + p];
        out[3 * (size_t)i] = r.x;
        out[3 * (size_t)i + 1] = r.y;
        out[3 * (size_t)i + 2] = r.z;
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Host side.

ChainSpec ParseChain(const std::string& xml, const std::string& base_dir) {
    ChainSpec s;
    const Input in = Input::FromString(xml);
    const Input rng = in.GetChild("RNG");
    s.seed = rng.IsNull() ? (uint32_t)time(nullptr) : (uint32_t)rng.GetAttribute<int>("seed", (int)time(nullptr));
    const Input sys = in.GetChild("System");
    if (sys.IsNull()) throw PimcError(kErrInput, "input has no <System> element");
    if (sys.GetAttribute<uint32_t>("n_d") != 3) throw PimcError(kErrUnsupported, "batched chains need n_d = 3");
    s.n_bead = sys.GetAttribute<uint32_t>("n_bead");
    s.beta = sys.GetAttribute<double>("beta");
    s.pbc = sys.GetAttribute<bool>("pbc", true);  // path_class.h:29 defaults to periodic
    s.L = s.pbc ? sys.GetAttribute<double>("L") : 0.;
    if (s.n_bead < 2 || !(s.beta > 0.) || (s.pbc && !(s.L > 0.))) throw PimcError(kErrInput, "bad <System> parameters");
    s.tau = s.beta / s.n_bead;
    const auto species = in.GetChild("Particles").GetChildList("Species");
    if (species.size() != 1) throw PimcError(kErrUnsupported, "batched chains need exactly one species");
    const std::string sp = species[0].GetAttribute<std::string>("name");
    s.n_part = species[0].GetAttribute<uint32_t>("n_part");
    s.lambda = species[0].GetAttribute<double>("lambda");
    if (species[0].GetAttribute<bool>("fermi", false) || species[0].GetAttribute<bool>("fixed_node", false))
        throw PimcError(kErrUnsupported, "batched chains are Boltzmannons");
    if (s.n_part < 1 || !(s.lambda > 0.)) throw PimcError(kErrInput, "bad <Species> parameters");
    if (s.n_part > 4096 || s.n_bead > 65536) throw PimcError(kErrUnsupported, "batched chains: n_part <= 4096, n_bead <= 65536");
    bool has_kinetic = false;
    for (const Input& a : in.GetChild("Actions").GetChildList("Action")) {
        const std::string type = a.GetAttribute<std::string>("type");
        if (type == "Kinetic") {
            if (a.GetAttribute<std::string>("species") != sp || a.GetAttribute<int>("n_images", 0) != 0)
                throw PimcError(kErrUnsupported, "batched Kinetic action: one species, n_images = 0");
            has_kinetic = true;
        } else if (type == "HarmonicTrap") {
            if (a.GetAttribute<std::string>("species") != sp) throw PimcError(kErrInput, "trap on an unknown species");
            s.has_trap = true;
            s.omega = a.GetAttribute<double>("omega");
            s.trap_max_level = a.GetAttribute<uint32_t>("max_level", 0);
        } else if (type == "BarePairAction") {
            if (a.GetAttribute<std::string>("species_a") != sp || a.GetAttribute<std::string>("species_b") != sp ||
                !a.GetAttribute<bool>("is_coulomb", false) || a.GetAttribute<bool>("use_long_range", false))
                throw PimcError(kErrUnsupported, "batched pair action: bare Coulomb within the species, no long range");
            std::string file = a.GetAttribute<std::string>("file");
            if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
            const TableFile tf = TableFile::Load(file);
            const auto& r = tf.Vec("v/diag/r");
            if (r.size() < 2) throw PimcError(kErrInput, "table '" + file + "': empty r grid");
            s.has_pair = true;
            s.r_min = r.front();
            s.r_max = r.back();
        } else {
            throw PimcError(kErrUnsupported, "batched chains do not support action type '" + type + "'");
        }
    }
    if (!has_kinetic) throw PimcError(kErrUnsupported, "batched chains need a Kinetic action");
    // One Bisect move and at most one HMC move; each keeps its index in the input as the key of its
    // random stream, as in a single-chain context.
    const auto moves = in.GetChild("Moves").GetChildList("Move");
    int bisect = -1;
    for (size_t i = 0; i < moves.size(); ++i) {
        const std::string type = moves[i].GetAttribute<std::string>("type");
        if (type == "Bisect" && bisect < 0) {
            bisect = (int)i;
        } else if (type == "HMC" && !s.has_hmc) {
            const std::string hs = moves[i].GetAttribute<std::string>("species", "");
            if (!hs.empty() && hs != sp) throw PimcError(kErrInput, "HMC on an unknown species");
            s.has_hmc = true;
            s.hmc_move = (uint32_t)i;
            s.hmc_eps = moves[i].GetAttribute<double>("step_size", 0.01);
            s.hmc_steps = moves[i].GetAttribute<uint32_t>("n_steps", 10);
            if (!(s.hmc_eps > 0.) || s.hmc_steps < 1 || s.hmc_steps > 100000) throw PimcError(kErrInput, "HMC needs step_size > 0, n_steps >= 1");
        } else {
            throw PimcError(kErrUnsupported, "batched chains take one Bisect move and at most one HMC move");
        }
    }
    if (bisect < 0) throw PimcError(kErrUnsupported, "batched chains need exactly one Bisect move");
    const Input& bm = moves[(size_t)bisect];
    if (bm.GetAttribute<std::string>("species") != sp) throw PimcError(kErrInput, "Bisect on an unknown species");
    if (bm.GetAttribute<bool>("adaptive", false) || bm.GetAttribute<int>("n_images", 0) != 0)
        throw PimcError(kErrUnsupported, "batched Bisect: fixed level, n_images = 0");
    s.n_level = bm.GetAttribute<uint32_t>("n_level");
    if (s.n_level < 1 || s.n_level > kBatchMaxLevels) throw PimcError(kErrUnsupported, "batched Bisect needs 1 <= n_level <= 5");
    if ((1u << s.n_level) > s.n_bead) throw PimcError(kErrInput, "bisection segment longer than the path");
    s.move = (uint32_t)bisect;
    // the HMC force leaves a particle's own term (r = 0) out by the clamp at the table's first point
    if (s.has_hmc && s.has_pair && !(s.r_min > 0.)) throw PimcError(kErrUnsupported, "batched HMC needs a pair table starting at r > 0");
    return s;
}

ChainBatch::ChainBatch(const std::vector<std::string>& xml, const std::string& base_dir, int dev) : device(dev) {
    if (xml.empty()) throw PimcError(kErrArg, "no chains");
    n_chains = (uint32_t)xml.size();
    for (const auto& x : xml) specs.push_back(ParseChain(x, base_dir));  // input errors before any CUDA call
    CudaCheck(cudaSetDevice(device), "cudaSetDevice");
    CudaCheck(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device), "device attribute");
    {
        // Shared memory left for a staged path next to the kernel's static shared memory.
        int optin = 0;
        cudaFuncAttributes fa{};
        CudaCheck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "device attribute");
        CudaCheck(cudaFuncGetAttributes(&fa, BatchSweepKernel), "kernel attributes");
        stage_cap = (size_t)optin > fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
    }
    chains.resize(n_chains);
    uint64_t off = 0;
    for (uint32_t i = 0; i < n_chains; ++i) {
        const ChainSpec& s = specs[i];
        ChainDev& c = chains[i];
        std::memset(&c, 0, sizeof(c));
        c.n_part = s.n_part;
        c.n_bead = s.n_bead;
        c.n_pad = (s.n_part + 7u) & ~7u;
        c.n_level = s.n_level;
        c.seed = s.seed;
        c.chain_id = i;
        c.move = s.move;
        c.pos_off = off;
        off += (uint64_t)c.n_pad * c.n_bead;
        const uint32_t B = 1u << s.n_level;
        c.attempts_per_sweep = (uint64_t)s.n_part * ((s.n_bead + B - 1) / B);
        c.L = (float)s.L;
        c.iL = s.pbc ? (float)(1. / s.L) : 0.f;
        c.lambda = (float)s.lambda;
        c.tau = (float)s.tau;
        for (uint32_t l = 0; l < s.n_level; ++l) {
            const double lt = s.tau * (double)(1u << l);
            c.sigma[l] = (float)std::sqrt(s.lambda * lt);
            c.i4lt_sample[l] = (float)(1. / (4. * s.lambda * 0.5 * lt));
            c.i4lt_level[l] = (float)(1. / (4. * s.lambda * lt));
        }
        c.pbc = s.pbc ? 1 : 0;
        c.has_trap = s.has_trap ? 1 : 0;
        c.has_pair = s.has_pair ? 1 : 0;
        c.trap_max_level = (int32_t)s.trap_max_level;
        const double w2 = s.omega * s.omega, t2 = s.tau * s.tau;
        c.trap_cofa = (float)(0.5 * s.tau * w2 * (1. + t2 * w2 / 12.));  // trap_class.h:14-15
        c.trap_cofb = 0.5 * w2 * (1. + 3. * t2 * w2 / 12.);
        c.r2_min = (float)(s.r_min * s.r_min);
        c.r2_max = (float)(s.r_max * s.r_max);
        c.kin_const = (double)s.n_part * s.n_bead * 3. / (2. * s.tau);  // kinetic_class.h:13
        c.i4ltt = 1. / (4. * s.lambda * s.tau * s.tau);
        if (s.has_hmc) {
            c.hmc_eps = (float)s.hmc_eps;
            c.hmc_steps = s.hmc_steps;
            c.hmc_move = s.hmc_move;
            bead_moves_per_hmc += (uint64_t)s.n_part * s.n_bead;
        }
        bead_moves_per_sweep += c.attempts_per_sweep * (B - 1);
        path_off_.push_back(path_doubles);
        path_doubles += (uint64_t)s.n_part * s.n_bead * 3;
    }
    series_cap = 4096;
    CudaCheck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream create");
    CudaCheck(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking), "stream create");
    CudaCheck(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming), "event create");
    CudaCheck(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming), "event create");
    pos_.reset(new DeviceBuffer(off * sizeof(float4)));
    pos_float4 = off;
    CudaCheck(cudaMemset(pos_->ptr, 0, off * sizeof(float4)), "memset");
    dstage_.reset(new DeviceBuffer(std::max<uint64_t>(path_doubles, 1) * sizeof(double)));
    path_off_dev_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
    CudaCheck(cudaMemcpy(path_off_dev_->ptr, path_off_.data(), n_chains * sizeof(uint64_t), cudaMemcpyHostToDevice), "path offsets");
    last_.reset(new DeviceBuffer((size_t)n_chains * kBatchSeriesComponents * sizeof(double)));
    CudaCheck(cudaMemset(last_->ptr, 0, last_->bytes), "memset");
    chains_dev_.reset(new DeviceBuffer(n_chains * sizeof(ChainDev)));
    order_dev_.reset(new DeviceBuffer(n_chains * sizeof(uint32_t)));
    att_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
    acc_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
    n_meas_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
    series_.reset(new DeviceBuffer((size_t)n_chains * series_cap * kBatchSeriesComponents * sizeof(double)));
    err_.reset(new DeviceBuffer(sizeof(int)));
    rounds_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
    CudaCheck(cudaMemset(rounds_->ptr, 0, n_chains * sizeof(uint64_t)), "memset");
    if (bead_moves_per_hmc) {
        int optin_h = 0;
        cudaFuncAttributes fh{};
        CudaCheck(cudaDeviceGetAttribute(&optin_h, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "device attribute");
        CudaCheck(cudaFuncGetAttributes(&fh, BatchHmcKernel), "kernel attributes");
        hmc_smem_cap = (size_t)optin_h > fh.sharedSizeBytes ? (size_t)optin_h - fh.sharedSizeBytes : 0;
        size_t need = 0;
        for (uint32_t k = 1; k <= 8; k *= 2)
            if (HmcSmem(k) && HmcSmem(k) <= hmc_smem_cap) need = std::max(need, HmcSmem(k));
        if (!need)
            throw PimcError(kErrUnsupported, "a batched HMC chain's path (24 n_part (n_bead / k + 1) bytes per block of a cluster of k <= 8) "
                                             "exceeds the shared memory of one block");
        CudaCheck(cudaFuncSetAttribute(BatchHmcKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need), "smem attribute");
        // Default split: the fewest blocks per chain that still give every SM a few blocks.
        hmc_cluster = 0;
        for (uint32_t k = 1; k <= 8; k *= 2)
            if (HmcClusterFits(k)) {
                hmc_cluster = k;
                if ((uint64_t)n_chains * k >= 4ull * (uint64_t)n_sm) break;
            }
        if (!hmc_cluster) throw PimcError(kErrUnsupported, "no thread-block cluster of 1-8 blocks fits the batched HMC launch");
        hmc_att_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
        hmc_acc_.reset(new DeviceBuffer(n_chains * sizeof(uint64_t)));
        CudaCheck(cudaMemset(hmc_att_->ptr, 0, n_chains * sizeof(uint64_t)), "memset");
        CudaCheck(cudaMemset(hmc_acc_->ptr, 0, n_chains * sizeof(uint64_t)), "memset");
    }
    CudaCheck(cudaMemset(att_->ptr, 0, n_chains * sizeof(uint64_t)), "memset");
    CudaCheck(cudaMemset(acc_->ptr, 0, n_chains * sizeof(uint64_t)), "memset");
    CudaCheck(cudaMemset(n_meas_->ptr, 0, n_chains * sizeof(uint64_t)), "memset");
    CudaCheck(cudaMemset(err_->ptr, 0, sizeof(int)), "memset");
    CudaCheck(cudaStreamSynchronize(cudaStreamLegacy), "memset completion");  // before any work on `stream`
    // Energy tasks: kEnergySlices slices of one chain each, chains in the launch order (most
    // expensive first, as SetTiles orders the blocks), so that a contiguous range of order positions
    // has a contiguous range of tasks.
    order.resize(n_chains);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const double wx = (double)chains[x].attempts_per_sweep * chains[x].n_part;
        const double wy = (double)chains[y].attempts_per_sweep * chains[y].n_part;
        return wx > wy;
    });
    std::vector<EnergyTask> tasks;
    std::vector<uint32_t> first(n_chains + 1, 0);
    for (uint32_t i = 0; i < n_chains; ++i) {
        const uint32_t ci = order[i];
        first[i] = (uint32_t)tasks.size();
        for (uint32_t b0 = 0; b0 < chains[ci].n_bead; b0 += kEnergySlices)
            tasks.push_back(EnergyTask{ci, b0, std::min(kEnergySlices, chains[ci].n_bead - b0), 0});
    }
    first[n_chains] = (uint32_t)tasks.size();
    n_energy_tasks_ = (uint32_t)tasks.size();
    // Shared memory of the largest task: its slices and the next one, N float4 each.
    energy_smem_ = 0;
    for (const auto& t : tasks) energy_smem_ = std::max(energy_smem_, (size_t)(t.nb + 1) * chains[t.chain].n_part * sizeof(float4));
    int optin_e = 0;
    CudaCheck(cudaDeviceGetAttribute(&optin_e, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "device attribute");
    if (energy_smem_ + 4096 > (size_t)optin_e) throw PimcError(kErrUnsupported, "batched chain too large for the energy kernel's shared memory");
    CudaCheck(cudaFuncSetAttribute(BatchEnergyPartKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)energy_smem_), "smem attribute");
    energy_tasks_.reset(new DeviceBuffer(tasks.size() * sizeof(EnergyTask)));
    energy_first_.reset(new DeviceBuffer(first.size() * sizeof(uint32_t)));
    energy_part_.reset(new DeviceBuffer(tasks.size() * 3 * sizeof(float2)));
    CudaCheck(cudaMemcpy(energy_tasks_->ptr, tasks.data(), tasks.size() * sizeof(EnergyTask), cudaMemcpyHostToDevice), "energy tasks");
    CudaCheck(cudaMemcpy(energy_first_->ptr, first.data(), first.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "energy tasks");
    energy_first_host_ = first;
    SetTiles(items_per_lane, max_warps, wave);
}

ChainBatch::~ChainBatch() {
    if (graph_) cudaGraphExecDestroy(graph_);
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    if (ev_join_) cudaEventDestroy(ev_join_);
    if (side_) cudaStreamDestroy(side_);
    if (stream) cudaStreamDestroy(stream);
}

void ChainBatch::ResetGraph() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    graph_sweeps_ = 0;
}

/// Pair tile: chain c gets ceil((N-1)(B-1) / (32 items_per_lane)) warps, at most max_warps.
/// Blocks are ordered by descending work so the longest chains start first.
void ChainBatch::SetTiles(uint32_t ipl, uint32_t mw, uint32_t wave) {
    if (ipl < 1 || mw < 1 || mw > kBatchMaxWarps || wave < 1 || wave > kMaxWave)
        throw PimcError(kErrArg, "tile: items_per_lane >= 1, 1 <= max_warps <= 16, 1 <= wave <= 8");
    items_per_lane = ipl;
    max_warps = mw;
    this->wave = wave;
    for (auto& c : chains) {
        const uint64_t items = (uint64_t)(c.n_part > 1 ? c.n_part - 1 : 1) * ((1u << c.n_level) - 1);
        const uint64_t g = (items + 32ull * ipl - 1) / (32ull * ipl);  // warps one attempt wants
        uint32_t W = wave;
        while (W > 1 && mw / W < 2) --W;  // a concurrent attempt needs a leader and a drawing warp
        if (W > 1) {
            const uint32_t gs = (uint32_t)std::max<uint64_t>(2, std::min<uint64_t>(g, mw / W));
            c.n_wave = W;
            c.sub_warps = gs;
            c.n_warps = W * gs;
            // The path in shared memory (three FP32 planes) when it fits next to the static part and
            // the ring of drawn attempts.
            c.staged = (size_t)12 * c.n_part * c.n_bead + RingBytes(1u << c.n_level, c.n_level) <= stage_cap ? 1u : 0u;
        } else {
            c.n_wave = 1;
            c.n_warps = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(g, mw));
            c.sub_warps = c.n_warps;
            c.staged = 0;
        }
    }
    stage_bytes = 0;
    for (const auto& c : chains)
        if (c.n_wave > 1)
            stage_bytes = std::max(stage_bytes, (c.staged ? (size_t)12 * c.n_part * c.n_bead : 0) + RingBytes(1u << c.n_level, c.n_level));
    stage_bytes = (stage_bytes + 15) & ~size_t(15);
    CudaCheck(cudaFuncSetAttribute(BatchSweepKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_bytes), "smem attribute");
    ApplySplit();  // `order` (most expensive first) was fixed at creation
    Upload();
    ResetGraph();
}

void ChainBatch::Upload() {
    CudaCheck(cudaMemcpyAsync(chains_dev_->ptr, chains.data(), n_chains * sizeof(ChainDev), cudaMemcpyHostToDevice, stream), "upload chains");
    CudaCheck(cudaMemcpyAsync(order_dev_->ptr, order.data(), n_chains * sizeof(uint32_t), cudaMemcpyHostToDevice, stream), "upload order");
    CudaCheck(cudaStreamSynchronize(stream), "sync");
}

void ChainBatch::SetPath(uint32_t chain, const double* p) {
    if (chain >= n_chains || !p) throw PimcError(kErrArg, "bad chain or null path");
    const ChainDev& c = chains[chain];
    std::vector<float4> h((size_t)c.n_bead * c.n_pad, make_float4(0.f, 0.f, 0.f, 0.f));
    for (uint32_t i = 0; i < c.n_part; ++i)
        for (uint32_t b = 0; b < c.n_bead; ++b) {
            const double* r = p + ((size_t)i * c.n_bead + b) * 3;
            if (!std::isfinite(r[0]) || !std::isfinite(r[1]) || !std::isfinite(r[2])) throw PimcError(kErrArg, "non-finite position");
            h[(size_t)b * c.n_pad + i] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.f);
        }
    CudaCheck(cudaMemcpyAsync(pos_->as<float4>() + c.pos_off, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice, stream), "set path");
    CudaCheck(cudaStreamSynchronize(stream), "sync");
}

void ChainBatch::GetPath(uint32_t chain, double* p) {
    if (chain >= n_chains || !p) throw PimcError(kErrArg, "bad chain or null path");
    const ChainDev& c = chains[chain];
    std::vector<float4> h((size_t)c.n_bead * c.n_pad);
    CudaCheck(cudaMemcpyAsync(h.data(), pos_->as<float4>() + c.pos_off, h.size() * sizeof(float4), cudaMemcpyDeviceToHost, stream), "get path");
    CudaCheck(cudaStreamSynchronize(stream), "sync");
    for (uint32_t i = 0; i < c.n_part; ++i)
        for (uint32_t b = 0; b < c.n_bead; ++b) {
            const float4 r = h[(size_t)b * c.n_pad + i];
            double* o = p + ((size_t)i * c.n_bead + b) * 3;
            o[0] = r.x;
            o[1] = r.y;
            o[2] = r.z;
        }
}

/// Every chain's path in one transfer: the caller's doubles are copied as they are (from pinned
/// memory at full link speed) and laid out as float4 on the device.
void ChainBatch::SetPaths(const double* all) {
    if (!all) throw PimcError(kErrArg, "null paths");
    CudaCheck(cudaMemcpyAsync(dstage_->ptr, all, path_doubles * sizeof(double), cudaMemcpyHostToDevice, stream), "set paths");
    CudaCheck(cudaMemsetAsync(err_->ptr, 0, sizeof(int), stream), "clear error");
    HostLayoutToPosKernel<<<n_chains, 256, 0, stream>>>(dstage_->as<double>(), chains_dev_->as<ChainDev>(), path_off_dev_->as<uint64_t>(),
                                                         pos_->as<float4>(), err_->as<int>());
    CudaCheck(cudaGetLastError(), "path layout launch");
    int e = 0;
    CudaCheck(cudaMemcpyAsync(&e, err_->ptr, sizeof(int), cudaMemcpyDeviceToHost, stream), "read error word");
    CudaCheck(cudaStreamSynchronize(stream), "sync");
    if (e & kDevErrNonFinite) {
        CudaCheck(cudaMemsetAsync(err_->ptr, 0, sizeof(int), stream), "clear error");
        CudaCheck(cudaStreamSynchronize(stream), "sync");
        throw PimcError(kErrArg, "non-finite position");
    }
}

void ChainBatch::GetPaths(double* all) {
    if (!all) throw PimcError(kErrArg, "null paths");
    PosToHostLayoutKernel<<<n_chains, 256, 0, stream>>>(pos_->as<float4>(), chains_dev_->as<ChainDev>(), path_off_dev_->as<uint64_t>(),
                                                         dstage_->as<double>());
    CudaCheck(cudaGetLastError(), "path layout launch");
    CudaCheck(cudaMemcpyAsync(all, dstage_->ptr, path_doubles * sizeof(double), cudaMemcpyDeviceToHost, stream), "get paths");
    CudaCheck(cudaStreamSynchronize(stream), "sync");
}

void ChainBatch::LastEnergy(double* out) {
    if (!out) throw PimcError(kErrArg, "null output");
    CudaCheck(cudaMemcpyAsync(out, last_->ptr, last_->bytes, cudaMemcpyDeviceToHost, stream), "last energy");
    Sync();
}

namespace {
BatchArgs MakeArgs(DeviceBuffer& pos, DeviceBuffer& ch, DeviceBuffer& ord, DeviceBuffer& att, DeviceBuffer& acc, DeviceBuffer& ser,
                   DeviceBuffer& nm, DeviceBuffer& last, DeviceBuffer& err, DeviceBuffer& rounds, uint32_t cap) {
    return BatchArgs{pos.as<float4>(), ch.as<ChainDev>(), ord.as<uint32_t>(), att.as<uint64_t>(), acc.as<uint64_t>(),
                     ser.as<double>(), nm.as<uint64_t>(), last.as<double>(), err.as<int>(), rounds.as<uint64_t>(), nullptr, cap};
}
}  // namespace

void ChainBatch::LaunchSweep(uint64_t n_sweeps, uint64_t n_attempts, uint32_t first, uint32_t count, cudaStream_t s) {
    uint32_t warps = 1;
    for (const auto& c : chains) warps = std::max(warps, c.n_warps);
    BatchArgs a = MakeArgs(*pos_, *chains_dev_, *order_dev_, *att_, *acc_, *series_, *n_meas_, *last_, *err_, *rounds_, series_cap);
    if (!s) s = stream;
    count = std::min(count, n_chains - std::min(first, n_chains));
    if (count == 0) return;
    if (n_split_ > 0) {
        if (first != 0 || count != n_chains) throw PimcError(kErrState, "split chains run in the whole-batch launch only");
        // Clusters of two blocks: a split chain on both, otherwise two chains side by side.
        a.cluster_tasks = cluster_tasks_->as<uint2>();
        cudaLaunchAttribute attr{};
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = 2;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(2 * n_clusters_);
        cfg.blockDim = dim3(warps * 32);
        cfg.dynamicSmemBytes = stage_bytes;
        cfg.stream = s;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        CudaCheck(cudaLaunchKernelEx(&cfg, BatchSweepKernel, a, n_sweeps, n_attempts), "batch sweep launch");
    } else {
        a.order = order_dev_->as<uint32_t>() + first;  // blocks run chains order[first .. first + count)
        BatchSweepKernel<<<count, warps * 32, stage_bytes, s>>>(a, n_sweeps, n_attempts);
        CudaCheck(cudaGetLastError(), "batch sweep launch");
    }
    ++kernel_launches;
}

/// The `split` most expensive chains that qualify (a wave tile of 16 warps and a staged path) run on
/// two blocks each with four groups of four warps per block; the others pair up, two chains per
/// cluster, in descending order of work. Called after every tile change.
void ChainBatch::ApplySplit() {
    n_split_ = 0;
    cluster_tasks_host_.clear();
    if (split_request == 0) return;
    std::vector<char> is_split(n_chains, 0);
    for (uint32_t i = 0; i < n_chains && n_split_ < split_request; ++i) {
        ChainDev& c = chains[order[i]];
        if (c.n_wave <= 1 || !c.staged || c.n_warps != kBatchMaxWarps) continue;
        c.n_wave = 4;
        c.sub_warps = 4;
        c.n_warps = 16;
        is_split[order[i]] = 1;
        cluster_tasks_host_.push_back(make_uint2(order[i], order[i]));
        ++n_split_;
    }
    if (n_split_ == 0) return;
    std::vector<uint32_t> rest;
    for (uint32_t i = 0; i < n_chains; ++i)
        if (!is_split[order[i]]) rest.push_back(order[i]);
    for (size_t i = 0; i < rest.size(); i += 2)
        cluster_tasks_host_.push_back(make_uint2(rest[i], i + 1 < rest.size() ? rest[i + 1] : 0xffffffffu));
    n_clusters_ = (uint32_t)cluster_tasks_host_.size();
    if (!cluster_tasks_ || cluster_tasks_->bytes < n_clusters_ * sizeof(uint2)) cluster_tasks_.reset(new DeviceBuffer(n_chains * sizeof(uint2)));
    CudaCheck(cudaMemcpyAsync(cluster_tasks_->ptr, cluster_tasks_host_.data(), n_clusters_ * sizeof(uint2), cudaMemcpyHostToDevice, stream),
              "upload cluster tasks");
    // Every cluster must be schedulable with the launch's shared memory.
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = 2;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(2 * n_clusters_);
    cfg.blockDim = dim3(kBatchMaxWarps * 32);
    cfg.dynamicSmemBytes = stage_bytes;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, BatchSweepKernel, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        throw PimcError(kErrUnsupported, "two-block clusters of the batch sweep do not fit this device");
    }
}

void ChainBatch::SetSplit(uint32_t n) {
    if (n > n_chains) throw PimcError(kErrArg, "more split chains than chains");
    split_request = n;
    SetTiles(items_per_lane, max_warps, wave);
}

size_t ChainBatch::HmcSmem(uint32_t k) const {
    // per block: three R planes of rows padded to an even length with one halo row on each side,
    // three P planes for its own beads
    size_t bytes = 0;
    for (const auto& s : specs) {
        if (!s.has_hmc) continue;
        if (k == 0 || s.n_bead % k != 0) return 0;
        const size_t nb = s.n_bead / k, n2 = s.n_part + (s.n_part & 1u);
        bytes = std::max(bytes, (size_t)12 * n2 * (nb + 2) + (size_t)12 * s.n_part * nb);
    }
    return bytes;
}

bool ChainBatch::HmcClusterFits(uint32_t k) const {
    const size_t smem = HmcSmem(k);
    if (!smem || smem > hmc_smem_cap) return false;
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = k;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.gridDim = dim3(n_chains * k);
    cfg.blockDim = dim3(kHmcThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, BatchHmcKernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return clusters > 0;
}

void ChainBatch::SetHmcCluster(uint32_t k) {
    if (!bead_moves_per_hmc) throw PimcError(kErrState, "no chain of the batch has an HMC move");
    if (k != 1 && k != 2 && k != 4 && k != 8) throw PimcError(kErrArg, "HMC cluster size must be 1, 2, 4 or 8");
    if (!HmcClusterFits(k)) throw PimcError(kErrUnsupported, "this HMC cluster size does not divide every HMC chain's n_bead or does not fit");
    if (k != hmc_cluster) ResetGraph();
    hmc_cluster = k;
}

void ChainBatch::LaunchHmc(uint64_t n_attempts, uint32_t first, uint32_t count, cudaStream_t s) {
    if (!bead_moves_per_hmc) throw PimcError(kErrState, "no chain of the batch has an HMC move");
    BatchArgs a = MakeArgs(*pos_, *chains_dev_, *order_dev_, *att_, *acc_, *series_, *n_meas_, *last_, *err_, *rounds_, series_cap);
    if (!s) s = stream;
    count = std::min(count, n_chains - std::min(first, n_chains));
    if (count == 0) return;
    a.order = order_dev_->as<uint32_t>() + first;  // clusters run chains order[first .. first + count)
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = hmc_cluster;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(count * hmc_cluster);
    cfg.blockDim = dim3(kHmcThreads);
    cfg.dynamicSmemBytes = HmcSmem(hmc_cluster);
    cfg.stream = s;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    for (uint64_t done = 0; done < n_attempts;) {
        const uint32_t k = (uint32_t)std::min<uint64_t>(n_attempts - done, 1u << 20);
        const HmcArgs h{hmc_att_->as<uint64_t>(), hmc_acc_->as<uint64_t>(), k};
        CudaCheck(cudaLaunchKernelEx(&cfg, BatchHmcKernel, a, h), "batch HMC launch");
        ++kernel_launches;
        done += k;
    }
}

void ChainBatch::HmcAttempts(uint64_t n) {
    if (n) LaunchHmc(n);
}

void ChainBatch::ReadHmcCounters(uint64_t* attempts, uint64_t* accepts) {
    if (!bead_moves_per_hmc) throw PimcError(kErrState, "no chain of the batch has an HMC move");
    Sync();
    if (attempts) CudaCheck(cudaMemcpy(attempts, hmc_att_->ptr, n_chains * sizeof(uint64_t), cudaMemcpyDeviceToHost), "read attempts");
    if (accepts) CudaCheck(cudaMemcpy(accepts, hmc_acc_->ptr, n_chains * sizeof(uint64_t), cudaMemcpyDeviceToHost), "read accepts");
}

void ChainBatch::SetHmcPerCycle(uint64_t n) {
    if (n && !bead_moves_per_hmc) throw PimcError(kErrState, "no chain of the batch has an HMC move");
    hmc_per_cycle = n;
}

void ChainBatch::LaunchMeasure(uint32_t i0, uint32_t i1, cudaStream_t s) {
    const BatchArgs a = MakeArgs(*pos_, *chains_dev_, *order_dev_, *att_, *acc_, *series_, *n_meas_, *last_, *err_, *rounds_, series_cap);
    if (!s) s = stream;
    i1 = std::min(i1, n_chains);
    if (i0 >= i1) return;
    const uint32_t t0 = energy_first_host_[i0], t1 = energy_first_host_[i1];
    BatchEnergyPartKernel<<<t1 - t0, kEnergyThreads, energy_smem_, s>>>(a, energy_tasks_->as<EnergyTask>() + t0, energy_part_->as<float2>() + (size_t)t0 * 3);
    CudaCheck(cudaGetLastError(), "batch energy launch");
    BatchEnergyFinishKernel<<<(i1 - i0 + 7) / 8, 256, 0, s>>>(a, energy_first_->as<uint32_t>(), energy_part_->as<float2>(), i0, i1);
    CudaCheck(cudaGetLastError(), "batch energy launch");
    kernel_launches += 2;
}

void ChainBatch::Attempts(uint64_t n) {
    if (n) LaunchSweep(0, n);
}

void ChainBatch::Sweeps(uint64_t n) {
    if (n) LaunchSweep(n, 0);
}

void ChainBatch::Measure() { LaunchMeasure(); }

void ChainBatch::Run(uint64_t n_cycles, uint64_t spm) {
    if (spm == 0) throw PimcError(kErrArg, "sweeps_per_measure must be positive");
    if (!graph_ || graph_sweeps_ != spm || graph_hmc_ != hmc_per_cycle || graph_heavy_ != overlap_heavy) {
        ResetGraph();
        cudaGraph_t g = nullptr;
        CudaCheck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        const uint64_t before = kernel_launches;
        const uint32_t heavy = overlap_heavy;
        try {
            if (hmc_per_cycle && n_split_ == 0 && heavy > 0 && heavy < n_chains) {
                // The heavy chains' sweep and HMC on the main stream, the others' sweep and HMC on
                // the side stream at the same time: a light chain's HMC fills SMs that its sweep left
                // while the heavy sweeps finish. Each chain's own kernels stay in order.
                CudaCheck(cudaEventRecord(ev_fork_, stream), "fork");
                CudaCheck(cudaStreamWaitEvent(side_, ev_fork_, 0), "fork wait");
                LaunchSweep(spm, 0, 0, heavy, stream);
                LaunchSweep(spm, 0, heavy, n_chains - heavy, side_);
                LaunchHmc(hmc_per_cycle, heavy, n_chains - heavy, side_);
                LaunchMeasure(heavy, n_chains, side_);
                LaunchHmc(hmc_per_cycle, 0, heavy, stream);
                LaunchMeasure(0, heavy, stream);
                CudaCheck(cudaEventRecord(ev_join_, side_), "join");
                CudaCheck(cudaStreamWaitEvent(stream, ev_join_, 0), "join wait");
            } else {
                LaunchSweep(spm, 0);
                if (hmc_per_cycle) LaunchHmc(hmc_per_cycle);
                LaunchMeasure();
            }
        } catch (...) {
            // end the capture so the batch's stream takes work again, drop the partial graph
            kernel_launches = before;
            cudaGraph_t partial = nullptr;
            cudaStreamEndCapture(stream, &partial);
            if (partial) cudaGraphDestroy(partial);
            cudaGetLastError();
            throw;
        }
        launches_per_cycle_ = (uint32_t)(kernel_launches - before);
        kernel_launches = before;
        CudaCheck(cudaStreamEndCapture(stream, &g), "end capture");
        const cudaError_t e = cudaGraphInstantiate(&graph_, g, 0);
        cudaGraphDestroy(g);
        CudaCheck(e, "graph instantiate");
        graph_sweeps_ = spm;
        graph_hmc_ = hmc_per_cycle;
        graph_heavy_ = overlap_heavy;
    }
    for (uint64_t i = 0; i < n_cycles; ++i) {
        CudaCheck(cudaGraphLaunch(graph_, stream), "graph launch");
        kernel_launches += launches_per_cycle_;
    }
}

void ChainBatch::Sync() {
    CudaCheck(cudaStreamSynchronize(stream), "sync");
    int e = 0;
    CudaCheck(cudaMemcpy(&e, err_->ptr, sizeof(int), cudaMemcpyDeviceToHost), "read error word");
    if (e & kDevErrNonFinite) throw PimcError(kErrNonFinite, "non-finite energy in a batched chain");
}

uint64_t ChainBatch::ReadEnergy(uint32_t chain, double* out, uint64_t cap) {
    if (chain >= n_chains) throw PimcError(kErrArg, "bad chain");
    Sync();
    uint64_t n = 0;
    CudaCheck(cudaMemcpy(&n, n_meas_->as<uint64_t>() + chain, sizeof(uint64_t), cudaMemcpyDeviceToHost), "read n");
    const uint64_t kept = std::min<uint64_t>(n, series_cap);
    if (out && cap) {
        const uint64_t m = std::min(kept, cap);
        CudaCheck(cudaMemcpy(out, series_->as<double>() + (size_t)chain * series_cap * kBatchSeriesComponents,
                             m * kBatchSeriesComponents * sizeof(double), cudaMemcpyDeviceToHost),
                  "read series");
    }
    return n;
}

void ChainBatch::ResetEnergy() {
    CudaCheck(cudaMemsetAsync(n_meas_->ptr, 0, n_chains * sizeof(uint64_t), stream), "reset");
    CudaCheck(cudaStreamSynchronize(stream), "sync");
}

void ChainBatch::ReadRounds(uint64_t* rounds) {
    Sync();
    CudaCheck(cudaMemcpy(rounds, rounds_->ptr, n_chains * sizeof(uint64_t), cudaMemcpyDeviceToHost), "read rounds");
}

void ChainBatch::ReadCounters(uint64_t* attempts, uint64_t* accepts) {
    Sync();
    if (attempts) CudaCheck(cudaMemcpy(attempts, att_->ptr, n_chains * sizeof(uint64_t), cudaMemcpyDeviceToHost), "read attempts");
    if (accepts) CudaCheck(cudaMemcpy(accepts, acc_->ptr, n_chains * sizeof(uint64_t), cudaMemcpyDeviceToHost), "read accepts");
}

/// Times trial sweeps for every (items_per_lane, max_warps) candidate on a copy of the chains'
/// state, restores the state after each trial and keeps the fastest tile.
double ChainBatch::Autotune(uint32_t trial_sweeps) {
    if (trial_sweeps == 0) trial_sweeps = 1;
    DeviceBuffer pos_save(pos_->bytes), att_save(att_->bytes), acc_save(acc_->bytes), rounds_save(rounds_->bytes);
    auto copy = [&](DeviceBuffer& dst, const DeviceBuffer& src) {
        CudaCheck(cudaMemcpyAsync(dst.ptr, src.ptr, src.bytes, cudaMemcpyDeviceToDevice, stream), "state copy");
    };
    copy(pos_save, *pos_);
    copy(att_save, *att_);
    copy(acc_save, *acc_);
    copy(rounds_save, *rounds_);
    cudaEvent_t e0, e1;
    CudaCheck(cudaEventCreate(&e0), "event");
    CudaCheck(cudaEventCreate(&e1), "event");
    const uint32_t ipls[] = {2, 4, 8};
    const uint32_t mws[] = {4, 8, 16};
    const uint32_t waves[] = {1, 2, 4, 8};
    double best = 1e300;
    uint32_t best_ipl = items_per_lane, best_mw = max_warps, best_wave = wave;
    for (uint32_t wv : waves)
    for (uint32_t ipl : ipls)
        for (uint32_t mw : mws) {
            SetTiles(ipl, mw, wv);
            LaunchSweep(1, 0);  // warm-up of this shape
            CudaCheck(cudaEventRecord(e0, stream), "event");
            LaunchSweep(trial_sweeps, 0);
            CudaCheck(cudaEventRecord(e1, stream), "event");
            CudaCheck(cudaEventSynchronize(e1), "event sync");
            float ms = 0.f;
            CudaCheck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            const double sec = ms * 1e-3 / trial_sweeps;
            if (sec < best) {
                best = sec;
                best_ipl = ipl;
                best_mw = mw;
                best_wave = wv;
            }
            copy(*pos_, pos_save);
            copy(*att_, att_save);
            copy(*acc_, acc_save);
            copy(*rounds_, rounds_save);
        }
    SetTiles(best_ipl, best_mw, best_wave);
    {
        // chains split over two-block clusters: none, or the 8, 16, 32 most expensive
        double best_s = best;
        uint32_t best_n = split_request;
        for (uint32_t n : {0u, 8u, 16u, 32u}) {
            if (n > n_chains) continue;
            SetSplit(n);
            if (n > 0 && n_split_ == 0) continue;
            LaunchSweep(1, 0);  // warm-up of this shape
            CudaCheck(cudaEventRecord(e0, stream), "event");
            LaunchSweep(trial_sweeps, 0);
            CudaCheck(cudaEventRecord(e1, stream), "event");
            CudaCheck(cudaEventSynchronize(e1), "event sync");
            float ms = 0.f;
            CudaCheck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            const double sec = ms * 1e-3 / trial_sweeps;
            if (n == 0 || sec < best_s) {
                best_s = sec;
                best_n = n;
            }
            copy(*pos_, pos_save);
            copy(*att_, att_save);
            copy(*acc_, acc_save);
            copy(*rounds_, rounds_save);
        }
        SetSplit(best_n);
        best = best_s;
    }
    if (bead_moves_per_hmc) {
        // blocks per chain of the HMC launch: one attempt per trial, the state put back after each
        DeviceBuffer hatt_save(hmc_att_->bytes), hacc_save(hmc_acc_->bytes);
        copy(hatt_save, *hmc_att_);
        copy(hacc_save, *hmc_acc_);
        float best_h = 1e30f;
        uint32_t best_k = hmc_cluster;
        for (uint32_t k = 1; k <= 8; k *= 2) {
            if (!HmcClusterFits(k)) continue;
            SetHmcCluster(k);
            LaunchHmc(1);  // warm-up of this shape
            CudaCheck(cudaEventRecord(e0, stream), "event");
            LaunchHmc(1);
            CudaCheck(cudaEventRecord(e1, stream), "event");
            CudaCheck(cudaEventSynchronize(e1), "event sync");
            float ms = 0.f;
            CudaCheck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            if (ms < best_h) {
                best_h = ms;
                best_k = k;
            }
            copy(*pos_, pos_save);
            copy(*hmc_att_, hatt_save);
            copy(*hmc_acc_, hacc_save);
        }
        SetHmcCluster(best_k);
        CudaCheck(cudaStreamSynchronize(stream), "sync");
        if (n_split_ == 0) {
            // The measurement cycle with the heaviest H chains beside the others (H = 0: one stream).
            DeviceBuffer meas_save(n_meas_->bytes), last_save(last_->bytes);
            copy(hatt_save, *hmc_att_);
            copy(hacc_save, *hmc_acc_);
            copy(meas_save, *n_meas_);
            copy(last_save, *last_);
            const uint64_t hpc = hmc_per_cycle;
            hmc_per_cycle = 1;
            float best_c = 1e30f;
            uint32_t best_h = 0;
            for (uint32_t eighths = 0; eighths <= 5; ++eighths) {  // H = 0, n/8, ..., 5n/8
                const uint32_t hv = n_chains * eighths / 8;
                if (eighths > 0 && (hv == 0 || hv >= n_chains)) continue;
                overlap_heavy = hv;
                Run(1, 1);  // builds the cycle's graph
                // the median of five single cycles: two streams schedule differently from run to run
                float cyc[5];
                for (float& ms : cyc) {
                    CudaCheck(cudaEventRecord(e0, stream), "event");
                    Run(1, 1);
                    CudaCheck(cudaEventRecord(e1, stream), "event");
                    CudaCheck(cudaEventSynchronize(e1), "event sync");
                    CudaCheck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                }
                std::sort(cyc, cyc + 5);
                const float ms = cyc[2];
                if (ms < best_c) {
                    best_c = ms;
                    best_h = hv;
                }
                copy(*pos_, pos_save);
                copy(*att_, att_save);
                copy(*acc_, acc_save);
                copy(*rounds_, rounds_save);
                copy(*hmc_att_, hatt_save);
                copy(*hmc_acc_, hacc_save);
                copy(*n_meas_, meas_save);
                copy(*last_, last_save);
            }
            hmc_per_cycle = hpc;
            overlap_heavy = best_h;
            ResetGraph();
            CudaCheck(cudaStreamSynchronize(stream), "sync");
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CudaCheck(cudaStreamSynchronize(stream), "sync");
    return best;
}

}  // namespace pimc

// ---------------------------------------------------------------------------------------------
// C interface.

struct pimc_batch {
    std::unique_ptr<pimc::ChainBatch> b;
    std::string err;
};

namespace {
thread_local std::string g_batch_create_error;

template <class F>
int BatchGuard(pimc_batch* h, F f) {
    if (!h || !h->b) return PIMC_ERR_ARG;
    try {
        f(*h->b);
        return PIMC_OK;
    } catch (const pimc::PimcError& e) {
        h->err = e.what();
        return e.code;
    } catch (const pimc::InputError& e) {
        h->err = e.what();
        return PIMC_ERR_INPUT;
    } catch (const std::exception& e) {
        h->err = e.what();
        return PIMC_ERR_STATE;
    }
}
}  // namespace

extern "C" {

int pimc_batch_create(const char* const* xml_texts, uint32_t n_chains, const char* base_dir, int device, pimc_batch** out) {
    if (!xml_texts || !out || n_chains == 0) return PIMC_ERR_ARG;
    *out = nullptr;
    try {
        std::vector<std::string> xml;
        for (uint32_t i = 0; i < n_chains; ++i) {
            if (!xml_texts[i]) return PIMC_ERR_ARG;
            xml.emplace_back(xml_texts[i]);
        }
        auto* h = new pimc_batch();
        try {
            h->b.reset(new pimc::ChainBatch(xml, base_dir ? base_dir : "", device));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return PIMC_OK;
    } catch (const pimc::PimcError& e) {
        g_batch_create_error = e.what();
        return e.code;
    } catch (const pimc::InputError& e) {
        g_batch_create_error = e.what();
        return PIMC_ERR_INPUT;
    } catch (const std::exception& e) {
        g_batch_create_error = e.what();
        return PIMC_ERR_STATE;
    }
}

void pimc_batch_destroy(pimc_batch* b) { delete b; }

const char* pimc_batch_last_error(const pimc_batch* b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

int pimc_batch_chain_info(pimc_batch* h, uint32_t chain, uint32_t* out4) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (chain >= b.n_chains || !out4) throw pimc::PimcError(pimc::kErrArg, "bad chain or null output");
        const auto& c = b.chains[chain];
        out4[0] = c.n_part;
        out4[1] = c.n_bead;
        out4[2] = c.n_level;
        out4[3] = c.n_warps;
    });
}

int pimc_batch_set_path(pimc_batch* h, uint32_t chain, const double* pos) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.SetPath(chain, pos); });
}

int pimc_batch_get_path(pimc_batch* h, uint32_t chain, double* pos) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.GetPath(chain, pos); });
}

int pimc_batch_set_paths(pimc_batch* h, const double* all) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.SetPaths(all); });
}

int pimc_batch_get_paths(pimc_batch* h, double* all) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.GetPaths(all); });
}

int pimc_batch_last_energy(pimc_batch* h, double* out) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.LastEnergy(out); });
}

int pimc_batch_attempts(pimc_batch* h, uint64_t n) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.Attempts(n); });
}

int pimc_batch_sweeps(pimc_batch* h, uint64_t n) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.Sweeps(n); });
}

int pimc_batch_measure(pimc_batch* h) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.Measure(); });
}

int pimc_batch_run(pimc_batch* h, uint64_t n_cycles, uint64_t sweeps_per_measure) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.Run(n_cycles, sweeps_per_measure); });
}

int pimc_batch_sync(pimc_batch* h) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.Sync(); });
}

int pimc_batch_energy(pimc_batch* h, uint32_t chain, double* out, uint64_t cap, uint64_t* n_measure) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        const uint64_t n = b.ReadEnergy(chain, out, cap);
        if (n_measure) *n_measure = n;
    });
}

int pimc_batch_reset_energy(pimc_batch* h) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.ResetEnergy(); });
}

int pimc_batch_counters(pimc_batch* h, uint64_t* attempts, uint64_t* accepts) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.ReadCounters(attempts, accepts); });
}

int pimc_batch_set_overlap(pimc_batch* h, uint32_t heavy) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (heavy > b.n_chains) throw pimc::PimcError(pimc::kErrArg, "more heavy chains than chains");
        b.overlap_heavy = heavy;
    });
}

int pimc_batch_get_overlap(pimc_batch* h, uint32_t* heavy) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (!heavy) throw pimc::PimcError(pimc::kErrArg, "null output");
        *heavy = b.overlap_heavy;
    });
}

int pimc_batch_set_split(pimc_batch* h, uint32_t n) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.SetSplit(n); });
}

int pimc_batch_get_split(pimc_batch* h, uint32_t* n) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (!n) throw pimc::PimcError(pimc::kErrArg, "null output");
        *n = b.n_split_;
    });
}

int pimc_batch_rounds(pimc_batch* h, uint64_t* rounds) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (!rounds) throw pimc::PimcError(pimc::kErrArg, "null output");
        b.ReadRounds(rounds);
    });
}

int pimc_batch_hmc_attempts(pimc_batch* h, uint64_t n) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.HmcAttempts(n); });
}

int pimc_batch_hmc_counters(pimc_batch* h, uint64_t* attempts, uint64_t* accepts) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.ReadHmcCounters(attempts, accepts); });
}

int pimc_batch_set_hmc_per_cycle(pimc_batch* h, uint64_t n) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.SetHmcPerCycle(n); });
}

int pimc_batch_set_hmc_cluster(pimc_batch* h, uint32_t k) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.SetHmcCluster(k); });
}

int pimc_batch_get_hmc_cluster(pimc_batch* h, uint32_t* k) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (!k) throw pimc::PimcError(pimc::kErrArg, "null output");
        if (!b.bead_moves_per_hmc) throw pimc::PimcError(pimc::kErrState, "no chain of the batch has an HMC move");
        *k = b.hmc_cluster;
    });
}

int pimc_batch_set_tiles(pimc_batch* h, uint32_t items_per_lane, uint32_t max_warps, uint32_t wave) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) { b.SetTiles(items_per_lane, max_warps, wave); });
}

int pimc_batch_autotune(pimc_batch* h, uint32_t trial_sweeps, uint32_t* items_per_lane, uint32_t* max_warps, uint32_t* wave,
                        double* sec_per_sweep) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        const double s = b.Autotune(trial_sweeps);
        if (items_per_lane) *items_per_lane = b.items_per_lane;
        if (max_warps) *max_warps = b.max_warps;
        if (wave) *wave = b.wave;
        if (sec_per_sweep) *sec_per_sweep = s;
    });
}

int pimc_batch_stats(pimc_batch* h, uint64_t* out4) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (!out4) throw pimc::PimcError(pimc::kErrArg, "null output");
        out4[0] = b.n_chains;
        out4[1] = b.bead_moves_per_sweep;
        out4[2] = b.kernel_launches;
        out4[3] = b.series_cap;
    });
}

int pimc_batch_stream(pimc_batch* h, void** stream) {
    return BatchGuard(h, [&](pimc::ChainBatch& b) {
        if (!stream) throw pimc::PimcError(pimc::kErrArg, "null output");
        *stream = (void*)b.stream;
    });
}

}  // extern "C"
