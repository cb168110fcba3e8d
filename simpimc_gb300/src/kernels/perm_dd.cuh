// Bisection moves of species whose paths exchange, in double-float: PermBisectIterative,
// PermBisectTable and the plain Bisect on a species that carries a path permutation
// (src/events/moves/single_species_move/bisect/perm_bisect/perm_bisect_class.h:7-133,
// perm_bisect_iterative_class.h:7-231, perm_bisect_table_class.h:7-240, bisect_class.h:39-139).
// Included by sweep.cu, whose double-float move and pair descriptors and helpers it uses; GB300
// issues FP64 at 1/64 of the FP32 rate, and a kernel whose phases each hold a few dependent FP64
// chains spends most of its time waiting on them.
//
// Representation. The reference links beads by pointers and relabels them after an accepted
// permutation (AssignParticleLabels, perm_bisect_class.h:47-56), so between moves every link keeps
// its particle label except at the ring closure. That closure is the array perm: bead (g, M - 1) is
// followed by bead (perm[g], 0); perm_inv is its inverse. A segment of particle p that passes the
// closure continues on perm[p]. During an attempt the cycle's new links (bead B - 1 of path i to the
// old end bead of path sigma(i)) and the proposed positions live in scratch; the committed
// double-float positions are only written on acceptance.
//
// Action changes. Kinetic links follow the paths (kinetic_class.h:105-122; a segment of the whole
// ring whose end bead is its start bead has no link in that mode). The trap and the Ewald part are
// sums over beads of the label-indexed particle list (trap_class.h:37-61,
// bare_pair_action_class.h:126-144); every moved bead lies on a listed label, so their changes are
// sums over the moved beads. The short-range pair actions are evaluated link by link over the
// list's labels as PairAction::GetAction does (pair_action_class.h:267-302, Path::DrDrpDrrp
// path_class.h:137-150): under periodic boundaries r' is the image nearest r, and the
// off-diagonal links keep the reference's label pairing across the permuted link.
//
// Weight table: t = exp(ex) with ex = -|r_i - r_j'|^2 / (4 lambda tau B) (relative to the
// identity for the table variant). exp in double-float reduces the argument by ln 2 and sums the
// Taylor series to the 14th power; a cycle's log weight is the sum of its exponents.
//
// One CTA runs the attempts of one move of one chain in order (PermBisectKernelDD, 256 threads;
// PermChainsKernelDD runs one chain per CTA of 128 threads, four per SM); the weight table, cycle
// weights, midpoints, links, beads and density changes are spread over the threads; the cycle
// walk runs on one warp (row sums by a warp reduction, the choice by a warp scan, in double-float;
// each decision compares the quantities the reference's loop compares); block sums are formed in
// a fixed order. Random numbers follow the block layout of the oracle's PermBisect (seed, chain,
// move, attempt) streams. No wait spins; every loop is bounded.

constexpr int kPermThreads = 256;
constexpr int kPermChainThreads = 128;  // many-chain launches: smaller CTAs, four per SM
constexpr uint32_t kPermMaxPart = 512;      // particles of an exchanging species
constexpr uint32_t kPermCycleCache = 4096;  // table cycles whose weights stay in shared memory
constexpr uint32_t kPermTabShared = 64;     // the walk's weight tables stay in shared memory up to N = 64
constexpr uint32_t kPermSegCap = 512;       // path beads (n (B + 1)) kept in shared memory
constexpr uint32_t kPermZCap = 512;         // midpoints (n (B - 1)) whose normals are drawn up front
constexpr int kPermVariantBisect = 0, kPermVariantIterative = 1, kPermVariantTable = 2;

/// Byte offsets of the kernel's dynamic shared memory: per-particle index arrays [11 N] uint32,
/// the walk's rows [2 N] and the table slices [6 N] float2, the cycle weights, the walk's weight
/// tables [2 N^2] float2, the old and new path beads [2 x 3 seg_cap] float2, the normals
/// [3 z_cap] float and the phase rows [6 stride] ddc.
struct PermSmem {
    size_t row, slices, cyc, tab, seg_old, seg_new, z, ph, total;
};
/// Path beads and midpoints a move can stage: its longest cycle (1 for the bisection, the table's
/// particle count, N for the walk) times B + 1 and B - 1, capped.
__host__ __device__ inline uint32_t PermSegCap(int variant, uint32_t N, uint32_t k_part, uint32_t B) {
    const uint32_t n_max = variant == kPermVariantBisect ? 1u : (variant == kPermVariantTable ? k_part : N);
    return n_max * (B + 1u) < kPermSegCap ? n_max * (B + 1u) : kPermSegCap;
}
__host__ __device__ inline uint32_t PermZCap(int variant, uint32_t N, uint32_t k_part, uint32_t B) {
    const uint32_t n_max = variant == kPermVariantBisect ? 1u : (variant == kPermVariantTable ? k_part : N);
    return n_max * (B - 1u) < kPermZCap ? n_max * (B - 1u) : kPermZCap;
}

__host__ __device__ inline PermSmem PermLayout(uint32_t N, uint32_t cyc_shared, bool tab_shared, uint32_t stride, uint32_t seg_cap,
                                               uint32_t z_cap) {
    PermSmem o;
    size_t at = (size_t)N * 11 * 4;
    at = (at + 15) & ~(size_t)15;
    o.row = at;
    at += (size_t)2 * N * 8;
    o.slices = at;
    at += (size_t)6 * N * 8;
    o.cyc = at;
    at += (size_t)cyc_shared * 8;
    o.tab = at;
    at += tab_shared ? (size_t)2 * N * N * 8 : 0;
    o.seg_old = at;
    at += (size_t)3 * seg_cap * 8;
    o.seg_new = at;
    at += (size_t)3 * seg_cap * 8;
    o.z = at;
    at += (size_t)3 * z_cap * 4;
    at = (at + 15) & ~(size_t)15;
    o.ph = at;
    at += (size_t)6 * stride * sizeof(ddc);
    o.total = at;
    return o;
}

struct PermArgsDD {
    uint32_t n_d, M, n_pad, K;
    dd L, iL, tau, two_pi, ln2, i4B, eps;
    float log_eps;
    uint32_t sp_off[kMaxSpecies], sp_n[kMaxSpecies];
    int32_t sp_rho[kMaxSpecies];
    int32_t max_index[3];
    float2* pos;              // committed positions [M][3][n_pad]
    float4* rho;              // densities [slots][M][K] (64-bit mode)
    float2* rho32;            // FP32 mode: densities [slots][M][K]; drho then holds float2 [B][K]
    const int32_t* kidx;
    const float4* phase256;
    const MoveDD* mv;
    const PairDD* pairs;
    int variant;
    uint32_t seed, chain, move_index, n_attempts;
    uint64_t attempt0;
    uint32_t k_part, n_comb, n_types;
    const uint32_t* combs;    // [n_comb][k_part]
    const uint32_t* types;    // [n_types][k_part]
    float2* ex;               // [N][N] exponents
    float2* tg;               // [2][N][N] weight tables when not in shared memory
    float2* seg_old_g;        // [N][B + 1][3] old path beads when not in shared memory
    float2* cw;               // [n_cycles] cycle weights (when not in shared memory)
    float2* cwl;              // [n_cycles] cycle log weights
    float2* ccon;             // [n_cycles] running sums of the kept cycles
    uint32_t* cidx;           // [n_cycles] kept cycle indices
    float2* prop;             // [N][B + 1][3] proposed positions per path and offset
    float4* drho;             // [B][K] density change per offset
    float2* hold;             // [N][M][3] relabelling buffer
    uint32_t* perm;
    uint32_t* perm_inv;
    unsigned long long* counters;  // accepts, level-0 tests, per cycle length attempts [N], accepts [N]
    int* err;
};

struct PermSharedDD {
    uint32_t n, bead0, p_first, nlist;
    int decide, overflow;
    Philox4 w0;
    dd prev0, tot0;
    float lu[kMaxLevels];
    dd lvl[kMaxLevels][3][kPermThreads / 32];  // per level: old / new sampling log densities, action change; per warp
    dd inv_fact[15];
};

/// exp(x) in double-float for |x| < 80: x = k ln 2 + r with |r| <= ln 2 / 2, exp(r) by its Taylor
/// series to r^14 / 14! (Horner), then scaled by 2^k.
__device__ __forceinline__ dd ExpDD(dd x, dd ln2, const dd* inv_fact) {
    const float k = rintf(__fmul_rn(x.hi, 1.44269504f));
    const dd r = Sub(x, MulF(ln2, k));
    dd p = inv_fact[14];
    for (int n = 13; n >= 0; --n) p = Add(inv_fact[n], Mul(r, p));
    const int ki = (int)k;
    return dd{ldexpf(p.hi, ki), ldexpf(p.lo, ki)};
}

__device__ __forceinline__ dd LoadPos(const float2* pos, uint32_t np, uint32_t b, uint32_t d, uint32_t g) {
    return LoadDD(&pos[((size_t)b * 3 + d) * np + g]);
}

/// Free-particle log density of a displacement: -|dr|^2 i4 - images (free_spline_class.h:76-84).
__device__ __forceinline__ dd LogRhoFreeDD(const dd* dr, uint32_t n_d, dd i4, const CubicDD* image, int has_images) {
    dd q{0.f, 0.f};
    for (uint32_t d = 0; d < n_d; ++d) q = Add(q, Sqr(dr[d]));
    dd v = Mul(q, i4);
    if (has_images) v = Add(v, ImageSum(*image, dr, n_d));
    return Neg(v);
}

/// Path::DrDrpDrrp (path_class.h:137-150): |r|, |r'| (r' the image nearest r) and s = |r - r'|.
__device__ __forceinline__ void DrDrpDrrpDD(const dd* A0, const dd* C0, const dd* A1, const dd* C1, uint32_t n_d, dd L, dd iL, dd& r,
                                            dd& rp, dd& s) {
    dd a{0.f, 0.f}, b{0.f, 0.f}, c{0.f, 0.f};
    for (uint32_t d = 0; d < n_d; ++d) {
        const dd rv = MinImageDD(Sub(A0[d], C0[d]), L, iL);
        dd rq = Sub(A1[d], C1[d]);
        const float n = Rint(Mul(Sub(rv, rq), iL));
        if (n != 0.f) rq = Add(rq, MulF(L, n));
        a = Add(a, Sqr(rv));
        b = Add(b, Sqr(rq));
        c = Add(c, Sqr(MinImageDD(Sub(rv, rq), L, iL)));
    }
    r = Sqrt(a);
    rp = Sqrt(b);
    s = Sqrt(c);
}

/// CalcU of one link (bare_pair_action_class.h:146-150 with level_tau; ilkka_pair_action_class.h:77-101;
/// david_pair_action_class.h:69-102).
__device__ __forceinline__ dd PairUDD(const PairDD& pa, dd r, dd rp, dd s, int level, dd tau) {
    if (pa.kind == kPairDavid) {  // the table u_kj(level)
        const int base = level * (int)pa.kj_stride;
        dd u0, u1;
        const int i0 = MultiIntervalDD(pa.u_kj, r, u0), i1 = MultiIntervalDD(pa.u_kj, rp, u1);
        dd f = Scale2(Add(MultiCompDD(pa.u_kj, i0, u0, base + 1), MultiCompDD(pa.u_kj, i1, u1, base + 1)), 0.5f);
        const dd q = Scale2(Add(r, rp), 0.5f);
        if (s.hi > 0.f && Less(q, pa.u_kj.x1)) f = Add(f, DavidOffDiagDD(pa, q, Sub(r, rp), s, base));
        return f;
    }
    if (pa.kind == kPairIlkka) {
        const dd q = Scale2(Add(r, rp), 0.5f), hs = Scale2(s, 0.5f);
        dd u = EvalBicubicDD(pa.u_xy, Add(q, hs), Sub(q, hs));
        if (pa.use_lr) {
            u = Sub(u, Scale2(EvalCubicDD(pa.u_long_r, Min(Max(r, pa.rumin), pa.rumax)), 0.5f));
            u = Sub(u, Scale2(EvalCubicDD(pa.u_long_r, Min(Max(rp, pa.rumin), pa.rumax)), 0.5f));
        }
        return u;
    }
    return level == 0 ? Mul(tau, PairVDD(pa, r, rp)) : dd{0.f, 0.f};
}

// The weight table of an end map: ex[i][j] = -|r_i - r_end(j)|^2 i4B (minus the same for end(i)
// when relative), t = exp(ex) above log epsilon and zero below. s0 holds the start beads [N][3],
// sE the beads at the end slice [N][3] by label; the end of particle j is its label there after
// the closure, or endmap[m] for cycle member m.
__device__ void BuildTableDD(const PermArgsDD& a, uint32_t N, uint32_t G0, uint32_t B, uint32_t tcross, bool relative, const int* lo_idx,
                             const uint32_t* endmap, const dd* inv_fact, const float2* s0, const float2* sE, float2* tt, float2* ttc,
                             int* overflow) {
    const uint32_t nd = a.n_d;
    auto end_of = [&](uint32_t j) -> uint32_t {
        const int m = endmap ? lo_idx[j] : -1;
        if (m >= 0) return endmap[m] - G0;
        return B >= tcross ? a.perm[G0 + j] - G0 : j;
    };
    for (uint32_t it = threadIdx.x; it < N * N; it += blockDim.x) {
        const uint32_t i = it / N, j = it % N, ej = end_of(j);
        dd dij{0.f, 0.f}, dii{0.f, 0.f};
        const uint32_t ei = relative ? end_of(i) : 0u;
        for (uint32_t d = 0; d < nd; ++d) {
            const dd ri = LoadDD(&s0[3 * i + d]);
            dij = Add(dij, Sqr(MinImageDD(Sub(ri, LoadDD(&sE[3 * ej + d])), a.L, a.iL)));
            if (relative) dii = Add(dii, Sqr(MinImageDD(Sub(ri, LoadDD(&sE[3 * ei + d])), a.L, a.iL)));
        }
        const dd e = relative ? Mul(Sub(dii, dij), a.i4B) : Neg(Mul(dij, a.i4B));
        dd v{0.f, 0.f};
        if (e.hi > a.log_eps) {
            if (e.hi > 80.f) atomicExch(overflow, 1);
            v = ExpDD(e.hi > 80.f ? DD(80.f) : e, a.ln2, inv_fact);
        }
        tt[it] = make_float2(v.hi, v.lo);
        a.ex[it] = make_float2(e.hi, e.lo);
        if (ttc) ttc[it] = make_float2(v.hi, v.lo);
    }
}

// Cycle weights (perm_bisect_table_class.h:15-26) and log weights of the table.
__device__ void CycleWeightsDD(const PermArgsDD& a, uint32_t N, const float2* tt, float2* cw) {
    const uint32_t n_cycles = a.n_comb * a.n_types, k = a.k_part;
    for (uint32_t c = threadIdx.x; c < n_cycles; c += blockDim.x) {
        const uint32_t* part = a.combs + (size_t)(c % a.n_comb) * k;
        const uint32_t* pm = a.types + (size_t)(c / a.n_comb) * k;
        dd w = DD(1.f), lw{0.f, 0.f};
        for (uint32_t i = 0; i < k; ++i) {
            const size_t ij = (size_t)part[i] * N + part[pm[i]];
            w = Mul(w, LoadDD(&tt[ij]));
            lw = Add(lw, LoadDD(&a.ex[ij]));
        }
        cw[c] = make_float2(w.hi, w.lo);
        a.cwl[c] = make_float2(lw.hi, lw.lo);
    }
}

/// The attempts attempt0 .. attempt0 + n_attempts - 1 of one move of one chain, by the whole CTA.
/// Word copy of a descriptor into shared memory by the whole CTA (the caller synchronises).
__device__ __forceinline__ void CopyToShared(void* dst, const void* src, size_t bytes) {
    uint32_t* d = static_cast<uint32_t*>(dst);
    const uint32_t* s = static_cast<const uint32_t*>(src);
    for (size_t i = threadIdx.x; i < bytes / 4; i += blockDim.x) d[i] = s[i];
}

__device__ void PermRun(const PermArgsDD& a_in, uint64_t attempt0, uint32_t n_attempts, unsigned char* dyn, PermSharedDD& sh) {
    // The arguments, the move descriptor and its pair descriptors in shared memory: the phases of an
    // attempt read them on their dependent chains.
    // (raw storage for the descriptors: their members have initialisers, which __shared__ cannot run)
    __shared__ PermArgsDD s_args;
    __shared__ __align__(16) unsigned char s_mv_raw[sizeof(MoveDD)];
    __shared__ __align__(16) unsigned char s_pairs_raw[sizeof(PairDD) * kMaxPair];
    MoveDD& s_mv = *reinterpret_cast<MoveDD*>(s_mv_raw);
    PairDD* s_pairs = reinterpret_cast<PairDD*>(s_pairs_raw);
    __syncthreads();  // the previous entry of a many-chain schedule is done with them
    CopyToShared(&s_args, &a_in, sizeof(PermArgsDD));
    CopyToShared(&s_mv, a_in.mv, sizeof(MoveDD));
    __syncthreads();
    for (int i = 0; i < s_mv.n_pair; ++i) CopyToShared(&s_pairs[i], a_in.pairs + s_mv.pair[i], sizeof(PairDD));
    const PermArgsDD& a = s_args;
    const MoveDD& mv = s_mv;
    const uint32_t sp = mv.species, N = a.sp_n[sp], G0 = a.sp_off[sp], M = a.M, nd = a.n_d, np = a.n_pad, K = a.K;
    const uint32_t B = 1u << mv.n_level;
    const int slot = a.sp_rho[sp];
    const uint32_t stride = (uint32_t)max(max(a.max_index[0], a.max_index[1]), a.max_index[2]) + 1u;
    const uint32_t n_cycles = a.n_comb * a.n_types;
    const bool cw_shared = a.variant == kPermVariantTable && n_cycles <= kPermCycleCache;
    const bool tab_shared = a.variant == kPermVariantIterative && N <= kPermTabShared;
    const uint32_t seg_cap = PermSegCap(a.variant, N, a.k_part, B), z_cap = PermZCap(a.variant, N, a.k_part, B);
    const PermSmem L = PermLayout(N, cw_shared ? n_cycles : 0u, tab_shared, stride, seg_cap, z_cap);
    int* lo_idx = reinterpret_cast<int*>(dyn);  // path of a start label
    int* hi_idx = lo_idx + N;                   // path of a label past the closure
    int* lpos = hi_idx + N;                     // place in the particle list
    uint32_t* part = reinterpret_cast<uint32_t*>(lpos + N);
    uint32_t* sigma = part + N;
    uint32_t* lab_lo = sigma + N;
    uint32_t* lab_hi = lab_lo + N;
    uint32_t* end_old = lab_hi + N;
    uint32_t* end_new = end_old + N;
    uint32_t* lst = end_new + N;  // [2N]
    float2* row = reinterpret_cast<float2*>(dyn + L.row);
    float2* s0 = reinterpret_cast<float2*>(dyn + L.slices);  // start slice [N][3]
    float2* sE = s0 + 3 * N;                                 // end slice [N][3], committed
    float2* cw = cw_shared ? reinterpret_cast<float2*>(dyn + L.cyc) : a.cw;
    float2* tt = tab_shared ? reinterpret_cast<float2*>(dyn + L.tab) : a.tg;
    float2* ttc = tt + (size_t)N * N;
    float* zb = reinterpret_cast<float*>(dyn + L.z);
    ddc* ph = reinterpret_cast<ddc*>(dyn + L.ph);
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) lo_idx[i] = hi_idx[i] = lpos[i] = -1;
    if (threadIdx.x == 0) {
        sh.inv_fact[0] = DD(1.f);
        for (int n = 1; n < 15; ++n) sh.inv_fact[n] = Div(sh.inv_fact[n - 1], DD((float)n));
        sh.overflow = 0;
    }
    const uint32_t base_m = a.variant == kPermVariantBisect ? 1u : 1u + N;
    const uint32_t base_u = a.variant == kPermVariantBisect ? 1u + (B - 1u) : base_m + N * (B - 1u);
    __syncthreads();

    for (uint32_t at = 0; at < n_attempts; ++at) {
        const MoveStream st{a.seed, a.chain, a.move_index, attempt0 + at};
        if (threadIdx.x == 0) {
            const Philox4 w0 = st.Block(0);
            sh.w0 = w0;
            if (a.variant == kPermVariantBisect) {
                sh.p_first = UniformIndex(w0.v[0], N);
                sh.bead0 = UniformIndex(w0.v[1], M);
            } else {
                sh.bead0 = UniformIndex(w0.v[0], M);
                sh.p_first = UniformIndex(w0.v[1], N);
            }
        }
        // the level tests' uniforms, drawn up front (bisect_class.h:113)
        if (threadIdx.x >= 32 && threadIdx.x < 32 + mv.n_level) {
            const uint32_t li = threadIdx.x - 32;
            sh.lu[li] = LogF(U24(st.Block(base_u + li).v[0]));
        }
        __syncthreads();
        const uint32_t bead0 = sh.bead0, tcross = M - bead0, es = (bead0 + B) % M;

        // ---- cycle selection ----
        if (a.variant != kPermVariantBisect) {
            for (uint32_t it = threadIdx.x; it < N * nd; it += blockDim.x) {
                const uint32_t j = it / nd, d = it % nd;
                s0[3 * j + d] = a.pos[((size_t)bead0 * 3 + d) * np + G0 + j];
                sE[3 * j + d] = a.pos[((size_t)es * 3 + d) * np + G0 + j];
            }
            __syncthreads();
            BuildTableDD(a, N, G0, B, tcross, a.variant == kPermVariantTable, lo_idx, nullptr, sh.inv_fact, s0, sE, tt,
                         a.variant == kPermVariantIterative ? ttc : nullptr, &sh.overflow);
            __syncthreads();
            if (a.variant == kPermVariantTable) {
                CycleWeightsDD(a, N, tt, cw);
                __syncthreads();
            }
            if (a.variant == kPermVariantIterative && threadIdx.x < 32) {
                // perm_bisect_iterative_class.h:32-110 on warp 0. The row sums and the running sum of
                // the choice are formed by the lanes (chunks, then a warp scan) in double-float;
                // every decision compares the same quantities as the reference's loop.
                const uint32_t lane = threadIdx.x, p0 = sh.p_first, c = (N + 31u) / 32u;
                const uint32_t i0 = min(N, lane * c), i1 = min(N, i0 + c);
                uint32_t p = p0, n = 0;
                bool ok = false;
                for (uint32_t step = 0; step < N; ++step) {
                    if (lane == 0) part[n] = p;
                    ++n;
                    __syncwarp();
                    float2* trow = tt + (size_t)p * N;
                    float2* crow = ttc + (size_t)p * N;
                    for (uint32_t i = lane; i < n; i += 32) crow[part[i]] = make_float2(0.f, 0.f);
                    __syncwarp();
                    if (lane == 0) crow[p0] = trow[p0];
                    __syncwarp();
                    dd Qp{0.f, 0.f}, Qpc{0.f, 0.f};
                    for (uint32_t i = i0; i < i1; ++i) {
                        Qp = Add(Qp, LoadDD(&trow[i]));
                        Qpc = Add(Qpc, LoadDD(&crow[i]));
                    }
                    WarpSum2DD(Qp, Qpc);
                    const Philox4 w = st.Block(1u + step);
                    dd u, x;
                    Split53(w.v[0], w.v[1], u);
                    Split53(w.v[2], w.v[3], x);
                    if (Less(Div(Qpc, Qp), u)) break;  // the walk stops: no cycle
                    dd loc{0.f, 0.f};
                    for (uint32_t i = i0; i < i1; ++i) loc = Add(loc, Div(LoadDD(&crow[i]), Qpc));
                    dd inc = loc;
                    for (int o = 1; o < 32; o <<= 1) {
                        const dd y = dd{__shfl_up_sync(0xffffffffu, inc.hi, o), __shfl_up_sync(0xffffffffu, inc.lo, o)};
                        if ((int)lane >= o) inc = Add(inc, y);
                    }
                    dd run = dd{__shfl_up_sync(0xffffffffu, inc.hi, 1), __shfl_up_sync(0xffffffffu, inc.lo, 1)};
                    if (lane == 0) run = dd{0.f, 0.f};
                    int hit = -1;
                    for (uint32_t i = i0; i < i1 && hit < 0; ++i) {
                        run = Add(run, Div(LoadDD(&crow[i]), Qpc));
                        if (Less(x, run)) hit = (int)i;
                    }
                    const unsigned hits = __ballot_sync(0xffffffffu, hit >= 0);
                    if (hits) p = (uint32_t)__shfl_sync(0xffffffffu, hit, __ffs(hits) - 1);
                    if (p == p0) {
                        ok = true;
                        break;
                    }
                }
                if (lane == 0) {
                    if (!ok) {
                        sh.n = 0;
                    } else {
                        // -log(weight) = sum of the exponents of the identity links minus the cycle's
                        dd lw{0.f, 0.f};
                        for (uint32_t i = 0; i < n; ++i) {
                            const uint32_t q = part[(i + 1) % n];
                            lw = Add(lw, Sub(LoadDD(&a.ex[(size_t)part[i] * N + part[i]]), LoadDD(&a.ex[(size_t)part[i] * N + q])));
                        }
                        sh.prev0 = lw;
                        sh.n = n;
                        for (uint32_t i = 0; i < n; ++i) sigma[i] = (i + 1) % n;
                    }
                }
            } else if (a.variant == kPermVariantTable && threadIdx.x == 0) {
                // perm_bisect_table_class.h:10-28, 105-119
                dd total{0.f, 0.f};
                uint32_t kept = 0;
                for (uint32_t cc = 0; cc < n_cycles; ++cc) {
                    const dd w = LoadDD(&cw[cc]);
                    if (Less(a.eps, w)) {
                        total = Add(total, w);
                        a.ccon[kept] = make_float2(total.hi, total.lo);
                        a.cidx[kept] = cc;
                        ++kept;
                    }
                }
                dd u;
                Split53(sh.w0.v[2], sh.w0.v[3], u);
                const dd x = Mul(u, total);
                uint32_t kk = 0;
                if (!Less(x, LoadDD(&a.ccon[0]))) {
                    uint32_t hi = kept, lo = 0;
                    while (hi - lo > 1) {
                        const uint32_t mid = (hi + lo) >> 1;
                        if (Less(x, LoadDD(&a.ccon[mid]))) hi = mid;
                        else lo = mid;
                    }
                    kk = min(hi, kept - 1);
                }
                const uint32_t cc = a.cidx[kk];
                const uint32_t* cp = a.combs + (size_t)(cc % a.n_comb) * a.k_part;
                const uint32_t* pm = a.types + (size_t)(cc / a.n_comb) * a.k_part;
                for (uint32_t i = 0; i < a.k_part; ++i) {
                    part[i] = cp[i];
                    sigma[i] = pm[i];
                }
                sh.n = a.k_part;
                sh.prev0 = Neg(LoadDD(&a.cwl[cc]));
                sh.tot0 = total;
            }
        } else if (threadIdx.x == 0) {
            part[0] = sh.p_first;
            sigma[0] = 0;
            sh.n = 1;
            sh.prev0 = dd{0.f, 0.f};
        }
        __syncthreads();
        const uint32_t n = sh.n;
        if (n == 0) {  // no cycle selected: rejected before any bisection
            __syncthreads();
            continue;
        }
        // ---- the cycle's paths, their end beads, the actions' particle list and the staged beads,
        // all formed from part, sigma and the committed permutation in one phase ----
        auto lo_of = [&](uint32_t m) -> uint32_t { return G0 + part[m]; };
        auto hi_of = [&](uint32_t m) -> uint32_t { return a.perm[G0 + part[m]]; };
        auto eold_of = [&](uint32_t m) -> uint32_t { return B < tcross ? lo_of(m) : hi_of(m); };
        for (uint32_t m = threadIdx.x; m < n; m += blockDim.x) {
            lab_lo[m] = lo_of(m);
            lab_hi[m] = hi_of(m);
            end_old[m] = eold_of(m);
            end_new[m] = eold_of(sigma[m]);
            lo_idx[part[m]] = (int)m;
            hi_idx[hi_of(m) - G0] = (int)m;
        }
        if (threadIdx.x == 0) {
            // the cycle, and the particles owning the end beads when the segment reaches past the
            // closure (perm_bisect_iterative_class.h:141-146, bisect_class.h:61-64)
            uint32_t nl = 0;
            for (uint32_t m = 0; m < n; ++m) {
                lpos[lo_of(m) - G0] = (int)nl;
                lst[nl++] = lo_of(m);
            }
            if (B >= tcross)
                for (uint32_t m = 0; m < n; ++m)
                    if (lpos[eold_of(m) - G0] < 0) {
                        lpos[eold_of(m) - G0] = (int)nl;
                        lst[nl++] = eold_of(m);
                    }
            sh.nlist = nl;
        }
        auto label = [&](uint32_t m, uint32_t t) -> uint32_t { return t < tcross ? lab_lo[m] : lab_hi[m]; };
        auto slice = [&](uint32_t t) -> uint32_t { return (bead0 + t) % M; };
        // old and new beads of the paths, offsets 0..B (the old end, the new end)
        const bool seg_shared = n * (B + 1u) <= seg_cap;
        float2* so = seg_shared ? reinterpret_cast<float2*>(dyn + L.seg_old) : a.seg_old_g;
        float2* sn = seg_shared ? reinterpret_cast<float2*>(dyn + L.seg_new) : a.prop;
        auto SO = [&](uint32_t m, uint32_t t, uint32_t d) -> float2* { return &so[((size_t)m * (B + 1u) + t) * 3 + d]; };
        auto SN = [&](uint32_t m, uint32_t t, uint32_t d) -> float2* { return &sn[((size_t)m * (B + 1u) + t) * 3 + d]; };
        for (uint32_t it = threadIdx.x; it < n * (B + 1u) * nd; it += blockDim.x) {
            const uint32_t d = it % nd, rest = it / nd, m = rest / (B + 1u), t = rest % (B + 1u);
            const uint32_t g = t == B ? eold_of(m) : (t < tcross ? lo_of(m) : hi_of(m));
            const float2 v = a.pos[((size_t)slice(t) * 3 + d) * np + g];
            *SO(m, t, d) = v;
            if (t == 0) *SN(m, 0, d) = v;
            if (t == B) *SN(m, B, d) = a.pos[((size_t)es * 3 + d) * np + eold_of(sigma[m])];
        }
        // the normals of every midpoint, drawn up front in the order of the reference's loop
        const bool z_up = n * (B - 1u) <= z_cap;
        if (z_up)
            for (uint32_t c = threadIdx.x; c < n * (B - 1u); c += blockDim.x) {
                float z[3];
                BisectNormals(st, base_m + c - 1u, z);
                zb[3 * c] = z[0];
                zb[3 * c + 1] = z[1];
                zb[3 * c + 2] = z[2];
            }
        // the new-mode coordinate of (label g, slice b): the proposal for a moved bead, else committed
        auto newc = [&](uint32_t g, uint32_t b, uint32_t d) -> dd {
            const uint32_t t = (b + M - bead0) % M;
            if (t >= 1u && t < B && g >= G0 && g < G0 + N) {
                const int m = t < tcross ? lo_idx[g - G0] : hi_idx[g - G0];
                if (m >= 0) return LoadDD(SN((uint32_t)m, t, d));
            }
            return LoadPos(a.pos, np, b, d, g);
        };
        __syncthreads();
        const uint32_t nlist = sh.nlist;

        // Every level's terms are formed before the level tests run (the draws of an attempt are
        // indexed per bead and per level, so the levels below a rejection change nothing): the
        // midpoints top-down, one barrier per level; then the density changes of the inner beads;
        // then every level's kinetic, trap, pair and Ewald terms in one pass, reduced per warp and
        // level; then the tests of bisect_class.h:103-118 in order on one thread.
        const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
        for (int level = (int)mv.n_level - 1; level >= 0; --level) {
            const uint32_t skip = 1u << level, nmid = B >> (level + 1);
            const uint32_t off = n * (nmid - 1u);
            dd old_lsp{0.f, 0.f}, new_lsp{0.f, 0.f};
            // midpoints (bisect_class.h:74-94 with the old end of each cycle path)
            for (uint32_t it = threadIdx.x; it < n * nmid; it += blockDim.x) {
                const uint32_t m = it / nmid, q = it % nmid;
                const uint32_t ta = 2u * skip * q, tb = ta + skip, tcc = ta + 2u * skip, c = off + m * nmid + q;
                float z[3];
                if (z_up) {
                    z[0] = zb[3 * c];
                    z[1] = zb[3 * c + 1];
                    z[2] = zb[3 * c + 2];
                } else {
                    BisectNormals(st, base_m + c - 1u, z);
                }
                dd dl[3], dn[3], nbv[3];
                for (uint32_t d = 0; d < nd; ++d) {
                    const dd ra = LoadDD(SO(m, ta, d)), rc = LoadDD(SO(m, tcc, d)), rb = LoadDD(SO(m, tb, d));
                    const dd na = LoadDD(SN(m, ta, d)), nc = LoadDD(SN(m, tcc, d));
                    const dd rbar = Add(ra, Scale2(MinImageDD(Sub(rc, ra), a.L, a.iL), 0.5f));
                    dl[d] = MinImageDD(Sub(rb, rbar), a.L, a.iL);
                    dn[d] = MinImageDD(MulF(mv.sigma[level], z[d]), a.L, a.iL);
                    const dd nbar = Add(na, Scale2(MinImageDD(Sub(nc, na), a.L, a.iL), 0.5f));
                    nbv[d] = Add(nbar, dn[d]);
                }
                for (uint32_t d = 0; d < nd; ++d) *SN(m, tb, d) = make_float2(nbv[d].hi, nbv[d].lo);
                old_lsp = Add(old_lsp, LogRhoFreeDD(dl, nd, mv.i4s[level], &mv.sample_image[level], mv.has_images));
                new_lsp = Add(new_lsp, LogRhoFreeDD(dn, nd, mv.i4s[level], &mv.sample_image[level], mv.has_images));
            }
            WarpSum2DD(old_lsp, new_lsp);
            if (lane == 0) {
                sh.lvl[level][0][warp] = old_lsp;
                sh.lvl[level][1][warp] = new_lsp;
            }
            __syncthreads();
        }
        // density changes of the inner beads (species_class.h:406-425), from their final positions
        // (FP32 mode: FP32 bead phases and density changes, as the sweep kernel's FP32 mode forms them)
        if (slot >= 0 && K > 0) {
            float2* phf = reinterpret_cast<float2*>(ph);
            float2* drho32 = reinterpret_cast<float2*>(a.drho);
            for (uint32_t t = 1; t < B; ++t)
                for (uint32_t m = 0; m < n; ++m) {
                    for (uint32_t it = threadIdx.x; it < 2u * nd * stride; it += blockDim.x) {
                        const uint32_t nn = it % stride, rest = it / stride, d = rest % nd, which = rest / nd;
                        const dd x = which ? LoadDD(SN(m, t, d)) : LoadDD(SO(m, t, d));
                        if (a.rho32) phf[((size_t)which * 3 + d) * stride + nn] = PhaseF(x, (int)nn, a.iL, a.phase256);
                        else ph[((size_t)which * 3 + d) * stride + nn] = PhaseDD(x, (int)nn, a.iL, a.two_pi, a.phase256);
                    }
                    __syncthreads();
                    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
                        const int32_t pk = a.kidx[k];
                        if (a.rho32) {
                            const float2 en = PhaseProductF(phf + 3 * stride, stride, nd, pk), eo = PhaseProductF(phf, stride, nd, pk);
                            const float2 dv = make_float2(__fsub_rn(en.x, eo.x), __fsub_rn(en.y, eo.y));
                            float2* cell = &drho32[(size_t)t * K + k];
                            *cell = m == 0 ? dv : make_float2(__fadd_rn(cell->x, dv.x), __fadd_rn(cell->y, dv.y));
                        } else {
                            const ddc dv = CSub(PhaseProductDD(ph + 3 * stride, stride, nd, pk), PhaseProductDD(ph, stride, nd, pk));
                            float4* cell = &a.drho[(size_t)t * K + k];
                            *cell = Pack(m == 0 ? dv : CAdd(Unpack(*cell), dv));
                        }
                    }
                    __syncthreads();
                }
        }
        for (int level = (int)mv.n_level - 1; level >= 0; --level) {
            const uint32_t skip = 1u << level, ngrid = B / skip - 1u;
            dd dS{0.f, 0.f};
            // kinetic links along the paths (kinetic_class.h:105-122)
            for (int ki = 0; ki < mv.n_kin; ++ki) {
                const uint32_t nl = B / skip;
                for (uint32_t it = threadIdx.x; it < n * nl; it += blockDim.x) {
                    const uint32_t m = it / nl, t0 = (it % nl) * skip, t1 = t0 + skip;
                    const bool old_empty = B == M && end_old[m] == lab_lo[m], new_empty = B == M && end_new[m] == lab_lo[m];
                    dd dro[3], drn[3];
                    for (uint32_t d = 0; d < nd; ++d) {
                        dro[d] = MinImageDD(Sub(LoadDD(SO(m, t0, d)), LoadDD(SO(m, t1, d))), a.L, a.iL);
                        drn[d] = MinImageDD(Sub(LoadDD(SN(m, t0, d)), LoadDD(SN(m, t1, d))), a.L, a.iL);
                    }
                    const dd lro = old_empty ? dd{0.f, 0.f} : LogRhoFreeDD(dro, nd, mv.kin_i4[ki][level], &mv.kin_image[ki][level], mv.kin_has_images[ki]);
                    const dd lrn = new_empty ? dd{0.f, 0.f} : LogRhoFreeDD(drn, nd, mv.kin_i4[ki][level], &mv.kin_image[ki][level], mv.kin_has_images[ki]);
                    dS = Add(dS, Sub(lro, lrn));  // action = -log rho
                }
            }
            // trap beads (trap_class.h:37-61)
            for (int ti = 0; ti < mv.n_trap; ++ti) {
                if ((uint32_t)level > mv.trap_max_level[ti]) continue;
                for (uint32_t it = threadIdx.x; it < n * ngrid; it += blockDim.x) {
                    const uint32_t m = it / ngrid, t = (it % ngrid + 1u) * skip;
                    dd qo{0.f, 0.f}, qn{0.f, 0.f};
                    for (uint32_t d = 0; d < nd; ++d) {
                        qo = Add(qo, Sqr(LoadDD(SO(m, t, d))));
                        qn = Add(qn, Sqr(LoadDD(SN(m, t, d))));
                    }
                    dS = Add(dS, MulF(Mul(Sub(qn, qo), mv.trap_cofa[ti]), (float)skip));
                }
            }
            // pair links over the particle list, label by label (pair_action_class.h:267-302)
            for (int pi = 0; pi < mv.n_pair; ++pi) {
                const PairDD& pa = s_pairs[pi];
                if (level > pa.max_level || pa.is_constant) continue;
                if (pa.kind == kPairBare && level != 0) continue;  // level_tau = 0
                const bool hom = pa.sa == pa.sb;
                const uint32_t other = hom ? sp : (pa.sa == sp ? pa.sb : pa.sa);
                const uint32_t nq = a.sp_n[other], goff = a.sp_off[other], nlk = B / skip;
                for (uint32_t it = threadIdx.x; it < nlk * nlist * nq; it += blockDim.x) {
                    const uint32_t q = it % nq, rest = it / nq, li = rest % nlist, t = (rest / nlist) * skip;
                    const uint32_t gx = lst[li], gy = goff + q;
                    if (hom) {
                        if (gy == gx) continue;
                        const int ly = lpos[q];
                        if (ly >= 0 && (uint32_t)ly < li) continue;  // a pair within the list: once
                    }
                    const uint32_t b = slice(t), bn = slice(t + skip);
                    dd A0[3], C0[3], A1[3], C1[3], r, rp, ss;
                    for (uint32_t d = 0; d < nd; ++d) {
                        A0[d] = LoadPos(a.pos, np, b, d, gy);
                        C0[d] = LoadPos(a.pos, np, b, d, gx);
                        A1[d] = LoadPos(a.pos, np, bn, d, gy);
                        C1[d] = LoadPos(a.pos, np, bn, d, gx);
                    }
                    DrDrpDrrpDD(A0, C0, A1, C1, nd, a.L, a.iL, r, rp, ss);
                    const dd uo = PairUDD(pa, r, rp, ss, level, a.tau);
                    for (uint32_t d = 0; d < nd; ++d) {
                        A0[d] = newc(gy, b, d);
                        C0[d] = newc(gx, b, d);
                        A1[d] = newc(gy, bn, d);
                        C1[d] = newc(gx, bn, d);
                    }
                    DrDrpDrrpDD(A0, C0, A1, C1, nd, a.L, a.iL, r, rp, ss);
                    dS = Add(dS, Sub(PairUDD(pa, r, rp, ss, level, a.tau), uo));
                }
            }
            // Ewald part: tau 2^level v_long_k (bare) or u_long_k (Ilkka, David) times the change of
            // CMag2 over the level's slices (bare_pair_action_class.h:126-144)
            if (slot >= 0 && K > 0)
                for (int pi = 0; pi < mv.n_pair; ++pi) {
                    const PairDD& pa = s_pairs[pi];
                    if (level > pa.max_level || pa.is_constant || !pa.use_lr || !pa.vk) continue;
                    const bool hom = pa.sa == pa.sb;
                    const int oslot = hom ? slot : a.sp_rho[pa.sa == sp ? pa.sb : pa.sa];
                    dd part_lr{0.f, 0.f};
                    if (a.rho32) {
                        // FP32 mode: FP32 terms in a compensated sum, joined to the double-float total
                        const float2* drho32 = reinterpret_cast<const float2*>(a.drho);
                        Comp lr32{0.f, 0.f};
                        for (uint32_t it = threadIdx.x; it < ngrid * K; it += blockDim.x) {
                            const uint32_t k = it % K, t = (it / K + 1u) * skip;
                            const float2 ro = a.rho32[((size_t)slot * M + slice(t)) * K + k];
                            const float2 dv = drho32[(size_t)t * K + k];
                            float tm;
                            if (hom) {
                                tm = __fmaf_rn(dv.x, __fmaf_rn(2.f, ro.x, dv.x), __fmul_rn(dv.y, __fmaf_rn(2.f, ro.y, dv.y)));
                            } else {
                                const float2 rb = a.rho32[((size_t)oslot * M + slice(t)) * K + k];
                                tm = __fmaf_rn(dv.x, rb.x, __fmul_rn(dv.y, rb.y));
                            }
                            CompAdd(lr32, __fmul_rn(pa.vk[k].x, tm));
                        }
                        part_lr = CompDD(lr32);
                    } else {
                        for (uint32_t it = threadIdx.x; it < ngrid * K; it += blockDim.x) {
                            const uint32_t k = it % K, t = (it / K + 1u) * skip;
                            const ddc ro = Unpack(a.rho[((size_t)slot * M + slice(t)) * K + k]);
                            const ddc dv = Unpack(a.drho[(size_t)t * K + k]);
                            dd dm;
                            if (hom) {
                                // |ro + dv|^2 - |ro|^2 = 2 Re(dv conj ro) + |dv|^2
                                dm = Add(Scale2(Add(Mul(dv.re, ro.re), Mul(dv.im, ro.im)), 2.f), Add(Sqr(dv.re), Sqr(dv.im)));
                            } else {
                                const ddc rb = Unpack(a.rho[((size_t)oslot * M + slice(t)) * K + k]);
                                dm = Add(Mul(dv.re, rb.re), Mul(dv.im, rb.im));
                            }
                            part_lr = Add(part_lr, Mul(LoadDD(&pa.vk[k]), dm));
                        }
                    }
                    const float f = (hom ? 1.f : 2.f) * (pa.kind == kPairBare ? (float)skip : 1.f);
                    dS = Add(dS, MulF(Mul(a.tau, part_lr), f));
                }
            dS = WarpSumDD(dS);
            if (lane == 0) sh.lvl[level][2][warp] = dS;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            // lanes add the warp partials of one (level, term) each, in warp order; lane 0 then runs the tests
            const uint32_t nw = blockDim.x >> 5;
            for (uint32_t i = lane; i < 3u * mv.n_level; i += 32) {
                dd t{0.f, 0.f};
                for (uint32_t w = 0; w < nw; ++w) t = Add(t, sh.lvl[i / 3][i % 3][w]);
                sh.lvl[i / 3][i % 3][0] = t;
            }
            __syncwarp();
        }
        if (threadIdx.x == 0) {
            dd prev = sh.prev0;
            int ok = 1;
            for (int level = (int)mv.n_level - 1; level >= 0 && ok; --level) {
                const dd so = sh.lvl[level][0][0], sn = sh.lvl[level][1][0], ds = sh.lvl[level][2][0];
                if (level == 0) atomicAdd(&a.counters[1], 1ull);  // the attempt reached the level-0 test
                const dd la = Add(Sub(Sub(so, sn), ds), prev);
                ok = !Less(la, DD(sh.lu[mv.n_level - 1u - (uint32_t)level]));
                if (!isfinite(la.hi)) {
                    atomicCAS(a.err, 0, kDevErrNonFinite);
                    ok = 0;
                }
                prev = ds;
            }
            sh.decide = ok;
        }
        __syncthreads();
        bool accepted = sh.decide != 0;
        // final test of the table with the new end map (perm_bisect_table_class.h:216-225)
        if (accepted && a.variant == kPermVariantTable && n < N) {
            BuildTableDD(a, N, G0, B, tcross, true, lo_idx, end_new, sh.inv_fact, s0, sE, tt, nullptr, &sh.overflow);
            __syncthreads();
            CycleWeightsDD(a, N, tt, cw);
            __syncthreads();
            if (threadIdx.x == 0) {
                dd total{0.f, 0.f};
                for (uint32_t cc = 0; cc < n_cycles; ++cc) {
                    const dd w = LoadDD(&cw[cc]);
                    if (Less(a.eps, w)) total = Add(total, w);
                }
                const Philox4 w = st.Block(base_u + mv.n_level);
                dd u;
                Split53(w.v[0], w.v[1], u);
                sh.decide = !Less(Div(sh.tot0, total), u);
            }
            __syncthreads();
            accepted = sh.decide != 0;
        }
        // ---- commit ----
        if (accepted) {
            for (uint32_t it = threadIdx.x; it < n * (B - 1u) * nd; it += blockDim.x) {
                const uint32_t d = it % nd, rest = it / nd, m = rest / (B - 1u), t = rest % (B - 1u) + 1u;
                a.pos[((size_t)slice(t) * 3 + d) * np + label(m, t)] = *SN(m, t, d);
            }
            if (slot >= 0 && K > 0)
                for (uint32_t it = threadIdx.x; it < (B - 1u) * K; it += blockDim.x) {
                    const uint32_t k = it % K, t = it / K + 1u;
                    if (a.rho32) {
                        float2* r = &a.rho32[((size_t)slot * M + slice(t)) * K + k];
                        const float2 dv = reinterpret_cast<const float2*>(a.drho)[(size_t)t * K + k];
                        *r = make_float2(__fadd_rn(r->x, dv.x), __fadd_rn(r->y, dv.y));
                    } else {
                        float4* r = &a.rho[((size_t)slot * M + slice(t)) * K + k];
                        *r = Pack(CAdd(Unpack(*r), Unpack(a.drho[(size_t)t * K + k])));
                    }
                }
        }
        __syncthreads();
        // AssignParticleLabels (perm_bisect_class.h:47-56): the beads after slice s0 of the paths'
        // labels there move to the label of the path that reaches them.
        bool moved_labels = false;
        for (uint32_t m = 0; m < n; ++m) moved_labels |= sigma[m] != m;
        if (accepted && moved_labels) {
            const uint32_t s0l = slice(B - 1u), ns = M - 1u - s0l;
            for (uint32_t it = threadIdx.x; it < n * ns * nd; it += blockDim.x) {
                const uint32_t d = it % nd, rest = it / nd, m = rest / ns, b = s0l + 1u + rest % ns;
                a.hold[((size_t)m * M + b) * 3 + d] = a.pos[((size_t)b * 3 + d) * np + label(sigma[m], B - 1u)];
            }
            __syncthreads();
            for (uint32_t it = threadIdx.x; it < n * ns * nd; it += blockDim.x) {
                const uint32_t d = it % nd, rest = it / nd, m = rest / ns, b = s0l + 1u + rest % ns;
                a.pos[((size_t)b * 3 + d) * np + label(m, B - 1u)] = a.hold[((size_t)m * M + b) * 3 + d];
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
            if (a.variant != kPermVariantBisect) {
                atomicAdd(&a.counters[2 + (n - 1)], 1ull);
                if (accepted) atomicAdd(&a.counters[2 + N + (n - 1)], 1ull);
            }
        }
        __syncthreads();
        for (uint32_t m = threadIdx.x; m < n; m += blockDim.x) {
            lo_idx[lab_lo[m] - G0] = -1;
            hi_idx[lab_hi[m] - G0] = -1;
        }
        for (uint32_t i = threadIdx.x; i < nlist; i += blockDim.x) lpos[lst[i] - G0] = -1;
        __syncthreads();
    }
    if (threadIdx.x == 0 && sh.overflow) atomicCAS(a.err, 0, kDevErrNonFinite);
    __syncthreads();
}

__global__ void __launch_bounds__(kPermThreads, 1) PermBisectKernelDD(const __grid_constant__ PermArgsDD a) {
    extern __shared__ __align__(16) unsigned char dyn[];
    __shared__ PermSharedDD sh;
    PermRun(a, a.attempt0, a.n_attempts, dyn, sh);
}

/// Many independent chains in one launch, one CTA of kPermChainThreads per chain: chain c runs its schedule
/// args[c n_entries + e] (e in order) n_rep times; repetition r of entry e starts at attempt
/// args.attempt0 + r rep_stride[c n_entries + e].
__global__ void __launch_bounds__(kPermChainThreads, 4) PermChainsKernelDD(const PermArgsDD* __restrict__ args, const uint64_t* __restrict__ rep_stride,
                                                                     uint32_t n_entries, uint64_t n_rep) {
    extern __shared__ __align__(16) unsigned char dyn[];
    __shared__ PermSharedDD sh;
    const size_t c = blockIdx.x;
    for (uint64_t r = 0; r < n_rep; ++r)
        for (uint32_t e = 0; e < n_entries; ++e) {
            const PermArgsDD& a = args[c * n_entries + e];
            PermRun(a, a.attempt0 + r * rep_stride[c * n_entries + e], a.n_attempts, dyn, sh);
        }
}
