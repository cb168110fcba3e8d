// Counter-based random numbers for the Monte Carlo moves (host and device).
//
// The reference draws from a stateful scaffold::rand::RNG (`UnifRand(n)` in 1..n, `UnifRand()` in
// [0,1), `NormRand(vec, mu, sigma)`; call sites src/events/moves/single_species_move/bisect/
// bisect_class.h:40-41,91,114). That library is not available, and a stateful generator cannot be
// shared by thousands of GPU threads anyway. Every draw here is instead a pure function of
// (seed, chain, move, attempt, block) through Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), so a bisection attempt can be replayed
// bit-for-bit by any thread, by a later launch, or by a CPU checker.
//
// Stream layout of one bisection attempt with n_bisect = 2^n_level beads:
//   block 0                       words 0,1 -> particle index, first bead (multiply-high ranges)
//   block 1+i                     3 normal deviates for the i-th resampled bead, in generation
//                                 order (top level first, left to right within a level)
//   block 1+(n_bisect-1)+li       word 0 -> acceptance uniform of level li (0 = top level)
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define PIMC_HD __host__ __device__ __forceinline__
#else
#define PIMC_HD inline
#endif

namespace pimc {

struct Philox4 {
    uint32_t v[4];
};

PIMC_HD uint32_t MulHi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return static_cast<uint32_t>((static_cast<uint64_t>(a) * b) >> 32);
#endif
}

/// Philox4x32 with 10 rounds: multipliers 0xD2511F53, 0xCD9E8D57; Weyl key increments
/// 0x9E3779B9, 0xBB67AE85 (the published parameter set).
PIMC_HD Philox4 Philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c0;
        const uint32_t hi0 = MulHi32(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2;
        const uint32_t hi1 = MulHi32(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n1 = lo1;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        const uint32_t n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    Philox4 out;
    out.v[0] = c0;
    out.v[1] = c1;
    out.v[2] = c2;
    out.v[3] = c3;
    return out;
}

/// 53-bit uniform in [0, 1) from two 32-bit words.
PIMC_HD double Uniform53(uint32_t a, uint32_t b) {
    return (static_cast<double>(a >> 5) * 67108864.0 + static_cast<double>(b >> 6)) * (1.0 / 9007199254740992.0);
}

/// Uniform integer in [0, n) by multiply-high (bias below 2^-32 * n, irrelevant here).
PIMC_HD uint32_t UniformIndex(uint32_t w, uint32_t n) { return MulHi32(w, n); }

/// Draw-stream coordinates of one Monte Carlo attempt.
struct MoveStream {
    uint32_t key0, key1;    // seed, chain
    uint32_t move;          // move index within the simulation
    uint64_t attempt;       // attempt counter of that move

    PIMC_HD Philox4 Block(uint32_t block) const {
        return Philox4x32_10(static_cast<uint32_t>(attempt), static_cast<uint32_t>(attempt >> 32), move, block, key0, key1);
    }
};

// ---------------------------------------------------------------------------------------------
// Exactly specified single-precision transforms. Every operation below is an IEEE-754 binary32
// operation with round-to-nearest and no contraction (explicit intrinsics on the device; the CPU
// checker compiles its restatement with -ffp-contract=off), so the GPU and any CPU produce the
// same bits. Methods: logarithm by reduction to m in [sqrt(1/2), sqrt(2)) and the series
// log m = 2 atanh((m-1)/(m+1)); sine/cosine of 2*pi*u by quadrant reduction in turns and Taylor
// polynomials on [-pi/4, pi/4]; normals by the Box-Muller transform.

#if defined(__CUDA_ARCH__)
#define PIMC_FADD(a, b) __fadd_rn(a, b)
#define PIMC_FSUB(a, b) __fsub_rn(a, b)
#define PIMC_FMUL(a, b) __fmul_rn(a, b)
#define PIMC_FDIV(a, b) __fdiv_rn(a, b)
#define PIMC_FFMA(a, b, c) __fmaf_rn(a, b, c)
#define PIMC_FSQRT(a) __fsqrt_rn(a)
#else
#define PIMC_FADD(a, b) ((a) + (b))
#define PIMC_FSUB(a, b) ((a) - (b))
#define PIMC_FMUL(a, b) ((a) * (b))
#define PIMC_FDIV(a, b) ((a) / (b))
#define PIMC_FFMA(a, b, c) fmaf(a, b, c)
#define PIMC_FSQRT(a) sqrtf(a)
#endif

PIMC_HD uint32_t FloatBits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t b;
    __builtin_memcpy(&b, &x, 4);
    return b;
#endif
}

PIMC_HD float BitsFloat(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    __builtin_memcpy(&x, &b, 4);
    return x;
#endif
}

/// 24-bit uniform in [0, 1), exact in binary32.
PIMC_HD float U24(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

/// Natural logarithm of a normal binary32 x in (0, 1]; -inf for 0.
PIMC_HD float LogF(float x) {
    if (x == 0.f) return -INFINITY;
    const uint32_t b = FloatBits(x);
    int e = (int)((b >> 23) & 0xffu) - 126;  // x = m 2^e, m in [1/2, 1)
    float m = BitsFloat((b & 0x007fffffu) | 0x3f000000u);
    if (m < 0.70710678f) {
        m = PIMC_FADD(m, m);
        e -= 1;
    }
    const float f = PIMC_FSUB(m, 1.0f);  // exact
    const float s = PIMC_FDIV(f, PIMC_FADD(2.0f, f));
    const float s2 = PIMC_FMUL(s, s);
    float p = PIMC_FFMA(s2, 1.0f / 9.0f, 1.0f / 7.0f);
    p = PIMC_FFMA(s2, p, 1.0f / 5.0f);
    p = PIMC_FFMA(s2, p, 1.0f / 3.0f);
    p = PIMC_FMUL(s2, p);
    const float two_s = PIMC_FADD(s, s);
    const float lm = PIMC_FFMA(two_s, p, two_s);
    const float ef = (float)e;
    return PIMC_FFMA(ef, 0.693145751953125f, PIMC_FFMA(ef, 1.428606765330187e-06f, lm));
}

/// sin and cos of 2 pi u for u in [0, 1).
PIMC_HD void SinCos2PiF(float u, float& s, float& c) {
    const float v = PIMC_FMUL(u, 4.0f);
    const float q = floorf(v);
    const float f = PIMC_FSUB(v, q);
    const int qi = (int)q & 3;
    const float t = PIMC_FMUL(PIMC_FSUB(f, 0.5f), 1.57079637f);
    const float t2 = PIMC_FMUL(t, t);
    float ps = PIMC_FFMA(t2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = PIMC_FFMA(t2, ps, 1.0f / 120.0f);
    ps = PIMC_FFMA(t2, ps, -1.0f / 6.0f);
    ps = PIMC_FMUL(t2, ps);
    const float st = PIMC_FFMA(t, ps, t);
    float pc = PIMC_FFMA(t2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = PIMC_FFMA(t2, pc, -1.0f / 720.0f);
    pc = PIMC_FFMA(t2, pc, 1.0f / 24.0f);
    pc = PIMC_FFMA(t2, pc, -0.5f);
    const float ct = PIMC_FFMA(t2, pc, 1.0f);
    const float sp = PIMC_FMUL(PIMC_FADD(st, ct), 0.70710678f);  // sin(pi/4 + t)
    const float cp = PIMC_FMUL(PIMC_FSUB(ct, st), 0.70710678f);  // cos(pi/4 + t)
    switch (qi) {
        case 0: s = sp; c = cp; break;
        case 1: s = cp; c = -sp; break;
        case 2: s = -sp; c = -cp; break;
        default: s = -cp; c = sp; break;
    }
}

/// Two standard normal deviates from two Philox words (Box-Muller on 24-bit uniforms; the
/// radius is bounded by sqrt(48 ln 2) = 5.77, a tail cut at probability 1e-8).
PIMC_HD void BoxMullerF(uint32_t w0, uint32_t w1, float& z0, float& z1) {
    const float u0 = U24(w0), u1 = U24(w1);
    const float r = PIMC_FSQRT(PIMC_FMUL(-2.0f, LogF(PIMC_FSUB(1.0f, u0))));
    float s, c;
    SinCos2PiF(u1, s, c);
    z0 = PIMC_FMUL(r, c);
    z1 = PIMC_FMUL(r, s);
}

/// The three normal deviates of resampled bead i of an attempt (one Philox block per bead).
PIMC_HD void BisectNormals(const MoveStream& st, uint32_t i, float z[3]) {
    const Philox4 w = st.Block(1u + i);
    float z3;
    BoxMullerF(w.v[0], w.v[1], z[0], z[1]);
    BoxMullerF(w.v[2], w.v[3], z[2], z3);
}

/// log of the acceptance uniform of level index li (0 = top level) of an attempt.
PIMC_HD float BisectLogU(const MoveStream& st, uint32_t n_bisect, uint32_t level_index) {
    const Philox4 w = st.Block(1u + (n_bisect - 1u) + level_index);
    return LogF(U24(w.v[0]));
}

}  // namespace pimc
