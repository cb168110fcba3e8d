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
//   blocks 1+2i, 2+2i             3 normal deviates for the i-th resampled bead, in generation
//                                 order (top level first, left to right within a level)
//   block 1+2(n_bisect-1)+li      words 0,1 -> acceptance uniform of level li (0 = top level)
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

/// Two standard normal deviates from one Philox block (Box-Muller on 53-bit uniforms).
PIMC_HD void BoxMuller(const Philox4& w, double& z0, double& z1) {
    const double u0 = Uniform53(w.v[0], w.v[1]);
    const double u1 = Uniform53(w.v[2], w.v[3]);
    const double r = sqrt(-2.0 * log(1.0 - u0));
    const double th = 6.283185307179586 * u1;
    z0 = r * cos(th);
    z1 = r * sin(th);
}

/// The three normal deviates of resampled bead i of an attempt.
PIMC_HD void BisectNormals(const MoveStream& s, uint32_t i, double z[3]) {
    double z3;
    BoxMuller(s.Block(1u + 2u * i), z[0], z[1]);
    BoxMuller(s.Block(2u + 2u * i), z[2], z3);
}

PIMC_HD double BisectAcceptUniform(const MoveStream& s, uint32_t n_bisect, uint32_t level_index) {
    Philox4 w = s.Block(1u + 2u * (n_bisect - 1u) + level_index);
    return Uniform53(w.v[0], w.v[1]);
}

}  // namespace pimc
