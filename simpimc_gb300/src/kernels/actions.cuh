// Per-link and per-k action terms shared by the estimator kernels and the bisection sweep.
#pragma once

#include "device_common.cuh"

namespace pimc {

/// BarePairAction::CalcV (bare_pair_action_class.h:99-123): clamp to the table grid, Coulomb or
/// spline short-range part, minus the long-range spline when the action has an Ewald part.
__device__ __forceinline__ double PairV(const PairDev& pa, double r, double rp) {
    r = fmin(fmax(r, pa.r_v_min), pa.r_v_max);
    rp = fmin(fmax(rp, pa.r_v_min), pa.r_v_max);
    double v = 0.;
    if (pa.is_coulomb) {
        v += (0.5 / r) + (0.5 / rp);
    } else {
        v += 0.5 * EvalCubic(pa.v_r, r);
        v += 0.5 * EvalCubic(pa.v_r, rp);
    }
    if (pa.use_long_range) {
        r = fmin(fmax(r, pa.r_vl_min), pa.r_vl_max);
        rp = fmin(fmax(rp, pa.r_vl_min), pa.r_vl_max);
        v -= 0.5 * EvalCubic(pa.v_long_r, r);
        v -= 0.5 * EvalCubic(pa.v_long_r, rp);
    }
    return v;
}

/// BarePairAction::CalcU (bare_pair_action_class.h:146-150). The reference scales by
/// (1 >> level) * tau, i.e. tau at level 0 and zero above; that behaviour is kept.
__device__ __forceinline__ double PairU(const PairDev& pa, double r, double rp, uint32_t level, double tau) {
    return level == 0 ? tau * PairV(pa, r, rp) : 0.;
}

/// Pair potential from two minimum-image distances (PairAction::Potential, pair_action_class.h:369-395).
__device__ __forceinline__ double DistMinImage(const double* a, const double* b, uint32_t n_d, double L, double iL) {
    double s = 0.;
    for (uint32_t d = 0; d < n_d; ++d) {
        double x = MinImage(a[d] - b[d], L, iL);
        s += x * x;
    }
    return sqrt(s);
}

/// Load the n_d components of bead (g, b) from a slice-major position array.
__device__ __forceinline__ void LoadBead(const double* __restrict__ pos, uint32_t n_pad, uint32_t n_d, uint32_t b, uint32_t g, double* r) {
#pragma unroll
    for (uint32_t d = 0; d < 3; ++d) r[d] = d < n_d ? PosAt(pos, n_pad, b, d, g) : 0.;
}

}  // namespace pimc
