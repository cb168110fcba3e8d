// Per-link and per-k action terms shared by the estimator kernels and the bisection sweep.
#pragma once

#include "device_common.cuh"

namespace pimc {

/// DavidPairAction: the endpoint terms of component `diag` at r and r' (clamped to the grid), plus
/// the off-diagonal expansion sum_{k=1..n} sum_{j=0..k} c_kj(q) z^2j s^2(k-j) at q = (r + r')/2
/// (clamped) when s > 0 and q < r_max (david_pair_action_class.h:69-102, 126-167). With `add_v` the
/// potential's endpoint terms (component 0) are added, as CalcdUdBeta does. `level` picks the table
/// u_kj(level) of the time step tau 2^level (the multi-spline's components from level * kj_stride).
__device__ __forceinline__ double DavidLink(const PairDev& pa, const MultiCubic& t, double r, double rp, double s, bool add_v,
                                            uint32_t level = 0) {
    const double q = 0.5 * (r + rp), z = r - rp;
    const int b = (int)(level * pa.kj_stride);
    double ur, urp;
    const int i = MultiInterval(t, r, ur), ip = MultiInterval(t, rp, urp);
    double u = 0.5 * (MultiComp(t, i, ur, b + 1) + MultiComp(t, ip, urp, b + 1));
    if (add_v) u += 0.5 * (MultiComp(t, i, ur, b) + MultiComp(t, ip, urp, b));
    if (s > 0. && q < pa.r_d_max) {
        double uq;
        const int iq = MultiInterval(t, q, uq);
        const double z2 = z * z, s2 = s * s, is2 = 1. / s2;
        double s2k = s2;
        for (uint32_t k = 1; k <= pa.n_order; ++k) {
            double z2j = 1., cs = s2k;
            for (uint32_t j = 0; j <= k; ++j) {
                u += MultiComp(t, iq, uq, b + (int)(k * (k + 1) / 2 + j + 1)) * z2j * cs;
                z2j *= z2;
                cs *= is2;
            }
            s2k *= s2;
        }
    }
    return u;
}

/// CalcV of a link. BarePairAction::CalcV (bare_pair_action_class.h:99-123): clamp to the table
/// grid, Coulomb or spline short-range part, minus the long-range spline when the action has an
/// Ewald part; IlkkaPairAction::CalcV is the same with its tables (ilkka_pair_action_class.h:34-54);
/// DavidPairAction::CalcV is the potential component at both ends (david_pair_action_class.h:34-47).
__device__ __forceinline__ double PairV(const PairDev& pa, double r, double rp) {
    if (pa.kind == kPairDavid) {
        double ur, urp;
        const int i = MultiInterval(pa.u_kj, r, ur), ip = MultiInterval(pa.u_kj, rp, urp);
        return 0.5 * (MultiComp(pa.u_kj, i, ur, 0) + MultiComp(pa.u_kj, ip, urp, 0));
    }
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

/// CalcU of a link with end distances r, r' and s = |r - r'|.
///  * BarePairAction (bare_pair_action_class.h:146-150): tau V(r, r') scaled by (1 >> level), i.e.
///    tau at level 0 and zero above; that behaviour is kept.
///  * IlkkaPairAction (ilkka_pair_action_class.h:77-101): u(q + s/2, q - s/2), q = (r + r')/2, minus
///    half the long-range action at each end (clamped to its grid) when the action has an Ewald part.
///  * DavidPairAction (david_pair_action_class.h:69-102): DavidLink of the action components of the
///    level's table u_kj(level).
__device__ __forceinline__ double PairU(const PairDev& pa, double r, double rp, double s, uint32_t level, double tau) {
    if (pa.kind == kPairDavid) return DavidLink(pa, pa.u_kj, r, rp, s, false, level);
    if (pa.kind == kPairIlkka) {
        const double q = 0.5 * (r + rp);
        double u = EvalBicubic(pa.u_xy, q + 0.5 * s, q - 0.5 * s);
        if (pa.use_long_range) {
            r = fmin(fmax(r, pa.r_u_min), pa.r_u_max);
            rp = fmin(fmax(rp, pa.r_u_min), pa.r_u_max);
            u -= 0.5 * EvalCubic(pa.u_long_r, r);
            u -= 0.5 * EvalCubic(pa.u_long_r, rp);
        }
        return u;
    }
    return level == 0 ? tau * PairV(pa, r, rp) : 0.;
}

/// CalcdUdBeta of a link: V(r, r') for the bare action (bare_pair_action_class.h:152-155);
/// du(q + s/2, q - s/2) minus half the long-range du at each end for IlkkaPairAction
/// (ilkka_pair_action_class.h:125-149).
__device__ __forceinline__ double PairdUdBeta(const PairDev& pa, double r, double rp, double s) {
    if (pa.kind == kPairDavid) return DavidLink(pa, pa.du_kj, r, rp, s, true);
    if (pa.kind == kPairIlkka) {
        const double q = 0.5 * (r + rp);
        double du = EvalBicubic(pa.du_xy, q + 0.5 * s, q - 0.5 * s);
        if (pa.use_long_range) {
            r = fmin(fmax(r, pa.r_du_min), pa.r_du_max);
            rp = fmin(fmax(rp, pa.r_du_min), pa.r_du_max);
            du -= 0.5 * EvalCubic(pa.du_long_r, r);
            du -= 0.5 * EvalCubic(pa.du_long_r, rp);
        }
        return du;
    }
    return PairV(pa, r, rp);
}

/// IlkkaPairAction::CalcGradientU (ilkka_pair_action_class.h:172-222): the gradient of the link
/// action with respect to the first particle's bead on the link's first slice, by the chain rule
/// through (x, y). A0/A1 are the second particle's beads, C0/C1 the first's (Path::DrDrpDrrp).
__device__ __forceinline__ void IlkkaGradientU(const PairDev& pa, const double* A0, const double* C0, const double* A1, const double* C1,
                                               uint32_t n_d, double L, double iL, double* g) {
    double rv[3] = {0., 0., 0.}, rq[3] = {0., 0., 0.}, rr[3] = {0., 0., 0.};
    double a = 0., b = 0., c = 0.;
#pragma unroll
    for (uint32_t d = 0; d < 3; ++d) {
        if (d < n_d) {
            rv[d] = A0[d] - C0[d];
            rq[d] = A1[d] - C1[d];
            rv[d] -= rint(rv[d] * iL) * L;
            rq[d] += rint((rv[d] - rq[d]) * iL) * L;
            rr[d] = rv[d] - rq[d];
            rr[d] -= rint(rr[d] * iL) * L;
            a += rv[d] * rv[d];
            b += rq[d] * rq[d];
            c += rr[d] * rr[d];
        }
    }
    double r = sqrt(a), rp = sqrt(b);
    const double s = sqrt(c);
    const double q = 0.5 * (r + rp);
    double ux, uy;
    EvalBicubic(pa.u_xy, q + 0.5 * s, q - 0.5 * s, &ux, &uy);
    double rh[3], sh[3];
#pragma unroll
    for (uint32_t d = 0; d < 3; ++d) {
        rh[d] = r == 0. ? 0. : rv[d] / r;
        sh[d] = s == 0. ? 0. : rr[d] / s;
        g[d] = d < n_d ? -0.5 * (ux * (rh[d] + sh[d]) + uy * (rh[d] - sh[d])) : 0.;
    }
    if (pa.use_long_range) {
        r = fmin(fmax(r, pa.r_u_min), pa.r_u_max);
        double tu, tdu;
        EvalCubicVG(pa.u_long_r, r, tu, tdu);
#pragma unroll
        for (uint32_t d = 0; d < 3; ++d)
            if (d < n_d) g[d] -= 0.5 * tdu * rh[d];
    }
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
