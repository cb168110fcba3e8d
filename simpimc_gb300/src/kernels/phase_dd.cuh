// Double-float bead phases exp(i k x) for the charge densities (k_space_class.h:83-94,
// bead_class.h:125-133): per-dimension rows exp(2 pi i n x / L), n = 0..max_index, and their
// products over dimensions for a packed k-vector.
#pragma once

#include <cmath>

#include "device_common.cuh"
#include "df64.cuh"

namespace pimc {

/// exp(2 pi i n t) for the turn count t = x / L of one coordinate: n t is reduced modulo 1, its
/// nearest 1/256 of a turn read from a table and the residue (|eps| <= pi/256) expanded in Taylor
/// series to eps^7 in double-float.
__device__ __forceinline__ ddc PhaseDD(dd x, int n, dd iL, dd two_pi, const float4* tab256) {
    if (n == 0) return ddc{DD(1.f), DD(0.f)};
    dd t = Mul(x, iL);
    t = Sub(t, DD(Rint(t)));
    dd a = MulF(t, (float)n);
    a = Sub(a, DD(Rint(a)));
    const float jf = rintf(__fmul_rn(a.hi, 256.f));
    const dd g = Sub(a, DD(__fmul_rn(jf, 1.f / 256.f)));
    const dd eps = Mul(g, two_pi);
    const dd e2 = Sqr(eps);
    const dd neg_inv6{-0.16666667f, 4.9670538e-09f};  // -1/6 as a float pair
    const dd ps = Add(neg_inv6, MulF(e2, __fmaf_rn(e2.hi, -1.f / 5040.f, 1.f / 120.f)));
    const dd sn = Add(eps, Mul(eps, Mul(e2, ps)));
    const dd pc = AddF(MulF(e2, __fmaf_rn(e2.hi, -1.f / 720.f, 1.f / 24.f)), -0.5f);
    const dd cs = AddF(Mul(e2, pc), 1.f);
    const int j = ((int)jf + 256) & 255;
    const ddc T = Unpack(tab256[j]);
    return CMulDD(T, ddc{cs, sn});
}

/// Product over dimensions of the per-dimension phases from tables [3][stride].
__device__ __forceinline__ ddc PhaseProductDD(const ddc* tab, uint32_t stride, uint32_t n_d, int32_t packed) {
    ddc f{DD(1.f), DD(0.f)};
    for (uint32_t d = 0; d < n_d; ++d) {
        const int n = KIdx(packed, (int)d);
        ddc c = tab[d * stride + (n < 0 ? -n : n)];
        if (n < 0) c.im = Neg(c.im);
        f = d == 0 ? c : CMulDD(f, c);
    }
    return f;
}

/// Host table of exp(2 pi i j / 256), j = 0..255, as double-float (re.hi, re.lo, im.hi, im.lo).
inline void PhaseTable256(float4* out) {
    for (int j = 0; j < 256; ++j) {
        const double th = 2. * 3.14159265358979323846 * j / 256.;
        const double c = std::cos(th), s = std::sin(th);
        float ch, cl, sh, sl;
        SplitDouble(c, ch, cl);
        SplitDouble(s, sh, sl);
        out[j] = make_float4(ch, cl, sh, sl);
    }
}

}  // namespace pimc
