// Double-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of two FP32 numbers,
// giving a 48-bit significand (relative rounding ~2^-46 = 1.4e-14 per operation) on the FP32 and
// integer pipes only.
//
// Why: GB300 (sm_103a) issues FP64 at 1/64 of its FP32 rate; a dependent chain of FP64
// instructions costs tens of cycles per instruction and one warp's FP64 work occupies the SM's
// FP64 pipe for everyone. The sweep kernel therefore does its bead geometry, pair terms, charge
// density phases and action sums in df64, which keeps FP64-grade accuracy (far inside the 1e-10
// relative parity tolerance against the FP64 oracle) at FP32 speed.
//
// The error-free transformations are the classical ones: TwoSum (Knuth, TAOCP vol. 2), FastTwoSum
// (Dekker 1971) and TwoProd through a fused multiply-add; the compound operations follow the
// double-double algorithms of Hida, Li and Bailey ("Algorithms for quad-double precision floating
// point arithmetic", ARITH-15, 2001) transposed to float pairs. Every operation is written with
// explicitly rounded intrinsics so the compiler cannot re-associate or contract it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pimc {

struct dd {
    float hi, lo;
};

struct ddc {  // complex df64
    dd re, im;
};

__device__ __forceinline__ dd DD(float h) { return dd{h, 0.f}; }

__device__ __forceinline__ dd FastTwoSum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return dd{s, e};
}

__device__ __forceinline__ dd TwoSum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return dd{s, e};
}

__device__ __forceinline__ dd TwoProd(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return dd{p, e};
}

/// df64 addition in the "sloppy" form of the double-double libraries: TwoSum of the high parts,
/// low parts added, one renormalisation. Its error is within a few units of 2^-46 of |a| + |b|,
/// which is the accuracy every use here needs (sums of positions, distances and action terms).
__device__ __forceinline__ dd Add(dd a, dd b) {
    dd s = TwoSum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return FastTwoSum(s.hi, s.lo);
}

/// df64 addition carrying both error terms (for long accumulations of cancelling terms).
__device__ __forceinline__ dd AddAccurate(dd a, dd b) {
    dd s = TwoSum(a.hi, b.hi);
    dd t = TwoSum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = FastTwoSum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return FastTwoSum(s.hi, s.lo);
}

__device__ __forceinline__ dd Neg(dd a) { return dd{-a.hi, -a.lo}; }
__device__ __forceinline__ dd Sub(dd a, dd b) { return Add(a, Neg(b)); }

__device__ __forceinline__ dd AddF(dd a, float b) {
    dd s = TwoSum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return FastTwoSum(s.hi, s.lo);
}

__device__ __forceinline__ dd Mul(dd a, dd b) {
    dd p = TwoProd(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return FastTwoSum(p.hi, p.lo);
}

__device__ __forceinline__ dd MulF(dd a, float b) {
    dd p = TwoProd(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return FastTwoSum(p.hi, p.lo);
}

/// Exact scaling by a power of two.
__device__ __forceinline__ dd Scale2(dd a, float two_pow) { return dd{__fmul_rn(a.hi, two_pow), __fmul_rn(a.lo, two_pow)}; }

__device__ __forceinline__ dd Sqr(dd a) {
    dd p = TwoProd(a.hi, a.hi);
    p.lo = __fmaf_rn(__fmul_rn(2.f, a.hi), a.lo, p.lo);
    return FastTwoSum(p.hi, p.lo);
}

__device__ __forceinline__ dd Div(dd a, dd b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    dd r = Sub(a, MulF(b, q1));
    const float q2 = __fdiv_rn(r.hi, b.hi);
    r = Sub(r, MulF(b, q2));
    const float q3 = __fdiv_rn(r.hi, b.hi);
    dd q = FastTwoSum(q1, q2);
    return AddF(q, q3);
}

__device__ __forceinline__ dd Sqrt(dd a) {
    if (a.hi <= 0.f) return dd{0.f, 0.f};
    const float x = __fsqrt_rn(a.hi);
    const dd x2 = TwoProd(x, x);
    const dd r = Sub(a, x2);
    const float corr = __fdiv_rn(r.hi, __fmul_rn(2.f, x));
    return FastTwoSum(x, corr);
}

__device__ __forceinline__ bool Less(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

__device__ __forceinline__ dd Min(dd a, dd b) { return Less(b, a) ? b : a; }
__device__ __forceinline__ dd Max(dd a, dd b) { return Less(a, b) ? b : a; }

/// Nearest integer of hi + lo, ties to even (nearbyint of the df64 value, for |value| < 2^22).
/// rintf(hi) is already correct unless hi sits exactly half-way, where the sign of lo decides.
__device__ __forceinline__ float Rint(dd a) {
    const float h = rintf(a.hi);
    const float d = __fsub_rn(a.hi, h);  // exact
    if (d == 0.5f && a.lo > 0.f) return __fadd_rn(h, 1.f);
    if (d == -0.5f && a.lo < 0.f) return __fsub_rn(h, 1.f);
    return h;
}

/// Minimum image x - rint(x / L) L with iL = 1/L (as the reference computes it, path_class.h:131-134).
__device__ __forceinline__ dd MinImageDD(dd x, dd L, dd iL) {
    const float n = Rint(Mul(x, iL));
    if (n == 0.f) return x;
    return Sub(x, MulF(L, n));
}

__device__ __forceinline__ double ToDouble(dd a) { return (double)a.hi + (double)a.lo; }

__host__ __device__ __forceinline__ void SplitDouble(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

/// Cascaded compensated sum (Neumaier / Ogita-Rump-Oishi Sum2): the running sum carries one FP32
/// add per term on its dependency chain; the TwoSum errors gather in a separate FP32 word. The
/// result is as accurate as a sum formed in twice the working precision.
struct Comp {
    float s, c;
};

__device__ __forceinline__ void CompAdd(Comp& a, float x) {
    const float t = __fadd_rn(a.s, x);
    const float bp = __fsub_rn(t, a.s);
    const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    a.s = t;
    a.c = __fadd_rn(a.c, e);
}

/// Merge of two compensated partial sums (TwoSum of the sums, errors added).
__device__ __forceinline__ Comp CompMerge(Comp a, Comp b) {
    const dd s = TwoSum(a.s, b.s);
    return Comp{s.hi, __fadd_rn(__fadd_rn(a.c, b.c), s.lo)};
}

__device__ __forceinline__ dd CompDD(Comp a) { return TwoSum(a.s, a.c); }

// Complex df64.
__device__ __forceinline__ ddc CAdd(ddc a, ddc b) { return ddc{Add(a.re, b.re), Add(a.im, b.im)}; }
__device__ __forceinline__ ddc CSub(ddc a, ddc b) { return ddc{Sub(a.re, b.re), Sub(a.im, b.im)}; }
__device__ __forceinline__ ddc CMulDD(ddc a, ddc b) {
    return ddc{Sub(Mul(a.re, b.re), Mul(a.im, b.im)), Add(Mul(a.re, b.im), Mul(a.im, b.re))};
}
__device__ __forceinline__ ddc CConj(ddc a) { return ddc{a.re, Neg(a.im)}; }

// Packed storage: float4 = (re.hi, re.lo, im.hi, im.lo).
__device__ __forceinline__ ddc Unpack(float4 v) { return ddc{dd{v.x, v.y}, dd{v.z, v.w}}; }
__device__ __forceinline__ float4 Pack(ddc a) { return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }

/// Warp-wide df64 sum (fixed xor tree; every lane returns the total).
__device__ __forceinline__ dd WarpSumDD(dd v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dd w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = Add(v, w);
    }
    return v;
}

/// Two warp-wide df64 sums in one shuffle tree (the two chains interleave).
__device__ __forceinline__ void WarpSum2DD(dd& a, dd& b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dd wa, wb;
        wa.hi = __shfl_xor_sync(0xffffffffu, a.hi, o);
        wa.lo = __shfl_xor_sync(0xffffffffu, a.lo, o);
        wb.hi = __shfl_xor_sync(0xffffffffu, b.hi, o);
        wb.lo = __shfl_xor_sync(0xffffffffu, b.lo, o);
        a = Add(a, wa);
        b = Add(b, wb);
    }
}

}  // namespace pimc
