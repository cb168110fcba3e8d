// Device helpers shared by every kernel: minimum-image geometry, spline evaluation, charge-density
// phases, deterministic reductions and a bounded grid barrier.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../data_structures/system.h"

namespace pimc {

// -------------------------------------------------------------------------------------------
// Geometry (src/data_structures/path_class.h:108-166). With open boundaries L = iL = 0 and the
// image shift vanishes, exactly as in the reference.

__device__ __forceinline__ double MinImage(double x, double L, double iL) { return x - rint(x * iL) * L; }

__device__ __forceinline__ double PosAt(const double* __restrict__ pos, uint32_t n_pad, uint32_t b, uint32_t d, uint32_t g) {
    return pos[((size_t)b * 3 + d) * n_pad + g];
}

/// Path::DrDrpDrrp (path_class.h:137-150): r = A0 - C0 (min image), r' = A1 - C1 shifted to the
/// image nearest r, s = |r - r'| (min image). A is the second particle of the pair, C the first.
__device__ __forceinline__ void DrDrpDrrp(const double* A0, const double* C0, const double* A1, const double* C1, uint32_t n_d,
                                          double L, double iL, double& r, double& rp, double& s) {
    double a = 0., b = 0., c = 0.;
#pragma unroll
    for (uint32_t d = 0; d < 3; ++d) {
        if (d < n_d) {
            double rv = A0[d] - C0[d];
            double rq = A1[d] - C1[d];
            rv -= rint(rv * iL) * L;
            rq += rint((rv - rq) * iL) * L;
            double rr = rv - rq;
            rr -= rint(rr * iL) * L;
            a += rv * rv;
            b += rq * rq;
            c += rr * rr;
        }
    }
    r = sqrt(a);
    rp = sqrt(b);
    s = sqrt(c);
}

// -------------------------------------------------------------------------------------------
// Splines.

__device__ __forceinline__ double EvalCubic(const CubicTable& t, double x) {
    x = fmin(fmax(x, t.x0), t.x1);
    int i;
    if (t.uniform) {
        i = (int)floor((x - t.x0) * t.inv_dx);
        i = min(max(i, 0), t.n - 2);
    } else {
        int j = (int)floor((x - t.x0) * t.inv_dx);
        j = min(max(j, 0), t.n_bucket - 1);
        i = t.bucket[j];
        while (i < t.n - 2 && __ldg(&t.x[i + 1]) <= x) ++i;
    }
    const Cubic4 c = t.c[i];
    const double u = x - __ldg(&t.x[i]);
    return c.c0 + u * (c.c1 + u * (c.c2 + u * c.c3));
}

/// Value and slope of a CubicTable at x clamped to the grid (the slope of the edge interval at an
/// end, as einspline's _vg evaluation of an argument the caller has clamped).
__device__ __forceinline__ void EvalCubicVG(const CubicTable& t, double x, double& v, double& g) {
    x = fmin(fmax(x, t.x0), t.x1);
    int i;
    if (t.uniform) {
        i = (int)floor((x - t.x0) * t.inv_dx);
        i = min(max(i, 0), t.n - 2);
    } else {
        int j = (int)floor((x - t.x0) * t.inv_dx);
        j = min(max(j, 0), t.n_bucket - 1);
        i = t.bucket[j];
        while (i < t.n - 2 && __ldg(&t.x[i + 1]) <= x) ++i;
    }
    const Cubic4 c = t.c[i];
    const double u = x - __ldg(&t.x[i]);
    v = c.c0 + u * (c.c1 + u * (c.c2 + u * c.c3));
    g = c.c1 + u * (2. * c.c2 + 3. * u * c.c3);
}

/// Cell of a 2-D table axis holding x: the last knot at or below x, within [0, n - 2] (so an
/// argument outside the grid takes the edge cell).
__device__ __forceinline__ int GridCell(const GridDev& g, double x) {
    int i;
    const double xc = fmin(fmax(x, g.x0), g.x1);
    if (g.uniform) {
        i = (int)floor((xc - g.x0) * g.inv_dx);
        i = min(max(i, 0), g.n - 2);
    } else {
        int j = (int)floor((xc - g.x0) * g.inv_dx);
        j = min(max(j, 0), g.n_bucket - 1);
        i = g.bucket[j];
        while (i < g.n - 2 && __ldg(&g.x[i + 1]) <= xc) ++i;
    }
    return i;
}

/// Value and partial derivatives of a BicubicTable at (x, y); the cell polynomial is evaluated at
/// the unclamped arguments.
__device__ __forceinline__ double EvalBicubic(const BicubicTable& t, double x, double y, double* fx = nullptr, double* fy = nullptr) {
    const int i = GridCell(t.gx, x), j = GridCell(t.gy, y);
    const double u = x - __ldg(&t.gx.x[i]), v = y - __ldg(&t.gy.x[j]);
    const double* c = t.c + ((size_t)i * (t.gy.n - 1) + j) * 16;
    double row[4], drow[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const double c0 = __ldg(&c[4 * a]), c1 = __ldg(&c[4 * a + 1]), c2 = __ldg(&c[4 * a + 2]), c3 = __ldg(&c[4 * a + 3]);
        row[a] = c0 + v * (c1 + v * (c2 + v * c3));
        drow[a] = c1 + v * (2. * c2 + 3. * v * c3);
    }
    if (fx) *fx = row[1] + u * (2. * row[2] + 3. * u * row[3]);
    if (fy) *fy = drow[0] + u * (drow[1] + u * (drow[2] + u * drow[3]));
    return row[0] + u * (row[1] + u * (row[2] + u * row[3]));
}

/// Component m of a MultiCubic on interval i at offset u from the interval's knot.
__device__ __forceinline__ double MultiComp(const MultiCubic& t, int i, double u, int m) {
    const Cubic4 c = t.c[(size_t)i * t.n_comp + m];
    return c.c0 + u * (c.c1 + u * (c.c2 + u * c.c3));
}

/// Interval of a MultiCubic holding x clamped to the grid, and the offset from its knot.
__device__ __forceinline__ int MultiInterval(const MultiCubic& t, double x, double& u) {
    x = fmin(fmax(x, t.g.x0), t.g.x1);
    const int i = GridCell(t.g, x);
    u = x - __ldg(&t.g.x[i]);
    return i;
}

/// Free-particle log density with periodic-image correction (free_spline_class.h:76-84):
/// -sum_d image(dr_d) - |dr|^2 / (4 lambda tau).
__device__ __forceinline__ double LogRhoFree(const double* dr, uint32_t n_d, double i4lt, const CubicTable* image, int has_images) {
    double tot = 0., r2 = 0.;
    for (uint32_t d = 0; d < n_d; ++d) {
        if (has_images) tot -= EvalCubic(*image, dr[d]);
        r2 += dr[d] * dr[d];
    }
    return tot - r2 * i4lt;
}

// -------------------------------------------------------------------------------------------
// Charge-density phases (k_space_class.h:83-94, bead_class.h:125-133).

__device__ __forceinline__ double2 CMul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

__device__ __forceinline__ int KIdx(int32_t packed, int d) { return (int)((packed >> (8 * d)) & 0xff) - 128; }

/// c_d(n) = exp(i n box_d r_d) for n = 0..max_index by the reference's recurrence; tab[n].
__device__ __forceinline__ void PhaseRow(double r, double box, int max_index, double2* tab) {
    double s, c;
    sincos(r * box, &s, &c);
    const double2 t = make_double2(c, s);
    double2 v = make_double2(1., 0.);
    tab[0] = v;
    for (int n = 1; n <= max_index; ++n) {
        v = CMul(t, v);
        tab[n] = v;
    }
}

/// prod_d c_d(n_d) for one packed k-vector from per-dimension tables (row stride `stride`).
__device__ __forceinline__ double2 PhaseProduct(const double2* tab, int stride, uint32_t n_d, int32_t packed) {
    double2 f = make_double2(1., 0.);
    for (uint32_t d = 0; d < n_d; ++d) {
        int n = KIdx(packed, (int)d);
        double2 c = tab[d * stride + (n < 0 ? -n : n)];
        if (n < 0) c.y = -c.y;
        f = d == 0 ? c : CMul(f, c);
    }
    return f;
}

// -------------------------------------------------------------------------------------------
// Deterministic reductions (fixed shuffle tree, fixed warp order).

__device__ __forceinline__ double WarpSum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/// Block-wide sum; every thread returns the same value. `red` holds >= blockDim.x/32 doubles.
__device__ __forceinline__ double BlockSum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = WarpSum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.;
    if (warp == 0) {
        t = lane < nw ? red[lane] : 0.;
        t = WarpSum(t);
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

// -------------------------------------------------------------------------------------------
// Bounded grid barrier for cooperative (co-resident) launches.
//
// A monotonic 64-bit arrival counter zeroed before the launch; generation g completes when the
// counter reaches g * gridDim.x. Every wait is bounded by `timeout_ns` of %globaltimer and by an
// iteration cap: on expiry the waiting block sets the error word and every block leaves its loop.

__device__ __forceinline__ uint64_t GlobalTimerNs() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint64_t LoadAcquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int LoadVolatile(const int* p) { return *(const volatile int*)p; }

/// Generation `gen` (1, 2, ...; every thread passes the same value) of the barrier. Returns false
/// if the barrier failed (timeout or another block's error); all threads of the block agree.
__device__ __forceinline__ bool GridBarrier(unsigned long long* ctr, uint64_t gen, int* err, uint64_t timeout_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint64_t target = gen * (uint64_t)gridDim.x;
        // Release-ordered arrival: this thread's earlier global writes (the block's partial) are
        // visible to any block that observes the incremented counter with an acquire load.
        asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(ctr), "l"(1ull) : "memory");
        const uint64_t t0 = GlobalTimerNs();
        uint32_t iters = 0;
        int ok = 1;
        for (;;) {
            if (LoadAcquire(ctr) >= target) break;
            ++iters;
            if ((iters & 63u) == 0u && LoadVolatile(err) != 0) { ok = 0; break; }
            if ((iters & 1023u) == 0u && (GlobalTimerNs() - t0 > timeout_ns || iters > (1u << 30))) {
                atomicCAS(err, 0, kDevErrTimeout);
                ok = 0;
                break;
            }
            if (iters > 4096u) __nanosleep(32);
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace pimc
