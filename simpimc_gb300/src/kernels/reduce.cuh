// Deterministic FP64 sums of per-item values on the context's stream: a fixed grid-stride split,
// block sums by a fixed shuffle tree, then one warp adding the block partials in order. The
// result does not depend on timing, so GPU parity against the oracle is reproducible.
#pragma once

#include <algorithm>
#include <cstdint>

#include "../framework/context.h"
#include "device_common.cuh"

namespace pimc {
namespace {

constexpr int kSumThreads = 256;

template <int N, class F>
__global__ void __launch_bounds__(kSumThreads) SumItemsKernel(uint64_t n, F f, double* __restrict__ partials) {
    __shared__ double red[kSumThreads / 32];
    double acc[N];
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] = 0.;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double v[N];
        f(i, v);
#pragma unroll
        for (int j = 0; j < N; ++j) acc[j] += v[j];
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const double s = BlockSum(acc[j], red);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * N + j] = s;
    }
}

template <int N>
__global__ void FinalSumKernel(const double* __restrict__ partials, int nb, double* __restrict__ out) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        double t = 0.;
        for (int b = lane; b < nb; b += 32) t += partials[(size_t)b * N + j];
        t = WarpSum(t);
        if (lane == 0) out[j] = t;
    }
}

/// Sum f(i) over i in [0, n) for N-component items; result copied to host `out`.
template <int N, class F>
void SumItems(Context& c, uint64_t n, F f, double* out) {
    for (int j = 0; j < N; ++j) out[j] = 0.;
    if (n == 0) return;
    const uint64_t want = (n + kSumThreads - 1) / kSumThreads;
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)c.n_sm * 8));
    double* part = c.Partials((size_t)blocks * N);
    SumItemsKernel<N><<<blocks, kSumThreads, 0, c.stream>>>(n, f, part);
    CudaCheck(cudaGetLastError(), "sum kernel launch");
    FinalSumKernel<N><<<1, 32, 0, c.stream>>>(part, blocks, c.Result());
    CudaCheck(cudaGetLastError(), "final sum launch");
    CudaCheck(cudaMemcpyAsync(out, c.Result(), N * sizeof(double), cudaMemcpyDeviceToHost, c.stream), "read result");
    c.Sync();
}

}  // namespace
}  // namespace pimc
