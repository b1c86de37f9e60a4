// reduce.cuh -- deterministic block and grid reductions.
//
// Every reduction runs in a fixed order (warp shuffle tree, then warps in
// index order, then per-CTA partials in CTA order), so a given launch
// configuration always returns the same bits.
#pragma once
#include "iegpu_internal.cuh"

namespace iegpu {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block of NV values per thread; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double sh[NV][32];  // up to 32 warps per block
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[q][w] = v[q];
    }
    __syncthreads();
    if (w == 0) {
        const int nw = (int)(blockDim.x >> 5);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double x = lane < nw ? sh[q][lane] : 0.0;
            v[q] = warp_sum(x);
        }
    }
    __syncthreads();
}

// Sum of part[b*NV + q] over b = 0..nb-1 by warp 0 in a fixed order; the
// result is valid in lane 0.  Each lane walks its slots once for all NV
// values, several slots' loads in flight.
template <int NV>
__device__ __forceinline__ void sum_partials(const double* part, int nb, double (&out)[NV]) {
    const int lane = threadIdx.x & 31;
    double s[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) s[q] = 0.0;
#pragma unroll 4
    for (int b = lane; b < nb; b += 32) {
#pragma unroll
        for (int q = 0; q < NV; ++q) s[q] += __ldcg(&part[(size_t)b * NV + q]);
    }
#pragma unroll
    for (int q = 0; q < NV; ++q) out[q] = warp_sum(s[q]);
}

// Last-CTA detection after each CTA wrote its partials.
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    return last;
}

}  // namespace iegpu
