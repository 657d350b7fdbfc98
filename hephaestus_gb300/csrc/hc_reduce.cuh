// hc_reduce.cuh -- deterministic block and grid reductions in FP64.
//
// A grid reduction writes one partial per block; the block that takes the last
// ticket sums the partials in a fixed order, so results do not depend on block
// scheduling.  The ticket counter is reset by that block for the next launch.
#pragma once
#include <cuda_runtime.h>

namespace hc {

// Sum of v over the block; the result is valid on thread 0.
template <int NV>
__device__ __forceinline__ void block_sum_n(double (&v)[NV]) {
  __shared__ double sh[NV][32];
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][w] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int i = 0; i < nw; ++i) s += sh[k][i];
      v[k] = s;
    }
  }
}

// Each block contributes v[0..NV-1] (valid on thread 0).  Returns true on
// thread 0 of the last block, with tot[] holding the grid totals.
template <int NV>
__device__ __forceinline__ bool grid_sum_n(double (&v)[NV], double* partials, unsigned int* counter,
                                           double (&tot)[NV]) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[(size_t)k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    s[k] = 0.0;
    for (unsigned int i = threadIdx.x; i < gridDim.x; i += blockDim.x)
      s[k] += ((volatile double*)partials)[(size_t)k * gridDim.x + i];
  }
  block_sum_n<NV>(s);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = s[k];
    *counter = 0u;
    return true;
  }
  return false;
}

}  // namespace hc
