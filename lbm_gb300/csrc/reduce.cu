// FP64 reductions: the reference's convergence residual sumAbsDiff
// (src/lbm/solver.cpp:808-815) and the global mass / momentum sums.
//
// Two passes with a fixed block count, warp-shuffle trees inside a block and a
// single-block final pass over the partials, so the result is deterministic
// (the same bits on every run) although its summation order differs from the
// reference's sequential loop.
#include <cuda_runtime.h>

#include "engine.h"
#include "lattice.cuh"

namespace lbm {
namespace {

constexpr int RTPB = 256;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// block-wide sum; valid in thread 0
__device__ __forceinline__ double block_sum(double x, double* sh) {
  x             = warp_sum(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if(lane == 0) sh[wid] = x;
  __syncthreads();
  x = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
  if(wid == 0) x = warp_sum(x);
  __syncthreads();
  return x;
}

// partials[v * gridDim.x + block] = sum over the block's stride of |a - b|
__global__ void __launch_bounds__(RTPB) k_absdiff_partial(const double* a, const double* b, int64_t n, int nvec, double* partials) {
  __shared__ double sh[RTPB / 32];
  for(int v = 0; v < nvec; ++v) {
    double acc = 0;
    for(int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x)
      acc += fabs(a[v * n + i] - b[v * n + i]);
    acc = block_sum(acc, sh);
    if(threadIdx.x == 0) partials[v * gridDim.x + blockIdx.x] = acc;
  }
}

// out[v] = sum of the nblocks partials of vector v (one block, fixed order)
__global__ void __launch_bounds__(RTPB) k_final(const double* partials, int nblocks, int nvec, double* out) {
  __shared__ double sh[RTPB / 32];
  for(int v = 0; v < nvec; ++v) {
    double acc = 0;
    for(int i = threadIdx.x; i < nblocks; i += blockDim.x) acc += partials[v * nblocks + i];
    acc = block_sum(acc, sh);
    if(threadIdx.x == 0) out[v] = acc;
  }
}

// zeroth and first moments summed over all cells: sum_q f, sum_q c_q f
template <int LAT>
__global__ void __launch_bounds__(RTPB) k_moment_partial(const double* f, int64_t n, double* partials) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  __shared__ double sh[RTPB / 32];
  double acc[D + 1];
#pragma unroll
  for(int k = 0; k <= D; ++k) acc[k] = 0;
  for(int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      const double x = f[q * n + i];
      acc[0] += x;
#pragma unroll
      for(int d = 0; d < D; ++d) acc[d + 1] += static_cast<double>(L::c(q, d)) * x;
    }
  }
#pragma unroll
  for(int k = 0; k <= D; ++k) {
    const double s = block_sum(acc[k], sh);
    if(threadIdx.x == 0) partials[k * gridDim.x + blockIdx.x] = s;
  }
}

}  // namespace

int reduce_blocks(int64_t n) {
  // two resident blocks per SM on a 152-SM part, fewer for small inputs
  const int64_t want = (n + RTPB * 8 - 1) / (RTPB * 8);
  return static_cast<int>(want < 1 ? 1 : (want > 304 ? 304 : want));
}

cudaError_t reduce_abs_diff(const double* a, const double* b, int64_t n, int nvec, double* partials, int nblocks, double* out,
                            cudaStream_t s) {
  k_absdiff_partial<<<nblocks, RTPB, 0, s>>>(a, b, n, nvec, partials);
  k_final<<<1, RTPB, 0, s>>>(partials, nblocks, nvec, out);
  return cudaGetLastError();
}

cudaError_t reduce_moments(const double* f, int64_t n, int Q, int lattice, double* partials, int nblocks, double* out,
                           cudaStream_t s) {
  (void)Q;
  int D = 0;
  switch(lattice) {
    case LBM_D1Q3: k_moment_partial<LBM_D1Q3><<<nblocks, RTPB, 0, s>>>(f, n, partials); D = 1; break;
    case LBM_D2Q5: k_moment_partial<LBM_D2Q5><<<nblocks, RTPB, 0, s>>>(f, n, partials); D = 2; break;
    case LBM_D2Q9: k_moment_partial<LBM_D2Q9><<<nblocks, RTPB, 0, s>>>(f, n, partials); D = 2; break;
    case LBM_D3Q7: k_moment_partial<LBM_D3Q7><<<nblocks, RTPB, 0, s>>>(f, n, partials); D = 3; break;
    case LBM_D3Q19: k_moment_partial<LBM_D3Q19><<<nblocks, RTPB, 0, s>>>(f, n, partials); D = 3; break;
    default: return cudaErrorInvalidValue;
  }
  k_final<<<1, RTPB, 0, s>>>(partials, nblocks, D + 1, out);
  return cudaGetLastError();
}

}  // namespace lbm
