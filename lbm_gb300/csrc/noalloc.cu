// Residual reduction for callers that cannot allocate device memory.
//
// lbm_gpu_residual() reduces a context's variables with scratch space the
// context allocated with cudaMalloc.  Some callers cannot make that call: code
// whose device memory belongs to another allocator (a framework's caching
// allocator or a fixed arena handed out by a host application), and code on a
// latency-critical path where cudaMalloc's implicit device-wide
// synchronisation is not acceptable.  lbm_gpu_residual_noalloc() runs the same
// two-pass FP64 reduction (reduce.cu) on device arrays the caller owns, with
// its per-block partial sums in a fixed-size array that lives in the
// library's own device image instead of in allocated memory.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/lbm_gpu.h"
#include "engine.h"

namespace {

// One partial sum per block of the first pass and per variable.  The first
// pass uses at most LBM_GPU_NOALLOC_MAX_BLOCKS blocks (reduce_blocks caps it),
// so this bounds the scratch at 304 x 8 doubles = 19 KB, held by every GPU
// that loads the library until the process exits.
constexpr int NOALLOC_MAX_BLOCKS = 304;
static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_BLOCKS * LBM_GPU_NOALLOC_MAX_VARS];

constexpr int MAX_DEVICES = 64;
std::mutex    g_setup_mutex;
double*       g_partials_addr[MAX_DEVICES] = {};  // device address of the array, per device ordinal

}  // namespace

extern "C" int lbm_gpu_residual_noalloc(const double* vars, const double* varsold, int64_t ncells, int32_t nvar, double* out,
                                        void* stream) {
  if(!vars || !varsold || !out || ncells <= 0 || nvar <= 0) return LBM_ERR_INVALID;
  if(nvar > LBM_GPU_NOALLOC_MAX_VARS) return LBM_ERR_INVALID;  // the scratch holds at most this many variables
  int dev = -1;
  if(cudaGetDevice(&dev) != cudaSuccess) return LBM_ERR_CUDA;
  if(dev < 0 || dev >= MAX_DEVICES) return LBM_ERR_UNSUPPORTED;
  double* scratch = nullptr;
  {
    // the address of the array in this device's copy of the module.  In host
    // code the name g_noalloc_partials is only a host-side stand-in, so
    // kernels must be given this address instead.  It is looked up on the
    // first call on a device and again on every call whose stream is not
    // being captured: a device reset (cudaDeviceReset, or another library
    // resetting the primary context) loads the module again, possibly at
    // another address.  A call during stream capture uses the address of the
    // last call outside capture on that device.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if(cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess) return LBM_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if(!g_partials_addr[dev] || cap == cudaStreamCaptureStatusNone) {
      if(cap != cudaStreamCaptureStatusNone) return LBM_ERR_INVALID;  // first call on this device inside a capture
      void*       addr = nullptr;
      cudaError_t e    = cudaGetSymbolAddress(&addr, g_noalloc_partials);
      if(e != cudaSuccess || !addr) return LBM_ERR_CUDA;
      g_partials_addr[dev] = static_cast<double*>(addr);
    }
    scratch = g_partials_addr[dev];
  }
  const int nblocks = lbm::reduce_blocks(ncells);
  if(nblocks > NOALLOC_MAX_BLOCKS) return LBM_ERR_UNSUPPORTED;
  // every partial slot the final pass reads is written by the first pass of
  // the same call, so the array needs no clearing between calls
  const cudaError_t e =
      lbm::reduce_abs_diff(vars, varsold, ncells, nvar, scratch, nblocks, out, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}
