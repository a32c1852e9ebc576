// Batched engine: many independent D2Q9 lid-driven cavities of different sizes
// advance together, one persistent launch per time step.
//
// Each cavity is its own n x n box (halfway bounce-back on all four walls, the
// +y wall moving in x, as the reference's moving-wall bounce-back,
// src/lbm/bnd/bnd_dirichlet.h:79-121 with rho_w = 1), stored as Q planes of
// scaled deviations (the dense-box engine's state, step_common.cuh) and
// streamed in place with the AA pattern.  The work of a step is a list of
// warp tiles -- 32 consecutive cells of one row of one active cavity -- and a
// fixed grid of resident blocks strides over it, so small and large cavities
// share the machine without one launch per cavity.  Converged cavities drop
// out of the active list between steps; the tile count is read from device
// memory, so the captured step graph stays valid as the list shrinks.
// Per-cavity residuals (the reference's sumAbsDiff, src/lbm/solver.cpp:808-815)
// are reduced deterministically: one partial per warp tile, then one block
// per cavity over its contiguous tile range.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "batch.h"
#include "lattice.cuh"
#include "step_common.cuh"

namespace lbm {
namespace {

using L9 = Lattice<LBM_D2Q9>;
constexpr int Q9 = 9, NV9 = 3;

template <class V>
__device__ __forceinline__ V wsum(V v) {
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// moving-lid momentum, in state units, for a population arriving in
// direction k through the +y wall
template <class C>
__device__ __forceinline__ C lid_term(int k, C lid) {
  return static_cast<C>(6.0 * STATE_SCALE) * static_cast<C>(L9::c(k, 0)) * lid;
}

template <int ST, bool ODD, int MOM>
__global__ void __launch_bounds__(256) k_batch(BatchParams P) {
  using S = Store<ST>;
  using T = typename S::T;
  using C = typename S::C;
  const int     lane   = threadIdx.x & 31;
  const int64_t warp   = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const int     na     = *P.nactive;
  if(na <= 0) return;
  const int64_t total = P.tile_start[na];
  T*            A     = static_cast<T*>(P.pop);
  const C       lid   = prm<C>(P.lid, P.lid_f);
  // each warp takes one contiguous run of tiles: the active domain is found
  // once by binary search and then advances only where the run crosses into
  // the next domain
  const int64_t chunk = (total + nwarps - 1) / nwarps;
  const int64_t t0 = warp * chunk, t1 = t0 + chunk < total ? t0 + chunk : total;
  int           lo = 0;
  if(t0 < t1) {
    int hi = na - 1;  // last active domain whose tiles start at or before t0
    while(lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if(P.tile_start[mid] <= t0) lo = mid;
      else hi = mid - 1;
    }
  }
  // the current domain and the tile's row and column, advanced tile by tile
  // (a division only where the run enters a domain)
  int     dom = -1, ty = 0, tx = 0;
  int64_t next_start = 0;
  for(int64_t t = t0; t < t1; ++t) {
    if(dom < 0 || t >= next_start) {
      while(lo + 1 < na && P.tile_start[lo + 1] <= t) ++lo;
      dom        = P.active[lo];
      next_start = lo + 1 < na ? P.tile_start[lo + 1] : total;
      const int64_t r   = t - P.tile_start[lo];
      const int     tpr = P.dom[dom].tiles_per_row;
      ty                = static_cast<int>(r / tpr);
      tx                = static_cast<int>(r - static_cast<int64_t>(ty) * tpr);
    }
    const BatchDomain D = P.dom[dom];
    const int         y = ty;
    const int         x = tx * 32 + lane;
    const int         n = D.n;
    if(++tx == D.tiles_per_row) {  // the next tile of this run
      tx = 0;
      ++ty;
    }
    C                 diff[NV9] = {C(0), C(0), C(0)};  // summed in the arithmetic type, stored as FP64
    if(x < n) {
      T*            Ad   = A + D.pop_off;
      const int64_t pl   = D.plane;
      const int     cell = x + n * y;
      C             v[Q9];
      C             prev[NV9];  // previous moments, read with the populations
      if constexpr(MOM == 2) {
        const C* M = static_cast<const C*>(P.mom) + D.mom_off;
#pragma unroll
        for(int k = 0; k < NV9; ++k) prev[k] = M[k * pl + cell];
      }
      const bool    fast = x > 0 && x < n - 1 && y > 0 && y < n - 1;
      if constexpr(!ODD) {
        static_for<Q9>([&](auto qc) { v[decltype(qc)::value] = S::load(Ad[decltype(qc)::value * pl + cell]); });
      } else if(fast) {
        static_for<Q9>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          v[q]            = S::load(Ad[L9::opp(q) * pl + cell - (L9::c(q, 0) + n * L9::c(q, 1))]);
        });
      } else {
        static_for<Q9>([&](auto qc) {
          constexpr int q  = decltype(qc)::value;
          const int     sx = x - L9::c(q, 0), sy = y - L9::c(q, 1);
          if(sx < 0 || sx >= n || sy < 0 || sy >= n) {
            C b = S::load(Ad[q * pl + cell]);  // the cell's own bounced population
            if(sy >= n) b += lid_term<C>(q, lid);
            v[q] = b;
          } else {
            v[q] = S::load(Ad[L9::opp(q) * pl + sx + n * sy]);
          }
        });
      }
      C mom[NV9];
      C F[3] = {0, 0, 0};
      collide_ns<LBM_D2Q9, C, false>(prm<C>(D.omega, D.omega_f), false, F, v, MOM ? mom : nullptr);
      if constexpr(MOM != 0) {
        C* M = static_cast<C*>(P.mom) + D.mom_off;
#pragma unroll
        for(int k = 0; k < NV9; ++k) {
          if constexpr(MOM == 2) diff[k] = fabs(mom[k] - prev[k]);
          M[k * pl + cell] = mom[k];
        }
      }
      if constexpr(!ODD) {
        static_for<Q9>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          Ad[L9::opp(q) * pl + cell] = S::store(v[q]);
        });
      } else if(fast) {
        static_for<Q9>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          Ad[q * pl + cell + L9::c(q, 0) + n * L9::c(q, 1)] = S::store(v[q]);
        });
      } else {
        static_for<Q9>([&](auto qc) {
          constexpr int q  = decltype(qc)::value;
          const int     tx = x + L9::c(q, 0), ty = y + L9::c(q, 1);
          if(tx < 0 || tx >= n || ty < 0 || ty >= n) {
            constexpr int o = L9::opp(q);
            C             b = v[q];
            if(ty >= n) b += lid_term<C>(o, lid);
            Ad[o * pl + cell] = S::store(b);
          } else {
            Ad[q * pl + tx + n * ty] = S::store(v[q]);
          }
        });
      }
    }
    if constexpr(MOM == 2) {
#pragma unroll
      for(int k = 0; k < NV9; ++k) {
        const C s = wsum(diff[k]);
        if(lane == 0) P.partials[k * P.partial_stride + t] = static_cast<double>(s);
      }
    }
  }
}

// per active domain: the sum of its tiles' partials
__global__ void k_batch_domain_sum(BatchParams P, double* out) {
  __shared__ double sh[32];
  const int     i  = blockIdx.x;
  const int     d  = P.active[i];
  const int64_t t0 = P.tile_start[i], t1 = P.tile_start[i + 1];
  for(int k = 0; k < NV9; ++k) {
    double acc = 0;
    for(int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) acc += P.partials[k * P.partial_stride + t];
    acc = wsum(acc);
    if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if(threadIdx.x < 32) {
      double s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
      s        = wsum(s);
      if(threadIdx.x == 0) out[d * NV9 + k] = s;
    }
    __syncthreads();
  }
}

template <int ST>
__global__ void k_batch_init(BatchParams P, int nd) {
  using S = Store<ST>;
  using T = typename S::T;
  // rest equilibrium: zero deviation everywhere (including padding)
  const int64_t total = P.dom[nd - 1].pop_off + Q9 * P.dom[nd - 1].plane;
  T*            A     = static_cast<T*>(P.pop);
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total; i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    A[i] = S::store(static_cast<typename S::C>(0));
}

// FP64 post-stream populations of one domain (odd: resolve the pull)
template <int ST>
__global__ void k_batch_readout(BatchParams P, int d, bool odd, double* out) {
  using S = Store<ST>;
  using T = typename S::T;
  using C = typename S::C;
  const BatchDomain D  = P.dom[d];
  const int         n  = D.n;
  const int64_t     nc = static_cast<int64_t>(n) * n;
  const int64_t     c  = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if(c >= nc) return;
  const int      x  = static_cast<int>(c % n), y = static_cast<int>(c / n);
  const T*       Ad = static_cast<const T*>(P.pop) + D.pop_off;
  const int64_t  pl = D.plane;
  const C        lid = prm<C>(P.lid, P.lid_f);
  for(int q = 0; q < Q9; ++q) {
    C val;
    if(!odd) {
      val = S::load(Ad[q * pl + c]);
    } else {
      const int sx = x - L9::c(q, 0), sy = y - L9::c(q, 1);
      if(sx < 0 || sx >= n || sy < 0 || sy >= n) {
        val = S::load(Ad[q * pl + c]);
        if(sy >= n) val += lid_term<C>(q, lid);
      } else {
        val = S::load(Ad[L9::opp(q) * pl + sx + n * sy]);
      }
    }
    out[q * nc + c] = L9::w(q) * (1.0 + static_cast<double>(val) / STATE_SCALE);
  }
}

template <int ST>
__global__ void k_batch_load(BatchParams P, int d, const double* in) {
  using S = Store<ST>;
  using T = typename S::T;
  const BatchDomain D  = P.dom[d];
  const int64_t     nc = static_cast<int64_t>(D.n) * D.n;
  const int64_t     c  = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if(c >= nc) return;
  T* Ad = static_cast<T*>(P.pop) + D.pop_off;
  for(int q = 0; q < Q9; ++q)
    Ad[q * D.plane + c] = S::store(static_cast<typename S::C>((in[q * nc + c] - L9::w(q)) * (STATE_SCALE / L9::w(q))));
}

template <int ST>
void launch(BatchState* b, bool odd, int mom, cudaStream_t s) {
  if(odd) {
    if(mom == 0) k_batch<ST, true, 0><<<b->grid, b->tpb, 0, s>>>(b->p);
    else if(mom == 1) k_batch<ST, true, 1><<<b->grid, b->tpb, 0, s>>>(b->p);
    else k_batch<ST, true, 2><<<b->grid, b->tpb, 0, s>>>(b->p);
  } else {
    if(mom == 0) k_batch<ST, false, 0><<<b->grid, b->tpb, 0, s>>>(b->p);
    else if(mom == 1) k_batch<ST, false, 1><<<b->grid, b->tpb, 0, s>>>(b->p);
    else k_batch<ST, false, 2><<<b->grid, b->tpb, 0, s>>>(b->p);
  }
}

cudaError_t step_launch(BatchState* b, bool odd, int mom, cudaStream_t s) {
  switch(b->storage) {
    case LBM_STORE_F64: launch<LBM_STORE_F64>(b, odd, mom, s); break;
    case LBM_STORE_F32: launch<LBM_STORE_F32>(b, odd, mom, s); break;
    case LBM_STORE_F16_DEV: launch<LBM_STORE_F16_DEV>(b, odd, mom, s); break;
    default: launch<LBM_STORE_BF16_DEV>(b, odd, mom, s); break;
  }
  return cudaGetLastError();
}

int cerr(std::string& err, cudaError_t e, const char* what) {
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return LBM_ERR_CUDA;
}

void drop_graphs(BatchState* b) {
  for(auto& g : b->graph)
    if(g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// upload the active list and its tile prefix
cudaError_t upload_active(BatchState* b, cudaStream_t s) {
  std::vector<int64_t> ts(b->active.size() + 1, 0);
  for(size_t i = 0; i < b->active.size(); ++i) {
    const BatchDomain& D = b->dom[b->active[i]];
    ts[i + 1]            = ts[i] + static_cast<int64_t>(D.n) * D.tiles_per_row;
  }
  b->total_tiles = ts.back();
  const int32_t na = static_cast<int32_t>(b->active.size());
  cudaError_t   e  = cudaMemcpyAsync(b->d_tile_start, ts.data(), sizeof(int64_t) * ts.size(), cudaMemcpyHostToDevice, s);
  if(e == cudaSuccess && na > 0) e = cudaMemcpyAsync(b->d_active, b->active.data(), sizeof(int32_t) * na, cudaMemcpyHostToDevice, s);
  if(e == cudaSuccess) e = cudaMemcpyAsync(b->d_nactive, &na, sizeof(int32_t), cudaMemcpyHostToDevice, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace

cudaError_t batch_initial_condition(BatchState* b, cudaStream_t s) {
  switch(b->storage) {
    case LBM_STORE_F64: k_batch_init<LBM_STORE_F64><<<1024, 256, 0, s>>>(b->p, b->ndomains); break;
    case LBM_STORE_F32: k_batch_init<LBM_STORE_F32><<<1024, 256, 0, s>>>(b->p, b->ndomains); break;
    case LBM_STORE_F16_DEV: k_batch_init<LBM_STORE_F16_DEV><<<1024, 256, 0, s>>>(b->p, b->ndomains); break;
    default: k_batch_init<LBM_STORE_BF16_DEV><<<1024, 256, 0, s>>>(b->p, b->ndomains); break;
  }
  b->active.resize(b->ndomains);
  for(int d = 0; d < b->ndomains; ++d) b->active[d] = d;
  std::fill(b->steps.begin(), b->steps.end(), 0);
  std::fill(b->status.begin(), b->status.end(), static_cast<int32_t>(LBM_BATCH_ACTIVE));
  b->global_steps = 0;
  b->mom_valid    = 0;
  b->res_ready    = 0;
  cudaError_t e   = cudaGetLastError();
  if(e == cudaSuccess) e = upload_active(b, s);
  return e;
}

int batch_step(BatchState* b, int64_t nsteps, cudaStream_t s, std::string& err) {
  if(b->active.empty()) return LBM_OK;
  const int64_t plain = nsteps >= 2 ? nsteps - 2 : 0;
  for(int64_t k = 0; k < plain; ++k) {
    const int parity = static_cast<int>(b->global_steps & 1);
    if(!b->graph[parity]) {
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      if(e != cudaSuccess) return cerr(err, e, "begin capture");
      e              = step_launch(b, parity != 0, 0, s);
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if(e != cudaSuccess) return cerr(err, e, "launch");
      if(e2 != cudaSuccess) return cerr(err, e2, "end capture");
      e = cudaGraphInstantiate(&b->graph[parity], g, 0);
      cudaGraphDestroy(g);
      if(e != cudaSuccess) return cerr(err, e, "instantiate");
    }
    cudaError_t e = cudaGraphLaunch(b->graph[parity], s);
    if(e != cudaSuccess) return cerr(err, e, "graph launch");
    ++b->global_steps;
    b->mom_valid = 0;
    b->res_ready = 0;
  }
  for(int64_t k = plain; k < nsteps; ++k) {
    const int   mom = b->mom_valid ? 2 : 1;
    cudaError_t e   = step_launch(b, (b->global_steps & 1) != 0, mom, s);
    if(e != cudaSuccess) return cerr(err, e, "step");
    ++b->global_steps;
    b->mom_valid = 1;
    b->res_ready = mom == 2;
  }
  for(int32_t d : b->active) b->steps[d] += nsteps;
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? LBM_OK : cerr(err, e, "step sync");
}

void batch_destroy(BatchState* b) {
  if(!b) return;
  drop_graphs(b);
  cudaFree(b->d_dom);
  cudaFree(b->d_active);
  cudaFree(b->d_tile_start);
  cudaFree(b->d_nactive);
  cudaFree(b->pop);
  cudaFree(b->mom);
  cudaFree(b->partials);
  cudaFree(b->d_res);
  cudaFree(b->f64);
  delete b;
}

int batch_info(const BatchState* b, int64_t* ncells, int32_t* q, int32_t* nvar) {
  int64_t n = 0;
  for(const auto& D : b->dom) n += static_cast<int64_t>(D.n) * D.n;
  if(ncells) *ncells = n;
  if(q) *q = Q9;
  if(nvar) *nvar = NV9;
  return LBM_OK;
}

}  // namespace lbm

using namespace lbm;

namespace {
int fail_ctx(lbm_gpu_ctx* ctx, int code, const std::string& msg);
}

extern void lbm_internal_set_error(lbm_gpu_ctx* ctx, const std::string& msg);
extern cudaStream_t lbm_internal_stream(lbm_gpu_ctx* ctx);

namespace {
int fail_ctx(lbm_gpu_ctx* ctx, int code, const std::string& msg) {
  lbm_internal_set_error(ctx, msg);
  return code;
}
}  // namespace

extern "C" {

int lbm_gpu_create_batch(const lbm_batch_desc* desc, const int32_t* sides, const double* omegas, lbm_gpu_ctx** out) {
  if(!desc || !sides || !omegas || !out) return LBM_ERR_INVALID;
  *out = nullptr;
  if(desc->lattice != LBM_D2Q9) return LBM_ERR_UNSUPPORTED;
  if(desc->storage < 0 || desc->storage > 3 || desc->ndomains <= 0) return LBM_ERR_INVALID;
  for(int d = 0; d < desc->ndomains; ++d) {
    if(sides[d] < 3 || sides[d] > 46340) return LBM_ERR_INVALID;
    if(!(omegas[d] > 0.0 && omegas[d] < 2.0)) return LBM_ERR_INVALID;
  }
  if(cudaSetDevice(desc->device) != cudaSuccess) return LBM_ERR_CUDA;
  BatchState* b = new(std::nothrow) BatchState();
  if(!b) return LBM_ERR_NOMEM;
  b->storage  = desc->storage;
  b->device   = desc->device;
  b->ndomains = desc->ndomains;
  b->dom.resize(b->ndomains);
  b->steps.assign(b->ndomains, 0);
  b->status.assign(b->ndomains, LBM_BATCH_ACTIVE);
  b->residual.assign(static_cast<size_t>(b->ndomains) * NV9, 0.0);
  int64_t pop = 0, mom = 0, tiles = 0;
  for(int d = 0; d < b->ndomains; ++d) {
    BatchDomain& D  = b->dom[d];
    D.n             = sides[d];
    D.tiles_per_row = (D.n + 31) / 32;
    D.plane         = (static_cast<int64_t>(D.n) * D.n + 31) / 32 * 32;
    D.pop_off       = pop;
    D.mom_off       = mom;
    D.omega         = omegas[d];
    D.omega_f       = static_cast<float>(omegas[d]);
    pop += Q9 * D.plane;
    mom += NV9 * D.plane;
    tiles += static_cast<int64_t>(D.n) * D.tiles_per_row;
    b->max_plane = std::max(b->max_plane, D.plane);
  }
  const size_t elem  = static_cast<size_t>(lbm_gpu_box_storage_bytes(desc->storage));
  const size_t celem = desc->storage == LBM_STORE_F64 ? 8 : 4;
  cudaError_t  e     = cudaMalloc(&b->pop, elem * pop);
  if(e == cudaSuccess) e = cudaMalloc(&b->mom, celem * mom);
  if(e == cudaSuccess) e = cudaMemset(b->mom, 0, celem * mom);
  if(e == cudaSuccess) e = cudaMalloc(&b->partials, sizeof(double) * NV9 * std::max<int64_t>(tiles, 1));
  if(e == cudaSuccess) e = cudaMalloc(&b->d_res, sizeof(double) * NV9 * b->ndomains);
  if(e == cudaSuccess) e = cudaMemset(b->d_res, 0, sizeof(double) * NV9 * b->ndomains);
  if(e == cudaSuccess) e = cudaMalloc(&b->d_dom, sizeof(BatchDomain) * b->ndomains);
  if(e == cudaSuccess) e = cudaMemcpy(b->d_dom, b->dom.data(), sizeof(BatchDomain) * b->ndomains, cudaMemcpyHostToDevice);
  if(e == cudaSuccess) e = cudaMalloc(&b->d_active, sizeof(int32_t) * b->ndomains);
  if(e == cudaSuccess) e = cudaMalloc(&b->d_tile_start, sizeof(int64_t) * (b->ndomains + 1));
  if(e == cudaSuccess) e = cudaMalloc(&b->d_nactive, sizeof(int32_t));
  if(e != cudaSuccess) {
    batch_destroy(b);
    return e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
  }
  BatchParams& p   = b->p;
  p.dom            = b->d_dom;
  p.active         = b->d_active;
  p.tile_start     = b->d_tile_start;
  p.nactive        = b->d_nactive;
  p.pop            = b->pop;
  p.mom            = b->mom;
  p.partials       = b->partials;
  p.partial_stride = std::max<int64_t>(tiles, 1);
  p.lid            = desc->lid_velocity;
  p.lid_f          = static_cast<float>(desc->lid_velocity);
  cudaStream_t s   = nullptr;
  e                = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if(e == cudaSuccess) e = batch_initial_condition(b, s);
  // autotune the resident grid: blocks per SM x threads per block
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, desc->device);
  if(e == cudaSuccess) {
    float best = 1e30f;
    int   bg = sms * 4, bt = 256;
    for(int tpb : {128, 256}) {
      for(int per : {2, 4, 8, 16}) {
        b->tpb  = tpb;
        b->grid = sms * per;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        step_launch(b, false, 0, s);
        step_launch(b, true, 0, s);
        cudaEventRecord(e0, s);
        step_launch(b, false, 0, s);
        step_launch(b, true, 0, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if(ms < best) {
          best = ms;
          bg   = b->grid;
          bt   = tpb;
        }
      }
    }
    b->grid = bg;
    b->tpb  = bt;
    e       = batch_initial_condition(b, s);
  }
  if(e != cudaSuccess) {
    if(s) cudaStreamDestroy(s);
    batch_destroy(b);
    return LBM_ERR_CUDA;
  }
  lbm_gpu_ctx* ctx = lbm_internal_new_batch_ctx(desc->device, b, s);
  if(!ctx) {
    cudaStreamDestroy(s);
    batch_destroy(b);
    return LBM_ERR_NOMEM;
  }
  *out = ctx;
  return LBM_OK;
}

int lbm_gpu_batch_residuals(lbm_gpu_ctx* ctx, double* res) {
  BatchState* b = lbm_internal_batch(ctx);
  if(!b || !res) return LBM_ERR_INVALID;
  cudaStream_t s = lbm_internal_stream(ctx);
  if(!b->res_ready) return fail_ctx(ctx, LBM_ERR_INVALID, "residuals need a step call of at least two steps");
  if(!b->active.empty()) k_batch_domain_sum<<<static_cast<unsigned>(b->active.size()), 256, 0, s>>>(b->p, b->d_res);
  cudaError_t e = cudaMemcpyAsync(b->residual.data(), b->d_res, sizeof(double) * b->residual.size(), cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return fail_ctx(ctx, LBM_ERR_CUDA, std::string("batch residuals: ") + cudaGetErrorString(e));
  std::copy(b->residual.begin(), b->residual.end(), res);
  return LBM_OK;
}

int lbm_gpu_batch_run(lbm_gpu_ctx* ctx, int64_t max_steps, int64_t check_interval, double tol, int64_t* steps_done) {
  BatchState* b = lbm_internal_batch(ctx);
  if(!b || max_steps < 0 || check_interval < 2) return LBM_ERR_INVALID;
  cudaStream_t s = lbm_internal_stream(ctx);
  std::string  err;
  int64_t      done = 0;
  std::vector<int32_t> diverged;  // cavities whose residual became NaN/Inf: taken out, reported at the end
  while(done < max_steps && !b->active.empty()) {
    const int64_t n  = std::min(check_interval, max_steps - done);
    int           rc = batch_step(b, n, s, err);
    if(rc) return fail_ctx(ctx, rc, err);
    done += n;
    if(n < 2) break;
    std::vector<double> r(b->residual.size());
    rc = lbm_gpu_batch_residuals(ctx, r.data());
    if(rc) return rc;
    std::vector<int32_t> keep;
    for(int32_t d : b->active) {
      const double m = std::max({r[d * NV9], r[d * NV9 + 1], r[d * NV9 + 2]});
      if(!std::isfinite(m)) {
        diverged.push_back(d);
        b->status[d] = LBM_BATCH_DIVERGED;
      } else if(!(m < tol)) {
        keep.push_back(d);
      } else {
        b->status[d] = LBM_BATCH_CONVERGED;
      }
    }
    if(keep.size() != b->active.size()) {
      b->active = keep;
      cudaError_t e = upload_active(b, s);
      if(e != cudaSuccess) return fail_ctx(ctx, LBM_ERR_CUDA, "active list upload");
      b->mom_valid = 0;  // the moment history of the remaining domains is kept, but recompute it to be safe
      b->res_ready = 0;
    }
  }
  if(steps_done) std::copy(b->steps.begin(), b->steps.end(), steps_done);
  if(!diverged.empty()) {
    std::string m = "cavities diverged (non-finite residual):";
    for(size_t i = 0; i < diverged.size() && i < 16; ++i) m += " " + std::to_string(diverged[i]);
    return fail_ctx(ctx, LBM_ERR_DIVERGED, m);
  }
  return LBM_OK;
}

int lbm_gpu_batch_status(lbm_gpu_ctx* ctx, int32_t* status) {
  BatchState* b = lbm_internal_batch(ctx);
  if(!b || !status) return LBM_ERR_INVALID;
  std::copy(b->status.begin(), b->status.end(), status);
  return LBM_OK;
}

int lbm_gpu_batch_get_domain(lbm_gpu_ctx* ctx, int32_t d, double* f) {
  BatchState* b = lbm_internal_batch(ctx);
  if(!b || !f || d < 0 || d >= b->ndomains) return LBM_ERR_INVALID;
  cudaStream_t s  = lbm_internal_stream(ctx);
  const int64_t nc = static_cast<int64_t>(b->dom[d].n) * b->dom[d].n;
  if(!b->f64 && cudaMalloc(&b->f64, sizeof(double) * Q9 * b->max_plane) != cudaSuccess) return LBM_ERR_NOMEM;
  const unsigned g   = static_cast<unsigned>((nc + 255) / 256);
  const bool     odd = (b->steps[d] & 1) != 0;
  switch(b->storage) {
    case LBM_STORE_F64: k_batch_readout<LBM_STORE_F64><<<g, 256, 0, s>>>(b->p, d, odd, b->f64); break;
    case LBM_STORE_F32: k_batch_readout<LBM_STORE_F32><<<g, 256, 0, s>>>(b->p, d, odd, b->f64); break;
    case LBM_STORE_F16_DEV: k_batch_readout<LBM_STORE_F16_DEV><<<g, 256, 0, s>>>(b->p, d, odd, b->f64); break;
    default: k_batch_readout<LBM_STORE_BF16_DEV><<<g, 256, 0, s>>>(b->p, d, odd, b->f64); break;
  }
  cudaError_t e = cudaMemcpyAsync(f, b->f64, sizeof(double) * Q9 * nc, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? LBM_OK : fail_ctx(ctx, LBM_ERR_CUDA, std::string("batch readout: ") + cudaGetErrorString(e));
}

int lbm_gpu_batch_profile_steps(lbm_gpu_ctx* ctx, int64_t nsteps, double* total_ms, double* kernel_ms, int64_t* launches) {
  BatchState* b = lbm_internal_batch(ctx);
  if(!b || nsteps < 0) return LBM_ERR_INVALID;
  cudaStream_t             s = lbm_internal_stream(ctx);
  std::vector<cudaEvent_t> ev(2 * nsteps + 2);
  for(auto& x : ev) cudaEventCreate(&x);
  cudaEventRecord(ev[0], s);
  cudaError_t e = cudaSuccess;
  for(int64_t k = 0; k < nsteps && e == cudaSuccess; ++k) {
    int mom = 0;
    if(nsteps >= 2 && k >= nsteps - 2) mom = b->mom_valid ? 2 : 1;
    cudaEventRecord(ev[2 + 2 * k], s);
    e = step_launch(b, (b->global_steps & 1) != 0, mom, s);
    cudaEventRecord(ev[3 + 2 * k], s);
    ++b->global_steps;
    b->mom_valid = mom != 0;
    b->res_ready = mom == 2;
  }
  for(int32_t d : b->active) b->steps[d] += nsteps;
  cudaEventRecord(ev[1], s);
  if(e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
  double tot = 0, ker = 0;
  if(e == cudaSuccess) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev[0], ev[1]);
    tot = ms;
    for(int64_t k = 0; k < nsteps; ++k) {
      cudaEventElapsedTime(&ms, ev[2 + 2 * k], ev[3 + 2 * k]);
      ker += ms;
    }
  }
  for(auto& x : ev) cudaEventDestroy(x);
  if(e != cudaSuccess) return fail_ctx(ctx, LBM_ERR_CUDA, std::string("batch profile: ") + cudaGetErrorString(e));
  if(total_ms) *total_ms = tot;
  if(kernel_ms) *kernel_ms = ker;
  if(launches) *launches = nsteps;
  return LBM_OK;
}

int lbm_gpu_batch_tuning(lbm_gpu_ctx* ctx, int32_t* grid, int32_t* threads_per_block) {
  BatchState* b = lbm_internal_batch(ctx);
  if(!b) return LBM_ERR_INVALID;
  if(grid) *grid = b->grid;
  if(threads_per_block) *threads_per_block = b->tpb;
  return LBM_OK;
}

}  // extern "C"
