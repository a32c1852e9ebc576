// Device build of the grid's cells (lbm_grid_create_device, include/lbm_grid.h).
//
// The host builder tests the positions of the level, keeps the cells cut by
// the geometry or inside it, and sorts them by the reference's curve index.
// On two and three dimensions that index is a bijection of the positions
// (each level's quadrant is the position's bit there, and the quadrant table
// permutes 0..2^D-1), so the device enumerates the curve indices in order
// instead of sorting: one thread per index decodes its position, tests it
// with the same geometry code as the host (grid_geom.h; this file is compiled
// without floating-point contraction, and sqrt is correctly rounded on both
// sides), and a prefix sum over the membership flags gives every kept cell its
// id in curve order.  In 1D the index is three times the position, so the
// order is the position order.  Then one thread per cell finds its main
// neighbours (the neighbour position's index, looked up in the id table) and
// its boundary property.  The result equals the host builder's bit for bit.
//
// Memory: one byte and one int32 per position of the level's cube
// (2^(D*level) positions, at most 2^30), plus the cell tables.  No kernel
// waits on another thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/lbm_grid.h"
#include "grid_geom.h"
#include "grid_internal.h"

namespace {

using namespace lbm_grid_geom;

constexpr int      kThreads = 256;
constexpr int      kPer     = 16;  // flags per thread in the scan: one 16-byte load
constexpr int64_t  kTile    = kThreads * kPer;

struct DevGrid {
  int           D = 0, L = 0;
  GeomSet       geom;
  const double* cv[3] = {nullptr, nullptr, nullptr};
  double        cell_length = 0;
  uint64_t      ntot        = 0;  // positions of the level's cube
};

__device__ __forceinline__ void position_of(const DevGrid& G, uint64_t idx, int64_t* p) {
  if(G.D == 1) {
    p[0] = static_cast<int64_t>(idx);
    return;
  }
  curve_position(idx, G.D, G.L, p);
}

__device__ __forceinline__ uint64_t index_of(const DevGrid& G, const int64_t* p) {
  return G.D == 1 ? static_cast<uint64_t>(p[0]) : curve_index_int(p, G.D, G.L);
}

// membership of every position, in curve order
__global__ void k_grid_member(DevGrid G, uint8_t* flag) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for(uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < G.ntot; i += stride) {
    int64_t p[3];
    position_of(G, i, p);
    double c[3];
    for(int d = 0; d < G.D; ++d) c[d] = G.cv[d][p[d]];
    flag[i] = (set_cut(G.geom, c, G.cell_length, G.D) || set_inside(G.geom, c, G.D)) ? 1 : 0;
  }
}

__device__ __forceinline__ int count16(const uint4 v) {
  // sixteen 0/1 bytes: add them as bytes within each word, then the words
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  int            s    = 0;
  for(int k = 0; k < 4; ++k) s += __popc(w[k]);  // flags are 0 or 1: one set bit each
  return s;
}

// members per tile of kTile flags (the flag array is padded to whole tiles)
__global__ void __launch_bounds__(kThreads) k_grid_tile_count(const uint8_t* flag, int64_t* tile_sum) {
  const uint4 v = reinterpret_cast<const uint4*>(flag + blockIdx.x * kTile)[threadIdx.x];
  int         s = count16(v);
  for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ int warp_sum[kThreads / 32];
  if((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
  __syncthreads();
  if(threadIdx.x == 0) {
    int t = 0;
    for(int w = 0; w < kThreads / 32; ++w) t += warp_sum[w];
    tile_sum[blockIdx.x] = t;
  }
}

// exclusive prefix of the tile sums, in place, and the total (one block)
__global__ void __launch_bounds__(1024) k_grid_scan_tiles(int64_t* tile_sum, int64_t ntiles, int64_t* total) {
  __shared__ int64_t buf[1024];
  __shared__ int64_t carry;
  if(threadIdx.x == 0) carry = 0;
  __syncthreads();
  for(int64_t base = 0; base < ntiles; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < ntiles ? tile_sum[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for(int o = 1; o < 1024; o <<= 1) {  // inclusive scan (Hillis-Steele)
      const int64_t add = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += add;
      __syncthreads();
    }
    if(i < ntiles) tile_sum[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if(threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if(threadIdx.x == 0) *total = carry;
}

// ids in curve order: centres and positions of the kept cells, and the id of
// every position (-1: not a cell)
__global__ void __launch_bounds__(kThreads) k_grid_emit(DevGrid G, const uint8_t* flag, const int64_t* tile_off, int64_t n,
                                                        int32_t* id_of, double* centers, int32_t* ipos) {
  const uint4 v = reinterpret_cast<const uint4*>(flag + blockIdx.x * kTile)[threadIdx.x];
  const int   s = count16(v);
  // exclusive prefix of the per-thread counts within the block
  int incl = s;
  for(int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if((threadIdx.x & 31) >= o) incl += t;
  }
  __shared__ int warp_sum[kThreads / 32];
  if((threadIdx.x & 31) == 31) warp_sum[threadIdx.x >> 5] = incl;
  __syncthreads();
  int before = 0;
  for(int w = 0; w < static_cast<int>(threadIdx.x >> 5); ++w) before += warp_sum[w];
  int64_t       id    = tile_off[blockIdx.x] + before + incl - s;
  const uint8_t* f    = reinterpret_cast<const uint8_t*>(&v);
  const uint64_t first = static_cast<uint64_t>(blockIdx.x) * kTile + static_cast<uint64_t>(threadIdx.x) * kPer;
  for(int j = 0; j < kPer; ++j) {
    const uint64_t i = first + j;
    if(i >= G.ntot) break;
    if(!f[j] || id >= n) {
      id_of[i] = -1;
      continue;
    }
    int64_t p[3];
    position_of(G, i, p);
    for(int d = 0; d < G.D; ++d) {
      centers[id * G.D + d] = G.cv[d][p[d]];
      ipos[id * G.D + d]    = static_cast<int32_t>(p[d]);
    }
    id_of[i] = static_cast<int32_t>(id);
    ++id;
  }
}

// main neighbours and the boundary property of every cell
__global__ void k_grid_links(DevGrid G, const int32_t* id_of, const double* centers, const int32_t* ipos, int64_t n, int64_t* nbr,
                             uint8_t* bndry) {
  const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if(c >= n) return;
  const int     M    = 2 * G.D;
  const int64_t side = int64_t(1) << G.L;
  bool          miss = false;
  for(int dir = 0; dir < M; ++dir) {
    int64_t q[3] = {0, 0, 0};
    for(int d = 0; d < G.D; ++d) q[d] = ipos[c * G.D + d];
    q[dir / 2] += (dir & 1) ? 1 : -1;
    int64_t m = -1;
    if(q[dir / 2] >= 0 && q[dir / 2] < side) m = id_of[index_of(G, q)];
    nbr[c * M + dir] = m;
    miss |= m == -1;
  }
  bndry[c] = (miss && set_cut(G.geom, &centers[c * G.D], G.cell_length, G.D)) ? 1 : 0;
}

struct DevBuffers {
  std::vector<void*> ptrs;
  ~DevBuffers() {
    for(void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    void*       raw = nullptr;
    cudaError_t e   = cudaMalloc(&raw, std::max<size_t>(1, count) * sizeof(T));
    if(e == cudaSuccess) ptrs.push_back(raw);
    *p = static_cast<T*>(raw);
    return e;
  }
};

int build_cells(lbm_grid& g, cudaStream_t s) {
  const int      D    = g.D;
  const uint64_t ntot = uint64_t(1) << (D * g.level);
  const int64_t  side = int64_t(1) << g.level;
  DevBuffers     buf;
  DevGrid        G;
  G.D           = D;
  G.L           = g.level;
  G.cell_length = g.cell_length;
  G.ntot        = ntot;
  lbm_geom_desc* objs = nullptr;
  int32_t*       body = nullptr;
  cudaError_t    e    = buf.alloc(&objs, g.objs.size());
  if(e == cudaSuccess) e = buf.alloc(&body, g.body.size());
  if(e == cudaSuccess && !g.objs.empty())
    e = cudaMemcpyAsync(objs, g.objs.data(), sizeof(lbm_geom_desc) * g.objs.size(), cudaMemcpyHostToDevice, s);
  if(e == cudaSuccess && !g.body.empty())
    e = cudaMemcpyAsync(body, g.body.data(), sizeof(int32_t) * g.body.size(), cudaMemcpyHostToDevice, s);
  G.geom.nobj  = static_cast<int>(g.objs.size());
  G.geom.nbody = g.nbody;
  G.geom.objs  = objs;
  G.geom.body  = body;
  for(int d = 0; d < D && e == cudaSuccess; ++d) {
    double* cv = nullptr;
    e          = buf.alloc(&cv, static_cast<size_t>(side));
    if(e == cudaSuccess) e = cudaMemcpyAsync(cv, g.cv[d].data(), sizeof(double) * side, cudaMemcpyHostToDevice, s);
    G.cv[d] = cv;
  }
  const int64_t ntiles = static_cast<int64_t>((ntot + kTile - 1) / kTile);
  uint8_t*      flag   = nullptr;
  int64_t *     tile   = nullptr, *total = nullptr;
  int32_t*      id_of  = nullptr;
  if(e == cudaSuccess) e = buf.alloc(&flag, static_cast<size_t>(ntiles * kTile));
  if(e == cudaSuccess) e = cudaMemsetAsync(flag, 0, static_cast<size_t>(ntiles * kTile), s);  // padding of the last tile
  if(e == cudaSuccess) e = buf.alloc(&tile, static_cast<size_t>(ntiles));
  if(e == cudaSuccess) e = buf.alloc(&total, 1);
  if(e == cudaSuccess) e = buf.alloc(&id_of, static_cast<size_t>(ntot));
  if(e != cudaSuccess) return e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t want = (ntot + kThreads - 1) / kThreads;
  const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>(want, static_cast<uint64_t>(std::max(sms, 1)) * 32));
  k_grid_member<<<blocks, kThreads, 0, s>>>(G, flag);
  k_grid_tile_count<<<static_cast<unsigned>(ntiles), kThreads, 0, s>>>(flag, tile);
  k_grid_scan_tiles<<<1, 1024, 0, s>>>(tile, ntiles, total);
  int64_t n = 0;
  e         = cudaMemcpyAsync(&n, total, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return LBM_ERR_CUDA;
  if(n <= 0 || n >= (int64_t(1) << 31)) return LBM_ERR_INVALID;
  const int M       = 2 * D;
  double*   centers = nullptr;
  int32_t*  ipos    = nullptr;
  int64_t*  nbr     = nullptr;
  uint8_t*  bndry   = nullptr;
  e                 = buf.alloc(&centers, static_cast<size_t>(n * D));
  if(e == cudaSuccess) e = buf.alloc(&ipos, static_cast<size_t>(n * D));
  if(e == cudaSuccess) e = buf.alloc(&nbr, static_cast<size_t>(n * M));
  if(e == cudaSuccess) e = buf.alloc(&bndry, static_cast<size_t>(n));
  if(e != cudaSuccess) return e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
  k_grid_emit<<<static_cast<unsigned>(ntiles), kThreads, 0, s>>>(G, flag, tile, n, id_of, centers, ipos);
  k_grid_links<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(G, id_of, centers, ipos, n, nbr, bndry);
  g.n = n;
  g.centers.resize(n * D);
  g.ipos.resize(n * D);
  g.nbr.resize(n * M);
  g.bndry.resize(n);
  e = cudaMemcpyAsync(g.centers.data(), centers, sizeof(double) * n * D, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaMemcpyAsync(g.ipos.data(), ipos, sizeof(int32_t) * n * D, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaMemcpyAsync(g.nbr.data(), nbr, sizeof(int64_t) * n * M, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaMemcpyAsync(g.bndry.data(), bndry, n, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}

}  // namespace

extern "C" int lbm_grid_create_device(int32_t ndim, int32_t level, const lbm_geom_desc* objs, int32_t nobj, const double* bbox,
                                      int32_t device, lbm_grid** out) {
  if(!out) return LBM_ERR_INVALID;
  *out        = nullptr;
  lbm_grid* g = new(std::nothrow) lbm_grid();
  if(!g) return LBM_ERR_NOMEM;
  int rc = lbm_grid_impl::setup(*g, ndim, level, objs, nobj, bbox);
  if(rc == LBM_OK && ndim * level > 30) rc = LBM_ERR_UNSUPPORTED;  // 2^30 positions at most
  if(rc != LBM_OK) {
    delete g;
    return rc;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaStream_t s = nullptr;
  if(cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaSetDevice(prev);
    delete g;
    return LBM_ERR_CUDA;
  }
  rc = build_cells(*g, s);
  cudaStreamDestroy(s);
  cudaSetDevice(prev);
  if(rc != LBM_OK) {
    delete g;
    return rc;
  }
  lbm_grid_impl::list_boundary_cells(*g);
  *out = g;
  return LBM_OK;
}
