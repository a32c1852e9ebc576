// Dense-box step with whole x-rows staged in shared memory and moved by bulk
// copies (TMA) in both directions.
//
// The per-thread step kernel (box.cu) issues one 2-byte global load and one
// 2-byte global store per population (FP16 storage), each with its own 64-bit
// address arithmetic: about 410 warp instructions per 32 cells, so it is bound
// by instruction issue and memory latency together.  Here one elected thread
// moves every row of the step with 1D bulk copies and the cell threads touch
// shared memory only, at compile-time offsets from one base per cell.
//
// One pipeline stage holds one x-row (y, z) of the step: per plane p a staged
// row of WR elements, the row's values at positions [0, nx) sitting at index
// H..H+nx-1 (H = one 16-byte vector of halo on either side).
//   even step: plane p, row (y, z).  Cell x reads f_q at [q][x] and writes its
//              post-collision f_q to [opp q][x] -- the AA even step, in place.
//   odd step:  plane p, row (y + c_py, z + c_pz), positions [-H, nx + H).  Cell
//              x pulls f_q = A[opp q][x - c_q], which is staged at
//              [opp q][x - c_qx], and pushes its post-collision f_q to
//              A[q][x + c_q], staged at [q][x + c_qx].  That slot is the one
//              the cell pulled f_{opp q} from: every staged slot is read and
//              then written by the one thread that owns it, so the update is
//              in place here too.
// After the row's cells, every plane's [0, nx) goes back to the same global
// row with one bulk store.  A cell the kernel does not step (a solid, a cell
// whose links the boundary kernel resolves) leaves its staged slots as they
// were loaded, so the store writes back unchanged values there.  The slots a
// row's store covers belong to that row's cells or to no cell at all: position
// 0 of a c_px = +1 plane and position nx-1 of a c_px = -1 plane receive
// nothing through an open face, and with periodic or wall x faces they belong
// to the row's own end cell, which the boundary kernel steps after this
// kernel.  Pushes through the row ends (the inlet's c_x < 0 populations, the
// outlet's c_x > 0 ones) land in the halo, which is never stored.
//
// The odd step covers the interior rows (the face rows hold only cells the
// boundary kernel steps); within them it steps what the per-thread odd step
// steps: fluid cells with no link to resolve, and the inlet / outlet face cells
// (XFACE) in line.  Results are bitwise those of the per-thread kernel: the
// same loads, collision and stores per cell.
//
// Pipeline per CTA: warp 0 lane 0 issues every copy.  It keeps NST rows of
// loads in flight (full barriers); eight cell warps step a loaded row in
// shared memory, fence their writes for the async proxy and mark it done
// (done barriers, one arrival per warp); the copy thread then issues the
// row's bulk stores and, once they have read the stage, loads the next row
// into it.  The cell warps never wait for a store.  Every mbarrier wait is
// bounded; a wait that runs out sets the error flag, and every role then
// leaves within its own bounded waits, the copies it issued having landed.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "box.h"
#include "box_device.cuh"
#include "bulk_copy.cuh"
#include "lattice.cuh"
#include "step_common.cuh"

namespace lbm {
namespace {

constexpr int kRowWarps   = 8;               // consumer warps per CTA
constexpr int kRowThreads = 32 * kRowWarps;  // consumer threads
constexpr int kRowBlock   = kRowThreads + 32;  // + the copy warp

#ifndef LBM_ROWS_STAGES_16
#define LBM_ROWS_STAGES_16 3
#endif
#ifndef LBM_ROWS_CTAS_16
#define LBM_ROWS_CTAS_16 3
#endif

// halo elements on either side of a staged row: one 16-byte vector
template <class T>
constexpr int row_halo() {
  return static_cast<int>(16 / sizeof(T));
}
// pipeline stages per CTA
template <class T>
constexpr int row_stages() {
  return sizeof(T) <= 2 ? LBM_ROWS_STAGES_16 : 2;
}
// staged row width (elements) for rows of up to 256*K cells
template <class T, int K>
constexpr int row_width() {
  return 256 * K + 2 * row_halo<T>();
}
// residual steps (MOM = 2): the previous moments of a cell thread's cells in
// the row (at most K, NV each, in the arithmetic type), fetched into shared
// memory with cp.async when the row starts and read after the collision, so
// that they hold no registers across it
template <class T, int K, int MOM>
constexpr size_t row_prev_bytes() {
  using C = typename std::conditional<sizeof(T) == 8, double, float>::type;
  return MOM == 2 ? sizeof(C) * static_cast<size_t>(K) * 4 * kRowThreads : 0;
}
template <int LAT, class T, int K, int MOM = 0>
constexpr size_t row_smem() {
  return sizeof(T) * row_stages<T>() * Lattice<LAT>::Q * row_width<T, K>() + sizeof(uint64_t) * 2 * row_stages<T>() +
         row_prev_bytes<T, K, MOM>();
}
constexpr size_t kRowSmemMax = 200 * 1024;  // the plain step's stages (box_rows_supported)
constexpr size_t kRowSmemHw  = 227 * 1024;  // per-CTA limit: the residual step's prefetch area comes on top

struct RowList {
  FastDiv  nrows;     // rows per z-slab in the list
  int      y0, z0;    // first row: y in [y0, y0 + nrows), z from z0
  int      count;     // rows in the list
  int*     err;       // set to 1 when a wait times out
  uint64_t limit_ns;  // limit of each pipeline wait
  int      starve;    // test only: the producer never arms the CTA's first row, so the waits on it run out
  int      outlet_inline;  // XFACE outlet cells read their upstream cell's values from the staged row
};

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// one element global -> shared without registers (cp.async, 4 or 8 bytes)
template <class C>
__device__ __forceinline__ void cp_async_elem(C* dst, const C* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"(static_cast<int>(sizeof(C))) : "memory");
}

// One cell of a staged row.  bx: the cell's element in plane 0 of the stage
// (index H + x).  MOM: 0 plain step, 1 also write the cell's moments, 2 also
// add |moments - previous moments| to dacc (the cell's residual share); the
// previous moments are at prev_s[v * kRowThreads], fetched with cp.async.
template <int LAT, int EQ, int ST, bool ODD, int WR, int MOM, int NV>
__device__ __forceinline__ void row_cell(const BoxParams& P, typename Store<ST>::T* bx, int x, int y, int z, bool outlet_inline,
                                         typename Store<ST>::C* dacc, const typename Store<ST>::C* prev_s) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  const int     cell = x + P.nx * (y + P.ny * z);
  const uint8_t flag = P.flags[cell];
  const uint8_t type = flag & TYPE_MASK;
  bool          work, special;
  if constexpr(ODD) {
    const bool xf = (flag & XFACE) != 0;
    work          = flag == LBM_CELL_FLUID || xf;  // fluid and not LINKED, or an inlet / outlet face cell
    special       = xf;
  } else {
    work    = type != LBM_CELL_SOLID;
    special = type != LBM_CELL_FLUID;
  }
  if(!work) return;
  C mom[NV];
#pragma unroll
  for(int k = 0; k < NV; ++k) mom[k] = 0;
  // one vote per warp: warps of plain fluid cells take the path without the
  // inlet / outlet / Dirichlet branches
  const unsigned active      = __activemask();
  const bool     any_special = __any_sync(active, special);
  C          f[Q];
  if(!any_special) {
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      if constexpr(ODD) f[q] = S::load(bx[L::opp(q) * WR - L::c(q, 0)]);
      else f[q] = S::load(bx[q * WR]);
    });
    collide<LAT, EQ, C>(P, z, f, MOM ? mom : nullptr);
  } else {
    const bool emit = ODD ? (special && type == LBM_CELL_INLET) : (type == LBM_CELL_INLET || type == LBM_CELL_DIRICHLET);
    if(emit) {
      emit_equilibrium<LAT, EQ, C>(P, f, cell);
    } else {
      static_for<Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        if constexpr(ODD) f[q] = S::load(bx[L::opp(q) * WR - L::c(q, 0)]);
        else f[q] = S::load(bx[q * WR]);
      });
      if(type == LBM_CELL_OUTLET) {
        if(outlet_inline && (flag & XFACE)) {
          // links from beyond +x: what the upstream cell x - 1 receives, read
          // from the staged row before that cell (the neighbouring lane)
          // overwrites the slot (the warp syncs before its stores)
          static_for<Q>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            if constexpr(L::c(q, 0) < 0) {
              if constexpr(ODD) f[q] = S::load(bx[L::opp(q) * WR - 1 - L::c(q, 0)]);
              else f[q] = S::load(bx[q * WR - 1]);
            }
          });
        } else {
          // links from beyond +x: what the upstream cell received (ghost plane)
          const T*  A  = static_cast<const T*>(P.pop);
          const int NA = static_cast<int>(P.nalloc);
          static_for<Q>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            if constexpr(L::c(q, 0) < 0) f[q] = S::load(A[Q * NA + static_cast<int>(ghost_index(P, q, y, z))]);
          });
        }
      }
      collide<LAT, EQ, C>(P, z, f, MOM ? mom : nullptr);
    }
    __syncwarp(active);  // every lane's staged reads come before any lane's stores
  }
  if constexpr(MOM != 0) {
    C prev[NV], diff[NV];
    if constexpr(MOM == 2) {
      cp_async_wait_all();
#pragma unroll
      for(int k = 0; k < NV; ++k) prev[k] = prev_s[k * kRowThreads];
    }
    moments_io<LAT, EQ, C, MOM, NV>(P, cell, mom, prev, diff);
    if constexpr(MOM == 2) {
#pragma unroll
      for(int k = 0; k < NV; ++k) dacc[k] += diff[k];
    }
  }
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    if constexpr(ODD) bx[q * WR + L::c(q, 0)] = S::store(f[q]);
    else bx[L::opp(q) * WR] = S::store(f[q]);
  });
}

// resident CTAs per SM the register budget aims at (what the stages of shared
// memory allow)
template <int ST>
constexpr int row_min_ctas() {
  return ST == LBM_STORE_F64 ? 1 : (ST == LBM_STORE_F32 ? 2 : LBM_ROWS_CTAS_16);
}

template <int LAT, int EQ, int ST, bool ODD, int K, int MOM>
__global__ void __launch_bounds__(kRowBlock, row_min_ctas<ST>()) k_box_rows(BoxParams P, RowList R) {
  using L             = Lattice<LAT>;
  using S             = Store<ST>;
  using T             = typename S::T;
  using C             = typename S::C;
  constexpr int Q     = L::Q;
  constexpr int NV    = EQ == LBM_NAVIER_STOKES ? L::D + 1 : 1;
  constexpr int H     = row_halo<T>();
  constexpr int NST   = row_stages<T>();
  constexpr int WR    = row_width<T, K>();
  constexpr int STAGE = Q * WR;  // staged elements per row
  extern __shared__ __align__(128) unsigned char smem[];
  T*        buf  = reinterpret_cast<T*>(smem);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + sizeof(T) * NST * STAGE);  // the row's loads landed
  uint64_t* done = full + NST;                                                   // the cell warps wrote the row
  C*        prevbuf = reinterpret_cast<C*>(done + NST);                          // MOM = 2: previous moments (4 per cell)

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G    = static_cast<int>(gridDim.x);
  // each CTA takes one contiguous run of rows
  const int per   = (R.count + G - 1) / G;
  const int first = static_cast<int>(blockIdx.x) * per;
  const int nloc  = first < R.count ? min(per, R.count - first) : 0;
  if(threadIdx.x == 0) {
#pragma unroll
    for(int s = 0; s < NST; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&done[s]), kRowWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  T* const  A  = static_cast<T*>(P.pop);
  const int NA = static_cast<int>(P.nalloc);
  const int nx = P.nx, ny = P.ny;
  auto      coords = [&](int i, int& y, int& z) {
    const uint32_t r  = static_cast<uint32_t>(first + i);
    const uint32_t zz = fdiv(r, R.nrows);
    y                 = R.y0 + static_cast<int>(r - zz * R.nrows.d);
    z                 = R.z0 + static_cast<int>(zz);
  };

  if(warp == 0) {
    // ---- copies: warp 0, lane 0 issues every load and every store ----
    if(lane == 0) {
      const uint32_t lbytes = static_cast<uint32_t>((ODD ? nx + 2 * H : nx) * sizeof(T));
      const uint32_t sbytes = static_cast<uint32_t>(nx * sizeof(T));
      auto           load   = [&](int i) {
        const int st = i % NST;
        int       y, z;
        coords(i, y, z);
        const uint32_t b = smem_u32(&full[st]);
        mbar_expect_tx(b, lbytes * Q);
        T* const dst0 = buf + st * STAGE + (ODD ? 0 : H);
        static_for<Q>([&](auto qc) {
          constexpr int p  = decltype(qc)::value;
          const int     ys = ODD ? y + L::c(p, 1) : y;
          const int     zs = ODD ? z + L::c(p, 2) : z;
          const T*      src = A + p * NA + nx * (ys + ny * zs) - (ODD ? H : 0);
          bulk_g2s(smem_u32(dst0 + p * WR), src, lbytes, b);
        });
      };
      // rows [0, issued) are armed (all but a starved one)
      int issued = 0;
      for(; issued < nloc && issued < NST; ++issued)
        if(!(R.starve && issued == 0)) load(issued);  // test only: nothing arms full[0], its waits run out
      for(int i = 0; i < nloc; ++i) {
        const int st = i % NST;
        if(!mbar_wait_bounded(smem_u32(&done[st]), static_cast<uint32_t>((i / NST) & 1), R.limit_ns)) {
          atomicExch(R.err, 1);
          break;
        }
        int y, z;
        coords(i, y, z);
        const T* const stage = buf + st * STAGE + H;
        static_for<Q>([&](auto qc) {
          constexpr int p  = decltype(qc)::value;
          const int     ys = ODD ? y + L::c(p, 1) : y;
          const int     zs = ODD ? z + L::c(p, 2) : z;
          bulk_s2g(A + p * NA + nx * (ys + ny * zs), smem_u32(stage + p * WR), sbytes);
        });
        bulk_commit();
        // the stage is free once its stores have read it; the cell warps are
        // meanwhile on the rows already loaded
        bulk_wait_read<0>();
        if(issued < nloc) load(issued++);
      }
      bulk_wait_all();  // every store issued has completed
      // and every load issued has landed before the CTA can exit (rows the
      // cell warps did not take after a wait ran out)
      for(int j = issued > NST ? issued - NST : 0; j < issued; ++j)
        if(!(R.starve && j == 0))
          mbar_wait_bounded(smem_u32(&full[j % NST]), static_cast<uint32_t>((j / NST) & 1), kDrainLimitNs);
    }
    return;
  }

  // ---- cells: warps 1 .. kRowWarps ----
  const int tid = threadIdx.x - 32;
  for(int i = 0; i < nloc; ++i) {
    const int st = i % NST;
    int       y, z;
    coords(i, y, z);
    // the wait result is made warp-uniform so the warp leaves together; a
    // warp that leaves never marks its rows done, so the copy thread's wait
    // runs out too and nothing more is loaded or stored
    if(!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&full[st]), static_cast<uint32_t>((i / NST) & 1), R.limit_ns))) {
      if(lane == 0) atomicExch(R.err, 1);
      return;
    }
    T* const stage = buf + st * STAGE + H;
    C        dacc[NV];
#pragma unroll
    for(int k = 0; k < NV; ++k) dacc[k] = C(0);
    if constexpr(MOM == 2) {
      // the previous moments of this thread's cells in the row, in flight
      // while the cells collide
      const C*      M   = static_cast<const C*>(P.mom);
      const int64_t row = static_cast<int64_t>(nx) * (y + static_cast<int64_t>(ny) * z);
      int           j   = 0;
#pragma unroll 1
      for(int x = tid; x < nx; x += kRowThreads, ++j)
#pragma unroll
        for(int v = 0; v < NV; ++v) cp_async_elem(prevbuf + (j * 4 + v) * kRowThreads + tid, M + v * P.ncells + row + x);
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
    {
      int j = 0;
#pragma unroll 1
      for(int x = tid; x < nx; x += kRowThreads, ++j)
        row_cell<LAT, EQ, ST, ODD, WR, MOM, NV>(P, stage + x, x, y, z, R.outlet_inline != 0, dacc, prevbuf + j * 4 * kRowThreads + tid);
    }
    if constexpr(MOM == 2) cp_async_wait_all();  // none left in flight (cells that did no work never waited)
    fence_async_smem();  // this thread's writes are visible to the bulk stores
    __syncwarp();
    if(lane == 0) mbar_arrive(smem_u32(&done[st]));
    // residual share of the row: one slot per (row, cell warp)
    if constexpr(MOM == 2)
      warp_partials<NV>(dacc, P.partials, P.partial_stride, static_cast<int64_t>(first + i) * kRowWarps + (warp - 1));
  }
}

template <int LAT, int EQ, int ST, bool ODD, int K, int MOM>
cudaError_t launch_rows_one(BoxState* b, const RowList& R, cudaStream_t s) {
  using T           = typename Store<ST>::T;
  constexpr size_t smem = row_smem<LAT, T, K, MOM>();
  if constexpr(smem > (MOM == 2 ? kRowSmemHw : kRowSmemMax)) {
    return cudaErrorInvalidValue;
  } else {
    auto kern = k_box_rows<LAT, EQ, ST, ODD, K, MOM>;
    // resident CTAs on the whole GPU, worked out once per instantiation
    static int resident = 0;
    if(resident == 0) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
      if(e != cudaSuccess) return e;
      int per_sm = 0;
      e          = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRowBlock, smem);
      if(e != cudaSuccess) return e;
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      resident = std::max(per_sm, 1) * sms;
    }
    const int64_t grid = std::min<int64_t>(R.count, resident);
    if(grid <= 0) return cudaSuccess;
    kern<<<static_cast<unsigned>(grid), kRowBlock, smem, s>>>(b->p, R);
    return cudaGetLastError();
  }
}

// smallest staged width that holds the row (0: none)
int row_k(int nx) {
  for(int k : {2, 4})
    if(nx <= 256 * k) return k;
  return 0;
}

template <int LAT, int EQ, int ST, int K>
cudaError_t launch_rows_k(BoxState* b, bool odd, int mom, const RowList& R, cudaStream_t s) {
  if(odd) {
    if(mom == 0) return launch_rows_one<LAT, EQ, ST, true, K, 0>(b, R, s);
    if(mom == 1) return launch_rows_one<LAT, EQ, ST, true, K, 1>(b, R, s);
    return launch_rows_one<LAT, EQ, ST, true, K, 2>(b, R, s);
  }
  if(mom == 0) return launch_rows_one<LAT, EQ, ST, false, K, 0>(b, R, s);
  if(mom == 1) return launch_rows_one<LAT, EQ, ST, false, K, 1>(b, R, s);
  return launch_rows_one<LAT, EQ, ST, false, K, 2>(b, R, s);
}

// *nbulk: the residual slots the launch writes (one per row and cell warp)
template <int LAT, int EQ, int ST>
cudaError_t launch_rows(BoxState* b, bool odd, int mom, cudaStream_t s, int64_t* nbulk) {
  using L = Lattice<LAT>;
  using T = typename Store<ST>::T;
  RowList R{};
  int     nrows, nz;
  if(odd) {
    R.y0  = L::D > 1 ? 1 : 0;
    nrows = L::D > 1 ? b->p.ny - 2 : b->p.ny;
    R.z0  = L::D > 2 ? 1 : 0;
    nz    = L::D > 2 ? b->p.nz - 2 : b->p.nz;
  } else {
    R.y0  = 0;
    nrows = b->p.ny;
    R.z0  = 0;
    nz    = b->p.nz;
  }
  R.count    = (nrows > 0 && nz > 0) ? nrows * nz : 0;
  R.nrows    = make_fastdiv(static_cast<uint32_t>(std::max(nrows, 1)));
  R.err      = b->d_err;
  R.limit_ns = b->wait_limit_ns;
  R.starve   = b->wait_starve;
  R.outlet_inline = box_rows_outlet_inline(b) ? 1 : 0;
  if(nbulk) *nbulk = static_cast<int64_t>(R.count) * kRowWarps;
  if(R.count == 0) return cudaSuccess;
  const int k = row_k(b->p.nx);
  if(k == 2) return launch_rows_k<LAT, EQ, ST, 2>(b, odd, mom, R, s);
  if(k == 4) return launch_rows_k<LAT, EQ, ST, 4>(b, odd, mom, R, s);
  return cudaErrorInvalidValue;
}

template <int LAT, class T>
size_t rows_smem_for(int nx) {
  const int k = row_k(nx);
  if(k == 2) return row_smem<LAT, T, 2>();
  if(k == 4) return row_smem<LAT, T, 4>();
  return 0;
}

}  // namespace

bool box_rows_outlet_inline(const BoxState* b) {
  // the outlet cell x = nx - 1 and its upstream cell x - 1 are stepped by two
  // lanes of one warp in the same pass over the row (cells x and x +
  // kRowThreads k per thread, 32 consecutive cells per warp)
  const int x = b->p.nx - 1;
  return b->p.has_outlet && x % 32 != 0;
}

bool box_rows_supported(const BoxState* b) {
  // every staged row starts on a 16-byte boundary (planes are padded to 128
  // cells, so rows are aligned when nx * sizeof(storage) is), the halo keeps
  // the odd step's loads 16-byte aligned too, and the stages fit shared memory
  if(!b->d_err) return false;
  if((static_cast<size_t>(b->p.nx) * b->elem) % 16 != 0) return false;
  if((static_cast<size_t>(b->p.nalloc) * b->elem) % 16 != 0) return false;
  size_t smem = 0;
  const int nx = b->p.nx;
  switch(b->desc.lattice) {
    case LBM_D2Q9:
      smem = b->elem == 8 ? rows_smem_for<LBM_D2Q9, double>(nx) : b->elem == 4 ? rows_smem_for<LBM_D2Q9, float>(nx) : rows_smem_for<LBM_D2Q9, uint16_t>(nx);
      break;
    case LBM_D3Q19:
      smem = b->elem == 8 ? rows_smem_for<LBM_D3Q19, double>(nx) : b->elem == 4 ? rows_smem_for<LBM_D3Q19, float>(nx) : rows_smem_for<LBM_D3Q19, uint16_t>(nx);
      break;
    case LBM_D3Q7:
      smem = b->elem == 8 ? rows_smem_for<LBM_D3Q7, double>(nx) : rows_smem_for<LBM_D3Q7, float>(nx);
      break;
    default: return false;
  }
  return smem > 0 && smem <= kRowSmemMax;
}

cudaError_t box_rows_bulk(BoxState* b, bool odd, int mom, cudaStream_t s, int64_t* nbulk) {
  const int key = b->desc.lattice * 100 + b->desc.equation * 10 + b->desc.storage;
  switch(key) {
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_F64: return launch_rows<LBM_D2Q9, 0, LBM_STORE_F64>(b, odd, mom, s, nbulk);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_F32: return launch_rows<LBM_D2Q9, 0, LBM_STORE_F32>(b, odd, mom, s, nbulk);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_F16_DEV: return launch_rows<LBM_D2Q9, 0, LBM_STORE_F16_DEV>(b, odd, mom, s, nbulk);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_BF16_DEV: return launch_rows<LBM_D2Q9, 0, LBM_STORE_BF16_DEV>(b, odd, mom, s, nbulk);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_E3M12_DEV: return launch_rows<LBM_D2Q9, 0, LBM_STORE_E3M12_DEV>(b, odd, mom, s, nbulk);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_F64: return launch_rows<LBM_D3Q19, 0, LBM_STORE_F64>(b, odd, mom, s, nbulk);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_F32: return launch_rows<LBM_D3Q19, 0, LBM_STORE_F32>(b, odd, mom, s, nbulk);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_F16_DEV: return launch_rows<LBM_D3Q19, 0, LBM_STORE_F16_DEV>(b, odd, mom, s, nbulk);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_BF16_DEV: return launch_rows<LBM_D3Q19, 0, LBM_STORE_BF16_DEV>(b, odd, mom, s, nbulk);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_E3M12_DEV: return launch_rows<LBM_D3Q19, 0, LBM_STORE_E3M12_DEV>(b, odd, mom, s, nbulk);
    case LBM_D3Q7 * 100 + 10 + LBM_STORE_F64: return launch_rows<LBM_D3Q7, 1, LBM_STORE_F64>(b, odd, mom, s, nbulk);
    case LBM_D3Q7 * 100 + 10 + LBM_STORE_F32: return launch_rows<LBM_D3Q7, 1, LBM_STORE_F32>(b, odd, mom, s, nbulk);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lbm
