// Dense-box step with bulk-copy (TMA) staging of the populations.
//
// The per-thread step kernel (box.cu) loads each population with its own
// global load; in FP16 storage that is 2 bytes per load and per register, so
// the bytes a warp can keep in flight are bounded by its registers and the
// kernel stalls on memory latency well below HBM bandwidth.  Here a CTA walks
// a list of row segments (SEG consecutive cells of one x-row) and, one
// segment per pipeline stage, has one thread issue a 1D bulk copy
// (cp.async.bulk, completion on an mbarrier) for every direction's row:
//   even step: row (y, z) of plane q, x in [x0, x0 + SEG);
//   odd step:  row (y - c_qy, z - c_qz) of plane opp(q), x in
//              [x0 - H, x0 + SEG + H), H = 16 bytes of halo on either side
//              so that the copy starts on a 16-byte boundary.
// NST segments are in flight per CTA while the threads collide the current
// one from shared memory and store the results straight to global memory
// (even: A[opp q][x]; odd: A[q][x + c_q]), exactly the AA update of the
// per-thread kernel.  Halo elements that belong to other segments may be
// stale by the time they are copied; only the cell's own slots are used, and
// each slot is read and written by the one thread that owns it.
//
// The odd step covers the cells of the per-thread bulk kernel (interior fluid
// cells with no solid neighbour, on rows 1..n-2); the boundary-list kernel of
// box.cu handles the rest afterwards.  Every mbarrier wait is bounded: after
// the wait limit (0.5 s unless a test lowers it) the CTA records an error
// flag, waits (bounded again, kDrainLimitNs) for its own copies still in
// flight and returns; the host reports the flag as LBM_ERR_TIMEOUT.
#include <cuda_runtime.h>

#include <algorithm>

#include "box.h"
#include "box_device.cuh"
#include "bulk_copy.cuh"
#include "lattice.cuh"
#include "step_common.cuh"

namespace lbm {
namespace {

constexpr int      kSeg        = 256;          // cells per segment = threads per CTA

template <class T>
constexpr int stages() {
  return sizeof(T) >= 8 ? 2 : 4;
}

struct SegList {
  FastDiv spr;      // segments per row, ceil(nx / kSeg)
  FastDiv nrows;    // rows per z-slab in the list
  int     y0, z0;   // first row: y in [y0, y0 + nrows), z from z0
  int     nseg;     // segments in the list
  int*    err;      // set to 1 when a wait times out
  uint64_t limit_ns;  // limit of each pipeline wait
  int     starve;   // test only: the producer never arms the CTA's first segment, so the waits on it run out
};

constexpr int kConsumers = kSeg / 32;  // consumer warps; warp 0 issues the copies

// Warp 0 is the producer: its lane 0 keeps NST segments of copies in flight,
// re-using a stage once every consumer warp has released it (empty barrier).
// Warps 1..kConsumers each own 32 cells of the segment: wait for the stage
// (full barrier), read their populations, release the stage, collide, store.
// No block-wide barrier after the set-up.
// resident CTAs per SM the register budget aims at: three for the plain
// FP32-arithmetic step, two where the moment bookkeeping or FP64 needs room
template <int ST, int MOM>
constexpr int min_ctas() {
  return (ST == LBM_STORE_F64 || MOM != 0) ? 2 : 3;
}

template <int LAT, int EQ, int ST, bool ODD, int MOM>
__global__ void __launch_bounds__(kSeg + 32, min_ctas<ST, MOM>()) k_box_tma(BoxParams P, SegList W) {
  using L               = Lattice<LAT>;
  using S               = Store<ST>;
  using T               = typename S::T;
  using C               = typename S::C;
  constexpr int Q       = L::Q;
  constexpr int NV      = EQ == LBM_NAVIER_STOKES ? L::D + 1 : 1;
  constexpr int NST     = stages<T>();
  constexpr int HALO    = ODD ? static_cast<int>(16 / sizeof(T)) : 0;
  constexpr int ROW     = kSeg + 2 * HALO;  // staged elements per direction
  constexpr int STAGE   = Q * ROW;          // staged elements per segment
  extern __shared__ __align__(128) unsigned char smem[];
  T*        buf   = reinterpret_cast<T*>(smem);
  uint64_t* full  = reinterpret_cast<uint64_t*>(smem + sizeof(T) * NST * STAGE);
  uint64_t* empty = full + NST;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G    = static_cast<int>(gridDim.x);
  // each CTA takes one contiguous run of segments
  const int per   = (W.nseg + G - 1) / G;
  const int first = static_cast<int>(blockIdx.x) * per;
  const int nloc  = first < W.nseg ? min(per, W.nseg - first) : 0;
  if(threadIdx.x == 0) {
#pragma unroll
    for(int s = 0; s < NST; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), kConsumers);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  T* const  A  = static_cast<T*>(P.pop);
  const int NA = static_cast<int>(P.nalloc);
  const int nx = P.nx, ny = P.ny;

  auto coords = [&](int i, int& x0, int& y, int& z) {
    const uint32_t s  = static_cast<uint32_t>(first + i);
    const uint32_t r  = fdiv(s, W.spr);
    const uint32_t zz = fdiv(r, W.nrows);
    x0                = static_cast<int>(s - r * W.spr.d) * kSeg;
    y                 = W.y0 + static_cast<int>(r - zz * W.nrows.d);
    z                 = W.z0 + static_cast<int>(zz);
  };

  if(warp == 0) {
    // ---- producer ----
    if(lane == 0) {
      int issued = 0;  // segments [0, issued) are armed (all but a starved one)
      for(int i = 0; i < nloc; ++i) {
        const int st = i % NST;
        if(i >= NST && !mbar_wait_bounded(smem_u32(&empty[st]), static_cast<uint32_t>((i / NST - 1) & 1), W.limit_ns)) {
          atomicExch(W.err, 1);
          break;
        }
        issued = i + 1;
        if(W.starve && i == 0) continue;  // test only: nothing arms full[0], its waits run out
        int x0, y, z;
        coords(i, x0, y, z);
        const int      lo    = ODD ? max(x0 - HALO, 0) : x0;
        const int      hi    = min(x0 + kSeg + HALO, nx);
        const uint32_t bytes = static_cast<uint32_t>(hi - lo) * sizeof(T);
        const uint32_t b     = smem_u32(&full[st]);
        mbar_expect_tx(b, bytes * Q);
        T* const dst0 = buf + st * STAGE + (lo - (x0 - HALO));
        static_for<Q>([&](auto qc) {
          constexpr int q     = decltype(qc)::value;
          constexpr int plane = ODD ? L::opp(q) : q;
          const int     ys    = ODD ? y - L::c(q, 1) : y;
          const int     zs    = ODD ? z - L::c(q, 2) : z;
          const T*      src   = A + plane * NA + lo + nx * (ys + ny * zs);
          bulk_g2s(smem_u32(dst0 + q * ROW), src, bytes, b);
        });
      }
      // every copy this CTA issued has landed before its threads can all
      // exit, also when consumer warps left early after a wait ran out (the
      // last NST armed segments; earlier ones were consumed before their
      // stage was re-armed).  Completed phases return at once.
      for(int j = issued > NST ? issued - NST : 0; j < issued; ++j)
        if(!(W.starve && j == 0))
          mbar_wait_bounded(smem_u32(&full[j % NST]), static_cast<uint32_t>((j / NST) & 1), kDrainLimitNs);
    }
    return;
  }

  // ---- consumers ----
  const int tid = threadIdx.x - 32;  // cell within the segment
  for(int i = 0; i < nloc; ++i) {
    int x0, y, z;
    coords(i, x0, y, z);
    const int     st    = i % NST;
    const int     x     = x0 + tid;
    const bool    valid = x < nx;
    const int     cell  = valid ? x + nx * (y + ny * z) : 0;
    const uint8_t flag  = valid ? P.flags[cell] : LBM_CELL_SOLID;
    const uint8_t type  = flag & TYPE_MASK;
    bool          work;
    if constexpr(ODD) work = flag == LBM_CELL_FLUID;  // fluid, and not LINKED
    else work = type != LBM_CELL_SOLID;
    const bool emit = !ODD && (type == LBM_CELL_INLET || type == LBM_CELL_DIRICHLET);
    C          mom[NV], prev[NV], diff[NV];
#pragma unroll
    for(int k = 0; k < NV; ++k) {
      mom[k]  = C(0);
      diff[k] = C(0);
    }
    if(work) prefetch_moments<C, MOM, NV>(P, cell, prev);

    // the wait result is made warp-uniform so the warp leaves together
    const bool ok =
        __all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&full[st]), static_cast<uint32_t>((i / NST) & 1), W.limit_ns));
    if(!ok) {
      if(lane == 0) atomicExch(W.err, 1);
      return;
    }
    C        f[Q];
    const T* row = buf + st * STAGE + HALO + tid;
    if(work && !emit)
      static_for<Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        f[q]            = S::load(row[q * ROW - (ODD ? L::c(q, 0) : 0)]);
      });
    __syncwarp();
    if(lane == 0) mbar_arrive(smem_u32(&empty[st]));  // this warp is done with the stage

    if(work) {
      if(emit) {
        emit_equilibrium<LAT, EQ, C>(P, f, cell);
      } else {
        if constexpr(!ODD) {
          if(type == LBM_CELL_OUTLET) {
            static_for<Q>([&](auto qc) {
              constexpr int q = decltype(qc)::value;
              if constexpr(L::c(q, 0) < 0) f[q] = S::load(A[Q * NA + static_cast<int>(ghost_index(P, q, y, z))]);
            });
          }
        }
        collide<LAT, EQ, C>(P, z, f, MOM ? mom : nullptr);
      }
      moments_io<LAT, EQ, C, MOM, NV>(P, cell, mom, prev, diff);
      if constexpr(!ODD) {
        static_for<Q>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          A[L::opp(q) * NA + cell] = S::store(f[q]);
        });
      } else {
        const int sy = nx, sz = nx * ny;
        static_for<Q>([&](auto qc) {
          constexpr int q   = decltype(qc)::value;
          const int     off = L::c(q, 0) + sy * L::c(q, 1) + sz * L::c(q, 2);
          A[q * NA + cell + off] = S::store(f[q]);
        });
      }
    }
    if constexpr(MOM == 2) {
      const int64_t s = static_cast<int64_t>(first) + i;
      warp_partials<NV>(diff, P.partials, P.partial_stride, s * kConsumers + (warp - 1));
    }
  }
}

template <int LAT, int EQ, int ST, bool ODD, int MOM>
cudaError_t launch_one(BoxState* b, const SegList& W, cudaStream_t s) {
  using T          = typename Store<ST>::T;
  constexpr int NST = stages<T>();
  constexpr int HALO = ODD ? static_cast<int>(16 / sizeof(T)) : 0;
  const size_t smem = sizeof(T) * NST * Lattice<LAT>::Q * (kSeg + 2 * HALO) + sizeof(uint64_t) * 2 * NST;
  auto         kern = k_box_tma<LAT, EQ, ST, ODD, MOM>;
  // resident CTAs on the whole GPU, worked out once per instantiation
  static int resident = 0;
  if(resident == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if(e != cudaSuccess) return e;
    int per_sm = 0;
    e          = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSeg + 32, smem);
    if(e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    resident = std::max(per_sm, 1) * sms;
  }
  const int64_t grid = std::min<int64_t>(W.nseg, resident);
  if(grid <= 0) return cudaSuccess;
  kern<<<static_cast<unsigned>(grid), kSeg + 32, smem, s>>>(b->p, W);
  return cudaGetLastError();
}

template <int LAT, int EQ, int ST>
cudaError_t launch_tma(BoxState* b, bool odd, int mom, cudaStream_t s, int64_t* slots) {
  using L = Lattice<LAT>;
  SegList   W{};
  const int spr = (b->p.nx + kSeg - 1) / kSeg;
  int       nrows, nz;
  if(odd) {
    W.y0  = L::D > 1 ? 1 : 0;
    nrows = L::D > 1 ? b->p.ny - 2 : b->p.ny;
    W.z0  = L::D > 2 ? 1 : 0;
    nz    = L::D > 2 ? b->p.nz - 2 : b->p.nz;
  } else {
    W.y0  = 0;
    nrows = b->p.ny;
    W.z0  = 0;
    nz    = b->p.nz;
  }
  W.nseg  = (nrows > 0 && nz > 0) ? spr * nrows * nz : 0;
  W.spr   = make_fastdiv(static_cast<uint32_t>(spr));
  W.nrows = make_fastdiv(static_cast<uint32_t>(std::max(nrows, 1)));
  W.err      = b->d_err;
  W.limit_ns = b->wait_limit_ns;
  W.starve   = b->wait_starve;
  *slots = static_cast<int64_t>(W.nseg) * kConsumers;
  if(W.nseg == 0) return cudaSuccess;
  if(odd) {
    if(mom == 0) return launch_one<LAT, EQ, ST, true, 0>(b, W, s);
    if(mom == 1) return launch_one<LAT, EQ, ST, true, 1>(b, W, s);
    return launch_one<LAT, EQ, ST, true, 2>(b, W, s);
  }
  if(mom == 0) return launch_one<LAT, EQ, ST, false, 0>(b, W, s);
  if(mom == 1) return launch_one<LAT, EQ, ST, false, 1>(b, W, s);
  return launch_one<LAT, EQ, ST, false, 2>(b, W, s);
}

}  // namespace

bool box_tma_supported(const BoxState* b) {
  // every staged row must start on a 16-byte boundary: planes are padded to
  // 128 cells, so rows are aligned when nx * sizeof(storage) is
  if(!b->d_err) return false;
  if((static_cast<size_t>(b->p.nx) * b->elem) % 16 != 0) return false;
  if((static_cast<size_t>(b->p.nalloc) * b->elem) % 16 != 0) return false;
  return true;
}

cudaError_t box_tma_bulk(BoxState* b, bool odd, int mom, cudaStream_t s, int64_t* slots) {
  const int key = b->desc.lattice * 100 + b->desc.equation * 10 + b->desc.storage;
  switch(key) {
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_F64: return launch_tma<LBM_D2Q9, 0, LBM_STORE_F64>(b, odd, mom, s, slots);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_F32: return launch_tma<LBM_D2Q9, 0, LBM_STORE_F32>(b, odd, mom, s, slots);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_F16_DEV: return launch_tma<LBM_D2Q9, 0, LBM_STORE_F16_DEV>(b, odd, mom, s, slots);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_BF16_DEV: return launch_tma<LBM_D2Q9, 0, LBM_STORE_BF16_DEV>(b, odd, mom, s, slots);
    case LBM_D2Q9 * 100 + 0 + LBM_STORE_E3M12_DEV: return launch_tma<LBM_D2Q9, 0, LBM_STORE_E3M12_DEV>(b, odd, mom, s, slots);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_F64: return launch_tma<LBM_D3Q19, 0, LBM_STORE_F64>(b, odd, mom, s, slots);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_F32: return launch_tma<LBM_D3Q19, 0, LBM_STORE_F32>(b, odd, mom, s, slots);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_F16_DEV: return launch_tma<LBM_D3Q19, 0, LBM_STORE_F16_DEV>(b, odd, mom, s, slots);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_BF16_DEV: return launch_tma<LBM_D3Q19, 0, LBM_STORE_BF16_DEV>(b, odd, mom, s, slots);
    case LBM_D3Q19 * 100 + 0 + LBM_STORE_E3M12_DEV: return launch_tma<LBM_D3Q19, 0, LBM_STORE_E3M12_DEV>(b, odd, mom, s, slots);
    case LBM_D3Q7 * 100 + 10 + LBM_STORE_F64: return launch_tma<LBM_D3Q7, 1, LBM_STORE_F64>(b, odd, mom, s, slots);
    case LBM_D3Q7 * 100 + 10 + LBM_STORE_F32: return launch_tma<LBM_D3Q7, 1, LBM_STORE_F32>(b, odd, mom, s, slots);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lbm
