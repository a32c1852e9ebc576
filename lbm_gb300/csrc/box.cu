// Dense-box engine: BGK / Poisson-Boltzmann step on a structured box, AA-pattern
// in-place streaming, FP64 / FP32 / FP16 / BF16 population storage.
//
// Physics per cell is the reference's BGK update (src/lbm/solver.cpp:512-622:
// moments, equilibrium eq::defaultEq, f = (1-omega) f + omega feq) with, where
// requested, Guo body forcing, and for D3Q7 the Chai-Shi Poisson collision of
// src/lbm/solver.cpp:589-611 with a sinh source.
//
// Streaming (the reference's push propagationStep, solver.cpp:714-740, plus its
// halfway bounce-back at wet-node boundary rows, bnd_dirichlet.h:79-121) uses
// the AA pattern: one population array, updated in place.
//   even step: cell x reads its own slots A[q][x], collides, writes the
//              post-collision value of direction q to A[opp(q)][x];
//   odd step:  cell x pulls f_q from A[opp(q)][x - c_q], collides, and pushes
//              the result of direction q to A[q][x + c_q].
// Every location is read and then written by the same thread, so the update is
// race-free without a second array.  Walls, solids, free slip, periodic wrap and
// the inlet/outlet planes are resolved per link: the pull side asks "which
// post-collision population arrives here" (src()), the push side asks "where
// does the population leaving here land" (dst()); the two are inverses.
//
// Storage: FP64 stores f; FP32 stores f - w; FP16 / BF16 store (f - w)/w * 2^12
// (the lattice weights make every direction's deviation O(1) before scaling,
// and the power-of-two scale keeps small deviations out of the subnormal
// range).  Arithmetic is FP64 for FP64 storage and FP32 otherwise; Navier-Stokes
// in reduced precision works on deviations from the weights throughout.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <utility>
#include <vector>

#include "box.h"
#include "box_device.cuh"
#include "lattice.cuh"
#include "step_common.cuh"

namespace lbm {
namespace {

// ---- the step kernels ----------------------------------------------------------
// k_box_bulk: 3D grid over the box, one thread per cell.
//   even step: every non-solid cell; reads and writes only its own slots.
//   odd step:  cells whose links all stay inside the box and avoid solids;
//              pull from x - c_q, push to x + c_q with constant offsets.
// k_box_bnd: odd step only, the remaining cells (next to a face or a solid,
//   inlet / outlet / Dirichlet planes) from a compact list; every link is
//   resolved through the faces.  Each population slot is read and then
//   written by the one thread that owns it, so the two kernels may run in
//   either order.
// MOM: 0 plain, 1 also write the moments, 2 also accumulate |moments - previous|
// The part of a bulk cell's step after its loads.  SPECIAL = false leaves the
// inlet / Dirichlet / outlet branches out of the instruction stream (the caller
// knows that no lane of the warp holds such a cell).
// XFP (odd step): some lane of the warp holds an XFACE or SFACE cell (xf, sf
// for this lane).  XFACE: an inlet emits its equilibrium, an outlet pulls its
// c_x < 0 links from the ghost plane, and neither pushes through its open
// face.  SFACE: the links through the free-slip face are reflected in it (the
// population arriving in direction q comes from the face neighbour x - c_q
// projected on the face, in the mirrored direction; a population leaving
// through the face lands mirrored on x + c_q projected on the face), as
// resolve() gives for the boundary kernel's link tables.
template <int LAT, int EQ, int ST, bool ODD, int MOM, bool SPECIAL, bool XFP = false>
__device__ __forceinline__ void bulk_finish(const BoxParams& P, int y, int z, int cell, uint8_t type, typename Store<ST>::C* f,
                                            const typename Store<ST>::C* prev, typename Store<ST>::C* diff, bool xf = false,
                                            int x = 0, bool sf = false) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  constexpr int NV = EQ == LBM_NAVIER_STOKES ? L::D + 1 : 1;
  T*            A    = static_cast<T*>(P.pop);
  T* const      Ac   = A + cell;
  const int     NA   = static_cast<int>(P.nalloc);
  C             mom[NV];
#pragma unroll
  for(int k = 0; k < NV; ++k) mom[k] = 0;
  const bool emit = (!ODD && SPECIAL && (type == LBM_CELL_INLET || type == LBM_CELL_DIRICHLET)) ||
                    (ODD && XFP && xf && type == LBM_CELL_INLET);
  // SFACE: the c_y (c_z) whose pull crosses the cell's free-slip face, 0 if
  // none (formed where it is used, so nothing extra lives across the collision)
  const auto pull_y = [&]() { return (L::D > 1 && sf) ? (y == 0 ? 1 : (y == P.ny - 1 ? -1 : 0)) : 0; };
  const auto pull_z = [&]() { return (L::D > 2 && sf) ? (z == 0 ? 1 : (z == P.nz - 1 ? -1 : 0)) : 0; };
  if(emit) {
    emit_equilibrium<LAT, EQ, C>(P, f, cell);
  } else {
    if constexpr(ODD && XFP) {
      if(xf) {
        // the outlet: links from beyond +x, the ghost plane
        static_for<Q>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          if constexpr(L::c(q, 0) < 0) f[q] = S::load(A[Q * NA + static_cast<int>(ghost_index(P, q, y, z))]);
        });
      }
      if(sf) {
        // links through the free-slip face: the mirrored population of the
        // face neighbour (inside the box: the cell is not on an x face or a
        // second y / z face)
        const int sy = P.nx, sz = P.nx * P.ny;
        const int py = pull_y(), pz = pull_z();
        static_for<Q>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          if constexpr(L::D > 1 && L::c(q, 1) != 0) {
            if(L::c(q, 1) == py)
              f[q] = S::load(Ac[L::opp(mirror_axis<LAT, 1>(q)) * NA - (L::c(q, 0) + sz * L::c(q, 2))]);
          }
          if constexpr(L::D > 2 && L::c(q, 2) != 0) {
            if(L::c(q, 2) == pz)
              f[q] = S::load(Ac[L::opp(mirror_axis<LAT, 2>(q)) * NA - (L::c(q, 0) + sy * L::c(q, 1))]);
          }
        });
      }
    }
    if constexpr(!ODD && SPECIAL) {
      if(type == LBM_CELL_OUTLET) {
        // links from beyond +x: what the upstream cell received (ghost plane)
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
      Ac[L::opp(q) * NA] = S::store(f[q]);
    });
  } else {
    const int  sy = P.nx, sz = P.nx * P.ny;
    const bool drop_neg = XFP && xf && x == 0;          // the inlet: nothing leaves through -x
    const bool drop_pos = XFP && xf && x == P.nx - 1;   // the outlet: nothing leaves through +x
    const int  py = XFP ? pull_y() : 0, pz = XFP ? pull_z() : 0;
    static_for<Q>([&](auto qc) {
      constexpr int q   = decltype(qc)::value;
      const int     off = L::c(q, 0) + sy * L::c(q, 1) + sz * L::c(q, 2);
      if constexpr(XFP && L::c(q, 0) < 0) {
        if(drop_neg) return;
      }
      if constexpr(XFP && L::c(q, 0) > 0) {
        if(drop_pos) return;
      }
      if constexpr(XFP && L::D > 1 && L::c(q, 1) != 0) {
        if(L::c(q, 1) == -py) {  // leaves through the free-slip face: lands mirrored on the face
          Ac[mirror_axis<LAT, 1>(q) * NA + L::c(q, 0) + sz * L::c(q, 2)] = S::store(f[q]);
          return;
        }
      }
      if constexpr(XFP && L::D > 2 && L::c(q, 2) != 0) {
        if(L::c(q, 2) == -pz) {
          Ac[mirror_axis<LAT, 2>(q) * NA + L::c(q, 0) + sy * L::c(q, 1)] = S::store(f[q]);
          return;
        }
      }
      Ac[q * NA + off] = S::store(f[q]);
    });
  }
}

// One cell of the bulk step (the body of k_box_bulk; also the fallback of
// k_box_pair for pairs that mix cell kinds).  Adds |moment change| to diff.
// XF (odd step): 0 plain; 1 the bulk kernel, which also steps the XFACE
// cells; 2 the face blocks of the boundary kernel, which step only the SFACE
// cells (kept out of the 40-register bulk kernel, whose registers the
// reflections would overflow).
template <int LAT, int EQ, int ST, bool ODD, int MOM, int XF = 0>
__device__ __forceinline__ void bulk_cell(const BoxParams& P, int x, int y, int z, int cell, uint8_t flag,
                                          typename Store<ST>::C* diff) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  constexpr int NV = EQ == LBM_NAVIER_STOKES ? L::D + 1 : 1;
  const uint8_t type = flag & TYPE_MASK;
  T* const      Ac   = static_cast<T*>(P.pop) + cell;  // the cell's slot in plane 0
  const int     NA   = static_cast<int>(P.nalloc);
  bool          work;
  const bool    xf = ODD && XF == 1 && (flag & XFACE);
  const bool    sf = ODD && XF == 2 && (flag & SFACE);
  if constexpr(ODD && XF == 2) work = sf;
  else if constexpr(ODD) work = flag == LBM_CELL_FLUID || xf;  // fluid and not LINKED, or stepped in line
  else work = type != LBM_CELL_SOLID;
  // the population loads do not wait for the flag: every address stays inside
  // the allocation (guard plane in front, ghost plane behind)
  C f[Q];
  if constexpr(!ODD) {
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      f[q]            = S::load(Ac[q * NA]);
    });
  } else {
    const int sy = P.nx, sz = P.nx * P.ny;
    static_for<Q>([&](auto qc) {
      constexpr int q   = decltype(qc)::value;
      const int     off = L::c(q, 0) + sy * L::c(q, 1) + sz * L::c(q, 2);
      f[q]              = S::load(Ac[L::opp(q) * NA - off]);  // warp-uniform offset from the cell's base
    });
  }
  C prev[NV];
  prefetch_moments<C, MOM, NV>(P, cell, prev);
  if(!work) return;
  if constexpr(ODD) {
    if constexpr(XF == 1) {
      if(__any_sync(__activemask(), xf)) {
        bulk_finish<LAT, EQ, ST, true, MOM, false, true>(P, y, z, cell, type, f, prev, diff, xf, x);
        return;
      }
    }
    if constexpr(XF == 2) {
      bulk_finish<LAT, EQ, ST, true, MOM, false, true>(P, y, z, cell, type, f, prev, diff, false, x, sf);
      return;
    }
    bulk_finish<LAT, EQ, ST, true, MOM, false>(P, y, z, cell, type, f, prev, diff);
  } else {
    // one vote per warp: warps of plain fluid (and solid) cells only take the
    // path without the inlet / Dirichlet / outlet branches.  Each lane votes
    // for its own cell, so a special cell always takes the full path.
    const bool special = type != LBM_CELL_FLUID;
    if(__any_sync(__activemask(), special)) bulk_finish<LAT, EQ, ST, false, MOM, true>(P, y, z, cell, type, f, prev, diff);
    else bulk_finish<LAT, EQ, ST, false, MOM, false>(P, y, z, cell, type, f, prev, diff);
  }
}

template <int LAT, int EQ, int ST, bool ODD, int MOM>
__device__ __forceinline__ void bulk_grid_cell(const BoxParams& P) {
  using C          = typename Store<ST>::C;
  constexpr int NV = EQ == LBM_NAVIER_STOKES ? Lattice<LAT>::D + 1 : 1;
  const int     x  = blockIdx.x * blockDim.x + threadIdx.x;
  const int     y  = blockIdx.y;
  const int     z  = blockIdx.z;
  C             diff[NV];
#pragma unroll
  for(int k = 0; k < NV; ++k) diff[k] = C(0);
  if(x < P.nx) {
    const int cell = x + P.nx * (y + P.ny * z);
    bulk_cell<LAT, EQ, ST, ODD, MOM, 1>(P, x, y, z, cell, P.flags[cell], diff);
  }
  if constexpr(MOM == 2) {
    const int64_t b = blockIdx.x + static_cast<int64_t>(gridDim.x) * (blockIdx.y + static_cast<int64_t>(gridDim.y) * blockIdx.z);
    warp_partials<NV>(diff, P.partials, P.partial_stride, b * (blockDim.x >> 5) + (threadIdx.x >> 5));
  }
}

template <int LAT, int EQ, int ST, bool ODD, int MOM>
__global__ void __launch_bounds__(256) k_box_bulk(BoxParams P) {
  bulk_grid_cell<LAT, EQ, ST, ODD, MOM>(P);
}

// The plain step of the FP32 / FP16 / BF16 storages with at most 48 registers
// per thread: the step is bound by memory latency and instruction issue
// together, and the extra resident warps hide more of the latency than the
// compiler's own register choice (64-72 on D3Q19) does.  40 registers spill
// the free-stream-shifted collision; 48 and 64 time alike on the 512x256x256
// sphere, 56 is slower.
#ifndef LBM_LEAN_REGS
#define LBM_LEAN_REGS 48
#endif
template <int LAT, int EQ, int ST, bool ODD>
__global__ void __maxnreg__(LBM_LEAN_REGS) k_box_bulk_lean(BoxParams P) {
  bulk_grid_cell<LAT, EQ, ST, ODD, 0>(P);
}

// Two populations of adjacent cells as one aligned load / store.
template <int ST>
struct Pair;
template <>
struct Pair<LBM_STORE_F32> {
  static __device__ __forceinline__ void load(const float* p, float& a, float& b) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    a              = v.x;
    b              = v.y;
  }
  static __device__ __forceinline__ void store(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }
};
template <>
struct Pair<LBM_STORE_F16_DEV> {
  static __device__ __forceinline__ void load(const __half* p, float& a, float& b) {
    const float2 v = __half22float2(*reinterpret_cast<const __half2*>(p));
    a              = v.x;
    b              = v.y;
  }
  static __device__ __forceinline__ void store(__half* p, float a, float b) { *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b); }
};
template <>
struct Pair<LBM_STORE_BF16_DEV> {
  static __device__ __forceinline__ void load(const __nv_bfloat16* p, float& a, float& b) {
    const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
    a              = v.x;
    b              = v.y;
  }
  static __device__ __forceinline__ void store(__nv_bfloat16* p, float a, float b) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
  }
};
template <>
struct Pair<LBM_STORE_E3M12_DEV> {
  static __device__ __forceinline__ void load(const uint16_t* p, float& a, float& b) {
    const uint32_t w = *reinterpret_cast<const uint32_t*>(p);
    a                = e3m12_decode(static_cast<uint16_t>(w & 0xffffu));
    b                = e3m12_decode(static_cast<uint16_t>(w >> 16));
  }
  static __device__ __forceinline__ void store(uint16_t* p, float a, float b) {
    *reinterpret_cast<uint32_t*>(p) = static_cast<uint32_t>(e3m12_encode(a)) | (static_cast<uint32_t>(e3m12_encode(b)) << 16);
  }
};

// k_box_pair: the plain (MOM = 0) bulk step with two x-adjacent cells per
// thread (nx even, so a pair never straddles a row and starts on an even
// cell).  Directions with c_x = 0 move both populations with one 2-element
// load and store; the others, one element apart from alignment, use two.
// Two independent collisions per thread also double the arithmetic in flight.
// Pairs that are not two plain fluid cells (even step) or two interior bulk
// cells (odd step) fall back to bulk_cell, cell by cell.
template <int LAT, int EQ, int ST, bool ODD>
__global__ void __launch_bounds__(256) k_box_pair(BoxParams P) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  using PR        = Pair<ST>;
  constexpr int Q = L::Q;
  const int     x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int     y = blockIdx.y;
  const int     z = blockIdx.z;
  if(x >= P.nx) return;
  const int      cell = x + P.nx * (y + P.ny * z);
  const uint16_t fl2  = *reinterpret_cast<const uint16_t*>(P.flags + cell);
  const uint8_t  fa = static_cast<uint8_t>(fl2 & 0xff), fb = static_cast<uint8_t>(fl2 >> 8);
  bool           fast;
  if constexpr(ODD) fast = fa == LBM_CELL_FLUID && fb == LBM_CELL_FLUID;  // both fluid, neither LINKED
  else fast = (fa & TYPE_MASK) == LBM_CELL_FLUID && (fb & TYPE_MASK) == LBM_CELL_FLUID;
  if(!fast) {
    C d[1];
    bulk_cell<LAT, EQ, ST, ODD, 0>(P, x, y, z, cell, fa, d);
    bulk_cell<LAT, EQ, ST, ODD, 0>(P, x + 1, y, z, cell + 1, fb, d);
    return;
  }
  T* const  Ac = static_cast<T*>(P.pop) + cell;  // the pair's first slot in plane 0
  const int NA = static_cast<int>(P.nalloc);
  const int sy = P.nx, sz = P.nx * P.ny;
  C         f0[Q], f1[Q];
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    if constexpr(!ODD) {
      PR::load(Ac + q * NA, f0[q], f1[q]);
    } else {
      const int off = L::c(q, 0) + sy * L::c(q, 1) + sz * L::c(q, 2);
      const T*  src = Ac + (L::opp(q) * NA - off);
      if constexpr(L::c(q, 0) == 0) {
        PR::load(src, f0[q], f1[q]);
      } else {
        f0[q] = S::load(src[0]);
        f1[q] = S::load(src[1]);
      }
    }
  });
  collide<LAT, EQ, C>(P, z, f0, nullptr);
  collide<LAT, EQ, C>(P, z, f1, nullptr);
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    if constexpr(!ODD) {
      PR::store(Ac + L::opp(q) * NA, f0[q], f1[q]);
    } else {
      const int off = L::c(q, 0) + sy * L::c(q, 1) + sz * L::c(q, 2);
      T*        dst = Ac + (q * NA + off);
      if constexpr(L::c(q, 0) == 0) {
        PR::store(dst, f0[q], f1[q]);
      } else {
        dst[0] = S::store(f0[q]);
        dst[1] = S::store(f1[q]);
      }
    }
  });
}

// Link tables of the boundary cells, built once: for list entry i and
// direction q, src[q*n+i] is the population slot the odd step pulls into f_q
// (a neighbour's slot, the cell's own slot for a bounce, or the outlet ghost)
// and dst[q*n+i] the slot the post-collision f_q is pushed to (-1: it leaves
// through an open face).  corr_* hold the moving-wall momentum in state units
// and, for a state shifted to a free stream (FP32 / FP16 / BF16 storage), the
// change of shift of a bounced population (only allocated when a wall moves
// or the state is shifted).
template <int LAT>
__global__ void k_box_build_links(BoxParams P, const int32_t* list, int n, int32_t* src, int32_t* dst, double* corr_src,
                                  double* corr_dst) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q;
  const int     i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  const int     cell = list[i];
  const int     x = cell % P.nx, y = (cell / P.nx) % P.ny, z = cell / (P.nx * P.ny);
  const int64_t NA   = P.nalloc;
  static_for<Q>([&](auto qc) {
    constexpr int q  = decltype(qc)::value;
    const Link    lp = resolve<LAT>(P, x, y, z, q, -1, q);
    int64_t       s;
    if(lp.kind == LINK_CELL) s = L::opp(lp.q) * NA + lp.cell;
    else if(lp.kind == LINK_BOUNCE) s = q * NA + cell;
    else s = Q * NA + ghost_index(P, q, y, z);
    src[q * n + i] = static_cast<int32_t>(s);
    const Link lq  = resolve<LAT>(P, x, y, z, q, +1, L::opp(q));
    int64_t    d   = -1;
    if(lq.kind == LINK_CELL) d = lq.q * NA + lq.cell;
    else if(lq.kind == LINK_BOUNCE) d = L::opp(q) * NA + cell;
    dst[q * n + i] = static_cast<int32_t>(d);
    if(corr_src) {
      // a bounced population changes direction, and with it the shift of a
      // shifted state: the pulled slot holds f_opp(q), the pushed slot
      // receives f_opp(q)
      const double dk = bounce_shift<LAT>(P, q);
      corr_src[q * n + i] = lp.kind == LINK_BOUNCE ? lp.corr + dk : 0.0;
      corr_dst[q * n + i] = lq.kind == LINK_BOUNCE ? lq.corr - dk : 0.0;
    }
  });
}

// The free-slip face cells that the boundary kernel steps without link tables
// (SFACE cells, per-thread odd step only): positions off the x faces on the
// two y faces (ny_part of them; for a 2D lattice every slice z) and then on
// the two z faces, x fastest.  Blocks from list_blocks on take one position
// per thread; positions without the SFACE bit do nothing.
struct FaceRange {
  int64_t ny_part     = 0;
  int64_t n           = 0;
  int     list_blocks = 0;
};

template <int LAT>
__device__ __forceinline__ void face_position(const BoxParams& P, const FaceRange& fr, int64_t j, int& x, int& y, int& z) {
  const int64_t w = P.nx - 2;
  if(j < fr.ny_part) {
    const int64_t per  = fr.ny_part / 2;
    const bool    high = j >= per;
    const int64_t r    = high ? j - per : j;
    x                  = 1 + static_cast<int>(r % w);
    z                  = (Lattice<LAT>::D > 2 ? 1 : 0) + static_cast<int>(r / w);
    y                  = high ? P.ny - 1 : 0;
  } else {
    const int64_t per  = (fr.n - fr.ny_part) / 2;
    const bool    high = j - fr.ny_part >= per;
    const int64_t r    = high ? j - fr.ny_part - per : j - fr.ny_part;
    x                  = 1 + static_cast<int>(r % w);
    y                  = 1 + static_cast<int>(r / w);
    z                  = high ? P.nz - 1 : 0;
  }
}

template <int LAT, int EQ, int ST, int MOM>
__global__ void __launch_bounds__(128) k_box_bnd(BoxParams P, const int32_t* list, int count, int n, int64_t slot0, const int32_t* src,
                                                 const int32_t* dst, const double* corr_src, const double* corr_dst, FaceRange fr) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  constexpr int NV   = EQ == LBM_NAVIER_STOKES ? L::D + 1 : 1;
  const int     i    = blockIdx.x * blockDim.x + threadIdx.x;
  C             diff[NV];
#pragma unroll
  for(int k = 0; k < NV; ++k) diff[k] = C(0);
  if(static_cast<int>(blockIdx.x) >= fr.list_blocks) {
    const int64_t j = static_cast<int64_t>(blockIdx.x - fr.list_blocks) * blockDim.x + threadIdx.x;
    if(j < fr.n) {
      int x, y, z;
      face_position<LAT>(P, fr, j, x, y, z);
      const int cell = x + P.nx * (y + P.ny * z);
      bulk_cell<LAT, EQ, ST, true, MOM, 2>(P, x, y, z, cell, P.flags[cell], diff);
    }
  } else if(i < count) {  // the first `count` entries; tables have stride n
    const int     cell = list[i];
    const uint8_t type = P.flags[cell] & TYPE_MASK;
    T*            A    = static_cast<T*>(P.pop);
    C             f[Q];
    C             mom[NV], prev[NV];
#pragma unroll
    for(int k = 0; k < NV; ++k) mom[k] = 0;
    prefetch_moments<C, MOM, NV>(P, cell, prev);
    // every table entry is read before the first population store: a table
    // load issued after a store would wait behind it (the compiler cannot
    // prove the two do not alias), one memory round trip per direction
    int32_t dsts[Q];
    static_for<Q>([&](auto qc) { dsts[decltype(qc)::value] = dst[decltype(qc)::value * n + i]; });
    if(type == LBM_CELL_INLET || type == LBM_CELL_DIRICHLET) {
      emit_equilibrium<LAT, EQ, C>(P, f, cell);
    } else {
      static_for<Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        f[q]            = S::load(A[src[q * n + i]]);
        if(corr_src) f[q] += static_cast<C>(corr_src[q * n + i]);
      });
      const int z = (P.slice_omega || P.slice_src) ? static_cast<int>(cell / (static_cast<int64_t>(P.nx) * P.ny)) : 0;
      collide<LAT, EQ, C>(P, z, f, MOM ? mom : nullptr);
    }
    if(corr_dst)
      static_for<Q>([&](auto qc) { f[decltype(qc)::value] += static_cast<C>(corr_dst[decltype(qc)::value * n + i]); });
    moments_io<LAT, EQ, C, MOM, NV>(P, cell, mom, prev, diff);
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      if(dsts[q] >= 0) A[dsts[q]] = S::store(f[q]);
    });
  }
  if constexpr(MOM == 2) warp_partials<NV>(diff, P.partials, P.partial_stride, slot0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
}

// outlet ghost fill, run before every step: for each outlet cell and each
// direction q with c_qx = -1, the population its upstream neighbour receives
// skip_xface: the outlet cells of the inlet / outlet face rows (XFACE) read
// their upstream cell from the row-staged kernel's shared memory instead
// (box_rows.cu), so only the other outlet cells need a ghost value
template <int LAT, int ST, bool ODD>
__global__ void k_box_outlet(BoxParams P, bool skip_xface) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  constexpr int Q = L::Q;
  const int     y = blockIdx.x * blockDim.x + threadIdx.x;
  const int     z = blockIdx.y;
  if(y >= P.ny) return;
  const int     x  = P.nx - 1;
  const int64_t r  = x + static_cast<int64_t>(P.nx) * (y + static_cast<int64_t>(P.ny) * z);
  const uint8_t fl = P.flags[r];
  if((fl & TYPE_MASK) != LBM_CELL_OUTLET || (skip_xface && (fl & XFACE))) return;
  T*            A  = static_cast<T*>(P.pop);
  const int64_t NA = P.nalloc;
  const int64_t u  = r - 1;
#pragma unroll
  for(int q = 0; q < Q; ++q) {
    if(L::c(q, 0) >= 0) continue;
    T v;
    if(!ODD) {
      v = A[q * NA + u];  // standard layout: what u received in the last odd step
    } else {
      const Link lk = resolve<LAT>(P, x - 1, y, z, q, -1, q);
      if(lk.kind == LINK_CELL) {
        v = A[L::opp(lk.q) * NA + lk.cell];
      } else {
        // bounce-back at the upstream cell (a wall or solid beside it)
        using C = typename S::C;
        // a bounced population changes direction, and with it the shift
        v = S::store(S::load(A[q * NA + u]) + static_cast<C>(bounce_shift<LAT>(P, q) + lk.corr));
      }
    }
    A[Q * NA + ghost_index(P, q, y, z)] = v;
  }
}

// FP64 post-stream populations of one cell of the current state (reference
// layout of m_fold), with inlet/Dirichlet cells reported as the equilibrium
// they emit and solids as zero; element q goes to out[q * stride]
template <int LAT, int EQ, int ST>
__device__ __forceinline__ void readout_cell(const BoxParams& P, bool odd, int x, int y, int z, double* out, int64_t stride) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  const int64_t cell = x + static_cast<int64_t>(P.nx) * (y + static_cast<int64_t>(P.ny) * z);
  const uint8_t type = P.flags[cell] & TYPE_MASK;
  const T*      A    = static_cast<const T*>(P.pop);
  const int64_t NA   = P.nalloc;
  C             f[Q];
  if(type == LBM_CELL_SOLID) {
#pragma unroll
    for(int q = 0; q < Q; ++q) out[q * stride] = 0.0;
    return;
  }
  if(type == LBM_CELL_INLET || type == LBM_CELL_DIRICHLET) {
    emit_equilibrium<LAT, EQ, C>(P, f, cell);
  } else {
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      if(!odd) {
        f[q] = S::load(A[q * NA + cell]);
        if(type == LBM_CELL_OUTLET && L::c(q, 0) < 0) f[q] = S::load(A[q * NA + cell - 1]);
      } else {
        int  xs = x;
        Link lk = resolve<LAT>(P, x, y, z, q, -1, q);
        if(lk.kind == LINK_OPEN) {  // beyond the outlet: what the upstream cell receives
          xs = x - 1;
          lk = resolve<LAT>(P, xs, y, z, q, -1, q);
        }
        const int64_t own = xs + static_cast<int64_t>(P.nx) * (y + static_cast<int64_t>(P.ny) * z);
        if(lk.kind == LINK_CELL) f[q] = S::load(A[L::opp(lk.q) * NA + lk.cell]);
        else  // bounced: f_opp(q) of the cell, with its change of shift
          f[q] = S::load(A[q * NA + own]) + static_cast<C>(bounce_shift<LAT>(P, q) + lk.corr);
      }
    }
  }
#pragma unroll
  for(int q = 0; q < Q; ++q) out[q * stride] = box_state_to_f<LAT, EQ, ST>(P, static_cast<double>(f[q]), q);
}

template <int LAT, int EQ, int ST>
__global__ void k_box_readout(BoxParams P, bool odd, double* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if(x >= P.nx) return;
  const int64_t cell = x + static_cast<int64_t>(P.nx) * (y + static_cast<int64_t>(P.ny) * z);
  readout_cell<LAT, EQ, ST>(P, odd, x, y, z, out + cell, P.ncells);
}

// store FP64 post-stream populations into the standard (even-parity) layout
template <int LAT, int EQ, int ST>
__global__ void k_box_load(BoxParams P, const double* in) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  const int64_t cell = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if(cell >= P.ncells) return;
  T* A = static_cast<T*>(P.pop);
  // every load before the first store (a load after a store the compiler
  // cannot prove disjoint would wait for it); `in` may be host memory read
  // over the CPU-GPU link, where a round trip per direction would be slow
  double v[Q];
#pragma unroll
  for(int q = 0; q < Q; ++q) v[q] = in[q * P.ncells + cell];
#pragma unroll
  for(int q = 0; q < Q; ++q) A[q * P.nalloc + cell] = S::store(static_cast<C>(box_f_to_state<LAT, EQ, ST>(P, v[q], q)));
}

// uniform initial state: the same FP64 population vector in every cell
struct InitVec {
  double f[19];
};
template <int LAT, int EQ, int ST>
__global__ void k_box_init(BoxParams P, InitVec v) {
  using L         = Lattice<LAT>;
  using S         = Store<ST>;
  using T         = typename S::T;
  using C         = typename S::C;
  constexpr int Q = L::Q;
  const int64_t cell = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if(cell >= P.ncells) return;
  T* A = static_cast<T*>(P.pop);
#pragma unroll
  for(int q = 0; q < Q; ++q) A[q * P.nalloc + cell] = S::store(static_cast<C>(box_f_to_state<LAT, EQ, ST>(P, v.f[q], q)));
}

// moments (rho or phi, u) of FP64 populations
// FP64 moments of one cell from its FP64 populations (f[q * stride]):
// rho and the velocity with the Guo half-force shift, or the potential;
// written to m[0] (rho or phi) and m[1 + d] (u_d)
template <int LAT, int EQ>
__device__ __forceinline__ void cell_moments_f64(const BoxParams& P, const double* f, int64_t stride, double* m) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  if constexpr(EQ == LBM_NAVIER_STOKES) {
    double r = 0, j[3] = {0, 0, 0};
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      const double v = f[q * stride];
      r += v;
#pragma unroll
      for(int d = 0; d < D; ++d) j[d] += L::c(q, d) * v;
    }
    const double F[3] = {P.has_force ? P.force[0] : 0.0, P.has_force ? P.force[1] : 0.0, P.has_force ? P.force[2] : 0.0};
    m[0] = r;
#pragma unroll
    for(int d = 0; d < D; ++d) m[1 + d] = r != 0.0 ? (j[d] + 0.5 * F[d]) / r : 0.0;
  } else {
    double acc = 0;
#pragma unroll
    for(int q = 0; q < Q - 1; ++q) acc += f[q * stride];
    m[0] = acc / (1.0 - L::w(Q - 1));
  }
}

template <int LAT, int EQ>
__global__ void k_box_moments_f64(BoxParams P, const double* f, double* rho, double* ux, double* uy, double* uz) {
  constexpr int D    = Lattice<LAT>::D;
  const int64_t cell = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if(cell >= P.ncells) return;
  double m[4];
  cell_moments_f64<LAT, EQ>(P, f + cell, P.ncells, m);
  if(rho) rho[cell] = m[0];
  if constexpr(EQ == LBM_NAVIER_STOKES) {
    double* uu[3] = {ux, uy, uz};
#pragma unroll
    for(int d = 0; d < D; ++d)
      if(uu[d]) uu[d][cell] = m[1 + d];
  }
}

// moments of a list of cells (line probes): the same populations and the same
// arithmetic as the full read-out, for n cells only; out[i * nv + k] with
// k = 0 rho (phi), 1.. the velocity
template <int LAT, int EQ, int ST>
__global__ void k_box_probe(BoxParams P, bool odd, const int64_t* cells, int64_t n, int nv, double* out) {
  constexpr int Q = Lattice<LAT>::Q;
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if(i >= n) return;
  const int64_t cell = cells[i];
  const int64_t row  = cell / P.nx;
  double        f[Q], m[4];
  readout_cell<LAT, EQ, ST>(P, odd, static_cast<int>(cell - row * P.nx), static_cast<int>(row % P.ny), static_cast<int>(row / P.ny), f, 1);
  cell_moments_f64<LAT, EQ>(P, f, 1, m);
  for(int k = 0; k < nv; ++k) out[i * nv + k] = m[k];
}

// sum over cells of the FP64 populations: mass and momentum
template <int LAT>
__global__ void k_box_sum(const double* f, int64_t n, double* partials) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  __shared__ double sh[D + 1][32];
  double acc[D + 1];
#pragma unroll
  for(int k = 0; k <= D; ++k) acc[k] = 0;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      const double v = f[q * n + i];
      acc[0] += v;
#pragma unroll
      for(int d = 0; d < D; ++d) acc[d + 1] += L::c(q, d) * v;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for(int k = 0; k <= D; ++k) {
    const double s = warp_sum(acc[k]);
    if(lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if(wid == 0) {
#pragma unroll
    for(int k = 0; k <= D; ++k) {
      double s = lane < nw ? sh[k][lane] : 0.0;
      s        = warp_sum(s);
      if(lane == 0) partials[k * gridDim.x + blockIdx.x] = s;
    }
  }
}

// first level of the residual reduction: block c sums the contiguous chunk
// [c*chunk, (c+1)*chunk) of every vector into mid[v*gridDim.x + c]
__global__ void k_chunk_sum(const double* partials, int64_t nb, int64_t stride, int nvec, int64_t chunk, double* mid) {
  __shared__ double sh[32];
  const int64_t lo = blockIdx.x * chunk, hi = lo + chunk < nb ? lo + chunk : nb;
  for(int v = 0; v < nvec; ++v) {
    double acc = 0;
    for(int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) acc += partials[v * stride + i];
    acc = warp_sum(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if(lane == 0) sh[wid] = acc;
    __syncthreads();
    if(wid == 0) {
      double t = lane < static_cast<int>(blockDim.x >> 5) ? sh[lane] : 0.0;
      t        = warp_sum(t);
      if(lane == 0) mid[v * gridDim.x + blockIdx.x] = t;
    }
    __syncthreads();
  }
}

__global__ void k_final_sum(const double* partials, int64_t nb, int64_t stride, int nvec, double* out) {
  __shared__ double sh[32];
  for(int v = 0; v < nvec; ++v) {
    double acc = 0;
    for(int64_t i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[v * stride + i];
    acc = warp_sum(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if(lane == 0) sh[wid] = acc;
    __syncthreads();
    if(wid == 0) {
      double s = lane < static_cast<int>(blockDim.x >> 5) ? sh[lane] : 0.0;
      s        = warp_sum(s);
      if(lane == 0) out[v] = s;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
dim3 step_grid(const BoxState* b, int tpb) {
  return dim3(static_cast<unsigned>((b->p.nx + tpb - 1) / tpb), static_cast<unsigned>(b->p.ny), static_cast<unsigned>(b->p.nz));
}

template <int LAT, int EQ, int ST>
cudaError_t launch_step(BoxState* b, bool odd, int mom, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1) {
  const int  tpb = b->tuned_tpb;
  const dim3 g   = step_grid(b, tpb);
  if(b->p.has_outlet) {
    const dim3 go(static_cast<unsigned>((b->p.ny + 127) / 128), static_cast<unsigned>(b->p.nz));
    // the row-staged kernel takes its outlet face cells' upstream values from
    // its own staged rows (when the outlet and upstream cells share a warp)
    const int  k    = odd ? b->kind_odd : b->kind_even;
    const bool skip = k == LBM_BOX_KERNEL_ROWS && box_rows_outlet_inline(b);
    if(odd) k_box_outlet<LAT, ST, true><<<go, 128, 0, s>>>(b->p, skip);
    else k_box_outlet<LAT, ST, false><<<go, 128, 0, s>>>(b->p, skip);
  }
  if(ev0) cudaEventRecord(ev0, s);
  int64_t        nbulk = static_cast<int64_t>(g.x) * g.y * g.z * (tpb / 32);  // residual slots (warps) of the bulk kernel
  const int      kind   = odd ? b->kind_odd : b->kind_even;
  const bool     staged = kind == LBM_BOX_KERNEL_STAGED;
  const bool     paired = kind == LBM_BOX_KERNEL_PAIRED && mom == 0;  // residual steps use the per-thread kernel
  const bool     rows   = kind == LBM_BOX_KERNEL_ROWS;                // like the per-thread kernel: XFACE cells in line
  // the per-thread odd kernel steps the XFACE cells itself; with the others the
  // boundary kernel takes them too (they close its list)
  // and its SFACE cells are taken by the boundary kernel's face blocks
  const bool     lean   = !(staged || paired);
  const int      nlist  = static_cast<int>(lean ? b->n_bnd_lean : b->n_bnd);
  FaceRange      fr;
  fr.list_blocks        = (nlist + 127) / 128;
  if(lean && b->n_sface > 0) {
    fr.ny_part = b->face_ny_part;
    fr.n       = b->face_n;
  }
  const unsigned nbb    = static_cast<unsigned>(fr.list_blocks + (fr.n + 127) / 128);
  const dim3     gp(static_cast<unsigned>((b->p.nx / 2 + tpb - 1) / tpb), static_cast<unsigned>(b->p.ny), static_cast<unsigned>(b->p.nz));
  if(staged) {
    const cudaError_t e = box_tma_bulk(b, odd, mom, s, &nbulk);
    if(e != cudaSuccess) return e;
  }
  if(rows) {
    // before the boundary kernel, whose cells' slots it writes back unchanged
    const cudaError_t e = box_rows_bulk(b, odd, mom, s, &nbulk);
    if(e != cudaSuccess) return e;
  }
  if(odd) {
    if(staged || rows) {
    } else if(paired) {
      if constexpr(ST != LBM_STORE_F64) k_box_pair<LAT, EQ, ST, true><<<gp, tpb, 0, s>>>(b->p);
    } else if(mom == 0) {
      if constexpr(ST == LBM_STORE_F64) k_box_bulk<LAT, EQ, ST, true, 0><<<g, tpb, 0, s>>>(b->p);
      else k_box_bulk_lean<LAT, EQ, ST, true><<<g, tpb, 0, s>>>(b->p);
    }
    else if(mom == 1) k_box_bulk<LAT, EQ, ST, true, 1><<<g, tpb, 0, s>>>(b->p);
    else k_box_bulk<LAT, EQ, ST, true, 2><<<g, tpb, 0, s>>>(b->p);
    if(nbb) {
      if(mom == 0) k_box_bnd<LAT, EQ, ST, 0><<<nbb, 128, 0, s>>>(b->p, b->bnd_list, nlist, static_cast<int>(b->n_bnd), nbulk, b->link_src, b->link_dst, b->corr_src, b->corr_dst, fr);
      else if(mom == 1) k_box_bnd<LAT, EQ, ST, 1><<<nbb, 128, 0, s>>>(b->p, b->bnd_list, nlist, static_cast<int>(b->n_bnd), nbulk, b->link_src, b->link_dst, b->corr_src, b->corr_dst, fr);
      else k_box_bnd<LAT, EQ, ST, 2><<<nbb, 128, 0, s>>>(b->p, b->bnd_list, nlist, static_cast<int>(b->n_bnd), nbulk, b->link_src, b->link_dst, b->corr_src, b->corr_dst, fr);
    }
    if(mom == 2) b->res_slots = nbulk + static_cast<int64_t>(nbb) * 4;
  } else {
    if(staged || rows) {
    } else if(paired) {
      if constexpr(ST != LBM_STORE_F64) k_box_pair<LAT, EQ, ST, false><<<gp, tpb, 0, s>>>(b->p);
    } else if(mom == 0) {
      if constexpr(ST == LBM_STORE_F64) k_box_bulk<LAT, EQ, ST, false, 0><<<g, tpb, 0, s>>>(b->p);
      else k_box_bulk_lean<LAT, EQ, ST, false><<<g, tpb, 0, s>>>(b->p);
    }
    else if(mom == 1) k_box_bulk<LAT, EQ, ST, false, 1><<<g, tpb, 0, s>>>(b->p);
    else k_box_bulk<LAT, EQ, ST, false, 2><<<g, tpb, 0, s>>>(b->p);
    if(mom == 2) b->res_slots = nbulk;
  }
  if(ev1) cudaEventRecord(ev1, s);
  return cudaGetLastError();
}

template <int LAT, int EQ, int ST>
cudaError_t launch_readout(BoxState* b, double* out, cudaStream_t s) {
  const dim3 g = step_grid(b, 128);
  k_box_readout<LAT, EQ, ST><<<g, 128, 0, s>>>(b->p, (b->steps & 1) != 0, out);
  return cudaGetLastError();
}

template <int LAT, int EQ, int ST>
cudaError_t launch_probe(BoxState* b, const int64_t* cells, int64_t n, double* out, cudaStream_t s) {
  k_box_probe<LAT, EQ, ST><<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(b->p, (b->steps & 1) != 0, cells, n, b->nvar, out);
  return cudaGetLastError();
}

template <int LAT, int EQ, int ST>
cudaError_t launch_load(BoxState* b, const double* in, cudaStream_t s) {
  k_box_load<LAT, EQ, ST><<<static_cast<unsigned>((b->p.ncells + 255) / 256), 256, 0, s>>>(b->p, in);
  return cudaGetLastError();
}

// one switch for every (lattice, equation, storage) instantiation
#define LBM_BOX_DISPATCH(FN, ...)                                                                          \
  do {                                                                                                     \
    const int key = b->desc.lattice * 100 + b->desc.equation * 10 + b->desc.storage;                        \
    switch(key) {                                                                                          \
      case LBM_D2Q9 * 100 + 0 + LBM_STORE_F64: return FN<LBM_D2Q9, 0, LBM_STORE_F64>(__VA_ARGS__);         \
      case LBM_D2Q9 * 100 + 0 + LBM_STORE_F32: return FN<LBM_D2Q9, 0, LBM_STORE_F32>(__VA_ARGS__);         \
      case LBM_D2Q9 * 100 + 0 + LBM_STORE_F16_DEV: return FN<LBM_D2Q9, 0, LBM_STORE_F16_DEV>(__VA_ARGS__); \
      case LBM_D2Q9 * 100 + 0 + LBM_STORE_BF16_DEV: return FN<LBM_D2Q9, 0, LBM_STORE_BF16_DEV>(__VA_ARGS__); \
      case LBM_D2Q9 * 100 + 0 + LBM_STORE_E3M12_DEV: return FN<LBM_D2Q9, 0, LBM_STORE_E3M12_DEV>(__VA_ARGS__); \
      case LBM_D3Q19 * 100 + 0 + LBM_STORE_F64: return FN<LBM_D3Q19, 0, LBM_STORE_F64>(__VA_ARGS__);       \
      case LBM_D3Q19 * 100 + 0 + LBM_STORE_F32: return FN<LBM_D3Q19, 0, LBM_STORE_F32>(__VA_ARGS__);       \
      case LBM_D3Q19 * 100 + 0 + LBM_STORE_F16_DEV: return FN<LBM_D3Q19, 0, LBM_STORE_F16_DEV>(__VA_ARGS__); \
      case LBM_D3Q19 * 100 + 0 + LBM_STORE_BF16_DEV: return FN<LBM_D3Q19, 0, LBM_STORE_BF16_DEV>(__VA_ARGS__); \
      case LBM_D3Q19 * 100 + 0 + LBM_STORE_E3M12_DEV: return FN<LBM_D3Q19, 0, LBM_STORE_E3M12_DEV>(__VA_ARGS__); \
      case LBM_D3Q7 * 100 + 10 + LBM_STORE_F64: return FN<LBM_D3Q7, 1, LBM_STORE_F64>(__VA_ARGS__);        \
      case LBM_D3Q7 * 100 + 10 + LBM_STORE_F32: return FN<LBM_D3Q7, 1, LBM_STORE_F32>(__VA_ARGS__);        \
      default: return cudaErrorInvalidValue;                                                               \
    }                                                                                                      \
  } while(0)

cudaError_t dispatch_step(BoxState* b, bool odd, int mom, cudaStream_t s, cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr) {
  LBM_BOX_DISPATCH(launch_step, b, odd, mom, s, ev0, ev1);
}
cudaError_t dispatch_readout(BoxState* b, double* out, cudaStream_t s) { LBM_BOX_DISPATCH(launch_readout, b, out, s); }
cudaError_t dispatch_load(BoxState* b, const double* in, cudaStream_t s) { LBM_BOX_DISPATCH(launch_load, b, in, s); }
cudaError_t dispatch_probe(BoxState* b, const int64_t* cells, int64_t n, double* out, cudaStream_t s) {
  LBM_BOX_DISPATCH(launch_probe, b, cells, n, out, s);
}

template <int LAT, int EQ, int ST>
cudaError_t launch_init(BoxState* b, const InitVec& v, cudaStream_t s) {
  k_box_init<LAT, EQ, ST><<<static_cast<unsigned>((b->p.ncells + 255) / 256), 256, 0, s>>>(b->p, v);
  return cudaGetLastError();
}
cudaError_t dispatch_init(BoxState* b, const InitVec& v, cudaStream_t s) { LBM_BOX_DISPATCH(launch_init, b, v, s); }


bool ensure_staging(BoxState* b) {
  if(b->f64) return true;
  return cudaMalloc(&b->f64, sizeof(double) * b->Q * b->p.ncells) == cudaSuccess;
}

int cerr(std::string& err, cudaError_t e, const char* what) {
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return LBM_ERR_CUDA;
}

// a staged kernel that gave up waiting for its copies leaves a flag behind
int check_wait_flag(BoxState* b, std::string& err) {
  const auto waits = [](int k) { return k == LBM_BOX_KERNEL_STAGED || k == LBM_BOX_KERNEL_ROWS; };
  if(!waits(b->kind_even) && !waits(b->kind_odd)) return LBM_OK;
  int         flag = 0;
  cudaError_t e    = cudaMemcpy(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if(e != cudaSuccess) return cerr(err, e, "wait flag");
  if(flag) {
    cudaMemset(b->d_err, 0, sizeof(int));
    err = "staged step kernel: a bulk-copy wait timed out (state of this step is invalid)";
    return LBM_ERR_TIMEOUT;
  }
  return LBM_OK;
}

bool box_kernel_supported(const BoxState* b, int kind) {
  if(kind == LBM_BOX_KERNEL_THREAD) return true;
  if(kind == LBM_BOX_KERNEL_STAGED) return box_tma_supported(b);
  if(kind == LBM_BOX_KERNEL_PAIRED) return b->p.nx % 2 == 0 && b->desc.storage != LBM_STORE_F64;
  if(kind == LBM_BOX_KERNEL_ROWS) return box_rows_supported(b);
  return false;
}

void drop_graphs(BoxState* b) {
  for(auto& g : b->graph)
    if(g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

}  // namespace

cudaError_t box_initial_condition(BoxState* b, cudaStream_t s) {
  // equilibrium at (init_density, init_velocity); Poisson starts from phi = 0
  const int Q = b->Q, D = b->D;
  double    c[19][3], w[19];
  auto fill = [&](auto L) {
    using LL = decltype(L);
    for(int q = 0; q < Q; ++q) {
      for(int d = 0; d < 3; ++d) c[q][d] = LL::c(q, d);
      w[q] = LL::w(q);
    }
  };
  if(b->desc.lattice == LBM_D2Q9) fill(Lattice<LBM_D2Q9>{});
  else if(b->desc.lattice == LBM_D3Q19) fill(Lattice<LBM_D3Q19>{});
  else fill(Lattice<LBM_D3Q7>{});
  InitVec v{};
  if(b->desc.equation == LBM_NAVIER_STOKES) {
    const double rho = b->desc.init_density;
    double       usq = 0;
    for(int d = 0; d < D; ++d) usq += b->desc.init_velocity[d] * b->desc.init_velocity[d];
    for(int q = 0; q < Q; ++q) {
      double cu = 0;
      for(int d = 0; d < D; ++d) cu += c[q][d] * b->desc.init_velocity[d];
      v.f[q] = w[q] * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
    }
  }
  cudaError_t e = dispatch_init(b, v, s);
  if(e != cudaSuccess) return e;
  b->steps     = 0;
  b->res_ready = 0;
  b->mom_valid = 0;
  return cudaStreamSynchronize(s);
}

// Enqueue nsteps on stream s (no synchronisation).
int box_step_enqueue(BoxState* b, int64_t nsteps, cudaStream_t s, std::string& err) {
  // All but the last two steps replay a captured one-step graph per parity.
  // The last two record the moments (mode 1) and then the residual partials
  // against them (mode 2), so lbm_gpu_residual is ready after any call of two
  // or more steps; a one-step call compares with the moments the previous call
  // left behind.
  const int64_t plain = nsteps >= 2 ? nsteps - 2 : 0;
  for(int64_t k = 0; k < plain; ++k) {
    const int parity = static_cast<int>(b->steps & 1);
    if(!b->graph[parity]) {
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      if(e != cudaSuccess) return cerr(err, e, "begin capture");
      e              = dispatch_step(b, parity != 0, 0, s);
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if(e != cudaSuccess) return cerr(err, e, "step launch");
      if(e2 != cudaSuccess) return cerr(err, e2, "end capture");
      e = cudaGraphInstantiate(&b->graph[parity], g, 0);
      cudaGraphDestroy(g);
      if(e != cudaSuccess) return cerr(err, e, "graph instantiate");
    }
    cudaError_t e = cudaGraphLaunch(b->graph[parity], s);
    if(e != cudaSuccess) return cerr(err, e, "graph launch");
    ++b->steps;
    b->mom_valid = 0;
    b->res_ready = 0;
  }
  for(int64_t k = plain; k < nsteps; ++k) {
    const int   mom = b->mom_valid ? 2 : 1;
    cudaError_t e   = dispatch_step(b, (b->steps & 1) != 0, mom, s);
    if(e != cudaSuccess) return cerr(err, e, "step");
    ++b->steps;
    b->mom_valid = 1;
    b->res_ready = mom == 2;
  }
  return LBM_OK;
}

int box_step(BoxState* b, int64_t nsteps, cudaStream_t s, std::string& err) {
  const int rc = box_step_enqueue(b, nsteps, s, err);
  if(rc != LBM_OK) return rc;
  cudaError_t e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return cerr(err, e, "step sync");
  return check_wait_flag(b, err);
}

int box_residual(BoxState* b, double* r, cudaStream_t s, std::string& err) {
  if(!b->res_ready) {
    err = "residual needs a step call of at least two steps";
    return LBM_ERR_INVALID;
  }
  // two levels, fixed shapes: deterministic bits for a given box and tuning
  const int64_t chunk = (b->res_slots + kMidBlocks - 1) / kMidBlocks;
  k_chunk_sum<<<kMidBlocks, 256, 0, s>>>(b->partials, b->res_slots, b->p.partial_stride, b->nvar, chunk, b->partials_mid);
  k_final_sum<<<1, 256, 0, s>>>(b->partials_mid, kMidBlocks, kMidBlocks, b->nvar, b->out);
  cudaError_t e = cudaMemcpyAsync(r, b->out, sizeof(double) * b->nvar, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return cerr(err, e, "residual");
  for(int v = 0; v < b->nvar; ++v)
    if(!std::isfinite(r[v])) {
      err = "Solution diverged";
      return LBM_ERR_DIVERGED;
    }
  return LBM_OK;
}

int box_get_populations(BoxState* b, double* f, cudaStream_t s, std::string& err) {
  if(!ensure_staging(b)) {
    err = "staging allocation failed";
    return LBM_ERR_NOMEM;
  }
  cudaError_t e = dispatch_readout(b, b->f64, s);
  if(e == cudaSuccess) e = cudaMemcpyAsync(f, b->f64, sizeof(double) * b->Q * b->p.ncells, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? LBM_OK : cerr(err, e, "get populations");
}

// A host array the device can read in place: page-locked memory mapped into
// the device's address space (on Grace-Blackwell the load kernel then streams
// it over the coherent CPU-GPU link and converts on the fly, with no staging
// copy); nullptr for anything else.
static const double* device_view_of_host(const double* f) {
  cudaPointerAttributes a{};
  if(cudaPointerGetAttributes(&a, f) != cudaSuccess) {
    cudaGetLastError();  // pageable memory of an older driver: clear the error
    return nullptr;
  }
  if(a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return static_cast<const double*>(a.devicePointer);
}

int box_set_populations(BoxState* b, const double* f, cudaStream_t s, std::string& err) {
  cudaError_t   e      = cudaSuccess;
  const double* direct = device_view_of_host(f);
  if(direct) {
    e = dispatch_load(b, direct, s);
  } else {
    if(!ensure_staging(b)) {
      err = "staging allocation failed";
      return LBM_ERR_NOMEM;
    }
    e = cudaMemcpyAsync(b->f64, f, sizeof(double) * b->Q * b->p.ncells, cudaMemcpyHostToDevice, s);
    if(e == cudaSuccess) e = dispatch_load(b, b->f64, s);
  }
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return cerr(err, e, "set populations");
  b->steps     = 0;  // the layout is now the even-parity (standard) one
  b->res_ready = 0;
  b->mom_valid = 0;
  return LBM_OK;
}

int box_mass_momentum(BoxState* b, double* out, cudaStream_t s, std::string& err) {
  if(!ensure_staging(b)) {
    err = "staging allocation failed";
    return LBM_ERR_NOMEM;
  }
  cudaError_t e = dispatch_readout(b, b->f64, s);
  if(e != cudaSuccess) return cerr(err, e, "readout");
  const int nb = 304;
  switch(b->desc.lattice) {
    case LBM_D2Q9: k_box_sum<LBM_D2Q9><<<nb, 256, 0, s>>>(b->f64, b->p.ncells, b->partials_mm); break;
    case LBM_D3Q19: k_box_sum<LBM_D3Q19><<<nb, 256, 0, s>>>(b->f64, b->p.ncells, b->partials_mm); break;
    default: k_box_sum<LBM_D3Q7><<<nb, 256, 0, s>>>(b->f64, b->p.ncells, b->partials_mm); break;
  }
  k_final_sum<<<1, 256, 0, s>>>(b->partials_mm, nb, nb, b->D + 1, b->out + 4);
  e = cudaMemcpyAsync(out, b->out + 4, sizeof(double) * (b->D + 1), cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? LBM_OK : cerr(err, e, "mass/momentum");
}

int box_info(const BoxState* b, int64_t* ncells, int32_t* q, int32_t* nvar) {
  if(ncells) *ncells = b->p.ncells;
  if(q) *q = b->Q;
  if(nvar) *nvar = b->nvar;
  return LBM_OK;
}

void box_destroy(BoxState* b) {
  if(!b) return;
  drop_graphs(b);
  cudaFree(b->pop_alloc);
  cudaFree(b->flags);
  cudaFree(b->dirichlet);
  cudaFree(b->slice_omega);
  cudaFree(b->slice_omega_f);
  cudaFree(b->slice_src);
  cudaFree(b->slice_src_f);
  cudaFree(b->mom);
  cudaFree(b->partials);
  cudaFree(b->out);
  cudaFree(b->f64);
  cudaFree(b->bnd_list);
  cudaFree(b->link_src);
  cudaFree(b->link_dst);
  cudaFree(b->corr_src);
  cudaFree(b->corr_dst);
  cudaFree(b->d_err);
  delete b;
}

// time one even+odd pair at a given block size (for the autotuner): the
// fastest of three pairs after two warm-up pairs
float time_pair(BoxState* b, int tpb, cudaStream_t s) {
  const int keep = b->tuned_tpb;
  b->tuned_tpb   = tpb;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for(int k = 0; k < 2; ++k) {
    dispatch_step(b, false, 0, s);
    dispatch_step(b, true, 0, s);
  }
  float best = 1e30f;
  for(int k = 0; k < 3; ++k) {
    cudaEventRecord(e0, s);
    dispatch_step(b, false, 0, s);
    dispatch_step(b, true, 0, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->tuned_tpb = keep;
  return best;
}

// time the even and the odd step separately: the fastest of four of each,
// after two warm-up pairs
void time_parities(BoxState* b, cudaStream_t s, float* even_ms, float* odd_ms) {
  cudaEvent_t ev[3];
  for(auto& e : ev) cudaEventCreate(&e);
  for(int k = 0; k < 2; ++k) {
    dispatch_step(b, false, 0, s);
    dispatch_step(b, true, 0, s);
  }
  float te = 1e30f, to = 1e30f;
  for(int k = 0; k < 4; ++k) {
    cudaEventRecord(ev[0], s);
    dispatch_step(b, false, 0, s);
    cudaEventRecord(ev[1], s);
    dispatch_step(b, true, 0, s);
    cudaEventRecord(ev[2], s);
    cudaEventSynchronize(ev[2]);
    float a = 0, c = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&c, ev[1], ev[2]);
    te = std::min(te, a);
    to = std::min(to, c);
  }
  for(auto& e : ev) cudaEventDestroy(e);
  *even_ms = te;
  *odd_ms  = to;
}

}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_gpu_box_storage_bytes(int32_t storage) {
  switch(storage) {
    case LBM_STORE_F64: return 8;
    case LBM_STORE_F32: return 4;
    case LBM_STORE_F16_DEV:
    case LBM_STORE_BF16_DEV:
    case LBM_STORE_E3M12_DEV: return 2;
    default: return 0;
  }
}

int lbm_gpu_create_box(const lbm_box_desc* desc, const uint8_t* flags, const double* dirichlet, lbm_gpu_ctx** out) {
  if(!desc || !out) return LBM_ERR_INVALID;
  *out = nullptr;
  const int lat = desc->lattice, eq = desc->equation, st = desc->storage;
  const bool ok = ((lat == LBM_D2Q9 || lat == LBM_D3Q19) && eq == LBM_NAVIER_STOKES && st >= 0 && st <= LBM_STORE_E3M12_DEV) ||
                  (lat == LBM_D3Q7 && eq == LBM_POISSON && (st == LBM_STORE_F64 || st == LBM_STORE_F32));
  if(!ok) return LBM_ERR_UNSUPPORTED;
  const int D = lat == LBM_D2Q9 ? 2 : 3;
  if(desc->nx < 2 || desc->ny < 2 || (D == 3 && desc->nz < 2) || desc->nz < 1) return LBM_ERR_INVALID;
  if(desc->ny > 65535 || desc->nz > 65535) return LBM_ERR_INVALID;
  if(!(desc->omega > 0.0 && desc->omega < 2.0)) return LBM_ERR_INVALID;
  for(int a = 0; a < D; ++a) {
    const bool p0 = desc->face[2 * a] == LBM_FACE_PERIODIC, p1 = desc->face[2 * a + 1] == LBM_FACE_PERIODIC;
    if(p0 != p1) return LBM_ERR_INVALID;
    for(int sd = 0; sd < 2; ++sd) {
      const int ft = desc->face[2 * a + sd];
      if(ft < 0 || ft > 3) return LBM_ERR_INVALID;
      if(ft == LBM_FACE_OPEN && a != 0) return LBM_ERR_UNSUPPORTED;  // open faces are the x inlet / outlet planes
    }
  }
  const int64_t ncells = static_cast<int64_t>(desc->nx) * desc->ny * desc->nz;
  std::vector<uint8_t> hflags(ncells, LBM_CELL_FLUID);
  if(flags) std::copy(flags, flags + ncells, hflags.begin());
  bool has_outlet = false, has_inlet = false;
  for(int64_t i = 0; i < ncells; ++i) {
    const uint8_t t = hflags[i];
    if(t > LBM_CELL_DIRICHLET) return LBM_ERR_INVALID;
    if(t == LBM_CELL_INLET) has_inlet = true;
    const int x = static_cast<int>(i % desc->nx);
    if(t == LBM_CELL_OUTLET) {
      if(x != desc->nx - 1 || desc->face[1] != LBM_FACE_OPEN) return LBM_ERR_INVALID;
      has_outlet = true;
    }
    if(t == LBM_CELL_DIRICHLET && (eq != LBM_POISSON || !dirichlet)) return LBM_ERR_INVALID;
    if(t == LBM_CELL_INLET && eq != LBM_NAVIER_STOKES) return LBM_ERR_INVALID;
    // a cell on an open face must emit (inlet) or be an outlet / solid
    if(x == 0 && desc->face[0] == LBM_FACE_OPEN && t != LBM_CELL_INLET && t != LBM_CELL_SOLID && t != LBM_CELL_DIRICHLET) return LBM_ERR_INVALID;
    if(x == desc->nx - 1 && desc->face[1] == LBM_FACE_OPEN && t != LBM_CELL_OUTLET && t != LBM_CELL_SOLID && t != LBM_CELL_INLET &&
       t != LBM_CELL_DIRICHLET)
      return LBM_ERR_INVALID;
  }
  if(cudaSetDevice(desc->device) != cudaSuccess) return LBM_ERR_CUDA;

  BoxState* b = new(std::nothrow) BoxState();
  if(!b) return LBM_ERR_NOMEM;
  b->desc = *desc;
  b->D    = D;
  b->Q    = lat == LBM_D2Q9 ? 9 : (lat == LBM_D3Q19 ? 19 : 7);
  b->nvar = eq == LBM_NAVIER_STOKES ? D + 1 : 1;
  b->elem = static_cast<size_t>(lbm_gpu_box_storage_bytes(st));
  BoxParams& p = b->p;
  p.nx = desc->nx;
  p.ny = desc->ny;
  p.nz = desc->nz;
  p.ncells = ncells;
  // plane size rounded to 128 cells so every plane starts 256-byte aligned;
  // the outlet ghost (Q x ny x nz values) is appended as plane Q
  const int64_t ghost = static_cast<int64_t>(b->Q) * desc->ny * desc->nz;
  p.nalloc = (std::max(ncells, ghost) + 127) / 128 * 128;
  if(p.nalloc * (b->Q + 1) >= (int64_t(1) << 31)) {
    delete b;
    return LBM_ERR_UNSUPPORTED;  // the step kernels index populations with 32-bit offsets
  }
  for(int i = 0; i < 6; ++i) {
    p.face[i] = desc->face[i];
    for(int d = 0; d < 3; ++d) p.wall_u[i][d] = desc->wall_velocity[i][d];
  }
  p.omega = desc->omega;
  p.has_force = 0;
  for(int d = 0; d < 3; ++d) {
    p.force[d]   = desc->body_force[d];
    p.inlet_u[d] = desc->inlet_velocity[d];
    if(desc->body_force[d] != 0.0) p.has_force = 1;
  }
  p.inlet_rho  = desc->inlet_density;
  p.kappa_sq   = desc->kappa_sq;
  p.pb_nonlinear = desc->pb_nonlinear;
  // D = alpha (1/2 - tau) in lattice units (src/lbm/solver.cpp:606 with dt = 1)
  p.pb_diffusivity = Lattice<LBM_D3Q7>::poisson_alpha * (0.5 - 1.0 / desc->omega);
  p.has_outlet = has_outlet ? 1 : 0;
  p.mom_mode   = 0;
  p.omega_f     = static_cast<float>(p.omega);
  p.inlet_rho_f = static_cast<float>(p.inlet_rho);
  p.pb_src_f    = static_cast<float>(p.pb_diffusivity * p.kappa_sq);
  for(int d = 0; d < 3; ++d) {
    p.force_f[d]   = static_cast<float>(p.force[d]);
    p.inlet_u_f[d] = static_cast<float>(p.inlet_u[d]);
  }
  // the FP32 / FP16 / BF16 Navier-Stokes state is shifted to the free
  // stream: each population's scaled deviation minus that of the equilibrium
  // at rho = 1 and the free-stream velocity U (the inlet velocity where the
  // box has inlet cells, else the initial velocity), and the single-precision
  // collision works on that state (collide_ns_shifted).  Only a velocity along
  // x is used (U = 0 otherwise): every direction then has the same shift as
  // its reflection in a y or z face, so free-slip reflections keep the state,
  // and only bounce-back changes it (bounce_shift).
  p.shift_u   = 0.0f;
  p.shift_u_d = 0.0;
  if(eq == LBM_NAVIER_STOKES && st != LBM_STORE_F64 && !desc->no_shift) {
    const double* uref = has_inlet ? desc->inlet_velocity : desc->init_velocity;
    p.shift_u          = (uref[1] == 0.0 && uref[2] == 0.0) ? static_cast<float>(uref[0]) : 0.0f;
    p.shift_u_d        = p.shift_u;  // the arithmetic's U, exactly
  }

  // one guard plane in front: the odd step issues its pull loads before it
  // knows whether the cell steps at all, and a boundary cell's pull address
  // may lie up to nx*ny + nx + 1 cells before plane 0 (behind the last plane
  // lies the ghost plane)
  cudaError_t e = cudaMalloc(&b->pop_alloc, b->elem * static_cast<size_t>(p.nalloc) * (b->Q + 2));
  if(e == cudaSuccess) e = cudaMemset(b->pop_alloc, 0, b->elem * static_cast<size_t>(p.nalloc) * (b->Q + 2));
  b->pop = static_cast<char*>(b->pop_alloc) + b->elem * static_cast<size_t>(p.nalloc);
  // engine bit: a stencil neighbour is solid; and the compact list of cells the
  // odd step must resolve link by link (next to a face or a solid, or not fluid)
  {
    const int nx = desc->nx, ny = desc->ny, nz = desc->nz;
    std::vector<int32_t> list, xlist;
    for(int64_t i = 0; i < ncells; ++i) {
      const int x = static_cast<int>(i % nx), y = static_cast<int>((i / nx) % ny), z = static_cast<int>(i / (static_cast<int64_t>(nx) * ny));
      if(hflags[i] == LBM_CELL_SOLID) continue;
      bool near = false;
      for(int dz = (D > 2 ? -1 : 0); dz <= (D > 2 ? 1 : 0) && !near; ++dz)
        for(int dy = -1; dy <= 1 && !near; ++dy)
          for(int dx = -1; dx <= 1 && !near; ++dx) {
            if(std::abs(dx) + std::abs(dy) + std::abs(dz) > (lat == LBM_D3Q7 ? 1 : 2)) continue;
            const int xx = x + dx, yy = y + dy, zz = z + dz;
            if(xx < 0 || yy < 0 || zz < 0 || xx >= nx || yy >= ny || zz >= nz) continue;
            if(hflags[xx + static_cast<int64_t>(nx) * (yy + static_cast<int64_t>(ny) * zz)] == LBM_CELL_SOLID) near = true;
          }
      const bool inside_yz = y > 0 && y < ny - 1 && (D < 3 || (z > 0 && z < nz - 1));
      const bool inside    = x > 0 && x < nx - 1 && inside_yz;
      const bool xface     = !near && inside_yz && nx >= 3 &&
                         ((x == 0 && hflags[i] == LBM_CELL_INLET && desc->face[0] == LBM_FACE_OPEN) ||
                          (x == nx - 1 && hflags[i] == LBM_CELL_OUTLET && desc->face[1] == LBM_FACE_OPEN));
      if(xface) {
        xlist.push_back(static_cast<int32_t>(i));
        hflags[i] = static_cast<uint8_t>(hflags[i] | XFACE);
        continue;
      }
      // a fluid cell on exactly one free-slip y / z face, off the x faces:
      // every link source and destination it reflects to is a non-solid cell
      // of the box (the cell has no solid stencil neighbour)
      const bool on_y  = D > 1 && ny >= 3 && (y == 0 || y == ny - 1);
      const bool on_z  = D > 2 && nz >= 3 && (z == 0 || z == nz - 1);
      const bool yz_ok = D > 2 ? (y > 0 && y < ny - 1) || (z > 0 && z < nz - 1) : true;
      const int  sface = on_y && !on_z ? (y == 0 ? 2 : 3) : (on_z && !on_y ? (z == 0 ? 4 : 5) : -1);
      if(!near && hflags[i] == LBM_CELL_FLUID && nx >= 3 && x > 0 && x < nx - 1 && yz_ok && sface >= 0 &&
         desc->face[sface] == LBM_FACE_FREESLIP) {
        xlist.push_back(static_cast<int32_t>(i));
        hflags[i] = static_cast<uint8_t>(hflags[i] | SFACE);
        ++b->n_sface;
        continue;
      }
      if(near || !inside || hflags[i] != LBM_CELL_FLUID) list.push_back(static_cast<int32_t>(i));
      if(near || !inside) hflags[i] = static_cast<uint8_t>(hflags[i] | LINKED);
    }
    b->n_bnd_lean = static_cast<int64_t>(list.size());
    // face positions the face blocks walk: every SFACE cell lies among them
    if(nx >= 3 && ny >= 3 && (D < 3 || nz >= 3) && D > 1) {
      b->face_ny_part = 2 * static_cast<int64_t>(nx - 2) * (D > 2 ? nz - 2 : nz);
      b->face_n       = b->face_ny_part + (D > 2 ? 2 * static_cast<int64_t>(nx - 2) * (ny - 2) : 0);
    }
    list.insert(list.end(), xlist.begin(), xlist.end());
    b->n_bnd = static_cast<int64_t>(list.size());
    if(e == cudaSuccess) e = cudaMalloc(&b->bnd_list, sizeof(int32_t) * std::max<size_t>(1, list.size()));
    if(e == cudaSuccess && !list.empty())
      e = cudaMemcpy(b->bnd_list, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice);
  }
  if(e == cudaSuccess) e = cudaMalloc(&b->flags, ncells);
  if(e == cudaSuccess) e = cudaMemcpy(b->flags, hflags.data(), ncells, cudaMemcpyHostToDevice);
  if(e == cudaSuccess && dirichlet) {
    e = cudaMalloc(&b->dirichlet, sizeof(double) * ncells);
    if(e == cudaSuccess) e = cudaMemcpy(b->dirichlet, dirichlet, sizeof(double) * ncells, cudaMemcpyHostToDevice);
  }
  const size_t csize = st == LBM_STORE_F64 ? 8 : 4;
  if(e == cudaSuccess) e = cudaMalloc(&b->mom, csize * b->nvar * ncells);
  if(e == cudaSuccess) e = cudaMemset(b->mom, 0, csize * b->nvar * ncells);
  // partials for the largest launch (smallest block size considered by the tuner)
  // residual slots: one per warp of the largest launch over the tuner's block sizes
  int64_t maxrow = 0;
  for(int t : kTunerBlocks) maxrow = std::max<int64_t>(maxrow, static_cast<int64_t>((desc->nx + t - 1) / t) * (t / 32));
  const int64_t maxblocks = maxrow * desc->ny * desc->nz + static_cast<int64_t>((b->n_bnd + 127) / 128 + (b->face_n + 127) / 128) * 4;
  if(e == cudaSuccess) e = cudaMalloc(&b->partials, sizeof(double) * (maxblocks * 4 + 304 * 4 + kMidBlocks * 4));
  b->partials_mm      = b->partials + maxblocks * 4;
  b->partials_mid     = b->partials_mm + 304 * 4;
  p.partial_stride    = maxblocks;
  if(e == cudaSuccess) e = cudaMalloc(&b->out, sizeof(double) * 8);
  if(e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(int));
  if(e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(int));
  p.flags     = b->flags;
  p.dirichlet = b->dirichlet;
  p.pop       = b->pop;
  p.mom       = b->mom;
  p.partials  = b->partials;
  bool moving = false;
  for(int i = 0; i < 6; ++i)
    for(int d = 0; d < 3; ++d)
      if(desc->wall_velocity[i][d] != 0.0 && desc->face[i] == LBM_FACE_WALL) moving = true;
  if(p.shift_u != 0.0f) moving = true;  // shifted state: bounced populations change shift
  if(e == cudaSuccess && b->n_bnd > 0) {
    const size_t nl = static_cast<size_t>(b->n_bnd) * b->Q;
    e = cudaMalloc(&b->link_src, sizeof(int32_t) * nl);
    if(e == cudaSuccess) e = cudaMalloc(&b->link_dst, sizeof(int32_t) * nl);
    if(e == cudaSuccess && moving) e = cudaMalloc(&b->corr_src, sizeof(double) * nl);
    if(e == cudaSuccess && moving) e = cudaMalloc(&b->corr_dst, sizeof(double) * nl);
    if(e == cudaSuccess) {
      const unsigned g = static_cast<unsigned>((b->n_bnd + 127) / 128);
      const int      n = static_cast<int>(b->n_bnd);
      switch(lat) {
        case LBM_D2Q9: k_box_build_links<LBM_D2Q9><<<g, 128>>>(p, b->bnd_list, n, b->link_src, b->link_dst, b->corr_src, b->corr_dst); break;
        case LBM_D3Q19: k_box_build_links<LBM_D3Q19><<<g, 128>>>(p, b->bnd_list, n, b->link_src, b->link_dst, b->corr_src, b->corr_dst); break;
        default: k_box_build_links<LBM_D3Q7><<<g, 128>>>(p, b->bnd_list, n, b->link_src, b->link_dst, b->corr_src, b->corr_dst); break;
      }
      e = cudaDeviceSynchronize();
    }
  }
  cudaStream_t stream = nullptr;
  if(e == cudaSuccess) e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  if(e != cudaSuccess) {
    box_destroy(b);
    return e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
  }
  // autotune the block size on the (not yet initialised) state
  {
    float best = 1e30f;
    for(int tpb : kTunerBlocks) {
      if(tpb > 2 * desc->nx && tpb > 64) continue;
      const float ms = time_pair(b, tpb, stream);
      if(ms < best) {
        best         = ms;
        b->tuned_tpb = tpb;
      }
    }
    // then every bulk kernel the box allows, timed per step parity: the even
    // (local) and odd (streaming) steps may each take a different one
    float best_even = 1e30f, best_odd = 1e30f;
    int   pick_even = LBM_BOX_KERNEL_THREAD, pick_odd = LBM_BOX_KERNEL_THREAD;
    for(int kind : {LBM_BOX_KERNEL_THREAD, LBM_BOX_KERNEL_STAGED, LBM_BOX_KERNEL_PAIRED, LBM_BOX_KERNEL_ROWS}) {
      if(!box_kernel_supported(b, kind)) continue;
      b->kind_even = b->kind_odd = kind;
      float       ev = 0, od = 0;
      time_parities(b, stream, &ev, &od);
      int         flag = 0;
      cudaMemcpy(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost);
      cudaMemset(b->d_err, 0, sizeof(int));
      if(flag) continue;
      if(ev < best_even) {
        best_even = ev;
        pick_even = kind;
      }
      if(od < best_odd) {
        best_odd = od;
        pick_odd = kind;
      }
    }
    // the mixed pick only stands if whole step pairs confirm it against the
    // best single kernel (the parities share the caches and the memory system)
    if(pick_even != pick_odd) {
      float best_pair = 1e30f;
      int   pe = pick_even, po = pick_odd;
      for(int kind : {LBM_BOX_KERNEL_THREAD, LBM_BOX_KERNEL_STAGED, LBM_BOX_KERNEL_PAIRED, LBM_BOX_KERNEL_ROWS}) {
        if(!box_kernel_supported(b, kind)) continue;
        b->kind_even = b->kind_odd = kind;
        const float ms = time_pair(b, b->tuned_tpb, stream);
        if(ms < best_pair) {
          best_pair = ms;
          pe = po = kind;
        }
      }
      b->kind_even = pick_even;
      b->kind_odd  = pick_odd;
      if(time_pair(b, b->tuned_tpb, stream) < 0.97f * best_pair) {  // a clear margin, or one kernel for both
        pe = pick_even;
        po = pick_odd;
      }
      pick_even = pe;
      pick_odd  = po;
    }
    b->kind_even = pick_even;
    b->kind_odd  = pick_odd;
    cudaMemsetAsync(b->pop, 0, b->elem * static_cast<size_t>(p.nalloc) * (b->Q + 1), stream);
    if(cudaStreamSynchronize(stream) != cudaSuccess) {
      cudaStreamDestroy(stream);
      box_destroy(b);
      return LBM_ERR_CUDA;
    }
  }
  lbm_gpu_ctx* ctx = lbm_internal_new_box_ctx(desc->device, b, stream);
  if(!ctx) {
    cudaStreamDestroy(stream);
    box_destroy(b);
    return LBM_ERR_NOMEM;
  }
  *out = ctx;
  return LBM_OK;
}

int lbm_gpu_box_moments(lbm_gpu_ctx* ctx, double* rho, double* ux, double* uy, double* uz) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b) return LBM_ERR_INVALID;
  cudaStream_t s = lbm_internal_stream(ctx);
  std::string  err;
  if(!ensure_staging(b)) return LBM_ERR_NOMEM;
  const int64_t N = b->p.ncells;
  double*       d = nullptr;
  cudaError_t   e = cudaMalloc(&d, sizeof(double) * N * 4);
  if(e == cudaSuccess) e = dispatch_readout(b, b->f64, s);
  if(e == cudaSuccess) {
    const unsigned g = static_cast<unsigned>((N + 255) / 256);
    switch(b->desc.lattice * 2 + b->desc.equation) {
      case LBM_D2Q9 * 2: k_box_moments_f64<LBM_D2Q9, 0><<<g, 256, 0, s>>>(b->p, b->f64, d, d + N, d + 2 * N, nullptr); break;
      case LBM_D3Q19 * 2: k_box_moments_f64<LBM_D3Q19, 0><<<g, 256, 0, s>>>(b->p, b->f64, d, d + N, d + 2 * N, d + 3 * N); break;
      default: k_box_moments_f64<LBM_D3Q7, 1><<<g, 256, 0, s>>>(b->p, b->f64, d, nullptr, nullptr, nullptr); break;
    }
    e = cudaGetLastError();
  }
  double* outs[4] = {rho, ux, uy, uz};
  for(int k = 0; k < 4 && e == cudaSuccess; ++k) {
    if(!outs[k]) continue;
    if(k > 0 && (b->desc.equation != LBM_NAVIER_STOKES || k > b->D)) continue;
    e = cudaMemcpyAsync(outs[k], d + k * N, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
  }
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if(e != cudaSuccess) {
    lbm_internal_set_error(ctx, std::string("box moments: ") + cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  return LBM_OK;
}

int lbm_gpu_box_probe(lbm_gpu_ctx* ctx, const int64_t* cells, int64_t n, double* out) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b || n < 0 || (n > 0 && (!cells || !out))) return LBM_ERR_INVALID;
  if(n == 0) return LBM_OK;
  for(int64_t i = 0; i < n; ++i)
    if(cells[i] < 0 || cells[i] >= b->p.ncells) {
      lbm_internal_set_error(ctx, "box probe: cell index out of range");
      return LBM_ERR_INVALID;
    }
  cudaStream_t s  = lbm_internal_stream(ctx);
  int64_t*     dc = nullptr;
  double*      dm = nullptr;
  cudaError_t  e  = cudaMalloc(&dc, sizeof(int64_t) * n);
  if(e == cudaSuccess) e = cudaMalloc(&dm, sizeof(double) * n * b->nvar);
  if(e == cudaSuccess) e = cudaMemcpyAsync(dc, cells, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
  if(e == cudaSuccess) e = dispatch_probe(b, dc, n, dm, s);
  if(e == cudaSuccess) e = cudaMemcpyAsync(out, dm, sizeof(double) * n * b->nvar, cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dc);
  cudaFree(dm);
  if(e != cudaSuccess) {
    lbm_internal_set_error(ctx, std::string("box probe: ") + cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  return LBM_OK;
}

int lbm_gpu_box_time_steps(lbm_gpu_ctx* ctx, int64_t nsteps, double* ms) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b || nsteps < 0 || !ms) return LBM_ERR_INVALID;
  cudaStream_t s = lbm_internal_stream(ctx);
  cudaEvent_t  ev[2];
  cudaEventCreate(&ev[0]);
  cudaEventCreate(&ev[1]);
  cudaEventRecord(ev[0], s);
  std::string err;
  int         rc = box_step_enqueue(b, nsteps, s, err);
  cudaEventRecord(ev[1], s);
  cudaError_t e = cudaEventSynchronize(ev[1]);
  float       t = 0;
  if(e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if(rc == LBM_OK && e != cudaSuccess) rc = cerr(err, e, "time steps");
  if(rc == LBM_OK) rc = check_wait_flag(b, err);
  if(rc != LBM_OK) {
    lbm_internal_set_error(ctx, err);
    return rc;
  }
  *ms = t;
  return LBM_OK;
}

int lbm_gpu_box_profile_steps(lbm_gpu_ctx* ctx, int64_t nsteps, double* total_ms, double* kernel_ms, int64_t* launches) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b || nsteps < 0) return LBM_ERR_INVALID;
  cudaStream_t             s = lbm_internal_stream(ctx);
  std::vector<cudaEvent_t> ev(2 * nsteps + 2);
  for(auto& e : ev) cudaEventCreate(&e);
  cudaEventRecord(ev[0], s);
  cudaError_t e = cudaSuccess;
  for(int64_t k = 0; k < nsteps && e == cudaSuccess; ++k) {
    // same moment bookkeeping as box_step: the last two steps record the residual
    int mom = 0;
    if(nsteps >= 2 && k >= nsteps - 2) mom = b->mom_valid ? 2 : 1;
    if(nsteps < 2) mom = b->mom_valid ? 2 : 1;
    e = dispatch_step(b, (b->steps & 1) != 0, mom, s, ev[2 + 2 * k], ev[3 + 2 * k]);
    ++b->steps;
    b->mom_valid = mom != 0;
    b->res_ready = mom == 2;
  }
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
  if(e != cudaSuccess) {
    lbm_internal_set_error(ctx, std::string("profile steps: ") + cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  std::string werr;
  if(check_wait_flag(b, werr) != LBM_OK) {
    lbm_internal_set_error(ctx, werr);
    return LBM_ERR_CUDA;
  }
  if(total_ms) *total_ms = tot;
  if(kernel_ms) *kernel_ms = ker;
  if(launches) *launches = nsteps;
  return LBM_OK;
}

int lbm_gpu_box_autotune(lbm_gpu_ctx* ctx, int32_t* threads_per_block) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b) return LBM_ERR_INVALID;
  if(threads_per_block) *threads_per_block = b->tuned_tpb;
  return LBM_OK;
}

int lbm_gpu_box_select_kernel(lbm_gpu_ctx* ctx, int32_t kernel, int32_t* selected) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b || kernel > LBM_BOX_KERNEL_ROWS) return LBM_ERR_INVALID;
  if(kernel >= 0 && !box_kernel_supported(b, kernel)) {
    lbm_internal_set_error(ctx, kernel == LBM_BOX_KERNEL_STAGED ? "box does not qualify for the staged kernel (rows must be 16-byte multiples)"
                                : kernel == LBM_BOX_KERNEL_ROWS ? "box does not qualify for the row-staged kernel (rows of 16-byte multiples, "
                                                                  "at most 1024 cells, stages within shared memory)"
                                                                : "box does not qualify for the paired kernel (nx even, FP32/FP16/BF16 storage)");
    return LBM_ERR_UNSUPPORTED;
  }
  if(kernel >= 0 && (kernel != b->kind_even || kernel != b->kind_odd)) {
    cudaStreamSynchronize(lbm_internal_stream(ctx));
    drop_graphs(b);
    b->kind_even = b->kind_odd = kernel;
  }
  if(selected) *selected = b->kind_even == b->kind_odd ? b->kind_even : -1;
  return LBM_OK;
}

int lbm_gpu_box_test_wait(lbm_gpu_ctx* ctx, int64_t limit_ns, int32_t starve) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b || limit_ns <= 0 || limit_ns > 500000000 || (starve != 0 && starve != 1)) return LBM_ERR_INVALID;
  cudaStreamSynchronize(lbm_internal_stream(ctx));
  drop_graphs(b);  // the graphs hold the old launch parameters
  b->wait_limit_ns = static_cast<uint64_t>(limit_ns);
  b->wait_starve   = starve;
  return LBM_OK;
}

int lbm_gpu_box_set_slice_omega(lbm_gpu_ctx* ctx, const double* omega, int32_t n) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b) return LBM_ERR_INVALID;
  if(b->desc.equation != LBM_NAVIER_STOKES) return LBM_ERR_UNSUPPORTED;
  cudaStream_t s = lbm_internal_stream(ctx);
  if(cudaStreamSynchronize(s) != cudaSuccess) return LBM_ERR_CUDA;
  if(!omega) {
    drop_graphs(b);  // the graphs hold the old launch parameters
    b->p.slice_omega   = nullptr;
    b->p.slice_omega_f = nullptr;
    return LBM_OK;
  }
  if(n != b->p.nz) return LBM_ERR_INVALID;
  std::vector<float> of(n);
  for(int z = 0; z < n; ++z) {
    if(!(omega[z] > 0.0 && omega[z] < 2.0)) return LBM_ERR_INVALID;
    of[z] = static_cast<float>(omega[z]);
  }
  if(!b->slice_omega) {
    if(cudaMalloc(&b->slice_omega, sizeof(double) * n) != cudaSuccess) return LBM_ERR_NOMEM;
    if(cudaMalloc(&b->slice_omega_f, sizeof(float) * n) != cudaSuccess) return LBM_ERR_NOMEM;
  }
  if(cudaMemcpy(b->slice_omega, omega, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
     cudaMemcpy(b->slice_omega_f, of.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    return LBM_ERR_CUDA;
  drop_graphs(b);
  b->p.slice_omega   = b->slice_omega;
  b->p.slice_omega_f = b->slice_omega_f;
  return LBM_OK;
}

int lbm_gpu_box_set_slice_kappa(lbm_gpu_ctx* ctx, const double* kappa_sq, int32_t n) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b) return LBM_ERR_INVALID;
  if(b->desc.equation != LBM_POISSON) return LBM_ERR_UNSUPPORTED;
  cudaStream_t s = lbm_internal_stream(ctx);
  if(cudaStreamSynchronize(s) != cudaSuccess) return LBM_ERR_CUDA;
  if(!kappa_sq) {
    drop_graphs(b);  // the graphs hold the old launch parameters
    b->p.slice_src   = nullptr;
    b->p.slice_src_f = nullptr;
    return LBM_OK;
  }
  if(n != b->p.nz) return LBM_ERR_INVALID;
  // the same products the single-coefficient box forms (pb_diffusivity * kappa_sq)
  std::vector<double> src(n);
  std::vector<float>  srcf(n);
  for(int z = 0; z < n; ++z) {
    if(!(kappa_sq[z] >= 0.0 && std::isfinite(kappa_sq[z]))) return LBM_ERR_INVALID;
    src[z]  = b->p.pb_diffusivity * kappa_sq[z];
    srcf[z] = static_cast<float>(src[z]);
  }
  if(!b->slice_src) {
    if(cudaMalloc(&b->slice_src, sizeof(double) * n) != cudaSuccess) return LBM_ERR_NOMEM;
    if(cudaMalloc(&b->slice_src_f, sizeof(float) * n) != cudaSuccess) return LBM_ERR_NOMEM;
  }
  if(cudaMemcpy(b->slice_src, src.data(), sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
     cudaMemcpy(b->slice_src_f, srcf.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    return LBM_ERR_CUDA;
  drop_graphs(b);
  b->p.slice_src   = b->slice_src;
  b->p.slice_src_f = b->slice_src_f;
  return LBM_OK;
}

int lbm_gpu_box_kernels(lbm_gpu_ctx* ctx, int32_t* even, int32_t* odd) {
  BoxState* b = lbm_internal_box(ctx);
  if(!b) return LBM_ERR_INVALID;
  if(even) *even = b->kind_even;
  if(odd) *odd = b->kind_odd;
  return LBM_OK;
}

}  // extern "C"
