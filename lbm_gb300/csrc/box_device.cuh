// Device helpers of the dense-box engine shared by its step kernels
// (box.cu: per-thread kernels; box_tma.cu: bulk-copy staged kernels): link
// resolution through the faces, collision dispatch, inlet / Dirichlet
// emission, and the residual bookkeeping of the moment-recording steps.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "box.h"
#include "lattice.cuh"
#include "step_common.cuh"

namespace lbm {

constexpr uint8_t TYPE_MASK  = 0x07;
constexpr uint8_t LINKED     = 0x08;  // set by the engine: the odd step resolves this cell's links in the
                                     // boundary kernel (a solid neighbour, or a face of the box)
constexpr uint8_t XFACE      = 0x10;  // set by the engine: an inlet cell on an open -x face or an outlet
                                     // cell on an open +x face, away from solids and the other faces; the
                                     // per-thread odd step handles it in line (emit, or ghost pulls, and
                                     // no push through the face), the other bulk kernels leave it to the
                                     // boundary kernel
constexpr uint8_t SFACE      = 0x20;  // set by the engine: a fluid cell on exactly one free-slip y or z face,
                                     // away from solids and the x faces; the per-thread odd step pulls
                                     // and pushes its links through that face by specular reflection in
                                     // line, the other bulk kernels leave it to the boundary kernel
// ---- link resolution ---------------------------------------------------------
// direction q with its component along axis AX reversed (compile-time form of
// mirror() for one axis)
template <int LAT, int AX>
LBM_HD constexpr int mirror_axis(int q) {
  using L = Lattice<LAT>;
  for(int k = 0; k < L::Q; ++k) {
    bool same = true;
    for(int a = 0; a < 3; ++a)
      if(L::c(k, a) != (a == AX ? -L::c(q, a) : L::c(q, a))) same = false;
    if(same) return k;
  }
  return q;
}

// mirror of direction q in the axes of `mask` (free-slip reflection)
template <int LAT>
__device__ __forceinline__ int mirror(int q, int mask) {
  using L = Lattice<LAT>;
  int c[3] = {L::c(q, 0), L::c(q, 1), L::c(q, 2)};
#pragma unroll
  for(int a = 0; a < 3; ++a)
    if(mask & (1 << a)) c[a] = -c[a];
#pragma unroll
  for(int k = 0; k < L::Q; ++k)
    if(L::c(k, 0) == c[0] && L::c(k, 1) == c[1] && L::c(k, 2) == c[2]) return k;
  return q;
}

enum LinkKind { LINK_CELL = 0, LINK_BOUNCE = 1, LINK_OPEN = 2 };

struct Link {
  int     kind;
  int64_t cell;  // LINK_CELL: cell to read / write
  int     q;     // LINK_CELL: direction of the population at that cell
  double  corr;  // LINK_BOUNCE: moving-wall momentum added to the arriving population
};

// Resolve the cell reached from (x,y,z) by displacement sign*c_q, through
// the box faces.  sign=-1: source of the population arriving at (x,y,z) in
// direction q; sign=+1: destination of the population leaving it.
// `arrive` is the direction of the population that arrives at (x,y,z) when the
// link bounces back (q for the pull side, opp(q) for the push side).
template <int LAT>
__device__ __forceinline__ Link resolve(const BoxParams& P, int x, int y, int z, int q, int sign, int arrive) {
  using L       = Lattice<LAT>;
  const int n[3] = {P.nx, P.ny, P.nz};
  int       p[3] = {x, y, z};
  int       s[3];
  int       mask = 0;
  bool      bb = false, open = false;
  double    corr = 0.0;
#pragma unroll
  for(int a = 0; a < L::D; ++a) {
    s[a] = p[a] + sign * L::c(q, a);
    if(s[a] < 0 || s[a] >= n[a]) {
      const int face = s[a] < 0 ? 2 * a : 2 * a + 1;
      const int ft   = P.face[face];
      if(ft == LBM_FACE_PERIODIC) {
        s[a] = s[a] < 0 ? s[a] + n[a] : s[a] - n[a];
      } else if(ft == LBM_FACE_FREESLIP) {
        s[a] = p[a];
        mask |= 1 << a;
      } else if(ft == LBM_FACE_OPEN) {
        open = true;
      } else {
        bb = true;
        double cu = 0;
#pragma unroll
        for(int d = 0; d < L::D; ++d) cu += static_cast<double>(L::c(arrive, d)) * P.wall_u[face][d];
        // 2 w (c.u_w) / c_s^2 with rho_w = 1, in state units S (delta f) / w
        corr += 6.0 * STATE_SCALE * cu;
      }
    }
  }
#pragma unroll
  for(int a = L::D; a < 3; ++a) s[a] = p[a];  // a 2D lattice on a stack of slices keeps its slice
  if(open) return Link{LINK_OPEN, 0, q, 0.0};
  if(bb) return Link{LINK_BOUNCE, 0, q, corr};
  const int64_t cell = s[0] + static_cast<int64_t>(P.nx) * (s[1] + static_cast<int64_t>(P.ny) * s[2]);
  if((P.flags[cell] & TYPE_MASK) == LBM_CELL_SOLID) return Link{LINK_BOUNCE, 0, q, 0.0};
  return Link{LINK_CELL, cell, mask ? mirror<LAT>(q, mask) : q, 0.0};
}

// The shift of the FP32 / FP16 / BF16 Navier-Stokes state (s_q = v_q -
// S P_q(U), box.h), FP64: the shift of direction q, and K_opp(q) - K_q, the
// change of shift of a population bounced from direction q into opp(q).
template <int LAT>
__device__ __forceinline__ double state_shift(const BoxParams& P, int q) {
  const double U = P.shift_u_d, cu = Lattice<LAT>::c(q, 0) * U;
  return STATE_SCALE * (3.0 * cu + 4.5 * cu * cu - 1.5 * U * U);
}
template <int LAT>
__device__ __forceinline__ double bounce_shift(const BoxParams& P, int q) {
  return -6.0 * STATE_SCALE * Lattice<LAT>::c(q, 0) * P.shift_u_d;
}
// state of a box <-> population f (FP64), with the shift
template <int LAT, int EQ, int ST>
__device__ __forceinline__ double box_state_to_f(const BoxParams& P, double s, int q) {
  if constexpr(EQ == LBM_NAVIER_STOKES && ST != LBM_STORE_F64) s += state_shift<LAT>(P, q);
  return state_to_f<LAT, EQ>(s, q);
}
template <int LAT, int EQ, int ST>
__device__ __forceinline__ double box_f_to_state(const BoxParams& P, double f, int q) {
  double s = f_to_state<LAT, EQ>(f, q);
  if constexpr(EQ == LBM_NAVIER_STOKES && ST != LBM_STORE_F64) s -= state_shift<LAT>(P, q);
  return s;
}

template <int LAT>
__device__ __forceinline__ int64_t offset(const BoxParams& P, int q) {
  using L = Lattice<LAT>;
  return L::c(q, 0) + static_cast<int64_t>(P.nx) * (L::c(q, 1) + static_cast<int64_t>(P.ny) * L::c(q, 2));
}

template <int LAT>
__device__ __forceinline__ bool interior(const BoxParams& P, int x, int y, int z) {
  using L = Lattice<LAT>;
  bool in = x > 0 && x < P.nx - 1;
  if(L::D > 1) in = in && y > 0 && y < P.ny - 1;
  if(L::D > 2) in = in && z > 0 && z < P.nz - 1;
  return in;
}

// outlet ghost: value of direction q (c_qx = -1) for the outlet cell (y,z)
__device__ __forceinline__ int64_t ghost_index(const BoxParams& P, int q, int y, int z) {
  return static_cast<int64_t>(q) * P.ny * P.nz + y + static_cast<int64_t>(P.ny) * z;
}

// The collision of one cell of z-slice z.  FP64 arithmetic (FP64 storage)
// works on the scaled deviation v; FP32 arithmetic (the other storages) on
// the state shifted to the free stream (collide_ns_shifted, U = P.shift_u).
// The relaxation rate (Navier-Stokes) or the source coefficient (Poisson) is
// the slice's where the box has one per slice.
template <int LAT, int EQ, class C>
__device__ __forceinline__ void collide(const BoxParams& P, int z, C* v, C* mom_out) {
  if constexpr(EQ == LBM_NAVIER_STOKES) {
    C F[3];
    F[0] = prm<C>(P.force[0], P.force_f[0]);
    F[1] = prm<C>(P.force[1], P.force_f[1]);
    F[2] = prm<C>(P.force[2], P.force_f[2]);
    if constexpr(sizeof(C) == 4) {
      const float om = P.slice_omega_f ? P.slice_omega_f[z] : P.omega_f;
      if(P.has_force) collide_ns_shifted<LAT, true>(om, true, F, P.shift_u, v, mom_out);
      else collide_ns_shifted<LAT, false>(om, false, F, P.shift_u, v, mom_out);
    } else {
      const C om = P.slice_omega ? static_cast<C>(P.slice_omega[z]) : prm<C>(P.omega, P.omega_f);
      if(P.has_force) collide_ns<LAT, C, true>(om, true, F, v, mom_out);
      else collide_ns<LAT, C, false>(om, false, F, v, mom_out);
    }
  } else {
    const C src = P.slice_src ? prm<C>(P.slice_src[z], P.slice_src_f[z]) : prm<C>(P.pb_diffusivity * P.kappa_sq, P.pb_src_f);
    collide_poisson<LAT, C>(prm<C>(P.omega, P.omega_f), P.pb_nonlinear != 0, src, v, mom_out);
  }
}

// state emitted by inlet / Dirichlet cells
template <int LAT, int EQ, class C>
__device__ __forceinline__ void emit_equilibrium(const BoxParams& P, C* v, int64_t cell) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  if constexpr(EQ == LBM_NAVIER_STOKES && sizeof(C) == 4) {
    const float ui[3] = {P.inlet_u_f[0], P.inlet_u_f[1], P.inlet_u_f[2]};
    equilibrium_shifted<LAT>(P.inlet_rho_f, ui, P.shift_u, v);
  } else if constexpr(EQ == LBM_NAVIER_STOKES) {
    const C rho = prm<C>(P.inlet_rho, P.inlet_rho_f);
    C       ui[3];
    static_for<D>([&](auto dc) { ui[decltype(dc)::value] = prm<C>(P.inlet_u[decltype(dc)::value], P.inlet_u_f[decltype(dc)::value]); });
    C usq = 0;
    static_for<D>([&](auto dc) { usq += ui[decltype(dc)::value] * ui[decltype(dc)::value]; });
    static_for<Q>([&](auto qc) {
      constexpr int q  = decltype(qc)::value;
      C             cu = 0;
      static_for<D>([&](auto dc) {
        constexpr int d = decltype(dc)::value;
        cu += static_cast<C>(L::c(q, d)) * ui[d];
      });
      const C poly = C(3) * cu + C(4.5) * cu * cu - C(1.5) * usq;
      v[q]         = static_cast<C>(STATE_SCALE) * ((rho - C(1)) + rho * poly);
    });
  } else {
    const C phi = P.dirichlet ? static_cast<C>(P.dirichlet[cell]) : C(0);
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      v[q]            = q == Q - 1 ? static_cast<C>(L::w(Q - 1) - 1.0) * phi : static_cast<C>(L::w(q)) * phi;
    });
  }
}

// warp sum of the per-thread residual contributions into
// partials[k*stride + slot], one slot per warp.  The sum runs in the
// arithmetic type C (FP32 storages stay off the narrow FP64 pipe) and needs
// no barrier; every later level is FP64.  All 32 lanes must arrive.
template <int NV, class C>
__device__ __forceinline__ void warp_partials(const C* diff, double* partials, int64_t stride, int64_t slot) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for(int k = 0; k < NV; ++k) {
    const C s = warp_sum(diff[k]);
    if(lane == 0) partials[k * stride + slot] = static_cast<double>(s);
  }
}

// The previous moments are read at the top of the kernel (prefetch_moments),
// together with the populations, so the residual adds no second round trip
// to memory; moments_io writes the new ones and forms |new - previous|.
template <class C, int MOM, int NV>
__device__ __forceinline__ void prefetch_moments(const BoxParams& P, int64_t cell, C* prev) {
  if constexpr(MOM == 2) {
    const C* M = static_cast<const C*>(P.mom);
#pragma unroll
    for(int k = 0; k < NV; ++k) prev[k] = M[k * P.ncells + cell];
  }
}

template <int LAT, int EQ, class C, int MOM, int NV>
__device__ __forceinline__ void moments_io(const BoxParams& P, int64_t cell, const C* mom, const C* prev, C* diff) {
  if constexpr(MOM != 0) {
    C* M = static_cast<C*>(P.mom);
#pragma unroll
    for(int k = 0; k < NV; ++k) {
      if constexpr(MOM == 2) diff[k] = fabs(mom[k] - prev[k]);
      M[k * P.ncells + cell] = mom[k];
    }
  }
}

}  // namespace lbm
