// Reference-table engine: the SFCMM/LBM time step on the reference's own cell
// list (curve order) and neighbour table, FP64.
//
// One step is the reference's phase sequence (src/lbm/solver.cpp:306-320):
//   k_collide   currToOldVars + updateMacroscopicValues + calcEquilibriumMoments
//               + collisionStep fused in one pass over the cells;
//   k_force_*   pressure forcing (solver.cpp:625-696);
//   k_pre_*     LBMBndManager::preApply (bnd.h:48-53);
//   k_stream    propagationStep (solver.cpp:714-740), written as a pull over
//               the inverse neighbour table built once on the host;
//   k_bnd_*     LBMBndManager::apply (bnd.h:60-65), one kernel per loop of
//               each BC object, in the reference's order.
// Populations are q-major SoA (a[q*n+cell]) so every per-direction access of a
// warp is one coalesced transaction.  This translation unit is compiled with
// -fmad=false and every expression keeps the reference's operation order, so
// on the same inputs the engine returns the reference's doubles bit for bit.
#include <cuda_runtime.h>

#include "engine.h"
#include "lattice.cuh"

namespace lbm {
namespace {

constexpr int TPB = 256;
constexpr double EPS = 2.220446049250313080847e-16;  // GDoubleEps

struct View {
  int64_t n;
  double *fold, *f, *feq, *vars, *varsold;
  const int32_t* src;
  const int32_t* nbr;
  double omega, dt, diffusivity, poisson_k;
  int need_feq;
};

inline View view(const TableState& t) {
  return View{t.n, t.fold, t.f, t.feq, t.vars, t.varsold, t.src, t.nbr, t.omega, t.dt, t.diffusivity, t.poisson_k, t.need_feq ? 1 : 0};
}

inline unsigned blocks(int64_t n) { return static_cast<unsigned>((n + TPB - 1) / TPB); }

__device__ __forceinline__ int64_t gid() { return static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; }

// x / c for the equilibrium's constant divisors c = c_s^2, 2 c_s^4, 2 c_s^2,
// correctly rounded, from y = RN(1/c): q0 = x y, r = x - c q0 (one fused
// multiply-add, exact), q = RN(q0 + r y).  For these three constants
// |y c - 1| = 2^-54, so q0 is within half an ulp of x / c and thus one of the
// two doubles around it, and Markstein's theorem (P. Markstein, IBM J. Res.
// Dev. 34(1), 1990: y within half an ulp of 1/c, q0 within one ulp of x / c
// => RN(q0 + r y) = RN(x / c)) makes q the IEEE quotient.  A full FP64
// division costs several times the three FP64 operations on this part's
// narrow FP64 pipe, which bounds the collision kernel.  Zeros, infinities
// and NaNs (exponent field 0 or all ones, tested on the integer side) pass
// through as x y; the state never reaches subnormal magnitudes.  Checked
// against IEEE division on 60 million doubles (tests/test_const_div.py) and,
// through the engine, bit for bit against the reference's solver.
struct ConstDiv {
  double c, y;
};
constexpr ConstDiv DIV_CS2{CSSQ, 1.0 / CSSQ};
constexpr ConstDiv DIV_2CS4{2.0 * CSSQ * CSSQ, 1.0 / (2.0 * CSSQ * CSSQ)};
constexpr ConstDiv DIV_2CS2{2.0 * CSSQ, 1.0 / (2.0 * CSSQ)};

__device__ __forceinline__ double div_const(double x, ConstDiv d) {
  const double q = x * d.y;
  const int    e = (__double2hiint(q) >> 20) & 0x7ff;
  if(e == 0 || e == 0x7ff) return q;
  const double r = __fma_rn(-q, d.c, x);
  return __fma_rn(r, d.y, q);
}

// eq::defaultEq(w, rho, cu, vsq), src/lbm/equilibrium_func.h:52-54
__device__ __forceinline__ double eq_default(double w, double rho, double cu, double vsq) {
  return w * rho * (1.0 + div_const(cu, DIV_CS2) + div_const(cu * cu, DIV_2CS4) - div_const(vsq, DIV_2CS2));
}
// eq::symmEq, src/lbm/equilibrium_func.h:109-111
__device__ __forceinline__ double eq_symm(double w, double rho, double cu, double vsq) {
  return w * rho * (1.0 + div_const(cu * cu, DIV_2CS4) - div_const(vsq, DIV_2CS2));
}

template <int LAT>
__device__ __forceinline__ double eq_dist(int q, double rho, const double* u) {
  using L    = Lattice<LAT>;
  double vsq = 0;
#pragma unroll
  for(int d = 0; d < L::D; ++d) vsq += u[d] * u[d];
  double cu = 0;
#pragma unroll
  for(int d = 0; d < L::D; ++d) cu += u[d] * static_cast<double>(L::c(q, d));
  return eq_default(L::w(q), rho, cu, vsq);
}

template <int LAT>
__device__ __forceinline__ double symm_dist(int q, double rho, const double* u) {
  using L    = Lattice<LAT>;
  double vsq = 0;
#pragma unroll
  for(int d = 0; d < L::D; ++d) vsq += u[d] * u[d];
  double cu = 0;
#pragma unroll
  for(int d = 0; d < L::D; ++d) cu += u[d] * static_cast<double>(L::c(q, d));
  return eq_symm(L::w(q), rho, cu, vsq);
}

// inDirection (src/lbm/constants.h:83-86) of a surface normal and direction q
template <int LAT>
__device__ __forceinline__ bool in_direction(const double* nrm, int q) {
  using L  = Lattice<LAT>;
  double s = 0;
#pragma unroll
  for(int d = 0; d < L::D; ++d) s += nrm[d] * static_cast<double>(L::c(q, d));
  return s >= EPS;
}

// ---------------------------------------------------------------------------
// fused moments + equilibrium + BGK collision (+ Poisson source)
template <int LAT, int EQ>
__global__ void __launch_bounds__(TPB) k_collide(View v) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t c = gid();
  if(c >= v.n) return;
  const int64_t n = v.n;
  double        fo[Q];
#pragma unroll
  for(int q = 0; q < Q; ++q) fo[q] = v.fold[q * n + c];
  constexpr int NVAR = EQ == LBM_POISSON ? 1 : D + 1;
#pragma unroll
  for(int k = 0; k < NVAR; ++k) v.varsold[k * n + c] = v.vars[k * n + c];  // currToOldVars

  if constexpr(EQ == LBM_NAVIER_STOKES) {
    double rho = 0.0;
#pragma unroll
    for(int q = 0; q < Q; ++q) rho += fo[q];
    double u[D];
#pragma unroll
    for(int d = 0; d < D; ++d) {
      double ud = 0;
#pragma unroll
      for(int q = 0; q < Q - 1; ++q) ud += static_cast<double>(L::c(q, d)) * fo[q];
      ud /= rho;
      u[d] = ud;
      v.vars[d * n + c] = ud;
    }
    v.vars[D * n + c] = rho;
    double vsq        = 0;
#pragma unroll
    for(int d = 0; d < D; ++d) vsq += u[d] * u[d];
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      double cu = 0;
#pragma unroll
      for(int d = 0; d < D; ++d) cu += u[d] * static_cast<double>(L::c(q, d));
      const double feq = eq_default(L::w(q), rho, cu, vsq);
      if(v.need_feq) v.feq[q * n + c] = feq;
      v.f[q * n + c] = (1 - v.omega) * fo[q] + v.omega * feq;
    }
  } else {
    double acc = 0.0;
#pragma unroll
    for(int q = 0; q < Q - 1; ++q) acc += fo[q];
    const double phi = 1.0 / (1.0 - L::w(Q - 1)) * acc;
    v.vars[c]        = phi;
    const double rhs = v.poisson_k * v.poisson_k * phi;
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      const double feq = q == Q - 1 ? (L::w(Q - 1) - 1.0) * phi : L::w(q) * phi;
      if(v.need_feq) v.feq[q * n + c] = feq;
      double f = (1 - v.omega) * fo[q] + v.omega * feq;
      if(q != Q - 1) f += v.dt * v.diffusivity * L::pw(q) * rhs;
      v.f[q * n + c] = f;
    }
  }
}

// updateMacroscopicValues alone (src/lbm/solver.cpp:512-553)
template <int LAT, int EQ>
__global__ void __launch_bounds__(TPB) k_moments(View v) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t c = gid();
  if(c >= v.n) return;
  const int64_t n = v.n;
  if constexpr(EQ == LBM_NAVIER_STOKES) {
    double rho = 0.0;
#pragma unroll
    for(int q = 0; q < Q; ++q) rho += v.fold[q * n + c];
#pragma unroll
    for(int d = 0; d < D; ++d) {
      double ud = 0;
#pragma unroll
      for(int q = 0; q < Q - 1; ++q) ud += static_cast<double>(L::c(q, d)) * v.fold[q * n + c];
      ud /= rho;
      v.vars[d * n + c] = ud;
    }
    v.vars[D * n + c] = rho;
  } else {
    double acc = 0.0;
#pragma unroll
    for(int q = 0; q < Q - 1; ++q) acc += v.fold[q * n + c];
    v.vars[c] = 1.0 / (1.0 - L::w(Q - 1)) * acc;
  }
}

// propagationStep as a pull: fold[q][c] = f[q][src], missing links keep fold
template <int LAT>
__global__ void __launch_bounds__(TPB) k_stream(View v) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q;
  const int64_t c = gid();
  if(c >= v.n) return;
  const int64_t n = v.n;
#pragma unroll
  for(int q = 0; q < Q - 1; ++q) {
    const int32_t s = v.src[q * n + c];
    if(s >= 0) v.fold[q * n + c] = v.f[q * n + s];
  }
  v.fold[(Q - 1) * n + c] = v.f[(Q - 1) * n + c];
}

// pressure forcing pass: f[target] = eq(p, cu_x only) + f[val] - feq[val]
template <int LAT>
__global__ void k_force(View v, const int32_t* tgt, const int32_t* val, int64_t np, double pressure) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= np) return;
  const int64_t n = v.n;
  const int32_t t = tgt[i], s = val[i];
  double        u[D];
#pragma unroll
  for(int d = 0; d < D; ++d) u[d] = v.vars[d * n + s];
  double vsq = 0;
#pragma unroll
  for(int d = 0; d < D; ++d) vsq += u[d] * u[d];
#pragma unroll
  for(int q = 0; q < Q; ++q) {
    const double cu = u[0] * static_cast<double>(L::c(q, 0));
    v.f[q * n + t]  = eq_default(L::w(q), pressure, cu, vsq) + v.f[q * n + s] - v.feq[q * n + s];
  }
}

// ---- preApply ---------------------------------------------------------------
__global__ void k_pre_periodic_copy(View v, const int32_t* dst, const int32_t* qq, const int32_t* srcc, int64_t ncopy) {
  const int64_t i = gid();
  if(i >= ncopy) return;
  v.fold[qq[i] * v.n + dst[i]] = v.f[qq[i] * v.n + srcc[i]];
}
__global__ void k_set_var(View v, const int32_t* cells, int64_t m, int var, double value) {
  const int64_t i = gid();
  if(i >= m) return;
  v.vars[var * v.n + cells[i]] = value;
}
template <int LAT>
__global__ void k_pre_periodic_pressure(View v, const int32_t* mapped, const int32_t* link0, int64_t m, double p) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= m) return;
  const int64_t n = v.n;
  const int32_t a = mapped[i], l = link0[i];
  double        u[D];
#pragma unroll
  for(int d = 0; d < D; ++d) u[d] = v.vars[d * n + a];
#pragma unroll
  for(int q = 0; q < Q; ++q) v.fold[q * n + l] = eq_dist<LAT>(q, p, u) + v.f[q * n + a] - v.feq[q * n + a];
  v.vars[D * n + l] = p;
}

// ---- apply ------------------------------------------------------------------
// LBMBnd_DirichletBB::apply<VALZERO,SCALAR> (bnd_dirichlet.h:79-121) for the
// wall, moving-wall and Dirichlet-vector variants
template <int LAT, int EQ, int KIND>
__global__ void k_bnd_bb(View v, TableBnd b) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n    = v.n;
  const int32_t cell = b.cells[i];
  double        nrm[D];
#pragma unroll
  for(int d = 0; d < D; ++d) nrm[d] = b.normals[i * D + d];
#pragma unroll
  for(int q = 0; q < Q - 1; ++q) {
    if(v.nbr[q * n + cell] < 0 && in_direction<LAT>(nrm, q)) {
      const int opp = L::opp(q);
      double    val = v.f[q * n + cell];
      if constexpr(EQ == LBM_NAVIER_STOKES) {
        const double density = 1.0;
        if constexpr(KIND == LBM_BND_WALL_BB_TANGENTIAL) {
          val += density * 2.0 / CSSQ * L::w(opp) * b.tang[i * Q + opp];
        } else if constexpr(KIND == LBM_BND_DIRICHLET_BB) {
#pragma unroll
          for(int d = 0; d < D; ++d) val += density * 2.0 / CSSQ * L::w(opp) * static_cast<double>(L::c(opp, d)) * b.vec[d];
        }
      }
      v.fold[opp * n + cell] = val;
    }
  }
}

// calcDensity_limited (src/lbm/moments.h:119-153) for list entry `idx`
template <int LAT>
__device__ __forceinline__ void density_limited(View v, const TableBnd& b, int64_t idx, int32_t cell, bool noslip) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  if(b.lim_empty[idx]) return;
  const int64_t n   = v.n;
  double        rho = 0;
#pragma unroll
  for(int q = 0; q < Q; ++q) {
    const double k = b.lim_const[idx * Q + q];
    if(k != 0.0) rho += k * v.fold[q * n + cell];
  }
  if(!noslip) {
#pragma unroll
    for(int d = 0; d < D; ++d) {
      const double nd = b.normals[idx * D + d];
      if(nd > EPS) rho *= 1.0 / (1.0 + v.vars[d * n + cell]);
      else if(nd < 0) rho *= 1.0 / (1.0 - v.vars[d * n + cell]);
    }
  }
  v.vars[D * n + cell] = rho;
}

// LBMBnd_DirichletEQ::apply<VALZERO> (bnd_dirichlet.h:211-241), the first
// part of the equilibrium and NEEM walls
template <int LAT>
__global__ void k_bnd_wall_eq(View v, TableBnd b) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n       = v.n;
  const int32_t cell    = b.cells[i];
  const bool    valzero = !b.has_vec;
  double        u[D];
#pragma unroll
  for(int d = 0; d < D; ++d) {
    u[d]              = valzero ? 0.0 : b.vec[d];
    v.vars[d * n + cell] = u[d];
  }
  density_limited<LAT>(v, b, b.widx[i], cell, valzero);
  const double rho = v.vars[D * n + cell];
#pragma unroll
  for(int q = 0; q < Q; ++q) v.fold[q * n + cell] = valzero ? eq_default(L::w(q), rho, 0, 0) : eq_dist<LAT>(q, rho, u);
}

// LBMBnd_wallNEEM::apply_general (bnd_wall.h:275-297): moments of the
// extrapolation cells from the post-stream populations ...
template <int LAT>
__global__ void k_bnd_neem_ext(View v, const int32_t* extu, int64_t m) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= m) return;
  const int64_t n   = v.n;
  const int32_t e   = extu[i];
  double        rho = v.fold[e];
#pragma unroll
  for(int q = 1; q < Q; ++q) rho += v.fold[q * n + e];
  v.vars[D * n + e] = rho;
#pragma unroll
  for(int d = 0; d < D; ++d) {
    double ud = 0;
#pragma unroll
    for(int q = 0; q < Q - 1; ++q) ud += static_cast<double>(L::c(q, d)) * v.fold[q * n + e];
    ud /= rho;
    v.vars[d * n + e] = ud;
  }
}
// ... then the non-equilibrium part added to the wall cells
template <int LAT>
__global__ void k_bnd_neem_add(View v, TableBnd b) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n    = v.n;
  const int32_t cell = b.cells[i], e = b.ext[i];
  if(e < 0) return;
  double u[D];
#pragma unroll
  for(int d = 0; d < D; ++d) u[d] = v.vars[d * n + e];
  const double rho = v.vars[D * n + e];
#pragma unroll
  for(int q = 0; q < Q; ++q) v.fold[q * n + cell] += v.fold[q * n + e] - eq_dist<LAT>(q, rho, u);
}

// LBMBnd_wallNEBB::apply_0 / apply_constV (bnd_wall.h:358-471), D2Q9 only
__global__ void k_bnd_nebb(View v, TableBnd b) {
  using L         = Lattice<LBM_D2Q9>;
  constexpr int Q = 9, D = 2;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n    = v.n;
  const int32_t cell = b.cells[i];
  double*       fo   = v.fold;
#define FO(q) fo[(q) * n + cell]
  if(!b.has_vec) {
    v.vars[0 * n + cell] = 0;
    v.vars[1 * n + cell] = 0;
    density_limited<LBM_D2Q9>(v, b, i, cell, true);
    for(int dist = 0; dist < 2 * D; ++dist)
      if(v.nbr[dist * n + cell] < 0) FO(dist + 1 - 2 * (dist % 2)) = FO(dist);
    // the reference never advances its index in this loop: every cell uses
    // the normal of the first list entry
    const double n0 = b.normals[0], n1 = b.normals[1];
    if(n0 < 0) {
      FO(6) = FO(4) + 0.5 * (FO(3) - FO(2));
      FO(7) = FO(5) - 0.5 * (FO(3) - FO(2));
    } else if(n0 > 0) {
      FO(4) = FO(6) - 0.5 * (FO(3) - FO(2));
      FO(5) = FO(7) + 0.5 * (FO(3) - FO(2));
    } else if(n1 < 0) {
      FO(5) = FO(7) - 0.5 * (FO(1) - FO(0));
      FO(6) = FO(4) + 0.5 * (FO(1) - FO(0));
    } else if(n1 > 0) {
      FO(7) = FO(5) + 0.5 * (FO(1) - FO(0));
      FO(4) = FO(6) - 0.5 * (FO(1) - FO(0));
    }
  } else {
    const double* wv = b.vec;
    density_limited<LBM_D2Q9>(v, b, i, cell, false);
    v.vars[0 * n + cell] = wv[0];
    v.vars[1 * n + cell] = wv[1];
    const double n0 = b.normals[i * D + 0], n1 = b.normals[i * D + 1];
    const double nn[2] = {n0, n1};
    for(int dist = 0; dist < 2 * D; ++dist) {
      const int dir = dist / 2;
      if(v.nbr[dist * n + cell] < 0 && fabs(nn[dir]) > 0) {
        const int od = dist + 1 - 2 * (dist % 2);
        FO(od)       = FO(dist);
        if(nn[dir] < 0) FO(od) -= 2.0 / 3.0 * v.vars[2 * n + cell] * wv[dir];
        else FO(od) += 2.0 / 3.0 * v.vars[2 * n + cell] * wv[dir];
      }
    }
    const double rho = v.vars[2 * n + cell];
    if(n0 > 0) {
      FO(6) = FO(4) + 0.5 * (FO(3) - FO(2)) - 0.5 * rho * wv[1] - 1.0 / 6.0 * rho * wv[0];
      FO(7) = FO(5) - 0.5 * (FO(3) - FO(2)) + 0.5 * rho * wv[1] - 1.0 / 6.0 * rho * wv[0];
    } else if(n0 < 0) {
      FO(4) = FO(6) - 0.5 * (FO(3) - FO(2)) + 0.5 * rho * wv[1] + 1.0 / 6.0 * rho * wv[0];
      FO(5) = FO(7) + 0.5 * (FO(3) - FO(2)) - 0.5 * rho * wv[1] + 1.0 / 6.0 * rho * wv[0];
    } else if(n1 > 0) {
      FO(5) = FO(7) - 0.5 * (FO(1) - FO(0)) + 0.5 * rho * wv[0] - 1.0 / 6.0 * rho * wv[1];
      FO(6) = FO(4) + 0.5 * (FO(1) - FO(0)) - 0.5 * rho * wv[0] - 1.0 / 6.0 * rho * wv[1];
    } else if(n1 < 0) {
      FO(7) = FO(5) + 0.5 * (FO(1) - FO(0)) - 0.5 * rho * wv[0] + 1.0 / 6.0 * rho * wv[1];
      FO(4) = FO(6) - 0.5 * (FO(1) - FO(0)) + 0.5 * rho * wv[0] + 1.0 / 6.0 * rho * wv[1];
    }
  }
#undef FO
  (void)Q;
  (void)L::Q;
}

// LBMBnd_Pressure::apply, anti-bounce-back (bnd_pressure.h:271-322)
template <int LAT>
__global__ void k_bnd_pressure(View v, TableBnd b) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n    = v.n;
  const int32_t cell = b.cells[i], n1 = b.ext[i], n2 = b.ext2[i];
  const double  p    = b.scalar;
  double        u[D], nrm[D];
#pragma unroll
  for(int d = 0; d < D; ++d) {
    u[d]   = 1.5 * v.vars[d * n + n1] - 0.5 * v.vars[d * n + n2];
    nrm[d] = b.normals[i * D + d];
  }
  v.vars[D * n + cell] = p;
#pragma unroll
  for(int d = 0; d < D; ++d) v.vars[d * n + cell] = u[d];
#pragma unroll
  for(int q = 0; q < Q - 1; ++q) {
    if(v.nbr[q * n + cell] < 0 && in_direction<LAT>(nrm, q)) {
      v.fold[L::opp(q) * n + cell] = -v.f[q * n + cell] + 2 * symm_dist<LAT>(q, p, u);
    }
  }
}

// LBMBnd_DirichletNEEM::apply (bnd_dirichlet.h:354-373): potentials of the
// extrapolation cells ...
template <int LAT>
__global__ void k_bnd_potential(View v, const int32_t* cells, int64_t m) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q;
  const int64_t i = gid();
  if(i >= m) return;
  const int64_t n   = v.n;
  const int32_t e   = cells[i];
  double        acc = 0;
#pragma unroll
  for(int q = 0; q < Q - 1; ++q) acc += v.fold[q * n + e];
  v.vars[e] = 1.0 / (1.0 - L::w(Q - 1)) * acc;
}
// ... then the wall populations
template <int LAT>
__global__ void k_bnd_dirichlet_neem(View v, TableBnd b) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n    = v.n;
  const int32_t cell = b.cells[i], e = b.ext[i];
  const double  val  = b.values[i];
  v.vars[cell]       = val;
  const double phie  = v.vars[e];
#pragma unroll
  for(int q = 0; q < Q - 1; ++q) {
    const double w       = L::w(q);
    v.fold[q * n + cell] = w * val + v.fold[q * n + e] - w * phie;
  }
  v.fold[(Q - 1) * n + cell] = (L::w(Q - 1) - 1.0) * val + v.fold[(Q - 1) * n + e] - (L::w(Q - 1) - 1.0) * phie;
}
// LBMBnd_NeumannNEEM::apply (bnd_neumann.h:373-392): the Dirichlet value from
// a second-order one-sided difference with zero gradient
template <int LAT>
__global__ void k_bnd_neumann_value(View v, TableBnd b) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q;
  const int64_t i = gid();
  if(i >= b.n) return;
  const int64_t n   = v.n;
  const int32_t e   = b.ext[i], e2 = b.ext2[i];
  double        acc = 0;
#pragma unroll
  for(int q = 0; q < Q - 1; ++q) acc += v.fold[q * n + e2];
  const double phi2 = 1.0 / (1.0 - L::w(Q - 1)) * acc;
  v.vars[e2]        = phi2;
  const double grad = 0.0;
  b.values[i]       = (4.0 * v.vars[e] - phi2 + grad) / 3.0;
}

// ---- initial condition (src/lbm/solver.cpp:266-295) -------------------------
template <int LAT, int EQ>
__global__ void k_init(View v) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  const int64_t c = gid();
  if(c >= v.n) return;
  const int64_t n = v.n;
  if constexpr(EQ == LBM_NAVIER_STOKES) {
    v.vars[D * n + c] = 1.0;
    double u[D];
#pragma unroll
    for(int d = 0; d < D; ++d) u[d] = v.vars[d * n + c];
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      const double fe = eq_dist<LAT>(q, 1.0, u);
      v.feq[q * n + c] = fe;
      v.f[q * n + c]    = fe;
      v.fold[q * n + c] = fe;
    }
  } else {
    const double phi = v.vars[c];
#pragma unroll
    for(int q = 0; q < Q; ++q) {
      const double fe   = q == Q - 1 ? (L::w(Q - 1) - 1.0) * phi : L::w(q) * phi;
      v.feq[q * n + c]  = fe;
      v.f[q * n + c]    = fe;
      v.fold[q * n + c] = fe;
    }
  }
}

// ---------------------------------------------------------------------------
template <int LAT, int EQ>
cudaError_t step_impl(TableState& t, cudaStream_t s) {
  const View v = view(t);
  k_collide<LAT, EQ><<<blocks(t.n), TPB, 0, s>>>(v);
  if(t.forcing) {
    if(t.nforce_out) k_force<LAT><<<blocks(t.nforce_out), TPB, 0, s>>>(v, t.force_out, t.force_out_val, t.nforce_out, 1.0);
    if(t.nforce_in)
      k_force<LAT><<<blocks(t.nforce_in), TPB, 0, s>>>(v, t.force_in, t.force_in_val, t.nforce_in, 1.0 + t.forcing_dp);
  }
  constexpr int D = Lattice<LAT>::D;
  for(const TableBnd& b : t.bnds) {
    if(b.kind == LBM_BND_PERIODIC) {
      if(b.has_press) {
        if constexpr(EQ == LBM_NAVIER_STOKES) k_pre_periodic_pressure<LAT><<<blocks(b.n), TPB, 0, s>>>(v, b.cells, b.link0, b.n, b.scalar);
      } else {
        if(b.ncopy) k_pre_periodic_copy<<<blocks(b.ncopy), TPB, 0, s>>>(v, b.copy_dst, b.copy_q, b.copy_src, b.ncopy);
        if constexpr(EQ == LBM_NAVIER_STOKES) k_set_var<<<blocks(b.n), TPB, 0, s>>>(v, b.link0, b.n, D, 1.0);
      }
    } else if(b.kind == LBM_BND_PRESSURE_ABB) {
      k_set_var<<<blocks(b.n), TPB, 0, s>>>(v, b.cells, b.n, D, b.scalar);
    }
  }
  k_stream<LAT><<<blocks(t.n), TPB, 0, s>>>(v);
  for(const TableBnd& b : t.bnds) {
    switch(b.kind) {
      case LBM_BND_WALL_BB:
        k_bnd_bb<LAT, EQ, LBM_BND_WALL_BB><<<blocks(b.n), TPB, 0, s>>>(v, b);
        break;
      case LBM_BND_WALL_BB_TANGENTIAL:
        k_bnd_bb<LAT, EQ, LBM_BND_WALL_BB_TANGENTIAL><<<blocks(b.n), TPB, 0, s>>>(v, b);
        break;
      case LBM_BND_DIRICHLET_BB:
        k_bnd_bb<LAT, EQ, LBM_BND_DIRICHLET_BB><<<blocks(b.n), TPB, 0, s>>>(v, b);
        break;
      case LBM_BND_WALL_EQ:
      case LBM_BND_WALL_NEEM:
        if constexpr(EQ == LBM_NAVIER_STOKES) {
          k_bnd_wall_eq<LAT><<<blocks(b.n), TPB, 0, s>>>(v, b);
          if(b.kind == LBM_BND_WALL_NEEM) {
            k_bnd_neem_ext<LAT><<<blocks(b.nextu), TPB, 0, s>>>(v, b.extu, b.nextu);
            k_bnd_neem_add<LAT><<<blocks(b.n), TPB, 0, s>>>(v, b);
          }
        }
        break;
      case LBM_BND_WALL_NEBB:
        if constexpr(LAT == LBM_D2Q9 && EQ == LBM_NAVIER_STOKES) k_bnd_nebb<<<blocks(b.n), TPB, 0, s>>>(v, b);
        break;
      case LBM_BND_PRESSURE_ABB:
        if constexpr(EQ == LBM_NAVIER_STOKES && D == 2) k_bnd_pressure<LAT><<<blocks(b.n), TPB, 0, s>>>(v, b);
        break;
      case LBM_BND_NEUMANN_NEEM:
        if constexpr(EQ == LBM_POISSON) k_bnd_neumann_value<LAT><<<blocks(b.n), TPB, 0, s>>>(v, b);
        [[fallthrough]];
      case LBM_BND_DIRICHLET_NEEM:
        if constexpr(EQ == LBM_POISSON) {
          k_bnd_potential<LAT><<<blocks(b.nextu), TPB, 0, s>>>(v, b.extu, b.nextu);
          k_bnd_dirichlet_neem<LAT><<<blocks(b.n), TPB, 0, s>>>(v, b);
        }
        break;
      default:
        break;
    }
  }
  return cudaGetLastError();
}

template <int LAT, int EQ>
cudaError_t init_impl(TableState& t, cudaStream_t s) {
  k_init<LAT, EQ><<<blocks(t.n), TPB, 0, s>>>(view(t));
  return cudaGetLastError();
}

template <int LAT, int EQ>
cudaError_t moments_impl(TableState& t, cudaStream_t s) {
  k_moments<LAT, EQ><<<blocks(t.n), TPB, 0, s>>>(view(t));
  return cudaGetLastError();
}

template <template <int, int> class F>
struct Dispatch;

#define LBM_TABLE_DISPATCH(FN)                                                           \
  switch(t.lattice * 2 + t.equation) {                                                   \
    case LBM_D2Q9 * 2 + LBM_NAVIER_STOKES: return FN<LBM_D2Q9, LBM_NAVIER_STOKES>(t, s); \
    case LBM_D2Q9 * 2 + LBM_POISSON: return FN<LBM_D2Q9, LBM_POISSON>(t, s);             \
    case LBM_D2Q5 * 2 + LBM_POISSON: return FN<LBM_D2Q5, LBM_POISSON>(t, s);             \
    case LBM_D1Q3 * 2 + LBM_POISSON: return FN<LBM_D1Q3, LBM_POISSON>(t, s);             \
    default: return cudaErrorInvalidValue;                                               \
  }

}  // namespace

cudaError_t table_step(TableState& t, cudaStream_t s) { LBM_TABLE_DISPATCH(step_impl) }
cudaError_t table_initial_condition(TableState& t, cudaStream_t s) { LBM_TABLE_DISPATCH(init_impl) }
cudaError_t table_update_moments(TableState& t, cudaStream_t s) { LBM_TABLE_DISPATCH(moments_impl) }

}  // namespace lbm
