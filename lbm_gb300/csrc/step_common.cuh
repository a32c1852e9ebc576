// Device building blocks shared by the dense-box and batched engines: the
// population state and its storage conversions, compile-time direction loops,
// and the BGK / Poisson-Boltzmann collisions.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <utility>

#include "../../include/lbm_gpu_box.h"
#include "lattice.cuh"

namespace lbm {

// Navier-Stokes populations are held as the scaled relative deviation from
// the lattice weight, v = S (f - w) / w, in every storage; Poisson populations
// are held as f.
constexpr double STATE_SCALE = 4096.0;

// ---- storage conversions ---------------------------------------------------
template <int ST>
struct Store;
// load(v) / store(v): the stored value is the state itself.  load(v, k) /
// store(v, k) (the dense-box engine): the 16-bit storages hold the state
// minus k, the state of a reference equilibrium for the population's
// direction, so that a population near that equilibrium is stored as a
// small number with FP16's / BF16's relative rounding; the 32- and 64-bit
// storages ignore k.
template <>
struct Store<LBM_STORE_F64> {
  using T = double;
  using C = double;
  static __device__ __forceinline__ C load(T v) { return v; }
  static __device__ __forceinline__ T store(C v) { return v; }
  static __device__ __forceinline__ C load(T v, float) { return v; }
  static __device__ __forceinline__ T store(C v, float) { return v; }
};
template <>
struct Store<LBM_STORE_F32> {
  using T = float;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return v; }
  static __device__ __forceinline__ T store(C v) { return v; }
  static __device__ __forceinline__ C load(T v, float) { return v; }
  static __device__ __forceinline__ T store(C v, float) { return v; }
};
template <>
struct Store<LBM_STORE_F16_DEV> {
  using T = __half;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return __half2float(v); }
  static __device__ __forceinline__ T store(C v) { return __float2half_rn(v); }
  static __device__ __forceinline__ C load(T v, float k) { return __half2float(v) + k; }
  static __device__ __forceinline__ T store(C v, float k) { return __float2half_rn(v - k); }
};
template <>
struct Store<LBM_STORE_BF16_DEV> {
  using T = __nv_bfloat16;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return __bfloat162float(v); }
  static __device__ __forceinline__ T store(C v) { return __float2bfloat16_rn(v); }
  static __device__ __forceinline__ C load(T v, float k) { return __bfloat162float(v) + k; }
  static __device__ __forceinline__ T store(C v, float k) { return __float2bfloat16_rn(v - k); }
};

// state value <-> population f of direction q
template <int LAT, int EQ>
__device__ __forceinline__ double state_to_f(double v, int q) {
  if constexpr(EQ == LBM_NAVIER_STOKES) return Lattice<LAT>::w(q) * (1.0 + v * (1.0 / STATE_SCALE));
  else return v;
}
template <int LAT, int EQ>
__device__ __forceinline__ double f_to_state(double f, int q) {
  if constexpr(EQ == LBM_NAVIER_STOKES) return (f - Lattice<LAT>::w(q)) * (STATE_SCALE / Lattice<LAT>::w(q));
  else return f;
}


// ---- compile-time loops over the directions ------------------------------
// Every per-direction statement of the step is instantiated with a constant q,
// so lattice velocities, weights and plane offsets fold into immediates and
// the populations stay in registers.
template <class F, int... Is>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// parameter in the arithmetic precision
template <class C>
__device__ __forceinline__ C prm(double d, float f) {
  if constexpr(sizeof(C) == 4) return f;
  else return d;
}

// ---- collision -------------------------------------------------------------
// Navier-Stokes BGK (+ Guo forcing) on the scaled deviations v_q:
//   S drho = sum w_q v_q,  S j = sum c_q w_q v_q  (sum c w = 0),
//   u = (j + F/2) / rho,
//   v_eq = S (drho + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u^2)),
//   v' = (1 - omega) v + omega v_eq + S (1 - omega/2) [3 (c - u).F + 9 (c.u)(c.F)].
// Opposite directions share the even part of v_eq and of the forcing term and
// differ in the sign of the odd part, so each pair costs one evaluation.
// 1/x: the correctly rounded single-precision reciprocal (no division
// slow path); plain division in FP64
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

// FORCE is a compile-time switch: without a body force the forcing terms and
// their branches are not generated at all.
template <int LAT, class C, bool FORCE = true>
__device__ __forceinline__ void collide_ns(C om, bool force_in, const C* Fin, C* v, C* mom_out) {
  const bool force = FORCE && force_in;
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  constexpr C   S = static_cast<C>(STATE_SCALE), IS = static_cast<C>(1.0 / STATE_SCALE);
  C             r0 = 0, j[3] = {0, 0, 0};
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    constexpr C   w = static_cast<C>(L::w(q));
    r0              = fma(w, v[q], r0);
    static_for<D>([&](auto dc) {
      constexpr int d = decltype(dc)::value;
      if constexpr(L::c(q, d) > 0) j[d] = fma(w, v[q], j[d]);
      if constexpr(L::c(q, d) < 0) j[d] = fma(-w, v[q], j[d]);
    });
  });
  const C    rho   = C(1) + r0 * IS;
  const C    irho  = recip(rho);
  C F[3] = {0, 0, 0}, u[3] = {0, 0, 0};
  if(force) static_for<D>([&](auto dc) { F[decltype(dc)::value] = Fin[decltype(dc)::value]; });
  C usq = 0, uf = 0;
  static_for<D>([&](auto dc) {
    constexpr int d = decltype(dc)::value;
    if constexpr(FORCE) {
      u[d] = fma(j[d], IS, C(0.5) * F[d]) * irho;
      uf   = fma(u[d], F[d], uf);
    } else {
      u[d] = j[d] * IS * irho;
    }
    usq = fma(u[d], u[d], usq);
  });
  if(mom_out) {
    mom_out[0] = rho;
    static_for<D>([&](auto dc) { mom_out[1 + decltype(dc)::value] = u[decltype(dc)::value]; });
  }
  const C keep = C(1) - om;
  const C Rs   = S * rho;
  const C K0w  = om * (r0 - C(1.5) * Rs * usq);  // omega S (drho - 1.5 rho u^2)
  const C A    = om * C(4.5) * Rs;
  const C B    = om * C(3) * Rs;
  const C G    = S * (C(1) - C(0.5) * om);  // Guo prefactor in state units
  C       E0   = K0w;
  if(force) E0 = fma(-C(3) * G, uf, E0);
  v[Q - 1] = fma(keep, v[Q - 1], E0);
  static_for<Q - 1>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    constexpr int o = L::opp(q);
    if constexpr(q < o) {
      // c_q.u and c_q.F, started from the first non-zero component (no 0 + x)
      constexpr int d0 = L::c(q, 0) != 0 ? 0 : (L::c(q, 1) != 0 ? 1 : 2);
      C             cu = L::c(q, d0) > 0 ? u[d0] : -u[d0];
      C             cf = L::c(q, d0) > 0 ? F[d0] : -F[d0];
      static_for<D>([&](auto dc) {
        constexpr int d = decltype(dc)::value;
        if constexpr(d > d0 && L::c(q, d) > 0) {
          cu += u[d];
          cf += F[d];
        }
        if constexpr(d > d0 && L::c(q, d) < 0) {
          cu -= u[d];
          cf -= F[d];
        }
      });
      C E = fma(A * cu, cu, E0);
      C O = B * cu;
      if(force) {
        E = fma(C(9) * G * cu, cf, E);
        O = fma(C(3) * G, cf, O);
      }
      v[q] = fma(keep, v[q], E + O);
      v[o] = fma(keep, v[o], E - O);
    }
  });
}

// Poisson(-Boltzmann), Chai & Shi (2008): phi from the moving populations,
// f' = f + omega (feq - f) + w'_q D kappa^2 g(phi), g = sinh or identity
template <int LAT, class C>
__device__ __forceinline__ void collide_poisson(C omega, bool nonlinear, C src_coef, C* f, C* mom_out) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q;
  C             acc = 0;
  static_for<Q - 1>([&](auto qc) { acc += f[decltype(qc)::value]; });
  const C phi = acc * static_cast<C>(1.0 / (1.0 - L::w(Q - 1)));
  if(mom_out) mom_out[0] = phi;
  const C g   = nonlinear ? sinh(phi) : phi;
  const C src = src_coef * g;
  static_for<Q>([&](auto qc) {
    constexpr int q   = decltype(qc)::value;
    const C       feq = q == Q - 1 ? static_cast<C>(L::w(Q - 1) - 1.0) * phi : static_cast<C>(L::w(q)) * phi;
    C             out = f[q] + omega * (feq - f[q]);
    if constexpr(q != Q - 1) out += static_cast<C>(L::pw(q)) * src;
    f[q] = out;
  });
}


template <class C>
__device__ __forceinline__ C warp_sum(C v) {
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}


}  // namespace lbm
