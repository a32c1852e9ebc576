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
template <>
struct Store<LBM_STORE_F64> {
  using T = double;
  using C = double;
  static __device__ __forceinline__ C load(T v) { return v; }
  static __device__ __forceinline__ T store(C v) { return v; }
};
template <>
struct Store<LBM_STORE_F32> {
  using T = float;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return v; }
  static __device__ __forceinline__ T store(C v) { return v; }
};
template <>
struct Store<LBM_STORE_F16_DEV> {
  using T = __half;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return __half2float(v); }
  static __device__ __forceinline__ T store(C v) { return __float2half_rn(v); }
};
template <>
struct Store<LBM_STORE_BF16_DEV> {
  using T = __nv_bfloat16;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return __bfloat162float(v); }
  static __device__ __forceinline__ T store(C v) { return __float2bfloat16_rn(v); }
};
// 1 sign, 3 exponent, 12 mantissa bits of t = s / 1024 (LBM_STORE_E3M12_DEV):
// code = E * 4096 + m, value 2^(E-7) (1 + m / 4096) for E >= 1 and
// 2^-6 m / 4096 for E = 0, saturating at code 0x7fff.  Encoding, for
// |s| >= 16 (t >= 2^-6, E >= 1): the FP32 bits of |s| rounded to 12 mantissa
// bits (round to nearest even on the 11 dropped bits, the carry moving into
// the exponent) and rebased from FP32's exponent bias and the 2^-10 scale to
// the code's (130 = 127 + 10 - 7); below: round(|s| 2^8) as an integer (the
// evenly spaced range, 2^-18 in t; 4096 rounds into the first normal code).
// Decoding: the code's 15 bits placed as FP32 bits (exponent field E,
// mantissa m << 11) are 2^-130 times the value, E = 0 included (an FP32
// subnormal then), so two exact power-of-two products restore it.
__device__ __forceinline__ uint16_t e3m12_encode(float s) {
  const uint32_t u = __float_as_uint(s);
  const uint32_t a = u & 0x7fffffffu;
  uint32_t       code;
  if(a >= 0x41800000u) {  // |s| >= 16
    const uint32_t r = a + 0x3ffu + ((a >> 11) & 1u);
    code             = min((r >> 11) - (130u << 12), 0x7fffu);
  } else {
    code = __float2uint_rn(__uint_as_float(a) * 256.0f);
  }
  return static_cast<uint16_t>(code | ((u >> 16) & 0x8000u));
}
__device__ __forceinline__ float e3m12_decode(uint16_t c) {
  const uint32_t bits = ((static_cast<uint32_t>(c) & 0x7fffu) << 11) | ((static_cast<uint32_t>(c) & 0x8000u) << 16);
  return __uint_as_float(bits) * 0x1p127f * 8.0f;
}
template <>
struct Store<LBM_STORE_E3M12_DEV> {
  using T = uint16_t;
  using C = float;
  static __device__ __forceinline__ C load(T v) { return e3m12_decode(v); }
  static __device__ __forceinline__ T store(C v) { return e3m12_encode(v); }
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
// 1/x for x near 1 (a density): the hardware reciprocal estimate refined by
// one Newton step, r (2 - x r), within an ulp or so of the correctly rounded
// value at a third of its instructions
__device__ __forceinline__ float recip_fast(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r * fmaf(-x, r, 2.0f);
}

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

// Navier-Stokes BGK (+ Guo forcing) in single precision on the state shifted
// to a free stream U along x (the dense-box engine's FP32 / FP16 / BF16
// storages):
//   s_q = v_q - S P_q(U),  P_q(u) = 3 c_q.u + 4.5 (c_q.u)^2 - 1.5 u^2,
// the deviation of each population from the equilibrium at rho = 1 and u = U.
// Every intermediate is a deviation from that free stream as well:
//   r = rho - 1 = (sum w_q s_q) / S   (sum w_q P_q(U) = 0),
//   du = u - U = (sum c_q w_q s_q / S + F/2 - r U) / rho,
//   s_eq_q = S [r (1 - 1.5 U^2) - 1.5 rho du.(2U + du)]
//            + 4.5 S [r (c_qx U)^2 + rho (c_q.du)(c_q.du + 2 c_qx U)]
//            + 3 S [r c_qx U + rho c_q.du],
// so in a flow near U the arithmetic rounds relative to small numbers.  (The
// same update on v = s + S P(U) rounds relative to |v| ~ 600 in a flow at
// U = 0.05, and over tens of thousands of steps that rounding acts like a
// small body force.)  It is the BGK update itself: v' = (1 - omega) v +
// omega v_eq maps to s' = (1 - omega) s + omega s_eq.  Opposite directions
// share the even part (first two lines) and differ in the sign of the odd
// part.  U = 0 gives the update on v.
template <int LAT, bool FORCE = true>
__device__ __forceinline__ void collide_ns_shifted(float om, bool force_in, const float* Fin, float U, float* sv, float* mom_out) {
  const bool force = FORCE && force_in;
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  constexpr float S = static_cast<float>(STATE_SCALE), IS = static_cast<float>(1.0 / STATE_SCALE);
  // moments from the sum and difference of each pair of opposite directions
  // (w_q = w_opp(q)): sum w s = sum_pairs w (s_q + s_o) + w_rest s_rest,
  // sum c w s = sum_pairs c_q w (s_q - s_o)
  float r0 = static_cast<float>(L::w(Q - 1)) * sv[Q - 1], j[3] = {0, 0, 0};
  static_for<Q - 1>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    constexpr int o = L::opp(q);
    if constexpr(q < o) {
      constexpr float w = static_cast<float>(L::w(q));
      r0                = fmaf(w, sv[q] + sv[o], r0);
      const float m     = sv[q] - sv[o];
      static_for<D>([&](auto dc) {
        constexpr int d = decltype(dc)::value;
        if constexpr(L::c(q, d) > 0) j[d] = fmaf(w, m, j[d]);
        if constexpr(L::c(q, d) < 0) j[d] = fmaf(-w, m, j[d]);
      });
    }
  });
  const float r    = r0 * IS;
  const float rho  = 1.0f + r;
  const float irho = recip_fast(rho);
  float       F[3] = {0, 0, 0}, du[3] = {0, 0, 0};
  if(force) static_for<D>([&](auto dc) { F[decltype(dc)::value] = Fin[decltype(dc)::value]; });
  static_for<D>([&](auto dc) {
    constexpr int d = decltype(dc)::value;
    float         m = FORCE ? fmaf(j[d], IS, 0.5f * F[d]) : j[d] * IS;
    if constexpr(d == 0) m = fmaf(-r, U, m);
    du[d] = m * irho;
  });
  // du.(2U + du) = u^2 - U^2, and u.F
  float dusq = du[0] * fmaf(2.0f, U, du[0]), uf = 0;
  static_for<D>([&](auto dc) {
    constexpr int d = decltype(dc)::value;
    if constexpr(d > 0) dusq = fmaf(du[d], du[d], dusq);
  });
  if(force) {
    uf = (U + du[0]) * F[0];
    static_for<D>([&](auto dc) {
      constexpr int d = decltype(dc)::value;
      if constexpr(d > 0) uf = fmaf(du[d], F[d], uf);
    });
  }
  if(mom_out) {
    mom_out[0] = rho;
    static_for<D>([&](auto dc) {
      constexpr int d = decltype(dc)::value;
      mom_out[1 + d]  = d == 0 ? U + du[0] : du[d];
    });
  }
  const float keep = 1.0f - om;
  const float oS   = om * S;
  const float A    = oS * 4.5f * rho;
  const float B    = oS * 3.0f * rho;
  const float G    = S * (1.0f - 0.5f * om);  // Guo prefactor in state units
  // the even constant part: rest and c_x = 0 directions, and c_x != 0 ones
  float E0 = oS * fmaf(r, fmaf(-1.5f * U, U, 1.0f), -1.5f * rho * dusq);
  if(force) E0 = fmaf(-3.0f * G, uf, E0);
  const float E0x = fmaf(oS * 4.5f * r * U, U, E0);
  const float Bu  = oS * 3.0f * r * U;
  sv[Q - 1]       = fmaf(keep, sv[Q - 1], E0);
  static_for<Q - 1>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    constexpr int o = L::opp(q);
    if constexpr(q < o) {
      // c_q.du and c_q.F, started from the first non-zero component (no 0 + x)
      constexpr int d0  = L::c(q, 0) != 0 ? 0 : (L::c(q, 1) != 0 ? 1 : 2);
      constexpr int cx  = L::c(q, 0);
      float         cdu = L::c(q, d0) > 0 ? du[d0] : -du[d0];
      float         cf  = L::c(q, d0) > 0 ? F[d0] : -F[d0];
      static_for<D>([&](auto dc) {
        constexpr int d = decltype(dc)::value;
        if constexpr(d > d0 && L::c(q, d) > 0) {
          cdu += du[d];
          cf += F[d];
        }
        if constexpr(d > d0 && L::c(q, d) < 0) {
          cdu -= du[d];
          cf -= F[d];
        }
      });
      float E, O;
      if constexpr(cx == 0) {
        E = fmaf(A * cdu, cdu, E0);
        O = B * cdu;
      } else {
        const float tu = cx > 0 ? 2.0f * U : -2.0f * U;  // 2 c_qx U
        E              = fmaf(A * cdu, cdu + tu, E0x);
        O              = fmaf(B, cdu, cx > 0 ? Bu : -Bu);
      }
      if(force) {
        const float cu = cx == 0 ? cdu : (cx > 0 ? cdu + U : cdu - U);
        E              = fmaf(9.0f * G * cu, cf, E);
        O              = fmaf(3.0f * G, cf, O);
      }
      sv[q] = fmaf(keep, sv[q], E + O);
      sv[o] = fmaf(keep, sv[o], E - O);
    }
  });
}

// The shifted state of the equilibrium at (rho, u) in single precision (free
// stream U along x): s_eq_q = v_eq_q - S P_q(U), the terms of
// collide_ns_shifted with omega = 1.
template <int LAT>
__device__ __forceinline__ void equilibrium_shifted(float rho, const float* u, float U, float* out) {
  using L         = Lattice<LAT>;
  constexpr int Q = L::Q, D = L::D;
  constexpr float S = static_cast<float>(STATE_SCALE);
  const float     r = rho - 1.0f;
  const float     du[3] = {u[0] - U, D > 1 ? u[1] : 0.0f, D > 2 ? u[2] : 0.0f};
  const float     dusq  = fmaf(du[0], fmaf(2.0f, U, du[0]), fmaf(du[1], du[1], du[2] * du[2]));
  const float     E0    = S * fmaf(r, fmaf(-1.5f * U, U, 1.0f), -1.5f * rho * dusq);
  static_for<Q>([&](auto qc) {
    constexpr int q   = decltype(qc)::value;
    constexpr int cx  = L::c(q, 0);
    float         cdu = 0;
    static_for<D>([&](auto dc) {
      constexpr int d = decltype(dc)::value;
      if constexpr(L::c(q, d) != 0) cdu += static_cast<float>(L::c(q, d)) * du[d];
    });
    const float ux = static_cast<float>(cx) * U;
    const float E  = E0 + S * 4.5f * fmaf(r * ux, ux, rho * cdu * (cdu + 2.0f * ux));
    const float O  = S * 3.0f * fmaf(r, ux, rho * cdu);
    out[q]         = E + O;
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
