// Lagrangian particles (include/lbm_lpt.h): the reference's particle step,
// LPTSolver::calcA + timeIntegration (src/lpt/solver.cpp:356-496, force models
// of src/lpt/forces.h), on the GPU.
//
// The reference loops over the particles once per step and reads and writes
// every particle's variables each time.  Here one thread owns a particle for
// a whole step call: its state is loaded once, stepped `nsteps` times in
// registers, and stored once, so a call of many steps costs one pass over
// memory.  Particles are independent (the reference has no collisions and
// deletes none), so nothing is shared between threads.
//
// Arithmetic: IEEE doubles in the reference's operation order; this unit is
// compiled without fused multiply-adds (-fmad=false), so every product and
// sum rounds as the reference's do.  The one difference is the power of the
// Putnam drag factor (gcem there, CUDA's pow here).
//
// Coupled to a dense-box LBM context, the ambient velocity of each step is
// read from the box's moments at the particle's cell (one-way coupling: the
// fluid moves the particles, the particles do not act on the fluid).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "../../include/lbm_lpt.h"
#include "box.h"

struct lbm_lpt_ctx {
  lbm_lpt_desc desc{};
  int          D  = 0;
  int          nv = 0;  // variables per particle, 3*D+5
  int64_t      n  = 0;
  cudaStream_t stream = nullptr;
  double*      soa    = nullptr;  // nv planes of `capacity` doubles
  std::string  err;
  lbm_gpu_ctx* box          = nullptr;
  double       origin[3]    = {0, 0, 0};
  double       cell_length  = 1.0;
  double       uscale       = 1.0;
};

namespace {

struct LptParams {
  int64_t n = 0, cap = 0;
  double  dt = 0, g[3] = {0, 0, 0}, rho_a = 0, nu_a = 0, va[3] = {0, 0, 0}, rho_p0 = 0;
  int     drag = 0, nlin = 0, buoyant = 0, own = 0;
  double* s = nullptr;  // plane k of variable k at s + k * cap
  // ambient velocity field of a coupled box: moments, k = 1..D the velocity
  const void* mom    = nullptr;
  int64_t     ncells = 0;
  int         nx = 1, ny = 1, nz = 1;
  double      origin[3] = {0, 0, 0}, inv_h = 1.0, uscale = 1.0;
};

// force::dragCoefficient<Putnam61> (src/lpt/forces.h)
__device__ __forceinline__ double putnam(double re) {
  if(re > 1000) return 0.424 * re / 24.0;
  if(re <= 0.1) return 1.0;
  return 1.0 + pow(re, 2.0 / 3.0) / 6.0;
}

__device__ __forceinline__ int64_t cell_of(double x, double origin, double inv_h, int n) {
  const double t = floor((x - origin) * inv_h);
  if(!(t >= 0.0)) return 0;  // below the box, or not a number
  if(t >= static_cast<double>(n)) return n - 1;
  return static_cast<int64_t>(t);
}

// FIELD: 0 constant ambient velocity, 1 FP32 box moments, 2 FP64 box moments
template <int D, bool IMPLICIT, int FIELD>
__global__ void __launch_bounds__(256) k_lpt_steps(LptParams P, int64_t nsteps) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if(i >= P.n) return;
  double* const S   = P.s;
  const int64_t cap = P.cap;
  double        x[D], v[D], a[D];
#pragma unroll
  for(int d = 0; d < D; ++d) {
    x[d] = S[d * cap + i];
    v[d] = S[(D + d) * cap + i];
    a[d] = S[(2 * D + d) * cap + i];
  }
  const double r     = S[(3 * D) * cap + i];
  const double rho   = S[(3 * D + 1) * cap + i];
  double       dc    = S[(3 * D + 4) * cap + i];
  const double rho_p = P.own ? rho : P.rho_p0;  // the density-ratio models use particle 0's density
  for(int64_t step = 0; step < nsteps; ++step) {
    double va[D];
    if constexpr(FIELD == 0) {
#pragma unroll
      for(int d = 0; d < D; ++d) va[d] = P.va[d];
    } else {
      const int64_t ix = cell_of(x[0], P.origin[0], P.inv_h, P.nx);
      const int64_t iy = cell_of(x[1], P.origin[1], P.inv_h, P.ny);
      const int64_t iz = D > 2 ? cell_of(x[D - 1], P.origin[D - 1], P.inv_h, P.nz) : 0;
      const int64_t c  = ix + P.nx * (iy + static_cast<int64_t>(P.ny) * iz);
#pragma unroll
      for(int d = 0; d < D; ++d) {
        const int64_t k = (1 + d) * P.ncells + c;
        va[d] = (FIELD == 1 ? static_cast<double>(static_cast<const float*>(P.mom)[k]) : static_cast<const double*>(P.mom)[k]) *
                P.uscale;
      }
    }
    // calcA: gravity (with buoyancy), then drag
    if(P.buoyant) {
      const double fac = 1.0 - P.rho_a / rho_p;
#pragma unroll
      for(int d = 0; d < D; ++d) a[d] = P.g[d] * fac;
    } else {
#pragma unroll
      for(int d = 0; d < D; ++d) a[d] = P.g[d];
    }
    if(P.drag) {
      dc = 18.0 * P.nu_a / (4.0 * r * r * rho_p);
      if(P.nlin) {
        double s2 = v[0] * v[0];
#pragma unroll
        for(int d = 1; d < D; ++d) s2 = s2 + v[d] * v[d];
        const double re = P.rho_a * sqrt(s2) * 2.0 * r / P.nu_a;
        dc *= putnam(re);
      }
      if constexpr(!IMPLICIT) {
#pragma unroll
        for(int d = 0; d < D; ++d) a[d] = a[d] + dc * (va[d] - v[d]);
      }
    } else {
      dc = 0.0;
    }
    // timeIntegration
    if constexpr(!IMPLICIT) {
#pragma unroll
      for(int d = 0; d < D; ++d) {
        v[d] = v[d] + a[d] * P.dt;
        x[d] = x[d] + v[d] * P.dt;
      }
    } else {
      const double den = 1.0 + dc * P.dt;
#pragma unroll
      for(int d = 0; d < D; ++d) {
        const double vo = v[d];
        const double vn = (vo + a[d] * P.dt + dc * va[d] * P.dt) / den;
        a[d]            = (vo - vn) / P.dt;
        x[d]            = x[d] + 0.5 * (vn + vo) * P.dt;
        v[d]            = vn;
      }
    }
  }
#pragma unroll
  for(int d = 0; d < D; ++d) {
    S[d * cap + i]           = x[d];
    S[(D + d) * cap + i]     = v[d];
    S[(2 * D + d) * cap + i] = a[d];
  }
  S[(3 * D + 4) * cap + i] = dc;
}

template <int D, bool IMPLICIT>
void launch_d(const LptParams& P, int field, int64_t nsteps, cudaStream_t s) {
  const unsigned g = static_cast<unsigned>((P.n + 255) / 256);
  if(field == 0) k_lpt_steps<D, IMPLICIT, 0><<<g, 256, 0, s>>>(P, nsteps);
  else if(field == 1) k_lpt_steps<D, IMPLICIT, 1><<<g, 256, 0, s>>>(P, nsteps);
  else k_lpt_steps<D, IMPLICIT, 2><<<g, 256, 0, s>>>(P, nsteps);
}

int fail(lbm_lpt_ctx* c, int code, const std::string& msg) {
  c->err = msg;
  return code;
}

int cuda_fail(lbm_lpt_ctx* c, cudaError_t e, const char* what) {
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return LBM_ERR_CUDA;
}

}  // namespace

extern "C" {

int lbm_lpt_create(const lbm_lpt_desc* desc, lbm_lpt_ctx** out) {
  if(!desc || !out) return LBM_ERR_INVALID;
  *out = nullptr;
  if((desc->ndim != 2 && desc->ndim != 3) || desc->model < 0 || desc->model > 8 || desc->integration < 0 || desc->integration > 1 ||
     desc->capacity <= 0 || !(desc->dt > 0.0))
    return LBM_ERR_INVALID;
  lbm_lpt_ctx* c = new(std::nothrow) lbm_lpt_ctx();
  if(!c) return LBM_ERR_NOMEM;
  c->desc = *desc;
  c->D    = desc->ndim;
  c->nv   = 3 * c->D + 5;
  cudaError_t e = cudaSetDevice(desc->device);
  if(e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if(e == cudaSuccess) e = cudaMalloc(&c->soa, sizeof(double) * c->nv * desc->capacity);
  if(e != cudaSuccess) {
    if(c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
  }
  *out = c;
  return LBM_OK;
}

int lbm_lpt_set_particles(lbm_lpt_ctx* c, int64_t n, const double* vars) {
  if(!c) return LBM_ERR_INVALID;
  if(n < 0 || n > c->desc.capacity || (n > 0 && !vars)) return fail(c, LBM_ERR_INVALID, "particle count outside [0, capacity]");
  const int64_t       cap = c->desc.capacity;
  std::vector<double> planes(static_cast<size_t>(c->nv) * n);
  for(int64_t p = 0; p < n; ++p)
    for(int k = 0; k < c->nv; ++k) planes[k * n + p] = vars[p * c->nv + k];
  cudaSetDevice(c->desc.device);
  for(int k = 0; k < c->nv && n > 0; ++k) {
    const cudaError_t e = cudaMemcpyAsync(c->soa + k * cap, planes.data() + k * n, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    if(e != cudaSuccess) return cuda_fail(c, e, "set particles");
  }
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  if(e != cudaSuccess) return cuda_fail(c, e, "set particles");
  c->n = n;
  return LBM_OK;
}

int lbm_lpt_get_particles(lbm_lpt_ctx* c, double* vars) {
  if(!c || (c->n > 0 && !vars)) return LBM_ERR_INVALID;
  const int64_t       n = c->n, cap = c->desc.capacity;
  std::vector<double> planes(static_cast<size_t>(c->nv) * n);
  cudaSetDevice(c->desc.device);
  for(int k = 0; k < c->nv && n > 0; ++k) {
    const cudaError_t e = cudaMemcpyAsync(planes.data() + k * n, c->soa + k * cap, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    if(e != cudaSuccess) return cuda_fail(c, e, "get particles");
  }
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  if(e != cudaSuccess) return cuda_fail(c, e, "get particles");
  for(int64_t p = 0; p < n; ++p)
    for(int k = 0; k < c->nv; ++k) vars[p * c->nv + k] = planes[k * n + p];
  return LBM_OK;
}

int64_t lbm_lpt_count(const lbm_lpt_ctx* c) { return c ? c->n : 0; }

int lbm_lpt_couple_box(lbm_lpt_ctx* c, lbm_gpu_ctx* box, const double* origin, double cell_length, double velocity_scale) {
  if(!c) return LBM_ERR_INVALID;
  if(!box) {
    c->box = nullptr;
    return LBM_OK;
  }
  lbm::BoxState* b = lbm_internal_box(box);
  if(!b) return fail(c, LBM_ERR_INVALID, "not a dense-box context");
  if(b->desc.equation != LBM_NAVIER_STOKES) return fail(c, LBM_ERR_UNSUPPORTED, "the box carries no velocity (Poisson)");
  if(!origin || !(cell_length > 0.0)) return fail(c, LBM_ERR_INVALID, "origin and a positive cell length needed");
  if(b->D != c->D) return fail(c, LBM_ERR_INVALID, "box and particles differ in dimension");
  c->box = box;
  for(int d = 0; d < 3; ++d) c->origin[d] = d < c->D ? origin[d] : 0.0;
  c->cell_length = cell_length;
  c->uscale      = velocity_scale;
  return LBM_OK;
}

int lbm_lpt_step(lbm_lpt_ctx* c, int64_t nsteps) {
  if(!c || nsteps < 0) return LBM_ERR_INVALID;
  if(c->n == 0 || nsteps == 0) return LBM_OK;
  const lbm_lpt_desc& d = c->desc;
  LptParams           P;
  P.n   = c->n;
  P.cap = d.capacity;
  P.dt  = d.dt;
  for(int k = 0; k < 3; ++k) {
    P.g[k]  = d.gravity[k];
    P.va[k] = d.v_ambient[k];
  }
  P.rho_a   = d.rho_ambient;
  P.nu_a    = d.nu_ambient;
  const int m = d.model;
  P.drag    = m == 1 || m == 2 || m == 4 || m == 5 || m == 7 || m == 8;
  P.nlin    = m == 2 || m == 5 || m == 8;
  P.buoyant = m >= 3;
  P.own     = m >= 6;
  P.s       = c->soa;
  cudaSetDevice(d.device);
  // particle 0's density (the density-ratio models use it for every particle)
  cudaError_t e = cudaMemcpyAsync(&P.rho_p0, c->soa + (3 * c->D + 1) * d.capacity, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if(e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if(e != cudaSuccess) return cuda_fail(c, e, "particle density");
  int field = 0;
  if(c->box) {
    lbm::BoxState* b = lbm_internal_box(c->box);
    if(!b || !b->mom_valid) return fail(c, LBM_ERR_INVALID, "the coupled box has no velocity field yet: run a step call first");
    field     = b->desc.storage == LBM_STORE_F64 ? 2 : 1;
    P.mom     = b->mom;
    P.ncells  = b->p.ncells;
    P.nx      = b->p.nx;
    P.ny      = b->p.ny;
    P.nz      = b->p.nz;
    P.inv_h   = 1.0 / c->cell_length;
    P.uscale  = c->uscale;
    for(int k = 0; k < 3; ++k) P.origin[k] = c->origin[k];
  }
  const bool implicit = d.integration == LBM_LPT_IMPLICIT_EULER;
  if(c->D == 2) {
    if(implicit) launch_d<2, true>(P, field, nsteps, c->stream);
    else launch_d<2, false>(P, field, nsteps, c->stream);
  } else {
    if(implicit) launch_d<3, true>(P, field, nsteps, c->stream);
    else launch_d<3, false>(P, field, nsteps, c->stream);
  }
  e = cudaGetLastError();
  if(e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if(e != cudaSuccess) return cuda_fail(c, e, "particle step");
  return LBM_OK;
}

const char* lbm_lpt_last_error(const lbm_lpt_ctx* c) { return c ? c->err.c_str() : "null context"; }

void lbm_lpt_destroy(lbm_lpt_ctx* c) {
  if(!c) return;
  cudaSetDevice(c->desc.device);
  if(c->soa) cudaFree(c->soa);
  if(c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

}  // extern "C"
