// Dense-box engine: the BGK step on a structured nx*ny*nz box with a flag byte
// per cell, AA-pattern in-place streaming and selectable population storage.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/lbm_gpu.h"
#include "../../include/lbm_gpu_box.h"

struct lbm_gpu_ctx;

namespace lbm {

// blocks of the first level of the residual reduction (two per SM on 152 SMs)
constexpr int kMidBlocks = 304;
// block sizes the step autotuner tries
constexpr int kTunerBlocks[3] = {64, 128, 256};

// Everything a box kernel needs, passed by value (kernel parameter space).
struct BoxParams {
  int     nx, ny, nz;       // fluid box
  int64_t ncells;           // nx*ny*nz
  int64_t nalloc;           // cells per population plane (ncells + outlet ghost plane)
  int     face[6];          // lbm_face per face (-x,+x,-y,+y,-z,+z)
  double  wall_u[6][3];     // velocity of each wall face (moving bounce-back)
  double  omega;
  double  force[3];         // Guo body force
  double  inlet_rho, inlet_u[3];
  double  kappa_sq;         // Poisson-Boltzmann kappa^2
  double  pb_diffusivity;   // alpha (1/2 - tau) in lattice units
  int     pb_nonlinear;
  int     has_force;
  // single-precision copies for the FP32-arithmetic kernels (GB300's FP64
  // pipe is narrow: converting a double parameter per cell is measurable)
  float   omega_f, force_f[3], inlet_rho_f, inlet_u_f[3], pb_src_f;
  int     has_outlet;
  // FP32 / FP16 / BF16 storage of Navier-Stokes populations: the state is
  // the scaled deviation shifted to the free stream U = (shift_u, 0, 0),
  // s_q = v_q - S P_q(U), S P_q(U) the scaled deviation of the equilibrium at
  // rho = 1 and u = U (0 for FP64 storage, for Poisson and without a free
  // stream); shift_u_d: the same U in double precision
  float   shift_u;
  double  shift_u_d;
  // per-z-slice relaxation rates (nz values each) or nullptr: one rate
  const double* slice_omega;
  const float*  slice_omega_f;
  // per-z-slice Poisson-Boltzmann source coefficients alpha (1/2 - tau)
  // kappa^2 (nz values each) or nullptr: pb_diffusivity * kappa_sq
  const double* slice_src;
  const float*  slice_src_f;
  const uint8_t* flags;     // ncells
  const double*  dirichlet; // ncells Poisson Dirichlet values or nullptr
  void*   pop;              // Q planes of nalloc values of the storage type
  // residual support: moments of the previous check step (ncells x nvar, compute precision)
  void*   mom;
  double* partials;         // per-block partial sums of |moment change|
  int64_t partial_stride;   // slots per variable in partials
  int     mom_mode;         // 0 none, 1 write moments, 2 accumulate |new-old| and write
};

struct BoxState {
  lbm_box_desc desc;
  BoxParams    p;
  int          Q = 0, D = 0, nvar = 0;
  int64_t      steps = 0;     // completed steps; parity selects the AA kernel
  size_t       elem  = 8;     // bytes per stored population
  void*        pop   = nullptr;  // plane 0 of the populations (inside pop_alloc, after one guard plane)
  void*        pop_alloc = nullptr;  // the allocation: one guard plane, Q planes, the outlet ghost plane
  uint8_t*     flags = nullptr;
  double*      dirichlet = nullptr;
  double*      slice_omega   = nullptr;  // per-z-slice relaxation rates (lbm_gpu_box_set_slice_omega)
  float*       slice_omega_f = nullptr;
  double*      slice_src     = nullptr;  // per-z-slice Poisson sources (lbm_gpu_box_set_slice_kappa)
  float*       slice_src_f   = nullptr;
  void*        mom   = nullptr;
  double*      partials = nullptr;     // residual partials (one per step block and variable)
  double*      partials_mm = nullptr;  // mass / momentum partials
  double*      partials_mid = nullptr; // first-level residual sums (kMidBlocks per variable)
  double*      out   = nullptr;
  double*      f64   = nullptr;  // FP64 staging for transfers (Q x ncells)
  int          res_ready = 0;  // partials hold the residual of the last step
  int          mom_valid = 0;  // mom holds the moments of the last step
  int          tuned_tpb = 128;
  int32_t*     bnd_list  = nullptr;  // cells the odd step resolves link by link; XFACE cells last
  int64_t      n_bnd     = 0;
  int64_t      n_bnd_lean = 0;       // leading entries without the XFACE / SFACE cells (per-thread odd kernel)
  int64_t      n_sface    = 0;       // SFACE cells (free-slip face cells the face blocks step)
  int64_t      face_ny_part = 0;     // face positions on the y faces, then
  int64_t      face_n       = 0;     // all face positions (y faces, then z faces)
  int32_t*     link_src  = nullptr;  // n_bnd x Q pull slots of the boundary cells
  int32_t*     link_dst  = nullptr;  // n_bnd x Q push slots (-1: leaves the box)
  double*      corr_src  = nullptr;  // moving-wall terms (allocated only when a wall moves)
  double*      corr_dst  = nullptr;
  int64_t      res_slots = 0;        // partial slots written by the last residual step
  int          kind_even = 0;        // lbm_box_kernel of the even steps: per-thread, staged (box_tma.cu) or paired
  int          kind_odd  = 0;        // and of the odd steps
  int*         d_err     = nullptr;  // set by a staged kernel whose bounded wait ran out
  // bounded waits of the staged kernel: the limit of each wait, and the
  // test-only starvation switch (the first segment of every CTA is never
  // armed, so its wait runs out); see lbm_gpu_box_test_wait
  uint64_t     wait_limit_ns = 500000000ull;
  int          wait_starve   = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one-step graphs for even and odd parity
};

cudaError_t box_initial_condition(BoxState* b, cudaStream_t s);
int         box_step(BoxState* b, int64_t nsteps, cudaStream_t s, std::string& err);
int         box_residual(BoxState* b, double* r, cudaStream_t s, std::string& err);
int         box_get_populations(BoxState* b, double* f, cudaStream_t s, std::string& err);
int         box_set_populations(BoxState* b, const double* f, cudaStream_t s, std::string& err);
int         box_mass_momentum(BoxState* b, double* out, cudaStream_t s, std::string& err);
int         box_info(const BoxState* b, int64_t* ncells, int32_t* q, int32_t* nvar);
void        box_destroy(BoxState* b);
// bulk-copy staged bulk kernel (box_tma.cu): whether the box qualifies, and
// the launch; *slots = residual partial slots the launch writes
bool        box_tma_supported(const BoxState* b);
cudaError_t box_tma_bulk(BoxState* b, bool odd, int mom, cudaStream_t s, int64_t* slots);
// row-staged bulk kernel (box_rows.cu): whether the box qualifies, and the
// launch (mom: 0 plain step, 1 / 2 the two halves of a residual step; *nbulk
// gets the residual slots it writes).  Its odd step must run before the
// boundary kernel: it writes back the unchanged slots of the cells it does
// not step.
bool        box_rows_supported(const BoxState* b);
// whether the row-staged kernel reads its XFACE outlet cells' upstream
// values from its staged rows (then the ghost fill skips those cells)
bool        box_rows_outlet_inline(const BoxState* b);
cudaError_t box_rows_bulk(BoxState* b, bool odd, int mom, cudaStream_t s, int64_t* nbulk);

}  // namespace lbm

// context plumbing shared with capi.cu
lbm_gpu_ctx*   lbm_internal_new_box_ctx(int device, lbm::BoxState* box, cudaStream_t stream);
lbm::BoxState* lbm_internal_box(lbm_gpu_ctx* ctx);
cudaStream_t   lbm_internal_stream(lbm_gpu_ctx* ctx);
void           lbm_internal_set_error(lbm_gpu_ctx* ctx, const std::string& msg);
