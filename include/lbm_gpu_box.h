/*
 * lbm_gpu_box.h -- C ABI of the dense-box engine of the GB300 LBM library.
 *
 * The reference stores its uniform grid as a curve-ordered cell list with an
 * int64 neighbour table (src/cartesiangrid.h:111-124).  For a uniform box the
 * same time step (LBMSolver::timeStep, src/lbm/solver.cpp:306-320) needs no
 * table at all: neighbours follow from coordinates, and a flag byte per cell
 * (fluid / solid / inlet / outlet / Dirichlet) carries the geometry.  This
 * header is the entry point for that layout: it is what the reference's
 * LBMSolver calls when its grid is a single uniform level (every test case
 * and every synthetic benchmark domain), and it is the only form in which the
 * features the reference lacks are available (D3Q19, D3Q7 Poisson-Boltzmann,
 * Guo body forcing, equilibrium inlet, zero-gradient outlet, free slip,
 * reduced-precision storage).
 *
 * Populations live on the device as q-major planes in the chosen storage and
 * stream in place with the AA pattern.  Transfers use FP64 SoA host arrays:
 * f[q * ncells + cell], cell = x + nx * (y + ny * z).  The context type and
 * every other entry point (step, residual, mass/momentum, destroy, errors) are
 * those of lbm_gpu.h.
 */
#ifndef LBM_GPU_BOX_H
#define LBM_GPU_BOX_H

#include <stdint.h>

#include "lbm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* population storage */
typedef enum lbm_storage {
  /* Navier-Stokes populations are held as the scaled deviation
   * v_i = (f_i - w_i) / w_i * 2^12 (FP64 storage) or as that deviation
   * shifted to the free stream, s_i = v_i - k_i (FP32 / FP16 / BF16 storage),
   * k_i the scaled deviation of the equilibrium at rho = 1 and the
   * free-stream velocity U: the inlet velocity where the box has inlet
   * cells, else the initial velocity, when it points along x (else U = 0).
   * The single-precision collision works on s_i, so that near the free
   * stream both the stored values and every intermediate are small numbers
   * with FP16's / FP32's relative rounding.  Poisson populations are held as
   * f_i.  See lbm_box_desc.no_shift. */
  LBM_STORE_F64     = 0, /* FP64 storage, FP64 arithmetic (the plain method) */
  LBM_STORE_F32     = 1, /* FP32 storage, FP32 arithmetic */
  LBM_STORE_F16_DEV = 2, /* FP16 storage, FP32 arithmetic */
  LBM_STORE_BF16_DEV = 3, /* BF16 storage, FP32 arithmetic */
  /* A 16-bit float of 1 sign, 3 exponent and 12 mantissa bits (13
   * significant bits) holding s_i / 1024: normal from 2^-6 to 2 - 2^-12,
   * evenly spaced (2^-18) below, rounded to nearest even, saturating at the
   * largest magnitude (no infinities or NaNs: a diverging state saturates).
   * Two more significant bits than FP16 over the range the shifted state
   * occupies, at the same bytes; FP32 arithmetic.  Navier-Stokes only. */
  LBM_STORE_E3M12_DEV = 4
} lbm_storage;

/* treatment of a face of the box */
typedef enum lbm_face {
  LBM_FACE_WALL     = 0, /* halfway bounce-back, optionally moving (wall_velocity) */
  LBM_FACE_PERIODIC = 1, /* wrap to the opposite face (both faces of the axis) */
  LBM_FACE_FREESLIP = 2, /* specular reflection */
  LBM_FACE_OPEN     = 3  /* -x: equilibrium inlet plane, +x: zero-gradient outlet plane */
} lbm_face;

/* per-cell flag byte */
typedef enum lbm_cell_flag {
  LBM_CELL_FLUID     = 0,
  LBM_CELL_SOLID     = 1, /* bounce-back obstacle, not updated */
  LBM_CELL_INLET     = 2, /* emits the equilibrium at (inlet_density, inlet_velocity) */
  LBM_CELL_OUTLET    = 3, /* fluid cell whose links from beyond +x copy the upstream cell */
  LBM_CELL_DIRICHLET = 4  /* Poisson: emits the equilibrium at its fixed potential */
} lbm_cell_flag;

typedef struct lbm_box_desc {
  int32_t lattice;          /* LBM_D2Q9, LBM_D3Q19 (Navier-Stokes) or LBM_D3Q7 (Poisson-Boltzmann) */
  int32_t equation;         /* LBM_NAVIER_STOKES or LBM_POISSON */
  int32_t storage;          /* lbm_storage */
  int32_t device;
  int32_t nx, ny, nz;       /* nz = 1 for D2Q9 */
  int32_t face[6];          /* lbm_face of -x,+x,-y,+y,-z,+z */
  double  omega;            /* 1/tau */
  double  wall_velocity[6][3];
  double  body_force[3];    /* Guo forcing, lattice units */
  double  inlet_density;
  double  inlet_velocity[3];
  double  init_density;     /* initial equilibrium */
  double  init_velocity[3];
  double  kappa_sq;         /* Poisson-Boltzmann: nabla^2 phi = kappa^2 sinh(phi) (or kappa^2 phi) */
  int32_t pb_nonlinear;     /* 1: sinh, 0: linear Debye-Hueckel */
  int32_t no_shift;         /* 1: U = 0 (the single-precision storages hold v_i itself); 0 (default): the free stream */
} lbm_box_desc;

/* flags: ncells bytes (NULL = all fluid); dirichlet: ncells potentials of the
 * LBM_CELL_DIRICHLET cells (Poisson) or NULL. */
int lbm_gpu_create_box(const lbm_box_desc* desc, const uint8_t* flags, const double* dirichlet, lbm_gpu_ctx** out);

/* Macroscopic fields of the current state, FP64 host arrays of ncells:
 * rho (or phi for Poisson) and ux, uy, uz (NULL to skip). */
int lbm_gpu_box_moments(lbm_gpu_ctx* ctx, double* rho, double* ux, double* uy, double* uz);

/* Moments of n listed cells of the current state (line probes and other
 * point samples, the cells of PostprocessCartesianFunctionLine,
 * src/postprocess/postprocessing_cartesian.h:17-39, whose values
 * src/postprocess/postprocessing.h:98-115 writes to line.csv): out[i * nvar + k]
 * with k = 0 rho (phi for Poisson) and k = 1.. the velocity components; the
 * values equal lbm_gpu_box_moments at those cells bit for bit.  Only the n
 * cells are read on the device.  LBM_ERR_INVALID for an index outside the box. */
int lbm_gpu_box_probe(lbm_gpu_ctx* ctx, const int64_t* cells, int64_t n, double* out);

/* Threads per block the autotuner chose for the per-thread step kernel. */
int lbm_gpu_box_autotune(lbm_gpu_ctx* ctx, int32_t* threads_per_block);
/* Bulk step kernel of a box context: LBM_BOX_KERNEL_THREAD (one cell per
 * thread, one global load per population), LBM_BOX_KERNEL_STAGED (each CTA
 * stages row segments in shared memory with bulk copies and stores straight
 * to global memory), LBM_BOX_KERNEL_PAIRED (two x-adjacent cells per thread,
 * 2-element loads and stores where aligned) or LBM_BOX_KERNEL_ROWS (each
 * stage holds one whole x-row; bulk copies load it and store it back, the
 * cells update it in place in shared memory); lbm_gpu_create_box picks the
 * fastest by timing them.  All give bit-identical results.  kernel < 0 only
 * queries.  LBM_ERR_UNSUPPORTED when the box does not qualify: staging needs
 * nx times the storage size to be a multiple of 16 bytes (row staging also
 * nx <= 1024 and, for FP64 D3Q19, nx <= 512); pairing needs nx even and a
 * 32- or 16-bit storage. */
typedef enum lbm_box_kernel {
  LBM_BOX_KERNEL_THREAD = 0,
  LBM_BOX_KERNEL_STAGED = 1,
  LBM_BOX_KERNEL_PAIRED = 2,
  LBM_BOX_KERNEL_ROWS   = 3
} lbm_box_kernel;
int lbm_gpu_box_select_kernel(lbm_gpu_ctx* ctx, int32_t kernel, int32_t* selected);
/* The autotuner times even (local) and odd (streaming) steps separately and
 * may pick a different kernel for each: the kernels of both parities
 * (lbm_gpu_box_select_kernel sets both, and reports -1 when they differ). */
int lbm_gpu_box_kernels(lbm_gpu_ctx* ctx, int32_t* even, int32_t* odd);

/* Navier-Stokes boxes: a relaxation rate per z-slice (omega[z], 0 < omega < 2,
 * n = nz values), so that the independent 2D slices of a D2Q9 box are a
 * sweep over Reynolds number (and geometry) stepped by one launch per step;
 * omega = NULL restores the box's single rate.  Every slice then steps
 * exactly as a box of its own with that rate.  The reference builds one
 * solver per configuration (src/lbm/solverExe.h:17-93); this has no
 * counterpart there.  LBM_ERR_UNSUPPORTED for Poisson boxes. */
int lbm_gpu_box_set_slice_omega(lbm_gpu_ctx* ctx, const double* omega, int32_t n);

/* Poisson-Boltzmann boxes: a kappa^2 per z-slice (kappa_sq[z] >= 0, n = nz
 * values), so that boxes stacked along z, each closed by planes of
 * LBM_CELL_DIRICHLET cells (which emit their own equilibrium whatever they
 * receive), are a sweep over Debye length 1/kappa (and charge placement)
 * stepped by one launch per step; kappa_sq = NULL restores the box's
 * single kappa^2.  Each stacked box then steps exactly as a box of its own
 * with its kappa^2.  Like the rate sweep, this has no counterpart in the
 * reference.  LBM_ERR_UNSUPPORTED for Navier-Stokes boxes. */
int lbm_gpu_box_set_slice_kappa(lbm_gpu_ctx* ctx, const double* kappa_sq, int32_t n);

/* TEST ONLY.  The staged kernels' (LBM_BOX_KERNEL_STAGED and
 * LBM_BOX_KERNEL_ROWS) pipeline waits are bounded (0.5 s each);
 * when one runs out the kernel records a flag, lets its copies in flight
 * land and returns, and the step call reports LBM_ERR_TIMEOUT (the state of
 * that step is invalid; re-initialise or reload it).  This sets the limit of
 * each wait (1 ns .. 0.5 s) and, with starve = 1, makes every CTA leave its
 * first segment unarmed, so the waits on it run out: a device-side timeout
 * without a fault.  starve = 0 and limit 500000000 restore the defaults.  No
 * counterpart in the reference, which has no device waits. */
int lbm_gpu_box_test_wait(lbm_gpu_ctx* ctx, int64_t limit_ns, int32_t starve);

/* Run nsteps exactly as lbm_gpu_step does (captured per-parity graphs, the
 * last two steps recording the residual) with one CUDA event pair around the
 * whole sequence on the context's stream: *ms is its device time. */
int lbm_gpu_box_time_steps(lbm_gpu_ctx* ctx, int64_t nsteps, double* ms);
/* Run nsteps exactly as lbm_gpu_step does, but with a CUDA event pair around
 * every launch of the step kernel on the context's stream: total_ms is the
 * device time of the whole sequence, kernel_ms the summed duration of the
 * step-kernel launches, launches their count (any pointer may be NULL). */
int lbm_gpu_box_profile_steps(lbm_gpu_ctx* ctx, int64_t nsteps, double* total_ms, double* kernel_ms, int64_t* launches);

/* ---- batched cavities --------------------------------------------------
 * Many independent D2Q9 lid-driven cavities (n x n, halfway bounce-back on
 * every wall, the +y wall moving in x at lid_velocity) advance together in one
 * persistent launch per step.  Used for parameter sweeps (Reynolds number,
 * size) that the reference runs one case at a time.  lbm_gpu_step,
 * lbm_gpu_initial_condition (rest equilibrium), lbm_gpu_info and
 * lbm_gpu_destroy apply to the returned context. */
typedef struct lbm_batch_desc {
  int32_t lattice;  /* LBM_D2Q9 */
  int32_t storage;  /* lbm_storage */
  int32_t device;
  int32_t ndomains;
  double  lid_velocity;
} lbm_batch_desc;

int lbm_gpu_create_batch(const lbm_batch_desc* desc, const int32_t* sides, const double* omegas, lbm_gpu_ctx** out);
/* res[d*3 + v]: residual (rho, ux, uy) of every cavity after the last step
 * call of at least two steps (cavities no longer active keep their last value) */
int lbm_gpu_batch_residuals(lbm_gpu_ctx* ctx, double* res);
/* Step all active cavities, checking every check_interval steps; a cavity
 * whose largest residual drops below tol stops.  steps_done[d]: steps taken.
 * A cavity whose residual is NaN/Inf stops too; the call then finishes the
 * others and returns LBM_ERR_DIVERGED, naming it in lbm_gpu_last_error. */
int lbm_gpu_batch_run(lbm_gpu_ctx* ctx, int64_t max_steps, int64_t check_interval, double tol, int64_t* steps_done);
/* per-cavity state after lbm_gpu_batch_run (reset by lbm_gpu_initial_condition) */
typedef enum lbm_batch_status {
  LBM_BATCH_ACTIVE    = 0, /* still stepping */
  LBM_BATCH_CONVERGED = 1, /* residual fell below the tolerance */
  LBM_BATCH_DIVERGED  = 2  /* residual became NaN/Inf */
} lbm_batch_status;
int lbm_gpu_batch_status(lbm_gpu_ctx* ctx, int32_t* status);
/* FP64 post-stream populations of cavity d, f[q * n*n + x + n*y] */
int lbm_gpu_batch_get_domain(lbm_gpu_ctx* ctx, int32_t d, double* f);
/* as lbm_gpu_box_profile_steps, for the batched step kernel */
int lbm_gpu_batch_profile_steps(lbm_gpu_ctx* ctx, int64_t nsteps, double* total_ms, double* kernel_ms, int64_t* launches);
/* the launch shape the autotuner chose */
int lbm_gpu_batch_tuning(lbm_gpu_ctx* ctx, int32_t* grid, int32_t* threads_per_block);

/* Bytes of one population in the chosen storage. */
int lbm_gpu_box_storage_bytes(int32_t storage);

#ifdef __cplusplus
}
#endif
#endif
