/*
 * lbm_gpu.h -- C ABI of the GB300 (sm_103a) lattice-Boltzmann time step.
 *
 * This is the drop-in boundary for the hot path of the SFCMM/LBM reference.
 * The reference has no plugin or FFI layer: its time step is the private
 * method LBMSolver<DEBUG,LBTYPE,EQ>::timeStep() (src/lbm/solver.cpp:306-320)
 * and the boundary conditions are LBMBndInterface objects driven through
 * std::function accessors (src/lbm/bnd/bnd_interface.h:7-24).  The entry
 * points below replace those, one for one, and are what a GPU branch inside
 * LBMSolver::run() calls:
 *
 *   lbm_gpu_create            <- LBMSolver::transferGrid + loadConfiguration
 *                                (src/lbm/solver.cpp:758-801, :70-163)
 *   lbm_gpu_add_boundary      <- LBMBndManager::setupBndryCnds, one BC object
 *                                (src/lbm/bnd/bnd.h:71-279)
 *   lbm_gpu_set_forcing       <- the pressure "forcing" set-up
 *                                (src/lbm/solver.cpp:625-648)
 *   lbm_gpu_initial_condition <- LBMSolver::initialCondition (solver.cpp:266-295)
 *   lbm_gpu_step              <- n x LBMSolver::timeStep (solver.cpp:306-320)
 *   lbm_gpu_residual          <- LBMSolver::sumAbsDiff for every variable
 *                                (solver.cpp:808-815, used at :232-263)
 *   lbm_gpu_update_moments    <- LBMSolver::updateMacroscopicValues (:512-553)
 *   lbm_gpu_get_vars          <- read of m_vars (output(), :322-384)
 *   lbm_gpu_get/set_populations <- read/write of m_fold (solver.h:206-210)
 *
 * Conventions: all host arrays are caller-owned, read or written only during
 * the call, and laid out as in the reference (cell-major AoS, curve order:
 * fold[cell*Q + dist], vars[cell*NVAR + var], nghbr[cell*NNGHBR + dir]).  Every
 * call is synchronous with respect to the host arrays it takes.  Every entry
 * point returns LBM_OK (0) or a negative lbm_status; the text of the last
 * error of a context is available from lbm_gpu_last_error().  Nothing traps on
 * the device: device-side failures are reported through the status.  One host
 * thread per context; a context is not re-entrant.
 */
#ifndef LBM_GPU_H
#define LBM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_GPU_ABI_VERSION 1

typedef enum lbm_status {
  LBM_OK              = 0,
  LBM_ERR_INVALID     = -1, /* bad argument */
  LBM_ERR_UNSUPPORTED = -2, /* valid in the reference's schema, not implemented here */
  LBM_ERR_TABLE       = -3, /* inconsistent neighbour / boundary tables */
  LBM_ERR_CUDA        = -4, /* CUDA runtime error (message in lbm_gpu_last_error) */
  LBM_ERR_DIVERGED    = -5, /* NaN/Inf in the state */
  LBM_ERR_TIMEOUT     = -6, /* a bounded device wait expired */
  LBM_ERR_NOMEM       = -7
} lbm_status;

/* lattices (src/lbm/constants.h:112; D3Q7 is new) */
typedef enum lbm_lattice { LBM_D1Q3 = 0, LBM_D2Q5 = 1, LBM_D2Q9 = 2, LBM_D3Q7 = 3, LBM_D3Q19 = 4 } lbm_lattice;
/* equations (src/lbm/constants.h:29) */
typedef enum lbm_equation { LBM_NAVIER_STOKES = 0, LBM_POISSON = 1 } lbm_equation;

/* boundary-condition classes of src/lbm/bnd/ (dispatch in bnd.h:71-279) */
typedef enum lbm_bnd_kind {
  LBM_BND_PERIODIC           = 1,  /* LBMBnd_Periodic, generateBndry=true (bnd_periodic.h:174-215) */
  LBM_BND_WALL_BB            = 2,  /* LBMBnd_wallBB<false> (bnd_wall.h:8-95) */
  LBM_BND_WALL_BB_TANGENTIAL = 3,  /* LBMBnd_wallBB<true>, scalar = tangentialVelocity */
  LBM_BND_DIRICHLET_BB       = 4,  /* LBMBnd_DirichletBB, vec = value (bnd_dirichlet.h:20-127) */
  LBM_BND_WALL_EQ            = 5,  /* LBMBnd_wallEq (bnd_wall.h:100-177), vec = velocity if has_vec */
  LBM_BND_WALL_NEEM          = 6,  /* LBMBnd_wallNEEM (bnd_wall.h:182-304) */
  LBM_BND_WALL_NEBB          = 7,  /* LBMBnd_wallNEBB, D2Q9 only (bnd_wall.h:312-479) */
  LBM_BND_PRESSURE_ABB       = 8,  /* LBMBnd_Pressure, scalar = pressure (bnd_pressure.h:11-113) */
  LBM_BND_DIRICHLET_NEEM     = 9,  /* LBMBnd_DirichletNEEM, Poisson (bnd_dirichlet.h:250-394) */
  LBM_BND_NEUMANN_NEEM       = 10  /* LBMBnd_NeumannNEEM, Poisson (bnd_neumann.h:15-66) */
} lbm_bnd_kind;

typedef struct lbm_gpu_ctx lbm_gpu_ctx;

/* Reference-table engine: the solver's own cell list and neighbour table. */
typedef struct lbm_table_desc {
  int32_t lattice;     /* lbm_lattice: D1Q3, D2Q5 or D2Q9 (the lattices LBMSolverExecutor builds) */
  int32_t equation;    /* lbm_equation */
  int64_t ncells;      /* grid().totalSize() */
  int32_t nnghbr;      /* neighbours per cell in nghbr: 2 (1D) or 8 (2D, diagonals appended) */
  int32_t device;      /* CUDA device ordinal */
  double  omega;       /* m_omega */
  double  relax_time;  /* m_relaxTime */
  double  dt;          /* m_dt */
  double  poisson_k;   /* Poisson source coefficient (27.79 or equation_th) */
  double  bbox[6];     /* grid bounding box min0,max0,min1,max1,min2,max2 */
  double  cell_length; /* cell length on the finest level */
} lbm_table_desc;

/* One boundary-condition object, as LBMBndManager builds it. */
typedef struct lbm_bnd_desc {
  int32_t        kind;         /* lbm_bnd_kind */
  int32_t        has_vec;      /* JSON carried "velocity" (wall eq/neem/nebb) */
  int32_t        has_pressure; /* periodic surface carries "pressure" */
  int32_t        reserved;
  int64_t        ncells;       /* Surface::getCellList().size() */
  const int64_t* cells;        /* Surface::getCellList() */
  const double*  normals;      /* ncells x ndim, Surface::normal_p(cell) */
  const double*  values;       /* ncells Dirichlet values (NEEM) or NULL */
  double         vec[3];       /* wall velocity / Dirichlet vector value */
  double         scalar;       /* pressure, tangential velocity, or constant Dirichlet value */
  int64_t        nconn;        /* periodic: connected surface */
  const int64_t* conn_cells;
  const double*  conn_normals;
} lbm_bnd_desc;

int lbm_gpu_abi_version(void);

/* Create a context on the reference's tables.  nghbr: ncells x nnghbr int64
 * (CartesianGrid::neighbor, -1 = none); centers: ncells x ndim. */
int lbm_gpu_create(const lbm_table_desc* desc, const int64_t* nghbr, const double* centers, lbm_gpu_ctx** out);
/* Append one BC object; call in the reference's application order. */
int lbm_gpu_add_boundary(lbm_gpu_ctx* ctx, const lbm_bnd_desc* bnd);
/* Pressure forcing between the inlet (cube_-x) and outlet (cube_+x) lists. */
int lbm_gpu_set_forcing(lbm_gpu_ctx* ctx, double pressure_gradient, int64_t nin, const int64_t* inlet_cells, int64_t nout,
                        const int64_t* outlet_cells);
/* vars = 0, BC initCnd, populations = equilibrium (initialCondition). */
int lbm_gpu_initial_condition(lbm_gpu_ctx* ctx);
/* Advance n time steps (captured as a CUDA graph). */
int lbm_gpu_step(lbm_gpu_ctx* ctx, int64_t nsteps);
/* r[v] = sum_cells |vars - varsold| for v < NVAR, double precision. */
int lbm_gpu_residual(lbm_gpu_ctx* ctx, double* r);
/* vars <- moments(fold) */
int lbm_gpu_update_moments(lbm_gpu_ctx* ctx);
int lbm_gpu_get_vars(lbm_gpu_ctx* ctx, double* vars);
int lbm_gpu_set_vars(lbm_gpu_ctx* ctx, const double* vars);
int lbm_gpu_get_varsold(lbm_gpu_ctx* ctx, double* varsold);
/* post-stream populations fold (m_fold), ncells x Q AoS */
int lbm_gpu_get_populations(lbm_gpu_ctx* ctx, double* fold);
int lbm_gpu_set_populations(lbm_gpu_ctx* ctx, const double* fold);
/* out[0] = sum rho-like zeroth moment, out[1..ndim] = sum of momentum, FP64 */
int lbm_gpu_reduce_mass_momentum(lbm_gpu_ctx* ctx, double* out);
int lbm_gpu_synchronize(lbm_gpu_ctx* ctx);
int lbm_gpu_info(const lbm_gpu_ctx* ctx, int64_t* ncells, int32_t* q, int32_t* nvar);
const char* lbm_gpu_last_error(const lbm_gpu_ctx* ctx);
void        lbm_gpu_destroy(lbm_gpu_ctx* ctx);

/* Residual without any device allocation.  No counterpart in the reference:
 * it serves callers that cannot call cudaMalloc -- code whose device memory
 * belongs to another allocator (a framework's caching allocator, a fixed
 * arena) and latency-critical code that cannot afford cudaMalloc's implicit
 * synchronisation.  It computes out[v] = sum_i |vars[v*ncells+i] -
 * varsold[v*ncells+i]| for v < nvar, the convergence residual of
 * lbm_gpu_residual, on caller-owned DEVICE arrays, variable-major, writing
 * nvar doubles to the DEVICE array `out`, asynchronously on `stream` (a
 * cudaStream_t; NULL = legacy default stream) of the current device.
 * Scratch: a fixed array in the library's device image (304 x
 * LBM_GPU_NOALLOC_MAX_VARS doubles per GPU, kept until the process exits),
 * shared by every call: calls that overlap on the GPU race.  nvar above
 * LBM_GPU_NOALLOC_MAX_VARS is rejected with LBM_ERR_INVALID.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture (a first call inside a
 * capture returns LBM_ERR_INVALID).  Calls outside capture look the address
 * up again, so the entry point stays valid across a device reset; a call
 * inside a capture uses the address of the last call outside one. */
#define LBM_GPU_NOALLOC_MAX_VARS 8
int lbm_gpu_residual_noalloc(const double* vars, const double* varsold, int64_t ncells, int32_t nvar, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
