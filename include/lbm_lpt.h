/* Lagrangian particles on the GPU (C ABI): the particle step of the SFCMM/LBM
 * reference's LPT solver, and its coupling to the LBM velocity field.
 *
 *   entry point              reference counterpart
 *   lbm_lpt_create           LPTSolver::loadConfiguration / setMethods / setForceModel
 *                            (src/lpt/solver.cpp:94-228): constants, force model, integrator
 *   lbm_lpt_set_particles    the particle array m_vars after initialCondition (src/lpt/solver.h:204,
 *                            layout src/lpt/particle.h:11-36)
 *   lbm_lpt_step             LPTSolver::timeStep (src/lpt/solver.cpp:335-347): calcA, then
 *                            timeIntegration (solver.cpp:356-496) with the models of src/lpt/forces.h
 *   lbm_lpt_get_particles    m_vars
 *   lbm_lpt_couple_box       no counterpart: the reference's particles see a constant ambient
 *                            velocity (v_infty); coupled, they see the velocity of the dense-box
 *                            LBM engine's last step at their cell
 *
 * Particle layout (the reference's "Normal" particle, per particle 3*ndim+5
 * doubles): center[ndim], velocity[ndim], a[ndim], radius, density,
 * temperature, volume, DC.  Temperature and volume are carried unchanged.
 * The step matches the reference bit for bit (IEEE doubles, the reference's
 * operation order, no contraction), except the Putnam drag factor's power
 * Re^(2/3) for 0.1 < Re <= 1000, which the reference takes from gcem and this
 * library from CUDA's pow.  Particle generation (injection) stays on the
 * host, as in the reference; new particles enter through
 * lbm_lpt_set_particles.
 *
 * Status codes are those of lbm_gpu.h; all calls are synchronous.
 */
#ifndef LBM_LPT_H
#define LBM_LPT_H

#include <stdint.h>

#include "lbm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* force models, in the order of force::Model (src/lpt/forces.h) */
typedef enum lbm_lpt_model {
  LBM_LPT_RATIO_GRAV                 = 0,
  LBM_LPT_RATIO_GRAV_STOKES_DRAG     = 1,
  LBM_LPT_RATIO_GRAV_NLIN_DRAG       = 2,
  LBM_LPT_RATIO_GRAV_BUO             = 3,
  LBM_LPT_RATIO_GRAV_BUO_STOKES_DRAG = 4, /* the reference's default */
  LBM_LPT_RATIO_GRAV_BUO_NLIN_DRAG   = 5,
  LBM_LPT_AMB_GRAV_BUO               = 6,
  LBM_LPT_AMB_GRAV_BUO_STOKES_DRAG   = 7,
  LBM_LPT_AMB_GRAV_BUO_NLIN_DRAG     = 8
} lbm_lpt_model;

typedef enum lbm_lpt_integration { LBM_LPT_FORWARD_EULER = 0, LBM_LPT_IMPLICIT_EULER = 1 } lbm_lpt_integration;

typedef struct lbm_lpt_desc {
  int32_t ndim;        /* 2 or 3 */
  int32_t model;       /* lbm_lpt_model */
  int32_t integration; /* lbm_lpt_integration */
  int32_t device;
  int64_t capacity;    /* particles at most */
  double  dt;          /* "dt" */
  double  gravity[3];  /* "gravity" */
  double  rho_ambient; /* "rho_infty" (reference default 1.205) */
  double  nu_ambient;  /* "nu_infty" (reference default 1.82e-5) */
  double  v_ambient[3]; /* "v_infty" */
} lbm_lpt_desc;

typedef struct lbm_lpt_ctx lbm_lpt_ctx;

int lbm_lpt_create(const lbm_lpt_desc* desc, lbm_lpt_ctx** out);
/* n particles in the reference's layout (n x (3*ndim+5) doubles) */
int lbm_lpt_set_particles(lbm_lpt_ctx* ctx, int64_t n, const double* vars);
int lbm_lpt_get_particles(lbm_lpt_ctx* ctx, double* vars);
int64_t lbm_lpt_count(const lbm_lpt_ctx* ctx);
/* nsteps particle steps, in one launch (each particle's state stays in
 * registers from the first step to the last) */
int lbm_lpt_step(lbm_lpt_ctx* ctx, int64_t nsteps);
/* Take the ambient velocity from a dense-box LBM context (lbm_gpu_create_box,
 * Navier-Stokes): the velocity its last step call left in its moments, at
 * the cell that holds the particle (cell (i,j,k) spans origin + [i,i+1) *
 * cell_length along each axis; positions outside the box use the nearest
 * cell), times velocity_scale (lattice to physical units).  NULL box: back
 * to the constant ambient velocity.  The box must have run a step call, and
 * must outlive the coupling. */
int lbm_lpt_couple_box(lbm_lpt_ctx* ctx, lbm_gpu_ctx* box, const double* origin, double cell_length, double velocity_scale);
const char* lbm_lpt_last_error(const lbm_lpt_ctx* ctx);
void lbm_lpt_destroy(lbm_lpt_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* LBM_LPT_H */
