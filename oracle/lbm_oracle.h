/*
 * CPU oracle for the SFCMM/LBM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * LBM step (src/lbm/solver.cpp and the headers in src/lbm/bnd/) used by tests/, by
 * __graft_entry__.smoke() and by the CPU-baseline legs of bench.py as the
 * checker the CUDA library is compared against.  The product never links it.
 *
 * Two engines live here:
 *   - the "table" engine restates the reference solver on the reference's own
 *     cell list and neighbour table, with every boundary-condition class the
 *     reference's JSON dispatcher can build (src/lbm/bnd/bnd.h:71-279).  It is
 *     pinned bit-for-bit against the reference built from source
 *     (oracle/build_ref.sh, tests/golden/).
 *   - the "box" engine (lbm_oracle_box.c) restates the same BGK update on a
 *     dense box with the features the reference lacks (D3Q19 neighbours
 *     computed from coordinates, Guo forcing, equilibrium inlet, zero-gradient
 *     outlet, free slip, D3Q7 Poisson-Boltzmann).  Its 2D/no-forcing limit is
 *     checked against the table engine.
 *
 * Enumerations mirror include/lbm_gpu.h value for value.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_ctx ora_ctx;

/* lattices and equations, same values as include/lbm_gpu.h */
enum { ORA_D1Q3 = 0, ORA_D2Q5 = 1, ORA_D2Q9 = 2, ORA_D3Q7 = 3, ORA_D3Q19 = 4 };
enum { ORA_NAVIER_STOKES = 0, ORA_POISSON = 1 };

/* boundary-condition kinds, same values as include/lbm_gpu.h */
enum {
  ORA_BND_PERIODIC = 1,
  ORA_BND_WALL_BB = 2,
  ORA_BND_WALL_BB_TANGENTIAL = 3,
  ORA_BND_DIRICHLET_BB = 4,
  ORA_BND_WALL_EQ = 5,
  ORA_BND_WALL_NEEM = 6,
  ORA_BND_WALL_NEBB = 7,
  ORA_BND_PRESSURE_ABB = 8,
  ORA_BND_DIRICHLET_NEEM = 9,
  ORA_BND_NEUMANN_NEEM = 10
};

/* Create a table-engine context.  nghbr is ncells x nnghbr (reference layout,
 * neighbor(cell,dir) = nghbr[cell*nnghbr+dir], -1 = missing), centers is
 * ncells x ndim, bbox is (min0,max0,min1,max1,...).  Returns NULL on error. */
ora_ctx* ora_create(int lattice, int equation, int64_t ncells, double omega, double relax_time, double dt, double poisson_k,
                    const int64_t* nghbr, int nnghbr, const double* centers, const double* bbox, double cell_length);
void ora_destroy(ora_ctx* c);

/* Add one boundary-condition object (JSON order).  values: per-cell scalar
 * values (Dirichlet NEEM) or NULL; vec: ndim velocity/value or NULL;
 * has_vec: the JSON carried "velocity"; scalar: pressure or tangential
 * velocity; has_pressure: periodic surface carries "pressure"; conn_*: the
 * connected surface of a periodic BC.  Returns 0 or a negative code. */
int ora_add_bnd(ora_ctx* c, int kind, int64_t ncells, const int64_t* cells, const double* normals, const double* values, const double* vec,
                int has_vec, double scalar, int has_pressure, int64_t nconn, const int64_t* conn_cells, const double* conn_normals);

/* Pressure "forcing" of src/lbm/solver.cpp:625-696 between the cube_-x (inlet)
 * and cube_+x (outlet) surfaces. */
int ora_set_forcing(ora_ctx* c, double pressure_gradient, int64_t nin, const int64_t* in_cells, int64_t nout, const int64_t* out_cells);

void ora_initial_condition(ora_ctx* c);
void ora_step(ora_ctx* c, int64_t nsteps);
/* recompute vars from the current fold (updateMacroscopicValues) */
void ora_update_moments(ora_ctx* c);
void ora_residual(const ora_ctx* c, double* r);
/* any pointer may be NULL; arrays are AoS cell-major as in the reference */
void ora_get(const ora_ctx* c, double* fold, double* f, double* vars, double* varsold);
void ora_set_state(ora_ctx* c, const double* fold, const double* vars);
int ora_nvar(const ora_ctx* c);
int ora_ndist(const ora_ctx* c);

/* ---------------- box engine (lbm_oracle_box.c) ---------------- */

/* per-cell flag byte of a dense box, same values as include/lbm_gpu.h */
enum { ORA_CELL_FLUID = 0, ORA_CELL_SOLID = 1, ORA_CELL_INLET = 2, ORA_CELL_OUTLET = 3, ORA_CELL_DIRICHLET = 4 };

typedef struct ora_box ora_box;

/* Dense box nx*ny*nz (nz=1, ny=1 for lower dimensions), x fastest.
 * face[6]: treatment of the -x,+x,-y,+y,-z,+z faces (wall, periodic, free
 * slip, open; the values of include/lbm_gpu_box.h), wall_u: 6x3 wall
 * velocities, flags: per-cell flag bytes (NULL = all fluid), body_force:
 * Guo forcing. */
ora_box* ora_box_create(int lattice, int equation, int nx, int ny, int nz, double omega, const uint8_t* flags, const int* face,
                        const double* wall_u, const double* body_force, const double* inlet_velocity, double inlet_density);
void ora_box_destroy(ora_box* b);
/* Poisson-Boltzmann: phi_dirichlet per cell for CELL_DIRICHLET cells,
 * kappa^2 and the sinh nonlinearity switch. */
int ora_box_set_poisson(ora_box* b, double kappa_sq, int nonlinear, const double* phi_dirichlet);
void ora_box_init_equilibrium(ora_box* b, double rho, const double* u);
/* hold Navier-Stokes populations as deviations f - w (call before init) */
int ora_box_set_deviation(ora_box* b, int on);
void ora_box_step(ora_box* b, int64_t nsteps, int nthreads);
/* post-stream populations (SoA, q-major: f[q*ncells+cell]) and moments */
void ora_box_get(const ora_box* b, double* f_soa, double* rho, double* u);
void ora_box_set(ora_box* b, const double* f_soa);

#ifdef __cplusplus
}
#endif
#endif
