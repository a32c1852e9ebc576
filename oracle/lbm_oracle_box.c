/* box engine: filled in below */
#include "lbm_oracle.h"
#include <stddef.h>
ora_box* ora_box_create(int lattice, int equation, int nx, int ny, int nz, double omega, const uint8_t* flags, const int* periodic,
                        const int* freeslip, const double* body_force, const double* inlet_velocity, double inlet_density,
                        double lid_velocity) {
  (void)lattice; (void)equation; (void)nx; (void)ny; (void)nz; (void)omega; (void)flags; (void)periodic; (void)freeslip;
  (void)body_force; (void)inlet_velocity; (void)inlet_density; (void)lid_velocity;
  return NULL;
}
void ora_box_destroy(ora_box* b) { (void)b; }
int ora_box_set_poisson(ora_box* b, double kappa_sq, int nonlinear, const double* phi) { (void)b; (void)kappa_sq; (void)nonlinear; (void)phi; return -1; }
void ora_box_init_equilibrium(ora_box* b, double rho, const double* u) { (void)b; (void)rho; (void)u; }
void ora_box_step(ora_box* b, int64_t nsteps, int nthreads) { (void)b; (void)nsteps; (void)nthreads; }
void ora_box_get(const ora_box* b, double* f, double* rho, double* u) { (void)b; (void)f; (void)rho; (void)u; }
void ora_box_set(ora_box* b, const double* f) { (void)b; (void)f; }
