/*
 * CPU oracle, box engine: the BGK / Poisson-Boltzmann step on a dense box.
 *
 * TEST INFRASTRUCTURE ONLY (see lbm_oracle.h).  A straightforward two-array
 * restatement (collide every cell, then pull every link) of the semantics the
 * GPU machine engine implements with in-place AA streaming, so the two can be
 * compared cell by cell:
 *   - collision: the reference's BGK (src/lbm/solver.cpp:555-622) written as
 *     f + omega (feq - f), plus Guo, Zheng & Shi (2002) forcing
 *     S_q = (1 - omega/2) w_q [3 (c_q - u) + 9 (c_q . u) c_q] . F with
 *     u = (sum c f + F/2) / rho;
 *   - Poisson-Boltzmann (D3Q7): the Chai & Shi (2008) collision of
 *     src/lbm/solver.cpp:589-611 in lattice units with the source
 *     kappa^2 sinh(phi) (or kappa^2 phi);
 *   - streaming: a population arriving at cell r in direction k comes from
 *     r - c_k; through a periodic face it wraps, through a wall face or into a
 *     solid cell it is the bounced post-collision population of r itself
 *     (halfway bounce-back, src/lbm/bnd/bnd_dirichlet.h:79-121) plus
 *     6 w_k (c_k . u_wall) for a moving wall, through a free-slip face it is
 *     the mirrored population, and through the open +x face of an outlet cell
 *     it is what the upstream cell r - e_x receives (zero gradient);
 *   - inlet and Dirichlet cells emit their equilibrium every step.
 * All arithmetic is FP64.  OpenMP parallelises the cell loops; the result does
 * not depend on the thread count.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "lbm_oracle.h"

typedef struct {
  int    D, Q;
  int    c[19][3];
  int    opp[19];
  double w[19];
  double alpha;
  double pw[19];
} blat_t;

static const blat_t B_D2Q9 = {2, 9, {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {-1, 1, 0}, {0, 0, 0}},
                              {1, 0, 3, 2, 6, 7, 4, 5, 8},
                              {1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 4.0 / 9},
                              1.0 / 3.0,
                              {0}};
static const blat_t B_D3Q19 = {3,
                               19,
                               {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}, {-1, -1, 0}, {-1, 1, 0}, {1, -1, 0}, {1, 1, 0},
                                {-1, 0, -1}, {-1, 0, 1}, {1, 0, -1}, {1, 0, 1}, {0, -1, -1}, {0, -1, 1}, {0, 1, -1}, {0, 1, 1}, {0, 0, 0}},
                               {1, 0, 3, 2, 5, 4, 9, 8, 7, 6, 13, 12, 11, 10, 17, 16, 15, 14, 18},
                               {1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                                1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 3},
                               0.0,
                               {0}};
/* D3Q7 Poisson lattice: w_rest = 1/4, links 1/8, alpha = sum w c_x^2 = 1/4,
 * source weights 1/6 on the six links */
static const blat_t B_D3Q7 = {3,
                              7,
                              {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}, {0, 0, 0}},
                              {1, 0, 3, 2, 5, 4, 6},
                              {1.0 / 8, 1.0 / 8, 1.0 / 8, 1.0 / 8, 1.0 / 8, 1.0 / 8, 1.0 / 4},
                              1.0 / 4.0,
                              {1.0 / 6, 1.0 / 6, 1.0 / 6, 1.0 / 6, 1.0 / 6, 1.0 / 6, 0}};

struct ora_box {
  blat_t   L;
  int      eq;
  int      n[3];
  int64_t  ncells;
  double   omega;
  uint8_t* flags;
  int      face[6];
  double   wall_u[6][3];
  double   force[3];
  int      has_force;
  double   inlet_u[3], inlet_rho;
  double   kappa_sq;
  double*  slice_kappa; /* nz values of kappa^2 (one per z-slice) or NULL: kappa_sq */
  int      nonlinear;
  double*  dirichlet;
  int      dev;  /* Navier-Stokes state held as deviations f - w (see ora_box_set_deviation) */
  double*  f;    /* post-stream, q-major */
  double*  fs;   /* post-collision scratch */
};

enum { F_WALL = 0, F_PERIODIC = 1, F_FREESLIP = 2, F_OPEN = 3 };

/* face[6]: lbm_face of -x,+x,-y,+y,-z,+z (same values as include/lbm_gpu_box.h);
 * wall_u: 6 x 3 wall velocities */
ora_box* ora_box_create(int lattice, int equation, int nx, int ny, int nz, double omega, const uint8_t* flags, const int* face,
                        const double* wall_u, const double* body_force, const double* inlet_velocity, double inlet_density) {
  ora_box* b = (ora_box*)calloc(1, sizeof(ora_box));
  if(!b) return NULL;
  if(lattice == ORA_D2Q9) b->L = B_D2Q9;
  else if(lattice == ORA_D3Q19) b->L = B_D3Q19;
  else if(lattice == ORA_D3Q7) b->L = B_D3Q7;
  else {
    free(b);
    return NULL;
  }
  b->eq     = equation;
  b->n[0]   = nx;
  b->n[1]   = ny;
  b->n[2]   = nz;
  b->ncells = (int64_t)nx * ny * nz;
  b->omega  = omega;
  b->flags  = (uint8_t*)calloc(b->ncells, 1);
  if(flags) memcpy(b->flags, flags, b->ncells);
  for(int i = 0; i < 6; ++i) {
    b->face[i] = face ? face[i] : F_WALL;
    for(int d = 0; d < 3; ++d) b->wall_u[i][d] = wall_u ? wall_u[3 * i + d] : 0.0;
  }
  for(int d = 0; d < 3; ++d) {
    b->force[d]   = body_force ? body_force[d] : 0.0;
    b->inlet_u[d] = inlet_velocity ? inlet_velocity[d] : 0.0;
    if(b->force[d] != 0.0) b->has_force = 1;
  }
  b->inlet_rho = inlet_density;
  b->f         = (double*)calloc((size_t)b->L.Q * b->ncells, sizeof(double));
  b->fs        = (double*)calloc((size_t)b->L.Q * b->ncells, sizeof(double));
  return b;
}

void ora_box_destroy(ora_box* b) {
  if(!b) return;
  free(b->flags);
  free(b->dirichlet);
  free(b->slice_kappa);
  free(b->f);
  free(b->fs);
  free(b);
}

/* a kappa^2 per z-slice (nz values; NULL: the box's single kappa^2), the
   engine's lbm_gpu_box_set_slice_kappa */
int ora_box_set_slice_kappa(ora_box* b, const double* kappa_sq) {
  free(b->slice_kappa);
  b->slice_kappa = NULL;
  if(!kappa_sq) return 0;
  b->slice_kappa = (double*)malloc(sizeof(double) * b->n[2]);
  memcpy(b->slice_kappa, kappa_sq, sizeof(double) * b->n[2]);
  return 0;
}

int ora_box_set_poisson(ora_box* b, double kappa_sq, int nonlinear, const double* phi) {
  b->kappa_sq  = kappa_sq;
  b->nonlinear = nonlinear;
  if(phi) {
    b->dirichlet = (double*)malloc(sizeof(double) * b->ncells);
    memcpy(b->dirichlet, phi, sizeof(double) * b->ncells);
  }
  return 0;
}

/* Deviation form: the same BGK update with every population held as f - w_q,
 * rho - 1 = sum (f - w) and j = sum c (f - w) (since sum c w = 0), and
 * feq - w = w (rho - 1 + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u^2)).  Algebraically
 * identical to the plain form; its rounding errors are relative to the
 * deviations instead of to f = O(w), which matters over tens of thousands
 * of steps. */
int ora_box_set_deviation(ora_box* b, int on) {
  if(b->eq != ORA_NAVIER_STOKES) return -1;
  b->dev = on ? 1 : 0;
  return 0;
}

static void equilibrium(const ora_box* b, double rho, const double* u, double* feq) {
  const blat_t* L   = &b->L;
  double        usq = 0;
  for(int d = 0; d < L->D; ++d) usq += u[d] * u[d];
  for(int q = 0; q < L->Q; ++q) {
    double cu = 0;
    for(int d = 0; d < L->D; ++d) cu += L->c[q][d] * u[d];
    feq[q] = L->w[q] * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
  }
}

static void equilibrium_dev(const ora_box* b, double rho, const double* u, double* deq) {
  const blat_t* L   = &b->L;
  double        usq = 0;
  for(int d = 0; d < L->D; ++d) usq += u[d] * u[d];
  for(int q = 0; q < L->Q; ++q) {
    double cu = 0;
    for(int d = 0; d < L->D; ++d) cu += L->c[q][d] * u[d];
    deq[q] = L->w[q] * ((rho - 1.0) + rho * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq));
  }
}

void ora_box_init_equilibrium(ora_box* b, double rho, const double* u) {
  double feq[19];
  if(b->eq == ORA_NAVIER_STOKES && b->dev) equilibrium_dev(b, rho, u, feq);
  else if(b->eq == ORA_NAVIER_STOKES) equilibrium(b, rho, u, feq);
  else
    for(int q = 0; q < b->L.Q; ++q) feq[q] = 0.0;
  for(int q = 0; q < b->L.Q; ++q)
    for(int64_t i = 0; i < b->ncells; ++i) b->f[q * b->ncells + i] = feq[q];
}

static void emit(const ora_box* b, int64_t cell, double* out) {
  const blat_t* L = &b->L;
  if(b->eq == ORA_NAVIER_STOKES) {
    if(b->dev) equilibrium_dev(b, b->inlet_rho, b->inlet_u, out);
    else equilibrium(b, b->inlet_rho, b->inlet_u, out);
  } else {
    const double phi = b->dirichlet ? b->dirichlet[cell] : 0.0;
    for(int q = 0; q < L->Q; ++q) out[q] = q == L->Q - 1 ? (L->w[q] - 1.0) * phi : L->w[q] * phi;
  }
}

static void collide_cell(const ora_box* b, const double* f, double* out, int z) {
  const blat_t* L = &b->L;
  const int     Q = L->Q, D = L->D;
  const double  om = b->omega;
  if(b->eq == ORA_NAVIER_STOKES) {
    double rho = 0, j[3] = {0, 0, 0};
    for(int q = 0; q < Q; ++q) {
      rho += f[q];
      for(int d = 0; d < D; ++d) j[d] += L->c[q][d] * f[q];
    }
    if(b->dev) rho += 1.0; /* f holds deviations: sum = rho - 1 */
    double u[3] = {0, 0, 0};
    for(int d = 0; d < D; ++d) u[d] = (j[d] + 0.5 * b->force[d]) / rho;
    double feq[19];
    if(b->dev) equilibrium_dev(b, rho, u, feq);
    else equilibrium(b, rho, u, feq);
    for(int q = 0; q < Q; ++q) {
      double o = f[q] + om * (feq[q] - f[q]);
      if(b->has_force) {
        double cf = 0, uf = 0, cu = 0;
        for(int d = 0; d < D; ++d) {
          cf += L->c[q][d] * b->force[d];
          uf += u[d] * b->force[d];
          cu += L->c[q][d] * u[d];
        }
        o += (1.0 - 0.5 * om) * L->w[q] * (3.0 * (cf - uf) + 9.0 * cu * cf);
      }
      out[q] = o;
    }
  } else {
    double acc = 0;
    for(int q = 0; q < Q - 1; ++q) acc += f[q];
    const double phi  = acc / (1.0 - L->w[Q - 1]);
    const double g    = b->nonlinear ? sinh(phi) : phi;
    const double diff = L->alpha * (0.5 - 1.0 / om);
    for(int q = 0; q < Q; ++q) {
      const double feq = q == Q - 1 ? (L->w[Q - 1] - 1.0) * phi : L->w[q] * phi;
      double       o   = f[q] + om * (feq - f[q]);
      if(q != Q - 1) o += L->pw[q] * diff * (b->slice_kappa ? b->slice_kappa[z] : b->kappa_sq) * g;
      out[q] = o;
    }
  }
}

static int find_dir(const blat_t* L, int cx, int cy, int cz) {
  for(int k = 0; k < L->Q; ++k)
    if(L->c[k][0] == cx && L->c[k][1] == cy && L->c[k][2] == cz) return k;
  return -1;
}

/* the post-collision population arriving at (x,y,z) in direction k */
static double pull(const ora_box* b, int x, int y, int z, int k, int allow_open) {
  const blat_t* L    = &b->L;
  int           p[3] = {x, y, z}, s[3] = {x, y, z}, c[3] = {L->c[k][0], L->c[k][1], L->c[k][2]};
  int           bb = 0, open = 0;
  double        corr = 0;
  for(int a = 0; a < L->D; ++a) {
    s[a] = p[a] - c[a];
    if(s[a] < 0 || s[a] >= b->n[a]) {
      const int face = s[a] < 0 ? 2 * a : 2 * a + 1;
      const int ft   = b->face[face];
      if(ft == F_PERIODIC) {
        s[a] = s[a] < 0 ? s[a] + b->n[a] : s[a] - b->n[a];
      } else if(ft == F_FREESLIP) {
        s[a] = p[a];
        c[a] = -c[a];
      } else if(ft == F_OPEN) {
        open = 1;
      } else {
        double cu = 0;
        for(int d = 0; d < L->D; ++d) cu += L->c[k][d] * b->wall_u[face][d];
        corr += 6.0 * L->w[k] * cu;
        bb = 1;
      }
    }
  }
  const int64_t own = x + (int64_t)b->n[0] * (y + (int64_t)b->n[1] * z);
  if(open) {
    /* zero gradient through the outlet face: what the upstream cell receives */
    if(allow_open && x > 0) return pull(b, x - 1, y, z, k, 0);
    return b->fs[L->opp[k] * b->ncells + own];
  }
  if(bb) return b->fs[L->opp[k] * b->ncells + own] + corr;
  const int64_t src = s[0] + (int64_t)b->n[0] * (s[1] + (int64_t)b->n[1] * s[2]);
  if(b->flags[src] == ORA_CELL_SOLID) return b->fs[L->opp[k] * b->ncells + own];
  const int q = find_dir(L, c[0], c[1], c[2]);
  return b->fs[q * b->ncells + src];
}

void ora_box_step(ora_box* b, int64_t nsteps, int nthreads) {
  const blat_t* L = &b->L;
  const int     Q = L->Q;
  const int64_t N = b->ncells;
  (void)nthreads;
  for(int64_t s = 0; s < nsteps; ++s) {
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for(int64_t cell = 0; cell < N; ++cell) {
      double f[19], o[19];
      const uint8_t t = b->flags[cell];
      if(t == ORA_CELL_SOLID) {
        for(int q = 0; q < Q; ++q) b->fs[q * N + cell] = 0.0;
        continue;
      }
      if(t == ORA_CELL_INLET || t == ORA_CELL_DIRICHLET) {
        emit(b, cell, o);
      } else {
        for(int q = 0; q < Q; ++q) f[q] = b->f[q * N + cell];
        collide_cell(b, f, o, (int)(cell / ((int64_t)b->n[0] * b->n[1])));
      }
      for(int q = 0; q < Q; ++q) b->fs[q * N + cell] = o[q];
    }
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for(int64_t cell = 0; cell < N; ++cell) {
      const uint8_t t = b->flags[cell];
      const int     x = (int)(cell % b->n[0]), y = (int)((cell / b->n[0]) % b->n[1]), z = (int)(cell / ((int64_t)b->n[0] * b->n[1]));
      if(t == ORA_CELL_SOLID) {
        for(int q = 0; q < Q; ++q) b->f[q * N + cell] = 0.0;
        continue;
      }
      if(t == ORA_CELL_INLET || t == ORA_CELL_DIRICHLET) {
        double o[19];
        emit(b, cell, o);
        for(int q = 0; q < Q; ++q) b->f[q * N + cell] = o[q];
        continue;
      }
      for(int k = 0; k < Q; ++k) b->f[k * N + cell] = pull(b, x, y, z, k, 1);
    }
  }
}

void ora_box_get(const ora_box* b, double* f_soa, double* rho, double* u) {
  const blat_t* L = &b->L;
  const int64_t N = b->ncells;
  if(f_soa) {
    memcpy(f_soa, b->f, sizeof(double) * L->Q * N);
    if(b->dev)
      for(int q = 0; q < L->Q; ++q)
        for(int64_t i = 0; i < N; ++i)
          if(b->flags[i] != ORA_CELL_SOLID) f_soa[q * N + i] += L->w[q];
  }
  for(int64_t cell = 0; cell < N; ++cell) {
    double r = 0, j[3] = {0, 0, 0}, acc = 0;
    for(int q = 0; q < L->Q; ++q) {
      const double v = b->f[q * N + cell] + (b->dev && b->flags[cell] != ORA_CELL_SOLID ? L->w[q] : 0.0);
      r += v;
      if(q < L->Q - 1) acc += v;
      for(int d = 0; d < L->D; ++d) j[d] += L->c[q][d] * v;
    }
    if(b->eq == ORA_POISSON) {
      if(rho) rho[cell] = acc / (1.0 - L->w[L->Q - 1]);
      continue;
    }
    if(rho) rho[cell] = r;
    if(u)
      for(int d = 0; d < L->D; ++d) u[d * N + cell] = r != 0.0 ? (j[d] + 0.5 * b->force[d]) / r : 0.0;
  }
}

void ora_box_set(ora_box* b, const double* f_soa) {
  memcpy(b->f, f_soa, sizeof(double) * b->L.Q * b->ncells);
  if(b->dev)
    for(int q = 0; q < b->L.Q; ++q)
      for(int64_t i = 0; i < b->ncells; ++i)
        if(b->flags[i] != ORA_CELL_SOLID) b->f[q * b->ncells + i] -= b->L.w[q];
}
