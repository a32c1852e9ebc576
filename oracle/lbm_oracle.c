/*
 * CPU oracle, table engine: a plain-C restatement of the SFCMM/LBM reference
 * time step on the reference's own cell list and neighbour table.
 *
 * TEST INFRASTRUCTURE ONLY (see lbm_oracle.h).  Every routine follows the
 * reference loop it cites, in the same floating-point operation order, and the
 * file is compiled with -ffp-contract=off so that no multiply-add is fused:
 * on the same inputs it reproduces the reference's doubles bit for bit
 * (tests/test_oracle_golden.py checks this against tests/golden/).
 */
#include "lbm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EPS DBL_EPSILON /* GDoubleEps, include/common/sfcmm_types.h:50 */
#define INVALID (-1)

/* lbm_cssq, src/lbm/constants.h:27 */
static const double CSSQ = 1.0 / 3.0;

/* ---- lattice tables, restated from src/lbm/constants.h:247-343 ------------
 * Direction order and weights must be the reference's: the reference's
 * neighbour table is indexed by the same direction ids. */
typedef struct {
  int    ndim, q;
  double c[19][3];
  int    opp[19];
  double w[19];
  double poisson_alpha;
  double poisson_w[19];
} lattice_t;

static const lattice_t L_D1Q3 = {1, 3, {{-1}, {1}, {0}}, {1, 0, 2}, {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}, 1.0 / 3.0, {0.5, 0.5, 0}};
static const lattice_t L_D2Q5 = {2,
                                 5,
                                 {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {0, 0}},
                                 {1, 0, 3, 2, 4},
                                 {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 1.0 / 3.0},
                                 1.0 / 2.0,
                                 {0.25, 0.25, 0.25, 0.25, 0.0}};
static const lattice_t L_D2Q9 = {
    2,
    9,
    {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {1, 1}, {1, -1}, {-1, -1}, {-1, 1}, {0, 0}},
    {1, 0, 3, 2, 6, 7, 4, 5, 8},
    {1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 4.0 / 9.0},
    1.0 / 3.0,
    {1.0 / 8.0, 1.0 / 8.0, 1.0 / 8.0, 1.0 / 8.0, 1.0 / 8.0, 1.0 / 8.0, 1.0 / 8.0, 1.0 / 8.0, 0.0}};

typedef struct {
  int      kind;
  int64_t  n;
  int64_t* cells;
  double*  normals; /* n x ndim, surface normal of each listed cell */
  double*  values;  /* per cell value (Dirichlet/Neumann NEEM) */
  double   vec[3];
  int      has_vec;
  double   scalar;
  int      has_pressure;
  /* derived tables */
  double*  tang;       /* n x q: tangential BB values (bnd_wall.h:31-72) */
  int*     lim_dist;   /* n x q: 1 if dist is in the limited set (bnd_wetnode.h:12-72) */
  double*  lim_const;  /* n x q */
  int*     lim_empty;  /* n: set cleared (corner) */
  int64_t* ext;        /* n: extrapolation cell */
  int*     ext_dir;    /* n: extrapolation direction (Dirichlet NEEM) */
  int*     nset;       /* n: periodic set dists */
  int*     set_dist;   /* n x q */
  int64_t* linked;     /* n x q */
  int64_t* cell2idx;   /* ncells: last index of a cell in the list (unordered_map semantics) */
} bnd_t;

struct ora_ctx {
  lattice_t L;
  int       eq, nvar, nnghbr;
  int64_t   n;
  double    omega, relax_time, dt, poisson_k;
  int64_t*  nghbr;
  double*   centers;
  double    bbox[6];
  double    cell_length;
  unsigned char* periodic;
  double *  fold, *f, *feq, *vars, *varsold;
  bnd_t*    bnds;
  int       nbnd;
  int       forcing;
  double    forcing_dp;
  int64_t   nin, nout;
  int64_t * in_cells, *out_cells;
  double    diffusivity;
  int       diffusivity_set;
};

static inline int64_t NB(const ora_ctx* c, int64_t cell, int dir) { return c->nghbr[cell * c->nnghbr + dir]; }

/* LBMVariables positions, src/lbm/variables.h:7-115 */
static inline int V_U(int d) { return d; }
static inline int V_RHO(const ora_ctx* c) { return c->L.ndim; }

/* inDirection: n . c >= eps, src/lbm/constants.h:83-86 */
static int in_direction(const double* n, const double* dir, int ndim) {
  double s = 0;
  for(int d = 0; d < ndim; ++d) s += n[d] * dir[d];
  return s >= EPS;
}
/* orthogonal: |n . c| <= eps, src/lbm/constants.h:88-91 */
static int orthogonal(const double* n, const double* dir, int ndim) {
  double s = 0;
  for(int d = 0; d < ndim; ++d) s += n[d] * dir[d];
  return fabs(s) <= EPS;
}

/* eq::defaultEq(w, rho, cu, vsq), src/lbm/equilibrium_func.h:52-54 */
static inline double eq_default(double w, double rho, double cu, double vsq) {
  return w * rho * (1.0 + cu / CSSQ + cu * cu / (2.0 * CSSQ * CSSQ) - vsq / (2.0 * CSSQ));
}
/* eq::symmEq, src/lbm/equilibrium_func.h:109-111 */
static inline double eq_symm(double w, double rho, double cu, double vsq) {
  return w * rho * (1.0 + cu * cu / (2.0 * CSSQ * CSSQ) - vsq / (2.0 * CSSQ));
}
/* defaultEq<LBTYPE>(dist, rho, u), src/lbm/equilibrium_func.h:86-101 */
static double eq_default_dist(const lattice_t* L, int dist, double rho, const double* u) {
  double vsq = 0;
  for(int d = 0; d < L->ndim; ++d) vsq += u[d] * u[d];
  double cu = 0;
  for(int d = 0; d < L->ndim; ++d) cu += u[d] * L->c[dist][d];
  return eq_default(L->w[dist], rho, cu, vsq);
}
static double eq_symm_dist(const lattice_t* L, int dist, double rho, const double* u) {
  double vsq = 0;
  for(int d = 0; d < L->ndim; ++d) vsq += u[d] * u[d];
  double cu = 0;
  for(int d = 0; d < L->ndim; ++d) cu += u[d] * L->c[dist][d];
  return eq_symm(L->w[dist], rho, cu, vsq);
}
/* defaultEq<LBTYPE>(feq*, rho, u), src/lbm/equilibrium_func.h:67-84 */
static void eq_default_all(const lattice_t* L, double* feq, double rho, const double* u) {
  double vsq = 0;
  for(int d = 0; d < L->ndim; ++d) vsq += u[d] * u[d];
  for(int q = 0; q < L->q; ++q) {
    double cu = 0;
    for(int d = 0; d < L->ndim; ++d) cu += u[d] * L->c[q][d];
    feq[q] = eq_default(L->w[q], rho, cu, vsq);
  }
}

/* ---- construction ------------------------------------------------------- */

ora_ctx* ora_create(int lattice, int equation, int64_t ncells, double omega, double relax_time, double dt, double poisson_k,
                    const int64_t* nghbr, int nnghbr, const double* centers, const double* bbox, double cell_length) {
  ora_ctx* c = (ora_ctx*)calloc(1, sizeof(ora_ctx));
  if(!c) return NULL;
  if(lattice == ORA_D1Q3) c->L = L_D1Q3;
  else if(lattice == ORA_D2Q5) c->L = L_D2Q5;
  else if(lattice == ORA_D2Q9) c->L = L_D2Q9;
  else {
    free(c);
    return NULL;
  }
  c->eq = equation;
  /* noVars, src/lbm/constants.h:424-439 */
  c->nvar       = equation == ORA_POISSON ? 1 : c->L.ndim + 1;
  c->nnghbr     = nnghbr;
  c->n          = ncells;
  c->omega      = omega;
  c->relax_time = relax_time;
  c->dt         = dt;
  c->poisson_k  = poisson_k;
  c->nghbr      = (int64_t*)malloc(sizeof(int64_t) * ncells * nnghbr);
  memcpy(c->nghbr, nghbr, sizeof(int64_t) * ncells * nnghbr);
  c->centers = (double*)malloc(sizeof(double) * ncells * c->L.ndim);
  memcpy(c->centers, centers, sizeof(double) * ncells * c->L.ndim);
  for(int i = 0; i < 2 * c->L.ndim; ++i) c->bbox[i] = bbox[i];
  c->cell_length = cell_length;
  c->periodic    = (unsigned char*)calloc(ncells, 1);
  const int64_t nq = ncells * c->L.q;
  c->fold    = (double*)calloc(nq, sizeof(double));
  c->f       = (double*)calloc(nq, sizeof(double));
  c->feq     = (double*)calloc(nq, sizeof(double));
  c->vars    = (double*)calloc(ncells * c->nvar, sizeof(double));
  c->varsold = (double*)calloc(ncells * c->nvar, sizeof(double));
  return c;
}

void ora_destroy(ora_ctx* c) {
  if(!c) return;
  for(int i = 0; i < c->nbnd; ++i) {
    bnd_t* b = &c->bnds[i];
    free(b->cells);
    free(b->normals);
    free(b->values);
    free(b->tang);
    free(b->lim_dist);
    free(b->lim_const);
    free(b->lim_empty);
    free(b->ext);
    free(b->ext_dir);
    free(b->nset);
    free(b->set_dist);
    free(b->linked);
    free(b->cell2idx);
  }
  free(c->bnds);
  free(c->nghbr);
  free(c->centers);
  free(c->periodic);
  free(c->fold);
  free(c->f);
  free(c->feq);
  free(c->vars);
  free(c->varsold);
  free(c->in_cells);
  free(c->out_cells);
  free(c);
}

int ora_nvar(const ora_ctx* c) { return c->nvar; }
int ora_ndist(const ora_ctx* c) { return c->L.q; }

/* LBMBnd_wallWetnode constructor, src/lbm/bnd/bnd_wetnode.h:21-60 */
static void build_wetnode(ora_ctx* c, bnd_t* b) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  b->lim_dist        = (int*)calloc(b->n * Q, sizeof(int));
  b->lim_const       = (double*)calloc(b->n * Q, sizeof(double));
  b->lim_empty       = (int*)calloc(b->n, sizeof(int));
  for(int64_t i = 0; i < b->n; ++i) {
    const int64_t cell = b->cells[i];
    const double* nrm  = &b->normals[i * L->ndim];
    const int     per  = c->periodic[cell];
    for(int dir = 0; dir < Q - 1; ++dir) {
      const int opp = L->opp[dir];
      if(in_direction(nrm, L->c[dir], L->ndim) && (per || NB(c, cell, opp) != INVALID)) {
        b->lim_dist[i * Q + dir]  = 1;
        b->lim_const[i * Q + dir] = 2;
      } else if(orthogonal(nrm, L->c[dir], L->ndim) && (per || NB(c, cell, opp) != INVALID)) {
        b->lim_dist[i * Q + dir] = 1;
        if(NB(c, cell, dir) == INVALID && !per) {
          b->lim_const[i * Q + dir] = 2;
        } else {
          b->lim_const[i * Q + dir] = 1;
        }
      }
    }
    /* std::accumulate(begin, end, 0): an int accumulator */
    int sumC = 0;
    for(int q = 0; q < Q; ++q) sumC = (int)(sumC + b->lim_const[i * Q + q]);
    if(sumC != Q - 1) {
      b->lim_empty[i] = 1;
      for(int q = 0; q < Q; ++q) b->lim_dist[i * Q + q] = 0;
    } else {
      b->lim_dist[i * Q + Q - 1]  = 1;
      b->lim_const[i * Q + Q - 1] = 1;
    }
  }
}

/* extrapolationDir lambda, src/lbm/bnd/bnd_wall.h:213-223 and bnd_pressure.h:274-284 */
static int inside_dir(const double* nrm, int ndim) {
  for(int d = 0; d < ndim; ++d) {
    if(nrm[d] < 0) return 2 * d + 1;
    if(nrm[d] > 0) return 2 * d;
  }
  return -1;
}

/* cartesian::oppositeDir<NDIM>, include/common/math/cartesian.h:22-33 */
static int opposite_dir_diag(int dir, int ndim) {
  if(dir < 2 * ndim) return dir + 1 - 2 * (dir % 2);
  return dir > 5 ? dir - 2 : dir + 2;
}

int ora_add_bnd(ora_ctx* c, int kind, int64_t ncells, const int64_t* cells, const double* normals, const double* values, const double* vec,
                int has_vec, double scalar, int has_pressure, int64_t nconn, const int64_t* conn_cells, const double* conn_normals) {
  (void)conn_normals;
  if(ncells <= 0) return 0; /* "Skipping ... no valid cells", bnd.h:82-86 */
  const lattice_t* L = &c->L;
  const int        Q = L->q, D = L->ndim;
  c->bnds            = (bnd_t*)realloc(c->bnds, sizeof(bnd_t) * (c->nbnd + 1));
  bnd_t* b           = &c->bnds[c->nbnd++];
  memset(b, 0, sizeof(*b));
  b->kind    = kind;
  b->n       = ncells;
  b->cells   = (int64_t*)malloc(sizeof(int64_t) * ncells);
  b->normals = (double*)malloc(sizeof(double) * ncells * D);
  memcpy(b->cells, cells, sizeof(int64_t) * ncells);
  memcpy(b->normals, normals, sizeof(double) * ncells * D);
  if(values) {
    b->values = (double*)malloc(sizeof(double) * ncells);
    memcpy(b->values, values, sizeof(double) * ncells);
  }
  for(int d = 0; d < 3; ++d) b->vec[d] = (vec && d < D) ? vec[d] : 0.0;
  b->has_vec      = has_vec;
  b->scalar       = scalar;
  b->has_pressure = has_pressure;
  b->cell2idx     = (int64_t*)malloc(sizeof(int64_t) * c->n);
  for(int64_t i = 0; i < c->n; ++i) b->cell2idx[i] = -1;
  for(int64_t i = 0; i < ncells; ++i) b->cell2idx[cells[i]] = i;

  switch(kind) {
    case ORA_BND_PERIODIC: {
      /* addPeriodicBndry marks both surfaces periodic, bnd.h:206-226 */
      for(int64_t i = 0; i < ncells; ++i) c->periodic[cells[i]] = 1;
      for(int64_t i = 0; i < nconn; ++i) c->periodic[conn_cells[i]] = 1;
      /* LBMBndCell_periodic::init, src/lbm/bnd/bnd_periodic.h:31-100 */
      b->nset     = (int*)calloc(ncells, sizeof(int));
      b->set_dist = (int*)calloc(ncells * Q, sizeof(int));
      b->linked   = (int64_t*)calloc(ncells * Q, sizeof(int64_t)); /* m_linkedCell{} is zero-initialised */
      for(int64_t i = 0; i < ncells; ++i) {
        const int64_t cell   = cells[i];
        const double* nrm    = &normals[i * D];
        const double* center = &c->centers[cell * D];
        for(int dist = 0; dist < Q; ++dist) {
          if(in_direction(nrm, L->c[dist], D)) {
            double coord[3];
            for(int d = 0; d < D; ++d) {
              if(fabs(nrm[d]) > 0) coord[d] = c->bbox[2 * d];
              else coord[d] = center[d] + L->c[dist][d] * c->cell_length;
            }
            int inside = 1;
            for(int d = 0; d < D; ++d)
              if(coord[d] < c->bbox[2 * d] || coord[d] > c->bbox[2 * d + 1]) inside = 0;
            if(inside) b->set_dist[i * Q + b->nset[i]++] = dist;
          }
        }
        for(int id = 0; id < b->nset[i]; ++id) {
          b->linked[i * Q + id] = INVALID;
          const int dist        = b->set_dist[i * Q + id];
          double    centerA[3];
          for(int d = 0; d < D; ++d) {
            centerA[d] = center[d];
            if(fabs(nrm[d]) > 0) continue;
            centerA[d] += L->c[dist][d] * c->cell_length;
          }
          const double max_cell_match_dist = 10 * EPS;
          for(int64_t j = 0; j < nconn; ++j) {
            const double* centerB = &c->centers[conn_cells[j] * D];
            int           match   = 0;
            for(int d = 0; d < D; ++d) {
              if(fabs(centerA[d] - centerB[d]) <= max_cell_match_dist) {
                match = 1; /* the reference accepts a match in any one direction */
                break;
              }
            }
            if(match) {
              b->linked[i * Q + id] = conn_cells[j];
              break;
            }
          }
          if(b->linked[i * Q + id] == INVALID) return -3;
        }
      }
      break;
    }
    case ORA_BND_WALL_BB_TANGENTIAL: {
      /* LBMBnd_wallBB<TANGENTIALVELO=true>::init, src/lbm/bnd/bnd_wall.h:31-72 (2D only) */
      if(D != 2) return -2;
      b->tang = (double*)calloc(ncells * Q, sizeof(double));
      for(int64_t i = 0; i < ncells; ++i) {
        const double* nrm = &normals[i * D];
        for(int id = 0; id < Q; ++id) {
          if(in_direction(nrm, L->c[id], D)) {
            const int     inside = L->opp[id];
            const double* dir    = L->c[inside];
            const double  t[2]   = {nrm[1], nrm[0]};
            /* angle(n, dir) == pi  <=>  dir is anti-parallel to n */
            const double ndot  = nrm[0] * dir[0] + nrm[1] * dir[1];
            const double cross = nrm[0] * dir[1] - nrm[1] * dir[0];
            const int    par   = cross == 0.0 && ndot < 0.0;
            if(!par) b->tang[i * Q + inside] = scalar * (t[0] * dir[0] + t[1] * dir[1]);
          }
        }
      }
      break;
    }
    case ORA_BND_WALL_EQ:
    case ORA_BND_WALL_NEBB:
      if(kind == ORA_BND_WALL_NEBB && !(L->q == 9 && D == 2)) return -2;
      build_wetnode(c, b);
      break;
    case ORA_BND_WALL_NEEM:
      build_wetnode(c, b);
      /* LBMBnd_wallNEEM::init, src/lbm/bnd/bnd_wall.h:212-248 */
      b->ext = (int64_t*)malloc(sizeof(int64_t) * ncells);
      for(int64_t i = 0; i < ncells; ++i) {
        const int dir = inside_dir(&normals[i * D], D);
        b->ext[i]     = dir < 0 ? INVALID : NB(c, cells[i], dir);
        if(b->ext[i] == INVALID) return -3;
      }
      break;
    case ORA_BND_DIRICHLET_NEEM:
    case ORA_BND_NEUMANN_NEEM: {
      /* LBMBnd_DirichletNEEM constructor, src/lbm/bnd/bnd_dirichlet.h:285-316 */
      if(c->eq != ORA_POISSON) return -2;
      b->ext     = (int64_t*)malloc(sizeof(int64_t) * ncells);
      b->ext_dir = (int*)malloc(sizeof(int) * ncells);
      if(!b->values) {
        b->values = (double*)malloc(sizeof(double) * ncells);
        for(int64_t i = 0; i < ncells; ++i) b->values[i] = scalar;
      }
      for(int64_t i = 0; i < ncells; ++i) {
        int ed = -1;
        for(int dist = 0; dist < 2 * D; ++dist) {
          if(NB(c, cells[i], dist) == INVALID) {
            if(ed < 0) {
              ed = dist;
            } else {
              if(ed == 0 && dist == 2) ed = 6;
              if(ed == 0 && dist == 3) ed = 7;
              if(ed == 1 && dist == 3) ed = 4;
              if(ed == 1 && dist == 2) ed = 5;
            }
          }
        }
        if(ed < 0) return -3;
        const int od  = opposite_dir_diag(ed, D);
        b->ext[i]     = NB(c, cells[i], od);
        b->ext_dir[i] = od;
        if(b->ext[i] == INVALID) return -3;
        /* the Neumann value extrapolates from a second cell further in; a
           grid without it (refined grids can lack it) is refused, as the
           library's table upload refuses it */
        if(kind == ORA_BND_NEUMANN_NEEM && NB(c, b->ext[i], od) == INVALID) return -3;
      }
      break;
    }
    case ORA_BND_PRESSURE_ABB:
      /* the extrapolation reads the two cells inside the boundary cell
         (bnd_pressure.h:73-78); the reference does not check that they
         exist, here a grid without them is refused */
      for(int64_t i = 0; i < ncells; ++i) {
        const int     id = inside_dir(&normals[i * D], D);
        const int64_t n1 = id < 0 ? INVALID : NB(c, cells[i], id);
        if(n1 == INVALID || NB(c, n1, id) == INVALID) return -3;
      }
      break;
    case ORA_BND_WALL_BB:
    case ORA_BND_DIRICHLET_BB:
      break;
    default:
      return -1;
  }
  return 0;
}

int ora_set_forcing(ora_ctx* c, double pressure_gradient, int64_t nin, const int64_t* in_cells, int64_t nout, const int64_t* out_cells) {
  c->forcing    = 1;
  c->forcing_dp = pressure_gradient;
  c->nin        = nin;
  c->nout       = nout;
  c->in_cells   = (int64_t*)malloc(sizeof(int64_t) * (nin > 0 ? nin : 1));
  c->out_cells  = (int64_t*)malloc(sizeof(int64_t) * (nout > 0 ? nout : 1));
  memcpy(c->in_cells, in_cells, sizeof(int64_t) * nin);
  memcpy(c->out_cells, out_cells, sizeof(int64_t) * nout);
  return 0;
}

/* ---- boundary initial conditions (initCnd) ------------------------------ */
static void bnd_init(ora_ctx* c, bnd_t* b) {
  const int D = c->L.ndim;
  switch(b->kind) {
    case ORA_BND_DIRICHLET_BB: /* bnd_dirichlet.h:44-50 */
      for(int64_t i = 0; i < b->n; ++i)
        for(int d = 0; d < D; ++d) c->vars[b->cells[i] * c->nvar + V_U(d)] = b->vec[d];
      break;
    case ORA_BND_PRESSURE_ABB: /* bnd_pressure.h:20-26 */
      for(int64_t i = 0; i < b->n; ++i) c->vars[b->cells[i] * c->nvar + V_RHO(c)] = b->scalar;
      break;
    case ORA_BND_DIRICHLET_NEEM: /* bnd_dirichlet.h:342-348 */
      for(int64_t i = 0; i < b->n; ++i) c->vars[b->cells[i] * c->nvar + 0] = b->values[i];
      break;
    default: /* wallBB, wallEq, wallNEEM, NEBB, periodic, Neumann: empty initCnd */
      break;
  }
}

/* initialCondition, src/lbm/solver.cpp:266-295 */
void ora_initial_condition(ora_ctx* c) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  memset(c->vars, 0, sizeof(double) * c->n * c->nvar);
  memset(c->varsold, 0, sizeof(double) * c->n * c->nvar);
  for(int i = 0; i < c->nbnd; ++i) bnd_init(c, &c->bnds[i]);
  for(int64_t cell = 0; cell < c->n; ++cell) {
    double* v = &c->vars[cell * c->nvar];
    if(c->eq == ORA_NAVIER_STOKES) {
      v[V_RHO(c)] = 1.0;
      for(int dist = 0; dist < Q; ++dist) {
        eq_default_all(L, &c->feq[cell * Q], v[V_RHO(c)], v);
        c->f[cell * Q + dist]    = c->feq[cell * Q + dist];
        c->fold[cell * Q + dist] = c->feq[cell * Q + dist];
      }
    } else {
      for(int dist = 0; dist < Q - 1; ++dist) {
        c->feq[cell * Q + dist]  = L->w[dist] * v[0];
        c->f[cell * Q + dist]    = c->feq[cell * Q + dist];
        c->fold[cell * Q + dist] = c->feq[cell * Q + dist];
      }
      const double centerFeq       = (L->w[Q - 1] - 1.0) * v[0];
      c->feq[cell * Q + Q - 1]     = centerFeq;
      c->f[cell * Q + Q - 1]       = centerFeq;
      c->fold[cell * Q + Q - 1]    = centerFeq;
    }
  }
}

/* ---- the step phases ---------------------------------------------------- */

/* updateMacroscopicValues, src/lbm/solver.cpp:512-553 */
void ora_update_moments(ora_ctx* c) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  for(int64_t cell = 0; cell < c->n; ++cell) {
    const double* fo = &c->fold[cell * Q];
    double*       v  = &c->vars[cell * c->nvar];
    if(c->eq == ORA_NAVIER_STOKES) {
      double rho = 0.0;
      for(int q = 0; q < Q; ++q) rho += fo[q];
      v[V_RHO(c)] = rho;
      for(int d = 0; d < L->ndim; ++d) {
        v[V_U(d)] = 0;
        for(int q = 0; q < Q - 1; ++q) v[V_U(d)] += L->c[q][d] * fo[q];
        v[V_U(d)] /= v[V_RHO(c)];
      }
    } else {
      double acc = 0.0;
      for(int q = 0; q < Q - 1; ++q) acc += fo[q];
      v[0] = 1.0 / (1.0 - L->w[Q - 1]) * acc;
    }
  }
}

/* calcEquilibriumMoments, src/lbm/solver.cpp:555-571 */
static void equilibrium(ora_ctx* c) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  for(int64_t cell = 0; cell < c->n; ++cell) {
    const double* v  = &c->vars[cell * c->nvar];
    double*       fe = &c->feq[cell * Q];
    if(c->eq == ORA_NAVIER_STOKES) {
      eq_default_all(L, fe, v[V_RHO(c)], v);
    } else {
      for(int q = 0; q < Q - 1; ++q) fe[q] = L->w[q] * v[0];
      fe[Q - 1] = (L->w[Q - 1] - 1.0) * v[0];
    }
  }
}

/* collisionStep, src/lbm/solver.cpp:573-622 */
static void collide(ora_ctx* c) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  if(c->eq == ORA_POISSON && !c->diffusivity_set) {
    /* `static const` in the reference: evaluated once, at the first step */
    const double latticeVelocity = 1.0;
    c->diffusivity               = L->poisson_alpha * (latticeVelocity * latticeVelocity) * (0.5 - c->relax_time) * c->dt;
    c->diffusivity_set           = 1;
  }
  for(int64_t cell = 0; cell < c->n; ++cell) {
    for(int q = 0; q < Q; ++q) {
      double f = (1 - c->omega) * c->fold[cell * Q + q] + c->omega * c->feq[cell * Q + q];
      if(c->eq == ORA_POISSON && q != Q - 1) {
        const double rhs = c->poisson_k * c->poisson_k * c->vars[cell * c->nvar + 0];
        f += c->dt * c->diffusivity * L->poisson_w[q] * rhs;
      }
      c->f[cell * Q + q] = f;
    }
  }
}

/* forcing, src/lbm/solver.cpp:625-696 */
static void forcing(ora_ctx* c) {
  if(!c->forcing) return;
  const lattice_t* L              = &c->L;
  const int        Q              = L->q, D = L->ndim;
  const double     outletPressure = 1.0;
  const double     inletPressure  = outletPressure + c->forcing_dp;
  for(int64_t i = 0; i < c->nin; ++i) {
    const int64_t valueCell   = NB(c, c->in_cells[i], 1);
    const double* centerInlet = &c->centers[valueCell * D];
    for(int64_t j = 0; j < c->nout; ++j) {
      const int64_t outCell = c->out_cells[j];
      if(fabs(centerInlet[1] - c->centers[outCell * D + 1]) < EPS) {
        const double* u   = &c->vars[valueCell * c->nvar];
        double        vsq = 0;
        for(int d = 0; d < D; ++d) vsq += u[d] * u[d];
        for(int q = 0; q < Q; ++q) {
          const double cu       = u[0] * L->c[q][0];
          c->f[outCell * Q + q] = eq_default(L->w[q], outletPressure, cu, vsq) + c->f[valueCell * Q + q] - c->feq[valueCell * Q + q];
        }
      }
    }
  }
  for(int64_t i = 0; i < c->nout; ++i) {
    const int64_t valueCell    = NB(c, c->out_cells[i], 0);
    const double* centerOutlet = &c->centers[valueCell * D];
    for(int64_t j = 0; j < c->nin; ++j) {
      const int64_t inCell = c->in_cells[j];
      if(fabs(c->centers[inCell * D + 1] - centerOutlet[1]) < EPS) {
        const double* u   = &c->vars[valueCell * c->nvar];
        double        vsq = 0;
        for(int d = 0; d < D; ++d) vsq += u[d] * u[d];
        for(int q = 0; q < Q; ++q) {
          const double cu      = u[0] * L->c[q][0];
          c->f[inCell * Q + q] = eq_default(L->w[q], inletPressure, cu, vsq) + c->f[valueCell * Q + q] - c->feq[valueCell * Q + q];
        }
      }
    }
  }
}

/* LBMBndManager::preApply, src/lbm/bnd/bnd.h:48-53 */
static void pre_apply(ora_ctx* c) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  for(int k = 0; k < c->nbnd; ++k) {
    bnd_t* b = &c->bnds[k];
    if(b->kind == ORA_BND_PERIODIC) {
      /* LBMBndCell_periodic::preApply, bnd_periodic.h:102-119 */
      for(int64_t i = 0; i < b->n; ++i) {
        const int64_t mapped = b->cells[i];
        const int64_t link0  = b->linked[i * Q + 0];
        if(b->has_pressure) {
          for(int dist = 0; dist < Q; ++dist) {
            c->fold[link0 * Q + dist] =
                eq_default_dist(L, dist, b->scalar, &c->vars[mapped * c->nvar]) + c->f[mapped * Q + dist] - c->feq[mapped * Q + dist];
          }
          c->vars[link0 * c->nvar + V_RHO(c)] = b->scalar;
        } else {
          for(int id = 0; id < b->nset[i]; ++id) {
            const int dist                                  = b->set_dist[i * Q + id];
            c->fold[b->linked[i * Q + id] * Q + dist] = c->f[mapped * Q + dist];
          }
          c->vars[link0 * c->nvar + V_RHO(c)] = 1.0;
        }
      }
    } else if(b->kind == ORA_BND_PRESSURE_ABB) {
      /* bnd_pressure.h:42-49 */
      for(int64_t i = 0; i < b->n; ++i) c->vars[b->cells[i] * c->nvar + V_RHO(c)] = b->scalar;
    }
  }
}

/* propagationStep, src/lbm/solver.cpp:714-740 */
static void propagate(ora_ctx* c) {
  const int Q = c->L.q;
  for(int64_t cell = 0; cell < c->n; ++cell) {
    for(int dist = 0; dist < Q - 1; ++dist) {
      const int64_t nb = NB(c, cell, dist);
      if(nb != INVALID) c->fold[nb * Q + dist] = c->f[cell * Q + dist];
    }
    c->fold[cell * Q + Q - 1] = c->f[cell * Q + Q - 1];
  }
}

/* calcDensity_limited, src/lbm/moments.h:119-153 */
static void density_limited(ora_ctx* c, const bnd_t* b, int64_t idx, int noslip) {
  const int     Q    = c->L.q, D = c->L.ndim;
  const int64_t cell = b->cells[idx];
  if(b->lim_empty[idx]) return;
  double* v   = &c->vars[cell * c->nvar];
  v[V_RHO(c)] = 0;
  for(int dist = 0; dist < Q; ++dist) /* std::set iterates in ascending order */
    if(b->lim_dist[idx * Q + dist]) v[V_RHO(c)] += b->lim_const[idx * Q + dist] * c->fold[cell * Q + dist];
  if(!noslip) {
    const double* nrm = &b->normals[idx * D];
    for(int d = 0; d < D; ++d) {
      if(nrm[d] > EPS) v[V_RHO(c)] *= 1.0 / (1.0 + v[V_U(d)]);
      else if(nrm[d] < 0) v[V_RHO(c)] *= 1.0 / (1.0 - v[V_U(d)]);
    }
  }
}

/* LBMBnd_DirichletEQ::apply<VALZERO>, src/lbm/bnd/bnd_dirichlet.h:211-241 */
static void dirichlet_eq_cell(ora_ctx* c, const bnd_t* b, int64_t cell, const double* values, int valzero) {
  const lattice_t* L     = &c->L;
  const int        Q     = L->q, D = L->ndim;
  const int64_t    index = b->cell2idx[cell];
  double*          v     = &c->vars[cell * c->nvar];
  for(int d = 0; d < D; ++d) v[V_U(d)] = values[d];
  density_limited(c, b, index, valzero);
  for(int dist = 0; dist < Q; ++dist) {
    if(valzero) {
      c->fold[cell * Q + dist] = eq_default(L->w[dist], v[V_RHO(c)], 0, 0);
    } else {
      eq_default_all(L, &c->fold[cell * Q], v[V_RHO(c)], v);
    }
  }
}

/* calcDensity + calcVelocity (NS), src/lbm/moments.h:17-45, 69-83 */
static void moments_ns_cell(ora_ctx* c, int64_t cell) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  double*          v = &c->vars[cell * c->nvar];
  v[V_RHO(c)]        = c->fold[cell * Q + 0];
  for(int dist = 1; dist < Q; ++dist) v[V_RHO(c)] += c->fold[cell * Q + dist];
}
static void velocity_ns_cell(ora_ctx* c, int64_t cell) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  double*          v = &c->vars[cell * c->nvar];
  for(int d = 0; d < L->ndim; ++d) {
    v[V_U(d)] = 0;
    for(int dist = 0; dist < Q - 1; ++dist) v[V_U(d)] += L->c[dist][d] * c->fold[cell * Q + dist];
    v[V_U(d)] /= v[V_RHO(c)];
  }
}
/* calcDensity (Poisson), src/lbm/moments.h:85-95 */
static void potential_cell(ora_ctx* c, int64_t cell) {
  const lattice_t* L   = &c->L;
  const int        Q   = L->q;
  double           acc = 0;
  for(int dist = 0; dist < Q - 1; ++dist) acc += c->fold[cell * Q + dist];
  c->vars[cell * c->nvar + 0] = 1.0 / (1.0 - L->w[Q - 1]) * acc;
}

/* LBMBnd_DirichletNEEM::apply, src/lbm/bnd/bnd_dirichlet.h:354-373 */
static void dirichlet_neem_apply(ora_ctx* c, bnd_t* b) {
  const lattice_t* L = &c->L;
  const int        Q = L->q;
  for(int64_t i = 0; i < b->n; ++i) potential_cell(c, b->ext[i]);
  for(int64_t i = 0; i < b->n; ++i) {
    const int64_t cell = b->cells[i], ext = b->ext[i];
    const double  val  = b->values[i];
    c->vars[cell * c->nvar + 0] = val;
    const double phiExt         = c->vars[ext * c->nvar + 0];
    for(int dist = 0; dist < Q - 1; ++dist) {
      const double w           = L->w[dist];
      c->fold[cell * Q + dist] = w * val + c->fold[ext * Q + dist] - w * phiExt;
    }
    c->fold[cell * Q + Q - 1] = (L->w[Q - 1] - 1.0) * val + c->fold[ext * Q + Q - 1] - (L->w[Q - 1] - 1.0) * phiExt;
  }
}

/* LBMBndManager::apply, src/lbm/bnd/bnd.h:60-65 */
static void apply_bnds(ora_ctx* c) {
  const lattice_t* L = &c->L;
  const int        Q = L->q, D = L->ndim;
  for(int k = 0; k < c->nbnd; ++k) {
    bnd_t* b = &c->bnds[k];
    switch(b->kind) {
      case ORA_BND_WALL_BB:
      case ORA_BND_WALL_BB_TANGENTIAL:
      case ORA_BND_DIRICHLET_BB: {
        /* LBMBnd_DirichletBB::apply<VALZERO,SCALAR>, bnd_dirichlet.h:79-121 */
        for(int64_t i = 0; i < b->n; ++i) {
          const int64_t cell = b->cells[i];
          const double* nrm  = &b->normals[i * D];
          for(int dist = 0; dist < Q - 1; ++dist) {
            if(NB(c, cell, dist) == INVALID && in_direction(nrm, L->c[dist], D)) {
              const int opp            = L->opp[dist];
              c->fold[cell * Q + opp] = c->f[cell * Q + dist];
              if(c->eq == ORA_NAVIER_STOKES) {
                const double density = 1.0;
                if(b->kind == ORA_BND_WALL_BB_TANGENTIAL) {
                  c->fold[cell * Q + opp] += density * 2.0 / CSSQ * L->w[opp] * b->tang[i * Q + opp];
                } else if(b->kind == ORA_BND_DIRICHLET_BB) {
                  for(int d = 0; d < D; ++d) c->fold[cell * Q + opp] += density * 2.0 / CSSQ * L->w[opp] * L->c[opp][d] * b->vec[d];
                }
              }
            }
          }
        }
        break;
      }
      case ORA_BND_PERIODIC:
        break;
      case ORA_BND_WALL_EQ:
      case ORA_BND_WALL_NEEM: {
        /* LBMBnd_wallEq::apply_0 / apply_constV, bnd_wall.h:143-155 */
        const int valzero = !b->has_vec;
        for(int64_t i = 0; i < b->n; ++i) dirichlet_eq_cell(c, b, b->cells[i], b->vec, valzero);
        if(b->kind == ORA_BND_WALL_NEEM) {
          /* LBMBnd_wallNEEM::apply_general, bnd_wall.h:275-297 */
          for(int64_t i = 0; i < b->n; ++i) moments_ns_cell(c, b->ext[i]);
          for(int64_t i = 0; i < b->n; ++i) velocity_ns_cell(c, b->ext[i]);
          for(int64_t i = 0; i < b->n; ++i) {
            const int64_t cell = b->cells[i], ext = b->ext[i];
            if(ext == INVALID) continue;
            for(int dist = 0; dist < Q; ++dist) {
              const double* ve = &c->vars[ext * c->nvar];
              c->fold[cell * Q + dist] += c->fold[ext * Q + dist] - eq_default_dist(L, dist, ve[V_RHO(c)], ve);
            }
          }
        }
        break;
      }
      case ORA_BND_WALL_NEBB: {
        if(!b->has_vec) {
          /* LBMBnd_wallNEBB::apply_0, bnd_wall.h:358-406 */
          for(int64_t i = 0; i < b->n; ++i)
            for(int d = 0; d < D; ++d) c->vars[b->cells[i] * c->nvar + V_U(d)] = 0;
          for(int64_t i = 0; i < b->n; ++i) density_limited(c, b, i, 1);
          for(int64_t i = 0; i < b->n; ++i) {
            const int64_t cell = b->cells[i];
            for(int dist = 0; dist < 2 * D; ++dist)
              if(NB(c, cell, dist) == INVALID) c->fold[cell * Q + (dist + 1 - 2 * (dist % 2))] = c->fold[cell * Q + dist];
          }
          /* the reference never advances `index` in this loop: every cell uses
             the first cell's normal */
          const double* nrm = &b->normals[0];
          for(int64_t i = 0; i < b->n; ++i) {
            double* fo = &c->fold[b->cells[i] * Q];
            if(nrm[0] < 0) {
              fo[6] = fo[4] + 0.5 * (fo[3] - fo[2]);
              fo[7] = fo[5] - 0.5 * (fo[3] - fo[2]);
            } else if(nrm[0] > 0) {
              fo[4] = fo[6] - 0.5 * (fo[3] - fo[2]);
              fo[5] = fo[7] + 0.5 * (fo[3] - fo[2]);
            } else if(nrm[1] < 0) {
              fo[5] = fo[7] - 0.5 * (fo[1] - fo[0]);
              fo[6] = fo[4] + 0.5 * (fo[1] - fo[0]);
            } else if(nrm[1] > 0) {
              fo[7] = fo[5] + 0.5 * (fo[1] - fo[0]);
              fo[4] = fo[6] - 0.5 * (fo[1] - fo[0]);
            }
          }
        } else {
          /* LBMBnd_wallNEBB::apply_constV, bnd_wall.h:408-471 */
          const double* wv = b->vec;
          for(int64_t i = 0; i < b->n; ++i) {
            density_limited(c, b, i, 0);
            for(int d = 0; d < D; ++d) c->vars[b->cells[i] * c->nvar + V_U(d)] = wv[d];
          }
          for(int64_t i = 0; i < b->n; ++i) {
            const int64_t cell = b->cells[i];
            const double* nrm  = &b->normals[i * D];
            double*       fo   = &c->fold[cell * Q];
            for(int dist = 0; dist < 2 * D; ++dist) {
              const int dir = dist / 2;
              if(NB(c, cell, dist) == INVALID && fabs(nrm[dir]) > 0) {
                const int od = dist + 1 - 2 * (dist % 2);
                fo[od]       = fo[dist];
                if(nrm[dir] < 0) fo[od] -= 2.0 / 3.0 * c->vars[cell * c->nvar + V_RHO(c)] * wv[dir];
                else fo[od] += 2.0 / 3.0 * c->vars[cell * c->nvar + V_RHO(c)] * wv[dir];
              }
            }
          }
          for(int64_t i = 0; i < b->n; ++i) {
            const int64_t cell = b->cells[i];
            const double  rho  = c->vars[cell * c->nvar + V_RHO(c)];
            const double* nrm  = &b->normals[i * D];
            double*       fo   = &c->fold[cell * Q];
            if(nrm[0] > 0) {
              fo[6] = fo[4] + 0.5 * (fo[3] - fo[2]) - 0.5 * rho * wv[1] - 1.0 / 6.0 * rho * wv[0];
              fo[7] = fo[5] - 0.5 * (fo[3] - fo[2]) + 0.5 * rho * wv[1] - 1.0 / 6.0 * rho * wv[0];
            } else if(nrm[0] < 0) {
              fo[4] = fo[6] - 0.5 * (fo[3] - fo[2]) + 0.5 * rho * wv[1] + 1.0 / 6.0 * rho * wv[0];
              fo[5] = fo[7] + 0.5 * (fo[3] - fo[2]) - 0.5 * rho * wv[1] + 1.0 / 6.0 * rho * wv[0];
            } else if(nrm[1] > 0) {
              fo[5] = fo[7] - 0.5 * (fo[1] - fo[0]) + 0.5 * rho * wv[0] - 1.0 / 6.0 * rho * wv[1];
              fo[6] = fo[4] + 0.5 * (fo[1] - fo[0]) - 0.5 * rho * wv[0] - 1.0 / 6.0 * rho * wv[1];
            } else if(nrm[1] < 0) {
              fo[7] = fo[5] + 0.5 * (fo[1] - fo[0]) - 0.5 * rho * wv[0] + 1.0 / 6.0 * rho * wv[1];
              fo[4] = fo[6] - 0.5 * (fo[1] - fo[0]) + 0.5 * rho * wv[0] + 1.0 / 6.0 * rho * wv[1];
            }
          }
        }
        break;
      }
      case ORA_BND_PRESSURE_ABB: {
        /* LBMBnd_Pressure::apply, bnd_pressure.h:271-322 */
        for(int64_t i = 0; i < b->n; ++i) {
          const int64_t cell = b->cells[i];
          const double* nrm  = &b->normals[i * D];
          const int     id   = inside_dir(nrm, D);
          const int64_t n1   = NB(c, cell, id);
          const int64_t n2   = NB(c, n1, id);
          double        u[3];
          for(int d = 0; d < D; ++d) u[d] = 1.5 * c->vars[n1 * c->nvar + V_U(d)] - 0.5 * c->vars[n2 * c->nvar + V_U(d)];
          for(int dist = 0; dist < Q; ++dist) {
            double* v   = &c->vars[cell * c->nvar];
            v[V_RHO(c)] = b->scalar;
            v[V_U(0)]   = u[0];
            v[V_U(1)]   = u[1];
            if(dist < Q - 1 && NB(c, cell, dist) == INVALID && in_direction(nrm, L->c[dist], D)) {
              const int opp            = L->opp[dist];
              c->fold[cell * Q + opp] = -c->f[cell * Q + dist] + 2 * eq_symm_dist(L, dist, b->scalar, u);
            }
          }
        }
        break;
      }
      case ORA_BND_DIRICHLET_NEEM:
        dirichlet_neem_apply(c, b);
        break;
      case ORA_BND_NEUMANN_NEEM: {
        /* LBMBnd_NeumannNEEM::apply, src/lbm/bnd/bnd_neumann.h:373-392 (m_gradValue = 0) */
        const double grad = 0.0;
        for(int64_t i = 0; i < b->n; ++i) {
          const int64_t ext = b->ext[i];
          const int64_t ex2 = NB(c, ext, b->ext_dir[i]);
          potential_cell(c, ex2);
          b->values[i] = (4.0 * c->vars[ext * c->nvar + 0] - c->vars[ex2 * c->nvar + 0] + grad) / 3.0;
        }
        dirichlet_neem_apply(c, b);
        break;
      }
      default:
        break;
    }
  }
}

/* timeStep, src/lbm/solver.cpp:306-320 */
void ora_step(ora_ctx* c, int64_t nsteps) {
  for(int64_t s = 0; s < nsteps; ++s) {
    memcpy(c->varsold, c->vars, sizeof(double) * c->n * c->nvar); /* currToOldVars */
    ora_update_moments(c);
    equilibrium(c);
    collide(c);
    forcing(c);
    pre_apply(c);
    propagate(c);
    apply_bnds(c);
  }
}

/* sumAbsDiff, src/lbm/solver.cpp:808-815 */
void ora_residual(const ora_ctx* c, double* r) {
  for(int v = 0; v < c->nvar; ++v) {
    double conv = 0.0;
    for(int64_t cell = 0; cell < c->n; ++cell) conv += fabs(c->vars[cell * c->nvar + v] - c->varsold[cell * c->nvar + v]);
    r[v] = conv;
  }
}

void ora_get(const ora_ctx* c, double* fold, double* f, double* vars, double* varsold) {
  const int64_t nq = c->n * c->L.q;
  if(fold) memcpy(fold, c->fold, sizeof(double) * nq);
  if(f) memcpy(f, c->f, sizeof(double) * nq);
  if(vars) memcpy(vars, c->vars, sizeof(double) * c->n * c->nvar);
  if(varsold) memcpy(varsold, c->varsold, sizeof(double) * c->n * c->nvar);
}

void ora_set_state(ora_ctx* c, const double* fold, const double* vars) {
  if(fold) memcpy(c->fold, fold, sizeof(double) * c->n * c->L.q);
  if(vars) memcpy(c->vars, vars, sizeof(double) * c->n * c->nvar);
}
