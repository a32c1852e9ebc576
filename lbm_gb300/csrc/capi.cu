// C ABI of the GB300 LBM library (include/lbm_gpu.h): contexts, the one-time
// table build from the reference's grid and boundary descriptions, and the
// step / reduction / transfer entry points.
//
// The derived boundary tables restate what the reference's BC constructors
// compute once (limited distribution sets, extrapolation cells, periodic
// links, tangential wall values) and flatten them into per-entry device
// arrays, so every boundary loop of the step becomes one data-parallel
// kernel.  Where the reference's sequential loop order would matter (two list
// entries writing the same slot) the build keeps the last writer, exactly as
// the sequential loop does, or rejects the configuration with
// LBM_ERR_UNSUPPORTED when no flat form preserves the order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <set>
#include <string>
#include <vector>

#include "batch.h"
#include "box.h"
#include "engine.h"
#include "lattice.cuh"

using namespace lbm;

struct HostBnd {
  int                  kind = 0;
  std::vector<int64_t> cells;
  std::vector<double>  values;
  double               vec[3] = {0, 0, 0};
  double               scalar = 0;
};

struct lbm_gpu_ctx {
  int                    mode   = 0;  // 0 reference tables, 1 dense box, 2 batched cavities
  int                    device = 0;
  cudaStream_t           stream = nullptr;
  std::string            err;
  TableState             t;
  int                    ndim = 0;
  std::vector<int64_t>   nghbr;  // host copy, cell-major
  std::vector<double>    centers;
  double                 bbox[6]     = {0, 0, 0, 0, 0, 0};
  double                 cell_length = 0;
  std::vector<uint8_t>   periodic;
  std::vector<HostBnd>   hbnds;
  std::vector<void*>     allocs;
  double*                d_partials = nullptr;
  double*                d_out      = nullptr;
  int                    nblocks    = 1;
  cudaGraphExec_t        graph      = nullptr;
  int                    graph_steps = 0;
  BoxState*              box        = nullptr;
  BatchState*            batch      = nullptr;
};

namespace {

constexpr double EPSD = 2.220446049250313080847e-16;

int fail(lbm_gpu_ctx* c, int code, const std::string& msg) {
  if(c) c->err = msg;
  return code;
}

int cuda_fail(lbm_gpu_ctx* c, cudaError_t e, const char* what) {
  return fail(c, LBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                  \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if(_e != cudaSuccess) return cuda_fail(ctx, _e, #call);       \
  } while(0)

template <class T>
T* dalloc(lbm_gpu_ctx* ctx, size_t count) {
  void* p = nullptr;
  if(count == 0) count = 1;
  if(cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
  ctx->allocs.push_back(p);
  return static_cast<T*>(p);
}

template <class T>
T* upload(lbm_gpu_ctx* ctx, const std::vector<T>& h) {
  T* d = dalloc<T>(ctx, h.size());
  if(!d) return nullptr;
  if(!h.empty() && cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
  return d;
}

int lattice_q(int lat) {
  switch(lat) {
    case LBM_D1Q3: return 3;
    case LBM_D2Q5: return 5;
    case LBM_D2Q9: return 9;
    case LBM_D3Q7: return 7;
    case LBM_D3Q19: return 19;
    default: return 0;
  }
}
int lattice_d(int lat) {
  switch(lat) {
    case LBM_D1Q3: return 1;
    case LBM_D2Q5:
    case LBM_D2Q9: return 2;
    default: return 3;
  }
}

// lattice velocity / opposite / weight lookup on the host
struct HostLattice {
  int    D = 0, Q = 0;
  int    c[19][3];
  int    opp[19];
  double w[19];
};

template <int LAT>
HostLattice make_host_lattice() {
  using L = Lattice<LAT>;
  HostLattice h;
  h.D = L::D;
  h.Q = L::Q;
  for(int q = 0; q < L::Q; ++q) {
    for(int d = 0; d < 3; ++d) h.c[q][d] = L::c(q, d);
    h.opp[q] = L::opp(q);
    h.w[q]   = L::w(q);
  }
  return h;
}

HostLattice host_lattice(int lat) {
  switch(lat) {
    case LBM_D1Q3: return make_host_lattice<LBM_D1Q3>();
    case LBM_D2Q5: return make_host_lattice<LBM_D2Q5>();
    case LBM_D2Q9: return make_host_lattice<LBM_D2Q9>();
    case LBM_D3Q7: return make_host_lattice<LBM_D3Q7>();
    default: return make_host_lattice<LBM_D3Q19>();
  }
}

bool in_direction(const double* n, const int* c, int D) {
  double s = 0;
  for(int d = 0; d < D; ++d) s += n[d] * static_cast<double>(c[d]);
  return s >= EPSD;
}
bool orthogonal(const double* n, const int* c, int D) {
  double s = 0;
  for(int d = 0; d < D; ++d) s += n[d] * static_cast<double>(c[d]);
  return std::fabs(s) <= EPSD;
}
// extrapolation / inside direction of a wall normal (bnd_wall.h:213-223)
int inside_dir(const double* n, int D) {
  for(int d = 0; d < D; ++d) {
    if(n[d] < 0) return 2 * d + 1;
    if(n[d] > 0) return 2 * d;
  }
  return -1;
}

void free_graph(lbm_gpu_ctx* ctx) {
  if(ctx->graph) cudaGraphExecDestroy(ctx->graph);
  ctx->graph       = nullptr;
  ctx->graph_steps = 0;
}

// LBMBnd_wallWetnode constructor (src/lbm/bnd/bnd_wetnode.h:21-60)
void build_wetnode(lbm_gpu_ctx* ctx, const HostLattice& L, const lbm_bnd_desc* b, std::vector<double>& lim_const,
                   std::vector<int8_t>& lim_empty) {
  const int Q = L.Q, D = L.D, nn = ctx->t.nnghbr;
  lim_const.assign(b->ncells * Q, 0.0);
  lim_empty.assign(b->ncells, 0);
  for(int64_t i = 0; i < b->ncells; ++i) {
    const int64_t cell = b->cells[i];
    const double* nrm  = &b->normals[i * D];
    const bool    per  = ctx->periodic[cell] != 0;
    double*       k    = &lim_const[i * Q];
    for(int dir = 0; dir < Q - 1; ++dir) {
      const int  opp     = L.opp[dir];
      const bool oppnbr  = ctx->nghbr[cell * nn + opp] != -1;
      if(in_direction(nrm, L.c[dir], D) && (per || oppnbr)) {
        k[dir] = 2;
      } else if(orthogonal(nrm, L.c[dir], D) && (per || oppnbr)) {
        k[dir] = (ctx->nghbr[cell * nn + dir] == -1 && !per) ? 2 : 1;
      }
    }
    int sumC = 0;
    for(int q = 0; q < Q; ++q) sumC = static_cast<int>(sumC + k[q]);
    if(sumC != Q - 1) {
      lim_empty[i] = 1;  // corner: the reference clears the set and skips the cell
    } else {
      k[Q - 1] = 1;
    }
  }
}

bool has_duplicates(const int64_t* a, int64_t n) {
  std::set<int64_t> s(a, a + n);
  return static_cast<int64_t>(s.size()) != n;
}

}  // namespace

extern "C" {

int lbm_gpu_abi_version(void) { return LBM_GPU_ABI_VERSION; }

const char* lbm_gpu_last_error(const lbm_gpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int lbm_gpu_create(const lbm_table_desc* desc, const int64_t* nghbr, const double* centers, lbm_gpu_ctx** out) {
  if(!desc || !nghbr || !centers || !out) return LBM_ERR_INVALID;
  *out = nullptr;
  const int lat = desc->lattice, eq = desc->equation;
  const bool supported = (lat == LBM_D2Q9 && (eq == LBM_NAVIER_STOKES || eq == LBM_POISSON)) ||
                         (lat == LBM_D2Q5 && eq == LBM_POISSON) || (lat == LBM_D1Q3 && eq == LBM_POISSON);
  if(!supported) return LBM_ERR_UNSUPPORTED;
  const int Q = lattice_q(lat), D = lattice_d(lat);
  if(desc->ncells <= 0 || desc->ncells >= (int64_t(1) << 31)) return LBM_ERR_INVALID;
  if(desc->nnghbr < Q - 1) return LBM_ERR_INVALID;
  if(!(desc->omega > 0.0)) return LBM_ERR_INVALID;
  lbm_gpu_ctx* ctx = new(std::nothrow) lbm_gpu_ctx();
  if(!ctx) return LBM_ERR_NOMEM;
  ctx->device = desc->device;
  if(cudaSetDevice(ctx->device) != cudaSuccess) {
    delete ctx;
    return LBM_ERR_CUDA;
  }
  const int64_t n = desc->ncells, nn = desc->nnghbr;
  for(int64_t i = 0; i < n * nn; ++i) {
    if(nghbr[i] < -1 || nghbr[i] >= n) {
      delete ctx;
      return LBM_ERR_TABLE;
    }
  }
  TableState& t = ctx->t;
  t.lattice = lat;
  t.equation = eq;
  t.D = D;
  t.Q = Q;
  t.nvar = eq == LBM_POISSON ? 1 : D + 1;
  t.nnghbr = static_cast<int>(nn);
  t.n = n;
  t.omega = desc->omega;
  t.relax_time = desc->relax_time;
  t.dt = desc->dt;
  t.poisson_k = desc->poisson_k;
  // `static const GDouble diffusivity` of collisionStep (src/lbm/solver.cpp:606)
  double alpha = 0;
  if(lat == LBM_D1Q3) alpha = Lattice<LBM_D1Q3>::poisson_alpha;
  if(lat == LBM_D2Q5) alpha = Lattice<LBM_D2Q5>::poisson_alpha;
  if(lat == LBM_D2Q9) alpha = Lattice<LBM_D2Q9>::poisson_alpha;
  const double lattice_velocity = 1.0;
  t.diffusivity = alpha * (lattice_velocity * lattice_velocity) * (0.5 - t.relax_time) * t.dt;
  ctx->ndim = D;
  ctx->nghbr.assign(nghbr, nghbr + n * nn);
  ctx->centers.assign(centers, centers + n * D);
  for(int i = 0; i < 6; ++i) ctx->bbox[i] = desc->bbox[i];
  ctx->cell_length = desc->cell_length;
  ctx->periodic.assign(n, 0);

  int rc = LBM_OK;
  if(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) rc = LBM_ERR_CUDA;
  // pull form of the push propagation: src[q][target] = the cell that pushes
  // into target along q (a sequential push keeps the last writer)
  std::vector<int32_t> src((Q - 1) * n, -1), nbr32(nn * n, -1);
  for(int64_t p = 0; p < n; ++p) {
    for(int q = 0; q < nn; ++q) nbr32[q * n + p] = static_cast<int32_t>(nghbr[p * nn + q]);
    for(int q = 0; q < Q - 1; ++q) {
      const int64_t tgt = nghbr[p * nn + q];
      if(tgt >= 0) src[q * n + tgt] = static_cast<int32_t>(p);
    }
  }
  if(rc == LBM_OK) {
    t.fold    = dalloc<double>(ctx, Q * n);
    t.f       = dalloc<double>(ctx, Q * n);
    t.feq     = dalloc<double>(ctx, Q * n);
    t.vars    = dalloc<double>(ctx, t.nvar * n);
    t.varsold = dalloc<double>(ctx, t.nvar * n);
    t.src     = upload(ctx, src);
    t.nbr     = upload(ctx, nbr32);
    ctx->nblocks    = reduce_blocks(n);
    ctx->d_partials = dalloc<double>(ctx, 8 * ctx->nblocks);
    ctx->d_out      = dalloc<double>(ctx, 8);
    if(!t.fold || !t.f || !t.feq || !t.vars || !t.varsold || !t.src || !t.nbr || !ctx->d_partials || !ctx->d_out) rc = LBM_ERR_NOMEM;
  }
  if(rc == LBM_OK) {
    cudaMemset(t.fold, 0, sizeof(double) * Q * n);
    cudaMemset(t.f, 0, sizeof(double) * Q * n);
    cudaMemset(t.feq, 0, sizeof(double) * Q * n);
    cudaMemset(t.vars, 0, sizeof(double) * t.nvar * n);
    cudaMemset(t.varsold, 0, sizeof(double) * t.nvar * n);
    if(cudaDeviceSynchronize() != cudaSuccess) rc = LBM_ERR_CUDA;
  }
  if(rc != LBM_OK) {
    lbm_gpu_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return LBM_OK;
}

int lbm_gpu_add_boundary(lbm_gpu_ctx* ctx, const lbm_bnd_desc* b) {
  if(!ctx || !b) return LBM_ERR_INVALID;
  if(ctx->mode != 0) return fail(ctx, LBM_ERR_INVALID, "boundary objects belong to reference-table contexts");
  if(b->ncells <= 0) return LBM_OK;  // "Skipping ... no valid cells" (bnd.h:82-86)
  if(!b->cells || !b->normals) return fail(ctx, LBM_ERR_INVALID, "boundary without cells or normals");
  CK(cudaSetDevice(ctx->device));
  TableState&       t = ctx->t;
  const HostLattice L = host_lattice(t.lattice);
  const int         Q = L.Q, D = L.D, nn = t.nnghbr;
  const int64_t     n = t.n, m = b->ncells;
  for(int64_t i = 0; i < m; ++i)
    if(b->cells[i] < 0 || b->cells[i] >= n) return fail(ctx, LBM_ERR_TABLE, "boundary cell id out of range");
  auto NB = [&](int64_t cell, int dir) { return ctx->nghbr[cell * nn + dir]; };

  TableBnd tb;
  tb.kind      = b->kind;
  tb.has_vec   = b->has_vec;
  tb.has_press = b->has_pressure;
  tb.n         = m;
  for(int d = 0; d < 3; ++d) tb.vec[d] = d < D ? b->vec[d] : 0.0;
  tb.scalar = b->scalar;
  HostBnd hb;
  hb.kind = b->kind;
  hb.cells.assign(b->cells, b->cells + m);
  for(int d = 0; d < 3; ++d) hb.vec[d] = tb.vec[d];
  hb.scalar = b->scalar;

  std::vector<int32_t> cells32(m);
  for(int64_t i = 0; i < m; ++i) cells32[i] = static_cast<int32_t>(b->cells[i]);
  std::vector<double> normals(b->normals, b->normals + m * D);
  tb.cells   = upload(ctx, cells32);
  tb.normals = upload(ctx, normals);
  if(!tb.cells || !tb.normals) return fail(ctx, LBM_ERR_NOMEM, "device allocation failed");
  const bool ns = t.equation == LBM_NAVIER_STOKES;

  auto finish_ext = [&](const std::vector<int32_t>& ext) -> int {
    std::vector<int32_t> extu;
    std::set<int32_t>    seen;
    for(int32_t e : ext)
      if(seen.insert(e).second) extu.push_back(e);
    std::set<int64_t> mine(b->cells, b->cells + m);
    for(int32_t e : extu)
      if(mine.count(e)) return fail(ctx, LBM_ERR_UNSUPPORTED, "extrapolation cell lies on its own boundary surface");
    tb.ext   = upload(ctx, ext);
    tb.extu  = upload(ctx, extu);
    tb.nextu = static_cast<int64_t>(extu.size());
    return (tb.ext && tb.extu) ? LBM_OK : fail(ctx, LBM_ERR_NOMEM, "device allocation failed");
  };

  switch(b->kind) {
    case LBM_BND_PERIODIC: {
      if(!b->conn_cells || b->nconn <= 0) return fail(ctx, LBM_ERR_INVALID, "periodic boundary without a connected surface");
      // addPeriodicBndry marks both surfaces periodic (bnd.h:217-221)
      for(int64_t i = 0; i < m; ++i) ctx->periodic[b->cells[i]] = 1;
      for(int64_t j = 0; j < b->nconn; ++j) {
        if(b->conn_cells[j] < 0 || b->conn_cells[j] >= n) return fail(ctx, LBM_ERR_TABLE, "connected cell id out of range");
        ctx->periodic[b->conn_cells[j]] = 1;
      }
      // LBMBndCell_periodic::init (src/lbm/bnd/bnd_periodic.h:31-100)
      std::map<std::pair<int64_t, int>, int64_t> last_copy;  // (dst,q) -> src, last writer wins
      std::vector<std::pair<std::pair<int64_t, int>, int64_t>> order;
      std::vector<int32_t> link0(m, 0);  // m_linkedCell{} is zero-initialised
      for(int64_t i = 0; i < m; ++i) {
        const int64_t cell   = b->cells[i];
        const double* nrm    = &b->normals[i * D];
        const double* center = &ctx->centers[cell * D];
        std::vector<int> set;
        for(int dist = 0; dist < Q; ++dist) {
          if(!in_direction(nrm, L.c[dist], D)) continue;
          double coord[3];
          for(int d = 0; d < D; ++d) coord[d] = std::fabs(nrm[d]) > 0 ? ctx->bbox[2 * d] : center[d] + L.c[dist][d] * ctx->cell_length;
          bool inside = true;
          for(int d = 0; d < D; ++d)
            if(coord[d] < ctx->bbox[2 * d] || coord[d] > ctx->bbox[2 * d + 1]) inside = false;
          if(inside) set.push_back(dist);
        }
        for(size_t id = 0; id < set.size(); ++id) {
          const int dist = set[id];
          double    centerA[3];
          for(int d = 0; d < D; ++d) centerA[d] = center[d] + (std::fabs(nrm[d]) > 0 ? 0.0 : L.c[dist][d] * ctx->cell_length);
          int64_t linked = -1;
          for(int64_t j = 0; j < b->nconn && linked < 0; ++j) {
            const double* cb = &ctx->centers[b->conn_cells[j] * D];
            for(int d = 0; d < D; ++d)
              if(std::fabs(centerA[d] - cb[d]) <= 10 * EPSD) {  // a match in any one direction, as in the reference
                linked = b->conn_cells[j];
                break;
              }
          }
          if(linked < 0) return fail(ctx, LBM_ERR_TABLE, "periodic boundary: no cell to link");
          for(size_t jd = 0; jd < id; ++jd) {
            (void)jd;
          }
          if(id == 0) link0[i] = static_cast<int32_t>(linked);
          const auto key = std::make_pair(linked, dist);
          last_copy[key]  = cell;
          order.push_back({key, cell});
        }
      }
      if(b->has_pressure) {
        if(!ns) return fail(ctx, LBM_ERR_UNSUPPORTED, "periodic pressure needs Navier-Stokes");
        // (mapped, link0) pairs; a later pair to the same link0 overwrites it
        std::map<int32_t, int64_t> last;
        for(int64_t i = 0; i < m; ++i) last[link0[i]] = i;
        std::vector<int32_t> mapped, l0;
        for(int64_t i = 0; i < m; ++i)
          if(last[link0[i]] == i) {
            mapped.push_back(cells32[i]);
            l0.push_back(link0[i]);
          }
        tb.n     = static_cast<int64_t>(mapped.size());
        tb.cells = upload(ctx, mapped);
        tb.link0 = upload(ctx, l0);
        t.need_feq = true;
      } else {
        std::vector<int32_t> dst, qq, srcc;
        std::set<std::pair<int64_t, int>> emitted;
        for(auto it = order.rbegin(); it != order.rend(); ++it) {
          if(!emitted.insert(it->first).second) continue;
          dst.push_back(static_cast<int32_t>(it->first.first));
          qq.push_back(it->first.second);
          srcc.push_back(static_cast<int32_t>(it->second));
        }
        tb.ncopy    = static_cast<int64_t>(dst.size());
        tb.copy_dst = upload(ctx, dst);
        tb.copy_q   = upload(ctx, qq);
        tb.copy_src = upload(ctx, srcc);
        tb.link0    = upload(ctx, link0);
      }
      break;
    }
    case LBM_BND_WALL_BB:
    case LBM_BND_DIRICHLET_BB:
      break;
    case LBM_BND_WALL_BB_TANGENTIAL: {
      if(D != 2) return fail(ctx, LBM_ERR_UNSUPPORTED, "tangential wall velocity is 2D only");
      // LBMBnd_wallBB<true>::init (src/lbm/bnd/bnd_wall.h:31-72)
      std::vector<double> tang(m * Q, 0.0);
      for(int64_t i = 0; i < m; ++i) {
        const double* nrm = &b->normals[i * D];
        for(int id = 0; id < Q; ++id) {
          if(!in_direction(nrm, L.c[id], D)) continue;
          const int    inside = L.opp[id];
          const int*   dir    = L.c[inside];
          const double ndot   = nrm[0] * dir[0] + nrm[1] * dir[1];
          const double cross  = nrm[0] * dir[1] - nrm[1] * dir[0];
          const bool   par    = cross == 0.0 && ndot < 0.0;  // angle(n, dir) == pi
          if(!par) tang[i * Q + inside] = b->scalar * (nrm[1] * dir[0] + nrm[0] * dir[1]);
        }
      }
      tb.tang = upload(ctx, tang);
      break;
    }
    case LBM_BND_WALL_EQ:
    case LBM_BND_WALL_NEEM:
    case LBM_BND_WALL_NEBB: {
      if(!ns) return fail(ctx, LBM_ERR_UNSUPPORTED, "wall models need Navier-Stokes");
      if(b->kind == LBM_BND_WALL_NEBB && t.lattice != LBM_D2Q9) return fail(ctx, LBM_ERR_UNSUPPORTED, "NEBB is D2Q9 only");
      if(has_duplicates(b->cells, m)) return fail(ctx, LBM_ERR_UNSUPPORTED, "wet-node wall with a repeated cell");
      std::vector<double> lim;
      std::vector<int8_t> empty;
      build_wetnode(ctx, L, b, lim, empty);
      tb.lim_const = upload(ctx, lim);
      tb.lim_empty = upload(ctx, empty);
      std::vector<int32_t> widx(m);
      for(int64_t i = 0; i < m; ++i) widx[i] = static_cast<int32_t>(i);
      tb.widx = upload(ctx, widx);
      if(b->kind == LBM_BND_WALL_NEEM) {
        // LBMBnd_wallNEEM::init (src/lbm/bnd/bnd_wall.h:212-248)
        std::vector<int32_t> ext(m);
        for(int64_t i = 0; i < m; ++i) {
          const int dir = inside_dir(&b->normals[i * D], D);
          const int64_t e = dir < 0 ? -1 : NB(b->cells[i], dir);
          if(e < 0) return fail(ctx, LBM_ERR_TABLE, "No valid extrapolation cellId");
          ext[i] = static_cast<int32_t>(e);
        }
        if(int rc = finish_ext(ext)) return rc;
      }
      break;
    }
    case LBM_BND_PRESSURE_ABB: {
      if(!ns || D != 2) return fail(ctx, LBM_ERR_UNSUPPORTED, "pressure boundary is 2D Navier-Stokes only");
      std::vector<int32_t> n1(m), n2(m);
      std::set<int64_t>    mine(b->cells, b->cells + m);
      for(int64_t i = 0; i < m; ++i) {
        const int dir = inside_dir(&b->normals[i * D], D);
        const int64_t a = dir < 0 ? -1 : NB(b->cells[i], dir);
        const int64_t c2 = a < 0 ? -1 : NB(a, dir);
        if(a < 0 || c2 < 0) return fail(ctx, LBM_ERR_TABLE, "pressure boundary: missing inside neighbours");
        if(mine.count(a) || mine.count(c2)) return fail(ctx, LBM_ERR_UNSUPPORTED, "pressure boundary: inside cell on the surface");
        n1[i] = static_cast<int32_t>(a);
        n2[i] = static_cast<int32_t>(c2);
      }
      tb.ext  = upload(ctx, n1);
      tb.ext2 = upload(ctx, n2);
      break;
    }
    case LBM_BND_DIRICHLET_NEEM:
    case LBM_BND_NEUMANN_NEEM: {
      if(ns) return fail(ctx, LBM_ERR_UNSUPPORTED, "NEEM Dirichlet/Neumann needs the Poisson equation");
      if(has_duplicates(b->cells, m)) return fail(ctx, LBM_ERR_UNSUPPORTED, "NEEM surface with a repeated cell");
      // LBMBnd_DirichletNEEM constructor (src/lbm/bnd/bnd_dirichlet.h:263-316)
      std::vector<int32_t> ext(m), ext2(m);
      std::vector<double>  values(m);
      for(int64_t i = 0; i < m; ++i) {
        const int64_t cell = b->cells[i];
        int           ed   = -1;
        for(int dist = 0; dist < 2 * D; ++dist) {
          if(NB(cell, dist) != -1) continue;
          if(ed < 0) {
            ed = dist;
          } else {
            if(ed == 0 && dist == 2) ed = 6;
            if(ed == 0 && dist == 3) ed = 7;
            if(ed == 1 && dist == 3) ed = 4;
            if(ed == 1 && dist == 2) ed = 5;
          }
        }
        if(ed < 0) return fail(ctx, LBM_ERR_TABLE, "No valid extrapolation cellId");
        const int od = ed < 2 * D ? ed + 1 - 2 * (ed % 2) : (ed > 5 ? ed - 2 : ed + 2);
        if(od >= nn) return fail(ctx, LBM_ERR_TABLE, "extrapolation direction outside the neighbour table");
        const int64_t e = NB(cell, od);
        if(e < 0) return fail(ctx, LBM_ERR_TABLE, "No valid extrapolation cellId");
        ext[i]    = static_cast<int32_t>(e);
        const int64_t e2 = NB(e, od);
        if(b->kind == LBM_BND_NEUMANN_NEEM && e2 < 0) return fail(ctx, LBM_ERR_TABLE, "Neumann: no second extrapolation cell");
        ext2[i]   = static_cast<int32_t>(e2);
        values[i] = b->values ? b->values[i] : b->scalar;
      }
      if(b->kind == LBM_BND_NEUMANN_NEEM) {
        std::set<int32_t> e1(ext.begin(), ext.end());
        for(int32_t e : ext2)
          if(e1.count(e)) return fail(ctx, LBM_ERR_UNSUPPORTED, "Neumann: overlapping extrapolation stencils");
      }
      tb.values = upload(ctx, values);
      tb.ext2   = upload(ctx, ext2);
      hb.values = values;
      if(int rc = finish_ext(ext)) return rc;
      break;
    }
    default:
      return fail(ctx, LBM_ERR_INVALID, "unknown boundary kind");
  }
  ctx->hbnds.push_back(hb);
  t.bnds.push_back(tb);
  free_graph(ctx);
  return LBM_OK;
}

int lbm_gpu_set_forcing(lbm_gpu_ctx* ctx, double dp, int64_t nin, const int64_t* in, int64_t nout, const int64_t* outc) {
  if(!ctx || (nin && !in) || (nout && !outc)) return LBM_ERR_INVALID;
  TableState& t = ctx->t;
  if(ctx->mode != 0 || t.equation != LBM_NAVIER_STOKES || t.D != 2) return fail(ctx, LBM_ERR_UNSUPPORTED, "forcing is 2D Navier-Stokes only");
  CK(cudaSetDevice(ctx->device));
  for(int64_t i = 0; i < nin; ++i)
    if(in[i] < 0 || in[i] >= t.n) return fail(ctx, LBM_ERR_TABLE, "forcing: inlet cell id out of range");
  for(int64_t i = 0; i < nout; ++i)
    if(outc[i] < 0 || outc[i] >= t.n) return fail(ctx, LBM_ERR_TABLE, "forcing: outlet cell id out of range");
  const int     nn = t.nnghbr, D = t.D;
  const double* C  = ctx->centers.data();
  // outlet pass (solver.cpp:650-672) then inlet pass (:674-693); pairs in loop
  // order with the last writer of a target kept
  auto pairs = [&](const int64_t* from, int64_t nf, int vdir, const int64_t* to, int64_t nt, std::vector<int32_t>& tg,
                   std::vector<int32_t>& vl) -> bool {
    std::map<int64_t, int64_t> last;
    for(int64_t i = 0; i < nf; ++i) {
      const int64_t v = ctx->nghbr[from[i] * nn + vdir];
      if(v < 0) return false;
      for(int64_t j = 0; j < nt; ++j)
        if(std::fabs(C[v * D + 1] - C[to[j] * D + 1]) < EPSD) last[to[j]] = v;
    }
    for(auto& kv : last) {
      tg.push_back(static_cast<int32_t>(kv.first));
      vl.push_back(static_cast<int32_t>(kv.second));
    }
    return true;
  };
  std::vector<int32_t> to, vo, ti, vi;
  if(!pairs(in, nin, 1, outc, nout, to, vo) || !pairs(outc, nout, 0, in, nin, ti, vi))
    return fail(ctx, LBM_ERR_TABLE, "forcing: missing value cell");
  std::set<int32_t> written(to.begin(), to.end());
  for(int32_t v : vi)
    if(written.count(v)) return fail(ctx, LBM_ERR_UNSUPPORTED, "forcing: inlet value cell is an outlet cell");
  t.force_out     = upload(ctx, to);
  t.force_out_val = upload(ctx, vo);
  t.force_in      = upload(ctx, ti);
  t.force_in_val  = upload(ctx, vi);
  t.nforce_out    = static_cast<int64_t>(to.size());
  t.nforce_in     = static_cast<int64_t>(ti.size());
  t.forcing_dp    = dp;
  t.forcing       = true;
  t.need_feq      = true;
  free_graph(ctx);
  return LBM_OK;
}

int lbm_gpu_initial_condition(lbm_gpu_ctx* ctx) {
  if(!ctx) return LBM_ERR_INVALID;
  if(ctx->mode == 1) return box_initial_condition(ctx->box, ctx->stream) == cudaSuccess ? LBM_OK : fail(ctx, LBM_ERR_CUDA, "box init");
  if(ctx->mode == 2) return batch_initial_condition(ctx->batch, ctx->stream) == cudaSuccess ? LBM_OK : fail(ctx, LBM_ERR_CUDA, "batch init");
  CK(cudaSetDevice(ctx->device));
  TableState&         t = ctx->t;
  const int64_t       n = t.n;
  std::vector<double> vars(t.nvar * n, 0.0);
  // initCnd of every BC object in order (initBndryValues, solver.cpp:298-304)
  for(const HostBnd& b : ctx->hbnds) {
    switch(b.kind) {
      case LBM_BND_DIRICHLET_BB:
        for(int64_t c : b.cells)
          for(int d = 0; d < t.D; ++d) vars[d * n + c] = b.vec[d];
        break;
      case LBM_BND_PRESSURE_ABB:
        for(int64_t c : b.cells) vars[t.D * n + c] = b.scalar;
        break;
      case LBM_BND_DIRICHLET_NEEM:
        for(size_t i = 0; i < b.cells.size(); ++i) vars[b.cells[i]] = b.values[i];
        break;
      default:
        break;
    }
  }
  CK(cudaMemcpyAsync(t.vars, vars.data(), sizeof(double) * vars.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(t.varsold, 0, sizeof(double) * vars.size(), ctx->stream));
  CK(table_initial_condition(t, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LBM_OK;
}

int lbm_gpu_step(lbm_gpu_ctx* ctx, int64_t nsteps) {
  if(!ctx || nsteps < 0) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  if(nsteps == 0) return LBM_OK;
  if(ctx->mode == 1) return box_step(ctx->box, nsteps, ctx->stream, ctx->err);
  if(ctx->mode == 2) return batch_step(ctx->batch, nsteps, ctx->stream, ctx->err);
  // the step's kernel sequence is captured once as a graph of G steps
  const int G = 8;
  if(!ctx->graph) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for(int k = 0; k < G && e == cudaSuccess; ++k) e = table_step(ctx->t, ctx->stream);
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
    if(e != cudaSuccess) return cuda_fail(ctx, e, "capture");
    if(e2 != cudaSuccess) return cuda_fail(ctx, e2, "end capture");
    e = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    if(e != cudaSuccess) return cuda_fail(ctx, e, "graph instantiate");
    ctx->graph_steps = G;
  }
  int64_t left = nsteps;
  while(left >= G) {
    CK(cudaGraphLaunch(ctx->graph, ctx->stream));
    left -= G;
  }
  for(; left > 0; --left) CK(table_step(ctx->t, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LBM_OK;
}

int lbm_gpu_residual(lbm_gpu_ctx* ctx, double* r) {
  if(!ctx || !r) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  if(ctx->mode == 1) return box_residual(ctx->box, r, ctx->stream, ctx->err);
  if(ctx->mode == 2) return fail(ctx, LBM_ERR_INVALID, "batched contexts report residuals per cavity (lbm_gpu_batch_residuals)");
  TableState& t = ctx->t;
  CK(reduce_abs_diff(t.vars, t.varsold, t.n, t.nvar, ctx->d_partials, ctx->nblocks, ctx->d_out, ctx->stream));
  CK(cudaMemcpyAsync(r, ctx->d_out, sizeof(double) * t.nvar, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for(int v = 0; v < t.nvar; ++v)
    if(!std::isfinite(r[v])) return fail(ctx, LBM_ERR_DIVERGED, "Solution diverged");
  return LBM_OK;
}

int lbm_gpu_update_moments(lbm_gpu_ctx* ctx) {
  if(!ctx) return LBM_ERR_INVALID;
  if(ctx->mode != 0) return fail(ctx, LBM_ERR_INVALID, "reference-table entry point");
  CK(cudaSetDevice(ctx->device));
  CK(table_update_moments(ctx->t, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LBM_OK;
}

static int soa_io(lbm_gpu_ctx* ctx, double* dev, int comps, double* host_out, const double* host_in) {
  TableState&         t = ctx->t;
  const int64_t       n = t.n;
  std::vector<double> tmp(comps * n);
  if(host_out) {
    CK(cudaMemcpyAsync(tmp.data(), dev, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for(int64_t c = 0; c < n; ++c)
      for(int k = 0; k < comps; ++k) host_out[c * comps + k] = tmp[k * n + c];
  } else {
    for(int64_t c = 0; c < n; ++c)
      for(int k = 0; k < comps; ++k) tmp[k * n + c] = host_in[c * comps + k];
    CK(cudaMemcpyAsync(dev, tmp.data(), sizeof(double) * tmp.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return LBM_OK;
}

int lbm_gpu_get_vars(lbm_gpu_ctx* ctx, double* vars) {
  if(!ctx || !vars || ctx->mode != 0) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  return soa_io(ctx, ctx->t.vars, ctx->t.nvar, vars, nullptr);
}
int lbm_gpu_get_varsold(lbm_gpu_ctx* ctx, double* vars) {
  if(!ctx || !vars || ctx->mode != 0) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  return soa_io(ctx, ctx->t.varsold, ctx->t.nvar, vars, nullptr);
}
int lbm_gpu_set_vars(lbm_gpu_ctx* ctx, const double* vars) {
  if(!ctx || !vars || ctx->mode != 0) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  return soa_io(ctx, ctx->t.vars, ctx->t.nvar, nullptr, vars);
}
int lbm_gpu_get_populations(lbm_gpu_ctx* ctx, double* fold) {
  if(!ctx || !fold) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  if(ctx->mode == 1) return box_get_populations(ctx->box, fold, ctx->stream, ctx->err);
  if(ctx->mode == 2) return fail(ctx, LBM_ERR_INVALID, "batched contexts: lbm_gpu_batch_get_domain");
  return soa_io(ctx, ctx->t.fold, ctx->t.Q, fold, nullptr);
}
int lbm_gpu_set_populations(lbm_gpu_ctx* ctx, const double* fold) {
  if(!ctx || !fold) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  if(ctx->mode == 1) return box_set_populations(ctx->box, fold, ctx->stream, ctx->err);
  if(ctx->mode == 2) return fail(ctx, LBM_ERR_INVALID, "batched contexts cannot take a whole-state upload");
  return soa_io(ctx, ctx->t.fold, ctx->t.Q, nullptr, fold);
}

int lbm_gpu_reduce_mass_momentum(lbm_gpu_ctx* ctx, double* out) {
  if(!ctx || !out) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  if(ctx->mode == 1) return box_mass_momentum(ctx->box, out, ctx->stream, ctx->err);
  if(ctx->mode == 2) return fail(ctx, LBM_ERR_INVALID, "batched contexts: not available");
  TableState& t = ctx->t;
  CK(reduce_moments(t.fold, t.n, t.Q, t.lattice, ctx->d_partials, ctx->nblocks, ctx->d_out, ctx->stream));
  CK(cudaMemcpyAsync(out, ctx->d_out, sizeof(double) * (t.D + 1), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LBM_OK;
}

int lbm_gpu_synchronize(lbm_gpu_ctx* ctx) {
  if(!ctx) return LBM_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  return LBM_OK;
}

int lbm_gpu_info(const lbm_gpu_ctx* ctx, int64_t* ncells, int32_t* q, int32_t* nvar) {
  if(!ctx) return LBM_ERR_INVALID;
  if(ctx->mode == 1) return box_info(ctx->box, ncells, q, nvar);
  if(ctx->mode == 2) return batch_info(ctx->batch, ncells, q, nvar);
  if(ncells) *ncells = ctx->t.n;
  if(q) *q = ctx->t.Q;
  if(nvar) *nvar = ctx->t.nvar;
  return LBM_OK;
}

void lbm_gpu_destroy(lbm_gpu_ctx* ctx) {
  if(!ctx) return;
  cudaSetDevice(ctx->device);
  if(ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_graph(ctx);
  if(ctx->box) box_destroy(ctx->box);
  if(ctx->batch) batch_destroy(ctx->batch);
  for(void* p : ctx->allocs) cudaFree(p);
  if(ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

}  // extern "C"

// box-engine contexts are created through lbm_gpu_create_box (box_api in box.cu)
lbm_gpu_ctx* lbm_internal_new_box_ctx(int device, BoxState* box, cudaStream_t stream) {
  lbm_gpu_ctx* ctx = new(std::nothrow) lbm_gpu_ctx();
  if(!ctx) return nullptr;
  ctx->mode   = 1;
  ctx->device = device;
  ctx->box    = box;
  ctx->stream = stream;
  return ctx;
}
BoxState* lbm_internal_box(lbm_gpu_ctx* ctx) { return ctx && ctx->mode == 1 ? ctx->box : nullptr; }
lbm_gpu_ctx* lbm_internal_new_batch_ctx(int device, BatchState* batch, cudaStream_t stream) {
  lbm_gpu_ctx* ctx = new(std::nothrow) lbm_gpu_ctx();
  if(!ctx) return nullptr;
  ctx->mode   = 2;
  ctx->device = device;
  ctx->batch  = batch;
  ctx->stream = stream;
  return ctx;
}
BatchState* lbm_internal_batch(lbm_gpu_ctx* ctx) { return ctx && ctx->mode == 2 ? ctx->batch : nullptr; }
cudaStream_t lbm_internal_stream(lbm_gpu_ctx* ctx) { return ctx ? ctx->stream : nullptr; }
void lbm_internal_set_error(lbm_gpu_ctx* ctx, const std::string& msg) {
  if(ctx) ctx->err = msg;
}
