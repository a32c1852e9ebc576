// Host-side grid and table build (include/lbm_grid.h): the uniform Cartesian
// grid of the SFCMM/LBM reference's grid generator for an analytic geometry,
// and the neighbour / boundary / surface tables of its CartesianGrid.
//
// What the reference does, and how it is done here:
//  * Cells.  The reference refines a root cell level by level, deletes the
//    cells that are neither cut by the geometry nor inside it (flood fill from
//    the cut layer), then sorts the partition level by its curve index
//    (src/gridgenerator/cartesiangrid_generation.h:71-149, 419-451, 505-610,
//    664-735).  On a single uniform level that leaves exactly the cells cut by
//    an object or with their centre inside the geometry, so each candidate
//    position is tested directly and the kept cells are sorted by the same
//    curve index.  Cell centres are formed as the reference forms them: the
//    root centre plus, level by level, half the child length with the child's
//    sign (refineCell), so the doubles are the same.
//  * Main neighbours: adjacent positions that both hold a cell.
//  * Boundary cells: cut and missing a main neighbour
//    (src/cartesiangrid.h:509-544).
//  * Surfaces, periodic wiring and diagonals: src/cartesiangrid.h:551-598,
//    636-703 and 450-487.
// The floating-point comparisons of the cut tests (src/geometry.h:660-807)
// are kept operation for operation; this file is compiled without
// floating-point contraction so that the host compilers of both machines
// round the same way.
#include "../../include/lbm_grid.h"
#include "grid_geom.h"
#include "grid_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <new>
#include <system_error>
#include <thread>
#include <unordered_map>
#include <vector>

namespace lbm_grid_impl {

using namespace lbm_grid_geom;

bool geom_inside(const lbm_grid& g, const double* x) { return set_inside(g.geom(), x, g.D); }

bool geom_cut(const lbm_grid& g, const double* c, double len) { return set_cut(g.geom(), c, len, g.D); }

// hilbert::index (include/common/math/hilbert.h:16-48) of a position in the
// unit cube
uint64_t curve_index(const double* x, int D, int level) {
  static constexpr int lut[16] = {0, 3, 1, 2, 5, 4, 6, 7, 10, 9, 11, 8, 15, 14, 12, 13};
  double               p[4];
  for(int d = 0; d < D; ++d) p[d] = x[d];
  uint64_t index = 0;
  for(int l = 0; l < level; ++l) {
    int q = 0;
    for(int d = 0; d < D; ++d)
      if(p[d] >= 0.5) q |= 1 << d;
    index += static_cast<uint64_t>(lut[q]) << (D * (level - 1 - l));
    for(int d = 0; d < D; ++d) p[d] = 2 * p[d] - ((q >> d) & 1);
  }
  return index;
}

int dir_axis(int dir) { return dir / 2; }
int dir_sign(int dir) { return (dir & 1) ? 1 : -1; }

// Run fn(begin, end, part) on `parts` contiguous slices of [0, n), one host
// thread each.  Every slice writes only its own outputs, so the result does
// not depend on the number of threads.
// LBM_GRID_THREADS sets the number of slices (1-16) regardless of size.
// Run the tasks on threads of their own.  If the process cannot start a
// thread (std::system_error, e.g. at its thread limit), the tasks not yet
// started run on the calling thread instead: every caller's result is the
// same for any split, so no error crosses the C boundary.
void run_tasks(std::vector<std::function<void()>>& tasks) {
  std::vector<std::thread> pool;
  size_t                   started = 0;
  try {
    for(; started < tasks.size(); ++started) pool.emplace_back(tasks[started]);
  } catch(const std::system_error&) {
  }
  for(size_t t = started; t < tasks.size(); ++t) tasks[t]();
  for(auto& th : pool) th.join();
}

template <class F>
void parallel_for(int64_t n, F fn, int* parts_out = nullptr) {
  const int64_t min_per_thread = 1 << 16;
  int           parts          = static_cast<int>(std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()), 16));
  parts                        = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(parts, n / min_per_thread)));
  if(const char* env = std::getenv("LBM_GRID_THREADS")) {
    const long want = std::strtol(env, nullptr, 10);
    if(want >= 1) parts = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({static_cast<int64_t>(want), 16, n})));
  }
  if(parts_out) *parts_out = parts;
  if(parts == 1) {
    fn(int64_t(0), n, 0);
    return;
  }
  std::vector<std::function<void()>> tasks;
  for(int t = 0; t < parts; ++t) tasks.emplace_back([&fn, n, t, parts]() { fn(n * t / parts, n * (t + 1) / parts, t); });
  run_tasks(tasks);
}

// Main neighbours (the adjacent positions that hold a cell) and the boundary
// property (cut, and missing a main neighbour: determineBoundaryCells,
// src/cartesiangrid.h:509-544) of the cells as they now stand.
void link_cells(lbm_grid& g) {
  const int     D = g.D, M = 2 * D;
  const int64_t nx = g.ext[0], ny = g.ext[1], nz = g.ext[2];
  std::vector<int32_t> at(static_cast<size_t>(nx * ny * nz), -1);  // position -> cell
  auto rel = [&](int64_t c, int d) -> int64_t { return d < D ? g.ipos[c * D + d] - g.lo[d] : 0; };
  for(int64_t c = 0; c < g.n; ++c) at[static_cast<size_t>(rel(c, 0) + nx * (rel(c, 1) + ny * rel(c, 2)))] = static_cast<int32_t>(c);
  const int64_t ext[3] = {nx, ny, nz};
  g.nbr.assign(g.n * M, -1);
  g.bndry.assign(g.n, 0);
  parallel_for(g.n, [&](int64_t c0, int64_t c1, int) {
    for(int64_t c = c0; c < c1; ++c) {
      int present = 0;
      for(int dir = 0; dir < M; ++dir) {
        int64_t r[3] = {rel(c, 0), rel(c, 1), rel(c, 2)};
        r[dir_axis(dir)] += dir_sign(dir);
        if(r[dir_axis(dir)] < 0 || r[dir_axis(dir)] >= ext[dir_axis(dir)]) continue;
        const int32_t m = at[static_cast<size_t>(r[0] + nx * (r[1] + ny * r[2]))];
        if(m >= 0) {
          g.nbr[c * M + dir] = m;
          ++present;
        }
      }
      g.bndry[c] = present < M && geom_cut(g, &g.centers[c * D], g.cell_length);
    }
  });
  list_boundary_cells(g);
}

void list_boundary_cells(lbm_grid& g) {
  g.assigned.assign(g.n, 0);
  g.bcells.clear();
  for(int64_t c = 0; c < g.n; ++c)
    if(g.bndry[c]) g.bcells.push_back(c);
}

int setup(lbm_grid& g, int ndim, int level, const lbm_geom_desc* objs, int nobj, const double* bbox) {
  if(ndim < 1 || ndim > 3 || level < 1 || level > 20 || nobj < 0 || (nobj > 0 && !objs) || (nobj == 0 && !bbox))
    return LBM_ERR_INVALID;
  for(int i = 0; i < nobj; ++i)
    if(objs[i].kind != LBM_GEOM_BOX && objs[i].kind != LBM_GEOM_SPHERE) return LBM_ERR_UNSUPPORTED;
  const int D = ndim;
  g.D         = D;
  g.level     = level;
  g.objs.assign(objs, objs + nobj);
  // bodies numbered in order of first appearance
  std::vector<int32_t> ids;
  g.body.assign(nobj, 0);
  for(int i = 0; i < nobj; ++i) {
    const auto it = std::find(ids.begin(), ids.end(), objs[i].body);
    g.body[i]     = static_cast<int32_t>(it - ids.begin());
    if(it == ids.end()) ids.push_back(objs[i].body);
  }
  g.nbody = static_cast<int>(ids.size());
  // bounding box: given, or the union of the objects' boxes
  // (GeometryManager::getBoundingBox, src/geometry.h:1080-1103)
  for(int d = 0; d < D; ++d) {
    if(bbox) {
      g.bmin[d] = bbox[2 * d];
      g.bmax[d] = bbox[2 * d + 1];
      continue;
    }
    for(int i = 0; i < nobj; ++i) {
      const lbm_geom_desc& o  = objs[i];
      const double         lo = o.kind == LBM_GEOM_SPHERE ? o.center[d] - o.radius : o.a[d];
      const double         hi = o.kind == LBM_GEOM_SPHERE ? o.center[d] + o.radius : o.b[d];
      if(i == 0 || g.bmin[d] > lo) g.bmin[d] = lo;
      if(i == 0 || g.bmax[d] < hi) g.bmax[d] = hi;
    }
  }
  // extents, decisive direction, centre and level lengths
  // (BaseCartesianGrid::setBoundingBox, src/cartesiangrid_base.h:125-142)
  int    dec = 0;
  double ext[3];
  for(int d = 0; d < D; ++d) {
    ext[d]   = std::abs(g.bmax[d] - g.bmin[d]);
    dec      = ext[d] > ext[dec] ? d : dec;
    g.cog[d] = g.bmin[d] + 0.5 * (g.bmax[d] - g.bmin[d]);
  }
  g.len0 = (1.0 + 1.0 / std::ldexp(1.0, 100)) * ext[dec];
  std::vector<double> len(level + 1);
  len[0] = g.len0;
  for(int l = 1; l <= level; ++l) len[l] = 0.5 * len[l - 1];
  g.cell_length = len[level];
  g.cut_length  = g.cell_length;
  if(!(g.cell_length > 0.0)) return LBM_ERR_INVALID;
  // centre coordinate of position i along an axis: the root centre plus the
  // child offsets level by level (refineCell,
  // src/gridgenerator/cartesiangrid_generation.h:419-451)
  const int64_t side = int64_t(1) << level;
  for(int d = 0; d < D; ++d) {
    g.cv[d].resize(side);
    for(int64_t i = 0; i < side; ++i) {
      double c = g.cog[d];
      for(int l = 0; l < level; ++l) c = c + (0.5 * len[l + 1]) * (((i >> (level - 1 - l)) & 1) ? 1.0 : -1.0);
      g.cv[d][i] = c;
    }
    // candidate range: a cell further than one cell length from the bounding
    // box and from every object's box is neither cut nor inside
    double umin = g.bmin[d], umax = g.bmax[d];
    for(int i = 0; i < nobj; ++i) {
      const lbm_geom_desc& o = objs[i];
      umin = std::min(umin, o.kind == LBM_GEOM_SPHERE ? o.center[d] - o.radius : std::min(o.a[d], o.b[d]));
      umax = std::max(umax, o.kind == LBM_GEOM_SPHERE ? o.center[d] + o.radius : std::max(o.a[d], o.b[d]));
    }
    int64_t lo = side, hi = -1;
    for(int64_t i = 0; i < side; ++i)
      if(g.cv[d][i] >= umin - g.cell_length && g.cv[d][i] <= umax + g.cell_length) {
        lo = std::min(lo, i);
        hi = std::max(hi, i);
      }
    if(hi < lo) return LBM_ERR_INVALID;
    g.lo[d]  = lo;
    g.ext[d] = hi - lo + 1;
  }
  return LBM_OK;
}

}  // namespace lbm_grid_impl

using namespace lbm_grid_impl;

extern "C" {

int lbm_grid_create(int32_t ndim, int32_t level, const lbm_geom_desc* objs, int32_t nobj, const double* bbox, lbm_grid** out) {
  if(!out) return LBM_ERR_INVALID;
  *out = nullptr;
  lbm_grid* g = new(std::nothrow) lbm_grid();
  if(!g) return LBM_ERR_NOMEM;
  int rc = setup(*g, ndim, level, objs, nobj, bbox);
  if(rc != LBM_OK) {
    delete g;
    return rc;
  }
  const int D = ndim;
  // kept cells: cut by an object, or centre inside the geometry
  struct Kept {
    uint64_t key;
    int32_t  p[3];
  };
  const int64_t nx = g->ext[0], ny = g->ext[1], nz = g->ext[2];
  // every slice of the candidate positions collects and sorts its own kept
  // cells; the sorted slices are then merged (the keys are distinct, so the
  // order does not depend on the slicing)
  std::vector<std::vector<Kept>> part(16);
  int                            parts = 1;
  const auto                     by_key = [](const Kept& a, const Kept& b) { return a.key < b.key; };
  parallel_for(
      nx * ny * nz,
      [&](int64_t q0, int64_t q1, int t) {
        std::vector<Kept>& kept = part[t];
        for(int64_t q = q0; q < q1; ++q) {
          const int64_t i = q % nx, j = (q / nx) % ny, k = q / (nx * ny);
          const int64_t p[3] = {g->lo[0] + i, D > 1 ? g->lo[1] + j : 0, D > 2 ? g->lo[2] + k : 0};
          double        c[3];
          for(int d = 0; d < D; ++d) c[d] = g->cv[d][p[d]];
          if(!(geom_cut(*g, c, g->cell_length) || geom_inside(*g, c))) continue;
          // curve index of the centre in the unit cube of the root cell
          // (reorderHilbertCurve, cartesiangrid_generation.h:677-680)
          double x[3];
          for(int d = 0; d < D; ++d) x[d] = ((c[d] - g->cog[d]) + 0.5 * g->len0) / g->len0;
          kept.push_back({curve_index(x, D, level), {static_cast<int32_t>(p[0]), static_cast<int32_t>(p[1]), static_cast<int32_t>(p[2])}});
        }
        std::sort(kept.begin(), kept.end(), by_key);
      },
      &parts);
  // pairwise merges of neighbouring slices until one is left
  for(int width = 1; width < parts; width *= 2) {
    std::vector<std::function<void()>> merges;
    for(int a = 0; a + width < parts; a += 2 * width)
      merges.emplace_back([&, a, width]() {
        std::vector<Kept> merged(part[a].size() + part[a + width].size());
        std::merge(part[a].begin(), part[a].end(), part[a + width].begin(), part[a + width].end(), merged.begin(), by_key);
        part[a].swap(merged);
        std::vector<Kept>().swap(part[a + width]);
      });
    run_tasks(merges);
  }
  std::vector<Kept>& kept = part[0];
  if(kept.empty() || kept.size() >= (size_t(1) << 31)) {
    delete g;
    return LBM_ERR_INVALID;
  }
  for(size_t i = 1; i < kept.size(); ++i)
    if(kept[i].key == kept[i - 1].key) {  // the reference stops on duplicated curve ids
      delete g;
      return LBM_ERR_INVALID;
    }
  const int64_t n = static_cast<int64_t>(kept.size());
  g->n            = n;
  g->centers.resize(n * D);
  g->ipos.resize(n * D);
  for(int64_t c = 0; c < n; ++c)
    for(int d = 0; d < D; ++d) {
      g->ipos[c * D + d]    = kept[c].p[d];
      g->centers[c * D + d] = g->cv[d][kept[c].p[d]];
    }
  link_cells(*g);
  *out = g;
  return LBM_OK;
}

int lbm_grid_align(lbm_grid* g, int32_t align_dir) {
  if(!g || align_dir < 0 || align_dir >= g->D) return LBM_ERR_INVALID;
  const int D = g->D;
  // extent of the cell centres (initial maximum: the smallest positive double)
  double emin[3], emax[3];
  for(int d = 0; d < D; ++d) {
    emin[d] = std::numeric_limits<double>::max();
    emax[d] = std::numeric_limits<double>::min();
  }
  for(int64_t c = 0; c < g->n; ++c)
    for(int d = 0; d < D; ++d) {
      const double v = g->centers[c * D + d];
      if(emin[d] > v) emin[d] = v;
      if(emax[d] < v) emax[d] = v;
    }
  // a domain with the same extent along every axis is aligned along all of them
  bool same = true;
  for(int d = 0; d < D && same; ++d)
    for(int e = d + 1; e < D; ++e)
      if(!(std::abs(emin[d] - emin[e]) < kEps) || !(std::abs(emax[d] - emax[e]) < kEps)) {
        same = false;
        break;
      }
  const double t = g->bmax[align_dir] / (emax[align_dir] - emin[align_dir]);
  for(int64_t c = 0; c < g->n; ++c)
    for(int d = 0; d < D; ++d) {
      double& v = g->centers[c * D + d];
      v         = (d == align_dir || same) ? v * t - (t * emax[d] - g->bmax[d]) : v * t;
    }
  // the generator's cell length of the level is scaled by t; the solver's grid
  // takes it over as the ratio of the two lengths (transformMaxLvl,
  // src/cartesiangrid.h:274)
  const double len_l = g->cell_length;
  g->cut_length      = len_l * t;
  g->cell_length     = len_l * (g->cut_length / len_l);
  // delete the cells that are now neither cut nor inside, from the last one
  // down; the last cell fills each hole (deleteOutsideCells<true>,
  // cartesiangrid_generation.h:505-552)
  std::vector<uint8_t> keep(g->n);
  for(int64_t c = 0; c < g->n; ++c) {
    const double* x = &g->centers[c * D];
    keep[c]         = geom_cut(*g, x, g->cut_length) || geom_inside(*g, x);
  }
  int64_t end = g->n;
  for(int64_t c = g->n - 1; c >= 0; --c) {
    if(keep[c]) continue;
    if(c != end - 1)
      for(int d = 0; d < D; ++d) {
        g->centers[c * D + d] = g->centers[(end - 1) * D + d];
        g->ipos[c * D + d]    = g->ipos[(end - 1) * D + d];
      }
    --end;
  }
  if(end == 0) return LBM_ERR_INVALID;
  g->n = end;
  g->centers.resize(end * D);
  g->ipos.resize(end * D);
  link_cells(*g);
  return LBM_OK;
}

int lbm_grid_curve_index(int32_t ndim, int32_t level, const double* x, uint64_t* out) {
  if(ndim < 1 || ndim > 4 || level < 0 || static_cast<int64_t>(ndim) * level > 64 || !x || !out) return LBM_ERR_INVALID;
  *out = curve_index(x, ndim, level);
  return LBM_OK;
}

int64_t lbm_grid_ncells(const lbm_grid* g) { return g ? g->n : 0; }

int32_t lbm_grid_nnghbr(const lbm_grid* g) {
  if(!g) return 0;
  return g->D == 1 ? 2 : (g->D == 2 ? 8 : 18);
}

int lbm_grid_info(const lbm_grid* g, double* bbox, double* cell_length) {
  if(!g) return LBM_ERR_INVALID;
  if(bbox)
    for(int d = 0; d < g->D; ++d) {
      bbox[2 * d]     = g->bmin[d];
      bbox[2 * d + 1] = g->bmax[d];
    }
  if(cell_length) *cell_length = g->cell_length;
  return LBM_OK;
}

int lbm_grid_centers(const lbm_grid* g, double* out) {
  if(!g || !out) return LBM_ERR_INVALID;
  std::copy(g->centers.begin(), g->centers.end(), out);
  return LBM_OK;
}

int lbm_grid_boundary(const lbm_grid* g, uint8_t* out) {
  if(!g || !out) return LBM_ERR_INVALID;
  std::copy(g->bndry.begin(), g->bndry.end(), out);
  return LBM_OK;
}

int lbm_grid_add_surface(lbm_grid* g, int32_t obj, int32_t dir_begin, int32_t dir_end, int64_t* cells, int8_t* dirs, int64_t cap,
                         int64_t* n) {
  if(!g || !n || obj < 0 || obj >= static_cast<int>(g->objs.size())) return LBM_ERR_INVALID;
  const int D = g->D, M = 2 * D;
  if(dir_begin < 0 || dir_end > M || dir_begin >= dir_end) return LBM_ERR_INVALID;
  // the pairs of this surface: a boundary cell without a main neighbour in
  // the direction, cut by the object, and not taken by an earlier surface
  // (within one call a pair cannot repeat, so counting needs no marks)
  // the cut test with the length of the cell's level
  auto member = [&](int64_t c, int dir) {
    const double len = g->cell_len.empty() ? g->cell_length : g->cell_len[c];
    return g->nbr[c * M + dir] == -1 && !(g->assigned[c] & (1u << dir)) && obj_cut(g->objs[obj], &g->centers[c * D], len, D);
  };
  int64_t count = 0;
  for(int dir = dir_begin; dir < dir_end; ++dir)
    for(const int64_t c : g->bcells) count += member(c, dir) ? 1 : 0;
  *n = count;
  if(!cells || !dirs) return cap == 0 ? LBM_OK : LBM_ERR_INVALID;  // count only: nothing taken
  if(count > cap) return LBM_ERR_INVALID;                          // nothing taken either
  int64_t k = 0;
  for(int dir = dir_begin; dir < dir_end; ++dir)
    for(const int64_t c : g->bcells) {  // the boundary cells in cell order
      if(!member(c, dir)) continue;
      g->assigned[c] = static_cast<uint8_t>(g->assigned[c] | (1u << dir));
      cells[k]       = c;
      dirs[k]        = static_cast<int8_t>(dir);
      ++k;
    }
  return LBM_OK;
}

int lbm_grid_connect_periodic(lbm_grid* g, const int64_t* cells_a, int64_t na, const int64_t* cells_b, int64_t nb) {
  if(!g || na < 0 || nb < 0 || (na && !cells_a) || (nb && !cells_b)) return LBM_ERR_INVALID;
  const int D = g->D, M = 2 * D;
  for(int64_t i = 0; i < na; ++i)
    if(cells_a[i] < 0 || cells_a[i] >= g->n) return LBM_ERR_INVALID;
  for(int64_t i = 0; i < nb; ++i)
    if(cells_b[i] < 0 || cells_b[i] >= g->n) return LBM_ERR_INVALID;
  // The reference tests every pair (a, b) in list order (a outer, b inner)
  // and connects those whose centres differ along exactly one axis.  Such a
  // pair shares the other coordinates bit for bit, so the pairs are looked up
  // by those coordinates (one table per axis) and then tested and applied in
  // the reference's order.
  struct Key {
    uint64_t k[2];
    bool     operator==(const Key& o) const { return k[0] == o.k[0] && k[1] == o.k[1]; }
  };
  struct KeyHash {
    size_t operator()(const Key& x) const { return std::hash<uint64_t>()(x.k[0] * 0x9e3779b97f4a7c15ull ^ x.k[1]); }
  };
  auto bits = [](double v) {
    uint64_t u;
    std::memcpy(&u, &v, sizeof u);
    return u;
  };
  auto key = [&](int64_t cell, int axis) {
    Key k{{0, 0}};
    int m = 0;
    for(int d = 0; d < D; ++d)
      if(d != axis) k.k[m++] = bits(g->centers[cell * D + d] + 0.0);  // +0.0: one key for -0 and +0
    return k;
  };
  std::vector<std::unordered_map<Key, std::vector<int64_t>, KeyHash>> by_axis(D);
  for(int64_t j = 0; j < nb; ++j)
    for(int d = 0; d < D; ++d) by_axis[d][key(cells_b[j], d)].push_back(j);
  std::vector<int64_t> cand;
  for(int64_t i = 0; i < na; ++i) {
    const int64_t a = cells_a[i];
    cand.clear();
    for(int d = 0; d < D; ++d) {
      const auto it = by_axis[d].find(key(a, d));
      if(it != by_axis[d].end()) cand.insert(cand.end(), it->second.begin(), it->second.end());
    }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    for(const int64_t j : cand) {
      const int64_t b  = cells_b[j];
      const double* ca = &g->centers[a * D];
      const double* cb = &g->centers[b * D];
      int           nm = -1;
      for(int d = 0; d < D; ++d) {
        if(std::abs(ca[d] - cb[d]) > kEps) {
          if(nm >= 0) {
            nm = -1;
            break;
          }
          nm = d;
        }
      }
      if(nm < 0) continue;
      const int dir = 2 * nm;
      if(ca[nm] > cb[nm]) {
        g->nbr[b * M + dir]     = a;
        g->nbr[a * M + dir + 1] = b;
      } else {
        g->nbr[a * M + dir]     = b;
        g->nbr[b * M + dir + 1] = a;
      }
    }
  }
  return LBM_OK;
}

int lbm_grid_neighbors(const lbm_grid* g, int64_t* out) {
  if(!g || !out) return LBM_ERR_INVALID;
  const int D = g->D, M = 2 * D, W = lbm_grid_nnghbr(g);
  auto      step = [&](int64_t c, int axis, int sign) -> int64_t {
    return c < 0 ? -1 : g->nbr[c * M + 2 * axis + (sign > 0 ? 1 : 0)];
  };
  // edge neighbours in the lattice's direction order: 2D as
  // CartesianGrid::addDiagonalNghbrs (+x+y, +x-y, -x-y, -x+y; x step first);
  // 3D the D3Q19 order of directions 6-17, first step along the first axis
  static constexpr int e2[4][2]  = {{1, 1}, {1, -1}, {-1, -1}, {-1, 1}};
  static constexpr int e3[12][3] = {{-1, -1, 0}, {-1, 1, 0}, {1, -1, 0}, {1, 1, 0},  {-1, 0, -1}, {-1, 0, 1},
                                    {1, 0, -1},  {1, 0, 1},  {0, -1, -1}, {0, -1, 1}, {0, 1, -1},  {0, 1, 1}};
  parallel_for(g->n, [&](int64_t c0, int64_t c1, int) {
  for(int64_t c = c0; c < c1; ++c) {
    int64_t* o = out + c * W;
    for(int dir = 0; dir < M; ++dir) o[dir] = g->nbr[c * M + dir];
    if(D == 2)
      for(int e = 0; e < 4; ++e) o[M + e] = step(step(c, 0, e2[e][0]), 1, e2[e][1]);
    if(D == 3)
      for(int e = 0; e < 12; ++e) {
        int ax[2], sg[2], m = 0;
        for(int a = 0; a < 3; ++a)
          if(e3[e][a] != 0) {
            ax[m]   = a;
            sg[m++] = e3[e][a];
          }
        o[M + e] = step(step(c, ax[0], sg[0]), ax[1], sg[1]);
      }
  }
  });
  return LBM_OK;
}

void lbm_grid_destroy(lbm_grid* g) { delete g; }

}  // extern "C"
