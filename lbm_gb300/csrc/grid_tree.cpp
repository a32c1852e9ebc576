// Multi-level grid generation (include/lbm_grid.h, lbm_grid_tree_*): the cell
// tree of the SFCMM/LBM reference's grid generator for an analytic geometry,
// for any partitionLevel <= uniformLevel <= maxRfnmtLvl.
//
// The reference (src/gridgenerator/gridGenerator.cpp:163-238,
// src/gridgenerator/cartesiangrid_generation.h) keeps every cell in one array
// of "maxNoCells" slots and builds it in three phases:
//  1. the partitioning level: the root cell refined level by level, the
//     levels placed alternately at the front and the back of the array so
//     that the partitioning level ends at slot 0, the cells outside the
//     geometry deleted after each refinement, and the partitioning level
//     sorted by its curve index (createPartitioningGrid, :71-147;
//     reorderHilbertCurve, :664-735);
//  2. uniform refinement up to uniformLevel: every cell of a level gets its
//     2^D children, appended after the grid (uniformRefineGrid, :151-169);
//  3. boundary refinement up to maxRfnmtLvl: the boundary cells of the
//     finest level get children, appended likewise (markBndryCells and
//     refineMarkedCells, :173-206).
// Each refinement links the children to their same-level neighbours through
// the parents' neighbours (findChildLevelNghbrs, :453-507), marks outside
// cells by a flood fill from the first unmarked cell of each region
// (markOutsideCells and floodCells, :555-603), and deletes them from the
// last one down, the level's last cell filling each hole (deleteCell and
// copyCell, :509-552, 616-646).  The optional alignNodesWithSurface step
// (transformMaxRfnmtLvlToExtent, :255-304) stretches the finest level.
//
// Here each level is held in arrays of its own, indexed locally; the
// reference's slot of a cell is the level's first slot plus the local index,
// which is how the global ids and the memory checks against maxNoCells are
// reproduced without allocating maxNoCells slots.  Every order-dependent step
// (flood fill, deletion, curve sort) is carried out in the reference's order,
// so the tree (centres, levels, parents, children, neighbours, boundary
// property and global ids) is the reference's cell for cell.
#include "../../include/lbm_grid.h"
#include "grid_geom.h"
#include "grid_internal.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <new>
#include <vector>

struct lbm_grid_tree {
  int                  D = 0, nc = 0, nn = 0;
  int                  partition_level = 0, highest_level = 0, max_level = 0;
  lbm_grid             geom;          // geometry, bounding box and root length (no cells)
  std::vector<double>  len;           // the generator's cell length per level (maxRfnmtLvl's stretched by alignment)
  double               max_len_solver = 0;  // maxRfnmtLvl's length as the solver's grid takes it over
  int64_t              n = 0;
  std::vector<double>  centers;   // n x D
  std::vector<int8_t>  level;     // n
  std::vector<int64_t> parent;    // n (-1: none)
  std::vector<int64_t> global;    // n
  std::vector<int64_t> children;  // n x nc (-1: none)
  std::vector<int64_t> nghbr;     // n x nn (-1: none)
  std::vector<int32_t> nchild;    // n
  std::vector<uint8_t> bndry;     // n
};

namespace {

using namespace lbm_grid_geom;

// one level of the tree, indexed locally
struct Level {
  int                  lvl    = 0;
  int64_t              vbegin = 0;  // the reference's slot of local cell 0 at creation
  int64_t              n      = 0;
  std::vector<double>  c;
  std::vector<int64_t> parent, gid, child, nb;
  std::vector<int32_t> nchild;
  std::vector<uint8_t> bndry, inside, marked;

  void resize(int64_t m, int D, int nc, int nn) {
    n = m;
    c.assign(m * D, 0.0);
    parent.assign(m, -1);
    gid.assign(m, -1);
    child.assign(m * nc, -1);
    nb.assign(m * nn, -1);
    nchild.assign(m, 0);
    bndry.assign(m, 0);
    inside.assign(m, 0);
    marked.assign(m, 0);
  }
};

struct Gen {
  int                 D, nc, nn;
  int                 partition_level;
  int64_t             capacity;
  GeomSet             geom;
  std::vector<double> len;  // cell length per level
  const double*       cog;
  double              len0;

  bool cut(const double* c, double l) const { return set_cut(geom, c, l, D); }
  bool inside(const double* x) const { return set_inside(geom, x, D); }

  // refineCell (cartesiangrid_generation.h:419-451) for the listed parents
  // of `up`, in order: the children of the k-th parent are the local cells
  // k*nc .. k*nc+nc-1 of `lo`, at slots lo.vbegin + local index
  void refine(Level& up, Level& lo, const std::vector<int64_t>& parents) const {
    lo.lvl = up.lvl + 1;
    lo.resize(static_cast<int64_t>(parents.size()) * nc, D, nc, nn);
    const double l  = len[lo.lvl];
    const double hl = 0.5 * l;
    for(size_t k = 0; k < parents.size(); ++k) {
      const int64_t p = parents[k];
      for(int ch = 0; ch < nc; ++ch) {
        const int64_t q = static_cast<int64_t>(k) * nc + ch;
        for(int d = 0; d < D; ++d) lo.c[q * D + d] = up.c[p * D + d] + hl * (((ch >> d) & 1) ? 1.0 : -1.0);
        lo.parent[q] = p;
        lo.gid[q]    = lo.vbegin + q;
        lo.bndry[q]  = up.bndry[p] ? (cut(&lo.c[q * D], l) ? 1 : 0) : 0;
        up.child[p * nc + ch] = q;
        ++up.nchild[p];
      }
    }
  }

  // findChildLevelNghbrs (cartesiangrid_generation.h:453-507): a child's
  // neighbour across a face inside its parent is the sibling there;
  // otherwise it is the matching child of the parent's neighbour, if any
  void link(const Level& up, Level& lo) const {
    for(int64_t p = 0; p < up.n; ++p)
      for(int ch = 0; ch < nc; ++ch) {
        const int64_t q = up.child[p * nc + ch];
        if(q < 0) continue;
        for(int dir = 0; dir < nn; ++dir) {
          const int axis = dir >> 1, plus = dir & 1;
          const int mate = ch ^ (1 << axis);  // the child on the other side of the face
          if(((ch >> axis) & 1) != plus) {
            lo.nb[q * nn + dir] = up.child[p * nc + mate];
          } else {
            const int64_t pn = up.nb[p * nn + dir];
            if(pn >= 0 && up.child[pn * nc + mate] >= 0) lo.nb[q * nn + dir] = up.child[pn * nc + mate];
          }
        }
      }
  }

  // markOutsideCells without CHECKALL (cartesiangrid_generation.h:555-603):
  // each unmarked cell in order decides its region (boundary cells are
  // always inside); the flood carries its decision to every non-boundary
  // cell it reaches through neighbour links, depth first from a stack
  void mark_flood(Level& lv) const {
    std::fill(lv.marked.begin(), lv.marked.end(), 0);
    std::vector<int64_t> stack;
    for(int64_t q = 0; q < lv.n; ++q) {
      if(lv.marked[q]) continue;
      lv.marked[q]  = 1;
      const bool bq = lv.bndry[q] != 0;
      lv.inside[q]  = (bq || inside(&lv.c[q * D])) ? 1 : 0;
      if(bq) continue;
      const uint8_t in = lv.inside[q];
      stack.assign(1, q);
      while(!stack.empty()) {
        const int64_t cur = stack.back();
        stack.pop_back();
        for(int dir = 0; dir < nn; ++dir) {
          const int64_t m = lv.nb[cur * nn + dir];
          if(m < 0 || lv.marked[m]) continue;
          lv.marked[m] = 1;
          if(!lv.bndry[m]) {
            lv.inside[m] = in;
            stack.push_back(m);
          } else {
            lv.inside[m] = 1;
          }
        }
      }
    }
  }

  // markOutsideCells with CHECKALL: every cell tested directly, the boundary
  // property recomputed with the level's (possibly stretched) length
  void mark_direct(Level& lv, double l) const {
    for(int64_t q = 0; q < lv.n; ++q) {
      const bool b = cut(&lv.c[q * D], l);
      lv.bndry[q]  = b ? 1 : 0;
      lv.inside[q] = (b || inside(&lv.c[q * D])) ? 1 : 0;
    }
  }

  // copyCell (cartesiangrid_generation.h:616-646) within a level
  void move(Level& lv, Level* up, Level* down, int64_t from, int64_t to) const {
    for(int d = 0; d < D; ++d) lv.c[to * D + d] = lv.c[from * D + d];
    lv.parent[to] = lv.parent[from];
    lv.gid[to]    = lv.gid[from];
    lv.nchild[to] = lv.nchild[from];
    lv.bndry[to]  = lv.bndry[from];
    lv.inside[to] = lv.inside[from];
    lv.marked[to] = lv.marked[from];
    for(int k = 0; k < nc; ++k) lv.child[to * nc + k] = lv.child[from * nc + k];
    for(int dir = 0; dir < nn; ++dir) {
      const int64_t m       = lv.nb[from * nn + dir];
      lv.nb[to * nn + dir] = m;
      if(m >= 0) lv.nb[m * nn + (dir ^ 1)] = to;
      lv.nb[from * nn + dir] = -1;
    }
    if(up && lv.parent[to] >= 0)
      for(int k = 0; k < nc; ++k)
        if(up->child[lv.parent[to] * nc + k] == from) {
          up->child[lv.parent[to] * nc + k] = to;
          break;
        }
    if(down)
      for(int k = 0; k < nc; ++k)
        if(lv.child[to * nc + k] >= 0) down->parent[lv.child[to * nc + k]] = to;
  }

  // deleteOutsideCells / deleteCell (cartesiangrid_generation.h:509-552):
  // from the last cell down, a cell not inside is unlinked from its parent
  // (not on the partitioning level) and from its neighbours, and the level's
  // last cell takes its place
  void delete_outside(Level& lv, Level* up, Level* down) const {
    int64_t end = lv.n;
    for(int64_t q = lv.n - 1; q >= 0; --q) {
      if(lv.inside[q]) continue;
      if(lv.lvl != partition_level && up) {
        const int64_t p = lv.parent[q];
        for(int k = 0; k < nc; ++k)
          if(up->child[p * nc + k] == q) {
            up->child[p * nc + k] = -1;
            break;
          }
        --up->nchild[p];
      }
      for(int dir = 0; dir < nn; ++dir) {
        const int64_t m = lv.nb[q * nn + dir];
        if(m >= 0) lv.nb[m * nn + (dir ^ 1)] = -1;
      }
      if(q != end - 1) move(lv, lv.lvl != partition_level ? up : nullptr, down, end - 1, q);
      --end;
    }
    lv.n = end;
    lv.c.resize(end * D);
    lv.parent.resize(end);
    lv.gid.resize(end);
    lv.child.resize(end * nc);
    lv.nb.resize(end * nn);
    lv.nchild.resize(end);
    lv.bndry.resize(end);
    lv.inside.resize(end);
    lv.marked.resize(end);
  }

  // reorderHilbertCurve (cartesiangrid_generation.h:664-735): the level
  // sorted by the curve index of its centres at the partitioning level; the
  // records move with their links.  Returns false on a repeated index.
  bool curve_sort(Level& lv) const {
    std::vector<uint64_t> key(lv.n);
    for(int64_t q = 0; q < lv.n; ++q) {
      double x[3];
      for(int d = 0; d < D; ++d) x[d] = ((lv.c[q * D + d] - cog[d]) + 0.5 * len0) / len0;
      key[q] = lbm_grid_impl::curve_index(x, D, partition_level);
    }
    std::vector<int64_t> order(lv.n);
    for(int64_t q = 0; q < lv.n; ++q) order[q] = q;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
    for(int64_t i = 1; i < lv.n; ++i)
      if(key[order[i]] == key[order[i - 1]]) return false;
    std::vector<int64_t> at(lv.n);
    for(int64_t i = 0; i < lv.n; ++i) at[order[i]] = i;
    Level s;
    s.lvl    = lv.lvl;
    s.vbegin = lv.vbegin;
    s.resize(lv.n, D, nc, nn);
    for(int64_t i = 0; i < lv.n; ++i) {
      const int64_t q = order[i];
      for(int d = 0; d < D; ++d) s.c[i * D + d] = lv.c[q * D + d];
      s.gid[i]    = lv.gid[q];
      s.nchild[i] = lv.nchild[q];
      s.bndry[i]  = lv.bndry[q];
      s.inside[i] = lv.inside[q];
      s.marked[i] = lv.marked[q];
      for(int dir = 0; dir < nn; ++dir) {
        const int64_t m    = lv.nb[q * nn + dir];
        s.nb[i * nn + dir] = m >= 0 ? at[m] : -1;
      }
      for(int k = 0; k < nc; ++k) s.child[i * nc + k] = lv.child[q * nc + k];
    }
    lv = std::move(s);
    return true;
  }
};

}  // namespace

using namespace lbm_grid_impl;

extern "C" {

static int tree_create(int32_t ndim, int32_t partition_level, int32_t uniform_level, int32_t max_level, int64_t max_cells,
                       const lbm_geom_desc* objs, int32_t nobj, const double* bbox, int32_t align_dir, lbm_grid_tree** out) {
  if(partition_level < 0 || partition_level > uniform_level || uniform_level > max_level || max_level > 20 || max_cells < 1)
    return LBM_ERR_INVALID;
  if(align_dir >= ndim) return LBM_ERR_INVALID;
  lbm_grid base;
  int      rc = setup(base, ndim, std::max(1, max_level), objs, nobj, bbox);
  if(rc != LBM_OK) return rc;
  Gen g;
  g.D               = ndim;
  g.nc              = 1 << ndim;
  g.nn              = 2 * ndim;
  g.partition_level = partition_level;
  g.capacity        = max_cells;
  g.geom            = base.geom();
  g.cog             = base.cog;
  g.len0            = base.len0;
  g.len.assign(max_level + 1, 0.0);
  g.len[0] = base.len0;
  for(int l = 1; l <= max_level; ++l) g.len[l] = 0.5 * g.len[l - 1];
  const int D = g.D, nc = g.nc, nn = g.nn;

  // 1. the partitioning level (createPartitioningGrid): the root at slot 0
  // when the partitioning level is even, at the last slot when it is odd
  Level cur;
  cur.lvl    = 0;
  cur.vbegin = (partition_level % 2 == 0) ? 0 : max_cells - 1;
  cur.resize(1, D, nc, nn);
  for(int d = 0; d < D; ++d) cur.c[d] = g.cog[d];
  cur.gid[0]   = cur.vbegin;
  cur.bndry[0] = 1;
  for(int l = 0; l < partition_level; ++l) {
    Level next;
    if(cur.vbegin == 0) {
      next.vbegin = max_cells - cur.n * nc;
      if(cur.vbegin + cur.n > next.vbegin) return LBM_ERR_NOMEM;
    } else {
      next.vbegin = 0;
      if(cur.vbegin < cur.n * nc) return LBM_ERR_NOMEM;
    }
    std::vector<int64_t> all(cur.n);
    for(int64_t q = 0; q < cur.n; ++q) all[q] = q;
    g.refine(cur, next, all);
    g.link(cur, next);
    g.mark_flood(next);
    g.delete_outside(next, &cur, nullptr);
    cur = std::move(next);
  }
  if(cur.n == 0 || !g.curve_sort(cur)) return LBM_ERR_INVALID;
  std::fill(cur.parent.begin(), cur.parent.end(), -1);

  // 2./3. uniform and boundary refinement, each level appended after the grid
  std::vector<Level> levels;
  levels.push_back(std::move(cur));
  int64_t size = levels.back().n;
  for(int l = partition_level; l < max_level; ++l) {
    Level&               up = levels.back();
    std::vector<int64_t> parents;
    for(int64_t q = 0; q < up.n; ++q)
      if(l < uniform_level || up.bndry[q]) parents.push_back(q);
    // no boundary cell left to refine: refineMarkedCells adds no level, and
    // every later pass finds the same finest level
    if(l >= uniform_level && parents.empty()) break;
    Level next;
    next.vbegin = size;
    if(size + static_cast<int64_t>(parents.size()) * nc > max_cells) return LBM_ERR_NOMEM;
    g.refine(up, next, parents);
    g.link(up, next);
    g.mark_flood(next);
    g.delete_outside(next, &up, nullptr);
    size += next.n;
    levels.push_back(std::move(next));
  }
  const int highest = partition_level + static_cast<int>(levels.size()) - 1;

  // optional alignNodesWithSurface on maxRfnmtLvl's cells
  if(align_dir >= 0) {
    if(highest != max_level) return LBM_ERR_INVALID;  // no cells on maxRfnmtLvl to align
    Level& lv = levels.back();
    double emin[3], emax[3];
    for(int d = 0; d < D; ++d) {
      emin[d] = std::numeric_limits<double>::max();
      emax[d] = std::numeric_limits<double>::min();
    }
    for(int64_t q = 0; q < lv.n; ++q)
      for(int d = 0; d < D; ++d) {
        const double v = lv.c[q * D + d];
        if(emin[d] > v) emin[d] = v;
        if(emax[d] < v) emax[d] = v;
      }
    bool same = true;
    for(int d = 0; d < D && same; ++d)
      for(int e = d + 1; e < D; ++e)
        if(!(std::abs(emin[d] - emin[e]) < kEps) || !(std::abs(emax[d] - emax[e]) < kEps)) {
          same = false;
          break;
        }
    const double t = base.bmax[align_dir] / (emax[align_dir] - emin[align_dir]);
    for(int64_t q = 0; q < lv.n; ++q)
      for(int d = 0; d < D; ++d) {
        double& v = lv.c[q * D + d];
        v         = (d == align_dir || same) ? v * t - (t * emax[d] - base.bmax[d]) : v * t;
      }
    g.len[max_level] *= t;
    g.mark_direct(lv, g.len[max_level]);
    Level* up = levels.size() > 1 ? &levels[levels.size() - 2] : nullptr;
    g.delete_outside(lv, up, nullptr);
    // the generator's size is then the finest level's cell count
    // (deleteOutsideCells sets it, and no refinement resets it)
    size = lv.n;
  }

  lbm_grid_tree* t = new(std::nothrow) lbm_grid_tree();
  if(!t) return LBM_ERR_NOMEM;
  t->D               = D;
  t->nc              = nc;
  t->nn              = nn;
  t->partition_level = partition_level;
  t->highest_level   = highest;
  t->max_level       = max_level;
  t->len             = g.len;
  // the solver's grid takes maxRfnmtLvl's length over as the ratio of the
  // generator's stretched length to its own (transformMaxLvl,
  // src/cartesiangrid.h:274)
  {
    double solver_len = base.len0;
    for(int l = 1; l <= max_level; ++l) solver_len = 0.5 * solver_len;
    t->max_len_solver = solver_len * (g.len[max_level] / solver_len);
  }
  base.cv[0].clear();
  base.cv[1].clear();
  base.cv[2].clear();
  t->geom = std::move(base);
  // flatten: the levels lie one after the other from slot 0
  std::vector<int64_t> off(levels.size() + 1, 0);
  for(size_t i = 0; i < levels.size(); ++i) off[i + 1] = off[i] + levels[i].n;
  const int64_t total = off.back();
  const int64_t n     = std::min(size, total);
  try {
    t->centers.resize(n * D);
    t->level.resize(n);
    t->parent.resize(n);
    t->global.resize(n);
    t->children.resize(n * nc);
    t->nghbr.resize(n * nn);
    t->nchild.resize(n);
    t->bndry.resize(n);
  } catch(const std::bad_alloc&) {
    delete t;
    return LBM_ERR_NOMEM;
  }
  t->n = n;
  for(size_t i = 0; i < levels.size(); ++i) {
    const Level& lv = levels[i];
    for(int64_t q = 0; q < lv.n; ++q) {
      const int64_t c = off[i] + q;
      if(c >= n) break;
      for(int d = 0; d < D; ++d) t->centers[c * D + d] = lv.c[q * D + d];
      t->level[c]  = static_cast<int8_t>(lv.lvl);
      t->parent[c] = (i > 0 && lv.parent[q] >= 0) ? off[i - 1] + lv.parent[q] : -1;
      t->global[c] = lv.gid[q];
      t->nchild[c] = lv.nchild[q];
      t->bndry[c]  = lv.bndry[q];
      for(int k = 0; k < nc; ++k) {
        const int64_t m        = lv.child[q * nc + k];
        t->children[c * nc + k] = (m >= 0 && i + 1 < levels.size()) ? off[i + 1] + m : -1;
      }
      for(int dir = 0; dir < nn; ++dir) {
        const int64_t m       = lv.nb[q * nn + dir];
        t->nghbr[c * nn + dir] = m >= 0 ? off[i] + m : -1;
      }
    }
  }
  *out = t;
  return LBM_OK;
}

int lbm_grid_tree_create(int32_t ndim, int32_t partition_level, int32_t uniform_level, int32_t max_level, int64_t max_cells,
                         const lbm_geom_desc* objs, int32_t nobj, const double* bbox, int32_t align_dir, lbm_grid_tree** out) {
  if(!out) return LBM_ERR_INVALID;
  *out = nullptr;
  try {
    return tree_create(ndim, partition_level, uniform_level, max_level, max_cells, objs, nobj, bbox, align_dir, out);
  } catch(const std::bad_alloc&) {  // no exception crosses the C boundary
    return LBM_ERR_NOMEM;
  }
}

int64_t lbm_grid_tree_ncells(const lbm_grid_tree* t) { return t ? t->n : 0; }

int lbm_grid_tree_levels(const lbm_grid_tree* t, int32_t* partition_level, int32_t* highest_level) {
  if(!t) return LBM_ERR_INVALID;
  if(partition_level) *partition_level = t->partition_level;
  if(highest_level) *highest_level = t->highest_level;
  return LBM_OK;
}

int lbm_grid_tree_cells(const lbm_grid_tree* t, double* centers, int8_t* level, int64_t* parent, int64_t* global_id, int32_t* nchildren,
                        uint8_t* bndry) {
  if(!t) return LBM_ERR_INVALID;
  if(centers) std::copy(t->centers.begin(), t->centers.end(), centers);
  if(level) std::copy(t->level.begin(), t->level.end(), level);
  if(parent) std::copy(t->parent.begin(), t->parent.end(), parent);
  if(global_id) std::copy(t->global.begin(), t->global.end(), global_id);
  if(nchildren) std::copy(t->nchild.begin(), t->nchild.end(), nchildren);
  if(bndry) std::copy(t->bndry.begin(), t->bndry.end(), bndry);
  return LBM_OK;
}

int lbm_grid_tree_children(const lbm_grid_tree* t, int64_t* out) {
  if(!t || !out) return LBM_ERR_INVALID;
  std::copy(t->children.begin(), t->children.end(), out);
  return LBM_OK;
}

int lbm_grid_tree_neighbors(const lbm_grid_tree* t, int64_t* out) {
  if(!t || !out) return LBM_ERR_INVALID;
  std::copy(t->nghbr.begin(), t->nghbr.end(), out);
  return LBM_OK;
}

int lbm_grid_tree_write_points(const lbm_grid_tree* t, const char* path, const int32_t* columns, int32_t ncolumns) {
  if(!t || !path || ncolumns < 0 || (ncolumns > 0 && !columns)) return LBM_ERR_INVALID;
  for(int32_t k = 0; k < ncolumns; ++k)
    if(columns[k] != LBM_TREE_COLUMN_LEVEL && columns[k] != LBM_TREE_COLUMN_NOCHILDREN) return LBM_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if(!f) return LBM_ERR_INVALID;
  static constexpr char axis[4] = {'x', 'y', 'z', 'w'};
  std::vector<char>     buf(1 << 16);
  std::setvbuf(f, buf.data(), _IOFBF, buf.size());
  bool ok = true;
  for(int d = 0; d < t->D; ++d) ok = ok && std::fprintf(f, d + 1 < t->D ? "%c," : "%c", axis[d]) > 0;
  for(int32_t k = 0; k < ncolumns; ++k) ok = ok && std::fprintf(f, columns[k] == LBM_TREE_COLUMN_LEVEL ? ",Level" : ",NoChildren") > 0;
  ok = ok && std::fputc('\n', f) != EOF;
  // coordinates as an ostream at precision 15 writes them (%.15g), integers plainly
  for(int64_t c = 0; c < t->n && ok; ++c) {
    for(int d = 0; d < t->D; ++d) ok = ok && std::fprintf(f, d + 1 < t->D ? "%.15g," : "%.15g", t->centers[c * t->D + d]) > 0;
    for(int32_t k = 0; k < ncolumns; ++k)
      ok = ok && std::fprintf(f, ",%d", columns[k] == LBM_TREE_COLUMN_LEVEL ? static_cast<int>(t->level[c]) : t->nchild[c]) > 0;
    ok = ok && std::fputc('\n', f) != EOF;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? LBM_OK : LBM_ERR_INVALID;
}

int lbm_grid_tree_grid(const lbm_grid_tree* t, lbm_grid** out) {
  if(!t || !out) return LBM_ERR_INVALID;
  *out = nullptr;
  if(t->n >= (int64_t(1) << 31)) return LBM_ERR_INVALID;
  lbm_grid* g = new(std::nothrow) lbm_grid();
  if(!g) return LBM_ERR_NOMEM;
  const int D = t->D, nn = t->nn;
  try {
    g->D     = D;
    g->level = t->max_level;
    g->objs  = t->geom.objs;
    g->body  = t->geom.body;
    g->nbody = t->geom.nbody;
    for(int d = 0; d < 3; ++d) {
      g->bmin[d] = t->geom.bmin[d];
      g->bmax[d] = t->geom.bmax[d];
      g->cog[d]  = t->geom.cog[d];
    }
    g->len0        = t->geom.len0;
    g->cell_length = t->max_len_solver;
    g->cut_length  = t->len[t->max_level];
    g->n           = t->n;
    g->centers     = t->centers;
    g->nbr         = t->nghbr;
    // the solver's length of each cell's level: the generator's, and
    // maxRfnmtLvl's as the solver takes it over
    g->cell_len.resize(t->n);
    for(int64_t c = 0; c < t->n; ++c)
      g->cell_len[c] = t->level[c] == t->max_level ? t->max_len_solver : t->len[t->level[c]];
    // determineBoundaryCells (src/cartesiangrid.h:509-544) in cell order: a
    // cell without a parent, or whose parent is a boundary cell, is one when
    // cut and missing a main neighbour; any other cell is not
    g->bndry.assign(t->n, 0);
    for(int64_t c = 0; c < t->n; ++c) {
      const int64_t p = t->parent[c];
      if(p >= 0 && !(p < c && g->bndry[p])) continue;
      if(!geom_cut(*g, &g->centers[c * D], g->cell_len[c])) continue;
      int present = 0;
      for(int dir = 0; dir < nn; ++dir) present += g->nbr[c * nn + dir] >= 0 ? 1 : 0;
      g->bndry[c] = present < nn ? 1 : 0;
    }
    list_boundary_cells(*g);
  } catch(const std::bad_alloc&) {
    delete g;
    return LBM_ERR_NOMEM;
  }
  *out = g;
  return LBM_OK;
}

void lbm_grid_tree_destroy(lbm_grid_tree* t) { delete t; }

}  // extern "C"
