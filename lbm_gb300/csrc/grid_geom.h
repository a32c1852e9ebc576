// Analytic geometry tests of the grid build (boxes and spheres), shared by
// the host builder (grid.cpp) and the device builder (grid_device.cu) so that
// both give the same bits: the same operations in the same order, compiled
// without floating-point contraction in both translation units.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>

#include "../../include/lbm_grid.h"

#ifdef __CUDACC__
#define LBM_GRID_HD __host__ __device__ inline
#else
#define LBM_GRID_HD inline
#endif

namespace lbm_grid_geom {

// gcem::sqrt(2) as the reference's constexpr evaluation rounds it (one unit in
// the last place below the correctly rounded square root); used by the 2D
// sphere cut test (src/geometry.h:667).
constexpr double kSqrt2Ref = 0x1.6a09e667f3bccp+0;
constexpr double kSqrt3    = 0x1.bb67ae8584caap+0;  // sqrt(3), correctly rounded
constexpr double kEps      = std::numeric_limits<double>::epsilon();

// Euclidean norm of a - b summed in axis order (Eigen's squaredNorm of a
// small fixed-size vector), then sqrt
LBM_GRID_HD double dist(const double* a, const double* b, int D) {
  double s = 0.0;
  for(int d = 0; d < D; ++d) {
    const double t = a[d] - b[d];
    s              = d == 0 ? t * t : s + t * t;
  }
  return sqrt(s);
}

// GeomBox::pointIsInside / GeomSphere::pointIsInside (src/geometry.h:660-662, 755-762)
LBM_GRID_HD bool obj_inside(const lbm_geom_desc& o, const double* x, int D) {
  if(o.kind == LBM_GEOM_SPHERE) return dist(x, o.center, D) < o.radius + kEps;
  for(int d = 0; d < D; ++d)
    if(o.a[d] > x[d] || o.b[d] < x[d]) return false;
  return true;
}

// GeomBox::cutWithCell (src/geometry.h:764-807); the 3D form extends the 2D
// rule to the six faces
LBM_GRID_HD bool box_cut(const lbm_geom_desc& o, const double* c, double len, int D) {
  const double h = 0.5 * len;
  if(D == 1) return fabs(o.a[0] - c[0]) <= h || fabs(o.b[0] - c[0]) <= h;
  for(int a = 0; a < D; ++a) {
    bool span = true;  // within the face's extent along the other axes
    for(int b = 0; b < D; ++b)
      if(b != a && !(o.a[b] - h <= c[b] && o.b[b] + h >= c[b])) span = false;
    if(!span) continue;
    if(fabs(c[a] - o.a[a]) <= h) return true;
    if(fabs(c[a] - o.b[a]) <= h) return true;
  }
  return false;
}

// GeomSphere::cutWithCell (src/geometry.h:664-698): a cell within the
// annulus of the circumscribed radius is cut unless all its vertices lie in
// the sphere.  3D: circumscribed radius sqrt(3) h and eight vertices.
LBM_GRID_HD bool sphere_cut(const lbm_geom_desc& o, const double* c, double len, int D) {
  const double distance = dist(c, o.center, D);
  const double h        = 0.5 * len;
  const double surr     = (D == 3 ? kSqrt3 : kSqrt2Ref) * h;
  if(!(distance <= o.radius + surr && distance >= o.radius - surr)) return false;
  if(D == 1) return true;  // the reference's vertex count stays 0 below 2D
  double origin[3];
  for(int d = 0; d < D; ++d) origin[d] = c[d] - h;
  int inside = 0;
  for(int v = 0; v < (1 << D); ++v) {
    double vert[3];
    for(int d = 0; d < D; ++d) vert[d] = ((v >> d) & 1) ? origin[d] + len : origin[d];
    if(dist(vert, o.center, D) <= o.radius) ++inside;
  }
  return inside < (1 << D);
}

LBM_GRID_HD bool obj_cut(const lbm_geom_desc& o, const double* c, double len, int D) {
  return o.kind == LBM_GEOM_SPHERE ? sphere_cut(o, c, len, D) : box_cut(o, c, len, D);
}

}  // namespace lbm_grid_geom

namespace lbm_grid_geom {

// The objects of a geometry with their bodies (body ids numbered in order of
// first appearance), usable on the host and, with device copies of the two
// arrays, on the device.
struct GeomSet {
  int                  nobj  = 0;
  int                  nbody = 0;
  const lbm_geom_desc* objs  = nullptr;
  const int32_t*       body  = nullptr;
};

// GeometryManager::pointIsInside (src/geometry.h:1011-1047): the first body
// (in order) with an object containing x decides
LBM_GRID_HD bool set_inside(const GeomSet& g, const double* x, int D) {
  for(int b = 0; b < g.nbody; ++b) {
    bool has_sub = false;
    for(int i = 0; i < g.nobj; ++i) has_sub |= g.body[i] == b && g.objs[i].subtract != 0;
    for(int i = 0; i < g.nobj; ++i) {
      if(g.body[i] != b || !obj_inside(g.objs[i], x, D)) continue;
      if(!has_sub) return true;
      if(g.objs[i].subtract) return false;
      for(int j = 0; j < g.nobj; ++j)
        if(g.body[j] == b && g.objs[j].subtract && obj_inside(g.objs[j], x, D)) return false;
      return true;
    }
  }
  return false;
}

// GeometryManager::cutWithCell (src/geometry.h:1055-1062): any object
LBM_GRID_HD bool set_cut(const GeomSet& g, const double* c, double len, int D) {
  for(int i = 0; i < g.nobj; ++i)
    if(obj_cut(g.objs[i], c, len, D)) return true;
  return false;
}

// hilbert::index (include/common/math/hilbert.h:16-48) of the cell at
// integer position p on the level: the quadrant of each level is the
// position's bit there, so the index is a bijection of the positions
LBM_GRID_HD uint64_t curve_index_int(const int64_t* p, int D, int level) {
  constexpr int lut[16] = {0, 3, 1, 2, 5, 4, 6, 7, 10, 9, 11, 8, 15, 14, 12, 13};
  uint64_t      index   = 0;
  for(int l = 0; l < level; ++l) {
    int q = 0;
    for(int d = 0; d < D; ++d) q |= static_cast<int>((p[d] >> (level - 1 - l)) & 1) << d;
    index |= static_cast<uint64_t>(lut[q]) << (D * (level - 1 - l));
  }
  return index;
}

// its inverse: the position of curve index `index`
LBM_GRID_HD void curve_position(uint64_t index, int D, int level, int64_t* p) {
  constexpr int inv[16] = {0, 2, 3, 1, 5, 4, 6, 7, 11, 9, 8, 10, 14, 15, 13, 12};
  for(int d = 0; d < D; ++d) p[d] = 0;
  for(int l = 0; l < level; ++l) {
    const int q = inv[(index >> (D * (level - 1 - l))) & ((1u << D) - 1)];
    for(int d = 0; d < D; ++d) p[d] = (p[d] << 1) | ((q >> d) & 1);
  }
}

}  // namespace lbm_grid_geom
