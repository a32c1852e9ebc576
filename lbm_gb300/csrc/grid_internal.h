// The grid object behind include/lbm_grid.h, shared by the host builder
// (grid.cpp) and the device builder (grid_device.cu).
#pragma once

#include <cstdint>
#include <vector>

#include "grid_geom.h"

struct lbm_grid {
  int                        D = 0, level = 0;
  std::vector<lbm_geom_desc> objs;
  std::vector<int32_t>       body;       // body of each object, numbered in order of first appearance
  int                        nbody = 0;
  double                     bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0}, cog[3] = {0, 0, 0};
  double                     len0 = 0, cell_length = 0;
  double                     cut_length = 0;  // length of the generator's cut tests (differs after alignment)
  std::vector<double>        cv[3];           // centre coordinate of each position of the level, per axis
  int64_t                    lo[3] = {0, 0, 0}, ext[3] = {1, 1, 1};  // candidate position range
  int64_t                    n = 0;
  std::vector<double>        centers;    // n x D
  std::vector<int32_t>       ipos;       // n x D integer positions on the level
  std::vector<int64_t>       nbr;        // n x 2D main neighbours
  std::vector<uint8_t>       bndry;      // boundary property
  std::vector<int64_t>       bcells;     // the boundary cells, ascending
  std::vector<uint8_t>       assigned;   // per cell: bit d set when (cell, d) belongs to a surface
  std::vector<double>        cell_len;   // per-cell level length (multi-level grids); empty: cell_length for all

  lbm_grid_geom::GeomSet geom() const {
    lbm_grid_geom::GeomSet s;
    s.nobj  = static_cast<int>(objs.size());
    s.nbody = nbody;
    s.objs  = objs.data();
    s.body  = body.data();
    return s;
  }
};

namespace lbm_grid_impl {
// validation, bounding box, level lengths, centre tables and candidate range
// (everything before the cells are enumerated); returns an LBM status
int setup(lbm_grid& g, int ndim, int level, const lbm_geom_desc* objs, int nobj, const double* bbox);
// main neighbours by position, boundary property and boundary-cell list
void link_cells(lbm_grid& g);
// boundary-cell list from the boundary property
void list_boundary_cells(lbm_grid& g);
// hilbert::index (include/common/math/hilbert.h:16-48) of a point of the unit cube
uint64_t curve_index(const double* x, int D, int level);
// analytic geometry tests of the grid's objects
bool geom_cut(const lbm_grid& g, const double* c, double len);
bool geom_inside(const lbm_grid& g, const double* x);
}  // namespace lbm_grid_impl
