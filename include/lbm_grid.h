/* Host-side grid and table build for the GB300 LBM library (C ABI).
 *
 * Builds, from an analytic geometry (boxes and spheres, bodies with
 * subtracted objects), the uniform Cartesian grid that the SFCMM/LBM
 * reference's grid generator and CartesianGrid produce when
 * partitionLevel == uniformLevel == maxRfnmtLvl (every reference LBM case),
 * and the tables its LBM solver reads (for multi-level grids the tree calls
 * at the end of this header build the cells, lbm_grid_tree_grid hands them
 * to the same table calls):
 *
 *   entry point                  reference step it replaces
 *   lbm_grid_create              GridGenerator::init / createPartitioningGrid, deleteOutsideCells,
 *                                reorderHilbertCurve (src/gridgenerator/gridGenerator.cpp:255-287,
 *                                src/gridgenerator/cartesiangrid_generation.h:71-149, 505-610, 664-735),
 *                                GeometryManager (src/geometry.h:923-1104), bounding box and level
 *                                lengths (src/cartesiangrid_base.h:125-142)
 *   lbm_grid_align               GridGenerator's alignNodesWithSurface step
 *                                (src/gridgenerator/cartesiangrid_generation.h:255-300)
 *   lbm_grid_boundary            CartesianGrid::determineBoundaryCells (src/cartesiangrid.h:509-544)
 *   lbm_grid_add_surface         CartesianGrid::identifyBndrySurfaces, one surface entry
 *                                (src/cartesiangrid.h:551-598)
 *   lbm_grid_connect_periodic    CartesianGrid::addPeriodicConnection (src/cartesiangrid.h:636-703)
 *   lbm_grid_neighbors           the neighbour table after addDiagonalNghbrs (src/cartesiangrid.h:450-487)
 *   lbm_grid_tree_create         GridGenerator::generateGrid for any partitionLevel <= uniformLevel <=
 *                                maxRfnmtLvl (src/gridgenerator/gridGenerator.cpp:163-238,
 *                                src/gridgenerator/cartesiangrid_generation.h)
 *   lbm_grid_tree_write_points   CartesianGridGen::save, ASCII points (cartesiangrid_generation.h:208-253)
 *   lbm_grid_tree_grid           CartesianGrid::loadGridInplace of the whole array, boundary cells included
 *                                (src/cartesiangrid.h:264-320, 509-544)
 *
 * In 2D (and 1D) every table equals the reference's bit for bit.  In 3D,
 * where the reference stops (box and sphere cut tests, src/geometry.h:690-692
 * and 796-798; diagonal neighbours, src/cartesiangrid.h:483-485), the same
 * rules are extended to the third dimension: a box cell is cut when it
 * touches one of the six faces within the face's extent, a sphere cell when
 * the sphere surface passes between its eight vertices, and the twelve
 * edge neighbours are formed through the main neighbours (x step first,
 * then y, then z), indexed in the D3Q19 direction order.
 *
 * All calls but lbm_grid_create_device are host-only (no device memory, no
 * CUDA call).  Status codes are those of lbm_gpu.h.
 */
#ifndef LBM_GRID_H
#define LBM_GRID_H

#include <stdint.h>

#include "lbm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_GEOM_BOX 0
#define LBM_GEOM_SPHERE 1

typedef struct lbm_geom_desc {
  int32_t kind;      /* LBM_GEOM_BOX or LBM_GEOM_SPHERE */
  int32_t body;      /* objects with the same body id form one body ("body" key) */
  int32_t subtract;  /* 1: the object is removed from its body ("subtract" key) */
  int32_t reserved;
  double  a[3];      /* box corner A */
  double  b[3];      /* box corner B */
  double  center[3]; /* sphere centre */
  double  radius;    /* sphere radius */
} lbm_geom_desc;

typedef struct lbm_grid lbm_grid;

/* The grid at `level` over `bbox` (2*ndim values min0,max0,min1,...; NULL:
 * the union of the objects' bounding boxes): the cells cut by an object or
 * with their centre inside the geometry, in the curve order of
 * hilbert::index (include/common/math/hilbert.h:16-48), with their main
 * neighbours.  Objects are given in the order of the config's "geometry"
 * keys (sorted). */
int lbm_grid_create(int32_t ndim, int32_t level, const lbm_geom_desc* objs, int32_t nobj, const double* bbox, lbm_grid** out);

/* lbm_grid_create with the cells enumerated on GPU `device`: the curve
 * indices of the level are walked in order (the index is a bijection of the
 * positions), each position tested with the host's geometry code, and the
 * kept cells numbered by a prefix sum; main neighbours and boundary cells are
 * found on the device too.  The grid equals lbm_grid_create's bit for bit.
 * Needs ndim*level <= 30 (one byte and one int32 of device memory per
 * position of the level's cube, plus the cell tables); everything after
 * creation runs on the host as for lbm_grid_create. */
int lbm_grid_create_device(int32_t ndim, int32_t level, const lbm_geom_desc* objs, int32_t nobj, const double* bbox, int32_t device,
                           lbm_grid** out);

/* "alignNodesWithSurface": stretch the grid so that the outermost cell
 * centres along `align_dir` (along every axis when the centres span the same
 * range on all of them) lie on the bounding box, scale the cell length with
 * it, and delete the cells that are then neither cut nor inside, as the
 * reference's GridGenerator does (transformMaxRfnmtLvlToExtent,
 * src/gridgenerator/cartesiangrid_generation.h:255-300).  Call before any
 * surface. */
int lbm_grid_align(lbm_grid* g, int32_t align_dir);

/* hilbert::index of a point x (ndim values in the unit cube, ndim <= 4) at
 * `level` (include/common/math/hilbert.h:16-48): the key the cells are
 * sorted by */
int lbm_grid_curve_index(int32_t ndim, int32_t level, const double* x, uint64_t* out);

int64_t lbm_grid_ncells(const lbm_grid* g);
/* width of the neighbour table: 2 (1D), 8 (2D), 18 (3D) */
int32_t lbm_grid_nnghbr(const lbm_grid* g);
/* bounding box (2*ndim) and the cell length of the grid level */
int lbm_grid_info(const lbm_grid* g, double* bbox, double* cell_length);
/* cell centres, ncells x ndim, curve order */
int lbm_grid_centers(const lbm_grid* g, double* out);
/* boundary property per cell: cut by the geometry and missing a main neighbour */
int lbm_grid_boundary(const lbm_grid* g, uint8_t* out);
/* One surface of a "boundary" entry: for each direction in [dir_begin,
 * dir_end) and each boundary cell without a main neighbour in it that
 * object `obj` cuts, the pair (cell, direction) unless an earlier call took
 * it.  *n = the number of pairs.  With cells and dirs NULL (and cap 0) the
 * call only counts; otherwise it writes the pairs in the reference's order
 * and takes them, or, when they are more than `cap`, returns
 * LBM_ERR_INVALID and takes none. */
int lbm_grid_add_surface(lbm_grid* g, int32_t obj, int32_t dir_begin, int32_t dir_end, int64_t* cells, int8_t* dirs, int64_t cap,
                         int64_t* n);
/* Connect the cells of two periodic surfaces whose centres differ along
 * exactly one axis (main neighbours across the period). */
int lbm_grid_connect_periodic(lbm_grid* g, const int64_t* cells_a, int64_t na, const int64_t* cells_b, int64_t nb);
/* neighbour table, ncells x nnghbr (-1: none): main directions, then the
 * diagonals built from them */
int lbm_grid_neighbors(const lbm_grid* g, int64_t* out);
void lbm_grid_destroy(lbm_grid* g);

/* ---- Multi-level grids: the reference generator's whole cell tree ------ */

typedef struct lbm_grid_tree lbm_grid_tree;

/* columns of lbm_grid_tree_write_points ("outputValues") */
#define LBM_TREE_COLUMN_LEVEL 0
#define LBM_TREE_COLUMN_NOCHILDREN 1

/* The cell tree GridGenerator::generateGrid builds
 * (src/gridgenerator/gridGenerator.cpp:163-238,
 * src/gridgenerator/cartesiangrid_generation.h) for
 * 0 <= partition_level <= uniform_level <= max_level <= 20 in an array of
 * max_cells slots ("maxNoCells"): the partitioning level in curve order
 * (createPartitioningGrid, :71-147), every cell refined up to uniform_level
 * (uniformRefineGrid, :151-169), then the boundary cells of the finest level
 * refined up to max_level (markBndryCells / refineMarkedCells, :173-206),
 * each new level appended after the grid with its outside cells deleted in
 * the reference's order.  align_dir >= 0 applies alignNodesWithSurface along
 * that axis to the cells of max_level (:255-304); -1 skips it.  The cells are
 * those of the reference's array, in its order: the partitioning level first,
 * then each finer level.  LBM_ERR_NOMEM: the grid does not fit in max_cells
 * slots (the reference stops with "Out of memory"). */
int lbm_grid_tree_create(int32_t ndim, int32_t partition_level, int32_t uniform_level, int32_t max_level, int64_t max_cells,
                         const lbm_geom_desc* objs, int32_t nobj, const double* bbox, int32_t align_dir, lbm_grid_tree** out);
int64_t lbm_grid_tree_ncells(const lbm_grid_tree* t);
/* partitioning level and the finest level built */
int lbm_grid_tree_levels(const lbm_grid_tree* t, int32_t* partition_level, int32_t* highest_level);
/* per cell (any pointer may be NULL): centres (ncells x ndim), level, parent
 * (-1: none), global id (the slot the cell was created in), number of
 * children, boundary property */
int lbm_grid_tree_cells(const lbm_grid_tree* t, double* centers, int8_t* level, int64_t* parent, int64_t* global_id, int32_t* nchildren,
                        uint8_t* bndry);
/* child ids, ncells x 2^ndim in child order (bit d set: the + half along
 * axis d), -1: none */
int lbm_grid_tree_children(const lbm_grid_tree* t, int64_t* out);
/* same-level neighbours, ncells x 2 ndim (-x, +x, -y, +y, -z, +z), -1: none */
int lbm_grid_tree_neighbors(const lbm_grid_tree* t, int64_t* out);
/* the generator's points file (ASCII::writePointsCSV, src/common/IO.h:36-81):
 * a header of the axis names and the columns, then one line per cell with
 * the centre at 15 significant digits and the listed columns */
int lbm_grid_tree_write_points(const lbm_grid_tree* t, const char* path, const int32_t* columns, int32_t ncolumns);
/* The tree's cells as the LBM solver's grid loads them
 * (CartesianGrid::loadGridInplace, src/cartesiangrid.h:264-320): every cell
 * of every level, in the tree's order, with its same-level neighbours; the
 * boundary property as determineBoundaryCells sets it (:509-544: a cell
 * whose parent is not a boundary cell is not one); surfaces cut with the
 * length of each cell's level.  The result takes the calls after
 * lbm_grid_create (lbm_grid_add_surface, lbm_grid_connect_periodic,
 * lbm_grid_neighbors, lbm_grid_destroy); alignment is the tree's own.  The
 * reference's solver steps every level of such a grid as a lattice of its
 * own (src/lbm/solver.cpp:525). */
int lbm_grid_tree_grid(const lbm_grid_tree* t, lbm_grid** out);
void lbm_grid_tree_destroy(lbm_grid_tree* t);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GRID_H */
