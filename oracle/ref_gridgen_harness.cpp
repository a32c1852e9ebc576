// Reference grid-generator harness: runs the SFCMM/LBM reference's own
// GridGenerator on one JSON config and dumps the cell tree it generated as raw
// little-endian arrays.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit is compiled by
// oracle/build_ref.sh against the copy of the reference sources kept in
// oracle/_ref/ (never committed).  Its outputs are the golden vectors that pin
// the project's multi-level grid generator (lbm_gb300/csrc/grid_tree.cpp).
// Nothing in the product links or runs it.
//
// GridGenerator::run() (src/gridgenerator/gridGenerator.cpp:83-110, 163-238)
// builds the partitioning level, refines it uniformly to "uniformLevel",
// refines the boundary cells level by level up to "maxRfnmtLvl", optionally
// stretches the finest level onto the geometry ("alignNodesWithSurface") and
// writes its points file <outputDir>/<gridFileName>.csv itself.  After it
// returns, this harness writes, for the size() cells of the generator's grid
// (src/gridgenerator/cartesiangrid_generation.h):
//   centers.f64   n x ndim cell centres
//   level.i64     n levels
//   parent.i64    n parent ids (-1: none)
//   global.i64    n global ids
//   children.i64  n x 2^ndim child ids (-1: none)
//   nghbr.i64     n x 2 ndim same-level neighbours (-1: none)
//   bndry.u8      n boundary properties
//   meta.json     n, ndim, partition level, highest level
//
// Usage: ref_gridgen_harness <config.json> <outdir>
// The generator's own outputDir (config key, default "out") is relative to the
// working directory and must exist.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <mpi.h>

#include <sfcmm_common.h>
#include "config.h"
#include "gridgenerator/cartesiangrid_generation.h"
#include "gridgenerator/gridGenerator.h"

namespace {

template <class T>
void writeRaw(const std::string& path, const std::vector<T>& v) {
  std::ofstream o(path, std::ios::binary);
  o.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

template <GInt NDIM>
int dumpTree(const GridInterface& gi, const std::string& out) {
  const auto& grid = static_cast<const CartesianGridGen<Debug_Level::no_debug, NDIM>&>(gi);
  const GInt n  = grid.size();
  const GInt nc = cartesian::maxNoChildren<NDIM>();
  const GInt nn = cartesian::maxNoNghbrs<NDIM>();
  std::vector<double>  centers(n * NDIM);
  std::vector<int64_t> level(n), parent(n), global(n), children(n * nc), nghbr(n * nn);
  std::vector<uint8_t> bndry(n);
  for(GInt c = 0; c < n; ++c) {
    for(GInt d = 0; d < NDIM; ++d) {
      centers[c * NDIM + d] = grid.center(c, d);
    }
    level[c]  = std::to_integer<GInt>(grid.level(c));
    parent[c] = grid.parent(c);
    global[c] = grid.globalId(c);
    for(GInt k = 0; k < nc; ++k) {
      children[c * nc + k] = grid.child(c, k);
    }
    for(GInt k = 0; k < nn; ++k) {
      nghbr[c * nn + k] = grid.neighbor(c, k);
    }
    bndry[c] = grid.property(c, CellProperties::bndry) ? 1 : 0;
  }
  writeRaw(out + "/centers.f64", centers);
  writeRaw(out + "/level.i64", level);
  writeRaw(out + "/parent.i64", parent);
  writeRaw(out + "/global.i64", global);
  writeRaw(out + "/children.i64", children);
  writeRaw(out + "/nghbr.i64", nghbr);
  writeRaw(out + "/bndry.u8", bndry);
  std::ofstream meta(out + "/meta.json");
  meta << "{\"n\": " << n << ", \"ndim\": " << NDIM << ", \"partitionLvl\": " << grid.partitionLvl()
       << ", \"currentHighestLvl\": " << grid.currentHighestLvl() << "}\n";
  return 0;
}

} // namespace

int main(int argc, char** argv) {
  if(argc < 3) {
    std::cerr << "usage: ref_gridgen_harness <config.json> <outdir>" << std::endl;
    return 1;
  }
  const std::string cfg = argv[1];
  const std::string out = argv[2];

  int provided = 0;
  MPI_Init_thread(&argc, &argv, MPI_THREAD_FUNNELED, &provided);
  MPI::g_mpiInformation.init(0, 1);
  cerr0.rdbuf(std::cerr.rdbuf());
  RESET_TIMERS();
  NEW_TIMER_GROUP_NOCREATE(TimeKeeper[Timers::AppGroup], "Application");
  NEW_TIMER_NOCREATE(TimeKeeper[Timers::timertotal], "Total", TimeKeeper[Timers::AppGroup]);
  RECORD_TIMER_START(TimeKeeper[Timers::timertotal]);

  std::ifstream cs(cfg);
  json          config;
  cs >> config;
  const GInt dim = config["dim"];

  int   hargc    = 1;
  char* hargv[2] = {argv[0], nullptr};
  GridGenerator<Debug_Level::no_debug> gridgen(0, 1);
  gridgen.init(hargc, hargv, cfg);
  int rc = static_cast<int>(gridgen.run());
  if(rc == 0) {
    switch(dim) {
      case 1:
        rc = dumpTree<1>(gridgen.grid(), out);
        break;
      case 2:
        rc = dumpTree<2>(gridgen.grid(), out);
        break;
      case 3:
        rc = dumpTree<3>(gridgen.grid(), out);
        break;
      default:
        std::cerr << "unsupported dim " << dim << std::endl;
        rc = 1;
    }
  }
  MPI_Finalize();
  return rc;
}
