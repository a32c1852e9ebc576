// Reference harness: drives the SFCMM/LBM reference's own LBMSolver on one JSON
// case and dumps its state as raw little-endian arrays.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit is compiled by
// oracle/build_ref.sh against a patched copy of the reference sources kept in
// oracle/_ref/ (never committed).  Its outputs are the golden vectors that pin
// the project's C oracle (oracle/lbm_oracle.c) and, through it, the GPU kernels.
// Nothing in the product links or runs it.
//
// What it reproduces, step for step, is LBMSolver::run() (src/lbm/solver.cpp:175-214)
// without the convergence printout and the VTK output: loadConfiguration,
// allocateMemory, POST::init, initialCondition, then `nsteps` calls of
// timeStep() (src/lbm/solver.cpp:306-320).  The residual written at the end is
// the reference's own sumAbsDiff() (src/lbm/solver.cpp:808-815) for every
// variable, i.e. the number convergenceCondition() would print before the next
// step.
//
// With --vtp it also calls the solver's own output(true) at the end, which
// writes its binary VTK PolyData file (src/lbm/solver.cpp:322-384,
// src/common/IO.h) into <outdir>: the golden file of the output writer.
//
// Like run() (src/lbm/solver.cpp:187, 199) it executes the post-processing
// hooks atStart and atEnd; a "postprocessing" line object in the case config
// then writes the reference's line.csv into the working directory
// (src/postprocess/postprocessing.h:87-119): the golden file of the line probe.
//
// With --run it instead calls the solver's own run() (src/lbm/solver.cpp:175-214):
// the reference's loop with its convergence check, extra step and analytic
// comparison (compareToAnalyticalResult, :387-482), which print the residual
// and the errors to cerr0, here at 17 significant digits; <nsteps> is ignored.
// It then prints one JSON line to stdout: the steps run (m_timeStep after the
// loop) and whether the solution diverged.
//
// Usage: ref_harness <config.json> <nsteps> <outdir> [--time] [--vtp] [--run]
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include <mpi.h>

// The harness needs the solver's private state (populations, variables, grid
// tables).  Opening the access specifiers is confined to this test-only TU.
#define private public
#define protected public
#include <sfcmm_common.h>
#include "config.h"
#include "gridgenerator/gridGenerator.h"
#include "lbm/solver.cpp"
#undef private
#undef protected

namespace {

template <class T>
void writeRaw(const std::string& path, const std::vector<T>& v) {
  std::ofstream o(path, std::ios::binary);
  o.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

std::string jnum(double x) {
  std::ostringstream s;
  s.precision(17);
  s << x;
  return s.str();
}

template <LBMethodType LBTYPE, LBEquationType EQ>
int runCase(int argc, char** argv, const std::string& cfg, long nsteps, const std::string& out, bool timing, bool vtp,
            bool runloop) {
  using S                 = LBMSolver<Debug_Level::no_debug, LBTYPE, EQ>;
  constexpr GInt NDIM     = S::NDIM;
  constexpr GInt NDIST    = S::NDIST;
  constexpr GInt NVAR     = S::NVAR;
  constexpr GInt NNGHBR   = NDIM == 1 ? 2 : (NDIM == 2 ? 8 : 6);
  using Grid              = CartesianGrid<Debug_Level::no_debug, NDIM>;

  GridGenerator<Debug_Level::no_debug> gridgen(0, 1);
  gridgen.init(argc, argv, cfg);
  if(gridgen.run() != 0) {
    std::cerr << "grid generation failed" << std::endl;
    return 2;
  }
  logger.close();

  S solver(0, 1);
  solver.init(argc, argv, cfg);
  solver.transferGrid(gridgen.grid());

  if(runloop) {
    cerr0.precision(17);
    solver.run();
    std::cout << "{\"steps\": " << solver.m_timeStep << ", \"diverged\": " << (solver.m_diverged ? "true" : "false") << "}"
              << std::endl;
    return 0;
  }

  solver.loadConfiguration();
  solver.allocateMemory();
  solver.POST::init();
  solver.initialCondition();

  const std::vector<GDouble> fold0 = solver.m_fold;

  solver.executePostprocess(pp::HOOK::ATSTART);
  const auto t0 = std::chrono::steady_clock::now();
  for(long t = 0; t < nsteps; ++t) {
    solver.m_timeStep = t;
    solver.timeStep();
    solver.m_currentTime += solver.m_dt;
  }
  const auto   t1      = std::chrono::steady_clock::now();
  solver.executePostprocess(pp::HOOK::ATEND);
  const double seconds = std::chrono::duration<double>(t1 - t0).count();

  const Grid& grid = *static_cast<Grid*>(solver.m_grid.get());
  const GInt  N    = solver.allCells();

  std::vector<double> residual(NVAR);
  for(GInt v = 0; v < NVAR; ++v) {
    residual[v] = solver.sumAbsDiff(v);
  }

  if(timing) {
    std::cout << "{\"cells\": " << N << ", \"steps\": " << nsteps << ", \"seconds\": " << jnum(seconds) << "}" << std::endl;
    return 0;
  }

  std::vector<double>  centers(N * NDIM);
  std::vector<int64_t> nghbr(N * NNGHBR);
  std::vector<uint8_t> props(N * 2);
  for(GInt c = 0; c < N; ++c) {
    for(GInt d = 0; d < NDIM; ++d) {
      centers[c * NDIM + d] = grid.center(c, d);
    }
    for(GInt d = 0; d < NNGHBR; ++d) {
      nghbr[c * NNGHBR + d] = grid.neighbor(c, d);
    }
    props[c * 2 + 0] = grid.property(c, CellProperties::bndry) ? 1 : 0;
    props[c * 2 + 1] = grid.property(c, CellProperties::periodic) ? 1 : 0;
  }
  writeRaw(out + "/centers.f64", centers);
  writeRaw(out + "/nghbr.i64", nghbr);
  writeRaw(out + "/props.u8", props);
  writeRaw(out + "/fold0.f64", fold0);
  writeRaw(out + "/fold.f64", solver.m_fold);
  writeRaw(out + "/f.f64", solver.m_f);
  writeRaw(out + "/vars.f64", solver.m_vars);
  writeRaw(out + "/varsold.f64", solver.m_varsold);
  writeRaw(out + "/residual.f64", residual);

  // boundary surfaces: names, cell lists and per-cell normals
  std::ofstream meta(out + "/meta.json");
  meta << "{\n";
  meta << "  \"ndim\": " << NDIM << ", \"ndist\": " << NDIST << ", \"nvar\": " << NVAR << ", \"nnghbr\": " << NNGHBR << ",\n";
  meta << "  \"cells\": " << N << ", \"steps\": " << nsteps << ",\n";
  meta << "  \"omega\": " << jnum(solver.m_omega) << ", \"relaxTime\": " << jnum(solver.m_relaxTime) << ", \"dt\": " << jnum(solver.m_dt)
       << ", \"nu\": " << jnum(solver.m_nu) << ", \"maxLvl\": " << solver.maxLvl() << ",\n";
  meta << "  \"cellLength\": " << jnum(grid.lengthOnLvl(grid.maxLvl())) << ",\n";
  meta << "  \"bbox\": [";
  for(GInt d = 0; d < NDIM; ++d) {
    meta << (d ? ", " : "") << jnum(grid.boundingBox().min(d)) << ", " << jnum(grid.boundingBox().max(d));
  }
  meta << "],\n  \"surfaces\": {";
  GBool first = true;
  for(const auto& [name, srf] : grid.m_bndrySurfaces) {
    meta << (first ? "\n" : ",\n") << "    \"" << name << "\": {\"cells\": [";
    first = false;
    GBool firstC = true;
    for(const GInt c : srf.getCellList()) {
      meta << (firstC ? "" : ", ") << c;
      firstC = false;
    }
    meta << "], \"normals\": [";
    firstC = true;
    for(const GInt c : srf.getCellList()) {
      const GDouble* n = srf.normal_p(c);
      for(GInt d = 0; d < NDIM; ++d) {
        meta << (firstC ? "" : ", ") << jnum(n[d]);
        firstC = false;
      }
    }
    meta << "]}";
  }
  meta << "\n  }\n}\n";
  meta.close();
  if(vtp) {
    solver.m_outputDir = out + "/";
    solver.output(true, "");
  }
  return 0;
}

} // namespace

int main(int argc, char** argv) {
  if(argc < 4) {
    std::cerr << "usage: ref_harness <config.json> <nsteps> <outdir> [--time]" << std::endl;
    return 1;
  }
  const std::string cfg    = argv[1];
  const long        nsteps = std::stol(argv[2]);
  const std::string out    = argv[3];
  bool              timing = false, vtp = false, runloop = false;
  for(int a = 4; a < argc; ++a) {
    timing  = timing || std::string(argv[a]) == "--time";
    vtp     = vtp || std::string(argv[a]) == "--vtp";
    runloop = runloop || std::string(argv[a]) == "--run";
  }

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
  const std::string model    = config::opt_config_value(config["solver"], "model", std::string("D2Q9"));
  const std::string equation = config::opt_config_value(config["solver"], "equation", std::string("navierstokes"));

  // the harness gets one argv without the harness-specific arguments
  int   hargc    = 1;
  char* hargv[2] = {argv[0], nullptr};

  int rc = 1;
  if(model == "D2Q9" && equation == "navierstokes") {
    rc = runCase<LBMethodType::D2Q9, LBEquationType::Navier_Stokes>(hargc, hargv, cfg, nsteps, out, timing, vtp, runloop);
  } else if(model == "D2Q9" && equation == "poisson") {
    rc = runCase<LBMethodType::D2Q9, LBEquationType::Poisson>(hargc, hargv, cfg, nsteps, out, timing, vtp, runloop);
  } else if(model == "D2Q5" && equation == "poisson") {
    rc = runCase<LBMethodType::D2Q5, LBEquationType::Poisson>(hargc, hargv, cfg, nsteps, out, timing, vtp, runloop);
  } else if(model == "D1Q3" && equation == "poisson") {
    rc = runCase<LBMethodType::D1Q3, LBEquationType::Poisson>(hargc, hargv, cfg, nsteps, out, timing, vtp, runloop);
  } else {
    std::cerr << "unsupported model/equation " << model << "/" << equation << std::endl;
  }
  MPI_Finalize();
  return rc;
}
