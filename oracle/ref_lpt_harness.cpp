// Reference harness for the particle solver: drives the SFCMM/LBM reference's
// own LPTSolver on one JSON case and dumps its particle state.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh against the
// patched copy of the reference sources in oracle/_ref/ (never committed).
// Its outputs are the golden vectors that pin the project's particle step.
//
// It reproduces LPTSolver::run() (src/lpt/solver.cpp:243-281) without output:
// loadConfiguration, allocateMemory, initialCondition, then `nsteps` calls of
// timeStep() (src/lpt/solver.cpp:335-349).  Written to <outdir>: vars0.f64
// and vars.f64 (the solver's m_vars, noParticles x NVARS, before and after),
// start.f64 (the start locations) and meta.json.
//
// Usage: ref_lpt_harness <config.json> <nsteps> <outdir> [--time]
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <mpi.h>

#define private public
#define protected public
#include <sfcmm_common.h>
#include "config.h"
#include "lpt/solver.cpp"
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

template <GInt NDIM>
int runCase(int argc, char** argv, const std::string& cfg, long nsteps, const std::string& out, bool timing) {
  using S = LPTSolver<Debug_Level::no_debug, NDIM, LPTType::Normal>;
  S solver(0, 1);
  solver.init(argc, argv, cfg);
  solver.loadConfiguration();
  solver.allocateMemory();
  solver.initialCondition();
  const std::vector<GDouble> vars0(solver.m_vars.begin(), solver.m_vars.begin() + solver.m_noParticles * S::NVARS);
  const auto                 t0 = std::chrono::steady_clock::now();
  for(long t = 0; t < nsteps; ++t) {
    solver.m_timeStep = t;
    solver.timeStep();
  }
  const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if(timing) {
    std::cout << "{\"particles\": " << solver.m_noParticles << ", \"steps\": " << nsteps << ", \"seconds\": " << jnum(seconds) << "}"
              << std::endl;
    return 0;
  }
  const std::vector<GDouble> vars(solver.m_vars.begin(), solver.m_vars.begin() + solver.m_noParticles * S::NVARS);
  std::vector<GDouble>       start;
  for(const auto& p : solver.m_start_location)
    for(GInt d = 0; d < NDIM; ++d) start.push_back(p[d]);
  writeRaw(out + "/vars0.f64", vars0);
  writeRaw(out + "/vars.f64", vars);
  writeRaw(out + "/start.f64", start);
  std::ofstream meta(out + "/meta.json");
  meta << "{\"ndim\": " << NDIM << ", \"nvars\": " << S::NVARS << ", \"particles\": " << solver.m_noParticles
       << ", \"steps\": " << nsteps << ", \"dt\": " << jnum(solver.m_dt) << ", \"time\": " << jnum(solver.m_currentTime)
       << ", \"rho_infty\": " << jnum(solver.m_rho_a_infty) << ", \"nu_infty\": " << jnum(solver.m_nu_a_infty) << ", \"gravity\": [";
  for(GInt d = 0; d < NDIM; ++d) meta << (d ? ", " : "") << jnum(solver.m_gravity[d]);
  meta << "], \"v_infty\": [";
  for(GInt d = 0; d < NDIM; ++d) meta << (d ? ", " : "") << jnum(solver.m_velo_a_infty[d]);
  meta << "]}" << std::endl;
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if(argc < 4) {
    std::cerr << "usage: ref_lpt_harness <config.json> <nsteps> <outdir> [--time]" << std::endl;
    return 1;
  }
  MPI_Init(&argc, &argv);
  // the application timers the solver's own timers hang from (src/main.cpp:212-214)
  NEW_TIMER_GROUP_NOCREATE(TimeKeeper[Timers::AppGroup], "Application");
  NEW_TIMER_NOCREATE(TimeKeeper[Timers::timertotal], "Total", TimeKeeper[Timers::AppGroup]);
  RECORD_TIMER_START(TimeKeeper[Timers::timertotal]);
  const std::string cfg    = argv[1];
  const long        nsteps = std::stol(argv[2]);
  const std::string out    = argv[3];
  const bool        timing = argc > 4 && std::string(argv[4]) == "--time";
  std::ifstream     in(cfg);
  json              j;
  in >> j;
  const GInt dim = j.value("dim", 2);
  int        rc  = dim == 3 ? runCase<3>(argc, argv, cfg, nsteps, out, timing) : runCase<2>(argc, argv, cfg, nsteps, out, timing);
  MPI_Finalize();
  return rc;
}
