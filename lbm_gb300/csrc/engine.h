// Internal interfaces between the C-ABI layer (capi.cu) and the two engines.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/lbm_gpu.h"

namespace lbm {

// ---- reference-table engine ------------------------------------------------
// Device image of one boundary-condition object (built once by tables.cpp).
struct TableBnd {
  int      kind      = 0;
  int      has_vec   = 0;
  int      has_press = 0;
  int64_t  n         = 0;       // list entries
  double   vec[3]    = {0, 0, 0};
  double   scalar    = 0.0;
  // device arrays (entry-indexed unless noted)
  int32_t* cells     = nullptr;
  double*  normals   = nullptr;  // n x D
  double*  values    = nullptr;  // n (NEEM values; rewritten by Neumann)
  double*  tang      = nullptr;  // n x Q tangential BB values
  double*  lim_const = nullptr;  // n x Q, 0 where dist is not in the limited set
  int8_t*  lim_empty = nullptr;  // n
  int32_t* ext       = nullptr;  // n extrapolation cell
  int32_t* ext2      = nullptr;  // n second cell (Neumann: ext's neighbour; pressure: 2nd inside cell)
  int32_t* widx      = nullptr;  // n wet-node table index (cell2Bnd) for the entry's cell
  int64_t  nextu     = 0;        // distinct extrapolation cells, in list order
  int32_t* extu      = nullptr;
  // periodic copy: flattened (target cell, dist, source cell) writes, last writer kept
  int64_t  ncopy     = 0;
  int32_t* copy_dst  = nullptr;
  int32_t* copy_q    = nullptr;
  int32_t* copy_src  = nullptr;
  // periodic with pressure: (link0, mapped) pairs
  int32_t* link0     = nullptr;
};

struct TableState {
  int      lattice = 0, equation = 0, D = 0, Q = 0, nvar = 0, nnghbr = 0;
  int64_t  n       = 0;
  double   omega = 0, relax_time = 0, dt = 0, poisson_k = 0, diffusivity = 0;
  // device arrays, q-major SoA: a[q * n + cell]
  double*  fold = nullptr;
  double*  f    = nullptr;
  double*  feq  = nullptr;
  double*  vars = nullptr;     // nvar x n
  double*  varsold = nullptr;  // nvar x n
  int32_t* src  = nullptr;     // (Q-1) x n pull source, -1 = keep
  int32_t* nbr  = nullptr;     // nnghbr x n neighbour table (int32)
  std::vector<TableBnd> bnds;
  bool     need_feq = false;
  // pressure forcing: (target, value cell) pairs for the outlet and inlet passes
  int64_t  nforce_out = 0, nforce_in = 0;
  int32_t *force_out = nullptr, *force_out_val = nullptr, *force_in = nullptr, *force_in_val = nullptr;
  double   forcing_dp = 0;
  bool     forcing = false;
};

// engine entry points (table_engine.cu); all enqueue on `s`
cudaError_t table_initial_condition(TableState& t, cudaStream_t s);
cudaError_t table_step(TableState& t, cudaStream_t s);
cudaError_t table_update_moments(TableState& t, cudaStream_t s);
// FP64 reductions (reduce.cu): out must hold nout doubles on the device
cudaError_t reduce_abs_diff(const double* a, const double* b, int64_t n, int nvec, double* partials, int nblocks, double* out,
                            cudaStream_t s);
cudaError_t reduce_moments(const double* f, int64_t n, int Q, int lattice, double* partials, int nblocks, double* out,
                           cudaStream_t s);
int reduce_blocks(int64_t n);

}  // namespace lbm
