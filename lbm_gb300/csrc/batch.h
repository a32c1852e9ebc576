// Batched engine: many independent D2Q9 lid-driven cavities in one launch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/lbm_gpu_box.h"

struct lbm_gpu_ctx;

namespace lbm {

// one domain in the device table
struct BatchDomain {
  int32_t n;              // side (cells)
  int32_t tiles_per_row;  // ceil(n / 32): one warp covers 32 cells of a row
  int64_t pop_off;        // first population element of the domain
  int64_t mom_off;        // first moment element of the domain
  int64_t plane;          // cells per population plane (n*n rounded up to 32)
  double  omega;
  float   omega_f;
  int32_t pad;
};

struct BatchParams {
  const BatchDomain* dom;
  const int32_t*     active;      // active domain ids
  const int64_t*     tile_start;  // warp-tile prefix over the active domains (nactive + 1)
  const int32_t*     nactive;     // device scalar
  void*              pop;
  void*              mom;
  double*            partials;    // one slot per warp tile and variable
  int64_t            partial_stride;
  double             lid, lid_f_pad;
  float              lid_f;
};

struct BatchState {
  int                      storage = 0, device = 0, ndomains = 0;
  std::vector<BatchDomain> dom;
  std::vector<int32_t>     active;      // host copy of the active list
  std::vector<int64_t>     steps;       // per-domain completed steps
  std::vector<int32_t>     status;      // per-domain lbm_batch_status
  std::vector<double>      residual;    // per-domain residual (3 per domain) of the last check
  BatchParams              p{};
  BatchDomain*             d_dom = nullptr;
  int32_t*                 d_active = nullptr;
  int64_t*                 d_tile_start = nullptr;
  int32_t*                 d_nactive = nullptr;
  void*                    pop = nullptr;
  void*                    mom = nullptr;
  double*                  partials = nullptr;
  double*                  d_res = nullptr;
  double*                  f64 = nullptr;  // staging for one domain
  int64_t                  total_tiles = 0, max_plane = 0;
  int                      grid = 0, tpb = 256;
  int                      mom_valid = 0, res_ready = 0;
  int64_t                  global_steps = 0;  // steps taken by the active set since the last activation change
  cudaGraphExec_t          graph[2] = {nullptr, nullptr};
};

cudaError_t batch_initial_condition(BatchState* b, cudaStream_t s);
int         batch_step(BatchState* b, int64_t nsteps, cudaStream_t s, std::string& err);
void        batch_destroy(BatchState* b);
int         batch_info(const BatchState* b, int64_t* ncells, int32_t* q, int32_t* nvar);

}  // namespace lbm

lbm_gpu_ctx*      lbm_internal_new_batch_ctx(int device, lbm::BatchState* batch, cudaStream_t stream);
lbm::BatchState*  lbm_internal_batch(lbm_gpu_ctx* ctx);
