// The objects behind the opaque gops_ctx / gops_graph handles.
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "gops_internal.cuh"

namespace gops {

// One unit of work of the pull kernels.  Normal items are a run of whole rows
// [r0, r1) whose in-edges fit the shared-memory stage; a row with more than
// `long_row` in-edges is split into `nchunks` items (first = index of its
// chunk 0) whose partial sums are combined by the chunk that finishes last.
struct Item {
  int32_t r0, r1;
  int32_t first;    // -1 for a normal item
  int32_t nchunks;  // chunks of the long row (0 for a normal item)
};

// Solver workspace held by a graph (allocated on first solve, reused).
struct Workspace {
  int64_t n = 0;
  float2 *gdf[2] = {nullptr, nullptr};  // gathered vector, double-float phase
  float *gf[2] = {nullptr, nullptr};    // gathered vector, FP32 phase
  float2 *acc = nullptr;                // x while in the double-float phase
  float *tail = nullptr;                // sum of the FP32-phase steps
  float2 *pdf = nullptr;                // personalization (normalised) as double-float
  double *scores = nullptr;             // final x = acc + tail
  long long *sums = nullptr;            // 3 slots x {dangling, l1, nonfinite, spare}
  float2 *lpart = nullptr;              // long-row chunk partials, per item
  unsigned *lcnt = nullptr;             // long-row arrival counters, per item
  struct SolveState *state = nullptr;   // device-side run record
};

struct SolveState {
  unsigned long long iterations;
  unsigned long long f32_from;  // first step run in the FP32 phase (0: none)
  double diff_l1;
  int done;
  int converged;
  int f32_phase;
  int pad;
};

struct Graph {
  struct Ctx *ctx = nullptr;
  int64_t n = 0, m = 0;
  bool weighted = false;
  // in-edge CSR (row v lists the sources u of edges u->v, in source order)
  int64_t *in_rp = nullptr;
  int32_t *in_col = nullptr;
  float *in_val = nullptr;    // max(w,0)/weight-sum of the source (weighted graphs)
  float *deg = nullptr;       // out-degree as float; 0 marks an unweighted-dangling node
  uint32_t *dmask_w = nullptr;  // weighted-dangling bitmask (weight sum == 0)
  // work partition of the pull kernels
  Item *items = nullptr;
  int32_t n_items = 0;
  int32_t window = 0;  // edge window W (normal items hold < 2W in-edges)
  int32_t max_chunks = 0;
  Workspace ws;
};

struct Ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  SolveState *host_state = nullptr;  // pinned
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // optional per-launch timing of the iteration kernels (gops_ctx_set_timing)
  bool timing = false;
  std::vector<cudaEvent_t> tev;
  std::string last_error;
  gops_stats stats{};
  const double *last_scores = nullptr;  // device scores of the last solve
  int set(const Status &s) {
    if (s.code != GOPS_OK) last_error = s.msg;
    return s.code;
  }
};

Status graph_build_from_out_csr_device(Ctx *ctx, Graph *g, const int64_t *d_out_rp,
                                       const int32_t *d_out_col, const double *d_w);
Status workspace_ensure(Ctx *ctx, Graph *g);
void workspace_free(Workspace &ws);

}  // namespace gops
