// The objects behind the opaque gops_ctx / gops_graph handles.
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "gops_internal.cuh"

namespace gops {

// Device layout of a graph.  Nodes are relabelled once at build time by a
// stable sort on in-degree (descending): row i of the in-edge CSR is node
// perm[i].  Rows of one degree class are then contiguous, and the most
// gathered nodes sit together at the front of every per-node vector.
//
// The pull kernel works in batches.  Rows [0, n_big) have more than kBigRow
// in-edges; each is split into kBatchEdges-edge chunks, one batch per chunk.
// The remaining rows form segments of one degree class each; a segment batch
// is rows_per_batch consecutive rows with sw lanes per row, at most
// kBatchEdges edges in all.  A batch's column indices, weights and row
// offsets are contiguous in memory and arrive in shared memory by one bulk
// copy each.
constexpr int kMaxSegments = 8;
constexpr int kPullThreads = 512;   // threads of a pull block
constexpr int kBatchEdges = 4096;   // edges per batch (shared-memory stage)
constexpr int kBigRow = 256;        // rows above this in-degree are chunked
#ifndef GOPS_LANE_EDGES
#define GOPS_LANE_EDGES 4
#endif
// target edges per lane when choosing a degree class's sub-warp width
constexpr int kLaneEdges = GOPS_LANE_EDGES;

struct Segment {
  int32_t row_begin, row_end;  // rows [row_begin, row_end) of this class
  int32_t sw;                  // lanes per row (1..32)
  int32_t rows_per_batch;
  int32_t batch_begin;         // first batch index of the segment
  int32_t pad;
};

struct Plan {
  int32_t n_big = 0;          // chunked rows [0, n_big)
  int32_t n_big_batches = 0;  // their chunks: batches [0, n_big_batches)
  int32_t n_segs = 0;
  int32_t n_batches = 0;      // all batches
  Segment segs[kMaxSegments];
};

// Solver workspace held by a graph (allocated on first solve, reused).
struct Workspace {
  int64_t n = 0;
  float2 *gdf[2] = {nullptr, nullptr};  // gathered vector, double-float phase
  float *gf[2] = {nullptr, nullptr};    // gathered vector, FP32 phase
  float2 *acc = nullptr;                // x while in the double-float phase
  float *tail = nullptr;                // sum of the FP32-phase steps
  float2 *pdf = nullptr;                // personalization (normalised) as double-float
  double *scores = nullptr;             // final x = acc + tail, in node order
  long long *sums = nullptr;            // 3 slots x {dangling, l1, nonfinite, spare}
  float2 *lpart = nullptr;              // chunk partials, per big-row batch
  unsigned *lcnt = nullptr;             // arrival counters, per big row
  int *err = nullptr;                   // device error word (bounded waits that ran out)
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
  // in-edge CSR over relabelled ids: row i lists the (relabelled) sources of
  // the edges into node perm[i], in ascending original source order
  int64_t *in_rp = nullptr;
  int32_t *in_col = nullptr;
  float *in_val = nullptr;      // max(w,0)/weight-sum of the source (weighted graphs)
  float *deg = nullptr;         // out-degree (relabelled order); 0 = unweighted-dangling
  uint32_t *dmask_w = nullptr;  // weighted-dangling bitmask (relabelled order)
  int32_t *perm = nullptr;      // relabelled row i -> original node id
  int32_t *big_first = nullptr;      // n_big + 1 chunk-batch offsets
  int32_t *big_batch_row = nullptr;  // chunk batch -> big row
  Plan plan;
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
void graph_free_device(Graph &g);

}  // namespace gops
