// The objects behind the opaque gops_ctx / gops_graph handles.
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "gops_internal.cuh"

namespace gops {

// Device layout of a graph.  Nodes are relabelled once at build time by a
// stable sort on in-degree (descending): row i of the in-edge CSR is node
// perm[i].  Rows of equal degree class are then contiguous, so each class is
// one "segment" processed with one sub-warp width, and the most-gathered
// nodes sit together at the front of every per-node vector.
constexpr int kMaxSegments = 8;

struct Segment {
  int32_t row_begin, row_end;  // rows [row_begin, row_end) of this class
  int32_t sw;                  // lanes per row (1..32); 32/sw rows per warp task
  int32_t task_begin;          // first task index of the segment
};

struct Plan {
  // hub rows (in-degree > kHubThreshold) are rows [0, n_hub); row h is split
  // into tasks hub_first[h] .. hub_first[h+1]-1 of kHubChunk edges each
  int32_t n_hub = 0;
  int32_t n_hub_tasks = 0;
  int32_t n_segs = 0;
  int32_t n_tasks = 0;  // n_hub_tasks + tasks of all segments
  Segment segs[kMaxSegments];
};

constexpr int kHubChunk = 1024;      // edges per hub task (one warp)
constexpr int kHubThreshold = 4096;  // rows above this in-degree are hubs
// Every in-row is padded to a multiple of four edges (padding: column n,
// weight 0; entry n of the gathered vectors is 0), so a lane loads four edges
// with one aligned 16-byte load.
constexpr int kRowAlign = 4;
// rows interleaved per sub-warp in one warp task of the pull step
constexpr int kRowsPerLane = 2;
// target edges per lane when choosing a degree class's sub-warp width
constexpr int kLaneEdges = 4;

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
  float2 *lpart = nullptr;              // hub chunk partials, per hub task
  unsigned *lcnt = nullptr;             // hub arrival counters, per hub row
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
  struct Ctx *ctx = nullptr;  // the creating context (not dereferenced on destroy)
  int device = 0;
  int64_t n = 0, m = 0;
  int64_t m_stored = 0;  // edges stored in the in-edge CSR (m plus row padding)
  bool weighted = false;
  // in-edge CSR over relabelled ids: row i lists the (relabelled) sources of
  // the edges into node perm[i], in ascending original source order
  int64_t *in_rp = nullptr;
  int32_t *in_col = nullptr;
  float *in_val = nullptr;      // max(w,0)/weight-sum of the source (weighted graphs)
  float *deg = nullptr;         // out-degree (relabelled order); 0 = unweighted-dangling
  uint32_t *dmask_w = nullptr;  // weighted-dangling bitmask (relabelled order)
  int32_t *perm = nullptr;      // relabelled row i -> original node id
  int64_t *out_rp = nullptr;    // the out-adjacency as uploaded (original ids, adapter order)
  int32_t *out_col = nullptr;
  int32_t *hub_first = nullptr;     // n_hub + 1 task offsets
  int32_t *hub_task_row = nullptr;  // hub task -> hub row
  Plan plan;
  Workspace ws;
  struct BatchState *batch = nullptr;  // batched-PPR plan and workspace (built on first use)
};

void batch_free(Graph &g);

struct Ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  SolveState *host_state = nullptr;  // pinned
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // a second stream for the weight upload, which overlaps the input checks
  // and the edge sort of gops_graph_upload; copy_ev orders it against stream
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[2] = {nullptr, nullptr};
  // the graph build's hand-over to and from the copy stream: build_ev[0]
  // after its structure pass (main stream), build_ev[1] after the weight
  // passes that run on the copy stream once the weights have arrived
  cudaEvent_t build_ev[2] = {nullptr, nullptr};
  // pinned host staging of the batched path's result blocks (two waves in
  // flight), kept across calls and graphs: pinning is slow next to a solve;
  // sev[q] follows the copy into hstage[q]
  float *hstage[2] = {nullptr, nullptr};
  size_t hstage_bytes = 0;
  cudaEvent_t sev[2] = {nullptr, nullptr};
  // optional per-launch timing of the iteration kernels (gops_ctx_set_timing)
  bool timing = false;
  std::vector<cudaEvent_t> tev;
  std::string last_error;
  gops_stats stats{};
  const double *last_scores = nullptr;  // device scores of the last solve
  bool noalloc_attached = false;        // counted in the no-alloc scratch's live contexts
  int set(const Status &s) {
    if (s.code != GOPS_OK) last_error = s.msg;
    return s.code;
  }
};

Status solve_plain_in_workspace(Ctx *ctx, Graph *g, const gops_config *cfg, Workspace &ws,
                                double *scores_host, gops_run *run);
// the no-allocation entry point's scratch array (csrc/noalloc.cu): mapped on
// a device with its first context, released with its last
Status noalloc_attach(int device);
void noalloc_detach(int device);
// w_ready (optional): an event after which d_w is complete; the build
// orders its first read of d_w after it.
Status graph_build_from_out_csr_device(Ctx *ctx, Graph *g, const int64_t *d_out_rp,
                                       const int32_t *d_out_col, const double *d_w,
                                       cudaEvent_t w_ready = nullptr);
Status workspace_ensure(Ctx *ctx, Graph *g);
void workspace_free(Workspace &ws);
void graph_free_device(Graph &g);

}  // namespace gops

// the opaque handles of include/gops.h
struct gops_ctx {
  gops::Ctx impl;
};
struct gops_graph {
  gops::Graph impl;
};
