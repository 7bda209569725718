// graphops.hpp -- C++ host API over libgops (include/gops.h), mirroring the
// graphops crate's PageRank path (graphops 0.4.1):
//
//   src/pagerank.rs  PageRankConfig (+validate), PageRankRun, pagerank,
//                    pagerank_run, pagerank_checked, pagerank_checked_run,
//                    pagerank_weighted (+_run, _checked, _checked_run)
//   src/ppr.rs       personalized_pagerank (+_run, _checked, _checked_run)
//   src/graph.rs     the Graph / WeightedGraph adapter protocol, AdjacencyMatrix
//   src/lib.rs       Error / InvalidParameter
//
// Same names, argument meaning, validation messages and n == 0 results; the
// power iteration runs on the GPU.  A graph adapter is any type with
//   size_t node_count() const;
//   std::vector<size_t> neighbors(size_t u) const;        // out-neighbors, adapter order
// and, for the weighted functions,
//   double edge_weight(size_t u, size_t v) const;          // 0.0 when absent
// Unchecked functions throw graphops::DeviceError when the device fails (the
// reference's unchecked functions cannot fail, so a device failure is the
// only error they report).  Link with -lgops.
#pragma once

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "gops.h"

namespace graphops {

// src/lib.rs:108-123
class Error : public std::runtime_error {
 public:
  explicit Error(const std::string &what) : std::runtime_error(what) {}
};

class InvalidParameter : public Error {
 public:
  explicit InvalidParameter(const std::string &msg) : Error("invalid parameter: " + msg), msg_(msg) {}
  const std::string &message() const { return msg_; }

 private:
  std::string msg_;
};

class DeviceError : public Error {
 public:
  explicit DeviceError(const std::string &what) : Error(what) {}
};

// src/pagerank.rs:39-86
struct PageRankConfig {
  double damping = 0.85;
  size_t max_iterations = 100;
  double tolerance = 1e-6;

  void validate() const {
    if (!std::isfinite(damping)) throw InvalidParameter("damping must be finite");
    if (!(damping >= 0.0 && damping <= 1.0)) throw InvalidParameter("damping must be in [0,1]");
    if (max_iterations == 0) throw InvalidParameter("max_iterations must be > 0");
    if (!std::isfinite(tolerance) || tolerance <= 0.0)
      throw InvalidParameter("tolerance must be finite and > 0");
  }
};

// src/pagerank.rs:16-29
struct PageRankRun {
  std::vector<double> scores;
  size_t iterations = 0;
  double diff_l1 = 0.0;
  bool converged = true;
};

// AdjacencyMatrix (src/graph.rs:122-142): edge u->j iff m[u][j] > 0.0.
class AdjacencyMatrix {
 public:
  explicit AdjacencyMatrix(const std::vector<std::vector<double>> &m) : m_(m) {}
  size_t node_count() const { return m_.size(); }
  std::vector<size_t> neighbors(size_t node) const {
    std::vector<size_t> out;
    const auto &row = m_[node];
    for (size_t j = 0; j < row.size(); ++j)
      if (row[j] > 0.0) out.push_back(j);
    return out;
  }
  double edge_weight(size_t source, size_t target) const { return m_[source][target]; }
  const std::vector<std::vector<double>> &rows() const { return m_; }

 private:
  const std::vector<std::vector<double>> &m_;
};

namespace detail {

template <class G, class = void>
struct has_edge_weight : std::false_type {};
template <class G>
struct has_edge_weight<G, std::void_t<decltype(std::declval<const G &>().edge_weight(size_t{}, size_t{}))>>
    : std::true_type {};

struct CtxDeleter {
  void operator()(gops_ctx *c) const { gops_ctx_destroy(c); }
};

// One context per host thread (the reference is reentrant and stateless).
inline gops_ctx *thread_ctx() {
  thread_local std::unique_ptr<gops_ctx, CtxDeleter> ctx;
  if (!ctx) {
    gops_ctx *c = nullptr;
    const int rc = gops_ctx_create(0, &c);
    if (rc != GOPS_OK) throw DeviceError("libgops: no usable CUDA device (status " + std::to_string(rc) + ")");
    ctx.reset(c);
  }
  return ctx.get();
}

inline void check(gops_ctx *ctx, int rc) {
  if (rc != GOPS_OK) throw DeviceError(std::string("libgops: ") + gops_last_error(ctx));
}

struct GraphDeleter {
  void operator()(gops_graph *g) const { gops_graph_destroy(g); }
};
using GraphPtr = std::unique_ptr<gops_graph, GraphDeleter>;

// Out-adjacency in adapter order, read exactly as src/pagerank.rs:136 and
// :226-234 read it.
template <class G>
GraphPtr upload(gops_ctx *ctx, const G &g, bool weighted) {
  const size_t n = g.node_count();
  std::vector<int64_t> rp(n + 1, 0);
  std::vector<int32_t> col;
  std::vector<double> w;
  for (size_t u = 0; u < n; ++u) {
    const auto nb = g.neighbors(u);
    for (size_t v : nb) {
      col.push_back(static_cast<int32_t>(v));
      if constexpr (has_edge_weight<G>::value)
        if (weighted) w.push_back(g.edge_weight(u, v));
    }
    rp[u + 1] = static_cast<int64_t>(col.size());
  }
  gops_graph *h = nullptr;
  check(ctx, gops_graph_upload(ctx, static_cast<int64_t>(n), rp.data(), col.data(),
                               weighted ? w.data() : nullptr, &h));
  return GraphPtr(h);
}

// AdjacencyMatrix: the dense matrix goes to the device, which does the scan.
inline GraphPtr upload(gops_ctx *ctx, const AdjacencyMatrix &g, bool) {
  const size_t n = g.node_count();
  std::vector<double> flat(n * n);
  for (size_t u = 0; u < n; ++u)
    for (size_t j = 0; j < n; ++j) flat[u * n + j] = g.rows()[u][j];
  gops_graph *h = nullptr;
  check(ctx, gops_graph_from_dense(ctx, static_cast<int64_t>(n), flat.data(), &h));
  return GraphPtr(h);
}

inline gops_config to_c(const PageRankConfig &c) {
  return gops_config{c.damping, static_cast<uint64_t>(c.max_iterations), c.tolerance};
}

inline PageRankRun from_c(std::vector<double> &&scores, const gops_run &r) {
  PageRankRun out;
  out.scores = std::move(scores);
  out.iterations = static_cast<size_t>(r.iterations);
  out.diff_l1 = r.diff_l1;
  out.converged = r.converged != 0;
  return out;
}

}  // namespace detail

// ---- unweighted (src/pagerank.rs:91-187, 321-324) ----
template <class G>
PageRankRun pagerank_run(const G &graph, PageRankConfig config = {}) {
  const size_t n = graph.node_count();
  if (n == 0) return PageRankRun{};  // src/pagerank.rs:123-131
  gops_ctx *ctx = detail::thread_ctx();
  auto h = detail::upload(ctx, graph, false);
  const gops_config c = detail::to_c(config);
  std::vector<double> scores(n);
  gops_run r{};
  detail::check(ctx, gops_pagerank_run(ctx, h.get(), &c, scores.data(), &r));
  return detail::from_c(std::move(scores), r);
}

template <class G>
std::vector<double> pagerank(const G &graph, PageRankConfig config = {}) {
  return pagerank_run(graph, config).scores;
}

template <class G>
std::vector<double> pagerank_checked(const G &graph, PageRankConfig config = {}) {
  config.validate();
  return pagerank(graph, config);
}

template <class G>
PageRankRun pagerank_checked_run(const G &graph, PageRankConfig config = {}) {
  config.validate();
  return pagerank_run(graph, config);
}

// ---- weighted (src/pagerank.rs:201-336) ----
template <class G>
PageRankRun pagerank_weighted_run(const G &graph, PageRankConfig config = {}) {
  const size_t n = graph.node_count();
  if (n == 0) return PageRankRun{};
  gops_ctx *ctx = detail::thread_ctx();
  auto h = detail::upload(ctx, graph, true);
  const gops_config c = detail::to_c(config);
  std::vector<double> scores(n);
  gops_run r{};
  detail::check(ctx, gops_pagerank_weighted_run(ctx, h.get(), &c, scores.data(), &r));
  return detail::from_c(std::move(scores), r);
}

template <class G>
std::vector<double> pagerank_weighted(const G &graph, PageRankConfig config = {}) {
  return pagerank_weighted_run(graph, config).scores;
}

namespace detail {
template <class G>
void check_weights(const G &graph) {  // src/pagerank.rs:299-314
  for (size_t u = 0; u < graph.node_count(); ++u)
    for (size_t v : graph.neighbors(u)) {
      const double w = graph.edge_weight(u, v);
      if (!std::isfinite(w)) throw InvalidParameter("edge weights must be finite");
      if (w < 0.0) throw InvalidParameter("edge weights must be non-negative");
    }
}
}  // namespace detail

template <class G>
std::vector<double> pagerank_weighted_checked(const G &graph, PageRankConfig config = {}) {
  config.validate();
  detail::check_weights(graph);
  return pagerank_weighted(graph, config);
}

template <class G>
PageRankRun pagerank_weighted_checked_run(const G &graph, PageRankConfig config = {}) {
  config.validate();
  detail::check_weights(graph);
  return pagerank_weighted_run(graph, config);
}

// ---- personalized (src/ppr.rs:11-156) ----
template <class G>
PageRankRun personalized_pagerank_run(const G &graph, PageRankConfig config,
                                      const std::vector<double> &personalization) {
  const size_t n = graph.node_count();
  if (n == 0) return PageRankRun{};
  if (personalization.size() < n) throw std::out_of_range("personalization shorter than node_count");
  gops_ctx *ctx = detail::thread_ctx();
  auto h = detail::upload(ctx, graph, false);
  const gops_config c = detail::to_c(config);
  std::vector<double> scores(n);
  gops_run r{};
  detail::check(ctx, gops_personalized_pagerank_run(ctx, h.get(), &c, personalization.data(), scores.data(), &r));
  return detail::from_c(std::move(scores), r);
}

template <class G>
std::vector<double> personalized_pagerank(const G &graph, PageRankConfig config,
                                          const std::vector<double> &personalization) {
  return personalized_pagerank_run(graph, config, personalization).scores;
}

namespace detail {
template <class G>
void check_personalization(const G &graph, const PageRankConfig &config, const std::vector<double> &p) {
  config.validate();
  char buf[200];
  if (gops_personalization_validate(static_cast<int64_t>(graph.node_count()), static_cast<int64_t>(p.size()),
                                    p.data(), buf, sizeof buf) != GOPS_OK)
    throw InvalidParameter(buf);
}
}  // namespace detail

template <class G>
std::vector<double> personalized_pagerank_checked(const G &graph, PageRankConfig config,
                                                  const std::vector<double> &personalization) {
  detail::check_personalization(graph, config, personalization);
  return personalized_pagerank(graph, config, personalization);
}

template <class G>
PageRankRun personalized_pagerank_checked_run(const G &graph, PageRankConfig config,
                                              const std::vector<double> &personalization) {
  detail::check_personalization(graph, config, personalization);
  return personalized_pagerank_run(graph, config, personalization);
}

// ---- Katz centrality (src/katz.rs:19-210) ----
struct KatzConfig {
  double alpha = 0.1;
  double beta = 1.0;
  size_t max_iterations = 100;
  double tolerance = 1e-6;
  // src/katz.rs:60-86: the library's checks and messages
  void validate() const {
    const gops_katz_config c{alpha, beta, static_cast<uint64_t>(max_iterations), tolerance};
    char msg[256] = {0};
    if (gops_katz_config_validate(&c, msg, sizeof(msg)) != GOPS_OK) throw InvalidParameter(msg);
  }
};

struct KatzRun {  // src/katz.rs:93-104
  std::vector<double> scores;
  size_t iterations = 0;
  double diff_l1 = 0.0;
  bool converged = true;
};

template <class G>
KatzRun katz_centrality_run(const G &graph, KatzConfig config = {}) {
  const size_t n = graph.node_count();
  if (n == 0) return KatzRun{};  // src/katz.rs:138-145
  gops_ctx *ctx = detail::thread_ctx();
  auto h = detail::upload(ctx, graph, false);
  const gops_katz_config c{config.alpha, config.beta, static_cast<uint64_t>(config.max_iterations),
                           config.tolerance};
  KatzRun out;
  out.scores.resize(n);
  gops_run r{};
  detail::check(ctx, gops_katz_run(ctx, h.get(), &c, out.scores.data(), &r));
  out.iterations = static_cast<size_t>(r.iterations);
  out.diff_l1 = r.diff_l1;
  out.converged = r.converged != 0;
  return out;
}

template <class G>
std::vector<double> katz_centrality(const G &graph, KatzConfig config = {}) {
  return katz_centrality_run(graph, config).scores;
}

template <class G>
std::vector<double> katz_centrality_checked(const G &graph, KatzConfig config = {}) {
  config.validate();
  return katz_centrality(graph, config);
}

// ---- eigenvector centrality (src/eigenvector.rs:13-125) ----
struct EigenvectorRun {
  std::vector<double> scores;
  size_t iterations = 0;
  double diff_l1 = 0.0;
  bool converged = true;
};

template <class G>
EigenvectorRun eigenvector_centrality_run(const G &graph, size_t max_iterations, double tolerance) {
  const size_t n = graph.node_count();
  if (n == 0) return EigenvectorRun{};
  gops_ctx *ctx = detail::thread_ctx();
  auto h = detail::upload(ctx, graph, false);
  EigenvectorRun out;
  out.scores.resize(n);
  gops_run r{};
  detail::check(ctx, gops_eigenvector_run(ctx, h.get(), static_cast<uint64_t>(max_iterations), tolerance,
                                          out.scores.data(), &r));
  out.iterations = static_cast<size_t>(r.iterations);
  out.diff_l1 = r.diff_l1;
  out.converged = r.converged != 0;
  return out;
}

template <class G>
std::vector<double> eigenvector_centrality(const G &graph) {  // src/eigenvector.rs:26-28
  return eigenvector_centrality_run(graph, 100, 1e-6).scores;
}

// ---- HITS (src/centrality.rs:114-166): (hub scores, authority scores) ----
template <class G>
std::pair<std::vector<double>, std::vector<double>> hits(const G &graph, size_t max_iter = 100,
                                                         double tol = 1e-6) {
  const size_t n = graph.node_count();
  if (n == 0) return {};
  gops_ctx *ctx = detail::thread_ctx();
  auto h = detail::upload(ctx, graph, false);
  std::vector<double> hub(n), auth(n);
  gops_run r{};
  detail::check(ctx, gops_hits_run(ctx, h.get(), static_cast<uint64_t>(max_iter), tol, hub.data(), auth.data(), &r));
  return {std::move(hub), std::move(auth)};
}

}  // namespace graphops
