// The reference's own PageRank/PPR tests, doctests and example, restated
// against the C++ host API (graphops_gb300/cpp/graphops.hpp).
//   --cpu-only  run only the checks that need no device (validation, adapters)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <random>
#include <string>
#include <vector>

#include "graphops.hpp"

using namespace graphops;

static int g_failed = 0, g_run = 0;

static void check(bool ok, const char *what) {
  ++g_run;
  if (!ok) {
    ++g_failed;
    std::fprintf(stderr, "FAIL: %s\n", what);
  }
}

template <class F>
static std::string error_of(F f) {
  try {
    f();
  } catch (const InvalidParameter &e) {
    return e.message();
  }
  return "";
}

static double sum(const std::vector<double> &v) {
  double s = 0.0;
  for (double x : v) s += x;
  return s;
}

// src/pagerank.rs:397-424: the reference's only hand-written adapter
struct TestWeighted {
  std::vector<std::vector<size_t>> nb;
  std::vector<std::vector<double>> w;
  size_t node_count() const { return nb.size(); }
  std::vector<size_t> neighbors(size_t u) const { return nb[u]; }
  double edge_weight(size_t s, size_t t) const { return w[s][t]; }
};

// petgraph-like multigraph: neighbors newest first (tests/invariants.rs:20-50)
struct DiGraph {
  std::vector<std::vector<size_t>> out;
  explicit DiGraph(size_t n) : out(n) {}
  void add_edge(size_t a, size_t b) { out[a].push_back(b); }
  size_t node_count() const { return out.size(); }
  std::vector<size_t> neighbors(size_t u) const { return {out[u].rbegin(), out[u].rend()}; }
};

static void cpu_tests() {
  PageRankConfig c;
  check(error_of([&] { c.validate(); }).empty(), "default config validates");
  PageRankConfig bad = c;
  bad.damping = NAN;
  check(error_of([&] { bad.validate(); }) == "damping must be finite", "nan damping message");
  bad = c;
  bad.damping = 1.5;
  check(error_of([&] { bad.validate(); }) == "damping must be in [0,1]", "damping range message");
  bad = c;
  bad.max_iterations = 0;
  check(error_of([&] { bad.validate(); }) == "max_iterations must be > 0", "max_iterations message");
  bad = c;
  bad.tolerance = 0.0;
  check(error_of([&] { bad.validate(); }) == "tolerance must be finite and > 0", "tolerance message");
  // src/graph.rs:107-121
  std::vector<std::vector<double>> cyc = {{0, 1, 0}, {0, 0, 1}, {1, 0, 0}};
  AdjacencyMatrix m(cyc);
  check(m.node_count() == 3 && m.neighbors(0) == std::vector<size_t>{1}, "AdjacencyMatrix doctest");
  // src/pagerank.rs:397-424
  for (size_t n = 2; n < 10; ++n) {
    TestWeighted tw{std::vector<std::vector<size_t>>(n), std::vector<std::vector<double>>(n, std::vector<double>(n, 0.0))};
    tw.nb[0].push_back(n - 1);
    tw.w[0][n - 1] = -1.0;
    check(error_of([&] { pagerank_weighted_checked(tw); }) == "edge weights must be non-negative",
          "weighted_checked rejects a negative weight");
  }
  // src/ppr.rs:163-181
  std::vector<std::vector<double>> two = {{0, 1}, {0, 0}};
  AdjacencyMatrix g2(two);
  check(error_of([&] { personalized_pagerank_checked(g2, PageRankConfig{}, {1.0}); }).find("personalization length") == 0,
        "ppr_checked rejects wrong length");
  check(error_of([&] { personalized_pagerank_checked(g2, PageRankConfig{}, {0.0, 0.0}); }).find("sum") != std::string::npos,
        "ppr_checked rejects zero sum");
  // src/katz.rs:60-86
  KatzConfig k;
  check(error_of([&] { k.validate(); }).empty(), "default Katz config validates");
  KatzConfig kb = k;
  kb.alpha = 0.0;
  check(error_of([&] { kb.validate(); }) == "alpha must be finite and > 0", "Katz alpha message");
  kb = k;
  kb.alpha = 1.0;
  check(error_of([&] { kb.validate(); }).find("alpha must be < 1") == 0, "Katz alpha bound message");
  kb = k;
  kb.beta = INFINITY;
  check(error_of([&] { kb.validate(); }) == "beta must be finite", "Katz beta message");
  kb = k;
  kb.max_iterations = 0;
  check(error_of([&] { kb.validate(); }) == "max_iterations must be > 0", "Katz max_iterations message");
  kb = k;
  kb.tolerance = -1.0;
  check(error_of([&] { kb.validate(); }) == "tolerance must be finite and > 0", "Katz tolerance message");
}

static void gpu_tests() {
  std::vector<std::vector<double>> cyc = {{0, 1, 0}, {0, 0, 1}, {1, 0, 0}};
  auto s = pagerank(AdjacencyMatrix(cyc));  // src/pagerank.rs:100-113
  check(s.size() == 3 && std::fabs(sum(s) - 1.0) < 1e-6, "3-cycle doctest");
  check(std::fabs(s[0] - 1.0 / 3) < 1e-12, "3-cycle is uniform");
  std::vector<std::vector<double>> w = {{0, 2, 1}, {0, 0, 1}, {0, 0, 0}};  // :344-359
  check(std::fabs(sum(pagerank_weighted(AdjacencyMatrix(w))) - 1.0) < 1e-6, "weighted sums to one");
  std::vector<std::vector<double>> h = {{0, 2, 1}, {0, 0, 0}, {0, 0, 0}};  // :361-377
  auto sh = pagerank_weighted(AdjacencyMatrix(h));
  check(sh[1] >= sh[2], "heavier edge ranks higher");
  // :379-395, proptest-style random 0/1 matrices
  std::mt19937 rng(7);
  for (int t = 0; t < 100; ++t) {
    const size_t n = 1 + rng() % 9;
    std::vector<std::vector<double>> M(n, std::vector<double>(n, 0.0));
    const int ne = rng() % 40;
    for (int e = 0; e < ne; ++e) {
      size_t u = rng() % 10, v = rng() % 10;
      if (u < n && v < n && u != v) M[u][v] = 1.0;
    }
    auto sc = pagerank_checked(AdjacencyMatrix(M));
    bool nonneg = true;
    for (double x : sc) nonneg = nonneg && x >= -1e-12;
    check(sc.size() == n && std::fabs(sum(sc) - 1.0) < 1e-6 && nonneg, "proptest: sums to one, non-negative");
  }
  // src/ppr.rs:50-65
  auto p = personalized_pagerank(AdjacencyMatrix(cyc), PageRankConfig{}, {1.0, 0.0, 0.0});
  check(p[0] > p[1], "ppr doctest: seed ranks first");
  // examples/pagerank.rs
  std::vector<std::vector<double>> ex = {{0, 1, 1, 0}, {0, 0, 1, 0}, {1, 0, 0, 0}, {0, 0, 1, 0}};
  PageRankConfig cex;
  cex.tolerance = 1e-8;
  auto se = pagerank(AdjacencyMatrix(ex), cex);
  size_t best = 0;
  for (size_t i = 1; i < se.size(); ++i)
    if (se[i] > se[best]) best = i;
  check(best == 2, "example: node 2 ranks highest");
  // tests/invariants.rs:20-50
  DiGraph chain(3);
  chain.add_edge(0, 1);
  chain.add_edge(1, 2);
  for (const auto &v : {pagerank(chain), personalized_pagerank(chain, PageRankConfig{}, {1.0, 0.0, 0.0})}) {
    bool ok = v.size() == 3 && std::fabs(sum(v) - 1.0) <= 1e-6;
    for (double x : v) ok = ok && std::isfinite(x) && x >= 0.0;
    check(ok, "petgraph chain invariants");
  }
  // run diagnostics (src/pagerank.rs:16-29)
  PageRankConfig c3;
  c3.max_iterations = 3;
  c3.tolerance = 1e-15;
  auto r = pagerank_run(AdjacencyMatrix(ex), c3);
  check(r.iterations == 3 && !r.converged && r.diff_l1 > 0.0, "non-converged run reports max_iterations");
  auto r0 = pagerank_run(AdjacencyMatrix(std::vector<std::vector<double>>{}));
  check(r0.scores.empty() && r0.iterations == 0 && r0.converged, "empty graph");
  // closed forms on the 3-cycle: Katz x = beta / (1 - alpha); eigenvector and
  // HITS scores 1/sqrt(3)
  auto kr = katz_centrality_run(AdjacencyMatrix(cyc));
  bool kok = kr.converged && kr.scores.size() == 3;
  for (double x : kr.scores) kok = kok && std::fabs(x - 1.0 / 0.9) < 1e-5;
  check(kok, "Katz on the 3-cycle");
  auto ev = eigenvector_centrality(AdjacencyMatrix(cyc));
  bool eok = ev.size() == 3;
  for (double x : ev) eok = eok && std::fabs(x - 1.0 / std::sqrt(3.0)) < 1e-9;
  check(eok, "eigenvector centrality on the 3-cycle");
  auto ha = hits(AdjacencyMatrix(cyc));
  bool hok = ha.first.size() == 3 && ha.second.size() == 3;
  for (size_t i = 0; i < 3 && hok; ++i)
    hok = std::fabs(ha.first[i] - 1.0 / std::sqrt(3.0)) < 1e-9 && std::fabs(ha.second[i] - 1.0 / std::sqrt(3.0)) < 1e-9;
  check(hok, "HITS on the 3-cycle");
  check(katz_centrality_run(AdjacencyMatrix(std::vector<std::vector<double>>{})).scores.empty(), "Katz empty graph");
}

int main(int argc, char **argv) {
  const bool cpu_only = argc > 1 && std::strcmp(argv[1], "--cpu-only") == 0;
  cpu_tests();
  if (!cpu_only) gpu_tests();
  std::printf("%d checks, %d failed\n", g_run, g_failed);
  return g_failed ? 1 : 0;
}
