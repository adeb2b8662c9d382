// pcc_oracle.cc -- THE ORACLE.  Test and baseline infrastructure only.
//
// A CPU restatement (C++17 + OpenMP) of the reference's parallel
// correlation / modularity clustering path.  Only tests/, the smoke check
// in __graft_entry__.py and bench.py's CPU-baseline leg load it; the GPU
// library never calls it and has no CPU fallback.
//
// Parity status: UNPINNED against the reference binary.  The reference
// needs Bazel, GBBS (commit d385adac), Abseil, protobuf and gflags, none of
// which exist here, so it cannot be built; it also ships no tests, golden
// vectors or fixtures.  This restatement is instead pinned against
// hand-derived known answers, a brute-force objective and an independent
// pure-Python restatement (tests/golden/).
//
// Each function cites the reference lines it restates (paths relative to
// the reference project).  Third-party semantics restated from GBBS/pbbslib
// at the pinned commit:
//   * pbbs::reduce: serial left fold for <= 1024 elements, otherwise a serial
//     fold of each 1024-element block followed by a reduce of the block sums.
//   * pbbs::sample_sort(..., stable=true): a stable sort.
//   * sparse_additive_map: concurrent additive hash (order unspecified; the
//     restatement adds in adjacency order).
// Build with -ffp-contract=off so every a - b*c rounds twice, as the GPU does.

#include "pcc_gb300.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <random>
#include <vector>

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr size_t kPbbsBlock = 1024;  // pbbslib _block_size (1 << 10)

int g_threads = 0;  // 0 = OpenMP default

int NumThreads() { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

// ---------------------------------------------------------------------------
// Graph: GBBS symmetric_ptr_graph<symmetric_vertex, float> as SoA CSR.
// ---------------------------------------------------------------------------
struct Graph {
  uint32_t n = 0;
  uint64_t m = 0;
  std::vector<uint64_t> off;
  std::vector<uint32_t> nbr;
  std::vector<float> w;        // empty => unit weights
  std::vector<double> node_w;  // node weights attached by compression
  float weight(uint64_t j) const { return w.empty() ? 1.0f : w[j]; }
  uint64_t degree(uint32_t v) const { return off[v + 1] - off[v]; }
};

// pbbs::reduce over a plain array with a binary op (see header comment).
template <class T, class F>
T BlockedReduce(const T* a, size_t len, F f) {
  if (len <= kPbbsBlock) {
    T r = a[0];
    for (size_t j = 1; j < len; ++j) r = f(r, a[j]);
    return r;
  }
  size_t nb = (len + kPbbsBlock - 1) / kPbbsBlock;
  std::vector<T> sums(nb);
  for (size_t b = 0; b < nb; ++b) {
    size_t s = b * kPbbsBlock, e = std::min(len, s + kPbbsBlock);
    T r = a[s];
    for (size_t j = s + 1; j < e; ++j) r = f(r, a[j]);
    sums[b] = r;
  }
  return BlockedReduce(sums.data(), nb, f);
}

// ---------------------------------------------------------------------------
// ClusteringHelper state (parallel-correlation-clusterer-internal.h:36-165).
// ---------------------------------------------------------------------------
struct Helper {
  uint32_t n = 0;
  std::vector<uint32_t> C;  // cluster_ids_
  std::vector<uint32_t> s;  // cluster_sizes_
  std::vector<double> k;    // node_weights_
  std::vector<double> K;    // cluster_weights_

  // Constructor + SetClustering with an empty clustering (internal.h:40-63,
  // internal.cc:60-67): singletons.
  void InitSingletons(uint32_t num, std::vector<double> weights) {
    n = num;
    k = std::move(weights);
    if (k.empty()) k.assign(n, 1.0);
    C.resize(n);
    s.assign(n, 1);
    K.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
      C[i] = i;
      K[i] = k[i];
    }
  }
  // SetClustering with a non-empty clustering (internal.cc:68-76); group g is
  // the list of members in ascending order.  ResetClustering zeroes first.
  void SetGroups(const std::vector<std::vector<uint32_t>>& groups) {
    std::fill(s.begin(), s.end(), 0u);
    std::fill(K.begin(), K.end(), 0.0);
    for (size_t g = 0; g < groups.size(); ++g) {
      s[g] = static_cast<uint32_t>(groups[g].size());
      for (uint32_t j : groups[g]) {
        C[j] = static_cast<uint32_t>(g);
        K[g] += k[j];
      }
    }
  }
};

// OutputIndicesById (parallel/parallel-sequence-ops.h:183-209): groups of
// indices by id, groups ordered by id, members ascending.
std::vector<std::vector<uint32_t>> GroupsById(const std::vector<uint32_t>& ids) {
  uint32_t mx = 0;
  for (uint32_t x : ids) mx = std::max(mx, x);
  std::vector<uint32_t> count(ids.empty() ? 0 : size_t(mx) + 1, 0);
  for (uint32_t x : ids) count[x]++;
  std::vector<uint32_t> rank(count.size(), kNone);
  uint32_t g = 0;
  for (size_t c = 0; c < count.size(); ++c)
    if (count[c]) rank[c] = g++;
  std::vector<std::vector<uint32_t>> groups(g);
  for (size_t c = 0; c < count.size(); ++c)
    if (count[c]) groups[rank[c]].reserve(count[c]);
  for (uint32_t i = 0; i < ids.size(); ++i) groups[rank[ids[i]]].push_back(i);
  return groups;
}

// Dense rank labels equivalent to GroupsById (group index of each vertex).
std::vector<uint32_t> DenseLabels(const std::vector<uint32_t>& ids,
                                  uint32_t* num_groups) {
  uint32_t mx = 0;
  for (uint32_t x : ids) mx = std::max(mx, x);
  std::vector<uint32_t> rank(ids.empty() ? 0 : size_t(mx) + 1, 0);
  for (uint32_t x : ids) rank[x] = 1;
  uint32_t g = 0;
  for (auto& r : rank) {
    uint32_t present = r;
    r = g;
    g += present;
  }
  std::vector<uint32_t> out(ids.size());
  for (size_t i = 0; i < ids.size(); ++i) out[i] = rank[ids[i]];
  if (num_groups) *num_groups = g;
  return out;
}

// ---------------------------------------------------------------------------
// Per-thread open-addressing map cluster id -> double sum; a flat_hash_map
// stand-in.  Values are accumulated in call order.
// ---------------------------------------------------------------------------
struct SumTable {
  std::vector<uint32_t> keys;
  std::vector<double> vals;
  std::vector<uint32_t> used;
  uint32_t mask = 0;
  void Reset(uint64_t expected) {
    uint64_t cap = 16;
    while (cap < 2 * expected + 2) cap <<= 1;
    if (keys.size() < cap) {
      keys.assign(cap, kNone);
      vals.assign(cap, 0.0);
    } else {
      for (uint32_t slot : used) keys[slot] = kNone;
    }
    used.clear();
    mask = static_cast<uint32_t>(cap - 1);
  }
  void Add(uint32_t key, double v) {
    // Fibonacci hashing on the high bits of the product (like absl's
    // flat_hash_map, it mixes all key bits into the slot index).
    uint32_t h = static_cast<uint32_t>((uint64_t(key) * 0x9E3779B97F4A7C15ull) >> 32) & mask;
    while (true) {
      if (keys[h] == key) {
        vals[h] += v;
        return;
      }
      if (keys[h] == kNone) {
        keys[h] = key;
        vals[h] = v;  // EdgeSum starts at 0.0: 0.0 + v == v
        used.push_back(h);
        return;
      }
      h = (h + 1) & mask;
    }
  }
};

struct Scratch {
  SumTable table;
  std::vector<double> seq;
};

template <bool kAtomic>
inline uint32_t LoadU32(const uint32_t* p) {
  if (kAtomic) return __atomic_load_n(p, __ATOMIC_RELAXED);
  return *p;
}
template <bool kAtomic>
inline double LoadF64(const double* p) {
  if (kAtomic) {
    double v;
    __atomic_load(p, &v, __ATOMIC_RELAXED);
    return v;
  }
  return *p;
}
inline void AtomicAddF64(double* p, double v) {
  double cur;
  __atomic_load(p, &cur, __ATOMIC_RELAXED);
  double next;
  do {
    next = cur + v;
  } while (!__atomic_compare_exchange(p, &cur, &next, true, __ATOMIC_RELAXED,
                                      __ATOMIC_RELAXED));
}

struct Move {
  uint32_t target;
  double value;
};

// ClusteringHelper::EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:448-583) with EdgeSum
// (correlation-clusterer-util.h:26-43).  Returns (target, value); target ==
// graph.n means "move to a new cluster".
template <bool kAtomic>
Move EfficientBestMove(const Graph& g, const Helper& h, uint32_t v,
                       double res, double offset, Scratch& sc) {
  const uint64_t b = g.off[v], e = g.off[v + 1];
  const uint64_t deg = e - b;
  const uint32_t c = LoadU32<kAtomic>(&h.C[v]);
  const double kv = h.k[v];
  double moving_nodes_weight = 0;
  moving_nodes_weight += kv;
  SumTable& t = sc.table;
  t.Reset(deg);
  if (deg <= 1000) {
    // :456-512 -- sequential accumulation in adjacency order.
    double together = 0.0;
    for (uint64_t j = b; j < e; ++j) {
      const uint32_t u = g.nbr[j];
      double weight = static_cast<double>(g.weight(j));
      weight -= offset;
      const uint32_t cu = LoadU32<kAtomic>(&h.C[u]);
      if (u != v) {
        if (cu == c) together += weight;
        t.Add(cu, weight);
      }
    }
    double change = 0;
    double max_edges = kv * (LoadF64<kAtomic>(&h.K[c]) - kv);
    change -= together - res * max_edges;
    bool has = false;
    uint32_t best_id = 0;
    double best = change;
    for (uint32_t slot : t.used) {
      const uint32_t cu = t.keys[slot];
      max_edges = moving_nodes_weight * LoadF64<kAtomic>(&h.K[cu]);
      const double val = change + (t.vals[slot] - res * max_edges);
      if (val > best || (val == best && has && cu < best_id)) {
        best = val;
        best_id = cu;
        has = true;
      }
    }
    return {has ? best_id : g.n, best};
  }
  // :516-582 -- hub path.  The weight is a float here, so w - offset is
  // rounded to float; the "together" sum is a pbbs reduce of a dense
  // sequence; cluster sums come from an additive map (adjacency order here).
  sc.seq.assign(deg, 0.0);
  for (uint64_t j = b; j < e; ++j) {
    const uint32_t u = g.nbr[j];
    float weight = g.weight(j);
    weight -= offset;
    const uint32_t cu = LoadU32<kAtomic>(&h.C[u]);
    if (u != v) {
      if (cu == c) sc.seq[j - b] = weight;
      t.Add(cu, static_cast<double>(weight));
    }
  }
  double change = 0;
  double max_edges = kv * (LoadF64<kAtomic>(&h.K[c]) - kv);
  double curr_together =
      BlockedReduce(sc.seq.data(), deg, [](double a, double x) { return a + x; }) -
      res * max_edges;
  change -= curr_together;
  uint32_t best_id = 0;  // monoid identity (0, 0.0) when there are no entries
  double best = 0.0;
  bool first = true;
  for (uint32_t slot : t.used) {
    const uint32_t cu = t.keys[slot];
    double data = t.vals[slot];
    max_edges = moving_nodes_weight * LoadF64<kAtomic>(&h.K[cu]);
    data -= res * max_edges;
    const double val = change + data;
    if (first || val > best || (val == best && cu < best_id)) {
      best = val;
      best_id = cu;
      first = false;
    }
  }
  if (change >= best) return {g.n, change};
  return {best_id, best};
}

struct Options {
  double res = 0;
  double offset = 0;
  int move_method = PCC_NBHR_CLUSTER_MOVE;
  bool whole_clusters = false;  // DEFAULT_CLUSTER_MOVES
  bool async = false;
  bool permute = false;
  uint64_t seed = 0;
  uint64_t round_counter = 0;
};

struct Counters {
  uint64_t edge_visits = 0;
  uint64_t vertex_visits = 0;
  uint64_t moves = 0;
  int32_t rounds = 0;
};

// ClusteringHelper::MoveNodesToCluster(moves)
// (parallel-correlation-clusterer-internal.cc:256-369).  moves[v] == kNone
// is "no move"; moves[v] == n is "new cluster".  Returns modified_cluster.
std::vector<uint8_t> MoveNodesToCluster(Helper& h,
                                        const std::vector<uint32_t>& moves,
                                        uint64_t* moved_count) {
  const uint32_t n = h.n;
  std::vector<uint8_t> modified(n, 0);
  std::vector<uint32_t> movers;
  for (uint32_t v = 0; v < n; ++v)
    if (moves[v] != kNone && moves[v] != h.C[v]) movers.push_back(v);
  if (moved_count) *moved_count += movers.size();
  if (movers.empty()) return modified;
  // Stable sort by old cluster id, then per group: sizes -= count, weights
  // -= node weight in ascending node order (:275-303).  Visiting movers in
  // ascending order gives every cluster the same operation order.
  for (uint32_t v : movers) {
    const uint32_t c = h.C[v];
    h.s[c] -= 1;
    modified[c] = 1;
    h.K[c] -= h.k[v];
  }
  // Stable sort by target, add to existing targets (:305-337).
  bool any_new = false;
  for (uint32_t v : movers) {
    const uint32_t t = moves[v];
    if (t != n) {
      h.s[t] += 1;
      modified[t] = 1;
      h.C[v] = t;
      h.K[t] += h.k[v];
    } else {
      any_new = true;
    }
  }
  // New clusters take the ascending list of empty ids, in ascending node
  // order (:339-366).
  if (any_new) {
    std::vector<uint32_t> zero;
    for (uint32_t i = 0; i < n; ++i)
      if (h.s[i] == 0) zero.push_back(i);
    size_t r = 0;
    for (uint32_t v : movers) {
      if (moves[v] != n) continue;
      const uint32_t cid = zero[r++];
      h.C[v] = cid;
      h.s[cid] = 1;
      modified[cid] = 1;
      h.K[cid] = h.k[v];
    }
  }
  return modified;
}

// ClusteringHelper::AsyncMove(node) (internal.cc:371-403).
bool AsyncMove(const Graph& g, Helper& h, uint32_t v, const Options& o,
               Scratch& sc) {
  const Move mv = EfficientBestMove<true>(g, h, v, o.res, o.offset, sc);
  const uint32_t cur = __atomic_load_n(&h.C[v], __ATOMIC_RELAXED);
  if (mv.value <= 0) return false;
  __atomic_fetch_sub(&h.s[cur], 1u, __ATOMIC_RELAXED);
  AtomicAddF64(&h.K[cur], -1 * h.k[v]);
  if (mv.target != h.n) {
    __atomic_fetch_add(&h.s[mv.target], 1u, __ATOMIC_RELAXED);
    AtomicAddF64(&h.K[mv.target], h.k[v]);
    __atomic_store_n(&h.C[v], mv.target, __ATOMIC_RELAXED);
    return true;
  }
  uint64_t i = v;
  while (true) {
    if (__atomic_load_n(&h.s[i], __ATOMIC_RELAXED) == 0) {
      uint32_t expected = 0;
      if (__atomic_compare_exchange_n(&h.s[i], &expected, 1u, false,
                                      __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
        AtomicAddF64(&h.K[i], h.k[v]);
        __atomic_store_n(&h.C[v], static_cast<uint32_t>(i), __ATOMIC_RELAXED);
        return true;
      }
    }
    i = (i + 1) % h.n;
  }
}

// Whole-cluster moves of one synchronous round: the DEFAULT_CLUSTER_MOVES
// block of BestMovesForVertexSubset (parallel-correlation-clusterer.cc:
// 167-297, subclustering NONE), with ClusteringHelper::BestMove(moving_nodes)
// (internal.cc:644-707) and BestMoveFromStats (correlation-clusterer-util.h:
// 70-113).  Every cluster (OutputIndicesById groups: members ascending) is a
// moving set whose members are exactly the vertices of that cluster, so
// class-2 entries (both ends moving) never cross clusters and class-1 entries
// never stay inside.  Returns the clusters MoveNodesToCluster modified.
std::vector<uint8_t> ClusterMoves(const Graph& g, Helper& h, const Options& o,
                                  uint64_t* moved_count) {
  const uint32_t n = g.n;
  const std::vector<std::vector<uint32_t>> groups = GroupsById(h.C);
  std::vector<uint32_t> moves(n, kNone);
  const int64_t ng = static_cast<int64_t>(groups.size());
#pragma omp parallel num_threads(NumThreads())
  {
    SumTable after;  // class_1_together_after: cluster -> EdgeSum
#pragma omp for schedule(dynamic, 16)
    for (int64_t gi = 0; gi < ng; ++gi) {
      const std::vector<uint32_t>& members = groups[gi];
      const uint32_t c = h.C[members[0]];
      uint64_t deg = 0;
      for (uint32_t v : members) deg += g.degree(v);
      after.Reset(deg);
      double weight = 0;    // moving_nodes_weight
      double weight_c = 0;  // cluster_moving_weights[c]
      for (uint32_t v : members) {
        weight_c += h.k[v];
        weight += h.k[v];
        for (uint64_t j = g.off[v]; j < g.off[v + 1]; ++j) {
          const uint32_t cu = h.C[g.nbr[j]];
          if (cu == c) continue;  // both ends moving
          // `float weight; weight -= offset;` then EdgeSum::Add(double).
          const float wf = static_cast<float>(static_cast<double>(g.weight(j)) - o.offset);
          after.Add(cu, static_cast<double>(wf));
        }
      }
      auto half_square = [](double x) { return x * x / 2; };
      double change = 0;
      change += 0.0 / 2 - o.res * (half_square(weight) - half_square(weight_c));
      change -= 0.0 - o.res * (weight_c * (h.K[c] - weight_c));
      uint32_t best = kNone;
      double best_val = change;
      for (uint32_t slot : after.used) {
        const uint32_t d = after.keys[slot];
        const double val = change + (after.vals[slot] - o.res * (weight * (h.K[d] - 0.0)));
        if (val > best_val || (val == best_val && best != kNone && d < best)) {
          best = d;
          best_val = val;
        }
      }
      const uint32_t target = best != kNone ? best : n;
      if (target < n && c >= target) best_val = 0;  // only towards a higher id
      if (best_val > 0)
        for (uint32_t v : members) moves[v] = target;
    }
  }
  return MoveNodesToCluster(h, moves, moved_count);
}

// ClusteringHelper::BestMove(moving_nodes) (internal.cc:644-707) with
// BestMoveFromStats (correlation-clusterer-util.h:70-113) on live state, for
// a moving set whose members share one cluster c (the async cluster-move
// step): class-2 entries (both ends moving) never cross clusters; class-1
// entries to c itself count as currently together.  Returns (target, value)
// with target == n for "no cluster" (nullopt).
Move BestMoveSet(const Graph& g, const Helper& h, const std::vector<uint32_t>& members,
                 const std::vector<uint8_t>& moving, const Options& o, SumTable& after) {
  const uint32_t c = h.C[members[0]];
  uint64_t deg = 0;
  for (uint32_t v : members) deg += g.degree(v);
  after.Reset(deg);
  double weight = 0, weight_c = 0, together = 0;
  for (uint32_t v : members) {
    weight_c += h.k[v];
    weight += h.k[v];
    for (uint64_t j = g.off[v]; j < g.off[v + 1]; ++j) {
      const uint32_t u = g.nbr[j];
      const float wf = static_cast<float>(static_cast<double>(g.weight(j)) - o.offset);
      if (moving[u]) continue;  // class 2: both ends in c
      const uint32_t cu = h.C[u];
      if (cu == c) together += static_cast<double>(wf);
      after.Add(cu, static_cast<double>(wf));
    }
  }
  auto half_square = [](double x) { return x * x / 2; };
  double change = 0;
  change += 0.0 / 2 - o.res * (half_square(weight) - half_square(weight_c));
  change -= together - o.res * (weight_c * (h.K[c] - weight_c));
  Move best{g.n, change};
  uint32_t best_id = kNone;
  for (uint32_t slot : after.used) {
    const uint32_t d = after.keys[slot];
    const double moving_d = d == c ? weight_c : 0.0;  // cluster_moving_weights[d]
    const double val = change + (after.vals[slot] - o.res * (weight * (h.K[d] - moving_d)));
    if (val > best.value || (val == best.value && best_id != kNone && d < best_id)) {
      best_id = d;
      best.value = val;
    }
  }
  if (best_id != kNone) best.target = best_id;
  return best;
}

// The async branch of the DEFAULT_CLUSTER_MOVES block (parallel-correlation-
// clusterer.cc:255-268): AsyncMove(moving_nodes) (internal.cc:405-446) for
// every cluster of the clustering after the round's vertex moves, restated
// sequentially in cluster order (each move sees the ones before it).  A
// one-member set takes the vertex AsyncMove; a larger one moves whole when
// its value is positive, with the moving weight summed in FP32 (the
// reference's delayed_seq<float>), to a new cluster by the linear probe
// from its own id.  The moved flags are set at the members' vertex ids, as
// the reference does.
void AsyncClusterMoves(const Graph& g, Helper& h, const Options& o,
                       std::vector<uint8_t>& moved_clusters, Counters& ctr) {
  const uint32_t n = g.n;
  const std::vector<std::vector<uint32_t>> groups = GroupsById(h.C);
  std::vector<uint8_t> additional(n, 0), moving(n, 0);
  Scratch sc;
  for (const std::vector<uint32_t>& members : groups) {
    bool moved = false;
    if (members.size() == 1) {
      moved = AsyncMove(g, h, members[0], o, sc);
    } else {
      for (uint32_t v : members) moving[v] = 1;
      const Move mv = BestMoveSet(g, h, members, moving, o, sc.table);
      for (uint32_t v : members) moving[v] = 0;
      if (mv.value > 0) {
        const uint32_t cur = h.C[members[0]];
        const uint32_t size = static_cast<uint32_t>(members.size());
        std::vector<float> wts(members.size());
        for (size_t i = 0; i < members.size(); ++i) wts[i] = static_cast<float>(h.k[members[i]]);
        const float total = BlockedReduce(wts.data(), wts.size(), [](float a, float b) { return a + b; });
        h.s[cur] -= size;
        h.K[cur] += -1 * total;
        uint32_t dest = mv.target;
        if (dest != n) {
          h.s[dest] += size;
          h.K[dest] += total;
        } else {
          uint64_t i = cur;
          while (h.s[i] != 0) i = (i + 1) % n;
          dest = static_cast<uint32_t>(i);
          h.s[dest] = size;
          h.K[dest] += total;
        }
        for (uint32_t v : members) h.C[v] = dest;
        moved = true;
      }
    }
    if (moved) {
      ctr.moves += members.size();
      for (uint32_t v : members) additional[v] = 1;
    }
  }
  for (uint32_t i = 0; i < n; ++i) moved_clusters[i] |= additional[i];
}

// N(marked) via gbbs::edgeMap with the always-true functor
// (parallel-correlation-clusterer.cc:46-55, 312-331): every neighbour of a
// marked vertex, as an ascending list.
std::vector<uint32_t> NeighborsOfMarked(const Graph& g,
                                        const std::vector<uint8_t>& marked) {
  const uint32_t n = g.n;
  std::vector<uint8_t> next(n, 0);
#pragma omp parallel for schedule(dynamic, 1024) num_threads(NumThreads())
  for (int64_t v = 0; v < int64_t(n); ++v) {
    if (!marked[v]) continue;
    for (uint64_t j = g.off[v]; j < g.off[v + 1]; ++j)
      __atomic_store_n(&next[g.nbr[j]], uint8_t(1), __ATOMIC_RELAXED);
  }
  std::vector<uint32_t> out;
  for (uint32_t v = 0; v < n; ++v)
    if (next[v]) out.push_back(v);
  return out;
}

std::vector<uint32_t> AllVertices(uint32_t n) {
  std::vector<uint32_t> out(n);
  std::iota(out.begin(), out.end(), 0u);
  return out;
}

// BestMovesForVertexSubset (parallel-correlation-clusterer.cc:115-338):
// vertex moves, then (DEFAULT_CLUSTER_MOVES, synchronous) whole-cluster
// moves.  Returns the next frontier.
std::vector<uint32_t> BestMovesForVertexSubset(const Graph& g, Helper& h,
                                               const std::vector<uint32_t>& frontier,
                                               Options& o, Counters& ctr) {
  const uint32_t n = g.n;
  std::vector<uint32_t> order = frontier;
  if (o.permute) {
    // vertexMapPermute (:69-109): a random processing order.
    std::mt19937_64 rng(o.seed * 0x9E3779B97F4A7C15ull + o.round_counter);
    std::shuffle(order.begin(), order.end(), rng);
  }
  o.round_counter++;
  for (uint32_t v : frontier) ctr.edge_visits += g.degree(v);
  ctr.vertex_visits += frontier.size();
  ctr.rounds += 1;

  std::vector<uint8_t> moved_vertex(n, 0);
  std::vector<uint8_t> moved_clusters;
  const int64_t nf = static_cast<int64_t>(order.size());
  if (o.async) {
    moved_clusters.assign(n, 0);
    std::atomic<uint64_t> moved_count{0};
#pragma omp parallel num_threads(NumThreads())
    {
      Scratch sc;
      uint64_t local = 0;
#pragma omp for schedule(dynamic, 64)
      for (int64_t x = 0; x < nf; ++x) {
        const uint32_t v = order[x];
        if (AsyncMove(g, h, v, o, sc)) {
          const uint32_t cid = __atomic_load_n(&h.C[v], __ATOMIC_RELAXED);
          __atomic_store_n(&moved_clusters[cid], uint8_t(1), __ATOMIC_RELAXED);
          moved_vertex[v] = 1;
          local++;
        }
      }
      moved_count += local;
    }
    ctr.moves += moved_count.load();
    if (o.whole_clusters) AsyncClusterMoves(g, h, o, moved_clusters, ctr);
  } else {
    std::vector<uint32_t> moves(n, kNone);
#pragma omp parallel num_threads(NumThreads())
    {
      Scratch sc;
#pragma omp for schedule(dynamic, 64)
      for (int64_t x = 0; x < nf; ++x) {
        const uint32_t v = order[x];
        Move mv = EfficientBestMove<false>(g, h, v, o.res, o.offset, sc);
        // Singleton rule (:142-152).
        const uint32_t cur = h.C[v];
        if (mv.target < n && h.s[mv.target] == 1 && h.s[cur] == 1 &&
            cur >= mv.target) {
          mv.target = cur;
          mv.value = 0;
        }
        if (mv.value > 0) {
          moves[v] = mv.target;
          moved_vertex[v] = 1;
        }
      }
    }
    moved_clusters = MoveNodesToCluster(h, moves, &ctr.moves);
    if (o.whole_clusters) {
      const std::vector<uint8_t> extra = ClusterMoves(g, h, o, &ctr.moves);
      for (uint32_t i = 0; i < n; ++i) moved_clusters[i] |= extra[i];
    }
  }

  if (o.move_method == PCC_ALL_MOVE) return AllVertices(n);
  std::vector<uint8_t> marked(n, 0);
  if (o.move_method == PCC_NBHR_CLUSTER_MOVE) {
    for (uint32_t v = 0; v < n; ++v) marked[v] = moved_clusters[h.C[v]];
  } else {
    marked = moved_vertex;
  }
  return NeighborsOfMarked(g, marked);
}

// IterateBestMoves (parallel-correlation-clusterer.cc:340-365).
bool IterateBestMoves(const Graph& g, Helper& h, int64_t num_inner, Options& o,
                      Counters& ctr) {
  std::vector<uint32_t> frontier = AllVertices(g.n);
  bool moved = false;
  bool local_moved = true;
  for (int64_t it = 0; it < num_inner && local_moved; ++it) {
    frontier = BestMovesForVertexSubset(g, h, frontier, o, ctr);
    local_moved = !frontier.empty();
    moved |= local_moved;
  }
  return moved;
}

// CompressGraph (parallel-correlation-clusterer-internal.cc:709-782) with
// ComputeInterClusterEdgesSort / RetrieveInterClusterEdges / GetOffsets
// (parallel/parallel-graph-utils.cc:33-122,156-231).
Graph CompressGraph(const Graph& g, const std::vector<uint32_t>& C,
                    const std::vector<double>& k) {
  const uint32_t n = g.n;
  uint32_t max_c = 0;
  for (uint32_t x : C) max_c = std::max(max_c, x);
  const uint32_t n2 = n == 0 ? 1 : max_c + 1;

  // Stable order of vertices by cluster (counting sort): the stable sort of
  // entries by C(u) keeps CSR order inside each cluster.
  std::vector<uint64_t> vstart(size_t(n2) + 1, 0);
  for (uint32_t v = 0; v < n; ++v) vstart[C[v] + 1]++;
  for (uint32_t c = 0; c < n2; ++c) vstart[c + 1] += vstart[c];
  std::vector<uint32_t> vorder(n);
  {
    std::vector<uint64_t> pos(vstart.begin(), vstart.end() - 1);
    for (uint32_t v = 0; v < n; ++v) vorder[pos[C[v]]++] = v;
  }

  // Per cluster: its kept entries (v <= u || C(v) != C(u), :102), stable
  // sorted by C(v), segment sums as a pbbs float reduce (:196-222).
  std::vector<std::vector<uint32_t>> out_nbr(n2);
  std::vector<std::vector<float>> out_w(n2);
#pragma omp parallel num_threads(NumThreads())
  {
    std::vector<std::pair<uint32_t, float>> ent;
    std::vector<float> seg;
#pragma omp for schedule(dynamic, 256)
    for (int64_t c = 0; c < int64_t(n2); ++c) {
      ent.clear();
      for (uint64_t x = vstart[c]; x < vstart[c + 1]; ++x) {
        const uint32_t u = vorder[x];
        for (uint64_t j = g.off[u]; j < g.off[u + 1]; ++j) {
          const uint32_t v = g.nbr[j];
          if (v <= u || C[v] != C[u]) ent.emplace_back(C[v], g.weight(j));
        }
      }
      std::stable_sort(ent.begin(), ent.end(),
                       [](const std::pair<uint32_t, float>& a,
                          const std::pair<uint32_t, float>& b) {
                         return a.first < b.first;
                       });
      size_t i = 0;
      while (i < ent.size()) {
        size_t j = i;
        seg.clear();
        while (j < ent.size() && ent[j].first == ent[i].first) {
          seg.push_back(ent[j].second);
          ++j;
        }
        const float sum = BlockedReduce(
            seg.data(), seg.size(), [](float a, float b) {
              return static_cast<float>(static_cast<double>(a) +
                                        static_cast<double>(b));
            });
        out_nbr[c].push_back(ent[i].first);
        out_w[c].push_back(sum);
        i = j;
      }
    }
  }
  Graph out;
  out.n = n2;
  out.off.assign(size_t(n2) + 1, 0);
  for (uint32_t c = 0; c < n2; ++c) out.off[c + 1] = out.off[c] + out_nbr[c].size();
  out.m = out.off[n2];
  out.nbr.resize(out.m);
  out.w.resize(out.m);
#pragma omp parallel for schedule(dynamic, 256) num_threads(NumThreads())
  for (int64_t c = 0; c < int64_t(n2); ++c) {
    std::copy(out_nbr[c].begin(), out_nbr[c].end(), out.nbr.begin() + out.off[c]);
    std::copy(out_w[c].begin(), out_w[c].end(), out.w.begin() + out.off[c]);
  }
  // New node weights: stable sort of (cluster, weight) + pbbs double reduce
  // per cluster (:732-777); absent ids keep weight 0.
  out.node_w.assign(n2, 0.0);
#pragma omp parallel num_threads(NumThreads())
  {
    std::vector<double> seg;
#pragma omp for schedule(dynamic, 1024)
    for (int64_t c = 0; c < int64_t(n2); ++c) {
      if (vstart[c] == vstart[c + 1]) continue;
      seg.clear();
      for (uint64_t x = vstart[c]; x < vstart[c + 1]; ++x) {
        const uint32_t v = vorder[x];
        seg.push_back(v < k.size() ? k[v] : 1.0);  // NodeWeight (:79-81)
      }
      out.node_w[c] = BlockedReduce(seg.data(), seg.size(),
                                    [](double a, double b) { return a + b; });
    }
  }
  return out;
}

// ClusteringHelper::ComputeObjective (internal.cc:118-149).
double ComputeObjective(const Graph& g, const std::vector<uint32_t>& C,
                        const std::vector<double>& k,
                        const std::vector<double>& K, double res,
                        double offset) {
  const uint32_t n = g.n;
  double edge_part = 0;
  double res_part = 0;
#pragma omp parallel for reduction(+ : edge_part, res_part) schedule(dynamic, 1024) num_threads(NumThreads())
  for (int64_t i = 0; i < int64_t(n); ++i) {
    double acc = 0;
    for (uint64_t j = g.off[i]; j < g.off[i + 1]; ++j) {
      if (C[i] == C[g.nbr[j]]) acc += (g.weight(j) - offset) / 2;
    }
    edge_part += acc;
    res_part += k[i] * (K[C[i]] - k[i]);
  }
  return edge_part - res * res_part / 2;
}

// Builds helper state from per-vertex group labels (SetClustering with
// clustering[c] = members of c, ascending).
void HelperFromLabels(Helper& h, uint32_t n, const std::vector<double>& k,
                      const std::vector<uint32_t>& labels) {
  h.n = n;
  h.k = k;
  if (h.k.empty()) h.k.assign(n, 1.0);
  h.C.assign(n, 0);
  h.s.assign(n, 0);
  h.K.assign(n, 0.0);
  for (uint32_t v = 0; v < n; ++v) {
    const uint32_t c = labels[v];
    h.C[v] = c;
    h.s[c] += 1;
    h.K[c] += h.k[v];
  }
}

// ---------------------------------------------------------------------------
// Subclustering before compression: CompressSubclusters (parallel-
// correlation-clusterer.cc:436-474) with ComputeSubcluster and its three
// methods (parallel-correlation-clusterer-internal.cc:784-1120).
//
// Every cluster (OutputIndicesById order: ids ascending, members ascending)
// is split into subclusters; cluster i owns the subcluster ids
// [next_i, next_i + B_i) (B_i = the method's block size, next = the
// exclusive scan of the blocks), and the graph is compressed by subcluster
// id.  The next level starts from the clustering "subclusters of one
// cluster together": compressed vertex j is in cluster i for j in i's block,
// and cluster i's size is its block size B_i (ids of the block that no
// vertex took included, as the reference's group sizes).
//
// Labels inside a cluster (local index x = rank of the member among the
// cluster's members):
//  * CONNECTIVITY: components of the member pairs joined by an entry, each
//    labelled by its smallest member's local index (union by the smaller
//    root, as GBBS's asynchronous union-find links a larger root to a
//    smaller one); B = the cluster size.
//  * TRIANGLE: components of the entries (v, u), C(u) = C(v), whose
//    triangle ratio |N(v) & N(u)| / (deg v + deg u) (a sorted-merge
//    intersection of the two rows) exceeds 0.25; B = 1 + the largest label.
//    The reference labels components with GBBS's work-efficient CC (LDD
//    centres); here a component is labelled by its smallest member, which
//    gives the same components under other ids.
//  * SLOW_CONNECTIVITY: the reference's sequential merge loop, step by step;
//    B = 1 + the largest label.
//
// Where this deliberately differs from the reference: its level loop keeps
// flattening through the level's cluster ids while the compressed graph is
// indexed by subcluster ids, and its next-level clustering names subcluster
// ids beyond the compressed graph (reads and writes outside the helper's
// vectors whenever a cluster's largest component label is below its block
// end).  Those are index confusions with undefined behaviour, so a
// level-i vertex maps to its subcluster id on level i + 1 (refinement
// projections and the final labels follow that map), and ids beyond the
// compressed graph count only in their cluster's size.
// ---------------------------------------------------------------------------
struct UnionFind {
  std::vector<uint32_t> p;
  explicit UnionFind(uint32_t n) : p(n) { std::iota(p.begin(), p.end(), 0u); }
  uint32_t Find(uint32_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
  void Unite(uint32_t a, uint32_t b) {
    a = Find(a);
    b = Find(b);
    if (a == b) return;
    if (a < b) std::swap(a, b);
    p[a] = b;  // the larger root under the smaller
  }
};

// |N(v) & N(u)| by a sorted-merge walk of the two rows (GBBS intersect),
// over the sum of the two degrees, for every entry.
std::vector<double> TriangleRatios(const Graph& g) {
  std::vector<double> out(g.m, 0.0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(NumThreads())
  for (int64_t v = 0; v < int64_t(g.n); ++v) {
    for (uint64_t j = g.off[v]; j < g.off[v + 1]; ++j) {
      const uint32_t u = g.nbr[j];
      uint64_t a = g.off[v], ae = g.off[v + 1], b = g.off[u], be = g.off[u + 1];
      uint64_t common = 0;
      while (a < ae && b < be) {
        if (g.nbr[a] == g.nbr[b]) {
          ++common;
          ++a;
          ++b;
        } else if (g.nbr[a] < g.nbr[b]) {
          ++a;
        } else {
          ++b;
        }
      }
      out[j] = static_cast<double>(common) / static_cast<double>(g.degree(v) + g.degree(u));
    }
  }
  return out;
}

// ComputeSubclusterConnectivitySlow (internal.cc:870-985) for one cluster:
// local labels into lab[0..size), returns 1 + the largest label.
uint32_t SlowSubclusters(const Graph& g, const std::vector<uint32_t>& members, const std::vector<uint32_t>& C,
                         const Options& o, std::vector<uint8_t>& mark, std::vector<uint32_t>& lab) {
  const size_t size = members.size();
  const uint32_t c = C[members[0]];
  std::vector<uint32_t> tmp(size);
  std::iota(tmp.begin(), tmp.end(), 0u);
  std::vector<char> single(size, 0);
  auto outside = [&](uint32_t x) { return C[x] != c; };
  for (size_t i = 0; i < size; ++i) {
    if (single[i] != 0) continue;
    const uint32_t cv = members[i];
    int curr_num_edges = 0;
    for (uint64_t j = g.off[cv]; j < g.off[cv + 1]; ++j)
      if (outside(g.nbr[j])) curr_num_edges++;
    if (static_cast<size_t>(curr_num_edges) < size - 1) continue;
    // OutputIndicesById(tmp): groups of local indices by label.
    std::vector<std::vector<uint32_t>> groups = GroupsById(tmp);
    std::vector<char> invalid(groups.size(), 0);
    int64_t num_valid = static_cast<int64_t>(groups.size());
    for (size_t j = 0; j < groups.size(); ++j) {
      const std::vector<uint32_t>& curr = groups[j];
      if (curr.empty() || curr[0] == i) {
        invalid[j] = 1;
        num_valid--;
        continue;
      }
      int num_edges = 0;
      for (uint32_t x : curr) {
        const uint32_t vx = members[x];
        for (uint64_t e = g.off[vx]; e < g.off[vx + 1]; ++e)
          if (outside(g.nbr[e])) num_edges++;
      }
      if (static_cast<size_t>(num_edges) < curr.size() * (size - curr.size())) {
        invalid[j] = 1;
        num_valid--;
      }
    }
    if (num_valid == 0) continue;
    double max_max = 0;
    size_t idx_idx = 0;
    for (size_t j = 0; j < groups.size(); ++j) {
      if (invalid[j] != 0) continue;
      const std::vector<uint32_t>& curr = groups[j];
      for (uint32_t x : curr) mark[members[x]] = 2;
      double weight = 0;
      const double offset = o.offset * double(curr.size()) + o.res * double(curr.size());
      for (uint64_t e = g.off[cv]; e < g.off[cv + 1]; ++e)
        if (mark[g.nbr[e]] == 2) weight++;
      for (uint32_t x : curr) mark[members[x]] = 0;
      if (weight < offset) {
        invalid[j] = 1;
        num_valid--;
      } else if (weight - offset >= max_max) {
        max_max = weight - offset;
        idx_idx = j;
      }
    }
    if (num_valid == 0) continue;
    const std::vector<uint32_t>& curr = groups[idx_idx];
    tmp[i] = tmp[curr[0]];
    single[i] = 1;
    single[curr[0]] = 1;
  }
  uint32_t mx = 0;
  for (size_t i = 0; i < size; ++i) {
    lab[i] = tmp[i];
    mx = std::max(mx, tmp[i]);
  }
  return mx + 1;
}

struct SubclusterMap {
  std::vector<uint32_t> id;     // subcluster id of every vertex
  std::vector<uint64_t> next;   // block start of every cluster (index order), then the total
};

SubclusterMap ComputeSubclusters(const Graph& g, const std::vector<uint32_t>& C, int method, const Options& o) {
  const std::vector<std::vector<uint32_t>> groups = GroupsById(C);
  const size_t G = groups.size();
  SubclusterMap out;
  out.id.assign(g.n, 0);
  out.next.assign(G + 1, 0);
  std::vector<uint32_t> local(g.n, 0);
  for (const auto& mem : groups)
    for (size_t x = 0; x < mem.size(); ++x) local[mem[x]] = static_cast<uint32_t>(x);
  std::vector<double> tri;
  if (method == PCC_TRIANGLE_SUBCLUSTERING) tri = TriangleRatios(g);
  std::vector<std::vector<uint32_t>> labels(G);
#pragma omp parallel num_threads(NumThreads())
  {
    std::vector<uint8_t> mark;
#pragma omp for schedule(dynamic, 16)
    for (int64_t gi = 0; gi < int64_t(G); ++gi) {
      const std::vector<uint32_t>& mem = groups[gi];
      std::vector<uint32_t>& lab = labels[gi];
      lab.assign(mem.size(), 0);
      uint32_t block = 0;
      if (method == PCC_SLOW_CONNECTIVITY_SUBCLUSTERING) {
        if (mark.size() != g.n) mark.assign(g.n, 0);
        block = SlowSubclusters(g, mem, C, o, mark, lab);
      } else {
        UnionFind uf(static_cast<uint32_t>(mem.size()));
        const uint32_t c = C[mem[0]];
        for (size_t x = 0; x < mem.size(); ++x) {
          const uint32_t v = mem[x];
          for (uint64_t j = g.off[v]; j < g.off[v + 1]; ++j) {
            const uint32_t u = g.nbr[j];
            if (C[u] != c) continue;
            if (method == PCC_TRIANGLE_SUBCLUSTERING && !(tri[j] > 0.25)) continue;
            uf.Unite(static_cast<uint32_t>(x), local[u]);
          }
        }
        uint32_t mx = 0;
        for (size_t x = 0; x < mem.size(); ++x) {
          lab[x] = uf.Find(static_cast<uint32_t>(x));
          mx = std::max(mx, lab[x]);
        }
        block = method == PCC_CONNECTIVITY_SUBCLUSTERING ? static_cast<uint32_t>(mem.size()) : mx + 1;
      }
      out.next[gi] = block;
    }
  }
  uint64_t run = 0;
  for (size_t gi = 0; gi < G; ++gi) {
    const uint64_t b = out.next[gi];
    out.next[gi] = run;
    run += b;
  }
  out.next[G] = run;
  for (size_t gi = 0; gi < G; ++gi)
    for (size_t x = 0; x < groups[gi].size(); ++x)
      out.id[groups[gi][x]] = static_cast<uint32_t>(out.next[gi] + labels[gi][x]);
  return out;
}

// The next level's starting clustering after compression by subcluster id.
void HelperFromSubclusters(Helper& h, uint32_t n2, std::vector<double> k2, const SubclusterMap& sm) {
  h.n = n2;
  h.k = std::move(k2);
  h.C.assign(n2, 0);
  h.s.assign(n2, 0);
  h.K.assign(n2, 0.0);
  const size_t G = sm.next.size() - 1;
  for (size_t gi = 0; gi < G; ++gi) {
    h.s[gi] = static_cast<uint32_t>(sm.next[gi + 1] - sm.next[gi]);
    for (uint64_t j = sm.next[gi]; j < sm.next[gi + 1] && j < n2; ++j) {
      h.C[j] = static_cast<uint32_t>(gi);
      h.K[gi] += h.k[j];
    }
  }
}

struct ClusterResult {
  std::vector<uint32_t> labels;  // dense group index
  uint32_t num_clusters = 0;
  double objective = 0;
  int32_t levels = 0;
  int32_t refine_passes = 0;
  Counters ctr;
};

// ParallelCorrelationClusterer::RefineClusters_subroutine
// (parallel-correlation-clusterer.cc:476-629).
int RefineClustersSubroutine(const Graph& graph, const pcc_config& cfg,
                             const std::vector<double>& node_weights,
                             const uint32_t* initial_labels,
                             ClusterResult* result) {
  int64_t num_iterations = 0, num_inner = 0;
  if (cfg.clustering_moves_method == PCC_LOUVAIN) {
    num_iterations = cfg.louvain_num_iterations > 0 ? cfg.louvain_num_iterations : 10;
    num_inner = cfg.louvain_num_inner_iterations > 0 ? cfg.louvain_num_inner_iterations : 10;
  } else if (cfg.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES) {
    // One level of up to num_iterations rounds (:487-492).
    num_iterations = 1;
    num_inner = cfg.num_iterations > 0 ? cfg.num_iterations : 20;
  } else {
    return PCC_UNIMPLEMENTED;
  }
  const int sub_method = cfg.subclustering_method;
  if (sub_method != PCC_NONE_SUBCLUSTERING && sub_method != PCC_TRIANGLE_SUBCLUSTERING &&
      sub_method != PCC_CONNECTIVITY_SUBCLUSTERING && sub_method != PCC_SLOW_CONNECTIVITY_SUBCLUSTERING)
    return PCC_UNIMPLEMENTED;
  // Subcluster moves inside the DEFAULT_CLUSTER_MOVES rounds are not
  // restated (the library answers UNIMPLEMENTED for them too).
  if (sub_method != PCC_NONE_SUBCLUSTERING && cfg.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES)
    return PCC_UNIMPLEMENTED;
  const bool subclusters = sub_method != PCC_NONE_SUBCLUSTERING;

  Options o;
  o.res = cfg.resolution;
  o.offset = cfg.edge_weight_offset;
  o.move_method = cfg.move_method;
  o.whole_clusters = cfg.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES;
  o.async = cfg.async != 0;
  o.permute = cfg.permute != 0;
  o.seed = cfg.random_seed;
  const bool refine = cfg.refine != 0;
  const uint32_t n = graph.n;

  std::vector<std::unique_ptr<Helper>> rec_helpers;
  std::vector<std::unique_ptr<Graph>> rec_graphs;
  std::vector<std::vector<uint32_t>> rec_maps;  // subclustering: level-i vertex -> level-(i+1) vertex
  if (refine) {
    rec_helpers.resize(num_iterations);
    rec_graphs.resize(num_iterations);
    rec_maps.resize(num_iterations);
  }
  bool vertex_ids = false;  // no refine, subclustering: cluster_ids hold vertex ids of the current level
  auto helper = std::make_unique<Helper>();
  {
    std::vector<double> k = node_weights;
    if (k.empty()) k.assign(n, 1.0);
    if (initial_labels) {
      std::vector<uint32_t> lab(initial_labels, initial_labels + n);
      HelperFromLabels(*helper, n, k, lab);
    } else {
      helper->InitSingletons(n, k);
    }
  }
  std::vector<uint32_t> cluster_ids(n);
  std::iota(cluster_ids.begin(), cluster_ids.end(), 0u);

  std::unique_ptr<Graph> compressed;
  int64_t iter = 0;
  for (iter = 0; iter < num_iterations; ++iter) {
    const Graph& cur = (iter == 0) ? graph : *compressed;
    bool moved = IterateBestMoves(cur, *helper, num_inner, o, result->ctr);
    if (!moved) {
      iter--;
      break;
    }
    result->levels++;
    const bool last = iter == num_iterations - 1;
    SubclusterMap sm;
    if (subclusters && !last) sm = ComputeSubclusters(cur, helper->C, sub_method, o);
    if (!refine) {
      // FlattenClustering (parallel-graph-utils.cc:233-243); with
      // subclusters the map to the next level is the subcluster id.
      const std::vector<uint32_t>& map = (subclusters && !last) ? sm.id : helper->C;
      for (uint32_t i = 0; i < n; ++i) cluster_ids[i] = map[cluster_ids[i]];
      vertex_ids = subclusters && !last;
    } else if (last) {
      rec_helpers[iter] = std::move(helper);
      rec_graphs[iter] = (iter == 0) ? nullptr : std::move(compressed);
    }
    if (last) break;

    auto next = std::make_unique<Graph>(CompressGraph(cur, subclusters ? sm.id : helper->C, helper->k));
    std::vector<double> next_k = std::move(next->node_w);
    next->node_w.clear();
    std::unique_ptr<Graph> prev = std::move(compressed);
    compressed = std::move(next);
    if (refine) {
      rec_helpers[iter] = std::move(helper);
      rec_graphs[iter] = std::move(prev);  // graph of level `iter` (nullptr at 0)
      if (subclusters) rec_maps[iter] = sm.id;
    }
    helper = std::make_unique<Helper>();
    if (subclusters) {
      HelperFromSubclusters(*helper, compressed->n, std::move(next_k), sm);
    } else {
      helper->InitSingletons(compressed->n, std::move(next_k));
    }
  }
  // No refine, subclusters: the last level did not move; its starting
  // clustering names the clusters of the vertices cluster_ids now hold.
  if (vertex_ids)
    for (uint32_t i = 0; i < n; ++i) cluster_ids[i] = helper->C[cluster_ids[i]];

  if (refine && iter > 0) {
    for (int64_t i = iter - 1; i >= 0; --i) {
      const Graph& cur = (i == 0) ? graph : *rec_graphs[i];
      Helper& hi = *rec_helpers[i];
      const Helper& hup = *rec_helpers[i + 1];
      std::vector<uint32_t> flat(hi.n);
      const std::vector<uint32_t>& map = subclusters ? rec_maps[i] : hi.C;
      for (uint32_t j = 0; j < hi.n; ++j) flat[j] = hup.C[map[j]];
      hi.SetGroups(GroupsById(flat));
      IterateBestMoves(cur, hi, num_inner, o, result->ctr);
      result->refine_passes++;
    }
    cluster_ids = rec_helpers[0]->C;
  }

  result->labels = DenseLabels(cluster_ids, &result->num_clusters);
  // Final objective with a fresh helper (:618-624).
  Helper h2;
  std::vector<double> k = node_weights;
  if (k.empty()) k.assign(n, 1.0);
  HelperFromLabels(h2, n, k, result->labels);
  result->objective = ComputeObjective(graph, h2.C, h2.k, h2.K, cfg.resolution,
                                       cfg.edge_weight_offset);
  return PCC_OK;
}

// ComputeModularity (parallel-modularity-clusterer.cc:36-66).
double ComputeModularity(const Graph& g, const std::vector<uint32_t>& labels,
                         double resolution) {
  double total = 0;
  double modularity = 0;
  uint32_t groups = 0;
  for (uint32_t x : labels) groups = std::max(groups, x + 1);
  for (uint32_t i = 0; i < g.n; ++i) {
    for (uint64_t j = g.off[i]; j < g.off[i + 1]; ++j) {
      total++;
      if (labels[i] == labels[g.nbr[j]]) modularity++;
    }
  }
  std::vector<double> degree(groups, 0.0);
  for (uint32_t i = 0; i < g.n; ++i) degree[labels[i]] += double(g.degree(i));
  for (uint32_t c = 0; c < groups; ++c)
    modularity -= (resolution * degree[c] * degree[c]) / total;
  return modularity / total;
}

void FillStats(const ClusterResult& r, pcc_stats* st) {
  if (!st) return;
  std::memset(st, 0, sizeof(*st));
  st->edge_visits = r.ctr.edge_visits;
  st->vertex_visits = r.ctr.vertex_visits;
  st->moves = r.ctr.moves;
  st->levels = r.levels;
  st->rounds = r.ctr.rounds;
  st->refine_passes = r.refine_passes;
  st->num_clusters = static_cast<int32_t>(r.num_clusters);
  st->objective = r.objective;
}

}  // namespace

// ---------------------------------------------------------------------------
// Seeded RMAT input for the CPU baseline.  Input generation, not part of the
// restated algorithm: it yields the same graph as the package's host
// generator (pcch_gen_rmat) from the same seed, written independently so a
// process that times the oracle loads no library of the GPU package.  The
// sample stream is a counter-based SplitMix64 hash of (seed, sample, level
// pair); each level picks a quadrant with probabilities a, b, c, 1-a-b-c.
// The CSR is symmetrised, self-loops dropped, rows sorted by neighbour id
// and deduplicated.  A CPU test checks the two generators agree entry for
// entry.
// ---------------------------------------------------------------------------
namespace {

inline uint64_t Mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

inline uint64_t SampleHash(uint64_t seed, uint64_t sample, uint64_t level) {
  return Mix64(Mix64(seed ^ Mix64(sample)) ^ (level * 0xD6E8FEB86659FD93ull));
}

Graph RmatGraph(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                uint64_t seed) {
  Graph g;
  g.n = scale >= 32 ? 0xFFFFFFFFu : (1u << scale);
  const uint64_t samples = uint64_t(edge_factor) << scale;
  const double ab = a + b, abc = a + b + c;
  std::vector<uint32_t> su(samples), sv(samples);
#pragma omp parallel for schedule(static) num_threads(NumThreads())
  for (int64_t e = 0; e < int64_t(samples); ++e) {
    uint32_t u = 0, v = 0;
    uint64_t h = 0;
    for (uint32_t l = 0; l < scale; ++l) {
      if (l % 2 == 0) h = SampleHash(seed, uint64_t(e), l);
      const uint32_t word = l % 2 ? uint32_t(h >> 32) : uint32_t(h & 0xFFFFFFFFu);
      const double x = double(word) / 4294967296.0;
      const uint32_t qu = x < ab ? 0u : 1u;
      const uint32_t qv = (x < a || (x >= ab && x < abc)) ? 0u : 1u;
      u = 2 * u + qu;
      v = 2 * v + qv;
    }
    su[e] = u;
    sv[e] = v;
  }
  // Both directions of every non-loop sample, bucketed by source row.
  std::vector<uint64_t> cnt(size_t(g.n) + 1, 0);
#pragma omp parallel for schedule(static) num_threads(NumThreads())
  for (int64_t e = 0; e < int64_t(samples); ++e) {
    if (su[e] == sv[e]) continue;
    __atomic_fetch_add(&cnt[su[e]], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&cnt[sv[e]], 1, __ATOMIC_RELAXED);
  }
  std::vector<uint64_t> start(size_t(g.n) + 1, 0);
  for (uint32_t i = 0; i < g.n; ++i) start[i + 1] = start[i] + cnt[i];
  std::vector<uint32_t> bucket(start[g.n]);
  std::vector<uint64_t> fill(start.begin(), start.end() - 1);
#pragma omp parallel for schedule(static) num_threads(NumThreads())
  for (int64_t e = 0; e < int64_t(samples); ++e) {
    if (su[e] == sv[e]) continue;
    bucket[__atomic_fetch_add(&fill[su[e]], 1, __ATOMIC_RELAXED)] = sv[e];
    bucket[__atomic_fetch_add(&fill[sv[e]], 1, __ATOMIC_RELAXED)] = su[e];
  }
  // Sort and deduplicate each row in place; then pack the rows.
  std::vector<uint64_t> deg(g.n, 0);
#pragma omp parallel for schedule(dynamic, 512) num_threads(NumThreads())
  for (int64_t i = 0; i < int64_t(g.n); ++i) {
    uint32_t* r = bucket.data() + start[i];
    const size_t len = start[i + 1] - start[i];
    std::sort(r, r + len);
    deg[i] = size_t(std::unique(r, r + len) - r);
  }
  g.off.assign(size_t(g.n) + 1, 0);
  for (uint32_t i = 0; i < g.n; ++i) g.off[i + 1] = g.off[i] + deg[i];
  g.m = g.off[g.n];
  g.nbr.resize(g.m);
#pragma omp parallel for schedule(dynamic, 512) num_threads(NumThreads())
  for (int64_t i = 0; i < int64_t(g.n); ++i)
    std::copy(bucket.begin() + start[i], bucket.begin() + start[i] + deg[i], g.nbr.begin() + g.off[i]);
  return g;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI of the oracle (ctypes from tests/ and bench.py).
// ---------------------------------------------------------------------------
extern "C" {

struct pcco_graph {
  Graph g;
};

void pcco_set_threads(int threads) { g_threads = threads; }
int pcco_get_threads(void) { return NumThreads(); }

pcco_graph* pcco_graph_create(uint32_t n, uint64_t m, const uint64_t* off,
                              const uint32_t* nbr, const float* w) {
  auto* h = new pcco_graph;
  h->g.n = n;
  h->g.m = m;
  h->g.off.assign(off, off + size_t(n) + 1);
  h->g.nbr.assign(nbr, nbr + m);
  if (w) h->g.w.assign(w, w + m);
  return h;
}

void pcco_graph_free(pcco_graph* g) { delete g; }

void pcco_graph_info(const pcco_graph* g, uint32_t* n, uint64_t* m) {
  *n = g->g.n;
  *m = g->g.m;
}

void pcco_graph_copy(const pcco_graph* g, uint64_t* off, uint32_t* nbr, float* w,
                     double* node_w) {
  std::copy(g->g.off.begin(), g->g.off.end(), off);
  std::copy(g->g.nbr.begin(), g->g.nbr.end(), nbr);
  if (w) {
    for (uint64_t j = 0; j < g->g.m; ++j) w[j] = g->g.weight(j);
  }
  if (node_w) std::copy(g->g.node_w.begin(), g->g.node_w.end(), node_w);
}

int pcco_correlation_cluster(const pcco_graph* g, const pcc_config* cfg,
                             const double* node_weights,
                             const uint32_t* initial_labels,
                             uint32_t* out_labels, pcc_stats* stats) {
  std::vector<double> k;
  if (node_weights) k.assign(node_weights, node_weights + g->g.n);
  ClusterResult r;
  int st = RefineClustersSubroutine(g->g, *cfg, k, initial_labels, &r);
  if (st != PCC_OK) return st;
  std::copy(r.labels.begin(), r.labels.end(), out_labels);
  FillStats(r, stats);
  return PCC_OK;
}

// ParallelModularityClusterer::RefineClusters (parallel-modularity-
// clusterer.cc:68-96) with ComputeModularityConfig (parallel-graph-
// utils.cc:141-153).
int pcco_modularity_cluster(const pcco_graph* g, const pcc_config* cfg,
                            const uint32_t* initial_labels, uint32_t* out_labels,
                            pcc_stats* stats) {
  const uint32_t n = g->g.n;
  std::vector<double> k(n);
  for (uint32_t i = 0; i < n; ++i) k[i] = double(g->g.degree(i));
  const double total = n ? BlockedReduce(k.data(), n, [](double a, double b) { return a + b; }) : 0.0;
  pcc_config c2 = *cfg;
  c2.resolution = cfg->resolution / total;
  c2.edge_weight_offset = 0;
  ClusterResult r;
  int st = RefineClustersSubroutine(g->g, c2, k, initial_labels, &r);
  if (st != PCC_OK) return st;
  std::copy(r.labels.begin(), r.labels.end(), out_labels);
  FillStats(r, stats);
  if (stats) stats->modularity = ComputeModularity(g->g, r.labels, cfg->resolution);
  return PCC_OK;
}

int pcco_objective(const pcco_graph* g, const pcc_config* cfg,
                   const double* node_weights, const uint32_t* labels,
                   double* out) {
  const uint32_t n = g->g.n;
  std::vector<double> k;
  if (node_weights) k.assign(node_weights, node_weights + n);
  std::vector<uint32_t> lab(labels, labels + n);
  for (uint32_t x : lab)
    if (x >= n) return PCC_INVALID_ARGUMENT;
  Helper h;
  HelperFromLabels(h, n, k, lab);
  *out = ComputeObjective(g->g, h.C, h.k, h.K, cfg->resolution, cfg->edge_weight_offset);
  return PCC_OK;
}

int pcco_modularity(const pcco_graph* g, double resolution, const uint32_t* labels,
                    double* out) {
  std::vector<uint32_t> lab(labels, labels + g->g.n);
  // ComputeModularity walks clusters in Clustering order; dense labels give it.
  uint32_t ng = 0;
  std::vector<uint32_t> dense = DenseLabels(lab, &ng);
  *out = ComputeModularity(g->g, dense, resolution);
  return PCC_OK;
}

// One synchronous best-move pass over all vertices from a given state.
int pcco_best_moves(const pcco_graph* g, const pcc_config* cfg,
                    const uint32_t* C, const uint32_t* s, const double* k,
                    const double* K, uint32_t* out_t, double* out_v,
                    uint32_t* out_moves) {
  const uint32_t n = g->g.n;
  Helper h;
  h.n = n;
  h.C.assign(C, C + n);
  h.s.assign(s, s + n);
  h.k.assign(k, k + n);
  h.K.assign(K, K + n);
#pragma omp parallel num_threads(NumThreads())
  {
    Scratch sc;
#pragma omp for schedule(dynamic, 64)
    for (int64_t v = 0; v < int64_t(n); ++v) {
      Move mv = EfficientBestMove<false>(g->g, h, uint32_t(v), cfg->resolution,
                                         cfg->edge_weight_offset, sc);
      out_t[v] = mv.target;
      out_v[v] = mv.value;
      if (out_moves) {
        const uint32_t cur = h.C[v];
        if (mv.target < n && h.s[mv.target] == 1 && h.s[cur] == 1 &&
            cur >= mv.target) {
          mv.target = cur;
          mv.value = 0;
        }
        out_moves[v] = mv.value > 0 ? mv.target : kNone;
      }
    }
  }
  return PCC_OK;
}

// MoveNodesToCluster in place on caller arrays.  modified may be NULL.
int pcco_move_nodes(uint32_t n, uint32_t* C, uint32_t* s, const double* k,
                    double* K, const uint32_t* moves, uint8_t* modified) {
  Helper h;
  h.n = n;
  h.C.assign(C, C + n);
  h.s.assign(s, s + n);
  h.k.assign(k, k + n);
  h.K.assign(K, K + n);
  std::vector<uint32_t> mv(moves, moves + n);
  std::vector<uint8_t> mod = MoveNodesToCluster(h, mv, nullptr);
  std::copy(h.C.begin(), h.C.end(), C);
  std::copy(h.s.begin(), h.s.end(), s);
  std::copy(h.K.begin(), h.K.end(), K);
  if (modified) std::copy(mod.begin(), mod.end(), modified);
  return PCC_OK;
}

// CompareCommunities (clustering/cluster-in-memory_main.cc:172-225), read
// literally: the clustering is OutputIndicesById of the labels (groups in
// ascending label order, members ascending), each community is sorted
// (ReadCommunities, :155-170), std::set_intersection against every cluster
// in order keeps the first largest, and the averages are pbbs::reduce_add
// over the per-community vectors divided by their count.  out[6] =
// {avg_precision, avg_recall, num_clusters, min_size, max_size, avg_size}.
int pcco_compare_communities(uint32_t n, const uint32_t* labels, uint32_t num_comm,
                             const uint64_t* off, const uint32_t* members,
                             double* precision, double* recall, double* out) {
  const std::vector<uint32_t> ids(labels, labels + n);
  const std::vector<std::vector<uint32_t>> clustering = GroupsById(ids);
  std::vector<double> prec(num_comm, 0.0), rec(num_comm, 0.0);
  for (uint32_t j = 0; j < num_comm; ++j) {
    std::vector<uint32_t> community(members + off[j], members + off[j + 1]);
    std::sort(community.begin(), community.end());
    std::vector<uint32_t> intersect(community.size());
    size_t max_intersect = 0, max_idx = 0;
    for (size_t i = 0; i < clustering.size(); ++i) {
      const std::vector<uint32_t>& cluster = clustering[i];
      auto it = std::set_intersection(cluster.begin(), cluster.end(), community.begin(),
                                      community.end(), intersect.begin());
      const size_t sz = static_cast<size_t>(it - intersect.begin());
      if (sz > max_intersect) {
        max_intersect = sz;
        max_idx = i;
      }
    }
    const size_t csize = clustering.empty() ? 0 : clustering[max_idx].size();
    prec[j] = csize ? static_cast<double>(max_intersect) / static_cast<double>(csize) : 0.0;
    rec[j] = community.empty() ? 0.0
                               : static_cast<double>(max_intersect) / static_cast<double>(community.size());
  }
  auto add = [](double a, double b) { return a + b; };
  const double sp = num_comm ? BlockedReduce(prec.data(), num_comm, add) : 0.0;
  const double sr = num_comm ? BlockedReduce(rec.data(), num_comm, add) : 0.0;
  out[0] = sp / static_cast<double>(num_comm);
  out[1] = sr / static_cast<double>(num_comm);
  size_t min_size = 0xFFFFFFFFu, max_size = 0;  // UINT_E_MAX
  double avg_size = 0;
  for (const auto& c : clustering) {
    min_size = std::min(min_size, c.size());
    max_size = std::max(max_size, c.size());
    avg_size += static_cast<double>(c.size());
  }
  avg_size /= static_cast<double>(clustering.size());
  out[2] = static_cast<double>(clustering.size());
  out[3] = static_cast<double>(min_size);
  out[4] = static_cast<double>(max_size);
  out[5] = avg_size;
  if (precision) std::copy(prec.begin(), prec.end(), precision);
  if (recall) std::copy(rec.begin(), rec.end(), recall);
  return PCC_OK;
}

pcco_graph* pcco_compress(const pcco_graph* g, const uint32_t* C,
                          const double* k) {
  std::vector<uint32_t> c(C, C + g->g.n);
  std::vector<double> kk;
  if (k) kk.assign(k, k + g->g.n);
  auto* out = new pcco_graph;
  out->g = CompressGraph(g->g, c, kk);
  return out;
}

// Subcluster ids of a clustering C (one level of CompressSubclusters):
// out_ids[n]; out_next[G + 1] block starts in cluster order, then the total
// (G = number of clusters; the array must hold n + 1 entries).
int pcco_subclusters(const pcco_graph* g, const uint32_t* C, int32_t method, double resolution,
                     double edge_weight_offset, uint32_t* out_ids, uint64_t* out_next, uint32_t* num_clusters) {
  std::vector<uint32_t> c(C, C + g->g.n);
  Options o;
  o.res = resolution;
  o.offset = edge_weight_offset;
  const SubclusterMap sm = ComputeSubclusters(g->g, c, method, o);
  std::copy(sm.id.begin(), sm.id.end(), out_ids);
  std::copy(sm.next.begin(), sm.next.end(), out_next);
  *num_clusters = static_cast<uint32_t>(sm.next.size() - 1);
  return PCC_OK;
}

pcco_graph* pcco_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                          uint64_t seed) {
  auto* out = new pcco_graph;
  out->g = RmatGraph(scale, edge_factor, a, b, c, seed);
  return out;
}

}  // extern "C"
