// louvain.cu -- the multilevel Louvain engine and the clustering C ABI.
//
// Restates ParallelCorrelationClusterer::RefineClusters_subroutine
// (clustering/clusterers/parallel-correlation-clusterer.cc:476-629),
// IterateBestMoves (:340-365), BestMovesForVertexSubset (:115-338, LOUVAIN
// vertex moves), MoveNodesToCluster (parallel-correlation-clusterer-
// internal.cc:256-369), FlattenClustering / OutputIndicesById
// (parallel/parallel-graph-utils.cc:233-243, parallel-sequence-ops.h:183-209),
// ComputeObjective (internal.cc:118-149) and the modularity wrapper
// (parallel-modularity-clusterer.cc:36-111).
//
// Host code only enqueues work on the context stream; it reads back a few
// counters once per best-move round and once per level.
#include <chrono>
#include <cmath>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "graphops.cuh"
#include "hubs.cuh"

namespace pcc {

Status CompressGraph(Context* ctx, const DevGraph& g, const uint32_t* C, const double* k,
                     std::unique_ptr<DevGraph>* out);
Status FindClusterMoves(Context* ctx, const DevGraph& g, const uint32_t* C, const double* k, const double* K,
                        double res, double offset, bool exact_sums, uint32_t* moves, uint32_t* movers,
                        DevCounters* ctr);
Status AsyncSetMoves(Context* ctx, const SetMoveArgs& a, const std::function<Status(uint32_t)>& vertex_moves);
Status ComputeSubclustersDevice(Context* ctx, const DevGraph& g, const uint32_t* C, int method, double res,
                                double offset, DBuf<uint32_t>* sub, DBuf<uint64_t>* next, uint32_t* num_clusters,
                                uint64_t* total);

namespace {

constexpr unsigned kT = 256;

unsigned GridFor(Context* ctx, uint64_t items, unsigned per_block = kT) {
  return Blocks(items, per_block, unsigned(ctx->num_sms) * 16);
}

// ---------------------------------------------------------------------------
// Small kernels.
// ---------------------------------------------------------------------------
__global__ void IotaKernel(uint32_t n, uint32_t* out) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    out[i] = static_cast<uint32_t>(i);
}

__global__ void FillF64Kernel(uint64_t n, double v, double* out) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    out[i] = v;
}

// Singletons: C = i, s = 1, K = k (SetClustering with an empty clustering).
__global__ void SingletonsKernel(uint32_t n, const double* __restrict__ k, uint32_t* C, uint32_t* s, double* K) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    C[i] = static_cast<uint32_t>(i);
    s[i] = 1u;
    K[i] = k[i];
  }
}

// s[C[i]] += 1, K[C[i]] += k[i] (SetClustering with a clustering; exact for
// integral node weights, which is every weight the clusterers create).
__global__ void AccumulateClustersKernel(uint32_t n, const uint32_t* __restrict__ C, const double* __restrict__ k,
                                         uint32_t* s, double* K) {
  const uint64_t limit = (uint64_t(n) + 31) & ~uint64_t(31);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * blockDim.x) {
    const bool in = i < n;
    const uint32_t c = in ? C[i] : kNone;
    const double x = in ? k[i] : 0.0;
    const unsigned peers = __match_any_sync(kFull, c);
    double tot = 0.0;
    unsigned mm = peers;
    while (mm) {
      const int j = __ffs(mm) - 1;
      tot += __shfl_sync(peers, x, j);
      mm &= mm - 1;
    }
    if (in && int(LaneId()) == __ffs(peers) - 1) {
      atomicAdd(&s[c], uint32_t(__popc(peers)));
      atomicAdd(&K[c], tot);
    }
  }
}

// Kf[c] = fl32(K[c]) for every c (stamp == 0) or for the clusters modified
// in the round `stamp` (the FP32 pre-filter of the best-move kernels needs
// Kf == fl32(K) exactly).
// Kf = FilterF32(K) on every cluster (stamp 0) or on the clusters modified
// in the round (mod_stamp == the round's stamp).
__global__ void RefreshKfKernel(uint32_t n, const double* __restrict__ K, float* Kf,
                                const uint32_t* __restrict__ mod_stamp, uint32_t stamp, const RoundState* rs) {
  const uint32_t st = StampIn(rs, stamp);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    if (st == 0 || mod_stamp[i] == st) Kf[i] = FilterF32(K[i]);
}

// kf = FilterF32(k): node weights for the FP32 pre-filter and certified
// decisions.
__global__ void NodeKfKernel(uint32_t n, const double* __restrict__ k, float* kf) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    kf[i] = FilterF32(k[i]);
}

// All node weights are integers of magnitude below 2^53 (host array).
bool IntegralWeights(const double* w, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i)
    if (!(w[i] == std::trunc(w[i]) && std::fabs(w[i]) < 9007199254740992.0)) return false;
  return true;
}

// cluster_ids[i] = C[cluster_ids[i]] (FlattenClustering).
// The starting cluster of every vertex of a level compressed by subcluster
// id: the cluster whose block [next[i], next[i + 1]) holds the id.
__global__ void BlockOfKernel(uint32_t n, const uint64_t* __restrict__ next, uint32_t G, uint32_t* __restrict__ out) {
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t lo = 0, hi = G;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (next[mid] <= j) lo = mid;
      else hi = mid;
    }
    out[j] = lo;
  }
}

__global__ void AddU32Kernel(uint32_t* p, uint32_t x) { *p += x; }

__global__ void FlattenKernel(uint32_t n, uint32_t* ids, const uint32_t* __restrict__ C) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    ids[i] = C[ids[i]];
}

// flat[j] = Cup[C[j]] and mark the flattened id as present.
__global__ void ProjectKernel(uint32_t n, const uint32_t* __restrict__ C, const uint32_t* __restrict__ Cup,
                              uint32_t* flat, uint32_t* present_stamp, uint32_t stamp) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t f = Cup[C[i]];
    flat[i] = f;
    present_stamp[f] = stamp;
  }
}

__global__ void MarkStampKernel(uint32_t n, const uint32_t* ids, uint32_t* st, uint32_t stamp) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    st[ids[i]] = stamp;
}

struct StampInput {
  const uint32_t* st;
  uint32_t stamp;
  __device__ uint32_t operator()(uint64_t i) const { return st[i] == stamp ? 1u : 0u; }
};

__global__ void GatherKernel(uint32_t n, const uint32_t* __restrict__ idx, const uint32_t* __restrict__ table,
                             uint32_t* out) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    out[i] = table[idx[i]];
}

// ---------------------------------------------------------------------------
// Sync apply: MoveNodesToCluster.
// ---------------------------------------------------------------------------
struct ApplyArgs {
  uint32_t n;
  uint32_t* C;
  uint32_t* s;
  const double* k;
  double* K;
  const uint32_t* moves;
  const uint32_t* movers;
  uint32_t* mod_stamp;
  uint32_t* new_stamp;
  uint32_t stamp;
  DevCounters* ctr;
  const RoundState* rs;  // non-null: the stamp comes from here
};

// Sum of x over the lanes of `peers` (the caller's match group), in lane
// order; every lane of the group gets the result.
__device__ __forceinline__ double GroupSum(unsigned peers, double x) {
  double tot = 0.0;
  unsigned mm = peers;
  while (mm) {
    const int j = __ffs(mm) - 1;
    tot += __shfl_sync(peers, x, j);
    mm &= mm - 1;
  }
  return tot;
}

// Leave: every mover leaves its cluster (sizes and weights), marks it
// modified; movers to a new cluster are flagged for ranking.  Equal
// clusters inside a warp are combined first (one atomic per cluster and
// warp); the FP64 sums are exact because node weights are integral.
__global__ void __launch_bounds__(kT) ApplyLeaveKernel(ApplyArgs a) {
  const uint32_t count = a.ctr->movers;
  const uint64_t limit = (uint64_t(count) + 31) & ~uint64_t(31);
  for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * kT) {
    const bool in = i < count;
    const uint32_t v = in ? a.movers[i] : 0u;
    const uint32_t c = in ? a.C[v] : kNone;
    const double kv = in ? a.k[v] : 0.0;
    const unsigned peers = __match_any_sync(kFull, c);
    const double tot = GroupSum(peers, kv);
    if (in && int(LaneId()) == __ffs(peers) - 1) {
      atomicSub(&a.s[c], uint32_t(__popc(peers)));
      atomicAdd(&a.K[c], -tot);
      a.mod_stamp[c] = StampIn(a.rs, a.stamp);
    }
    const bool isnew = in && a.moves[v] == a.n;
    if (isnew) a.new_stamp[v] = StampIn(a.rs, a.stamp);
    const unsigned nb = __ballot_sync(kFull, isnew);
    if (nb && LaneId() == 0) atomicAdd(&a.ctr->new_movers, uint32_t(__popc(nb)));
  }
}

// Leave and join in one pass over the movers: every size and weight update
// is an atomic add, and the adds commute (the FP64 weight sums are exact for
// integral node weights), so each mover can leave its cluster and enter its
// target at once.  Equal clusters inside a warp are combined first, for the
// leave and for the join.
__global__ void __launch_bounds__(kT) ApplyMoveKernel(ApplyArgs a) {
  const uint32_t count = a.ctr->movers;
  const uint64_t limit = (uint64_t(count) + 31) & ~uint64_t(31);
  for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * kT) {
    const bool in = i < count;
    const uint32_t v = in ? a.movers[i] : 0u;
    const uint32_t c = in ? a.C[v] : kNone;
    const uint32_t t = in ? a.moves[v] : a.n;
    const double kv = in ? a.k[v] : 0.0;
    {
      const unsigned peers = __match_any_sync(kFull, c);
      const double tot = GroupSum(peers, kv);
      if (in && int(LaneId()) == __ffs(peers) - 1) {
        atomicSub(&a.s[c], uint32_t(__popc(peers)));
        atomicAdd(&a.K[c], -tot);
        a.mod_stamp[c] = StampIn(a.rs, a.stamp);
      }
    }
    const bool isnew = in && t == a.n;
    if (isnew) a.new_stamp[v] = StampIn(a.rs, a.stamp);
    const unsigned nb = __ballot_sync(kFull, isnew);
    if (nb && LaneId() == 0) atomicAdd(&a.ctr->new_movers, uint32_t(__popc(nb)));
    const bool join = in && t != a.n;
    {
      const uint32_t key = join ? t : kNone;
      const unsigned peers = __match_any_sync(kFull, key);
      const double tot = GroupSum(peers, join ? kv : 0.0);
      if (join && int(LaneId()) == __ffs(peers) - 1) {
        atomicAdd(&a.s[t], uint32_t(__popc(peers)));
        atomicAdd(&a.K[t], tot);
        a.mod_stamp[t] = StampIn(a.rs, a.stamp);
      }
    }
    if (join) a.C[v] = t;
  }
}

// Join: movers to existing clusters enter them.
__global__ void __launch_bounds__(kT) ApplyJoinKernel(ApplyArgs a) {
  const uint32_t count = a.ctr->movers;
  const uint64_t limit = (uint64_t(count) + 31) & ~uint64_t(31);
  for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * kT) {
    const uint32_t v = i < count ? a.movers[i] : 0u;
    const uint32_t t = i < count ? a.moves[v] : a.n;
    const bool in = i < count && t != a.n;
    const uint32_t key = in ? t : kNone;
    const double kv = in ? a.k[v] : 0.0;
    const unsigned peers = __match_any_sync(kFull, key);
    const double tot = GroupSum(peers, kv);
    if (in && int(LaneId()) == __ffs(peers) - 1) {
      atomicAdd(&a.s[t], uint32_t(__popc(peers)));
      atomicAdd(&a.K[t], tot);
      a.mod_stamp[t] = StampIn(a.rs, a.stamp);
    }
    if (in) a.C[v] = t;
  }
}

// Gated inputs for the new-cluster compactions: nothing to do when no
// vertex moves to a new cluster.
struct ZeroSizeInput {
  const uint32_t* s;
  const DevCounters* ctr;
  __device__ uint32_t operator()(uint64_t i) const { return ctr->new_movers && s[i] == 0u ? 1u : 0u; }
};
struct EmptyClusterInput {
  const uint32_t* s;
  __device__ uint32_t operator()(uint64_t i) const { return s[i] == 0u ? 1u : 0u; }
};
struct NewMoverInput {
  const uint32_t* st;
  uint32_t stamp;
  const DevCounters* ctr;
  const RoundState* rs = nullptr;
  __device__ uint32_t operator()(uint64_t i) const {
    return ctr->new_movers && st[i] == StampIn(rs, stamp) ? 1u : 0u;
  }
};

// New clusters take the ascending list of empty ids, in ascending node order.
__global__ void __launch_bounds__(kT) AssignNewKernel(ApplyArgs a, const uint32_t* __restrict__ zero_ids,
                                                      const uint32_t* __restrict__ new_list) {
  const uint32_t count = a.ctr->new_movers;
  for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < count; i += uint64_t(gridDim.x) * kT) {
    const uint32_t v = new_list[i];
    const uint32_t cid = zero_ids[i];
    a.C[v] = cid;
    a.s[cid] = 1u;
    a.K[cid] = a.k[v];
    a.mod_stamp[cid] = StampIn(a.rs, a.stamp);
  }
}

// ---------------------------------------------------------------------------
// Disjoint-union kernels (batched graphs; vbase: B + 1 vertex bases).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t LowerBound(const uint32_t* __restrict__ a, uint32_t len, uint32_t x) {
  uint32_t lo = 0, hi = len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// New clusters of a union: graph j's i-th new mover (ascending id) takes
// graph j's i-th empty id (ascending), as it would alone.  Graph j always
// has at least as many empty ids as new movers (its other clusters hold the
// rest of its vertices); an index outside graph j's range is reported as
// kErrUnionRange and skipped.
__global__ void __launch_bounds__(kT) AssignNewUnionKernel(ApplyArgs a, const uint32_t* __restrict__ zero_ids,
                                                           const uint32_t* __restrict__ zcount,
                                                           const uint32_t* __restrict__ new_list,
                                                           const uint32_t* __restrict__ vbase, uint32_t B) {
  const uint32_t count = a.ctr->new_movers;
  const uint32_t zc = *zcount;
  for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < count; i += uint64_t(gridDim.x) * kT) {
    const uint32_t v = new_list[i];
    const uint32_t j = GraphOf(vbase, B, v);
    const uint32_t lo = vbase[j];
    const uint32_t nb = LowerBound(new_list, count, lo);
    const uint32_t zb = LowerBound(zero_ids, zc, lo);
    const uint64_t zi = uint64_t(zb) + (i - nb);
    if (zi >= zc || zero_ids[zi] >= vbase[j + 1]) {
      atomicExch(&a.ctr->error, kErrUnionRange);
      continue;
    }
    const uint32_t cid = zero_ids[zi];
    a.C[v] = cid;
    a.s[cid] = 1u;
    a.K[cid] = a.k[v];
    a.mod_stamp[cid] = StampIn(a.rs, a.stamp);
  }
}

// Per graph: flags[j] = stamp when the frontier (st == stamp) holds a vertex
// of graph j, and edges[j] += the degrees of those vertices.
__global__ void __launch_bounds__(kT) GraphFrontierKernel(uint32_t n, const uint64_t* __restrict__ off,
                                                          const uint32_t* __restrict__ st, uint32_t stamp_arg,
                                                          const RoundState* rs, const uint32_t* __restrict__ vbase,
                                                          uint32_t B, uint32_t* flags, unsigned long long* edges) {
  const uint32_t stamp = StampIn(rs, stamp_arg);
  const uint64_t limit = (uint64_t(n) + 31) & ~uint64_t(31);
  for (uint64_t v = uint64_t(blockIdx.x) * kT + threadIdx.x; v < limit; v += uint64_t(gridDim.x) * kT) {
    const bool in = v < n && st[v] == stamp;
    const uint32_t j = in ? GraphOf(vbase, B, static_cast<uint32_t>(v)) : kNone;
    const unsigned long long d = in ? off[v + 1] - off[v] : 0ull;
    const unsigned peers = __match_any_sync(kFull, j);
    unsigned long long tot = 0;
    for (unsigned mm = peers; mm; mm &= mm - 1) tot += __shfl_sync(peers, d, __ffs(mm) - 1);
    if (in && int(LaneId()) == __ffs(peers) - 1) {
      if (flags[j] != stamp) flags[j] = stamp;
      if (tot) atomicAdd(&edges[j], tot);
    }
  }
}

// Round-0 frontier of the graphs with mask[j] != 0: st = stamp on their
// vertices of degree > 0.
__global__ void __launch_bounds__(kT) MarkGraphsKernel(uint32_t n, const uint64_t* __restrict__ off,
                                                       const uint32_t* __restrict__ vbase, uint32_t B,
                                                       const uint32_t* __restrict__ mask, uint32_t* st,
                                                       uint32_t stamp) {
  for (uint64_t v = uint64_t(blockIdx.x) * kT + threadIdx.x; v < n; v += uint64_t(gridDim.x) * kT)
    if (off[v + 1] > off[v] && mask[GraphOf(vbase, B, static_cast<uint32_t>(v))]) st[v] = stamp;
}

// Per-graph dense rank: out[v] = rank[ids[v]] - rank[vbase[j]] (+ vbase[j]
// when add_base), rank the exclusive prefix count of the ids in use.
__global__ void __launch_bounds__(kT) GraphRankKernel(uint32_t n, const uint32_t* __restrict__ ids,
                                                      const uint32_t* __restrict__ rank, uint32_t* out,
                                                      const uint32_t* __restrict__ vbase, uint32_t B,
                                                      int add_base) {
  for (uint64_t v = uint64_t(blockIdx.x) * kT + threadIdx.x; v < n; v += uint64_t(gridDim.x) * kT) {
    const uint32_t j = GraphOf(vbase, B, static_cast<uint32_t>(v));
    out[v] = rank[ids[v]] - rank[vbase[j]] + (add_base ? vbase[j] : 0u);
  }
}

// out[j] = rank[vbase[j]] (j < B), out[B] = *total.
__global__ void GraphRankBaseKernel(uint32_t B, const uint32_t* __restrict__ vbase, const uint32_t* __restrict__ rank,
                                    const uint32_t* __restrict__ total, uint32_t* out) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j <= B; j += gridDim.x * blockDim.x)
    out[j] = j < B ? rank[vbase[j]] : *total;
}

// Per-vertex resolution of a union level: the owning graph's.
__global__ void __launch_bounds__(kT) GraphResKernel(uint32_t n, const uint32_t* __restrict__ vbase, uint32_t B,
                                                     const double* __restrict__ res, const float* __restrict__ res32,
                                                     double* vres, float* vres32) {
  for (uint64_t v = uint64_t(blockIdx.x) * kT + threadIdx.x; v < n; v += uint64_t(gridDim.x) * kT) {
    const uint32_t j = GraphOf(vbase, B, static_cast<uint32_t>(v));
    vres[v] = res[j];
    vres32[v] = res32[j];
  }
}

// ids[v] = v on the graphs with mask[j] != 0.
__global__ void __launch_bounds__(kT) IdentityGraphsKernel(uint32_t n, uint32_t* ids,
                                                           const uint32_t* __restrict__ vbase, uint32_t B,
                                                           const uint32_t* __restrict__ mask) {
  for (uint64_t v = uint64_t(blockIdx.x) * kT + threadIdx.x; v < n; v += uint64_t(gridDim.x) * kT)
    if (mask[GraphOf(vbase, B, static_cast<uint32_t>(v))]) ids[v] = static_cast<uint32_t>(v);
}

// Entries of each graph at a level of n vertices.
__global__ void GraphEntriesKernel(uint32_t B, uint32_t n, const uint32_t* __restrict__ vbase,
                                   const uint64_t* __restrict__ off, unsigned long long* out) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < B; j += gridDim.x * blockDim.x) {
    const uint32_t a = vbase[j], b = j + 1 < B ? vbase[j + 1] : n;
    out[j] = off[b < n ? b : n] - off[a];
  }
}

// ComputeObjective (parallel-correlation-clusterer-internal.cc:118-149) per
// graph of a union: edge[j] = sum over graph j's entries with equal labels
// of (w - offset) / 2, res[j] = sum over its vertices of k (K[L] - k).  The
// terms are the single-graph ones; with integer weights and node weights
// every partial sum is exact, so the result equals the single-graph value.
__global__ void __launch_bounds__(kT) ObjectiveUnionKernel(uint32_t n, const uint64_t* __restrict__ off,
                                                           const uint32_t* __restrict__ nbr,
                                                           const float* __restrict__ w,
                                                           const uint32_t* __restrict__ L,
                                                           const double* __restrict__ k,
                                                           const double* __restrict__ K, double offset,
                                                           const uint32_t* __restrict__ vbase, uint32_t B,
                                                           double* edge, double* res) {
  for (uint64_t u = uint64_t(blockIdx.x) * kT + threadIdx.x; u < n; u += uint64_t(gridDim.x) * kT) {
    const uint32_t cu = L[u];
    double x = 0.0;
    for (uint64_t e = off[u]; e < off[u + 1]; ++e)
      if (L[nbr[e]] == cu) x += Dsub(static_cast<double>(w ? w[e] : 1.0f), offset) / 2;
    const double r = Dmul(k[u], Dsub(K[cu], k[u]));
    const uint32_t j = GraphOf(vbase, B, static_cast<uint32_t>(u));
    if (x != 0.0) atomicAdd(&edge[j], x);
    if (r != 0.0) atomicAdd(&res[j], r);
  }
}

// Marked vertices for the next frontier.

// Marked vertices of the next frontier.
struct PredModifiedCluster {  // NBHR_CLUSTER_MOVE: vertices of modified clusters
  const uint32_t* C;
  const uint32_t* mod_stamp;
  uint32_t stamp;
  const RoundState* rs = nullptr;
  __device__ bool operator()(uint32_t v) const { return mod_stamp[C[v]] == StampIn(rs, stamp); }
};

// Rows the frontier push expands: marked (pred) and not empty.
template <class P>
struct PredMarkedRow {
  const uint64_t* off;
  P pred;
  __device__ bool operator()(uint32_t v) const { return off[v + 1] > off[v] && pred(v); }
};

// ---------------------------------------------------------------------------
// Objective / modularity.
// ---------------------------------------------------------------------------
struct ObjEdgeTerm {
  const uint32_t* nbr;
  const float* w;
  const uint32_t* C;
  double offset;
  double* acc;  // per-thread accumulators (indexed by the iteration slot)
  __device__ void operator()(uint32_t u, uint64_t j, uint64_t slot) const {
    if (C[u] == C[nbr[j]]) {
      const double x = Dsub(static_cast<double>(w ? w[j] : 1.0f), offset) / 2;
      acc[slot] += x;
    }
  }
};

struct ResTerm {
  const uint32_t* C;
  const double* k;
  const double* K;
  __device__ double operator()(uint64_t i) const { return Dmul(k[i], Dsub(K[C[i]], k[i])); }
};

struct ArrayInputF64 {
  const double* a;
  __device__ double operator()(uint64_t i) const { return a[i]; }
};

struct SameLabelCount {
  const uint32_t* nbr;
  const uint32_t* L;
  unsigned long long* acc;
  __device__ void operator()(uint32_t u, uint64_t j, uint64_t slot) const {
    if (L[u] == L[nbr[j]]) acc[slot] += 1ull;
  }
};

// deg[L[i]] += deg(i), one atomic per distinct label per warp.
__global__ void DegreeSumKernel(uint32_t n, const uint64_t* __restrict__ off, const uint32_t* __restrict__ L,
                                unsigned long long* deg) {
  const uint64_t limit = (uint64_t(n) + 31) & ~uint64_t(31);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * blockDim.x) {
    const bool in = i < n;
    const uint32_t lab = in ? L[i] : kNone;
    unsigned long long d = in ? static_cast<unsigned long long>(off[i + 1] - off[i]) : 0ull;
    const unsigned peers = __match_any_sync(kFull, lab);
    // Sum over peers (any order: integers).
    unsigned long long tot = 0;
    unsigned mm = peers;
    while (mm) {
      const int j = __ffs(mm) - 1;
      tot += __shfl_sync(peers, d, j);
      mm &= mm - 1;
    }
    if (in && int(LaneId()) == __ffs(peers) - 1) atomicAdd(&deg[lab], tot);
  }
}

struct ModTerm {
  const unsigned long long* deg;
  double res;
  double total;
  __device__ double operator()(uint64_t c) const {
    const double d = static_cast<double>(deg[c]);
    return Dmul(Dmul(res, d), d) / total;
  }
};

struct U64Input {
  const unsigned long long* a;
  __device__ unsigned long long operator()(uint64_t i) const { return a[i]; }
};

__global__ void DegreeF64Kernel(uint32_t n, const uint64_t* __restrict__ off, double* k) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    k[i] = static_cast<double>(off[i + 1] - off[i]);
}

// ---------------------------------------------------------------------------
// Device-side round loop (IterateBestMoves inside a graph WHILE node).
// ---------------------------------------------------------------------------
__global__ void RoundBeginKernel(RoundState* rs) { rs->stamp += 1; }

// End of a round: accounts it (the frontier it evaluated, its movers), sets
// the next round's frontier and whether the loop goes on -- the next frontier
// is non-empty (ALL_MOVE: n > 0, every vertex again) and rounds are left.
__global__ void RoundEndKernel(RoundState* rs, DevCounters* ctr, cudaGraphConditionalHandle loop, uint32_t num_inner,
                               int all_move, uint32_t n, uint64_t m, uint64_t binned) {
  ctr->rounds += 1;
  ctr->edge_visits += rs->front_edges;
  ctr->vertex_visits += rs->front_size;
  ctr->visited += rs->visited;
  ctr->sync_moves += ctr->movers;
  bool next;
  if (all_move) {
    next = n > 0;
    rs->front_all = 1;
    rs->front_edges = m;
    rs->front_size = n;
    rs->visited = binned;
  } else {
    next = ctr->frontier > 0;
    rs->front_all = 0;
    rs->front_val = rs->stamp;
    rs->front_edges = ctr->pend_edges;
    rs->front_size = ctr->frontier;
    rs->visited = ctr->frontier;
  }
  if (next) ctr->level_moved = 1;
  rs->iter += 1;
  cudaGraphSetConditional(loop, (next && rs->iter < num_inner) ? 1u : 0u);
}

// Per-graph bookkeeping of a union round in the device-side loop (after the
// round's per-graph frontier flags): every graph still in the loop counts
// the round and its frontier's entries; a graph whose next frontier is empty
// leaves the loop, as it would alone.  ub: in_loop[B] (bytes) | moved[B]
// (bytes); pend/ev: per-graph frontier entries and edge visits; rounds.
struct UnionBook {
  uint8_t* in_loop;
  uint8_t* moved;
  unsigned long long* pend;
  unsigned long long* ev;
  uint32_t* rounds;
};

__global__ void UnionRoundEndKernel(uint32_t B, const RoundState* rs, int all_move, UnionBook ub,
                                    const uint32_t* __restrict__ gflags, const unsigned long long* __restrict__ gedges) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < B; j += gridDim.x * blockDim.x) {
    if (!ub.in_loop[j]) continue;
    ub.rounds[j] += 1;
    ub.ev[j] += ub.pend[j];
    if (all_move) {
      ub.moved[j] = 1;
    } else if (gflags[j] == rs->stamp) {
      ub.moved[j] = 1;
      ub.pend[j] = gedges[j];
    } else {
      ub.in_loop[j] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Level state (one ClusteringHelper + its graph).
// ---------------------------------------------------------------------------
struct Level {
  const DevGraph* g = nullptr;
  std::unique_ptr<DevGraph> own;
  DBuf<uint32_t> C, s;
  DBuf<double> k, K;
  DBuf<float> Kf;  // FilterF32(K)
  DBuf<float> kf;  // FilterF32(k)
  // Vertices the best-move kernels visit: the degree > 0 bins, or all
  // vertices when isolated ones may sit in shared clusters (level 0 started
  // from given labels).  From singletons an isolated vertex never moves:
  // its value is 0 and no vertex can join it.
  const BinSet* bins = nullptr;
  bool int_mode = false;
  // Subclustering: the vertex of the next level every vertex became (its
  // subcluster id); empty when the level was compressed by cluster id.
  DBuf<uint32_t> sub;
  // Per-vertex resolution (unions of graphs with different resolutions).
  DBuf<double> vres;
  DBuf<float> vres32;
};

struct RunResult {
  uint64_t edge_visits = 0;
  uint64_t vertex_visits = 0;
  uint64_t moves = 0;
  int32_t levels = 0;
  int32_t rounds = 0;
  int32_t refine_passes = 0;
  uint64_t algo_bytes = 0;
  // CompressGraph: (12 or 8) m + 8 m' + 20 n + 16 n' per contraction.
  uint64_t algo_bytes_compress = 0;
};

// INT mode with every neighbour-cluster sum below 2^30 in magnitude (so
// sums and their differences fit in int): a cluster sum is at most the
// row's sum of |w| plus degree * |offset|.
bool NarrowSums(const DevGraph& g, double offset) {
  return g.row_abs_bound + std::fabs(offset) * static_cast<double>(g.max_deg) < 1073741824.0;
}

// Sequential waves of an async round (see Round); 16 keeps the mean quality
// over seeds within 0.15% of the reference restatement on SBM, RMAT and
// LFR-like graphs, where one wave loses up to 1.6%.
constexpr uint32_t kAsyncWaves = 16;

// Algorithmic bytes of one contraction (CompressGraph): read the CSR and
// gather C per entry ((4 + 4) or (4 + 4 + 4) B), write CSR' (8 B per entry),
// read C and k per vertex (12 B) plus the offsets (8 B), write the offsets'
// and k' (16 B per new vertex).
uint64_t CompressBytes(const DevGraph& in, const DevGraph& out) {
  return (in.w.p ? 12ull : 8ull) * in.m + 8ull * out.m + 20ull * in.n + 16ull * out.n;
}

bool IntModeFor(const DevGraph& g, double offset) {
  if (!g.integral) return false;
  if (offset != std::floor(offset) || std::fabs(offset) > 4194304.0) return false;
  return g.max_abs_w + std::fabs(offset) <= 4194304.0;  // 2^22
}

class Engine {
 public:
  Engine(Context* ctx, const pcc_config& cfg, bool int_nw)
      : ctx_(ctx), cfg_(cfg), int_nw_(int_nw), timer_(ctx), fam_timer_(ctx) {
    ctx_->fam_timer = &fam_timer_;
    for (int f = 0; f < kNumFamilies; ++f) ctx_->fam_launches[f] = 0;
  }
  ~Engine() { ctx_->fam_timer = nullptr; }
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  Status Init(uint32_t n_max, uint32_t max_deg) {
    n_max_ = n_max;
    const uint64_t nn = std::max<uint64_t>(n_max, 1);
    PCC_RETURN_IF_ERROR(moves_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(movers_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(moved_stamp_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(mod_stamp_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(next_stamp_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(new_stamp_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(aux_stamp_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(moved_stamp_.Zero());
    PCC_RETURN_IF_ERROR(mod_stamp_.Zero());
    PCC_RETURN_IF_ERROR(next_stamp_.Zero());
    PCC_RETURN_IF_ERROR(new_stamp_.Zero());
    PCC_RETURN_IF_ERROR(aux_stamp_.Zero());
    PCC_RETURN_IF_ERROR(zero_ids_.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(new_list_.Alloc(ctx_, nn));

    if (cfg_.async) {
      PCC_RETURN_IF_ERROR(free_ids_.Alloc(ctx_, nn));
      PCC_RETURN_IF_ERROR(free_ctr_.Alloc(ctx_, 2));
      if (cfg_.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES) {
        PCC_RETURN_IF_ERROR(sm_front_.Alloc(ctx_, nn));
        PCC_RETURN_IF_ERROR(sm_moved_.Alloc(ctx_, nn));
        PCC_RETURN_IF_ERROR(sm_dummy_.Alloc(ctx_, nn));
        PCC_RETURN_IF_ERROR(sm_front_.Zero());
        PCC_RETURN_IF_ERROR(sm_moved_.Zero());
      }
    }
    PCC_RETURN_IF_ERROR(ctr_.Alloc(ctx_, 1));
    PCC_RETURN_IF_ERROR(ctr_.Zero());
    PCC_RETURN_IF_ERROR(rs_.Alloc(ctx_, 1));
    // Scan scratch for every level (no allocation inside a captured round).
    PCC_RETURN_IF_ERROR(scan_tiles_.Reserve(ctx_, (nn + kScanTile - 1) / kScanTile + 1));
    (void)max_deg;
    return Status::Ok();
  }

  // Async mode: the free-id list of a level (or refinement pass) starts as
  // the ids of its empty clusters (none from singletons).
  Status SeedFreeIds(uint32_t n, const uint32_t* s) {
    if (!cfg_.async || n == 0) return Status::Ok();
    PCC_CUDA(cudaMemsetAsync(free_ids_.p, 0xFF, sizeof(uint32_t) * n, ctx_->stream));
    PCC_RETURN_IF_ERROR(free_ctr_.Zero());
    return ScanApply<uint32_t>(ctx_, n, EmptyClusterInput{s}, StoreIndexIfSet{free_ids_.p}, scan_tiles_,
                               free_ctr_.p);
  }

  // Builds level state over graph g: singletons with node weights k (device,
  // copied) or from initial labels.
  Status MakeLevel(const DevGraph* g, std::unique_ptr<DevGraph> own, const double* d_k, bool k_is_ones,
                   const uint32_t* d_labels, std::unique_ptr<Level>* out) {
    auto L = std::make_unique<Level>();
    L->g = g;
    L->own = std::move(own);
    const uint32_t n = g->n;
    const uint64_t nn = std::max<uint64_t>(n, 1);
    PCC_RETURN_IF_ERROR(L->C.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(L->s.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(L->k.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(L->K.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(L->Kf.Alloc(ctx_, nn));
    PCC_RETURN_IF_ERROR(L->kf.Alloc(ctx_, nn));
    if (n) {
      if (k_is_ones || !d_k) {
        FillF64Kernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, 1.0, L->k.p); PCC_COUNT(1);
      } else {
        PCC_CUDA(cudaMemcpyAsync(L->k.p, d_k, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx_->stream));
      }
      if (d_labels) {
        PCC_CUDA(cudaMemcpyAsync(L->C.p, d_labels, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx_->stream));
        PCC_RETURN_IF_ERROR(L->s.Zero());
        PCC_RETURN_IF_ERROR(L->K.Zero());
        AccumulateClustersKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, L->C.p, L->k.p, L->s.p, L->K.p); PCC_COUNT(1);
      } else {
        SingletonsKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, L->k.p, L->C.p, L->s.p, L->K.p); PCC_COUNT(1);
      }
      RefreshKfKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, L->K.p, L->Kf.p, nullptr, 0, nullptr); PCC_COUNT(1);
      NodeKfKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, L->k.p, L->kf.p); PCC_COUNT(1);
      PCC_RETURN_IF_ERROR(LaunchCheck());
    }
    L->int_mode = IntModeFor(*g, cfg_.edge_weight_offset);
    PCC_RETURN_IF_ERROR(SeedFreeIds(n, L->s.p));
    if (un_ && un_->d_res.p && n) {
      PCC_RETURN_IF_ERROR(L->vres.Alloc(ctx_, n));
      PCC_RETURN_IF_ERROR(L->vres32.Alloc(ctx_, n));
      GraphResKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, un_->d_vbase.p, un_->B, un_->d_res.p,
                                                                un_->d_res32.p, L->vres.p, L->vres32.p);
      PCC_COUNT(1);
    }
    if (d_labels) {
      PCC_RETURN_IF_ERROR(EnsureAllBins(ctx_, g));
      L->bins = &g->bins_all;
    } else {
      L->bins = &g->bins;
    }
    PCC_RETURN_IF_ERROR(EnsureHubPlan(ctx_, g));
    PCC_RETURN_IF_ERROR(AllocHubState(ctx_, *g->hub_plan, &hub_state_));
    *out = std::move(L);
    return Status::Ok();
  }

  // The work of one best-move round, enqueued on the context stream with no
  // host read: counter resets, the best-move kernels, the application of the
  // moves (sync) and, unless ALL_MOVE, the next frontier with its size and
  // degree sum in the counters.  rs == null: the stamp is stamp_ and the
  // frontier is front_stamp (0: every vertex); else both come from rs in
  // device memory (rounds of a device-side loop).
  Status EnqueueRound(Level* L, uint32_t front_stamp, uint64_t front_size, const RoundState* rs) {
    const DevGraph& g = *L->g;
    const uint32_t n = g.n;
    // Reset per-round counters: frontier, movers, new_movers, marked, pend_edges.
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->frontier, 0, sizeof(uint32_t) * 4, ctx_->stream));
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->pend_edges, 0, sizeof(unsigned long long), ctx_->stream));

    BMArgs a{};
    a.n = n;
    a.off = g.off.p;
    a.nbr = g.nbr.p;
    a.w = g.wp();
    a.C = L->C.p;
    a.s = L->s.p;
    a.k = L->k.p;
    a.K = L->K.p;
    a.Kf = L->Kf.p;
    a.kf = L->kf.p;
    a.int_nw = int_nw_ ? 1 : 0;
    a.narrow = (L->int_mode && NarrowSums(g, cfg_.edge_weight_offset)) ? 1 : 0;
    a.res = cfg_.resolution;
    a.res32 = FilterF32(cfg_.resolution);
    a.offset = cfg_.edge_weight_offset;
    a.ioffset = static_cast<int32_t>(cfg_.edge_weight_offset);
    a.stamp = stamp_;
    a.moves = moves_.p;
    a.moved_stamp = moved_stamp_.p;
    a.movers = movers_.p;
    a.ctr = ctr_.p;
    a.async = cfg_.async ? 1 : 0;
    a.s_mut = L->s.p;
    a.K_mut = L->K.p;
    a.C_mut = L->C.p;
    a.moved_cluster_stamp = mod_stamp_.p;
    if (cfg_.async) {
      a.free_ids = free_ids_.p;
      a.free_ctr = free_ctr_.p;
      a.free_cap = n;
    }
    a.rs = rs;
    a.vres = L->vres.p;
    a.vres32 = L->vres32.p;
    a.front_stamp = (rs || front_stamp) ? next_stamp_.p : nullptr;
    a.front_val = front_stamp;
    const BinSet& bins = *L->bins;
    timer_.Begin(kPhaseBestMoves);
    // Async rounds run in waves: the reference's AsyncMove applies each move
    // before most other vertices of the round are evaluated (a handful of CPU
    // threads in flight); evaluating the whole frontier at once on the GPU
    // would decide every vertex on the round's initial state.  Each wave sees
    // the moves of the waves before it.
    a.waves = cfg_.async ? kAsyncWaves : 1;
    a.wave_salt = static_cast<uint32_t>(cfg_.random_seed * 0x9E3779B97F4A7C15ull >> 32) ^ (stamp_ * 0x85EBCA6Bu);

    if (!cfg_.async && !ctx_->detailed_timing && ctx_->overlap_families) {
      PCC_RETURN_IF_ERROR(OverlappedBestMoves(L, a));
    } else {
      for (uint32_t w = 0; w < a.waves; ++w) {
        a.wave = w;
        PCC_RETURN_IF_ERROR(LaunchBestMoves(ctx_, a, bins.list.p, bins.counts.p, bins.counts.p + kNumBins,
                                            bins.host_counts, L->int_mode, g.max_deg));
        PCC_RETURN_IF_ERROR(LaunchHubBestMoves(ctx_, a, *g.hub_plan, hub_state_, L->int_mode, a.narrow != 0));
      }
    }
    timer_.End(kPhaseBestMoves);

    timer_.Begin(kPhaseApply);
    if (!cfg_.async) {
      ApplyArgs ap{n, L->C.p, L->s.p, L->k.p, L->K.p, moves_.p, movers_.p, mod_stamp_.p, new_stamp_.p, stamp_,
                   ctr_.p, rs};
      const unsigned grid = GridFor(ctx_, rs ? uint64_t(n) : front_size);
      ApplyMoveKernel<<<grid, kT, 0, ctx_->stream>>>(ap); PCC_COUNT(1);
      PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, n, ZeroSizeInput{L->s.p, ctr_.p},
                                              StoreIndexIfSet{zero_ids_.p}, scan_tiles_,
                                              un_ ? zcount_.p : static_cast<uint32_t*>(nullptr)));
      PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, n, NewMoverInput{new_stamp_.p, stamp_, ctr_.p, rs},
                                              StoreIndexIfSet{new_list_.p}, scan_tiles_,
                                              static_cast<uint32_t*>(nullptr)));
      if (un_) {
        AssignNewUnionKernel<<<grid, kT, 0, ctx_->stream>>>(ap, zero_ids_.p, zcount_.p, new_list_.p,
                                                             un_->d_vbase.p, un_->B); PCC_COUNT(1);
      } else {
        AssignNewKernel<<<grid, kT, 0, ctx_->stream>>>(ap, zero_ids_.p, new_list_.p); PCC_COUNT(1);
      }
      if (n) {
        RefreshKfKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, L->K.p, L->Kf.p, mod_stamp_.p, stamp_, rs);
        PCC_COUNT(1);
      }
      PCC_RETURN_IF_ERROR(LaunchCheck());
      if (cfg_.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES) PCC_RETURN_IF_ERROR(WholeClusterMoves(L));
    } else if (cfg_.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES) {
      PCC_RETURN_IF_ERROR(AsyncWholeClusterMoves(L, a));
    }
    timer_.End(kPhaseApply);
    if (cfg_.move_method == PCC_ALL_MOVE) return Status::Ok();

    // Neighbourhood of the marked set (edgeMap), rows taken from the static
    // degree bins with a marked-row predicate, then the next frontier's size.
    timer_.Begin(kPhaseFrontier);
    const StampValue sv{stamp_, rs};
    if (cfg_.move_method == PCC_NBHR_CLUSTER_MOVE) {
      LaunchPush(ctx_, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                 g.nbr.p, next_stamp_.p, sv, PredModifiedCluster{L->C.p, mod_stamp_.p, stamp_, rs});  // rows with d > 0
    } else {
      LaunchPush(ctx_, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                 g.nbr.p, next_stamp_.p, sv, PredStamp{moved_stamp_.p, stamp_, rs});
    }
    if (n) {
      CountDegreesKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, g.off.p, PredStamp{next_stamp_.p, stamp_, rs},
                                                                    &ctr_.p->pend_edges, &ctr_.p->frontier);
      PCC_COUNT(1);
      if (un_) {
        PCC_RETURN_IF_ERROR(gedges_.Zero());
        GraphFrontierKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, g.off.p, next_stamp_.p, stamp_, rs,
                                                                       un_->d_vbase.p, un_->B, gflags_.p,
                                                                       gedges_.p); PCC_COUNT(1);
      }
    }
    PCC_RETURN_IF_ERROR(LaunchCheck());
    timer_.End(kPhaseFrontier);
    if (ctx_->detailed_timing && !rs && n) {
      // Untimed: the rows the push expanded and their entries, for the
      // frontier phase's algorithmic bytes.
      if (cfg_.move_method == PCC_NBHR_CLUSTER_MOVE) {
        const PredMarkedRow<PredModifiedCluster> pred{g.off.p, PredModifiedCluster{L->C.p, mod_stamp_.p, stamp_, rs}};
        CountDegreesKernel<PredMarkedRow<PredModifiedCluster>, unsigned long long>
            <<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, g.off.p, pred, &ctr_.p->push_entries, &ctr_.p->push_rows);
      } else {
        const PredMarkedRow<PredStamp> pred{g.off.p, PredStamp{moved_stamp_.p, stamp_, rs}};
        CountDegreesKernel<PredMarkedRow<PredStamp>, unsigned long long>
            <<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, g.off.p, pred, &ctr_.p->push_entries, &ctr_.p->push_rows);
      }
      PCC_COUNT(1);
      PCC_RETURN_IF_ERROR(LaunchCheck());
    }
    return Status::Ok();
  }

  // The best-move families of one synchronous round as parallel branches:
  // big hubs, warps and small hubs on side streams forked from the context
  // stream, the lane groups on the context stream, then a join.  The
  // families read the same round state and write disjoint per-vertex
  // outputs (moves, moved stamps) plus atomic counters and the atomic
  // movers list, so their order does not matter.  The join runs even when
  // a launch failed, so a stream capture is never left with unjoined work.
  Status OverlappedBestMoves(Level* L, const BMArgs& a) {
    const DevGraph& g = *L->g;
    const BinSet& bins = *L->bins;
    PCC_RETURN_IF_ERROR(ctx_->EnsureSideStreams());
    PCC_CUDA(cudaEventRecord(ctx_->fork_ev, ctx_->stream));
    for (int i = 0; i < Context::kSideStreams; ++i) PCC_CUDA(cudaStreamWaitEvent(ctx_->side[i], ctx_->fork_ev, 0));
    Status st;
    {
      OnSideStream on(ctx_, 0);
      st = LaunchHubBestMoves(ctx_, a, *g.hub_plan, hub_state_, L->int_mode, a.narrow != 0, kLaunchBigHubs);
    }
    if (st.ok()) {
      OnSideStream on(ctx_, 1);
      st = LaunchBestMoves(ctx_, a, bins.list.p, bins.counts.p, bins.counts.p + kNumBins, bins.host_counts,
                           L->int_mode, g.max_deg, kLaunchWarps);
    }
    if (st.ok()) {
      OnSideStream on(ctx_, 2);
      st = LaunchHubBestMoves(ctx_, a, *g.hub_plan, hub_state_, L->int_mode, a.narrow != 0, kLaunchSmallHubs);
    }
    if (st.ok())
      st = LaunchBestMoves(ctx_, a, bins.list.p, bins.counts.p, bins.counts.p + kNumBins, bins.host_counts,
                           L->int_mode, g.max_deg, kLaunchGroups);
    for (int i = 0; i < Context::kSideStreams; ++i) {
      PCC_CUDA(cudaEventRecord(ctx_->join_ev[i], ctx_->side[i]));
      PCC_CUDA(cudaStreamWaitEvent(ctx_->stream, ctx_->join_ev[i], 0));
    }
    return st;
  }

  // Whole-cluster moves after the round's vertex moves (DEFAULT_CLUSTER_MOVES,
  // parallel-correlation-clusterer.cc:167-297): the moving clusters'
  // members go through the same apply as vertex movers, and the clusters it
  // modifies carry this round's stamp, so the NBHR_CLUSTER_MOVE frontier
  // sees them (moved_clusters |= additional_moved_clusters).  Host-driven
  // rounds only (the step reads sizes on the host).
  Status WholeClusterMoves(Level* L) {
    const DevGraph& g = *L->g;
    const uint32_t n = g.n;
    DevCounters hc;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    res_.moves += hc.movers;  // the vertex movers; the caller adds the cluster movers
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->movers, 0, sizeof(uint32_t), ctx_->stream));
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->new_movers, 0, sizeof(uint32_t), ctx_->stream));
    // The vertex movers' new-cluster marks of this round are spent (0 is no stamp).
    PCC_CUDA(cudaMemsetAsync(new_stamp_.p, 0, sizeof(uint32_t) * n, ctx_->stream));
    // Integral entry values whose every partial sum stays below 2^53 sum
    // exactly in any order.
    const bool exact = L->int_mode && static_cast<double>(g.m) * (g.max_abs_w + std::fabs(cfg_.edge_weight_offset)) <
                                          9007199254740992.0;
    PCC_RETURN_IF_ERROR(FindClusterMoves(ctx_, g, L->C.p, L->k.p, L->K.p, cfg_.resolution, cfg_.edge_weight_offset,
                                         exact, moves_.p, movers_.p, ctr_.p));
    ApplyArgs ap{n, L->C.p, L->s.p, L->k.p, L->K.p, moves_.p, movers_.p, mod_stamp_.p, new_stamp_.p, stamp_,
                 ctr_.p, nullptr};
    const unsigned grid = GridFor(ctx_, n);
    ApplyLeaveKernel<<<grid, kT, 0, ctx_->stream>>>(ap); PCC_COUNT(1);
    ApplyJoinKernel<<<grid, kT, 0, ctx_->stream>>>(ap); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, n, ZeroSizeInput{L->s.p, ctr_.p}, StoreIndexIfSet{zero_ids_.p},
                                            scan_tiles_, static_cast<uint32_t*>(nullptr)));
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, n, NewMoverInput{new_stamp_.p, stamp_, ctr_.p, nullptr},
                                            StoreIndexIfSet{new_list_.p}, scan_tiles_,
                                            static_cast<uint32_t*>(nullptr)));
    AssignNewKernel<<<grid, kT, 0, ctx_->stream>>>(ap, zero_ids_.p, new_list_.p); PCC_COUNT(1);
    RefreshKfKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, L->K.p, L->Kf.p, mod_stamp_.p, stamp_, nullptr);
    PCC_COUNT(1);
    return LaunchCheck();
  }

  // The async branch of the whole-cluster moves (parallel-correlation-
  // clusterer.cc:255-268): every cluster's members, fixed after the round's
  // vertex moves, move as a set (AsyncSetMoves); one-member sets take the
  // vertex AsyncMove through the async best-move kernels, evaluated over the
  // wave's marked vertices with their moved flags redirected.
  Status AsyncWholeClusterMoves(Level* L, const BMArgs& round_args) {
    const DevGraph& g = *L->g;
    const BinSet& bins = *L->bins;
    const bool exact = L->int_mode && static_cast<double>(g.m) * (g.max_abs_w + std::fabs(cfg_.edge_weight_offset)) <
                                          9007199254740992.0;
    SetMoveArgs sm{};
    sm.g = &g;
    sm.C = L->C.p;
    sm.s = L->s.p;
    sm.k = L->k.p;
    sm.K = L->K.p;
    sm.res = cfg_.resolution;
    sm.offset = cfg_.edge_weight_offset;
    sm.exact_sums = exact;
    sm.waves = kAsyncWaves;
    sm.salt = round_args.wave_salt ^ 0xA511E9B3u;
    sm.free_ids = free_ids_.p;
    sm.free_ctr = free_ctr_.p;
    sm.free_cap = g.n;
    sm.mod_stamp = mod_stamp_.p;
    sm.stamp = stamp_;
    sm.ctr = ctr_.p;
    sm.aux_front = sm_front_.p;
    sm.aux_moved = sm_moved_.p;
    sm.aux_base = sm_val_ + 1;
    sm_val_ += kAsyncWaves;
    auto vertex_moves = [&](uint32_t val) -> Status {
      BMArgs b = round_args;
      b.waves = 1;
      b.wave = 0;
      b.rs = nullptr;
      b.front_stamp = sm_front_.p;
      b.front_val = val;
      b.stamp = val;
      b.moved_stamp = sm_moved_.p;
      b.moved_cluster_stamp = sm_dummy_.p;
      PCC_RETURN_IF_ERROR(LaunchBestMoves(ctx_, b, bins.list.p, bins.counts.p, bins.counts.p + kNumBins,
                                          bins.host_counts, L->int_mode, g.max_deg));
      return LaunchHubBestMoves(ctx_, b, *g.hub_plan, hub_state_, L->int_mode, b.narrow != 0);
    };
    return AsyncSetMoves(ctx_, sm, vertex_moves);
  }

  // One best-move round over `front` (host_counts known), driven from the
  // host.  Builds the next frontier unless ALL_MOVE.  Returns whether the
  // next frontier is non-empty (local_moved).
  // front_stamp == 0: all vertices; else vertices with next_stamp == it.
  Status Round(Level* L, uint32_t front_stamp, uint64_t front_edges, uint64_t front_size, bool* next_nonempty,
               uint32_t* next_front_stamp, uint64_t* next_edges, uint64_t* next_size) {
    const DevGraph& g = *L->g;
    const uint32_t n = g.n;
    stamp_++;
    res_.rounds++;
    res_.edge_visits += front_edges;
    res_.vertex_visits += front_size;
    // Isolated vertices outside L->bins are not visited by any kernel.
    const uint64_t visited = front_stamp ? front_size : L->bins->size;
    res_.algo_bytes += (g.w.p ? 12ull : 8ull) * front_edges + 40ull * visited;
    PCC_RETURN_IF_ERROR(EnqueueRound(L, front_stamp, front_size, nullptr));
    DevCounters hc;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    if (un_ && cfg_.move_method != PCC_ALL_MOVE) {
      PCC_RETURN_IF_ERROR(gflags_.ToHost(h_gflags_.data(), un_->B));
      PCC_RETURN_IF_ERROR(gedges_.ToHost(h_gedges_.data(), un_->B));
    }
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    if (!cfg_.async) res_.moves += hc.movers;
    if (cfg_.move_method == PCC_ALL_MOVE) {
      *next_nonempty = n > 0;
      *next_front_stamp = 0;
      *next_size = n;
      *next_edges = g.m;
      return Status::Ok();
    }
    *next_front_stamp = stamp_;
    *next_size = hc.frontier;
    *next_edges = hc.pend_edges;
    *next_nonempty = hc.frontier > 0;
    return Status::Ok();
  }

  // IterateBestMoves with the round loop on the device: one round is
  // captured into the body of a graph WHILE node, RoundEndKernel decides
  // whether it runs again, and the host reads the counters once the loop is
  // over.  Same kernels and arguments as the host-driven loop, with the stamp
  // and the frontier taken from rs_.
  // init: the round-0 frontier (null: every vertex); book: the union's
  // per-graph bookkeeping (null: one graph).  *fell_back (when given) is set
  // instead of running the host-driven loop if CUDA graphs are unavailable.
  Status IterateDevice(Level* L, int64_t num_inner, bool* moved_out, const RoundState* init = nullptr,
                       const UnionBook* book = nullptr, bool* fell_back = nullptr) {
    const DevGraph& g = *L->g;
    PCC_RETURN_IF_ERROR(PrepareBestMoveKernels());
    PCC_RETURN_IF_ERROR(PrepareHubKernels());
    PCC_RETURN_IF_ERROR(ctx_->EnsureSideStreams());
    RoundState h{};
    if (init) {
      h = *init;
    } else {
      h.front_all = 1;
      h.front_edges = g.m;
      h.front_size = g.n;
      h.visited = L->bins->size;
    }
    h.stamp = stamp_;  // RoundBeginKernel increments it first
    h.iter = 0;
    PCC_RETURN_IF_ERROR(rs_.FromHost(&h, 1));
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->level_moved, 0, sizeof(uint32_t) * 2, ctx_->stream));  // level_moved, rounds
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->edge_visits, 0, sizeof(unsigned long long) * 2, ctx_->stream));
    PCC_CUDA(cudaMemsetAsync(&ctr_.p->sync_moves, 0, sizeof(unsigned long long) * 2, ctx_->stream));

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&] {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
    };
    PCC_CUDA(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle loop;
    cudaError_t e = cudaGraphConditionalHandleCreate(&loop, graph, num_inner > 0 ? 1u : 0u,
                                                     cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    if (e != cudaSuccess) {
      cleanup();
      cudaGetLastError();
      ctx_->graphs_failed = true;
      if (fell_back) {
        *fell_back = true;
        return Status::Ok();
      }
      return IterateBestMoves(L, num_inner, moved_out);
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const uint64_t launches0 = LaunchCounter();
    const uint64_t fam0[kNumFamilies] = {ctx_->fam_launches[0], ctx_->fam_launches[1], ctx_->fam_launches[2],
                                         ctx_->fam_launches[3]};
    PhaseTimer* fam = ctx_->fam_timer;
    ctx_->fam_timer = nullptr;
    timer_.enabled = false;
    if (cudaStreamBeginCaptureToGraph(ctx_->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess) {
      timer_.enabled = true;
      ctx_->fam_timer = fam;
      cleanup();
      cudaGetLastError();
      ctx_->graphs_failed = true;
      if (fell_back) {
        *fell_back = true;
        return Status::Ok();
      }
      return IterateBestMoves(L, num_inner, moved_out);
    }
    RoundBeginKernel<<<1, 1, 0, ctx_->stream>>>(rs_.p); PCC_COUNT(1);
    Status st = EnqueueRound(L, 0, g.n, rs_.p);
    if (book && st.ok()) {
      UnionRoundEndKernel<<<Blocks(un_->B, 256, 1024), 256, 0, ctx_->stream>>>(
          un_->B, rs_.p, cfg_.move_method == PCC_ALL_MOVE ? 1 : 0, *book, gflags_.p, gedges_.p);
      PCC_COUNT(1);
    }
    RoundEndKernel<<<1, 1, 0, ctx_->stream>>>(rs_.p, ctr_.p, loop, static_cast<uint32_t>(num_inner),
                                              cfg_.move_method == PCC_ALL_MOVE ? 1 : 0, g.n, g.m, L->bins->size);
    PCC_COUNT(1);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(ctx_->stream, &captured);
    timer_.enabled = true;
    ctx_->fam_timer = fam;
    const uint64_t body_launches = LaunchCounter() - launches0;
    uint64_t body_fam[kNumFamilies];
    for (int f = 0; f < kNumFamilies; ++f) body_fam[f] = ctx_->fam_launches[f] - fam0[f];
    if (!st.ok()) {
      cleanup();
      return st;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, ctx_->stream);
    if (e != cudaSuccess) {
      cleanup();
      cudaGetLastError();
      return MakeError(PCC_INTERNAL, std::string("device round loop: ") + cudaGetErrorString(e));
    }
    DevCounters hc;
    RoundState hr;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    PCC_RETURN_IF_ERROR(rs_.ToHost(&hr, 1));
    const Status ss = Sync(ctx_);
    cleanup();
    PCC_RETURN_IF_ERROR(ss);
    stamp_ = hr.stamp;
    res_.rounds += static_cast<int32_t>(hc.rounds);
    res_.edge_visits += hc.edge_visits;
    res_.vertex_visits += hc.vertex_visits;
    res_.algo_bytes += (g.w.p ? 12ull : 8ull) * hc.edge_visits + 40ull * hc.visited;
    res_.moves += hc.sync_moves;
    // Launch counts: the captured round once per executed round.
    if (hc.rounds > 1) {
      LaunchCounter() += body_launches * (hc.rounds - 1);
      for (int f = 0; f < kNumFamilies; ++f) ctx_->fam_launches[f] += body_fam[f] * (hc.rounds - 1);
    }
    *moved_out = hc.level_moved != 0;
    return Status::Ok();
  }

  // The round loop of one level: on the device when it can be (synchronous
  // moves, one graph, no detailed timing), else driven from the host.
  Status Iterate(Level* L, int64_t num_inner, bool* moved_out) {
    if (!cfg_.async && !un_ && !ctx_->detailed_timing && !ctx_->graphs_failed &&
        cfg_.clustering_moves_method == PCC_LOUVAIN && L->g->m >= ctx_->device_loop_min_entries)
      return IterateDevice(L, num_inner, moved_out);
    return IterateBestMoves(L, num_inner, moved_out);
  }

  // IterateBestMoves (parallel-correlation-clusterer.cc:340-365).
  Status IterateBestMoves(Level* L, int64_t num_inner, bool* moved_out) {
    bool moved = false;
    bool local_moved = true;
    uint32_t front = 0;  // all vertices
    uint64_t front_edges = L->g->m, front_size = L->g->n;
    for (int64_t it = 0; it < num_inner && local_moved; ++it) {
      bool next = false;
      PCC_RETURN_IF_ERROR(Round(L, front, front_edges, front_size, &next, &front, &front_edges, &front_size));
      local_moved = next;
      moved |= local_moved;
    }
    *moved_out = moved;
    return Status::Ok();
  }

  // RefineClusters_subroutine (parallel-correlation-clusterer.cc:476-629).
  // d_k: device node weights or null (all 1); d_init: device labels or null.
  // On success d_out (device uint32[n]) holds the final dense labels.
  Status Run(const DevGraph& g0, const double* d_k, const uint32_t* d_init, uint32_t* d_out,
             uint32_t* num_clusters) {
    int64_t num_iterations = 0, num_inner = 0;
    if (cfg_.clustering_moves_method == PCC_LOUVAIN) {
      num_iterations = cfg_.louvain_num_iterations > 0 ? cfg_.louvain_num_iterations : 10;
      num_inner = cfg_.louvain_num_inner_iterations > 0 ? cfg_.louvain_num_inner_iterations : 10;
    } else if (cfg_.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES) {
      // One level of up to num_iterations rounds (:487-492), each with
      // whole-cluster moves after the vertex moves.
      num_iterations = 1;
      num_inner = cfg_.num_iterations > 0 ? cfg_.num_iterations : 20;
    } else {
      return MakeError(PCC_UNIMPLEMENTED,
                       "Correlation clustering moves must be DEFAULT_CLUSTER_MOVES or LOUVAIN.");
    }
    const int sub_method = cfg_.subclustering_method;
    if (sub_method < PCC_NONE_SUBCLUSTERING || sub_method > PCC_SLOW_CONNECTIVITY_SUBCLUSTERING)
      return MakeError(PCC_UNIMPLEMENTED, "unknown subclustering_method");
    if (sub_method != PCC_NONE_SUBCLUSTERING && cfg_.clustering_moves_method == PCC_DEFAULT_CLUSTER_MOVES)
      return MakeError(PCC_UNIMPLEMENTED, "subcluster moves inside DEFAULT_CLUSTER_MOVES rounds are not available");
    const bool subclusters = sub_method != PCC_NONE_SUBCLUSTERING;
    const bool refine = cfg_.refine != 0;
    const uint32_t n = g0.n;
    PCC_RETURN_IF_ERROR(Init(n, g0.max_deg));
    bool vertex_ids = false;  // no refine, subclusters: cluster_ids hold vertex ids of the current level

    std::vector<std::unique_ptr<Level>> rec;
    if (refine) rec.resize(static_cast<size_t>(num_iterations));
    std::unique_ptr<Level> helper;
    PCC_RETURN_IF_ERROR(MakeLevel(&g0, nullptr, d_k, d_k == nullptr, d_init, &helper));
    DBuf<uint32_t> cluster_ids;
    PCC_RETURN_IF_ERROR(cluster_ids.Alloc(ctx_, std::max<uint64_t>(n, 1)));
    if (n) IotaKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p); PCC_COUNT(1);

    int64_t iter = 0;
    for (iter = 0; iter < num_iterations; ++iter) {
      bool moved = false;
      PCC_RETURN_IF_ERROR(Iterate(helper.get(), num_inner, &moved));
      if (!moved) {
        iter--;
        break;
      }
      res_.levels++;
      const bool last = iter == num_iterations - 1;
      // Subclustering before compression (CompressSubclusters,
      // parallel-correlation-clusterer.cc:436-474).
      DBuf<uint32_t> sub;
      DBuf<uint64_t> blocks;
      uint32_t nclust = 0;
      uint64_t nsub = 0;
      if (subclusters && !last)
        PCC_RETURN_IF_ERROR(ComputeSubclustersDevice(ctx_, *helper->g, helper->C.p, sub_method, cfg_.resolution,
                                                     cfg_.edge_weight_offset, &sub, &blocks, &nclust, &nsub));
      const uint32_t* map = (subclusters && !last) ? sub.p : helper->C.p;
      if (!refine) {
        if (n) FlattenKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p, map); PCC_COUNT(1);
        vertex_ids = subclusters && !last;
      } else if (last) {
        rec[static_cast<size_t>(iter)] = std::move(helper);
      }
      if (last) break;
      std::unique_ptr<DevGraph> next;
      timer_.Begin(kPhaseCompress);
      PCC_RETURN_IF_ERROR(CompressGraph(ctx_, *helper->g, map, helper->k.p, &next));
      timer_.End(kPhaseCompress);
      res_.algo_bytes_compress += CompressBytes(*helper->g, *next);
      DevGraph* ng = next.get();
      std::unique_ptr<Level> nl;
      if (subclusters) {
        // The next level starts with the subclusters of one cluster together;
        // a cluster's size is its block size, ids beyond the compressed graph
        // (the last block's unused tail) included.
        DBuf<uint32_t> start_labels;
        const uint32_t n2 = ng->n;
        PCC_RETURN_IF_ERROR(start_labels.Alloc(ctx_, std::max<uint64_t>(n2, 1)));
        if (n2) {
          BlockOfKernel<<<GridFor(ctx_, n2), kT, 0, ctx_->stream>>>(n2, blocks.p, nclust, start_labels.p);
          PCC_COUNT(1);
        }
        PCC_RETURN_IF_ERROR(MakeLevel(ng, std::move(next), ng->node_w.p, false, start_labels.p, &nl));
        if (nsub > n2 && nclust > 0) {
          AddU32Kernel<<<1, 1, 0, ctx_->stream>>>(nl->s.p + (nclust - 1), static_cast<uint32_t>(nsub - n2));
          PCC_COUNT(1);
        }
        PCC_RETURN_IF_ERROR(LaunchCheck());
      } else {
        PCC_RETURN_IF_ERROR(MakeLevel(ng, std::move(next), ng->node_w.p, false, nullptr, &nl));
      }
      if (refine) {
        if (subclusters) helper->sub = std::move(sub);
        rec[static_cast<size_t>(iter)] = std::move(helper);
      }
      helper = std::move(nl);
    }
    // No refine, subclusters, and the last level did not move: its starting
    // clustering names the clusters of the vertices cluster_ids now hold.
    if (vertex_ids && n) {
      FlattenKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p, helper->C.p);
      PCC_COUNT(1);
    }

    if (refine && iter > 0) {
      DBuf<uint32_t> flat, rank;
      PCC_RETURN_IF_ERROR(flat.Alloc(ctx_, std::max<uint64_t>(n, 1)));
      PCC_RETURN_IF_ERROR(rank.Alloc(ctx_, std::max<uint64_t>(n, 1)));
      for (int64_t i = iter - 1; i >= 0; --i) {
        Level* Li = rec[static_cast<size_t>(i)].get();
        Level* Lu = rec[static_cast<size_t>(i + 1)].get();
        const uint32_t ni = Li->g->n, nu = Lu->g->n;
        stamp_++;
        if (ni) {
          ProjectKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, Li->sub.p ? Li->sub.p : Li->C.p, Lu->C.p,
                                                                    flat.p, aux_stamp_.p, stamp_); PCC_COUNT(1);
          PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, nu, StampInput{aux_stamp_.p, stamp_},
                                                  StorePrefix<uint32_t>{rank.p}, scan_tiles_,
                                                  static_cast<uint32_t*>(nullptr)));
          GatherKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, flat.p, rank.p, Li->C.p); PCC_COUNT(1);
          PCC_RETURN_IF_ERROR(Li->s.Zero());
          PCC_RETURN_IF_ERROR(Li->K.Zero());
          AccumulateClustersKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, Li->C.p, Li->k.p, Li->s.p,
                                                                                Li->K.p); PCC_COUNT(1);
          RefreshKfKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, Li->K.p, Li->Kf.p, nullptr, 0, nullptr);
          PCC_COUNT(1);
          PCC_RETURN_IF_ERROR(LaunchCheck());
          PCC_RETURN_IF_ERROR(SeedFreeIds(ni, Li->s.p));
        }
        bool moved = false;
        PCC_RETURN_IF_ERROR(Iterate(Li, num_inner, &moved));
        res_.refine_passes++;
        rec[static_cast<size_t>(i + 1)].reset();
      }
      PCC_CUDA(cudaMemcpyAsync(cluster_ids.p, rec[0]->C.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice,
                               ctx_->stream));
    }
    rec.clear();
    helper.reset();
    PCC_RETURN_IF_ERROR(DenseRank(n, cluster_ids.p, d_out, num_clusters));
    DevCounters hc;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    if (hc.error) return MakeError(PCC_INTERNAL, "device error flag " + std::to_string(hc.error));
    res_.moves += hc.moves;
    return Status::Ok();
  }

  // OutputIndicesById as labels: out[i] = rank of ids[i] among distinct ids.
  Status DenseRank(uint32_t n, const uint32_t* ids, uint32_t* out, uint32_t* num_groups) {
    if (n == 0) {
      *num_groups = 0;
      return Status::Ok();
    }
    stamp_++;
    DBuf<uint32_t> rank, tot;
    PCC_RETURN_IF_ERROR(rank.Alloc(ctx_, n));
    PCC_RETURN_IF_ERROR(tot.Alloc(ctx_, 1));
    MarkStampKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, ids, aux_stamp_.p, stamp_); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, n, StampInput{aux_stamp_.p, stamp_},
                                            StorePrefix<uint32_t>{rank.p}, scan_tiles_, tot.p));
    GatherKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, ids, rank.p, out); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(tot.ToHost(num_groups, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    return Status::Ok();
  }

  // ---- Disjoint-union mode -------------------------------------------------
  // What RefineClusters_subroutine would record for one graph run alone.
  struct GraphRun {
    int64_t iter = -1;  // the subroutine's final `iter`
    int32_t levels = 0, rounds = 0, refine_passes = 0;
    uint64_t edge_visits = 0;
  };

  // IterateBestMoves for every graph j with in_loop[j], all in the same
  // rounds.  A graph leaves the loop when its next frontier is empty, as it
  // would alone; its vertices are then in no frontier, so the rounds the
  // other graphs still run do not touch it.  Round 0 visits every vertex when
  // all graphs take part, else the vertices of the taking-part graphs.
  // moved[j] = the graph's IterateBestMoves result.
  Status IterateUnion(Level* L, int64_t num_inner, std::vector<uint8_t> in_loop, std::vector<uint8_t>* moved,
                      std::vector<GraphRun>& gr) {
    const uint32_t B = un_->B;
    const DevGraph& g = *L->g;
    bool all = true, any = false;
    for (uint32_t j = 0; j < B; ++j) {
      all &= in_loop[j] != 0;
      any |= in_loop[j] != 0;
    }
    moved->assign(B, 0);
    if (!any) return Status::Ok();
    if (!all && cfg_.move_method == PCC_ALL_MOVE)
      return MakeError(PCC_INTERNAL, "ALL_MOVE union rounds must include every graph");
    GraphEntriesKernel<<<Blocks(B, kT, 1024), kT, 0, ctx_->stream>>>(B, g.n, un_->d_vbase.p, g.off.p, gedges_.p);
    PCC_COUNT(1);
    const bool device_loop = !ctx_->detailed_timing && !ctx_->graphs_failed && g.m >= ctx_->device_loop_min_entries;
    if (device_loop) {
      // Round-0 per-graph frontier entries, flags and counters on the device.
      PCC_CUDA(cudaMemcpyAsync(ub_pend_.p, gedges_.p, sizeof(unsigned long long) * B, cudaMemcpyDeviceToDevice,
                               ctx_->stream));
      PCC_RETURN_IF_ERROR(ub_flags_.FromHost(in_loop.data(), B));
      PCC_CUDA(cudaMemsetAsync(ub_flags_.p + B, 0, B, ctx_->stream));  // moved
      PCC_RETURN_IF_ERROR(ub_ev_.Zero());
      PCC_RETURN_IF_ERROR(ub_rounds_.Zero());
    }
    PCC_RETURN_IF_ERROR(gedges_.ToHost(h_gent_.data(), B));
    uint32_t front = 0;
    uint64_t fe = g.m, fs = g.n;
    if (!all) {
      for (uint32_t j = 0; j < B; ++j) h_mask_[j] = in_loop[j];
      PCC_RETURN_IF_ERROR(gmask_.FromHost(h_mask_.data(), B));
      const uint32_t s0 = ++stamp_;
      MarkGraphsKernel<<<GridFor(ctx_, g.n), kT, 0, ctx_->stream>>>(g.n, g.off.p, un_->d_vbase.p, B, gmask_.p,
                                                                    next_stamp_.p, s0); PCC_COUNT(1);
      PCC_CUDA(cudaMemsetAsync(&ctr_.p->frontier, 0, sizeof(uint32_t), ctx_->stream));
      PCC_CUDA(cudaMemsetAsync(&ctr_.p->pend_edges, 0, sizeof(unsigned long long), ctx_->stream));
      CountDegreesKernel<<<GridFor(ctx_, g.n), kT, 0, ctx_->stream>>>(g.n, g.off.p, PredStamp{next_stamp_.p, s0},
                                                                      &ctr_.p->pend_edges, &ctr_.p->frontier);
      PCC_COUNT(1);
      DevCounters hc;
      PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
      PCC_RETURN_IF_ERROR(Sync(ctx_));
      front = s0;
      fe = hc.pend_edges;
      fs = hc.frontier;
    } else {
      PCC_RETURN_IF_ERROR(Sync(ctx_));
    }
    if (device_loop) {
      RoundState init{};
      init.front_all = all ? 1 : 0;
      init.front_val = front;
      init.front_edges = fe;
      init.front_size = fs;
      init.visited = all ? L->bins->size : fs;
      const UnionBook book{ub_flags_.p, ub_flags_.p + B, ub_pend_.p, ub_ev_.p, ub_rounds_.p};
      bool fell_back = false, any_moved = false;
      PCC_RETURN_IF_ERROR(IterateDevice(L, num_inner, &any_moved, &init, &book, &fell_back));
      if (!fell_back) {
        std::vector<uint8_t> flags(2 * size_t(B));
        std::vector<unsigned long long> ev(B);
        std::vector<uint32_t> rounds(B);
        PCC_RETURN_IF_ERROR(ub_flags_.ToHost(flags.data(), 2 * size_t(B)));
        PCC_RETURN_IF_ERROR(ub_ev_.ToHost(ev.data(), B));
        PCC_RETURN_IF_ERROR(ub_rounds_.ToHost(rounds.data(), B));
        PCC_RETURN_IF_ERROR(Sync(ctx_));
        for (uint32_t j = 0; j < B; ++j) {
          gr[j].rounds += static_cast<int32_t>(rounds[j]);
          gr[j].edge_visits += ev[j];
          (*moved)[j] = flags[B + j];
        }
        return Status::Ok();
      }
    }
    std::vector<unsigned long long> pend(h_gent_.begin(), h_gent_.begin() + B);
    bool local_moved = true;
    for (int64_t it = 0; it < num_inner && local_moved; ++it) {
      for (uint32_t j = 0; j < B; ++j) {
        if (!in_loop[j]) continue;
        gr[j].rounds++;
        gr[j].edge_visits += pend[j];
      }
      bool next = false;
      PCC_RETURN_IF_ERROR(Round(L, front, fe, fs, &next, &front, &fe, &fs));
      for (uint32_t j = 0; j < B; ++j) {
        if (!in_loop[j]) continue;
        if (cfg_.move_method == PCC_ALL_MOVE) {
          (*moved)[j] = 1;  // local_moved = n > 0 (every round visits every vertex)
        } else if (h_gflags_[j] == stamp_) {
          (*moved)[j] = 1;
          pend[j] = h_gedges_[j];
        } else {
          in_loop[j] = 0;
        }
      }
      local_moved = next;
    }
    return Status::Ok();
  }

  // RefineClusters_subroutine (parallel-correlation-clusterer.cc:476-629)
  // for the B graphs of a disjoint union, each following its own control
  // flow: a graph whose level did not move stops taking part in later levels
  // (its vertices stay singletons there), refinement visits a graph only on
  // the levels below its own final level, and a graph whose final `iter` is
  // not positive keeps the subroutine's singleton output.  d_out receives
  // each graph's dense labels (local ids); d_ids the cluster ids behind them
  // (inside each graph's id range); nclusters[j] the graph's cluster count.
  Status RunUnion(const DevGraph& g0, const UnionLayout& u, const double* d_k, uint32_t* d_out, uint32_t* d_ids,
                  std::vector<GraphRun>* runs, std::vector<uint32_t>* nclusters) {
    if (cfg_.clustering_moves_method != PCC_LOUVAIN)
      return MakeError(PCC_UNIMPLEMENTED, "union batches need clustering_moves_method LOUVAIN");
    if (cfg_.subclustering_method != PCC_NONE_SUBCLUSTERING)
      return MakeError(PCC_UNIMPLEMENTED, "subclustering_method other than NONE_SUBCLUSTERING is not available");
    if (cfg_.async) return MakeError(PCC_INVALID_ARGUMENT, "union batches run synchronous moves only");
    const int64_t num_iterations = cfg_.louvain_num_iterations > 0 ? cfg_.louvain_num_iterations : 10;
    const int64_t num_inner = cfg_.louvain_num_inner_iterations > 0 ? cfg_.louvain_num_inner_iterations : 10;
    const bool refine = cfg_.refine != 0;
    const uint32_t n = g0.n, B = u.B;
    un_ = &u;
    PCC_RETURN_IF_ERROR(Init(n, g0.max_deg));
    PCC_RETURN_IF_ERROR(gflags_.Alloc(ctx_, B));
    PCC_RETURN_IF_ERROR(gflags_.Zero());
    PCC_RETURN_IF_ERROR(gmask_.Alloc(ctx_, B));
    PCC_RETURN_IF_ERROR(gedges_.Alloc(ctx_, B));
    PCC_RETURN_IF_ERROR(ub_flags_.Alloc(ctx_, 2 * uint64_t(B)));
    PCC_RETURN_IF_ERROR(ub_pend_.Alloc(ctx_, B));
    PCC_RETURN_IF_ERROR(ub_ev_.Alloc(ctx_, B));
    PCC_RETURN_IF_ERROR(ub_rounds_.Alloc(ctx_, B));
    PCC_RETURN_IF_ERROR(zcount_.Alloc(ctx_, 1));
    h_gflags_.assign(B, 0);
    h_mask_.assign(B, 0);
    h_gedges_.assign(B, 0);
    h_gent_.assign(B, 0);
    runs->assign(B, GraphRun{});
    std::vector<GraphRun>& gr = *runs;

    std::vector<std::unique_ptr<Level>> rec;
    if (refine) rec.resize(static_cast<size_t>(num_iterations));
    std::unique_ptr<Level> helper;
    PCC_RETURN_IF_ERROR(MakeLevel(&g0, nullptr, d_k, d_k == nullptr, nullptr, &helper));
    DBuf<uint32_t> cluster_ids;
    PCC_RETURN_IF_ERROR(cluster_ids.Alloc(ctx_, n));
    IotaKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p); PCC_COUNT(1);

    std::vector<uint8_t> active(B, 1), moved;
    int64_t iter = 0;
    for (iter = 0; iter < num_iterations; ++iter) {
      PCC_RETURN_IF_ERROR(IterateUnion(helper.get(), num_inner, active, &moved, gr));
      bool any = false;
      for (uint32_t j = 0; j < B; ++j) {
        if (!active[j]) continue;
        if (!moved[j]) {
          active[j] = 0;
          gr[j].iter = iter - 1;
        } else {
          gr[j].levels++;
          any = true;
        }
      }
      if (!any) {
        iter--;
        break;
      }
      res_.levels++;
      if (!refine) {
        FlattenKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p, helper->C.p); PCC_COUNT(1);
      } else if (iter == num_iterations - 1) {
        rec[static_cast<size_t>(iter)] = std::move(helper);
      }
      if (iter == num_iterations - 1) {
        for (uint32_t j = 0; j < B; ++j)
          if (active[j]) gr[j].iter = iter;
        break;
      }
      std::unique_ptr<DevGraph> next;
      timer_.Begin(kPhaseCompress);
      PCC_RETURN_IF_ERROR(CompressGraph(ctx_, *helper->g, helper->C.p, helper->k.p, &next));
      timer_.End(kPhaseCompress);
      res_.algo_bytes_compress += CompressBytes(*helper->g, *next);
      DevGraph* ng = next.get();
      if (ng->n <= u.vbase[B - 1]) return MakeError(PCC_INTERNAL, "union contraction lost a graph's range");
      std::unique_ptr<Level> nl;
      PCC_RETURN_IF_ERROR(MakeLevel(ng, std::move(next), ng->node_w.p, false, nullptr, &nl));
      if (refine) rec[static_cast<size_t>(iter)] = std::move(helper);
      helper = std::move(nl);
    }

    DBuf<uint32_t> rank, tot;
    PCC_RETURN_IF_ERROR(rank.Alloc(ctx_, n));
    PCC_RETURN_IF_ERROR(tot.Alloc(ctx_, 1));
    if (refine && iter > 0) {
      DBuf<uint32_t> flat;
      PCC_RETURN_IF_ERROR(flat.Alloc(ctx_, n));
      std::vector<uint8_t> in_loop(B);
      for (int64_t i = iter - 1; i >= 0; --i) {
        Level* Li = rec[static_cast<size_t>(i)].get();
        Level* Lu = rec[static_cast<size_t>(i + 1)].get();
        const uint32_t ni = Li->g->n, nu = Lu->g->n;
        stamp_++;
        ProjectKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, Li->C.p, Lu->C.p, flat.p, aux_stamp_.p,
                                                                  stamp_); PCC_COUNT(1);
        PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, nu, StampInput{aux_stamp_.p, stamp_},
                                                StorePrefix<uint32_t>{rank.p}, scan_tiles_,
                                                static_cast<uint32_t*>(nullptr)));
        GraphRankKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, flat.p, rank.p, Li->C.p, u.d_vbase.p, B, 1);
        PCC_COUNT(1);
        PCC_RETURN_IF_ERROR(Li->s.Zero());
        PCC_RETURN_IF_ERROR(Li->K.Zero());
        AccumulateClustersKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, Li->C.p, Li->k.p, Li->s.p,
                                                                              Li->K.p); PCC_COUNT(1);
        RefreshKfKernel<<<GridFor(ctx_, ni), kT, 0, ctx_->stream>>>(ni, Li->K.p, Li->Kf.p, nullptr, 0, nullptr);
        PCC_COUNT(1);
        PCC_RETURN_IF_ERROR(LaunchCheck());
        for (uint32_t j = 0; j < B; ++j) {
          in_loop[j] = i <= gr[j].iter - 1;
          if (in_loop[j]) gr[j].refine_passes++;
        }
        PCC_RETURN_IF_ERROR(IterateUnion(Li, num_inner, in_loop, &moved, gr));
        res_.refine_passes++;
        rec[static_cast<size_t>(i + 1)].reset();
      }
      PCC_CUDA(cudaMemcpyAsync(cluster_ids.p, rec[0]->C.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice,
                               ctx_->stream));
      // A graph whose own `iter` is not positive outputs singletons.
      bool anyid = false;
      for (uint32_t j = 0; j < B; ++j) {
        h_mask_[j] = gr[j].iter <= 0;
        anyid |= h_mask_[j] != 0;
      }
      if (anyid) {
        PCC_RETURN_IF_ERROR(gmask_.FromHost(h_mask_.data(), B));
        IdentityGraphsKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p, u.d_vbase.p, B, gmask_.p);
        PCC_COUNT(1);
      }
    }
    rec.clear();
    helper.reset();

    // OutputIndicesById per graph.
    stamp_++;
    MarkStampKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p, aux_stamp_.p, stamp_); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx_, n, StampInput{aux_stamp_.p, stamp_}, StorePrefix<uint32_t>{rank.p},
                                            scan_tiles_, tot.p));
    GraphRankKernel<<<GridFor(ctx_, n), kT, 0, ctx_->stream>>>(n, cluster_ids.p, rank.p, d_out, u.d_vbase.p, B, 0);
    PCC_COUNT(1);
    DBuf<uint32_t> base;
    PCC_RETURN_IF_ERROR(base.Alloc(ctx_, B + 1));
    GraphRankBaseKernel<<<Blocks(B + 1, kT, 1024), kT, 0, ctx_->stream>>>(B, u.d_vbase.p, rank.p, tot.p, base.p);
    PCC_COUNT(1);
    PCC_CUDA(cudaMemcpyAsync(d_ids, cluster_ids.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx_->stream));
    std::vector<uint32_t> hb(B + 1);
    PCC_RETURN_IF_ERROR(base.ToHost(hb.data(), B + 1));
    DevCounters hc;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    if (hc.error) return MakeError(PCC_INTERNAL, "device error flag " + std::to_string(hc.error));
    nclusters->resize(B);
    for (uint32_t j = 0; j < B; ++j) (*nclusters)[j] = hb[j + 1] - hb[j];
    res_.moves += hc.moves;
    return Status::Ok();
  }

  const RunResult& result() const { return res_; }
  double PhaseMs(int k) const { return timer_.TotalMs(k); }
  double FamilyMs(int f) const { return fam_timer_.TotalMs(f); }
  // Family counters of the call (reads the device counters).
  // Rows the frontier push expanded and their entries (detailed timing).
  Status PushCounts(uint64_t* entries, uint64_t* rows) {
    DevCounters hc;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    *entries = hc.push_entries;
    *rows = hc.push_rows;
    return Status::Ok();
  }
  Status FamilyCounts(uint64_t* entries, uint64_t* vertices) {
    DevCounters hc;
    PCC_RETURN_IF_ERROR(ctr_.ToHost(&hc, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx_));
    for (int f = 0; f < kNumFamilies; ++f) {
      entries[f] = hc.fam_entries[f];
      vertices[f] = hc.fam_vertices[f];
    }
    return Status::Ok();
  }
  DevCounters* ctr() { return ctr_.p; }

 private:
  Context* ctx_;
  pcc_config cfg_;
  bool int_nw_ = false;  // integer node weights (certified decisions)
  uint32_t n_max_ = 0;
  uint32_t stamp_ = 0;
  DBuf<uint32_t> moves_, movers_, moved_stamp_, mod_stamp_, next_stamp_, new_stamp_, aux_stamp_;
  DBuf<uint32_t> zero_ids_, new_list_;
  DBuf<uint32_t> free_ids_, free_ctr_;  // async: ids of clusters emptied during the level
  // Async whole-cluster moves: the one-member sets' vertex frontier and moved
  // flags (values sm_val_ + 1, + 2, ...), and a sink for their cluster flags.
  DBuf<uint32_t> sm_front_, sm_moved_, sm_dummy_;
  uint32_t sm_val_ = 0;
  DBuf<uint32_t> scan_tiles_;
  HubState hub_state_;
  DBuf<DevCounters> ctr_;
  RunResult res_;
  PhaseTimer timer_;
  PhaseTimer fam_timer_;  // best-move kernel families (kFam*)
  // Disjoint-union mode (null for a single graph): per-graph frontier flags
  // and degree sums of the round, round-0 masks, the empty-id count.
  DBuf<RoundState> rs_;  // device-side round loop state
  const UnionLayout* un_ = nullptr;
  DBuf<uint32_t> gflags_, gmask_, zcount_;
  DBuf<unsigned long long> gedges_;
  // Device-side union loop: in_loop[B] | moved[B], per-graph frontier
  // entries, edge visits and rounds.
  DBuf<uint8_t> ub_flags_;
  DBuf<unsigned long long> ub_pend_, ub_ev_;
  DBuf<uint32_t> ub_rounds_;
  std::vector<uint32_t> h_gflags_, h_mask_;
  std::vector<unsigned long long> h_gedges_, h_gent_;
};

// Objective of dense labels L (< n) with node weights k (device, or null).
Status ComputeObjectiveDevice(Context* ctx, const DevGraph& g, const uint32_t* L, const double* d_k,
                              double res, double offset, double* out) {
  const uint32_t n = g.n;
  if (n == 0) {
    *out = 0;
    return Status::Ok();
  }
  DBuf<uint32_t> s;
  DBuf<double> k, K;
  PCC_RETURN_IF_ERROR(s.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(k.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(K.Alloc(ctx, n));
  if (d_k) {
    PCC_CUDA(cudaMemcpyAsync(k.p, d_k, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    FillF64Kernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, 1.0, k.p); PCC_COUNT(1);
  }
  PCC_RETURN_IF_ERROR(s.Zero());
  PCC_RETURN_IF_ERROR(K.Zero());
  AccumulateClustersKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, L, k.p, s.p, K.p); PCC_COUNT(1);
  const uint64_t slots = EdgeIterSlots(ctx);
  DBuf<double> acc;
  PCC_RETURN_IF_ERROR(acc.Alloc(ctx, slots));
  PCC_RETURN_IF_ERROR(acc.Zero());
  LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                 ObjEdgeTerm{g.nbr.p, g.wp(), L, offset, acc.p});
  DBuf<double> part, sums;
  PCC_RETURN_IF_ERROR(sums.Alloc(ctx, 2));
  PCC_RETURN_IF_ERROR(Reduce<double>(ctx, slots, ArrayInputF64{acc.p}, OpAdd{}, 0.0, sums.p, part));
  PCC_RETURN_IF_ERROR(Reduce<double>(ctx, n, ResTerm{L, k.p, K.p}, OpAdd{}, 0.0, sums.p + 1, part));
  double h[2];
  PCC_RETURN_IF_ERROR(sums.ToHost(h, 2));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  *out = h[0] - res * h[1] / 2;
  return Status::Ok();
}

// ComputeModularity of dense labels (< n).
Status ComputeModularityDevice(Context* ctx, const DevGraph& g, const uint32_t* L, double resolution,
                               double* out) {
  const uint32_t n = g.n;
  if (n == 0 || g.m == 0) {
    *out = 0;
    return Status::Ok();
  }
  DBuf<unsigned long long> cnt, deg;
  const uint64_t slots = EdgeIterSlots(ctx);
  PCC_RETURN_IF_ERROR(cnt.Alloc(ctx, slots));
  PCC_RETURN_IF_ERROR(cnt.Zero());
  PCC_RETURN_IF_ERROR(deg.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(deg.Zero());
  LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                 SameLabelCount{g.nbr.p, L, cnt.p});
  DegreeSumKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, g.off.p, L, deg.p); PCC_COUNT(1);
  DBuf<unsigned long long> part64, tot64;
  PCC_RETURN_IF_ERROR(tot64.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(Reduce<unsigned long long>(ctx, slots, U64Input{cnt.p}, OpAdd{}, 0ull, tot64.p, part64));
  const double total = static_cast<double>(g.m);
  DBuf<double> part, sum;
  PCC_RETURN_IF_ERROR(sum.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(Reduce<double>(ctx, n, ModTerm{deg.p, resolution, total}, OpAdd{}, 0.0, sum.p, part));
  unsigned long long same = 0;
  double sub = 0;
  PCC_RETURN_IF_ERROR(tot64.ToHost(&same, 1));
  PCC_RETURN_IF_ERROR(sum.ToHost(&sub, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  *out = (static_cast<double>(same) - sub) / total;
  return Status::Ok();
}

Status ValidateGraphArgs(pcc_context* ctx, const pcc_graph* graph, const pcc_config* cfg) {
  if (!ctx) return MakeError(PCC_INVALID_ARGUMENT, "null context");
  // The calling thread may have another device current (worker threads).
  if (cudaSetDevice(ctx->c.device) != cudaSuccess) return MakeError(PCC_UNAVAILABLE, "cannot select the device");
  if (!graph) return MakeError(PCC_INVALID_ARGUMENT, "null graph");
  if (!cfg) return MakeError(PCC_INVALID_ARGUMENT, "null config");
  if (cfg->move_method < 0 || cfg->move_method > 2)
    return MakeError(PCC_INVALID_ARGUMENT, "move_method must be NBHR_CLUSTER_MOVE, ALL_MOVE or NBHR_MOVE");
  return Status::Ok();
}

Status CheckLabels(const uint32_t* labels, uint32_t n) {
  if (!labels) return Status::Ok();
  for (uint32_t i = 0; i < n; ++i)
    if (labels[i] >= n)
      return MakeError(PCC_INVALID_ARGUMENT, "label of node " + std::to_string(i) + " is " +
                                                 std::to_string(labels[i]) + ", not below n = " + std::to_string(n));
  return Status::Ok();
}

pcc_status Finish(pcc_context* ctx, const Status& st) {
  if (ctx) ctx->c.last_error = st.ok() ? std::string() : st.msg;
  return st.code;
}

struct EventTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t s;
  explicit EventTimer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double StopMs() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~EventTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

// Shared body of the correlation / modularity entry points.  `modularity`
// switches to ComputeModularityConfig's node weights and resolution.
Status ClusterImpl(pcc_context* pctx, const pcc_graph* graph, const pcc_config* config, const double* node_weights,
                   const uint32_t* initial_labels, uint32_t* out_labels, pcc_stats* stats, bool modularity) {
  PCC_RETURN_IF_ERROR(ValidateGraphArgs(pctx, graph, config));
  if (!out_labels) return MakeError(PCC_INVALID_ARGUMENT, "null out_labels");
  Context* ctx = &pctx->c;
  const DevGraph& g = graph->g;
  const uint32_t n = g.n;
  PCC_RETURN_IF_ERROR(CheckLabels(initial_labels, n));
  EventTimer timer(ctx->stream);
  const uint64_t launches0 = LaunchCounter();
  pcc_config cfg = *config;
  DBuf<double> dk;
  DBuf<uint32_t> dinit, dout;
  const uint64_t nn = std::max<uint64_t>(n, 1);
  if (modularity) {
    // ComputeModularityConfig (parallel/parallel-graph-utils.cc:141-153).
    PCC_RETURN_IF_ERROR(dk.Alloc(ctx, nn));
    if (n) DegreeF64Kernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, g.off.p, dk.p); PCC_COUNT(1);
    const double total = static_cast<double>(g.m);  // sum of degrees, exact
    cfg.resolution = config->resolution / total;
    cfg.edge_weight_offset = 0;
  } else if (node_weights) {
    PCC_RETURN_IF_ERROR(dk.Alloc(ctx, nn));
    PCC_RETURN_IF_ERROR(dk.FromHost(node_weights, n));
  }
  if (initial_labels) {
    PCC_RETURN_IF_ERROR(dinit.Alloc(ctx, nn));
    PCC_RETURN_IF_ERROR(dinit.FromHost(initial_labels, n));
  }
  PCC_RETURN_IF_ERROR(dout.Alloc(ctx, nn));
  // Integer node weights: degrees, the default ones, or given integers (sums
  // of integers stay integers on the compressed levels).
  const bool int_nw = modularity || !node_weights || IntegralWeights(node_weights, n);
  Engine eng(ctx, cfg, int_nw);
  uint32_t groups = 0;
  PCC_RETURN_IF_ERROR(eng.Run(g, dk.p, dinit.p, dout.p, &groups));
  double obj = 0;
  PCC_RETURN_IF_ERROR(ComputeObjectiveDevice(ctx, g, dout.p, dk.p, cfg.resolution, cfg.edge_weight_offset, &obj));
  double mod = 0;
  if (modularity) PCC_RETURN_IF_ERROR(ComputeModularityDevice(ctx, g, dout.p, config->resolution, &mod));
  PCC_RETURN_IF_ERROR(dout.ToHost(out_labels, n));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  const double ms = timer.StopMs();
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    const RunResult& r = eng.result();
    stats->edge_visits = r.edge_visits;
    stats->vertex_visits = r.vertex_visits;
    stats->moves = r.moves;
    stats->levels = r.levels;
    stats->rounds = r.rounds;
    stats->refine_passes = r.refine_passes;
    stats->num_clusters = static_cast<int32_t>(groups);
    stats->objective = obj;
    stats->modularity = mod;
    stats->ms_total = ms;
    stats->ms_best_moves = eng.PhaseMs(kPhaseBestMoves);
    stats->ms_compress = eng.PhaseMs(kPhaseCompress);
    stats->ms_apply = eng.PhaseMs(kPhaseApply);
    stats->ms_frontier = eng.PhaseMs(kPhaseFrontier);
    stats->kernel_launches = LaunchCounter() - launches0;
    stats->algo_bytes_best_moves = eng.result().algo_bytes;
    stats->algo_bytes_compress = eng.result().algo_bytes_compress;
    uint64_t pe = 0, pr = 0;
    PCC_RETURN_IF_ERROR(eng.PushCounts(&pe, &pr));
    stats->algo_bytes_frontier = 4 * pe + 4 * pr;
    uint64_t fe[kNumFamilies], fv[kNumFamilies];
    PCC_RETURN_IF_ERROR(eng.FamilyCounts(fe, fv));
    for (int f = 0; f < kNumFamilies; ++f) {
      stats->family_ms[f] = eng.FamilyMs(f);
      stats->family_launches[f] = ctx->fam_launches[f];
      stats->family_entries[f] = fe[f];
      stats->family_vertices[f] = fv[f];
    }
  }
  return Status::Ok();
}

// Modularity of the union's modularity graphs (want[j] != 0), segmented by
// graph: entries whose ends share a label, and degree sums per label.
__global__ void __launch_bounds__(kT) ModularityCountsKernel(uint32_t n, const uint64_t* __restrict__ off,
                                                             const uint32_t* __restrict__ nbr,
                                                             const uint32_t* __restrict__ L,
                                                             const uint32_t* __restrict__ vbase, uint32_t B,
                                                             const uint8_t* __restrict__ want,
                                                             unsigned long long* same, unsigned long long* deg) {
  for (uint64_t u = uint64_t(blockIdx.x) * kT + threadIdx.x; u < n; u += uint64_t(gridDim.x) * kT) {
    const uint32_t j = GraphOf(vbase, B, static_cast<uint32_t>(u));
    if (!want[j]) continue;
    const uint32_t lu = L[u];
    unsigned long long cnt = 0;
    for (uint64_t e = off[u]; e < off[u + 1]; ++e) cnt += L[nbr[e]] == lu ? 1ull : 0ull;
    if (cnt) atomicAdd(&same[j], cnt);
    if (off[u + 1] > off[u]) atomicAdd(&deg[lu], static_cast<unsigned long long>(off[u + 1] - off[u]));
  }
}

// sub[j] = sum over graph j's labels c of res_j * d_c * d_c / total_j
// (ComputeModularity, parallel-modularity-clusterer.cc:36-66).
__global__ void __launch_bounds__(kT) ModularitySubKernel(uint32_t n, const unsigned long long* __restrict__ deg,
                                                          const uint32_t* __restrict__ vbase, uint32_t B,
                                                          const double* __restrict__ res,
                                                          const double* __restrict__ total, double* sub) {
  for (uint64_t c = uint64_t(blockIdx.x) * kT + threadIdx.x; c < n; c += uint64_t(gridDim.x) * kT) {
    if (!deg[c]) continue;
    const uint32_t j = GraphOf(vbase, B, static_cast<uint32_t>(c));
    const double d = static_cast<double>(deg[c]);
    atomicAdd(&sub[j], Dmul(Dmul(res[j], d), d) / total[j]);
  }
}

// One disjoint union: graphs gs (each n > 0) with their own resolutions and
// objectives (modularity: node weights = degrees, resolution / sum of
// degrees), results into out_labels[idx[j]] and stats[idx[j]]; totals added
// to *tot.
Status UnionChunk(Context* ctx, const pcc_config& cfg, const std::vector<const pcc_batch_graph*>& gs,
                  const std::vector<uint32_t>& idx, const std::vector<double>& res_in,
                  const std::vector<uint8_t>& modularity, uint32_t* const* out_labels, pcc_stats* stats,
                  pcc_stats* tot) {
  const uint32_t B = static_cast<uint32_t>(gs.size());
  EventTimer timer(ctx->stream);
  const uint64_t launches0 = LaunchCounter();
  DevGraph g0;
  UnionLayout u;
  DBuf<double> dk;
  bool int_nw = true;
  PCC_RETURN_IF_ERROR(UploadUnion(ctx, B, gs.data(), modularity.data(), &g0, &u, &dk, &int_nw));
  const uint32_t n = g0.n;
  // ComputeModularityConfig (parallel/parallel-graph-utils.cc:141-153) per
  // modularity graph: resolution / sum of degrees (= its entries).
  u.res.resize(B);
  bool uniform = true;
  for (uint32_t j = 0; j < B; ++j) {
    u.res[j] = modularity[j] ? res_in[j] / static_cast<double>(gs[j]->m) : res_in[j];
    uniform = uniform && u.res[j] == u.res[0];
  }
  if (!uniform) {
    std::vector<float> r32(B);
    for (uint32_t j = 0; j < B; ++j) r32[j] = FilterF32(u.res[j]);
    PCC_RETURN_IF_ERROR(u.d_res.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(u.d_res32.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(u.d_res.FromHost(u.res.data(), B));
    PCC_RETURN_IF_ERROR(u.d_res32.FromHost(r32.data(), B));
  }
  pcc_config ecfg = cfg;
  ecfg.resolution = u.res[0];  // every vertex's resolution when uniform
  std::vector<Engine::GraphRun> runs;
  std::vector<uint32_t> ncl;
  DBuf<uint32_t> dout, dids;
  PCC_RETURN_IF_ERROR(dout.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(dids.Alloc(ctx, n));
  Engine eng(ctx, ecfg, int_nw);
  PCC_RETURN_IF_ERROR(eng.RunUnion(g0, u, dk.p, dout.p, dids.p, &runs, &ncl));
  // ComputeObjective per graph.
  DBuf<double> ones, K, acc;
  DBuf<uint32_t> s;
  const double* kp = dk.p;
  if (!kp) {
    PCC_RETURN_IF_ERROR(ones.Alloc(ctx, n));
    FillF64Kernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, 1.0, ones.p); PCC_COUNT(1);
    kp = ones.p;
  }
  PCC_RETURN_IF_ERROR(s.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(K.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(acc.Alloc(ctx, 2ull * B));
  PCC_RETURN_IF_ERROR(s.Zero());
  PCC_RETURN_IF_ERROR(K.Zero());
  PCC_RETURN_IF_ERROR(acc.Zero());
  AccumulateClustersKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, dids.p, kp, s.p, K.p); PCC_COUNT(1);
  ObjectiveUnionKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, g0.off.p, g0.nbr.p, g0.wp(), dids.p, kp, K.p,
                                                                ecfg.edge_weight_offset, u.d_vbase.p, B, acc.p,
                                                                acc.p + B); PCC_COUNT(1);
  // ComputeModularity per modularity graph.
  bool any_mod = false;
  for (uint32_t j = 0; j < B; ++j) any_mod = any_mod || modularity[j];
  std::vector<unsigned long long> hsame(B, 0);
  std::vector<double> hsub(B, 0.0);
  DBuf<unsigned long long> same, deg;
  DBuf<double> sub, mres, mtot;
  DBuf<uint8_t> want;
  if (any_mod) {
    std::vector<double> r(B), t(B);
    for (uint32_t j = 0; j < B; ++j) {
      r[j] = res_in[j];
      t[j] = static_cast<double>(gs[j]->m);
    }
    PCC_RETURN_IF_ERROR(same.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(sub.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(deg.Alloc(ctx, n));
    PCC_RETURN_IF_ERROR(mres.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(mtot.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(want.Alloc(ctx, B));
    PCC_RETURN_IF_ERROR(same.Zero());
    PCC_RETURN_IF_ERROR(sub.Zero());
    PCC_RETURN_IF_ERROR(deg.Zero());
    PCC_RETURN_IF_ERROR(mres.FromHost(r.data(), B));
    PCC_RETURN_IF_ERROR(mtot.FromHost(t.data(), B));
    PCC_RETURN_IF_ERROR(want.FromHost(modularity.data(), B));
    ModularityCountsKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, g0.off.p, g0.nbr.p, dids.p, u.d_vbase.p, B,
                                                                    want.p, same.p, deg.p); PCC_COUNT(1);
    ModularitySubKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, deg.p, u.d_vbase.p, B, mres.p, mtot.p, sub.p);
    PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(same.ToHost(hsame.data(), B));
    PCC_RETURN_IF_ERROR(sub.ToHost(hsub.data(), B));
  }
  PCC_RETURN_IF_ERROR(LaunchCheck());
  std::vector<double> hacc(2ull * B);
  std::vector<uint32_t> hl(n);
  PCC_RETURN_IF_ERROR(acc.ToHost(hacc.data(), 2ull * B));
  PCC_RETURN_IF_ERROR(dout.ToHost(hl.data(), n));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  const double ms = timer.StopMs();
  for (uint32_t j = 0; j < B; ++j) {
    const uint32_t i = idx[j];
    std::memcpy(out_labels[i], hl.data() + u.vbase[j], sizeof(uint32_t) * gs[j]->n);
    if (!stats) continue;
    pcc_stats& st = stats[i];
    std::memset(&st, 0, sizeof(st));
    st.objective = hacc[j] - u.res[j] * hacc[B + j] / 2;
    if (modularity[j] && gs[j]->m) {
      const double total = static_cast<double>(gs[j]->m);
      st.modularity = (static_cast<double>(hsame[j]) - hsub[j]) / total;
    }
    st.num_clusters = static_cast<int32_t>(ncl[j]);
    st.levels = runs[j].levels;
    st.rounds = runs[j].rounds;
    st.refine_passes = runs[j].refine_passes;
    st.edge_visits = runs[j].edge_visits;
  }
  if (tot) {
    const RunResult& r = eng.result();
    tot->edge_visits += r.edge_visits;
    tot->vertex_visits += r.vertex_visits;
    tot->moves += r.moves;
    tot->levels = std::max(tot->levels, r.levels);
    tot->rounds += r.rounds;
    tot->refine_passes += r.refine_passes;
    tot->ms_total += ms;
    tot->ms_best_moves += eng.PhaseMs(kPhaseBestMoves);
    tot->ms_compress += eng.PhaseMs(kPhaseCompress);
    tot->ms_apply += eng.PhaseMs(kPhaseApply);
    tot->ms_frontier += eng.PhaseMs(kPhaseFrontier);
    tot->kernel_launches += LaunchCounter() - launches0;
    tot->algo_bytes_best_moves += r.algo_bytes;
    tot->algo_bytes_compress += r.algo_bytes_compress;
    uint64_t pe = 0, pr = 0;
    PCC_RETURN_IF_ERROR(eng.PushCounts(&pe, &pr));
    tot->algo_bytes_frontier += 4 * pe + 4 * pr;
    uint64_t fe[kNumFamilies], fv[kNumFamilies];
    PCC_RETURN_IF_ERROR(eng.FamilyCounts(fe, fv));
    for (int f = 0; f < kNumFamilies; ++f) {
      tot->family_ms[f] += eng.FamilyMs(f);
      tot->family_launches[f] += ctx->fam_launches[f];
      tot->family_entries[f] += fe[f];
      tot->family_vertices[f] += fv[f];
    }
  }
  return Status::Ok();
}

// Configs that can share a union run: equal in every field but the
// resolution.
bool UnionCompatible(const pcc_config& a, const pcc_config& b) {
  pcc_config x = a, y = b;
  x.resolution = 0;
  y.resolution = 0;
  return std::memcmp(&x, &y, sizeof(pcc_config)) == 0;
}

Status ClusterUnionImpl(pcc_context* pctx, uint32_t num_graphs, const pcc_batch_graph* graphs,
                        const pcc_config* configs, uint32_t num_configs, const int32_t* objectives,
                        uint64_t max_entries, uint32_t* const* out_labels, pcc_stats* stats,
                        pcc_stats* batch_stats) {
  if (!pctx || !configs) return MakeError(PCC_INVALID_ARGUMENT, "null context or config");
  if (num_graphs && (!graphs || !out_labels)) return MakeError(PCC_INVALID_ARGUMENT, "null graphs or out_labels");
  if (num_configs != 1 && num_configs != num_graphs)
    return MakeError(PCC_INVALID_ARGUMENT, "num_configs must be 1 or num_graphs");
  Context* ctx = &pctx->c;
  PCC_CUDA(cudaSetDevice(ctx->device));
  if (batch_stats) std::memset(batch_stats, 0, sizeof(*batch_stats));
  if (max_entries == 0) max_entries = 1ull << 31;
  const pcc_config& cfg0 = configs[0];
  bool any_mod = false;
  for (uint32_t i = 0; i < num_graphs; ++i) {
    if (!out_labels[i] && graphs[i].n) return MakeError(PCC_INVALID_ARGUMENT, "null out_labels entry");
    if (graphs[i].n > kMaxVertices) return MakeError(PCC_INVALID_ARGUMENT, "n must be at most 2^32 - 32");
    if (graphs[i].m >= 0xFFFFFFFFull)
      return MakeError(PCC_INVALID_ARGUMENT, "graphs with 2^32 or more entries are not supported");
    if (objectives && objectives[i] != 0 && objectives[i] != 1)
      return MakeError(PCC_INVALID_ARGUMENT, "objective must be 0 (correlation) or 1 (modularity)");
    if (num_configs > 1 && !UnionCompatible(configs[i], cfg0))
      return MakeError(PCC_INVALID_ARGUMENT, "union configs may differ in resolution only");
    any_mod = any_mod || (objectives && objectives[i] == 1);
    if (graphs[i].n == 0 && stats) std::memset(&stats[i], 0, sizeof(pcc_stats));
  }
  // ComputeModularityConfig sets the offset to 0 for modularity graphs.
  if (any_mod && cfg0.edge_weight_offset != 0)
    return MakeError(PCC_INVALID_ARGUMENT, "a union with modularity graphs needs edge_weight_offset 0");
  std::vector<const pcc_batch_graph*> gs;
  std::vector<uint32_t> idx;
  std::vector<double> res;
  std::vector<uint8_t> mod;
  uint64_t nv = 0, ne = 0;
  for (uint32_t i = 0; i <= num_graphs; ++i) {
    const bool flush = i == num_graphs ||
                       (!gs.empty() && (ne + graphs[i].m > max_entries || nv + graphs[i].n > kMaxVertices / 2));
    if (flush && !gs.empty()) {
      PCC_RETURN_IF_ERROR(UnionChunk(ctx, cfg0, gs, idx, res, mod, out_labels, stats, batch_stats));
      gs.clear();
      idx.clear();
      res.clear();
      mod.clear();
      nv = ne = 0;
    }
    if (i == num_graphs) break;
    if (graphs[i].n == 0) continue;  // empty labels, zero stats
    gs.push_back(&graphs[i]);
    idx.push_back(i);
    res.push_back(configs[num_configs == 1 ? 0 : i].resolution);
    mod.push_back(objectives && objectives[i] == 1 ? 1 : 0);
    nv += graphs[i].n;
    ne += graphs[i].m;
  }
  return Status::Ok();
}

}  // namespace

}  // namespace pcc

using namespace pcc;

extern "C" {

pcc_status pcc_cluster_union(pcc_context* ctx, uint32_t num_graphs, const pcc_batch_graph* graphs,
                             const pcc_config* configs, uint32_t num_configs, const int32_t* objectives,
                             uint64_t max_union_entries, uint32_t* const* out_labels, pcc_stats* stats,
                             pcc_stats* batch_stats) {
  try {
    return Finish(ctx, ClusterUnionImpl(ctx, num_graphs, graphs, configs, num_configs, objectives, max_union_entries,
                                        out_labels, stats, batch_stats));
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_correlation_cluster(pcc_context* ctx, const pcc_graph* graph, const pcc_config* config,
                                   const double* node_weights, const uint32_t* initial_labels,
                                   uint32_t* out_labels, pcc_stats* stats) {
  try {
    return Finish(ctx, ClusterImpl(ctx, graph, config, node_weights, initial_labels, out_labels, stats, false));
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_modularity_cluster(pcc_context* ctx, const pcc_graph* graph, const pcc_config* config,
                                  const uint32_t* initial_labels, uint32_t* out_labels, pcc_stats* stats) {
  try {
    return Finish(ctx, ClusterImpl(ctx, graph, config, nullptr, initial_labels, out_labels, stats, true));
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_objective(pcc_context* pctx, const pcc_graph* graph, const pcc_config* config,
                         const double* node_weights, const uint32_t* labels, double* out_objective) {
  Status st = ValidateGraphArgs(pctx, graph, config);
  if (st.ok() && (!labels || !out_objective)) st = MakeError(PCC_INVALID_ARGUMENT, "null labels or output");
  if (st.ok()) st = CheckLabels(labels, graph->g.n);
  if (st.ok()) {
    Context* ctx = &pctx->c;
    const uint32_t n = graph->g.n;
    const uint64_t nn = std::max<uint64_t>(n, 1);
    DBuf<uint32_t> dl;
    DBuf<double> dk;
    st = dl.Alloc(ctx, nn);
    if (st.ok()) st = dl.FromHost(labels, n);
    if (st.ok() && node_weights) {
      st = dk.Alloc(ctx, nn);
      if (st.ok()) st = dk.FromHost(node_weights, n);
    }
    if (st.ok())
      st = ComputeObjectiveDevice(ctx, graph->g, dl.p, dk.p, config->resolution, config->edge_weight_offset,
                                  out_objective);
  }
  return Finish(pctx, st);
}

pcc_status pcc_modularity(pcc_context* pctx, const pcc_graph* graph, double resolution, const uint32_t* labels,
                          double* out_modularity) {
  Status st;
  if (!pctx || !graph || !labels || !out_modularity) st = MakeError(PCC_INVALID_ARGUMENT, "null argument");
  if (st.ok()) st = CheckLabels(labels, graph->g.n);
  if (st.ok()) {
    Context* ctx = &pctx->c;
    const uint32_t n = graph->g.n;
    // ComputeModularity walks the clustering in id order; dense ranks give it.
    std::vector<uint32_t> present(n, 0), dense(n);
    for (uint32_t i = 0; i < n; ++i) present[labels[i]] = 1;
    uint32_t acc = 0;
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t p = present[i];
      present[i] = acc;
      acc += p;
    }
    for (uint32_t i = 0; i < n; ++i) dense[i] = present[labels[i]];
    DBuf<uint32_t> dl;
    st = dl.Alloc(ctx, std::max<uint64_t>(n, 1));
    if (st.ok()) st = dl.FromHost(dense.data(), n);
    if (st.ok()) st = ComputeModularityDevice(ctx, graph->g, dl.p, resolution, out_modularity);
  }
  return Finish(pctx, st);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Kernel-level entry points used by replay tests: one best-move pass from a
// given state, and one contraction.
// ---------------------------------------------------------------------------
namespace pcc {
namespace {

Status BestMovesImpl(pcc_context* pctx, const pcc_graph* graph, const pcc_config* config, const uint32_t* C,
                     const uint32_t* s, const double* k, const double* K, uint32_t* out_t, double* out_v,
                     uint32_t* out_moves) {
  PCC_RETURN_IF_ERROR(ValidateGraphArgs(pctx, graph, config));
  if (!C || !s || !k || !K || !out_t || !out_v)
    return MakeError(PCC_INVALID_ARGUMENT, "null state or output array");
  Context* ctx = &pctx->c;
  const DevGraph& g = graph->g;
  const uint32_t n = g.n;
  PCC_RETURN_IF_ERROR(CheckLabels(C, n));
  const uint64_t nn = std::max<uint64_t>(n, 1);
  DBuf<uint32_t> dC, ds, dt, dm, dmoves, dmovers, dstamp;
  DBuf<double> dk, dK, dv;
  DBuf<float> dKf, dkf;
  PCC_RETURN_IF_ERROR(dKf.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dkf.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dC.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(ds.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dk.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dK.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dt.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dv.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dm.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dmoves.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dmovers.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dstamp.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dstamp.Zero());
  PCC_RETURN_IF_ERROR(dC.FromHost(C, n));
  PCC_RETURN_IF_ERROR(ds.FromHost(s, n));
  PCC_RETURN_IF_ERROR(dk.FromHost(k, n));
  PCC_RETURN_IF_ERROR(dK.FromHost(K, n));
  if (n) {
    RefreshKfKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, dK.p, dKf.p, nullptr, 0, nullptr);
    PCC_COUNT(1);
    NodeKfKernel<<<GridFor(ctx, n), kT, 0, ctx->stream>>>(n, dk.p, dkf.p);
    PCC_COUNT(1);
  }
  DBuf<DevCounters> ctr;
  PCC_RETURN_IF_ERROR(ctr.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(ctr.Zero());
  PCC_RETURN_IF_ERROR(EnsureHubPlan(ctx, &g));
  HubState hs;
  PCC_RETURN_IF_ERROR(AllocHubState(ctx, *g.hub_plan, &hs));
  BMArgs a{};
  a.n = n;
  a.off = g.off.p;
  a.nbr = g.nbr.p;
  a.w = g.wp();
  a.C = dC.p;
  a.s = ds.p;
  a.k = dk.p;
  a.K = dK.p;
  a.Kf = dKf.p;
  a.kf = dkf.p;
  a.int_nw = IntegralWeights(k, n) ? 1 : 0;
  a.narrow = (IntModeFor(g, config->edge_weight_offset) && NarrowSums(g, config->edge_weight_offset)) ? 1 : 0;
  a.res = config->resolution;
  a.res32 = FilterF32(config->resolution);
  a.offset = config->edge_weight_offset;
  a.ioffset = static_cast<int32_t>(config->edge_weight_offset);
  a.stamp = 1;
  a.moves = dmoves.p;
  a.moved_stamp = dstamp.p;
  a.movers = dmovers.p;
  a.ctr = ctr.p;
  a.out_target = dt.p;
  a.out_value = dv.p;
  a.out_moves = dm.p;
  a.async = 0;
  PCC_RETURN_IF_ERROR(EnsureAllBins(ctx, &g));
  const BinSet& ab = g.bins_all;
  PCC_RETURN_IF_ERROR(LaunchBestMoves(ctx, a, ab.list.p, ab.counts.p, ab.counts.p + kNumBins, ab.host_counts,
                                      IntModeFor(g, config->edge_weight_offset), g.max_deg));
  const bool im = IntModeFor(g, config->edge_weight_offset);
  PCC_RETURN_IF_ERROR(LaunchHubBestMoves(ctx, a, *g.hub_plan, hs, im, im && NarrowSums(g, config->edge_weight_offset)));
  PCC_RETURN_IF_ERROR(dt.ToHost(out_t, n));
  PCC_RETURN_IF_ERROR(dv.ToHost(out_v, n));
  if (out_moves) PCC_RETURN_IF_ERROR(dm.ToHost(out_moves, n));
  DevCounters hc;
  PCC_RETURN_IF_ERROR(ctr.ToHost(&hc, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  if (hc.error) return MakeError(PCC_INTERNAL, "device error flag " + std::to_string(hc.error));
  return Status::Ok();
}

}  // namespace
}  // namespace pcc

extern "C" {

pcc_status pcc_best_moves(pcc_context* ctx, const pcc_graph* graph, const pcc_config* config,
                          const uint32_t* cluster_ids, const uint32_t* cluster_sizes, const double* node_weights,
                          const double* cluster_weights, uint32_t* out_targets, double* out_values,
                          uint32_t* out_moves) {
  try {
    return Finish(ctx, BestMovesImpl(ctx, graph, config, cluster_ids, cluster_sizes, node_weights, cluster_weights,
                                     out_targets, out_values, out_moves));
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_compress(pcc_context* pctx, const pcc_graph* graph, const uint32_t* cluster_ids,
                        const double* node_weights, pcc_graph** out) {
  Status st;
  if (!pctx || !graph || !cluster_ids || !out) st = MakeError(PCC_INVALID_ARGUMENT, "null argument");
  if (st.ok()) st = CheckLabels(cluster_ids, graph->g.n);
  if (st.ok()) {
    Context* ctx = &pctx->c;
    const uint32_t n = graph->g.n;
    const uint64_t nn = std::max<uint64_t>(n, 1);
    DBuf<uint32_t> dC;
    DBuf<double> dk;
    st = dC.Alloc(ctx, nn);
    if (st.ok()) st = dC.FromHost(cluster_ids, n);
    if (st.ok() && node_weights) {
      st = dk.Alloc(ctx, nn);
      if (st.ok()) st = dk.FromHost(node_weights, n);
    }
    std::unique_ptr<DevGraph> res;
    if (st.ok()) st = CompressGraph(ctx, graph->g, dC.p, dk.p, &res);
    if (st.ok()) st = Sync(ctx);
    if (st.ok()) {
      auto* h = new pcc_graph;
      h->g = std::move(*res);
      *out = h;
    }
  }
  return Finish(pctx, st);
}

pcc_status pcc_cluster_host_csr(pcc_context* ctx, uint32_t n, uint64_t m, const uint64_t* offsets,
                                const uint32_t* neighbors, const float* weights, const pcc_config* config,
                                int32_t objective, const double* node_weights, uint32_t* out_labels,
                                pcc_stats* stats) {
  pcc_graph* g = nullptr;
  pcc_status st = pcc_graph_upload(ctx, n, m, offsets, neighbors, weights, &g);
  if (st != PCC_OK) return st;
  if (objective == 1)
    st = pcc_modularity_cluster(ctx, g, config, nullptr, out_labels, stats);
  else if (objective == 0)
    st = pcc_correlation_cluster(ctx, g, config, node_weights, nullptr, out_labels, stats);
  else
    st = Finish(ctx, MakeError(PCC_INVALID_ARGUMENT, "objective must be 0 (correlation) or 1 (modularity)"));
  std::string err = ctx ? ctx->c.last_error : std::string();
  pcc_graph_free(ctx, g);
  if (ctx) ctx->c.last_error = err;
  return st;
}

}  // extern "C"
