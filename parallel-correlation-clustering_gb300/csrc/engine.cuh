// engine.cuh -- device data layout of the clustering engine and the
// launchers shared between translation units.
//
// HBM layout (SoA, one set per compression level):
//   graph   off u64[n+1], nbr u32[m], w f32[m] (absent for unit weights)
//   state   C u32[n] (cluster_ids_), s u32[n] (cluster_sizes_),
//           k f64[n] (node_weights_), K f64[n] (cluster_weights_)
// mirroring ClusteringHelper (parallel-correlation-clusterer-internal.h:
// 36-165).  Per-round scratch (sized by the level-0 vertex count) holds the
// degree-binned frontier, the decided moves and round-stamped flags, so no
// per-round clearing pass is needed.
#pragma once

#include "primitives.cuh"

namespace pcc {

// ---------------------------------------------------------------------------
// Degree bins.  Each bin is served by one best-move kernel shape:
//   d <= 4, 8, 16, 32    lane groups of 4/8/16/32 lanes, one chunk
//   d <= 128/256/512     one warp, shared-memory hash of 256/512/1024 slots
//   d <= 1000            one warp, shared-memory hash of 2048 slots
//                        (the reference's sequential path ends at 1000)
//   d >  1000            hubs: hash-partitioned CTAs (hubs.cuh); the two
//                        top bins only split the static vertex list
// ---------------------------------------------------------------------------
enum Bin : int {
  kBinG4 = 0, kBinG8, kBinG16, kBinG32,
  kBinW128, kBinW256, kBinW512, kBinW1000,
  kBinCta, kBinGlobal,
  kNumBins
};
constexpr uint32_t kBinMaxDeg[kNumBins] = {4, 8, 16, 32, 128, 256, 512, 1000, 4096, 0xFFFFFFFFu};
constexpr uint32_t kCtaHashSlots = 8192;

__host__ __device__ inline int BinOf(uint64_t d) {
  if (d <= 4) return kBinG4;
  if (d <= 8) return kBinG8;
  if (d <= 16) return kBinG16;
  if (d <= 32) return kBinG32;
  if (d <= 128) return kBinW128;
  if (d <= 256) return kBinW256;
  if (d <= 512) return kBinW512;
  if (d <= 1000) return kBinW1000;
  if (d <= 4096) return kBinCta;
  return kBinGlobal;
}

// Degree-binned vertex list: bins are contiguous segments of `list`.
struct BinSet {
  DBuf<uint32_t> list;       // n entries
  DBuf<uint32_t> counts;     // [kNumBins] counts, then [kNumBins+1] starts
  uint64_t edges = 0;        // sum of degrees (host copy, static bins only)
  uint32_t size = 0;         // vertices (host copy, static bins only)
  uint32_t host_counts[kNumBins] = {0};
};

struct HubPlan;

// ---------------------------------------------------------------------------
// Graph resident in HBM.
// ---------------------------------------------------------------------------
struct DevGraph {
  uint32_t n = 0;
  uint64_t m = 0;
  DBuf<uint64_t> off;
  DBuf<uint32_t> nbr;
  DBuf<float> w;          // empty => unit weights
  DBuf<double> node_w;    // node weights attached by compression
  BinSet bins;            // static degree bins of the vertices with degree > 0
  mutable BinSet bins_all;  // all vertices (built on first use)
  mutable std::shared_ptr<HubPlan> hub_plan;  // degree > 1000 (built on first use)
  uint32_t max_deg = 0;
  bool integral = true;   // every weight is an integer value
  double max_abs_w = 1.0; // max |w| (1 for unit weights)
  double row_abs_bound = 0; // upper bound of any row's sum of |w|
  const float* wp() const { return w.p; }
};

// Computes max degree / weight properties and the static degree bins on
// the device (one sync).
Status ComputeGraphProperties(Context* ctx, DevGraph* g);
// Builds g->bins_all (degree bins including isolated vertices) if absent.
Status EnsureAllBins(Context* ctx, const DevGraph* g);

// ---------------------------------------------------------------------------
// Disjoint union of independent graphs (batched clustering).  Graph j owns
// the vertex ids [vbase[j], vbase[j+1]) at every level: contraction keeps
// cluster ids as vertex ids (1 + max C vertices), and new-cluster ids and
// refinement relabels are drawn inside each graph's range, so every graph
// runs exactly as it would alone, with its ids shifted by vbase[j].
// ---------------------------------------------------------------------------
struct UnionLayout {
  uint32_t B = 0;               // graphs (each with n > 0)
  std::vector<uint32_t> vbase;  // B + 1 (host)
  std::vector<uint64_t> ebase;  // B + 1 (host)
  DBuf<uint32_t> d_vbase;       // B + 1
  // Per-graph resolution the moves use (modularity graphs: res / sum of
  // degrees); d_res / d_res32 are set when the graphs' resolutions differ.
  std::vector<double> res;
  DBuf<double> d_res;
  DBuf<float> d_res32;
};

// Index j < B of the last base[j] <= x (bases ascending): the graph owning
// vertex id (or entry index) x.
template <class T>
__device__ __forceinline__ uint32_t GraphOf(const T* __restrict__ base, uint32_t B, T x) {
  uint32_t lo = 0, hi = B;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (base[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Uploads graphs[0..B) (host CSR, each n > 0) as one union graph with
// shifted offsets and neighbour ids, validating every graph's CSR.  Node
// weights: *k receives the union's node weights when any graph has them or
// takes its degrees (degree_weights[j], modularity), 1 for the others;
// *int_nw = every node weight is an integer.
Status UploadUnion(Context* ctx, uint32_t B, const pcc_batch_graph* const* graphs, const uint8_t* degree_weights,
                   DevGraph* g, UnionLayout* u, DBuf<double>* k, bool* int_nw);

// Device counters of one call (all in one allocation).
struct DevCounters {
  uint32_t bin_count[kNumBins];
  uint32_t bin_start[kNumBins + 1];
  uint32_t frontier;        // vertices in the frontier being built
  uint32_t movers;          // real movers of this round
  uint32_t new_movers;      // movers to a new cluster
  uint32_t marked;          // vertices marked for the next frontier
  uint32_t level_moved;     // OR over rounds of "next frontier non-empty"
  uint32_t rounds;          // best-move rounds executed
  uint32_t present;         // generic count used by compaction steps
  uint32_t max_u32;         // generic max used by reductions
  unsigned long long pend_edges;     // sum deg of the frontier being built
  unsigned long long edge_visits;    // sum deg over executed rounds
  unsigned long long vertex_visits;  // sum |F| over executed rounds
  unsigned long long moves;          // real moves (sync) / moves (async)
  int error;                // nonzero: a bounded wait gave up (see kErr*)
  int pad;
  // Per kernel family (kFam*): entries and vertices evaluated (algorithmic
  // bytes of the roofline); accumulated over the call.
  unsigned long long fam_entries[kNumFamilies];
  unsigned long long fam_vertices[kNumFamilies];
  // Accumulated by the device-side round loop (sync mode).
  unsigned long long sync_moves;     // real movers over the loop's rounds
  unsigned long long visited;        // vertices evaluated over the loop's rounds
  // Detailed timing only: rows the frontier push expanded and their entries,
  // over the call (algorithmic bytes of the push).
  unsigned long long push_entries;
  unsigned long long push_rows;
};

constexpr int kErrProbeLimit = 1;   // async new-cluster probe exceeded its bound
constexpr int kErrHashFull = 2;     // a best-move hash table filled up
constexpr int kErrCertMismatch = 3; // a certified decision differed from FP64 (replay self-check)
constexpr int kErrUnionRange = 4;   // a union graph's new-cluster id fell outside its range

// Round state in device memory for rounds that run inside a device-side
// graph loop: the kernel arguments stay fixed from round to round, and the
// kernels take the stamp and the frontier from here.
struct RoundState {
  uint32_t stamp;                  // this round's stamp
  uint32_t front_val;              // frontier: front_stamp[v] == front_val
  uint32_t front_all;              // 1: every binned vertex is in the frontier
  uint32_t iter;                   // rounds run in this loop so far
  unsigned long long front_edges;  // degree sum of this round's frontier
  unsigned long long front_size;   // its vertices (n when front_all)
  unsigned long long visited;      // vertices evaluated (the binned ones when front_all)
};

__host__ __device__ __forceinline__ uint32_t StampIn(const RoundState* rs, uint32_t stamp) {
#ifdef __CUDA_ARCH__
  return rs ? rs->stamp : stamp;
#else
  return stamp;
#endif
}

// Best-move kernel arguments.
struct BMArgs {
  uint32_t n;
  const uint64_t* off;
  const uint32_t* nbr;
  const float* w;
  const uint32_t* C;
  const uint32_t* s;
  const double* k;
  const double* K;
  const float* Kf;          // FilterF32(K), current for the sync round (filter input)
  const float* kf;          // FilterF32(k), node weights (certified decisions)
  double res;
  float res32;              // FilterF32(res)
  int int_nw;               // all node weights are integers (certified decisions)
  int narrow;               // INT mode and every cluster sum fits in 32 bits
  double offset;
  int32_t ioffset;          // integer offset (INT mode)
  uint32_t stamp;
  // frontier: vertices v with front_stamp[v] == front_val (all when null)
  const uint32_t* front_stamp;
  uint32_t front_val;
  // async waves: with waves > 1 only the frontier vertices of wave `wave`
  // (a salted hash of the id) are evaluated by this launch
  uint32_t waves;
  uint32_t wave;
  uint32_t wave_salt;
  // sync outputs
  uint32_t* moves;          // decided target per vertex (read for movers)
  uint32_t* moved_stamp;    // moved_vertex: = stamp when value > 0
  uint32_t* movers;         // list of real movers (target != current)
  DevCounters* ctr;
  // replay outputs (nullable)
  uint32_t* out_target;
  double* out_value;
  uint32_t* out_moves;
  // async mode: apply moves immediately with atomics
  int async;
  uint32_t* s_mut;
  double* K_mut;
  uint32_t* C_mut;
  uint32_t* moved_cluster_stamp;
  // async mode: ids of empty clusters (at the start of the level, then as
  // clusters empty), offered to vertices that found a new cluster
  // (free_ctr[0] = pushed, [1] = taken; slots hold kNone until published
  // and after being taken)
  uint32_t* free_ids;
  uint32_t* free_ctr;
  uint32_t free_cap;
  // non-null: stamp and frontier come from here (front_stamp is the array)
  const RoundState* rs;
  // non-null: per-vertex resolution (graphs of a union with their own
  // resolutions); else res / res32 for every vertex
  const double* vres;
  const float* vres32;
};

__device__ __forceinline__ double ResOf(const BMArgs& a, uint32_t v) { return a.vres ? a.vres[v] : a.res; }
__device__ __forceinline__ float Res32Of(const BMArgs& a, uint32_t v) { return a.vres32 ? a.vres32[v] : a.res32; }

// Asynchronous whole-cluster moves (AsyncSetMoves, clustermoves.cu).
struct SetMoveArgs {
  const DevGraph* g;
  uint32_t* C;          // live state
  uint32_t* s;
  const double* k;
  double* K;
  double res;
  double offset;
  bool exact_sums;      // integral entry values: run sums in any order
  uint32_t waves;       // hashed waves of sets
  uint32_t salt;
  uint32_t* free_ids;   // empty ids offered to new clusters (as the vertex moves)
  uint32_t* free_ctr;
  uint32_t free_cap;
  uint32_t* mod_stamp;  // moved-cluster flags (set at the members' vertex ids)
  uint32_t stamp;
  DevCounters* ctr;
  // One-member sets go through the vertex AsyncMove: the caller's kernels
  // evaluate the vertices with aux_front[v] == val (val = aux_base + wave)
  // and leave aux_moved[v] == val for the ones that moved.
  uint32_t* aux_front;
  const uint32_t* aux_moved;
  uint32_t aux_base;
};

// Configures (shared-memory limit, occupancy) every synchronous best-move
// kernel once per process, so that launches captured into a graph make no
// runtime configuration calls.
Status PrepareBestMoveKernels();

// Launches the best-move kernels of the bins up to degree 1000 over `bins`
// (counts read on the device); hubs go through LaunchHubBestMoves.
// int_mode selects exact integer accumulation (all weights and the offset
// integral and small) over FP64 accumulation in adjacency order.
// families: kLaunchGroups (degree <= 32) and/or kLaunchWarps (33-1000).
constexpr int kLaunchGroups = 1;
constexpr int kLaunchWarps = 2;

// Launch shape of the best-move bins: lane-group bins whose degree cap is
// above group_max_degree run on the warp kernel instead (4, 8, 16 or 32);
// certified warp bins whose degree cap is above cta_min_degree run one CTA
// per vertex (64, 128, 256, 512, or 1000 for none); the grid-stride kernels
// get grid_waves times one wave of resident CTAs.  Every choice changes the
// schedule only: each vertex's decision is the same, so the labels are too.
struct LaunchTuning {
  uint32_t group_max_degree;
  uint32_t cta_min_degree;
  float grid_waves;
};
struct TuningRow {
  uint32_t max_vertices;  // the row applies to level graphs with n <= this
  uint32_t group_max_degree;
  uint32_t cta_min_degree;
  float grid_waves;
};
}  // namespace pcc
#include "tuning_table.cuh"
namespace pcc {
inline LaunchTuning TuningFor(const Context* ctx, uint32_t n) {
  if (ctx->tuned) return LaunchTuning{ctx->group_max_degree, ctx->cta_min_degree, ctx->grid_waves};
  for (const TuningRow& r : kTuningTable)
    if (n <= r.max_vertices) return LaunchTuning{r.group_max_degree, r.cta_min_degree, r.grid_waves};
  return LaunchTuning{32, 1000, 1.0f};
}

Status LaunchBestMoves(Context* ctx, const BMArgs& a, const uint32_t* list, const uint32_t* bin_counts,
                       const uint32_t* bin_starts, const uint32_t* host_counts, bool int_mode,
                       uint32_t max_deg, int families = kLaunchGroups | kLaunchWarps);

// The hub plan of a graph (built on first use).
Status EnsureHubPlan(Context* ctx, const DevGraph* g);

}  // namespace pcc

struct pcc_graph {
  pcc::DevGraph g;
};
