// hubs.cuh -- best moves of hub vertices (degree > 1000) without per-hub
// serial tails.
//
// The reference gives hubs their own path (EfficientBestMove, degree > 1000:
// a concurrent sparse_additive_map and a parallel reduce, parallel-
// correlation-clusterer-internal.cc:516-582).  Here every hub owns a region
// of a global open-addressing table (capacity: the next power of two >= 2 *
// degree), and a round runs flat kernels over static chunk lists:
//   accumulate  CTA per 2048-entry chunk of a hub's row: gather C(u),
//               aggregation in a shared-memory table, then one atomic add
//               per distinct cluster into the hub's global table (new slots
//               appended to the hub's used list, warp-aggregated)
//   change      thread per hub: T = S_c, change
//   gather      CTA per 2048-slot chunk of a hub's used list: (key, sum)
//               pairs compacted, table slots cleared for the next round
//   smax / bound / best / tie   CTA per used chunk over the compacted pairs:
//               the FP32 pre-filter (INT mode) and the exact FP64 argmax
//               (value, then lowest id) by atomics
//   decide      thread per hub: the sync / async decision
#pragma once

#include "engine.cuh"

namespace pcc {

// Static part (depends on the graph only).
struct HubPlan {
  uint32_t num_hubs = 0;
  uint64_t total_slots = 0;
  uint32_t num_echunks = 0;
  uint32_t num_uchunks = 0;
  DBuf<uint32_t> hub_v;      // hub vertex ids
  DBuf<uint32_t> hub_cap;    // table capacity (power of two)
  DBuf<uint64_t> hub_toff;   // table offset (slots); used list at toff / 2
  DBuf<uint32_t> ech_hub, ech_e0;  // row chunks
  DBuf<uint32_t> uch_hub, uch_u0;  // used-list chunks
};

// Per-level mutable state (clean between rounds).
struct HubState {
  DBuf<uint32_t> keys;                // kNone when empty
  DBuf<unsigned long long> vals;      // int64 (INT) or double bits; 0 when empty
  DBuf<uint32_t> used;                // slot indices, total_slots / 2
  DBuf<uint32_t> pkeys;               // compacted keys of the used slots
  DBuf<unsigned long long> pvals;     // compacted sums of the used slots
  DBuf<uint32_t> used_count;          // per hub
  DBuf<long long> smax;               // per hub (INT filter)
  DBuf<uint32_t> ubound;              // per hub: ordered-float max of Y' - e
  DBuf<unsigned long long> best;      // per hub: ordered-double max value
  DBuf<uint32_t> best_id;             // per hub: lowest id among the best
  DBuf<double> change;                // per hub
};

constexpr uint32_t kHubEdgeChunk = 2048;
constexpr uint32_t kHubUsedChunk = 2048;
constexpr uint32_t kHubMinDegree = 1000;  // hub = degree > 1000

Status BuildHubPlan(Context* ctx, const DevGraph& g, const BinSet& bins, HubPlan* plan);
Status AllocHubState(Context* ctx, const HubPlan& plan, HubState* st);
Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode);

}  // namespace pcc
