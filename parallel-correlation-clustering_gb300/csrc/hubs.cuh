// hubs.cuh -- best moves of hub vertices (degree > 1000).
//
// The reference gives hubs their own path (EfficientBestMove, degree > 1000:
// a concurrent sparse_additive_map and a parallel reduce, parallel-
// correlation-clusterer-internal.cc:516-582).  Here a hub's neighbour
// clusters are split by a hash of the cluster id into P partitions, each
// small enough for one CTA's shared-memory table (P = ceil(degree /
// kHubPartKeys)).  A work item is (hub, partition); its CTA
//   1. scans the whole row (entries are re-read by the P CTAs of a hub, from
//      L2 after the first), sums w - offset of the entries whose cluster
//      falls in its partition into the shared table, and sums the entries of
//      the hub's own cluster ("together");
//   2. evaluates its table: FP32 pre-filter, exact FP64 value of the
//      survivors, argmax (value desc, id asc);
//   3. writes its partial best; the last CTA of the hub (atomic counter)
//      combines the P partials and makes the sync / async decision.
// A partition whose keys overflow the table is split again by further hash
// bits and rescanned (sub-passes), so correctness does not depend on the
// hash distribution.  No global hash tables, no spin-waits.
#pragma once

#include "engine.cuh"

namespace pcc {

constexpr uint32_t kHubMinDegree = 1000;  // hub = degree > 1000
constexpr uint32_t kHubSlots = 4096;      // shared table capacity per CTA
constexpr uint32_t kHubPartKeys = 2048;   // expected distinct keys per partition

// Static part (depends on the graph only).
struct HubPlan {
  uint32_t num_hubs = 0;
  uint32_t num_items = 0;
  uint64_t num_partials = 0;
  DBuf<uint32_t> hub_v;       // hub vertex ids
  DBuf<uint32_t> hub_parts;   // P per hub
  DBuf<uint32_t> hub_pbase;   // first partial of the hub
  DBuf<uint32_t> item_hub;    // work items, largest hubs first
  DBuf<uint32_t> item_part;
};

// Per-context mutable state; counters are zero between rounds.
struct HubState {
  DBuf<double> part_val;
  DBuf<uint32_t> part_id;
  DBuf<uint32_t> done;
};

Status BuildHubPlan(Context* ctx, const DevGraph& g, const BinSet& bins, HubPlan* plan);
Status AllocHubState(Context* ctx, const HubPlan& plan, HubState* st);
Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode);

}  // namespace pcc
