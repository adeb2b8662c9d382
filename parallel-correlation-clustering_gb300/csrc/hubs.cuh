// hubs.cuh -- best moves of hub vertices (degree > 1000).
//
// The reference gives hubs their own path (EfficientBestMove, degree > 1000:
// a concurrent sparse_additive_map and a parallel reduce, parallel-
// correlation-clusterer-internal.cc:516-582).  Here a hub's neighbour-cluster
// sums live in shared memory only:
//
//   small hubs (1000 < degree <= kHubSmallMax): one 256-thread CTA per hub,
//     a table of at least 2 * degree + 2 slots, so it never fills (4096
//     slots up to degree 2047, else 8192);
//   big hubs (degree > kHubSmallMax): one 1024-thread CTA per (hub,
//     partition) with a ~192 KB table.  Hubs with more than kHubBigKeys
//     distinct neighbour clusters are split into P hash partitions (P =
//     ceil(degree / kHubBigKeys)), whose CTAs re-read the row from L2.  A
//     partition whose keys overflow its table is split again by further hash
//     bits and rescanned (sub-passes), so correctness does not depend on the
//     hash distribution.
//
// Each CTA evaluates its table (FP32 pre-filter, exact FP64 values of the
// survivors, argmax by value desc / id asc); for big hubs the partitions'
// bests are combined by the hub's last CTA (atomic counter).  No global hash
// tables, no spin-waits.
#pragma once

#include "engine.cuh"

namespace pcc {

constexpr uint32_t kHubMinDegree = 1000;  // hub = degree > 1000
constexpr uint32_t kHubSmallMax = 4096;   // one-partition hubs
constexpr uint32_t kHubBigKeys = 12288;   // expected distinct keys per big-hub partition
constexpr uint32_t kHubGlobalParts = 4;    // big hubs with >= this many partitions take the global path
constexpr uint32_t kHubGlobalSlice = 1024;   // table slots evaluated by one CTA

// Static part (depends on the graph only).
struct HubPlan {
  uint32_t num_hubs = 0;
  uint32_t num_small = 0;      // hubs with degree <= kHubSmallMax
  uint32_t num_small_wide = 0; // of those, the first ones, with 2 * degree + 2 > 6144 slots
  uint32_t num_small_mid = 0;  // then those with 4096 < 2 * degree + 2 <= 6144
  uint32_t num_big = 0;
  uint32_t num_items = 0;      // big-hub work items (hub, partition)
  uint64_t num_partials = 0;   // one per big-hub item
  DBuf<uint32_t> small_v;      // small hubs, largest first
  DBuf<uint32_t> big_v;        // big hubs, largest first
  DBuf<uint32_t> big_parts;    // P per big hub
  DBuf<uint32_t> big_pbase;    // first partial of the big hub
  DBuf<uint32_t> item_hub;     // work items, largest hubs first
  DBuf<uint32_t> item_part;
  // Big hubs with at least kHubGlobalParts partitions, synchronous rounds:
  // many CTAs accumulate a row's chunks into one per-hub table in HBM, then
  // one CTA per hub evaluates it (a row of millions of entries would
  // otherwise keep a few CTAs busy while the rest of the GPU idles).
  uint32_t num_glob = 0;
  uint32_t num_glob_items = 0;
  uint64_t glob_slots = 0;
  DBuf<uint32_t> glob_hub;               // per global hub: its big-hub index
  DBuf<unsigned long long> glob_base;    // first table slot
  DBuf<uint32_t> glob_cap;               // table slots (2 * degree + 2: never full)
  DBuf<uint32_t> glob_item;              // per work item: global hub index
  DBuf<uint32_t> glob_item_start;        // first entry of the item's chunk
  DBuf<uint32_t> big_glob;               // per big hub: global hub index or kNone
  // Evaluation: the table is split into slices of kHubGlobalSlice slots, one
  // CTA each; the hub's last CTA combines the slices' bests.
  uint32_t num_glob_slices = 0;
  DBuf<uint32_t> glob_nslices;           // per global hub
  DBuf<uint32_t> glob_sbase;             // per global hub: first partial
  DBuf<uint32_t> slice_hub;              // per slice: global hub index
  DBuf<uint32_t> slice_start;            // per slice: first slot (within the hub's table)
};

// Per-context mutable state; counters are zero between rounds.
struct HubState {
  DBuf<double> part_val;
  DBuf<uint32_t> part_id;
  DBuf<uint32_t> done;
  // Global-path tables (keys kNone / values 0 between rounds) and per-hub
  // accumulators (reset by the evaluating CTA).
  DBuf<uint32_t> gkeys;
  DBuf<unsigned long long> gvals;
  DBuf<long long> gt_int;
  DBuf<double> gt_dbl;
  DBuf<long long> gsmax;
  DBuf<double> gpart_val;                // per slice: best (value, id)
  DBuf<uint32_t> gpart_id;
  DBuf<uint32_t> gdone;                  // per global hub: slices evaluated (0 between rounds)
};

Status BuildHubPlan(Context* ctx, const DevGraph& g, const BinSet& bins, HubPlan* plan);
// Configures every synchronous hub kernel once per process (for launches
// captured into a graph).
Status PrepareHubKernels();
Status AllocHubState(Context* ctx, const HubPlan& plan, HubState* st);
// narrow: INT mode with every neighbour-cluster sum below 2^31 in
// magnitude, so the tables hold 32-bit sums.  families: kLaunchSmallHubs
// (degree <= 4096, one CTA per hub) and/or kLaunchBigHubs (the partitioned
// and global paths).
constexpr int kLaunchSmallHubs = 4;
constexpr int kLaunchBigHubs = 8;
Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode,
                          bool narrow, int families = kLaunchSmallHubs | kLaunchBigHubs);

}  // namespace pcc
