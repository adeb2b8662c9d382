// batch.cuh -- batched best moves (INT mode, sync rounds) of the vertices
// with degree <= 1000: see batch.cu.
#pragma once

#include "engine.cuh"

namespace pcc {

constexpr uint32_t kBatchEdges = 1024;  // entries per batch (degree <= 1000 fits)
constexpr uint32_t kBatchVerts = 256;   // vertices per batch

// Static packing of a degree-binned list (bins G4..W1000) into batches.
struct BatchPlan {
  const uint32_t* list = nullptr;
  uint32_t num_batches = 0;
  DBuf<uint32_t> starts;  // num_batches + 1 positions in list
};

Status BuildBatchPlan(Context* ctx, const DevGraph& g, const BinSet& bins, BatchPlan* plan);
Status LaunchBatchBestMoves(Context* ctx, const BMArgs& a, const BatchPlan& plan);

}  // namespace pcc
