// graphops.cuh -- load-balanced iteration over CSR entries.
#pragma once

#include "engine.cuh"

namespace pcc {

// Calls f(u, j) for every entry j of every vertex u in [0, n).  A warp owns
// 32 consecutive vertices, whose rows are contiguous in CSR, and walks their
// entries 32 at a time (coalesced); each lane finds the owner of its entry
// by a binary search over the warp's inclusive degree scan.
template <class F>
__global__ void __launch_bounds__(256) ForEachEntryKernel(uint32_t n, const uint64_t* __restrict__ off, F f) {
  __shared__ uint64_t incl[8][32];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint64_t stride = uint64_t(gridDim.x) * 8 * 32;
  for (uint64_t v0 = (uint64_t(blockIdx.x) * 8 + warp) * 32; v0 < n; v0 += stride) {
    const uint64_t v = v0 + lane;
    uint64_t b = 0, d = 0;
    if (v < n) {
      b = off[v];
      d = off[v + 1] - b;
    }
    const uint64_t inc = WarpInclusiveScan<uint64_t>(d);
    incl[warp][lane] = inc;
    const uint64_t total = __shfl_sync(kFull, inc, 31);
    const uint64_t base = __shfl_sync(kFull, b, 0);
    __syncwarp();
    for (uint64_t e = lane; e < total; e += 32) {
      int lo = 0, hi = 31;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (incl[warp][mid] > e) hi = mid; else lo = mid + 1;
      }
      f(static_cast<uint32_t>(v0 + lo), base + e);
    }
    __syncwarp();
  }
}

// Same for an arbitrary vertex list (count read on the device).
template <class F>
__global__ void __launch_bounds__(256) ForEachListEntryKernel(const uint32_t* __restrict__ list,
                                                             const uint32_t* __restrict__ count_ptr,
                                                             const uint64_t* __restrict__ off, F f) {
  __shared__ uint64_t incl[8][32];
  __shared__ uint64_t begin[8][32];
  __shared__ uint32_t vert[8][32];
  const uint32_t count = *count_ptr;
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint64_t stride = uint64_t(gridDim.x) * 8 * 32;
  for (uint64_t i0 = (uint64_t(blockIdx.x) * 8 + warp) * 32; i0 < count; i0 += stride) {
    const uint64_t i = i0 + lane;
    uint64_t b = 0, d = 0;
    uint32_t v = 0;
    if (i < count) {
      v = list[i];
      b = off[v];
      d = off[v + 1] - b;
    }
    const uint64_t inc = WarpInclusiveScan<uint64_t>(d);
    incl[warp][lane] = inc;
    begin[warp][lane] = b;
    vert[warp][lane] = v;
    const uint64_t total = __shfl_sync(kFull, inc, 31);
    __syncwarp();
    for (uint64_t e = lane; e < total; e += 32) {
      int lo = 0, hi = 31;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (incl[warp][mid] > e) hi = mid; else lo = mid + 1;
      }
      const uint64_t excl = lo ? incl[warp][lo - 1] : 0;
      f(vert[warp][lo], begin[warp][lo] + (e - excl));
    }
    __syncwarp();
  }
}

}  // namespace pcc
