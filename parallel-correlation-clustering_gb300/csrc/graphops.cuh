// graphops.cuh -- load-balanced iteration over CSR entries of a
// degree-binned vertex list.
//
// Rows are served by three kernel shapes so that no warp walks a hub row on
// its own (a 64k-entry row walked by one warp is a ~1 ms latency chain):
//   small rows (bins d <= 32):   a warp takes 32 rows and walks their entries
//                                32 at a time (warp-level load balancing);
//   mid rows (32 < d <= 1000):   one warp per row, 4 entries per lane in
//                                flight;
//   big rows (d > 1000):         one CTA of 512 threads per row.
// The functor is called as f(u, j, slot): vertex u, entry j, and a
// per-thread slot in [0, EdgeIterSlots(ctx)) for deterministic per-thread
// accumulation.
#pragma once

#include "engine.cuh"

namespace pcc {

constexpr int kIterThreads = 256;
constexpr int kIterBigThreads = 512;

inline unsigned IterSmallGrid(const Context* ctx) { return unsigned(ctx->num_sms) * 8; }
inline unsigned IterMidGrid(const Context* ctx) { return unsigned(ctx->num_sms) * 8; }
inline unsigned IterBigGrid(const Context* ctx) { return unsigned(ctx->num_sms) * 2; }
inline uint64_t EdgeIterSlots(const Context* ctx) {
  return uint64_t(IterSmallGrid(ctx)) * kIterThreads + uint64_t(IterMidGrid(ctx)) * kIterThreads +
         uint64_t(IterBigGrid(ctx)) * kIterBigThreads;
}

struct RowAll {
  __device__ bool operator()(uint32_t) const { return true; }
};

template <class F, class R>
__global__ void __launch_bounds__(kIterThreads) EdgeIterSmallKernel(const uint32_t* __restrict__ list,
                                                                   const uint32_t* __restrict__ counts,
                                                                   const uint32_t* __restrict__ starts,
                                                                   const uint64_t* __restrict__ off, F f, R row) {
  __shared__ uint32_t incl[kIterThreads / 32][32];
  __shared__ uint64_t begin[kIterThreads / 32][32];
  __shared__ uint32_t vert[kIterThreads / 32][32];
  const uint32_t s0 = starts[kBinG4];
  const uint32_t count = starts[kBinW128] - s0;  // bins G4..G32 are contiguous
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint64_t slot = uint64_t(blockIdx.x) * kIterThreads + threadIdx.x;
  const uint64_t stride = uint64_t(gridDim.x) * kIterThreads;
  for (uint64_t i0 = (uint64_t(blockIdx.x) * (kIterThreads / 32) + warp) * 32; i0 < count; i0 += stride) {
    const uint64_t i = i0 + lane;
    uint32_t d = 0, v = 0;
    uint64_t b = 0;
    if (i < count) {
      v = list[s0 + i];
      if (row(v)) {
        b = off[v];
        d = static_cast<uint32_t>(off[v + 1] - b);
      }
    }
    const uint32_t inc = WarpInclusiveScan<uint32_t>(d);
    incl[warp][lane] = inc;
    begin[warp][lane] = b;
    vert[warp][lane] = v;
    const uint32_t total = __shfl_sync(kFull, inc, 31);
    __syncwarp();
    for (uint32_t e = lane; e < total; e += 32) {
      int lo = 0, hi = 31;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (incl[warp][mid] > e) hi = mid; else lo = mid + 1;
      }
      const uint32_t excl = lo ? incl[warp][lo - 1] : 0u;
      f(vert[warp][lo], begin[warp][lo] + (e - excl), slot);
    }
    __syncwarp();
  }
  (void)counts;
}

template <class F, class R>
__global__ void __launch_bounds__(kIterThreads) EdgeIterMidKernel(const uint32_t* __restrict__ list,
                                                                 const uint32_t* __restrict__ counts,
                                                                 const uint32_t* __restrict__ starts,
                                                                 const uint64_t* __restrict__ off, F f,
                                                                 uint64_t slot_base, R row) {
  const uint32_t s0 = starts[kBinW128];
  const uint32_t count = starts[kBinCta] - s0;  // bins W128..W1000
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint64_t slot = slot_base + uint64_t(blockIdx.x) * kIterThreads + threadIdx.x;
  for (uint64_t i = uint64_t(blockIdx.x) * (kIterThreads / 32) + warp; i < count;
       i += uint64_t(gridDim.x) * (kIterThreads / 32)) {
    const uint32_t v = list[s0 + i];
    if (!row(v)) continue;
    const uint64_t b = off[v], e = off[v + 1];
    for (uint64_t j = b + lane; j < e; j += 128) {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (j + 32 * k < e) f(v, j + 32 * k, slot);
    }
  }
  (void)counts;
}

template <class F, class R>
__global__ void __launch_bounds__(kIterBigThreads) EdgeIterBigKernel(const uint32_t* __restrict__ list,
                                                                    const uint32_t* __restrict__ counts,
                                                                    const uint32_t* __restrict__ starts,
                                                                    const uint64_t* __restrict__ off, F f,
                                                                    uint64_t slot_base, R row) {
  const uint32_t s0 = starts[kBinCta];
  const uint32_t count = starts[kNumBins] - s0;  // bins Cta, Global
  const uint64_t slot = slot_base + uint64_t(blockIdx.x) * kIterBigThreads + threadIdx.x;
  for (uint64_t i = blockIdx.x; i < count; i += gridDim.x) {
    const uint32_t v = list[s0 + i];
    if (!row(v)) continue;
    const uint64_t b = off[v], e = off[v + 1];
    for (uint64_t j = b + threadIdx.x; j < e; j += 4 * kIterBigThreads) {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (j + uint64_t(kIterBigThreads) * k < e) f(v, j + uint64_t(kIterBigThreads) * k, slot);
    }
  }
  (void)counts;
}

// Launches the three shapes over a BinSet-layout list (starts on device);
// rows failing `row` are skipped.  host_counts (per bin) may be null; then
// every shape is launched.
template <class F, class R = RowAll>
inline void LaunchEdgeIter(Context* ctx, const uint32_t* list, const uint32_t* counts, const uint32_t* starts,
                           const uint32_t* host_counts, const uint64_t* off, F f, R row = R()) {
  auto any = [&](int b0, int b1) {
    if (!host_counts) return true;
    for (int b = b0; b < b1; ++b)
      if (host_counts[b]) return true;
    return false;
  };
  cudaStream_t st = ctx->stream;
  if (any(kBinG4, kBinW128)) {
    EdgeIterSmallKernel<F, R><<<IterSmallGrid(ctx), kIterThreads, 0, st>>>(list, counts, starts, off, f, row);
    PCC_COUNT(1);
  }
  const uint64_t base_mid = uint64_t(IterSmallGrid(ctx)) * kIterThreads;
  if (any(kBinW128, kBinCta)) {
    EdgeIterMidKernel<F, R><<<IterMidGrid(ctx), kIterThreads, 0, st>>>(list, counts, starts, off, f, base_mid, row);
    PCC_COUNT(1);
  }
  const uint64_t base_big = base_mid + uint64_t(IterMidGrid(ctx)) * kIterThreads;
  if (any(kBinCta, kNumBins)) {
    EdgeIterBigKernel<F, R><<<IterBigGrid(ctx), kIterBigThreads, 0, st>>>(list, counts, starts, off, f, base_big,
                                                                          row);
    PCC_COUNT(1);
  }
}

// ---------------------------------------------------------------------------
// Frontier push (gbbs edgeMap with an always-true update): stamp[u] = value
// for every neighbour u of a row passing `row`.  The mid and big shapes load
// kPushBatch neighbour ids per thread before storing any stamp: through the
// generic functor the compiler must assume a store may alias the next id and
// keeps one load in flight.  Small rows use EdgeIterSmallKernel.  A stamp
// already equal to the value is not stored again: hub vertices are
// neighbours of a large share of all rows, and same-address stores
// serialise at their L2 slice while the loads are served by L1.
// ---------------------------------------------------------------------------
constexpr int kPushBatch = 8;

struct StampValue {
  uint32_t stamp;
  const RoundState* rs;  // non-null: the value comes from here
};

template <class R>
__global__ void __launch_bounds__(kIterThreads) PushMidKernel(const uint32_t* __restrict__ list,
                                                             const uint32_t* __restrict__ starts,
                                                             const uint64_t* __restrict__ off,
                                                             const uint32_t* __restrict__ nbr,
                                                             uint32_t* __restrict__ stamp, StampValue sv, R row) {
  const uint32_t s0 = starts[kBinW128];
  const uint32_t count = starts[kBinCta] - s0;  // bins W128..W1000
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint32_t value = StampIn(sv.rs, sv.stamp);
  for (uint64_t i = uint64_t(blockIdx.x) * (kIterThreads / 32) + warp; i < count;
       i += uint64_t(gridDim.x) * (kIterThreads / 32)) {
    const uint32_t v = list[s0 + i];
    if (!row(v)) continue;
    const uint64_t b = off[v], e = off[v + 1];
    for (uint64_t j0 = b; j0 < e; j0 += 32 * kPushBatch) {
      uint32_t u[kPushBatch];
#pragma unroll
      for (int k = 0; k < kPushBatch; ++k) {
        const uint64_t j = j0 + 32 * k + lane;
        u[k] = j < e ? nbr[j] : kNone;
      }
      uint32_t cur[kPushBatch];
#pragma unroll
      for (int k = 0; k < kPushBatch; ++k) cur[k] = u[k] != kNone ? stamp[u[k]] : value;
#pragma unroll
      for (int k = 0; k < kPushBatch; ++k)
        if (cur[k] != value) stamp[u[k]] = value;
    }
  }
}

template <class R>
__global__ void __launch_bounds__(kIterBigThreads) PushBigKernel(const uint32_t* __restrict__ list,
                                                                const uint32_t* __restrict__ starts,
                                                                const uint64_t* __restrict__ off,
                                                                const uint32_t* __restrict__ nbr,
                                                                uint32_t* __restrict__ stamp, StampValue sv, R row) {
  const uint32_t s0 = starts[kBinCta];
  const uint32_t count = starts[kNumBins] - s0;  // bins Cta, Global
  const uint32_t value = StampIn(sv.rs, sv.stamp);
  for (uint64_t i = blockIdx.x; i < count; i += gridDim.x) {
    const uint32_t v = list[s0 + i];
    if (!row(v)) continue;
    const uint64_t b = off[v], e = off[v + 1];
    for (uint64_t j0 = b; j0 < e; j0 += uint64_t(kIterBigThreads) * kPushBatch) {
      uint32_t u[kPushBatch];
#pragma unroll
      for (int k = 0; k < kPushBatch; ++k) {
        const uint64_t j = j0 + uint64_t(kIterBigThreads) * k + threadIdx.x;
        u[k] = j < e ? nbr[j] : kNone;
      }
      uint32_t cur[kPushBatch];
#pragma unroll
      for (int k = 0; k < kPushBatch; ++k) cur[k] = u[k] != kNone ? stamp[u[k]] : value;
#pragma unroll
      for (int k = 0; k < kPushBatch; ++k)
        if (cur[k] != value) stamp[u[k]] = value;
    }
  }
}

struct PushStampFn {
  const uint32_t* nbr;
  uint32_t* stamp;
  StampValue sv;
  __device__ void operator()(uint32_t, uint64_t j, uint64_t) const {
    const uint32_t u = nbr[j], value = StampIn(sv.rs, sv.stamp);
    if (stamp[u] != value) stamp[u] = value;
  }
};

// The push over a BinSet-layout list (starts on device; host_counts may be
// null: every shape launched).
template <class R>
inline void LaunchPush(Context* ctx, const uint32_t* list, const uint32_t* counts, const uint32_t* starts,
                       const uint32_t* host_counts, const uint64_t* off, const uint32_t* nbr, uint32_t* stamp,
                       StampValue sv, R row) {
  auto any = [&](int b0, int b1) {
    if (!host_counts) return true;
    for (int b = b0; b < b1; ++b)
      if (host_counts[b]) return true;
    return false;
  };
  cudaStream_t st = ctx->stream;
  if (any(kBinG4, kBinW128)) {
    EdgeIterSmallKernel<PushStampFn, R><<<IterSmallGrid(ctx), kIterThreads, 0, st>>>(
        list, counts, starts, off, PushStampFn{nbr, stamp, sv}, row);
    PCC_COUNT(1);
  }
  if (any(kBinW128, kBinCta)) {
    PushMidKernel<R><<<IterMidGrid(ctx), kIterThreads, 0, st>>>(list, starts, off, nbr, stamp, sv, row);
    PCC_COUNT(1);
  }
  if (any(kBinCta, kNumBins)) {
    PushBigKernel<R><<<IterBigGrid(ctx), kIterBigThreads, 0, st>>>(list, starts, off, nbr, stamp, sv, row);
    PCC_COUNT(1);
  }
}

// ---------------------------------------------------------------------------
// Degree binning of a vertex predicate over [0, n): count, starts, scatter.
// The order inside a bin is not specified (warp-aggregated atomics).
// ---------------------------------------------------------------------------
struct PredAll {
  __device__ bool operator()(uint32_t) const { return true; }
};
struct PredStamp {
  const uint32_t* st;
  uint32_t stamp;
  const RoundState* rs = nullptr;  // non-null: the stamp comes from here
  __device__ bool operator()(uint32_t v) const { return st[v] == StampIn(rs, stamp); }
};

template <class P>
__global__ void __launch_bounds__(256) BinCountKernel(uint32_t n, const uint64_t* __restrict__ off, P pred,
                                                      uint32_t* counts, unsigned long long* deg_sum,
                                                      uint32_t* vcount) {
  __shared__ uint32_t sh[kNumBins];
  __shared__ unsigned long long sh_deg;
  __shared__ uint32_t sh_cnt;
  if (threadIdx.x < kNumBins) sh[threadIdx.x] = 0;
  if (threadIdx.x == 0) {
    sh_deg = 0;
    sh_cnt = 0;
  }
  __syncthreads();
  uint32_t local[kNumBins];
#pragma unroll
  for (int b = 0; b < kNumBins; ++b) local[b] = 0;
  unsigned long long deg_acc = 0;
  uint32_t cnt = 0;
  for (uint64_t v = uint64_t(blockIdx.x) * 256 + threadIdx.x; v < n; v += uint64_t(gridDim.x) * 256) {
    if (!pred(static_cast<uint32_t>(v))) continue;
    const uint64_t d = off[v + 1] - off[v];
    const int b = BinOf(d);
#pragma unroll
    for (int q = 0; q < kNumBins; ++q) local[q] += (q == b);
    deg_acc += d;
    cnt++;
  }
#pragma unroll
  for (int q = 0; q < kNumBins; ++q)
    if (local[q]) atomicAdd(&sh[q], local[q]);
  if (deg_acc) atomicAdd(&sh_deg, deg_acc);
  if (cnt) atomicAdd(&sh_cnt, cnt);
  __syncthreads();
  if (threadIdx.x < kNumBins && sh[threadIdx.x]) atomicAdd(&counts[threadIdx.x], sh[threadIdx.x]);
  if (threadIdx.x == 0) {
    if (deg_sum && sh_deg) atomicAdd(deg_sum, sh_deg);
    if (vcount && sh_cnt) atomicAdd(vcount, sh_cnt);
  }
}

// Number and degree sum of the vertices satisfying pred (one pass over n).
template <class P, class CountT = uint32_t>
__global__ void __launch_bounds__(256) CountDegreesKernel(uint32_t n, const uint64_t* __restrict__ off, P pred,
                                                          unsigned long long* deg_sum, CountT* vcount) {
  unsigned long long dacc = 0;
  CountT cnt = 0;
  for (uint64_t v = uint64_t(blockIdx.x) * 256 + threadIdx.x; v < n; v += uint64_t(gridDim.x) * 256) {
    if (!pred(static_cast<uint32_t>(v))) continue;
    dacc += off[v + 1] - off[v];
    cnt++;
  }
  for (int o = 16; o >= 1; o >>= 1) {
    dacc += __shfl_xor_sync(kFull, dacc, o);
    cnt += __shfl_xor_sync(kFull, cnt, o);
  }
  __shared__ unsigned long long sd[8];
  __shared__ CountT sc[8];
  if (LaneId() == 0) {
    sd[threadIdx.x >> 5] = dacc;
    sc[threadIdx.x >> 5] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    CountT c = 0;
    for (int w = 0; w < 8; ++w) {
      t += sd[w];
      c += sc[w];
    }
    if (t) atomicAdd(deg_sum, t);
    if (c) atomicAdd(vcount, c);
  }
}

// counts[0..B) -> starts[0..B] and cursors zeroed.
__global__ void BinStartsKernel(const uint32_t* counts, uint32_t* starts, uint32_t* cursor);

template <class P>
__global__ void __launch_bounds__(256) BinScatterKernel(uint32_t n, const uint64_t* __restrict__ off, P pred,
                                                        const uint32_t* __restrict__ starts, uint32_t* cursor,
                                                        uint32_t* list) {
  const uint64_t stride = uint64_t(gridDim.x) * 256;
  const uint64_t limit = (uint64_t(n) + 31) & ~uint64_t(31);
  for (uint64_t v = uint64_t(blockIdx.x) * 256 + threadIdx.x; v < limit; v += stride) {
    const bool in = v < n && pred(static_cast<uint32_t>(v));
    const int bin = in ? BinOf(off[v + 1] - off[v]) : kNumBins + int(LaneId());
    const unsigned peers = __match_any_sync(kFull, bin);
    uint32_t base = 0;
    const int leader = __ffs(peers) - 1;
    if (in && int(LaneId()) == leader) base = atomicAdd(&cursor[bin], uint32_t(__popc(peers)));
    base = __shfl_sync(kFull, base, leader);
    if (in) list[starts[bin] + base + __popc(peers & LaneMaskLt())] = static_cast<uint32_t>(v);
  }
}

// Bins the vertices of [0, n) that satisfy pred into b (list must hold n
// entries, counts 3 * kNumBins + 1).  deg_sum / vcount (device, nullable)
// accumulate the sum of degrees and the number of binned vertices.
template <class P>
Status BinVertices(Context* ctx, uint32_t n, const uint64_t* off, P pred, BinSet* b,
                   unsigned long long* deg_sum, uint32_t* vcount) {
  uint32_t* counts = b->counts.p;
  uint32_t* starts = counts + kNumBins;
  uint32_t* cursor = starts + kNumBins + 1;
  PCC_CUDA(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * kNumBins, ctx->stream));
  const unsigned grid = Blocks(n, 256, unsigned(ctx->num_sms) * 16);
  if (n) {
    BinCountKernel<P><<<grid, 256, 0, ctx->stream>>>(n, off, pred, counts, deg_sum, vcount);
    PCC_COUNT(1);
  }
  BinStartsKernel<<<1, 1, 0, ctx->stream>>>(counts, starts, cursor);
  PCC_COUNT(1);
  if (n) {
    BinScatterKernel<P><<<grid, 256, 0, ctx->stream>>>(n, off, pred, starts, cursor, b->list.p);
    PCC_COUNT(1);
  }
  return LaunchCheck();
}

inline Status AllocBins(Context* ctx, uint32_t n, BinSet* b) {
  PCC_RETURN_IF_ERROR(b->list.Reserve(ctx, std::max<uint64_t>(n, 1)));
  PCC_RETURN_IF_ERROR(b->counts.Reserve(ctx, 3 * kNumBins + 1));
  return Status::Ok();
}

}  // namespace pcc
