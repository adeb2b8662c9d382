// primitives.cuh -- device-wide scan / compaction / reduction and a stable
// LSD radix sort of (uint64 key, uint32 value) pairs.  These replace the
// pbbslib scan, filter, reduce and stable sample sort that the reference
// calls (parallel/parallel-sequence-ops.h:38-232).
#pragma once

#include <mutex>

#include "common.cuh"

namespace pcc {

// ---------------------------------------------------------------------------
// Exclusive scan in three phases over a functor input f(i) -> T (uint32 or
// uint64): per-tile reduce, scan of the tile sums, per-tile scan + write.
// The writer w(i, exclusive_prefix, value) consumes the result, which lets
// the same code express prefix sums, compactions and offset arrays.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ T WarpInclusiveScan(T x) {
  const unsigned lane = LaneId();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= unsigned(o)) x += y;
  }
  return x;
}

// Exclusive block scan of one value per thread (256 threads); returns the
// prefix and writes the block total to *total.
template <class T>
__device__ __forceinline__ T BlockExclusiveScan(T x, T* total) {
  __shared__ T warp_sums[kScanThreads / 32];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  T inc = WarpInclusiveScan(x);
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T s = lane < kScanThreads / 32 ? warp_sums[lane] : T(0);
    T si = WarpInclusiveScan(s);
    if (lane < kScanThreads / 32) warp_sums[lane] = si - s;
    if (lane == kScanThreads / 32 - 1) *total = si;
  }
  __syncthreads();
  T r = inc - x + warp_sums[warp];
  __syncthreads();
  return r;
}

template <class T, class F>
__global__ void __launch_bounds__(kScanThreads) ScanTileReduceKernel(uint64_t n, F f, T* tile_sums) {
  const uint64_t base = uint64_t(blockIdx.x) * kScanTile;
  T acc = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = base + uint64_t(j) * kScanThreads + threadIdx.x;
    if (i < n) acc += f(i);
  }
  __shared__ T total;
  BlockExclusiveScan<T>(acc, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Single block: exclusive scan of tile_sums in place; grand total to *total.
template <class T>
__global__ void __launch_bounds__(1024) ScanTileSumsKernel(uint64_t tiles, T* tile_sums, T* total) {
  __shared__ T part[1024];
  const uint64_t per = (tiles + 1023) / 1024;
  const uint64_t s = uint64_t(threadIdx.x) * per;
  const uint64_t e = s + per < tiles ? s + per : tiles;
  T acc = 0;
  for (uint64_t i = s; i < e; ++i) acc += tile_sums[i];
  part[threadIdx.x] = acc;
  __syncthreads();
  // Hillis-Steele over 1024 partials.
  for (int o = 1; o < 1024; o <<= 1) {
    T y = threadIdx.x >= unsigned(o) ? part[threadIdx.x - o] : T(0);
    __syncthreads();
    part[threadIdx.x] += y;
    __syncthreads();
  }
  T run = part[threadIdx.x] - acc;
  for (uint64_t i = s; i < e; ++i) {
    T v = tile_sums[i];
    tile_sums[i] = run;
    run += v;
  }
  if (threadIdx.x == 1023 && total) *total = part[1023];
}

template <class T, class F, class W>
__global__ void __launch_bounds__(kScanThreads) ScanTileApplyKernel(uint64_t n, F f, const T* tile_sums, W w) {
  __shared__ T vals[kScanTile];
  const uint64_t base = uint64_t(blockIdx.x) * kScanTile;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = base + uint64_t(j) * kScanThreads + threadIdx.x;
    vals[j * kScanThreads + threadIdx.x] = i < n ? f(i) : T(0);
  }
  __syncthreads();
  T local[kScanItems];
  T acc = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    local[j] = vals[threadIdx.x * kScanItems + j];
    acc += local[j];
  }
  __shared__ T total;
  T pre = BlockExclusiveScan<T>(acc, &total) + tile_sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = base + uint64_t(threadIdx.x) * kScanItems + j;
    if (i < n) w(i, pre, local[j]);
    pre += local[j];
  }
}

// Scratch for scans: tile sums.  `total` (device) receives the grand total.
template <class T, class F, class W>
Status ScanApply(Context* ctx, uint64_t n, F f, W w, DBuf<T>& tile_buf, T* d_total) {
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 0) {
    if (d_total) PCC_CUDA(cudaMemsetAsync(d_total, 0, sizeof(T), ctx->stream));
    return Status::Ok();
  }
  PCC_RETURN_IF_ERROR(tile_buf.Reserve(ctx, tiles));
  ScanTileReduceKernel<T, F><<<unsigned(tiles), kScanThreads, 0, ctx->stream>>>(n, f, tile_buf.p); PCC_COUNT(1);
  ScanTileSumsKernel<T><<<1, 1024, 0, ctx->stream>>>(tiles, tile_buf.p, d_total); PCC_COUNT(1);
  ScanTileApplyKernel<T, F, W><<<unsigned(tiles), kScanThreads, 0, ctx->stream>>>(n, f, tile_buf.p, w); PCC_COUNT(1);
  return LaunchCheck();
}

// Writers / inputs used with ScanApply.
template <class T>
struct StorePrefix {
  T* out;
  __device__ void operator()(uint64_t i, T pre, T) const { out[i] = pre; }
};
// Compaction: appends index i when value != 0, in ascending order.
struct StoreIndexIfSet {
  uint32_t* out;
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t v) const {
    if (v) out[pre] = static_cast<uint32_t>(i);
  }
};

// ---------------------------------------------------------------------------
// Reductions (deterministic: per-block partials then one block).
// ---------------------------------------------------------------------------
template <class T, class F, class Op>
__global__ void __launch_bounds__(256) BlockReduceKernel(uint64_t n, F f, Op op, T ident, T* partial) {
  T acc = ident;
  for (uint64_t i = uint64_t(blockIdx.x) * 256 + threadIdx.x; i < n; i += uint64_t(gridDim.x) * 256)
    acc = op(acc, f(i));
  __shared__ T sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < unsigned(o)) sh[threadIdx.x] = op(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

template <class T, class Op>
__global__ void __launch_bounds__(256) FinalReduceKernel(const T* partial, unsigned parts, Op op, T ident, T* out) {
  T acc = ident;
  for (unsigned i = threadIdx.x; i < parts; i += 256) acc = op(acc, partial[i]);
  __shared__ T sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < unsigned(o)) sh[threadIdx.x] = op(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

template <class T, class F, class Op>
Status Reduce(Context* ctx, uint64_t n, F f, Op op, T ident, T* d_out, DBuf<T>& partial) {
  const unsigned blocks = Blocks(n, 256 * 4, unsigned(ctx->num_sms) * 4);
  PCC_RETURN_IF_ERROR(partial.Reserve(ctx, blocks));
  BlockReduceKernel<T, F, Op><<<blocks, 256, 0, ctx->stream>>>(n, f, op, ident, partial.p); PCC_COUNT(1);
  FinalReduceKernel<T, Op><<<1, 256, 0, ctx->stream>>>(partial.p, blocks, op, ident, d_out); PCC_COUNT(1);
  return LaunchCheck();
}

struct OpAdd {
  template <class T>
  __device__ T operator()(T a, T b) const { return a + b; }
};
struct OpMax {
  template <class T>
  __device__ T operator()(T a, T b) const { return a > b ? a : b; }
};

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (uint64 key, uint32 value) pairs, 8-bit digits.
// Per pass: per-tile digit histograms, a scan of the digit-major histogram
// table, and a scatter whose in-tile ranks come from warp-level match
// (lanes in order, rounds in order, warps in order), which keeps the sort
// stable -- the property ComputeInterClusterEdgesSort relies on.
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;

static __global__ void __launch_bounds__(kSortThreads) RadixHistKernel(const uint64_t* keys, uint64_t n, int shift,
                                                                uint32_t* hist, uint32_t tiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint64_t wbase = uint64_t(blockIdx.x) * kSortTile + uint64_t(warp) * 32 * kSortItems;
#pragma unroll 4
  for (int r = 0; r < kSortItems; ++r) {
    const uint64_t i = wbase + uint64_t(r) * 32 + lane;
    const bool valid = i < n;
    const uint32_t d = valid ? uint32_t((keys[i] >> shift) & 255u) : 256u + lane;
    const unsigned peers = __match_any_sync(kFull, d);
    if (valid && int(lane) == __ffs(peers) - 1) atomicAdd(&h[d], __popc(peers));
  }
  __syncthreads();
  hist[uint64_t(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

// Scatter of one tile: ranks inside the tile in stable order (digit, then
// item order: warps, rounds, lanes), the tile staged in shared memory in
// that order, then each digit's run written by consecutive threads to its
// global range (coalesced stores).  Dynamic shared memory: kSortScatterSmem.
constexpr size_t kSortScatterSmem = size_t(kSortTile) * (sizeof(uint64_t) + sizeof(uint32_t));

static __global__ void __launch_bounds__(kSortThreads) RadixScatterKernel(const uint64_t* keys_in, const uint32_t* vals_in,
                                                                   uint64_t* keys_out, uint32_t* vals_out, uint64_t n,
                                                                   int shift, const uint32_t* offsets, uint32_t tiles) {
  extern __shared__ __align__(16) unsigned char sort_smem[];
  uint64_t* sk = reinterpret_cast<uint64_t*>(sort_smem);
  uint32_t* sv = reinterpret_cast<uint32_t*>(sort_smem + size_t(kSortTile) * sizeof(uint64_t));
  __shared__ uint32_t wcount[kSortWarps][256];
  __shared__ uint32_t dstart[256];   // tile-local start of each digit's run
  __shared__ uint32_t goff[256];     // global start of this tile's run of each digit
  __shared__ uint32_t wsum[kSortWarps];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  for (int d = lane; d < 256; d += 32) wcount[warp][d] = 0;
  __syncwarp();
  const uint64_t tbase = uint64_t(blockIdx.x) * kSortTile;
  const uint64_t wbase = tbase + uint64_t(warp) * 32 * kSortItems;
  // Only the digit and the in-warp rank of each item stay in registers
  // across the block-wide scan (16 bits each); the key and value are read
  // again for the staging writes (the tile is still in L1/L2), which keeps
  // the register count, and so the warps resident per SM, in check.
  uint32_t dp[kSortItems];  // (digit << 16) | rank within the warp's digit run
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const uint64_t i = wbase + uint64_t(r) * 32 + lane;
    const bool valid = i < n;
    const uint32_t d = valid ? uint32_t((keys_in[i] >> shift) & 255u) : 256u + lane;
    const unsigned peers = __match_any_sync(kFull, d);
    uint32_t base = 0;
    if (valid) base = wcount[warp][d];
    __syncwarp();
    if (valid && int(lane) == __ffs(peers) - 1) wcount[warp][d] = base + __popc(peers);
    __syncwarp();
    dp[r] = ((d & 255u) << 16) | (base + __popc(peers & LaneMaskLt()));
  }
  __syncthreads();
  // Thread d: exclusive scan across warps of digit d (in place), the
  // digit's tile total, and its global offset.
  const unsigned d = threadIdx.x;
  uint32_t tot = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) {
    const uint32_t t = wcount[w][d];
    wcount[w][d] = tot;
    tot += t;
  }
  goff[d] = offsets[uint64_t(d) * tiles + blockIdx.x];
  // Exclusive scan of the digit totals over the block (digit order).
  uint32_t incl = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, incl, o);
    if (lane >= unsigned(o)) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  uint32_t wpre = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) wpre += unsigned(w) < warp ? wsum[w] : 0u;
  dstart[d] = wpre + incl - tot;
  __syncthreads();
#pragma unroll 4
  for (int r = 0; r < kSortItems; ++r) {
    const uint64_t i = wbase + uint64_t(r) * 32 + lane;
    if (i < n) {
      const uint32_t dg = dp[r] >> 16;
      const uint32_t li = dstart[dg] + wcount[warp][dg] + (dp[r] & 0xFFFFu);
      sk[li] = keys_in[i];
      sv[li] = vals_in[i];
    }
  }
  __syncthreads();
  const uint32_t cnt = n - tbase < uint64_t(kSortTile) ? uint32_t(n - tbase) : uint32_t(kSortTile);
  for (uint32_t t = threadIdx.x; t < cnt; t += kSortThreads) {
    const uint64_t key = sk[t];
    const uint32_t dg = uint32_t((key >> shift) & 255u);
    const uint32_t o = goff[dg] + (t - dstart[dg]);
    keys_out[o] = key;
    vals_out[o] = sv[t];
  }
}

struct HistInput {
  const uint32_t* h;
  __device__ uint32_t operator()(uint64_t i) const { return h[i]; }
};

struct SortScratch {
  DBuf<uint64_t> keys;
  DBuf<uint32_t> vals;
  DBuf<uint32_t> hist;
  DBuf<uint32_t> tile_sums;
};

// Sorts keys[0..n) (with vals) by the low `bits` bits of the key; the
// result is left in keys/vals.  n < 2^32.
static inline Status RadixSortPairs(Context* ctx, uint64_t* keys, uint32_t* vals, uint64_t n, int bits,
                             SortScratch& sc) {
  if (n <= 1 || bits <= 0) return Status::Ok();
  const uint32_t tiles = uint32_t((n + kSortTile - 1) / kSortTile);
  PCC_RETURN_IF_ERROR(sc.keys.Reserve(ctx, n));
  PCC_RETURN_IF_ERROR(sc.vals.Reserve(ctx, n));
  PCC_RETURN_IF_ERROR(sc.hist.Reserve(ctx, uint64_t(tiles) * 256));
  uint64_t* kin = keys;
  uint32_t* vin = vals;
  uint64_t* kout = sc.keys.p;
  uint32_t* vout = sc.vals.p;
  const int passes = (bits + 7) / 8;
  {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
      attr = cudaFuncSetAttribute(RadixScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(kSortScatterSmem));
    });
    PCC_CUDA(attr);
  }
  for (int p = 0; p < passes; ++p) {
    const int shift = p * 8;
    RadixHistKernel<<<tiles, kSortThreads, 0, ctx->stream>>>(kin, n, shift, sc.hist.p, tiles); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, uint64_t(tiles) * 256, HistInput{sc.hist.p},
                                            StorePrefix<uint32_t>{sc.hist.p}, sc.tile_sums,
                                            static_cast<uint32_t*>(nullptr)));
    RadixScatterKernel<<<tiles, kSortThreads, kSortScatterSmem, ctx->stream>>>(kin, vin, kout, vout, n, shift,
                                                                               sc.hist.p, tiles); PCC_COUNT(1);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys) {
    PCC_CUDA(cudaMemcpyAsync(keys, kin, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, ctx->stream));
    PCC_CUDA(cudaMemcpyAsync(vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return LaunchCheck();
}

}  // namespace pcc
