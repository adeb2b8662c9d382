// compress.cu -- graph contraction.
//
// Restates CompressGraph (clustering/clusterers/parallel-correlation-
// clusterer-internal.cc:709-782) with ComputeInterClusterEdgesSort,
// RetrieveInterClusterEdges and GetOffsets (parallel/parallel-graph-utils.cc:
// 33-122, 156-231):
//   * entry (u, v, w) is kept when v <= u or C(u) != C(v) (one copy of each
//     intra-cluster edge, :102);
//   * kept entries, in CSR order, are stably sorted by (C(u), C(v));
//   * equal pairs are summed in FP32 in that order with the pbbs blocked
//     reduce (serial fold of <= 1024 items, else serial folds of 1024-item
//     blocks followed by a reduce of the block sums);
//   * the new graph has 1 + max C vertices (cluster ids are not compacted);
//   * new node weight of cluster c = sum of the node weights of its members.
//
// GB300 shape: most-significant key first, without a global sort of the
// entries.  The vertices are stably sorted by cluster (a radix sort over n,
// not m), so the rows of a cluster's members, in ascending vertex order and
// each in CSR order, form the cluster's contiguous segment of a cluster-
// ordered entry array -- exactly the kept entries stably sorted by C(u), plus
// the dropped second copies of intra-cluster edges, marked with a key above
// every cluster rank.  One pass moves every row into place (4-byte keys: the
// dense rank of C(v)).  Each segment is then sorted by key and folded where
// it lies: segments of up to kSegWarpMax entries by one warp (rank by
// counting in shared memory), up to kSegCtaMax by one CTA (stable LSD radix
// passes in shared memory), longer ones by the global stable radix sort of
// primitives.cuh over (segment, key).  The unique pairs of a segment are
// written over its own start, and a final pass copies them into the new CSR.
// Traffic per level: the CSR once (ids, weights, cluster gathers), the
// 8-byte moved entries written and read once, the unique pairs twice.
#include "graphops.cuh"

namespace pcc {

namespace {

constexpr uint32_t kSegWarpMax = 64;    // one warp: two entries per lane
constexpr uint32_t kSegMidMax = 512;    // one warp: radix passes in shared memory
constexpr uint32_t kSegCtaMax = 4096;   // one CTA: the segment in shared memory
constexpr int kSegMidItems = kSegMidMax / 32;
constexpr int kSegCtaThreads = 256;
constexpr int kSegCtaItems = kSegCtaMax / kSegCtaThreads;
constexpr int kSegCtaWarps = kSegCtaThreads / 32;

struct MaxOfU32 {
  const uint32_t* a;
  __device__ uint32_t operator()(uint64_t i) const { return a[i]; }
};

__global__ void MarkPresentKernel(uint32_t n, const uint32_t* __restrict__ C, uint32_t* __restrict__ pres) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    pres[C[i]] = 1u;
}

struct PresInput {
  const uint32_t* pres;
  __device__ uint32_t operator()(uint64_t i) const { return pres[i]; }
};
struct RankWriter {
  uint32_t* rank;
  uint32_t* ids;
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t v) const {
    rank[i] = pre;
    if (v) ids[pre] = static_cast<uint32_t>(i);
  }
};

// Vertex sort keys: the dense rank of the vertex's cluster.
__global__ void VertexKeysKernel(uint32_t n, const uint32_t* __restrict__ C, const uint32_t* __restrict__ rank,
                                 uint64_t* __restrict__ vkey, uint32_t* __restrict__ vval) {
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < n; u += uint64_t(gridDim.x) * blockDim.x) {
    vkey[u] = rank[C[u]];
    vval[u] = static_cast<uint32_t>(u);
  }
}

// Degree of the p-th vertex in cluster order; the writer records where its
// row starts in the cluster-ordered entry array.
struct SortedDegInput {
  const uint64_t* off;
  const uint32_t* vval;
  __device__ uint64_t operator()(uint64_t p) const {
    const uint32_t u = vval[p];
    return off[u + 1] - off[u];
  }
};
struct RowStartWriter {
  const uint32_t* vval;
  uint64_t* dstart;
  __device__ void operator()(uint64_t p, uint64_t pre, uint64_t) const { dstart[vval[p]] = pre; }
};

// segbase[r] = first slot of cluster rank r's segment; segbase[R] = m.
__global__ void SegBaseKernel(uint32_t n, const uint64_t* __restrict__ vkey, const uint32_t* __restrict__ vval,
                              const uint64_t* __restrict__ dstart, uint64_t* __restrict__ segbase, uint32_t R,
                              uint64_t m) {
  for (uint64_t p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += uint64_t(gridDim.x) * blockDim.x) {
    if (p == 0 || vkey[p] != vkey[p - 1]) segbase[vkey[p]] = dstart[vval[p]];
    if (p == 0) segbase[R] = m;
  }
}

// Moves every entry to its row's place in the cluster-ordered array.
struct MoveEntries {
  const uint64_t* off;
  const uint32_t* nbr;
  const float* w;
  const uint32_t* C;
  const uint32_t* rank;
  const uint64_t* dstart;
  uint32_t drop;
  uint32_t* akey;
  uint32_t* aval;
  __device__ void operator()(uint32_t u, uint64_t j, uint64_t) const {
    const uint32_t v = nbr[j];
    const uint32_t cu = C[u], cv = C[v];
    const bool keep = v <= u || cu != cv;
    const uint64_t d = dstart[u] + (j - off[u]);
    akey[d] = keep ? rank[cv] : drop;
    aval[d] = __float_as_uint(w ? w[j] : 1.0f);
  }
};

// Segment classes (by entries): counting warp, radix warp, CTA, global.
// counts[c] = length of class c's list (lists[c] holds R slots).
__global__ void ClassifyKernel(uint32_t R, const uint64_t* __restrict__ segbase, uint32_t* __restrict__ lists,
                               uint32_t* __restrict__ counts, unsigned long long* __restrict__ big_entries) {
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < R; r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t len = segbase[r + 1] - segbase[r];
    if (len == 0) continue;
    const int c = len <= kSegWarpMax ? 0 : len <= kSegMidMax ? 1 : len <= kSegCtaMax ? 2 : 3;
    lists[uint64_t(c) * R + atomicAdd(&counts[c], 1u)] = static_cast<uint32_t>(r);
    if (c == 3) atomicAdd(big_entries, static_cast<unsigned long long>(len));
  }
}

// pbbs blocked FP32 sum of x[0..len) (len >= 1), x as float bits.
__device__ __forceinline__ float BlockedFold(const uint32_t* x, uint32_t len) {
  auto serial = [&](uint32_t a, uint32_t l) {
    float r = __uint_as_float(x[a]);
    for (uint32_t j = 1; j < l; ++j) r = __fadd_rn(r, __uint_as_float(x[a + j]));
    return r;
  };
  if (len <= 1024) return serial(0, len);
  float r = serial(0, 1024);
  for (uint32_t b = 1024; b < len; b += 1024) r = __fadd_rn(r, serial(b, min(1024u, len - b)));
  return r;
}

// Segments of at most kSegWarpMax entries, one warp each: an entry's output
// rank is the number of distinct smaller keys; the first entry of each key
// folds its run in segment (= CSR) order.  Runs are at most 64 entries, so
// the fold is the serial one.
__global__ void __launch_bounds__(256) SegWarpKernel(const uint32_t* __restrict__ list,
                                                     const uint32_t* __restrict__ counts,
                                                     const uint64_t* __restrict__ segbase,
                                                     const uint32_t* __restrict__ ids, uint32_t drop,
                                                     uint32_t* __restrict__ akey, uint32_t* __restrict__ aval,
                                                     uint32_t* __restrict__ ucount) {
  __shared__ uint32_t sk[8][kSegWarpMax], sv[8][kSegWarpMax];
  __shared__ uint8_t sf[8][kSegWarpMax];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  const uint32_t cnt = counts[0];
  for (uint64_t i = uint64_t(blockIdx.x) * 8 + warp; i < cnt; i += uint64_t(gridDim.x) * 8) {
    const uint32_t r = list[i];
    const uint64_t b = segbase[r];
    const uint32_t len = static_cast<uint32_t>(segbase[r + 1] - b);
    uint32_t k[2], v[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t t = lane + 32 * h;
      k[h] = t < len ? akey[b + t] : kNone;
      v[h] = t < len ? aval[b + t] : 0u;
      sk[warp][t] = k[h];
      sv[warp][t] = v[h];
    }
    __syncwarp();
    bool first[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t t = lane + 32 * h;
      bool f = t < len && k[h] < drop;
      for (uint32_t j = 0; f && j < t; ++j) f = sk[warp][j] != k[h];
      first[h] = f;
      sf[warp][t] = f ? 1 : 0;
    }
    __syncwarp();
    uint32_t orank[2] = {0, 0};
    float sum[2] = {0.f, 0.f};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!first[h]) continue;
      const uint32_t t = lane + 32 * h;
      uint32_t rk = 0;
      float acc = __uint_as_float(v[h]);
      for (uint32_t j = 0; j < len; ++j) {
        const uint32_t kj = sk[warp][j];
        if (sf[warp][j] && kj < k[h]) ++rk;
        if (j > t && kj == k[h]) acc = __fadd_rn(acc, __uint_as_float(sv[warp][j]));
      }
      orank[h] = rk;
      sum[h] = acc;
    }
    __syncwarp();  // every read of the segment is done: write over its start
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!first[h]) continue;
      akey[b + orank[h]] = ids[k[h]];
      aval[b + orank[h]] = __float_as_uint(sum[h]);
    }
    const uint32_t u = __popc(__ballot_sync(kFull, first[0])) + __popc(__ballot_sync(kFull, first[1]));
    if (lane == 0) ucount[r] = u;
    __syncwarp();
  }
}

// Segments of kSegWarpMax+1 .. kSegMidMax entries, one warp each: stable
// LSD radix passes (8-bit digits, ranks by match in index order) between two
// shared-memory buffers of the warp, then the heads of the kept runs, their
// output ranks by ballot, and the head lane folding its run (at most 512
// entries: the serial fold).
constexpr int kSegMidWarps = 4;
constexpr size_t kSegMidSmem = size_t(kSegMidWarps) * (size_t(kSegMidMax) * 16 + 256 * 4);

__global__ void __launch_bounds__(kSegMidWarps * 32) SegMidKernel(const uint32_t* __restrict__ list,
                                                                 const uint32_t* __restrict__ counts,
                                                                 const uint64_t* __restrict__ segbase,
                                                                 const uint32_t* __restrict__ ids, uint32_t drop,
                                                                 int passes, uint32_t* __restrict__ akey,
                                                                 uint32_t* __restrict__ aval,
                                                                 uint32_t* __restrict__ ucount) {
  extern __shared__ __align__(16) unsigned char mid_smem[];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  uint32_t* k0 = reinterpret_cast<uint32_t*>(mid_smem + size_t(warp) * (size_t(kSegMidMax) * 16 + 256 * 4));
  uint32_t* v0 = k0 + kSegMidMax;
  uint32_t* k1 = v0 + kSegMidMax;
  uint32_t* v1 = k1 + kSegMidMax;
  uint32_t* hist = v1 + kSegMidMax;  // 256 digit counters
  const uint32_t cnt = counts[1];
  for (uint64_t i = uint64_t(blockIdx.x) * kSegMidWarps + warp; i < cnt; i += uint64_t(gridDim.x) * kSegMidWarps) {
    const uint32_t r = list[i];
    const uint64_t b = segbase[r];
    const uint32_t len = static_cast<uint32_t>(segbase[r + 1] - b);
    const int nq = int((len + 31) / 32);
    for (uint32_t t = lane; t < len; t += 32) {
      k0[t] = akey[b + t];
      v0[t] = aval[b + t];
    }
    __syncwarp();
    uint32_t* kin = k0;
    uint32_t* vin = v0;
    uint32_t* kout = k1;
    uint32_t* vout = v1;
    for (int pass = 0; pass < passes; ++pass) {
      const int shift = pass * 8;
      for (int d = lane; d < 256; d += 32) hist[d] = 0;
      __syncwarp();
      uint32_t dp[kSegMidItems];
#pragma unroll
      for (int q = 0; q < kSegMidItems; ++q) {
        if (q >= nq) break;
        const uint32_t t = uint32_t(q) * 32 + lane;
        const bool valid = t < len;
        const uint32_t d = valid ? (kin[t] >> shift) & 255u : 256u + lane;
        const unsigned peers = __match_any_sync(kFull, d);
        uint32_t base = 0;
        if (valid) base = hist[d];
        __syncwarp();
        if (valid && int(lane) == __ffs(peers) - 1) hist[d] = base + __popc(peers);
        __syncwarp();
        dp[q] = ((d & 255u) << 16) | (base + __popc(peers & LaneMaskLt()));
      }
      // Exclusive scan of the 256 digit counts: 8 per lane, lanes in order.
      uint32_t c8[8], sum = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        c8[j] = hist[lane * 8 + j];
        sum += c8[j];
      }
      const uint32_t incl = WarpInclusiveScan<uint32_t>(sum);
      uint32_t run = incl - sum;
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        hist[lane * 8 + j] = run;
        run += c8[j];
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < kSegMidItems; ++q) {
        if (q >= nq) break;
        const uint32_t t = uint32_t(q) * 32 + lane;
        if (t < len) {
          const uint32_t o = hist[dp[q] >> 16] + (dp[q] & 0xFFFFu);
          kout[o] = kin[t];
          vout[o] = vin[t];
        }
      }
      __syncwarp();
      uint32_t* tk = kin;
      kin = kout;
      kout = tk;
      uint32_t* tv = vin;
      vin = vout;
      vout = tv;
    }
    uint32_t pre = 0;
    for (int q = 0; q < nq; ++q) {
      const uint32_t t = uint32_t(q) * 32 + lane;
      const bool head = t < len && kin[t] < drop && (t == 0 || kin[t - 1] != kin[t]);
      const unsigned hb = __ballot_sync(kFull, head);
      if (head) {
        uint32_t e = t + 1;
        float acc = __uint_as_float(vin[t]);
        while (e < len && kin[e] == kin[t]) {
          acc = __fadd_rn(acc, __uint_as_float(vin[e]));
          ++e;
        }
        const uint32_t o = pre + __popc(hb & LaneMaskLt());
        akey[b + o] = ids[kin[t]];
        aval[b + o] = __float_as_uint(acc);
      }
      pre += __popc(hb);
    }
    if (lane == 0) ucount[r] = pre;
    __syncwarp();
  }
}

// Segments of kSegMidMax+1 .. kSegCtaMax entries, one CTA each: stable LSD
// radix passes (8-bit digits, ranks by warp match in item order) between two
// shared-memory buffers, then heads, a block scan of the heads for the
// output ranks, and one thread per run folding it (pbbs blocked rule).
constexpr size_t kSegCtaSmem = size_t(kSegCtaMax) * 4 * 4;  // two (key, value) buffers

__global__ void __launch_bounds__(kSegCtaThreads) SegCtaKernel(const uint32_t* __restrict__ list,
                                                              const uint32_t* __restrict__ counts,
                                                              const uint64_t* __restrict__ segbase,
                                                              const uint32_t* __restrict__ ids, uint32_t drop,
                                                              int passes, uint32_t* __restrict__ akey,
                                                              uint32_t* __restrict__ aval,
                                                              uint32_t* __restrict__ ucount) {
  extern __shared__ __align__(16) unsigned char seg_smem[];
  uint32_t* k0 = reinterpret_cast<uint32_t*>(seg_smem);
  uint32_t* v0 = k0 + kSegCtaMax;
  uint32_t* k1 = v0 + kSegCtaMax;
  uint32_t* v1 = k1 + kSegCtaMax;
  __shared__ uint32_t wcount[kSegCtaWarps][256];
  __shared__ uint32_t dstart[256];
  __shared__ uint32_t wsum[kSegCtaWarps];
  __shared__ uint32_t s_total;
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5, tid = threadIdx.x;
  const uint32_t cnt = counts[2];
  for (uint32_t li = blockIdx.x; li < cnt; li += gridDim.x) {
    const uint32_t r = list[li];
    const uint64_t b = segbase[r];
    const uint32_t len = static_cast<uint32_t>(segbase[r + 1] - b);
    for (uint32_t t = tid; t < len; t += kSegCtaThreads) {
      k0[t] = akey[b + t];
      v0[t] = aval[b + t];
    }
    // Rounds of 32 items this warp holds (its items are [warp * 32 *
    // kSegCtaItems, ...)), so the cost follows the segment's length.
    const uint32_t wfirst = warp * 32 * kSegCtaItems;
    const int nq = len > wfirst ? int(min(uint32_t(kSegCtaItems), (len - wfirst + 31) / 32)) : 0;
    __syncthreads();
    uint32_t* kin = k0;
    uint32_t* vin = v0;
    uint32_t* kout = k1;
    uint32_t* vout = v1;
    for (int pass = 0; pass < passes; ++pass) {
      const int shift = pass * 8;
      for (int d = lane; d < 256; d += 32) wcount[warp][d] = 0;
      __syncwarp();
      // Items of warp w: [w * 32 * kSegCtaItems, (w + 1) * 32 * kSegCtaItems),
      // visited in index order (rounds, then lanes).
      uint32_t dp[kSegCtaItems];
#pragma unroll
      for (int q = 0; q < kSegCtaItems; ++q) {
        if (q >= nq) break;
        const uint32_t t = (warp * kSegCtaItems + q) * 32 + lane;
        const bool valid = t < len;
        const uint32_t d = valid ? (kin[t] >> shift) & 255u : 256u + lane;
        const unsigned peers = __match_any_sync(kFull, d);
        uint32_t base = 0;
        if (valid) base = wcount[warp][d];
        __syncwarp();
        if (valid && int(lane) == __ffs(peers) - 1) wcount[warp][d] = base + __popc(peers);
        __syncwarp();
        dp[q] = ((d & 255u) << 16) | (base + __popc(peers & LaneMaskLt()));
      }
      __syncthreads();
      const unsigned d = tid;  // 256 threads = 256 digits
      uint32_t tot = 0;
#pragma unroll
      for (int w = 0; w < kSegCtaWarps; ++w) {
        const uint32_t x = wcount[w][d];
        wcount[w][d] = tot;
        tot += x;
      }
      uint32_t incl = WarpInclusiveScan<uint32_t>(tot);
      if (lane == 31) wsum[warp] = incl;
      __syncthreads();
      uint32_t wpre = 0;
#pragma unroll
      for (int w = 0; w < kSegCtaWarps; ++w) wpre += unsigned(w) < warp ? wsum[w] : 0u;
      dstart[d] = wpre + incl - tot;
      __syncthreads();
#pragma unroll
      for (int q = 0; q < kSegCtaItems; ++q) {
        if (q >= nq) break;
        const uint32_t t = (warp * kSegCtaItems + q) * 32 + lane;
        if (t < len) {
          const uint32_t dg = dp[q] >> 16;
          const uint32_t o = dstart[dg] + wcount[warp][dg] + (dp[q] & 0xFFFFu);
          kout[o] = kin[t];
          vout[o] = vin[t];
        }
      }
      __syncthreads();
      uint32_t* tk = kin;
      kin = kout;
      kout = tk;
      uint32_t* tv = vin;
      vin = vout;
      vout = tv;
    }
    // Heads of the kept runs and their output ranks (items t = tid * kSegCtaItems + q).
    uint32_t heads = 0;
#pragma unroll
    for (int q = 0; q < kSegCtaItems; ++q) {
      const uint32_t t = tid * kSegCtaItems + q;
      if (t < len && kin[t] < drop && (t == 0 || kin[t - 1] != kin[t])) heads |= 1u << q;
    }
    uint32_t pre = BlockExclusiveScan<uint32_t>(uint32_t(__popc(heads)), &s_total);
#pragma unroll
    for (int q = 0; q < kSegCtaItems; ++q) {
      if (!(heads & (1u << q))) continue;
      const uint32_t t = tid * kSegCtaItems + q;
      uint32_t e = t + 1;
      while (e < len && kin[e] == kin[t]) ++e;
      const float sum = BlockedFold(vin + t, e - t);
      // The segment was read into shared memory before the first pass.
      akey[b + pre] = ids[kin[t]];
      aval[b + pre] = __float_as_uint(sum);
      ++pre;
    }
    if (tid == 0) ucount[r] = s_total;
    __syncthreads();
  }
}

// Global path: the entries of segments longer than kSegCtaMax, keyed by
// (index in big_list, key) for the stable radix sort.  Work is split into
// chunks of kSegCtaMax entries of the gathered array; a chunk spans at most
// two segments (each is longer than a chunk), found by one binary search.
__global__ void __launch_bounds__(256) BigGatherKernel(const uint32_t* __restrict__ big_list, uint32_t nbig,
                                                       uint64_t E, const uint64_t* __restrict__ segbase,
                                                       const uint64_t* __restrict__ ebase,
                                                       const uint32_t* __restrict__ akey,
                                                       const uint32_t* __restrict__ aval, int kbits,
                                                       uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  __shared__ uint32_t s_bi;
  for (uint64_t c0 = uint64_t(blockIdx.x) * kSegCtaMax; c0 < E; c0 += uint64_t(gridDim.x) * kSegCtaMax) {
    if (threadIdx.x == 0) {
      uint32_t lo = 0, hi = nbig;  // last segment with ebase <= c0
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ebase[mid] <= c0) lo = mid;
        else hi = mid;
      }
      s_bi = lo;
    }
    __syncthreads();
    const uint32_t b0 = s_bi;
    const uint64_t next = b0 + 1 < nbig ? ebase[b0 + 1] : E;
    const uint64_t c1 = c0 + kSegCtaMax < E ? c0 + kSegCtaMax : E;
    for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
      const uint32_t bi = i < next ? b0 : b0 + 1;
      const uint64_t src = segbase[big_list[bi]] + (i - ebase[bi]);
      keys[i] = (uint64_t(bi) << kbits) | akey[src];
      vals[i] = aval[src];
    }
    __syncthreads();
  }
}
struct BigLenInput {
  const uint32_t* big_list;
  const uint64_t* segbase;
  __device__ uint64_t operator()(uint64_t i) const {
    const uint32_t r = big_list[i];
    return segbase[r + 1] - segbase[r];
  }
};

struct HeadInput {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};

// Global path, per run s of equal (segment, key) in the sorted entries:
// grun[g] = first run of big segment g.
__global__ void BigGroupKernel(uint32_t S, const uint32_t* __restrict__ seg_start, const uint64_t* __restrict__ keys,
                               int kbits, uint32_t* __restrict__ grun) {
  for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < S; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t g = keys[seg_start[s]] >> kbits;
    if (s == 0 || (keys[seg_start[s - 1]] >> kbits) != g) grun[g] = static_cast<uint32_t>(s);
  }
}

// Global path: each kept run's neighbour id and sum, stored at the run's
// index (a segment's kept runs are consecutive and first: the dropped key
// sorts last), folded here when at most 1024 long, else listed for
// BigLongKernel; the segment's unique count is set by its last kept run.
__global__ void BigRunKernel(uint32_t S, uint64_t E, const uint32_t* __restrict__ seg_start,
                             const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, int kbits,
                             uint32_t drop, const uint32_t* __restrict__ grun, const uint32_t* __restrict__ big_list,
                             const uint32_t* __restrict__ ids, uint32_t* __restrict__ bkey,
                             uint32_t* __restrict__ bval, uint32_t* __restrict__ ucount,
                             uint32_t* __restrict__ long_run, uint32_t* __restrict__ long_count) {
  const uint64_t low_mask = (uint64_t(1) << kbits) - 1;
  for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < S; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t a = seg_start[s];
    const uint64_t e = s + 1 < S ? seg_start[s + 1] : E;
    const uint64_t key = keys[a];
    const uint32_t low = static_cast<uint32_t>(key & low_mask);
    if (low >= drop) continue;
    const uint32_t g = static_cast<uint32_t>(key >> kbits);
    const uint32_t r = big_list[g];
    const uint32_t local = static_cast<uint32_t>(s) - grun[g];
    bkey[s] = ids[low];
    const uint64_t len = e - a;
    if (len <= 1024) {
      float acc = __uint_as_float(vals[a]);
      for (uint64_t j = 1; j < len; ++j) acc = __fadd_rn(acc, __uint_as_float(vals[a + j]));
      bval[s] = __float_as_uint(acc);
    } else {
      long_run[atomicAdd(long_count, 1u)] = static_cast<uint32_t>(s);
    }
    bool last = s + 1 == S;
    if (!last) {
      const uint64_t kn = keys[seg_start[s + 1]];
      last = (kn >> kbits) != g || static_cast<uint32_t>(kn & low_mask) >= drop;
    }
    if (last) ucount[r] = local + 1;
  }
}

// First level of the pbbs blocked fold of every run longer than 1024, over
// the whole grid: one thread per 1024-item block (bbase: exclusive prefix of
// the runs' block counts), written to the run's scratch slots.
struct LongBlocksInput {
  const uint32_t* long_run;
  const uint32_t* seg_start;
  uint32_t S;
  uint64_t E;
  __device__ uint64_t operator()(uint64_t li) const {
    const uint32_t s = long_run[li];
    const uint64_t len = (s + 1 < S ? seg_start[s + 1] : E) - seg_start[s];
    return (len + 1023) / 1024;
  }
};

__global__ void LongBlocksKernel(uint32_t cnt, uint64_t NB, const uint64_t* __restrict__ bbase,
                                 const uint32_t* __restrict__ long_run, const uint32_t* __restrict__ seg_start,
                                 uint32_t S, uint64_t E, const uint32_t* __restrict__ vals,
                                 float* __restrict__ scratch) {
  for (uint64_t b = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; b < NB; b += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t lo = 0, hi = cnt;  // the last run with bbase <= b
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (bbase[mid] <= b) lo = mid;
      else hi = mid;
    }
    const uint32_t s = long_run[lo];
    const uint64_t a = seg_start[s];
    const uint64_t len = (s + 1 < S ? seg_start[s + 1] : E) - a;
    const uint64_t blk = b - bbase[lo];
    const uint64_t s0 = blk * 1024;
    const uint64_t l = min(uint64_t(1024), len - s0);
    float r = __uint_as_float(vals[a + s0]);
    for (uint64_t j = 1; j < l; ++j) r = __fadd_rn(r, __uint_as_float(vals[a + s0 + j]));
    scratch[a / 256 + blk] = r;
  }
}

// One CTA per run longer than 1024: the pbbs blocked fold from the first
// level's partials (LongBlocksKernel) on, level by level, with partials in
// global scratch (two regions of ceil(len/1024) floats per run at the run's
// scratch offset).
constexpr int kLongThreads = 1024;
__global__ void __launch_bounds__(kLongThreads) BigLongKernel(const uint32_t* __restrict__ long_run,
                                                             const uint32_t* __restrict__ long_count,
                                                             const uint32_t* __restrict__ seg_start, uint32_t S,
                                                             uint64_t E, const uint32_t* __restrict__ vals,
                                                             float* __restrict__ scratch, uint32_t* __restrict__ bval) {
  const uint32_t cnt = *long_count;
  for (uint32_t li = blockIdx.x; li < cnt; li += gridDim.x) {
    const uint32_t s = long_run[li];
    const uint64_t a = seg_start[s];
    const uint64_t len = (s + 1 < S ? seg_start[s + 1] : E) - a;
    // Scratch: the run's items start at a and number len > 1024, so the
    // slots [a/256, a/256 + 2*ceil(len/1024)) lie below the next long run's
    // a'/256 (a' >= a + len) and no two runs overlap.
    float* p0 = scratch + (a / 256);
    uint64_t nb = (len + 1023) / 1024;
    float* p1 = p0 + nb;
    float* cur = p0;
    float* nxt = p1;
    while (nb > 1024) {
      const uint64_t nb2 = (nb + 1023) / 1024;
      for (uint64_t blk = threadIdx.x; blk < nb2; blk += kLongThreads) {
        const uint64_t s0 = blk * 1024;
        const uint64_t l = min(uint64_t(1024), nb - s0);
        float r = __ldcg(cur + s0);
        for (uint64_t j = 1; j < l; ++j) r = __fadd_rn(r, __ldcg(cur + s0 + j));
        nxt[blk] = r;
      }
      __syncthreads();
      float* t = cur;
      cur = nxt;
      nxt = t;
      nb = nb2;
    }
    if (threadIdx.x == 0) {
      float r = __ldcg(cur);
      for (uint64_t j = 1; j < nb; ++j) r = __fadd_rn(r, __ldcg(cur + j));
      bval[s] = __float_as_uint(r);
    }
    __syncthreads();
  }
}

__global__ void RowCountKernel(uint32_t R, const uint32_t* __restrict__ ids, const uint32_t* __restrict__ ucount,
                               uint32_t* __restrict__ row_count) {
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < R; r += uint64_t(gridDim.x) * blockDim.x)
    row_count[ids[r]] = ucount[r];
}

// The unique pairs of each segment (at its start) into the new CSR; one
// warp per cluster.
__global__ void __launch_bounds__(256) GatherRowsKernel(uint32_t R, const uint32_t* __restrict__ ids,
                                                        const uint32_t* __restrict__ ucount,
                                                        const uint64_t* __restrict__ segbase,
                                                        const uint64_t* __restrict__ off2,
                                                        const uint32_t* __restrict__ akey,
                                                        const uint32_t* __restrict__ aval,
                                                        uint32_t* __restrict__ nbr2, float* __restrict__ w2) {
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  for (uint64_t r = uint64_t(blockIdx.x) * 8 + warp; r < R; r += uint64_t(gridDim.x) * 8) {
    const uint32_t cnt = ucount[r];
    const uint64_t src = segbase[r];
    if (cnt == 0 || segbase[r + 1] - src > kSegCtaMax) continue;  // global-path rows: BigPlaceKernel
    const uint64_t dst = off2[ids[r]];
    for (uint32_t t = lane; t < cnt; t += 32) {
      nbr2[dst + t] = akey[src + t];
      w2[dst + t] = __uint_as_float(aval[src + t]);
    }
  }
}

// Global-path rows into the new CSR, one thread per kept run.
__global__ void BigPlaceKernel(uint32_t S, const uint32_t* __restrict__ seg_start, const uint64_t* __restrict__ keys,
                               int kbits, uint32_t drop, const uint32_t* __restrict__ grun,
                               const uint32_t* __restrict__ big_list, const uint32_t* __restrict__ ids,
                               const uint64_t* __restrict__ off2, const uint32_t* __restrict__ bkey,
                               const uint32_t* __restrict__ bval, uint32_t* __restrict__ nbr2,
                               float* __restrict__ w2) {
  const uint64_t low_mask = (uint64_t(1) << kbits) - 1;
  for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < S; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = keys[seg_start[s]];
    if (static_cast<uint32_t>(key & low_mask) >= drop) continue;
    const uint32_t g = static_cast<uint32_t>(key >> kbits);
    const uint64_t pos = off2[ids[big_list[g]]] + (static_cast<uint32_t>(s) - grun[g]);
    nbr2[pos] = bkey[s];
    w2[pos] = __uint_as_float(bval[s]);
  }
}

__global__ void NodeWeightKernel(uint32_t n, const uint32_t* __restrict__ C, const double* __restrict__ k,
                                 double* __restrict__ k2) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    atomicAdd(&k2[C[i]], k ? k[i] : 1.0);
}

struct CountInput {
  const uint32_t* c;
  uint32_t n;
  __device__ uint64_t operator()(uint64_t i) const { return i < n ? c[i] : 0ull; }
};

int BitsFor(uint64_t count) {
  int b = 1;
  while ((uint64_t(1) << b) < count) ++b;
  return b;
}

}  // namespace

// Contracts g by C (device uint32[n]); k = node weights (device, or null for
// 1).  The new graph carries its node weights in node_w.
Status CompressGraph(Context* ctx, const DevGraph& g, const uint32_t* C, const double* k,
                     std::unique_ptr<DevGraph>* out) {
  const uint32_t n = g.n;
  cudaStream_t st = ctx->stream;
  DBuf<uint32_t> tmp32;
  PCC_RETURN_IF_ERROR(tmp32.Alloc(ctx, 8));
  DBuf<uint32_t> part32;
  // n2 = 1 + max C
  uint32_t maxc = 0;
  if (n > 0) {
    PCC_RETURN_IF_ERROR(Reduce<uint32_t>(ctx, n, MaxOfU32{C}, OpMax{}, 0u, tmp32.p, part32));
    PCC_RETURN_IF_ERROR(tmp32.ToHost(&maxc, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx));
  }
  const uint32_t n2 = maxc + 1;

  // Dense order-preserving rank of the cluster ids in use.
  DBuf<uint32_t> pres, rank, ids;
  PCC_RETURN_IF_ERROR(pres.Alloc(ctx, n2));
  PCC_RETURN_IF_ERROR(pres.Zero());
  PCC_RETURN_IF_ERROR(rank.Alloc(ctx, n2));
  PCC_RETURN_IF_ERROR(ids.Alloc(ctx, n2));
  MarkPresentKernel<<<Blocks(n, 256, ctx->num_sms * 8), 256, 0, st>>>(n, C, pres.p); PCC_COUNT(1);
  DBuf<uint32_t> scan_tiles;
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, n2, PresInput{pres.p}, RankWriter{rank.p, ids.p}, scan_tiles,
                                          tmp32.p));
  uint32_t R = 0;  // clusters in use
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&R, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  pres.Release();
  // Keys: a rank (< R) or the dropped-copy mark above every rank, in kbits
  // bits (32 when the ranks need 31 or more).
  const int bits = BitsFor(R);
  const int kbits = bits >= 31 ? 32 : bits + 1;
  const uint32_t drop = bits >= 31 ? kNone : (1u << bits);

  auto res = std::make_unique<DevGraph>();
  res->n = n2;
  PCC_RETURN_IF_ERROR(res->off.Alloc(ctx, uint64_t(n2) + 1));
  DBuf<uint32_t> row_count;
  PCC_RETURN_IF_ERROR(row_count.Alloc(ctx, uint64_t(n2) + 1));
  PCC_RETURN_IF_ERROR(row_count.Zero());
  DBuf<uint32_t> akey, aval;
  DBuf<uint64_t> segbase;
  DBuf<uint32_t> ucount;
  // Global path, kept until its rows are placed: sorted keys, run starts,
  // first run per segment, and each kept run's neighbour id and sum.
  DBuf<uint64_t> bkeys;
  DBuf<uint32_t> seg_start, grun, bkey, bval, lists;
  uint32_t S = 0;
  int place_kbits = 0;
  if (g.m) {
    // Vertices in cluster order (stable: ascending id inside a cluster) and
    // where each row starts in the cluster-ordered entry array.
    DBuf<uint64_t> vkey;
    DBuf<uint32_t> vval;
    PCC_RETURN_IF_ERROR(vkey.Alloc(ctx, n));
    PCC_RETURN_IF_ERROR(vval.Alloc(ctx, n));
    VertexKeysKernel<<<Blocks(n, 256, ctx->num_sms * 8), 256, 0, st>>>(n, C, rank.p, vkey.p, vval.p);
    PCC_COUNT(1);
    {
      SortScratch sc;
      PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, vkey.p, vval.p, n, bits, sc));
    }
    DBuf<uint64_t> dstart, scan64;
    PCC_RETURN_IF_ERROR(dstart.Alloc(ctx, n));
    PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, n, SortedDegInput{g.off.p, vval.p}, RowStartWriter{vval.p, dstart.p},
                                            scan64, static_cast<uint64_t*>(nullptr)));
    PCC_RETURN_IF_ERROR(segbase.Alloc(ctx, uint64_t(R) + 1));
    SegBaseKernel<<<Blocks(n, 256, ctx->num_sms * 8), 256, 0, st>>>(n, vkey.p, vval.p, dstart.p, segbase.p, R, g.m);
    PCC_COUNT(1);
    vkey.Release();
    vval.Release();
    // Every row moved into its cluster's segment.
    PCC_RETURN_IF_ERROR(akey.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(aval.Alloc(ctx, g.m));
    LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                   MoveEntries{g.off.p, g.nbr.p, g.wp(), C, rank.p, dstart.p, drop, akey.p, aval.p});
    PCC_RETURN_IF_ERROR(LaunchCheck());
    dstart.Release();
    // Segment classes.
    DBuf<uint32_t> counts;
    DBuf<unsigned long long> big_e;
    PCC_RETURN_IF_ERROR(lists.Alloc(ctx, uint64_t(R) * 4));
    const uint32_t* wlist = lists.p;
    const uint32_t* mlist = lists.p + uint64_t(R);
    const uint32_t* clist = lists.p + 2 * uint64_t(R);
    const uint32_t* blist = lists.p + 3 * uint64_t(R);
    PCC_RETURN_IF_ERROR(counts.Alloc(ctx, 4));
    PCC_RETURN_IF_ERROR(counts.Zero());
    PCC_RETURN_IF_ERROR(big_e.Alloc(ctx, 1));
    PCC_RETURN_IF_ERROR(big_e.Zero());
    PCC_RETURN_IF_ERROR(ucount.Alloc(ctx, R));
    PCC_RETURN_IF_ERROR(ucount.Zero());
    ClassifyKernel<<<Blocks(R, 256, ctx->num_sms * 8), 256, 0, st>>>(R, segbase.p, lists.p, counts.p, big_e.p);
    PCC_COUNT(1);
    uint32_t hc[4];
    unsigned long long E = 0;
    PCC_RETURN_IF_ERROR(counts.ToHost(hc, 4));
    PCC_RETURN_IF_ERROR(big_e.ToHost(&E, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx));
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
      attr = cudaFuncSetAttribute(SegMidKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSegMidSmem));
      if (attr == cudaSuccess)
        attr = cudaFuncSetAttribute(SegCtaKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSegCtaSmem));
    });
    PCC_CUDA(attr);
    const int passes = (kbits + 7) / 8;
    if (hc[0]) {
      SegWarpKernel<<<Blocks(hc[0], 8, ctx->num_sms * 16), 256, 0, st>>>(wlist, counts.p, segbase.p, ids.p, drop,
                                                                         akey.p, aval.p, ucount.p);
      PCC_COUNT(1);
    }
    if (hc[1]) {
      SegMidKernel<<<Blocks(hc[1], kSegMidWarps, ctx->num_sms * 12), kSegMidWarps * 32, kSegMidSmem, st>>>(
          mlist, counts.p, segbase.p, ids.p, drop, passes, akey.p, aval.p, ucount.p);
      PCC_COUNT(1);
    }
    if (hc[2]) {
      SegCtaKernel<<<Blocks(hc[2], 1, ctx->num_sms * 3), kSegCtaThreads, kSegCtaSmem, st>>>(
          clist, counts.p, segbase.p, ids.p, drop, passes, akey.p, aval.p, ucount.p);
      PCC_COUNT(1);
    }
    if (hc[3]) {
      const uint32_t nbig = hc[3];
      place_kbits = kbits;
      DBuf<uint64_t> ebase;
      DBuf<uint32_t> bvals, long_run, long_count;
      PCC_RETURN_IF_ERROR(ebase.Alloc(ctx, nbig));
      PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, nbig, BigLenInput{blist, segbase.p}, StorePrefix<uint64_t>{ebase.p},
                                              scan64, static_cast<uint64_t*>(nullptr)));
      PCC_RETURN_IF_ERROR(bkeys.Alloc(ctx, E));
      PCC_RETURN_IF_ERROR(bvals.Alloc(ctx, E));
      BigGatherKernel<<<Blocks(E, kSegCtaMax, unsigned(ctx->num_sms) * 8), 256, 0, st>>>(
          blist, nbig, E, segbase.p, ebase.p, akey.p, aval.p, kbits, bkeys.p, bvals.p);
      PCC_COUNT(1);
      {
        SortScratch sc;
        PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, bkeys.p, bvals.p, E, kbits + BitsFor(nbig), sc));
      }
      PCC_RETURN_IF_ERROR(seg_start.Alloc(ctx, E));
      PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, E, HeadInput{bkeys.p}, StoreIndexIfSet{seg_start.p}, scan_tiles,
                                              tmp32.p));
      PCC_RETURN_IF_ERROR(tmp32.ToHost(&S, 1));
      PCC_RETURN_IF_ERROR(Sync(ctx));
      PCC_RETURN_IF_ERROR(grun.Alloc(ctx, nbig));
      PCC_RETURN_IF_ERROR(long_run.Alloc(ctx, S));
      PCC_RETURN_IF_ERROR(bkey.Alloc(ctx, S));
      PCC_RETURN_IF_ERROR(bval.Alloc(ctx, S));
      PCC_RETURN_IF_ERROR(long_count.Alloc(ctx, 1));
      PCC_RETURN_IF_ERROR(long_count.Zero());
      BigGroupKernel<<<Blocks(S, 256, ctx->num_sms * 8), 256, 0, st>>>(S, seg_start.p, bkeys.p, kbits, grun.p);
      PCC_COUNT(1);
      BigRunKernel<<<Blocks(S, 256, ctx->num_sms * 16), 256, 0, st>>>(
          S, E, seg_start.p, bkeys.p, bvals.p, kbits, drop, grun.p, blist, ids.p, bkey.p, bval.p, ucount.p,
          long_run.p, long_count.p);
      PCC_COUNT(1);
      uint32_t nlong = 0;
      PCC_RETURN_IF_ERROR(long_count.ToHost(&nlong, 1));
      PCC_RETURN_IF_ERROR(Sync(ctx));
      if (nlong) {
        DBuf<float> scratch;
        PCC_RETURN_IF_ERROR(scratch.Alloc(ctx, E / 256 + 64));
        DBuf<uint64_t> bbase, nbtot;
        PCC_RETURN_IF_ERROR(bbase.Alloc(ctx, nlong));
        PCC_RETURN_IF_ERROR(nbtot.Alloc(ctx, 1));
        PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, nlong, LongBlocksInput{long_run.p, seg_start.p, S, E},
                                                StorePrefix<uint64_t>{bbase.p}, scan64, nbtot.p));
        uint64_t NB = 0;
        PCC_RETURN_IF_ERROR(nbtot.ToHost(&NB, 1));
        PCC_RETURN_IF_ERROR(Sync(ctx));
        LongBlocksKernel<<<Blocks(NB, 256, unsigned(ctx->num_sms) * 16), 256, 0, st>>>(
            nlong, NB, bbase.p, long_run.p, seg_start.p, S, E, bvals.p, scratch.p);
        PCC_COUNT(1);
        BigLongKernel<<<unsigned(ctx->num_sms) * 2, kLongThreads, 0, st>>>(long_run.p, long_count.p, seg_start.p,
                                                                           S, E, bvals.p, scratch.p, bval.p);
        PCC_COUNT(1);
      }
    }
    PCC_RETURN_IF_ERROR(LaunchCheck());
    RowCountKernel<<<Blocks(R, 256, ctx->num_sms * 8), 256, 0, st>>>(R, ids.p, ucount.p, row_count.p);
    PCC_COUNT(1);
  }
  // Offsets over the sparse id space [0, n2].
  DBuf<uint64_t> scan64b, total;
  PCC_RETURN_IF_ERROR(total.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, uint64_t(n2) + 1, CountInput{row_count.p, n2},
                                          StorePrefix<uint64_t>{res->off.p}, scan64b, total.p));
  uint64_t m2 = 0;
  PCC_RETURN_IF_ERROR(total.ToHost(&m2, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  res->m = m2;
  PCC_RETURN_IF_ERROR(res->nbr.Alloc(ctx, m2 ? m2 : 1));
  PCC_RETURN_IF_ERROR(res->w.Alloc(ctx, m2 ? m2 : 1));
  if (m2) {
    GatherRowsKernel<<<Blocks(R, 8, ctx->num_sms * 16), 256, 0, st>>>(R, ids.p, ucount.p, segbase.p, res->off.p,
                                                                      akey.p, aval.p, res->nbr.p, res->w.p);
    PCC_COUNT(1);
    if (S) {
      BigPlaceKernel<<<Blocks(S, 256, ctx->num_sms * 16), 256, 0, st>>>(
          S, seg_start.p, bkeys.p, place_kbits, drop, grun.p, lists.p + 3 * uint64_t(R), ids.p, res->off.p, bkey.p,
          bval.p, res->nbr.p, res->w.p);
      PCC_COUNT(1);
    }
  }
  bkeys.Release();
  seg_start.Release();
  grun.Release();
  bkey.Release();
  bval.Release();
  lists.Release();
  akey.Release();
  aval.Release();
  // Node weights.
  PCC_RETURN_IF_ERROR(res->node_w.Alloc(ctx, n2));
  PCC_RETURN_IF_ERROR(res->node_w.Zero());
  NodeWeightKernel<<<Blocks(n, 256, ctx->num_sms * 8), 256, 0, st>>>(n, C, k, res->node_w.p); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(LaunchCheck());
  PCC_RETURN_IF_ERROR(ComputeGraphProperties(ctx, res.get()));
  *out = std::move(res);
  return Status::Ok();
}

}  // namespace pcc
