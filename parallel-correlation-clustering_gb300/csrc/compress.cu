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
// GB300 shape: cluster ids are ranked densely (order-preserving) so the sort
// key (rank C(u), rank C(v)) needs only 2*ceil(log2 #clusters) bits; the
// stable LSD radix sort of primitives.cuh does the sort.
#include "graphops.cuh"

namespace pcc {

namespace {

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

struct KeyBuilder {
  const uint32_t* nbr;
  const uint32_t* C;
  const uint32_t* rank;
  uint32_t bits;
  uint8_t* keep;
  uint64_t* key;
  __device__ void operator()(uint32_t u, uint64_t j, uint64_t) const {
    const uint32_t v = nbr[j];
    const uint32_t cu = C[u], cv = C[v];
    const bool k = v <= u || cu != cv;
    keep[j] = k;
    if (k) key[j] = (static_cast<uint64_t>(rank[cu]) << bits) | rank[cv];
  }
};

struct KeepInput {
  const uint8_t* keep;
  __device__ uint32_t operator()(uint64_t i) const { return keep[i]; }
};
struct KeepWriter {
  const uint64_t* key_full;
  const float* w;
  uint64_t* keys;
  uint32_t* vals;
  __device__ void operator()(uint64_t j, uint32_t pre, uint32_t v) const {
    if (v) {
      keys[pre] = key_full[j];
      vals[pre] = __float_as_uint(w ? w[j] : 1.0f);
    }
  }
};

struct HeadInput {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};

__global__ void SetU32Kernel(uint32_t* p, const uint32_t* value) { *p = *value; }

// pbbs serial fold of x[0..len) (len >= 1) in FP32.
__device__ __forceinline__ float SerialFold(const uint32_t* x, uint32_t len) {
  float r = __uint_as_float(x[0]);
  for (uint32_t j = 1; j < len; ++j) r = __fadd_rn(r, __uint_as_float(x[j]));
  return r;
}

// Short segments (<= 1024 items): one thread each.  Long segments are
// listed for the CTA kernel.
__global__ void SegReduceShortKernel(uint32_t m2, const uint32_t* __restrict__ seg_start,
                                     const uint32_t* __restrict__ vals, const uint64_t* __restrict__ keys,
                                     uint32_t bits, const uint32_t* __restrict__ ids, uint32_t* __restrict__ nbr2,
                                     float* __restrict__ w2, uint32_t* __restrict__ row_count,
                                     uint32_t* __restrict__ long_list, uint32_t* __restrict__ long_count) {
  const uint64_t mask = (uint64_t(1) << bits) - 1;
  for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < m2; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t a = seg_start[s], e = seg_start[s + 1];
    const uint64_t key = keys[a];
    nbr2[s] = ids[key & mask];
    atomicAdd(&row_count[ids[key >> bits]], 1u);
    const uint32_t len = e - a;
    if (len <= 1024) {
      w2[s] = SerialFold(vals + a, len);
    } else {
      long_list[atomicAdd(long_count, 1u)] = static_cast<uint32_t>(s);
    }
  }
}

// One CTA per long segment: the pbbs blocked fold, level by level, with
// partials in global scratch (two regions of ceil(len/1024) floats per
// segment at the segment's scratch offset).
constexpr int kLongThreads = 1024;
__global__ void __launch_bounds__(kLongThreads) SegReduceLongKernel(const uint32_t* __restrict__ long_list,
                                                                   const uint32_t* __restrict__ long_count,
                                                                   const uint32_t* __restrict__ seg_start,
                                                                   const uint32_t* __restrict__ vals,
                                                                   float* __restrict__ scratch, float* __restrict__ w2) {
  const uint32_t cnt = *long_count;
  for (uint32_t li = blockIdx.x; li < cnt; li += gridDim.x) {
    const uint32_t s = long_list[li];
    const uint32_t a = seg_start[s], e = seg_start[s + 1];
    const uint32_t len = e - a;
    // Scratch: the segment's items start at a and number len > 1024, so the
    // slots [a/256, a/256 + 2*ceil(len/1024)) lie below the next segment's
    // a'/256 (a' >= a + len) and no two segments overlap.
    float* p0 = scratch + (a / 256);
    uint32_t nb = (len + 1023) / 1024;
    float* p1 = p0 + nb;
    for (uint32_t b = threadIdx.x; b < nb; b += kLongThreads) {
      const uint32_t s0 = b * 1024;
      const uint32_t l = min(1024u, len - s0);
      p0[b] = SerialFold(vals + a + s0, l);
    }
    __syncthreads();
    float* cur = p0;
    float* nxt = p1;
    while (nb > 1024) {
      const uint32_t nb2 = (nb + 1023) / 1024;
      for (uint32_t b = threadIdx.x; b < nb2; b += kLongThreads) {
        const uint32_t s0 = b * 1024;
        const uint32_t l = min(1024u, nb - s0);
        float r = __ldcg(cur + s0);
        for (uint32_t j = 1; j < l; ++j) r = __fadd_rn(r, __ldcg(cur + s0 + j));
        nxt[b] = r;
      }
      __syncthreads();
      float* t = cur;
      cur = nxt;
      nxt = t;
      nb = nb2;
    }
    if (threadIdx.x == 0) {
      float r = __ldcg(cur);
      for (uint32_t j = 1; j < nb; ++j) r = __fadd_rn(r, __ldcg(cur + j));
      w2[s] = r;
    }
    __syncthreads();
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
  uint32_t nclusters = 0;
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&nclusters, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  uint32_t bits = 1;
  while ((uint64_t(1) << bits) < nclusters) ++bits;

  // Kept entries with their keys, in CSR order.
  DBuf<uint8_t> keep;
  DBuf<uint64_t> key_full;
  PCC_RETURN_IF_ERROR(keep.Alloc(ctx, g.m ? g.m : 1));
  PCC_RETURN_IF_ERROR(key_full.Alloc(ctx, g.m ? g.m : 1));
  if (g.m) {
    LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                   KeyBuilder{g.nbr.p, C, rank.p, bits, keep.p, key_full.p});
    PCC_RETURN_IF_ERROR(LaunchCheck());
  }
  DBuf<uint64_t> keys;
  DBuf<uint32_t> vals;
  PCC_RETURN_IF_ERROR(keys.Alloc(ctx, g.m ? g.m : 1));
  PCC_RETURN_IF_ERROR(vals.Alloc(ctx, g.m ? g.m : 1));
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, g.m, KeepInput{keep.p},
                                          KeepWriter{key_full.p, g.wp(), keys.p, vals.p}, scan_tiles, tmp32.p));
  uint32_t M = 0;
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&M, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  keep.Release();
  key_full.Release();

  {
    SortScratch sc;
    PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys.p, vals.p, M, int(2 * bits), sc));
  }

  // Segments of equal (C(u), C(v)).
  DBuf<uint32_t> seg_start;
  PCC_RETURN_IF_ERROR(seg_start.Alloc(ctx, uint64_t(M) + 1));
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, M, HeadInput{keys.p}, StoreIndexIfSet{seg_start.p}, scan_tiles,
                                          tmp32.p));
  uint32_t m2 = 0;
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&m2, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  // seg_start[m2] = M
  PCC_RETURN_IF_ERROR(tmp32.FromHost(&M, 1));
  SetU32Kernel<<<1, 1, 0, st>>>(seg_start.p + m2, tmp32.p); PCC_COUNT(1);

  auto res = std::make_unique<DevGraph>();
  res->n = n2;
  res->m = m2;
  PCC_RETURN_IF_ERROR(res->off.Alloc(ctx, uint64_t(n2) + 1));
  PCC_RETURN_IF_ERROR(res->nbr.Alloc(ctx, m2 ? m2 : 1));
  PCC_RETURN_IF_ERROR(res->w.Alloc(ctx, m2 ? m2 : 1));
  DBuf<uint32_t> row_count, long_list;
  PCC_RETURN_IF_ERROR(row_count.Alloc(ctx, uint64_t(n2) + 1));
  PCC_RETURN_IF_ERROR(row_count.Zero());
  PCC_RETURN_IF_ERROR(long_list.Alloc(ctx, m2 ? m2 : 1));
  DBuf<uint32_t> long_count;
  PCC_RETURN_IF_ERROR(long_count.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(long_count.Zero());
  if (m2) {
    SegReduceShortKernel<<<Blocks(m2, 256, ctx->num_sms * 16), 256, 0, st>>>(
        m2, seg_start.p, vals.p, keys.p, bits, ids.p, res->nbr.p, res->w.p, row_count.p, long_list.p,
        long_count.p); PCC_COUNT(1);
    DBuf<float> scratch;
    PCC_RETURN_IF_ERROR(scratch.Alloc(ctx, uint64_t(M) / 256 + 64));
    SegReduceLongKernel<<<unsigned(ctx->num_sms) * 2, kLongThreads, 0, st>>>(long_list.p, long_count.p,
                                                                             seg_start.p, vals.p, scratch.p,
                                                                             res->w.p); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(LaunchCheck());
  }
  // Offsets over the sparse id space [0, n2].
  DBuf<uint64_t> scan64;
  PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, uint64_t(n2) + 1, CountInput{row_count.p, n2},
                                          StorePrefix<uint64_t>{res->off.p}, scan64,
                                          static_cast<uint64_t*>(nullptr)));
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
