// scoring.cu -- ground-truth scoring of a clustering on the device.
//
// Restates CompareCommunities (clustering/cluster-in-memory_main.cc:172-225),
// which the reference CLI runs on the host after Cluster() when it is given
// --input_communities:
//   * the intersection of community j with cluster i counts the distinct
//     members of j whose label is cluster i (std::set_intersection of the
//     sorted community with the sorted cluster counts a repeated member
//     once, since the cluster holds it once; a member that is no vertex of
//     the graph meets no cluster but counts in the community's size);
//   * the best cluster of j is the first one, in cluster order (ascending
//     labels, as OutputIndicesById lists them), with the largest
//     intersection; with no intersection at all it is cluster 0;
//   * precision_j = best / |that cluster|, recall_j = best / |community j|
//     (0 for an empty community); each average is pbbs::reduce_add (serial
//     folds of 1024-element blocks, then the same reduce over the block
//     sums) divided by the number of communities;
//   * cluster sizes: count, minimum (UINT_E_MAX when there is no cluster),
//     maximum, and the mean, whose sequential FP64 sum of integer sizes is
//     exactly n.
// GB300 shape: (community, vertex) keys are radix-sorted and deduplicated;
// the distinct members' (community, label) keys are sorted again, so the
// lengths of equal-key runs are the intersections.  One 64-bit atomicMax
// per run keeps, for each community, the largest count and, among equal
// counts, the lowest label.
#include <cmath>

#include "graphops.cuh"

namespace pcc {

namespace {

constexpr uint32_t kLow32 = 0xFFFFFFFFu;

// Key (community, vertex) of every member entry and the vertex's label; the
// community comes from a binary search over the offsets.
__global__ void ScMemberKeysKernel(uint64_t total, uint32_t ncomm, uint32_t n, const uint64_t* __restrict__ off,
                                   const uint32_t* __restrict__ members, const uint32_t* __restrict__ labels,
                                   uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t lo = 0, hi = ncomm;  // off[lo] <= e < off[hi]
    while (hi - lo > 1) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (off[mid] <= e)
        lo = mid;
      else
        hi = mid;
    }
    const uint32_t v = members[e];
    keys[e] = (static_cast<uint64_t>(lo) << 32) | v;
    vals[e] = v < n ? labels[v] : kLow32;  // a vertex no cluster holds
  }
}

// First occurrence of each (community, vertex): the distinct members.
struct ScDistinctInput {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};
// Rewrites a distinct member as its (community, label) key.
struct ScLabelKeyWriter {
  const uint64_t* keys;
  const uint32_t* labels_of;
  uint64_t* out_keys;
  uint32_t* out_vals;
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t v) const {
    if (v) {
      out_keys[pre] = (keys[i] & ~uint64_t(kLow32)) | labels_of[i];
      out_vals[pre] = 0u;
    }
  }
};
struct ScRunHead {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};

__global__ void ScSetKernel(uint32_t* p, const uint32_t* value) { *p = *value; }

// Largest intersection of each community, lowest label on ties.
__global__ void ScRunBestKernel(const uint32_t* __restrict__ nruns_p, const uint32_t* __restrict__ run_start,
                                const uint64_t* __restrict__ keys, unsigned long long* __restrict__ best) {
  const uint32_t nruns = *nruns_p;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = keys[run_start[r]];
    const uint32_t count = run_start[r + 1] - run_start[r];
    const uint32_t label = static_cast<uint32_t>(key & kLow32);
    if (label == kLow32) continue;  // members that are not vertices of the graph
    atomicMax(&best[key >> 32], (static_cast<unsigned long long>(count) << 32) | (kLow32 - label));
  }
}

// Cluster sizes by label and the lowest label in use (cluster 0).
__global__ void ScSizesKernel(uint32_t n, const uint32_t* __restrict__ labels, uint32_t* __restrict__ size,
                              uint32_t* __restrict__ min_label) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
    atomicAdd(&size[labels[v]], 1u);
    atomicMin(min_label, labels[v]);
  }
}

struct ScStats {
  unsigned long long clusters;
  unsigned long long min_size;
  unsigned long long max_size;
};

__global__ void ScClusterStatsKernel(uint32_t n, const uint32_t* __restrict__ size, ScStats* st) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t s = size[i];
    if (s == 0) continue;
    atomicAdd(&st->clusters, 1ull);
    atomicMin(&st->min_size, static_cast<unsigned long long>(s));
    atomicMax(&st->max_size, static_cast<unsigned long long>(s));
  }
}

// precision_j and recall_j.
__global__ void ScScoreKernel(uint32_t ncomm, const uint64_t* __restrict__ off,
                              const unsigned long long* __restrict__ best, const uint32_t* __restrict__ size,
                              const uint32_t* __restrict__ min_label, uint32_t n, double* __restrict__ prec,
                              double* __restrict__ rec) {
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < ncomm;
       j += uint64_t(gridDim.x) * blockDim.x) {
    const unsigned long long b = best[j];
    const uint32_t count = static_cast<uint32_t>(b >> 32);
    const uint32_t label = count ? kLow32 - static_cast<uint32_t>(b & kLow32) : *min_label;
    const uint32_t csize = label < n ? size[label] : 0u;
    const uint64_t comm = off[j + 1] - off[j];
    prec[j] = csize ? __ddiv_rn(static_cast<double>(count), static_cast<double>(csize)) : 0.0;
    rec[j] = comm == 0 ? 0.0 : __ddiv_rn(static_cast<double>(count), static_cast<double>(comm));
  }
}

// One level of pbbs::reduce_add: a serial fold per 1024-element block.
__global__ void ScBlockFoldKernel(uint64_t len, const double* __restrict__ a, double* __restrict__ sums) {
  const uint64_t nb = (len + 1023) / 1024;
  for (uint64_t b = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; b < nb; b += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t s = b * 1024, e = s + 1024 < len ? s + 1024 : len;
    double r = a[s];
    for (uint64_t j = s + 1; j < e; ++j) r = Dadd(r, a[j]);
    sums[b] = r;
  }
}

// pbbs::reduce_add of a device array (len >= 1) into *out (device).
Status BlockedSum(Context* ctx, const double* a, uint64_t len, double* out) {
  DBuf<double> cur, nxt;
  const double* src = a;
  while (len > 1024) {
    const uint64_t nb = (len + 1023) / 1024;
    PCC_RETURN_IF_ERROR(nxt.Alloc(ctx, nb));
    ScBlockFoldKernel<<<Blocks(nb, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(len, src, nxt.p); PCC_COUNT(1);
    std::swap(cur, nxt);
    src = cur.p;
    len = nb;
  }
  ScBlockFoldKernel<<<1, 32, 0, ctx->stream>>>(len, src, out); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(LaunchCheck());
  return Sync(ctx);  // cur / nxt go out of scope
}

Status CompareCommunities(Context* ctx, uint32_t n, const uint32_t* labels, uint32_t ncomm, const uint64_t* offsets,
                          const uint32_t* members, double* precision, double* recall, pcc_community_scores* out) {
  cudaStream_t st = ctx->stream;
  const uint64_t total = ncomm ? offsets[ncomm] : 0;
  const uint64_t nn = n ? n : 1;
  DBuf<uint32_t> dlab, size, min_label;
  PCC_RETURN_IF_ERROR(dlab.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(dlab.FromHost(labels, n));
  PCC_RETURN_IF_ERROR(size.Alloc(ctx, nn));
  PCC_RETURN_IF_ERROR(size.Zero());
  PCC_RETURN_IF_ERROR(min_label.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(min_label.Fill(0xFF));
  DBuf<ScStats> stats;
  PCC_RETURN_IF_ERROR(stats.Alloc(ctx, 1));
  const ScStats init{0ull, 0xFFFFFFFFull, 0ull};  // UINT_E_MAX
  PCC_RETURN_IF_ERROR(stats.FromHost(&init, 1));
  const unsigned grid_n = Blocks(nn, 256, ctx->num_sms * 8);
  if (n) {
    ScSizesKernel<<<grid_n, 256, 0, st>>>(n, dlab.p, size.p, min_label.p); PCC_COUNT(1);
    ScClusterStatsKernel<<<grid_n, 256, 0, st>>>(n, size.p, stats.p); PCC_COUNT(1);
  }

  // Per community: best intersection, precision, recall.
  const uint64_t nc = ncomm ? ncomm : 1;
  DBuf<uint64_t> doff;
  DBuf<unsigned long long> best;
  DBuf<double> prec, rec;
  PCC_RETURN_IF_ERROR(doff.Alloc(ctx, uint64_t(ncomm) + 1));
  PCC_RETURN_IF_ERROR(doff.FromHost(offsets, uint64_t(ncomm) + 1));
  PCC_RETURN_IF_ERROR(best.Alloc(ctx, nc));
  PCC_RETURN_IF_ERROR(best.Zero());
  PCC_RETURN_IF_ERROR(prec.Alloc(ctx, nc));
  PCC_RETURN_IF_ERROR(rec.Alloc(ctx, nc));
  if (total) {
    DBuf<uint32_t> dmem, vals, vals2, tmp32, run_start, scan_tiles;
    DBuf<uint64_t> keys, keys2;
    PCC_RETURN_IF_ERROR(dmem.Alloc(ctx, total));
    PCC_RETURN_IF_ERROR(dmem.FromHost(members, total));
    PCC_RETURN_IF_ERROR(keys.Alloc(ctx, total));
    PCC_RETURN_IF_ERROR(vals.Alloc(ctx, total));
    ScMemberKeysKernel<<<Blocks(total, 256, ctx->num_sms * 8), 256, 0, st>>>(total, ncomm, n, doff.p, dmem.p,
                                                                             dlab.p, keys.p, vals.p); PCC_COUNT(1);
    uint32_t bits_c = 1;
    while ((uint64_t(1) << bits_c) < ncomm) ++bits_c;
    const int bits = int(32 + bits_c);
    SortScratch sc;
    PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys.p, vals.p, total, bits, sc));
    PCC_RETURN_IF_ERROR(tmp32.Alloc(ctx, 2));
    PCC_RETURN_IF_ERROR(keys2.Alloc(ctx, total));
    PCC_RETURN_IF_ERROR(vals2.Alloc(ctx, total));
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, total, ScDistinctInput{keys.p},
                                            ScLabelKeyWriter{keys.p, vals.p, keys2.p, vals2.p}, scan_tiles, tmp32.p));
    uint32_t distinct = 0;
    PCC_RETURN_IF_ERROR(tmp32.ToHost(&distinct, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx));
    PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys2.p, vals2.p, distinct, bits, sc));
    PCC_RETURN_IF_ERROR(run_start.Alloc(ctx, uint64_t(distinct) + 1));
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, distinct, ScRunHead{keys2.p}, StoreIndexIfSet{run_start.p},
                                            scan_tiles, tmp32.p));
    uint32_t nruns = 0;
    PCC_RETURN_IF_ERROR(tmp32.ToHost(&nruns, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx));
    PCC_RETURN_IF_ERROR(tmp32.FromHost(&distinct, 1));
    ScSetKernel<<<1, 1, 0, st>>>(run_start.p + nruns, tmp32.p); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(tmp32.FromHost(&nruns, 1));
    ScRunBestKernel<<<Blocks(nruns, 256, ctx->num_sms * 8), 256, 0, st>>>(tmp32.p, run_start.p, keys2.p, best.p);
    PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(LaunchCheck());
    PCC_RETURN_IF_ERROR(Sync(ctx));  // scratch goes out of scope
  }
  double sums[2] = {0.0, 0.0};
  if (ncomm) {
    ScScoreKernel<<<Blocks(ncomm, 256, ctx->num_sms * 8), 256, 0, st>>>(ncomm, doff.p, best.p, size.p, min_label.p,
                                                                        n, prec.p, rec.p); PCC_COUNT(1);
    DBuf<double> dsum;
    PCC_RETURN_IF_ERROR(dsum.Alloc(ctx, 2));
    PCC_RETURN_IF_ERROR(BlockedSum(ctx, prec.p, ncomm, dsum.p));
    PCC_RETURN_IF_ERROR(BlockedSum(ctx, rec.p, ncomm, dsum.p + 1));
    PCC_RETURN_IF_ERROR(dsum.ToHost(sums, 2));
    if (precision) PCC_RETURN_IF_ERROR(prec.ToHost(precision, ncomm));
    if (recall) PCC_RETURN_IF_ERROR(rec.ToHost(recall, ncomm));
  }
  ScStats hs;
  PCC_RETURN_IF_ERROR(stats.ToHost(&hs, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  out->avg_precision = sums[0] / static_cast<double>(ncomm);
  out->avg_recall = sums[1] / static_cast<double>(ncomm);
  out->num_clusters = hs.clusters;
  out->min_size = hs.min_size;
  out->max_size = hs.max_size;
  double size_sum = 0;  // the reference's sequential sum of the sizes: exactly n
  size_sum += static_cast<double>(n);
  out->avg_size = size_sum / static_cast<double>(hs.clusters);
  return Status::Ok();
}

pcc_status Done(pcc_context* ctx, const Status& st) {
  if (ctx) ctx->c.last_error = st.ok() ? std::string() : st.msg;
  return st.code;
}

}  // namespace
}  // namespace pcc

using pcc::Status;
using pcc::MakeError;

extern "C" {

pcc_status pcc_compare_communities(pcc_context* pctx, uint32_t n, const uint32_t* labels, uint32_t num_communities,
                                   const uint64_t* offsets, const uint32_t* members, double* precision,
                                   double* recall, pcc_community_scores* out) {
  Status st;
  if (!pctx || !out || !offsets || (n && !labels)) st = MakeError(PCC_INVALID_ARGUMENT, "null argument");
  if (st.ok() && offsets[0] != 0) st = MakeError(PCC_INVALID_ARGUMENT, "offsets[0] must be 0");
  for (uint32_t j = 0; st.ok() && j < num_communities; ++j)
    if (offsets[j + 1] < offsets[j]) st = MakeError(PCC_INVALID_ARGUMENT, "offsets must not decrease");
  const uint64_t total = st.ok() && num_communities ? offsets[num_communities] : 0;
  if (st.ok() && total && !members) st = MakeError(PCC_INVALID_ARGUMENT, "null members");
  if (st.ok() && total > 0xFFFFFFFFull) st = MakeError(PCC_INVALID_ARGUMENT, "more than 2^32 - 1 members");
  for (uint32_t v = 0; st.ok() && v < n; ++v)
    if (labels[v] >= n) st = MakeError(PCC_INVALID_ARGUMENT, "label " + std::to_string(labels[v]) + " is not below n");
  if (st.ok())
    st = pcc::CompareCommunities(&pctx->c, n, labels, num_communities, offsets, members, precision, recall, out);
  return pcc::Done(pctx, st);
}

}  // extern "C"
