// batch.cu -- batched best moves of all vertices with degree <= 1000 (INT
// mode, synchronous rounds).
//
// Restates the <= 1000-degree branch of ClusteringHelper::EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:456-512) plus the sync
// decision (parallel-correlation-clusterer.cc:139-157).  In INT mode every
// per-cluster sum is an exact integer, so the summation order is free and
// the vertices of a batch can be aggregated together:
//   * a static plan packs the degree-binned vertex list into batches of at
//     most kBatchEdges entries and kBatchVerts vertices;
//   * one CTA per batch: every thread takes entries of the batch (binary
//     search over the batch's degree prefix), gathers C(u) and adds
//     (w - offset) into a shared-memory table keyed by (vertex, cluster);
//   * per-vertex work that needs FP64 (change, the exact values of the
//     candidates that survive the FP32 pre-filter, the decision) runs one
//     vertex or one candidate per lane, so an FP64 warp instruction serves
//     up to 32 vertices -- GB300's FP64 pipe is ~1/64 of FP32.
#include <algorithm>
#include <vector>

#include "batch.cuh"
#include "moves.cuh"

namespace pcc {
namespace {

constexpr int kBT = 512;
constexpr uint32_t kBSlots = 2 * kBatchEdges;
constexpr unsigned long long kEmpty64 = ~0ull;

struct BatchShared {
  unsigned long long key[kBSlots];  // (local vertex << 32) | cluster, kEmpty64
  long long val[kBSlots];
  uint16_t used[kBatchEdges];
  uint16_t cand[kBatchEdges];       // contenders (index into used)
  double cval[kBatchEdges];         // contender exact values
  uint32_t vtx[kBatchVerts];        // vertex id, kNone when not in the frontier
  uint32_t epre[kBatchVerts + 1];   // exclusive prefix of frontier degrees
  uint64_t vbeg[kBatchVerts];
  long long smax[kBatchVerts];
  uint32_t ubound[kBatchVerts];
  unsigned long long best[kBatchVerts];
  uint32_t best_id[kBatchVerts];
  double change[kBatchVerts];
  uint32_t nused, ncand, nv, E;
};

__device__ __forceinline__ uint32_t Hash64(unsigned long long key, uint32_t mask) {
  const uint32_t lo = static_cast<uint32_t>(key), hi = static_cast<uint32_t>(key >> 32);
  const uint32_t x = lo * 0x9E3779B1u ^ (hi * 0x85EBCA77u + 0x27D4EB2Fu);
  return ((x * 0x9E3779B1u) >> (__clz(mask) & 31u)) & mask;
}

__device__ __forceinline__ uint32_t FindOrInsert64(unsigned long long* keys, unsigned long long key, bool* ins) {
  const uint32_t mask = kBSlots - 1;
  uint32_t h = Hash64(key, mask);
  *ins = false;
  for (uint32_t p = 0; p < kBSlots; ++p) {
    const unsigned long long k = keys[h];
    if (k == key) return h;
    if (k == kEmpty64) {
      const unsigned long long old = atomicCAS(&keys[h], kEmpty64, key);
      if (old == kEmpty64) {
        *ins = true;
        return h;
      }
      if (old == key) return h;
    }
    h = (h + 1) & mask;
  }
  return kNone;
}

__device__ __forceinline__ uint32_t Find64(const unsigned long long* keys, unsigned long long key) {
  const uint32_t mask = kBSlots - 1;
  uint32_t h = Hash64(key, mask);
  for (uint32_t p = 0; p < kBSlots; ++p) {
    const unsigned long long k = keys[h];
    if (k == key) return h;
    if (k == kEmpty64) return kNone;
    h = (h + 1) & mask;
  }
  return kNone;
}

__device__ __forceinline__ uint32_t OrderF32(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float UnorderF32(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ unsigned long long OrderF64(double d) {
  if (d == 0) d = 0.0;
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double UnorderF64(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double(static_cast<long long>(b));
}

__global__ void __launch_bounds__(kBT) BatchBestMoveKernel(BMArgs a, const uint32_t* __restrict__ list,
                                                          const uint32_t* __restrict__ bstart, uint32_t nbatches) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BatchShared& sh = *reinterpret_cast<BatchShared*>(smem_raw);
  const unsigned tid = threadIdx.x, lane = LaneId();
  for (uint32_t i = tid; i < kBSlots; i += kBT) {
    sh.key[i] = kEmpty64;
    sh.val[i] = 0;
  }
  if (tid == 0) sh.nused = 0;
  __syncthreads();
  for (uint32_t bi = blockIdx.x; bi < nbatches; bi += gridDim.x) {
    const uint32_t s0 = bstart[bi], s1 = bstart[bi + 1];
    const uint32_t nvb = s1 - s0;  // <= kBatchVerts
    // 1. Vertices of the batch in the frontier and their row prefix.
    uint32_t d = 0;
    if (tid < nvb) {
      const uint32_t v = list[s0 + tid];
      const bool in = InFront(a, v);
      const uint64_t b = a.off[v];
      d = in ? static_cast<uint32_t>(a.off[v + 1] - b) : 0u;
      sh.vtx[tid] = in ? v : kNone;
      sh.vbeg[tid] = b;
      sh.smax[tid] = LLONG_MIN;
      sh.ubound[tid] = 0;
      sh.best[tid] = 0;
      sh.best_id[tid] = kNone;
    }
    // Block exclusive scan of d over the first kBatchVerts threads.
    {
      __shared__ uint32_t wsum[kBT / 32];
      const uint32_t inc = WarpInclusiveScan<uint32_t>(d);
      if (lane == 31) wsum[tid >> 5] = inc;
      __syncthreads();
      if (tid < 32) {
        const uint32_t x = tid < kBT / 32 ? wsum[tid] : 0u;
        const uint32_t xi = WarpInclusiveScan<uint32_t>(x);
        if (tid < kBT / 32) wsum[tid] = xi - x;
      }
      __syncthreads();
      const uint32_t ex = inc - d + wsum[tid >> 5];
      if (tid < nvb) sh.epre[tid] = ex;
      if (tid == nvb) {
        sh.epre[nvb] = ex;
        sh.E = ex;
      }
    }
    __syncthreads();
    const uint32_t E = sh.E;
    bool any_front = false;
    if (tid < nvb) any_front = sh.vtx[tid] != kNone;
    if (!__syncthreads_or(any_front)) continue;
    // 2. Aggregate the entries into the (vertex, cluster) table.
    const uint32_t rounds = (E + kBT - 1) / kBT;
    for (uint32_t r = 0; r < rounds; ++r) {
      const uint32_t e = r * kBT + tid;
      const bool valid = e < E;
      uint32_t j = 0, v = 0, u = 0;
      float wt = 0.f;
      if (valid) {
        int lo = 0, hi = int(nvb) - 1;  // last j with epre[j] <= e
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (sh.epre[mid] <= e) lo = mid; else hi = mid - 1;
        }
        j = uint32_t(lo);
        v = sh.vtx[j];
        const uint64_t p = sh.vbeg[j] + (e - sh.epre[j]);
        u = a.nbr[p];
        wt = a.w ? a.w[p] : 1.0f;
      }
      const bool cand = valid && u != v;
      const uint32_t cu = cand ? __ldg(a.C + u) : kNone;
      const unsigned long long key = cand ? ((static_cast<unsigned long long>(j) << 32) | cu) : (kEmpty64 - lane);
      const unsigned peers = __match_any_sync(kFull, key);
      const bool leader = cand && int(lane) == __ffs(peers) - 1;
      const int xi = cand ? (static_cast<int>(wt) - a.ioffset) : 0;
      const int S = __reduce_add_sync(peers, xi);
      uint32_t slot = kNone;
      bool ins = false;
      if (leader) {
        slot = FindOrInsert64(sh.key, key, &ins);
        if (slot == kNone) {
          atomicExch(&a.ctr->error, kErrHashFull);
        } else {
          atomicAdd(reinterpret_cast<unsigned long long*>(&sh.val[slot]),
                    static_cast<unsigned long long>(static_cast<long long>(S)));
        }
      }
      // Used-list append, one shared atomic per warp.
      const unsigned im = __ballot_sync(kFull, ins);
      if (im) {
        uint32_t base = 0;
        const int ld = __ffs(im) - 1;
        if (int(lane) == ld) base = atomicAdd(&sh.nused, uint32_t(__popc(im)));
        base = __shfl_sync(kFull, base, ld);
        if (ins) sh.used[base + __popc(im & LaneMaskLt())] = static_cast<uint16_t>(slot);
      }
    }
    __syncthreads();
    const uint32_t nused = sh.nused;
    // 3. Per vertex: T = S of its own cluster, change (one vertex per lane).
    if (tid < nvb && sh.vtx[tid] != kNone) {
      const VertexCtx x = LoadVertex<false>(a, sh.vtx[tid]);
      const uint32_t slot = Find64(sh.key, (static_cast<unsigned long long>(tid) << 32) | x.c);
      const double T = slot != kNone ? static_cast<double>(sh.val[slot]) : 0.0;
      sh.change[tid] = ChangeOf(a, x, T);
    }
    // 4. Max S per vertex (the pre-filter's shift).
    for (uint32_t i = tid; i < nused; i += kBT) {
      const uint32_t slot = sh.used[i];
      atomicMax(&sh.smax[sh.key[slot] >> 32], sh.val[slot]);
    }
    __syncthreads();
    // 5. Filter bound U per vertex.
    for (uint32_t i = tid; i < nused; i += kBT) {
      const uint32_t slot = sh.used[i];
      const unsigned long long key = sh.key[slot];
      const uint32_t j = static_cast<uint32_t>(key >> 32);
      const long long Si = sh.val[slot];
      const float R = __fmul_rn(a.res32, __fmul_rn(static_cast<float>(a.k[sh.vtx[j]]),
                                                   a.Kf[static_cast<uint32_t>(key)]));
      const float Y = __fsub_rn(static_cast<float>(Si - sh.smax[j]), R);
      const float e = FilterBound(R, Y, static_cast<float>(Si), static_cast<float>(sh.change[j]));
      atomicMax(&sh.ubound[j], OrderF32(__fsub_rn(Y, e)));
    }
    if (tid == 0) sh.ncand = 0;
    __syncthreads();
    // 6. Contenders (compacted, one shared atomic per warp).
    const uint32_t nused32 = (nused + 31) & ~31u;
    for (uint32_t i = tid; i < nused32; i += kBT) {
      bool is_c = false;
      if (i < nused) {
        const uint32_t slot = sh.used[i];
        const unsigned long long key = sh.key[slot];
        const uint32_t j = static_cast<uint32_t>(key >> 32);
        const long long Si = sh.val[slot];
        const float R = __fmul_rn(a.res32, __fmul_rn(static_cast<float>(a.k[sh.vtx[j]]),
                                                     a.Kf[static_cast<uint32_t>(key)]));
        const float Y = __fsub_rn(static_cast<float>(Si - sh.smax[j]), R);
        const float e = FilterBound(R, Y, static_cast<float>(Si), static_cast<float>(sh.change[j]));
        is_c = __fadd_rn(Y, e) >= UnorderF32(sh.ubound[j]);
      }
      const unsigned cm = __ballot_sync(kFull, is_c);
      if (cm) {
        uint32_t base = 0;
        const int ld = __ffs(cm) - 1;
        if (int(lane) == ld) base = atomicAdd(&sh.ncand, uint32_t(__popc(cm)));
        base = __shfl_sync(kFull, base, ld);
        if (is_c) sh.cand[base + __popc(cm & LaneMaskLt())] = static_cast<uint16_t>(i);
      }
    }
    __syncthreads();
    const uint32_t ncand = sh.ncand;
    // 7. Exact FP64 values of the contenders (one per lane).
    for (uint32_t c = tid; c < ncand; c += kBT) {
      const uint32_t slot = sh.used[sh.cand[c]];
      const unsigned long long key = sh.key[slot];
      const uint32_t j = static_cast<uint32_t>(key >> 32);
      const double val = ValOf(a, a.k[sh.vtx[j]], sh.change[j], static_cast<double>(sh.val[slot]),
                               __ldg(a.K + static_cast<uint32_t>(key)));
      sh.cval[c] = val;
      atomicMax(&sh.best[j], OrderF64(val));
    }
    __syncthreads();
    // 8. Lowest cluster id among each vertex's best.
    for (uint32_t c = tid; c < ncand; c += kBT) {
      const uint32_t slot = sh.used[sh.cand[c]];
      const unsigned long long key = sh.key[slot];
      const uint32_t j = static_cast<uint32_t>(key >> 32);
      if (OrderF64(sh.cval[c]) == sh.best[j]) atomicMin(&sh.best_id[j], static_cast<uint32_t>(key));
    }
    __syncthreads();
    // 9. Decisions (one vertex per lane) and table cleanup.
    bool append = false;
    uint32_t mv = 0;
    if (tid < nvb && sh.vtx[tid] != kNone) {
      const VertexCtx x = LoadVertex<false>(a, sh.vtx[tid]);
      const unsigned long long bk = sh.best[tid];
      const double best = bk ? UnorderF64(bk) : -CUDART_INF;
      const uint32_t bid = bk ? sh.best_id[tid] : kNone;
      append = Decide<false>(a, x, best, bid, sh.change[tid]);
      mv = x.v;
    }
    if (tid < kBatchVerts) {  // warps 0 .. kBatchVerts/32-1, converged
      const uint32_t pos = WarpAppendFull(&a.ctr->movers, append);
      if (append) a.movers[pos] = mv;
    }
    for (uint32_t i = tid; i < nused; i += kBT) {
      const uint32_t slot = sh.used[i];
      sh.key[slot] = kEmpty64;
      sh.val[slot] = 0;
    }
    __syncthreads();
    if (tid == 0) sh.nused = 0;
    __syncthreads();
  }
}

__global__ void ListDegreesKernel(const uint32_t* list, uint32_t count, const uint64_t* off, uint32_t* deg) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    deg[i] = static_cast<uint32_t>(off[list[i] + 1] - off[list[i]]);
}

}  // namespace

size_t BatchSmemBytes() { return sizeof(BatchShared); }

Status BuildBatchPlan(Context* ctx, const DevGraph& g, const BinSet& bins, BatchPlan* plan) {
  // Vertices of the bins up to kBinW1000 (degree <= 1000), in list order.
  uint32_t count = 0;
  for (int b = 0; b <= kBinW1000; ++b) count += bins.host_counts[b];
  plan->list = bins.list.p;  // bins G4..W1000 start at the beginning of the list
  plan->num_batches = 0;
  if (count == 0) return Status::Ok();
  DBuf<uint32_t> ddeg;
  PCC_RETURN_IF_ERROR(ddeg.Alloc(ctx, count));
  ListDegreesKernel<<<Blocks(count, 256, unsigned(ctx->num_sms) * 8), 256, 0, ctx->stream>>>(bins.list.p, count,
                                                                                            g.off.p, ddeg.p);
  PCC_COUNT(1);
  std::vector<uint32_t> deg(count);
  PCC_RETURN_IF_ERROR(ddeg.ToHost(deg.data(), count));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  std::vector<uint32_t> starts;
  starts.reserve(count / 8 + 2);
  uint32_t e = 0, nv = 0;
  starts.push_back(0);
  for (uint32_t i = 0; i < count; ++i) {
    if (nv > 0 && (nv == kBatchVerts || e + deg[i] > kBatchEdges)) {
      starts.push_back(i);
      e = 0;
      nv = 0;
    }
    e += deg[i];
    nv++;
  }
  starts.push_back(count);
  plan->num_batches = static_cast<uint32_t>(starts.size() - 1);
  PCC_RETURN_IF_ERROR(plan->starts.Alloc(ctx, starts.size()));
  PCC_RETURN_IF_ERROR(plan->starts.FromHost(starts.data(), starts.size()));
  return Sync(ctx);
}

Status LaunchBatchBestMoves(Context* ctx, const BMArgs& a, const BatchPlan& plan) {
  if (plan.num_batches == 0) return Status::Ok();
  const size_t smem = BatchSmemBytes();
  PCC_CUDA(cudaFuncSetAttribute(BatchBestMoveKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const unsigned grid = Blocks(plan.num_batches, 1, unsigned(ctx->num_sms) * 4);
  BatchBestMoveKernel<<<grid, kBT, smem, ctx->stream>>>(a, plan.list, plan.starts.p, plan.num_batches);
  PCC_COUNT(1);
  return LaunchCheck();
}

}  // namespace pcc
