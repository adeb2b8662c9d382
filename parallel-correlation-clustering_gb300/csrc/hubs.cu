// hubs.cu -- flat best-move kernels for hub vertices (degree > 1000); see
// hubs.cuh for the scheme.  Restates the hub branch of
// ClusteringHelper::EfficientBestMove (parallel-correlation-clusterer-
// internal.cc:516-582): per-cluster sums in any order (the reference adds
// concurrently), FP64-mode weights rounded to float after the offset, the
// argmax by (value desc, id asc), and "no entries" giving the reduce
// identity (0, 0.0) unless change >= 0.
#include <algorithm>
#include <vector>

#include "hubs.cuh"
#include "moves.cuh"

namespace pcc {
namespace {

constexpr int kHubThreads = 512;
constexpr int kHubScanThreads = 256;

// Order-preserving unsigned encodings (0 is below every encoded value).
__device__ __forceinline__ uint32_t OrderF32(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float UnorderF32(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ unsigned long long OrderF64(double d) {
  if (d == 0) d = 0.0;  // one encoding for +-0
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double UnorderF64(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double(static_cast<long long>(b));
}

struct HubArgs {
  BMArgs a;
  const uint32_t* hub_v;
  const uint32_t* hub_cap;
  const uint64_t* hub_toff;
  const uint32_t* ech_hub;
  const uint32_t* ech_e0;
  const uint32_t* uch_hub;
  const uint32_t* uch_u0;
  uint32_t num_hubs, num_echunks, num_uchunks;
  uint32_t* keys;
  unsigned long long* vals;
  uint32_t* used;
  uint32_t* used_count;
  long long* smax;
  uint32_t* ubound;
  unsigned long long* best;
  uint32_t* best_id;
  double* change;
};

__global__ void HubResetKernel(HubArgs h) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < h.num_hubs; i += gridDim.x * blockDim.x) {
    h.used_count[i] = 0;
    h.smax[i] = LLONG_MIN;
    h.ubound[i] = 0;
    h.best[i] = 0;
    h.best_id[i] = kNone;
  }
}

// Shared-memory pre-aggregation table of one row chunk (<= 2048 distinct
// keys, 4096 slots): keys, sums and the used list.
constexpr uint32_t kHubSmemSlots = 2 * kHubEdgeChunk;
constexpr size_t kHubAccSmem = size_t(kHubSmemSlots) * 12 + size_t(kHubEdgeChunk) * 2 +
                               size_t(kHubThreads / 32) * 32 * 8;

template <bool kInt, bool kAsync>
__global__ void __launch_bounds__(kHubThreads) HubAccumulateKernel(HubArgs h) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* svals = reinterpret_cast<unsigned long long*>(smem);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem + size_t(kHubSmemSlots) * 8);
  uint16_t* sused = reinterpret_cast<uint16_t*>(smem + size_t(kHubSmemSlots) * 12);
  double* stage = reinterpret_cast<double*>(smem + size_t(kHubSmemSlots) * 12 + size_t(kHubEdgeChunk) * 2);
  __shared__ uint32_t s_nused;
  const BMArgs& a = h.a;
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  for (uint32_t i = threadIdx.x; i < kHubSmemSlots; i += kHubThreads) {
    skeys[i] = kNone;
    svals[i] = 0ull;
  }
  if (threadIdx.x == 0) s_nused = 0;
  __syncthreads();
  for (uint32_t ci = blockIdx.x; ci < h.num_echunks; ci += gridDim.x) {
    const uint32_t hb = h.ech_hub[ci];
    const uint32_t v = h.hub_v[hb];
    if (!InFront(a, v)) continue;
    const uint64_t b = a.off[v];
    const uint32_t d = static_cast<uint32_t>(a.off[v + 1] - b);
    const uint32_t e0 = h.ech_e0[ci];
    const uint32_t e1 = min(d, e0 + kHubEdgeChunk);
    const uint32_t rounds = (e1 - e0 + kHubThreads - 1) / kHubThreads;
    // 1. Aggregate the chunk in shared memory.
    for (uint32_t r = 0; r < rounds; ++r) {
      const uint32_t e = e0 + r * kHubThreads + threadIdx.x;
      const bool has = e < e1;
      uint32_t u = v;
      float wt = 0.f;
      if (has) {
        u = a.nbr[b + e];
        wt = a.w ? a.w[b + e] : 1.0f;
      }
      const bool cand = has && u != v;
      const uint32_t cu = cand ? LdC<kAsync>(a.C + u) : kNone;
      const unsigned long long key = cand ? cu : (0x100000000ull | lane);
      const unsigned peers = __match_any_sync(kFull, key);
      const bool leader = cand && int(lane) == __ffs(peers) - 1;
      uint32_t slot = kNone;
      bool ins = false;
      if (leader) slot = FindOrInsertT<false>(skeys, kHubSmemSlots, cu, &ins);
      const unsigned im = __ballot_sync(kFull, ins);
      if (im) {
        uint32_t base = 0;
        const int ld = __ffs(im) - 1;
        if (int(lane) == ld) base = atomicAdd(&s_nused, uint32_t(__popc(im)));
        base = __shfl_sync(kFull, base, ld);
        if (ins) sused[base + __popc(im & LaneMaskLt())] = static_cast<uint16_t>(slot);
      }
      if (kInt) {
        const int xi = cand ? (static_cast<int>(wt) - a.ioffset) : 0;
        const int S = __reduce_add_sync(peers, xi);
        if (slot != kNone) atomicAdd(&svals[slot], static_cast<unsigned long long>(static_cast<long long>(S)));
      } else {
        // Hub path of the reference: `float weight; weight -= offset;`
        const float wf = static_cast<float>(Dsub(static_cast<double>(wt), a.offset));
        stage[warp * 32 + lane] = cand ? static_cast<double>(wf) : 0.0;
        __syncwarp();
        if (slot != kNone) {
          double acc = 0.0;
          unsigned mm = peers;
          while (mm) {
            const int j = __ffs(mm) - 1;
            acc = Dadd(acc, stage[warp * 32 + j]);
            mm &= mm - 1;
          }
          atomicAdd(reinterpret_cast<double*>(&svals[slot]), acc);
        }
        __syncwarp();
      }
    }
    __syncthreads();
    // 2. Flush the distinct keys into the hub's global table; clear smem.
    const uint32_t nl = s_nused;
    const uint32_t cap = h.hub_cap[hb];
    const uint64_t toff = h.hub_toff[hb];
    uint32_t* keys = h.keys + toff;
    unsigned long long* vals = h.vals + toff;
    uint32_t* used = h.used + toff / 2;
    const uint32_t nl32 = (nl + 31) & ~31u;
    for (uint32_t i = threadIdx.x; i < nl32; i += kHubThreads) {
      const bool in = i < nl;
      uint32_t gslot = kNone;
      bool ins = false;
      unsigned long long sv = 0;
      if (in) {
        const uint32_t ss = sused[i];
        const uint32_t key = skeys[ss];
        sv = svals[ss];
        skeys[ss] = kNone;
        svals[ss] = 0ull;
        gslot = FindOrInsertT<true>(keys, cap, key, &ins);
        if (gslot == kNone) atomicExch(&a.ctr->error, kErrHashFull);
      }
      const unsigned im = __ballot_sync(kFull, ins);
      uint32_t base = 0;
      if (im) {
        const int ld = __ffs(im) - 1;
        if (int(lane) == ld) base = atomicAdd(&h.used_count[hb], uint32_t(__popc(im)));
        base = __shfl_sync(kFull, base, ld);
      }
      if (ins) used[base + __popc(im & LaneMaskLt())] = gslot;
      if (in && gslot != kNone) {
        if (kInt)
          atomicAdd(&vals[gslot], sv);
        else
          atomicAdd(reinterpret_cast<double*>(&vals[gslot]), __longlong_as_double(static_cast<long long>(sv)));
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_nused = 0;
    __syncthreads();
  }
}

// Compacts each hub's (key, sum) pairs and clears the table slots.
__global__ void __launch_bounds__(256) HubGatherKernel(HubArgs h, uint32_t* pkeys, unsigned long long* pvals) {
  for (uint32_t ci = blockIdx.x; ci < h.num_uchunks; ci += gridDim.x) {
    const uint32_t hb = h.uch_hub[ci];
    const uint32_t nused = h.used_count[hb];
    const uint32_t u0 = h.uch_u0[ci];
    if (u0 >= nused) continue;
    const uint32_t u1 = min(nused, u0 + kHubUsedChunk);
    const uint64_t toff = h.hub_toff[hb];
    for (uint32_t i = u0 + threadIdx.x; i < u1; i += 256) {
      const uint32_t slot = h.used[toff / 2 + i];
      pkeys[toff / 2 + i] = h.keys[toff + slot];
      pvals[toff / 2 + i] = h.vals[toff + slot];
      h.keys[toff + slot] = kNone;
      h.vals[toff + slot] = 0ull;
    }
  }
}

template <bool kInt, bool kAsync>
__global__ void HubChangeKernel(HubArgs h) {
  const BMArgs& a = h.a;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < h.num_hubs; i += gridDim.x * blockDim.x) {
    const uint32_t v = h.hub_v[i];
    if (!InFront(a, v)) continue;
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    const uint64_t toff = h.hub_toff[i];
    const uint32_t slot = FindT<true>(h.keys + toff, h.hub_cap[i], x.c);
    const double T = slot != kNone ? AsDouble<kInt>(__ldcg(h.vals + toff + slot)) : 0.0;
    h.change[i] = ChangeOf(a, x, T);
  }
}

// Phases over the used lists: 0 = max S (INT filter), 1 = filter bound,
// 2 = best exact value, 3 = lowest id among the best.
template <bool kInt, bool kFilter, bool kAsync, int kPhase>
__global__ void __launch_bounds__(kHubScanThreads) HubScanKernel(HubArgs h, const uint32_t* __restrict__ pkeys,
                                                                const unsigned long long* __restrict__ pvals) {
  const BMArgs& a = h.a;
  for (uint32_t ci = blockIdx.x; ci < h.num_uchunks; ci += gridDim.x) {
    const uint32_t hb = h.uch_hub[ci];
    const uint32_t v = h.hub_v[hb];
    if (!InFront(a, v)) continue;
    const uint32_t nused = __ldcg(h.used_count + hb);
    const uint32_t u0 = h.uch_u0[ci];
    if (u0 >= nused) continue;
    const uint32_t u1 = min(nused, u0 + kHubUsedChunk);
    const uint64_t poff = h.hub_toff[hb] / 2;
    const double kv = a.k[v];
    const double change = __ldcg(h.change + hb);
    const long long smax = kFilter ? __ldcg(h.smax + hb) : 0;
    const float U = (kFilter && kPhase >= 2) ? UnorderF32(__ldcg(h.ubound + hb)) : 0.f;
    const unsigned long long bestk = kPhase == 3 ? __ldcg(h.best + hb) : 0ull;
    long long m0 = LLONG_MIN;
    uint32_t m1 = 0;
    unsigned long long m2 = 0;
    uint32_t m3 = kNone;
    for (uint32_t i = u0 + threadIdx.x; i < u1; i += kHubScanThreads) {
      const uint32_t key = pkeys[poff + i];
      const unsigned long long sv = pvals[poff + i];
      if (kPhase == 0) {
        m0 = max(m0, static_cast<long long>(sv));
        continue;
      }
      bool contender = true;
      if (kFilter) {
        const long long Si = static_cast<long long>(sv);
        const float R = __fmul_rn(a.res32, __fmul_rn(static_cast<float>(kv), a.Kf[key]));
        const float Y = __fsub_rn(static_cast<float>(Si - smax), R);
        const float e = FilterBound(R, Y, static_cast<float>(Si), static_cast<float>(change));
        if (kPhase == 1) {
          m1 = max(m1, OrderF32(__fsub_rn(Y, e)));
          continue;
        }
        contender = __fadd_rn(Y, e) >= U;
      } else if (kPhase == 1) {
        continue;
      }
      if (!contender) continue;
      const double val = ValOf(a, kv, change, AsDouble<kInt>(sv), LdK<kAsync>(a.K + key));
      const unsigned long long ok = OrderF64(val);
      if (kPhase == 2) m2 = max(m2, ok);
      if (kPhase == 3 && ok == bestk) m3 = min(m3, key);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      if (kPhase == 0) m0 = max(m0, __shfl_xor_sync(kFull, m0, o));
      if (kPhase == 1) m1 = max(m1, __shfl_xor_sync(kFull, m1, o));
      if (kPhase == 2) m2 = max(m2, __shfl_xor_sync(kFull, m2, o));
      if (kPhase == 3) m3 = min(m3, __shfl_xor_sync(kFull, m3, o));
    }
    if (LaneId() == 0) {
      if (kPhase == 0 && m0 != LLONG_MIN) atomicMax(h.smax + hb, m0);
      if (kPhase == 1 && m1) atomicMax(h.ubound + hb, m1);
      if (kPhase == 2 && m2) atomicMax(h.best + hb, m2);
      if (kPhase == 3 && m3 != kNone) atomicMin(h.best_id + hb, m3);
    }
  }
}

template <bool kAsync>
__global__ void HubDecideKernel(HubArgs h) {
  const BMArgs& a = h.a;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < h.num_hubs; i += gridDim.x * blockDim.x) {
    const uint32_t v = h.hub_v[i];
    if (!InFront(a, v)) continue;
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    const double change = h.change[i];
    const unsigned long long bk = h.best[i];
    double best;
    uint32_t bid;
    if (bk == 0) {  // no entries: the reduce identity (0, 0.0)
      best = 0.0;
      bid = 0;
    } else {
      best = UnorderF64(bk);
      bid = h.best_id[i];
    }
    const bool append = Decide<kAsync>(a, x, best, bid, change);
    if (!kAsync && append) a.movers[atomicAdd(&a.ctr->movers, 1u)] = v;
  }
}

__global__ void HubDegreesKernel(const uint32_t* list, uint32_t count, const uint64_t* off, uint32_t* deg) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    deg[i] = static_cast<uint32_t>(off[list[i] + 1] - off[list[i]]);
}

template <bool kInt, bool kAsync>
Status LaunchHub(Context* ctx, const HubArgs& h, uint32_t* pkeys, unsigned long long* pvals) {
  cudaStream_t st = ctx->stream;
  const unsigned sms = unsigned(ctx->num_sms);
  const unsigned hb = Blocks(h.num_hubs, 256, sms * 4);
  const unsigned eg = Blocks(h.num_echunks, 1, sms * 4);
  const unsigned ug = Blocks(h.num_uchunks, 1, sms * 8);
  auto acc = HubAccumulateKernel<kInt, kAsync>;
  PCC_CUDA(cudaFuncSetAttribute(acc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kHubAccSmem)));
  HubResetKernel<<<hb, 256, 0, st>>>(h); PCC_COUNT(1);
  acc<<<eg, kHubThreads, kHubAccSmem, st>>>(h); PCC_COUNT(1);
  HubChangeKernel<kInt, kAsync><<<hb, 256, 0, st>>>(h); PCC_COUNT(1);
  HubGatherKernel<<<ug, 256, 0, st>>>(h, pkeys, pvals); PCC_COUNT(1);
  constexpr bool kFilter = kInt && !kAsync;
  if (kFilter) {
    HubScanKernel<kInt, kFilter, kAsync, 0><<<ug, kHubScanThreads, 0, st>>>(h, pkeys, pvals); PCC_COUNT(1);
    HubScanKernel<kInt, kFilter, kAsync, 1><<<ug, kHubScanThreads, 0, st>>>(h, pkeys, pvals); PCC_COUNT(1);
  }
  // Without the filter every candidate gets its exact value.
  HubScanKernel<kInt, kFilter, kAsync, 2><<<ug, kHubScanThreads, 0, st>>>(h, pkeys, pvals); PCC_COUNT(1);
  HubScanKernel<kInt, kFilter, kAsync, 3><<<ug, kHubScanThreads, 0, st>>>(h, pkeys, pvals); PCC_COUNT(1);
  HubDecideKernel<kAsync><<<hb, 256, 0, st>>>(h); PCC_COUNT(1);
  return LaunchCheck();
}

}  // namespace

Status BuildHubPlan(Context* ctx, const DevGraph& g, const BinSet& bins, HubPlan* plan) {
  // Hubs are the static bins above the warp bins (degree > 1000).
  uint32_t start = 0, count = 0;
  for (int b = 0; b < kBinCta; ++b) start += bins.host_counts[b];
  for (int b = kBinCta; b < kNumBins; ++b) count += bins.host_counts[b];
  plan->num_hubs = count;
  if (count == 0) return Status::Ok();
  std::vector<uint32_t> hv(count), hd(count);
  DBuf<uint32_t> ddeg;
  PCC_RETURN_IF_ERROR(ddeg.Alloc(ctx, count));
  HubDegreesKernel<<<Blocks(count, 256, 1024), 256, 0, ctx->stream>>>(bins.list.p + start, count, g.off.p, ddeg.p);
  PCC_COUNT(1);
  PCC_CUDA(cudaMemcpyAsync(hv.data(), bins.list.p + start, sizeof(uint32_t) * count, cudaMemcpyDeviceToHost,
                           ctx->stream));
  PCC_RETURN_IF_ERROR(ddeg.ToHost(hd.data(), count));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  std::vector<uint32_t> cap(count), ech_hub, ech_e0, uch_hub, uch_u0;
  std::vector<uint64_t> toff(count);
  uint64_t total = 0;
  for (uint32_t i = 0; i < count; ++i) {
    uint32_t c = 2048;
    while (c < 2ull * hd[i] + 2) c <<= 1;
    cap[i] = c;
    toff[i] = total;
    total += c;
    for (uint32_t e = 0; e < hd[i]; e += kHubEdgeChunk) {
      ech_hub.push_back(i);
      ech_e0.push_back(e);
    }
    for (uint32_t u = 0; u < c / 2; u += kHubUsedChunk) {
      uch_hub.push_back(i);
      uch_u0.push_back(u);
    }
  }
  plan->total_slots = total;
  plan->num_echunks = static_cast<uint32_t>(ech_hub.size());
  plan->num_uchunks = static_cast<uint32_t>(uch_hub.size());
  PCC_RETURN_IF_ERROR(plan->hub_v.Alloc(ctx, count));
  PCC_RETURN_IF_ERROR(plan->hub_v.FromHost(hv.data(), count));
  PCC_RETURN_IF_ERROR(plan->hub_cap.Alloc(ctx, count));
  PCC_RETURN_IF_ERROR(plan->hub_cap.FromHost(cap.data(), count));
  PCC_RETURN_IF_ERROR(plan->hub_toff.Alloc(ctx, count));
  PCC_RETURN_IF_ERROR(plan->hub_toff.FromHost(toff.data(), count));
  PCC_RETURN_IF_ERROR(plan->ech_hub.Alloc(ctx, ech_hub.size()));
  PCC_RETURN_IF_ERROR(plan->ech_hub.FromHost(ech_hub.data(), ech_hub.size()));
  PCC_RETURN_IF_ERROR(plan->ech_e0.Alloc(ctx, ech_e0.size()));
  PCC_RETURN_IF_ERROR(plan->ech_e0.FromHost(ech_e0.data(), ech_e0.size()));
  PCC_RETURN_IF_ERROR(plan->uch_hub.Alloc(ctx, uch_hub.size()));
  PCC_RETURN_IF_ERROR(plan->uch_hub.FromHost(uch_hub.data(), uch_hub.size()));
  PCC_RETURN_IF_ERROR(plan->uch_u0.Alloc(ctx, uch_u0.size()));
  PCC_RETURN_IF_ERROR(plan->uch_u0.FromHost(uch_u0.data(), uch_u0.size()));
  return Sync(ctx);  // host vectors go out of scope
}

Status AllocHubState(Context* ctx, const HubPlan& plan, HubState* st) {
  const uint64_t slots = std::max<uint64_t>(plan.total_slots, 1);
  if (st->keys.count < slots) {
    PCC_RETURN_IF_ERROR(st->keys.Alloc(ctx, slots));
    PCC_RETURN_IF_ERROR(st->vals.Alloc(ctx, slots));
    PCC_RETURN_IF_ERROR(st->used.Alloc(ctx, slots / 2 + 1));
    PCC_RETURN_IF_ERROR(st->pkeys.Alloc(ctx, slots / 2 + 1));
    PCC_RETURN_IF_ERROR(st->pvals.Alloc(ctx, slots / 2 + 1));
    PCC_RETURN_IF_ERROR(st->keys.Fill(0xFF));
    PCC_RETURN_IF_ERROR(st->vals.Zero());
  }
  const uint64_t h = std::max<uint32_t>(plan.num_hubs, 1);
  if (st->used_count.count < h) {
    PCC_RETURN_IF_ERROR(st->used_count.Alloc(ctx, h));
    PCC_RETURN_IF_ERROR(st->smax.Alloc(ctx, h));
    PCC_RETURN_IF_ERROR(st->ubound.Alloc(ctx, h));
    PCC_RETURN_IF_ERROR(st->best.Alloc(ctx, h));
    PCC_RETURN_IF_ERROR(st->best_id.Alloc(ctx, h));
    PCC_RETURN_IF_ERROR(st->change.Alloc(ctx, h));
  }
  return Status::Ok();
}

Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode) {
  if (plan.num_hubs == 0) return Status::Ok();
  HubArgs h;
  h.a = a;
  h.hub_v = plan.hub_v.p;
  h.hub_cap = plan.hub_cap.p;
  h.hub_toff = plan.hub_toff.p;
  h.ech_hub = plan.ech_hub.p;
  h.ech_e0 = plan.ech_e0.p;
  h.uch_hub = plan.uch_hub.p;
  h.uch_u0 = plan.uch_u0.p;
  h.num_hubs = plan.num_hubs;
  h.num_echunks = plan.num_echunks;
  h.num_uchunks = plan.num_uchunks;
  h.keys = st.keys.p;
  h.vals = st.vals.p;
  h.used = st.used.p;
  h.used_count = st.used_count.p;
  h.smax = st.smax.p;
  h.ubound = st.ubound.p;
  h.best = st.best.p;
  h.best_id = st.best_id.p;
  h.change = st.change.p;
  uint32_t* pk = st.pkeys.p;
  unsigned long long* pv = st.pvals.p;
  if (a.async) return int_mode ? LaunchHub<true, true>(ctx, h, pk, pv) : LaunchHub<false, true>(ctx, h, pk, pv);
  return int_mode ? LaunchHub<true, false>(ctx, h, pk, pv) : LaunchHub<false, false>(ctx, h, pk, pv);
}

}  // namespace pcc
