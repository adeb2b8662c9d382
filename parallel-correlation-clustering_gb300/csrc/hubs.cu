// hubs.cu -- best moves of hub vertices (degree > 1000); the scheme is in
// hubs.cuh.  Restates the hub branch of ClusteringHelper::EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:516-582): per-cluster sums in
// any order (the reference adds concurrently), FP64-mode weights rounded to
// float after the offset, the argmax by (value desc, id asc), and "no
// entries" giving the reduce identity (0, 0.0) unless change >= 0.
#include <algorithm>
#include <numeric>
#include <type_traits>
#include <vector>

#include "hubs.cuh"
#include "moves.cuh"

namespace pcc {
namespace {

constexpr int kHT = 256;                  // threads per hub CTA
constexpr int kHW = kHT / 32;
constexpr int kHubUnroll = 4;             // entries per thread in flight
constexpr uint32_t kHubMaxSub = 1u << 12; // sub-partitions before giving up
constexpr size_t kHubSmem = size_t(kHubSlots) * 12;

struct HubArgs {
  BMArgs a;
  const uint32_t* hub_v;
  const uint32_t* hub_parts;
  const uint32_t* hub_pbase;
  const uint32_t* item_hub;
  const uint32_t* item_part;
  uint32_t num_items;
  double* part_val;
  uint32_t* part_id;
  uint32_t* done;
};

// MurmurHash3's 32-bit finalizer (a bijection; all output bits depend on all
// input bits).  Top bits pick the partition, bits 12.. the sub-partition,
// low bits the slot.
__device__ __forceinline__ uint32_t Mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ void KeepBest(double& bv, uint32_t& bi, double v, uint32_t i) {
  if (i == kNone) return;
  if (bi == kNone || v > bv || (v == bv && i < bi)) {
    bv = v;
    bi = i;
  }
}

// Block reductions; every thread receives the result.  `red` holds kHW
// entries of 8 bytes.
__device__ __forceinline__ long long BlockMaxLL(long long x, long long* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x = max(x, __shfl_xor_sync(kFull, x, o));
  if (LaneId() == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  long long r = red[0];
#pragma unroll
  for (int w = 1; w < kHW; ++w) r = max(r, red[w]);
  __syncthreads();
  return r;
}

__device__ __forceinline__ float BlockMaxF(float x, float* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x = fmaxf(x, __shfl_xor_sync(kFull, x, o));
  if (LaneId() == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  float r = red[0];
#pragma unroll
  for (int w = 1; w < kHW; ++w) r = fmaxf(r, red[w]);
  __syncthreads();
  return r;
}

// Deterministic sum: butterfly inside warps, then the warps in order.
template <class T>
__device__ __forceinline__ T BlockSum(T x, T* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    if constexpr (std::is_floating_point<T>::value) {
      x = Dadd(x, __shfl_xor_sync(kFull, x, o));
    } else {
      x += __shfl_xor_sync(kFull, x, o);
    }
  }
  if (LaneId() == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  T r = red[0];
#pragma unroll
  for (int w = 1; w < kHW; ++w) {
    if constexpr (std::is_floating_point<T>::value) {
      r = Dadd(r, red[w]);
    } else {
      r += red[w];
    }
  }
  __syncthreads();
  return r;
}

__device__ __forceinline__ void BlockArgmax(double& v, uint32_t& id, double* redv, uint32_t* redi) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const double ov = __shfl_xor_sync(kFull, v, o);
    const uint32_t oi = __shfl_xor_sync(kFull, id, o);
    KeepBest(v, id, ov, oi);
  }
  if (LaneId() == 0) {
    redv[threadIdx.x >> 5] = v;
    redi[threadIdx.x >> 5] = id;
  }
  __syncthreads();
  double rv = redv[0];
  uint32_t ri = redi[0];
#pragma unroll
  for (int w = 1; w < kHW; ++w) KeepBest(rv, ri, redv[w], redi[w]);
  __syncthreads();
  v = rv;
  id = ri;
}

// Order-preserving integer image of a double (no FP64 instruction); -0 and
// +0 map to the same value.
__device__ __forceinline__ unsigned long long KOrder(double d) {
  unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// (S desc, K asc, id asc) lexicographic leader; id kNone = none.
struct LexKey {
  long long S = LLONG_MIN;
  unsigned long long K = ~0ull;
  uint32_t id = kNone;
  __device__ __forceinline__ void Keep(long long s, unsigned long long k, uint32_t i) {
    if (i == kNone) return;
    if (id == kNone || s > S || (s == S && (k < K || (k == K && i < id)))) {
      S = s;
      K = k;
      id = i;
    }
  }
};

__device__ __forceinline__ LexKey BlockLex(LexKey x, long long* rs, unsigned long long* rk, uint32_t* ri) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const long long s = __shfl_xor_sync(kFull, x.S, o);
    const unsigned long long k = __shfl_xor_sync(kFull, x.K, o);
    const uint32_t i = __shfl_xor_sync(kFull, x.id, o);
    x.Keep(s, k, i);
  }
  if (LaneId() == 0) {
    rs[threadIdx.x >> 5] = x.S;
    rk[threadIdx.x >> 5] = x.K;
    ri[threadIdx.x >> 5] = x.id;
  }
  __syncthreads();
  LexKey r;
#pragma unroll
  for (int w = 0; w < kHW; ++w) r.Keep(rs[w], rk[w], ri[w]);
  __syncthreads();
  return r;
}

// Finds or inserts `key`, probing from the hash's low bits; kNone when the
// table is full.
__device__ __forceinline__ uint32_t HubInsert(uint32_t* keys, uint32_t cap, uint32_t hsh, uint32_t key, bool* ins) {
  const uint32_t mask = cap - 1;
  uint32_t s = hsh & mask;
  *ins = false;
  for (uint32_t pr = 0; pr < cap; ++pr) {
    const uint32_t k = *reinterpret_cast<volatile uint32_t*>(keys + s);
    if (k == key) return s;
    if (k == kNone) {
      const uint32_t old = atomicCAS(keys + s, kNone, key);
      if (old == kNone) {
        *ins = true;
        return s;
      }
      if (old == key) return s;
    }
    s = (s + 1) & mask;
  }
  return kNone;
}

template <bool kInt, bool kAsync>
__global__ void __launch_bounds__(kHT, 4) HubPartKernel(HubArgs h) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* svals = reinterpret_cast<unsigned long long*>(smem);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem + size_t(kHubSlots) * 8);
  __shared__ __align__(8) unsigned char red_raw[kHW * 8];
  __shared__ uint32_t redi[kHW];
  __shared__ unsigned long long red_lex[kHW];
  __shared__ double s_change;
  __shared__ double stage[kHW][32];
  __shared__ uint32_t s_nkeys, s_overflow;
  long long* red_ll = reinterpret_cast<long long*>(red_raw);
  float* red_f = reinterpret_cast<float*>(red_raw);
  double* red_d = reinterpret_cast<double*>(red_raw);
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x, lane = LaneId(), warp = tid >> 5;
  constexpr bool kFilter = kInt && !kAsync;

  for (uint32_t i = tid; i < kHubSlots; i += kHT) {
    skeys[i] = kNone;
    svals[i] = 0ull;
  }
  if (tid == 0) {
    s_nkeys = 0;
    s_overflow = 0;
  }
  __syncthreads();

  for (uint32_t item = blockIdx.x; item < h.num_items; item += gridDim.x) {
    const uint32_t hb = h.item_hub[item];
    const uint32_t p = h.item_part[item];
    const uint32_t v = h.hub_v[hb];
    if (!InFront(a, v)) continue;  // uniform over the CTA
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    const uint32_t P = h.hub_parts[hb];
    const uint32_t per_part = (x.d + P - 1) / P;
    uint32_t cap = 256;
    while (cap < 2 * per_part + 2 && cap < kHubSlots) cap <<= 1;
    const uint32_t maxkeys = cap - cap / 4;
    const float k32 = a.kf[v];

    uint32_t Q = 1, q = 0;
    bool have_T = false;
    double change = 0.0;
    double bestv = 0.0;
    uint32_t bestid = kNone;
    while (true) {
      // 1. Scan the row: partition sums into the table, "together" once.
      long long t_int = 0;
      double t_dbl = 0.0;
      for (uint32_t e0 = 0; e0 < x.d; e0 += kHT * kHubUnroll) {
        uint32_t uu[kHubUnroll];
        float ww[kHubUnroll];
#pragma unroll
        for (int k = 0; k < kHubUnroll; ++k) {
          const uint32_t e = e0 + k * kHT + tid;
          uu[k] = v;
          ww[k] = 0.f;
          if (e < x.d) {
            uu[k] = a.nbr[x.b + e];
            ww[k] = a.w ? a.w[x.b + e] : 1.0f;
          }
        }
        uint32_t cc[kHubUnroll];
#pragma unroll
        for (int k = 0; k < kHubUnroll; ++k) cc[k] = uu[k] != v ? LdC<kAsync>(a.C + uu[k]) : kNone;
#pragma unroll
        for (int k = 0; k < kHubUnroll; ++k) {
          const bool cand = uu[k] != v;
          const uint32_t cu = cc[k];
          int xi = 0;
          double xd = 0.0;
          if (kInt) {
            xi = cand ? (static_cast<int>(ww[k]) - a.ioffset) : 0;
          } else if (cand) {
            // `float weight; weight -= offset;` of the reference's hub path.
            xd = static_cast<double>(static_cast<float>(Dsub(static_cast<double>(ww[k]), a.offset)));
          }
          if (!have_T && cand && cu == x.c) {
            if (kInt)
              t_int += xi;
            else
              t_dbl = Dadd(t_dbl, xd);
          }
          const uint32_t hsh = Mix32(cu);
          const bool mine = cand && __umulhi(hsh, P) == p && ((hsh >> 12) & (Q - 1)) == q &&
                            *reinterpret_cast<volatile uint32_t*>(&s_overflow) == 0;
          const unsigned peers = __match_any_sync(kFull, mine ? cu : LaneSentinel(lane));
          const bool leader = mine && int(lane) == __ffs(peers) - 1;
          uint32_t slot = kNone;
          bool ins = false;
          if (leader) {
            slot = HubInsert(skeys, cap, hsh, cu, &ins);
            if (slot == kNone) s_overflow = 1;
          }
          const unsigned im = __ballot_sync(kFull, ins);
          if (im && int(lane) == __ffs(im) - 1) {
            const uint32_t nk = atomicAdd(&s_nkeys, uint32_t(__popc(im))) + uint32_t(__popc(im));
            if (nk > maxkeys) s_overflow = 1;
          }
          if (kInt) {
            const int S = GroupSumInt(peers, xi, a.w == nullptr, leader, reinterpret_cast<int*>(stage[warp]));
            if (slot != kNone) atomicAdd(&svals[slot], static_cast<unsigned long long>(static_cast<long long>(S)));
          } else {
            stage[warp][lane] = xd;
            __syncwarp();
            if (slot != kNone) {
              double acc = 0.0;
              unsigned mm = peers;
              while (mm) {
                const int j = __ffs(mm) - 1;
                acc = Dadd(acc, stage[warp][j]);
                mm &= mm - 1;
              }
              atomicAdd(reinterpret_cast<double*>(&svals[slot]), acc);
            }
            __syncwarp();
          }
        }
      }
      __syncthreads();
      if (!have_T) {
        double T;
        if (kInt)
          T = static_cast<double>(BlockSum<long long>(t_int, red_ll));
        else
          T = BlockSum<double>(t_dbl, red_d);
        if (tid == 0) s_change = ChangeOf(a, x, T);  // FP64: once per CTA
        __syncthreads();
        change = s_change;
        have_T = true;
      }
      const bool overflow = s_overflow != 0;
      __syncthreads();
      if (overflow) {
        // Split the partition further and rescan from the first sub-pass.
        for (uint32_t s = tid; s < cap; s += kHT) {
          skeys[s] = kNone;
          svals[s] = 0ull;
        }
        __syncthreads();
        if (tid == 0) {
          s_overflow = 0;
          s_nkeys = 0;
        }
        __syncthreads();
        Q *= 2;
        q = 0;
        bestv = 0.0;
        bestid = kNone;
        if (Q > kHubMaxSub) {
          if (tid == 0) atomicExch(&a.ctr->error, kErrHashFull);
          break;
        }
        continue;
      }
      // 2. Evaluate the table.
      double lv = 0.0;
      uint32_t lid = kNone;
      if (kFilter) {
        // FP32 pre-filter (FilterBound): U = max(Y' - e); contenders have
        // Y' + e >= U.  Contenders with equal (S, K) have equal FP64 values,
        // so the class that leads by (S desc, K asc) is represented by its
        // lowest id and evaluated once; only the other contenders get their
        // own FP64 value.
        long long smax = LLONG_MIN;
        for (uint32_t s = tid; s < cap; s += kHT)
          if (skeys[s] != kNone) smax = max(smax, static_cast<long long>(svals[s]));
        smax = BlockMaxLL(smax, red_ll);
        const float c32 = static_cast<float>(change);
        float U = -CUDART_INF_F;
        for (uint32_t s = tid; s < cap; s += kHT) {
          const uint32_t key = skeys[s];
          if (key == kNone) continue;
          const long long Si = static_cast<long long>(svals[s]);
          const float R = __fmul_rn(a.res32, __fmul_rn(k32, a.Kf[key]));
          const float Y = __fsub_rn(static_cast<float>(Si - smax), R);
          U = fmaxf(U, __fsub_rn(Y, FilterBound(R, Y, static_cast<float>(Si), c32)));
        }
        U = BlockMaxF(U, red_f);
        LexKey lead;
        for (uint32_t s = tid; s < cap; s += kHT) {
          const uint32_t key = skeys[s];
          if (key == kNone) continue;
          const long long Si = static_cast<long long>(svals[s]);
          const float R = __fmul_rn(a.res32, __fmul_rn(k32, a.Kf[key]));
          const float Y = __fsub_rn(static_cast<float>(Si - smax), R);
          if (__fadd_rn(Y, FilterBound(R, Y, static_cast<float>(Si), c32)) < U) {
            skeys[s] = kNone;  // never the best: drop now
            svals[s] = 0ull;
            continue;
          }
          lead.Keep(Si, KOrder(a.K[key]), key);
        }
        lead = BlockLex(lead, red_ll, reinterpret_cast<unsigned long long*>(red_lex), redi);
        for (uint32_t s = tid; s < cap; s += kHT) {
          const uint32_t key = skeys[s];
          if (key == kNone) continue;
          const long long Si = static_cast<long long>(svals[s]);
          skeys[s] = kNone;
          svals[s] = 0ull;
          const double KD = a.K[key];
          if (Si == lead.S && KOrder(KD) == lead.K) continue;  // the leading class
          KeepBest(lv, lid, ValOf(a, x.kv, change, static_cast<double>(Si), KD), key);
        }
        if (tid == 0 && lead.id != kNone)
          KeepBest(lv, lid, ValOf(a, x.kv, change, static_cast<double>(lead.S), a.K[lead.id]), lead.id);
      } else {
        for (uint32_t s = tid; s < cap; s += kHT) {
          const uint32_t key = skeys[s];
          if (key == kNone) continue;
          const unsigned long long sv = svals[s];
          skeys[s] = kNone;
          svals[s] = 0ull;
          KeepBest(lv, lid, ValOf(a, x.kv, change, AsDouble<kInt>(sv), LdK<kAsync>(a.K + key)), key);
        }
      }
      BlockArgmax(lv, lid, red_d, redi);
      KeepBest(bestv, bestid, lv, lid);
      if (tid == 0) s_nkeys = 0;
      __syncthreads();
      if (++q == Q) break;
    }

    // 3. Partial result; the hub's last CTA combines and decides.
    if (tid == 0) {
      const uint32_t pb = h.hub_pbase[hb];
      h.part_val[pb + p] = bestv;
      h.part_id[pb + p] = bestid;
      __threadfence();
      const uint32_t old = atomicAdd(&h.done[hb], 1u);
      if (old == P - 1) {
        __threadfence();
        double bv = 0.0;
        uint32_t bi = kNone;
        for (uint32_t j = 0; j < P; ++j) KeepBest(bv, bi, __ldcg(h.part_val + pb + j), __ldcg(h.part_id + pb + j));
        h.done[hb] = 0;
        if (bi == kNone) {  // no entries: the reduce identity (0, 0.0)
          bv = 0.0;
          bi = 0;
        }
        const bool append = Decide<kAsync>(a, x, bv, bi, change);
        if (!kAsync && append) a.movers[atomicAdd(&a.ctr->movers, 1u)] = v;
      }
    }
  }
}

__global__ void HubDegreesKernel(const uint32_t* list, uint32_t count, const uint64_t* off, uint32_t* deg) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    deg[i] = static_cast<uint32_t>(off[list[i] + 1] - off[list[i]]);
}

template <bool kInt, bool kAsync>
Status LaunchHub(Context* ctx, const HubArgs& h) {
  auto k = HubPartKernel<kInt, kAsync>;
  PCC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kHubSmem)));
  const unsigned grid = Blocks(h.num_items, 1, unsigned(ctx->num_sms) * 4);
  k<<<grid, kHT, kHubSmem, ctx->stream>>>(h);
  PCC_COUNT(1);
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
  // Largest hubs first; a hub's partitions are consecutive items, so they
  // run on different CTAs at the same time and share the row through L2.
  std::vector<uint32_t> order(count);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t i, uint32_t j) { return hd[i] > hd[j]; });
  std::vector<uint32_t> v_sorted(count), parts(count), pbase(count), item_hub, item_part;
  uint64_t total = 0;
  for (uint32_t r = 0; r < count; ++r) {
    const uint32_t i = order[r];
    v_sorted[r] = hv[i];
    const uint32_t P = std::max<uint32_t>(1, (hd[i] + kHubPartKeys - 1) / kHubPartKeys);
    parts[r] = P;
    pbase[r] = static_cast<uint32_t>(total);
    total += P;
    for (uint32_t p = 0; p < P; ++p) {
      item_hub.push_back(r);
      item_part.push_back(p);
    }
  }
  if (total > 0xFFFFFFFFull) return MakeError(PCC_OUT_OF_RANGE, "too many hub partitions");
  plan->num_items = static_cast<uint32_t>(item_hub.size());
  plan->num_partials = total;
  PCC_RETURN_IF_ERROR(plan->hub_v.Alloc(ctx, count));
  PCC_RETURN_IF_ERROR(plan->hub_v.FromHost(v_sorted.data(), count));
  PCC_RETURN_IF_ERROR(plan->hub_parts.Alloc(ctx, count));
  PCC_RETURN_IF_ERROR(plan->hub_parts.FromHost(parts.data(), count));
  PCC_RETURN_IF_ERROR(plan->hub_pbase.Alloc(ctx, count));
  PCC_RETURN_IF_ERROR(plan->hub_pbase.FromHost(pbase.data(), count));
  PCC_RETURN_IF_ERROR(plan->item_hub.Alloc(ctx, item_hub.size()));
  PCC_RETURN_IF_ERROR(plan->item_hub.FromHost(item_hub.data(), item_hub.size()));
  PCC_RETURN_IF_ERROR(plan->item_part.Alloc(ctx, item_part.size()));
  PCC_RETURN_IF_ERROR(plan->item_part.FromHost(item_part.data(), item_part.size()));
  return Sync(ctx);  // host vectors go out of scope
}

Status AllocHubState(Context* ctx, const HubPlan& plan, HubState* st) {
  const uint64_t np = std::max<uint64_t>(plan.num_partials, 1);
  if (st->part_val.count < np) {
    PCC_RETURN_IF_ERROR(st->part_val.Alloc(ctx, np));
    PCC_RETURN_IF_ERROR(st->part_id.Alloc(ctx, np));
  }
  const uint64_t nh = std::max<uint32_t>(plan.num_hubs, 1);
  if (st->done.count < nh) PCC_RETURN_IF_ERROR(st->done.Alloc(ctx, nh));
  return st->done.Zero();
}

Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode) {
  if (plan.num_hubs == 0) return Status::Ok();
  HubArgs h;
  h.a = a;
  h.hub_v = plan.hub_v.p;
  h.hub_parts = plan.hub_parts.p;
  h.hub_pbase = plan.hub_pbase.p;
  h.item_hub = plan.item_hub.p;
  h.item_part = plan.item_part.p;
  h.num_items = plan.num_items;
  h.part_val = st.part_val.p;
  h.part_id = st.part_id.p;
  h.done = st.done.p;
  if (a.async) return int_mode ? LaunchHub<true, true>(ctx, h) : LaunchHub<false, true>(ctx, h);
  return int_mode ? LaunchHub<true, false>(ctx, h) : LaunchHub<false, false>(ctx, h);
}

}  // namespace pcc
