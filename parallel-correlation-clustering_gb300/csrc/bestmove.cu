// bestmove.cu -- degree-binned best-move kernels.
//
// Restates ClusteringHelper::EfficientBestMove
// (clustering/clusterers/parallel-correlation-clusterer-internal.cc:448-583)
// with EdgeSum (correlation-clusterer-util.h:26-43), the sync decision of
// BestMovesForVertexSubset (parallel-correlation-clusterer.cc:139-157) and
// AsyncMove (parallel-correlation-clusterer-internal.cc:371-403).
//
// For vertex v in cluster c with node weight kv, over neighbours u != v:
//   S_D    = sum over neighbours in cluster D of (w - offset)
//   T      = S_c
//   change = 0 - (T - res * (kv * (K_c - kv)))
//   val_D  = change + (S_D - res * (kv * K_D))
// The chosen move is argmax_D val_D (ties -> lowest D), unless change >= max
// val, in which case it is "new cluster" (target n, value change).  Every
// operation is a separately rounded IEEE double op (no FMA), as in the
// reference.
//
// Accumulation of S_D:
//   INT mode  (weights and offset integral, |w - offset| <= 2^22): exact
//             integer sums, so any order gives the reference's doubles.
//   FP64 mode: degree <= 1000 adds in adjacency order (the reference's
//             sequential flat_hash_map path, bit-exact); hubs add in any
//             order, as the reference's concurrent map does.
#include "engine.cuh"

#include <math_constants.h>

#include <type_traits>

namespace pcc {

namespace {

__device__ __forceinline__ uint32_t WarpAppendFull(uint32_t* counter, bool pred) {
  const unsigned mask = __ballot_sync(kFull, pred);
  uint32_t base = 0;
  if (mask) {
    const int leader = __ffs(mask) - 1;
    if (int(LaneId()) == leader) base = atomicAdd(counter, uint32_t(__popc(mask)));
    base = __shfl_sync(kFull, base, leader);
  }
  return base + __popc(mask & LaneMaskLt());
}

template <bool kAsync>
__device__ __forceinline__ uint32_t LdC(const uint32_t* p) {
  return kAsync ? __ldcg(p) : __ldg(p);
}
template <bool kAsync>
__device__ __forceinline__ double LdK(const double* p) {
  return kAsync ? __ldcg(p) : __ldg(p);
}

__device__ __forceinline__ uint32_t HashSlot(uint32_t key, uint32_t mask) {
  return (key * 0x9E3779B1u) & mask;
}

// Open addressing with linear probing; keys are cluster ids, kNone = empty.
// Capacity is at least twice the number of keys, so a free slot exists.

// (val desc, id asc) ordering used by every argmax.
__device__ __forceinline__ bool Better(double va, uint32_t ia, double vb, uint32_t ib) {
  return va > vb || (va == vb && ia < ib);
}

struct VertexCtx {
  uint32_t v;
  uint64_t b;
  uint32_t d;
  uint32_t c;
  double kv;
  double Kc;
};

template <bool kAsync>
__device__ __forceinline__ VertexCtx LoadVertex(const BMArgs& a, uint32_t v) {
  VertexCtx x;
  x.v = v;
  x.b = a.off[v];
  x.d = uint32_t(a.off[v + 1] - x.b);
  x.c = LdC<kAsync>(a.C + v);
  x.kv = a.k[v];
  x.Kc = LdK<kAsync>(a.K + x.c);
  return x;
}

__device__ __forceinline__ double ChangeOf(const BMArgs& a, const VertexCtx& x, double T) {
  // change_in_objective -= together.NetWeight(kv * (K_c - kv))   (:483-488)
  return Dsub(0.0, Dsub(T, Dmul(a.res, Dmul(x.kv, Dsub(x.Kc, x.kv)))));
}

__device__ __forceinline__ double ValOf(const BMArgs& a, double kv, double change, double S, double KD) {
  // change + data.NetWeight(moving_nodes_weight * K_D)   (:493-497)
  return Dadd(change, Dsub(S, Dmul(a.res, Dmul(kv, KD))));
}

// Finishes one vertex: the chosen move and the sync / async decision.
// Returns true when the vertex must be appended to the movers list (sync).
template <bool kAsync>
__device__ __forceinline__ bool Decide(const BMArgs& a, const VertexCtx& x, double best, uint32_t bid,
                                       double change) {
  uint32_t target;
  double value;
  if (bid == kNone || change >= best) {
    target = a.n;
    value = change;
  } else {
    target = bid;
    value = best;
  }
  if (a.out_target) {
    a.out_target[x.v] = target;
    a.out_value[x.v] = value;
  }
  if (kAsync) {
    // AsyncMove (internal.cc:371-403): apply immediately.
    if (!(value > 0)) return false;
    const uint32_t cur = x.c;
    atomicSub(&a.s_mut[cur], 1u);
    atomicAdd(&a.K_mut[cur], -1 * x.kv);
    uint32_t dest = target;
    if (target != a.n) {
      atomicAdd(&a.s_mut[target], 1u);
      atomicAdd(&a.K_mut[target], x.kv);
    } else {
      // Claim an empty id by CAS, probing linearly from the vertex's own id.
      // Bounded: after 4n probes the kernel records an error and leaves the
      // vertex where it was (its leave is undone).
      uint64_t i = x.v;
      const uint64_t limit = 4ull * a.n + 64;
      bool got = false;
      for (uint64_t p = 0; p < limit; ++p) {
        if (__ldcg(&a.s_mut[i]) == 0u && atomicCAS(&a.s_mut[i], 0u, 1u) == 0u) {
          got = true;
          break;
        }
        i = (i + 1 == a.n) ? 0 : i + 1;
      }
      if (!got) {
        atomicAdd(&a.s_mut[cur], 1u);
        atomicAdd(&a.K_mut[cur], x.kv);
        atomicExch(&a.ctr->error, kErrProbeLimit);
        return false;
      }
      atomicAdd(&a.K_mut[i], x.kv);
      dest = uint32_t(i);
    }
    __stcg(&a.C_mut[x.v], dest);
    a.moved_cluster_stamp[dest] = a.stamp;
    a.moved_stamp[x.v] = a.stamp;
    atomicAdd(&a.ctr->moves, 1ull);
    return false;
  }
  // Sync decision (parallel-correlation-clusterer.cc:142-156): the singleton
  // rule, then move only on a positive value.
  uint32_t t2 = target;
  double v2 = value;
  if (target < a.n && a.s[target] == 1u && a.s[x.c] == 1u && x.c >= target) {
    t2 = x.c;
    v2 = 0;
  }
  if (a.out_moves) a.out_moves[x.v] = v2 > 0 ? t2 : kNone;
  if (v2 > 0) {
    a.moved_stamp[x.v] = a.stamp;
    if (t2 != x.c) {
      a.moves[x.v] = t2;
      return true;
    }
  }
  return false;
}

// ---------------------------------------------------------------------------
// Lane groups of G lanes, one vertex per group, degree <= G (one chunk).
// Equal cluster ids inside the group are found with match.any; the group
// leader of each id sums its peers in lane (= adjacency) order.
// ---------------------------------------------------------------------------
template <int G, bool kInt, bool kAsync>
__global__ void __launch_bounds__(256) BestMoveGroupKernel(BMArgs a, const uint32_t* __restrict__ list,
                                                          const uint32_t* __restrict__ bin_counts,
                                                          const uint32_t* __restrict__ bin_starts, int bin) {
  __shared__ double stage[8][32];
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  constexpr unsigned kVpw = 32 / G;
  const unsigned g = lane / G, gl = lane % G;
  const unsigned gmask = G == 32 ? kFull : (((1u << G) - 1u) << (g * G));
  const uint64_t stride = uint64_t(gridDim.x) * 8 * kVpw;
  for (uint64_t base = (uint64_t(blockIdx.x) * 8 + warp) * kVpw; base < count; base += stride) {
    const uint64_t idx = base + g;
    const bool vvalid = idx < count;
    VertexCtx x{};
    if (vvalid) x = LoadVertex<kAsync>(a, list[start + idx]);
    const bool has = vvalid && gl < x.d;
    uint32_t u = x.v;
    float wt = 0.f;
    if (has) {
      u = a.nbr[x.b + gl];
      wt = a.w ? a.w[x.b + gl] : 1.0f;
    }
    const bool cand = has && u != x.v;
    const uint32_t cu = cand ? LdC<kAsync>(a.C + u) : kNone;
    const unsigned long long key =
        cand ? ((static_cast<unsigned long long>(g) << 32) | cu) : (0xFFFFFFFF00000000ull | lane);
    const unsigned peers = __match_any_sync(kFull, key);
    const bool leader = cand && int(lane) == __ffs(peers) - 1;
    double S;
    if (kInt) {
      const int xi = cand ? (static_cast<int>(wt) - a.ioffset) : 0;
      S = static_cast<double>(__reduce_add_sync(peers, xi));
    } else {
      stage[warp][lane] = cand ? Dsub(static_cast<double>(wt), a.offset) : 0.0;
      __syncwarp();
      S = 0.0;
      if (leader) {
        unsigned mm = peers;
        while (mm) {
          const int j = __ffs(mm) - 1;
          S = Dadd(S, stage[warp][j]);
          mm &= mm - 1;
        }
      }
      __syncwarp();
    }
    const unsigned tmask = __ballot_sync(kFull, leader && cu == x.c) & gmask;
    const double Tsh = __shfl_sync(kFull, S, tmask ? __ffs(tmask) - 1 : int(lane));
    const double T = tmask ? Tsh : 0.0;
    const double change = ChangeOf(a, x, T);
    double val = -CUDART_INF;
    uint32_t id = kNone;
    if (leader) {
      val = ValOf(a, x.kv, change, S, LdK<kAsync>(a.K + cu));
      id = cu;
    }
#pragma unroll
    for (int o = G / 2; o >= 1; o >>= 1) {
      const double ov = __shfl_xor_sync(kFull, val, o);
      const uint32_t oid = __shfl_xor_sync(kFull, id, o);
      if (Better(ov, oid, val, id)) {
        val = ov;
        id = oid;
      }
    }
    bool append = false;
    if (vvalid && gl == 0) append = Decide<kAsync>(a, x, val, id, change);
    if (!kAsync) {
      const uint32_t slot = WarpAppendFull(&a.ctr->movers, append);
      if (append) a.movers[slot] = x.v;
    }
  }
}

// ---------------------------------------------------------------------------
// Hash tables with an occupied-slot list.  The table starts clean (keys
// kNone, values 0); each insert appends its slot to `used`, and after the
// vertex only the used slots are read and cleared, so the cost per vertex is
// proportional to its distinct neighbour clusters, not to the capacity.
// ---------------------------------------------------------------------------
template <bool kGlobal>
__device__ __forceinline__ uint32_t HKey(const uint32_t* keys, uint32_t i) {
  return kGlobal ? __ldcg(keys + i) : keys[i];
}
template <bool kGlobal>
__device__ __forceinline__ unsigned long long HVal(const unsigned long long* vals, uint32_t i) {
  return kGlobal ? __ldcg(vals + i) : vals[i];
}

// Finds or inserts `key`; *inserted is set when this call claimed the slot.
template <bool kGlobal>
__device__ __forceinline__ uint32_t FindOrInsertT(uint32_t* keys, uint32_t cap, uint32_t key, bool* inserted) {
  const uint32_t mask = cap - 1;
  uint32_t h = HashSlot(key, mask);
  *inserted = false;
  for (uint32_t probes = 0; probes < cap; ++probes) {
    const uint32_t k = HKey<kGlobal>(keys, h);
    if (k == key) return h;
    if (k == kNone) {
      const uint32_t old = atomicCAS(&keys[h], kNone, key);
      if (old == kNone) {
        *inserted = true;
        return h;
      }
      if (old == key) return h;
    }
    h = (h + 1) & mask;
  }
  return kNone;
}

template <bool kGlobal>
__device__ __forceinline__ uint32_t FindT(const uint32_t* keys, uint32_t cap, uint32_t key) {
  const uint32_t mask = cap - 1;
  uint32_t h = HashSlot(key, mask);
  for (uint32_t probes = 0; probes < cap; ++probes) {
    const uint32_t k = HKey<kGlobal>(keys, h);
    if (k == key) return h;
    if (k == kNone) return kNone;
    h = (h + 1) & mask;
  }
  return kNone;
}

template <bool kInt>
__device__ __forceinline__ double AsDouble(unsigned long long bits) {
  return kInt ? static_cast<double>(static_cast<long long>(bits))
              : __longlong_as_double(static_cast<long long>(bits));
}

// ---------------------------------------------------------------------------
// One warp per vertex, degree <= 1000, shared-memory hash of HC slots.
// Chunks of 32 entries in adjacency order; per chunk the leader of each
// cluster id adds its peers one by one (FP64) onto the slot's running sum,
// which keeps the reference's adjacency-order summation exactly.
// ---------------------------------------------------------------------------
constexpr int kWarpKernelWarps = 4;

template <int HC>
constexpr size_t WarpKernelSmem() {
  // per warp: vals HC*8, keys HC*4, used HC/2 * 2, stage 32*8, count 16
  return size_t(kWarpKernelWarps) * (size_t(HC) * 13 + 32 * 8 + 16);
}

template <int HC, bool kInt, bool kAsync>
__global__ void __launch_bounds__(kWarpKernelWarps * 32) BestMoveWarpKernel(BMArgs a,
                                                                           const uint32_t* __restrict__ list,
                                                                           const uint32_t* __restrict__ bin_counts,
                                                                           const uint32_t* __restrict__ bin_starts,
                                                                           int bin) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  unsigned char* base = smem + size_t(warp) * (size_t(HC) * 13 + 32 * 8 + 16);
  unsigned long long* vals = reinterpret_cast<unsigned long long*>(base);
  uint32_t* keys = reinterpret_cast<uint32_t*>(base + size_t(HC) * 8);
  double* stage = reinterpret_cast<double*>(base + size_t(HC) * 12);
  uint16_t* used = reinterpret_cast<uint16_t*>(base + size_t(HC) * 12 + 32 * 8);
  uint32_t* used_count = reinterpret_cast<uint32_t*>(base + size_t(HC) * 13 + 32 * 8);
  for (int i = lane; i < HC; i += 32) {
    keys[i] = kNone;
    vals[i] = 0ull;
  }
  if (lane == 0) *used_count = 0;
  __syncwarp();
  for (uint64_t idx = uint64_t(blockIdx.x) * kWarpKernelWarps + warp; idx < count;
       idx += uint64_t(gridDim.x) * kWarpKernelWarps) {
    const VertexCtx x = LoadVertex<kAsync>(a, list[start + idx]);
    for (uint32_t e0 = 0; e0 < x.d; e0 += 32) {
      const uint32_t e = e0 + lane;
      const bool has = e < x.d;
      uint32_t u = x.v;
      float wt = 0.f;
      if (has) {
        u = a.nbr[x.b + e];
        wt = a.w ? a.w[x.b + e] : 1.0f;
      }
      const bool cand = has && u != x.v;
      const uint32_t cu = cand ? LdC<kAsync>(a.C + u) : kNone;
      const unsigned long long key = cand ? cu : (0x100000000ull | lane);
      const unsigned peers = __match_any_sync(kFull, key);
      const bool leader = cand && int(lane) == __ffs(peers) - 1;
      uint32_t slot = kNone;
      if (leader) {
        bool ins = false;
        slot = FindOrInsertT<false>(keys, HC, cu, &ins);
        if (slot == kNone) {
          atomicExch(&a.ctr->error, kErrHashFull);
        } else if (ins) {
          used[atomicAdd(used_count, 1u)] = static_cast<uint16_t>(slot);
        }
      }
      if (kInt) {
        const int xi = cand ? (static_cast<int>(wt) - a.ioffset) : 0;
        const int S = __reduce_add_sync(peers, xi);
        if (slot != kNone) vals[slot] += static_cast<unsigned long long>(static_cast<long long>(S));
      } else {
        stage[lane] = cand ? Dsub(static_cast<double>(wt), a.offset) : 0.0;
        __syncwarp();
        if (slot != kNone) {
          double acc = __longlong_as_double(static_cast<long long>(vals[slot]));
          unsigned mm = peers;
          while (mm) {
            const int j = __ffs(mm) - 1;
            acc = Dadd(acc, stage[j]);
            mm &= mm - 1;
          }
          vals[slot] = static_cast<unsigned long long>(__double_as_longlong(acc));
        }
      }
      __syncwarp();
    }
    double T = 0.0;
    if (lane == 0) {
      const uint32_t slot = FindT<false>(keys, HC, x.c);
      if (slot != kNone) T = AsDouble<kInt>(vals[slot]);
    }
    T = __shfl_sync(kFull, T, 0);
    const double change = ChangeOf(a, x, T);
    const uint32_t nused = *used_count;
    double best = -CUDART_INF;
    uint32_t bid = kNone;
    for (uint32_t i = lane; i < nused; i += 32) {
      const uint32_t slot = used[i];
      const uint32_t key = keys[slot];
      const double S = AsDouble<kInt>(vals[slot]);
      const double val = ValOf(a, x.kv, change, S, LdK<kAsync>(a.K + key));
      if (Better(val, key, best, bid)) {
        best = val;
        bid = key;
      }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      const double ov = __shfl_xor_sync(kFull, best, o);
      const uint32_t oid = __shfl_xor_sync(kFull, bid, o);
      if (Better(ov, oid, best, bid)) {
        best = ov;
        bid = oid;
      }
    }
    __syncwarp();
    for (uint32_t i = lane; i < nused; i += 32) {
      const uint32_t slot = used[i];
      keys[slot] = kNone;
      vals[slot] = 0ull;
    }
    bool append = false;
    if (lane == 0) append = Decide<kAsync>(a, x, best, bid, change);
    if (!kAsync) {
      const uint32_t pos = WarpAppendFull(&a.ctr->movers, append);
      if (append) a.movers[pos] = x.v;
    }
    __syncwarp();
    if (lane == 0) *used_count = 0;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// One CTA per hub vertex (degree > 1000).  The hash lives in shared memory
// (kCtaHashSlots) or, for kGlobal, in a per-CTA region of global scratch
// that stays clean between vertices (only used slots are cleared).
// Warp-level pre-aggregation (match.any), then atomic adds into the table.
// FP64 mode follows the reference's hub path: w - offset rounded to float.
// ---------------------------------------------------------------------------
constexpr int kCtaThreads = 512;
constexpr size_t kCtaStage = size_t(kCtaThreads / 32) * 32 * 8;
constexpr size_t kCtaSmem = kCtaStage + size_t(kCtaHashSlots) * 12 + size_t(kCtaHashSlots / 2) * 2;

template <bool kInt, bool kGlobal, bool kAsync>
__global__ void __launch_bounds__(kCtaThreads) BestMoveCtaKernel(BMArgs a, const uint32_t* __restrict__ list,
                                                                const uint32_t* __restrict__ bin_counts,
                                                                const uint32_t* __restrict__ bin_starts, int bin) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red_val[kCtaThreads / 32];
  __shared__ uint32_t red_id[kCtaThreads / 32];
  __shared__ double sh_T;
  __shared__ uint32_t sh_used;
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  double* stage = reinterpret_cast<double*>(smem) + size_t(warp) * 32;
  using UsedT = typename std::conditional<kGlobal, uint32_t, uint16_t>::type;
  unsigned long long* vals;
  uint32_t* keys;
  UsedT* used;
  if (kGlobal) {
    vals = a.g_vals + size_t(blockIdx.x) * a.g_cap;
    keys = a.g_keys + size_t(blockIdx.x) * a.g_cap;
    used = reinterpret_cast<UsedT*>(a.g_used + size_t(blockIdx.x) * (a.g_cap / 2));
  } else {
    vals = reinterpret_cast<unsigned long long*>(smem + kCtaStage);
    keys = reinterpret_cast<uint32_t*>(smem + kCtaStage + size_t(kCtaHashSlots) * 8);
    used = reinterpret_cast<UsedT*>(smem + kCtaStage + size_t(kCtaHashSlots) * 12);
    for (uint32_t i = threadIdx.x; i < kCtaHashSlots; i += kCtaThreads) {
      keys[i] = kNone;
      vals[i] = 0ull;
    }
  }
  if (threadIdx.x == 0) sh_used = 0;
  __syncthreads();
  for (uint64_t idx = blockIdx.x; idx < count; idx += gridDim.x) {
    const VertexCtx x = LoadVertex<kAsync>(a, list[start + idx]);
    uint32_t cap = kCtaHashSlots;
    if (kGlobal) {
      cap = 1024;
      while (cap < 2ull * x.d + 2) cap <<= 1;
      if (cap > a.g_cap) {  // cannot happen: scratch is sized by the max degree
        if (threadIdx.x == 0) atomicExch(&a.ctr->error, kErrHashFull);
        continue;
      }
    }
    const uint32_t rounds = (x.d + kCtaThreads - 1) / kCtaThreads;
    for (uint32_t r = 0; r < rounds; ++r) {
      const uint32_t e = r * kCtaThreads + threadIdx.x;
      const bool has = e < x.d;
      uint32_t u = x.v;
      float wt = 0.f;
      if (has) {
        u = a.nbr[x.b + e];
        wt = a.w ? a.w[x.b + e] : 1.0f;
      }
      const bool cand = has && u != x.v;
      const uint32_t cu = cand ? LdC<kAsync>(a.C + u) : kNone;
      const unsigned long long key = cand ? cu : (0x100000000ull | lane);
      const unsigned peers = __match_any_sync(kFull, key);
      const bool leader = cand && int(lane) == __ffs(peers) - 1;
      uint32_t slot = kNone;
      if (leader) {
        bool ins = false;
        slot = FindOrInsertT<kGlobal>(keys, cap, cu, &ins);
        if (slot == kNone) {
          atomicExch(&a.ctr->error, kErrHashFull);
        } else if (ins) {
          used[atomicAdd(&sh_used, 1u)] = static_cast<UsedT>(slot);
        }
      }
      if (kInt) {
        const int xi = cand ? (static_cast<int>(wt) - a.ioffset) : 0;
        const int S = __reduce_add_sync(peers, xi);
        if (slot != kNone) atomicAdd(&vals[slot], static_cast<unsigned long long>(static_cast<long long>(S)));
      } else {
        // Hub path of the reference: `float weight; weight -= offset;`
        const float wf = static_cast<float>(Dsub(static_cast<double>(wt), a.offset));
        stage[lane] = cand ? static_cast<double>(wf) : 0.0;
        __syncwarp();
        if (slot != kNone) {
          double acc = 0.0;
          unsigned mm = peers;
          while (mm) {
            const int j = __ffs(mm) - 1;
            acc = Dadd(acc, stage[j]);
            mm &= mm - 1;
          }
          atomicAdd(reinterpret_cast<double*>(&vals[slot]), acc);
        }
        __syncwarp();
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t slot = FindT<kGlobal>(keys, cap, x.c);
      sh_T = slot != kNone ? AsDouble<kInt>(HVal<kGlobal>(vals, slot)) : 0.0;
    }
    __syncthreads();
    const double change = ChangeOf(a, x, sh_T);
    const uint32_t nused = sh_used;
    double best = -CUDART_INF;
    uint32_t bid = kNone;
    for (uint32_t i = threadIdx.x; i < nused; i += kCtaThreads) {
      const uint32_t slot = kGlobal ? __ldcg(reinterpret_cast<const uint32_t*>(used) + i) : uint32_t(used[i]);
      const uint32_t key = HKey<kGlobal>(keys, slot);
      const double S = AsDouble<kInt>(HVal<kGlobal>(vals, slot));
      const double val = ValOf(a, x.kv, change, S, LdK<kAsync>(a.K + key));
      if (Better(val, key, best, bid)) {
        best = val;
        bid = key;
      }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      const double ov = __shfl_xor_sync(kFull, best, o);
      const uint32_t oid = __shfl_xor_sync(kFull, bid, o);
      if (Better(ov, oid, best, bid)) {
        best = ov;
        bid = oid;
      }
    }
    if (lane == 0) {
      red_val[warp] = best;
      red_id[warp] = bid;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nused; i += kCtaThreads) {
      const uint32_t slot = kGlobal ? __ldcg(reinterpret_cast<const uint32_t*>(used) + i) : uint32_t(used[i]);
      keys[slot] = kNone;
      vals[slot] = 0ull;
    }
    if (threadIdx.x == 0) {
      for (int w = 1; w < kCtaThreads / 32; ++w) {
        if (Better(red_val[w], red_id[w], best, bid)) {
          best = red_val[w];
          bid = red_id[w];
        }
      }
      const bool append = Decide<kAsync>(a, x, best, bid, change);
      if (!kAsync && append) a.movers[atomicAdd(&a.ctr->movers, 1u)] = x.v;
      sh_used = 0;
    }
    __syncthreads();
  }
}

template <class K>
Status SetSmem(K kernel, size_t bytes) {
  PCC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
  return Status::Ok();
}

template <bool kInt, bool kAsync>
Status LaunchAll(Context* ctx, const BMArgs& a, const uint32_t* list, const uint32_t* counts,
                 const uint32_t* starts, const uint32_t* host_counts, uint32_t max_deg) {
  const unsigned sms = unsigned(ctx->num_sms);
  auto grid = [&](int bin, uint64_t per_block, unsigned cap) -> unsigned {
    if (!host_counts) return cap;
    return Blocks(host_counts[bin], unsigned(per_block), cap);
  };
  auto want = [&](int bin) { return !host_counts || host_counts[bin] > 0; };
  cudaStream_t st = ctx->stream;
  if (want(kBinG4))
    BestMoveGroupKernel<4, kInt, kAsync><<<grid(kBinG4, 64, sms * 8), 256, 0, st>>>(a, list, counts, starts, kBinG4); PCC_COUNT(1);
  if (want(kBinG8))
    BestMoveGroupKernel<8, kInt, kAsync><<<grid(kBinG8, 32, sms * 8), 256, 0, st>>>(a, list, counts, starts, kBinG8); PCC_COUNT(1);
  if (want(kBinG16))
    BestMoveGroupKernel<16, kInt, kAsync><<<grid(kBinG16, 16, sms * 8), 256, 0, st>>>(a, list, counts, starts, kBinG16); PCC_COUNT(1);
  if (want(kBinG32))
    BestMoveGroupKernel<32, kInt, kAsync><<<grid(kBinG32, 8, sms * 8), 256, 0, st>>>(a, list, counts, starts, kBinG32); PCC_COUNT(1);
  if (want(kBinW128)) {
    auto k = BestMoveWarpKernel<256, kInt, kAsync>;
    PCC_RETURN_IF_ERROR(SetSmem(k, WarpKernelSmem<256>()));
    k<<<grid(kBinW128, kWarpKernelWarps, sms * 8), kWarpKernelWarps * 32, WarpKernelSmem<256>(), st>>>(
        a, list, counts, starts, kBinW128); PCC_COUNT(1);
  }
  if (want(kBinW256)) {
    auto k = BestMoveWarpKernel<512, kInt, kAsync>;
    PCC_RETURN_IF_ERROR(SetSmem(k, WarpKernelSmem<512>()));
    k<<<grid(kBinW256, kWarpKernelWarps, sms * 8), kWarpKernelWarps * 32, WarpKernelSmem<512>(), st>>>(
        a, list, counts, starts, kBinW256); PCC_COUNT(1);
  }
  if (want(kBinW512)) {
    auto k = BestMoveWarpKernel<1024, kInt, kAsync>;
    PCC_RETURN_IF_ERROR(SetSmem(k, WarpKernelSmem<1024>()));
    k<<<grid(kBinW512, kWarpKernelWarps, sms * 4), kWarpKernelWarps * 32, WarpKernelSmem<1024>(), st>>>(
        a, list, counts, starts, kBinW512); PCC_COUNT(1);
  }
  if (want(kBinW1000)) {
    auto k = BestMoveWarpKernel<2048, kInt, kAsync>;
    PCC_RETURN_IF_ERROR(SetSmem(k, WarpKernelSmem<2048>()));
    k<<<grid(kBinW1000, kWarpKernelWarps, sms * 2), kWarpKernelWarps * 32, WarpKernelSmem<2048>(), st>>>(
        a, list, counts, starts, kBinW1000); PCC_COUNT(1);
  }
  if (want(kBinCta)) {
    auto k = BestMoveCtaKernel<kInt, false, kAsync>;
    PCC_RETURN_IF_ERROR(SetSmem(k, kCtaSmem));
    k<<<grid(kBinCta, 1, sms * 2), kCtaThreads, kCtaSmem, st>>>(a, list, counts, starts, kBinCta); PCC_COUNT(1);
  }
  if (want(kBinGlobal) && max_deg > kBinMaxDeg[kBinCta]) {
    auto k = BestMoveCtaKernel<kInt, true, kAsync>;
    k<<<grid(kBinGlobal, 1, sms * 2), kCtaThreads, kCtaStage, st>>>(a, list, counts, starts, kBinGlobal); PCC_COUNT(1);
  }
  return LaunchCheck();
}

}  // namespace

uint64_t GlobalHashSlots(Context* ctx, uint32_t max_deg) {
  // Per CTA: a table of the next power of two >= 2 * max degree; one CTA per
  // grid slot of the hub kernel (2 per SM).
  if (max_deg <= kBinMaxDeg[kBinCta]) return 0;
  uint64_t cap = 1024;
  while (cap < 2ull * max_deg + 2) cap <<= 1;
  return cap * uint64_t(ctx->num_sms) * 2;
}

Status LaunchBestMoves(Context* ctx, const BMArgs& a, const uint32_t* list, const uint32_t* bin_counts,
                       const uint32_t* bin_starts, const uint32_t* host_counts, bool int_mode,
                       uint32_t max_deg) {
  if (a.async) {
    return int_mode ? LaunchAll<true, true>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg)
                    : LaunchAll<false, true>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg);
  }
  return int_mode ? LaunchAll<true, false>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg)
                  : LaunchAll<false, false>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg);
}

}  // namespace pcc
