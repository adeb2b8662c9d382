// hubs.cu -- best moves of hub vertices (degree > 1000); the scheme is in
// hubs.cuh.  Restates the hub branch of ClusteringHelper::EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:516-582): per-cluster sums in
// any order (the reference adds concurrently), FP64-mode weights rounded to
// float after the offset, the argmax by (value desc, id asc), and "no
// entries" giving the reduce identity (0, 0.0) unless change >= 0.
#include <cooperative_groups.h>

#include <algorithm>
#include <numeric>
#include <type_traits>
#include <vector>

#include "certify.cuh"
#include "hubs.cuh"
#include "moves.cuh"

namespace cg = cooperative_groups;

namespace pcc {
namespace {

constexpr int kHT = 256;                   // threads per hub CTA
constexpr int kHW = kHT / 32;
constexpr int kHubUnroll = 4;              // entries per thread in flight
constexpr uint32_t kHubMaxSub = 1u << 12;  // sub-partitions before giving up
constexpr uint32_t kMaxCont = 256;         // contender list per CTA

struct HubArgs {
  BMArgs a;
  const uint32_t* small_v;
  uint32_t num_small;
  const uint32_t* big_v;
  const uint32_t* big_parts;
  const uint32_t* big_pbase;
  const uint32_t* item_hub;
  const uint32_t* item_part;
  uint32_t num_items;
  double* part_val;
  uint32_t* part_id;
  uint32_t* done;
};

// MurmurHash3's 32-bit finalizer (a bijection; every output bit depends on
// every input bit).  Low bits pick the slot, bits 13..15 the owning CTA of a
// cluster, bits 16.. the sub-partition, the top bits the partition.
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

// Value types of the tables: int (narrow INT sums), long long (INT sums),
// double (FP64 sums).
template <typename V>
__device__ __forceinline__ V AtomicAddV(V* p, V x) {
  if constexpr (std::is_same<V, int>::value) {
    return atomicAdd(p, x);
  } else if constexpr (std::is_same<V, long long>::value) {
    return static_cast<long long>(atomicAdd(reinterpret_cast<unsigned long long*>(p),
                                            static_cast<unsigned long long>(x)));
  } else {
    return atomicAdd(p, x);
  }
}

template <typename V>
__device__ __forceinline__ double VToDouble(V x) {
  return static_cast<double>(x);
}

// Block reductions; every thread receives the result.
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

__device__ __forceinline__ LexKey BlockLex(LexKey x, long long* rs, unsigned long long* rk, uint32_t* ri) {
  LexGroupReduce<32>(x);
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

// Finds or inserts `key` (local or distributed shared memory), probing from
// `start`; kNone when the table is full.
__device__ __forceinline__ uint32_t HubInsert(uint32_t* keys, uint32_t cap, uint32_t start, uint32_t key,
                                              bool* ins) {
  const uint32_t mask = cap - 1;
  uint32_t s = start & mask;
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

// Shared scratch of a hub CTA besides its table.
struct HubShared {
  long long red_ll[kHW];
  unsigned long long red_k[kHW];
  double red_d[kHW];
  float red_f[kHW];
  uint32_t red_i[kHW];
  int stage_i[kHW][32];
  double stage_d[kHW][32];
  uint32_t cont_key[kMaxCont];
  long long cont_S[kMaxCont];
  uint32_t ncont;
  double change;
  float change32;
  // Cluster exchange (big hubs); flags and key counts double-buffered by
  // sub-pass parity.
  long long xT;
  double xTd;
  long long xsmax;
  uint32_t flags[2];
  uint32_t nkeys[2];
};

// Entry contribution w - offset: integer in INT mode, the reference hub
// path's float-rounded value in FP64 mode.
template <bool kInt>
__device__ __forceinline__ void EntryWeight(const BMArgs& a, float wt, int* xi, double* xd) {
  if (kInt) {
    *xi = static_cast<int>(wt) - a.ioffset;
  } else {
    *xd = static_cast<double>(static_cast<float>(Dsub(static_cast<double>(wt), a.offset)));
  }
}

// Evaluates this CTA's table: returns (to every thread) the best (exact FP64
// value, id) of its keys and clears the table.  INT sync mode: FP32
// pre-filter, then FP64 only for the survivors outside the leading (S, K)
// class, whose members share one FP64 value (evaluated once).
template <bool kInt, bool kAsync, typename V>
__device__ void EvalTable(const BMArgs& a, const VertexCtx& x, float k32, double change, long long smax,
                          uint32_t* skeys, V* svals, uint32_t cap, HubShared& sh, double* out_v, uint32_t* out_id) {
  const unsigned tid = threadIdx.x;
  constexpr bool kFilter = kInt && !kAsync;
  double lv = 0.0;
  uint32_t lid = kNone;
  if (kFilter) {
    const float c32 = sh.change32;
    float U = -CUDART_INF_F;
    for (uint32_t s = tid; s < cap; s += kHT) {
      const uint32_t key = skeys[s];
      if (key == kNone) continue;
      const FilterVal f = FilterOf(a.res32, k32, a.Kf[key], static_cast<long long>(svals[s]), smax, c32);
      if (f.sane) U = fmaxf(U, __fsub_rn(f.Y, f.e));
    }
    if (tid == 0) sh.ncont = 0;
    U = BlockMaxF(U, sh.red_f);
    LexKey lead, tail;
    for (uint32_t s = tid; s < cap; s += kHT) {
      const uint32_t key = skeys[s];
      if (key == kNone) continue;
      const long long S = static_cast<long long>(svals[s]);
      skeys[s] = kNone;
      svals[s] = V(0);
      const FilterVal f = FilterOf(a.res32, k32, a.Kf[key], S, smax, c32);
      if (f.sane && __fadd_rn(f.Y, f.e) < U) continue;
      const double KD = a.K[key];
      const unsigned long long ko = KOrder(KD);
      lead.Keep(S, ko, key);
      tail.Keep(-S, ~ko, key);
      const uint32_t pos = atomicAdd(&sh.ncont, 1u);
      if (pos < kMaxCont) {
        sh.cont_key[pos] = key;
        sh.cont_S[pos] = S;
      } else {
        KeepBest(lv, lid, ValOf(a, x.kv, change, static_cast<double>(S), KD), key);  // list full: now
      }
    }
    lead = BlockLex(lead, sh.red_ll, sh.red_k, sh.red_i);
    tail = BlockLex(tail, sh.red_ll, sh.red_k, sh.red_i);
    const uint32_t nc = min(sh.ncont, kMaxCont);
    const bool single = lead.id == kNone || (-tail.S == lead.S && ~tail.K == lead.K);
    if (!single) {
      for (uint32_t i = tid; i < nc; i += kHT) {
        const uint32_t key = sh.cont_key[i];
        const long long S = sh.cont_S[i];
        const double KD = a.K[key];
        if (S == lead.S && KOrder(KD) == lead.K) continue;  // the leading class
        KeepBest(lv, lid, ValOf(a, x.kv, change, static_cast<double>(S), KD), key);
      }
    }
    if (tid == 0 && lead.id != kNone)
      KeepBest(lv, lid, ValOf(a, x.kv, change, static_cast<double>(lead.S), a.K[lead.id]), lead.id);
  } else {
    for (uint32_t s = tid; s < cap; s += kHT) {
      const uint32_t key = skeys[s];
      if (key == kNone) continue;
      const V sv = svals[s];
      skeys[s] = kNone;
      svals[s] = V(0);
      KeepBest(lv, lid, ValOf(a, x.kv, change, VToDouble(sv), LdK<kAsync>(a.K + key)), key);
    }
  }
  BlockArgmax(lv, lid, sh.red_d, sh.red_i);
  *out_v = lv;
  *out_id = lid;
}

// Warp-aggregated sum of the entry weights of each match group.
template <bool kInt>
__device__ __forceinline__ void GroupWeights(const BMArgs& a, unsigned peers, bool leader, int xi, double xd,
                                             HubShared& sh, int* Si, double* Sd) {
  const unsigned warp = threadIdx.x >> 5, lane = LaneId();
  if (kInt) {
    *Si = GroupSumInt(peers, xi, a.w == nullptr, leader, sh.stage_i[warp]);
  } else {
    sh.stage_d[warp][lane] = xd;
    __syncwarp();
    double acc = 0.0;
    if (leader) {
      unsigned mm = peers;
      while (mm) {
        acc = Dadd(acc, sh.stage_d[warp][__ffs(mm) - 1]);
        mm &= mm - 1;
      }
    }
    __syncwarp();
    *Sd = acc;
  }
}

template <bool kAsync>
__device__ __forceinline__ void HubDecide(const BMArgs& a, const VertexCtx& x, double bv, uint32_t bi,
                                          double change) {
  if (bi == kNone) {  // no entries: the reduce identity (0, 0.0)
    bv = 0.0;
    bi = 0;
  }
  const bool append = Decide<kAsync>(a, x, bv, bi, change);
  if (!kAsync && append) a.movers[atomicAdd(&a.ctr->movers, 1u)] = x.v;
}

// ---------------------------------------------------------------------------
// Small hubs: one CTA per hub, a table of nextpow2(2 * degree + 2) slots.
// ---------------------------------------------------------------------------
template <bool kInt, bool kAsync, typename V>
__global__ void __launch_bounds__(kHT) HubSmallKernel(HubArgs h) {
  extern __shared__ __align__(16) unsigned char smem[];
  V* svals = reinterpret_cast<V*>(smem);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem + size_t(kHubSlots) * sizeof(V));
  __shared__ HubShared sh;
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x, lane = LaneId();
  for (uint32_t i = tid; i < kHubSlots; i += kHT) {
    skeys[i] = kNone;
    svals[i] = V(0);
  }
  __syncthreads();
  for (uint32_t item = blockIdx.x; item < h.num_small; item += gridDim.x) {
    const uint32_t v = h.small_v[item];
    if (!InFront(a, v)) continue;  // uniform over the CTA
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    uint32_t cap = 256;
    while (cap < 2 * x.d + 2 && cap < kHubSlots) cap <<= 1;
    long long t_int = 0, smax = LLONG_MIN;
    double t_dbl = 0.0;
    for (uint32_t e0 = 0; e0 < x.d; e0 += kHT * kHubUnroll) {
      uint32_t uu[kHubUnroll], cc[kHubUnroll];
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
#pragma unroll
      for (int k = 0; k < kHubUnroll; ++k) cc[k] = uu[k] != v ? LdC<kAsync>(a.C + uu[k]) : kNone;
#pragma unroll
      for (int k = 0; k < kHubUnroll; ++k) {
        const bool cand = uu[k] != v;
        const uint32_t cu = cc[k];
        int xi = 0;
        double xd = 0.0;
        if (cand) EntryWeight<kInt>(a, ww[k], &xi, &xd);
        if (cand && cu == x.c) {
          if (kInt)
            t_int += xi;
          else
            t_dbl = Dadd(t_dbl, xd);
        }
        const unsigned peers = __match_any_sync(kFull, cand ? cu : LaneSentinel(lane));
        const bool leader = cand && int(lane) == __ffs(peers) - 1;
        int Si = 0;
        double Sd = 0.0;
        GroupWeights<kInt>(a, peers, leader, xi, xd, sh, &Si, &Sd);
        if (leader) {
          bool ins;
          const uint32_t slot = HubInsert(skeys, cap, Mix32(cu), cu, &ins);
          if (slot == kNone) {
            atomicExch(&a.ctr->error, kErrHashFull);
          } else if (kInt) {
            const V old = AtomicAddV<V>(svals + slot, static_cast<V>(Si));
            smax = max(smax, static_cast<long long>(old) + Si);
          } else {
            AtomicAddV<V>(svals + slot, static_cast<V>(Sd));
          }
        }
      }
    }
    __syncthreads();
    double T;
    if (kInt) {
      T = static_cast<double>(BlockSum<long long>(t_int, sh.red_ll));
      smax = BlockMaxLL(smax, sh.red_ll);
    } else {
      T = BlockSum<double>(t_dbl, sh.red_d);
    }
    if (tid == 0) {
      sh.change = ChangeOf(a, x, T);  // FP64 once per CTA
      sh.change32 = static_cast<float>(sh.change);
    }
    __syncthreads();
    const double change = sh.change;
    double bv;
    uint32_t bi;
    EvalTable<kInt, kAsync, V>(a, x, a.kf[v], change, smax, skeys, svals, cap, sh, &bv, &bi);
    if (tid == 0) HubDecide<kAsync>(a, x, bv, bi, change);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Big hubs: a cluster of kCS CTAs per (hub, partition) sharing one
// distributed table.  All control flow between cluster barriers is uniform
// over the cluster (it depends on the item and on values every CTA reads
// after a barrier), so every CTA reaches every cluster.sync().  kCS = 1 (no
// distributed shared memory) serves the 64-bit and FP64 sums, which keep
// their atomics local; the overflow sub-passes then split the partitions.
// ---------------------------------------------------------------------------
template <unsigned kCS, typename T>
__device__ __forceinline__ T* Owner(cg::cluster_group& cluster, T* p, unsigned r) {
  if constexpr (kCS == 1) {
    return p;
  } else {
    return cluster.map_shared_rank(p, r);
  }
}

template <unsigned kCS>
__device__ __forceinline__ void ClusterSync(cg::cluster_group& cluster) {
  if constexpr (kCS == 1) {
    __syncthreads();
  } else {
    cluster.sync();
  }
}

template <bool kInt, bool kAsync, typename V, unsigned kCS>
__global__ void __cluster_dims__(kCS, 1, 1) __launch_bounds__(kHT) HubClusterKernel(HubArgs h) {
  extern __shared__ __align__(16) unsigned char smem[];
  V* svals = reinterpret_cast<V*>(smem);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem + size_t(kHubSlots) * sizeof(V));
  __shared__ HubShared sh;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = kCS == 1 ? 0u : cluster.block_rank();
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x, lane = LaneId();
  for (uint32_t i = tid; i < kHubSlots; i += kHT) {
    skeys[i] = kNone;
    svals[i] = V(0);
  }
  if (tid == 0) {
    sh.flags[0] = sh.flags[1] = 0;
    sh.nkeys[0] = sh.nkeys[1] = 0;
  }
  ClusterSync<kCS>(cluster);  // every table is initialised before any remote insert
  const uint32_t cid = blockIdx.x / kCS, ncl = gridDim.x / kCS;
  unsigned parity = 0;
  for (uint32_t item = cid; item < h.num_items; item += ncl) {
    const uint32_t hb = h.item_hub[item];
    const uint32_t p = h.item_part[item];
    const uint32_t v = h.big_v[hb];
    if (!InFront(a, v)) continue;  // uniform over the cluster
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    const uint32_t P = h.big_parts[hb];
    const uint32_t per_cta = (x.d + P * kCS - 1) / (P * kCS);
    uint32_t cap = 256;
    while (cap < 2 * per_cta + 2 && cap < kHubSlots) cap <<= 1;
    const uint32_t maxkeys = cap - cap / 4;
    const uint32_t seg = (x.d + kCS - 1) / kCS;
    const uint32_t e_lo = min(x.d, rank * seg), e_hi = min(x.d, e_lo + seg);
    uint32_t Q = 1, q = 0;
    bool have_T = false;
    double change = 0.0;
    double bestv = 0.0;
    uint32_t bestid = kNone;
    while (true) {
      long long t_int = 0, smax = LLONG_MIN;
      double t_dbl = 0.0;
      for (uint32_t e0 = e_lo; e0 < e_hi; e0 += kHT * kHubUnroll) {
        uint32_t uu[kHubUnroll], cc[kHubUnroll];
        float ww[kHubUnroll];
#pragma unroll
        for (int k = 0; k < kHubUnroll; ++k) {
          const uint32_t e = e0 + k * kHT + tid;
          uu[k] = v;
          ww[k] = 0.f;
          if (e < e_hi) {
            uu[k] = a.nbr[x.b + e];
            ww[k] = a.w ? a.w[x.b + e] : 1.0f;
          }
        }
#pragma unroll
        for (int k = 0; k < kHubUnroll; ++k) cc[k] = uu[k] != v ? LdC<kAsync>(a.C + uu[k]) : kNone;
#pragma unroll
        for (int k = 0; k < kHubUnroll; ++k) {
          const bool cand = uu[k] != v;
          const uint32_t cu = cc[k];
          int xi = 0;
          double xd = 0.0;
          if (cand) EntryWeight<kInt>(a, ww[k], &xi, &xd);
          if (!have_T && cand && cu == x.c) {
            if (kInt)
              t_int += xi;
            else
              t_dbl = Dadd(t_dbl, xd);
          }
          const uint32_t hsh = Mix32(cu);
          const bool mine = cand && __umulhi(hsh, P) == p && ((hsh >> 16) & (Q - 1)) == q;
          const unsigned peers = __match_any_sync(kFull, mine ? cu : LaneSentinel(lane));
          const bool leader = mine && int(lane) == __ffs(peers) - 1;
          int Si = 0;
          double Sd = 0.0;
          GroupWeights<kInt>(a, peers, leader, xi, xd, sh, &Si, &Sd);
          if (leader) {
            const unsigned owner = (hsh >> 13) & (kCS - 1);
            uint32_t* rkeys = Owner<kCS>(cluster, skeys, owner);
            V* rvals = Owner<kCS>(cluster, svals, owner);
            HubShared* rsh = Owner<kCS>(cluster, &sh, owner);
            bool ins;
            const uint32_t slot = HubInsert(rkeys, cap, hsh, cu, &ins);
            if (slot == kNone) {
              atomicExch(&rsh->flags[parity], 1u);
            } else {
              if (ins && atomicAdd(&rsh->nkeys[parity], 1u) + 1 > maxkeys) atomicExch(&rsh->flags[parity], 1u);
              if (kInt) {
                const V old = AtomicAddV<V>(rvals + slot, static_cast<V>(Si));
                smax = max(smax, static_cast<long long>(old) + Si);
              } else {
                AtomicAddV<V>(rvals + slot, static_cast<V>(Sd));
              }
            }
          }
        }
      }
      // Per-CTA partials of "together" and of the largest sum, then the
      // cluster barrier that also publishes every remote insert.
      if (!have_T) {
        if (kInt) {
          const long long t = BlockSum<long long>(t_int, sh.red_ll);
          if (tid == 0) sh.xT = t;
        } else {
          const double t = BlockSum<double>(t_dbl, sh.red_d);
          if (tid == 0) sh.xTd = t;
        }
      }
      if (kInt) {
        const long long m = BlockMaxLL(smax, sh.red_ll);
        if (tid == 0) sh.xsmax = m;
      }
      ClusterSync<kCS>(cluster);  // (1) tables, partials and flags complete
      bool overflow = false;
      long long csmax = LLONG_MIN;
      for (unsigned r = 0; r < kCS; ++r) {
        const HubShared* rsh = Owner<kCS>(cluster, &sh, r);
        overflow = overflow || (*reinterpret_cast<const volatile uint32_t*>(&rsh->flags[parity]) != 0);
        if (kInt) csmax = max(csmax, rsh->xsmax);
      }
      if (!have_T) {
        double T;
        if (kInt) {
          long long t = 0;
          for (unsigned r = 0; r < kCS; ++r) t += Owner<kCS>(cluster, &sh, r)->xT;
          T = static_cast<double>(t);
        } else {
          T = 0.0;
          for (unsigned r = 0; r < kCS; ++r) T = Dadd(T, Owner<kCS>(cluster, &sh, r)->xTd);
        }
        if (tid == 0) {
          sh.change = ChangeOf(a, x, T);  // FP64 once per CTA
          sh.change32 = static_cast<float>(sh.change);
        }
        __syncthreads();
        change = sh.change;
        have_T = true;
      }
      // The next sub-pass uses the other parity; reset it here (it was last
      // read before the previous cluster barrier).
      if (tid == 0) {
        sh.flags[parity ^ 1] = 0;
        sh.nkeys[parity ^ 1] = 0;
      }
      if (overflow) {
        for (uint32_t s = tid; s < cap; s += kHT) {
          skeys[s] = kNone;
          svals[s] = V(0);
        }
        Q *= 2;
        q = 0;
        bestv = 0.0;
        bestid = kNone;
        ClusterSync<kCS>(cluster);  // (2) cleared before the rescan's inserts
        parity ^= 1;
        if (Q > kHubMaxSub) {
          if (tid == 0) atomicExch(&a.ctr->error, kErrHashFull);
          break;
        }
        continue;
      }
      double lv;
      uint32_t lid;
      EvalTable<kInt, kAsync, V>(a, x, a.kf[v], change, csmax, skeys, svals, cap, sh, &lv, &lid);
      KeepBest(bestv, bestid, lv, lid);
      ClusterSync<kCS>(cluster);  // (2) every table cleared before the next inserts
      parity ^= 1;
      if (++q == Q) break;
    }
    // Partial result; the hub's last CTA combines and decides.
    if (tid == 0) {
      const uint32_t pb = h.big_pbase[hb] + p * kCS + rank;
      h.part_val[pb] = bestv;
      h.part_id[pb] = bestid;
      __threadfence();
      const uint32_t total = P * kCS;
      if (atomicAdd(&h.done[hb], 1u) == total - 1) {
        __threadfence();
        double bv = 0.0;
        uint32_t bi = kNone;
        const uint32_t b0 = h.big_pbase[hb];
        for (uint32_t j = 0; j < total; ++j) KeepBest(bv, bi, __ldcg(h.part_val + b0 + j), __ldcg(h.part_id + b0 + j));
        h.done[hb] = 0;
        HubDecide<kAsync>(a, x, bv, bi, change);
      }
    }
  }
  ClusterSync<kCS>(cluster);  // no CTA leaves while its table may still be read
}

__global__ void HubDegreesKernel(const uint32_t* list, uint32_t count, const uint64_t* off, uint32_t* deg) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    deg[i] = static_cast<uint32_t>(off[list[i] + 1] - off[list[i]]);
}

template <bool kInt, bool kAsync, typename V>
Status LaunchHubT(Context* ctx, const HubArgs& h) {
  constexpr size_t smem = size_t(kHubSlots) * (sizeof(V) + sizeof(uint32_t));
  // Distributed tables only with 32-bit sums (32-bit remote atomics).
  constexpr unsigned kCS = std::is_same<V, int>::value ? kHubClusterSize : 1u;
  const unsigned sms = unsigned(ctx->num_sms);
  if (h.num_small) {
    auto k = HubSmallKernel<kInt, kAsync, V>;
    PCC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    PCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kHT, smem));
    const unsigned grid = Blocks(h.num_small, 1, sms * unsigned(std::max(per_sm, 1)));
    k<<<grid, kHT, smem, ctx->stream>>>(h);
    PCC_COUNT(1);
  }
  if (h.num_items) {
    auto k = HubClusterKernel<kInt, kAsync, V, kCS>;
    PCC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int max_clusters = 0;
    if (kCS > 1) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kCS * sms, 1, 1);
      cfg.blockDim = dim3(kHT, 1, 1);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = ctx->stream;
      if (cudaOccupancyMaxActiveClusters(&max_clusters, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        max_clusters = 0;
      }
      if (max_clusters < 1) max_clusters = int(sms / kCS);
    } else {
      int per_sm = 0;
      PCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kHT, smem));
      max_clusters = int(sms) * std::max(per_sm, 1);
    }
    const unsigned clusters = std::min<unsigned>(h.num_items, unsigned(std::max(max_clusters, 1)));
    k<<<clusters * kCS, kHT, smem, ctx->stream>>>(h);
    PCC_COUNT(1);
  }
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
  // Largest hubs first (the longest work items start first); a big hub's
  // partitions are consecutive items, so they run at the same time and share
  // the row through L2.
  std::vector<uint32_t> order(count);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t i, uint32_t j) { return hd[i] > hd[j]; });
  std::vector<uint32_t> small_v, big_v, parts, pbase, item_hub, item_part;
  uint64_t total = 0;
  for (uint32_t r = 0; r < count; ++r) {
    const uint32_t i = order[r];
    if (hd[i] <= kHubSmallMax) {
      small_v.push_back(hv[i]);
      continue;
    }
    const uint32_t P = std::max<uint32_t>(1, (hd[i] + kHubClusterKeys - 1) / kHubClusterKeys);
    const uint32_t hb = static_cast<uint32_t>(big_v.size());
    big_v.push_back(hv[i]);
    parts.push_back(P);
    pbase.push_back(static_cast<uint32_t>(total));
    total += uint64_t(P) * kHubClusterSize;
    for (uint32_t p = 0; p < P; ++p) {
      item_hub.push_back(hb);
      item_part.push_back(p);
    }
  }
  if (total > 0xFFFFFFFFull) return MakeError(PCC_OUT_OF_RANGE, "too many hub partitions");
  plan->num_small = static_cast<uint32_t>(small_v.size());
  plan->num_big = static_cast<uint32_t>(big_v.size());
  plan->num_items = static_cast<uint32_t>(item_hub.size());
  plan->num_partials = total;
  auto up = [&](DBuf<uint32_t>& d, const std::vector<uint32_t>& hvec) -> Status {
    if (hvec.empty()) return Status::Ok();
    PCC_RETURN_IF_ERROR(d.Alloc(ctx, hvec.size()));
    return d.FromHost(hvec.data(), hvec.size());
  };
  PCC_RETURN_IF_ERROR(up(plan->small_v, small_v));
  PCC_RETURN_IF_ERROR(up(plan->big_v, big_v));
  PCC_RETURN_IF_ERROR(up(plan->big_parts, parts));
  PCC_RETURN_IF_ERROR(up(plan->big_pbase, pbase));
  PCC_RETURN_IF_ERROR(up(plan->item_hub, item_hub));
  PCC_RETURN_IF_ERROR(up(plan->item_part, item_part));
  return Sync(ctx);  // host vectors go out of scope
}

Status AllocHubState(Context* ctx, const HubPlan& plan, HubState* st) {
  const uint64_t np = std::max<uint64_t>(plan.num_partials, 1);
  if (st->part_val.count < np) {
    PCC_RETURN_IF_ERROR(st->part_val.Alloc(ctx, np));
    PCC_RETURN_IF_ERROR(st->part_id.Alloc(ctx, np));
  }
  const uint64_t nh = std::max<uint32_t>(plan.num_big, 1);
  if (st->done.count < nh) PCC_RETURN_IF_ERROR(st->done.Alloc(ctx, nh));
  return st->done.Zero();
}

Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode,
                          bool narrow) {
  if (plan.num_hubs == 0) return Status::Ok();
  HubArgs h;
  h.a = a;
  h.small_v = plan.small_v.p;
  h.num_small = plan.num_small;
  h.big_v = plan.big_v.p;
  h.big_parts = plan.big_parts.p;
  h.big_pbase = plan.big_pbase.p;
  h.item_hub = plan.item_hub.p;
  h.item_part = plan.item_part.p;
  h.num_items = plan.num_items;
  h.part_val = st.part_val.p;
  h.part_id = st.part_id.p;
  h.done = st.done.p;
  if (a.async) {
    if (!int_mode) return LaunchHubT<false, true, double>(ctx, h);
    return narrow ? LaunchHubT<true, true, int>(ctx, h) : LaunchHubT<true, true, long long>(ctx, h);
  }
  if (!int_mode) return LaunchHubT<false, false, double>(ctx, h);
  return narrow ? LaunchHubT<true, false, int>(ctx, h) : LaunchHubT<true, false, long long>(ctx, h);
}

}  // namespace pcc
