// hubs.cu -- best moves of hub vertices (degree > 1000); the scheme is in
// hubs.cuh.  Restates the hub branch of ClusteringHelper::EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:516-582): per-cluster sums in
// any order (the reference adds concurrently), FP64-mode weights rounded to
// float after the offset, the argmax by (value desc, id asc), and "no
// entries" giving the reduce identity (0, 0.0) unless change >= 0.
#include <algorithm>
#include <mutex>
#include <numeric>
#include <unordered_map>
#include <type_traits>
#include <vector>

#include "certify.cuh"
#include "hubs.cuh"
#include "moves.cuh"

namespace pcc {
namespace {

constexpr int kHubUnroll = 4;              // entries per thread in flight
constexpr uint32_t kHubMaxSub = 1u << 12;  // sub-partitions before giving up
constexpr uint32_t kMaxCont = 256;         // contender list per CTA
constexpr int kEvalBatch = 4;              // table slots per thread in flight (EvalTable)

constexpr int kSmallThreads = 256;         // small hubs: CTA size, table slots
constexpr uint32_t kSmallSlots = 2 * kHubSmallMax;
constexpr uint32_t kSmallMidSlots = 3 * kHubSmallMax / 2;  // hubs with 2d + 2 <= kSmallMidSlots
constexpr uint32_t kSmallNarrowSlots = kHubSmallMax;  // hubs with 2d + 2 <= kSmallNarrowSlots
constexpr int kBigThreads = 1024;          // big hubs
// Big-hub table: ~192 KB of (key, sum) slots.
template <typename V>
__host__ __device__ constexpr uint32_t BigSlots() {
  return sizeof(V) == 4 ? 2 * kHubBigKeys : 16384;
}

struct HubArgs {
  BMArgs a;
  const uint32_t* small_v;
  uint32_t small_lo, small_hi;  // this launch's items of small_v
  const uint32_t* big_v;
  const uint32_t* big_parts;
  const uint32_t* big_pbase;
  const uint32_t* item_hub;
  const uint32_t* item_part;
  uint32_t num_items;
  double* part_val;
  uint32_t* part_id;
  uint32_t* done;
  // Global path (sync): tables, accumulators, plan (num_glob 0: none).
  uint32_t num_glob;
  uint32_t num_glob_items;
  const uint32_t* glob_hub;
  const unsigned long long* glob_base;
  const uint32_t* glob_cap;
  const uint32_t* glob_item;
  const uint32_t* glob_item_start;
  const uint32_t* big_glob;
  uint32_t* gkeys;
  unsigned long long* gvals;
  long long* gt_int;
  double* gt_dbl;
  long long* gsmax;
  uint32_t num_glob_slices;
  const uint32_t* glob_nslices;
  const uint32_t* glob_sbase;
  const uint32_t* slice_hub;
  const uint32_t* slice_start;
  double* gpart_val;
  uint32_t* gpart_id;
  uint32_t* gdone;
};

// MurmurHash3's 32-bit finalizer (a bijection; every output bit depends on
// every input bit).  The product with the capacity's high half picks the
// slot, bits 8..19 the sub-partition, the top bits (again through a
// product) the partition.
__device__ __forceinline__ uint32_t Mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ uint32_t SlotHash(uint32_t cu) {
  // A second mix so that the slot is independent of the partition bits.
  return Mix32(cu ^ 0x9E3779B9u);
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

// Shared scratch of a hub CTA of BT threads besides its table.  The
// reduction arrays hold one partial per warp; their last element carries a
// result that warp 0 publishes (wide CTAs, HubChangeSmax).
template <int BT>
struct HubShared {
  static constexpr int kW = BT / 32;
  long long red_ll[kW + 1];
  long long red_mx[kW + 1];
  unsigned long long red_k[kW + 1];
  double red_d[kW];
  float red_f[kW + 1];
  uint32_t red_i[kW + 1];
  int stage_i[kW][32];
  double stage_d[kW][32];
  uint32_t cont_key[kMaxCont];
  long long cont_S[kMaxCont];
  uint32_t ncont;
  uint32_t overflow;
  uint32_t nkeys;
  uint32_t last;  // global path: this CTA evaluated the hub's last slice
  double change;
  float change32;
};

// Block reductions; every thread receives the result.  In wide CTAs (512
// threads and more) warp 0 combines the warps' partials and publishes the
// result in red[BT / 32], so that the other threads read one value instead
// of BT / 32; the combines here (max, integer sum, lexicographic and
// (value, id) selections) give the same result in any order.
template <int BT>
constexpr bool kWideBlock = BT >= 512;

template <int BT>
__device__ __forceinline__ long long BlockMaxLL(long long x, long long* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x = max(x, __shfl_xor_sync(kFull, x, o));
  if (LaneId() == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if constexpr (kWideBlock<BT>) {
    if (threadIdx.x < 32) {
      long long r = threadIdx.x < BT / 32 ? red[threadIdx.x] : LLONG_MIN;
#pragma unroll
      for (int o = 16; o; o >>= 1) r = max(r, __shfl_xor_sync(kFull, r, o));
      if (threadIdx.x == 0) red[BT / 32] = r;
    }
    __syncthreads();
    return red[BT / 32];
  }
  long long r = red[0];
#pragma unroll
  for (int w = 1; w < BT / 32; ++w) r = max(r, red[w]);
  __syncthreads();
  return r;
}

template <int BT>
__device__ __forceinline__ float BlockMaxF(float x, float* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x = fmaxf(x, __shfl_xor_sync(kFull, x, o));
  if (LaneId() == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if constexpr (kWideBlock<BT>) {
    if (threadIdx.x < 32) {
      float r = threadIdx.x < BT / 32 ? red[threadIdx.x] : -CUDART_INF_F;
#pragma unroll
      for (int o = 16; o; o >>= 1) r = fmaxf(r, __shfl_xor_sync(kFull, r, o));
      if (threadIdx.x == 0) red[BT / 32] = r;
    }
    __syncthreads();
    return red[BT / 32];
  }
  float r = red[0];
#pragma unroll
  for (int w = 1; w < BT / 32; ++w) r = fmaxf(r, red[w]);
  __syncthreads();
  return r;
}

// Deterministic sum: butterfly inside warps, then the warps in order.
template <int BT, class T>
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
  if constexpr (kWideBlock<BT> && std::is_integral<T>::value) {
    if (threadIdx.x < 32) {
      T r = threadIdx.x < BT / 32 ? red[threadIdx.x] : T(0);
#pragma unroll
      for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(kFull, r, o);
      if (threadIdx.x == 0) red[BT / 32] = r;
    }
    __syncthreads();
    return red[BT / 32];
  }
  T r = red[0];
#pragma unroll
  for (int w = 1; w < BT / 32; ++w) {
    if constexpr (std::is_floating_point<T>::value) {
      r = Dadd(r, red[w]);
    } else {
      r += red[w];
    }
  }
  __syncthreads();
  return r;
}

// Argmax over (value desc, id asc) with integer compares: the values are
// mapped to order-preserving 64-bit images (no FP64 instruction; the values
// here are never -0, the only case where the image order and IEEE equality
// differ).
__device__ __forceinline__ unsigned long long ValBits(double d) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double BitsVal(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double(static_cast<long long>(b));
}
__device__ __forceinline__ void KeepBits(unsigned long long& bo, uint32_t& bi, unsigned long long o, uint32_t i) {
  if (i == kNone) return;
  if (bi == kNone || o > bo || (o == bo && i < bi)) {
    bo = o;
    bi = i;
  }
}

template <int BT>
__device__ __forceinline__ void BlockArgmax(double& v, uint32_t& id, unsigned long long* redv, uint32_t* redi) {
  unsigned long long o = ValBits(v);
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const unsigned long long oo = __shfl_xor_sync(kFull, o, off);
    const uint32_t oi = __shfl_xor_sync(kFull, id, off);
    KeepBits(o, id, oo, oi);
  }
  if (LaneId() == 0) {
    redv[threadIdx.x >> 5] = o;
    redi[threadIdx.x >> 5] = id;
  }
  __syncthreads();
  if constexpr (kWideBlock<BT>) {
    if (threadIdx.x < 32) {
      const bool in = threadIdx.x < BT / 32;
      unsigned long long wo = redv[in ? threadIdx.x : 0];
      uint32_t wi = in ? redi[threadIdx.x] : kNone;
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const unsigned long long oo = __shfl_xor_sync(kFull, wo, off);
        const uint32_t oi = __shfl_xor_sync(kFull, wi, off);
        KeepBits(wo, wi, oo, oi);
      }
      if (threadIdx.x == 0) {
        redv[BT / 32] = wo;
        redi[BT / 32] = wi;
      }
    }
    __syncthreads();
    v = BitsVal(redv[BT / 32]);
    id = redi[BT / 32];
    return;
  }
  unsigned long long ro = redv[0];
  uint32_t ri = redi[0];
#pragma unroll
  for (int w = 1; w < BT / 32; ++w) KeepBits(ro, ri, redv[w], redi[w]);
  __syncthreads();
  v = BitsVal(ro);
  id = ri;
}

template <int BT, typename I>
__device__ __forceinline__ LexKeyT<I> BlockLex(LexKeyT<I> x, long long* rs, unsigned long long* rk, uint32_t* ri) {
  LexGroupReduce<32, I>(x);
  if (LaneId() == 0) {
    rs[threadIdx.x >> 5] = x.S;
    rk[threadIdx.x >> 5] = x.K;
    ri[threadIdx.x >> 5] = x.id;
  }
  __syncthreads();
  if constexpr (kWideBlock<BT>) {
    if (threadIdx.x < 32) {
      LexKeyT<I> w;
      if (threadIdx.x < BT / 32) w.Keep(static_cast<I>(rs[threadIdx.x]), rk[threadIdx.x], ri[threadIdx.x]);
      LexGroupReduce<32, I>(w);
      if (threadIdx.x == 0) {
        rs[BT / 32] = w.S;
        rk[BT / 32] = w.K;
        ri[BT / 32] = w.id;
      }
    }
    __syncthreads();
    LexKeyT<I> r;
    r.Keep(static_cast<I>(rs[BT / 32]), rk[BT / 32], ri[BT / 32]);
    return r;
  }
  LexKeyT<I> r;
#pragma unroll
  for (int w = 0; w < BT / 32; ++w) r.Keep(static_cast<I>(rs[w]), rk[w], ri[w]);
  __syncthreads();
  return r;
}

// Block leader of `lead` and the class test over `tail` (the two BlockLex
// calls and the (S, K) comparison) with 32-bit sums: warp leaders by REDUX,
// the warps' leaders combined by every thread, the test by one barrier with
// a predicate.
template <int BT>
__device__ __forceinline__ bool BlockLexLeadInt(LexKeyT<int>& lead, const LexKeyT<int>& tail, long long* rs,
                                                unsigned long long* rk, uint32_t* ri) {
  LexWarpLeaderInt(lead);
  if (LaneId() == 0) {
    rs[threadIdx.x >> 5] = lead.S;
    rk[threadIdx.x >> 5] = lead.K;
    ri[threadIdx.x >> 5] = lead.id;
  }
  __syncthreads();
  LexKeyT<int> r;
  if constexpr (kWideBlock<BT>) {
    if (threadIdx.x < 32) {
      LexKeyT<int> w;
      if (threadIdx.x < BT / 32) w.Keep(static_cast<int>(rs[threadIdx.x]), rk[threadIdx.x], ri[threadIdx.x]);
      LexWarpLeaderInt(w);
      if (threadIdx.x == 0) {
        rs[BT / 32] = w.S;
        rk[BT / 32] = w.K;
        ri[BT / 32] = w.id;
      }
    }
    __syncthreads();
    r.Keep(static_cast<int>(rs[BT / 32]), rk[BT / 32], ri[BT / 32]);
  } else {
#pragma unroll
    for (int w = 0; w < BT / 32; ++w) r.Keep(static_cast<int>(rs[w]), rk[w], ri[w]);
  }
  lead = r;
  const bool diff = r.id != kNone && tail.id != kNone && (-tail.S != r.S || ~tail.K != r.K);
  return !__syncthreads_or(diff);  // also orders the reads of rs/rk/ri before their next use
}

// Finds or inserts `key` in a table of `cap` slots (any capacity), probing
// linearly from the slot the hash picks; kNone when the table is full.
__device__ __forceinline__ uint32_t HubInsert(uint32_t* keys, uint32_t cap, uint32_t hsh, uint32_t key,
                                              bool* ins) {
  uint32_t s = __umulhi(hsh, cap);
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
    s = s + 1 == cap ? 0 : s + 1;
  }
  return kNone;
}

// Entry contribution w - offset: integer in INT mode, the reference hub
// path's float-rounded value in FP64 mode.
template <bool kInt>
__device__ __forceinline__ void EntryWeight(const BMArgs& a, float wt, int* xi, double* xd) {
  if (kInt) {
    *xi = WeightToInt(wt) - a.ioffset;
  } else {
    *xd = static_cast<double>(static_cast<float>(Dsub(static_cast<double>(wt), a.offset)));
  }
}

// Warp-aggregated sum of the entry weights of each match group.
template <int BT, bool kInt>
__device__ __forceinline__ void GroupWeights(const BMArgs& a, unsigned peers, bool leader, int xi, double xd,
                                             HubShared<BT>& sh, int* Si, double* Sd) {
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

// Evaluates the CTA's table: returns (to every thread) the best (exact FP64
// value, id) of its keys and clears the table.  INT sync mode: FP32
// pre-filter, then FP64 only for the survivors outside the leading (S, K)
// class, whose members share one FP64 value (evaluated once).
template <int BT, bool kInt, bool kAsync, typename V>
__device__ void EvalTable(const BMArgs& a, const VertexCtx& x, float k32, double change, long long smax_ll,
                          uint32_t* skeys, V* svals, uint32_t cap, HubShared<BT>& sh, double* out_v,
                          uint32_t* out_id) {
  // Integer type of the sums: int for narrow tables (32-bit conversions).
  using I = typename std::conditional<std::is_same<V, int>::value, int, long long>::type;
  const unsigned tid = threadIdx.x;
  constexpr bool kFilter = kInt && !kAsync;
  double lv = 0.0;
  uint32_t lid = kNone;
  // Slots are read kEvalBatch at a time per thread, so that the gathers of
  // their cluster weights are in flight together.
  constexpr int kB = kEvalBatch;
  if (kFilter) {
    const I smax = static_cast<I>(smax_ll);
    const float c32 = sh.change32;
    const float r32 = Res32Of(a, x.v);
    float U = -CUDART_INF_F;
    // The two largest upper ends (Y + e; +inf for a candidate outside the
    // error model) among this thread's slots, and the slot of the largest:
    // when the second is below the block's U, no other slot of the thread
    // can be a contender and the second pass need not re-evaluate them.
    float hi1 = -CUDART_INF_F, hi2 = -CUDART_INF_F;
    uint32_t slot1 = kNone;
    for (uint32_t s0 = tid; s0 < cap; s0 += BT * kB) {
      uint32_t kk[kB];
      I ss[kB];
      float kf[kB];
#pragma unroll
      for (int j = 0; j < kB; ++j) {
        const uint32_t s = s0 + j * BT;
        kk[j] = s < cap ? skeys[s] : kNone;
        ss[j] = s < cap ? static_cast<I>(svals[s]) : I(0);
      }
#pragma unroll
      for (int j = 0; j < kB; ++j) kf[j] = kk[j] != kNone ? a.Kf[kk[j]] : 0.f;
#pragma unroll
      for (int j = 0; j < kB; ++j) {
        if (kk[j] == kNone) continue;
        const FilterVal f = FilterOf<I>(r32, k32, kf[j], ss[j], smax, c32);
        if (f.sane) U = fmaxf(U, __fsub_rn(f.Y, f.e));
        KeepTop2(hi1, hi2, slot1, f.sane ? __fadd_rn(f.Y, f.e) : CUDART_INF_F, s0 + j * BT);
      }
    }
    if (tid == 0) sh.ncont = 0;
    U = BlockMaxF<BT>(U, sh.red_f);
    LexKeyT<I> lead, tail;
    // The contenders are the slots with hi >= U (every slot when U = -inf).
    const bool rescan = !(hi2 < U);
    if (!rescan) {
      // At most slot1 is a contender; the thread's other slots are cleared.
      if (slot1 != kNone && !(hi1 < U)) {
        const uint32_t key = skeys[slot1];
        const I S = static_cast<I>(svals[slot1]);
        const double KD = a.K[key];
        const unsigned long long ko = KOrder(KD);
        lead.Keep(S, ko, key);
        tail.Keep(-S, ~ko, key);
        const uint32_t pos = atomicAdd(&sh.ncont, 1u);
        if (pos < kMaxCont) {
          sh.cont_key[pos] = key;
          sh.cont_S[pos] = S;
        } else {
          KeepBest(lv, lid, ValOf(a, x, change, static_cast<double>(S), KD), key);  // list full: now
        }
      }
      for (uint32_t s = tid; s < cap; s += BT) {
        if (skeys[s] != kNone) {
          skeys[s] = kNone;
          svals[s] = V(0);
        }
      }
    }
    for (uint32_t s0 = rescan ? tid : cap; s0 < cap; s0 += BT * kB) {
      uint32_t kk[kB];
      I ss[kB];
      float kf[kB];
#pragma unroll
      for (int j = 0; j < kB; ++j) {
        const uint32_t s = s0 + j * BT;
        kk[j] = kNone;
        ss[j] = I(0);
        if (s < cap) {
          kk[j] = skeys[s];
          if (kk[j] != kNone) {
            ss[j] = static_cast<I>(svals[s]);
            skeys[s] = kNone;
            svals[s] = V(0);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < kB; ++j) kf[j] = kk[j] != kNone ? a.Kf[kk[j]] : 0.f;
#pragma unroll
      for (int j = 0; j < kB; ++j) {
        const uint32_t key = kk[j];
        if (key == kNone) continue;
        const I S = ss[j];
        const FilterVal f = FilterOf<I>(r32, k32, kf[j], S, smax, c32);
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
          KeepBest(lv, lid, ValOf(a, x, change, static_cast<double>(S), KD), key);  // list full: now
        }
      }
    }
    bool single;
    if constexpr (std::is_same<I, int>::value) {
      single = BlockLexLeadInt<BT>(lead, tail, sh.red_ll, sh.red_k, sh.red_i);
    } else {
      lead = BlockLex<BT, I>(lead, sh.red_ll, sh.red_k, sh.red_i);
      tail = BlockLex<BT, I>(tail, sh.red_ll, sh.red_k, sh.red_i);
      single = lead.id == kNone || (-tail.S == lead.S && ~tail.K == lead.K);
    }
    const uint32_t nc = min(sh.ncont, kMaxCont);
    if (!single) {
      for (uint32_t i = tid; i < nc; i += BT) {
        const uint32_t key = sh.cont_key[i];
        const I S = static_cast<I>(sh.cont_S[i]);
        const double KD = a.K[key];
        if (S == lead.S && KOrder(KD) == lead.K) continue;  // the leading class
        KeepBest(lv, lid, ValOf(a, x, change, static_cast<double>(S), KD), key);
      }
    }
    if (tid == 0 && lead.id != kNone)
      KeepBest(lv, lid, ValOf(a, x, change, static_cast<double>(lead.S), a.K[lead.id]), lead.id);
  } else {
    for (uint32_t s0 = tid; s0 < cap; s0 += BT * kB) {
      uint32_t kk[kB];
      V sv[kB];
      double kd[kB];
#pragma unroll
      for (int j = 0; j < kB; ++j) {
        const uint32_t s = s0 + j * BT;
        kk[j] = kNone;
        sv[j] = V(0);
        if (s < cap) {
          kk[j] = skeys[s];
          if (kk[j] != kNone) {
            sv[j] = svals[s];
            skeys[s] = kNone;
            svals[s] = V(0);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < kB; ++j) kd[j] = kk[j] != kNone ? LdK<kAsync>(a.K + kk[j]) : 0.0;
#pragma unroll
      for (int j = 0; j < kB; ++j)
        if (kk[j] != kNone) KeepBest(lv, lid, ValOf(a, x, change, static_cast<double>(sv[j]), kd[j]), kk[j]);
    }
  }
  BlockArgmax<BT>(lv, lid, sh.red_k, sh.red_i);
  *out_v = lv;
  *out_id = lid;
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

// One CTA's scan of a hub row: the entries whose cluster falls in partition
// p / sub-partition q are added into the CTA's table; "together" (the hub's
// own cluster) accumulates when want_T.  Returns the largest sum seen
// (INT mode) through *smax.
template <int BT, bool kInt, bool kAsync, typename V>
__device__ __forceinline__ void ScanRow(const BMArgs& a, const VertexCtx& x, uint32_t P, uint32_t p, uint32_t Q,
                                        uint32_t q, bool want_T, uint32_t* skeys, V* svals, uint32_t cap,
                                        uint32_t maxkeys, HubShared<BT>& sh, long long* t_int, double* t_dbl,
                                        long long* smax) {
  const unsigned tid = threadIdx.x, lane = LaneId();
  const uint32_t v = x.v;
  for (uint32_t e0 = 0; e0 < x.d; e0 += BT * kHubUnroll) {
    uint32_t uu[kHubUnroll], cc[kHubUnroll];
    float ww[kHubUnroll];
#pragma unroll
    for (int k = 0; k < kHubUnroll; ++k) {
      const uint32_t e = e0 + k * BT + tid;
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
      if (e0 + k * BT >= x.d) break;  // uniform over the CTA
      const bool cand = uu[k] != v;
      const uint32_t cu = cc[k];
      int xi = 0;
      double xd = 0.0;
      if (cand) EntryWeight<kInt>(a, ww[k], &xi, &xd);
      if (want_T && cand && cu == x.c) {
        if (kInt)
          *t_int += xi;
        else
          *t_dbl = Dadd(*t_dbl, xd);
      }
      bool mine = cand;
      if (P > 1 || Q > 1) {
        const uint32_t hp = Mix32(cu);
        mine = mine && __umulhi(hp, P) == p && ((hp >> 8) & (Q - 1)) == q;
      }
      // INT mode: every entry adds its own integer weight (exact in any
      // order); FP64 mode: equal clusters of the warp are summed in lane
      // order first, one atomic per cluster.
      unsigned peers = 0;
      bool leader = mine;
      int Si = xi;
      double Sd = 0.0;
      if (!kInt) {
        peers = __match_any_sync(kFull, mine ? cu : LaneSentinel(lane));
        leader = mine && int(lane) == __ffs(peers) - 1;
        GroupWeights<BT, kInt>(a, peers, leader, xi, xd, sh, &Si, &Sd);
      }
      if (leader && *reinterpret_cast<volatile uint32_t*>(&sh.overflow) == 0) {
        bool ins;
        const uint32_t slot = HubInsert(skeys, cap, SlotHash(cu), cu, &ins);
        if (slot == kNone) {
          sh.overflow = 1;
        } else {
          if (ins && atomicAdd(&sh.nkeys, 1u) + 1 > maxkeys) sh.overflow = 1;
          if (kInt) {
            const V old = AtomicAddV<V>(svals + slot, static_cast<V>(Si));
            *smax = max(*smax, static_cast<long long>(old) + Si);
          } else {
            AtomicAddV<V>(svals + slot, static_cast<V>(Sd));
          }
        }
      }
    }
  }
}

// The hub's "together" and change, once per item (FP64 by one thread).
template <int BT, bool kInt>
__device__ __forceinline__ double HubChange(const BMArgs& a, const VertexCtx& x, long long t_int, double t_dbl,
                                            HubShared<BT>& sh) {
  double T;
  if (kInt)
    T = static_cast<double>(BlockSum<BT, long long>(t_int, sh.red_ll));
  else
    T = BlockSum<BT, double>(t_dbl, sh.red_d);
  if (threadIdx.x == 0) {
    sh.change = ChangeOf(a, x, T);
    sh.change32 = static_cast<float>(sh.change);
  }
  __syncthreads();
  return sh.change;
}

// HubChange and, in INT mode, the block maximum of the running sums.  Wide
// CTAs take both in one reduction: warp 0 combines the warps' (sum, max)
// partials and its lane 0 computes the change, so that the table scan's end
// costs two barriers.
template <int BT, bool kInt>
__device__ __forceinline__ double HubChangeSmax(const BMArgs& a, const VertexCtx& x, long long t_int, double t_dbl,
                                                long long* smax, HubShared<BT>& sh) {
  if constexpr (!kWideBlock<BT>) {
    __syncthreads();
    const double change = HubChange<BT, kInt>(a, x, t_int, t_dbl, sh);
    if (kInt) *smax = BlockMaxLL<BT>(*smax, sh.red_ll);
    return change;
  } else if constexpr (!kInt) {
    return HubChange<BT, kInt>(a, x, t_int, t_dbl, sh);
  } else {
    constexpr int kW = BT / 32;
    long long t = t_int, m = *smax;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      t += __shfl_xor_sync(kFull, t, o);
      m = max(m, __shfl_xor_sync(kFull, m, o));
    }
    if (LaneId() == 0) {
      sh.red_ll[threadIdx.x >> 5] = t;
      sh.red_mx[threadIdx.x >> 5] = m;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      long long wt = threadIdx.x < kW ? sh.red_ll[threadIdx.x] : 0;
      long long wm = threadIdx.x < kW ? sh.red_mx[threadIdx.x] : LLONG_MIN;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        wt += __shfl_xor_sync(kFull, wt, o);
        wm = max(wm, __shfl_xor_sync(kFull, wm, o));
      }
      if (threadIdx.x == 0) {
        sh.change = ChangeOf(a, x, static_cast<double>(wt));
        sh.change32 = static_cast<float>(sh.change);
        sh.red_mx[kW] = wm;
      }
    }
    __syncthreads();
    *smax = sh.red_mx[kW];
    return sh.change;
  }
}

// ---------------------------------------------------------------------------
// Small hubs: one CTA per hub, a table of 2 * degree slots (never full).
// ---------------------------------------------------------------------------
template <bool kInt, bool kAsync, typename V, uint32_t kSlots>
__global__ void __launch_bounds__(kSmallThreads) HubSmallKernel(HubArgs h) {
  constexpr int BT = kSmallThreads;
  extern __shared__ __align__(16) unsigned char smem[];
  V* svals = reinterpret_cast<V*>(smem);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem + size_t(kSlots) * sizeof(V));
  __shared__ HubShared<BT> sh;
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x;
  unsigned long long fam_e = 0, fam_v = 0;  // entries and vertices evaluated (tid 0)
  for (uint32_t i = tid; i < kSlots; i += BT) {
    skeys[i] = kNone;
    svals[i] = V(0);
  }
  if (tid == 0) {
    sh.overflow = 0;
    sh.nkeys = 0;
  }
  __syncthreads();
  for (uint32_t item = h.small_lo + blockIdx.x; item < h.small_hi; item += gridDim.x) {
    const uint32_t v = h.small_v[item];
    if (!InFront(a, v)) continue;  // uniform over the CTA
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    const uint32_t cap = min(kSlots, 2 * x.d + 2);
    if (tid == 0) {
      fam_e += x.d;
      fam_v += 1;
    }
    long long t_int = 0, smax = LLONG_MIN;
    double t_dbl = 0.0;
    ScanRow<BT, kInt, kAsync, V>(a, x, 1, 0, 1, 0, true, skeys, svals, cap, cap, sh, &t_int, &t_dbl, &smax);
    // Its barriers also complete the table and sh.overflow before they are read.
    const double change = HubChangeSmax<BT, kInt>(a, x, t_int, t_dbl, &smax, sh);
    if (tid == 0) {
      if (sh.overflow) atomicExch(&a.ctr->error, kErrHashFull);  // cannot happen: 2d + 2 slots
      sh.nkeys = 0;
    }
    double bv;
    uint32_t bi;
    EvalTable<BT, kInt, kAsync, V>(a, x, a.kf[v], change, smax, skeys, svals, cap, sh, &bv, &bi);
    if (tid == 0) HubDecide<kAsync>(a, x, bv, bi, change);
    __syncthreads();
  }
  if (tid == 0 && fam_v) {
    atomicAdd(&a.ctr->fam_entries[kFamHubSmall], fam_e);
    atomicAdd(&a.ctr->fam_vertices[kFamHubSmall], fam_v);
  }
}

// ---------------------------------------------------------------------------
// Big hubs: one CTA per (hub, partition), sub-passes on overflow.
// ---------------------------------------------------------------------------
template <bool kInt, bool kAsync, typename V>
__global__ void __launch_bounds__(kBigThreads) HubBigKernel(HubArgs h) {
  constexpr int BT = kBigThreads;
  constexpr uint32_t kSlots = BigSlots<V>();
  extern __shared__ __align__(16) unsigned char smem[];
  V* svals = reinterpret_cast<V*>(smem);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem + size_t(kSlots) * sizeof(V));
  __shared__ HubShared<BT> sh;
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x;
  unsigned long long fam_e = 0, fam_v = 0;  // entries and vertices evaluated once per hub (tid 0)
  for (uint32_t i = tid; i < kSlots; i += BT) {
    skeys[i] = kNone;
    svals[i] = V(0);
  }
  if (tid == 0) {
    sh.overflow = 0;
    sh.nkeys = 0;
  }
  __syncthreads();
  for (uint32_t item = blockIdx.x; item < h.num_items; item += gridDim.x) {
    const uint32_t hb = h.item_hub[item];
    const uint32_t p = h.item_part[item];
    const uint32_t v = h.big_v[hb];
    if (!kAsync && h.num_glob && h.big_glob[hb] != kNone) continue;  // global path
    if (!InFront(a, v)) continue;  // uniform over the CTA
    const VertexCtx x = LoadVertex<kAsync>(a, v);
    const uint32_t P = h.big_parts[hb];
    if (tid == 0 && p == 0) {
      fam_e += x.d;
      fam_v += 1;
    }
    const uint32_t cap = min(kSlots, 2 * ((x.d + P - 1) / P) + 2);
    const uint32_t maxkeys = cap - cap / 4;
    uint32_t Q = 1, q = 0;
    bool have_T = false;
    double change = 0.0;
    double bestv = 0.0;
    uint32_t bestid = kNone;
    while (true) {
      long long t_int = 0, smax = LLONG_MIN;
      double t_dbl = 0.0;
      ScanRow<BT, kInt, kAsync, V>(a, x, P, p, Q, q, !have_T, skeys, svals, cap, maxkeys, sh, &t_int, &t_dbl,
                                   &smax);
      // The reductions' barriers also order the reads of sh.overflow.
      if (!have_T) {
        change = HubChangeSmax<BT, kInt>(a, x, t_int, t_dbl, &smax, sh);
        have_T = true;
      } else {
        __syncthreads();
        if (kInt) smax = BlockMaxLL<BT>(smax, sh.red_ll);
      }
      const bool overflow = sh.overflow != 0;
      __syncthreads();
      if (tid == 0) {
        sh.overflow = 0;
        sh.nkeys = 0;
      }
      if (overflow) {
        // Split the partition further and rescan from the first sub-pass.
        for (uint32_t s = tid; s < cap; s += BT) {
          skeys[s] = kNone;
          svals[s] = V(0);
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
      double lv;
      uint32_t lid;
      EvalTable<BT, kInt, kAsync, V>(a, x, a.kf[v], change, smax, skeys, svals, cap, sh, &lv, &lid);
      KeepBest(bestv, bestid, lv, lid);
      __syncthreads();
      if (++q == Q) break;
    }
    // Partial result; the hub's last CTA combines and decides.
    if (tid == 0) {
      const uint32_t pb = h.big_pbase[hb];
      h.part_val[pb + p] = bestv;
      h.part_id[pb + p] = bestid;
      __threadfence();
      if (atomicAdd(&h.done[hb], 1u) == P - 1) {
        __threadfence();
        double bv = 0.0;
        uint32_t bi = kNone;
        for (uint32_t j = 0; j < P; ++j) KeepBest(bv, bi, __ldcg(h.part_val + pb + j), __ldcg(h.part_id + pb + j));
        h.done[hb] = 0;
        HubDecide<kAsync>(a, x, bv, bi, change);
      }
    }
    __syncthreads();
  }
  if (tid == 0 && fam_v) {
    atomicAdd(&a.ctr->fam_entries[kFamHubBig], fam_e);
    atomicAdd(&a.ctr->fam_vertices[kFamHubBig], fam_v);
  }
}

// ---------------------------------------------------------------------------
// Global path: rows of the largest hubs split over many CTAs.
// ---------------------------------------------------------------------------
constexpr int kGlobThreads = 256;
constexpr uint32_t kGlobChunk = kGlobThreads;  // row entries per work item: one per thread

// Accumulates row chunks into the hubs' HBM tables (warp-aggregated inserts
// and adds), the together-sum and (INT) the largest running sum.
template <bool kInt, typename V>
__global__ void __launch_bounds__(kGlobThreads) HubGlobalAccumKernel(HubArgs h) {
  constexpr int BT = kGlobThreads;
  __shared__ HubShared<BT> sh;
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x, lane = LaneId();
  for (uint32_t item = blockIdx.x; item < h.num_glob_items; item += gridDim.x) {
    const uint32_t gi = h.glob_item[item];
    const uint32_t v = h.big_v[h.glob_hub[gi]];
    if (!InFront(a, v)) continue;  // uniform over the CTA
    const VertexCtx x = LoadVertex<false>(a, v);
    const uint32_t e_begin = h.glob_item_start[item];
    const uint32_t e_end = min(x.d, e_begin + kGlobChunk);
    uint32_t* keys = h.gkeys + h.glob_base[gi];
    V* vals = reinterpret_cast<V*>(h.gvals) + h.glob_base[gi];
    const uint32_t cap = h.glob_cap[gi];
    long long t_int = 0, smax = LLONG_MIN;
    double t_dbl = 0.0;
    for (uint32_t e0 = e_begin; e0 < e_end; e0 += BT * kHubUnroll) {
      uint32_t uu[kHubUnroll], cc[kHubUnroll];
      float ww[kHubUnroll];
#pragma unroll
      for (int k = 0; k < kHubUnroll; ++k) {
        const uint32_t e = e0 + k * BT + tid;
        uu[k] = v;
        ww[k] = 0.f;
        if (e < e_end) {
          uu[k] = a.nbr[x.b + e];
          ww[k] = a.w ? a.w[x.b + e] : 1.0f;
        }
      }
#pragma unroll
      for (int k = 0; k < kHubUnroll; ++k) cc[k] = uu[k] != v ? __ldg(a.C + uu[k]) : kNone;
#pragma unroll
      for (int k = 0; k < kHubUnroll; ++k) {
        if (e0 + k * BT >= e_end) break;  // uniform over the CTA
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
        unsigned peers = 0;
        bool leader = cand;
        int Si = xi;
        double Sd = 0.0;
        if (!kInt) {
          peers = __match_any_sync(kFull, cand ? cu : LaneSentinel(lane));
          leader = cand && int(lane) == __ffs(peers) - 1;
          GroupWeights<BT, kInt>(a, peers, leader, xi, xd, sh, &Si, &Sd);
        }
        if (leader) {
          bool ins;
          const uint32_t slot = HubInsert(keys, cap, SlotHash(cu), cu, &ins);
          if (slot == kNone) {
            atomicExch(&a.ctr->error, kErrHashFull);  // cannot happen: 2 * degree + 2 slots
          } else if (kInt) {
            const V old = AtomicAddV<V>(vals + slot, static_cast<V>(Si));
            smax = max(smax, static_cast<long long>(old) + Si);
          } else {
            AtomicAddV<V>(vals + slot, static_cast<V>(Sd));
          }
        }
      }
    }
    if (kInt) {
      const long long t = BlockSum<BT, long long>(t_int, sh.red_ll);
      const long long mx = BlockMaxLL<BT>(smax, sh.red_ll);
      if (tid == 0) {
        if (t) atomicAdd(reinterpret_cast<unsigned long long*>(h.gt_int + gi), static_cast<unsigned long long>(t));
        atomicMax(h.gsmax + gi, mx);
      }
    } else {
      const double t = BlockSum<BT, double>(t_dbl, sh.red_d);
      if (tid == 0 && t != 0.0) atomicAdd(h.gt_dbl + gi, t);
    }
  }
}

// Evaluates the HBM tables of the frontier hubs, one slice per CTA (the
// small-hub evaluation of the slice's keys: FP32 pre-filter, certified leading
// class, FP64 survivors), clearing the slots (EvalTable).  The hub's last CTA
// combines the slices' (value, id) bests, decides and resets the hub's
// accumulators.
template <bool kInt, typename V>
__global__ void __launch_bounds__(kGlobThreads) HubGlobalEvalKernel(HubArgs h) {
  constexpr int BT = kGlobThreads;
  __shared__ HubShared<BT> sh;
  const BMArgs& a = h.a;
  const unsigned tid = threadIdx.x;
  unsigned long long fam_e = 0, fam_v = 0;
  for (uint32_t item = blockIdx.x; item < h.num_glob_slices; item += gridDim.x) {
    const uint32_t gi = h.slice_hub[item];
    const uint32_t v = h.big_v[h.glob_hub[gi]];
    if (!InFront(a, v)) continue;  // uniform over the CTA
    const VertexCtx x = LoadVertex<false>(a, v);
    const uint32_t s0 = h.slice_start[item];
    const uint32_t len = min(kHubGlobalSlice, h.glob_cap[gi] - s0);
    const long long smax = __ldcg(h.gsmax + gi);
    if (tid == 0) {
      if (s0 == 0) {
        fam_e += x.d;
        fam_v += 1;
      }
      const double T = kInt ? static_cast<double>(__ldcg(h.gt_int + gi)) : __ldcg(h.gt_dbl + gi);
      sh.change = ChangeOf(a, x, T);
      sh.change32 = static_cast<float>(sh.change);
    }
    __syncthreads();
    const double change = sh.change;
    double bv;
    uint32_t bi;
    const unsigned long long base = h.glob_base[gi] + s0;
    EvalTable<BT, kInt, false, V>(a, x, a.kf[v], change, smax, h.gkeys + base, reinterpret_cast<V*>(h.gvals) + base,
                                  len, sh, &bv, &bi);
    const uint32_t sb = h.glob_sbase[gi];
    const uint32_t ns = h.glob_nslices[gi];
    if (tid == 0) {
      h.gpart_val[sb + s0 / kHubGlobalSlice] = bv;
      h.gpart_id[sb + s0 / kHubGlobalSlice] = bi;
      __threadfence();
      sh.last = atomicAdd(&h.gdone[gi], 1u) == ns - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (sh.last) {  // uniform: the whole CTA combines the slices' bests
      __threadfence();
      double cv = 0.0;
      uint32_t ci = kNone;
      for (uint32_t j = tid; j < ns; j += BT) KeepBest(cv, ci, __ldcg(h.gpart_val + sb + j), __ldcg(h.gpart_id + sb + j));
      BlockArgmax<BT>(cv, ci, sh.red_k, sh.red_i);
      if (tid == 0) {
        HubDecide<false>(a, x, cv, ci, change);
        h.gdone[gi] = 0;
        h.gt_int[gi] = 0;
        h.gt_dbl[gi] = 0.0;
        h.gsmax[gi] = LLONG_MIN;
      }
    }
    __syncthreads();
  }
  if (tid == 0 && fam_v) {
    atomicAdd(&a.ctr->fam_entries[kFamHubBig], fam_e);
    atomicAdd(&a.ctr->fam_vertices[kFamHubBig], fam_v);
  }
}

__global__ void GlobalStateInitKernel(uint32_t num, long long* gt_int, double* gt_dbl, long long* gsmax,
                                      uint32_t* gdone) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
    gt_int[i] = 0;
    gt_dbl[i] = 0.0;
    gsmax[i] = LLONG_MIN;
    gdone[i] = 0;
  }
}

__global__ void HubDegreesKernel(const uint32_t* list, uint32_t count, const uint64_t* off, uint32_t* deg) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    deg[i] = static_cast<uint32_t>(off[list[i] + 1] - off[list[i]]);
}

// Dynamic shared-memory limit and resident CTAs per SM of a kernel, set up
// and queried once per process (the runtime calls take a lock that
// serialises concurrent contexts).  Returns 0 on failure.
template <class K>
int PrepareOnce(K kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> per_sm_of;
  std::lock_guard<std::mutex> lk(mu);
  auto it = per_sm_of.find(reinterpret_cast<const void*>(kernel));
  if (it != per_sm_of.end()) return it->second;
  int per_sm = 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  per_sm_of[reinterpret_cast<const void*>(kernel)] = per_sm;
  return per_sm;
}

// One small-hub table class over small_v[lo, hi).
template <bool kInt, bool kAsync, typename V, uint32_t kSlots>
Status LaunchSmallClass(Context* ctx, const HubArgs& h, uint32_t lo, uint32_t hi) {
  if (hi <= lo) return Status::Ok();
  constexpr size_t smem = size_t(kSlots) * (sizeof(V) + sizeof(uint32_t));
  auto k = HubSmallKernel<kInt, kAsync, V, kSlots>;
  const int per_sm = PrepareOnce(k, kSmallThreads, smem);
  if (per_sm <= 0) return MakeError(PCC_INTERNAL, "small-hub kernel cannot be configured");
  HubArgs hc = h;
  hc.small_lo = lo;
  hc.small_hi = hi;
  k<<<Blocks(hi - lo, 1, unsigned(ctx->num_sms) * unsigned(per_sm)), kSmallThreads, smem, ctx->stream>>>(hc);
  PCC_COUNT(1);
  return Status::Ok();
}

template <bool kInt, bool kAsync, typename V>
Status LaunchHubT(Context* ctx, const HubArgs& h, uint32_t num_small, uint32_t num_wide, uint32_t num_mid,
                  int families) {
  const unsigned sms = unsigned(ctx->num_sms);
  if (num_small && (families & kLaunchSmallHubs)) {
    // Three table sizes, each hub in the smallest that holds its 2d + 2
    // slots (the classes are consecutive in small_v, widest first): smaller
    // tables fit more CTAs per SM.
    const uint32_t end_mid = num_wide + num_mid;
    const int nl = (num_wide > 0) + (num_mid > 0) + (num_small > end_mid);
    FamBegin(ctx, kFamHubSmall);
    PCC_RETURN_IF_ERROR((LaunchSmallClass<kInt, kAsync, V, kSmallSlots>(ctx, h, 0, num_wide)));
    PCC_RETURN_IF_ERROR((LaunchSmallClass<kInt, kAsync, V, kSmallMidSlots>(ctx, h, num_wide, end_mid)));
    PCC_RETURN_IF_ERROR((LaunchSmallClass<kInt, kAsync, V, kSmallNarrowSlots>(ctx, h, end_mid, num_small)));
    FamEnd(ctx, kFamHubSmall, nl);
  }
  const bool glob = !kAsync && h.num_glob;
  if (h.num_items && (families & kLaunchBigHubs)) {
    FamBegin(ctx, kFamHubBig);
    if (glob) {
      HubGlobalAccumKernel<kInt, V><<<std::min<unsigned>(h.num_glob_items, sms * 8), kGlobThreads, 0,
                                      ctx->stream>>>(h);
      PCC_COUNT(1);
    }
    FamEnd(ctx, kFamHubBig, glob ? 1 : 0);
    constexpr size_t smem = size_t(BigSlots<V>()) * (sizeof(V) + sizeof(uint32_t));
    auto k = HubBigKernel<kInt, kAsync, V>;
    const int per_sm = PrepareOnce(k, kBigThreads, smem);
    if (per_sm <= 0) return MakeError(PCC_INTERNAL, "big-hub kernel cannot be configured");
    const unsigned grid = Blocks(h.num_items, 1, sms * unsigned(std::max(per_sm, 1)));
    FamBegin(ctx, kFamHubBig);
    k<<<grid, kBigThreads, smem, ctx->stream>>>(h);
    FamEnd(ctx, kFamHubBig, 1);
    PCC_COUNT(1);
    if (glob) {
      FamBegin(ctx, kFamHubBig);
      HubGlobalEvalKernel<kInt, V><<<std::min<unsigned>(h.num_glob_slices, 8 * sms), kGlobThreads, 0,
                                     ctx->stream>>>(h);
      FamEnd(ctx, kFamHubBig, 1);
      PCC_COUNT(1);
    }
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
  std::vector<uint32_t> big_glob, glob_hub, glob_cap, glob_item, glob_item_start;
  std::vector<uint32_t> glob_nslices, glob_sbase, slice_hub, slice_start;
  std::vector<unsigned long long> glob_base;
  uint64_t total = 0;
  for (uint32_t r = 0; r < count; ++r) {
    const uint32_t i = order[r];
    if (hd[i] <= kHubSmallMax) {
      small_v.push_back(hv[i]);
      if (2 * hd[i] + 2 > kSmallMidSlots) plan->num_small_wide++;
      else if (2 * hd[i] + 2 > kSmallNarrowSlots) plan->num_small_mid++;
      continue;
    }
    const uint32_t P = std::max<uint32_t>(1, (hd[i] + kHubBigKeys - 1) / kHubBigKeys);
    const uint32_t hb = static_cast<uint32_t>(big_v.size());
    big_v.push_back(hv[i]);
    if (P >= kHubGlobalParts) {
      const uint32_t gi = static_cast<uint32_t>(glob_hub.size());
      big_glob.push_back(gi);
      glob_hub.push_back(hb);
      glob_base.push_back(plan->glob_slots);
      const uint32_t gcap = 2 * hd[i] + 2;
      glob_cap.push_back(gcap);
      plan->glob_slots += gcap;
      glob_sbase.push_back(static_cast<uint32_t>(slice_hub.size()));
      glob_nslices.push_back((gcap + kHubGlobalSlice - 1) / kHubGlobalSlice);
      for (uint32_t s0 = 0; s0 < gcap; s0 += kHubGlobalSlice) {
        slice_hub.push_back(gi);
        slice_start.push_back(s0);
      }
      for (uint32_t e = 0; e < hd[i]; e += kGlobChunk) {
        glob_item.push_back(gi);
        glob_item_start.push_back(e);
      }
    } else {
      big_glob.push_back(kNone);
    }
    parts.push_back(P);
    pbase.push_back(static_cast<uint32_t>(total));
    total += P;
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
  plan->num_glob = static_cast<uint32_t>(glob_hub.size());
  plan->num_glob_items = static_cast<uint32_t>(glob_item.size());
  if (plan->num_glob) {
    PCC_RETURN_IF_ERROR(up(plan->big_glob, big_glob));
    PCC_RETURN_IF_ERROR(up(plan->glob_hub, glob_hub));
    PCC_RETURN_IF_ERROR(up(plan->glob_cap, glob_cap));
    PCC_RETURN_IF_ERROR(up(plan->glob_item, glob_item));
    PCC_RETURN_IF_ERROR(up(plan->glob_item_start, glob_item_start));
    plan->num_glob_slices = static_cast<uint32_t>(slice_hub.size());
    PCC_RETURN_IF_ERROR(up(plan->glob_nslices, glob_nslices));
    PCC_RETURN_IF_ERROR(up(plan->glob_sbase, glob_sbase));
    PCC_RETURN_IF_ERROR(up(plan->slice_hub, slice_hub));
    PCC_RETURN_IF_ERROR(up(plan->slice_start, slice_start));
    PCC_RETURN_IF_ERROR(plan->glob_base.Alloc(ctx, glob_base.size()));
    PCC_RETURN_IF_ERROR(plan->glob_base.FromHost(glob_base.data(), glob_base.size()));
  }
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
  if (plan.num_glob) {
    // The rounds leave the tables clean; they are reset here all the same,
    // at every level, so that a run cut short cannot leave keys behind.
    if (st->gkeys.count < plan.glob_slots) {
      PCC_RETURN_IF_ERROR(st->gkeys.Alloc(ctx, plan.glob_slots));
      PCC_RETURN_IF_ERROR(st->gvals.Alloc(ctx, plan.glob_slots));
    }
    if (st->gt_int.count < plan.num_glob) {
      PCC_RETURN_IF_ERROR(st->gt_int.Alloc(ctx, plan.num_glob));
      PCC_RETURN_IF_ERROR(st->gt_dbl.Alloc(ctx, plan.num_glob));
      PCC_RETURN_IF_ERROR(st->gsmax.Alloc(ctx, plan.num_glob));
      PCC_RETURN_IF_ERROR(st->gdone.Alloc(ctx, plan.num_glob));
    }
    if (st->gpart_val.count < plan.num_glob_slices) {
      PCC_RETURN_IF_ERROR(st->gpart_val.Alloc(ctx, plan.num_glob_slices));
      PCC_RETURN_IF_ERROR(st->gpart_id.Alloc(ctx, plan.num_glob_slices));
    }
    PCC_CUDA(cudaMemsetAsync(st->gkeys.p, 0xFF, plan.glob_slots * sizeof(uint32_t), ctx->stream));  // kNone
    PCC_CUDA(cudaMemsetAsync(st->gvals.p, 0, plan.glob_slots * sizeof(unsigned long long), ctx->stream));
    GlobalStateInitKernel<<<Blocks(plan.num_glob, 256, 1024), 256, 0, ctx->stream>>>(
        plan.num_glob, st->gt_int.p, st->gt_dbl.p, st->gsmax.p, st->gdone.p);
    PCC_COUNT(1);
  }
  return st->done.Zero();
}

Status PrepareHubKernels() {
  static std::mutex mu;
  static bool done = false;
  std::lock_guard<std::mutex> lk(mu);
  if (done) return Status::Ok();
  bool ok = true;
  auto small = [&](auto k, size_t slots, size_t vsize) {
    ok = ok && PrepareOnce(k, kSmallThreads, slots * (vsize + sizeof(uint32_t))) > 0;
  };
  auto big = [&](auto k, size_t slots, size_t vsize) {
    ok = ok && PrepareOnce(k, kBigThreads, slots * (vsize + sizeof(uint32_t))) > 0;
  };
  small(HubSmallKernel<true, false, int, kSmallSlots>, kSmallSlots, sizeof(int));
  small(HubSmallKernel<true, false, int, kSmallNarrowSlots>, kSmallNarrowSlots, sizeof(int));
  small(HubSmallKernel<true, false, int, kSmallMidSlots>, kSmallMidSlots, sizeof(int));
  small(HubSmallKernel<true, false, long long, kSmallMidSlots>, kSmallMidSlots, sizeof(long long));
  small(HubSmallKernel<false, false, double, kSmallMidSlots>, kSmallMidSlots, sizeof(double));
  small(HubSmallKernel<true, false, long long, kSmallSlots>, kSmallSlots, sizeof(long long));
  small(HubSmallKernel<true, false, long long, kSmallNarrowSlots>, kSmallNarrowSlots, sizeof(long long));
  small(HubSmallKernel<false, false, double, kSmallSlots>, kSmallSlots, sizeof(double));
  small(HubSmallKernel<false, false, double, kSmallNarrowSlots>, kSmallNarrowSlots, sizeof(double));
  big(HubBigKernel<true, false, int>, BigSlots<int>(), sizeof(int));
  big(HubBigKernel<true, false, long long>, BigSlots<long long>(), sizeof(long long));
  big(HubBigKernel<false, false, double>, BigSlots<double>(), sizeof(double));
  if (!ok) return MakeError(PCC_INTERNAL, "hub kernels cannot be configured");
  done = true;
  return Status::Ok();
}

Status LaunchHubBestMoves(Context* ctx, const BMArgs& a, const HubPlan& plan, HubState& st, bool int_mode,
                          bool narrow, int families) {
  if (plan.num_hubs == 0) return Status::Ok();
  HubArgs h;
  h.a = a;
  h.small_v = plan.small_v.p;
  h.small_lo = 0;
  h.small_hi = plan.num_small;
  h.big_v = plan.big_v.p;
  h.big_parts = plan.big_parts.p;
  h.big_pbase = plan.big_pbase.p;
  h.item_hub = plan.item_hub.p;
  h.item_part = plan.item_part.p;
  h.num_items = plan.num_items;
  h.part_val = st.part_val.p;
  h.part_id = st.part_id.p;
  h.done = st.done.p;
  h.num_glob = plan.num_glob;
  h.num_glob_items = plan.num_glob_items;
  h.glob_hub = plan.glob_hub.p;
  h.glob_base = plan.glob_base.p;
  h.glob_cap = plan.glob_cap.p;
  h.glob_item = plan.glob_item.p;
  h.glob_item_start = plan.glob_item_start.p;
  h.big_glob = plan.big_glob.p;
  h.gkeys = st.gkeys.p;
  h.gvals = st.gvals.p;
  h.gt_int = st.gt_int.p;
  h.gt_dbl = st.gt_dbl.p;
  h.gsmax = st.gsmax.p;
  h.num_glob_slices = plan.num_glob_slices;
  h.glob_nslices = plan.glob_nslices.p;
  h.glob_sbase = plan.glob_sbase.p;
  h.slice_hub = plan.slice_hub.p;
  h.slice_start = plan.slice_start.p;
  h.gpart_val = st.gpart_val.p;
  h.gpart_id = st.gpart_id.p;
  h.gdone = st.gdone.p;
  if (a.async) {
    if (!int_mode)
      return LaunchHubT<false, true, double>(ctx, h, plan.num_small, plan.num_small_wide, plan.num_small_mid, families);
    return narrow ? LaunchHubT<true, true, int>(ctx, h, plan.num_small, plan.num_small_wide, plan.num_small_mid, families)
                  : LaunchHubT<true, true, long long>(ctx, h, plan.num_small, plan.num_small_wide, plan.num_small_mid,
                                                      families);
  }
  if (!int_mode)
    return LaunchHubT<false, false, double>(ctx, h, plan.num_small, plan.num_small_wide, plan.num_small_mid, families);
  return narrow ? LaunchHubT<true, false, int>(ctx, h, plan.num_small, plan.num_small_wide, plan.num_small_mid, families)
                : LaunchHubT<true, false, long long>(ctx, h, plan.num_small, plan.num_small_wide, plan.num_small_mid,
                                                     families);
}

}  // namespace pcc
