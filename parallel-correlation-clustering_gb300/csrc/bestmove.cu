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
#include "certify.cuh"
#include "moves.cuh"

namespace pcc {

namespace {

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
  __shared__ uint32_t mover_buf[8][64];
  WarpMoverBuffer mb{mover_buf[threadIdx.x >> 5]};
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  constexpr unsigned kVpw = 32 / G;
  const unsigned g = lane / G, gl = lane % G;
  const unsigned gmask = G == 32 ? kFull : (((1u << G) - 1u) << (g * G));
  unsigned long long fam_e = 0, fam_v = 0;
  const uint64_t stride = uint64_t(gridDim.x) * 8 * kVpw;
  // Vertex ids are loaded one iteration ahead (latency-bound kernel).
  uint64_t base = (uint64_t(blockIdx.x) * 8 + warp) * kVpw;
  uint32_t vid = base + g < count ? list[start + base + g] : 0u;
  for (; base < count; base += stride) {
    const uint64_t idx = base + g;
    const uint32_t nvid = base + stride + g < count ? list[start + base + stride + g] : 0u;
    bool vvalid = idx < count;
    VertexCtx x{};
    if (vvalid) {
      vvalid = InFront(a, vid);
      if (vvalid) x = LoadVertex<kAsync>(a, vid);
    }
    vid = nvid;
    if (__ballot_sync(kFull, vvalid) == 0) continue;
    if (vvalid && gl == 0) {
      fam_e += x.d;
      fam_v += 1;
    }  // no frontier vertex in this warp
    const bool has = vvalid && gl < x.d;
    uint32_t u = x.v;
    float wt = 0.f;
    if (has) {
      u = a.nbr[x.b + gl];
      wt = a.w ? a.w[x.b + gl] : 1.0f;
    }
    const bool cand = has && u != x.v;
    const uint32_t cu = cand ? LdC<kAsync>(a.C + u) : kNone;
    const unsigned peers = __match_any_sync(kFull, cand ? cu : LaneSentinel(lane)) & gmask;
    const bool leader = cand && int(lane) == __ffs(peers) - 1;
    double S;
    if (kInt) {
      const int xi = cand ? (WeightToInt(wt) - a.ioffset) : 0;
      S = static_cast<double>(GroupSumInt(peers, xi, a.w == nullptr, leader, reinterpret_cast<int*>(stage[warp])));
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
      val = ValOf(a, x, change, S, LdK<kAsync>(a.K + cu));
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
    if (!kAsync) mb.Add(&a.ctr->movers, a.movers, append, x.v);
  }
  if (!kAsync) mb.Flush(&a.ctr->movers, a.movers);
  FlushFamily(a, kFamGroup, fam_e, fam_v);
}

// ---------------------------------------------------------------------------
// One warp per vertex, degree <= 1000, shared-memory hash of HC slots.
// Chunks of 32 entries in adjacency order; per chunk the leader of each
// cluster id adds its peers one by one (FP64) onto the slot's running sum,
// which keeps the reference's adjacency-order summation exactly.
// ---------------------------------------------------------------------------
constexpr int kWarpKernelWarps = 4;
constexpr int kCertUnroll = 4;  // chunks of 32 entries loaded together
constexpr int kCertRegRounds = 1;  // candidates per lane held in registers

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
  __shared__ uint32_t mover_buf[kWarpKernelWarps][64];
  WarpMoverBuffer mb{mover_buf[threadIdx.x >> 5]};
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
  unsigned long long fam_e = 0, fam_v = 0;
  for (int i = lane; i < HC; i += 32) {
    keys[i] = kNone;
    vals[i] = 0ull;
  }
  if (lane == 0) *used_count = 0;
  __syncwarp();
  // The next vertex id is loaded one iteration ahead and each vertex's
  // entries kCertUnroll chunks at a time (the loads of the chunks are in
  // flight together; the sums still run chunk by chunk, in adjacency order).
  const uint64_t wstride = uint64_t(gridDim.x) * kWarpKernelWarps;
  uint64_t idx = uint64_t(blockIdx.x) * kWarpKernelWarps + warp;
  uint32_t vid = idx < count ? list[start + idx] : 0u;
  for (; idx < count; idx += wstride) {
    const uint64_t nidx = idx + wstride;
    const uint32_t nvid = nidx < count ? list[start + nidx] : 0u;
    if (!InFront(a, vid)) {
      vid = nvid;
      continue;
    }
    const VertexCtx x = LoadVertex<kAsync>(a, vid);
    vid = nvid;
    if (lane == 0) {
      fam_e += x.d;
      fam_v += 1;
    }
    for (uint32_t e00 = 0; e00 < x.d; e00 += 32 * kCertUnroll) {
      uint32_t uu[kCertUnroll], cc[kCertUnroll];
      float ww[kCertUnroll];
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) {
        const uint32_t e = e00 + 32 * k + lane;
        uu[k] = x.v;
        ww[k] = 0.f;
        if (e < x.d) {
          uu[k] = a.nbr[x.b + e];
          ww[k] = a.w ? a.w[x.b + e] : 1.0f;
        }
      }
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) cc[k] = uu[k] != x.v ? LdC<kAsync>(a.C + uu[k]) : kNone;
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) {
      if (e00 + 32 * k >= x.d) break;  // warp-uniform
      const uint32_t u = uu[k];
      const float wt = ww[k];
      const bool cand = u != x.v;
      const uint32_t cu = cc[k];
      const unsigned peers = __match_any_sync(kFull, cand ? cu : LaneSentinel(lane));
      const bool leader = cand && int(lane) == __ffs(peers) - 1;
      uint32_t slot = kNone;
      bool ins = false;
      if (leader) {
        slot = FindOrInsertT<false>(keys, HC, cu, &ins);
        if (slot == kNone) atomicExch(&a.ctr->error, kErrHashFull);
      }
      const unsigned im = __ballot_sync(kFull, ins);
      if (im) {
        uint32_t base = 0;
        const int ld = __ffs(im) - 1;
        if (int(lane) == ld) base = atomicAdd(used_count, uint32_t(__popc(im)));
        base = __shfl_sync(kFull, base, ld);
        if (ins) used[base + __popc(im & LaneMaskLt())] = static_cast<uint16_t>(slot);
      }
      if (kInt) {
        const int xi = cand ? (WeightToInt(wt) - a.ioffset) : 0;
        const int S = GroupSumInt(peers, xi, a.w == nullptr, leader, reinterpret_cast<int*>(stage));
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
      const double val = ValOf(a, x, change, S, LdK<kAsync>(a.K + key));
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
    if (!kAsync) mb.Add(&a.ctr->movers, a.movers, append, x.v);
    __syncwarp();
    if (lane == 0) *used_count = 0;
    __syncwarp();
  }
  if (!kAsync) mb.Flush(&a.ctr->movers, a.movers);
  FlushFamily(a, kFamWarp, fam_e, fam_v);
}

// ---------------------------------------------------------------------------
// INT-mode synchronous rounds: certified decisions (certify.cuh).  The FP32
// pre-filter selects the survivors; when they form one (S, K) class and the
// FP32 bounds decide the move, no FP64 instruction runs for the vertex.
// Otherwise -- and always in replay mode, where the exact values are outputs
// -- the exact FP64 values decide; in replay mode a certified decision that
// differs from the FP64 one raises kErrCertMismatch (a self-check).
// ---------------------------------------------------------------------------
// Exact FP64 fallbacks of the certified kernels.  They are separate
// non-inlined functions so that the compiler cannot hoist their FP64
// arithmetic onto the certified path (an FP64 warp instruction costs ~19
// SM cycles on this GPU).  Both return whether the vertex must be appended
// to the movers list; in replay mode they also run the self-check.
template <int G>
__device__ __noinline__ bool GroupExact(const BMArgs& a, const VertexCtx& x, bool fp64, bool contender, unsigned gl,
                                        int T, int S, double KD, uint32_t cu, bool replay, int cres,
                                        uint32_t cmove) {
  double change = 0.0, val = -CUDART_INF;
  uint32_t id = kNone;
  if (fp64) {
    change = ChangeOf(a, x, static_cast<double>(T));
    if (contender) {
      val = ValOf(a, x, change, static_cast<double>(S), KD);
      id = cu;
    }
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
  if (fp64 && gl == 0) {
    append = Decide<false>(a, x, val, id, change);
    if (replay && cres != kUncertain && a.out_moves && a.out_moves[x.v] != cmove)
      atomicExch(&a.ctr->error, kErrCertMismatch);
  }
  return append;
}

template <int HC, typename V>
__device__ __noinline__ bool WarpExact(const BMArgs& a, const VertexCtx& x, V T, const uint32_t* keys,
                                       const V* vals, const uint16_t* used, uint32_t nused, bool replay, int cres,
                                       uint32_t cmove) {
  const unsigned lane = LaneId();
  const double change = ChangeOf(a, x, static_cast<double>(T));
  double best = -CUDART_INF;
  uint32_t bid = kNone;
  for (uint32_t i = lane; i < nused; i += 32) {
    const uint32_t slot = used[i];
    if (slot == 0xFFFFu) continue;
    const uint32_t key = keys[slot];
    const double val = ValOf(a, x, change, static_cast<double>(vals[slot]), a.K[key]);
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
  bool append = false;
  if (lane == 0) {
    append = Decide<false>(a, x, best, bid, change);
    if (replay && cres != kUncertain && a.out_moves && a.out_moves[x.v] != cmove)
      atomicExch(&a.ctr->error, kErrCertMismatch);
  }
  return append;
}

template <int G>
__global__ void __launch_bounds__(256) CertGroupKernel(BMArgs a, const uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ bin_counts,
                                                      const uint32_t* __restrict__ bin_starts, int bin) {
  __shared__ int stage[8][32];
  __shared__ uint32_t mover_buf[8][64];
  WarpMoverBuffer mb{mover_buf[threadIdx.x >> 5]};
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  constexpr unsigned kVpw = 32 / G;
  const unsigned g = lane / G, gl = lane % G;
  const unsigned gmask = G == 32 ? kFull : (((1u << G) - 1u) << (g * G));
  unsigned long long fam_e = 0, fam_v = 0;
  const bool replay = a.out_target != nullptr;
  const bool unit = a.w == nullptr;
  const uint64_t stride = uint64_t(gridDim.x) * 8 * kVpw;
  // Vertex ids are loaded one iteration ahead (latency-bound kernel).
  uint64_t base = (uint64_t(blockIdx.x) * 8 + warp) * kVpw;
  uint32_t vid = base + g < count ? list[start + base + g] : 0u;
  for (; base < count; base += stride) {
    const uint64_t idx = base + g;
    const uint32_t nvid = base + stride + g < count ? list[start + base + stride + g] : 0u;
    bool vvalid = idx < count;
    VertexCtx x{};
    if (vvalid) {
      vvalid = InFront(a, vid);
      if (vvalid) x = LoadVertex<false>(a, vid);
    }
    vid = nvid;
    if (__ballot_sync(kFull, vvalid) == 0) continue;
    if (vvalid && gl == 0) {
      fam_e += x.d;
      fam_v += 1;
    }
    const bool has = vvalid && gl < x.d;
    uint32_t u = x.v;
    float wt = 0.f;
    if (has) {
      u = a.nbr[x.b + gl];
      wt = a.w ? a.w[x.b + gl] : 1.0f;
    }
    const bool cand = has && u != x.v;
    const uint32_t cu = cand ? __ldg(a.C + u) : kNone;
    const unsigned peers = __match_any_sync(kFull, cand ? cu : LaneSentinel(lane)) & gmask;
    const bool leader = cand && int(lane) == __ffs(peers) - 1;
    const int xi = cand ? (WeightToInt(wt) - a.ioffset) : 0;
    const int S = GroupSumInt(peers, xi, unit, leader, stage[warp]);
    const unsigned tmask = __ballot_sync(kFull, leader && cu == x.c) & gmask;
    const int Tsh = __shfl_sync(kFull, S, tmask ? __ffs(tmask) - 1 : int(lane));
    const int T = tmask ? Tsh : 0;  // group sums stay below 2^29 in INT mode
    int smax = leader ? S : INT_MIN;
    if constexpr (G == 32) {
      smax = __reduce_max_sync(kFull, smax);
    } else {
#pragma unroll
      for (int o = G / 2; o >= 1; o >>= 1) smax = max(smax, __shfl_xor_sync(kFull, smax, o));
    }
    const float k32 = vvalid ? a.kf[x.v] : 0.f;
    const float Kc32 = vvalid ? a.Kf[x.c] : 0.f;
    const ChangeApproxT<int> ca = ApproxChange<int>(Res32Of(a, x.v), a.int_nw != 0, k32, Kc32, T);
    const float cabs = ChangeAbsBound(ca);
    // FP32 pre-filter over the group's leaders.
    FilterVal f{0.f, 0.f, false};
    float KfD = 0.f;
    float lo = -CUDART_INF_F;
    if (leader) {
      KfD = a.Kf[cu];
      f = FilterOf<int>(Res32Of(a, x.v), k32, KfD, S, smax, cabs);
      if (f.sane) lo = __fsub_rn(f.Y, f.e);
    }
    float U = lo;
    if constexpr (G == 32) {
      U = WarpMaxFinite(U);
    } else {
#pragma unroll
      for (int o = G / 2; o >= 1; o >>= 1) U = fmaxf(U, __shfl_xor_sync(kFull, U, o));
    }
    const bool contender = leader && (!f.sane || __fadd_rn(f.Y, f.e) >= U);
    // The leading (S, K) class of the contenders and the trailing one.
    LexKeyT<int> lead, tail;
    double KD = 0.0;
    if (contender) {
      KD = a.K[cu];
      const unsigned long long ko = KOrder(KD);
      lead.Keep(S, ko, cu);
      tail.Keep(-S, ~ko, cu);
    }
    bool single;
    if constexpr (G == 32) {
      single = LexWarpLeadInt(lead, tail);
    } else {
      LexGroupReduce<G>(lead);
      LexGroupReduce<G>(tail);
      single = lead.id == kNone || (-tail.S == lead.S && ~tail.K == lead.K);
    }
    int cres = kUncertain;
    uint32_t ctarget = kNone;
    if (vvalid && single) {
      const float KfA = lead.id != kNone ? a.Kf[lead.id] : 0.f;
      cres = CertifyDecision<int>(ca, Res32Of(a, x.v), k32, lead.id != kNone, lead.S, KfA, lead.id, a.n, &ctarget);
    }
    const uint32_t cmove = cres == kUncertain ? kNone : CertifiedMove(a, x, ctarget, cres == kCertMove);
    const bool fp64 = vvalid && (replay || cres == kUncertain);
    bool append = false;
    if (vvalid && !fp64 && gl == 0) append = ApplyCertified(a, x, cmove);
    if (__ballot_sync(kFull, fp64)) {
      const bool app = GroupExact<G>(a, x, fp64, contender, gl, T, S, KD, cu, replay, cres, cmove);
      append = append || app;
    }
    mb.Add(&a.ctr->movers, a.movers, append, x.v);
  }
  mb.Flush(&a.ctr->movers, a.movers);
  FlushFamily(a, kFamGroup, fam_e, fam_v);
}

// Per-warp shared bytes: vals HC*sizeof(V), keys HC*4, stage 32*4, used
// HC/2 * 2, count 16.
template <int HC, typename V>
__host__ __device__ constexpr size_t CertWarpStride() {
  return size_t(HC) * (sizeof(V) + 5) + 32 * 4 + 16;
}
template <int HC, typename V>
constexpr size_t CertWarpSmem() {
  return size_t(kWarpKernelWarps) * CertWarpStride<HC, V>();
}

// V: int when every cluster sum fits in 32 bits (narrow), else long long.
// Every entry inserts its cluster itself (atomicCAS claims a slot) and adds
// its integer weight with a shared-memory atomic: INT-mode sums are exact in
// any order, and grouping equal clusters first with match.any cost more than
// the atomics it saves.
template <int HC, typename V>
__global__ void __launch_bounds__(kWarpKernelWarps * 32) CertWarpKernel(BMArgs a, const uint32_t* __restrict__ list,
                                                                       const uint32_t* __restrict__ bin_counts,
                                                                       const uint32_t* __restrict__ bin_starts,
                                                                       int bin) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t mover_buf[kWarpKernelWarps][64];
  WarpMoverBuffer mb{mover_buf[threadIdx.x >> 5]};
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned lane = LaneId(), warp = threadIdx.x >> 5;
  unsigned char* base = smem + size_t(warp) * CertWarpStride<HC, V>();
  V* vals = reinterpret_cast<V*>(base);
  uint32_t* keys = reinterpret_cast<uint32_t*>(base + size_t(HC) * sizeof(V));
  uint16_t* used = reinterpret_cast<uint16_t*>(base + size_t(HC) * (sizeof(V) + 4) + 32 * 4);
  unsigned long long fam_e = 0, fam_v = 0;
  const bool replay = a.out_target != nullptr;
  for (int i = lane; i < HC; i += 32) {
    keys[i] = kNone;
    vals[i] = 0;
  }
  __syncwarp();
  // The next vertex id is loaded one iteration ahead, and each vertex's
  // entries are loaded kCertUnroll chunks at a time (up to 128 neighbour ids
  // and their cluster ids in flight per warp): the kernel is bound by the
  // latency of the dependent loads list -> offsets -> neighbours -> clusters.
  const uint64_t wstride = uint64_t(gridDim.x) * kWarpKernelWarps;
  uint64_t idx = uint64_t(blockIdx.x) * kWarpKernelWarps + warp;
  uint32_t vid = idx < count ? list[start + idx] : 0u;
  for (; idx < count; idx += wstride) {
    const uint64_t nidx = idx + wstride;
    const uint32_t nvid = nidx < count ? list[start + nidx] : 0u;
    if (!InFront(a, vid)) {
      vid = nvid;
      continue;
    }
    const VertexCtx x = LoadVertex<false>(a, vid);
    vid = nvid;
    if (lane == 0) {
      fam_e += x.d;
      fam_v += 1;
    }
    uint32_t nused = 0;  // used[] entries (warp-uniform)
    int tpart = 0;       // this lane's part of T (entries in the vertex's own cluster)
    for (uint32_t e0 = 0; e0 < x.d; e0 += 32 * kCertUnroll) {
      uint32_t uu[kCertUnroll], cc[kCertUnroll];
      float ww[kCertUnroll];
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) {
        const uint32_t e = e0 + 32 * k + lane;
        uu[k] = x.v;
        ww[k] = 0.f;
        if (e < x.d) {
          uu[k] = a.nbr[x.b + e];
          ww[k] = a.w ? a.w[x.b + e] : 1.0f;
        }
      }
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) cc[k] = uu[k] != x.v ? __ldg(a.C + uu[k]) : kNone;
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) {
      if (e0 + 32 * k >= x.d) break;  // warp-uniform
      const float wt = ww[k];
      const bool cand = uu[k] != x.v;
      const uint32_t cu = cc[k];
      uint32_t slot = kNone;
      bool ins = false;
      if (cand) {
        slot = FindOrInsertT<false>(keys, HC, cu, &ins);
        if (slot == kNone) atomicExch(&a.ctr->error, kErrHashFull);
      }
      const unsigned im = __ballot_sync(kFull, ins);
      if (im) {
        if (ins) used[nused + __popc(im & LaneMaskLt())] = static_cast<uint16_t>(slot);
        nused += __popc(im);
      }
      const int xi = cand ? (WeightToInt(wt) - a.ioffset) : 0;
      if (cand && cu == x.c) tpart += xi;
      if (slot != kNone) {
        if constexpr (sizeof(V) == 4) atomicAdd(reinterpret_cast<int*>(&vals[slot]), xi);
        else atomicAdd(reinterpret_cast<unsigned long long*>(&vals[slot]), static_cast<unsigned long long>(static_cast<long long>(xi)));
      }
      __syncwarp();
      }
    }
    // T: the lanes' own-cluster parts (a lane's part is at most
    // ceil(1000 / 32) weights of |w - offset| <= 2^22, so it fits an int).
    V T;
    if constexpr (sizeof(V) == 4) {
      T = __reduce_add_sync(kFull, tpart);
    } else {
      T = tpart;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) T += __shfl_xor_sync(kFull, T, o);
    }
    const float r32 = Res32Of(a, x.v);
    const float k32 = a.kf[x.v];
    const ChangeApproxT<V> ca = ApproxChange<V>(r32, a.int_nw != 0, k32, a.Kf[x.c], T);
    const float cabs = ChangeAbsBound(ca);
    // The first kCertRegRounds candidates of each lane (i = lane + 32 r) keep
    // their slot, sum, Kf and filter value in registers across the passes;
    // any further ones are read again.
    uint32_t rslot[kCertRegRounds];
    V rS[kCertRegRounds];
    float rKf[kCertRegRounds];
    V vmax = sizeof(V) == 4 ? V(INT_MIN) : V(LLONG_MIN);
#pragma unroll
    for (int r = 0; r < kCertRegRounds; ++r) {
      const uint32_t i = lane + 32 * r;
      rslot[r] = 0xFFFFu;
      rS[r] = 0;
      rKf[r] = 0.f;
      if (i < nused) {
        rslot[r] = used[i];
        rS[r] = vals[rslot[r]];
        rKf[r] = a.Kf[keys[rslot[r]]];
        vmax = max(vmax, rS[r]);
      }
    }
    for (uint32_t i = lane + 32 * kCertRegRounds; i < nused; i += 32) vmax = max(vmax, vals[used[i]]);
    if constexpr (sizeof(V) == 4) {
      vmax = __reduce_max_sync(kFull, vmax);
    } else {
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) vmax = max(vmax, __shfl_xor_sync(kFull, vmax, o));
    }
    const V smax = vmax;
    float U = -CUDART_INF_F;
    // The two largest upper ends (Y + e; +inf outside the error model) of
    // this lane's candidates and the index of the largest: when the second
    // is below U, only that one can be a contender.  Kept for the bins of
    // more than 128 entries, where lanes hold several candidates (in the
    // 33-128 bin it costs about what it saves).
    constexpr bool kTop2 = HC >= 512;
    float hi1 = -CUDART_INF_F, hi2 = -CUDART_INF_F;
    uint32_t i1 = kNone;
    FilterVal rf[kCertRegRounds];
#pragma unroll
    for (int r = 0; r < kCertRegRounds; ++r) {
      rf[r].sane = false;
      if (lane + 32 * r < nused) {
        rf[r] = FilterOf<V>(r32, k32, rKf[r], rS[r], smax, cabs);
        if (rf[r].sane) U = fmaxf(U, __fsub_rn(rf[r].Y, rf[r].e));
        if (kTop2) KeepTop2(hi1, hi2, i1, rf[r].sane ? __fadd_rn(rf[r].Y, rf[r].e) : CUDART_INF_F, lane + 32 * r);
      }
    }
    for (uint32_t i = lane + 32 * kCertRegRounds; i < nused; i += 32) {
      const uint32_t slot = used[i];
      const FilterVal f = FilterOf<V>(r32, k32, a.Kf[keys[slot]], vals[slot], smax, cabs);
      if (f.sane) U = fmaxf(U, __fsub_rn(f.Y, f.e));
      if (kTop2) KeepTop2(hi1, hi2, i1, f.sane ? __fadd_rn(f.Y, f.e) : CUDART_INF_F, i);
    }
    U = WarpMaxFinite(U);
    LexKeyT<V> lead, tail;
    // The contenders are the candidates with Y + e >= U (all when U = -inf).
    const bool skip = kTop2 && hi2 < U;
    if (skip) {
      // At most candidate i1 is a contender: the others are cleared and
      // marked without evaluating them again.
      for (uint32_t i = lane; i < nused; i += 32) {
        const uint32_t slot = used[i];
        if (i == i1 && !(hi1 < U)) {
          const uint32_t key = keys[slot];
          const V S = vals[slot];
          const unsigned long long ko = KOrder(a.K[key]);
          lead.Keep(S, ko, key);
          tail.Keep(-S, ~ko, key);
          continue;
        }
        keys[slot] = kNone;
        vals[slot] = 0;
        used[i] = 0xFFFFu;
      }
    }
    const uint32_t rescan_end = skip ? 0u : nused;
#pragma unroll
    for (int r = 0; r < kCertRegRounds; ++r) {
      const uint32_t i = lane + 32 * r;
      if (i >= rescan_end) continue;
      const uint32_t slot = rslot[r];
      if (rf[r].sane && __fadd_rn(rf[r].Y, rf[r].e) < U) {
        keys[slot] = kNone;  // not a contender: cleared now, skipped later
        vals[slot] = 0;
        used[i] = 0xFFFFu;
        continue;
      }
      const uint32_t key = keys[slot];
      const unsigned long long ko = KOrder(a.K[key]);
      lead.Keep(rS[r], ko, key);
      tail.Keep(-rS[r], ~ko, key);
    }
    for (uint32_t i = lane + 32 * kCertRegRounds; i < rescan_end; i += 32) {
      const uint32_t slot = used[i];
      const uint32_t key = keys[slot];
      const FilterVal f = FilterOf<V>(r32, k32, a.Kf[key], vals[slot], smax, cabs);
      if (f.sane && __fadd_rn(f.Y, f.e) < U) {
        keys[slot] = kNone;  // not a contender: cleared now, skipped later
        vals[slot] = 0;
        used[i] = 0xFFFFu;
        continue;
      }
      const unsigned long long ko = KOrder(a.K[key]);
      const V S = vals[slot];
      lead.Keep(S, ko, key);
      tail.Keep(-S, ~ko, key);
    }
    bool single;
    if constexpr (sizeof(V) == 4) {
      single = LexWarpLeadInt(lead, tail);
    } else {
      LexGroupReduce<32>(lead);
      LexGroupReduce<32>(tail);
      single = lead.id == kNone || (-tail.S == lead.S && ~tail.K == lead.K);
    }
    int cres = kUncertain;
    uint32_t ctarget = kNone;
    if (single) {
      const float KfA = lead.id != kNone ? a.Kf[lead.id] : 0.f;
      cres = CertifyDecision<V>(ca, r32, k32, lead.id != kNone, lead.S, KfA, lead.id, a.n, &ctarget);
    }
    const uint32_t cmove = cres == kUncertain ? kNone : CertifiedMove(a, x, ctarget, cres == kCertMove);
    bool append = false;
    if (replay || cres == kUncertain) {
      append = WarpExact<HC, V>(a, x, T, keys, vals, used, nused, replay, cres, cmove);
    } else if (lane == 0) {
      append = ApplyCertified(a, x, cmove);
    }
    __syncwarp();
    // Clear the table through the key list (used[] may hold 0xFFFF marks).
    for (uint32_t i = lane; i < nused; i += 32) {
      const uint32_t slot = used[i];
      if (slot != 0xFFFFu) {
        keys[slot] = kNone;
        vals[slot] = 0;
      }
    }
    mb.Add(&a.ctr->movers, a.movers, append, x.v);
    __syncwarp();
  }
  mb.Flush(&a.ctr->movers, a.movers);
  FlushFamily(a, kFamWarp, fam_e, fam_v);
}

// ---------------------------------------------------------------------------
// One CTA of kCtaWarps warps per vertex (degree 129-1000, INT mode, sync):
// the same certified decision as CertWarpKernel, with the row and the
// epilogue split over the CTA's warps.  One table of HC slots per CTA
// instead of one per warp, so several times more vertices are in flight per
// SM for the same shared memory, and each vertex's chain of dependent loads
// and candidate loops is kCtaWarps times shorter.  Inserts claim slots with
// atomicCAS and add with shared-memory atomics (any order: INT-mode sums
// are exact); the warp maxima and lexicographic leaders are combined through
// shared memory.  An uncertain (or replayed) vertex takes WarpExact on warp 0
// over the whole table, exactly as in the warp kernel.
// ---------------------------------------------------------------------------
constexpr int kCtaWarps = 4;

template <int HC, typename V>
constexpr size_t CertCtaSmem() {
  return size_t(HC) * (sizeof(V) + 4 + 2);  // vals, keys, used
}

template <typename V>
__device__ __forceinline__ V WarpMaxV(V x) {
  if constexpr (sizeof(V) == 4) {
    return __reduce_max_sync(kFull, x);
  } else {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) x = max(x, __shfl_xor_sync(kFull, x, o));
    return x;
  }
}

template <int HC, typename V>
__global__ void __launch_bounds__(kCtaWarps * 32) CertCtaKernel(BMArgs a, const uint32_t* __restrict__ list,
                                                               const uint32_t* __restrict__ bin_counts,
                                                               const uint32_t* __restrict__ bin_starts, int bin) {
  constexpr int BT = kCtaWarps * 32;
  extern __shared__ __align__(16) unsigned char smem[];
  V* vals = reinterpret_cast<V*>(smem);
  uint32_t* keys = reinterpret_cast<uint32_t*>(smem + size_t(HC) * sizeof(V));
  uint16_t* used = reinterpret_cast<uint16_t*>(smem + size_t(HC) * (sizeof(V) + 4));
  __shared__ uint32_t s_nused;
  __shared__ V s_max[kCtaWarps];
  __shared__ float s_u[kCtaWarps];
  __shared__ V s_ls[kCtaWarps], s_ts[kCtaWarps];
  __shared__ unsigned long long s_lk[kCtaWarps], s_tk[kCtaWarps];
  __shared__ uint32_t s_li[kCtaWarps], s_ti[kCtaWarps];
  __shared__ uint32_t mover_buf[64];  // warp 0's
  WarpMoverBuffer mb{mover_buf};
  const uint32_t count = bin_counts[bin];
  const uint32_t start = bin_starts[bin];
  const unsigned tid = threadIdx.x, lane = LaneId(), warp = tid >> 5;
  unsigned long long fam_e = 0, fam_v = 0;
  const bool replay = a.out_target != nullptr;
  for (int i = tid; i < HC; i += BT) {
    keys[i] = kNone;
    vals[i] = 0;
  }
  if (tid == 0) s_nused = 0;
  __syncthreads();
  uint32_t vid = blockIdx.x < count ? list[start + blockIdx.x] : 0u;
  for (uint64_t idx = blockIdx.x; idx < count; idx += gridDim.x) {
    const uint64_t nidx = idx + gridDim.x;
    const uint32_t nvid = nidx < count ? list[start + nidx] : 0u;
    if (!InFront(a, vid)) {  // uniform over the CTA
      vid = nvid;
      continue;
    }
    const VertexCtx x = LoadVertex<false>(a, vid);
    vid = nvid;
    if (tid == 0) {
      fam_e += x.d;
      fam_v += 1;
    }
    for (uint32_t e0 = 0; e0 < x.d; e0 += BT * kCertUnroll) {
      uint32_t uu[kCertUnroll], cc[kCertUnroll];
      float ww[kCertUnroll];
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) {
        const uint32_t e = e0 + BT * k + tid;
        uu[k] = x.v;
        ww[k] = 0.f;
        if (e < x.d) {
          uu[k] = a.nbr[x.b + e];
          ww[k] = a.w ? a.w[x.b + e] : 1.0f;
        }
      }
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) cc[k] = uu[k] != x.v ? __ldg(a.C + uu[k]) : kNone;
#pragma unroll
      for (int k = 0; k < kCertUnroll; ++k) {
        if (e0 + BT * k + 32 * warp >= x.d) break;  // uniform over the warp
        const bool cand = uu[k] != x.v;
        const uint32_t cu = cc[k];
        uint32_t slot = kNone;
        bool ins = false;
        if (cand) {
          slot = FindOrInsertT<false>(keys, HC, cu, &ins);
          if (slot == kNone) atomicExch(&a.ctr->error, kErrHashFull);
        }
        const unsigned im = __ballot_sync(kFull, ins);
        if (im) {
          const int first = __ffs(im) - 1;
          uint32_t base = 0;
          if (int(lane) == first) base = atomicAdd(&s_nused, uint32_t(__popc(im)));
          base = __shfl_sync(kFull, base, first);
          if (ins) used[base + __popc(im & LaneMaskLt())] = static_cast<uint16_t>(slot);
        }
        const int xi = cand ? (WeightToInt(ww[k]) - a.ioffset) : 0;
        if (slot != kNone) {
          if constexpr (sizeof(V) == 4)
            atomicAdd(reinterpret_cast<int*>(&vals[slot]), xi);
          else
            atomicAdd(reinterpret_cast<unsigned long long*>(&vals[slot]),
                      static_cast<unsigned long long>(static_cast<long long>(xi)));
        }
      }
    }
    __syncthreads();  // table complete
    const uint32_t nused = s_nused;
    V T = 0;
    {
      const uint32_t slot = FindT<false>(keys, HC, x.c);
      if (slot != kNone) T = vals[slot];
    }
    const float k32 = a.kf[x.v];
    const ChangeApproxT<V> ca = ApproxChange<V>(Res32Of(a, x.v), a.int_nw != 0, k32, a.Kf[x.c], T);
    const float cabs = ChangeAbsBound(ca);
    V vmax = sizeof(V) == 4 ? V(INT_MIN) : V(LLONG_MIN);
    for (uint32_t i = tid; i < nused; i += BT) vmax = max(vmax, vals[used[i]]);
    vmax = WarpMaxV<V>(vmax);
    if (lane == 0) s_max[warp] = vmax;
    __syncthreads();
    V smax = s_max[0];
#pragma unroll
    for (int w = 1; w < kCtaWarps; ++w) smax = max(smax, s_max[w]);
    float U = -CUDART_INF_F;
    float hi1 = -CUDART_INF_F, hi2 = -CUDART_INF_F;  // KeepTop2 of this thread's candidates
    uint32_t i1 = kNone;
    for (uint32_t i = tid; i < nused; i += BT) {
      const uint32_t slot = used[i];
      const FilterVal f = FilterOf<V>(Res32Of(a, x.v), k32, a.Kf[keys[slot]], vals[slot], smax, cabs);
      if (f.sane) U = fmaxf(U, __fsub_rn(f.Y, f.e));
      KeepTop2(hi1, hi2, i1, f.sane ? __fadd_rn(f.Y, f.e) : CUDART_INF_F, i);
    }
    U = WarpMaxFinite(U);
    if (lane == 0) s_u[warp] = U;
    __syncthreads();
    U = s_u[0];
#pragma unroll
    for (int w = 1; w < kCtaWarps; ++w) U = fmaxf(U, s_u[w]);
    LexKeyT<V> lead, tail;
    // The contenders are the candidates with Y + e >= U (all when U = -inf);
    // when this thread's runner-up is below U, at most its candidate i1 is
    // one, and the others are cleared and marked without a second
    // evaluation.
    const bool rescan = !(hi2 < U);
    if (!rescan) {
      for (uint32_t i = tid; i < nused; i += BT) {
        const uint32_t slot = used[i];
        if (i == i1 && !(hi1 < U)) {
          const uint32_t key = keys[slot];
          const V S = vals[slot];
          const unsigned long long ko = KOrder(a.K[key]);
          lead.Keep(S, ko, key);
          tail.Keep(-S, ~ko, key);
          continue;
        }
        keys[slot] = kNone;
        vals[slot] = 0;
        used[i] = 0xFFFFu;
      }
    }
    for (uint32_t i = tid; i < (rescan ? nused : 0u); i += BT) {
      const uint32_t slot = used[i];
      const uint32_t key = keys[slot];
      const FilterVal f = FilterOf<V>(Res32Of(a, x.v), k32, a.Kf[key], vals[slot], smax, cabs);
      if (f.sane && __fadd_rn(f.Y, f.e) < U) {
        keys[slot] = kNone;  // not a contender: cleared now, skipped later
        vals[slot] = 0;
        used[i] = 0xFFFFu;
        continue;
      }
      const unsigned long long ko = KOrder(a.K[key]);
      const V S = vals[slot];
      lead.Keep(S, ko, key);
      tail.Keep(-S, ~ko, key);
    }
    if constexpr (sizeof(V) == 4) {
      LexWarpLeaderInt(lead);
      LexWarpLeaderInt(tail);
    } else {
      LexGroupReduce<32>(lead);
      LexGroupReduce<32>(tail);
    }
    if (lane == 0) {
      s_ls[warp] = lead.S;
      s_lk[warp] = lead.K;
      s_li[warp] = lead.id;
      s_ts[warp] = tail.S;
      s_tk[warp] = tail.K;
      s_ti[warp] = tail.id;
    }
    __syncthreads();
    if (warp == 0) {
      LexKeyT<V> L, Tl;
#pragma unroll
      for (int w = 0; w < kCtaWarps; ++w) {
        L.Keep(s_ls[w], s_lk[w], s_li[w]);
        Tl.Keep(s_ts[w], s_tk[w], s_ti[w]);
      }
      // One (S, K) class among the contenders iff the lowest-ranked one
      // (Tl: smallest S, then largest K) is in the leader's class.
      const bool single = L.id == kNone || (-Tl.S == L.S && ~Tl.K == L.K);
      int cres = kUncertain;
      uint32_t ctarget = kNone;
      if (single) {
        const float KfA = L.id != kNone ? a.Kf[L.id] : 0.f;
        cres = CertifyDecision<V>(ca, Res32Of(a, x.v), k32, L.id != kNone, L.S, KfA, L.id, a.n, &ctarget);
      }
      const uint32_t cmove = cres == kUncertain ? kNone : CertifiedMove(a, x, ctarget, cres == kCertMove);
      bool append = false;
      if (replay || cres == kUncertain) {
        append = WarpExact<HC, V>(a, x, T, keys, vals, used, nused, replay, cres, cmove);
      } else if (lane == 0) {
        append = ApplyCertified(a, x, cmove);
      }
      mb.Add(&a.ctr->movers, a.movers, append, x.v);
    }
    __syncthreads();  // the table is read by WarpExact up to here
    for (uint32_t i = tid; i < nused; i += BT) {
      const uint32_t slot = used[i];
      if (slot != 0xFFFFu) {
        keys[slot] = kNone;
        vals[slot] = 0;
      }
    }
    if (tid == 0) s_nused = 0;
    __syncthreads();
  }
  if (warp == 0) {
    mb.Flush(&a.ctr->movers, a.movers);
    FlushFamily(a, kFamWarp, fam_e, fam_v);
  }
}

// Sets the kernel's dynamic shared-memory limit and queries its resident
// CTAs per SM once per process (the runtime calls take a lock that
// serialises concurrent contexts).  Each kernel is launched with one fixed
// shared-memory size.
template <class K>
Status SetSmem(K kernel, size_t bytes, int threads, int* per_sm) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> occ;
  std::lock_guard<std::mutex> lk(mu);
  auto it = occ.find(reinterpret_cast<const void*>(kernel));
  if (it != occ.end()) {
    *per_sm = it->second;
    return Status::Ok();
  }
  PCC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
  int n = 0;
  PCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, bytes));
  occ[reinterpret_cast<const void*>(kernel)] = n;
  *per_sm = n;
  return Status::Ok();
}

template <bool kInt, bool kAsync>
Status LaunchAll(Context* ctx, const BMArgs& a, const uint32_t* list, const uint32_t* counts,
                 const uint32_t* starts, const uint32_t* host_counts, uint32_t max_deg, int families) {
  const unsigned sms = unsigned(ctx->num_sms);
  const LaunchTuning tune = TuningFor(ctx, a.n);
  // Resident CTAs of one wave scaled by the tuned wave count.
  auto waves = [&](unsigned one_wave) -> unsigned {
    return std::max(1u, unsigned(double(one_wave) * double(tune.grid_waves) + 0.5));
  };
  auto grid = [&](int bin, uint64_t per_block, unsigned cap) -> unsigned {
    if (!host_counts) return cap;
    return Blocks(host_counts[bin], unsigned(per_block), cap);
  };
  // Warp bins above the tuned degree run one CTA per vertex (INT mode).
  auto on_cta = [&](int bin) {
    return bin >= kBinW128 && bin <= kBinW1000 && kBinMaxDeg[bin] > tune.cta_min_degree;
  };
  // Lane-group bins above the tuned degree run on the 256-slot warp kernel,
  // as part of the warp family (launched, timed and counted with it).
  auto routed = [&](int bin) { return bin <= kBinG32 && kBinMaxDeg[bin] > tune.group_max_degree; };
  auto want = [&](int bin) {
    const int fam = bin <= kBinG32 && !routed(bin) ? kLaunchGroups : kLaunchWarps;
    return (families & fam) && (!host_counts || host_counts[bin] > 0);
  };
  cudaStream_t st = ctx->stream;
  constexpr bool kCert = kInt && !kAsync;
  // Grid-stride kernels: at most one wave of resident CTAs, so no partial
  // last wave.
  auto warp_bin = [&](auto k, size_t smem, int bin, unsigned cap) -> Status {
    if (!want(bin)) return Status::Ok();
    int per_sm = 0;
    PCC_RETURN_IF_ERROR(SetSmem(k, smem, kWarpKernelWarps * 32, &per_sm));
    if (per_sm > 0) cap = sms * unsigned(per_sm);
    k<<<grid(bin, kWarpKernelWarps, waves(cap)), kWarpKernelWarps * 32, smem, st>>>(a, list, counts, starts, bin);
    PCC_COUNT(1);
    return Status::Ok();
  };
  auto cta_bin = [&](auto k, size_t smem, int bin) -> Status {
    if (!want(bin)) return Status::Ok();
    int per_sm = 0;
    PCC_RETURN_IF_ERROR(SetSmem(k, smem, kCtaWarps * 32, &per_sm));
    const unsigned cap = sms * unsigned(per_sm > 0 ? per_sm : 4);
    k<<<grid(bin, 1, waves(cap)), kCtaWarps * 32, smem, st>>>(a, list, counts, starts, bin);
    PCC_COUNT(1);
    return Status::Ok();
  };
  // A certified warp bin on the warp kernel or, above the tuned degree, the
  // CTA kernel of the same table size.
  auto cert_bin = [&](auto kw, size_t smem_w, auto kc, size_t smem_c, int bin, unsigned cap) -> Status {
    return on_cta(bin) ? cta_bin(kc, smem_c, bin) : warp_bin(kw, smem_w, bin, cap);
  };
  // The routed lane-group bins, on the warp kernel of the smallest table.
  auto routed_bins = [&](auto k, size_t smem, unsigned cap) -> Status {
    for (int b = kBinG4; b <= kBinG32; ++b)
      if (routed(b)) PCC_RETURN_IF_ERROR(warp_bin(k, smem, b, cap));
    return Status::Ok();
  };
  int ng = 0;
  for (int b = kBinG4; b <= kBinG32; ++b) ng += want(b) && !routed(b) ? 1 : 0;
  if (families & kLaunchGroups) FamBegin(ctx, kFamGroup);
  if constexpr (kCert) {
    // One wave of resident CTAs (grid-stride kernels).
    auto group_bin = [&](auto k, int bin, uint64_t per_block) -> Status {
      if (!want(bin) || routed(bin)) return Status::Ok();
      int per_sm = 0;
      PCC_RETURN_IF_ERROR(SetSmem(k, 0, 256, &per_sm));
      k<<<grid(bin, per_block, waves(sms * unsigned(per_sm > 0 ? per_sm : 8))), 256, 0, st>>>(a, list, counts, starts,
                                                                                          bin);
      PCC_COUNT(1);
      return Status::Ok();
    };
    PCC_RETURN_IF_ERROR(group_bin(CertGroupKernel<4>, kBinG4, 64));
    PCC_RETURN_IF_ERROR(group_bin(CertGroupKernel<8>, kBinG8, 32));
    PCC_RETURN_IF_ERROR(group_bin(CertGroupKernel<16>, kBinG16, 16));
    PCC_RETURN_IF_ERROR(group_bin(CertGroupKernel<32>, kBinG32, 8));
  } else {
    if (want(kBinG4) && !routed(kBinG4)) {
      BestMoveGroupKernel<4, kInt, kAsync><<<grid(kBinG4, 64, waves(sms * 8)), 256, 0, st>>>(a, list, counts, starts,
                                                                                            kBinG4);
      PCC_COUNT(1);
    }
    if (want(kBinG8) && !routed(kBinG8)) {
      BestMoveGroupKernel<8, kInt, kAsync><<<grid(kBinG8, 32, waves(sms * 8)), 256, 0, st>>>(a, list, counts, starts,
                                                                                            kBinG8);
      PCC_COUNT(1);
    }
    if (want(kBinG16) && !routed(kBinG16)) {
      BestMoveGroupKernel<16, kInt, kAsync><<<grid(kBinG16, 16, waves(sms * 8)), 256, 0, st>>>(a, list, counts, starts,
                                                                                            kBinG16);
      PCC_COUNT(1);
    }
    if (want(kBinG32) && !routed(kBinG32)) {
      BestMoveGroupKernel<32, kInt, kAsync><<<grid(kBinG32, 8, waves(sms * 8)), 256, 0, st>>>(a, list, counts, starts,
                                                                                            kBinG32);
      PCC_COUNT(1);
    }
  }
  if (families & kLaunchGroups) FamEnd(ctx, kFamGroup, ng);
  int nw = 0;
  for (int b = kBinG4; b <= kBinW1000; ++b) nw += want(b) && (b > kBinG32 || routed(b)) ? 1 : 0;
  if (families & kLaunchWarps) FamBegin(ctx, kFamWarp);
  if constexpr (kCert) {
    if (a.narrow) {
      PCC_RETURN_IF_ERROR(routed_bins(CertWarpKernel<256, int>, CertWarpSmem<256, int>(), sms * 16));
      PCC_RETURN_IF_ERROR(cert_bin(CertWarpKernel<256, int>, CertWarpSmem<256, int>(), CertCtaKernel<256, int>,
                   CertCtaSmem<256, int>(), kBinW128, sms * 16));
      PCC_RETURN_IF_ERROR(cert_bin(CertWarpKernel<512, int>, CertWarpSmem<512, int>(), CertCtaKernel<512, int>,
                   CertCtaSmem<512, int>(), kBinW256, sms * 8));
      PCC_RETURN_IF_ERROR(cert_bin(CertWarpKernel<1024, int>, CertWarpSmem<1024, int>(), CertCtaKernel<1024, int>,
                   CertCtaSmem<1024, int>(), kBinW512, sms * 6));
      PCC_RETURN_IF_ERROR(cert_bin(CertWarpKernel<2048, int>, CertWarpSmem<2048, int>(), CertCtaKernel<2048, int>,
                   CertCtaSmem<2048, int>(), kBinW1000, sms * 3));
    } else {
      PCC_RETURN_IF_ERROR(routed_bins(CertWarpKernel<256, long long>, CertWarpSmem<256, long long>(), sms * 16));
      PCC_RETURN_IF_ERROR(
          cert_bin(CertWarpKernel<256, long long>, CertWarpSmem<256, long long>(), CertCtaKernel<256, long long>,
                   CertCtaSmem<256, long long>(), kBinW128, sms * 16));
      PCC_RETURN_IF_ERROR(
          cert_bin(CertWarpKernel<512, long long>, CertWarpSmem<512, long long>(), CertCtaKernel<512, long long>,
                   CertCtaSmem<512, long long>(), kBinW256, sms * 8));
      PCC_RETURN_IF_ERROR(
          cert_bin(CertWarpKernel<1024, long long>, CertWarpSmem<1024, long long>(), CertCtaKernel<1024, long long>,
                   CertCtaSmem<1024, long long>(), kBinW512, sms * 4));
      PCC_RETURN_IF_ERROR(
          cert_bin(CertWarpKernel<2048, long long>, CertWarpSmem<2048, long long>(), CertCtaKernel<2048, long long>,
                   CertCtaSmem<2048, long long>(), kBinW1000, sms * 2));
    }
  } else {
    PCC_RETURN_IF_ERROR(routed_bins(BestMoveWarpKernel<256, kInt, kAsync>, WarpKernelSmem<256>(), sms * 16));
    PCC_RETURN_IF_ERROR(warp_bin(BestMoveWarpKernel<256, kInt, kAsync>, WarpKernelSmem<256>(), kBinW128, sms * 16));
    PCC_RETURN_IF_ERROR(warp_bin(BestMoveWarpKernel<512, kInt, kAsync>, WarpKernelSmem<512>(), kBinW256, sms * 8));
    PCC_RETURN_IF_ERROR(warp_bin(BestMoveWarpKernel<1024, kInt, kAsync>, WarpKernelSmem<1024>(), kBinW512, sms * 4));
    PCC_RETURN_IF_ERROR(warp_bin(BestMoveWarpKernel<2048, kInt, kAsync>, WarpKernelSmem<2048>(), kBinW1000, sms * 2));
  }
  if (families & kLaunchWarps) FamEnd(ctx, kFamWarp, nw);
  return LaunchCheck();
}

template <class K>
Status Prep(K kernel, size_t smem, int threads) {
  int per_sm = 0;
  return SetSmem(kernel, smem, threads, &per_sm);
}

}  // namespace

Status PrepareBestMoveKernels() {
  static std::mutex mu;
  static bool done = false;
  std::lock_guard<std::mutex> lk(mu);
  if (done) return Status::Ok();
  PCC_RETURN_IF_ERROR(Prep(CertGroupKernel<4>, 0, 256));
  PCC_RETURN_IF_ERROR(Prep(CertGroupKernel<8>, 0, 256));
  PCC_RETURN_IF_ERROR(Prep(CertGroupKernel<16>, 0, 256));
  PCC_RETURN_IF_ERROR(Prep(CertGroupKernel<32>, 0, 256));
  constexpr int kW = kWarpKernelWarps * 32;
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<256, int>, CertWarpSmem<256, int>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<512, int>, CertWarpSmem<512, int>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<1024, int>, CertWarpSmem<1024, int>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<2048, int>, CertWarpSmem<2048, int>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<256, long long>, CertWarpSmem<256, long long>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<512, long long>, CertWarpSmem<512, long long>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<1024, long long>, CertWarpSmem<1024, long long>(), kW));
  PCC_RETURN_IF_ERROR(Prep(CertWarpKernel<2048, long long>, CertWarpSmem<2048, long long>(), kW));
  constexpr int kC = kCtaWarps * 32;
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<256, int>, CertCtaSmem<256, int>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<512, int>, CertCtaSmem<512, int>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<1024, int>, CertCtaSmem<1024, int>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<2048, int>, CertCtaSmem<2048, int>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<256, long long>, CertCtaSmem<256, long long>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<512, long long>, CertCtaSmem<512, long long>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<1024, long long>, CertCtaSmem<1024, long long>(), kC));
  PCC_RETURN_IF_ERROR(Prep(CertCtaKernel<2048, long long>, CertCtaSmem<2048, long long>(), kC));
  PCC_RETURN_IF_ERROR(Prep(BestMoveWarpKernel<256, false, false>, WarpKernelSmem<256>(), kW));
  PCC_RETURN_IF_ERROR(Prep(BestMoveWarpKernel<512, false, false>, WarpKernelSmem<512>(), kW));
  PCC_RETURN_IF_ERROR(Prep(BestMoveWarpKernel<1024, false, false>, WarpKernelSmem<1024>(), kW));
  PCC_RETURN_IF_ERROR(Prep(BestMoveWarpKernel<2048, false, false>, WarpKernelSmem<2048>(), kW));
  done = true;
  return Status::Ok();
}

Status LaunchBestMoves(Context* ctx, const BMArgs& a, const uint32_t* list, const uint32_t* bin_counts,
                       const uint32_t* bin_starts, const uint32_t* host_counts, bool int_mode,
                       uint32_t max_deg, int families) {
  if (a.async) {
    return int_mode ? LaunchAll<true, true>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg, families)
                    : LaunchAll<false, true>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg, families);
  }
  return int_mode ? LaunchAll<true, false>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg, families)
                  : LaunchAll<false, false>(ctx, a, list, bin_counts, bin_starts, host_counts, max_deg, families);
}

}  // namespace pcc
