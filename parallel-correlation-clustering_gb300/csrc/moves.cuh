// moves.cuh -- device helpers shared by the best-move kernels: the move
// value formulas of ClusteringHelper::EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:448-583, EdgeSum in
// correlation-clusterer-util.h:26-43), the sync / async decision
// (parallel-correlation-clusterer.cc:139-157, internal.cc:371-403), the FP32
// pre-filter bound and the open-addressing hash used for aggregation.
#pragma once

#include <math_constants.h>

#include <climits>
#include <type_traits>

#include "engine.cuh"

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

// Movers appended through a per-warp buffer of 64 ids in shared memory: one
// atomic per 32 movers instead of one per evaluation step.  The movers
// counter is shared by every CTA of a round, and an atomic whose result is
// needed is a round trip the warp waits for.  Every lane calls Add and
// Flush; the order of the movers list carries no meaning.
struct WarpMoverBuffer {
  uint32_t* buf;       // 64 entries, owned by the calling warp
  uint32_t count = 0;  // warp-uniform
  __device__ void Add(uint32_t* counter, uint32_t* movers, bool pred, uint32_t v) {
    const unsigned m = __ballot_sync(kFull, pred);
    if (!m) return;
    const unsigned lane = LaneId();
    if (pred) buf[count + __popc(m & LaneMaskLt())] = v;
    count += __popc(m);
    if (count < 32) return;
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, 32u);
    base = __shfl_sync(kFull, base, 0);
    movers[base + lane] = buf[lane];
    __syncwarp();
    if (lane < count - 32) buf[lane] = buf[32 + lane];
    count -= 32;
    __syncwarp();
  }
  __device__ void Flush(uint32_t* counter, uint32_t* movers) {
    __syncwarp();
    if (count == 0) return;
    const unsigned lane = LaneId();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, count);
    base = __shfl_sync(kFull, base, 0);
    if (lane < count) movers[base + lane] = buf[lane];
    count = 0;
    __syncwarp();
  }
};

template <bool kAsync>
__device__ __forceinline__ uint32_t LdC(const uint32_t* p) {
  return kAsync ? __ldcg(p) : __ldg(p);
}
template <bool kAsync>
__device__ __forceinline__ double LdK(const double* p) {
  return kAsync ? __ldcg(p) : __ldg(p);
}

// Fibonacci hashing: the HIGH bits of key * 2^32/phi.  (The low bits of the
// product depend only on the key's low bits, which are shared by many
// structured ids -- e.g. RMAT vertex ids -- and would chain the probes.)
__device__ __forceinline__ uint32_t HashSlot(uint32_t key, uint32_t mask) {
  const uint32_t shift = __clz(mask) & 31u;  // mask = cap - 1, cap a power of two
  return ((key * 0x9E3779B1u) >> shift) & mask;
}

// Open addressing with linear probing; keys are cluster ids, kNone = empty.
// Capacity is at least twice the number of keys, so a free slot exists.

// (val desc, id asc) ordering used by every argmax.
__device__ __forceinline__ bool Better(double va, uint32_t ia, double vb, uint32_t ib) {
  return va > vb || (va == vb && ia < ib);
}

// Adds a warp's per-lane counts of evaluated entries and vertices to the
// kernel family's counters (one atomic per warp; every lane calls).
__device__ __forceinline__ void FlushFamily(const BMArgs& a, int fam, unsigned long long e, unsigned long long v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    e += __shfl_xor_sync(kFull, e, o);
    v += __shfl_xor_sync(kFull, v, o);
  }
  if (LaneId() == 0 && v) {
    atomicAdd(&a.ctr->fam_entries[fam], e);
    atomicAdd(&a.ctr->fam_vertices[fam], v);
  }
}

// Wave of vertex v in an async round: a salted MurmurHash3 finalizer of the
// id, scaled to [0, waves).
__device__ __forceinline__ uint32_t WaveOf(uint32_t v, uint32_t salt, uint32_t waves) {
  uint32_t x = v ^ salt;
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return __umulhi(x, waves);
}

__device__ __forceinline__ bool InFront(const BMArgs& a, uint32_t v) {
  if (a.waves > 1 && WaveOf(v, a.wave_salt, a.waves) != a.wave) return false;
  if (a.rs) return a.rs->front_all || a.front_stamp[v] == a.rs->front_val;
  return a.front_stamp == nullptr || a.front_stamp[v] == a.front_val;
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
  return Dsub(0.0, Dsub(T, Dmul(ResOf(a, x.v), Dmul(x.kv, Dsub(x.Kc, x.kv)))));
}

__device__ __forceinline__ double ValOf(const BMArgs& a, const VertexCtx& x, double change, double S, double KD) {
  // change + data.NetWeight(moving_nodes_weight * K_D)   (:493-497)
  return Dadd(change, Dsub(S, Dmul(ResOf(a, x.v), Dmul(x.kv, KD))));
}

// FP32 pre-filter of the INT-mode sync path.  For candidate D with exact
// integer sum S_D, Y_D = (S_D - S_max) - res*kv*K_D orders the candidates
// exactly like the reference's val_D = change + (S_D - res*(kv*K_D)).  Y' is
// Y in FP32 from fl32 inputs: |Y' - Y| <= 2^-21 (R + |Y|) (five roundings of
// 2^-24 in R, one in the subtraction; S_D - S_max is an exact integer).  The
// bound below adds a 4x margin plus an absolute term that covers the FP64
// roundings of val_D (<= 2^-50 (|change| + |S| + R)), so a candidate with
// Y' + e < max(Y' - e) is strictly below the best in FP64 as well and never
// needs its FP64 value; the survivors are evaluated exactly.
__device__ __forceinline__ float FilterBound(float R, float Y, float S, float change32) {
  return __fadd_rn(__fmul_rn(3.814697265625e-06f /* 2^-18 */, __fadd_rn(R, fabsf(Y))),
                   __fmul_rn(3.552713678800501e-15f /* 2^-48 */,
                             __fadd_rn(__fadd_rn(fabsf(change32), fabsf(S)), R)));
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
    const uint32_t left = atomicSub(&a.s_mut[cur], 1u);
    atomicAdd(&a.K_mut[cur], -1 * x.kv);
    if (left == 1u && a.free_ids) {  // cur emptied: offer its id to new clusters
      const uint32_t pos = atomicAdd(&a.free_ctr[0], 1u);
      if (pos < a.free_cap) atomicExch(&a.free_ids[pos], cur);
    }
    uint32_t dest = target;
    if (target != a.n) {
      atomicAdd(&a.s_mut[target], 1u);
      atomicAdd(&a.K_mut[target], x.kv);
    } else {
      // Claim an empty id by CAS.  The reference probes linearly from the
      // vertex's own id (internal.cc:390-401); any empty id gives the same
      // clustering up to renaming, and on graphs with long runs of occupied
      // ids (isolated vertices of RMAT) that probe can walk a million ids
      // while the rest of the kernel waits on one thread.  So the ids empty
      // at the start of the level and those of clusters emptied during it
      // are tried first (a taken or re-occupied one fails the CAS), then the
      // linear probe.  Bounded:
      // after 4n probes the kernel records an error and leaves the vertex
      // where it was (its leave is undone).
      uint64_t i = x.v;
      bool got = false;
      if (a.free_ids) {
        for (int t = 0; t < 16; ++t) {
          const uint32_t pushed = min(__ldcg(&a.free_ctr[0]), a.free_cap);
          if (__ldcg(&a.free_ctr[1]) >= pushed) break;
          const uint32_t pos = atomicAdd(&a.free_ctr[1], 1u);
          if (pos >= pushed) break;
          const uint32_t id = atomicExch(&a.free_ids[pos], kNone);
          if (id != kNone && atomicCAS(&a.s_mut[id], 0u, 1u) == 0u) {
            i = id;
            got = true;
            break;
          }
        }
      }
      const uint64_t limit = got ? 0 : 4ull * a.n + 64;
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
    a.moved_cluster_stamp[dest] = StampIn(a.rs, a.stamp);
    a.moved_stamp[x.v] = StampIn(a.rs, a.stamp);
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
    a.moved_stamp[x.v] = StampIn(a.rs, a.stamp);
    if (t2 != x.c) {
      a.moves[x.v] = t2;
      return true;
    }
  }
  return false;
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

// An integral weight |w| <= 2^22 (INT mode) as an int, with integer and FP32
// arithmetic (no conversion instruction): w + 1.5 * 2^23 is exact and its
// bit pattern minus 0x4B400000 is w.
__device__ __forceinline__ int WeightToInt(float w) {
  return __float_as_int(__fadd_rn(w, 12582912.0f)) - 0x4B400000;
}

// Sum of the integer weights x over the calling lane's match_any group
// `peers`; every lane of the warp calls it.  (__reduce_add_sync with a
// different mask per group executes once per distinct group -- up to 32
// passes per instruction.)  Unit weights: every lane's x is the same, so the
// sum is x * |group|.  Other weights: the group's leader adds its peers'
// values from the warp's 32-int stage row (passes = the largest group).
__device__ __forceinline__ int GroupSumInt(unsigned peers, int x, bool unit, bool leader, int* stage) {
  if (unit) return x * __popc(peers);
  stage[LaneId()] = x;
  __syncwarp();
  int s = 0;
  if (leader) {
    unsigned mm = peers;
    while (mm) {
      s += stage[__ffs(mm) - 1];
      mm &= mm - 1;
    }
  }
  __syncwarp();
  return s;
}

template <bool kInt>
__device__ __forceinline__ double AsDouble(unsigned long long bits) {
  return kInt ? static_cast<double>(static_cast<long long>(bits))
              : __longlong_as_double(static_cast<long long>(bits));
}

}  // namespace
}  // namespace pcc
