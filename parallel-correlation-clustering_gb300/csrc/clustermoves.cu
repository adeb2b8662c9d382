// clustermoves.cu -- whole-cluster moves (DEFAULT_CLUSTER_MOVES).
//
// Restates the cluster-move block of BestMovesForVertexSubset
// (clustering/clusterers/parallel-correlation-clusterer.cc:167-297, with
// subclustering NONE, synchronous moves), ClusteringHelper::BestMove
// (parallel-correlation-clusterer-internal.cc:644-707) and BestMoveFromStats
// (correlation-clusterer-util.h:70-113).  After the round's vertex moves
// are applied, every cluster c is a moving set whose members are exactly
// the vertices of c, so:
//   * S_D = the sum, over member entries (v, u) with C(u) = D != c, of
//     double(float(double(w) - offset)), in member order (ascending ids)
//     and then adjacency order (EdgeSum::Add in the reference's loop);
//   * W = the sum of the members' node weights;
//   * change = 0 + (0/2 - res*(W*W/2 - W*W/2)), then
//     change -= 0 - res*(W*(K_c - W));
//   * value(D) = change + (S_D - res*(W*(K_D - 0)));
//   * the best D has the largest value, ties to the lowest id, and must
//     beat `change` (staying); the cluster moves when the value is > 0 and
//     c < D (the reference's id rule for simultaneous moves).
// GB300 shape: the entries with C(u) != C(v) are keyed (rank C(v), rank
// C(u)) in CSR order and stably radix-sorted, so each (c, D) run holds its
// entries in the reference's summation order.  A run's sum is a sequential
// FP64 fold (real weights) or warp-combined FP64 atomics (integral values,
// exact in any order).  Every run's value is computed in parallel; the
// per-cluster best is an atomic max over order-preserving bits, then an
// atomic min of the id over the runs at that max.
#include <functional>

#include "graphops.cuh"

namespace pcc {

namespace {

__global__ void CmPresentKernel(uint32_t n, const uint32_t* __restrict__ C, uint32_t* __restrict__ pres) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    pres[C[i]] = 1u;
}

struct CmPresInput {
  const uint32_t* pres;
  __device__ uint32_t operator()(uint64_t i) const { return pres[i]; }
};
struct CmRankWriter {
  uint32_t* rank;
  uint32_t* ids;
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t v) const {
    rank[i] = pre;
    if (v) ids[pre] = static_cast<uint32_t>(i);
  }
};

// Entries that leave their cluster (a self-loop never does), keyed by the
// ranks of (C(v), C(u)).
struct CmKeyBuilder {
  const uint32_t* nbr;
  const uint32_t* C;
  const uint32_t* rank;
  uint32_t bits;
  uint8_t* keep;
  uint64_t* key;
  __device__ void operator()(uint32_t v, uint64_t j, uint64_t) const {
    const uint32_t cv = C[v], cu = C[nbr[j]];
    const bool k = cv != cu;
    keep[j] = k;
    if (k) key[j] = (static_cast<uint64_t>(rank[cv]) << bits) | rank[cu];
  }
};

struct CmKeepInput {
  const uint8_t* keep;
  __device__ uint32_t operator()(uint64_t i) const { return keep[i]; }
};
// Compacts the kept keys in CSR order with the entry's float(w - offset).
struct CmKeepWriter {
  const uint64_t* key_full;
  const float* w;
  double offset;
  uint64_t* keys;
  uint32_t* vals;
  __device__ void operator()(uint64_t j, uint32_t pre, uint32_t v) const {
    if (v) {
      keys[pre] = key_full[j];
      const double wd = w ? static_cast<double>(w[j]) : 1.0;
      vals[pre] = __float_as_uint(__double2float_rn(Dsub(wd, offset)));
    }
  }
};

struct CmRunHead {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};
// Run starts, and (for the integral path) the run of every entry.
struct CmRunWriter {
  uint32_t* run_start;
  uint32_t* run_of;  // nullable
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t v) const {
    if (v) run_start[pre] = static_cast<uint32_t>(i);
    if (run_of) run_of[i] = pre + v - 1;
  }
};

__global__ void CmSetKernel(uint32_t* p, const uint32_t* value) { *p = *value; }

// S of each (c, D) run, real weights: a left fold from 0.0 in run order (the
// reference's EdgeSum::Add sequence).
__global__ void CmRunFoldKernel(const uint32_t* __restrict__ nruns_p, const uint32_t* __restrict__ run_start,
                                const uint32_t* __restrict__ vals, double* __restrict__ run_sum) {
  const uint32_t nruns = *nruns_p;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t a = run_start[r], e = run_start[r + 1];
    double s = 0.0;
    for (uint32_t j = a; j < e; ++j) s = Dadd(s, static_cast<double>(__uint_as_float(vals[j])));
    run_sum[r] = s;
  }
}

// S of each run, integral values (every partial sum an integer below 2^53,
// so any order gives the fold's result): lanes of a warp that share a run
// add first, then one FP64 atomic per run and warp.
__global__ void CmRunAtomicKernel(uint32_t M, const uint32_t* __restrict__ run_of, const uint32_t* __restrict__ vals,
                                  double* __restrict__ run_sum) {
  const uint64_t limit = (uint64_t(M) + 31) & ~uint64_t(31);
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < limit;
       j += uint64_t(gridDim.x) * blockDim.x) {
    const bool in = j < M;
    const uint32_t r = in ? run_of[j] : kNone;
    double x = in ? static_cast<double>(__uint_as_float(vals[j])) : 0.0;
    const unsigned peers = __match_any_sync(kFull, r);
    const int leader = __ffs(peers) - 1;
    double tot = 0.0;
    unsigned mm = peers;
    while (mm) {
      const int l = __ffs(mm) - 1;
      tot = Dadd(tot, __shfl_sync(peers, x, l));
      mm &= mm - 1;
    }
    if (in && int(LaneId()) == leader) atomicAdd(&run_sum[r], tot);
  }
}

// W of each cluster (exact for integral node weights, as on every path of
// the reference's clusterers).
__global__ void CmWeightKernel(uint32_t n, const uint32_t* __restrict__ C, const double* __restrict__ k,
                               double* __restrict__ W) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    atomicAdd(&W[C[i]], k[i]);
}

__device__ __forceinline__ double HalfSquare(double x) { return __ddiv_rn(Dmul(x, x), 2.0); }

// change of BestMoveFromStats for a cluster of weight w (K_c its cluster
// weight): the class-2 and class-1-together terms, both empty sums.
__device__ __forceinline__ double StayValue(double res, double w, double Kc) {
  double change = 0.0;
  change = Dadd(change, Dsub(0.0 / 2, Dmul(res, Dsub(HalfSquare(w), HalfSquare(w)))));
  return Dsub(change, Dsub(0.0, Dmul(res, Dmul(w, Dsub(Kc, w)))));
}

// Total order of doubles as unsigned integers (-0 taken as +0, which
// compares equal to it).
__device__ __forceinline__ unsigned long long OrdBits(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(Dadd(v, 0.0)));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double FromOrd(unsigned long long o) {
  const unsigned long long b = (o >> 63) ? (o & 0x7FFFFFFFFFFFFFFFull) : ~o;
  return __longlong_as_double(static_cast<long long>(b));
}

struct CmRunArgs {
  const uint32_t* nruns_p;
  const uint32_t* run_start;
  const uint64_t* keys;
  const double* run_sum;
  const uint32_t* ids;
  uint32_t bits;
  const double* W;
  const double* K;
  double res;
  double* run_val;
  unsigned long long* best_bits;  // per cluster id: max OrdBits(value) (0: no runs)
  uint32_t* best_id;              // per cluster id: lowest D with the max value
};

// value(D) = change + (S_D - res*(W*(K_D - 0))) of every run, and the max
// per moving cluster.
__global__ void CmRunValueKernel(CmRunArgs a) {
  const uint32_t nruns = *a.nruns_p;
  const uint64_t mask = (uint64_t(1) << a.bits) - 1;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = a.keys[a.run_start[r]];
    const uint32_t c = a.ids[key >> a.bits], d = a.ids[key & mask];
    const double w = a.W[c];
    const double val = Dadd(StayValue(a.res, w, a.K[c]), Dsub(a.run_sum[r], Dmul(a.res, Dmul(w, Dsub(a.K[d], 0.0)))));
    a.run_val[r] = val;
    atomicMax(&a.best_bits[c], OrdBits(val));
  }
}

// Ties at the max go to the lowest cluster id.
__global__ void CmRunTieKernel(CmRunArgs a) {
  const uint32_t nruns = *a.nruns_p;
  const uint64_t mask = (uint64_t(1) << a.bits) - 1;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = a.keys[a.run_start[r]];
    const uint32_t c = a.ids[key >> a.bits];
    if (OrdBits(a.run_val[r]) == a.best_bits[c]) atomicMin(&a.best_id[c], a.ids[key & mask]);
  }
}

// The decision of every cluster with runs: the best D when its value beats
// staying (a D that only ties with staying never replaces it), the id rule,
// then a move when the value is > 0.
__global__ void CmDecideKernel(uint32_t n, const uint32_t* __restrict__ best_id,
                               const unsigned long long* __restrict__ best_bits, const double* __restrict__ W,
                               const double* __restrict__ K, double res, uint32_t* __restrict__ cmove) {
  for (uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n; c += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t d = best_id[c];
    if (d == kNone) continue;
    const double change = StayValue(res, W[c], K[c]);
    const double bv = FromOrd(best_bits[c]);
    uint32_t target = n;
    double val = change;
    if (bv > change) {
      target = d;
      val = bv;
    }
    if (target < n && c >= target) val = 0.0;
    cmove[c] = val > 0 ? target : kNone;
  }
}

// Members of moving clusters become movers (warp-aggregated append).
__global__ void CmMoversKernel(uint32_t n, const uint32_t* __restrict__ C, const uint32_t* __restrict__ cmove,
                               uint32_t* __restrict__ moves, uint32_t* __restrict__ movers, DevCounters* ctr) {
  const uint64_t limit = (uint64_t(n) + 31) & ~uint64_t(31);
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < limit;
       v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t t = v < n ? cmove[C[v]] : kNone;
    const bool in = t != kNone;
    if (in) moves[v] = t;
    const unsigned b = __ballot_sync(kFull, in);
    if (!b) continue;
    uint32_t base = 0;
    if (LaneId() == 0) base = atomicAdd(&ctr->movers, uint32_t(__popc(b)));
    base = __shfl_sync(kFull, base, 0);
    if (in) movers[base + __popc(b & LaneMaskLt())] = static_cast<uint32_t>(v);
  }
}

// ---------------------------------------------------------------------------
// Asynchronous whole-cluster moves: AsyncMove(moving_nodes) (parallel-
// correlation-clusterer-internal.cc:405-446) for every cluster of the
// clustering after the round's vertex moves (parallel-correlation-
// clusterer.cc:255-268).  The moving sets are those clusters' members,
// fixed when the step starts; each set is evaluated on the live state in
// one of `waves` hashed waves, and the moves of a wave are applied before the
// next wave is evaluated (the reference applies each move as it is found,
// with a few CPU threads in flight).  A set's members always share one
// cluster c, which other vertices may have joined, so for member entries
// (v, u) with u outside the set:
//   * T = the sum over C(u) = c (class 1 "currently together");
//   * S_D = the sum over C(u) = D, D = c included;
//   * change = (0 - res*(W*W/2 - W*W/2)) - (T - res*(W*(K_c - W)));
//   * value(D) = change + (S_D - res*(W*(K_D - (D == c ? W : 0))));
// the best D has the largest value (ties to the lowest id) and must beat
// staying, which otherwise means a new cluster; the set moves when its
// value is > 0 (no id rule in async mode).  K moves by the FP32 sum of the
// members' node weights (the reference's delayed_seq<float> reduce, in the
// pbbs block order).  A one-member set takes the vertex AsyncMove (run by
// the caller's vertex kernels).  The moved flags are set at the members'
// vertex ids, as the reference does.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t SetWave(uint32_t set, uint32_t salt, uint32_t waves) {
  uint32_t x = set ^ salt;
  x ^= x >> 16;
  x *= 0x7FEB352Du;
  x ^= x >> 15;
  x *= 0x846CA68Bu;
  x ^= x >> 16;
  return __umulhi(x, waves);
}

struct SmFrame {
  uint32_t n;
  const uint32_t* set_of;   // the set (cluster at the start of the step) of every vertex
  const uint32_t* set_size; // members per set id
  uint32_t wave, waves, salt;
  __device__ bool Active(uint32_t set) const { return SetWave(set, salt, waves) == wave; }
};

__global__ void IotaKeysKernel(uint32_t n, const uint32_t* __restrict__ set_of, uint64_t* __restrict__ keys,
                               uint32_t* __restrict__ vals) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
    keys[v] = set_of[v];
    vals[v] = static_cast<uint32_t>(v);
  }
}

__global__ void SmSizeKernel(uint32_t n, const uint32_t* __restrict__ C, uint32_t* __restrict__ set_of,
                             uint32_t* __restrict__ size, const double* __restrict__ k, double* __restrict__ W) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t c = C[v];
    set_of[v] = c;
    atomicAdd(&size[c], 1u);
    atomicAdd(&W[c], k[v]);
  }
}

// Vertices of the wave's one-member sets, for the vertex AsyncMove.
__global__ void SmMarkSinglesKernel(SmFrame f, uint32_t* __restrict__ front, uint32_t val) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < f.n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t set = f.set_of[v];
    if (f.set_size[set] == 1 && f.Active(set)) front[v] = val;
  }
}

// A one-member set that moved: its flag at the vertex id.
__global__ void SmFlagSinglesKernel(SmFrame f, const uint32_t* __restrict__ moved, uint32_t val,
                                    uint32_t* __restrict__ mod_stamp, uint32_t stamp) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < f.n; v += uint64_t(gridDim.x) * blockDim.x)
    if (moved[v] == val) mod_stamp[v] = stamp;
}

// The live cluster of every active multi-member set.
__global__ void SmClusterKernel(SmFrame f, const uint32_t* __restrict__ C, uint32_t* __restrict__ cset) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < f.n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t set = f.set_of[v];
    if (f.set_size[set] > 1 && f.Active(set)) cset[set] = C[v];
  }
}

// Entries of active multi-member sets to vertices outside the set, keyed
// (set, C(u)) in CSR order.
struct SmKeyBuilder {
  SmFrame f;
  const uint32_t* nbr;
  const uint32_t* C;
  uint32_t bits;
  uint8_t* keep;
  uint64_t* key;
  __device__ void operator()(uint32_t v, uint64_t j, uint64_t) const {
    const uint32_t set = f.set_of[v];
    const uint32_t u = nbr[j];
    const bool k = f.set_size[set] > 1 && f.Active(set) && f.set_of[u] != set;
    keep[j] = k;
    if (k) key[j] = (static_cast<uint64_t>(set) << bits) | C[u];
  }
};

struct SmRunArgs {
  const uint32_t* nruns_p;
  const uint32_t* run_start;
  const uint64_t* keys;
  const double* run_sum;
  uint32_t bits;
  const uint32_t* cset;
  const double* W;
  const double* K;
  double res;
  double* T;                      // per set: the together sum (0 when no entry)
  double* run_val;
  unsigned long long* best_bits;  // per set: max OrdBits(value) over its runs
  uint32_t* best_id;              // per set: lowest D at that max
};

__device__ __forceinline__ double SetChange(double res, double w, double Kc, double T) {
  double change = 0.0;
  change = Dadd(change, Dsub(0.0 / 2, Dmul(res, Dsub(HalfSquare(w), HalfSquare(w)))));
  return Dsub(change, Dsub(T, Dmul(res, Dmul(w, Dsub(Kc, w)))));
}

__global__ void SmTogetherKernel(SmRunArgs a) {
  const uint32_t nruns = *a.nruns_p;
  const uint64_t mask = (uint64_t(1) << a.bits) - 1;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = a.keys[a.run_start[r]];
    const uint32_t set = uint32_t(key >> a.bits), d = uint32_t(key & mask);
    if (d == a.cset[set]) a.T[set] = a.run_sum[r];
  }
}

__global__ void SmRunValueKernel(SmRunArgs a) {
  const uint32_t nruns = *a.nruns_p;
  const uint64_t mask = (uint64_t(1) << a.bits) - 1;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = a.keys[a.run_start[r]];
    const uint32_t set = uint32_t(key >> a.bits), d = uint32_t(key & mask);
    const uint32_t c = a.cset[set];
    const double w = a.W[set];
    const double moving_d = d == c ? w : 0.0;
    const double val = Dadd(SetChange(a.res, w, a.K[c], a.T[set]),
                            Dsub(a.run_sum[r], Dmul(a.res, Dmul(w, Dsub(a.K[d], moving_d)))));
    a.run_val[r] = val;
    atomicMax(&a.best_bits[set], OrdBits(val));
  }
}

__global__ void SmRunTieKernel(SmRunArgs a) {
  const uint32_t nruns = *a.nruns_p;
  const uint64_t mask = (uint64_t(1) << a.bits) - 1;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nruns;
       r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = a.keys[a.run_start[r]];
    const uint32_t set = uint32_t(key >> a.bits);
    if (OrdBits(a.run_val[r]) == a.best_bits[set]) atomicMin(&a.best_id[set], uint32_t(key & mask));
  }
}

struct SmApplyArgs {
  SmFrame f;
  const uint32_t* member;     // vertices sorted by (set, id)
  const uint32_t* set_first;  // per set id: first index in member (valid for sets with members)
  const uint32_t* cset;
  const double* W;
  const double* T;
  const double* k;
  const unsigned long long* best_bits;
  const uint32_t* best_id;
  double res;
  uint32_t* s;
  double* K;
  uint32_t* dest;             // per set: destination (kNone: stays)
  uint32_t* free_ids;
  uint32_t* free_ctr;
  uint32_t free_cap;
  DevCounters* ctr;
};

// pbbs::reduce_add over the members' node weights as floats: serial folds
// of 1024-item blocks, then the same reduce over the block sums.
__device__ float BlockedFloatSum(const uint32_t* member, uint32_t len, const double* k) {
  if (len <= 1024) {
    float r = static_cast<float>(k[member[0]]);
    for (uint32_t j = 1; j < len; ++j) r = __fadd_rn(r, static_cast<float>(k[member[j]]));
    return r;
  }
  // Block sums fold in order; their reduce is again blocked (1024 blocks
  // hold a million members; beyond that the blocks of block sums fold in
  // order too).
  float outer = 0.f, inner = 0.f;
  const uint32_t nb = (len + 1023) / 1024;
  for (uint32_t b = 0; b < nb; ++b) {
    const uint32_t s0 = b * 1024, e0 = min(len, s0 + 1024);
    float r = static_cast<float>(k[member[s0]]);
    for (uint32_t j = s0 + 1; j < e0; ++j) r = __fadd_rn(r, static_cast<float>(k[member[j]]));
    if (nb <= 1024) {
      inner = b == 0 ? r : __fadd_rn(inner, r);
    } else {
      const uint32_t bb = b % 1024;
      inner = bb == 0 ? r : __fadd_rn(inner, r);
      if (bb == 1023 || b + 1 == nb) {
        outer = b < 1024 ? inner : __fadd_rn(outer, inner);
      }
    }
  }
  return nb <= 1024 ? inner : outer;
}

// One thread per active multi-member set: the decision, then the size and
// weight updates and the destination.
__global__ void SmApplyKernel(SmApplyArgs a, uint32_t nsets_ids) {
  for (uint64_t set = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; set < nsets_ids;
       set += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t size = a.f.set_size[set];
    if (size <= 1 || !a.f.Active(uint32_t(set))) continue;
    const uint32_t c = a.cset[set];
    const double w = a.W[set];
    const double change = SetChange(a.res, w, a.K[c], a.T[set]);
    uint32_t target = a.f.n;
    double val = change;
    if (a.best_id[set] != kNone) {
      const double bv = FromOrd(a.best_bits[set]);
      if (bv > change) {
        target = a.best_id[set];
        val = bv;
      }
    }
    if (!(val > 0)) continue;
    const float total = BlockedFloatSum(a.member + a.set_first[set], size, a.k);
    const uint32_t left = atomicSub(&a.s[c], size);
    atomicAdd(&a.K[c], -1 * static_cast<double>(total));
    uint32_t d = target;
    if (target != a.f.n) {
      if (left == size && a.free_ids) {  // c emptied: offer its id to new clusters
        const uint32_t pos = atomicAdd(&a.free_ctr[0], 1u);
        if (pos < a.free_cap) atomicExch(&a.free_ids[pos], c);
      }
      atomicAdd(&a.s[target], size);
      atomicAdd(&a.K[target], static_cast<double>(total));
    } else {
      // The reference probes from c itself, which the set just emptied when
      // it was all of c; otherwise an empty id (free list, then a bounded
      // linear probe), as the vertex move.
      uint64_t i = c;
      bool got = atomicCAS(&a.s[c], 0u, size) == 0u;
      if (!got && a.free_ids) {
        for (int t = 0; t < 16 && !got; ++t) {
          const uint32_t pushed = min(__ldcg(&a.free_ctr[0]), a.free_cap);
          if (__ldcg(&a.free_ctr[1]) >= pushed) break;
          const uint32_t pos = atomicAdd(&a.free_ctr[1], 1u);
          if (pos >= pushed) break;
          const uint32_t id = atomicExch(&a.free_ids[pos], kNone);
          if (id != kNone && atomicCAS(&a.s[id], 0u, size) == 0u) {
            i = id;
            got = true;
          }
        }
      }
      const uint64_t limit = got ? 0 : 4ull * a.f.n + 64;
      for (uint64_t p = 0; p < limit; ++p) {
        i = (i + 1 == a.f.n) ? 0 : i + 1;
        if (__ldcg(&a.s[i]) == 0u && atomicCAS(&a.s[i], 0u, size) == 0u) {
          got = true;
          break;
        }
      }
      if (!got) {  // undo the leave
        atomicAdd(&a.s[c], size);
        atomicAdd(&a.K[c], static_cast<double>(total));
        atomicExch(&a.ctr->error, kErrProbeLimit);
        continue;
      }
      atomicAdd(&a.K[i], static_cast<double>(total));
      d = uint32_t(i);
    }
    a.dest[set] = d;
  }
}

// Members of the sets that moved take the destination; the moved flag is
// set at the member's vertex id.
__global__ void SmMembersKernel(SmFrame f, uint32_t* __restrict__ dest, uint32_t* __restrict__ C,
                                uint32_t* __restrict__ mod_stamp, uint32_t stamp, DevCounters* ctr) {
  const uint64_t limit = (uint64_t(f.n) + 31) & ~uint64_t(31);
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < limit;
       v += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t d = kNone;
    if (v < f.n) {
      const uint32_t set = f.set_of[v];
      if (f.set_size[set] > 1 && f.Active(set)) d = dest[set];
    }
    if (d != kNone) {
      __stcg(&C[v], d);
      mod_stamp[v] = stamp;
    }
    const unsigned b = __ballot_sync(kFull, d != kNone);
    if (b && LaneId() == 0) atomicAdd(&ctr->moves, (unsigned long long)__popc(b));
  }
}

struct SmSetInput {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};
struct SmFirstWriter {
  const uint64_t* keys;
  uint32_t* set_first;
  __device__ void operator()(uint64_t i, uint32_t, uint32_t v) const {
    if (v) set_first[keys[i]] = static_cast<uint32_t>(i);
  }
};

}  // namespace

Status AsyncSetMoves(Context* ctx, const SetMoveArgs& a, const std::function<Status(uint32_t)>& vertex_moves) {
  const DevGraph& g = *a.g;
  const uint32_t n = g.n;
  if (n == 0) return Status::Ok();
  cudaStream_t st = ctx->stream;
  const unsigned grid_n = Blocks(n, 256, ctx->num_sms * 8);
  DBuf<uint32_t> set_of, size, cset, dest, best_id, member, set_first, tmp32, scan_tiles;
  DBuf<double> W, T;
  DBuf<unsigned long long> best_bits;
  DBuf<uint64_t> mkeys;
  PCC_RETURN_IF_ERROR(set_of.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(size.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(W.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(size.Zero());
  PCC_RETURN_IF_ERROR(W.Zero());
  PCC_RETURN_IF_ERROR(cset.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(dest.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(T.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(best_bits.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(best_id.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(member.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(set_first.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(mkeys.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(tmp32.Alloc(ctx, 4));
  SmSizeKernel<<<grid_n, 256, 0, st>>>(n, a.C, set_of.p, size.p, a.k, W.p); PCC_COUNT(1);
  // Members grouped by set in ascending id order (stable sort by set).
  IotaKeysKernel<<<grid_n, 256, 0, st>>>(n, set_of.p, mkeys.p, member.p); PCC_COUNT(1);
  uint32_t bits = 1;
  while ((uint64_t(1) << bits) < n) ++bits;
  {
    SortScratch sc;
    PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, mkeys.p, member.p, n, int(bits), sc));
  }
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, n, SmSetInput{mkeys.p}, SmFirstWriter{mkeys.p, set_first.p},
                                          scan_tiles, tmp32.p));
  mkeys.Release();

  DBuf<uint8_t> keep;
  DBuf<uint64_t> key_full, keys;
  DBuf<uint32_t> vals, run_start, run_of, counts;
  DBuf<double> run_sum, run_val;
  if (g.m) {
    PCC_RETURN_IF_ERROR(keep.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(key_full.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(keys.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(vals.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(run_start.Alloc(ctx, g.m + 1));
    if (a.exact_sums) PCC_RETURN_IF_ERROR(run_of.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(run_sum.Alloc(ctx, g.m));
    PCC_RETURN_IF_ERROR(run_val.Alloc(ctx, g.m));
  }
  PCC_RETURN_IF_ERROR(counts.Alloc(ctx, 1));
  for (uint32_t w = 0; w < a.waves; ++w) {
    SmFrame f{n, set_of.p, size.p, w, a.waves, a.salt};
    // One-member sets: the vertex AsyncMove through the caller's kernels,
    // with their own moved flags (aux) turned into flags at the vertex ids.
    const uint32_t val = a.aux_base + w;
    SmMarkSinglesKernel<<<grid_n, 256, 0, st>>>(f, a.aux_front, val); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(vertex_moves(val));
    SmFlagSinglesKernel<<<grid_n, 256, 0, st>>>(f, a.aux_moved, val, a.mod_stamp, a.stamp); PCC_COUNT(1);
    if (g.m == 0) continue;
    // Multi-member sets on the live state.
    SmClusterKernel<<<grid_n, 256, 0, st>>>(f, a.C, cset.p); PCC_COUNT(1);
    LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                   SmKeyBuilder{f, g.nbr.p, a.C, bits, keep.p, key_full.p});
    PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, g.m, CmKeepInput{keep.p},
                                            CmKeepWriter{key_full.p, g.wp(), a.offset, keys.p, vals.p}, scan_tiles,
                                            tmp32.p));
    uint32_t M = 0;
    PCC_RETURN_IF_ERROR(tmp32.ToHost(&M, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx));
    PCC_RETURN_IF_ERROR(T.Zero());
    PCC_RETURN_IF_ERROR(best_bits.Zero());
    PCC_RETURN_IF_ERROR(best_id.Fill(0xFF));
    PCC_RETURN_IF_ERROR(dest.Fill(0xFF));
    uint32_t nruns = 0;
    if (M) {
      SortScratch sc;
      PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys.p, vals.p, M, int(2 * bits), sc));
      PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, M, CmRunHead{keys.p}, CmRunWriter{run_start.p, run_of.p},
                                              scan_tiles, counts.p));
      PCC_RETURN_IF_ERROR(counts.ToHost(&nruns, 1));
      PCC_RETURN_IF_ERROR(Sync(ctx));
      PCC_RETURN_IF_ERROR(tmp32.FromHost(&M, 1));
      CmSetKernel<<<1, 1, 0, st>>>(run_start.p + nruns, tmp32.p); PCC_COUNT(1);
      const unsigned grid_runs = Blocks(nruns, 256, ctx->num_sms * 16);
      if (a.exact_sums) {
        PCC_RETURN_IF_ERROR(run_sum.Zero());
        CmRunAtomicKernel<<<Blocks(M, 256, ctx->num_sms * 16), 256, 0, st>>>(M, run_of.p, vals.p, run_sum.p);
      } else {
        CmRunFoldKernel<<<grid_runs, 256, 0, st>>>(counts.p, run_start.p, vals.p, run_sum.p);
      }
      PCC_COUNT(1);
      SmRunArgs ra{counts.p, run_start.p, keys.p, run_sum.p, bits, cset.p, W.p, a.K, a.res, T.p, run_val.p,
                   best_bits.p, best_id.p};
      SmTogetherKernel<<<grid_runs, 256, 0, st>>>(ra); PCC_COUNT(1);
      SmRunValueKernel<<<grid_runs, 256, 0, st>>>(ra); PCC_COUNT(1);
      SmRunTieKernel<<<grid_runs, 256, 0, st>>>(ra); PCC_COUNT(1);
    }
    SmApplyArgs aa{f, member.p, set_first.p, cset.p, W.p, T.p, a.k, best_bits.p, best_id.p, a.res, a.s, a.K,
                   dest.p, a.free_ids, a.free_ctr, a.free_cap, a.ctr};
    SmApplyKernel<<<grid_n, 256, 0, st>>>(aa, n); PCC_COUNT(1);
    SmMembersKernel<<<grid_n, 256, 0, st>>>(f, dest.p, a.C, a.mod_stamp, a.stamp, a.ctr); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(LaunchCheck());
  }
  return Sync(ctx);  // scratch buffers go out of scope
}

Status FindClusterMoves(Context* ctx, const DevGraph& g, const uint32_t* C, const double* k, const double* K,
                        double res, double offset, bool exact_sums, uint32_t* moves, uint32_t* movers,
                        DevCounters* ctr) {
  const uint32_t n = g.n;
  if (n == 0 || g.m == 0) return Status::Ok();
  cudaStream_t st = ctx->stream;
  const unsigned grid_n = Blocks(n, 256, ctx->num_sms * 8);
  DBuf<uint32_t> tmp32;
  PCC_RETURN_IF_ERROR(tmp32.Alloc(ctx, 4));
  DBuf<uint32_t> scan_tiles;

  // Dense order-preserving rank of the cluster ids in use (ids are < n).
  DBuf<uint32_t> pres, rank, ids;
  PCC_RETURN_IF_ERROR(pres.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(pres.Zero());
  PCC_RETURN_IF_ERROR(rank.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(ids.Alloc(ctx, n));
  CmPresentKernel<<<grid_n, 256, 0, st>>>(n, C, pres.p); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, n, CmPresInput{pres.p}, CmRankWriter{rank.p, ids.p}, scan_tiles,
                                          tmp32.p));
  uint32_t nclusters = 0;
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&nclusters, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  if (nclusters < 2) return Status::Ok();  // nowhere to move
  uint32_t bits = 1;
  while ((uint64_t(1) << bits) < nclusters) ++bits;

  // Leaving entries with their keys and float(w - offset), in CSR order.
  DBuf<uint8_t> keep;
  DBuf<uint64_t> key_full;
  PCC_RETURN_IF_ERROR(keep.Alloc(ctx, g.m));
  PCC_RETURN_IF_ERROR(key_full.Alloc(ctx, g.m));
  LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                 CmKeyBuilder{g.nbr.p, C, rank.p, bits, keep.p, key_full.p});
  PCC_RETURN_IF_ERROR(LaunchCheck());
  DBuf<uint64_t> keys;
  DBuf<uint32_t> vals;
  PCC_RETURN_IF_ERROR(keys.Alloc(ctx, g.m));
  PCC_RETURN_IF_ERROR(vals.Alloc(ctx, g.m));
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, g.m, CmKeepInput{keep.p},
                                          CmKeepWriter{key_full.p, g.wp(), offset, keys.p, vals.p}, scan_tiles,
                                          tmp32.p));
  uint32_t M = 0;
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&M, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  keep.Release();
  key_full.Release();
  if (M == 0) return Status::Ok();  // no cluster has a neighbouring cluster
  {
    SortScratch sc;
    PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys.p, vals.p, M, int(2 * bits), sc));
  }

  // Runs of equal (c, D) and their sums.
  DBuf<uint32_t> run_start, run_of, counts;
  PCC_RETURN_IF_ERROR(run_start.Alloc(ctx, uint64_t(M) + 1));
  if (exact_sums) PCC_RETURN_IF_ERROR(run_of.Alloc(ctx, M));
  PCC_RETURN_IF_ERROR(counts.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, M, CmRunHead{keys.p}, CmRunWriter{run_start.p, run_of.p}, scan_tiles,
                                          counts.p));
  uint32_t nruns = 0;
  PCC_RETURN_IF_ERROR(counts.ToHost(&nruns, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  PCC_RETURN_IF_ERROR(tmp32.FromHost(&M, 1));
  CmSetKernel<<<1, 1, 0, st>>>(run_start.p + nruns, tmp32.p); PCC_COUNT(1);
  DBuf<double> run_sum;
  PCC_RETURN_IF_ERROR(run_sum.Alloc(ctx, nruns));
  const unsigned grid_runs = Blocks(nruns, 256, ctx->num_sms * 16);
  if (exact_sums) {
    PCC_RETURN_IF_ERROR(run_sum.Zero());
    CmRunAtomicKernel<<<Blocks(M, 256, ctx->num_sms * 16), 256, 0, st>>>(M, run_of.p, vals.p, run_sum.p);
    PCC_COUNT(1);
  } else {
    CmRunFoldKernel<<<grid_runs, 256, 0, st>>>(counts.p, run_start.p, vals.p, run_sum.p); PCC_COUNT(1);
  }

  // Cluster weights, run values, and the decisions.
  DBuf<double> W, run_val;
  PCC_RETURN_IF_ERROR(W.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(W.Zero());
  CmWeightKernel<<<grid_n, 256, 0, st>>>(n, C, k, W.p); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(run_val.Alloc(ctx, nruns));
  DBuf<unsigned long long> best_bits;
  DBuf<uint32_t> best_id, cmove;
  PCC_RETURN_IF_ERROR(best_bits.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(best_bits.Zero());
  PCC_RETURN_IF_ERROR(best_id.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(best_id.Fill(0xFF));
  PCC_RETURN_IF_ERROR(cmove.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(cmove.Fill(0xFF));
  CmRunArgs ra{counts.p, run_start.p, keys.p, run_sum.p, ids.p, bits, W.p, K, res, run_val.p, best_bits.p, best_id.p};
  CmRunValueKernel<<<grid_runs, 256, 0, st>>>(ra); PCC_COUNT(1);
  CmRunTieKernel<<<grid_runs, 256, 0, st>>>(ra); PCC_COUNT(1);
  CmDecideKernel<<<grid_n, 256, 0, st>>>(n, best_id.p, best_bits.p, W.p, K, res, cmove.p); PCC_COUNT(1);
  CmMoversKernel<<<grid_n, 256, 0, st>>>(n, C, cmove.p, moves, movers, ctr); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(LaunchCheck());
  return Sync(ctx);  // scratch buffers go out of scope
}

}  // namespace pcc
