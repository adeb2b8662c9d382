// static_moves.cu -- pcc_best_moves_static: EfficientBestMove for a list of
// vertices on caller-owned device arrays, with every scratch byte taken from
// one file-scope device array.  The call allocates no device memory.
//
// Who needs it: callers that own every byte of HBM through their own
// allocator and cannot let a library allocate on the request path -- a
// serving loop that has admitted requests against a fixed HBM budget, or a
// framework whose caching allocator holds the device's free memory.  A
// cudaMalloc there can fail on fragmentation or stall the device.
//
// Kernel: one CTA per vertex at a time (grid-stride over the list).  Each
// CTA owns a fixed region of the scratch table: an open-addressing map from
// neighbour cluster id to the summed edge weight (the block-per-vertex
// global-hash form of the hub path, parallel-correlation-clusterer-
// internal.cc:516-582), used at capacity nextpow2(2 * degree + 2) for the
// current vertex, then read, reduced to the best move and cleared back to
// zero by the same CTA.  The value semantics follow EfficientBestMove
// (parallel-correlation-clusterer-internal.cc:448-583) per vertex degree:
// degree <= 1000 takes w - offset in double and lets the new cluster win
// unless a neighbour cluster is strictly better; degree > 1000 rounds
// w - offset to float and starts the reduce at the monoid identity (0, 0.0).
// Sums are accumulated by FP64 atomics, so on real weights values match the
// context path within rounding (exact on integer weights).
//
// Scratch: kStaticSlots slots of (uint32 key, double sum), key = cluster + 1
// (0 = empty), all zero between calls, plus one error word.  The first call
// on a device resolves the array's address (cudaGetSymbolAddress) with that
// device current; make that first call before any stream capture begins.
// Every call synchronises its stream and copies the error word to the host
// before it returns.  Calls that overlap in time on one device (two host
// threads, two streams) share the scratch and race; callers serialise them.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "pcc_gb300.h"

namespace {

constexpr uint32_t kStaticSlots = 1u << 21;           // 2,097,152 slots
constexpr uint32_t kStaticMaxDegree = (kStaticSlots - 2) / 2;  // one CTA, whole table
constexpr uint32_t kHubDegree = 1000;
constexpr uint32_t kThreads = 256;
constexpr uint32_t kNoTarget = 0xFFFFFFFFu;
constexpr int kMaxDevices = 64;

// keys (4 B/slot), then sums (8 B/slot), then the error word.
constexpr size_t kKeysBytes = size_t(kStaticSlots) * 4;
constexpr size_t kScratchBytes = kKeysBytes + size_t(kStaticSlots) * 8 + 256;
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

enum : uint32_t { kErrDegree = 1, kErrProbe = 2, kErrRange = 4 };

struct StaticArgs {
  uint32_t n;
  const uint64_t* off;
  const uint32_t* nbr;
  const float* w;
  const uint32_t* C;
  const double* k;
  const double* K;
  double res;
  double offset;
  const uint32_t* list;
  uint32_t count;
  uint32_t max_degree;
  uint32_t region;  // slots per CTA (power of two)
  uint32_t* out_t;
  double* out_v;
  uint32_t* keys;
  double* sums;
  uint32_t* error;
};

__device__ __forceinline__ uint32_t Slot(uint32_t key, uint32_t cap) {
  const uint32_t shift = __clz(cap - 1) & 31u;
  return ((key * 0x9E3779B1u) >> shift) & (cap - 1);
}

// (value desc, id asc) argmax of two candidates; id kNoTarget = none.
__device__ __forceinline__ void Keep(double& bv, uint32_t& bi, double v, uint32_t i) {
  if (i == kNoTarget) return;
  if (bi == kNoTarget || v > bv || (v == bv && i < bi)) {
    bv = v;
    bi = i;
  }
}

__global__ void __launch_bounds__(kThreads) StaticBestMoveKernel(StaticArgs a) {
  __shared__ double s_red[kThreads / 32];
  __shared__ double s_val[kThreads / 32];
  __shared__ uint32_t s_id[kThreads / 32];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, wid = tid >> 5;
  uint32_t* keys = a.keys + size_t(blockIdx.x) * a.region;
  double* sums = a.sums + size_t(blockIdx.x) * a.region;
  for (uint32_t i = blockIdx.x; i < a.count; i += gridDim.x) {
    const uint32_t v = a.list ? a.list[i] : i;
    if (v >= a.n) {
      if (tid == 0) {
        atomicOr(a.error, kErrRange);
        a.out_t[i] = kNoTarget;
        a.out_v[i] = 0.0;
      }
      continue;
    }
    const uint64_t b = a.off[v], e = a.off[v + 1];
    const uint64_t deg = e - b;
    if (deg > a.max_degree) {
      if (tid == 0) {
        atomicOr(a.error, kErrDegree);
        a.out_t[i] = kNoTarget;
        a.out_v[i] = 0.0;
      }
      continue;
    }
    uint32_t cap = 32;
    while (cap < 2 * deg + 2) cap <<= 1;
    const bool hub = deg > kHubDegree;
    uint32_t c = a.C[v];
    if (c >= a.n) {
      if (tid == 0) atomicOr(a.error, kErrRange);
      c = 0;
    }
    const double kv = a.k[v];
    // Phase 1: cluster sums into the CTA's region, "together" in registers.
    double together = 0.0;
    for (uint64_t j = b + tid; j < e; j += kThreads) {
      const uint32_t u = a.nbr[j];
      if (u == v) continue;
      if (u >= a.n) {
        atomicOr(a.error, kErrRange);
        continue;
      }
      const float wf = a.w ? a.w[j] : 1.0f;
      // Hub rows take `float weight; weight -= offset;` (rounded to float).
      double wt = __dsub_rn(static_cast<double>(wf), a.offset);
      if (hub) wt = static_cast<double>(static_cast<float>(wt));
      const uint32_t cu = a.C[u];
      if (cu >= a.n) {
        atomicOr(a.error, kErrRange);
        continue;
      }
      if (cu == c) together += wt;
      const uint32_t key = cu + 1;
      uint32_t h = Slot(key, cap);
      bool placed = false;
      for (uint32_t p = 0; p < cap; ++p) {
        uint32_t cur = __ldcg(keys + h);
        if (cur == 0) cur = atomicCAS(keys + h, 0u, key);
        if (cur == 0 || cur == key) {
          placed = true;
          break;
        }
        h = (h + 1) & (cap - 1);
      }
      if (placed) {
        atomicAdd(sums + h, wt);
      } else {
        atomicOr(a.error, kErrProbe);
      }
    }
    for (int o = 16; o; o >>= 1) together += __shfl_xor_sync(0xFFFFFFFFu, together, o);
    if (lane == 0) s_red[wid] = together;
    __syncthreads();
    double T = 0.0;
    for (uint32_t q = 0; q < kThreads / 32; ++q) T += s_red[q];
    const double max_edges = kv * (a.K[c] - kv);
    double change = 0.0;
    change -= T - a.res * max_edges;
    // Phase 2: values of the used slots, argmax, slots cleared.
    double bv = 0.0;
    uint32_t bi = kNoTarget;
    for (uint32_t s = tid; s < cap; s += kThreads) {
      const uint32_t key = __ldcg(keys + s);
      if (key == 0) continue;
      const uint32_t cu = key - 1;
      double data = __ldcg(sums + s);
      data -= a.res * (kv * a.K[cu]);
      Keep(bv, bi, change + data, cu);
      keys[s] = 0;
      sums[s] = 0.0;
    }
    for (int o = 16; o; o >>= 1) {
      const double ov = __shfl_xor_sync(0xFFFFFFFFu, bv, o);
      const uint32_t oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
      Keep(bv, bi, ov, oi);
    }
    if (lane == 0) {
      s_val[wid] = bv;
      s_id[wid] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double best = 0.0;
      uint32_t id = kNoTarget;
      for (uint32_t q = 0; q < kThreads / 32; ++q) Keep(best, id, s_val[q], s_id[q]);
      uint32_t target;
      double value;
      if (!hub) {
        // :495-512: the new cluster unless a cluster is strictly better.
        if (id != kNoTarget && best > change) {
          target = id;
          value = best;
        } else {
          target = a.n;
          value = change;
        }
      } else {
        // :562-582: reduce from the identity (0, 0.0); new cluster on ties.
        if (id == kNoTarget) {
          best = 0.0;
          id = 0;
        }
        if (change >= best) {
          target = a.n;
          value = change;
        } else {
          target = id;
          value = best;
        }
      }
      a.out_t[i] = target;
      a.out_v[i] = value;
    }
    __syncthreads();  // region clear and shared reductions done before reuse
  }
}

// The scratch array's device address, per device.  Only a successful
// lookup is recorded: a lookup that failed (for example while another
// stream was capturing in global mode) is retried by the next call.
struct DeviceScratch {
  std::mutex mu;
  unsigned char* base = nullptr;
};
DeviceScratch g_devices[kMaxDevices];

unsigned char* ScratchBase(int dev) {
  DeviceScratch& ds = g_devices[dev];
  std::lock_guard<std::mutex> lk(ds.mu);
  if (!ds.base) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ds.base = static_cast<unsigned char*>(p);
  }
  return ds.base;
}

}  // namespace

extern "C" pcc_status pcc_best_moves_static(
    uint32_t n, const uint64_t* d_offsets, const uint32_t* d_neighbors, const float* d_weights,
    const uint32_t* d_cluster_ids, const double* d_node_weights, const double* d_cluster_weights,
    double resolution, double edge_weight_offset, const uint32_t* d_vertices, uint32_t num_vertices,
    uint32_t max_degree, uint32_t* d_out_targets, double* d_out_values, void* stream) {
  if (!d_offsets || (!d_neighbors && num_vertices) || !d_cluster_ids || !d_node_weights ||
      !d_cluster_weights || !d_out_targets || !d_out_values)
    return PCC_INVALID_ARGUMENT;
  if (!d_vertices && num_vertices != n) return PCC_INVALID_ARGUMENT;
  if (max_degree > kStaticMaxDegree) return PCC_OUT_OF_RANGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PCC_UNAVAILABLE;
  if (dev < 0 || dev >= kMaxDevices) return PCC_OUT_OF_RANGE;
  unsigned char* const base = ScratchBase(dev);
  if (!base) return PCC_INTERNAL;
  if (num_vertices == 0) return PCC_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint32_t* error = reinterpret_cast<uint32_t*>(base + kKeysBytes + size_t(kStaticSlots) * 8);
  if (cudaMemsetAsync(error, 0, sizeof(uint32_t), st) != cudaSuccess) return PCC_INTERNAL;
  uint32_t region = 32;
  while (region < 2ull * max_degree + 2) region <<= 1;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PCC_INTERNAL;
  uint64_t grid = uint64_t(sms) * 8;
  grid = std::min<uint64_t>(grid, kStaticSlots / region);
  grid = std::min<uint64_t>(grid, num_vertices);
  if (grid == 0) grid = 1;
  StaticArgs a;
  a.n = n;
  a.off = d_offsets;
  a.nbr = d_neighbors;
  a.w = d_weights;
  a.C = d_cluster_ids;
  a.k = d_node_weights;
  a.K = d_cluster_weights;
  a.res = resolution;
  a.offset = edge_weight_offset;
  a.list = d_vertices;
  a.count = num_vertices;
  a.max_degree = max_degree;
  a.region = region;
  a.out_t = d_out_targets;
  a.out_v = d_out_values;
  a.keys = reinterpret_cast<uint32_t*>(base);
  a.sums = reinterpret_cast<double*>(base + kKeysBytes);
  a.error = error;
  StaticBestMoveKernel<<<static_cast<unsigned>(grid), kThreads, 0, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return PCC_INTERNAL;
  uint32_t herr = 0;
  if (cudaMemcpyAsync(&herr, error, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return PCC_INTERNAL;
  if (cudaStreamSynchronize(st) != cudaSuccess) return PCC_INTERNAL;
  if (herr & kErrRange) return PCC_INVALID_ARGUMENT;
  if (herr & kErrDegree) return PCC_OUT_OF_RANGE;
  if (herr & kErrProbe) return PCC_INTERNAL;
  return PCC_OK;
}
