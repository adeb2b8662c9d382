// common.cuh -- shared host/device infrastructure of libpcc_gb300.so:
// status plumbing, the per-call device context, stream-ordered device
// buffers and small warp utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "pcc_gb300.h"

namespace pcc {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kFull = 0xFFFFFFFFu;

// Status carried through host code; converts 1:1 to pcc_status / absl codes.
struct Status {
  pcc_status code = PCC_OK;
  std::string msg;
  bool ok() const { return code == PCC_OK; }
  static Status Ok() { return {}; }
};

inline Status MakeError(pcc_status code, std::string msg) {
  Status s;
  s.code = code;
  s.msg = std::move(msg);
  return s;
}

#define PCC_RETURN_IF_ERROR(expr)            \
  do {                                       \
    ::pcc::Status _st = (expr);              \
    if (!_st.ok()) return _st;               \
  } while (0)

#define PCC_CUDA(expr)                                                          \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess)                                                      \
      return ::pcc::MakeError(PCC_INTERNAL, std::string(#expr) + ": " +         \
                                                cudaGetErrorString(_e));        \
  } while (0)

// ---------------------------------------------------------------------------
// Context: one device, one stream, one stream-ordered pool with an optional
// HBM budget.  All kernels of a call run on `stream`.
// ---------------------------------------------------------------------------
struct PhaseTimer;

// Best-move kernel families, timed and counted separately (roofline of the
// dominant kernel): lane groups (degree <= 32), warps (<= 1000), small hubs,
// big hubs.
constexpr int kFamGroup = 0;
constexpr int kFamWarp = 1;
constexpr int kFamHubSmall = 2;
constexpr int kFamHubBig = 3;
constexpr int kNumFamilies = 4;

struct Context {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;             // 0 = device capacity
  // Synchronous rounds run as a device-side graph loop (one host read per
  // level) unless detailed timing (CUDA events around every phase and kernel
  // family, host-driven rounds) is on, or graphs are unavailable.
  bool detailed_timing = false;
  bool graphs_failed = false;
  // Levels (and union levels) with fewer entries run host-driven rounds.
  // Capturing and instantiating a level's loop takes driver locks that
  // concurrent worker contexts contend for, so the serving pool's workers set
  // it above any graph size.
  uint64_t device_loop_min_entries = 0;
  std::atomic<uint64_t> in_use{0};
  std::atomic<uint64_t> peak{0};   // high-water mark of in_use
  std::mutex mu;
  std::unordered_map<void*, uint64_t> sizes;
  std::string last_error;
  // Kernel-family timing of the running call (null when not requested).
  PhaseTimer* fam_timer = nullptr;
  uint64_t fam_launches[kNumFamilies] = {0, 0, 0, 0};
  // CUDA events reused across calls (event creation takes a runtime lock
  // that serialises concurrent contexts).
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t GetEvent() {
    if (event_pool.empty()) {
      cudaEvent_t e = nullptr;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = event_pool.back();
    event_pool.pop_back();
    return e;
  }
  void PutEvent(cudaEvent_t e) {
    if (e) event_pool.push_back(e);
  }
  // Side streams for the best-move kernel families of a synchronous round:
  // the warp and hub launches run on streams forked from `stream` (an event
  // recorded there) and joined back into it, so their kernels overlap the
  // lane-group kernels and each other.  Under stream capture the fork and
  // the join become parallel branches of the captured graph.
  static constexpr int kSideStreams = 3;
  cudaStream_t side[kSideStreams] = {nullptr, nullptr, nullptr};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[kSideStreams] = {nullptr, nullptr, nullptr};
  bool overlap_families = true;  // off: every family on `stream` in turn
  // Best-move launch shape set by pcc_set_launch_tuning (tuned false: the
  // compiled-in table by graph size).
  bool tuned = false;
  uint32_t group_max_degree = 32;
  uint32_t cta_min_degree = 1000;
  float grid_waves = 1.0f;
  Status EnsureSideStreams() {
    if (fork_ev) return Status::Ok();
    for (int i = 0; i < kSideStreams; ++i) {
      PCC_CUDA(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
      PCC_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
    }
    PCC_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    return Status::Ok();
  }
  ~Context() {
    for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
    for (int i = 0; i < kSideStreams; ++i) {
      if (side[i]) cudaStreamDestroy(side[i]);
      if (join_ev[i]) cudaEventDestroy(join_ev[i]);
    }
    if (fork_ev) cudaEventDestroy(fork_ev);
  }

  Status Alloc(void** p, uint64_t bytes) {
    *p = nullptr;
    if (bytes == 0) return Status::Ok();
    bytes = (bytes + 255) & ~uint64_t(255);
    if (budget && in_use.load() + bytes > budget)
      return MakeError(PCC_RESOURCE_EXHAUSTED,
                       "HBM budget exceeded: need " + std::to_string(bytes) +
                           " more bytes, " + std::to_string(in_use.load()) +
                           " of " + std::to_string(budget) + " in use");
    cudaError_t e = cudaMallocAsync(p, bytes, stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return MakeError(PCC_RESOURCE_EXHAUSTED,
                       std::string("device allocation of ") +
                           std::to_string(bytes) + " bytes failed: " +
                           cudaGetErrorString(e));
    }
    const uint64_t now = in_use += bytes;
    uint64_t pk = peak.load();
    while (now > pk && !peak.compare_exchange_weak(pk, now)) {
    }
    std::lock_guard<std::mutex> lk(mu);
    sizes[*p] = bytes;
    return Status::Ok();
  }
  void Free(void* p) {
    if (!p) return;
    cudaFreeAsync(p, stream);
    std::lock_guard<std::mutex> lk(mu);
    auto it = sizes.find(p);
    if (it != sizes.end()) {
      in_use -= it->second;
      sizes.erase(it);
    }
  }
};

// Stream-ordered device array owned by a context.
template <class T>
struct DBuf {
  Context* ctx = nullptr;
  T* p = nullptr;
  uint64_t count = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept { *this = std::move(o); }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      Release();
      ctx = o.ctx;
      p = o.p;
      count = o.count;
      o.p = nullptr;
      o.count = 0;
    }
    return *this;
  }
  ~DBuf() { Release(); }
  Status Alloc(Context* c, uint64_t n) {
    Release();
    ctx = c;
    count = n;
    void* q = nullptr;
    PCC_RETURN_IF_ERROR(c->Alloc(&q, n * sizeof(T)));
    p = static_cast<T*>(q);
    return Status::Ok();
  }
  // Grows to at least n elements (contents not preserved).
  Status Reserve(Context* c, uint64_t n) {
    if (p && count >= n) return Status::Ok();
    return Alloc(c, n);
  }
  void Release() {
    if (p && ctx) ctx->Free(p);
    p = nullptr;
    count = 0;
  }
  Status Zero() {
    if (count) PCC_CUDA(cudaMemsetAsync(p, 0, count * sizeof(T), ctx->stream));
    return Status::Ok();
  }
  Status Fill(int byte) {
    if (count) PCC_CUDA(cudaMemsetAsync(p, byte, count * sizeof(T), ctx->stream));
    return Status::Ok();
  }
  Status FromHost(const T* h, uint64_t n) {
    if (n) PCC_CUDA(cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return Status::Ok();
  }
  Status ToHost(T* h, uint64_t n) const {
    if (n) PCC_CUDA(cudaMemcpyAsync(h, p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    return Status::Ok();
  }
};

// Launches issued while this is alive go to side stream i of the context
// (the launchers read ctx->stream).
struct OnSideStream {
  Context* ctx;
  cudaStream_t saved;
  OnSideStream(Context* c, int i) : ctx(c), saved(c->stream) { c->stream = c->side[i]; }
  ~OnSideStream() { ctx->stream = saved; }
  OnSideStream(const OnSideStream&) = delete;
  OnSideStream& operator=(const OnSideStream&) = delete;
};

inline Status Sync(Context* c) {
  PCC_CUDA(cudaStreamSynchronize(c->stream));
  PCC_CUDA(cudaGetLastError());
  return Status::Ok();
}

inline Status LaunchCheck() {
  PCC_CUDA(cudaGetLastError());
  return Status::Ok();
}

// Count of kernel launches issued by this library on the calling host
// thread (a call runs on one thread and reports the difference across its
// own duration; concurrent calls on other threads do not disturb it).
inline uint64_t& LaunchCounter() {
  thread_local uint64_t c = 0;
  return c;
}
#define PCC_COUNT(k) (::pcc::LaunchCounter() += (k))

// CUDA-event spans of named phases on the context stream; totals are read
// after the stream has been synchronised.  Events come from the context's
// pool and go back to it.
struct PhaseTimer {
  Context* ctx;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> spans[4];
  cudaEvent_t open[4] = {nullptr, nullptr, nullptr, nullptr};
  bool enabled = true;  // off while work is captured into a graph
  explicit PhaseTimer(Context* c) : ctx(c) {}
  PhaseTimer(const PhaseTimer&) = delete;
  PhaseTimer& operator=(const PhaseTimer&) = delete;
  void Begin(int k) {
    if (!enabled) return;
    open[k] = ctx->GetEvent();
    cudaEventRecord(open[k], ctx->stream);
  }
  void End(int k) {
    if (!enabled) return;
    cudaEvent_t e = ctx->GetEvent();
    cudaEventRecord(e, ctx->stream);
    spans[k].emplace_back(open[k], e);
    open[k] = nullptr;
  }
  double TotalMs(int k) const {
    double t = 0;
    for (const auto& sp : spans[k]) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, sp.first, sp.second) == cudaSuccess) t += ms;
    }
    return t;
  }
  ~PhaseTimer() {
    for (auto& v : spans)
      for (auto& sp : v) {
        ctx->PutEvent(sp.first);
        ctx->PutEvent(sp.second);
      }
    for (auto e : open) ctx->PutEvent(e);
  }
};
inline void FamBegin(Context* ctx, int f) {
  if (ctx->fam_timer) ctx->fam_timer->Begin(f);
}
inline void FamEnd(Context* ctx, int f, int launches) {
  if (ctx->fam_timer) ctx->fam_timer->End(f);
  ctx->fam_launches[f] += uint64_t(launches);
}

constexpr int kPhaseBestMoves = 0;
constexpr int kPhaseCompress = 1;
constexpr int kPhaseApply = 2;
constexpr int kPhaseFrontier = 3;

inline unsigned Blocks(uint64_t items, unsigned per_block, unsigned cap) {
  uint64_t b = (items + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return static_cast<unsigned>(b);
}

// ---------------------------------------------------------------------------
// Device helpers.
// ---------------------------------------------------------------------------
// FP32 image of an FP64 quantity for the pre-filter and the certified
// decision: the nearest float when the value is 0 or within [2^-100, 2^100],
// NaN otherwise (the relative-error model needs normal floats; a NaN
// candidate always survives the filter and makes a decision uncertain).
__host__ __device__ inline float FilterF32(double d) {
  const double m = d < 0 ? -d : d;
  if (d == 0.0 || (m >= 7.888609052210118e-31 && m <= 1.2676506002282294e30)) return static_cast<float>(d);
#ifdef __CUDA_ARCH__
  return __int_as_float(0x7fc00000);
#else
  return std::numeric_limits<float>::quiet_NaN();
#endif
}

// A 32-bit match key no cluster id can take: graphs have at most
// kMaxVertices vertices, so ids stay below 0xFFFFFFE0.  (A 64-bit
// __match_any_sync key costs far more than a 32-bit one.)
constexpr uint32_t kMaxVertices = 0xFFFFFFE0u;
__device__ __forceinline__ uint32_t LaneSentinel(unsigned lane) { return 0xFFFFFFE0u | lane; }

__device__ __forceinline__ unsigned LaneId() {
  unsigned r;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned LaneMaskLt() {
  unsigned r;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}

// IEEE double arithmetic without contraction into FMA: the reference's
// values are computed with separate roundings (built with the oracle's
// -ffp-contract=off), so every step here rounds separately too.
__device__ __forceinline__ double Dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double Dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double Dsub(double a, double b) { return __dsub_rn(a, b); }

}  // namespace pcc

// The opaque C-ABI types.
struct pcc_context {
  pcc::Context c;
};
