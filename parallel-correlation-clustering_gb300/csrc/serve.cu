// serve.cu -- batched clustering and the serving loop (host code).
//
// Many independent graphs run concurrently on one GPU: a pool of worker
// threads, each owning a context (its own non-blocking CUDA stream), takes
// requests from a FIFO queue and runs the single-graph path
// (pcc_cluster_host_csr) on them, so the kernels of different graphs overlap
// on the device while every result stays identical to a standalone call.
// Admission is continuous: a queued request starts as soon as a worker is
// free and its device-memory estimate fits the HBM budget beside the
// requests already running.  pcc_cluster_batch drives the same pool with
// requests that point at the caller's arrays; the server copies them.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace pcc {
namespace {

using Clock = std::chrono::steady_clock;

// Pool workers drive the rounds from the host: concurrent per-level graph
// captures and instantiations contend for driver locks, which cost the
// serving mix more capacity than the device-side loop saves.
constexpr uint64_t kPoolDeviceLoopMinEntries = ~0ull;

double MsBetween(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
  uint64_t ticket = 0;
  uint32_t n = 0;
  uint64_t m = 0;
  // Graph arrays: the owned copies (server) or the caller's arrays (batch).
  std::vector<uint64_t> off_own;
  std::vector<uint32_t> nbr_own;
  std::vector<float> w_own;
  std::vector<double> k_own;
  const uint64_t* off = nullptr;
  const uint32_t* nbr = nullptr;
  const float* w = nullptr;
  const double* k = nullptr;
  pcc_config cfg{};
  int32_t objective = 0;
  uint64_t est_bytes = 0;
  // Results.
  uint32_t* labels_out = nullptr;       // batch: the caller's array
  std::vector<uint32_t> labels;         // server: kept until waited for
  pcc_stats stats{};
  pcc_stats* stats_out = nullptr;       // batch: the caller's slot
  pcc_status status = PCC_OK;
  bool done = false;
  Clock::time_point t_submit, t_start, t_end;
};

// A request that can share a disjoint-union run (pcc_cluster_union):
// synchronous LOUVAIN moves without subclustering; modularity needs offset 0.
bool UnionEligible(const Request& r) {
  return r.n > 0 && r.cfg.clustering_moves_method == PCC_LOUVAIN && !r.cfg.async &&
         r.cfg.subclustering_method == PCC_NONE_SUBCLUSTERING &&
         (r.objective == 0 || r.cfg.edge_weight_offset == 0);
}

// Two eligible requests share a run when their configs differ in resolution
// only (and, with modularity in the run, the offset is 0 -- checked above).
bool SameRunConfig(const Request& a, const Request& b) {
  pcc_config x = a.cfg, y = b.cfg;
  x.resolution = 0;
  y.resolution = 0;
  if (std::memcmp(&x, &y, sizeof(pcc_config)) != 0) return false;
  return (a.objective == 0 && b.objective == 0) || a.cfg.edge_weight_offset == 0;
}

constexpr size_t kMaxGroupGraphs = 64;
constexpr uint64_t kMaxGroupEntries = 8ull << 20;

class Pool {
 public:
  // group_unions: a worker that takes a union-eligible request also takes
  // the queued requests with the same config (up to kMaxGroupGraphs graphs
  // and kMaxGroupEntries entries, within the budget) and runs them as one
  // disjoint union; every label and objective equals its standalone call.
  Pool(int device, uint32_t slots, uint64_t budget, bool group_unions = false)
      : device_(device), budget_(budget), group_unions_(group_unions) {
    slots_ = std::max<uint32_t>(1, slots);
  }

  pcc_status Start() {
    for (uint32_t i = 0; i < slots_; ++i) {
      pcc_context* c = nullptr;
      const pcc_status s = pcc_create(&c, device_, 0);
      if (s != PCC_OK) {
        Stop();
        return s;
      }
      c->c.device_loop_min_entries = kPoolDeviceLoopMinEntries;
      ctxs_.push_back(c);
    }
    for (uint32_t i = 0; i < slots_; ++i) workers_.emplace_back([this, i] { Work(i); });
    return PCC_OK;
  }

  // Finishes running requests, cancels queued ones, joins the workers.
  void Stop() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      for (Request* r : queue_) Finish(r, PCC_CANCELLED);
      queue_.clear();
    }
    cv_work_.notify_all();
    for (auto& t : workers_) t.join();
    workers_.clear();
    for (pcc_context* c : ctxs_) pcc_destroy(c);
    ctxs_.clear();
  }

  ~Pool() { Stop(); }

  pcc_status Submit(Request* r) {
    r->t_submit = Clock::now();
    if (budget_ && r->est_bytes > budget_) return PCC_RESOURCE_EXHAUSTED;
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (stop_) return PCC_CANCELLED;
      queue_.push_back(r);
    }
    cv_work_.notify_all();
    return PCC_OK;
  }

  // Waits until r is done or the deadline passes; true when done.
  bool Wait(Request* r, int32_t wait_ms) {
    std::unique_lock<std::mutex> lk(mu_);
    if (wait_ms < 0) {
      cv_done_.wait(lk, [&] { return r->done; });
      return true;
    }
    return cv_done_.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return r->done; });
  }

  std::mutex& mu() { return mu_; }

 private:
  void Finish(Request* r, pcc_status s) {  // mu_ held
    r->status = s;
    r->t_end = Clock::now();
    r->done = true;
    cv_done_.notify_all();
  }

  static uint32_t* OutOf(Request* r) {
    if (r->labels_out) return r->labels_out;
    r->labels.resize(std::max<uint32_t>(r->n, 1));
    return r->labels.data();
  }

  void Work(uint32_t slot) {
    pcc_context* ctx = ctxs_[slot];
    cudaSetDevice(device_);
    for (;;) {
      std::vector<Request*> group;
      {
        std::unique_lock<std::mutex> lk(mu_);
        // First come, first served: the head of the queue runs when its
        // estimate fits beside the admitted requests.
        cv_work_.wait(lk, [&] {
          return stop_ || (!queue_.empty() && (!budget_ || reserved_ + queue_.front()->est_bytes <= budget_));
        });
        if (stop_) return;
        const auto now = Clock::now();
        Request* r = queue_.front();
        queue_.pop_front();
        reserved_ += r->est_bytes;
        r->t_start = now;
        group.push_back(r);
        if (group_unions_ && UnionEligible(*r)) {
          uint64_t entries = r->m;
          for (auto it = queue_.begin(); it != queue_.end() && group.size() < kMaxGroupGraphs;) {
            Request* q = *it;
            if (UnionEligible(*q) && SameRunConfig(*q, *r) &&
                entries + q->m <= kMaxGroupEntries && (!budget_ || reserved_ + q->est_bytes <= budget_)) {
              reserved_ += q->est_bytes;
              q->t_start = now;
              entries += q->m;
              group.push_back(q);
              it = queue_.erase(it);
            } else {
              ++it;
            }
          }
        }
      }
      std::vector<pcc_status> st(group.size(), PCC_OK);
      bool done = false;
      if (group.size() > 1) {
        std::vector<pcc_batch_graph> gs;
        std::vector<uint32_t*> outs;
        std::vector<pcc_stats> stats(group.size());
        std::vector<pcc_config> cfgs;
        std::vector<int32_t> objs;
        for (Request* q : group) {
          gs.push_back(pcc_batch_graph{q->n, q->m, q->off, q->nbr, q->w, q->objective == 1 ? nullptr : q->k});
          outs.push_back(OutOf(q));
          cfgs.push_back(q->cfg);
          objs.push_back(q->objective);
        }
        if (pcc_cluster_union(ctx, static_cast<uint32_t>(group.size()), gs.data(), cfgs.data(),
                              static_cast<uint32_t>(cfgs.size()), objs.data(), 0, outs.data(), stats.data(),
                              nullptr) == PCC_OK) {
          for (size_t i = 0; i < group.size(); ++i) group[i]->stats = stats[i];
          done = true;
        }
      }
      if (!done) {  // one request, or the union failed: standalone calls
        for (size_t i = 0; i < group.size(); ++i) {
          Request* r = group[i];
          st[i] = pcc_cluster_host_csr(ctx, r->n, r->m, r->off, r->nbr, r->w, &r->cfg, r->objective,
                                       r->objective == 1 ? nullptr : r->k, OutOf(r), &r->stats);
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu_);
        for (size_t i = 0; i < group.size(); ++i) {
          Request* r = group[i];
          if (r->stats_out) *r->stats_out = r->stats;
          reserved_ -= r->est_bytes;
          Finish(r, st[i]);
        }
      }
      cv_work_.notify_all();  // memory was released: the queue head may fit now
    }
  }

  int device_;
  uint32_t slots_;
  uint64_t budget_;
  bool group_unions_ = false;
  uint64_t reserved_ = 0;
  bool stop_ = false;
  std::vector<pcc_context*> ctxs_;
  std::vector<std::thread> workers_;
  std::deque<Request*> queue_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
};

}  // namespace
}  // namespace pcc

using pcc::Clock;
using pcc::Pool;
using pcc::Request;

struct pcc_server {
  std::unique_ptr<Pool> pool;
  std::mutex mu;
  uint64_t next_ticket = 1;
  // Shared so that a waiter keeps its request alive after another waiter of
  // the same ticket has collected and erased it.
  std::unordered_map<uint64_t, std::shared_ptr<Request>> requests;
};

extern "C" {

// Device memory of one clustering call: the uploaded CSR and per-level
// state, the engine's per-round arrays, and the contraction of level 0
// (sort keys and values with their double buffers) -- the peak -- plus a
// fixed allowance for pools and small tables.
uint64_t pcc_request_bytes_estimate(uint32_t n, uint64_t m, int32_t has_weights) {
  const uint64_t per_entry = 52 + (has_weights ? 8 : 0);
  return per_entry * m + 192ull * n + (64ull << 20);
}

pcc_status pcc_cluster_batch(int device, uint32_t num_graphs, const pcc_batch_graph* graphs,
                             const pcc_config* configs, uint32_t num_configs, const int32_t* objectives,
                             uint32_t concurrency, uint64_t hbm_budget, uint32_t* const* out_labels,
                             pcc_stats* stats, double* wall_ms) {
  if (num_graphs == 0) {
    if (wall_ms) *wall_ms = 0;
    return PCC_OK;
  }
  if (!graphs || !configs || !out_labels || (num_configs != 1 && num_configs != num_graphs))
    return PCC_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < num_graphs; ++i) {
    if (!out_labels[i] || !graphs[i].offsets || (graphs[i].m && !graphs[i].neighbors)) return PCC_INVALID_ARGUMENT;
    if (objectives && objectives[i] != 0 && objectives[i] != 1) return PCC_INVALID_ARGUMENT;
  }
  const auto t0 = Clock::now();
  // Configs that differ in resolution only: disjoint unions on one context.
  bool as_union = configs[0].clustering_moves_method == PCC_LOUVAIN && !configs[0].async &&
                  configs[0].subclustering_method == PCC_NONE_SUBCLUSTERING;
  for (uint32_t i = 1; as_union && i < num_configs; ++i) {
    pcc_config x = configs[i], y = configs[0];
    x.resolution = 0;
    y.resolution = 0;
    as_union = std::memcmp(&x, &y, sizeof(pcc_config)) == 0;
  }
  for (uint32_t i = 0; as_union && objectives && i < num_graphs; ++i)
    as_union = objectives[i] == 0 || configs[0].edge_weight_offset == 0;
  if (as_union) {
    pcc_context* c = nullptr;
    pcc_status s = pcc_create(&c, device, hbm_budget);
    if (s != PCC_OK) return s;
    // Under a budget, a union's entries are capped so that its device bytes
    // (about 60 B per entry plus 192 B per vertex, at most one new vertex
    // per entry counted) fit next to the fixed 64 MB.
    const uint64_t fixed = 64ull << 20;
    const uint64_t cap = hbm_budget == 0 ? 0 : std::max<uint64_t>(1, (hbm_budget > fixed ? hbm_budget - fixed : 0) / 252);
    // Graphs packed in ascending entry count (stable): unions of similar
    // graphs end their levels and rounds closer together, so fewer launches
    // run for a few stragglers.  Every graph's result is independent of its
    // union, so the order changes no label.
    std::vector<uint32_t> order(num_graphs);
    for (uint32_t i = 0; i < num_graphs; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return graphs[a].m < graphs[b].m; });
    std::vector<pcc_batch_graph> sg(num_graphs);
    std::vector<pcc_config> sc(num_configs);
    std::vector<int32_t> so(objectives ? num_graphs : 0);
    std::vector<uint32_t*> sl(num_graphs);
    std::vector<pcc_stats> ss(stats ? num_graphs : 0);
    for (uint32_t i = 0; i < num_graphs; ++i) {
      sg[i] = graphs[order[i]];
      sl[i] = out_labels[order[i]];
      if (objectives) so[i] = objectives[order[i]];
      if (num_configs != 1) sc[i] = configs[order[i]];
    }
    if (num_configs == 1) sc[0] = configs[0];
    s = pcc_cluster_union(c, num_graphs, sg.data(), sc.data(), num_configs, objectives ? so.data() : nullptr, cap,
                          sl.data(), stats ? ss.data() : nullptr, nullptr);
    if (stats)
      for (uint32_t i = 0; i < num_graphs; ++i) stats[order[i]] = ss[i];
    pcc_destroy(c);
    if (wall_ms) *wall_ms = pcc::MsBetween(t0, Clock::now());
    return s;
  }
  Pool pool(device, std::min(std::max<uint32_t>(concurrency, 1), num_graphs), hbm_budget);
  pcc_status s = pool.Start();
  if (s != PCC_OK) return s;
  std::vector<Request> reqs(num_graphs);
  for (uint32_t i = 0; i < num_graphs; ++i) {
    Request& r = reqs[i];
    const pcc_batch_graph& g = graphs[i];
    r.ticket = i;
    r.n = g.n;
    r.m = g.m;
    r.off = g.offsets;
    r.nbr = g.neighbors;
    r.w = g.weights;
    r.k = g.node_weights;
    r.cfg = configs[num_configs == 1 ? 0 : i];
    r.objective = objectives ? objectives[i] : 0;
    r.est_bytes = pcc_request_bytes_estimate(g.n, g.m, g.weights != nullptr);
    r.labels_out = out_labels[i];
    r.stats_out = stats ? stats + i : nullptr;
  }
  pcc_status first = PCC_OK;
  uint32_t submitted = 0;
  for (; submitted < num_graphs; ++submitted) {
    const pcc_status ss = pool.Submit(&reqs[submitted]);
    if (ss != PCC_OK) {
      first = ss;
      break;
    }
  }
  for (uint32_t i = 0; i < submitted; ++i) {
    pool.Wait(&reqs[i], -1);
    if (first == PCC_OK && reqs[i].status != PCC_OK) first = reqs[i].status;
  }
  pool.Stop();
  if (wall_ms) *wall_ms = pcc::MsBetween(t0, Clock::now());
  return first;
}

pcc_status pcc_server_create(pcc_server** out, int device, uint32_t slots, uint64_t hbm_budget) {
  if (!out) return PCC_INVALID_ARGUMENT;
  *out = nullptr;
  auto s = std::make_unique<pcc_server>();
  s->pool = std::make_unique<Pool>(device, slots, hbm_budget, /*group_unions=*/true);
  const pcc_status st = s->pool->Start();
  if (st != PCC_OK) return st;
  *out = s.release();
  return PCC_OK;
}

pcc_status pcc_server_submit(pcc_server* server, uint32_t n, uint64_t m, const uint64_t* offsets,
                             const uint32_t* neighbors, const float* weights, const double* node_weights,
                             const pcc_config* config, int32_t objective, uint64_t* ticket) {
  if (!server || !offsets || (m && !neighbors) || !config || !ticket || (objective != 0 && objective != 1))
    return PCC_INVALID_ARGUMENT;
  auto r = std::make_shared<Request>();
  r->n = n;
  r->m = m;
  r->off_own.assign(offsets, offsets + uint64_t(n) + 1);
  r->nbr_own.assign(neighbors, neighbors + m);
  if (weights) r->w_own.assign(weights, weights + m);
  if (node_weights) r->k_own.assign(node_weights, node_weights + n);
  r->off = r->off_own.data();
  r->nbr = r->nbr_own.data();
  r->w = weights ? r->w_own.data() : nullptr;
  r->k = node_weights ? r->k_own.data() : nullptr;
  r->cfg = *config;
  r->objective = objective;
  r->est_bytes = pcc_request_bytes_estimate(n, m, weights != nullptr);
  Request* raw = r.get();
  {
    std::lock_guard<std::mutex> lk(server->mu);
    r->ticket = server->next_ticket++;
    *ticket = r->ticket;
    server->requests[r->ticket] = r;
  }
  const pcc_status s = server->pool->Submit(raw);
  if (s != PCC_OK) {
    std::lock_guard<std::mutex> lk(server->mu);
    server->requests.erase(*ticket);
    *ticket = 0;
  }
  return s;
}

pcc_status pcc_server_wait(pcc_server* server, uint64_t ticket, int32_t wait_ms, uint32_t* out_labels,
                           pcc_stats* stats, double* latency_ms, double* queue_ms) {
  if (!server) return PCC_INVALID_ARGUMENT;
  std::shared_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lk(server->mu);
    auto it = server->requests.find(ticket);
    if (it == server->requests.end()) return PCC_NOT_FOUND;
    r = it->second;
  }
  if (!server->pool->Wait(r.get(), wait_ms)) return PCC_DEADLINE_EXCEEDED;
  const pcc_status s = r->status;
  if (s == PCC_OK && out_labels && r->n) std::memcpy(out_labels, r->labels.data(), sizeof(uint32_t) * r->n);
  if (stats) *stats = r->stats;
  if (latency_ms) *latency_ms = pcc::MsBetween(r->t_submit, r->t_end);
  if (queue_ms) *queue_ms = r->t_start.time_since_epoch().count() ? pcc::MsBetween(r->t_submit, r->t_start) : 0.0;
  std::lock_guard<std::mutex> lk(server->mu);
  server->requests.erase(ticket);
  return s;
}

void pcc_server_destroy(pcc_server* server) {
  if (!server) return;
  server->pool->Stop();
  delete server;
}

}  // extern "C"
