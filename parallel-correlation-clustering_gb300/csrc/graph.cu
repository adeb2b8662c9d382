// graph.cu -- context lifetime, graph upload / download and graph
// properties (C ABI).  A graph upload replaces GbbsGraph::Import /
// FinishImport (clustering/gbbs-graph.cc:32-76) and the CLI's CopyGraph
// (clustering/cluster-in-memory_main.cc:231-306): the CSR arrays are copied
// once into HBM and stay there for every clustering call.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "graphops.cuh"
#include "hubs.cuh"

namespace pcc {

namespace {

struct DegreeInput {
  const uint64_t* off;
  __device__ uint32_t operator()(uint64_t i) const { return static_cast<uint32_t>(off[i + 1] - off[i]); }
};

// Non-integral weight count and max |w| (as float bits of the magnitude).
// Weight statistics: non-integral count, max |w| and the sum of |w| over
// integral weights below 2^32 (saturating; it bounds every row's sum).
struct WeightStats {
  unsigned long long nonint;
  float maxabs;
  unsigned long long sumabs;
};
struct WeightInput {
  const float* w;
  __device__ WeightStats operator()(uint64_t i) const {
    const float x = w[i];
    WeightStats r;
    r.nonint = (x != truncf(x) || isnan(x) || isinf(x)) ? 1ull : 0ull;
    r.maxabs = fabsf(x);
    r.sumabs = r.maxabs < 4294967296.0f ? __float2uint_rz(r.maxabs) : 0xFFFFFFFFull;
    return r;
  }
};
struct WeightOp {
  __device__ WeightStats operator()(WeightStats a, WeightStats b) const {
    WeightStats r;
    r.nonint = a.nonint + b.nonint;
    r.maxabs = fmaxf(a.maxabs, b.maxabs);
    r.sumabs = a.sumabs + b.sumabs;
    if (r.sumabs < a.sumabs) r.sumabs = ~0ull;
    return r;
  }
};

__global__ void CheckCsrKernel(uint32_t n, uint64_t m, const uint64_t* __restrict__ off,
                               const uint32_t* __restrict__ nbr, int* bad) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i <= n; i += uint64_t(gridDim.x) * blockDim.x) {
    if (i == 0 && off[0] != 0) atomicExch(bad, 1);
    if (i == n && off[n] != m) atomicExch(bad, 2);
    if (i < n && off[i] > off[i + 1]) atomicExch(bad, 3);
  }
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < m; j += uint64_t(gridDim.x) * blockDim.x)
    if (nbr[j] >= n) atomicExch(bad, 4);
}

struct PredNonZeroDegree {
  const uint64_t* off;
  __device__ bool operator()(uint32_t v) const { return off[v + 1] > off[v]; }
};

Status BuildBins(Context* ctx, const DevGraph* g, BinSet* b, bool include_isolated) {
  PCC_RETURN_IF_ERROR(AllocBins(ctx, g->n, b));
  DBuf<unsigned long long> sum;
  DBuf<uint32_t> cnt;
  PCC_RETURN_IF_ERROR(sum.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(cnt.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(sum.Zero());
  PCC_RETURN_IF_ERROR(cnt.Zero());
  if (include_isolated) {
    PCC_RETURN_IF_ERROR(BinVertices(ctx, g->n, g->off.p, PredAll{}, b, sum.p, cnt.p));
  } else {
    PCC_RETURN_IF_ERROR(BinVertices(ctx, g->n, g->off.p, PredNonZeroDegree{g->off.p}, b, sum.p, cnt.p));
  }
  uint32_t hc[kNumBins];
  uint32_t hcnt = 0;
  unsigned long long hsum = 0;
  PCC_RETURN_IF_ERROR(b->counts.ToHost(hc, kNumBins));
  PCC_RETURN_IF_ERROR(cnt.ToHost(&hcnt, 1));
  PCC_RETURN_IF_ERROR(sum.ToHost(&hsum, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  for (int i = 0; i < kNumBins; ++i) b->host_counts[i] = hc[i];
  b->size = hcnt;
  b->edges = hsum;
  return Status::Ok();
}

}  // namespace

Status EnsureHubPlan(Context* ctx, const DevGraph* g) {
  if (g->hub_plan) return Status::Ok();
  auto plan = std::make_shared<HubPlan>();
  PCC_RETURN_IF_ERROR(BuildHubPlan(ctx, *g, g->bins, plan.get()));
  g->hub_plan = std::move(plan);
  return Status::Ok();
}

Status EnsureAllBins(Context* ctx, const DevGraph* g) {
  if (g->bins_all.list.p) return Status::Ok();
  return BuildBins(ctx, g, &g->bins_all, true);
}

__global__ void BinStartsKernel(const uint32_t* counts, uint32_t* starts, uint32_t* cursor) {
  uint32_t acc = 0;
  for (int b = 0; b < kNumBins; ++b) {
    starts[b] = acc;
    acc += counts[b];
    cursor[b] = 0;
  }
  starts[kNumBins] = acc;
}

Status ComputeGraphProperties(Context* ctx, DevGraph* g) {
  DBuf<uint32_t> part, out;
  PCC_RETURN_IF_ERROR(out.Alloc(ctx, 1));
  uint32_t maxd = 0;
  if (g->n) {
    PCC_RETURN_IF_ERROR(Reduce<uint32_t>(ctx, g->n, DegreeInput{g->off.p}, OpMax{}, 0u, out.p, part));
    PCC_RETURN_IF_ERROR(out.ToHost(&maxd, 1));
  }
  WeightStats ws{0, 1.0f, g->m};
  if (g->w.p && g->m) {
    DBuf<WeightStats> wpart, wout;
    PCC_RETURN_IF_ERROR(wout.Alloc(ctx, 1));
    PCC_RETURN_IF_ERROR(Reduce<WeightStats>(ctx, g->m, WeightInput{g->w.p}, WeightOp{}, WeightStats{0, 0.0f, 0},
                                            wout.p, wpart));
    PCC_RETURN_IF_ERROR(wout.ToHost(&ws, 1));
    PCC_RETURN_IF_ERROR(Sync(ctx));
  }
  PCC_RETURN_IF_ERROR(BuildBins(ctx, g, &g->bins, false));
  g->max_deg = maxd;
  g->integral = ws.nonint == 0;
  g->max_abs_w = ws.maxabs;
  // A row's sum of |w| is at most max|w| * degree and at most the total.
  g->row_abs_bound = std::min(static_cast<double>(ws.maxabs) * static_cast<double>(maxd),
                              static_cast<double>(ws.sumabs));
  return Status::Ok();
}

namespace {

// Union fix-up, vertices: offsets of graph j are shifted by ebase[j] (index
// vbase[j+1] belongs to graph j+1, whose copy wrote 0 there last); node
// weights of graphs without them are 1.
__global__ void UnionVertexFixKernel(uint32_t n, const uint32_t* __restrict__ vbase,
                                     const uint64_t* __restrict__ ebase, uint32_t B, uint64_t* off, double* k,
                                     const uint8_t* __restrict__ has_k) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v <= n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t j = GraphOf(vbase, B, static_cast<uint32_t>(v));
    off[v] += ebase[j];
    if (k && v < n && !has_k[j]) k[v] = 1.0;
  }
}

// Union fix-up, entries: local neighbour ids are checked against the
// graph's own n and shifted by vbase[j]; unweighted graphs get weight 1.
__global__ void UnionEntryFixKernel(uint64_t m, const uint32_t* __restrict__ vbase,
                                    const uint64_t* __restrict__ ebase, uint32_t B, uint32_t* nbr, float* w,
                                    const uint8_t* __restrict__ has_w, int* bad) {
  for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t j = GraphOf(ebase, B, e);
    const uint32_t x = nbr[e];
    if (x >= vbase[j + 1] - vbase[j]) {
      atomicExch(bad, 4);
      continue;
    }
    nbr[e] = x + vbase[j];
    if (w && !has_w[j]) w[e] = 1.0f;
  }
}

// Node weights = degrees on the graphs with has_k[j] == 2 (modularity).
__global__ void UnionDegreeWeightsKernel(uint32_t n, const uint64_t* __restrict__ off,
                                         const uint32_t* __restrict__ vbase, uint32_t B,
                                         const uint8_t* __restrict__ has_k, double* k) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x)
    if (has_k[GraphOf(vbase, B, static_cast<uint32_t>(v))] == 2)
      k[v] = static_cast<double>(off[v + 1] - off[v]);
}

}  // namespace

Status UploadUnion(Context* ctx, uint32_t B, const pcc_batch_graph* const* graphs, const uint8_t* degree_weights,
                   DevGraph* g, UnionLayout* u, DBuf<double>* k, bool* int_nw) {
  if (B == 0) return MakeError(PCC_INVALID_ARGUMENT, "empty union");
  u->B = B;
  u->vbase.assign(B + 1, 0);
  u->ebase.assign(B + 1, 0);
  bool any_w = false, any_k = false;
  *int_nw = true;
  std::vector<uint8_t> has_w(B), has_k(B);
  for (uint32_t j = 0; j < B; ++j) {
    const pcc_batch_graph& x = *graphs[j];
    if (x.n == 0) return MakeError(PCC_INVALID_ARGUMENT, "union graphs must have n > 0");
    if (!x.offsets || (x.m && !x.neighbors)) return MakeError(PCC_INVALID_ARGUMENT, "null offsets or neighbors");
    if (x.offsets[0] != 0 || x.offsets[x.n] != x.m)
      return MakeError(PCC_INVALID_ARGUMENT, "offsets must start at 0 and end at m");
    const uint64_t nv = uint64_t(u->vbase[j]) + x.n;
    const uint64_t ne = u->ebase[j] + x.m;
    if (nv > kMaxVertices) return MakeError(PCC_INVALID_ARGUMENT, "union has more than 2^32 - 32 vertices");
    if (ne >= 0xFFFFFFFFull) return MakeError(PCC_INVALID_ARGUMENT, "union has 2^32 or more entries");
    u->vbase[j + 1] = static_cast<uint32_t>(nv);
    u->ebase[j + 1] = ne;
    has_w[j] = x.weights != nullptr;
    has_k[j] = (degree_weights && degree_weights[j]) ? 2 : (x.node_weights != nullptr ? 1 : 0);
    any_w |= has_w[j] != 0;
    any_k |= has_k[j] != 0;
    if (x.node_weights && has_k[j] == 1)
      for (uint32_t v = 0; v < x.n && *int_nw; ++v)
        if (x.node_weights[v] != std::floor(x.node_weights[v])) *int_nw = false;
  }
  const uint32_t n = u->vbase[B];
  const uint64_t m = u->ebase[B];
  g->n = n;
  g->m = m;
  PCC_RETURN_IF_ERROR(g->off.Alloc(ctx, uint64_t(n) + 1));
  PCC_RETURN_IF_ERROR(g->nbr.Alloc(ctx, m ? m : 1));
  if (any_w) PCC_RETURN_IF_ERROR(g->w.Alloc(ctx, m ? m : 1));
  if (any_k) PCC_RETURN_IF_ERROR(k->Alloc(ctx, n));
  // Stream order matters for the offsets: graph j+1's copy overwrites the
  // shared index vbase[j+1] (graph j's value m_j) with 0.
  for (uint32_t j = 0; j < B; ++j) {
    const pcc_batch_graph& x = *graphs[j];
    PCC_CUDA(cudaMemcpyAsync(g->off.p + u->vbase[j], x.offsets, sizeof(uint64_t) * (uint64_t(x.n) + 1),
                             cudaMemcpyHostToDevice, ctx->stream));
    if (x.m) {
      PCC_CUDA(cudaMemcpyAsync(g->nbr.p + u->ebase[j], x.neighbors, sizeof(uint32_t) * x.m, cudaMemcpyHostToDevice,
                               ctx->stream));
      if (x.weights)
        PCC_CUDA(cudaMemcpyAsync(g->w.p + u->ebase[j], x.weights, sizeof(float) * x.m, cudaMemcpyHostToDevice,
                                 ctx->stream));
    }
    if (has_k[j] == 1)
      PCC_CUDA(cudaMemcpyAsync(k->p + u->vbase[j], x.node_weights, sizeof(double) * x.n, cudaMemcpyHostToDevice,
                               ctx->stream));
  }
  DBuf<uint64_t> d_ebase;
  DBuf<uint8_t> d_has_w, d_has_k;
  PCC_RETURN_IF_ERROR(u->d_vbase.Alloc(ctx, B + 1));
  PCC_RETURN_IF_ERROR(d_ebase.Alloc(ctx, B + 1));
  PCC_RETURN_IF_ERROR(d_has_w.Alloc(ctx, B));
  PCC_RETURN_IF_ERROR(d_has_k.Alloc(ctx, B));
  PCC_RETURN_IF_ERROR(u->d_vbase.FromHost(u->vbase.data(), B + 1));
  PCC_RETURN_IF_ERROR(d_ebase.FromHost(u->ebase.data(), B + 1));
  PCC_RETURN_IF_ERROR(d_has_w.FromHost(has_w.data(), B));
  PCC_RETURN_IF_ERROR(d_has_k.FromHost(has_k.data(), B));
  DBuf<int> bad;
  PCC_RETURN_IF_ERROR(bad.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(bad.Zero());
  const unsigned cap = unsigned(ctx->num_sms) * 8;
  UnionVertexFixKernel<<<Blocks(uint64_t(n) + 1, 256, cap), 256, 0, ctx->stream>>>(
      n, u->d_vbase.p, d_ebase.p, B, g->off.p, any_k ? k->p : nullptr, d_has_k.p); PCC_COUNT(1);
  if (m) {
    UnionEntryFixKernel<<<Blocks(m, 256, cap), 256, 0, ctx->stream>>>(m, u->d_vbase.p, d_ebase.p, B, g->nbr.p,
                                                                       g->w.p, d_has_w.p, bad.p); PCC_COUNT(1);
  }
  CheckCsrKernel<<<Blocks(std::max<uint64_t>(m, uint64_t(n) + 1), 256, cap), 256, 0, ctx->stream>>>(
      n, m, g->off.p, g->nbr.p, bad.p); PCC_COUNT(1);
  if (any_k) {
    UnionDegreeWeightsKernel<<<Blocks(n, 256, cap), 256, 0, ctx->stream>>>(n, g->off.p, u->d_vbase.p, B, d_has_k.p,
                                                                          k->p); PCC_COUNT(1);
  }
  int hbad = 0;
  PCC_RETURN_IF_ERROR(bad.ToHost(&hbad, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  if (hbad)
    return MakeError(PCC_INVALID_ARGUMENT,
                     hbad == 4 ? "neighbor id out of range" : "offsets are not a valid CSR row index");
  return ComputeGraphProperties(ctx, g);
}

namespace {

Status Upload(pcc_context* pctx, uint32_t n, uint64_t m, const uint64_t* off, const uint32_t* nbr, const float* w,
              bool device_src, pcc_graph** out) {
  if (!pctx || !out) return MakeError(PCC_INVALID_ARGUMENT, "null context or output");
  if (!off || (m && !nbr)) return MakeError(PCC_INVALID_ARGUMENT, "null offsets or neighbors");
  if (m >= 0xFFFFFFFFull) return MakeError(PCC_INVALID_ARGUMENT, "graphs with 2^32 or more entries are not supported");
  if (n > kMaxVertices) return MakeError(PCC_INVALID_ARGUMENT, "n must be at most 2^32 - 32");
  Context* ctx = &pctx->c;
  if (!device_src) {
    if (off[0] != 0 || off[n] != m)
      return MakeError(PCC_INVALID_ARGUMENT, "offsets must start at 0 and end at m");
  }
  auto h = std::make_unique<pcc_graph>();
  DevGraph& g = h->g;
  g.n = n;
  g.m = m;
  const cudaMemcpyKind kind = device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  PCC_RETURN_IF_ERROR(g.off.Alloc(ctx, uint64_t(n) + 1));
  PCC_RETURN_IF_ERROR(g.nbr.Alloc(ctx, m ? m : 1));
  PCC_CUDA(cudaMemcpyAsync(g.off.p, off, sizeof(uint64_t) * (uint64_t(n) + 1), kind, ctx->stream));
  if (m) PCC_CUDA(cudaMemcpyAsync(g.nbr.p, nbr, sizeof(uint32_t) * m, kind, ctx->stream));
  if (w) {
    PCC_RETURN_IF_ERROR(g.w.Alloc(ctx, m ? m : 1));
    if (m) PCC_CUDA(cudaMemcpyAsync(g.w.p, w, sizeof(float) * m, kind, ctx->stream));
  }
  DBuf<int> bad;
  PCC_RETURN_IF_ERROR(bad.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(bad.Zero());
  CheckCsrKernel<<<Blocks(std::max<uint64_t>(m, n + 1), 256, unsigned(ctx->num_sms) * 8), 256, 0, ctx->stream>>>(
      n, m, g.off.p, g.nbr.p, bad.p); PCC_COUNT(1);
  int hbad = 0;
  PCC_RETURN_IF_ERROR(bad.ToHost(&hbad, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  if (hbad)
    return MakeError(PCC_INVALID_ARGUMENT,
                     hbad == 4 ? "neighbor id out of range" : "offsets are not a valid CSR row index");
  PCC_RETURN_IF_ERROR(ComputeGraphProperties(ctx, &g));
  *out = h.release();
  return Status::Ok();
}

pcc_status Done(pcc_context* ctx, const Status& st) {
  if (ctx) ctx->c.last_error = st.ok() ? std::string() : st.msg;
  return st.code;
}

}  // namespace
}  // namespace pcc

using namespace pcc;

extern "C" {

void pcc_config_default(pcc_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->clustering_moves_method = PCC_LOUVAIN;
  c->subclustering_method = PCC_NONE_SUBCLUSTERING;
  c->move_method = PCC_NBHR_CLUSTER_MOVE;
}

const char* pcc_version(void) { return "pcc_gb300 0.1.0 (sm_103a)"; }

pcc_status pcc_create(pcc_context** out, int device, uint64_t hbm_budget_bytes) {
  if (!out) return PCC_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return PCC_UNAVAILABLE;
  }
  if (device < 0 || device >= count) return PCC_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return PCC_UNAVAILABLE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PCC_UNAVAILABLE;
  auto* h = new pcc_context;
  Context& c = h->c;
  c.device = device;
  c.num_sms = prop.multiProcessorCount;
  c.smem_optin = prop.sharedMemPerBlockOptin;
  c.budget = hbm_budget_bytes;
  // PCC_SERIAL_FAMILIES=1 runs the best-move kernel families one after the
  // other on the context stream instead of as parallel branches (same
  // results; for comparisons).
  if (const char* e = std::getenv("PCC_SERIAL_FAMILIES")) c.overlap_families = std::strcmp(e, "1") != 0;
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return PCC_UNAVAILABLE;
  }
  // Keep freed pool memory cached between calls (no release to the OS).
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t threshold = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  *out = h;
  return PCC_OK;
}

void pcc_destroy(pcc_context* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  cudaStreamDestroy(ctx->c.stream);
  delete ctx;
}

const char* pcc_last_error(const pcc_context* ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

uint64_t pcc_device_bytes_in_use(const pcc_context* ctx) { return ctx ? ctx->c.in_use.load() : 0; }

void pcc_set_detailed_timing(pcc_context* ctx, int32_t on) {
  if (ctx) ctx->c.detailed_timing = on != 0;
}

pcc_status pcc_set_launch_tuning(pcc_context* ctx, uint32_t group_max_degree, uint32_t cta_min_degree,
                                 float grid_waves) {
  if (!ctx) return PCC_INVALID_ARGUMENT;
  if (group_max_degree == 0 && cta_min_degree == 0 && grid_waves == 0.0f) {
    ctx->c.tuned = false;
    return PCC_OK;
  }
  const bool g_ok = group_max_degree == 4 || group_max_degree == 8 || group_max_degree == 16 ||
                    group_max_degree == 32;
  const bool c_ok = cta_min_degree == 64 || cta_min_degree == 128 || cta_min_degree == 256 ||
                    cta_min_degree == 512 || cta_min_degree == 1000;
  if (!g_ok || !c_ok || !(grid_waves >= 0.125f && grid_waves <= 16.0f)) return PCC_INVALID_ARGUMENT;
  ctx->c.tuned = true;
  ctx->c.group_max_degree = group_max_degree;
  ctx->c.cta_min_degree = cta_min_degree;
  ctx->c.grid_waves = grid_waves;
  return PCC_OK;
}

uint64_t pcc_device_peak_bytes(pcc_context* ctx, int32_t reset) {
  if (!ctx) return 0;
  const uint64_t p = ctx->c.peak.load();
  if (reset) ctx->c.peak.store(ctx->c.in_use.load());
  return p;
}

pcc_status pcc_graph_upload(pcc_context* ctx, uint32_t n, uint64_t m, const uint64_t* offsets,
                            const uint32_t* neighbors, const float* weights, pcc_graph** out) {
  try {
    if (ctx) cudaSetDevice(ctx->c.device);
    return Done(ctx, Upload(ctx, n, m, offsets, neighbors, weights, false, out));
  } catch (const std::exception& e) {
    return Done(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_graph_upload_device(pcc_context* ctx, uint32_t n, uint64_t m, const uint64_t* d_offsets,
                                   const uint32_t* d_neighbors, const float* d_weights, pcc_graph** out) {
  try {
    if (ctx) cudaSetDevice(ctx->c.device);
    return Done(ctx, Upload(ctx, n, m, d_offsets, d_neighbors, d_weights, true, out));
  } catch (const std::exception& e) {
    return Done(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

void pcc_graph_free(pcc_context* ctx, pcc_graph* graph) {
  (void)ctx;
  delete graph;
}

pcc_status pcc_graph_info(const pcc_graph* graph, uint32_t* n, uint64_t* m, int32_t* has_weights) {
  if (!graph) return PCC_INVALID_ARGUMENT;
  if (n) *n = graph->g.n;
  if (m) *m = graph->g.m;
  if (has_weights) *has_weights = graph->g.w.p != nullptr;
  return PCC_OK;
}

pcc_status pcc_graph_download(pcc_context* pctx, const pcc_graph* graph, uint64_t* offsets, uint32_t* neighbors,
                              float* weights) {
  Status st;
  if (!pctx || !graph || !offsets || !neighbors) st = MakeError(PCC_INVALID_ARGUMENT, "null argument");
  if (st.ok()) st = graph->g.off.ToHost(offsets, uint64_t(graph->g.n) + 1);
  if (st.ok()) st = graph->g.nbr.ToHost(neighbors, graph->g.m);
  if (st.ok() && weights) {
    if (graph->g.w.p) {
      st = graph->g.w.ToHost(weights, graph->g.m);
    } else {
      for (uint64_t j = 0; j < graph->g.m; ++j) weights[j] = 1.0f;
    }
  }
  if (st.ok()) st = Sync(&pctx->c);
  return Done(pctx, st);
}

pcc_status pcc_graph_node_weights(pcc_context* pctx, const pcc_graph* graph, double* out) {
  Status st;
  if (!pctx || !graph || !out) st = MakeError(PCC_INVALID_ARGUMENT, "null argument");
  if (st.ok()) {
    if (graph->g.node_w.p) {
      st = graph->g.node_w.ToHost(out, graph->g.n);
    } else {
      for (uint32_t i = 0; i < graph->g.n; ++i) out[i] = 1.0;
    }
  }
  if (st.ok()) st = Sync(&pctx->c);
  return Done(pctx, st);
}

}  // extern "C"
