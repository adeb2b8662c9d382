// subcluster.cu -- subclustering before compression (CompressSubclusters,
// clustering/clusterers/parallel-correlation-clusterer.cc:436-474, with
// ComputeSubcluster and its three methods, parallel-correlation-clusterer-
// internal.cc:784-1120).
//
// Every cluster is split into subclusters; cluster i (clusters in id order)
// owns the subcluster ids [next_i, next_i + B_i), B_i its block size, and
// the level's graph is then compressed by subcluster id.  Inside a cluster
// a member's local index is its rank among the cluster's members (ids
// ascending).
//   * CONNECTIVITY: components of the member pairs joined by an entry,
//     labelled by the smallest member's local index; B = the cluster size.
//   * TRIANGLE: components over the entries (v, u), C(u) = C(v), whose
//     ratio |N(v) & N(u)| / (deg v + deg u) (a sorted-merge count of the
//     two rows, GBBS's intersect) exceeds 0.25; B = 1 + the largest label.
//   * SLOW_CONNECTIVITY: the reference's sequential merge loop, one thread
//     per cluster; B = 1 + the largest label.
// Components come from a lock-free union-find over the vertex ids that
// always links the larger root under the smaller one (the rule of GBBS's
// asynchronous union-find), so a component's root is its smallest vertex,
// i.e. its smallest local index.  (The reference labels triangle components
// with GBBS's work-efficient CC, whose labels are LDD centres; the
// components are the same.)
#include "graphops.cuh"

namespace pcc {

namespace {

__global__ void ScPresentKernel(uint32_t n, const uint32_t* __restrict__ C, uint32_t* __restrict__ pres) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    pres[C[i]] = 1u;
}
struct ScPresInput {
  const uint32_t* pres;
  __device__ uint32_t operator()(uint64_t i) const { return pres[i]; }
};
struct ScRankWriter {
  uint32_t* rank;
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t) const { rank[i] = pre; }
};

// (cluster index, vertex) pairs for the stable member sort, and the
// union-find roots.
__global__ void ScInitKernel(uint32_t n, const uint32_t* __restrict__ C, const uint32_t* __restrict__ rank,
                             uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t* __restrict__ parent,
                             uint32_t* __restrict__ csize) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t gi = rank[C[v]];
    keys[v] = gi;
    vals[v] = static_cast<uint32_t>(v);
    parent[v] = static_cast<uint32_t>(v);
    atomicAdd(&csize[gi], 1u);
  }
}

struct ScHeadInput {
  const uint64_t* keys;
  __device__ uint32_t operator()(uint64_t i) const { return i == 0 || keys[i] != keys[i - 1]; }
};
// first[gi] = the sorted position of cluster gi's smallest member; local[v].
struct ScFirstWriter {
  const uint64_t* keys;
  uint32_t* first;
  __device__ void operator()(uint64_t i, uint32_t, uint32_t v) const {
    if (v) first[keys[i]] = static_cast<uint32_t>(i);
  }
};
__global__ void ScLocalKernel(uint32_t n, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ member,
                              const uint32_t* __restrict__ first, uint32_t* __restrict__ local) {
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += uint64_t(gridDim.x) * blockDim.x)
    local[member[k]] = static_cast<uint32_t>(k - first[keys[k]]);
}

__device__ __forceinline__ uint32_t UfFind(uint32_t* parent, uint32_t x) {
  uint32_t p = __ldcg(&parent[x]);
  while (p != x) {
    const uint32_t gp = __ldcg(&parent[p]);
    if (gp != p) atomicCAS(&parent[x], p, gp);  // path halving
    x = p;
    p = __ldcg(&parent[x]);
  }
  return x;
}

// Links the two components (the larger root under the smaller).  Each
// failed CAS means another thread changed a root, so the loop ends.
__device__ __forceinline__ void UfUnite(uint32_t* parent, uint32_t a, uint32_t b) {
  while (true) {
    a = UfFind(parent, a);
    b = UfFind(parent, b);
    if (a == b) return;
    if (a < b) {
      const uint32_t t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(&parent[a], a, b) == a) return;
  }
}

// |N(v) & N(u)| by the sorted-merge walk of the two rows.
__device__ uint64_t MergeCount(const uint64_t* off, const uint32_t* nbr, uint32_t v, uint32_t u) {
  uint64_t a = off[v], ae = off[v + 1], b = off[u], be = off[u + 1];
  uint64_t common = 0;
  while (a < ae && b < be) {
    const uint32_t x = nbr[a], y = nbr[b];
    if (x == y) {
      ++common;
      ++a;
      ++b;
    } else if (x < y) {
      ++a;
    } else {
      ++b;
    }
  }
  return common;
}

struct ScUnion {
  const uint64_t* off;
  const uint32_t* nbr;
  const uint32_t* C;
  uint32_t* parent;
  bool triangle;
  __device__ void operator()(uint32_t v, uint64_t j, uint64_t) const {
    const uint32_t u = nbr[j];
    if (C[u] != C[v]) return;
    if (triangle) {
      const double ratio = static_cast<double>(MergeCount(off, nbr, v, u)) /
                           static_cast<double>((off[v + 1] - off[v]) + (off[u + 1] - off[u]));
      if (!(ratio > 0.25)) return;
    }
    UfUnite(parent, v, u);
  }
};

// Label = the root's local index; the block of a cluster is its size
// (connectivity) or 1 + its largest label (triangle).
__global__ void ScLabelKernel(uint32_t n, const uint32_t* __restrict__ C, const uint32_t* __restrict__ rank,
                              uint32_t* parent, const uint32_t* __restrict__ local, uint32_t* __restrict__ label,
                              uint32_t* __restrict__ block, bool by_size, const uint32_t* __restrict__ csize) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t lab = local[UfFind(parent, static_cast<uint32_t>(v))];
    label[v] = lab;
    const uint32_t gi = rank[C[v]];
    if (by_size) {
      block[gi] = csize[gi];
    } else {
      atomicMax(&block[gi], lab + 1);
    }
  }
}

// ComputeSubclusterConnectivitySlow (internal.cc:870-985) for one cluster
// per thread.  Scratch indexed by sorted member position: tmp (labels) and
// single; mark[v] = 2 while v is in the subcluster being measured.
struct SlowArgs {
  uint32_t G;
  const uint64_t* off;
  const uint32_t* nbr;
  const uint32_t* C;
  const uint32_t* member;  // vertices sorted by (cluster index, id)
  const uint32_t* first;   // per cluster index: first sorted position
  const uint32_t* csize;
  uint32_t* tmp;
  uint8_t* single;
  uint8_t* mark;
  uint32_t* label;         // per vertex
  uint32_t* block;         // per cluster index
  double res;
  double offset;
};

__device__ uint32_t OutsideEdges(const SlowArgs& a, uint32_t v, uint32_t c) {
  uint32_t e = 0;
  for (uint64_t j = a.off[v]; j < a.off[v + 1]; ++j) e += a.C[a.nbr[j]] != c ? 1u : 0u;
  return e;
}

__global__ void ScSlowKernel(SlowArgs a) {
  for (uint64_t gi = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; gi < a.G; gi += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t base = a.first[gi];
    const uint32_t size = a.csize[gi];
    const uint32_t* mem = a.member + base;
    uint32_t* tmp = a.tmp + base;
    uint8_t* single = a.single + base;
    const uint32_t c = a.C[mem[0]];
    for (uint32_t i = 0; i < size; ++i) {
      tmp[i] = i;
      single[i] = 0;
    }
    for (uint32_t i = 0; i < size; ++i) {
      if (single[i] != 0) continue;
      const uint32_t cv = mem[i];
      if (OutsideEdges(a, cv, c) < size - 1) continue;
      // Groups of local indices by label (ascending label, members
      // ascending): walked label by label.  First pass: validity.
      int64_t num_valid = 0;
      double max_max = 0;
      uint32_t best_label = kNone;
      for (uint32_t t = 0; t < size; ++t) {
        uint32_t gsize = 0, g0 = kNone;
        for (uint32_t x = 0; x < size; ++x)
          if (tmp[x] == t) {
            if (g0 == kNone) g0 = x;
            ++gsize;
          }
        if (gsize == 0 || g0 == i) continue;
        uint64_t num_edges = 0;
        for (uint32_t x = 0; x < size; ++x)
          if (tmp[x] == t) num_edges += OutsideEdges(a, mem[x], c);
        if (num_edges < uint64_t(gsize) * (size - gsize)) continue;
        // Second pass (same group order): the objective requirement.
        for (uint32_t x = 0; x < size; ++x)
          if (tmp[x] == t) a.mark[mem[x]] = 2;
        double weight = 0;
        // Marks are shared by all clusters' threads: a neighbour counts only
        // if it is in this cluster, whose marks this thread alone writes.
        for (uint64_t j = a.off[cv]; j < a.off[cv + 1]; ++j) {
          const uint32_t u = a.nbr[j];
          if (a.C[u] == c && a.mark[u] == 2) weight += 1.0;
        }
        for (uint32_t x = 0; x < size; ++x)
          if (tmp[x] == t) a.mark[mem[x]] = 0;
        const double offset = a.offset * double(gsize) + a.res * double(gsize);
        if (weight < offset) continue;
        ++num_valid;
        if (weight - offset >= max_max) {
          max_max = weight - offset;
          best_label = t;
        }
      }
      if (num_valid == 0) continue;
      uint32_t g0 = 0;
      for (uint32_t x = 0; x < size; ++x)
        if (tmp[x] == best_label) {
          g0 = x;
          break;
        }
      tmp[i] = tmp[g0];
      single[i] = 1;
      single[g0] = 1;
    }
    uint32_t mx = 0;
    for (uint32_t i = 0; i < size; ++i) {
      a.label[mem[i]] = tmp[i];
      mx = max(mx, tmp[i]);
    }
    a.block[gi] = mx + 1;
  }
}

struct BlockInput {
  const uint32_t* block;
  __device__ uint64_t operator()(uint64_t i) const { return block[i]; }
};

__global__ void ScIdsKernel(uint32_t n, const uint32_t* __restrict__ C, const uint32_t* __restrict__ rank,
                            const uint64_t* __restrict__ next, const uint32_t* __restrict__ label,
                            uint32_t* __restrict__ sub) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x)
    sub[v] = static_cast<uint32_t>(next[rank[C[v]]] + label[v]);
}

}  // namespace

Status ComputeSubclustersDevice(Context* ctx, const DevGraph& g, const uint32_t* C, int method, double res,
                                double offset, DBuf<uint32_t>* sub, DBuf<uint64_t>* next, uint32_t* num_clusters,
                                uint64_t* total) {
  const uint32_t n = g.n;
  *num_clusters = 0;
  *total = 0;
  if (n == 0) return Status::Ok();
  cudaStream_t st = ctx->stream;
  const unsigned grid = Blocks(n, 256, unsigned(ctx->num_sms) * 8);
  DBuf<uint32_t> pres, rank, tmp32, scan32;
  PCC_RETURN_IF_ERROR(pres.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(rank.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(tmp32.Alloc(ctx, 2));
  PCC_RETURN_IF_ERROR(pres.Zero());
  ScPresentKernel<<<grid, 256, 0, st>>>(n, C, pres.p); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, n, ScPresInput{pres.p}, ScRankWriter{rank.p}, scan32, tmp32.p));
  uint32_t G = 0;
  PCC_RETURN_IF_ERROR(tmp32.ToHost(&G, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));

  DBuf<uint64_t> keys;
  DBuf<uint32_t> member, parent, csize, first, local, label, block;
  PCC_RETURN_IF_ERROR(keys.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(member.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(parent.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(csize.Alloc(ctx, G));
  PCC_RETURN_IF_ERROR(first.Alloc(ctx, G));
  PCC_RETURN_IF_ERROR(local.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(label.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(block.Alloc(ctx, G));
  PCC_RETURN_IF_ERROR(csize.Zero());
  PCC_RETURN_IF_ERROR(block.Zero());
  ScInitKernel<<<grid, 256, 0, st>>>(n, C, rank.p, keys.p, member.p, parent.p, csize.p); PCC_COUNT(1);
  int bits = 1;
  while ((uint64_t(1) << bits) < G) ++bits;
  {
    SortScratch sc;  // stable: members ascending inside each cluster
    PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys.p, member.p, n, bits, sc));
  }
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, n, ScHeadInput{keys.p}, ScFirstWriter{keys.p, first.p}, scan32,
                                          tmp32.p));
  ScLocalKernel<<<grid, 256, 0, st>>>(n, keys.p, member.p, first.p, local.p); PCC_COUNT(1);

  if (method == PCC_SLOW_CONNECTIVITY_SUBCLUSTERING) {
    DBuf<uint32_t> tmp;
    DBuf<uint8_t> single, mark;
    PCC_RETURN_IF_ERROR(tmp.Alloc(ctx, n));
    PCC_RETURN_IF_ERROR(single.Alloc(ctx, n));
    PCC_RETURN_IF_ERROR(mark.Alloc(ctx, n));
    PCC_RETURN_IF_ERROR(mark.Zero());
    SlowArgs a{G, g.off.p, g.nbr.p, C, member.p, first.p, csize.p, tmp.p, single.p, mark.p, label.p, block.p,
               res, offset};
    ScSlowKernel<<<Blocks(G, 64, unsigned(ctx->num_sms) * 16), 64, 0, st>>>(a); PCC_COUNT(1);
    PCC_RETURN_IF_ERROR(LaunchCheck());
    PCC_RETURN_IF_ERROR(Sync(ctx));  // scratch freed on return
  } else {
    if (g.m)
      LaunchEdgeIter(ctx, g.bins.list.p, g.bins.counts.p, g.bins.counts.p + kNumBins, g.bins.host_counts, g.off.p,
                     ScUnion{g.off.p, g.nbr.p, C, parent.p, method == PCC_TRIANGLE_SUBCLUSTERING});
    ScLabelKernel<<<grid, 256, 0, st>>>(n, C, rank.p, parent.p, local.p, label.p, block.p,
                                        method == PCC_CONNECTIVITY_SUBCLUSTERING, csize.p); PCC_COUNT(1);
  }
  PCC_RETURN_IF_ERROR(next->Alloc(ctx, uint64_t(G) + 1));
  DBuf<uint64_t> scan64;
  PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, G, BlockInput{block.p}, StorePrefix<uint64_t>{next->p}, scan64,
                                          next->p + G));
  PCC_RETURN_IF_ERROR(sub->Alloc(ctx, n));
  ScIdsKernel<<<grid, 256, 0, st>>>(n, C, rank.p, next->p, label.p, sub->p); PCC_COUNT(1);
  PCC_RETURN_IF_ERROR(LaunchCheck());
  uint64_t tot = 0;
  PCC_CUDA(cudaMemcpyAsync(&tot, next->p + G, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  *num_clusters = G;
  *total = tot;
  return Status::Ok();
}

}  // namespace pcc
