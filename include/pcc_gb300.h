/*
 * pcc_gb300.h -- C ABI of the GB300 (sm_103a) correlation / modularity
 * clustering library (libpcc_gb300.so).
 *
 * This is the drop-in boundary for the Louvain-style hot path of the
 * reference's ParallelCorrelationClusterer / ParallelModularityClusterer:
 * best-move rounds, graph compression and multilevel refinement.  Every
 * signature uses plain pointers and sizes; no C++ or torch types cross it.
 * The C++ InMemoryClusterer mirror (pcc_clusterer.h) and the Python
 * binding are the callers.
 *
 * Graph layout (host and device): symmetric CSR.
 *   offsets   uint64[n+1]   row i = entries [offsets[i], offsets[i+1])
 *   neighbors uint32[m]     neighbour vertex id of each entry
 *   weights   float[m]      edge weight of each entry, or NULL for unit weights
 * Each undirected edge appears in both rows, as in the reference's GBBS
 * symmetric_ptr_graph<symmetric_vertex, float> (clustering/gbbs-graph.h:39-56).
 *
 * Status codes are numerically identical to absl::StatusCode, the error
 * type of the reference (clustering/status_macros.h:26-60).
 */
#ifndef PCC_GB300_H_
#define PCC_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pcc_status {
  PCC_OK = 0,
  PCC_CANCELLED = 1,
  PCC_UNKNOWN = 2,
  PCC_INVALID_ARGUMENT = 3,
  PCC_DEADLINE_EXCEEDED = 4,
  PCC_NOT_FOUND = 5,
  PCC_ALREADY_EXISTS = 6,
  PCC_PERMISSION_DENIED = 7,
  PCC_RESOURCE_EXHAUSTED = 8,
  PCC_FAILED_PRECONDITION = 9,
  PCC_ABORTED = 10,
  PCC_OUT_OF_RANGE = 11,
  PCC_UNIMPLEMENTED = 12,
  PCC_INTERNAL = 13,
  PCC_UNAVAILABLE = 14,
  PCC_DATA_LOSS = 15
} pcc_status;

/* CorrelationClustererConfig.ClusteringMovesMethod (clustering/config.proto:122-130) */
enum { PCC_DEFAULT_CLUSTER_MOVES = 0, PCC_LOUVAIN = 1 };
/* CorrelationClustererConfig.SubclusteringMethod (config.proto:132-137) */
enum {
  PCC_NONE_SUBCLUSTERING = 0,
  PCC_TRIANGLE_SUBCLUSTERING = 1,
  PCC_CONNECTIVITY_SUBCLUSTERING = 2,
  PCC_SLOW_CONNECTIVITY_SUBCLUSTERING = 3
};
/* CorrelationClustererConfig.MoveMethod (config.proto:155-160) */
enum { PCC_NBHR_CLUSTER_MOVE = 0, PCC_ALL_MOVE = 1, PCC_NBHR_MOVE = 2 };

/*
 * Plain-C mirror of research_graph.in_memory.CorrelationClustererConfig
 * (clustering/config.proto:94-165) plus LouvainConfig (config.proto:176-183).
 * pcc_config_default() gives the proto defaults: every number 0, LOUVAIN,
 * NONE_SUBCLUSTERING, NBHR_CLUSTER_MOVE, all flags false.
 */
typedef struct pcc_config {
  double resolution;                   /* tag 1 */
  double edge_weight_offset;           /* tag 2 */
  int64_t num_iterations;              /* tag 4 (DEFAULT_CLUSTER_MOVES rounds) */
  int64_t louvain_num_iterations;      /* louvain_config.num_iterations */
  int64_t louvain_num_inner_iterations;/* louvain_config.num_inner_iterations */
  int32_t clustering_moves_method;     /* tag 9 */
  int32_t subclustering_method;        /* tag 10 */
  int32_t preclustering_method;        /* tag 11, parsed and ignored as in the reference */
  int32_t move_method;                 /* tag 16 */
  int32_t refine;                      /* tag 13 */
  int32_t async;                       /* tag 14 */
  int32_t permute;                     /* tag 18 */
  int32_t all_iter;                    /* tag 17, sequential clusterers only */
  uint64_t random_seed;                /* tag 3; also seeds permute / async order */
} pcc_config;

/* Per-call counters and phase times, filled by the clustering entry points. */
typedef struct pcc_stats {
  uint64_t edge_visits;      /* sum of deg(v) over every best-move evaluation */
  uint64_t vertex_visits;    /* number of best-move evaluations */
  uint64_t moves;            /* vertices that changed cluster */
  int32_t levels;            /* compression levels whose best moves ran */
  int32_t rounds;            /* best-move rounds, all levels and refinement */
  int32_t refine_passes;     /* refinement levels run */
  int32_t num_clusters;      /* clusters in the returned clustering */
  double objective;          /* ComputeObjective of the result on the input graph */
  double modularity;         /* modularity runs: ComputeModularity, else 0 */
  double ms_total;           /* device time of the whole call (CUDA events) */
  double ms_best_moves;      /* device time spent in best-move kernels */
  double ms_compress;        /* device time spent in graph compression */
  double ms_apply;           /* device time applying sync moves */
  double ms_frontier;        /* device time building next frontiers */
  uint64_t kernel_launches;  /* CUDA kernels this call launched */
  uint64_t algo_bytes_best_moves; /* algorithmic bytes of the best-move kernels:
                                     (8 or 12) per edge visit + 40 per vertex
                                     visit (8 when the graph has no weights) */
  /* Best-move kernel families: [0] lane groups (degree <= 32), [1] warps
     (degree <= 1000), [2] small hubs (<= 4096), [3] big hubs.  Device time
     (CUDA events around the family's launches), launches, and the entries
     and vertices evaluated (a big hub counts once however many partitions
     it is split into). */
  double family_ms[4];
  uint64_t family_launches[4];
  uint64_t family_entries[4];
  uint64_t family_vertices[4];
  /* Algorithmic bytes of graph compression: (12, or 8 without weights) per
     input entry + 8 per output entry + 20 per input vertex + 16 per output
     vertex, summed over the contractions. */
  uint64_t algo_bytes_compress;
  /* Algorithmic bytes of the frontier push with detailed timing on (0 off):
     4 per entry of every expanded row + 4 per expanded row. */
  uint64_t algo_bytes_frontier;
} pcc_stats;

void pcc_config_default(pcc_config* config);

/* ------------------------------------------------------------------------
 * Context: one GPU, one CUDA stream, one stream-ordered memory pool.
 * Replaces the reference's implicit global GBBS scheduler; one context per
 * host thread.  hbm_budget_bytes = 0 means "no budget" (device capacity).
 * ---------------------------------------------------------------------- */
typedef struct pcc_context pcc_context;
typedef struct pcc_graph pcc_graph;

pcc_status pcc_create(pcc_context** out, int device, uint64_t hbm_budget_bytes);
void pcc_destroy(pcc_context* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* pcc_last_error(const pcc_context* ctx);
/* Library version string. */
const char* pcc_version(void);
/* Bytes of device memory currently held by the context. */
uint64_t pcc_device_bytes_in_use(const pcc_context* ctx);
/* High-water mark of the context's device memory since creation or the last
 * reset (reset != 0 restarts it from the current use). */
uint64_t pcc_device_peak_bytes(pcc_context* ctx, int32_t reset);
/*
 * Detailed timing (no reference counterpart).  Off (the default):
 * synchronous best-move rounds run as a device-side loop, one round captured
 * into a CUDA graph WHILE node, with one host read per level; pcc_stats
 * then carries the compress time but no per-phase or per-family kernel
 * times.  On: the host drives every round and CUDA events time each phase
 * and best-move kernel family.  Results are identical either way.
 */
void pcc_set_detailed_timing(pcc_context* ctx, int32_t on);

/*
 * Best-move launch shape (no reference counterpart).  Lane-group bins (degree
 * <= 4, 8, 16, 32) above group_max_degree (4, 8, 16 or 32) run on the warp
 * kernel; certified (INT-mode, synchronous) warp bins (degree <= 128, 256,
 * 512, 1000) above cta_min_degree (64, 128, 256, 512, or 1000 for none) run
 * one CTA per vertex; the grid-stride best-move kernels launch grid_waves
 * (0.125-16) times one wave of resident CTAs.  (0, 0, 0) returns to the
 * compiled-in table, chosen per level-graph size class by tune_launch.py.
 * Results are identical under every setting; only the time changes.
 */
pcc_status pcc_set_launch_tuning(pcc_context* ctx, uint32_t group_max_degree, uint32_t cta_min_degree,
                                 float grid_waves);

/*
 * Graph upload.  Copies a host CSR graph into HBM.  Replaces
 * GbbsGraph::Import/FinishImport (clustering/gbbs-graph.cc:32-76) and the
 * CLI's CopyGraph injection (clustering/cluster-in-memory_main.cc:231-306).
 * weights == NULL stores a unit-weight graph with no weight array.
 * n must be at most 2^32 - 32 (INVALID_ARGUMENT otherwise).
 */
pcc_status pcc_graph_upload(pcc_context* ctx, uint32_t n, uint64_t m,
                            const uint64_t* offsets, const uint32_t* neighbors,
                            const float* weights, pcc_graph** out);
/* Same, from device pointers (device-to-device copy on the context stream). */
pcc_status pcc_graph_upload_device(pcc_context* ctx, uint32_t n, uint64_t m,
                                   const uint64_t* d_offsets,
                                   const uint32_t* d_neighbors,
                                   const float* d_weights, pcc_graph** out);
void pcc_graph_free(pcc_context* ctx, pcc_graph* graph);
pcc_status pcc_graph_info(const pcc_graph* graph, uint32_t* n, uint64_t* m,
                          int32_t* has_weights);
/* Copies the graph back to host buffers (weights may be NULL to skip). */
pcc_status pcc_graph_download(pcc_context* ctx, const pcc_graph* graph,
                              uint64_t* offsets, uint32_t* neighbors,
                              float* weights);

/*
 * GBBS adjacency text parsed on the device into a resident graph, in place
 * of gbbs_io::read_unweighted_symmetric_graph /
 * read_weighted_symmetric_graph<float> + CopyGraph
 * (clustering/cluster-in-memory_main.cc:285-306).  The text is
 * "AdjacencyGraph" or "WeightedAdjacencyGraph", n, m, n offsets, m neighbour
 * ids and, when weighted, m weights, separated by whitespace; float_weighted
 * must match the header.  Results and errors equal the host reader's
 * (pcch_read_gbbs): offsets and ids are decimal digits; weights round as
 * strtof (nearest float, ties to even); all-one weights give a unit-weight
 * graph; tokens after the last one needed are ignored.  Hexadecimal floats,
 * nan(...) payloads and weights of more than 200 significant digits are
 * INVALID_ARGUMENT here.  Bad or missing tokens are INVALID_ARGUMENT (the
 * first in file order is named), n > 2^32 - 1 is OUT_OF_RANGE.
 *   text / size   the file's bytes in host memory
 */
pcc_status pcc_graph_parse_gbbs(pcc_context* ctx, const char* text, uint64_t size,
                                int32_t float_weighted, pcc_graph** out);
/* Reads the file at `path` into pinned host memory, then parses it on the
 * device as pcc_graph_parse_gbbs.  NOT_FOUND if it cannot be opened. */
pcc_status pcc_graph_read_gbbs(pcc_context* ctx, const char* path,
                               int32_t float_weighted, pcc_graph** out);

/*
 * WriteClustering (clustering/cluster-in-memory_main.cc:132-145) formatted
 * on the device.  labels[n] (host) gives each node's cluster index; cluster
 * i is the set of nodes labelled i, for i up to the largest label.  The text
 * has one line per cluster in index order, each member id (ascending)
 * followed by a tab, then a newline (an empty line for an empty cluster).
 * pcc_format_clustering stores the length in *length and, when out is not
 * NULL, the text in out[0..length) (RESOURCE_EXHAUSTED if capacity is
 * smaller; call with out = NULL to size the buffer).  pcc_write_clustering
 * writes the text to the file at `path` (NOT_FOUND if it cannot be opened).
 */
pcc_status pcc_format_clustering(pcc_context* ctx, uint32_t n,
                                 const uint32_t* labels, char* out,
                                 uint64_t capacity, uint64_t* length);
pcc_status pcc_write_clustering(pcc_context* ctx, const char* path, uint32_t n,
                                const uint32_t* labels);

/*
 * ParallelCorrelationClusterer::RefineClusters / Cluster
 * (clustering/clusterers/parallel-correlation-clusterer.cc:392-653).
 *   node_weights    host double[n] or NULL (all 1, parallel-correlation-
 *                   clusterer-internal.h:47)
 *   initial_labels  host uint32[n] or NULL.  NULL = all singletons (Cluster).
 *                   Otherwise vertex i starts in cluster initial_labels[i]
 *                   (< n), like RefineClusters(config, &clustering) with
 *                   clustering[c] = { i : initial_labels[i] == c }.
 *   out_labels      host uint32[n]: index of the vertex's cluster in the
 *                   returned InMemoryClusterer::Clustering (clusters ordered
 *                   by internal id, members ascending -- OutputIndicesById,
 *                   parallel/parallel-sequence-ops.h:183-209).
 */
pcc_status pcc_correlation_cluster(pcc_context* ctx, const pcc_graph* graph,
                                   const pcc_config* config,
                                   const double* node_weights,
                                   const uint32_t* initial_labels,
                                   uint32_t* out_labels, pcc_stats* stats);

/*
 * ParallelModularityClusterer::RefineClusters / Cluster
 * (clustering/clusterers/parallel-modularity-clusterer.cc:68-111):
 * node weight = degree, resolution' = resolution / sum(degree), offset 0,
 * then the correlation path; stats->modularity = ComputeModularity with the
 * original resolution (parallel-modularity-clusterer.cc:36-66).
 */
pcc_status pcc_modularity_cluster(pcc_context* ctx, const pcc_graph* graph,
                                  const pcc_config* config,
                                  const uint32_t* initial_labels,
                                  uint32_t* out_labels, pcc_stats* stats);

/*
 * End-to-end convenience call on host CSR buffers: upload, cluster (objective
 * 0 = correlation, 1 = modularity), download labels, free.  The call a user
 * without a persistent graph handle makes.
 */
pcc_status pcc_cluster_host_csr(pcc_context* ctx, uint32_t n, uint64_t m,
                                const uint64_t* offsets,
                                const uint32_t* neighbors, const float* weights,
                                const pcc_config* config, int32_t objective,
                                const double* node_weights,
                                uint32_t* out_labels, pcc_stats* stats);

/*
 * ClusteringHelper::ComputeObjective on host labels
 * (parallel-correlation-clusterer-internal.cc:118-149).  Labels < n.
 */
pcc_status pcc_objective(pcc_context* ctx, const pcc_graph* graph,
                         const pcc_config* config, const double* node_weights,
                         const uint32_t* labels, double* out_objective);

/* ComputeModularity (parallel-modularity-clusterer.cc:36-66). */
pcc_status pcc_modularity(pcc_context* ctx, const pcc_graph* graph,
                          double resolution, const uint32_t* labels,
                          double* out_modularity);

/*
 * Ground-truth scoring on the device: CompareCommunities
 * (clustering/cluster-in-memory_main.cc:172-225), the CLI's
 * --input_communities step.  Replaces the host loops the reference runs
 * after Cluster() returns.
 *
 * labels[n] (< n) is a clustering: cluster i is the i-th distinct label in
 * ascending order, as OutputIndicesById lists the clustering.  Community j
 * is members[offsets[j] .. offsets[j+1]) (order and repeats as read from
 * the file, see ReadCommunities :155-170; an id >= n meets no cluster but
 * counts in the community's size).  For each
 * community: the cluster with the largest intersection (the first such
 * cluster on ties; cluster 0 when every intersection is empty), precision
 * = intersection / that cluster's size, recall = intersection / community
 * size (0 for an empty community).  Averages use pbbs::reduce_add order.
 * precision / recall (num_communities each) may be NULL.
 */
typedef struct pcc_community_scores {
  double avg_precision;
  double avg_recall;
  uint64_t num_clusters;  /* "Num communities" of the reference's report */
  uint64_t min_size;      /* UINT32_MAX (UINT_E_MAX) when there is no cluster */
  uint64_t max_size;
  double avg_size;
} pcc_community_scores;

pcc_status pcc_compare_communities(pcc_context* ctx, uint32_t n,
                                   const uint32_t* labels,
                                   uint32_t num_communities,
                                   const uint64_t* offsets,
                                   const uint32_t* members,
                                   double* precision, double* recall,
                                   pcc_community_scores* out);

/*
 * One synchronous best-move pass over ALL vertices from a given state:
 * ClusteringHelper::EfficientBestMove plus the sync decision of
 * BestMovesForVertexSubset (parallel-correlation-clusterer-internal.cc:
 * 448-583, parallel-correlation-clusterer.cc:139-157).  Host arrays of n.
 *   out_targets[v]  cluster id (n = new cluster) chosen by EfficientBestMove
 *   out_values[v]   its objective change (before the singleton rule)
 *   out_moves[v]    decided move after the singleton rule and value > 0,
 *                   or 0xFFFFFFFF for "no move"; may be NULL.
 */
pcc_status pcc_best_moves(pcc_context* ctx, const pcc_graph* graph,
                          const pcc_config* config,
                          const uint32_t* cluster_ids,
                          const uint32_t* cluster_sizes,
                          const double* node_weights,
                          const double* cluster_weights, uint32_t* out_targets,
                          double* out_values, uint32_t* out_moves);

/*
 * CompressGraph (parallel-correlation-clusterer-internal.cc:709-782 with
 * ComputeInterClusterEdgesSort, parallel/parallel-graph-utils.cc:156-231):
 * contracts `graph` by cluster_ids (host uint32[n]) into a new graph over
 * 1 + max(cluster_ids) vertices.  node_weights host double[n] or NULL (1).
 * The new graph's node weights are downloaded with pcc_graph_node_weights.
 */
pcc_status pcc_compress(pcc_context* ctx, const pcc_graph* graph,
                        const uint32_t* cluster_ids, const double* node_weights,
                        pcc_graph** out);
/* Node weights attached to a compressed graph (host double[n]). */
pcc_status pcc_graph_node_weights(pcc_context* ctx, const pcc_graph* graph,
                                  double* out);

/* ------------------------------------------------------------------------
 * Batched clustering and the serving loop (no reference counterpart; the
 * reference clusters one graph per process).  Many independent graphs run
 * concurrently on one GPU: `concurrency` worker threads each own a context
 * (its own CUDA stream and memory pool share), so the kernels of different
 * graphs overlap on the device.  Every result is identical to a call of
 * pcc_cluster_host_csr on that graph alone.
 * ---------------------------------------------------------------------- */
typedef struct pcc_batch_graph {
  uint32_t n;
  uint64_t m;
  const uint64_t* offsets;      /* host CSR, as pcc_graph_upload */
  const uint32_t* neighbors;
  const float* weights;         /* NULL = unit weights */
  const double* node_weights;   /* correlation only; NULL = all 1 */
} pcc_batch_graph;

/*
 * Clusters graphs[0..num_graphs).  configs: one config for all graphs
 * (num_configs == 1) or one per graph; objectives: NULL (all correlation) or
 * one per graph (0 correlation, 1 modularity).  out_labels[i]: host
 * uint32[n_i].  stats: NULL or one per graph.  hbm_budget: 0 = none, else
 * the limit on the device memory all workers hold together.  *wall_ms (may
 * be NULL) receives the batch's wall time.  The first failing graph's
 * status is returned; the others stop taking new work.
 *
 * When the configs differ in resolution only (num_configs == 1 included), are
 * LOUVAIN, synchronous and without subclustering, and the offset is 0 or every
 * objective is correlation, the batch runs as disjoint unions
 * (pcc_cluster_union on one context; stats as documented there), with the
 * graphs packed in ascending order of entry count (stable; results and stats
 * are returned in the caller's order).  Otherwise each graph runs on the
 * worker pool and its stats equal a standalone call's.
 */
pcc_status pcc_cluster_batch(int device, uint32_t num_graphs, const pcc_batch_graph* graphs,
                             const pcc_config* configs, uint32_t num_configs,
                             const int32_t* objectives, uint32_t concurrency,
                             uint64_t hbm_budget, uint32_t* const* out_labels,
                             pcc_stats* stats, double* wall_ms);

/*
 * Batched clustering as a disjoint-union graph: the graphs run as one engine
 * run, and each kernel launch of a round covers all of them.  Each graph keeps
 * the control flow of RefineClusters_subroutine
 * (clustering/clusterers/parallel-correlation-clusterer.cc:476-629) for itself:
 *   - its own level count;
 *   - its own inner-loop exit;
 *   - its own refinement levels;
 *   - new-cluster ids from its own empty ids;
 *   - its own resolution.
 * So its labels and objective equal those of a standalone call (bit for bit
 * with integer weights and node weights, else within FP64 summation order for
 * the objective; modularity within 1e-12 relative).  The rounds of a level
 * run as one device-side loop (a CUDA graph WHILE node) that keeps each
 * graph's rounds, edge visits and in-loop flag on the device, with one host
 * read per level; with detailed timing on, the host drives them.
 * configs: one for all graphs or one per graph, equal in every field but the
 * resolution; LOUVAIN, synchronous, NONE_SUBCLUSTERING.  objectives: NULL
 * (correlation) or one per graph (0 correlation, 1 modularity: node weights
 * = degrees, resolution / sum of degrees, which needs edge_weight_offset 0).
 * Graphs are packed in order into unions of at most max_union_entries
 * adjacency entries (0: 2^31) and 2^31 vertices.  out_labels[i]: host
 * uint32[n_i] (may be NULL when n_i == 0).  stats (NULL or one per graph)
 * carries objective, modularity, num_clusters, levels, rounds,
 * refine_passes and edge_visits of each graph (the other fields are 0).
 * batch_stats (may be NULL) receives the totals, phase times and kernel
 * launches of the whole call.
 */
pcc_status pcc_cluster_union(pcc_context* ctx, uint32_t num_graphs, const pcc_batch_graph* graphs,
                             const pcc_config* configs, uint32_t num_configs,
                             const int32_t* objectives, uint64_t max_union_entries,
                             uint32_t* const* out_labels, pcc_stats* stats,
                             pcc_stats* batch_stats);

/*
 * Serving loop with continuous batching: requests are queued by
 * pcc_server_submit and admitted, first come first served, as soon as a
 * worker slot is free and the request's device-memory estimate fits the HBM
 * budget next to the requests already running; admitted requests run
 * concurrently.  A worker that admits a request with a synchronous LOUVAIN
 * config without subclustering also admits the queued requests whose config
 * differs in resolution only (and objective, with offset 0), up to 64 graphs
 * and 8M entries, and runs them as one disjoint-union engine run
 * (pcc_cluster_union).  The stats of such requests
 * are the per-graph stats pcc_cluster_union documents.  Each label set and
 * objective is identical to a standalone pcc_cluster_host_csr call.
 */
typedef struct pcc_server pcc_server;

pcc_status pcc_server_create(pcc_server** out, int device, uint32_t slots,
                             uint64_t hbm_budget);
/* Copies the graph; returns a ticket.  RESOURCE_EXHAUSTED when the request
 * alone exceeds the budget. */
pcc_status pcc_server_submit(pcc_server* server, uint32_t n, uint64_t m,
                             const uint64_t* offsets, const uint32_t* neighbors,
                             const float* weights, const double* node_weights,
                             const pcc_config* config, int32_t objective,
                             uint64_t* ticket);
/*
 * Waits up to wait_ms (< 0: no limit) for a request.  When it has finished,
 * copies its labels (host uint32[n]) and stats (may be NULL), sets
 * *latency_ms (submit to completion) and *queue_ms (submit to admission),
 * releases the ticket and returns the request's status.  Returns
 * DEADLINE_EXCEEDED (ticket kept) while it is still queued or running, and
 * NOT_FOUND for an unknown ticket.
 */
pcc_status pcc_server_wait(pcc_server* server, uint64_t ticket, int32_t wait_ms,
                           uint32_t* out_labels, pcc_stats* stats,
                           double* latency_ms, double* queue_ms);
/* Device-memory estimate the admission control uses for a request. */
uint64_t pcc_request_bytes_estimate(uint32_t n, uint64_t m, int32_t has_weights);
/* Finishes the running requests, fails the queued ones (CANCELLED) and
 * frees the server. */
void pcc_server_destroy(pcc_server* server);

/*
 * No reference counterpart.  EfficientBestMove (target and value, before the
 * sync decision; the out_targets / out_values of pcc_best_moves) for a list
 * of vertices, on caller-owned DEVICE arrays, allocating no device memory.
 * For callers that hold all device memory in their own allocator (a serving
 * loop with a fixed HBM budget, a framework's caching allocator) and cannot
 * let a library call cudaMalloc on the request path.
 *
 * Scratch is one file-scope device array of 24 MiB (2^21 hash slots); each
 * listed vertex needs nextpow2(2 * degree + 2) slots, so degrees up to
 * 1,048,575.  max_degree (>= every listed vertex's degree) above that limit
 * returns OUT_OF_RANGE before launching; a listed vertex whose degree
 * exceeds max_degree gets target 0xFFFFFFFF and the call returns
 * OUT_OF_RANGE.  Vertex or cluster ids >= n return INVALID_ARGUMENT.
 *
 *   d_offsets / d_neighbors / d_weights   device CSR (d_weights NULL = 1)
 *   d_cluster_ids (uint32[n]), d_node_weights (double[n]),
 *   d_cluster_weights (double[n], per cluster id)
 *   d_vertices    device uint32[num_vertices], or NULL for all n vertices
 *   d_out_targets / d_out_values   device arrays of num_vertices
 *   stream        cudaStream_t (NULL = default stream) of the current device
 *
 * Runs on the current device.  The first call on a device resolves the
 * scratch address (cudaGetSymbolAddress); make that first call before any
 * stream capture begins.  Every call synchronises `stream` and copies a
 * status word to the host before it returns.  Calls that overlap in time on
 * one device share the scratch and race: serialise them.  Sums use FP64
 * atomics: equal to pcc_best_moves on integer weights, within rounding on
 * real weights.
 */
pcc_status pcc_best_moves_static(
    uint32_t n, const uint64_t* d_offsets, const uint32_t* d_neighbors,
    const float* d_weights, const uint32_t* d_cluster_ids,
    const double* d_node_weights, const double* d_cluster_weights,
    double resolution, double edge_weight_offset, const uint32_t* d_vertices,
    uint32_t num_vertices, uint32_t max_degree, uint32_t* d_out_targets,
    double* d_out_values, void* stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* PCC_GB300_H_ */
