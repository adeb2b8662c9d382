// pcc_clusterer.h -- C++ host mirror of the reference's clusterer interface
// on top of the C ABI of libpcc_gb300.so (pcc_gb300.h).
//
// Mirrors, with the same names, argument meaning and error behaviour:
//   InMemoryClusterer, Graph::Import / FinishImport, Clustering
//       (clustering/in-memory-clusterer.h:34-121)
//   GbbsGraph import semantics (clustering/gbbs-graph.cc:28-76)
//   ClustererConfig / CorrelationClustererConfig / LouvainConfig / KcoreConfig
//       and their text format (clustering/config.proto:94-197)
//   ParallelCorrelationClusterer::Cluster / RefineClusters
//       (clustering/clusterers/parallel-correlation-clusterer.cc:392-653)
//   ParallelModularityClusterer::Cluster / RefineClusters
//       (clustering/clusterers/parallel-modularity-clusterer.cc:68-111)
//   the CLI helpers: GBBS adjacency reading, WriteClustering,
//       ReadCommunities / CompareCommunities, name dispatch
//       (clustering/cluster-in-memory_main.cc:131-306)
// absl::Status / StatusOr are replaced by the small Status / StatusOr below
// (same numeric codes).  The implementation lives in libpcc_host.so.
#ifndef PCC_CLUSTERER_H_
#define PCC_CLUSTERER_H_

#include <stddef.h>
#include <stdint.h>

#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "pcc_gb300.h"

namespace pcc_gb300 {

class Status {
 public:
  Status() = default;
  Status(pcc_status code, std::string message) : code_(code), message_(std::move(message)) {}
  static Status Ok() { return Status(); }
  bool ok() const { return code_ == PCC_OK; }
  pcc_status code() const { return code_; }
  const std::string& message() const { return message_; }
  std::string ToString() const;

 private:
  pcc_status code_ = PCC_OK;
  std::string message_;
};

template <class T>
class StatusOr {
 public:
  StatusOr(Status s) : status_(std::move(s)) {}  // NOLINT: implicit like absl
  StatusOr(T value) : value_(std::move(value)) {}  // NOLINT
  bool ok() const { return status_.ok(); }
  const Status& status() const { return status_; }
  T& value() { return value_; }
  const T& value() const { return value_; }
  T& operator*() { return value_; }
  const T& operator*() const { return value_; }

 private:
  Status status_;
  T value_{};
};

// ---------------------------------------------------------------------------
// Configuration (config.proto).  Fields keep the proto's names and defaults.
// ---------------------------------------------------------------------------
struct LouvainConfig {
  int64_t num_iterations = 0;
  int64_t num_inner_iterations = 0;
};

struct KcoreConfig {
  int32_t kcore_cutoff = 0;
  bool fix_preclusters = false;
  bool connect_only = false;
  double percent_cutoff = 0;
};

struct CorrelationClustererConfig {
  enum ClusteringMovesMethod { DEFAULT_CLUSTER_MOVES = 0, LOUVAIN = 1 };
  enum SubclusteringMethod {
    NONE_SUBCLUSTERING = 0,
    TRIANGLE_SUBCLUSTERING = 1,
    CONNECTIVITY_SUBCLUSTERING = 2,
    SLOW_CONNECTIVITY_SUBCLUSTERING = 3
  };
  enum PreclusteringMethod { NONE_PRECLUSTERING = 0, KCORE_PRECLUSTERING = 1 };
  enum MoveMethod { NBHR_CLUSTER_MOVE = 0, ALL_MOVE = 1, NBHR_MOVE = 2 };

  double resolution = 0;
  double edge_weight_offset = 0;
  uint32_t random_seed = 0;
  int64_t num_iterations = 0;
  LouvainConfig louvain_config;
  int32_t clustering_moves_method = LOUVAIN;
  int32_t subclustering_method = NONE_SUBCLUSTERING;
  int32_t preclustering_method = NONE_PRECLUSTERING;
  KcoreConfig kcore_config;
  bool refine = false;
  bool async = false;
  bool connect_stats = false;
  int32_t move_method = NBHR_CLUSTER_MOVE;
  bool all_iter = false;
  bool permute = false;
};

struct ClustererConfig {
  // The oneof of config.proto:188-197.
  enum ConfigCase { CONFIG_NOT_SET = 0, kParameterString = 1, kAffinityClustererConfig = 4,
                    kCorrelationClustererConfig = 7 };
  ConfigCase config_case = CONFIG_NOT_SET;
  std::string parameter_string;
  CorrelationClustererConfig correlation_clusterer_config;
};

// Parses a text-format ClustererConfig (google.protobuf.TextFormat syntax:
// `field: value`, nested `field { ... }` / `field < ... >`, optional `,` or
// `;` separators, `#` comments, enum names or numbers).  Unknown fields of
// the correlation config are errors, as in TextFormat::ParseFromString;
// the contents of affinity_clusterer_config are checked for syntax only.
Status ParseClustererConfig(const std::string& text, ClustererConfig* out);
// CorrelationClustererConfig -> the C ABI's pcc_config.
pcc_config ToPccConfig(const ClustererConfig& config);

// ---------------------------------------------------------------------------
// InMemoryClusterer (in-memory-clusterer.h:34-121)
// ---------------------------------------------------------------------------
class InMemoryClusterer {
 public:
  class Graph {
   public:
    using NodeId = uint32_t;
    struct AdjacencyList {
      NodeId id = static_cast<NodeId>(-1);
      double weight = 1;
      std::vector<std::pair<NodeId, double>> outgoing_edges;
    };
    virtual ~Graph() = default;
    // Safe to call concurrently.  Import must be called at most once per node.
    virtual Status Import(AdjacencyList adjacency_list) = 0;
    virtual Status FinishImport() { return Status::Ok(); }
  };

  using NodeId = Graph::NodeId;
  using AdjacencyList = Graph::AdjacencyList;
  using Clustering = std::vector<std::vector<NodeId>>;

  virtual ~InMemoryClusterer() = default;
  virtual Graph* MutableGraph() = 0;
  virtual StatusOr<Clustering> Cluster(const ClustererConfig& config) const = 0;
  virtual Status RefineClusters(const ClustererConfig& config, Clustering* clustering) const {
    return Status::Ok();
  }
};

// A symmetric CSR graph in host memory with GbbsGraph's import semantics:
// edges kept in the order given (weights stored as float), no
// symmetrisation, n = max(imported id, neighbour id) + 1, node weights of
// the adjacency lists ignored.  FinishImport builds the CSR.
class CsrGraph : public InMemoryClusterer::Graph {
 public:
  Status Import(AdjacencyList adjacency_list) override;
  Status FinishImport() override;
  // Direct CSR hand-over (the CLI's CopyGraph injection path).
  Status SetCsr(std::vector<uint64_t> offsets, std::vector<uint32_t> neighbors,
                std::vector<float> weights);
  uint32_t num_nodes() const { return n_; }
  uint64_t num_entries() const { return offsets_.empty() ? 0 : offsets_.back(); }
  const std::vector<uint64_t>& offsets() const { return offsets_; }
  const std::vector<uint32_t>& neighbors() const { return neighbors_; }
  // Empty for unit-weight graphs.
  const std::vector<float>& weights() const { return weights_; }
  bool finished() const { return finished_; }

 private:
  std::mutex mu_;
  std::vector<std::vector<std::pair<NodeId, float>>> rows_;
  std::vector<uint64_t> offsets_{0};
  std::vector<uint32_t> neighbors_;
  std::vector<float> weights_;
  uint32_t n_ = 0;
  bool finished_ = false;
};

// Options of the GPU clusterers (no reference counterpart).
struct GpuOptions {
  int device = 0;
  uint64_t hbm_budget_bytes = 0;  // 0 = device capacity
};

// ParallelCorrelationClusterer on the GB300 library.  Clustering order and
// error behaviour follow the reference: RefineClusters needs a clustering
// covering every node exactly once (INVALID_ARGUMENT otherwise).
class ParallelCorrelationClustererGB300 : public InMemoryClusterer {
 public:
  explicit ParallelCorrelationClustererGB300(GpuOptions options = {}) : options_(options) {}
  ~ParallelCorrelationClustererGB300() override;
  Graph* MutableGraph() override { return &graph_; }
  StatusOr<Clustering> Cluster(const ClustererConfig& config) const override;
  Status RefineClusters(const ClustererConfig& config, Clustering* clustering) const override;
  // Statistics of the last call (edge visits, rounds, timings).
  const pcc_stats& last_stats() const { return stats_; }
  // The CLI's graph read (cluster-in-memory_main.cc:285-306) on the device:
  // the GBBS adjacency file is parsed straight into the resident graph
  // (pcc_graph_read_gbbs) and replaces whatever MutableGraph() holds for
  // the following Cluster / RefineClusters calls.
  Status ReadGraphOnDevice(const std::string& path, bool float_weighted);

 protected:
  virtual int objective() const { return 0; }
  Status Run(const ClustererConfig& config, const std::vector<uint32_t>* initial,
             Clustering* out) const;
  Status EnsureDevice() const;
  Status EnsureContext() const;
  uint32_t num_nodes() const { return device_graph_only_ ? device_nodes_ : graph_.num_nodes(); }

  GpuOptions options_;
  CsrGraph graph_;
  mutable pcc_context* ctx_ = nullptr;
  mutable pcc_graph* dgraph_ = nullptr;
  mutable uint64_t uploaded_entries_ = 0;
  mutable uint32_t uploaded_nodes_ = 0;
  mutable pcc_stats stats_{};
  bool device_graph_only_ = false;  // dgraph_ came from ReadGraphOnDevice
  uint32_t device_nodes_ = 0;
};

// ParallelModularityClusterer: node weight = degree, resolution / total
// degree, offset 0 (parallel-modularity-clusterer.cc:68-111).
class ParallelModularityClustererGB300 : public ParallelCorrelationClustererGB300 {
 public:
  using ParallelCorrelationClustererGB300::ParallelCorrelationClustererGB300;

 protected:
  int objective() const override { return 1; }
};

// The CLI's clusterer dispatch (cluster-in-memory_main.cc:267-284).
// "ParallelCorrelationClusterer" / "ParallelModularityClusterer" (and their
// "...GB300" spellings) create the GPU clusterers; the reference's other
// names return UNIMPLEMENTED.
StatusOr<std::unique_ptr<InMemoryClusterer>> CreateClusterer(const std::string& name,
                                                             GpuOptions options = {});

// GBBS adjacency text format ("AdjacencyGraph" / "WeightedAdjacencyGraph":
// n, m, n offsets, m neighbour ids [, m weights]).
Status ReadGbbsAdjacencyGraph(const std::string& path, bool float_weighted, CsrGraph* graph);
Status WriteGbbsAdjacencyGraph(const std::string& path, const CsrGraph& graph);

// One cluster per line, node ids each followed by a tab
// (cluster-in-memory_main.cc:131-144).
Status WriteClustering(const std::string& path, const InMemoryClusterer::Clustering& clustering);
// The same file formatted on GPU `device` (pcc_write_clustering).
Status WriteClusteringOnDevice(const std::string& path, const InMemoryClusterer::Clustering& clustering,
                               int device);
Status ReadCommunities(const std::string& path, std::vector<std::vector<uint32_t>>* communities);

// Ground-truth scoring of CompareCommunities (cluster-in-memory_main.cc:
// 167-222): for each community the cluster with the largest intersection
// (first one on ties), precision = |intersection| / |cluster|, recall =
// |intersection| / |community|, averaged over communities; plus cluster
// size statistics.
struct CommunityScores {
  double avg_precision = 0;
  double avg_recall = 0;
  size_t num_clusters = 0;
  size_t min_size = 0;
  size_t max_size = 0;
  double avg_size = 0;
};
CommunityScores CompareCommunities(const std::vector<std::vector<uint32_t>>& communities,
                                   const InMemoryClusterer::Clustering& clustering);
// The same scores computed on the device (pcc_compare_communities) on GPU
// `device`; what the CLI's --input_communities step runs.
Status CompareCommunitiesOnDevice(const std::vector<std::vector<uint32_t>>& communities,
                                  const InMemoryClusterer::Clustering& clustering, int device,
                                  CommunityScores* out);

}  // namespace pcc_gb300

#endif  // PCC_CLUSTERER_H_
