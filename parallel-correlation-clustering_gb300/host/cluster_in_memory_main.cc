// cluster_in_memory_main.cc -- command-line clusterer with the flags of the
// reference's cluster-in-memory_main (clustering/cluster-in-memory_main.cc:
// 24-54, 250-333): reads a GBBS adjacency graph, clusters it on the GPU and
// writes the clustering (one cluster per line, tab-separated node ids).
//
//   --clusterer_name      ParallelCorrelationClusterer | ParallelModularityClusterer
//   --clusterer_config    text-format ClustererConfig
//   --input_graph         GBBS adjacency file
//   --output_clustering   output path (optional)
//   --float_weighted      the file is a WeightedAdjacencyGraph
//   --is_symmetric_graph  accepted for compatibility (the adjacency input is
//                         symmetric already)
//   --input_communities   ground-truth communities: prints precision / recall
// GPU options (no reference counterpart): --device, --hbm_budget_gb,
// --device_io (default true: the graph file is parsed and the clustering
// file formatted on the GPU; --nodevice_io uses the host reader and writer).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>

#include "pcc_clusterer.h"

namespace {

using pcc_gb300::Status;

struct Flags {
  std::map<std::string, std::string> values;
  bool Has(const std::string& k) const { return values.count(k) != 0; }
  std::string Str(const std::string& k, const std::string& def = "") const {
    auto it = values.find(k);
    return it == values.end() ? def : it->second;
  }
  bool Bool(const std::string& k, bool def) const {
    auto it = values.find(k);
    if (it == values.end()) return def;
    return it->second == "true" || it->second == "1" || it->second.empty();
  }
};

const char* const kBoolFlags[] = {"float_weighted", "is_symmetric_graph", "device_io"};
const char* const kKnownFlags[] = {"clusterer_name", "clusterer_config", "input_graph", "output_clustering",
                                   "float_weighted", "is_symmetric_graph", "input_communities", "device",
                                   "hbm_budget_gb", "device_io"};

bool IsBool(const std::string& k) {
  for (const char* b : kBoolFlags)
    if (k == b) return true;
  return false;
}

Status ParseFlags(int argc, char** argv, Flags* f) {
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a.rfind("--", 0) != 0 && a.rfind("-", 0) == 0) a = "-" + a;
    if (a.rfind("--", 0) != 0) return Status(PCC_INVALID_ARGUMENT, "unexpected argument '" + a + "'");
    a = a.substr(2);
    std::string key = a, val;
    bool has_val = false;
    const size_t eq = a.find('=');
    if (eq != std::string::npos) {
      key = a.substr(0, eq);
      val = a.substr(eq + 1);
      has_val = true;
    }
    if (!has_val && key.rfind("no", 0) == 0 && IsBool(key.substr(2))) {
      key = key.substr(2);
      val = "false";
      has_val = true;
    }
    bool known = false;
    for (const char* k : kKnownFlags) known = known || key == k;
    if (!known) return Status(PCC_INVALID_ARGUMENT, "unknown flag --" + key);
    if (!has_val) {
      if (IsBool(key)) {
        val = "true";
      } else if (i + 1 < argc) {
        val = argv[++i];
      } else {
        return Status(PCC_INVALID_ARGUMENT, "flag --" + key + " needs a value");
      }
    }
    f->values[key] = val;
  }
  return Status::Ok();
}

void PrintTime(std::chrono::steady_clock::time_point b, std::chrono::steady_clock::time_point e,
               const std::string& what) {
  std::cout << what << " Time: "
            << std::chrono::duration_cast<std::chrono::microseconds>(e - b).count() / 1000000.0 << std::endl;
}

Status Main(int argc, char** argv) {
  Flags flags;
  Status s = ParseFlags(argc, argv, &flags);
  if (!s.ok()) return s;

  pcc_gb300::ClustererConfig config;
  const std::string text = flags.Str("clusterer_config");
  s = pcc_gb300::ParseClustererConfig(text, &config);
  if (!s.ok())
    return Status(PCC_INVALID_ARGUMENT,
                  "Cannot parse --clusterer_config as a text-format research_graph.in_memory.ClustererConfig "
                  "proto: " + text + " (" + s.message() + ")");

  pcc_gb300::GpuOptions opt;
  opt.device = std::atoi(flags.Str("device", "0").c_str());
  opt.hbm_budget_bytes = static_cast<uint64_t>(std::atof(flags.Str("hbm_budget_gb", "0").c_str()) * 1e9);
  auto made = pcc_gb300::CreateClusterer(flags.Str("clusterer_name"), opt);
  if (!made.ok()) return made.status();
  std::unique_ptr<pcc_gb300::InMemoryClusterer> clusterer = std::move(made.value());

  const bool device_io = flags.Bool("device_io", true);
  const auto begin_read = std::chrono::steady_clock::now();
  if (device_io) {
    auto* gpu = static_cast<pcc_gb300::ParallelCorrelationClustererGB300*>(clusterer.get());
    s = gpu->ReadGraphOnDevice(flags.Str("input_graph"), flags.Bool("float_weighted", false));
  } else {
    auto* graph = static_cast<pcc_gb300::CsrGraph*>(clusterer->MutableGraph());
    s = pcc_gb300::ReadGbbsAdjacencyGraph(flags.Str("input_graph"), flags.Bool("float_weighted", false), graph);
  }
  if (!s.ok()) return s;
  PrintTime(begin_read, std::chrono::steady_clock::now(), "Read graph");

  const auto begin_cluster = std::chrono::steady_clock::now();
  auto clustering = clusterer->Cluster(config);
  if (!clustering.ok()) return clustering.status();
  PrintTime(begin_cluster, std::chrono::steady_clock::now(), "Cluster");

  const std::string communities = flags.Str("input_communities");
  if (!communities.empty()) {
    std::vector<std::vector<uint32_t>> comm;
    s = pcc_gb300::ReadCommunities(communities, &comm);
    if (!s.ok()) return s;
    pcc_gb300::CommunityScores r;  // scored on the device
    s = pcc_gb300::CompareCommunitiesOnDevice(comm, *clustering, 0, &r);
    if (!s.ok()) return s;
    std::cout << "Avg precision: " << std::setprecision(17) << r.avg_precision << std::endl;
    std::cout << "Avg recall: " << std::setprecision(17) << r.avg_recall << std::endl;
    std::cout << "Num communities: " << r.num_clusters << std::endl;
    std::cout << "Min size: " << r.min_size << std::endl;
    std::cout << "Max size: " << r.max_size << std::endl;
    std::cout << "Avg size: " << r.avg_size << std::endl;
  }

  const std::string out = flags.Str("output_clustering");
  if (!out.empty()) {
    s = device_io ? pcc_gb300::WriteClusteringOnDevice(out, *clustering, opt.device)
                  : pcc_gb300::WriteClustering(out, *clustering);
    if (!s.ok()) return s;
  }
  return Status::Ok();
}

}  // namespace

int main(int argc, char** argv) {
  const Status s = Main(argc, argv);
  if (!s.ok()) {
    std::cerr << s.ToString() << std::endl;
    return EXIT_FAILURE;
  }
  return 0;
}
