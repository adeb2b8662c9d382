// clusterer.cc -- the C++ host mirror of the reference's clusterer
// interface (pcc_clusterer.h): text-format config parsing, GbbsGraph import
// semantics, the GPU clusterers over the C ABI, GBBS adjacency I/O and the
// CLI's clustering output / ground-truth scoring.
#include "pcc_clusterer.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <sstream>

#include "pcc_host.h"

namespace pcc_gb300 {

namespace {

const char* CodeName(pcc_status c) {
  switch (c) {
    case PCC_OK: return "OK";
    case PCC_CANCELLED: return "CANCELLED";
    case PCC_UNKNOWN: return "UNKNOWN";
    case PCC_INVALID_ARGUMENT: return "INVALID_ARGUMENT";
    case PCC_DEADLINE_EXCEEDED: return "DEADLINE_EXCEEDED";
    case PCC_NOT_FOUND: return "NOT_FOUND";
    case PCC_ALREADY_EXISTS: return "ALREADY_EXISTS";
    case PCC_PERMISSION_DENIED: return "PERMISSION_DENIED";
    case PCC_RESOURCE_EXHAUSTED: return "RESOURCE_EXHAUSTED";
    case PCC_FAILED_PRECONDITION: return "FAILED_PRECONDITION";
    case PCC_ABORTED: return "ABORTED";
    case PCC_OUT_OF_RANGE: return "OUT_OF_RANGE";
    case PCC_UNIMPLEMENTED: return "UNIMPLEMENTED";
    case PCC_INTERNAL: return "INTERNAL";
    case PCC_UNAVAILABLE: return "UNAVAILABLE";
    case PCC_DATA_LOSS: return "DATA_LOSS";
  }
  return "UNKNOWN";
}

Status Invalid(std::string m) { return Status(PCC_INVALID_ARGUMENT, std::move(m)); }

#define PCC_TRY(expr)             \
  do {                            \
    Status _s = (expr);           \
    if (!_s.ok()) return _s;      \
  } while (0)

// ---------------------------------------------------------------------------
// Text-format tokenizer and a generic message tree.
// ---------------------------------------------------------------------------
struct Token {
  enum Kind { kEnd, kIdent, kNumber, kString, kPunct } kind = kEnd;
  std::string text;
  int line = 1;
};

class Lexer {
 public:
  explicit Lexer(const std::string& s) : s_(s) {}

  Status Next(Token* t) {
    SkipSpace();
    t->line = line_;
    t->text.clear();
    if (i_ >= s_.size()) {
      t->kind = Token::kEnd;
      return Status::Ok();
    }
    const char c = s_[i_];
    if (std::isalpha(static_cast<unsigned char>(c)) || c == '_') {
      size_t j = i_;
      while (j < s_.size() && (std::isalnum(static_cast<unsigned char>(s_[j])) || s_[j] == '_' || s_[j] == '.'))
        ++j;
      t->kind = Token::kIdent;
      t->text = s_.substr(i_, j - i_);
      i_ = j;
      return Status::Ok();
    }
    if (std::isdigit(static_cast<unsigned char>(c)) || c == '-' || c == '+' || c == '.') {
      size_t j = i_ + 1;
      while (j < s_.size() && (std::isalnum(static_cast<unsigned char>(s_[j])) || s_[j] == '.' ||
                               ((s_[j] == '-' || s_[j] == '+') && (s_[j - 1] == 'e' || s_[j - 1] == 'E'))))
        ++j;
      t->kind = Token::kNumber;
      t->text = s_.substr(i_, j - i_);
      i_ = j;
      return Status::Ok();
    }
    if (c == '"' || c == '\'') {
      size_t j = i_ + 1;
      std::string out;
      while (j < s_.size() && s_[j] != c) {
        if (s_[j] == '\\' && j + 1 < s_.size()) {
          ++j;
          const char e = s_[j];
          out.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e);
        } else {
          if (s_[j] == '\n') ++line_;
          out.push_back(s_[j]);
        }
        ++j;
      }
      if (j >= s_.size()) return Invalid("line " + std::to_string(line_) + ": unterminated string");
      t->kind = Token::kString;
      t->text = out;
      i_ = j + 1;
      return Status::Ok();
    }
    if (std::strchr("{}<>:,;[]", c)) {
      t->kind = Token::kPunct;
      t->text = std::string(1, c);
      ++i_;
      return Status::Ok();
    }
    return Invalid("line " + std::to_string(line_) + ": unexpected character '" + std::string(1, c) + "'");
  }

 private:
  void SkipSpace() {
    while (i_ < s_.size()) {
      const char c = s_[i_];
      if (c == '\n') {
        ++line_;
        ++i_;
      } else if (std::isspace(static_cast<unsigned char>(c))) {
        ++i_;
      } else if (c == '#') {
        while (i_ < s_.size() && s_[i_] != '\n') ++i_;
      } else {
        break;
      }
    }
  }
  const std::string& s_;
  size_t i_ = 0;
  int line_ = 1;
};

struct Field;
struct Message {
  std::vector<Field> fields;
};
struct Field {
  std::string name;
  bool is_message = false;
  Token value;
  std::shared_ptr<Message> message;
  int line = 1;
};

class Parser {
 public:
  explicit Parser(const std::string& s) : lex_(s) {}

  Status ParseTop(Message* m) {
    PCC_TRY(Advance());
    return ParseFields(m, "");
  }

 private:

  Status Advance() { return lex_.Next(&tok_); }

  Status ParseFields(Message* m, const std::string& close) {
    while (true) {
      if (tok_.kind == Token::kEnd) {
        if (!close.empty()) return Invalid("line " + std::to_string(tok_.line) + ": expected '" + close + "'");
        return Status::Ok();
      }
      if (tok_.kind == Token::kPunct && tok_.text == close) return Status::Ok();
      if (tok_.kind != Token::kIdent)
        return Invalid("line " + std::to_string(tok_.line) + ": expected a field name, got '" + tok_.text + "'");
      Field f;
      f.name = tok_.text;
      f.line = tok_.line;
      PCC_TRY(Advance());
      bool colon = false;
      if (tok_.kind == Token::kPunct && tok_.text == ":") {
        colon = true;
        PCC_TRY(Advance());
      }
      if (tok_.kind == Token::kPunct && (tok_.text == "{" || tok_.text == "<")) {
        const std::string end = tok_.text == "{" ? "}" : ">";
        f.is_message = true;
        f.message = std::make_shared<Message>();
        PCC_TRY(Advance());
        PCC_TRY(ParseFields(f.message.get(), end));
        PCC_TRY(Advance());
      } else {
        if (!colon)
          return Invalid("line " + std::to_string(f.line) + ": expected ':' after field '" + f.name + "'");
        if (tok_.kind != Token::kIdent && tok_.kind != Token::kNumber && tok_.kind != Token::kString)
          return Invalid("line " + std::to_string(f.line) + ": missing value of field '" + f.name + "'");
        f.value = tok_;
        PCC_TRY(Advance());
        // Adjacent string literals concatenate.
        while (f.value.kind == Token::kString && tok_.kind == Token::kString) {
          f.value.text += tok_.text;
          PCC_TRY(Advance());
        }
      }
      m->fields.push_back(std::move(f));
      if (tok_.kind == Token::kPunct && (tok_.text == "," || tok_.text == ";")) PCC_TRY(Advance());
    }
  }

  Lexer lex_;
  Token tok_;
};

std::string Where(const Field& f) { return "line " + std::to_string(f.line) + ": field '" + f.name + "'"; }

Status ScalarExpected(const Field& f) {
  if (f.is_message) return Invalid(Where(f) + " is not a message");
  return Status::Ok();
}

Status GetDouble(const Field& f, double* out) {
  Status s = ScalarExpected(f);
  if (!s.ok()) return s;
  std::string t = f.value.text;
  if (f.value.kind == Token::kIdent) {
    std::string l = t;
    std::transform(l.begin(), l.end(), l.begin(), [](unsigned char c) { return std::tolower(c); });
    if (l == "inf" || l == "infinity") {
      *out = std::numeric_limits<double>::infinity();
      return Status::Ok();
    }
    if (l == "nan") {
      *out = std::numeric_limits<double>::quiet_NaN();
      return Status::Ok();
    }
    return Invalid(Where(f) + ": expected a number, got '" + t + "'");
  }
  if (f.value.kind != Token::kNumber) return Invalid(Where(f) + ": expected a number");
  std::string l = t;
  std::transform(l.begin(), l.end(), l.begin(), [](unsigned char c) { return std::tolower(c); });
  if (l == "-inf" || l == "-infinity") {
    *out = -std::numeric_limits<double>::infinity();
    return Status::Ok();
  }
  if (!l.empty() && l.back() == 'f' && l.find('x') == std::string::npos) t.pop_back();
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str() || *end != '\0') return Invalid(Where(f) + ": invalid number '" + f.value.text + "'");
  *out = v;
  return Status::Ok();
}

Status GetInt(const Field& f, int64_t lo, int64_t hi, int64_t* out) {
  Status s = ScalarExpected(f);
  if (!s.ok()) return s;
  if (f.value.kind != Token::kNumber) return Invalid(Where(f) + ": expected an integer");
  const std::string& t = f.value.text;
  char* end = nullptr;
  errno = 0;
  long long v = 0;
  if (!t.empty() && t[0] != '-') {
    const unsigned long long u = std::strtoull(t.c_str(), &end, 0);
    if (u > static_cast<unsigned long long>(std::numeric_limits<long long>::max())) errno = ERANGE;
    v = static_cast<long long>(u);
  } else {
    v = std::strtoll(t.c_str(), &end, 0);
  }
  if (end == t.c_str() || *end != '\0' || errno == ERANGE || v < lo || v > hi)
    return Invalid(Where(f) + ": invalid or out-of-range integer '" + t + "'");
  *out = v;
  return Status::Ok();
}

Status GetBool(const Field& f, bool* out) {
  Status s = ScalarExpected(f);
  if (!s.ok()) return s;
  const std::string& t = f.value.text;
  if (t == "true" || t == "True" || t == "t" || t == "1") {
    *out = true;
  } else if (t == "false" || t == "False" || t == "f" || t == "0") {
    *out = false;
  } else {
    return Invalid(Where(f) + ": expected a bool, got '" + t + "'");
  }
  return Status::Ok();
}

Status GetEnum(const Field& f, const std::vector<std::pair<const char*, int>>& values, int32_t* out) {
  Status s = ScalarExpected(f);
  if (!s.ok()) return s;
  if (f.value.kind == Token::kIdent) {
    for (const auto& [name, num] : values) {
      if (f.value.text == name) {
        *out = num;
        return Status::Ok();
      }
    }
    return Invalid(Where(f) + ": unknown enum value '" + f.value.text + "'");
  }
  int64_t v = 0;
  s = GetInt(f, std::numeric_limits<int32_t>::min(), std::numeric_limits<int32_t>::max(), &v);
  if (!s.ok()) return s;
  for (const auto& [name, num] : values) {
    if (v == num) {
      *out = static_cast<int32_t>(v);
      return Status::Ok();
    }
  }
  return Invalid(Where(f) + ": unknown enum number " + f.value.text);
}

Status MessageExpected(const Field& f) {
  if (!f.is_message) return Invalid(Where(f) + " is a message; expected '{'");
  return Status::Ok();
}


Status ApplyLouvain(const Message& m, LouvainConfig* c) {
  for (const Field& f : m.fields) {
    if (f.name == "num_iterations") {
      PCC_TRY(GetInt(f, INT64_MIN, INT64_MAX, &c->num_iterations));
    } else if (f.name == "num_inner_iterations") {
      PCC_TRY(GetInt(f, INT64_MIN, INT64_MAX, &c->num_inner_iterations));
    } else {
      return Invalid(Where(f) + ": no such field in LouvainConfig");
    }
  }
  return Status::Ok();
}

Status ApplyKcore(const Message& m, KcoreConfig* c) {
  for (const Field& f : m.fields) {
    int64_t v = 0;
    if (f.name == "kcore_cutoff") {
      PCC_TRY(GetInt(f, INT32_MIN, INT32_MAX, &v));
      c->kcore_cutoff = static_cast<int32_t>(v);
    } else if (f.name == "fix_preclusters") {
      PCC_TRY(GetBool(f, &c->fix_preclusters));
    } else if (f.name == "connect_only") {
      PCC_TRY(GetBool(f, &c->connect_only));
    } else if (f.name == "percent_cutoff") {
      PCC_TRY(GetDouble(f, &c->percent_cutoff));
    } else {
      return Invalid(Where(f) + ": no such field in KcoreConfig");
    }
  }
  return Status::Ok();
}

Status ApplyCorrelation(const Message& m, CorrelationClustererConfig* c) {
  using C = CorrelationClustererConfig;
  for (const Field& f : m.fields) {
    int64_t v = 0;
    if (f.name == "resolution") {
      PCC_TRY(GetDouble(f, &c->resolution));
    } else if (f.name == "edge_weight_offset") {
      PCC_TRY(GetDouble(f, &c->edge_weight_offset));
    } else if (f.name == "random_seed") {
      PCC_TRY(GetInt(f, 0, UINT32_MAX, &v));
      c->random_seed = static_cast<uint32_t>(v);
    } else if (f.name == "num_iterations") {
      PCC_TRY(GetInt(f, INT64_MIN, INT64_MAX, &c->num_iterations));
    } else if (f.name == "louvain_config") {
      PCC_TRY(MessageExpected(f));
      PCC_TRY(ApplyLouvain(*f.message, &c->louvain_config));
    } else if (f.name == "clustering_moves_method") {
      PCC_TRY(GetEnum(f, {{"DEFAULT_CLUSTER_MOVES", C::DEFAULT_CLUSTER_MOVES}, {"LOUVAIN", C::LOUVAIN}},
                      &c->clustering_moves_method));
    } else if (f.name == "subclustering_method") {
      PCC_TRY(GetEnum(f,
                      {{"NONE_SUBCLUSTERING", C::NONE_SUBCLUSTERING},
                       {"TRIANGLE_SUBCLUSTERING", C::TRIANGLE_SUBCLUSTERING},
                       {"CONNECTIVITY_SUBCLUSTERING", C::CONNECTIVITY_SUBCLUSTERING},
                       {"SLOW_CONNECTIVITY_SUBCLUSTERING", C::SLOW_CONNECTIVITY_SUBCLUSTERING}},
                      &c->subclustering_method));
    } else if (f.name == "preclustering_method") {
      PCC_TRY(GetEnum(f, {{"NONE_PRECLUSTERING", C::NONE_PRECLUSTERING},
                          {"KCORE_PRECLUSTERING", C::KCORE_PRECLUSTERING}},
                      &c->preclustering_method));
    } else if (f.name == "kcore_config") {
      PCC_TRY(MessageExpected(f));
      PCC_TRY(ApplyKcore(*f.message, &c->kcore_config));
    } else if (f.name == "refine") {
      PCC_TRY(GetBool(f, &c->refine));
    } else if (f.name == "async") {
      PCC_TRY(GetBool(f, &c->async));
    } else if (f.name == "connect_stats") {
      PCC_TRY(GetBool(f, &c->connect_stats));
    } else if (f.name == "move_method") {
      PCC_TRY(GetEnum(f, {{"NBHR_CLUSTER_MOVE", C::NBHR_CLUSTER_MOVE}, {"ALL_MOVE", C::ALL_MOVE},
                          {"NBHR_MOVE", C::NBHR_MOVE}},
                      &c->move_method));
    } else if (f.name == "all_iter") {
      PCC_TRY(GetBool(f, &c->all_iter));
    } else if (f.name == "permute") {
      PCC_TRY(GetBool(f, &c->permute));
    } else {
      return Invalid(Where(f) + ": no such field in CorrelationClustererConfig");
    }
  }
  return Status::Ok();
}

Status CheckAffinity(const Message& m) {
  // Syntax only: the affinity clusterer is not part of this library.
  for (const Field& f : m.fields) {
    static const char* kKnown[] = {"num_iterations", "weight_threshold", "edge_aggregation_function",
                                   "active_cluster_conditions"};
    bool ok = false;
    for (const char* k : kKnown) ok = ok || f.name == k;
    if (!ok) return Invalid(Where(f) + ": no such field in AffinityClustererConfig");
  }
  return Status::Ok();
}

}  // namespace

std::string Status::ToString() const {
  if (ok()) return "OK";
  return std::string(CodeName(code_)) + ": " + message_;
}

Status ParseClustererConfig(const std::string& text, ClustererConfig* out) {
  ClustererConfig cfg;
  Message top;
  Parser p(text);
  PCC_TRY(p.ParseTop(&top));
  for (const Field& f : top.fields) {
    if (f.name == "correlation_clusterer_config") {
      PCC_TRY(MessageExpected(f));
      cfg.config_case = ClustererConfig::kCorrelationClustererConfig;
      cfg.correlation_clusterer_config = CorrelationClustererConfig();
      PCC_TRY(ApplyCorrelation(*f.message, &cfg.correlation_clusterer_config));
    } else if (f.name == "affinity_clusterer_config") {
      PCC_TRY(MessageExpected(f));
      PCC_TRY(CheckAffinity(*f.message));
      cfg.config_case = ClustererConfig::kAffinityClustererConfig;
      cfg.correlation_clusterer_config = CorrelationClustererConfig();
    } else if (f.name == "parameter_string") {
      if (f.is_message || f.value.kind != Token::kString) return Invalid(Where(f) + ": expected a string");
      cfg.config_case = ClustererConfig::kParameterString;
      cfg.parameter_string = f.value.text;
      cfg.correlation_clusterer_config = CorrelationClustererConfig();
    } else {
      return Invalid(Where(f) + ": no such field in ClustererConfig");
    }
  }
  *out = cfg;
  return Status::Ok();
}

pcc_config ToPccConfig(const ClustererConfig& config) {
  const CorrelationClustererConfig& c = config.correlation_clusterer_config;
  pcc_config p;
  pcc_config_default(&p);
  p.resolution = c.resolution;
  p.edge_weight_offset = c.edge_weight_offset;
  p.num_iterations = c.num_iterations;
  p.louvain_num_iterations = c.louvain_config.num_iterations;
  p.louvain_num_inner_iterations = c.louvain_config.num_inner_iterations;
  p.clustering_moves_method = c.clustering_moves_method;
  p.subclustering_method = c.subclustering_method;
  p.preclustering_method = c.preclustering_method;
  p.move_method = c.move_method;
  p.refine = c.refine ? 1 : 0;
  p.async = c.async ? 1 : 0;
  p.permute = c.permute ? 1 : 0;
  p.all_iter = c.all_iter ? 1 : 0;
  p.random_seed = c.random_seed;
  return p;
}

// ---------------------------------------------------------------------------
// CsrGraph (GbbsGraph import semantics, gbbs-graph.cc:28-76)
// ---------------------------------------------------------------------------
Status CsrGraph::Import(AdjacencyList adjacency_list) {
  if (adjacency_list.id == static_cast<NodeId>(-1)) return Invalid("adjacency list without a node id");
  std::vector<std::pair<NodeId, float>> row(adjacency_list.outgoing_edges.size());
  for (size_t i = 0; i < row.size(); ++i)
    row[i] = {adjacency_list.outgoing_edges[i].first, static_cast<float>(adjacency_list.outgoing_edges[i].second)};
  std::lock_guard<std::mutex> lock(mu_);
  if (rows_.size() <= adjacency_list.id) rows_.resize(size_t(adjacency_list.id) + 1);
  rows_[adjacency_list.id] = std::move(row);
  finished_ = false;
  return Status::Ok();
}

Status CsrGraph::FinishImport() {
  std::lock_guard<std::mutex> lock(mu_);
  uint64_t n = rows_.size();
  for (const auto& r : rows_)
    for (const auto& e : r) n = std::max<uint64_t>(n, uint64_t(e.first) + 1);
  if (n > 0xFFFFFFFFull) return Status(PCC_OUT_OF_RANGE, "more than 2^32 - 1 nodes");
  rows_.resize(n);
  offsets_.assign(n + 1, 0);
  bool unit = true;
  for (uint64_t v = 0; v < n; ++v) {
    offsets_[v + 1] = offsets_[v] + rows_[v].size();
    for (const auto& e : rows_[v]) unit = unit && e.second == 1.0f;
  }
  neighbors_.resize(offsets_[n]);
  weights_.clear();
  if (!unit) weights_.resize(offsets_[n]);
  for (uint64_t v = 0; v < n; ++v) {
    uint64_t j = offsets_[v];
    for (const auto& e : rows_[v]) {
      neighbors_[j] = e.first;
      if (!unit) weights_[j] = e.second;
      ++j;
    }
  }
  n_ = static_cast<uint32_t>(n);
  finished_ = true;
  return Status::Ok();
}

Status CsrGraph::SetCsr(std::vector<uint64_t> offsets, std::vector<uint32_t> neighbors,
                        std::vector<float> weights) {
  if (offsets.empty() || offsets.front() != 0) return Invalid("offsets must start at 0");
  if (offsets.size() - 1 > 0xFFFFFFFFull) return Status(PCC_OUT_OF_RANGE, "more than 2^32 - 1 nodes");
  for (size_t i = 1; i < offsets.size(); ++i)
    if (offsets[i] < offsets[i - 1]) return Invalid("offsets must be non-decreasing");
  if (offsets.back() != neighbors.size()) return Invalid("offsets[n] must equal the number of neighbours");
  if (!weights.empty() && weights.size() != neighbors.size()) return Invalid("one weight per entry");
  const uint64_t n = offsets.size() - 1;
  for (uint32_t u : neighbors)
    if (u >= n) return Invalid("neighbour id out of range");
  std::lock_guard<std::mutex> lock(mu_);
  rows_.clear();
  offsets_ = std::move(offsets);
  neighbors_ = std::move(neighbors);
  weights_ = std::move(weights);
  n_ = static_cast<uint32_t>(n);
  finished_ = true;
  return Status::Ok();
}

// ---------------------------------------------------------------------------
// GPU clusterers
// ---------------------------------------------------------------------------
ParallelCorrelationClustererGB300::~ParallelCorrelationClustererGB300() {
  if (ctx_) {
    if (dgraph_) pcc_graph_free(ctx_, dgraph_);
    pcc_destroy(ctx_);
  }
}

Status ParallelCorrelationClustererGB300::EnsureContext() const {
  if (!ctx_) {
    const pcc_status s = pcc_create(&ctx_, options_.device, options_.hbm_budget_bytes);
    if (s != PCC_OK) {
      ctx_ = nullptr;
      return Status(s, "pcc_create failed (no usable GPU)");
    }
  }
  return Status::Ok();
}

Status ParallelCorrelationClustererGB300::ReadGraphOnDevice(const std::string& path, bool float_weighted) {
  PCC_TRY(EnsureContext());
  pcc_graph* g = nullptr;
  const pcc_status s = pcc_graph_read_gbbs(ctx_, path.c_str(), float_weighted ? 1 : 0, &g);
  if (s != PCC_OK) return Status(s, pcc_last_error(ctx_));
  uint64_t m = 0;
  int32_t hw = 0;
  pcc_graph_info(g, &device_nodes_, &m, &hw);
  if (dgraph_) pcc_graph_free(ctx_, dgraph_);
  dgraph_ = g;
  device_graph_only_ = true;
  return Status::Ok();
}

Status ParallelCorrelationClustererGB300::EnsureDevice() const {
  if (device_graph_only_) return Status::Ok();
  if (!graph_.finished()) return Status(PCC_FAILED_PRECONDITION, "FinishImport has not been called");
  PCC_TRY(EnsureContext());
  // Re-upload when the graph changed since the last upload.
  if (dgraph_ && (uploaded_nodes_ != graph_.num_nodes() || uploaded_entries_ != graph_.num_entries())) {
    pcc_graph_free(ctx_, dgraph_);
    dgraph_ = nullptr;
  }
  if (!dgraph_) {
    const auto& w = graph_.weights();
    const pcc_status s = pcc_graph_upload(ctx_, graph_.num_nodes(), graph_.num_entries(),
                                          graph_.offsets().data(), graph_.neighbors().data(),
                                          w.empty() ? nullptr : w.data(), &dgraph_);
    if (s != PCC_OK) {
      dgraph_ = nullptr;
      return Status(s, pcc_last_error(ctx_));
    }
    uploaded_nodes_ = graph_.num_nodes();
    uploaded_entries_ = graph_.num_entries();
  }
  return Status::Ok();
}

Status ParallelCorrelationClustererGB300::Run(const ClustererConfig& config,
                                             const std::vector<uint32_t>* initial,
                                             Clustering* out) const {
  PCC_TRY(EnsureDevice());
  const pcc_config p = ToPccConfig(config);
  const uint32_t n = num_nodes();
  std::vector<uint32_t> labels(n);
  stats_ = pcc_stats{};
  const uint32_t* init = initial ? initial->data() : nullptr;
  const pcc_status s = objective() == 1
                           ? pcc_modularity_cluster(ctx_, dgraph_, &p, init, labels.data(), &stats_)
                           : pcc_correlation_cluster(ctx_, dgraph_, &p, nullptr, init, labels.data(), &stats_);
  if (s != PCC_OK) return Status(s, pcc_last_error(ctx_));
  uint32_t k = 0;
  for (uint32_t l : labels) k = std::max(k, l + 1);
  out->assign(k, {});
  for (uint32_t v = 0; v < n; ++v) (*out)[labels[v]].push_back(v);
  return Status::Ok();
}

StatusOr<InMemoryClusterer::Clustering> ParallelCorrelationClustererGB300::Cluster(
    const ClustererConfig& config) const {
  Clustering c;
  Status s = Run(config, nullptr, &c);
  if (!s.ok()) return s;
  return c;
}

Status ParallelCorrelationClustererGB300::RefineClusters(const ClustererConfig& config,
                                                        Clustering* clustering) const {
  if (!clustering) return Invalid("null clustering");
  if (!device_graph_only_ && !graph_.finished())
    return Status(PCC_FAILED_PRECONDITION, "FinishImport has not been called");
  const uint32_t n = num_nodes();
  std::vector<uint32_t> init(n, 0xFFFFFFFFu);
  for (size_t c = 0; c < clustering->size(); ++c) {
    for (NodeId v : (*clustering)[c]) {
      if (v >= n) return Invalid("clustering names node " + std::to_string(v) + " >= n");
      if (init[v] != 0xFFFFFFFFu) return Invalid("node " + std::to_string(v) + " is in two clusters");
      init[v] = static_cast<uint32_t>(c);
    }
  }
  for (uint32_t v = 0; v < n; ++v)
    if (init[v] == 0xFFFFFFFFu) return Invalid("node " + std::to_string(v) + " is in no cluster");
  // Cluster ids must be < n for the C ABI: compact them (the order of the
  // given clusters is kept, so the result does not depend on empty ones).
  std::vector<uint32_t> remap(clustering->size(), 0xFFFFFFFFu);
  uint32_t next = 0;
  for (uint32_t v = 0; v < n; ++v) {
    uint32_t& r = remap[init[v]];
    if (r == 0xFFFFFFFFu) r = next++;
  }
  for (uint32_t v = 0; v < n; ++v) init[v] = remap[init[v]];
  Clustering out;
  PCC_TRY(Run(config, &init, &out));
  *clustering = std::move(out);
  return Status::Ok();
}

StatusOr<std::unique_ptr<InMemoryClusterer>> CreateClusterer(const std::string& name, GpuOptions options) {
  std::unique_ptr<InMemoryClusterer> c;
  if (name == "ParallelCorrelationClusterer" || name == "ParallelCorrelationClustererGB300") {
    c.reset(new ParallelCorrelationClustererGB300(options));
  } else if (name == "ParallelModularityClusterer" || name == "ParallelModularityClustererGB300") {
    c.reset(new ParallelModularityClustererGB300(options));
  } else {
    return Status(PCC_UNIMPLEMENTED,
                  "ParallelCorrelationClusterer and ParallelModularityClusterer are the only supported "
                  "clusterers (got '" + name + "')");
  }
  return c;
}

// ---------------------------------------------------------------------------
// GBBS adjacency text format
// ---------------------------------------------------------------------------
namespace {

class WordReader {
 public:
  explicit WordReader(const std::string& data) : d_(data) {}
  bool Next(std::string* w) {
    while (i_ < d_.size() && std::isspace(static_cast<unsigned char>(d_[i_]))) ++i_;
    if (i_ >= d_.size()) return false;
    const size_t j0 = i_;
    while (i_ < d_.size() && !std::isspace(static_cast<unsigned char>(d_[i_]))) ++i_;
    w->assign(d_, j0, i_ - j0);
    return true;
  }
  bool NextU64(uint64_t* v) {
    while (i_ < d_.size() && std::isspace(static_cast<unsigned char>(d_[i_]))) ++i_;
    if (i_ >= d_.size() || !std::isdigit(static_cast<unsigned char>(d_[i_]))) return false;
    uint64_t x = 0;
    while (i_ < d_.size() && std::isdigit(static_cast<unsigned char>(d_[i_]))) {
      const uint64_t dgt = static_cast<uint64_t>(d_[i_] - '0');
      if (x > (UINT64_MAX - dgt) / 10) return false;
      x = x * 10 + dgt;
      ++i_;
    }
    *v = x;
    return i_ >= d_.size() || std::isspace(static_cast<unsigned char>(d_[i_]));
  }
  bool NextFloat(float* v) {
    std::string w;
    if (!Next(&w)) return false;
    char* end = nullptr;
    *v = std::strtof(w.c_str(), &end);
    return end != w.c_str() && *end == '\0';
  }

 private:
  const std::string& d_;
  size_t i_ = 0;
};

}  // namespace

Status ReadGbbsAdjacencyGraph(const std::string& path, bool float_weighted, CsrGraph* graph) {
  std::ifstream f(path, std::ios::binary);
  if (!f.is_open()) return Status(PCC_NOT_FOUND, "Unable to open file " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string data = ss.str();
  WordReader r(data);
  std::string header;
  if (!r.Next(&header)) return Invalid(path + ": empty file");
  const bool weighted = header == "WeightedAdjacencyGraph";
  if (!weighted && header != "AdjacencyGraph") return Invalid(path + ": bad header '" + header + "'");
  if (weighted != float_weighted)
    return Invalid(path + ": header '" + header + "' does not match float_weighted=" +
                   (float_weighted ? "true" : "false"));
  uint64_t n = 0, m = 0;
  if (!r.NextU64(&n) || !r.NextU64(&m)) return Invalid(path + ": bad n / m");
  if (n > 0xFFFFFFFFull) return Status(PCC_OUT_OF_RANGE, path + ": more than 2^32 - 1 nodes");
  std::vector<uint64_t> off(n + 1);
  for (uint64_t i = 0; i < n; ++i)
    if (!r.NextU64(&off[i])) return Invalid(path + ": bad offset " + std::to_string(i));
  off[n] = m;
  std::vector<uint32_t> nbr(m);
  for (uint64_t j = 0; j < m; ++j) {
    uint64_t x = 0;
    if (!r.NextU64(&x) || x >= n) return Invalid(path + ": bad neighbour id at entry " + std::to_string(j));
    nbr[j] = static_cast<uint32_t>(x);
  }
  std::vector<float> w;
  if (weighted) {
    w.resize(m);
    bool unit = true;
    for (uint64_t j = 0; j < m; ++j) {
      if (!r.NextFloat(&w[j])) return Invalid(path + ": bad weight at entry " + std::to_string(j));
      unit = unit && w[j] == 1.0f;
    }
    if (unit) w.clear();
  }
  return graph->SetCsr(std::move(off), std::move(nbr), std::move(w));
}

Status WriteGbbsAdjacencyGraph(const std::string& path, const CsrGraph& graph) {
  std::ofstream f(path);
  if (!f.is_open()) return Status(PCC_NOT_FOUND, "Unable to open file " + path);
  const bool weighted = !graph.weights().empty();
  const uint32_t n = graph.num_nodes();
  f << (weighted ? "WeightedAdjacencyGraph" : "AdjacencyGraph") << "\n" << n << "\n" << graph.num_entries() << "\n";
  for (uint32_t i = 0; i < n; ++i) f << graph.offsets()[i] << "\n";
  for (uint32_t u : graph.neighbors()) f << u << "\n";
  if (weighted) {
    f.precision(9);
    for (float w : graph.weights()) f << w << "\n";
  }
  return f.good() ? Status::Ok() : Status(PCC_DATA_LOSS, "write failed: " + path);
}

Status WriteClustering(const std::string& path, const InMemoryClusterer::Clustering& clustering) {
  std::ofstream f(path);
  if (!f.is_open()) return Status(PCC_NOT_FOUND, "Unable to open file.");
  for (const auto& cluster : clustering) {
    for (auto v : cluster) f << v << "\t";
    f << "\n";
  }
  return Status::Ok();
}

Status WriteClusteringOnDevice(const std::string& path, const InMemoryClusterer::Clustering& clustering,
                               int device) {
  size_t n = 0;
  for (const auto& c : clustering) n += c.size();
  std::vector<uint32_t> labels(n, 0xFFFFFFFFu);
  for (size_t c = 0; c < clustering.size(); ++c)
    for (auto v : clustering[c]) {
      if (v >= n || labels[v] != 0xFFFFFFFFu) return Invalid("the clustering must cover nodes 0..n-1 once each");
      labels[v] = static_cast<uint32_t>(c);
    }
  if (n > 0xFFFFFFFFull) return Status(PCC_OUT_OF_RANGE, "more than 2^32 - 1 nodes");
  pcc_context* ctx = nullptr;
  pcc_status s = pcc_create(&ctx, device, 0);
  if (s != PCC_OK) return Status(s, "pcc_create failed (no usable GPU)");
  s = pcc_write_clustering(ctx, path.c_str(), static_cast<uint32_t>(n), labels.data());
  const std::string msg = s == PCC_OK ? "" : pcc_last_error(ctx);
  pcc_destroy(ctx);
  return Status(s, msg);
}

Status ReadCommunities(const std::string& path, std::vector<std::vector<uint32_t>>* communities) {
  std::ifstream f(path);
  if (!f.is_open()) return Status(PCC_NOT_FOUND, "Unable to open file.");
  std::string line;
  while (std::getline(f, line)) {
    std::vector<uint32_t> row;
    std::stringstream ls(line);
    std::string item;
    while (std::getline(ls, item, '\t')) {
      if (item.empty()) continue;
      row.push_back(static_cast<uint32_t>(std::stoul(item)));
    }
    std::sort(row.begin(), row.end());
    communities->push_back(std::move(row));
  }
  return Status::Ok();
}

// pbbs::reduce_add order: a serial fold of <= 1024 items, else serial folds
// of 1024-item blocks followed by the same reduce over the block sums.
static double BlockedSum(const std::vector<double>& a) {
  if (a.empty()) return 0.0;
  if (a.size() <= 1024) {
    double r = a[0];
    for (size_t j = 1; j < a.size(); ++j) r += a[j];
    return r;
  }
  std::vector<double> sums((a.size() + 1023) / 1024);
  for (size_t b = 0; b < sums.size(); ++b) {
    const size_t s = b * 1024, e = std::min(a.size(), s + 1024);
    double r = a[s];
    for (size_t j = s + 1; j < e; ++j) r += a[j];
    sums[b] = r;
  }
  return BlockedSum(sums);
}

CommunityScores CompareCommunities(const std::vector<std::vector<uint32_t>>& communities,
                                   const InMemoryClusterer::Clustering& clustering) {
  CommunityScores out;
  std::vector<std::vector<uint32_t>> sorted(clustering.begin(), clustering.end());
  for (auto& c : sorted) std::sort(c.begin(), c.end());
  // node -> cluster index, to count intersections in one pass per community.
  uint32_t max_node = 0;
  for (const auto& c : sorted)
    for (uint32_t v : c) max_node = std::max(max_node, v + 1);
  std::vector<uint32_t> owner(max_node, 0xFFFFFFFFu);
  for (size_t i = 0; i < sorted.size(); ++i)
    for (uint32_t v : sorted[i]) owner[v] = static_cast<uint32_t>(i);
  std::vector<double> prec(communities.size(), 0.0), rec(communities.size(), 0.0);
  std::map<uint32_t, size_t> count;
  std::vector<uint32_t> distinct;
  for (size_t j = 0; j < communities.size(); ++j) {
    const std::vector<uint32_t>& community = communities[j];
    // std::set_intersection counts a repeated member once: the cluster
    // holds it once.
    distinct.assign(community.begin(), community.end());
    std::sort(distinct.begin(), distinct.end());
    distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
    count.clear();
    for (uint32_t v : distinct)
      if (v < max_node && owner[v] != 0xFFFFFFFFu) ++count[owner[v]];
    // The largest intersection, the first cluster (lowest index) on ties;
    // cluster 0 when nothing intersects.
    size_t best = 0, best_idx = 0;
    for (const auto& [idx, cnt] : count) {
      if (cnt > best) {
        best = cnt;
        best_idx = idx;
      }
    }
    const double denom = sorted.empty() ? 0.0 : static_cast<double>(sorted[best_idx].size());
    prec[j] = denom > 0 ? static_cast<double>(best) / denom : 0.0;
    rec[j] = community.empty() ? 0.0 : static_cast<double>(best) / static_cast<double>(community.size());
  }
  out.avg_precision = BlockedSum(prec) / static_cast<double>(communities.size());
  out.avg_recall = BlockedSum(rec) / static_cast<double>(communities.size());
  out.num_clusters = sorted.size();
  out.min_size = 0xFFFFFFFFu;  // UINT_E_MAX, the reference's start value
  for (const auto& c : sorted) {
    out.min_size = std::min(out.min_size, c.size());
    out.max_size = std::max(out.max_size, c.size());
    out.avg_size += static_cast<double>(c.size());
  }
  out.avg_size /= static_cast<double>(sorted.size());
  return out;
}

Status CompareCommunitiesOnDevice(const std::vector<std::vector<uint32_t>>& communities,
                                  const InMemoryClusterer::Clustering& clustering, int device,
                                  CommunityScores* out) {
  // Labels: cluster i of the clustering is label i (OutputIndicesById order).
  uint64_t n64 = 0;
  for (const auto& c : clustering) n64 += c.size();
  if (n64 > 0xFFFFFFFFull) return Status(PCC_INVALID_ARGUMENT, "clustering too large");
  const uint32_t n = static_cast<uint32_t>(n64);
  std::vector<uint32_t> labels(n, 0xFFFFFFFFu);
  for (size_t i = 0; i < clustering.size(); ++i)
    for (uint32_t v : clustering[i]) {
      if (v >= n || labels[v] != 0xFFFFFFFFu)
        return Status(PCC_INVALID_ARGUMENT, "the clustering must cover nodes 0..n-1 once");
      labels[v] = static_cast<uint32_t>(i);
    }
  std::vector<uint64_t> offsets(communities.size() + 1, 0);
  std::vector<uint32_t> members;
  for (size_t j = 0; j < communities.size(); ++j) {
    members.insert(members.end(), communities[j].begin(), communities[j].end());
    offsets[j + 1] = members.size();
  }
  pcc_context* ctx = nullptr;
  pcc_status st = pcc_create(&ctx, device, 0);
  if (st != PCC_OK) return Status(st, "pcc_create failed (no usable GPU)");
  pcc_community_scores r{};
  st = pcc_compare_communities(ctx, n, labels.data(), static_cast<uint32_t>(communities.size()), offsets.data(),
                               members.empty() ? nullptr : members.data(), nullptr, nullptr, &r);
  const std::string msg = st == PCC_OK ? std::string() : std::string(pcc_last_error(ctx));
  pcc_destroy(ctx);
  if (st != PCC_OK) return Status(st, msg);
  out->avg_precision = r.avg_precision;
  out->avg_recall = r.avg_recall;
  out->num_clusters = static_cast<size_t>(r.num_clusters);
  out->min_size = static_cast<size_t>(r.min_size);
  out->max_size = static_cast<size_t>(r.max_size);
  out->avg_size = r.avg_size;
  return Status::Ok();
}

}  // namespace pcc_gb300

// ---------------------------------------------------------------------------
// C entry points of the host library for bindings and tests
// ---------------------------------------------------------------------------
extern "C" {

int32_t pcch_parse_config(const char* text, pcc_config* out, int32_t* config_case, char* err, size_t err_len) {
  if (!text || !out) return PCC_INVALID_ARGUMENT;
  pcc_gb300::ClustererConfig cfg;
  const pcc_gb300::Status s = pcc_gb300::ParseClustererConfig(text, &cfg);
  if (err && err_len) {
    std::strncpy(err, s.message().c_str(), err_len - 1);
    err[err_len - 1] = '\0';
  }
  if (!s.ok()) return s.code();
  *out = pcc_gb300::ToPccConfig(cfg);
  if (config_case) *config_case = cfg.config_case;
  return PCC_OK;
}

pcch_graph* pcch_read_gbbs(const char* path, int32_t float_weighted, int32_t* status) {
  int32_t dummy = 0;
  int32_t& st = status ? *status : dummy;
  st = PCC_INVALID_ARGUMENT;
  if (!path) return nullptr;
  pcc_gb300::CsrGraph g;
  const pcc_gb300::Status s = pcc_gb300::ReadGbbsAdjacencyGraph(path, float_weighted != 0, &g);
  if (!s.ok()) {
    st = s.code();
    return nullptr;
  }
  auto* out = static_cast<pcch_graph*>(std::calloc(1, sizeof(pcch_graph)));
  if (!out) {
    st = PCC_RESOURCE_EXHAUSTED;
    return nullptr;
  }
  out->n = g.num_nodes();
  out->m = g.num_entries();
  out->off = static_cast<uint64_t*>(std::malloc(sizeof(uint64_t) * (size_t(out->n) + 1)));
  out->nbr = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * std::max<uint64_t>(out->m, 1)));
  if (!g.weights().empty()) out->w = static_cast<float*>(std::malloc(sizeof(float) * out->m));
  if (!out->off || !out->nbr || (!g.weights().empty() && !out->w)) {
    pcch_graph_free(out);
    st = PCC_RESOURCE_EXHAUSTED;
    return nullptr;
  }
  std::memcpy(out->off, g.offsets().data(), sizeof(uint64_t) * (size_t(out->n) + 1));
  if (out->m) std::memcpy(out->nbr, g.neighbors().data(), sizeof(uint32_t) * out->m);
  if (out->w) std::memcpy(out->w, g.weights().data(), sizeof(float) * out->m);
  st = PCC_OK;
  return out;
}

int32_t pcch_compare_communities(const char* communities_path, uint32_t n, const uint32_t* labels,
                                 double* out6) {
  if (!communities_path || (!labels && n) || !out6) return PCC_INVALID_ARGUMENT;
  std::vector<std::vector<uint32_t>> comm;
  const pcc_gb300::Status s = pcc_gb300::ReadCommunities(communities_path, &comm);
  if (!s.ok()) return s.code();
  uint32_t k = 0;
  for (uint32_t v = 0; v < n; ++v) k = std::max(k, labels[v] + 1);
  pcc_gb300::InMemoryClusterer::Clustering cl(k);
  for (uint32_t v = 0; v < n; ++v) cl[labels[v]].push_back(v);
  // OutputIndicesById lists only the labels in use, in ascending order.
  cl.erase(std::remove_if(cl.begin(), cl.end(), [](const std::vector<uint32_t>& c) { return c.empty(); }),
           cl.end());
  const pcc_gb300::CommunityScores r = pcc_gb300::CompareCommunities(comm, cl);
  out6[0] = r.avg_precision;
  out6[1] = r.avg_recall;
  out6[2] = static_cast<double>(r.num_clusters);
  out6[3] = static_cast<double>(r.min_size);
  out6[4] = static_cast<double>(r.max_size);
  out6[5] = r.avg_size;
  return PCC_OK;
}

}  // extern "C"
