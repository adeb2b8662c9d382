// generators.cc -- seeded synthetic graph generators for the workloads the
// clusterer is measured on (stand-ins for the paper's datasets): stochastic
// block models, RMAT (Graph500-style quadrant recursion) and LFR-like
// planted partitions.  Counter-based RNG (SplitMix64 of seed and index), so
// the output is the same for any thread count and on x86 and Arm.
//
// Every generator returns a symmetric CSR graph without self-loops or
// duplicate entries, rows sorted by neighbour id.

#include "pcc_host.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

namespace {

inline uint64_t SplitMix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

inline uint64_t Hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return SplitMix64(SplitMix64(seed ^ SplitMix64(a)) ^ (b * 0xD6E8FEB86659FD93ull));
}

// Uniform double in [0, 1) from 53 random bits.
inline double U01(uint64_t r) { return static_cast<double>(r >> 11) * (1.0 / 9007199254740992.0); }

struct Rng {
  uint64_t state;
  explicit Rng(uint64_t s) : state(s) {}
  uint64_t Next() {
    state += 0x9E3779B97F4A7C15ull;
    return SplitMix64(state);
  }
  double Uniform() { return U01(Next()); }
};

pcch_graph* NewGraph() {
  auto* g = static_cast<pcch_graph*>(std::calloc(1, sizeof(pcch_graph)));
  return g;
}

// Builds CSR from directed (u, v) pairs (both directions already present or
// added by `symmetrize`), dropping self-loops and duplicates; optional
// per-pair weights (the weight of the first copy of a duplicate is kept).
pcch_graph* BuildCsr(uint32_t n, std::vector<uint32_t>& src, std::vector<uint32_t>& dst,
                     std::vector<float>* wts, bool symmetrize) {
  const size_t E = src.size();
  const size_t total = symmetrize ? 2 * E : E;
  std::vector<std::atomic<uint64_t>> deg(size_t(n) + 1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(n) + 1; ++i) deg[i].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < int64_t(E); ++e) {
    if (src[e] == dst[e]) continue;
    deg[src[e]].fetch_add(1, std::memory_order_relaxed);
    if (symmetrize) deg[dst[e]].fetch_add(1, std::memory_order_relaxed);
  }
  std::vector<uint64_t> off(size_t(n) + 1, 0);
  for (uint32_t i = 0; i < n; ++i) off[i + 1] = off[i] + deg[i].load(std::memory_order_relaxed);
  std::vector<std::atomic<uint64_t>>& cur = deg;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(n); ++i) cur[i].store(off[i], std::memory_order_relaxed);
  std::vector<uint64_t> packed(off[n]);  // (neighbour << 32) | weight-index low bits unused
  std::vector<float> pw(wts ? off[n] : 0);
  (void)total;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < int64_t(E); ++e) {
    const uint32_t u = src[e], v = dst[e];
    if (u == v) continue;
    uint64_t p = cur[u].fetch_add(1, std::memory_order_relaxed);
    packed[p] = (uint64_t(v) << 32) | uint32_t(e & 0xFFFFFFFFu);
    if (wts) pw[p] = (*wts)[e];
    if (symmetrize) {
      p = cur[v].fetch_add(1, std::memory_order_relaxed);
      packed[p] = (uint64_t(u) << 32) | uint32_t(e & 0xFFFFFFFFu);
      if (wts) pw[p] = (*wts)[e];
    }
  }
  // Sort each row by (neighbour, source edge index) -- deterministic -- and
  // drop duplicates.
  std::vector<uint64_t> newdeg(size_t(n) + 1, 0);
#pragma omp parallel
  {
    std::vector<std::pair<uint64_t, float>> row;
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < int64_t(n); ++i) {
      const uint64_t b = off[i], e = off[i + 1];
      row.clear();
      for (uint64_t j = b; j < e; ++j) row.emplace_back(packed[j], wts ? pw[j] : 1.0f);
      std::sort(row.begin(), row.end(),
                [](const std::pair<uint64_t, float>& x, const std::pair<uint64_t, float>& y) {
                  return x.first < y.first;
                });
      uint64_t k = b;
      for (size_t j = 0; j < row.size(); ++j) {
        if (j > 0 && (row[j].first >> 32) == (row[j - 1].first >> 32)) continue;
        packed[k] = row[j].first;
        if (wts) pw[k] = row[j].second;
        ++k;
      }
      newdeg[i] = k - b;
    }
  }
  pcch_graph* g = NewGraph();
  g->n = n;
  g->off = static_cast<uint64_t*>(std::malloc(sizeof(uint64_t) * (size_t(n) + 1)));
  g->off[0] = 0;
  for (uint32_t i = 0; i < n; ++i) g->off[i + 1] = g->off[i] + newdeg[i];
  g->m = g->off[n];
  g->nbr = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * std::max<uint64_t>(g->m, 1)));
  if (wts) g->w = static_cast<float*>(std::malloc(sizeof(float) * std::max<uint64_t>(g->m, 1)));
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    const uint64_t b = off[i];
    const uint64_t o = g->off[i];
    for (uint64_t j = 0; j < newdeg[i]; ++j) {
      g->nbr[o + j] = static_cast<uint32_t>(packed[b + j] >> 32);
      if (wts) g->w[o + j] = pw[b + j];
    }
  }
  return g;
}

// Geometric skip sampling of Bernoulli(p) successes among `count` slots;
// calls f(slot) for each success in ascending order.
template <class F>
void SkipSample(Rng& rng, uint64_t count, double p, F f) {
  if (p <= 0 || count == 0) return;
  if (p >= 1) {
    for (uint64_t i = 0; i < count; ++i) f(i);
    return;
  }
  const double lq = std::log1p(-p);
  uint64_t i = 0;
  while (true) {
    const double u = 1.0 - rng.Uniform();  // (0, 1]
    const double skip = std::floor(std::log(u) / lq);
    if (skip >= double(count - i)) return;
    i += static_cast<uint64_t>(skip);
    f(i);
    ++i;
    if (i >= count) return;
  }
}

}  // namespace

extern "C" {

void pcch_graph_free(pcch_graph* g) {
  if (!g) return;
  std::free(g->off);
  std::free(g->nbr);
  std::free(g->w);
  std::free(g->truth);
  std::free(g);
}

// Stochastic block model: vertex i joins block Uniform[0, blocks) (so block
// sizes are multinomial with uniform probabilities); each unordered pair is
// an edge with p_in inside a block and p_out across blocks.  truth[i] is the
// block of vertex i.
pcch_graph* pcch_gen_sbm(uint32_t n, uint32_t blocks, double p_in, double p_out, uint64_t seed) {
  if (blocks == 0) blocks = 1;
  std::vector<uint32_t> block(n);
  for (uint32_t i = 0; i < n; ++i) block[i] = static_cast<uint32_t>(Hash3(seed, 1, i) % blocks);
  std::vector<std::vector<uint32_t>> members(blocks);
  for (uint32_t i = 0; i < n; ++i) members[block[i]].push_back(i);
  const int T = omp_get_max_threads();
  std::vector<std::vector<uint32_t>> ts(T), td(T);
#pragma omp parallel
  {
    const int t = omp_get_thread_num();
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < int64_t(n); ++i) {
      for (uint32_t b = 0; b < blocks; ++b) {
        const auto& mb = members[b];
        // Members of b greater than i.
        const size_t first = std::upper_bound(mb.begin(), mb.end(), uint32_t(i)) - mb.begin();
        const uint64_t count = mb.size() - first;
        Rng rng(Hash3(seed, 2 + uint64_t(i), b));
        const double p = (b == block[i]) ? p_in : p_out;
        SkipSample(rng, count, p, [&](uint64_t k) {
          ts[t].push_back(uint32_t(i));
          td[t].push_back(mb[first + k]);
        });
      }
    }
  }
  std::vector<uint32_t> src, dst;
  for (int t = 0; t < T; ++t) {
    src.insert(src.end(), ts[t].begin(), ts[t].end());
    dst.insert(dst.end(), td[t].begin(), td[t].end());
  }
  pcch_graph* g = BuildCsr(n, src, dst, nullptr, true);
  g->truth = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * std::max<uint32_t>(n, 1)));
  std::copy(block.begin(), block.end(), g->truth);
  return g;
}

// RMAT: edge_factor * 2^scale samples, each choosing one of four quadrants
// per level with probabilities a, b, c, 1-a-b-c; symmetrised, deduplicated,
// self-loops removed, unit weights.
pcch_graph* pcch_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed) {
  const uint32_t n = scale >= 32 ? 0xFFFFFFFFu : (1u << scale);
  const uint64_t M = uint64_t(edge_factor) << scale;
  std::vector<uint32_t> src(M), dst(M);
  const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < int64_t(M); ++e) {
    uint32_t u = 0, v = 0;
    uint64_t r = 0;
    for (uint32_t l = 0; l < scale; ++l) {
      if ((l & 1) == 0) r = Hash3(seed, uint64_t(e), l);
      const uint32_t bits32 = (l & 1) ? uint32_t(r >> 32) : uint32_t(r);
      const double x = bits32 * (1.0 / 4294967296.0);
      uint32_t bu, bv;
      if (x < a) {
        bu = 0; bv = 0;
      } else if (x < ab) {
        bu = 0; bv = 1;
      } else if (x < abc) {
        bu = 1; bv = 0;
      } else {
        bu = 1; bv = 1;
      }
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    src[e] = u;
    dst[e] = v;
  }
  return BuildCsr(n, src, dst, nullptr, true);
}

// LFR-like planted partition.  Degrees follow a discrete power law
// (exponent tau1) on [dmin, dmax]; a fraction q of the draws comes from
// [dmin + 1, dmax] instead, with dmin and q chosen so the sequence's mean is
// the target.  Community sizes follow a power law (exponent tau2) on
// [cmin, cmax].  Each vertex sends round((1 - mu) d) stubs inside its
// community and the rest outside; stubs are paired uniformly at random
// (configuration model) within each community and globally.  Self-loops and
// duplicates are dropped.  Weights are Uniform[w_lo, w_hi] per undirected
// edge (0 / 0 for unit weights).  truth[i] is the community of vertex i.
static pcch_graph* LfrOnce(uint32_t n, double mean_degree, uint32_t dmax, double tau1, uint32_t cmin, uint32_t cmax,
                    double tau2, double mu, double w_lo, double w_hi, uint64_t seed) {
  // Degree distribution.
  auto pl_mean = [&](uint32_t dmin) {
    double num = 0, den = 0;
    for (uint32_t d = dmin; d <= dmax; ++d) {
      const double p = std::pow(double(d), -tau1);
      num += d * p;
      den += p;
    }
    return num / den;
  };
  uint32_t dmin = 1;
  while (dmin < dmax && pl_mean(dmin + 1) <= mean_degree) ++dmin;
  auto make_cdf = [&](uint32_t lo) {
    std::vector<double> cdf;
    for (uint32_t d = lo; d <= dmax; ++d) cdf.push_back(std::pow(double(d), -tau1));
    for (size_t i = 1; i < cdf.size(); ++i) cdf[i] += cdf[i - 1];
    for (auto& x : cdf) x /= cdf.back();
    return cdf;
  };
  const std::vector<double> cdf = make_cdf(dmin);
  const std::vector<double> cdf_up = make_cdf(dmin < dmax ? dmin + 1 : dmin);
  const uint32_t dmin_up = dmin < dmax ? dmin + 1 : dmin;
  // Mix the laws from dmin and dmin + 1: fraction q from the upper one, so
  // (1 - q) mean(dmin) + q mean(dmin + 1) equals the target.
  const double m_lo = pl_mean(dmin), m_hi = pl_mean(dmin_up);
  const double q = m_hi > m_lo ? std::min(1.0, std::max(0.0, (mean_degree - m_lo) / (m_hi - m_lo))) : 0.0;
  std::vector<uint32_t> deg(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    const double u = U01(Hash3(seed, 11, uint64_t(i)));
    const bool up = U01(Hash3(seed, 16, uint64_t(i))) < q;
    const std::vector<double>& c = up ? cdf_up : cdf;
    const size_t k = std::lower_bound(c.begin(), c.end(), u) - c.begin();
    deg[i] = (up ? dmin_up : dmin) + static_cast<uint32_t>(std::min(k, c.size() - 1));
  }
  // Community sizes.
  std::vector<double> ccdf;
  for (uint32_t s = cmin; s <= cmax; ++s) ccdf.push_back(std::pow(double(s), -tau2));
  for (size_t i = 1; i < ccdf.size(); ++i) ccdf[i] += ccdf[i - 1];
  for (auto& x : ccdf) x /= ccdf.back();
  std::vector<uint32_t> csize;
  uint64_t covered = 0;
  for (uint64_t j = 0; covered < n; ++j) {
    const double u = U01(Hash3(seed, 12, j));
    const size_t k = std::lower_bound(ccdf.begin(), ccdf.end(), u) - ccdf.begin();
    uint32_t s = cmin + static_cast<uint32_t>(std::min(k, ccdf.size() - 1));
    if (covered + s > n) s = static_cast<uint32_t>(n - covered);
    csize.push_back(s);
    covered += s;
  }
  // Assign vertices to communities in a seeded random order.
  std::vector<uint32_t> order(n);
  std::iota(order.begin(), order.end(), 0u);
  {
    Rng rng(Hash3(seed, 13, 0));
    for (uint32_t i = n; i > 1; --i) std::swap(order[i - 1], order[rng.Next() % i]);
  }
  std::vector<uint32_t> comm(n);
  std::vector<uint64_t> cstart(csize.size() + 1, 0);
  for (size_t c = 0; c < csize.size(); ++c) cstart[c + 1] = cstart[c] + csize[c];
  for (size_t c = 0; c < csize.size(); ++c)
    for (uint64_t x = cstart[c]; x < cstart[c + 1]; ++x) comm[order[x]] = uint32_t(c);
  // Stubs.
  std::vector<std::vector<uint32_t>> inner(csize.size());
  std::vector<uint32_t> outer;
  for (size_t c = 0; c < csize.size(); ++c) {
    for (uint64_t x = cstart[c]; x < cstart[c + 1]; ++x) {
      const uint32_t v = order[x];
      uint32_t din = static_cast<uint32_t>(std::lround((1.0 - mu) * deg[v]));
      din = std::min<uint32_t>(din, csize[c] > 1 ? csize[c] - 1 : 0);
      for (uint32_t k = 0; k < din; ++k) inner[c].push_back(v);
      for (uint32_t k = din; k < deg[v]; ++k) outer.push_back(v);
    }
  }
  std::vector<uint32_t> src, dst;
  auto pair_up = [&](std::vector<uint32_t>& stubs, uint64_t salt) {
    Rng rng(Hash3(seed, 14, salt));
    for (size_t i = stubs.size(); i > 1; --i) std::swap(stubs[i - 1], stubs[rng.Next() % i]);
    for (size_t i = 0; i + 1 < stubs.size(); i += 2) {
      src.push_back(stubs[i]);
      dst.push_back(stubs[i + 1]);
    }
  };
  for (size_t c = 0; c < csize.size(); ++c) pair_up(inner[c], c + 1);
  pair_up(outer, 0);
  std::vector<float> w;
  const bool weighted = w_hi > 0;
  if (weighted) {
    w.resize(src.size());
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < int64_t(src.size()); ++e) {
      const uint32_t lo = std::min(src[e], dst[e]), hi = std::max(src[e], dst[e]);
      const double u = U01(Hash3(seed, 15, (uint64_t(lo) << 32) | hi));
      w[e] = static_cast<float>(w_lo + (w_hi - w_lo) * u);
    }
  }
  pcch_graph* g = BuildCsr(n, src, dst, weighted ? &w : nullptr, true);
  g->truth = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * std::max<uint32_t>(n, 1)));
  std::copy(comm.begin(), comm.end(), g->truth);
  return g;
}

// The realised mean degree falls short of the degree sequence's mean by the
// self-loops and duplicates dropped after pairing (small communities pair
// many stubs among few vertices).  One measured pass gives the shortfall; a
// second pass from the same seed asks for a mean raised by it, so that the
// realised mean lands on the configured one.
pcch_graph* pcch_gen_lfr(uint32_t n, double mean_degree, uint32_t dmax, double tau1, uint32_t cmin, uint32_t cmax,
                         double tau2, double mu, double w_lo, double w_hi, uint64_t seed) {
  pcch_graph* g = LfrOnce(n, mean_degree, dmax, tau1, cmin, cmax, tau2, mu, w_lo, w_hi, seed);
  if (!g || n == 0 || g->m == 0) return g;
  const double realised = double(g->m) / double(n);
  if (realised >= 0.998 * mean_degree) return g;
  const double target = std::min(double(dmax), mean_degree * mean_degree / realised);
  pcch_graph_free(g);
  return LfrOnce(n, target, dmax, tau1, cmin, cmax, tau2, mu, w_lo, w_hi, seed);
}

}  // extern "C"
