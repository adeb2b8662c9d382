// ingest.cu -- the CLI's input and output steps on the device.
//
// * GBBS adjacency text ("AdjacencyGraph" / "WeightedAdjacencyGraph": the
//   header, n, m, n offsets, m neighbour ids, then m weights) parsed straight
//   into a resident graph.  Replaces gbbs_io::read_(un)weighted_symmetric_
//   graph + CopyGraph in clustering/cluster-in-memory_main.cc:285-306.  The
//   result equals the host reader of this package (ReadGbbsAdjacencyGraph in
//   host/clusterer.cc) on every input that reader accepts, and errors arise
//   in the same order: the first bad token in file order, then the offset
//   checks of CsrGraph::SetCsr.
// * WriteClustering (cluster-in-memory_main.cc:132-145) formatted on the
//   device: one line per cluster in cluster order, each member id followed by
//   a tab, then a newline.
//
// Parsing: the bytes after the m token are copied to the device once.  An
// exclusive scan over "token starts here" flags gives every token its index
// (kScanTile bytes per CTA); the thread owning a token's first byte parses
// it and stores it in the offsets, neighbour or weight array.  Whitespace is
// the C locale's isspace set.  Offsets and ids are decimal digits only, with
// overflow checks (the host reader's NextU64).  Weights are converted as
// strtof does: the nearest float, ties to even, for the decimal forms
// [+-]digits[.digits][(e|E)[+-]digits] and inf / infinity / nan.  The
// conversion takes Clinger's fast path (an exact double product or quotient,
// then a float rounding that cannot double-round unless the double lands on
// a float midpoint) and otherwise decides between neighbouring floats by an
// exact big-integer comparison of the decimal value with their midpoint.
// Hexadecimal floats, nan(...) payloads and tokens of more than
// kMaxSigDigits significant digits are rejected as INVALID_ARGUMENT with a
// message naming the device reader's limit.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include <math_constants.h>

#include "engine.cuh"

namespace pcc {
namespace {

constexpr int kMaxSigDigits = 200;

__host__ __device__ __forceinline__ bool IsSpace(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }
__host__ __device__ __forceinline__ bool IsDigit(unsigned char c) { return c >= '0' && c <= '9'; }
__host__ __device__ __forceinline__ unsigned char Lower(unsigned char c) {
  return (c >= 'A' && c <= 'Z') ? static_cast<unsigned char>(c + 32) : c;
}

// ---------------------------------------------------------------------------
// Big unsigned integers for the exact comparison (little-endian 32-bit limbs).
// ---------------------------------------------------------------------------
constexpr int kLimbs = 40;  // 1280 bits: 200 digits (665 bits) times 5^246 fits

struct Big {
  uint32_t d[kLimbs];
  int len;  // limbs in use (d[len..) are zero)
};

__device__ void BigSet(Big& a, uint64_t v) {
  for (int i = 0; i < kLimbs; ++i) a.d[i] = 0;
  a.d[0] = static_cast<uint32_t>(v);
  a.d[1] = static_cast<uint32_t>(v >> 32);
  a.len = a.d[1] ? 2 : (a.d[0] ? 1 : 0);
}

// a = a * f + add; false if the result needs more than kLimbs limbs.
__device__ bool BigMulAdd(Big& a, uint32_t f, uint32_t add) {
  uint64_t carry = add;
  for (int i = 0; i < a.len; ++i) {
    const uint64_t t = uint64_t(a.d[i]) * f + carry;
    a.d[i] = static_cast<uint32_t>(t);
    carry = t >> 32;
  }
  if (carry) {
    if (a.len == kLimbs) return false;
    a.d[a.len++] = static_cast<uint32_t>(carry);
  }
  return true;
}

__device__ bool BigMulPow5(Big& a, int e) {
  constexpr uint32_t k5_13 = 1220703125u;  // 5^13 < 2^32
  while (e >= 13) {
    if (!BigMulAdd(a, k5_13, 0)) return false;
    e -= 13;
  }
  uint32_t f = 1;
  while (e-- > 0) f *= 5;
  return BigMulAdd(a, f, 0);
}

__device__ bool BigShl(Big& a, int k) {
  if (a.len == 0 || k == 0) return true;
  const int limbs = k / 32, bits = k % 32;
  if (a.len + limbs + 1 > kLimbs) return false;
  for (int i = a.len - 1; i >= 0; --i) {
    const uint32_t v = a.d[i];
    a.d[i + limbs + 1] |= bits ? (v >> (32 - bits)) : 0u;
    a.d[i + limbs] = bits ? (v << bits) : v;
  }
  for (int i = 0; i < limbs; ++i) a.d[i] = 0;
  a.len += limbs + 1;
  while (a.len > 0 && a.d[a.len - 1] == 0) --a.len;
  return true;
}

__device__ int BigCmp(const Big& a, const Big& b) {
  if (a.len != b.len) return a.len < b.len ? -1 : 1;
  for (int i = a.len - 1; i >= 0; --i)
    if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
  return 0;
}

// ---------------------------------------------------------------------------
// Decimal -> float.
// ---------------------------------------------------------------------------
enum ParseResult : int { kParsed = 0, kBadToken = 1, kUnsupported = 2 };

struct DecimalToken {
  const unsigned char* p;  // the significant digits are read again from here
  uint64_t len;            // token length
  bool neg;
  uint64_t m19;            // first (up to) 19 significant digits
  int nd;                  // significant digits in total
  int64_t e19;             // value ~= m19 * 10^e19
  int64_t eall;            // value == digits * 10^eall (all significant digits)
};

// Exact comparison of the token's decimal value with the positive double q.
__device__ int CompareExact(const DecimalToken& t, double q, bool* ok) {
  Big L, R;
  // The significant digits as an integer.
  BigSet(L, 0);
  int seen = 0;
  bool started = false;
  for (uint64_t i = 0; i < t.len && seen < t.nd; ++i) {
    const unsigned char c = t.p[i];
    if (c == 'e' || c == 'E') break;
    if (!IsDigit(c)) continue;
    if (!started && c == '0') continue;
    started = true;
    if (!BigMulAdd(L, 10u, uint32_t(c - '0'))) {
      *ok = false;
      return 0;
    }
    ++seen;
  }
  // q = Q * 2^qe, Q < 2^53.
  const unsigned long long bits = __double_as_longlong(q);
  const int be = int((bits >> 52) & 0x7FF);
  const uint64_t Q = (bits & ((1ull << 52) - 1)) | (be ? (1ull << 52) : 0ull);
  const int qe = (be ? be : 1) - 1075;
  BigSet(R, Q);
  // digits * 5^e * 2^e  vs  Q * 2^qe.
  const int64_t e = t.eall;
  bool good = e >= 0 ? BigMulPow5(L, int(e)) : BigMulPow5(R, int(-e));
  const int64_t dl = e - qe;  // power of two on the left minus the right
  if (good) good = dl >= 0 ? BigShl(L, int(dl)) : BigShl(R, int(-dl));
  *ok = good;
  return good ? BigCmp(L, R) : 0;
}

__device__ __forceinline__ float NextUp(float f) {  // f >= 0, finite
  return __uint_as_float(__float_as_uint(f) + 1u);
}
__device__ __forceinline__ float NextDown(float f) {  // f > 0
  return __uint_as_float(__float_as_uint(f) - 1u);
}
// Midpoint of adjacent non-negative floats a < b (b may be +inf: the
// overflow threshold, 2^128 - 2^103).
__device__ __forceinline__ double Midpoint(float a, float b) {
  if (isinf(b)) return 340282356779733661637539395458142568448.0;  // 2^128 - 2^103
  return (double(a) + double(b)) * 0.5;
}
__device__ __forceinline__ bool EvenMantissa(float f) {
  return isinf(f) || (__float_as_uint(f) & 1u) == 0;
}

// Powers of ten that doubles hold exactly (10^22 < 2^53 * 2^22).
__constant__ double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                  1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

__device__ int ParseFloatToken(const unsigned char* p, uint64_t len, float* out) {
  uint64_t i = 0;
  bool neg = false;
  if (i < len && (p[i] == '+' || p[i] == '-')) {
    neg = p[i] == '-';
    ++i;
  }
  // inf, infinity, nan (case-insensitive), as strtof.
  auto word = [&](const char* w) {
    uint64_t k = 0;
    while (w[k]) {
      if (i + k >= len || Lower(p[i + k]) != static_cast<unsigned char>(w[k])) return false;
      ++k;
    }
    return i + k == len;
  };
  if (i < len && (Lower(p[i]) == 'i' || Lower(p[i]) == 'n')) {
    if (word("inf") || word("infinity")) {
      *out = neg ? -CUDART_INF_F : CUDART_INF_F;
      return kParsed;
    }
    if (word("nan")) {
      *out = __uint_as_float(neg ? 0xFFC00000u : 0x7FC00000u);
      return kParsed;
    }
    if (i + 3 < len && Lower(p[i]) == 'n' && Lower(p[i + 1]) == 'a' && Lower(p[i + 2]) == 'n' && p[i + 3] == '(')
      return kUnsupported;
    return kBadToken;
  }
  if (i + 1 < len && p[i] == '0' && Lower(p[i + 1]) == 'x') return kUnsupported;
  DecimalToken t;
  t.p = p + i;
  t.len = len - i;
  t.neg = neg;
  t.m19 = 0;
  t.nd = 0;
  int64_t e19 = 0, eall = 0;
  bool any = false, point = false, started = false;
  for (; i < len; ++i) {
    const unsigned char c = p[i];
    if (c == '.') {
      if (point) return kBadToken;
      point = true;
      continue;
    }
    if (!IsDigit(c)) break;
    any = true;
    const int dg = c - '0';
    if (!started && dg == 0) {
      if (point) {
        --e19;
        --eall;
      }
      continue;
    }
    started = true;
    if (t.nd < 19) {
      t.m19 = t.m19 * 10 + uint64_t(dg);
      if (point) --e19;
    } else if (!point) {
      ++e19;
    }
    if (point) --eall;
    if (++t.nd > kMaxSigDigits) return kUnsupported;
  }
  if (!any) return kBadToken;
  int64_t ex = 0;
  if (i < len && (p[i] == 'e' || p[i] == 'E')) {
    uint64_t j = i + 1;
    bool eneg = false;
    if (j < len && (p[j] == '+' || p[j] == '-')) {
      eneg = p[j] == '-';
      ++j;
    }
    if (j >= len || !IsDigit(p[j])) return kBadToken;  // strtof stops before the 'e'
    for (; j < len && IsDigit(p[j]); ++j)
      if (ex < 100000) ex = ex * 10 + (p[j] - '0');
    ex = eneg ? -ex : ex;
    i = j;
  }
  if (i != len) return kBadToken;
  t.e19 = e19 + ex;
  t.eall = eall + ex;
  float r;
  if (t.nd == 0) {
    r = 0.f;
  } else if (t.nd + t.eall >= 40) {  // >= 10^39 > FLT_MAX
    r = CUDART_INF_F;
  } else if (t.nd + t.eall <= -46) {  // < 10^-46 < 2^-150: rounds to 0
    r = 0.f;
  } else {
    // Approximation d of the value (relative error far below a float ulp).
    double d = double(t.m19);
    int64_t e = t.e19;
    const bool fast = t.nd <= 19 && t.m19 < (1ull << 53) && e >= -22 && e <= 22;
    while (e > 22) {
      d *= 1e22;
      e -= 22;
    }
    while (e < -22) {
      d /= 1e22;
      e += 22;
    }
    d = e >= 0 ? d * kPow10[e] : d / kPow10[-e];
    const float f0 = __double2float_rn(d);
    bool exact_needed = !fast;
    if (fast && double(f0) != d) {
      // d is the correctly rounded double of the value; rounding it to float
      // is right unless d sits exactly on a float midpoint.
      const float g = double(f0) < d ? (isinf(f0) ? f0 : NextUp(f0)) : (f0 > 0.f ? NextDown(f0) : f0);
      const double mid = double(f0) < d ? Midpoint(f0, g) : Midpoint(g, f0);
      exact_needed = d == mid;
    }
    if (!exact_needed) {
      r = f0;
    } else {
      // The result is f0 or one of its neighbours.
      const float hi = isinf(f0) ? f0 : NextUp(f0);
      const float lo = f0 > 0.f ? NextDown(f0) : f0;
      bool ok = true;
      int c2 = -1;
      if (!isinf(f0)) c2 = CompareExact(t, Midpoint(f0, hi), &ok);
      if (!ok) return kUnsupported;
      if (c2 > 0) {
        r = hi;
      } else if (c2 == 0) {
        r = EvenMantissa(f0) ? f0 : hi;
      } else {
        int c1 = 1;
        if (f0 > 0.f) c1 = CompareExact(t, Midpoint(lo, f0), &ok);
        if (!ok) return kUnsupported;
        if (c1 < 0) r = lo;
        else if (c1 == 0) r = EvenMantissa(lo) ? lo : f0;
        else r = f0;
      }
    }
  }
  *out = neg ? -r : r;
  return kParsed;
}

// Digits only, no overflow, as NextU64 of the host reader.
__device__ bool ParseU64Token(const unsigned char* p, uint64_t len, uint64_t* out) {
  if (len == 0) return false;
  uint64_t x = 0;
  for (uint64_t i = 0; i < len; ++i) {
    if (!IsDigit(p[i])) return false;
    const uint64_t dg = uint64_t(p[i] - '0');
    if (x > (~0ull - dg) / 10) return false;
    x = x * 10 + dg;
  }
  *out = x;
  return true;
}

// ---------------------------------------------------------------------------
// Token scan and parse.
// ---------------------------------------------------------------------------
struct TokenStart {
  const unsigned char* b;
  uint64_t len;
  __device__ uint64_t operator()(uint64_t i) const {
    return (!IsSpace(b[i]) && (i == 0 || IsSpace(b[i - 1]))) ? 1ull : 0ull;
  }
};

// Error key: (token index << 2) | kind; the smallest key is the first error
// in file order.
constexpr unsigned long long kNoError = ~0ull;

struct TokenParse {
  const unsigned char* b;
  uint64_t len;
  uint32_t n;
  uint64_t m;
  bool weighted;
  uint64_t* off;
  uint32_t* nbr;
  float* w;
  unsigned long long* err;
  unsigned int* nonunit;
  __device__ void operator()(uint64_t i, uint64_t k, uint64_t v) const {
    if (!v) return;
    const uint64_t need = uint64_t(n) + m + (weighted ? m : 0);
    if (k >= need) return;  // trailing tokens are ignored, as the host reader does
    uint64_t e = i;
    while (e < len && !IsSpace(b[e])) ++e;
    const unsigned char* p = b + i;
    const uint64_t tl = e - i;
    if (k < n) {
      uint64_t x;
      if (ParseU64Token(p, tl, &x)) off[k] = x;
      else atomicMin(err, (k << 2) | kBadToken);
    } else if (k < uint64_t(n) + m) {
      uint64_t x;
      if (ParseU64Token(p, tl, &x) && x < n) nbr[k - n] = static_cast<uint32_t>(x);
      else atomicMin(err, (k << 2) | kBadToken);
    } else {
      float f;
      const int r = ParseFloatToken(p, tl, &f);
      if (r == kParsed) {
        w[k - n - m] = f;
        if (!(f == 1.0f)) atomicOr(nonunit, 1u);
      } else {
        atomicMin(err, (k << 2) | unsigned(r));
      }
    }
  }
};

// SetCsr's offset checks: 1 = does not start at 0, 2 = decreasing.
__global__ void OffsetOrderKernel(uint32_t n, const uint64_t* __restrict__ off, int* bad) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i <= n; i += uint64_t(gridDim.x) * blockDim.x) {
    if (i == 0 && off[0] != 0) atomicMin(bad, 1);
    if (i < n && off[i] > off[i + 1]) atomicMin(bad, 2);
  }
}

// Host-side reading of the first tokens (header, n, m), as WordReader.
struct HostWords {
  const char* d;
  uint64_t size;
  uint64_t i = 0;
  bool Next(std::string* w) {
    while (i < size && IsSpace(static_cast<unsigned char>(d[i]))) ++i;
    if (i >= size) return false;
    const uint64_t j = i;
    while (i < size && !IsSpace(static_cast<unsigned char>(d[i]))) ++i;
    w->assign(d + j, i - j);
    return true;
  }
  bool NextU64(uint64_t* v) {
    while (i < size && IsSpace(static_cast<unsigned char>(d[i]))) ++i;
    if (i >= size || !IsDigit(static_cast<unsigned char>(d[i]))) return false;
    uint64_t x = 0;
    while (i < size && IsDigit(static_cast<unsigned char>(d[i]))) {
      const uint64_t dg = uint64_t(d[i] - '0');
      if (x > (~0ull - dg) / 10) return false;
      x = x * 10 + dg;
      ++i;
    }
    *v = x;
    return i >= size || IsSpace(static_cast<unsigned char>(d[i]));
  }
};

Status Invalid(const std::string& msg) { return MakeError(PCC_INVALID_ARGUMENT, msg); }

Status ParseGbbs(Context* ctx, const char* text, uint64_t size, bool float_weighted, const std::string& name,
                 std::unique_ptr<pcc_graph>* out) {
  HostWords r{text, size};
  std::string header;
  if (!r.Next(&header)) return Invalid(name + ": empty file");
  const bool weighted = header == "WeightedAdjacencyGraph";
  if (!weighted && header != "AdjacencyGraph") return Invalid(name + ": bad header '" + header + "'");
  if (weighted != float_weighted)
    return Invalid(name + ": header '" + header + "' does not match float_weighted=" +
                   (float_weighted ? "true" : "false"));
  uint64_t n64 = 0, m = 0;
  if (!r.NextU64(&n64) || !r.NextU64(&m)) return Invalid(name + ": bad n / m");
  if (n64 > 0xFFFFFFFFull) return MakeError(PCC_OUT_OF_RANGE, name + ": more than 2^32 - 1 nodes");
  if (n64 > 0xFFFFFFFFull - 31) return Invalid(name + ": n must be at most 2^32 - 32 for the GPU library");
  if (m >= 0xFFFFFFFFull) return Invalid(name + ": graphs with 2^32 or more entries are not supported");
  const uint32_t n = static_cast<uint32_t>(n64);
  const uint64_t rest = size - r.i;  // bytes after the m token (starts with whitespace or is empty)

  auto h = std::make_unique<pcc_graph>();
  DevGraph& g = h->g;
  g.n = n;
  g.m = m;
  PCC_RETURN_IF_ERROR(g.off.Alloc(ctx, uint64_t(n) + 1));
  PCC_RETURN_IF_ERROR(g.nbr.Alloc(ctx, m ? m : 1));
  if (weighted) PCC_RETURN_IF_ERROR(g.w.Alloc(ctx, m ? m : 1));
  DBuf<unsigned char> bytes;
  PCC_RETURN_IF_ERROR(bytes.Alloc(ctx, rest ? rest : 1));
  if (rest) PCC_CUDA(cudaMemcpyAsync(bytes.p, text + r.i, rest, cudaMemcpyHostToDevice, ctx->stream));
  DBuf<unsigned long long> err;
  DBuf<unsigned int> nonunit;
  DBuf<uint64_t> total, tiles;
  DBuf<int> bad;
  PCC_RETURN_IF_ERROR(err.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(nonunit.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(total.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(bad.Alloc(ctx, 1));
  PCC_RETURN_IF_ERROR(err.Fill(0xFF));
  PCC_RETURN_IF_ERROR(nonunit.Zero());
  PCC_RETURN_IF_ERROR(bad.Fill(0x7F));
  const TokenStart ts{bytes.p, rest};
  const TokenParse tp{bytes.p, rest, n, m, weighted, g.off.p, g.nbr.p, g.w.p, err.p, nonunit.p};
  PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, rest, ts, tp, tiles, total.p));
  // off[n] = m (the host reader's off[n]), then SetCsr's order checks.
  PCC_CUDA(cudaMemcpyAsync(g.off.p + n, &m, sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
  OffsetOrderKernel<<<Blocks(uint64_t(n) + 1, 256, unsigned(ctx->num_sms) * 8), 256, 0, ctx->stream>>>(n, g.off.p,
                                                                                                        bad.p);
  PCC_COUNT(1);
  unsigned long long herr = 0;
  uint64_t htotal = 0;
  unsigned int hnonunit = 0;
  int hbad = 0;
  PCC_RETURN_IF_ERROR(err.ToHost(&herr, 1));
  PCC_RETURN_IF_ERROR(total.ToHost(&htotal, 1));
  PCC_RETURN_IF_ERROR(nonunit.ToHost(&hnonunit, 1));
  PCC_RETURN_IF_ERROR(bad.ToHost(&hbad, 1));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  const uint64_t need = uint64_t(n) + m + (weighted ? m : 0);
  uint64_t first = herr == kNoError ? ~0ull : (herr >> 2);
  int kind = herr == kNoError ? kBadToken : int(herr & 3);
  if (htotal < need && htotal <= first) {
    first = htotal;  // the first missing token
    kind = kBadToken;
  }
  if (first < need) {
    const std::string limit =
        kind == kUnsupported ? " (the device reader takes decimal, inf and nan weights of at most " +
                                   std::to_string(kMaxSigDigits) + " significant digits)"
                             : "";
    if (first < n) return Invalid(name + ": bad offset " + std::to_string(first));
    if (first < uint64_t(n) + m) return Invalid(name + ": bad neighbour id at entry " + std::to_string(first - n));
    return Invalid(name + ": bad weight at entry " + std::to_string(first - n - m) + limit);
  }
  if (hbad == 1) return Invalid("offsets must start at 0");
  if (hbad == 2) return Invalid("offsets must be non-decreasing");
  if (weighted && !hnonunit) g.w.Release();  // all-one weights: a unit-weight graph
  PCC_RETURN_IF_ERROR(ComputeGraphProperties(ctx, &g));
  *out = std::move(h);
  return Status::Ok();
}

// ---------------------------------------------------------------------------
// WriteClustering on the device.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t DecimalDigits(uint32_t v) {
  uint32_t d = 1;
  while (v >= 10) {
    v /= 10;
    ++d;
  }
  return d;
}

__global__ void LabelKeysKernel(uint32_t n, const uint32_t* __restrict__ labels, uint64_t* keys, uint32_t* vals,
                                uint32_t* counts) {
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t c = labels[v];
    keys[v] = c;
    vals[v] = static_cast<uint32_t>(v);
    atomicAdd(&counts[c], 1u);
  }
}

// Characters of sorted position k: the id and a tab.
struct IdChars {
  const uint32_t* vals;
  __device__ uint64_t operator()(uint64_t k) const { return DecimalDigits(vals[k]) + 1; }
};

struct CountInput {
  const uint32_t* counts;
  __device__ uint32_t operator()(uint64_t c) const { return counts[c]; }
};
struct StoreInclusive {
  uint32_t* out;
  __device__ void operator()(uint64_t i, uint32_t pre, uint32_t v) const { out[i] = pre + v; }
};

// Member k of the sorted (cluster, id) order starts at S[k] + its cluster
// index (one newline per earlier cluster line, empty lines included).
__global__ void WriteIdsKernel(uint32_t n, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                               const uint64_t* __restrict__ S, char* out) {
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t v = vals[k];
    const uint64_t pos = S[k] + keys[k];
    const uint32_t nd = uint32_t(S[k + 1] - S[k]) - 1;
    for (uint32_t j = nd; j > 0; --j) {
      out[pos + j - 1] = static_cast<char>('0' + v % 10);
      v /= 10;
    }
    out[pos + nd] = '\t';
  }
}

// The newline of cluster c follows its members: S[end of c] + c.
__global__ void WriteNewlinesKernel(uint32_t groups, const uint32_t* __restrict__ cend,
                                    const uint64_t* __restrict__ S, char* out) {
  for (uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < groups;
       c += uint64_t(gridDim.x) * blockDim.x)
    out[S[cend[c]] + c] = '\n';
}

// Formats a clustering given as labels (host array; cluster i is the set of
// vertices labelled i, for i up to the largest label) as the reference's
// clustering file, empty clusters as empty lines; the text is left in *text
// (device).
Status FormatClustering(Context* ctx, uint32_t n, const uint32_t* labels, DBuf<char>* text, uint64_t* length) {
  *length = 0;
  if (n == 0) return Status::Ok();
  uint32_t maxl = 0;
  for (uint32_t v = 0; v < n; ++v) maxl = std::max(maxl, labels[v]);
  if (maxl == 0xFFFFFFFFu) return Invalid("label 2^32 - 1 is reserved");
  const uint32_t groups = maxl + 1;
  DBuf<uint32_t> dl, counts, cend;
  DBuf<uint64_t> keys, S, tiles64;
  DBuf<uint32_t> vals, tiles32;
  PCC_RETURN_IF_ERROR(dl.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(dl.FromHost(labels, n));
  PCC_RETURN_IF_ERROR(keys.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(vals.Alloc(ctx, n));
  PCC_RETURN_IF_ERROR(counts.Alloc(ctx, groups));
  PCC_RETURN_IF_ERROR(cend.Alloc(ctx, groups));
  PCC_RETURN_IF_ERROR(S.Alloc(ctx, uint64_t(n) + 1));
  PCC_RETURN_IF_ERROR(counts.Zero());
  const unsigned grid = Blocks(n, 256, unsigned(ctx->num_sms) * 8);
  LabelKeysKernel<<<grid, 256, 0, ctx->stream>>>(n, dl.p, keys.p, vals.p, counts.p);
  PCC_COUNT(1);
  int bits = 0;
  while (bits < 32 && (uint64_t(maxl) >> bits)) ++bits;
  SortScratch sc;
  // Stable: members stay in ascending id order inside each cluster.
  PCC_RETURN_IF_ERROR(RadixSortPairs(ctx, keys.p, vals.p, n, bits, sc));
  PCC_RETURN_IF_ERROR(ScanApply<uint64_t>(ctx, n, IdChars{vals.p}, StorePrefix<uint64_t>{S.p}, tiles64, S.p + n));
  PCC_RETURN_IF_ERROR(ScanApply<uint32_t>(ctx, groups, CountInput{counts.p}, StoreInclusive{cend.p}, tiles32,
                                          static_cast<uint32_t*>(nullptr)));
  uint64_t chars = 0;
  PCC_CUDA(cudaMemcpyAsync(&chars, S.p + n, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
  PCC_RETURN_IF_ERROR(Sync(ctx));
  const uint64_t len = chars + groups;
  PCC_RETURN_IF_ERROR(text->Alloc(ctx, len));
  WriteIdsKernel<<<grid, 256, 0, ctx->stream>>>(n, keys.p, vals.p, S.p, text->p);
  PCC_COUNT(1);
  WriteNewlinesKernel<<<Blocks(groups, 256, unsigned(ctx->num_sms) * 8), 256, 0, ctx->stream>>>(groups, cend.p, S.p,
                                                                                               text->p);
  PCC_COUNT(1);
  *length = len;
  return LaunchCheck();
}

pcc_status Finish(pcc_context* ctx, const Status& st) {
  if (ctx) ctx->c.last_error = st.ok() ? std::string() : st.msg;
  return st.code;
}

}  // namespace
}  // namespace pcc

using namespace pcc;

extern "C" {

pcc_status pcc_graph_parse_gbbs(pcc_context* ctx, const char* text, uint64_t size, int32_t float_weighted,
                                pcc_graph** out) {
  if (!ctx || !out || (!text && size)) return PCC_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    cudaSetDevice(ctx->c.device);
    std::unique_ptr<pcc_graph> g;
    const Status st = ParseGbbs(&ctx->c, text, size, float_weighted != 0, "graph text", &g);
    if (st.ok()) *out = g.release();
    return Finish(ctx, st);
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_graph_read_gbbs(pcc_context* ctx, const char* path, int32_t float_weighted, pcc_graph** out) {
  if (!ctx || !out || !path) return PCC_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    cudaSetDevice(ctx->c.device);
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f.is_open()) return Finish(ctx, MakeError(PCC_NOT_FOUND, std::string("Unable to open file ") + path));
    const std::streamsize size = f.tellg();
    f.seekg(0);
    // Pinned staging buffer: one DMA to the device.
    char* buf = nullptr;
    if (cudaMallocHost(&buf, size > 0 ? size_t(size) : 1) != cudaSuccess) {
      cudaGetLastError();
      return Finish(ctx, MakeError(PCC_RESOURCE_EXHAUSTED, "pinned staging buffer for the graph file"));
    }
    std::unique_ptr<char, decltype(&cudaFreeHost)> hold(buf, &cudaFreeHost);
    if (size > 0 && !f.read(buf, size)) return Finish(ctx, MakeError(PCC_DATA_LOSS, std::string("read failed: ") + path));
    std::unique_ptr<pcc_graph> g;
    const Status st = ParseGbbs(&ctx->c, buf, uint64_t(size > 0 ? size : 0), float_weighted != 0, path, &g);
    if (st.ok()) {
      const Status ss = Sync(&ctx->c);  // the staging buffer is freed on return
      if (!ss.ok()) return Finish(ctx, ss);
      *out = g.release();
    }
    return Finish(ctx, st);
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_format_clustering(pcc_context* ctx, uint32_t n, const uint32_t* labels, char* out,
                                 uint64_t capacity, uint64_t* length) {
  if (!ctx || !length || (n && !labels)) return PCC_INVALID_ARGUMENT;
  try {
    cudaSetDevice(ctx->c.device);
    DBuf<char> text;
    uint64_t len = 0;
    Status st = FormatClustering(&ctx->c, n, labels, &text, &len);
    if (!st.ok()) return Finish(ctx, st);
    *length = len;
    if (!out) return Finish(ctx, Sync(&ctx->c));
    if (capacity < len)
      return Finish(ctx, MakeError(PCC_RESOURCE_EXHAUSTED, "output buffer holds " + std::to_string(capacity) +
                                                                " bytes, the text needs " + std::to_string(len)));
    if (len) st = text.ToHost(out, len);
    if (st.ok()) st = Sync(&ctx->c);
    return Finish(ctx, st);
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

pcc_status pcc_write_clustering(pcc_context* ctx, const char* path, uint32_t n, const uint32_t* labels) {
  if (!ctx || !path || (n && !labels)) return PCC_INVALID_ARGUMENT;
  try {
    cudaSetDevice(ctx->c.device);
    DBuf<char> text;
    uint64_t len = 0;
    Status st = FormatClustering(&ctx->c, n, labels, &text, &len);
    if (!st.ok()) return Finish(ctx, st);
    std::vector<char> host(len);
    if (len) st = text.ToHost(host.data(), len);
    if (st.ok()) st = Sync(&ctx->c);
    if (!st.ok()) return Finish(ctx, st);
    std::ofstream f(path, std::ios::binary);
    if (!f.is_open()) return Finish(ctx, MakeError(PCC_NOT_FOUND, "Unable to open file."));
    f.write(host.data(), std::streamsize(len));
    return Finish(ctx, f.good() ? Status::Ok() : MakeError(PCC_DATA_LOSS, std::string("write failed: ") + path));
  } catch (const std::exception& e) {
    return Finish(ctx, MakeError(PCC_INTERNAL, e.what()));
  }
}

}  // extern "C"
