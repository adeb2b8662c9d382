// certify.cuh -- FP32 certification of the synchronous best-move decision
// (INT mode).  GB300 runs FP64 at ~1/64 of FP32 and an FP64 warp
// instruction costs ~19 SM cycles however few lanes are active, so the
// per-vertex FP64 of EfficientBestMove (parallel-correlation-clusterer-
// internal.cc:483-512) and of the sync decision (parallel-correlation-
// clusterer.cc:139-157) dominates a naive kernel.  Here the decision is
// taken from FP32 approximations with rigorous error bounds when they
// determine it, and from the exact FP64 values otherwise.
//
// Reference quantities (FP64, every operation separately rounded):
//   X_D    = S_D - res * (kv * K_D)          val_D = change + X_D
//   change = 0 - (T - res * (kv * (K_c - kv)))
// with S_D, T exact integers (INT mode).  The reference moves v to
// argmax_D val_D (ties: lowest D) if that value exceeds change, else to a new
// cluster with value change; then the singleton rule, then "move iff value
// > 0".
//
// Certification, u = 2^-24 (FP32 unit roundoff):
//   * the winner: the FP32 pre-filter keeps every D that can be the FP64
//     argmax; if all survivors share one (S, K) pair, their FP64 values are
//     equal and the winner is the lowest id (no FP64 needed);
//   * X' = fl32(S) - fl32(r32 * fl32(k32 * Kf_D)) is within
//     eX = 2^-21 |R'| + 2^-23 |X'| + [|S| > 2^24] 2^-23 |S| + 2^-48 (...)
//     of the FP64 X_D (five relative roundings of u in R', one in the
//     subtraction, the conversion of S, and the reference's own FP64
//     roundings), each bound doubled for margin;
//   * change' = -(fl32(T) - M'), M' = r32 * (k32 * (Kc32 - k32)): the
//     difference K_c - kv is exact in FP32 when both are integers below 2^24
//     (integer node weights), otherwise it carries 2^-23 of each operand;
//     that error is scaled by |r32 k32|, plus 2^-21 |M'| for the products;
//   * the decision: X_D > 2^-50 |change| (so change + X_D > change in FP64)
//     -> target D, value sign from (S_D - T) + (M' - R'), the integer part
//     exact; X_D <= 0 -> new cluster, value change; anything the bounds do
//     not separate -> FP64.
// Inputs that are zero, infinite, NaN or outside [2^-100, 2^100] in FP32
// make the vertex uncertain (the relative-error model needs normal floats).
#pragma once

#include "moves.cuh"

namespace pcc {
namespace {

constexpr float kU21 = 4.76837158203125e-07f;   // 2^-21
constexpr float kU23 = 1.1920928955078125e-07f; // 2^-23
constexpr float kU48 = 3.552713678800501e-15f;  // 2^-48
constexpr float kU50 = 8.881784197001252e-16f;  // 2^-50
constexpr float kTwo24 = 16777216.0f;

// Integer -> float.  The kernels keep sums in int when they are narrow
// (every sum and difference below 2^31 in magnitude) and convert them with
// integer and FP32 arithmetic only: conversion instructions run on this
// GPU's slow double-precision path.  For |y| < 2^22 the float with bit
// pattern 0x4B400000 + y is exactly 1.5 * 2^23 + y (the ulp there is 1), so
// subtracting 1.5 * 2^23 gives y exactly.  x = hi * 2^16 + lo with both
// halves in that range; hi * 2^16 is exact and the final addition rounds
// once, so the result is x correctly rounded, like __int2float_rn.
__device__ __forceinline__ float SmallIntToFloat(int y) {
  return __fsub_rn(__int_as_float(0x4B400000 + y), 12582912.0f);
}
__device__ __forceinline__ float I2F(int x) {
  const float fh = SmallIntToFloat(x >> 16);
  const float fl = SmallIntToFloat(x & 0xFFFF);
  return __fadd_rn(__fmul_rn(fh, 65536.0f), fl);
}
__device__ __forceinline__ float I2F(long long x) { return __ll2float_rn(x); }

__device__ __forceinline__ bool SaneF(float z) {
  const float m = fabsf(z);
  return z == 0.0f || (m >= 7.888609052210118e-31f /* 2^-100 */ && m <= 1.2676506002282294e30f /* 2^100 */);
}

// Order-preserving integer image of a double (integer instructions only);
// -0 and +0 map to one value.
__device__ __forceinline__ unsigned long long KOrder(double d) {
  unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// (S desc, K asc, id asc) lexicographic leader of the filter's survivors;
// id kNone = none.
template <typename I>
struct LexKeyT {
  I S = sizeof(I) == 4 ? I(INT_MIN) : I(LLONG_MIN);
  unsigned long long K = ~0ull;
  uint32_t id = kNone;
  __device__ __forceinline__ void Keep(I s, unsigned long long k, uint32_t i) {
    if (i == kNone) return;
    if (id == kNone || s > S || (s == S && (k < K || (k == K && i < id)))) {
      S = s;
      K = k;
      id = i;
    }
  }
};

// Butterfly over lane groups of G lanes (G = 32: the warp).
using LexKey = LexKeyT<long long>;

template <int G, typename I>
__device__ __forceinline__ void LexGroupReduce(LexKeyT<I>& x) {
#pragma unroll
  for (int o = G / 2; o >= 1; o >>= 1) {
    const I s = __shfl_xor_sync(kFull, x.S, o);
    const unsigned long long k = __shfl_xor_sync(kFull, x.K, o);
    const uint32_t i = __shfl_xor_sync(kFull, x.id, o);
    x.Keep(s, k, i);
  }
}

// Warp-wide form of LexGroupReduce<32> for 32-bit sums, by single-
// instruction warp reductions (REDUX) instead of a shuffle butterfly: the
// leader's S is the largest S, then the smallest K among those (high word,
// then low word), then the lowest id.
__device__ __forceinline__ void LexWarpLeaderInt(LexKeyT<int>& lead) {
  const bool has = lead.id != kNone;
  const int sm = __reduce_max_sync(kFull, has ? lead.S : INT_MIN);
  const bool m1 = has && lead.S == sm;
  const unsigned hi = static_cast<unsigned>(lead.K >> 32), lo = static_cast<unsigned>(lead.K);
  const unsigned khi = __reduce_min_sync(kFull, m1 ? hi : 0xFFFFFFFFu);
  const bool m2 = m1 && hi == khi;
  const unsigned klo = __reduce_min_sync(kFull, m2 ? lo : 0xFFFFFFFFu);
  const bool m3 = m2 && lo == klo;
  const unsigned id = __reduce_min_sync(kFull, m3 ? lead.id : kNone);
  if (id == kNone) {
    lead = LexKeyT<int>{};
    return;
  }
  lead.S = sm;
  lead.K = (static_cast<unsigned long long>(khi) << 32) | klo;
  lead.id = id;
}

// The warp leader, and whether every lane's trailing contender (`tail`,
// kept with (-S, ~K)) lies in the leader's (S, K) class, i.e. the test the
// butterfly over `tail` decided.
__device__ __forceinline__ bool LexWarpLeadInt(LexKeyT<int>& lead, const LexKeyT<int>& tail) {
  LexWarpLeaderInt(lead);
  if (lead.id == kNone) return true;
  const bool diff = tail.id != kNone && (-tail.S != lead.S || ~tail.K != lead.K);
  return !__any_sync(kFull, diff);
}

// Warp maximum of finite floats (or -inf) by one integer REDUX: the map
// i -> i ^ 0x7FFFFFFF on negative bit patterns orders floats as signed ints
// and is its own inverse.
__device__ __forceinline__ float WarpMaxFinite(float x) {
  int i = __float_as_int(x);
  i = i >= 0 ? i : (i ^ 0x7FFFFFFF);
  i = __reduce_max_sync(kFull, i);
  return __int_as_float(i >= 0 ? i : (i ^ 0x7FFFFFFF));
}

// FP32 filter value of a candidate (FilterBound): Y' = fl32(S - Smax) - R'
// and its bound e; the shift keeps the top-S candidates apart by R alone.
// (An S - Smax above 2^24 adds at most u (|Y| + R), inside FilterBound's
// 2^-21 (R + |Y|) model.)  sane = false when the inputs leave the
// relative-error model; such candidates are always kept.
struct FilterVal {
  float Y, e;
  bool sane;
};

template <typename I>
__device__ __forceinline__ FilterVal FilterOf(float r32, float k32, float KfD, I S, I Smax, float change32) {
  FilterVal f;
  const float R = __fmul_rn(r32, __fmul_rn(k32, KfD));
  f.Y = __fsub_rn(I2F(S - Smax), R);
  f.e = FilterBound(R, f.Y, I2F(S), change32);
  f.sane = SaneF(R) && SaneF(KfD) && isfinite(f.Y) && isfinite(f.e);
  return f;
}

// Running top two of the candidates' upper ends (Y + e), with the index of
// the largest.  A pre-filter pass keeps them so that its second pass can
// skip re-evaluating a thread's candidates when the runner-up is below the
// pass's U: then at most the largest can be a contender.
__device__ __forceinline__ void KeepTop2(float& hi1, float& hi2, uint32_t& i1, float hi, uint32_t i) {
  if (hi > hi1) {
    hi2 = hi1;
    hi1 = hi;
    i1 = i;
  } else if (hi > hi2) {
    hi2 = hi;
  }
}

// Result of the certification: kUncertain = take the FP64 path.
enum CertResult : int { kCertNoMove = 0, kCertMove = 1, kUncertain = 2 };

// FP32 approximation of change = 0 - (T - res*(kv*(K_c - kv))) and its
// bound; ok = false when the inputs leave the relative-error model.
template <typename I>
struct ChangeApproxT {
  float ch, ec;  // change' and its bound
  float M, eM;   // res*kv*(K_c - kv) in FP32 and its bound
  I T;
  bool ok;
};

template <typename I>
__device__ __forceinline__ ChangeApproxT<I> ApproxChange(float r32, bool int_nw, float k32, float Kc32, I T) {
  ChangeApproxT<I> c;
  const float diff = __fsub_rn(Kc32, k32);
  const bool kc_exact = int_nw && fabsf(Kc32) < kTwo24;
  const bool kv_exact = int_nw && fabsf(k32) < kTwo24;
  const float ed = __fadd_rn(__fadd_rn(kc_exact ? 0.0f : __fmul_rn(kU23, fabsf(Kc32)),
                                       kv_exact ? 0.0f : __fmul_rn(kU23, fabsf(k32))),
                             __fmul_rn(kU23, fabsf(diff)));
  const float rk = __fmul_rn(fabsf(r32), fabsf(k32));
  const float M = __fmul_rn(r32, __fmul_rn(k32, diff));
  const float eM = __fadd_rn(__fmul_rn(__fmul_rn(rk, ed), 1.0001f), __fmul_rn(kU21, fabsf(M)));
  const float T32 = I2F(T);
  const float eT = fabsf(T32) > kTwo24 ? __fmul_rn(kU23, fabsf(T32)) : 0.0f;
  c.M = M;
  c.eM = eM;
  c.T = T;
  c.ch = -__fsub_rn(T32, M);
  c.ec = __fadd_rn(__fadd_rn(__fadd_rn(eM, eT), __fmul_rn(kU23, fabsf(c.ch))),
                   __fmul_rn(kU48, __fadd_rn(fabsf(T32), fabsf(M))));
  c.ok = SaneF(r32) && SaneF(k32) && SaneF(Kc32) && SaneF(M) && SaneF(c.ch) && isfinite(c.ec) && isfinite(ed);
  return c;
}

// An upper bound of |change| for FilterBound's absolute term (inf when the
// approximation is not usable, which keeps every candidate).
template <typename I>
__device__ __forceinline__ float ChangeAbsBound(const ChangeApproxT<I>& c) {
  return c.ok ? __fmul_rn(__fadd_rn(fabsf(c.ch), c.ec), 1.0001f) : CUDART_INF_F;
}

// Certifies the decision given the single-class winner A (has_cand) or no
// candidate at all.  *target receives the target (n = new cluster) when the
// result is kCertMove.
template <typename I>
__device__ __forceinline__ int CertifyDecision(const ChangeApproxT<I>& c, float r32, float k32, bool has_cand,
                                               I SA, float KfA, uint32_t idA, uint32_t n, uint32_t* target) {
  if (!c.ok) return kUncertain;
  if (has_cand) {
    const float RA = __fmul_rn(r32, __fmul_rn(k32, KfA));
    const float SA32 = I2F(SA);
    const float X = __fsub_rn(SA32, RA);
    float eX = __fadd_rn(__fmul_rn(kU21, fabsf(RA)), __fmul_rn(kU23, fabsf(X)));
    if (fabsf(SA32) > kTwo24) eX = __fadd_rn(eX, __fmul_rn(kU23, fabsf(SA32)));
    eX = __fadd_rn(eX, __fmul_rn(kU48, __fadd_rn(__fadd_rn(fabsf(RA), fabsf(X)), fabsf(SA32))));
    if (!(SaneF(KfA) && SaneF(RA) && SaneF(X) && isfinite(eX))) return kUncertain;
    if (__fsub_rn(X, eX) > __fmul_rn(kU50, __fadd_rn(fabsf(c.ch), c.ec))) {
      // val_A = fl(change + X_A) > change: target A, value val_A, whose sign
      // is that of (S_A - T) + (M - R_A): the integer part is exact, so the
      // bound carries only the FP32 error of M and R_A (a vertex tied
      // between its own cluster and A has S_A = T and a tiny value).
      const I dI = SA - c.T;
      const float I32 = I2F(dI);
      const float mr = __fsub_rn(c.M, RA);
      const float vs = __fadd_rn(I32, mr);
      float ev = __fadd_rn(__fadd_rn(c.eM, __fmul_rn(kU21, fabsf(RA))),
                           __fmul_rn(kU23, __fadd_rn(fabsf(mr), fabsf(vs))));
      if (fabsf(I32) > kTwo24) ev = __fadd_rn(ev, __fmul_rn(kU23, fabsf(I32)));
      ev = __fadd_rn(ev, __fmul_rn(kU48, __fadd_rn(__fadd_rn(fabsf(I2F(c.T)), fabsf(SA32)),
                                                    __fadd_rn(fabsf(c.M), fabsf(RA)))));
      *target = idA;
      if (!isfinite(ev)) return kUncertain;
      if (__fsub_rn(vs, ev) > 0.0f) return kCertMove;
      if (__fadd_rn(vs, ev) < 0.0f) return kCertNoMove;
      return kUncertain;
    }
    if (!(__fadd_rn(X, eX) <= 0.0f)) return kUncertain;
    // X_A <= 0: change >= val_A, the new cluster.
  }
  *target = n;
  if (__fsub_rn(c.ch, c.ec) > 0.0f) return kCertMove;
  if (__fadd_rn(c.ch, c.ec) <= 0.0f) return kCertNoMove;
  return kUncertain;
}

// The move the sync decision makes for a certified (target, value > 0?):
// the singleton rule, then kNone unless the value is positive.
__device__ __forceinline__ uint32_t CertifiedMove(const BMArgs& a, const VertexCtx& x, uint32_t target,
                                                  bool positive) {
  if (target < a.n && a.s[target] == 1u && a.s[x.c] == 1u && x.c >= target) return kNone;
  return positive ? target : kNone;
}

// Effects of a certified sync decision (moved flag, mover list): returns
// true when the vertex must be appended to the movers list.
__device__ __forceinline__ bool ApplyCertified(const BMArgs& a, const VertexCtx& x, uint32_t move) {
  if (move == kNone) return false;
  a.moved_stamp[x.v] = StampIn(a.rs, a.stamp);
  if (move == x.c) return false;
  a.moves[x.v] = move;
  return true;
}

}  // namespace
}  // namespace pcc
