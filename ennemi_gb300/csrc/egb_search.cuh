// egb_search.cuh -- bound searches in a sorted key segment through two
// levels of samples.
//
// A sorted segment keys[0 .. len) carries s1[j] = keys[32 j] and s2[j] =
// keys[1024 j] (launch_samples).  A bound is found level by level: a binary
// search over s2 (a few KB per million keys, resident in L1), then over the
// 32 samples of s1 under that s2 entry (256 bytes), then over the 32 keys
// under that s1 entry (256 bytes).  About a dozen loads per bound, all but
// four or so cache hits, against the 25-30 dependent loads spread over the
// whole range that a gallop from the query's own position takes for the
// ranges of thousands of keys that ball counts cover.
#pragma once
#include <cstdint>

namespace egb {

constexpr int SAMPLE1 = 32;      // keys per s1 sample
constexpr int SAMPLE2 = 1024;    // keys per s2 sample

// sample arrays of a segment of len keys
__host__ __device__ __forceinline__ int64_t samples1_of(int64_t len) {
  return (len + SAMPLE1 - 1) / SAMPLE1;
}
__host__ __device__ __forceinline__ int64_t samples2_of(int64_t len) {
  return (len + SAMPLE2 - 1) / SAMPLE2;
}

#ifdef __CUDACC__
// First index i in [lo, hi) with a[i] > x (upper) or a[i] >= x (lower);
// hi if none.
template <bool UPPER>
__device__ __forceinline__ int first_above(const uint64_t* __restrict__ a, int lo, int hi, uint64_t x) {
  int n = hi - lo;
  while (n > 0) {
    const int h = n >> 1;
    const uint64_t v = __ldg(a + lo + h);
    if (UPPER ? (v <= x) : (v < x)) {
      lo += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return lo;
}

// First position of the segment with key > x (UPPER) or key >= x (lower).
template <bool UPPER>
__device__ __forceinline__ int sampled_bound(const uint64_t* __restrict__ keys,
                                             const uint64_t* __restrict__ s1,
                                             const uint64_t* __restrict__ s2, int len, uint64_t x) {
  const int n2 = (int)samples2_of(len), n1 = (int)samples1_of(len);
  // c2 = number of s2 entries before the bound; the bound lies in
  // (1024 (c2 - 1), 1024 c2]
  const int c2 = first_above<UPPER>(s2, 0, n2, x);
  if (c2 == 0) return 0;
  const int b1 = (c2 - 1) * (SAMPLE2 / SAMPLE1);
  const int c1 = first_above<UPPER>(s1, b1 + 1, min(b1 + SAMPLE2 / SAMPLE1, n1), x);
  const int b0 = (c1 - 1) * SAMPLE1;
  return first_above<UPPER>(keys, b0 + 1, min(b0 + SAMPLE1, len), x);
}

// The same from a position g of the segment near the bound (the query's
// own position): a gallop over s1 from g's sample, then the 32 keys under
// the sample found.  Lanes holding consecutive positions read the same
// sample lines, and no search starts from the top of the segment.
template <bool UPPER>
__device__ __forceinline__ int sampled_bound_from(const uint64_t* __restrict__ keys,
                                                  const uint64_t* __restrict__ s1, int len,
                                                  uint64_t x, int g) {
  const int n1 = (int)samples1_of(len);
  auto before = [&](uint64_t v) { return UPPER ? (v <= x) : (v < x); };  // v precedes the bound
  int j = min(max(g, 0), len - 1) / SAMPLE1;
  int c1;  // first sample index that does not precede the bound (n1 if none)
  if (before(__ldg(s1 + j))) {
    int lo = j, step = 1, hi;  // s1[lo] precedes
    for (;;) {
      const int t = lo + step;
      if (t >= n1) { hi = n1; break; }
      if (!before(__ldg(s1 + t))) { hi = t; break; }
      lo = t;
      step <<= 1;
    }
    c1 = first_above<UPPER>(s1, lo + 1, hi, x);
  } else {
    int hi = j, step = 1, lo;  // s1[hi] does not precede
    for (;;) {
      const int t = hi - step;
      if (t < 0) { lo = -1; break; }
      if (before(__ldg(s1 + t))) { lo = t; break; }
      hi = t;
      step <<= 1;
    }
    c1 = first_above<UPPER>(s1, lo + 1, hi, x);
  }
  if (c1 == 0) return 0;
  const int b0 = (c1 - 1) * SAMPLE1;
  return first_above<UPPER>(keys, b0 + 1, min(b0 + SAMPLE1, len), x);
}

// ---------------------------------------------------- ball as positions --
// Largest float <= the non-negative double with bit pattern u (integer
// operations only; 0 below the normal range, FLT_MAX above it).
__device__ __forceinline__ float f32_down_of_bits(uint64_t u) {
  const int e = (int)(u >> 52);
  if (e >= 1023 + 128) return __int_as_float(0x7f7fffff);
  if (e < 1023 - 126) return 0.0f;
  return __int_as_float((int)(((uint32_t)(e - 1023 + 127) << 23) |
                              (uint32_t)((u & 0xfffffffffffffull) >> 29)));
}
// Floats bounding a double from below and above (integer operations only).
__device__ __forceinline__ float f32_below(double v) {
  const uint64_t u = (uint64_t)__double_as_longlong(v);
  const uint64_t a = u & 0x7fffffffffffffffull;
  return (u >> 63) ? -f32_up_of_bits(a) : f32_down_of_bits(a);
}
__device__ __forceinline__ float f32_above(double v) {
  const uint64_t u = (uint64_t)__double_as_longlong(v);
  const uint64_t a = u & 0x7fffffffffffffffull;
  return (u >> 63) ? -f32_down_of_bits(a) : f32_up_of_bits(a);
}
// Sort key (key_of) of the double equal to a finite float, by integer
// widening: exact, -0 folded into +0.
__device__ __forceinline__ uint64_t key_of_f32(float f) {
  const uint32_t b = (uint32_t)__float_as_int(f);
  const uint64_t s = (uint64_t)(b >> 31) << 63;
  const uint32_t e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  uint64_t d;
  if (e != 0) {
    d = s | ((uint64_t)(e - 127 + 1023) << 52) | ((uint64_t)m << 29);
  } else if (m != 0) {  // subnormal float: a normal double
    const int p = 31 - __clz((int)m);                 // highest set bit, 0 .. 22
    d = s | ((uint64_t)(p - 149 + 1023) << 52) | (((uint64_t)m << (52 - p)) & 0xfffffffffffffull);
  } else {
    d = 0;  // +0 and -0
  }
  return (d >> 63) ? ~d : (d | 0x8000000000000000ull);
}

// Positions [lo, hi) of the sorted keys of a segment whose values x have
// fl64(|x - q|) <= r (q finite, r finite and >= 0): the inclusive ball of
// query_ball_point in one coordinate.
//
// The ends come from FP32 brackets, not from FP64 arithmetic (GB300 issues
// FP64 at a small fraction of its FP32 and integer rates).  With P(x) =
// [fl64(x - q) <= r] (true for small x) and Q(x) = [fl64(q - x) <= r] (true
// for large x), both monotone because rounding is:
//   x <= q + r            => P(x)   (x - q <= r, r representable)
//   x >= q + next_up(r)   => !P(x)  (x - q >= next_up(r) rounds to >= it)
// and symmetrically for Q.  The floats a1 <= q + r, b1 >= q + next_up(r)
// (and b0 >= q - r, a0 <= q - next_up(r)) come from FP32 additions rounded
// down / up on floats bounding q and r.  Every key below key(a1) satisfies
// P, every key above key(b1) fails it; the few keys between -- usually
// none -- are decided by the exact FP64 predicate.  A bracket that is not
// finite or holds more than BALL_SCAN keys (values far outside the FP32
// range, or all crowded into a few FP32 ulps) takes the exact FP64 search
// of ball_keys instead.
constexpr int BALL_SCAN = 16;
// g: the query's own position in the segment (where q sits), the start of
// galloping bound searches (measured faster for the 1-D counts, whose warps
// hold consecutive positions), or -1: searches from the top of the samples.
__device__ __forceinline__ void ball_positions(const uint64_t* __restrict__ keys,
                                               const uint64_t* __restrict__ s1,
                                               const uint64_t* __restrict__ s2, int len, double q,
                                               double r, int g, int& lo, int& hi) {
  const float qd = f32_below(q), qu = f32_above(q), rd = f32_below(r), ru = f32_above(r);
  const float rn = __int_as_float(__float_as_int(ru) + 1);   // next float above ru (ru >= 0)
  const float a1 = __fadd_rd(qd, rd), b1 = __fadd_ru(qu, rn);
  const float a0 = __fsub_rd(qd, rn), b0 = __fsub_ru(qu, rd);
  bool exact = isfinite(a1) && isfinite(b1) && isfinite(a0) && isfinite(b0) && isfinite(q);
  if (exact) {
    const uint64_t ka1 = key_of_f32(a1), kb1 = key_of_f32(b1);
    int p = g >= 0 ? sampled_bound_from<false>(keys, s1, len, ka1, g)
                   : sampled_bound<false>(keys, s1, s2, len, ka1);
    int n = 0;
    for (; p < len; ++p, ++n) {
      const uint64_t k = __ldg(keys + p);
      if (k > kb1 || n == BALL_SCAN || !(value_of(k) - q <= r)) break;
    }
    hi = p;
    exact = n < BALL_SCAN;
  }
  if (exact) {
    const uint64_t ka0 = key_of_f32(a0), kb0 = key_of_f32(b0);
    int p = g >= 0 ? sampled_bound_from<true>(keys, s1, len, kb0, g)
                   : sampled_bound<true>(keys, s1, s2, len, kb0);
    int n = 0;
    for (; p > 0; --p, ++n) {
      const uint64_t k = __ldg(keys + p - 1);
      if (k < ka0 || n == BALL_SCAN || !(q - value_of(k) <= r)) break;
    }
    lo = p;
    exact = n < BALL_SCAN;
  }
  if (!exact) {  // the exact key range, then its positions
    uint64_t kl, kr;
    ball_keys(q, r, kl, kr);
    kl = kl == 0x7fffffffffffffffull ? 0x8000000000000000ull : kl;  // raw -0 -> +0
    lo = sampled_bound<false>(keys, s1, s2, len, kl);
    hi = sampled_bound<true>(keys, s1, s2, len, kr);
  }
}
#endif

}  // namespace egb
