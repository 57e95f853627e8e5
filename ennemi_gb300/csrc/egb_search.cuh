// egb_search.cuh -- bound searches in a sorted key segment through two
// levels of samples.
//
// A sorted segment keys[0 .. len) carries s1[j] = keys[32 j] and s2[j] =
// keys[1024 j] (launch_samples), and the same of its FP32 copy (each value
// rounded down).  A bound is found level by level: a binary search over s2
// (a few KB per million keys, resident in L1), then over the 32 samples of
// s1 under that s2 entry, then over the 32 keys under that s1 entry.  About
// a dozen loads per bound, all but four or so cache hits, against the 25-30
// dependent loads spread over the whole range that a gallop from the query's
// own position takes for the ranges of thousands of keys that ball counts
// cover.  The FP32 copy halves the bytes of each level.
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
// One sorted segment of a KeyIndex.
struct SegView {
  const uint64_t* keys;
  const float* fk;
  const uint64_t* s1;
  const uint64_t* s2;
  const float* fs1;
  const float* fs2;
  int len;
};
__device__ __forceinline__ SegView seg_view(const KeyIndex& I, int64_t base, int64_t s1b,
                                            int64_t s2b, int len) {
  return SegView{I.keys + base, I.fkeys + base, I.s1 + s1b, I.s2 + s2b, I.fs1 + s1b, I.fs2 + s2b, len};
}

// First index i in [lo, hi) with a[i] > x (UPPER) or a[i] >= x (lower);
// hi if none.
template <typename T, bool UPPER>
__device__ __forceinline__ int first_above(const T* __restrict__ a, int lo, int hi, T x) {
  int n = hi - lo;
  while (n > 0) {
    const int h = n >> 1;
    const T v = __ldg(a + lo + h);
    if (UPPER ? (v <= x) : (v < x)) {
      lo += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return lo;
}

// First position of a sorted array with element > x (UPPER) or >= x
// (lower), through its two levels of samples: the bound lies under the first
// s2 entry past it, then under the first s1 entry past it.
template <typename T, bool UPPER>
__device__ __forceinline__ int sampled_bound(const T* __restrict__ keys, const T* __restrict__ s1,
                                             const T* __restrict__ s2, int len, T x) {
  const int n2 = (int)samples2_of(len), n1 = (int)samples1_of(len);
  const int c2 = first_above<T, UPPER>(s2, 0, n2, x);
  if (c2 == 0) return 0;
  const int b1 = (c2 - 1) * (SAMPLE2 / SAMPLE1);
  const int c1 = first_above<T, UPPER>(s1, b1 + 1, min(b1 + SAMPLE2 / SAMPLE1, n1), x);
  const int b0 = (c1 - 1) * SAMPLE1;
  return first_above<T, UPPER>(keys, b0 + 1, min(b0 + SAMPLE1, len), x);
}

// The same from a position g near the bound (the query's own position): a
// gallop over s1 from g's sample, then the 32 elements under the sample
// found.  Lanes holding consecutive positions read the same sample lines.
template <typename T, bool UPPER>
__device__ __forceinline__ int sampled_bound_from(const T* __restrict__ keys,
                                                  const T* __restrict__ s1, int len, T x, int g) {
  const int n1 = (int)samples1_of(len);
  auto before = [&](T v) { return UPPER ? (v <= x) : (v < x); };  // v precedes the bound
  const int j = min(max(g, 0), len - 1) / SAMPLE1;
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
    c1 = first_above<T, UPPER>(s1, lo + 1, hi, x);
  } else {
    int hi = j, step = 1, lo;  // s1[hi] does not precede
    for (;;) {
      const int t = hi - step;
      if (t < 0) { lo = -1; break; }
      if (before(__ldg(s1 + t))) { lo = t; break; }
      hi = t;
      step <<= 1;
    }
    c1 = first_above<T, UPPER>(s1, lo + 1, hi, x);
  }
  if (c1 == 0) return 0;
  const int b0 = (c1 - 1) * SAMPLE1;
  return first_above<T, UPPER>(keys, b0 + 1, min(b0 + SAMPLE1, len), x);
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
// Positions [lo, hi) of the sorted values x of a segment with
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
// down / up on floats bounding q and r.  For a float a, x >= a exactly when
// the largest float <= x is >= a, so the searches run on the FP32 copy of
// the keys: every value below a1 satisfies P, every value above b1 fails it,
// and the few between -- usually none -- are decided by the exact FP64
// predicate on the 8-byte keys (the left end alike with Q, a0, b0).  A
// bracket that is not finite or holds more than BALL_SCAN values (values far
// outside the FP32 range, or all crowded into a few FP32 ulps) takes the
// exact FP64 search of ball_keys on the 8-byte keys instead.
//
// g: the query's own position in the segment, the start of galloping
// searches (measured faster for the 1-D counts, whose warps hold
// consecutive positions), or -1: searches from the top of the samples.
constexpr int BALL_SCAN = 16;
__device__ __forceinline__ void ball_positions(const SegView& v, double q, double r, int g, int& lo,
                                               int& hi) {
  const int len = v.len;
  const uint64_t rb = (uint64_t)__double_as_longlong(r) & 0x7fffffffffffffffull;  // -0 as +0
  const float qd = f32_below(q), qu = f32_above(q);
  const float rd = f32_down_of_bits(rb), ru = f32_up_of_bits(rb);  // ru >= 2^-126
  const float rn = __int_as_float(__float_as_int(ru) + 1);         // next float above ru
  const float a1 = __fadd_rd(qd, rd), b1 = __fadd_ru(qu, rn);
  const float a0 = __fsub_rd(qd, rn), b0 = __fsub_ru(qu, rd);
  const uint64_t qb = (uint64_t)__double_as_longlong(q);
  bool exact = isfinite(a1) && isfinite(b1) && isfinite(a0) && isfinite(b0) &&
               ((qb >> 52) & 0x7ffu) != 0x7ffu;  // q finite, by its exponent bits
  auto fbound = [&](float a) {  // first position whose value is >= a
    return g >= 0 ? sampled_bound_from<float, false>(v.fk, v.fs1, len, a, g)
                  : sampled_bound<float, false>(v.fk, v.fs1, v.fs2, len, a);
  };
  if (exact) {  // right end: the first value failing P
    int p = fbound(a1), n = 0;
    for (; p < len; ++p, ++n) {
      if (__ldg(v.fk + p) > b1 || n == BALL_SCAN) break;  // value > b1: fails P
      if (!(value_of(__ldg(v.keys + p)) - q <= r)) break;
    }
    hi = p;
    exact = n < BALL_SCAN;
  }
  if (exact) {  // left end: the first value satisfying Q
    int p = fbound(a0), n = 0;
    for (; p < len; ++p, ++n) {
      if (__ldg(v.fk + p) > b0 || n == BALL_SCAN) break;  // value > b0: satisfies Q
      if (q - value_of(__ldg(v.keys + p)) <= r) break;
    }
    lo = p;
    exact = n < BALL_SCAN;
  }
  if (!exact) {  // the exact key range, then its positions
    uint64_t kl, kr;
    ball_keys(q, r, kl, kr);
    kl = kl == 0x7fffffffffffffffull ? 0x8000000000000000ull : kl;  // raw -0 -> +0
    lo = sampled_bound<uint64_t, false>(v.keys, v.s1, v.s2, len, kl);
    hi = sampled_bound<uint64_t, true>(v.keys, v.s1, v.s2, len, kr);
  }
}
#endif

}  // namespace egb
