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
#endif

}  // namespace egb
