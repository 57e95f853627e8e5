// egb_tile.cuh -- candidate-tile machinery shared by the kNN and ball-count
// tile kernels.
//
// A work item is a tile of consecutive query positions of one materialised
// job (JobDev).  Candidates are the same positions; they are staged through
// shared memory in tiles of TILE points per column by cp.async.bulk, double
// buffered, one mbarrier per buffer, every wait bounded.
//
// Candidate schedule:
//   brute force  every tile of the job, in order;
//   slab         the job is sorted by its first column.  First the "home"
//                tiles that hold the item's queries, then alternately the
//                next tile to the right and to the left.  A side closes when,
//                for every query q of the item, fl64(X - q_0) > t_q, where X
//                is the first column of the nearest unvisited point on that
//                side and t_q the query's current threshold (k-th distance,
//                or count radius).  Every unvisited point p on that side has
//                |p_0 - q_0| >= |X - q_0| (sorted order), and the FP64
//                distance is at least fl64(|p_0 - q_0|) (rounding is
//                monotone), so no unvisited point can enter a kNN list or a
//                count.  Thresholds only shrink, so a closed side stays
//                closed.
#pragma once
#include <type_traits>
#include "egb_internal.cuh"
#include "egb_tma.cuh"

namespace egb {

template <bool PLAIN>
using CoordT = typename std::conditional<PLAIN, double, float>::type;

template <int TILE, bool SLAB>
struct TileSched {
  int ntiles, home, h1, nextR, nextL;
  bool doneR, doneL, turnR;

  __device__ __forceinline__ void init(int len, int q0, int qend) {
    ntiles = (len + TILE - 1) / TILE;
    if (SLAB) {
      home = q0 / TILE;
      h1 = (qend - 1) / TILE;
    } else {
      home = 0;
      h1 = ntiles - 1;
    }
    nextR = h1 + 1;
    nextL = home - 1;
    doneR = nextR >= ntiles;
    doneL = nextL < 0;
    turnR = true;
  }
  // Next tile to stage, or -1.  Uniform across the CTA (every thread runs
  // the same sequence of calls with the same done flags).
  __device__ __forceinline__ int next() {
    if (home <= h1) return home++;
    if (!SLAB) return -1;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      if (turnR) {
        turnR = false;
        if (!doneR) {
          const int t = nextR++;
          if (nextR >= ntiles) doneR = true;
          return t;
        }
      } else {
        turnR = true;
        if (!doneL) {
          const int t = nextL--;
          if (nextL < 0) doneL = true;
          return t;
        }
      }
    }
    return -1;
  }
};

// Stage tile `t` of a job into buffer `buf` (thread 0 only).
template <typename T, int TILE>
__device__ __forceinline__ void stage_tile(T* tiles, int DM, int buf, const T* g, int64_t lds,
                                           int d, int len, int t, uint64_t* bar) {
  const int A = t * TILE;
  const int cnt = min(TILE, len - A);
  constexpr int V = 16 / (int)sizeof(T);  // elements per 16 bytes
  const uint32_t bytes = (uint32_t)((cnt + V - 1) / V * V) * (uint32_t)sizeof(T);
  fence_proxy_async_smem();
  mbar_expect_tx(bar, bytes * (uint32_t)d);
#pragma unroll 1
  for (int c = 0; c < d; ++c)
    bulk_g2s(tiles + ((size_t)buf * DM + c) * TILE, g + (int64_t)c * lds + A, bytes, bar);
}

// Number of positions p of a sorted column with |col[p] - v| <= t (within
// rounding; used only to choose a scan order), and the first position with
// col[p] >= v.
__device__ __forceinline__ int lower_bound_d(const double* col, int len, double v) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (col[m] < v) lo = m + 1; else hi = m;
  }
  return lo;
}
__device__ __forceinline__ int upper_bound_d(const double* col, int len, double v) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (col[m] <= v) lo = m + 1; else hi = m;
  }
  return lo;
}

// Scan order for a deferred slab query: its first-column slab or, when the
// job has a second copy sorted by column 1 and that slab is narrower, the
// second.  Returns the arrays to scan, the start position, the sorted
// column's query value and the column index used for termination.
template <typename T>
struct ScanOrder {
  const double* c64;
  const T* g;
  int start;       // first position to the right (inclusive)
  int col;         // sorted column (0 or 1)
  double qs;       // query value in that column
};

template <typename T, bool PLAIN>
__device__ __forceinline__ ScanOrder<T> choose_order(const JobDev* J, int pos, double tb) {
  ScanOrder<T> o;
  o.c64 = J->c64;
  o.g = PLAIN ? reinterpret_cast<const T*>(J->c64) : reinterpret_cast<const T*>(J->c32);
  o.start = pos;
  o.col = 0;
  o.qs = J->c64[pos];
  if (J->c64b == nullptr || J->sp.d < 2 || !(tb < __longlong_as_double((long long)INF_BITS)))
    return o;
  const int len = J->len;
  const double* x = J->c64;
  const double* y = J->c64b + J->lds;  // column 1 of the second copy, sorted
  const double qy = J->c64[J->lds + pos];
  const int w0 = upper_bound_d(x, len, o.qs + tb) - lower_bound_d(x, len, o.qs - tb);
  const int w1 = upper_bound_d(y, len, qy + tb) - lower_bound_d(y, len, qy - tb);
  if (w1 < w0) {
    o.c64 = J->c64b;
    o.g = PLAIN ? reinterpret_cast<const T*>(J->c64b) : reinterpret_cast<const T*>(J->c32b);
    o.start = lower_bound_d(y, len, qy);
    o.col = 1;
    o.qs = qy;
  }
  return o;
}

}  // namespace egb
