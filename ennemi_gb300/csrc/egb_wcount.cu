// egb_wcount.cu -- ball counts of d = 2, 3 and 4 warp-grid jobs by key
// ranges: integer comparisons only, no distance arithmetic.
//
// The count of query q is #{j : max_c fl64(|p_jc - q_c|) <= r}, r =
// fl64(eps_q - 1e-12) (query_ball_point with p=inf and return_length=True,
// ennemi/_entropy_estimators.py:109-110, :152-154).  Per coordinate,
// x -> fl64(x - q_c) is monotone, so {x : fl64(|x - q_c|) <= r} is one range
// of doubles, and -- mapping doubles to order-preserving integer keys -- one
// key range [kl_c, kr_c] whose ends ball_keys() finds with a few exact FP64
// steps per query.  The ball is then the box of those key ranges, exactly.
//
// Layout: the job's grid copy (strips by column 1, nested cells by column 2
// for d >= 3, column-0 order inside), holding the keys themselves as high and
// low 32-bit words (JobDev::kform): most comparisons are settled by the high
// words, and the low word is read only on a tie.  A warp takes an item of up to 32
// queries of one strip (cell) and visits the strips outward from its own
// while some lane's column-1 key range reaches them; in a nested grid, the
// cells of each strip whose column-2 range meets some lane's.  In each strip
// (cell) every lane finds its own column-0 key range by galloping from a
// guess -- its own position at home, the same relative positions elsewhere --
// and bisecting.  A strip (cell) whose column-1 (and column-2) bounds
// lie inside the lane's ball adds the length of that range; otherwise the
// lane checks the column-1 (column-2) keys of the candidates in its range.
#include "egb_internal.cuh"

namespace egb {
namespace {

constexpr int WC_WARPS = 4;

// One key column of the grid copy: high words, then low words.
struct KeyCol {
  const uint32_t* __restrict__ hi;
  const uint32_t* __restrict__ lo;
  __device__ __forceinline__ uint64_t key(int p) const {
    return ((uint64_t)hi[p] << 32) | lo[p];
  }
  __device__ __forceinline__ bool lt(int p, uint64_t k) const {  // key(p) < k
    const uint32_t h = hi[p], kh = (uint32_t)(k >> 32);
    return h < kh || (h == kh && lo[p] < (uint32_t)k);
  }
  __device__ __forceinline__ bool le(int p, uint64_t k) const {  // key(p) <= k
    const uint32_t h = hi[p], kh = (uint32_t)(k >> 32);
    return h < kh || (h == kh && lo[p] <= (uint32_t)k);
  }
  // key(p) in [a, b]
  __device__ __forceinline__ bool in(int p, uint64_t a, uint64_t b) const {
    const uint32_t h = hi[p], ah = (uint32_t)(a >> 32), bh = (uint32_t)(b >> 32);
    if (h > ah && h < bh) return true;
    if (h < ah || h > bh) return false;
    const uint64_t k = ((uint64_t)h << 32) | lo[p];
    return k >= a && k <= b;
  }
};

// 1 if position p, whose high word w equals that of a or b, has its key in [a, b]
__device__ __forceinline__ int tied_in(const KeyCol& c, uint32_t w, int p, uint64_t a, uint64_t b) {
  if (w != (uint32_t)(a >> 32) && w != (uint32_t)(b >> 32)) return 0;
  const uint64_t k = ((uint64_t)w << 32) | c.lo[p];
  return (k >= a && k <= b) ? 1 : 0;
}

// #{p in [pl, ph) : key(p) in [a, b]}, four high words per 16-byte load
// (the key columns start 128-byte aligned: lds is a multiple of 32); a
// high word strictly between those of a and b settles the point, one equal
// to either is settled by the full key.
__device__ __forceinline__ int count_in(const KeyCol& c, int pl, int ph, uint64_t a, uint64_t b) {
  const uint32_t ah = (uint32_t)(a >> 32), bh = (uint32_t)(b >> 32);
  int cnt = 0;
  int p = pl;
  for (; p < ph && (p & 3); ++p) cnt += c.in(p, a, b) ? 1 : 0;
  for (; p + 4 <= ph; p += 4) {
    const uint4 h = *reinterpret_cast<const uint4*>(c.hi + p);
    cnt += (h.x > ah && h.x < bh) + (h.y > ah && h.y < bh) + (h.z > ah && h.z < bh) +
           (h.w > ah && h.w < bh);
    const bool tie = h.x == ah || h.x == bh || h.y == ah || h.y == bh || h.z == ah ||
                     h.z == bh || h.w == ah || h.w == bh;
    if (tie) cnt += tied_in(c, h.x, p, a, b) + tied_in(c, h.y, p + 1, a, b) +
                    tied_in(c, h.z, p + 2, a, b) + tied_in(c, h.w, p + 3, a, b);
  }
  for (; p < ph; ++p) cnt += c.in(p, a, b) ? 1 : 0;
  return cnt;
}

__device__ __forceinline__ uint64_t rkey(uint64_t u) { return raw_key(u); }

__device__ __forceinline__ uint64_t wmin64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}
__device__ __forceinline__ uint64_t wmax64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// First position of [a, b) with key >= k (keys sorted).
__device__ __forceinline__ int lower_key(const KeyCol& x, int a, int b, uint64_t k) {
  int n = b - a;
  while (n > 0) {
    const int h = n >> 1;
    if (x.lt(a + h, k)) {
      a += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return a;
}
// First position of [a, b) with key > k.
__device__ __forceinline__ int upper_key(const KeyCol& x, int a, int b, uint64_t k) {
  int n = b - a;
  while (n > 0) {
    const int h = n >> 1;
    if (x.le(a + h, k)) {
      a += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return a;
}

// First position of [a, b) with key >= k (lt = false) or > k (lt = true:
// first key not <= k), from a guessed position g: gallop towards the
// answer, then bisect (exact for any g).
__device__ __forceinline__ int bound_from(const KeyCol& x, int a, int b, uint64_t k, bool upper,
                                          int g) {
  if (b <= a) return a;
  g = g < a ? a : (g >= b ? b - 1 : g);
  auto before = [&](int p) { return upper ? x.le(p, k) : x.lt(p, k); };  // p precedes the bound
  int lo, hi;
  if (before(g)) {
    lo = g + 1;
    int step = 1;
    for (;;) {
      const int t = g + step;
      if (t >= b) { hi = b; break; }
      if (!before(t)) { hi = t; break; }
      lo = t + 1;
      step <<= 1;
    }
  } else {
    hi = g;
    int step = 1;
    for (;;) {
      const int t = g - step;
      if (t < a) { lo = a; break; }
      if (before(t)) { lo = t + 1; break; }
      hi = t;
      step <<= 1;
    }
  }
  return upper ? upper_key(x, lo, hi, k) : lower_key(x, lo, hi, k);
}

template <int D>
__global__ void __launch_bounds__(WC_WARPS * 32)
wcount_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items, int nitems,
              int* __restrict__ counter) {
  static_assert(D >= 2 && D <= 4, "d = 2 strips, d = 3 and 4 nested cells");
  constexpr bool NEST = D >= 3;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const WorkItem wi = items[it];
    const JobDev* __restrict__ J = jobs + wi.job;
    const int len = J->len;
    const int64_t lds = J->lds;
    const uint32_t* kw = reinterpret_cast<const uint32_t*>(J->c64g);
    const KeyCol xk{kw, kw + lds}, yk{kw + 2 * lds, kw + 3 * lds};
    const KeyCol zk{kw + 4 * lds, kw + 5 * lds};  // d >= 3
    const KeyCol wk{kw + 6 * lds, kw + 7 * lds};  // d = 4
    const int32_t* __restrict__ sst = J->sstart;
    const unsigned long long* __restrict__ sylo = reinterpret_cast<const unsigned long long*>(J->sylo);
    const unsigned long long* __restrict__ syhi = reinterpret_cast<const unsigned long long*>(J->syhi);
    const int S = J->nstrips;
    const int S2 = NEST ? J->nsub : 1;
    const int32_t* __restrict__ cst = J->cstart;
    const unsigned long long* __restrict__ czlo = reinterpret_cast<const unsigned long long*>(J->czlo);
    const unsigned long long* __restrict__ czhi = reinterpret_cast<const unsigned long long*>(J->czhi);

    const int qp = wi.q0 + lane;
    const bool exists = qp < wi.q1;
    const double qr = exists ? J->rad[J->idxg[qp]] : -1.0;
    const bool qok = exists && qr >= 0.0;
    const bool every = qok && isinf(qr);  // an infinite radius holds every point
    uint64_t kxl = 1, kxr = 0, kyl = 1, kyr = 0, kzl = 1, kzr = 0, kwl = 1, kwr = 0;  // empty
    const bool act = qok && !every;
    if (act) {
      ball_keys(raw_value(xk.key(qp)), qr, kxl, kxr);
      ball_keys(raw_value(yk.key(qp)), qr, kyl, kyr);
      if (D >= 3) ball_keys(raw_value(zk.key(qp)), qr, kzl, kzr);
      if (D == 4) ball_keys(raw_value(wk.key(qp)), qr, kwl, kwr);
    }
    int cnt = every ? len : 0;
    unsigned long long checked = 0;

    // Count this lane's ball in the positions [a, b) of one strip or cell.
    // In its own strip (cell) the lane searches its column-0 range from its
    // own position; elsewhere from the same relative positions, which the
    // equal-count layout makes close guesses.
    const int sq = NEST ? (wi.strip & 0xffff) : wi.strip;
    const int hc2 = NEST ? (wi.strip >> 16) : 0;
    float frl = 0.0f, frh = 0.0f;
    auto count_range = [&](int a, int b, bool inner, bool reach, bool home) {
      if (!reach) return;
      int pl, ph;
      if (home) {
        pl = bound_from(xk, a, b, kxl, false, qp);
        ph = bound_from(xk, pl, b, kxr, true, qp);
        frl = b > a ? (float)(pl - a) / (float)(b - a) : 0.0f;
        frh = b > a ? (float)(ph - a) / (float)(b - a) : 0.0f;
      } else {
        pl = bound_from(xk, a, b, kxl, false, a + (int)(frl * (float)(b - a)));
        ph = bound_from(xk, pl, b, kxr, true, a + (int)(frh * (float)(b - a)));
      }
      if (inner) {
        cnt += ph - pl;
        return;
      }
      checked += (unsigned long long)(ph - pl);
      if (D == 2) {
        cnt += count_in(yk, pl, ph, kyl, kyr);
        return;
      }
      for (int p = pl; p < ph; ++p) {
        bool in = yk.in(p, kyl, kyr);
        if (D >= 3) in = in && zk.in(p, kzl, kzr);
        if (D == 4) in = in && wk.in(p, kwl, kwr);
        cnt += in ? 1 : 0;
      }
    };
    // Strip s: its cells (nested) or the strip itself.
    auto visit = [&](int s) {
      const uint64_t lo1 = rkey(sylo[s]), hi1 = rkey(syhi[s]);
      const bool reach = act && hi1 >= kyl && lo1 <= kyr;
      if (!__any_sync(0xffffffffu, reach)) return;
      const bool in1 = reach && lo1 >= kyl && hi1 <= kyr;
      if (D == 2) {
        count_range(sst[s], sst[s + 1], in1, reach, s == sq);
        return;
      }
      // cells whose column-2 range meets a reaching lane's: a contiguous run
      const uint64_t zl = wmin64(reach ? kzl : ~0ull);
      const uint64_t zh = wmax64(reach ? kzr : 0ull);
      int c0 = 0, c1 = 0;
      for (int b = 0; b < S2; b += 32) {
        const int c = b + lane;
        c0 += __popc(__ballot_sync(0xffffffffu, c < S2 && rkey(czhi[s * S2 + c]) < zl));
        c1 += __popc(__ballot_sync(0xffffffffu, c < S2 && rkey(czlo[s * S2 + c]) <= zh));
      }
      for (int c = c0; c < c1; ++c) {
        const uint64_t lo2 = rkey(czlo[s * S2 + c]), hi2 = rkey(czhi[s * S2 + c]);
        const bool rc = reach && hi2 >= kzl && lo2 <= kzr;
        if (!__any_sync(0xffffffffu, rc)) continue;
        // d = 4: column 3 has no cell bounds, so every candidate is checked
        const bool in2 = D == 3 && rc && in1 && lo2 >= kzl && hi2 <= kzr;
        count_range(cst[s * S2 + c], cst[s * S2 + c + 1], in2, rc, s == sq && c == hc2);
      }
    };

    visit(sq);
    // strips above: their lower bounds grow, so the first one that no lane
    // reaches ends the direction (every lane's ball starts below its own
    // strip's upper bound); the same below
    for (int s = sq + 1; s < S; ++s) {
      if (!__any_sync(0xffffffffu, act && rkey(sylo[s]) <= kyr)) break;
      visit(s);
    }
    for (int s = sq - 1; s >= 0; --s) {
      if (!__any_sync(0xffffffffu, act && rkey(syhi[s]) >= kyl)) break;
      visit(s);
    }

    if (exists) J->cnt[J->idxg[qp]] = qok ? cnt : 0;
    const unsigned long long tot = __reduce_add_sync(0xffffffffu, (unsigned)checked);
    if (lane == 0) atomicAdd(J->stats + 0, tot);
  }
}

template <int D>
void launch_t(const JobDev* jobs, const WorkItem* items, int nitems, int* counter, int num_sms,
              cudaStream_t st) {
  auto kern = wcount_kernel<D>;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WC_WARPS * 32, 0);
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  const int need = (nitems + WC_WARPS - 1) / WC_WARPS;
  if (grid > need) grid = need;
  if (grid < 1) return;
  kern<<<grid, WC_WARPS * 32, 0, st>>>(jobs, items, nitems, counter);
  count_launch();
}

}  // namespace

// d = 2: measured faster than the FP32 union-window counts on every workload
// here; for d = 3 and 4 the radii of those workloads are large and few cells
// lie wholly inside a ball, so the FP32 kernel (egb_wgrid.cuh) is kept there
bool count_keys_supported(int dclass) { return dclass == 2; }

void launch_count_keys(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                       int* counter, int num_sms, cudaStream_t st) {
  if (dclass == 2) launch_t<2>(jobs_d, items_d, nitems, counter, num_sms, st);
  else if (dclass == 3) launch_t<3>(jobs_d, items_d, nitems, counter, num_sms, st);
  else launch_t<4>(jobs_d, items_d, nitems, counter, num_sms, st);
}

}  // namespace egb
