// egb_wavelet.cu -- exact 2-D ball counts in rank space (wavelet matrix).
//
// query_ball_point(..., r, p=inf, return_length=True) in two dimensions
// (ennemi/_entropy_estimators.py:152-154 for the (x, z) and (y, z) spaces of
// the conditional MI, :196 and :243 for two-column semidiscrete spaces)
// counts #{j : max(fl64(|a_j - a_q|), fl64(|b_j - b_q|)) <= r}.  Per column,
// {v : fl64(|v - q|) <= r} is one range of order-preserving keys (ball_keys),
// hence one range of positions in the column's sorted order: [a_lo, a_hi) and
// [b_lo, b_hi).  With S[i] = position in the b order of the point at position
// i of the a order, the count is #{i in [a_lo, a_hi) : S[i] in [b_lo, b_hi)}
// -- integer arithmetic on ranks, exact for any data, ties included.
//
// The wavelet matrix answers that in O(log len): level l (l = 0 .. L-1)
// stores bit L-1-l of every value of the sequence S_l, where S_0 = S and
// S_{l+1} is S_l stably partitioned by that bit (zeros first).  A value range
// [c, d) is descended bit by bit; at each level a position range [a, b)
// maps to [rank0(a), rank0(b)) on the zero side or [Z + rank1(a), Z +
// rank1(b)) on the one side.  While c and d agree on their leading bits both
// descend together; below the first differing bit the count splits into "at
// least c" on the zero side and "below d" on the one side.
//
// Build: one block per tile of WM_TILE values and one launch per level.  A
// block needs the ones of its level before its tile: the previous level's
// pass adds the ones it sends to each destination tile (and super tile) of
// the next level, so the sums are ready when the next launch starts.
#include "egb_internal.cuh"

namespace egb {
namespace {

constexpr int WM_THREADS = 256;
constexpr int WM_PER = WM_TILE / WM_THREADS;  // values per thread (k-major)
static_assert(WM_TILE % (32 * WM_THREADS / 32) == 0, "tiles hold whole warps");
static_assert(WM_PER == 8, "eight values per thread");

// job of a block: last j with jobs[j].first <= b
template <typename F>
__device__ __forceinline__ int job_of(const WmJob* __restrict__ jobs, int njobs, int b, F first) {
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (first(jobs[m]) <= b) lo = m; else hi = m;
  }
  return lo;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = __reduce_add_sync(0xffffffffu, v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  uint32_t t = 0;
#pragma unroll
  for (int w = 0; w < WM_THREADS / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

// inv_b[w] = position of working offset w in the b order
__global__ void __launch_bounds__(WM_THREADS)
wm_inv_kernel(const WmJob* __restrict__ jobs, int njobs, const int32_t* __restrict__ vals) {
  const WmJob J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.tile0; })];
  const int t0 = ((int)blockIdx.x - J.tile0) * WM_TILE;
  const int t1 = min(t0 + WM_TILE, J.len);
  for (int p = t0 + threadIdx.x; p < t1; p += WM_THREADS) {
    const int w = vals[J.base_b + p] - J.seg_begin;
    if ((unsigned)w < (unsigned)J.len) J.inv_b[w] = p;
  }
}

// S_0[i] = inv_b[point at position i of the a order]; ones of the top bit
// per tile and super tile
__global__ void __launch_bounds__(WM_THREADS)
wm_seq_kernel(const WmJob* __restrict__ jobs, int njobs, const int32_t* __restrict__ vals) {
  __shared__ uint32_t red[WM_THREADS / 32];
  const WmJob J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.tile0; })];
  const int tile = (int)blockIdx.x - J.tile0;
  const int t0 = tile * WM_TILE;
  const int t1 = min(t0 + WM_TILE, J.len);
  const int top = J.L - 1;
  uint32_t ones = 0;
  for (int i = t0 + threadIdx.x; i < t1; i += WM_THREADS) {
    const int w = vals[J.base_a + i] - J.seg_begin;
    const int s = (unsigned)w < (unsigned)J.len ? J.inv_b[w] : 0;
    J.seq0[i] = s;
    ones += (uint32_t)(s >> top) & 1u;
  }
  const uint32_t tot = block_sum(ones, red);
  if (threadIdx.x == 0 && tot) {
    J.tcount[tile] = tot;
    atomicAdd(J.scount + tile / WM_SUPER, tot);
  }
}

// One level of every job: bits and word prefixes of level l, the stable
// partition into the sequence of level l + 1, and that level's ones per
// destination tile.
__global__ void __launch_bounds__(WM_THREADS)
wm_level_kernel(const WmJob* __restrict__ jobs, int njobs, int l) {
  __shared__ uint32_t red[WM_THREADS / 32];
  __shared__ uint32_t wpre[WM_PER][WM_THREADS / 32];  // ones of (k, warp), then their prefix
  __shared__ uint32_t next[4];                        // next level's ones per destination tile
  const WmJob J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.tile0; })];
  if (l >= J.L) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tile = (int)blockIdx.x - J.tile0;
  const int t0 = tile * WM_TILE;
  const int len = J.len;
  const int bit = J.L - 1 - l;
  const int32_t* __restrict__ src = (l & 1) ? J.seq1 : J.seq0;
  int32_t* __restrict__ dst = (l & 1) ? J.seq0 : J.seq1;
  const uint32_t* __restrict__ tc = J.tcount + (size_t)l * J.ntiles;
  const uint32_t* __restrict__ sc = J.scount + (size_t)l * J.nsuper;
  uint2* __restrict__ lv = J.levels + (size_t)l * J.nwords;

  // ones of this level before the tile, and in all
  uint32_t before = 0, total = 0;
  const int sup = tile / WM_SUPER;
  for (int s = tid; s < J.nsuper; s += WM_THREADS) {
    const uint32_t v = sc[s];
    total += v;
    before += s < sup ? v : 0u;
  }
  for (int t = sup * WM_SUPER + tid; t < tile; t += WM_THREADS) before += tc[t];
  if (tid < 4) next[tid] = 0;
  const uint32_t ones_before = block_sum(before, red);
  const uint32_t ones_total = block_sum(total, red);
  const int Z = len - (int)ones_total;
  if (tile == 0 && tid == 0) J.zeros[l] = Z;
  const int zeros_before = t0 - (int)ones_before;

  int32_t v[WM_PER];
  uint32_t bal[WM_PER];
#pragma unroll
  for (int k = 0; k < WM_PER; ++k) {
    const int e = t0 + k * WM_THREADS + tid;
    const bool ok = e < len;
    v[k] = ok ? src[e] : 0;
    bal[k] = __ballot_sync(0xffffffffu, ok && ((v[k] >> bit) & 1));
    if (lane == 0) wpre[k][warp] = __popc(bal[k]);
  }
  __syncthreads();
  if (tid == 0) {  // exclusive prefix in value order: (k, warp) k-major
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < WM_PER; ++k)
      for (int w = 0; w < WM_THREADS / 32; ++w) {
        const uint32_t c = wpre[k][w];
        wpre[k][w] = run;
        run += c;
      }
  }
  __syncthreads();
  const bool more = l + 1 < J.L;
  const int nbit = bit - 1;
  const int zt0 = zeros_before / WM_TILE;                 // first destination tile, zeros
  const int ot0 = (Z + (int)ones_before) / WM_TILE;       // ... ones
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < WM_PER; ++k) {
    const int w0 = t0 + k * WM_THREADS + warp * 32;       // first value of this word
    if (lane == 0 && w0 < len) lv[w0 >> 5] = make_uint2(bal[k], ones_before + wpre[k][warp]);
    const int e = w0 + lane;
    const bool ok = e < len;
    const int r1 = (int)(wpre[k][warp] + __popc(bal[k] & lt));   // ones before e in the tile
    const int r0 = (e - t0) - r1;
    const bool one = (bal[k] >> lane) & 1u;
    const int dest = one ? Z + (int)ones_before + r1 : zeros_before + r0;
    if (more) {
      if (ok && (unsigned)dest < (unsigned)len) dst[dest] = v[k];
      const bool nb = ok && ((v[k] >> nbit) & 1);
      const int slot = one ? 2 + (dest / WM_TILE - ot0) : (dest / WM_TILE - zt0);
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const uint32_t c = __popc(__ballot_sync(0xffffffffu, nb && slot == s));
        if (lane == 0 && c) atomicAdd(&next[s], c);
      }
    }
  }
  // a length that is a multiple of 32 leaves one more word: no bits, every one
  if (tid == 0 && (len & 31) == 0 && t0 + WM_TILE >= len) lv[len >> 5] = make_uint2(0u, ones_total);
  if (more) {
    __syncthreads();
    if (tid < 4 && next[tid]) {
      const int dtile = tid < 2 ? zt0 + tid : ot0 + (tid - 2);
      if (dtile >= 0 && dtile < J.ntiles) {
        atomicAdd(J.tcount + (size_t)(l + 1) * J.ntiles + dtile, next[tid]);
        atomicAdd(J.scount + (size_t)(l + 1) * J.nsuper + dtile / WM_SUPER, next[tid]);
      }
    }
  }
}

// ------------------------------------------------------------- queries --
// i is clamped into [0, len]: positions of a consistent matrix never leave
// it, and the clamp keeps every read inside the level
__device__ __forceinline__ int rank1(const uint2* __restrict__ lv, int i, int len) {
  i = min(max(i, 0), len);
  const uint2 w = __ldg(lv + (i >> 5));
  return (int)w.y + __popc(w.x & ((1u << (i & 31)) - 1u));
}

// #{i in [a, b) : S[i] in [c, d)} for 0 <= a <= b <= len, 0 <= c <= d <= len.
__device__ int wm_rect(const WmJob& J, int a, int b, int c, int d) {
  if (a >= b || c >= d) return 0;
  const uint2* __restrict__ base = J.levels;
  const int L = J.L;
  int l = 0;
  for (; l < L; ++l) {  // c and d agree on this bit: one descent
    const int sh = L - 1 - l;
    const int cb = (c >> sh) & 1;
    if (cb != ((d >> sh) & 1)) break;
    const uint2* lv = base + (size_t)l * J.nwords;
    const int ra = a - rank1(lv, a, J.len), rb = b - rank1(lv, b, J.len);
    if (cb) {
      const int Z = __ldg(J.zeros + l);
      a = Z + (a - ra);
      b = Z + (b - rb);
    } else {
      a = ra;
      b = rb;
    }
    if (a >= b) return 0;
  }
  if (l >= L) return 0;  // c == d (excluded above)
  // c has bit 0 here and d bit 1: the zero side counts values >= c, the
  // one side values < d; the two descents run side by side
  const uint2* lv = base + (size_t)l * J.nwords;
  const int ra = a - rank1(lv, a, J.len), rb = b - rank1(lv, b, J.len);
  const int Zl = __ldg(J.zeros + l);
  int a0 = ra, b0 = rb;                          // zero side: count < c, subtract
  int a1 = Zl + (a - ra), b1 = Zl + (b - rb);    // one side: count < d
  int res = b0 - a0;
  for (++l; l < L; ++l) {
    const int sh = L - 1 - l;
    const uint2* lv2 = base + (size_t)l * J.nwords;
    const int Z = __ldg(J.zeros + l);
    if (a0 < b0) {
      const int r0a = a0 - rank1(lv2, a0, J.len), r0b = b0 - rank1(lv2, b0, J.len);
      if ((c >> sh) & 1) {
        res -= r0b - r0a;
        a0 = Z + (a0 - r0a);
        b0 = Z + (b0 - r0b);
      } else {
        a0 = r0a;
        b0 = r0b;
      }
    }
    if (a1 < b1) {
      const int r1a = a1 - rank1(lv2, a1, J.len), r1b = b1 - rank1(lv2, b1, J.len);
      if ((d >> sh) & 1) {
        res += r1b - r1a;
        a1 = Z + (a1 - r1a);
        b1 = Z + (b1 - r1b);
      } else {
        a1 = r1a;
        b1 = r1b;
      }
    }
    if (a0 >= b0 && a1 >= b1) break;
  }
  return res;
}

// [lo, hi): the positions of the sorted keys within [kl, kr], around p (whose
// key lies inside): gallop outward, then bisect.
__device__ __forceinline__ void key_range(const uint64_t* __restrict__ keys, int len, int p,
                                          uint64_t kl, uint64_t kr, int& lo, int& hi) {
  int a = p, step = 1;
  while (a + step < len && __ldg(keys + a + step) <= kr) {
    a += step;
    step <<= 1;
  }
  int b = a + step < len ? a + step : len;
  while (b - a > 1) {
    const int m = a + ((b - a) >> 1);
    if (__ldg(keys + m) <= kr) a = m; else b = m;
  }
  hi = a + 1;
  a = p;
  step = 1;
  while (a - step >= 0 && __ldg(keys + a - step) >= kl) {
    a -= step;
    step <<= 1;
  }
  b = a - step >= 0 ? a - step : -1;
  while (a - b > 1) {
    const int m = b + ((a - b) >> 1);
    if (__ldg(keys + m) >= kl) a = m; else b = m;
  }
  lo = a;
}

__global__ void __launch_bounds__(WM_QBLOCK)
wm_count_kernel(const TaskDev* __restrict__ tasks, const WmJob* __restrict__ jobs, int njobs,
                const uint64_t* __restrict__ keys_all, const int32_t* __restrict__ vals_all) {
  const WmJob& J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.qblk0; })];
  const int i = ((int)blockIdx.x - J.qblk0) * WM_QBLOCK + threadIdx.x;
  if (i >= J.len) return;
  const TaskDev& t = tasks[J.task];
  const int32_t w = vals_all[J.base_a + i];          // working index of the query
  const double r = t.rad[w];
  int32_t count;
  if (!(r >= 0.0)) {
    count = 0;
  } else if (isinf(r)) {
    count = J.len;
  } else {
    const uint64_t* __restrict__ ka = keys_all + J.base_a;
    const uint64_t* __restrict__ kb = keys_all + J.base_b;
    const int jb = min(max(J.inv_b[w - J.seg_begin], 0), J.len - 1);
    uint64_t al, ar, bl, br;
    ball_keys(value_of(ka[i]), r, al, ar);
    ball_keys(value_of(kb[jb]), r, bl, br);
    // the sorted keys fold -0 into +0, as the predicate does
    al = al == 0x7fffffffffffffffull ? 0x8000000000000000ull : al;
    bl = bl == 0x7fffffffffffffffull ? 0x8000000000000000ull : bl;
    int alo, ahi, blo, bhi;
    key_range(ka, J.len, i, al, ar, alo, ahi);
    key_range(kb, J.len, jb, bl, br, blo, bhi);
    count = wm_rect(J, alo, ahi, blo, bhi);
  }
  t.cnt[J.slot][w] = count;
}

}  // namespace

void launch_wm_build(const WmJob* jobs_d, int njobs, int total_tiles, int max_levels,
                     const int32_t* sorted_vals, cudaStream_t st) {
  if (njobs <= 0 || total_tiles <= 0) return;
  wm_inv_kernel<<<total_tiles, WM_THREADS, 0, st>>>(jobs_d, njobs, sorted_vals);
  count_launch();
  wm_seq_kernel<<<total_tiles, WM_THREADS, 0, st>>>(jobs_d, njobs, sorted_vals);
  count_launch();
  for (int l = 0; l < max_levels; ++l) {
    wm_level_kernel<<<total_tiles, WM_THREADS, 0, st>>>(jobs_d, njobs, l);
    count_launch();
  }
}

void launch_wm_count(const TaskDev* tasks_d, const WmJob* jobs_d, int njobs, int total_blocks,
                     const uint64_t* sorted_keys, const int32_t* sorted_vals, cudaStream_t st) {
  if (njobs <= 0 || total_blocks <= 0) return;
  wm_count_kernel<<<total_blocks, WM_QBLOCK, 0, st>>>(tasks_d, jobs_d, njobs, sorted_keys,
                                                      sorted_vals);
  count_launch();
}

}  // namespace egb
