// egb_wavelet.cu -- exact 2-D ball counts in rank space (4-ary wavelet matrix).
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
// The wavelet matrix answers that in O(log len).  Values are written as D
// base-4 digits; level l (l = 0 .. D-1) stores digit D-1-l of every value
// of the sequence S_l, where S_0 = S and S_{l+1} is S_l stably partitioned
// by that digit (digit 0 first, then 1, 2, 3).  A position range [a, b) of
// level l maps, for digit t, to [B_t + rank_t(a), B_t + rank_t(b)) in level
// l + 1 (B_t: digits below t in the whole level).  A value range [c, d) is
// descended digit by digit: while c and d share their leading digits both
// descend together; at the first digit where they differ the values with a
// digit strictly between count whole, and two descents continue -- "at
// least c" in c's digit and "below d" in d's.
//
// Storage: each level is a sequence of 32-byte blocks of 64 digits (two bit
// planes and the counts of digits <= 0, <= 1, <= 2 before the block), so a
// rank costs one block read.  Range ends come from the sorted keys through
// FP32 brackets and two levels of samples (ball_positions, egb_search.cuh).
//
// Build: one block per tile of WM_TILE values and one launch per level.  A
// block needs the digit counts of its level before its tile: the previous
// level's pass adds the digits it sends to each destination tile (and super
// tile) of the next level, so the sums are complete when the next launch
// starts.
#include "egb_internal.cuh"
#include "egb_search.cuh"

namespace egb {
namespace {

constexpr int WM_THREADS = 256;
constexpr int WM_WARPS = WM_THREADS / 32;
constexpr int WM_ROUNDS = WM_TILE / WM_THREADS;  // rounds of 32 values per warp
static_assert(WM_ROUNDS == 8 && WM_ROUNDS % 2 == 0, "pairs of rounds fill 64-digit blocks");

// job of a block: last j with first(jobs[j]) <= b
template <typename F>
__device__ __forceinline__ int job_of(const WmJob* __restrict__ jobs, int njobs, int b, F first) {
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (first(jobs[m]) <= b) lo = m; else hi = m;
  }
  return lo;
}

// inv_b[w] = position of working offset w in the b order
__global__ void __launch_bounds__(WM_THREADS)
wm_inv_kernel(const WmJob* __restrict__ jobs, int njobs, const int32_t* __restrict__ vals) {
  const WmJob& J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.tile0; })];
  const int len = J.len;
  const int t0 = ((int)blockIdx.x - J.tile0) * WM_TILE;
  const int t1 = min(t0 + WM_TILE, len);
  const int32_t* __restrict__ vb = vals + J.base_b;
  int32_t* __restrict__ inv = J.inv_b;
  const int sb = J.seg_begin;
  for (int p = t0 + threadIdx.x; p < t1; p += WM_THREADS) {
    const int w = vb[p] - sb;
    if ((unsigned)w < (unsigned)len) inv[w] = p;
  }
}

// S_0[i] = inv_b[point at position i of the a order], and the digits of
// level 0 per tile and super tile
__global__ void __launch_bounds__(WM_THREADS)
wm_seq_kernel(const WmJob* __restrict__ jobs, int njobs, const int32_t* __restrict__ vals) {
  __shared__ uint32_t cnt[4];
  const WmJob& J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.tile0; })];
  const int len = J.len;
  const int tile = (int)blockIdx.x - J.tile0;
  const int t0 = tile * WM_TILE;
  const int t1 = min(t0 + WM_TILE, len);
  const int sh = 2 * (J.D - 1);
  const int32_t* __restrict__ va = vals + J.base_a;
  const int32_t* __restrict__ inv = J.inv_b;
  int32_t* __restrict__ seq = J.seq0;
  const int sb = J.seg_begin;
  if (threadIdx.x < 4) cnt[threadIdx.x] = 0;
  __syncthreads();
  uint32_t c[4] = {0, 0, 0, 0};
  for (int i = t0 + threadIdx.x; i < t1; i += WM_THREADS) {
    const int w = va[i] - sb;
    const int s = (unsigned)w < (unsigned)len ? inv[w] : 0;
    seq[i] = s;
    const int dg = (s >> sh) & 3;
#pragma unroll
    for (int t = 0; t < 4; ++t) c[t] += dg == t;
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const uint32_t v = __reduce_add_sync(0xffffffffu, c[t]);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&cnt[t], v);
  }
  __syncthreads();
  if (threadIdx.x < 4 && cnt[threadIdx.x]) {
    J.tcount[(size_t)tile * 4 + threadIdx.x] = cnt[threadIdx.x];
    atomicAdd(J.scount + (size_t)(tile / WM_SUPER) * 4 + threadIdx.x, cnt[threadIdx.x]);
  }
}

// One level of every job: the 64-digit blocks of level l, the stable
// partition into the sequence of level l + 1, and that level's digits per
// destination tile.  Warp w holds the values [w * 256, (w + 1) * 256) of the
// tile in eight rounds of 32; rounds 2m and 2m + 1 form one block.
__global__ void __launch_bounds__(WM_THREADS)
wm_level_kernel(const WmJob* __restrict__ jobs, int njobs, int l) {
  __shared__ uint32_t red[WM_WARPS][8];
  __shared__ uint32_t wtot[WM_WARPS][4];     // digits of each warp's 256 values
  __shared__ uint32_t nxt[32];               // next level: [digit t][tile offset][next digit]
  __shared__ int32_t base[4];                // first destination of each digit from this tile
  __shared__ uint32_t before_s[4];           // digits of this level before the tile
  __shared__ uint32_t total_s[4];            // digits of the whole level
  const WmJob& J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.tile0; })];
  const int D = J.D;
  if (l >= D) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int len = J.len;
  const int ntiles = J.ntiles, nsuper = J.nsuper;
  const int tile = (int)blockIdx.x - J.tile0;
  const int t0 = tile * WM_TILE;
  const int sh = 2 * (D - 1 - l);
  const int32_t* __restrict__ src = (l & 1) ? J.seq1 : J.seq0;
  int32_t* __restrict__ dst = (l & 1) ? J.seq0 : J.seq1;
  const uint4* __restrict__ tc = reinterpret_cast<const uint4*>(J.tcount) + (size_t)l * ntiles;
  const uint4* __restrict__ sc = reinterpret_cast<const uint4*>(J.scount) + (size_t)l * nsuper;
  WmBlock* __restrict__ lv = J.levels + (size_t)l * J.nblocks;

  // digits of this level before the tile, and in all
  uint32_t bf[4] = {0, 0, 0, 0}, tt[4] = {0, 0, 0, 0};
  const int sup = tile / WM_SUPER;
  for (int s = tid; s < nsuper; s += WM_THREADS) {
    const uint4 v = sc[s];
    tt[0] += v.x; tt[1] += v.y; tt[2] += v.z; tt[3] += v.w;
    if (s < sup) { bf[0] += v.x; bf[1] += v.y; bf[2] += v.z; bf[3] += v.w; }
  }
  for (int t = sup * WM_SUPER + tid; t < tile; t += WM_THREADS) {
    const uint4 v = tc[t];
    bf[0] += v.x; bf[1] += v.y; bf[2] += v.z; bf[3] += v.w;
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    bf[t] = __reduce_add_sync(0xffffffffu, bf[t]);
    tt[t] = __reduce_add_sync(0xffffffffu, tt[t]);
  }
  if (lane == 0) {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      red[warp][t] = bf[t];
      red[warp][4 + t] = tt[t];
    }
  }
  if (tid < 32) nxt[tid] = 0;

  // this warp's values and their digits
  const int wbase = t0 + warp * (WM_TILE / WM_WARPS);
  int32_t v[WM_ROUNDS];
  uint32_t bh[WM_ROUNDS], bl[WM_ROUNDS], bv[WM_ROUNDS];
  uint32_t wc[4] = {0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < WM_ROUNDS; ++k) {
    const int e = wbase + k * 32 + lane;
    const bool ok = e < len;
    v[k] = ok ? src[e] : 0;
    const int dg = (v[k] >> sh) & 3;
    bh[k] = __ballot_sync(0xffffffffu, ok && (dg & 2));
    bl[k] = __ballot_sync(0xffffffffu, ok && (dg & 1));
    bv[k] = __ballot_sync(0xffffffffu, ok);
    wc[0] += __popc(bv[k] & ~bh[k] & ~bl[k]);
    wc[1] += __popc(bv[k] & ~bh[k] & bl[k]);
    wc[2] += __popc(bh[k] & ~bl[k]);
    wc[3] += __popc(bh[k] & bl[k]);
  }
  if (lane == 0) {
#pragma unroll
    for (int t = 0; t < 4; ++t) wtot[warp][t] = wc[t];
  }
  __syncthreads();
  if (tid == 0) {
    int32_t run = 0;
    for (int t = 0; t < 4; ++t) {
      uint32_t b = 0, tot = 0;
      for (int w = 0; w < WM_WARPS; ++w) {
        b += red[w][t];
        tot += red[w][4 + t];
      }
      before_s[t] = b;
      total_s[t] = tot;
      if (tile == 0) J.bucket[l * 4 + t] = run;   // first position of digit t next level
      base[t] = run + (int32_t)b;
      run += (int32_t)tot;
    }
  }
  __syncthreads();
  // digits before this warp's values in the tile
  uint32_t wp[4] = {0, 0, 0, 0};
  for (int w = 0; w < warp; ++w) {
#pragma unroll
    for (int t = 0; t < 4; ++t) wp[t] += wtot[w][t];
  }
  const uint32_t lt = (1u << lane) - 1u;
  const bool more = l + 1 < D;
  const int nsh = sh - 2;
  int32_t dbase[4], dtile0[4];
  uint32_t gb[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    dbase[t] = base[t] + (int32_t)wp[t];     // this warp's first destination per digit
    dtile0[t] = base[t] / WM_TILE;
    gb[t] = before_s[t] + wp[t];             // digits of the level before this warp
  }
#pragma unroll
  for (int k = 0; k < WM_ROUNDS; ++k) {
    const uint32_t m0 = bv[k] & ~bh[k] & ~bl[k], m1 = bv[k] & ~bh[k] & bl[k];
    const uint32_t m2 = bh[k] & ~bl[k], m3 = bh[k] & bl[k];
    const int e0 = wbase + k * 32;
    if ((k & 1) == 0 && lane == 0 && e0 < len) {
      WmBlock B;
      B.hi[0] = bh[k];
      B.hi[1] = bh[k + 1];
      B.lo[0] = bl[k];
      B.lo[1] = bl[k + 1];
      B.le[0] = gb[0];
      B.le[1] = gb[0] + gb[1];
      B.le[2] = gb[0] + gb[1] + gb[2];
      B.pad = 0;
      lv[e0 >> 6] = B;
    }
    const int e = e0 + lane;
    const bool ok = e < len;
    const int dg = (int)((bh[k] >> lane) & 1u) * 2 + (int)((bl[k] >> lane) & 1u);
    const uint32_t mine = dg == 0 ? m0 : dg == 1 ? m1 : dg == 2 ? m2 : m3;
    const int db = dg == 0 ? dbase[0] : dg == 1 ? dbase[1] : dg == 2 ? dbase[2] : dbase[3];
    const int dt0 = dg == 0 ? dtile0[0] : dg == 1 ? dtile0[1] : dg == 2 ? dtile0[2] : dtile0[3];
    const int dest = db + __popc(mine & lt);
    if (more) {
      if (ok && (unsigned)dest < (unsigned)len) dst[dest] = v[k];
      const int off = dest / WM_TILE - dt0;
      const int key = ok && off >= 0 && off < 2 ? dg * 8 + off * 4 + ((v[k] >> nsh) & 3) : -1;
      const uint32_t peers = __match_any_sync(0xffffffffu, key);
      if (key >= 0 && (peers & lt) == 0) atomicAdd(&nxt[key], (uint32_t)__popc(peers));
    }
    dbase[0] += __popc(m0); dbase[1] += __popc(m1); dbase[2] += __popc(m2); dbase[3] += __popc(m3);
    gb[0] += __popc(m0); gb[1] += __popc(m1); gb[2] += __popc(m2); gb[3] += __popc(m3);
  }
  // a length that is a multiple of 64 leaves one more block: no digits, every count
  if (tid == 0 && (len & 63) == 0 && t0 + WM_TILE >= len) {
    WmBlock B;
    B.hi[0] = B.hi[1] = B.lo[0] = B.lo[1] = 0u;
    B.le[0] = total_s[0];
    B.le[1] = total_s[0] + total_s[1];
    B.le[2] = total_s[0] + total_s[1] + total_s[2];
    B.pad = 0;
    lv[len >> 6] = B;
  }
  if (more) {
    __syncthreads();
    if (tid < 32 && nxt[tid]) {
      const int t = tid >> 3, off = (tid >> 2) & 1, nd = tid & 3;
      const int dt = base[t] / WM_TILE + off;
      if (dt >= 0 && dt < ntiles) {
        atomicAdd(J.tcount + ((size_t)(l + 1) * ntiles + dt) * 4 + nd, nxt[tid]);
        atomicAdd(J.scount + ((size_t)(l + 1) * nsuper + dt / WM_SUPER) * 4 + nd, nxt[tid]);
      }
    }
  }
}

// ------------------------------------------------------------- queries --
// Digits <= t (t = 0, 1, 2) before position i of a level, i clamped to
// [0, len] (positions of a consistent matrix never leave it; the clamp keeps
// every read inside the level).
struct Rank4 {
  uint32_t le[3];
};
__device__ __forceinline__ Rank4 rank4(const WmBlock* __restrict__ lv, int i, int len) {
  i = min(max(i, 0), len);
  const uint4* p = reinterpret_cast<const uint4*>(lv + (i >> 6));
  const uint4 planes = __ldg(p);
  const uint4 cnts = __ldg(p + 1);
  const int r = i & 63;
  const uint64_t mask = r ? (~0ull >> (64 - r)) : 0ull;
  const uint64_t hi = ((uint64_t)planes.y << 32) | planes.x;
  const uint64_t lo = ((uint64_t)planes.w << 32) | planes.z;
  Rank4 R;
  R.le[0] = cnts.x + (uint32_t)__popcll(~hi & ~lo & mask);
  R.le[1] = cnts.y + (uint32_t)__popcll(~hi & mask);
  R.le[2] = cnts.z + (uint32_t)__popcll(~(hi & lo) & mask);
  return R;
}
// digits <= t before i (t = -1 .. 3); selects, not an indexed array, so
// the ranks stay in registers
__device__ __forceinline__ int le_of(const Rank4& R, int t, int i) {
  return t < 0 ? 0 : t == 0 ? (int)R.le[0] : t == 1 ? (int)R.le[1] : t == 2 ? (int)R.le[2] : i;
}

// #{i in [a, b) : S[i] in [c, d)} for 0 <= a <= b <= len, 0 <= c <= d <= len.
__device__ int wm_rect(const WmJob& J, int a, int b, int c, int d) {
  if (a >= b || c >= d) return 0;
  const WmBlock* __restrict__ levels = J.levels;
  const int32_t* __restrict__ bucket = J.bucket;
  const int D = J.D, nb = J.nblocks, len = J.len;
  int l = 0, tc = 0, td = 0;
  for (; l < D; ++l) {  // c and d share this digit: one descent
    const int sh = 2 * (D - 1 - l);
    tc = (c >> sh) & 3;
    td = (d >> sh) & 3;
    if (tc != td) break;
    const WmBlock* lv = levels + (size_t)l * nb;
    const Rank4 A = rank4(lv, a, len), B = rank4(lv, b, len);
    const int bt = __ldg(bucket + 4 * l + tc);
    a = bt + le_of(A, tc, a) - le_of(A, tc - 1, a);
    b = bt + le_of(B, tc, b) - le_of(B, tc - 1, b);
    if (a >= b) return 0;
  }
  if (l >= D) return 0;  // c == d (excluded above)
  // first differing digit tc < td: digits strictly between count whole
  const WmBlock* lv = levels + (size_t)l * nb;
  const Rank4 A = rank4(lv, a, len), B = rank4(lv, b, len);
  int res = (le_of(B, td - 1, b) - le_of(A, td - 1, a)) - (le_of(B, tc, b) - le_of(A, tc, a));
  const int bc = __ldg(bucket + 4 * l + tc), bd = __ldg(bucket + 4 * l + td);
  int a0 = bc + le_of(A, tc, a) - le_of(A, tc - 1, a);   // digit tc: count values >= c
  int b0 = bc + le_of(B, tc, b) - le_of(B, tc - 1, b);
  int a1 = bd + le_of(A, td, a) - le_of(A, td - 1, a);   // digit td: count values < d
  int b1 = bd + le_of(B, td, b) - le_of(B, td - 1, b);
  res += b0 - a0;
  for (++l; l < D; ++l) {
    const int sh = 2 * (D - 1 - l);
    const WmBlock* lv2 = levels + (size_t)l * nb;
    if (a0 < b0) {  // values >= c: subtract those below c's digit
      const int t = (c >> sh) & 3;
      const Rank4 P = rank4(lv2, a0, len), Q = rank4(lv2, b0, len);
      res -= le_of(Q, t - 1, b0) - le_of(P, t - 1, a0);
      const int bt = __ldg(bucket + 4 * l + t);
      a0 = bt + le_of(P, t, a0) - le_of(P, t - 1, a0);
      b0 = bt + le_of(Q, t, b0) - le_of(Q, t - 1, b0);
    }
    if (a1 < b1) {  // values < d: add those below d's digit
      const int t = (d >> sh) & 3;
      const Rank4 P = rank4(lv2, a1, len), Q = rank4(lv2, b1, len);
      res += le_of(Q, t - 1, b1) - le_of(P, t - 1, a1);
      const int bt = __ldg(bucket + 4 * l + t);
      a1 = bt + le_of(P, t, a1) - le_of(P, t - 1, a1);
      b1 = bt + le_of(Q, t, b1) - le_of(Q, t - 1, b1);
    }
    if (a0 >= b0 && a1 >= b1) break;
  }
  return res;
}

__global__ void __launch_bounds__(WM_QBLOCK)
wm_count_kernel(const TaskDev* __restrict__ tasks, const WmJob* __restrict__ jobs, int njobs,
                const KeyIndex kx, const int32_t* __restrict__ vals_all) {
  const WmJob& J = jobs[job_of(jobs, njobs, blockIdx.x, [](const WmJob& j) { return j.qblk0; })];
  const int len = J.len;
  const int i = ((int)blockIdx.x - J.qblk0) * WM_QBLOCK + threadIdx.x;
  if (i >= len) return;
  const TaskDev& t = tasks[J.task];
  const int32_t w = vals_all[J.base_a + i];          // working index of the query
  const double r = t.rad[w];
  const int rc = radius_class(r);
  int32_t count;
  if (rc == 0) {
    count = 0;
  } else if (rc == 2) {
    count = len;
  } else {
    const SegView va = seg_view(kx, J.base_a, J.s1_a, J.s2_a, len);
    int alo, ahi, blo, bhi;
    ball_positions(va, value_of(va.keys[i]), r, -1, alo, ahi);
    if (J.brange) {  // the b ball, as the 1-D count of column b found it
      const int2 br = __ldg(J.brange + w);
      blo = br.x;
      bhi = br.y;
    } else {
      const SegView vb = seg_view(kx, J.base_b, J.s1_b, J.s2_b, len);
      const int jb = min(max(J.inv_b[w - J.seg_begin], 0), len - 1);
      ball_positions(vb, value_of(__ldg(vb.keys + jb)), r, -1, blo, bhi);
    }
    count = wm_rect(J, alo, ahi, blo, bhi);
  }
  t.cnt[J.slot][w] = count;
}

// fkeys[p] = the largest float <= the value of keys[p]; s1[j] = keys[32 j],
// s2[j] = keys[1024 j] and the same of fkeys, for every sorted segment.
// One block of SAMPLE_THREADS per 2048-key tile of the sort.
constexpr int SAMPLE_THREADS = 256;
__global__ void __launch_bounds__(SAMPLE_THREADS)
samples_kernel(const SortSeg* __restrict__ segs, const int32_t* __restrict__ blk_seg,
               const uint64_t* __restrict__ keys, KeyIndexOut out) {
  const SortSeg sg = segs[blk_seg[blockIdx.x]];
  const int i0 = ((int)blockIdx.x - sg.blk0) * SORT_TILE;
  const int i1 = min(i0 + SORT_TILE, sg.len);
  for (int p = i0 + (int)threadIdx.x; p < i1; p += SAMPLE_THREADS) {
    const uint64_t k = __ldg(keys + sg.out_base + p);
    const float f = __double2float_rd(value_of(k));
    out.fkeys[sg.out_base + p] = f;
    if (p % SAMPLE1 == 0) {
      out.s1[sg.s1_base + p / SAMPLE1] = k;
      out.fs1[sg.s1_base + p / SAMPLE1] = f;
      if (p % SAMPLE2 == 0) {
        out.s2[sg.s2_base + p / SAMPLE2] = k;
        out.fs2[sg.s2_base + p / SAMPLE2] = f;
      }
    }
  }
}
static_assert(SORT_TILE % SAMPLE1 == 0, "sample grid");

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
                     const KeyIndex& kx, const int32_t* sorted_vals, cudaStream_t st) {
  if (njobs <= 0 || total_blocks <= 0) return;
  wm_count_kernel<<<total_blocks, WM_QBLOCK, 0, st>>>(tasks_d, jobs_d, njobs, kx, sorted_vals);
  count_launch();
}

void launch_samples(const SortSeg* segs_d, const int32_t* blk_seg_d, int nblk,
                    const uint64_t* keys, const KeyIndexOut& out, cudaStream_t st) {
  if (nblk <= 0) return;
  samples_kernel<<<nblk, SAMPLE_THREADS, 0, st>>>(segs_d, blk_seg_d, keys, out);
  count_launch();
}

}  // namespace egb
