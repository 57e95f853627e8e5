// egb_sort.cu -- batched segmented LSD radix sort of FP64 columns, and the
// 1-D estimator kernels that run on the sorted arrays.
//
// Sort.  Every requested (task, column, segment) is one segment of a single
// concatenated key array.  Keys are the order-preserving uint64 image of the
// FP64 value (key_of), the payload is the working index of the point.  The
// batch sort takes stable 8-bit single-sweep LSD passes over the high 48 key
// bits and repairs the rare runs tied there (below); the three-kernel pass
// -- histogram, exclusive scan, stable scatter -- serves the strip-key
// passes of the grid layouts: its per-block histograms are laid out
// segment-major, digit-next, block-minor, so ONE global exclusive scan
// yields absolute output positions that never leave a segment.
//
// 1-D kNN (entropy of one column, Ross MI with 1-D x): for the point at
// sorted position p the (k+1)-th smallest |x_j - x_p| (self included) is
// found by merging outward from p -- the exact FP64 distances, as cKDTree.
//
// 1-D counts (marginal spaces of KSG / CMI): #{j : fl64(|x_j - q|) <= r},
// r = fl64(eps - 1e-12).  fl64(s_j - q) is monotone in s_j (rounding is
// monotone), so on each side of q the predicate holds on one contiguous run
// of sorted positions -- one key range (ball_keys), whose ends are found
// through the segment's samples (egb_search.cuh).
#include <algorithm>

#include "egb_internal.cuh"
#include "egb_search.cuh"

namespace egb {

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;
constexpr int SORTED_THREADS = SORTED_BLOCK;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < SCAN_THREADS / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_THREADS / 32) ws[lane] = w;
  }
  __syncthreads();
  const uint32_t wprefix = warp ? ws[warp - 1] : 0;
  if (total) *total = ws[SCAN_THREADS / 32 - 1];
  const uint32_t r = wprefix + x - v;
  __syncthreads();
  return r;
}

__global__ void sort_hist_kernel(const SortSeg* __restrict__ segs,
                                 const int32_t* __restrict__ blk_seg,
                                 const uint64_t* __restrict__ keys, int shift,
                                 uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  const int b = blockIdx.x;
  const SortSeg s = segs[blk_seg[b]];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int i0 = (b - s.blk0) * SORT_TILE;
  const int i1 = min(i0 + SORT_TILE, s.len);
  for (int i = i0 + threadIdx.x; i < i1; i += SORT_THREADS)
    atomicAdd(&h[(uint32_t)(keys[s.out_base + i] >> shift) & 255u], 1u);
  __syncthreads();
  const int lb = b - s.blk0;
  hist[(int64_t)256 * s.blk0 + (int64_t)threadIdx.x * s.nblk + lb] = h[threadIdx.x];
}

// Stable scatter of one tile.  Warp w ranks the keys [w * CH, (w + 1) * CH)
// of the tile in rounds of 32: per-bit ballots give a key's rank among the
// equal digits of its round, per-warp counters carry the rank across rounds.  One
// block scan then turns the per-warp digit counts into the tile's layout in
// digit order, staged in shared memory and written out so that consecutive
// threads store to consecutive addresses of each digit's output run.
// offs[] holds absolute positions in the concatenated buffer.
__global__ void __launch_bounds__(SORT_THREADS)
sort_scatter_kernel(const SortSeg* __restrict__ segs, const int32_t* __restrict__ blk_seg,
                    const uint64_t* __restrict__ kin, const int32_t* __restrict__ vin, int shift,
                    const uint32_t* __restrict__ offs, uint64_t* __restrict__ kout,
                    int32_t* __restrict__ vout) {
  constexpr int NW = SORT_THREADS / 32;
  constexpr int CH = SORT_TILE / NW;  // keys per warp
  constexpr int R = CH / 32;          // rounds per warp
  static_assert(SORT_THREADS == 256 && SCAN_THREADS == 256, "one thread per digit");
  __shared__ uint32_t wcnt[NW][256];  // per-warp digit counts, then offsets
  __shared__ uint32_t dstart[256];    // first tile slot of each digit
  __shared__ uint32_t gbase[256];     // first output position of each digit
  __shared__ uint64_t sk[SORT_TILE];
  __shared__ int32_t sv[SORT_TILE];
  const int b = blockIdx.x;
  const SortSeg s = segs[blk_seg[b]];
  const int lb = b - s.blk0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  gbase[tid] = offs[(int64_t)256 * s.blk0 + (int64_t)tid * s.nblk + lb];
#pragma unroll
  for (int w = 0; w < NW; ++w) wcnt[w][tid] = 0;
  __syncthreads();
  const int i0 = lb * SORT_TILE;
  const int n = min(SORT_TILE, s.len - i0);
  const uint32_t lt = (1u << lane) - 1u;
  uint64_t key[R];
  int32_t val[R];
  uint32_t dg[R], rk[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t = warp * CH + r * 32 + lane;
    const bool valid = t < n;
    key[r] = valid ? kin[s.out_base + i0 + t] : 0ull;
    val[r] = valid ? vin[s.out_base + i0 + t] : 0;
    const uint32_t d = valid ? (uint32_t)(key[r] >> shift) & 255u : 256u + lane;
    dg[r] = d;
    // lanes with the same digit (9 bits: invalid lanes carry 256 + lane),
    // from one ballot per bit (measured faster than match_any here)
    uint32_t peers = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < 9; ++bit) {
      const uint32_t bb = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
      peers &= ((d >> bit) & 1u) ? bb : ~bb;
    }
    const uint32_t before = valid ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
    rk[r] = before + __popc(peers & lt);
  }
  __syncthreads();
  uint32_t run = 0;  // digit tid: offsets of the warps, then of the digit
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    const uint32_t c = wcnt[w][tid];
    wcnt[w][tid] = run;
    run += c;
  }
  dstart[tid] = block_excl_scan(run, nullptr);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t = warp * CH + r * 32 + lane;
    if (t < n) {
      const uint32_t d = dg[r];
      const uint32_t slot = dstart[d] + wcnt[warp][d] + rk[r];
      sk[slot] = key[r];
      sv[slot] = val[r];
    }
  }
  __syncthreads();
  for (int t = tid; t < n; t += SORT_THREADS) {
    const uint64_t k = sk[t];
    const uint32_t d = (uint32_t)(k >> shift) & 255u;
    const uint32_t pos = gbase[d] + ((uint32_t)t - dstart[d]);
    kout[pos] = k;
    vout[pos] = sv[t];
  }
}

// ------------------------------------------------------- single sweep --
// The batch sort proper: stable 8-bit LSD passes, one launch each,
// after Adinets and Merrill's single-sweep radix sort (Onesweep, 2022).  The
// load kernel computes the digit totals of all the passes per segment at
// once; each pass then needs, per tile and digit, only the count of that
// digit in the segment's earlier tiles.  A tile takes its id from an atomic
// counter (so every earlier tile of its segment has started), publishes its
// own digit counts at once, and looks back over its predecessors' published
// words -- aggregates or inclusive prefixes -- until it meets an inclusive
// one; it then publishes its own inclusive prefix and scatters.  A flag word
// holds the pass + 1 (bits 56-63; other passes' words read as "not yet"),
// an inclusive bit (55) and the count (bits 0-31), and is written and read
// whole, so no other data needs ordering.  Every wait is bounded: past
// OS_SPIN_LIMIT polls the tile records DERR_WAIT_TIMEOUT (the batch then
// reports EGB_ERR_DEVICE) and goes on.
constexpr int OS_PASSES = 8;
constexpr int OS_SPIN_LIMIT = 1 << 22;

__device__ __forceinline__ uint64_t key_of_bits(uint64_t u) {
  u = u == 0x8000000000000000ull ? 0ull : u;  // -0 -> +0
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__global__ void __launch_bounds__(SORT_THREADS)
onesweep_load_kernel(const TaskDev* __restrict__ tasks, const SortSeg* __restrict__ segs,
                     const int32_t* __restrict__ blk_seg, uint64_t* __restrict__ keys,
                     int32_t* __restrict__ vals, uint32_t* __restrict__ seg_hist, int first) {
  __shared__ uint32_t h[OS_PASSES * 256];
  const int b = blockIdx.x;
  const int si = blk_seg[b];
  const SortSeg s = segs[si];
  for (int i = threadIdx.x; i < OS_PASSES * 256; i += SORT_THREADS) h[i] = 0;
  __syncthreads();
  const TaskDev& t = tasks[s.task];
  const uint64_t* __restrict__ x =
      reinterpret_cast<const uint64_t*>(t.x64 + (int64_t)s.col * t.ld + s.src_begin);
  const int i0 = (b - s.blk0) * SORT_TILE;
  const int i1 = min(i0 + SORT_TILE, s.len);
  for (int i = i0 + threadIdx.x; i < i1; i += SORT_THREADS) {
    const uint64_t k = key_of_bits(x[i]);
    keys[s.out_base + i] = k;
    vals[s.out_base + i] = s.src_begin + i;
#pragma unroll
    for (int p = 0; p < OS_PASSES; ++p)
      if (p >= first) atomicAdd(&h[p * 256 + (uint32_t)((k >> (8 * p)) & 255u)], 1u);
  }
  __syncthreads();
  uint32_t* g = seg_hist + (size_t)si * OS_PASSES * 256;
  for (int i = threadIdx.x; i < OS_PASSES * 256; i += SORT_THREADS)
    if (h[i]) atomicAdd(g + i, h[i]);
}

// A pass tile is OS_TILE keys on OS_THREADS threads (eight keys a thread);
// its staging arrays exceed the 48 KB of static shared memory.
constexpr int OS_THREADS = 512;
constexpr int OS_NW = OS_THREADS / 32;
struct OsSmem {
  uint32_t wcnt[OS_NW][256];  // per-warp digit counts, then offsets
  uint32_t dstart[256];       // first tile slot of each digit
  uint32_t gbase[256];        // first output position of each digit
  uint32_t ws[8];             // digit-scan scratch
  int tile;
  uint64_t sk[OS_TILE];
  int32_t sv[OS_TILE];
};
static_assert(OS_TILE % OS_NW == 0 && (OS_TILE / OS_NW) % 32 == 0, "whole warp rounds");

// Exclusive scan over the 256 digits, one value per digit thread (tid <
// 256: warps 0-7); every thread of the block calls it.
__device__ __forceinline__ uint32_t digit_excl_scan(uint32_t v, uint32_t* ws) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t x = v;
  if (tid < 256) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < 8 ? ws[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < 8) ws[lane] = w;
  }
  __syncthreads();
  const uint32_t r = tid < 256 ? (warp ? ws[warp - 1] : 0u) + x - v : 0u;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(OS_THREADS)
onesweep_pass_kernel(const SortSeg* __restrict__ segs, const int32_t* __restrict__ os_blk_seg,
                     const uint64_t* __restrict__ kin, const int32_t* __restrict__ vin,
                     uint64_t* __restrict__ kout, int32_t* __restrict__ vout, int pass,
                     const uint32_t* __restrict__ seg_hist, unsigned long long* flags,
                     int* tile_counter, uint32_t* err) {
  constexpr int CH = OS_TILE / OS_NW;  // keys per warp
  constexpr int R = CH / 32;           // rounds per warp
  extern __shared__ __align__(16) unsigned char os_raw[];
  OsSmem& S = *reinterpret_cast<OsSmem*>(os_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) S.tile = atomicAdd(tile_counter, 1);
  for (int i = tid; i < OS_NW * 256; i += OS_THREADS) (&S.wcnt[0][0])[i] = 0u;
  __syncthreads();
  const int b = S.tile;
  const int si = os_blk_seg[b];
  const SortSeg s = segs[si];
  const int lb = b - s.os_blk0;
  const int shift = 8 * pass;
  const int i0 = lb * OS_TILE;
  const int n = min(OS_TILE, s.len - i0);
  const uint32_t lt = (1u << lane) - 1u;
  uint64_t key[R];
  int32_t val[R];
  uint32_t dg[R], rk[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t = warp * CH + r * 32 + lane;
    const bool valid = t < n;
    key[r] = valid ? kin[s.out_base + i0 + t] : 0ull;
    val[r] = valid ? vin[s.out_base + i0 + t] : 0;
    const uint32_t d = valid ? (uint32_t)(key[r] >> shift) & 255u : 256u + lane;
    dg[r] = d;
    uint32_t peers = 0xffffffffu;  // lanes with the same 9-bit digit
#pragma unroll
    for (int bit = 0; bit < 9; ++bit) {
      const uint32_t bb = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
      peers &= ((d >> bit) & 1u) ? bb : ~bb;
    }
    const uint32_t before = valid ? S.wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && (peers & lt) == 0) S.wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
    rk[r] = before + __popc(peers & lt);
  }
  __syncthreads();
  uint32_t cnt = 0;  // digit tid: offsets of the warps, then its count in the tile
  if (tid < 256) {
#pragma unroll
    for (int w = 0; w < OS_NW; ++w) {
      const uint32_t c = S.wcnt[w][tid];
      S.wcnt[w][tid] = cnt;
      cnt += c;
    }
  }
  // publish this tile's count of digit tid, then look back for the count of
  // digit tid in the segment's earlier tiles
  uint32_t excl = 0;
  if (tid < 256) {
    const unsigned long long tag = (unsigned long long)(pass + 1) << 56;
    const unsigned long long INCL = 1ull << 55;
    unsigned long long* mine = flags + (size_t)b * 256 + tid;
    if (lb == 0) {
      atomicExch(mine, tag | INCL | cnt);
    } else {
      atomicExch(mine, tag | cnt);
      int pb = b - 1;
      for (;;) {
        const volatile unsigned long long* f = flags + (size_t)pb * 256 + tid;
        unsigned long long w = *f;
        int spins = 0;
        while ((w >> 56) != (unsigned long long)(pass + 1)) {
          if (++spins > OS_SPIN_LIMIT) {
            atomicOr(err, DERR_WAIT_TIMEOUT);
            w = tag | INCL;
            break;
          }
          w = *f;
        }
        excl += (uint32_t)w;
        if ((w & INCL) || pb <= s.os_blk0) break;
        --pb;
      }
      atomicExch(mine, tag | INCL | (excl + cnt));
    }
  }
  // digit tid of the whole segment starts after the smaller digits
  const uint32_t seg_tot = tid < 256 ? seg_hist[((size_t)si * OS_PASSES + pass) * 256 + tid] : 0u;
  const uint32_t seg_off = digit_excl_scan(seg_tot, S.ws);
  const uint32_t ds = digit_excl_scan(cnt, S.ws);
  if (tid < 256) {
    S.gbase[tid] = seg_off + excl;
    S.dstart[tid] = ds;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t = warp * CH + r * 32 + lane;
    if (t < n) {
      const uint32_t d = dg[r];
      const uint32_t slot = S.dstart[d] + S.wcnt[warp][d] + rk[r];
      S.sk[slot] = key[r];
      S.sv[slot] = val[r];
    }
  }
  __syncthreads();
  for (int t = tid; t < n; t += OS_THREADS) {
    const uint64_t k = S.sk[t];
    const uint32_t d = (uint32_t)(k >> shift) & 255u;
    const uint32_t pos = S.gbase[d] + ((uint32_t)t - S.dstart[d]);
    if (pos < (uint32_t)s.len) {
      kout[s.out_base + pos] = k;
      vout[s.out_base + pos] = S.sv[t];
    } else {
      atomicOr(err, DERR_BAD_INDEX);
    }
  }
}

// ----------------------------------------------------------- tie repair --
// After the passes over digits 2..7 the keys of a segment are ordered by
// their high 48 bits (sign, exponent and 36 mantissa bits of the value),
// stably.  Keys equal there but not in the low 16 bits -- values within a
// relative 2^-36 of each other -- are rare, and sit in short runs: the first
// thread of a run of at most TIE_RUN keys sorts it by the whole key with an
// insertion sort (stable, so equal keys keep their input order and the
// result is the permutation of the eight-pass sort).  A longer run that is
// out of order is not repaired: its threads set DERR_SORT_TIES and the host
// runs the batch again with all eight passes.  Repairs permute keys only
// within runs, so the high bits read at any position never change while the
// kernel runs: run boundaries are read race-free.
constexpr int TIE_RUN = 32;

__global__ void __launch_bounds__(SORT_THREADS)
tie_fix_kernel(const SortSeg* __restrict__ segs, const int32_t* __restrict__ blk_seg,
               uint64_t* keys_all, int32_t* vals_all, uint32_t* __restrict__ err) {
  const SortSeg sg = segs[blk_seg[blockIdx.x]];
  const int len = sg.len;
  const int i0 = ((int)blockIdx.x - sg.blk0) * SORT_TILE;
  const int i1 = min(i0 + SORT_TILE, len);
  uint64_t* keys = keys_all + sg.out_base;  // written by run owners: no __restrict__
  int32_t* vals = vals_all + sg.out_base;
  for (int q = i0 + (int)threadIdx.x; q < i1; q += SORT_THREADS) {
    const uint64_t k = keys[q];
    const uint64_t hi = k >> 16;
    const bool starts = q == 0 || (keys[q - 1] >> 16) != hi;
    if (!starts) {
      // inside a run: out of order against the previous key and the run
      // too long to be repaired -> the batch needs the full sort
      if (k < keys[q - 1]) {
        int s = q - 1, e = q + 1;
        while (s > 0 && (keys[s - 1] >> 16) == hi && q - s <= TIE_RUN) --s;
        while (e < len && (keys[e] >> 16) == hi && e - s <= TIE_RUN) ++e;
        if (e - s > TIE_RUN) atomicOr(err, (uint32_t)DERR_SORT_TIES);
      }
      continue;
    }
    if (q + 1 >= len || (keys[q + 1] >> 16) != hi) continue;  // a run of one
    int e = q + 1;
    while (e < len && (keys[e] >> 16) == hi && e - q <= TIE_RUN) ++e;
    if (e - q > TIE_RUN) continue;
    for (int i = q + 1; i < e; ++i) {  // stable insertion sort of [q, e)
      const uint64_t ki = keys[i];
      if (ki >= keys[i - 1]) continue;
      const int32_t vi = vals[i];
      int j = i;
      while (j > q && keys[j - 1] > ki) {
        keys[j] = keys[j - 1];
        vals[j] = vals[j - 1];
        --j;
      }
      keys[j] = ki;
      vals[j] = vi;
    }
  }
}

// ------------------------------------------------------------------ scan --
__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, int64_t n,
                                   uint32_t* __restrict__ sums) {
  const int64_t c0 = (int64_t)blockIdx.x * SCAN_CHUNK;
  uint32_t s = 0;
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    const int64_t i = c0 + (int64_t)j * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint32_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_top_kernel(uint32_t* __restrict__ sums, int nchunks) {
  uint32_t carry = 0;
  for (int c0 = 0; c0 < nchunks; c0 += SCAN_THREADS) {
    const int i = c0 + threadIdx.x;
    const uint32_t v = i < nchunks ? sums[i] : 0;
    uint32_t tot;
    const uint32_t ex = block_excl_scan(v, &tot);
    if (i < nchunks) sums[i] = carry + ex;
    carry += tot;
  }
}

__global__ void scan_down_kernel(uint32_t* __restrict__ data, int64_t n,
                                 const uint32_t* __restrict__ sums) {
  const int64_t c0 = (int64_t)blockIdx.x * SCAN_CHUNK;
  // blocked arrangement: thread t owns items [t*ITEMS, (t+1)*ITEMS)
  uint32_t v[SCAN_ITEMS];
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    const int64_t i = c0 + (int64_t)threadIdx.x * SCAN_ITEMS + j;
    v[j] = i < n ? data[i] : 0;
    s += v[j];
  }
  uint32_t run = block_excl_scan(s, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    const int64_t i = c0 + (int64_t)threadIdx.x * SCAN_ITEMS + j;
    if (i < n) data[i] = run;
    run += v[j];
  }
}

// --------------------------------------------------------- sorted jobs ----
__global__ void sorted_jobs_kernel(const TaskDev* __restrict__ tasks,
                                   const SortedJob* __restrict__ jobs, int njobs,
                                   const KeyIndex kx, const int32_t* __restrict__ perm_all) {
  // the job of this block: last j with jobs[j].blk0 <= blockIdx.x
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (jobs[m].blk0 <= (int)blockIdx.x) lo = m; else hi = m;
  }
  const SortedJob jb = jobs[lo];
  const int64_t p = (int64_t)((int)blockIdx.x - jb.blk0) * SORTED_THREADS + threadIdx.x;
  const int64_t len = jb.len;
  if (p >= len) return;
  const uint64_t* __restrict__ keys = kx.keys + jb.base;
  const int32_t i = perm_all[jb.base + p];
  const TaskDev t = tasks[jb.task];
  const double q = value_of(keys[p]);
  const double INF = __longlong_as_double((long long)INF_BITS);

  if (jb.kind == 0) {  // (k+1)-NN distance, self included; +inf if too few
    int64_t L = p - 1, R = p + 1;
    double d = (jb.K <= len) ? 0.0 : INF;
    if (jb.K <= len) {
      for (int s = 1; s < jb.K; ++s) {
        const double dl = L >= 0 ? q - value_of(keys[L]) : INF;
        const double dr = R < len ? value_of(keys[R]) - q : INF;
        if (dl <= dr) { d = dl; --L; } else { d = dr; ++R; }
      }
    }
    t.eps[i] = d;
    return;
  }

  const double r = t.rad[i];
  const int rc = radius_class(r);
  int32_t count;
  if (rc == 0) {
    count = 0;
  } else if (rc == 2) {
    count = (int32_t)len;
  } else {
    // The ball is one run of sorted positions; its ends come from FP32
    // brackets and the segment's samples (ball_positions, egb_search.cuh).
    int lo, hi;
    ball_positions(seg_view(kx, jb.base, jb.s1_base, jb.s2_base, (int)len), q, r, (int)p, lo, hi);
    count = (int32_t)(hi - lo);
    if (jb.ranges) jb.ranges[i] = make_int2(lo, hi);
  }
  t.cnt[jb.slot][i] = count;
}

// ----------------------------------------------------------- grid keys ----
// inv[out + (w_B - seg_begin)] = p_B for the column-1 order of each grid job.
__global__ void grid_inv_kernel(const JobDev* __restrict__ jobs,
                                const int32_t* __restrict__ grid_jobs, int ngrid,
                                const SortSeg* __restrict__ gsegs,
                                const int32_t* __restrict__ sorted_vals,
                                const SortSeg* __restrict__ segs, int32_t* __restrict__ inv) {
  for (int g = blockIdx.y; g < ngrid; g += gridDim.y) {
    const JobDev& J = jobs[grid_jobs[g]];
    const int64_t out = gsegs[J.gseg].out_base;
    const int32_t* vb = sorted_vals + segs[J.sort_seg_b].out_base;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < J.len;
         p += (int64_t)gridDim.x * blockDim.x)
      inv[out + (vb[p] - J.seg_begin)] = (int32_t)p;
  }
}

// keys[out + p_A] = cell key of the point at column-0 position p_A; vals = p_A.
__global__ void grid_key_kernel(const JobDev* __restrict__ jobs,
                                const int32_t* __restrict__ grid_jobs, int ngrid,
                                const SortSeg* __restrict__ gsegs,
                                const int32_t* __restrict__ sorted_vals,
                                const SortSeg* __restrict__ segs,
                                const int32_t* __restrict__ inv, const int32_t* __restrict__ sub,
                                uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
  for (int g = blockIdx.y; g < ngrid; g += gridDim.y) {
    const JobDev& J = jobs[grid_jobs[g]];
    const int64_t out = gsegs[J.gseg].out_base;
    const int32_t* va = sorted_vals + segs[J.sort_seg].out_base;
    const int64_t len = J.len;
    const int nsub = J.nsub;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < len;
         p += (int64_t)gridDim.x * blockDim.x) {
      const int64_t w = va[p] - J.seg_begin;
      const int64_t strip = (int64_t)inv[out + w] * J.nstrips / len;
      keys[out + p] = (uint64_t)(nsub > 0 ? strip * nsub + sub[out + w] : strip);
      vals[out + p] = (int32_t)p;
    }
  }
}

// keys[out + r] = strip of the point at column-2 position r; vals = its offset.
__global__ void nest_key_kernel(const JobDev* __restrict__ jobs,
                                const int32_t* __restrict__ grid_jobs, int ngrid,
                                const SortSeg* __restrict__ gsegs,
                                const int32_t* __restrict__ sorted_vals,
                                const SortSeg* __restrict__ segs,
                                const int32_t* __restrict__ inv, uint64_t* __restrict__ keys,
                                int32_t* __restrict__ vals) {
  for (int g = blockIdx.y; g < ngrid; g += gridDim.y) {
    const JobDev& J = jobs[grid_jobs[g]];
    const int64_t out = gsegs[J.gseg].out_base;
    const int64_t len = J.len;
    const bool nested = J.nsub > 0;
    const int32_t* vc = nested ? sorted_vals + segs[J.sort_seg_c].out_base : nullptr;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < len;
         r += (int64_t)gridDim.x * blockDim.x) {
      if (nested) {
        const int32_t w = vc[r] - J.seg_begin;
        keys[out + r] = (uint64_t)((int64_t)inv[out + w] * J.nstrips / len);
        vals[out + r] = w;
      } else {
        keys[out + r] = 0;
        vals[out + r] = (int32_t)r;
      }
    }
  }
}

// After the strip pass over the column-2 order: position p2 of strip s1
// holds within-strip column-2 rank p2 - sstart[s1].
__global__ void nest_sub_kernel(const TaskDev* __restrict__ tasks,
                                const JobDev* __restrict__ jobs,
                                const int32_t* __restrict__ grid_jobs, int ngrid,
                                const SortSeg* __restrict__ gsegs,
                                const uint64_t* __restrict__ keys_sorted,
                                const int32_t* __restrict__ vals_sorted,
                                int32_t* __restrict__ sub) {
  for (int g = blockIdx.y; g < ngrid; g += gridDim.y) {
    const JobDev& J = jobs[grid_jobs[g]];
    if (J.nsub <= 0) continue;
    const TaskDev& t = tasks[J.task];
    const int64_t out = gsegs[J.gseg].out_base;
    const int nsub = J.nsub;
    const double* z = t.x64 + (int64_t)J.sp.cols[2] * t.ld + J.seg_begin;
    for (int64_t p2 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p2 < J.len;
         p2 += (int64_t)gridDim.x * blockDim.x) {
      const int s1 = (int)keys_sorted[out + p2];
      const int32_t w = vals_sorted[out + p2];
      const int32_t s0 = J.sstart[s1];
      const int32_t L = J.sstart[s1 + 1] - s0;
      const int c2 = (int)((p2 - s0) * nsub / L);
      sub[out + w] = c2;
      const int cell = s1 * nsub + c2;
      if (p2 == J.cstart[cell]) {
        J.czlo[cell] = z[w];
        J.czlo32[cell] = __double2float_rd(__dsub_rd(z[w], J.center[2]));
      }
      if (p2 == J.cstart[cell + 1] - 1) {
        J.czhi[cell] = z[w];
        J.czhi32[cell] = __double2float_ru(__dsub_ru(z[w], J.center[2]));
      }
    }
  }
}

dim3 grid_of(int ngrid, int64_t max_len) {
  int gx = (int)((max_len + 255) / 256);
  if (gx > 1024) gx = 1024;
  if (gx < 1) gx = 1;
  return dim3(gx, ngrid > 65535 ? 65535 : ngrid);
}

}  // namespace

void launch_grid_inv(const JobDev* jobs_d, const int32_t* grid_jobs_d, int ngrid,
                     const SortSeg* gsegs_d, const int32_t* sorted_vals, const SortSeg* segs_d,
                     int32_t* inv_scratch, int64_t max_len, cudaStream_t st) {
  if (ngrid <= 0) return;
  grid_inv_kernel<<<grid_of(ngrid, max_len), 256, 0, st>>>(jobs_d, grid_jobs_d, ngrid, gsegs_d,
                                                           sorted_vals, segs_d, inv_scratch);
  count_launch();
}

void launch_grid_key(const JobDev* jobs_d, const int32_t* grid_jobs_d, int ngrid,
                     const SortSeg* gsegs_d, const int32_t* sorted_vals, const SortSeg* segs_d,
                     const int32_t* inv_scratch, const int32_t* sub, uint64_t* gkeys,
                     int32_t* gvals, int64_t max_len, cudaStream_t st) {
  if (ngrid <= 0) return;
  grid_key_kernel<<<grid_of(ngrid, max_len), 256, 0, st>>>(jobs_d, grid_jobs_d, ngrid, gsegs_d,
                                                           sorted_vals, segs_d, inv_scratch, sub,
                                                           gkeys, gvals);
  count_launch();
}

void launch_nest_key(const JobDev* jobs_d, const int32_t* grid_jobs_d, int ngrid,
                     const SortSeg* gsegs_d, const int32_t* sorted_vals, const SortSeg* segs_d,
                     const int32_t* inv_scratch, uint64_t* keys, int32_t* vals, int64_t max_len,
                     cudaStream_t st) {
  if (ngrid <= 0) return;
  nest_key_kernel<<<grid_of(ngrid, max_len), 256, 0, st>>>(jobs_d, grid_jobs_d, ngrid, gsegs_d,
                                                           sorted_vals, segs_d, inv_scratch, keys,
                                                           vals);
  count_launch();
}

void launch_nest_sub(const TaskDev* tasks_d, const JobDev* jobs_d, const int32_t* grid_jobs_d,
                     int ngrid, const SortSeg* gsegs_d, const uint64_t* keys_sorted,
                     const int32_t* vals_sorted, int32_t* sub, int64_t max_len, cudaStream_t st) {
  if (ngrid <= 0) return;
  nest_sub_kernel<<<grid_of(ngrid, max_len), 256, 0, st>>>(tasks_d, jobs_d, grid_jobs_d, ngrid,
                                                           gsegs_d, keys_sorted, vals_sorted, sub);
  count_launch();
}

size_t sort_scan_tmp_elems(int nblk) {
  const int64_t n = (int64_t)256 * nblk;
  return (size_t)((n + SCAN_CHUNK - 1) / SCAN_CHUNK) + 1;
}

static void excl_scan(uint32_t* data, int64_t n, uint32_t* tmp, cudaStream_t st) {
  const int nchunks = (int)((n + SCAN_CHUNK - 1) / SCAN_CHUNK);
  scan_reduce_kernel<<<nchunks, SCAN_THREADS, 0, st>>>(data, n, tmp);
  count_launch();
  scan_top_kernel<<<1, SCAN_THREADS, 0, st>>>(tmp, nchunks);
  count_launch();
  scan_down_kernel<<<nchunks, SCAN_THREADS, 0, st>>>(data, n, tmp);
  count_launch();
}

int init_sort_kernels() {
  return (int)cudaFuncSetAttribute(onesweep_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sizeof(OsSmem));
}

size_t sort_sweep_bytes(int os_nblk, int nseg) {
  return sizeof(unsigned long long) * 256 * (size_t)std::max(os_nblk, 1) +
         sizeof(uint32_t) * OS_PASSES * 256 * (size_t)std::max(nseg, 1) + 64;
}

void launch_sort(const TaskDev* tasks_d, const SortSeg* segs_d, const int32_t* blk_seg_d,
                 int nblk, const int32_t* os_blk_seg_d, int os_nblk, int nseg, uint64_t* keys_a,
                 uint64_t* keys_b, int32_t* vals_a, int32_t* vals_b, void* sweep, int first,
                 uint32_t* err, cudaStream_t st, cudaEvent_t* pass_events) {
  if (nblk <= 0 || os_nblk <= 0) return;
  // sweep (zeroed by the caller): flag words, segment digit totals, tile counters
  unsigned long long* flags = (unsigned long long*)sweep;
  uint32_t* seg_hist = (uint32_t*)(flags + 256 * (size_t)os_nblk);
  int* counters = (int*)(seg_hist + OS_PASSES * 256 * (size_t)std::max(nseg, 1));
  onesweep_load_kernel<<<nblk, SORT_THREADS, 0, st>>>(tasks_d, segs_d, blk_seg_d, keys_a, vals_a,
                                                     seg_hist, first);
  count_launch();
  uint64_t* kin = keys_a;
  uint64_t* kout = keys_b;
  int32_t* vin = vals_a;
  int32_t* vout = vals_b;
  if (pass_events) cudaEventRecord(pass_events[0], st);
  for (int pass = first; pass < OS_PASSES; ++pass) {
    onesweep_pass_kernel<<<os_nblk, OS_THREADS, sizeof(OsSmem), st>>>(
        segs_d, os_blk_seg_d, kin, vin, kout, vout, pass, seg_hist, flags, counters + pass, err);
    count_launch();
    uint64_t* tk = kin; kin = kout; kout = tk;
    int32_t* tv = vin; vin = vout; vout = tv;
  }
  if (pass_events) cudaEventRecord(pass_events[1], st);
  // an even number of passes: the sorted keys and values are back in
  // keys_a / vals_a
  if (first > 0) {
    tie_fix_kernel<<<nblk, SORT_THREADS, 0, st>>>(segs_d, blk_seg_d, keys_a, vals_a, err);
    count_launch();
  }
}

void launch_radix_pass(const SortSeg* segs_d, const int32_t* blk_seg_d, int nblk,
                       const uint64_t* kin, const int32_t* vin, uint64_t* kout, int32_t* vout,
                       int shift, uint32_t* hist, uint32_t* scan_tmp, cudaStream_t st) {
  if (nblk <= 0) return;
  sort_hist_kernel<<<nblk, SORT_THREADS, 0, st>>>(segs_d, blk_seg_d, kin, shift, hist);
  count_launch();
  excl_scan(hist, (int64_t)256 * nblk, scan_tmp, st);
  sort_scatter_kernel<<<nblk, SORT_THREADS, 0, st>>>(segs_d, blk_seg_d, kin, vin, shift, hist,
                                                     kout, vout);
  count_launch();
}

void launch_sorted_jobs(const TaskDev* tasks_d, const SortedJob* jobs_d, int njobs,
                        int total_blocks, const KeyIndex& kx, const int32_t* perm, cudaStream_t st) {
  if (njobs <= 0 || total_blocks <= 0) return;
  sorted_jobs_kernel<<<(unsigned)total_blocks, SORTED_THREADS, 0, st>>>(tasks_d, jobs_d, njobs, kx,
                                                                        perm);
  count_launch();
}

}  // namespace egb
