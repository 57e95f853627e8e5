// egb_knn.cu -- dispatch of the tile kernels, and the any-K selection kernel.
//
// knn_select_kernel handles k+1 above the register lists of the tile kernels
// (k >= 32): one warp per query finds the K-th smallest FP64 max-norm
// distance by an 8-pass radix select over the bit pattern of the distance
// (non-negative doubles order like their bits), 8 bits per pass with a
// 256-bin shared-memory histogram per warp.  Exact; O(8 * len) distance
// evaluations per query, so it serves the large-k cases of the reference
// (k = 50, 100 in tests/integration/test_unbiasedness.py) at moderate N.
#include "egb_internal.cuh"

namespace egb {

template <bool PLAIN, bool SLAB>
TileShape knn_shape_v(int kclass, int dclass, int dmax);
template <bool PLAIN, bool SLAB>
void launch_knn_v(int kclass, int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                  int* counter, uint32_t* err, int dmax, DeferEntry* df, int* dc, int num_sms,
                  cudaStream_t st);
template <bool PLAIN>
void launch_knn_defer_v(int kclass, int dclass, const JobDev* jobs, const DeferEntry* list,
                        const int* count, int cap, int num_sms, cudaStream_t st);

TileShape count_shape_f32b(int, int);
TileShape count_shape_f32s(int, int);
TileShape count_shape_f64b(int, int);
TileShape count_shape_f64s(int, int);
void launch_count_f32b(int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                       DeferEntry*, int*, int, cudaStream_t);
void launch_count_f32s(int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                       DeferEntry*, int*, int, cudaStream_t);
void launch_count_f64b(int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                       DeferEntry*, int*, int, cudaStream_t);
void launch_count_f64s(int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                       DeferEntry*, int*, int, cudaStream_t);
void count_defer_f32s(int, const JobDev*, const DeferEntry*, const int*, int, int, cudaStream_t);
void count_defer_f64s(int, const JobDev*, const DeferEntry*, const int*, int, int, cudaStream_t);

TileShape grid_shape_f32(int, int);
TileShape grid_shape_f64(int, int);
void launch_knn_grid_f32(int, int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                         DeferEntry*, int*, int, cudaStream_t);
void launch_knn_grid_f64(int, int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                         DeferEntry*, int*, int, cudaStream_t);
void launch_count_grid_f32(int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                           DeferEntry*, int*, int, cudaStream_t);
void launch_count_grid_f64(int, const JobDev*, const WorkItem*, int, int*, uint32_t*, int,
                           DeferEntry*, int*, int, cudaStream_t);

void launch_knn_wgrid_f32(int, int, const JobDev*, const WorkItem*, int, int*, int, int, cudaStream_t);
void launch_knn_wgrid_f64(int, int, const JobDev*, const WorkItem*, int, int*, int, int, cudaStream_t);
void launch_count_wgrid_f32(int, const JobDev*, const WorkItem*, int, int*, int, int, cudaStream_t);
void launch_count_wgrid_f64(int, const JobDev*, const WorkItem*, int, int*, int, int, cudaStream_t);

void launch_knn_wgrid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                      int dclass, int plain, int dmax, int* counter, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  // the FP32 path walks per lane (egb_wwalk.cu); the FP64 comparator keeps
  // the warp-window kernel
  if (plain) launch_knn_wgrid_f64(kclass, dclass, jobs_d, items_d, nitems, counter, dmax, num_sms, st);
  else launch_knn_walk(jobs_d, items_d, nitems, kclass, dclass, counter, num_sms, st);
}

void launch_count_wgrid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                        int plain, int dmax, int* counter, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  if (plain) launch_count_wgrid_f64(dclass, jobs_d, items_d, nitems, counter, dmax, num_sms, st);
  else launch_count_wgrid_f32(dclass, jobs_d, items_d, nitems, counter, dmax, num_sms, st);
}

TileShape grid_shape(int dclass, int plain, int dmax) {
  return plain ? grid_shape_f64(dclass, dmax) : grid_shape_f32(dclass, dmax);
}

void launch_knn_grid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                     int dclass, int plain, int dmax, int* counter, uint32_t* err,
                     DeferEntry* defer, int* defer_count, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  if (plain) launch_knn_grid_f64(kclass, dclass, jobs_d, items_d, nitems, counter, err, dmax, defer, defer_count, num_sms, st);
  else launch_knn_grid_f32(kclass, dclass, jobs_d, items_d, nitems, counter, err, dmax, defer, defer_count, num_sms, st);
}

void launch_count_grid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                       int plain, int dmax, int* counter, uint32_t* err, DeferEntry* defer,
                       int* defer_count, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  if (plain) launch_count_grid_f64(dclass, jobs_d, items_d, nitems, counter, err, dmax, defer, defer_count, num_sms, st);
  else launch_count_grid_f32(dclass, jobs_d, items_d, nitems, counter, err, dmax, defer, defer_count, num_sms, st);
}

TileShape knn_shape(int kclass, int dclass, int plain, int slab, int dmax) {
  if (plain) return slab ? knn_shape_v<true, true>(kclass, dclass, dmax)
                         : knn_shape_v<true, false>(kclass, dclass, dmax);
  return slab ? knn_shape_v<false, true>(kclass, dclass, dmax)
              : knn_shape_v<false, false>(kclass, dclass, dmax);
}

void launch_knn_tile(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                     int dclass, int plain, int slab, int dmax, int* counter, uint32_t* err,
                     DeferEntry* df, int* dc, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  if (plain) {
    if (slab) launch_knn_v<true, true>(kclass, dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
    else launch_knn_v<true, false>(kclass, dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
  } else {
    if (slab) launch_knn_v<false, true>(kclass, dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
    else launch_knn_v<false, false>(kclass, dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
  }
}

void launch_knn_defer(const JobDev* jobs_d, const DeferEntry* defer, const int* defer_count,
                      int defer_cap, int kclass, int dclass, int plain, int num_sms,
                      cudaStream_t st) {
  if (defer_cap <= 0) return;
  if (plain) launch_knn_defer_v<true>(kclass, dclass, jobs_d, defer, defer_count, defer_cap, num_sms, st);
  else launch_knn_defer_v<false>(kclass, dclass, jobs_d, defer, defer_count, defer_cap, num_sms, st);
}

TileShape count_shape(int dclass, int plain, int slab, int dmax) {
  if (plain) return slab ? count_shape_f64s(dclass, dmax) : count_shape_f64b(dclass, dmax);
  return slab ? count_shape_f32s(dclass, dmax) : count_shape_f32b(dclass, dmax);
}

void launch_count_tile(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                       int plain, int slab, int dmax, int* counter, uint32_t* err,
                       DeferEntry* df, int* dc, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  if (plain) {
    if (slab) launch_count_f64s(dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
    else launch_count_f64b(dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
  } else {
    if (slab) launch_count_f32s(dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
    else launch_count_f32b(dclass, jobs_d, items_d, nitems, counter, err, dmax, df, dc, num_sms, st);
  }
}

void launch_count_defer(const JobDev* jobs_d, const DeferEntry* defer, const int* defer_count,
                        int defer_cap, int dclass, int plain, int num_sms, cudaStream_t st) {
  if (defer_cap <= 0) return;
  if (plain) count_defer_f64s(dclass, jobs_d, defer, defer_count, defer_cap, num_sms, st);
  else count_defer_f32s(dclass, jobs_d, defer, defer_count, defer_cap, num_sms, st);
}

namespace {

__global__ void __launch_bounds__(SELECT_WARPS * 32)
knn_select_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items,
                  int nitems) {
  __shared__ uint32_t hist[SELECT_WARPS][256];
  __shared__ double qsm[SELECT_WARPS][EGB_DMAX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x;
  if (item >= nitems) return;
  const WorkItem wi = items[item];
  const JobDev* jb = jobs + wi.job;
  const int qp = wi.q0 + warp;
  const int len = jb->len;
  if (qp >= len) return;  // whole warp leaves; no block-wide barrier below
  const int d = jb->sp.d;
  const int K = jb->K;
  const int64_t lds = jb->lds;
  const double* __restrict__ c64 = jb->c64;
  double* out = jb->eps + jb->idx[qp];
  if (len < K) {
    if (lane == 0) *out = __longlong_as_double((long long)INF_BITS);
    return;
  }
  if (lane < d) qsm[warp][lane] = c64[(int64_t)lane * lds + qp];
  __syncwarp();
  uint64_t prefix = 0, mask = 0;
  uint32_t rank = (uint32_t)K;  // 1-based rank among candidates matching prefix
#pragma unroll 1
  for (int pass = 0; pass < 8; ++pass) {
    const int shift = 56 - 8 * pass;
    for (int b = lane; b < 256; b += 32) hist[warp][b] = 0u;
    __syncwarp();
    for (int j = lane; j < len; j += 32) {
      uint64_t m = 0;
      for (int c = 0; c < d; ++c) {
        const uint64_t v = absdiff_bits(c64[(int64_t)c * lds + j], qsm[warp][c]);
        m = v > m ? v : m;
      }
      if ((m & mask) == prefix) atomicAdd(&hist[warp][(m >> shift) & 255u], 1u);
    }
    __syncwarp();
    uint32_t loc[8];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      loc[i] = hist[warp][8 * lane + i];
      s += loc[i];
    }
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t excl = incl - s;
    const unsigned hit = __ballot_sync(0xffffffffu, excl < rank && rank <= incl);
    const int src = __ffs(hit) - 1;
    int digit = 0;
    uint32_t before = 0;
    if (lane == src) {
      uint32_t run = excl;
      bool found = false;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (!found && run + loc[i] >= rank) {
          digit = 8 * lane + i;
          before = run;
          found = true;
        }
        run += loc[i];
      }
    }
    digit = __shfl_sync(0xffffffffu, digit, src < 0 ? 0 : src);
    before = __shfl_sync(0xffffffffu, before, src < 0 ? 0 : src);
    prefix |= (uint64_t)digit << shift;
    mask |= 255ull << shift;
    rank -= before;
    __syncwarp();
  }
  if (lane == 0) *out = bits_to_double(prefix);
}

}  // namespace

void launch_knn_select(const JobDev* jobs_d, const WorkItem* items_d, int nitems, uint32_t* err,
                       int num_sms, cudaStream_t st) {
  (void)err;
  (void)num_sms;
  if (nitems <= 0) return;
  knn_select_kernel<<<nitems, SELECT_WARPS * 32, 0, st>>>(jobs_d, items_d, nitems);
  count_launch();
}

}  // namespace egb
