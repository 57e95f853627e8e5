// egb_internal.cuh -- device structures and helpers shared by the kernels of
// libennemi_gb.so.
//
// Layout of one batch in HBM (all inside one arena):
//   * task t owns ncol_t float64 columns in *working order* (samples of a
//     class-partitioned task grouped by class, stable); column c lives at
//     x64 + c*ld with ld a multiple of 32 elements, so every column start is
//     256-byte aligned relative to the arena;
//   * eps[ld] (float64), rad[ld] = fl64(eps - 1e-12) or a caller radius, and
//     up to three int32 count arrays cnt[s][ld];
//   * per sorted 1-D space: the order-preserving uint64 keys and the working
//     index of each key, concatenated over all spaces of the batch;
//   * per multi-D job: its columns copied into one SoA block (see JobDev),
//     with an FP32 copy fl32(x - center_c) (center_c = the task column's
//     midrange) read by the FP32 distance filters.
// All distances are max-norm.  Every decision that fixes a neighbour count or
// a k-th distance is taken on the exact FP64 distance max_c fl64(|a_c - b_c|)
// -- the value scipy's cKDTree compares -- either directly or behind an FP32
// filter whose guard band is proven below (band()).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define EGB_DMAX 32        // most columns in one space
#define EGB_KREG_MAX 32    // largest k+1 kept in registers by the tile kernels

namespace egb {

// Device-side error word: kernels OR bits in, the host reads it after a batch.
enum DevErr : uint32_t {
  DERR_NONE = 0,
  DERR_WAIT_TIMEOUT = 1u << 0,  // a bounded mbarrier wait gave up
  DERR_BAD_INDEX = 1u << 1,     // an index guard tripped
  DERR_SORT_TIES = 1u << 2,     // keys equal in their high 48 bits need the
                                // full sort: the host runs the batch again
};

// Per-job flag bits (JobDev::jflags).
enum JobFlag : uint32_t {
  TF_UNSAFE32 = 1u << 0,  // some centred value does not fit FP32 comfortably:
                          // every candidate of the job is checked in FP64
};

// ------------------------------------------------------------ key helpers --
// Order-preserving map float64 -> uint64 (after folding -0.0 into +0.0).
__host__ __device__ __forceinline__ uint64_t key_of(double v) {
  v = v + 0.0;  // -0.0 + 0.0 = +0.0 in round-to-nearest
  uint64_t u;
#ifdef __CUDA_ARCH__
  u = (uint64_t)__double_as_longlong(v);
#else
  __builtin_memcpy(&u, &v, 8);
#endif
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double value_of(uint64_t k) {
  uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
#ifdef __CUDA_ARCH__
  v = __longlong_as_double((long long)u);
#else
  __builtin_memcpy(&v, &u, 8);
#endif
  return v;
}

// A count radius by its bits, with integer compares (GB300 issues FP64,
// comparisons included, at a few operations per clock per SM): 0 = no ball
// (negative or NaN: the count is 0), 1 = finite and >= 0 (-0 included),
// 2 = +inf (every point).
__host__ __device__ __forceinline__ int radius_class(double r) {
  uint64_t u;
#ifdef __CUDA_ARCH__
  u = (uint64_t)__double_as_longlong(r);
#else
  __builtin_memcpy(&u, &r, 8);
#endif
  if (u == 0x7ff0000000000000ull) return 2;
  if (u < 0x7ff0000000000000ull || u == 0x8000000000000000ull) return 1;
  return 0;
}

#ifdef __CUDACC__
// Smallest float >= the non-negative double with bit pattern u (integer
// operations only: GB300 issues FP64 at 2 lanes per clock per SM, so this
// keeps conversions off that pipe).
__device__ __forceinline__ float f32_up_of_bits(uint64_t u) {
  const int e = (int)(u >> 52);                       // biased exponent (sign is 0)
  if (e >= 1023 + 128) return __int_as_float(0x7f800000);
  if (e < 1023 - 126) return __int_as_float(0x00800000);  // 2^-126 bounds it
  const uint64_t mant = u & 0xfffffffffffffull;
  uint32_t b = ((uint32_t)(e - 1023 + 127) << 23) | (uint32_t)(mant >> 29);
  b += (mant & 0x1fffffffull) ? 1u : 0u;              // carry into the exponent is exact
  return __int_as_float((int)b);
}

// fl64(|a - b|) as the bit pattern of a non-negative double.  Non-negative
// doubles order like their bit patterns, so the max over coordinates and the
// comparisons run on the integer pipe; only the subtraction is FP64.
__device__ __forceinline__ uint64_t absdiff_bits(double a, double b) {
  return (uint64_t)__double_as_longlong(a - b) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ double bits_to_double(uint64_t u) {
  return __longlong_as_double((long long)u);
}

// Order-preserving integer image of a double's bit pattern (raw: -0 sorts
// just below +0) and its inverse.
__device__ __forceinline__ uint64_t raw_key(uint64_t u) {
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double raw_value(uint64_t k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// Raw keys [kl, kr] of the doubles x with fl64(|x - q|) <= r, for q and r
// finite, r >= 0.  x -> fl64(x - q) is monotone (rounding is), so the set
// is one key range.  Its ends usually lie an ulp or two from fl64(q -+ r),
// but where q -+ r is much smaller in magnitude than q many doubles share
// one fl64 difference, so each end is found by galloping from there and
// bisecting on the exact predicate (at most about 128 FP64 steps).
__device__ __forceinline__ void ball_keys(double q, double r, uint64_t& kl, uint64_t& kr) {
  // right end: largest k with value(k) - q <= r
  {
    uint64_t k = raw_key((uint64_t)__double_as_longlong(q + r));
    auto P = [&](uint64_t x) { return raw_value(x) - q <= r; };
    uint64_t good, bad;  // P(good), !P(bad), good < bad
    if (P(k)) {
      good = k;
      uint64_t step = 1;
      for (;;) {
        const uint64_t nx = good + step;
        if (nx < good || !P(nx)) {
          bad = nx < good ? ~0ull : nx;
          break;
        }
        good = nx;
        step <<= 1;
      }
    } else {
      bad = k;
      uint64_t step = 1;
      for (;;) {
        const uint64_t nx = bad - step;
        if (P(nx)) {  // value(key(q)) - q = 0 <= r bounds the walk
          good = nx;
          break;
        }
        bad = nx;
        step <<= 1;
      }
    }
    while (bad - good > 1) {
      const uint64_t m = good + ((bad - good) >> 1);
      if (P(m)) good = m; else bad = m;
    }
    kr = good;
  }
  // left end: smallest k with q - value(k) <= r
  {
    uint64_t k = raw_key((uint64_t)__double_as_longlong(q - r));
    auto Q = [&](uint64_t x) { return q - raw_value(x) <= r; };
    uint64_t good, bad;  // Q(good), !Q(bad), bad < good
    if (Q(k)) {
      good = k;
      uint64_t step = 1;
      for (;;) {
        const uint64_t nx = good - step;
        if (nx > good || !Q(nx)) {
          bad = nx > good ? 0ull : nx;
          break;
        }
        good = nx;
        step <<= 1;
      }
    } else {
      bad = k;
      uint64_t step = 1;
      for (;;) {
        const uint64_t nx = bad + step;
        if (Q(nx)) {
          good = nx;
          break;
        }
        bad = nx;
        step <<= 1;
      }
    }
    while (good - bad > 1) {
      const uint64_t m = bad + ((good - bad) >> 1);
      if (Q(m)) good = m; else bad = m;
    }
    kl = good;
  }
}

// FP32 guard band.
// Let c be a column centre (a double), q the query, p a candidate, and
// D = max_c |p_c - q_c| the exact max-norm distance.  The filter works on
// f = fl32(fl64(v - c)) per coordinate and d32 = max_c fl32(|f_p - f_q|).
// With u = 2^-24 and M = max_c |q_c - c|:
//   |f - (v - c)| <= (u + 2^-53 + u 2^-53)|v - c| + 2^-150   (subnormals),
//   |p_c - c| <= M + D,   |q_c - c| <= M,
//   the FP32 subtraction adds at most u |f_p - f_q|,
// so |d32 - D| <= 2^-23 (M + D)(1 + 2^-20) + 2^-148, and the FP64 distance
// fl64(D) is within 2^-53 D of D.  band(M, t) = 2^-21 (M + t) + 2^-100 is
// four times that bound for every D <= t (1 + 2^-20):
//   kNN:    a candidate with fl64 distance < t has d32 <= t + band(M, t);
//   counts: d32 <= r - band(M, r)  =>  fl64 distance <= r,
//           d32 >  r + band(M, r)  =>  fl64 distance >  r.
// Everything in between is decided in FP64.
__device__ __forceinline__ double band(double m, double t) {
  return 0x1p-21 * (m + t) + 0x1p-100;
}
#endif

constexpr uint64_t INF_BITS = 0x7ff0000000000000ull;

// ------------------------------------------------------------ job structs --
struct TaskDev {          // per-task device view
  const double* x64;      // working FP64 columns, column c at x64 + c*ld
  const double* center;   // [ncol] column midranges (FP32 copies are x - center)
  double* eps;            // [ld]
  double* rad;            // [ld] count radius per sample
  int32_t* cnt[4];        // count slots (working order)
  int64_t ld;
  int32_t n;
  int32_t ncol;
  int32_t rad_given;      // 1: rad holds caller radii (egb_ball_count)
  int32_t pad_;
};

struct SpaceCols {        // the columns of one (sub)space of a task
  int32_t d;
  int8_t cols[EGB_DMAX];
};

// A multi-D job: the samples [seg_begin, seg_end) of one task restricted to
// the columns `sp`, materialised as a contiguous structure-of-arrays block
// (FP64 and FP32 copies, column c at +c*lds).  Brute-force jobs keep working
// order; slab jobs are sorted by their first column, so that the candidates
// within distance t of a query lie in a contiguous run around it.  Queries
// and candidates are the same point set (every kNN and ball-count query of
// the reference searches the set it belongs to).
struct JobDev {
  double* c64;            // [d][lds]
  float* c32;             // [d][lds] fl32(c64 - center)
  int32_t* idx;           // [lds] position -> working index of the task
  double* center;         // [d]
  uint32_t* jflags;       // TF_* bits of this job (set by materialise)
  double* eps;            // task eps  (kNN: written; counts: unused)
  const double* rad;      // task radius (counts)
  int32_t* cnt;           // task count slot (counts)
  int64_t lds;
  int32_t task;
  int32_t seg_begin;
  int32_t len;            // seg_end - seg_begin
  int32_t K;              // k + 1 (kNN) or 0 (count)
  int32_t slab;           // 1: sorted by the first column
  int32_t sort_seg;       // slab: index of the sort segment of column 0
  int32_t sort_seg_b;     // slab: sort segment of column 1 (second order)
  int32_t kform;          // grid copy holds order-preserving keys, not values:
                          // column c's high words at (uint32*)c64g + 2c*lds,
                          // low words at + (2c+1)*lds (key-range count jobs)
  // slab jobs: a second copy sorted by column 1, scanned by deferred queries
  // whose column-1 slab is narrower than their column-0 slab
  double* c64b;
  float* c32b;
  int32_t* idxb;
  // grid jobs: a third copy in strip order -- the points split into nstrips
  // equal-count strips by their rank in column 1, each strip sorted by
  // column 0 -- with, per position, its position in the column-0 order
  double* c64g;
  float* c32g;
  int32_t* idxg;
  int32_t* posg;
  int32_t nstrips;
  int32_t gseg;           // grid: its segment in the strip-key sort
  const int32_t* sstart;  // grid: nstrips + 1 strip starts (strip_start table)
  double* sylo;           // grid: smallest column-1 value of each strip
  double* syhi;           // grid: largest column-1 value of each strip
  // nested grid (warp-grid jobs of d >= 3): every strip split again into nsub
  // equal-count cells by the rank of column 2 within the strip, each cell
  // sorted by column 0; nsub == 0 for plain strips
  int32_t nsub;
  int32_t sort_seg_c;     // nested: sort segment of column 2
  const int32_t* cstart;  // nstrips * nsub + 1 cell starts (cell_start table)
  double* czlo;           // smallest column-2 value of each cell
  double* czhi;           // largest column-2 value of each cell
  // the strip and cell bounds centred and rounded outward to FP32
  // (lower bounds down, upper bounds up): the FP32 kernels plan on these
  float* sylo32;
  float* syhi32;
  float* czlo32;
  float* czhi32;
  // work counters of this job's launch group: [0] pairs screened by tile
  // items, [1] pairs screened by deferred-query warps, [2] queries deferred
  unsigned long long* stats;
  SpaceCols sp;
};

// Strip s of a grid job of length len holds the column-1 ranks
// [strip_start(s), strip_start(s + 1)).
__host__ __device__ __forceinline__ int32_t strip_start(int64_t s, int64_t len, int32_t nstrips) {
  return (int32_t)((s * len + nstrips - 1) / nstrips);
}
// Cell c2 of a strip starting at s0 with length L holds the within-strip
// column-2 ranks [strip_start(c2, L, nsub), strip_start(c2 + 1, L, nsub)).
__host__ __device__ __forceinline__ int32_t cell_start(int32_t s0, int32_t L, int32_t c2,
                                                       int32_t nsub) {
  return s0 + strip_start(c2, L, nsub);
}
constexpr int NEST_CELL_3D = 384;     // target points per nested-grid cell, kNN jobs of d = 3
constexpr int NEST_CELL_4D = 256;     // the same for d >= 4 (measured best for each)
constexpr int NEST_CELL_COUNT = 768;  // the same for count jobs, which also take at least
constexpr double NEST_SIDE_C = 1.07;  // NEST_SIDE_C * len^(1/dj) cells per side (dj: see strips)
constexpr int GRID_QB = 128;     // queries per grid work item
constexpr int GRID_TILE = 128;   // candidates per grid tile
constexpr int GRID_MIN_STRIP = 64;
// Strips of a 2-D warp-grid job: about c * len^(1/dj), dj the dimension of
// the kNN search that sets the job's radii (the job's own for a kNN job, the
// task's joint space for a count job), so that a strip stays a few ball widths
// wide (balls shrink as len^(-1/dj)).  c measured on GB300: 500 kNN strips
// and 128 count strips (3-D joint kNN) at 1e6 points.
constexpr double GRID_STRIPS_KNN_C = 0.5;
constexpr double GRID_STRIPS_COUNT_C = 1.28;
constexpr int GRID_STRIPS_MAX = 1024;

struct WorkItem {         // one tile of queries of one job
  int32_t job;
  int32_t q0;
  int32_t q1;             // grid items: end of the query range (exclusive)
  int32_t strip;          // grid items: the strip holding the queries (nested
                          // grids: strip | cell << 16)
};

// Grid work items built on the device (launch_emit_items): per grid job of a
// launch group, its cells -- strips, or strips x cells when nested -- in
// order; cell c of the run holds the group's items [cum[cum0 + c],
// cum[cum0 + c + 1]), each of up to qb consecutive positions.
struct ItemRun {
  int32_t job;
  int32_t ncell;
  int32_t cum0;   // offset of the run's ncell + 1 item offsets in cum[]
  int32_t qb;     // queries per item
  int64_t cell0;  // index of the run's first cell among the group's cells
};

// A slab query whose search a tile work item left unfinished (it needed a
// much wider window than the rest of its item); finished one warp per query.
struct DeferEntry {
  int32_t job;
  int32_t pos;      // position in the job's first-column order
  double tb;        // upper bound of the query's threshold (kNN: K-th distance
                    // so far; counts: the radius)
};
constexpr int DEFER_FRAC = 8;    // an item stops when <= 1/8 of its threads
                                 // still have unfinished queries
constexpr int SIDE_CAP = 128;    // ... or after this many tiles beyond home

// 1-D jobs on sorted arrays: one thread per sorted position.
struct SortedJob {
  int32_t task;
  int32_t kind;           // 0 = kNN (writes eps), 1 = count (writes cnt[slot])
  int32_t slot;
  int32_t K;              // k + 1 for kNN
  int64_t base;           // offset of the sorted segment in the key buffer
  int64_t s1_base;        // its samples (egb_search.cuh)
  int64_t s2_base;
  int32_t len;            // its length
  int32_t blk0;           // first block of this job in the launch
  int2* ranges;           // count jobs: [lo, hi) of each query's ball in the
                          // segment, by working index (null: not kept), for
                          // the rank-space counts whose b order it is
};

struct SortSeg {          // one segment of the batched radix sort
  int64_t out_base;       // offset into the concatenated key buffer
  int64_t s1_base;        // offset of its samples keys[32 j] (egb_search.cuh)
  int64_t s2_base;        // offset of its samples keys[1024 j]
  int32_t len;
  int32_t blk0;           // first tile (block) of the segment
  int32_t nblk;
  int32_t task;
  int32_t col;            // source column of the task
  int32_t src_begin;      // first working index of the segment
  int32_t os_blk0;        // its first tile of the single-sweep passes (OS_TILE keys)
  int32_t os_nblk;
};

struct GatherCol {        // working column <- caller column (strided, permuted)
  const double* src;
  int64_t stride;
  const int32_t* perm;    // working -> caller index, or null (identity)
  int32_t task;
  int32_t col;
};

// Device rescale (EGB_RESCALE).  A column's sum in NumPy's pairwise order
// is a tree: leaves of at most 128 samples summed with eight accumulators,
// inner nodes the sum of their two children.  Nodes of one tree are stored
// leaves first ((offset, length) in .x/.y), then inner nodes by height
// ((left, right) child), heights 1 .. nlvl starting at levels[lvl0 + h - 1]
// (local node indices; levels[lvl0 + nlvl] = nnode).  The root is the last.
struct PwTree {
  int32_t node0, nleaf, nnode, lvl0, nlvl;
};
struct RescaleStat {      // one distinct column of the batch: its mean and std
  int32_t task, col;      // a task column holding it (working order)
  int32_t tree;           // its summation tree (group == 1)
  int32_t group;          // > 1: one of `group` condition columns, which NumPy
                          // reduces along axis 0 -- row by row, in order
  int64_t scratch;        // first node-sum slot (tree.nnode doubles)
  const int32_t* inv;     // sample -> working position (class-ordered tasks), or null
};
struct RescaleCol {       // one task column to rescale in place
  int32_t task, col;
  int32_t stat;           // its RescaleStat
  int32_t group;          // noise stride: condition columns of an n x group array
  int64_t noise_pos;      // noise value of the column's first sample
  const int32_t* inv;
};
// zero_flags bit of a task with a column whose standard deviation was below
// 1e-20: left as given, the task is reported EGB_TASK_CONSTANT
constexpr uint32_t RESCALE_CONSTANT = 1u << 31;
// stats: one block per distinct column -> ms[u] = (mean, std); then one block
// per task column: x = (x - mean) / std + noise
void launch_rescale(const TaskDev* tasks_d, const RescaleStat* stats_d, int nstats,
                    const RescaleCol* cols_d, int ncols, const PwTree* trees_d,
                    const int2* nodes_d, const int32_t* levels_d, double* scratch, double2* ms,
                    const double* noise, uint32_t* zero_flags, int64_t max_n, cudaStream_t st);
// egb_debug_divide: the rescale's division (div_rn) over n pairs
void launch_divide(const double* a_d, const double* b_d, int64_t n, double* out_d, cudaStream_t st);

struct CombineJob {       // per-task reduction of per-sample terms
  int32_t task;
  int32_t kind;           // egb_kind
  int32_t chunk0;         // first partial-sum slot of the task
  int32_t nchunk;
};
constexpr int COMBINE_CHUNK = 4096;

// Kernels launched by this library since the counter was last read (every
// <<<>>> site calls count_launch(); the planner reports the count per batch).
void count_launch();

// ----------------------------------------------------------- entry points --
// Launch wrappers implemented in the kernel translation units.  Every wrapper
// launches on `st` and never synchronises.

// egb_prep.cu
void launch_gather(const TaskDev* tasks_d, const GatherCol* cols_d, int ncols,
                   int64_t max_ld, cudaStream_t st);
void launch_prepare(const TaskDev* tasks_d, const int32_t* col_task_d, const int32_t* col_idx_d,
                    int ncols_total, int64_t max_n, unsigned long long* minmax_d,
                    double* centers_d, cudaStream_t st);
void launch_materialize(const TaskDev* tasks_d, const JobDev* jobs_d, int njobs,
                        const int32_t* sorted_vals, const SortSeg* segs_d, int64_t max_lds,
                        cudaStream_t st);
void launch_materialize_grid(const TaskDev* tasks_d, const JobDev* jobs_d,
                             const int32_t* grid_jobs_d, int ngrid, const int32_t* sorted_vals,
                             const SortSeg* segs_d, const int32_t* gvals_sorted,
                             const SortSeg* gsegs_d, int64_t max_lds, cudaStream_t st);
void launch_radius(const TaskDev* tasks_d, int ntasks, int64_t max_ld, cudaStream_t st);
void launch_emit_items(const JobDev* jobs_d, const ItemRun* runs_d, int nruns, const int32_t* cum_d,
                       int64_t nitems, WorkItem* items_d, cudaStream_t st);
void launch_combine(const TaskDev* tasks_d, const CombineJob* jobs_d, const int32_t* chunk_job_d,
                    int nchunks, const double* psi_tab, int64_t psi_len, double* partial,
                    uint32_t* zero_flags, uint32_t* err, cudaStream_t st);

// egb_sort.cu
constexpr int SORT_TILE = 2048;
constexpr int OS_TILE = 4096;   // keys per tile of the batch sort's single-sweep passes
// The batch's sorted keys and the arrays searched in their place: each
// key's value rounded down to FP32 (exact comparisons against FP32 bounds in
// half the bytes), and samples of both (egb_search.cuh), at each segment's
// out_base / s1_base / s2_base.
struct KeyIndex {
  const uint64_t* keys;   // sorted keys of every segment (key_of)
  const float* fkeys;     // the largest float <= each key's value
  const uint64_t* s1;     // keys[32 j]
  const uint64_t* s2;     // keys[1024 j]
  const float* fs1;       // fkeys[32 j]
  const float* fs2;       // fkeys[1024 j]
};
// Strip keys of the grid jobs.  launch_grid_inv: inv[p_B] = column-1 rank
// of each point (by working offset).  launch_grid_key: keys[p] = cell key of
// the point at column-0 position p -- its strip (column-1 rank * nstrips /
// len), times nsub plus its cell (nested grids, from sub[]) -- and vals[p] =
// p; stable 8-bit radix passes then order each segment by (key, column 0).
void launch_grid_inv(const JobDev* jobs_d, const int32_t* grid_jobs_d, int ngrid,
                     const SortSeg* gsegs_d, const int32_t* sorted_vals, const SortSeg* segs_d,
                     int32_t* inv_scratch, int64_t max_len, cudaStream_t st);
void launch_grid_key(const JobDev* jobs_d, const int32_t* grid_jobs_d, int ngrid,
                     const SortSeg* gsegs_d, const int32_t* sorted_vals, const SortSeg* segs_d,
                     const int32_t* inv_scratch, const int32_t* sub, uint64_t* gkeys,
                     int32_t* gvals, int64_t max_len, cudaStream_t st);
// Nested grids.  launch_nest_key: over the column-2 order of each nested job,
// keys[r] = strip of the point at column-2 position r, vals[r] = its working
// offset (non-nested jobs: zeros).  After one stable radix pass (strips in
// column-2 order), launch_nest_sub: sub[w] = cell of point w within its strip
// (its within-strip column-2 rank * nsub / strip length), and the column-2
// bounds czlo / czhi of every cell.
void launch_nest_key(const JobDev* jobs_d, const int32_t* grid_jobs_d, int ngrid,
                     const SortSeg* gsegs_d, const int32_t* sorted_vals, const SortSeg* segs_d,
                     const int32_t* inv_scratch, uint64_t* keys, int32_t* vals, int64_t max_len,
                     cudaStream_t st);
void launch_nest_sub(const TaskDev* tasks_d, const JobDev* jobs_d, const int32_t* grid_jobs_d,
                     int ngrid, const SortSeg* gsegs_d, const uint64_t* keys_sorted,
                     const int32_t* vals_sorted, int32_t* sub, int64_t max_len, cudaStream_t st);
void launch_radix_pass(const SortSeg* segs_d, const int32_t* blk_seg_d, int nblk,
                       const uint64_t* kin, const int32_t* vin, uint64_t* kout, int32_t* vout,
                       int shift, uint32_t* hist, uint32_t* scan_tmp, cudaStream_t st);
size_t sort_scan_tmp_elems(int nblk);
// The batch sort: single-sweep LSD passes over the 8-bit digits first..7 of
// the keys (first = 0: all; first = 2: the high 48 bits, then a repair of
// the rare runs tied there, which sets DERR_SORT_TIES when one is too long);
// `sweep` (sort_sweep_bytes, zeroed before the launch) holds its look-back
// flags, digit totals and tile counters.  `first` is even: the result is in
// keys_a / vals_a.
// blk_seg_d / nblk: the segments' SORT_TILE tiles (load and repair
// kernels); os_blk_seg_d / os_nblk: their OS_TILE tiles (the passes).
size_t sort_sweep_bytes(int os_nblk, int nseg);
// Once per context, on its device: lets the passes use their shared memory
// (above the 48 KB default); returns the cudaError_t.
int init_sort_kernels();
void launch_sort(const TaskDev* tasks_d, const SortSeg* segs_d, const int32_t* blk_seg_d,
                 int nblk, const int32_t* os_blk_seg_d, int os_nblk, int nseg, uint64_t* keys_a,
                 uint64_t* keys_b, int32_t* vals_a, int32_t* vals_b, void* sweep, int first,
                 uint32_t* err, cudaStream_t st,
                 cudaEvent_t* pass_events = nullptr);  // recorded around the passes alone
constexpr int SORTED_BLOCK = 128;
void launch_sorted_jobs(const TaskDev* tasks_d, const SortedJob* jobs_d, int njobs,
                        int total_blocks, const KeyIndex& kx, const int32_t* perm, cudaStream_t st);

// egb_knn.cu / egb_count.cu: tile kernels over materialised jobs.
// dclass in {2, 3, 4} or 0 (generic d <= EGB_DMAX); kclass in {4, 8, 16, 32}.
struct TileShape {
  int threads;            // CTA size
  int qpt;                // queries per thread
  int tile;               // candidates per shared-memory tile
  size_t smem;            // dynamic shared memory bytes
  int queries() const { return threads * qpt; }
};
TileShape knn_shape(int kclass, int dclass, int plain, int slab, int dmax);
void launch_knn_tile(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                     int dclass, int plain, int slab, int dmax, int* counter, uint32_t* err,
                     DeferEntry* defer, int* defer_count, int num_sms, cudaStream_t st);
void launch_knn_defer(const JobDev* jobs_d, const DeferEntry* defer, const int* defer_count,
                      int defer_cap, int kclass, int dclass, int plain, int num_sms,
                      cudaStream_t st);
TileShape count_shape(int dclass, int plain, int slab, int dmax);
void launch_count_tile(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                       int plain, int slab, int dmax, int* counter, uint32_t* err,
                       DeferEntry* defer, int* defer_count, int num_sms, cudaStream_t st);
void launch_count_defer(const JobDev* jobs_d, const DeferEntry* defer, const int* defer_count,
                        int defer_cap, int dclass, int plain, int num_sms, cudaStream_t st);

// egb_grid.cu: grid (strip) tile kernels; deferred queries go to the same
// warp-per-query kernels as the slab form.
TileShape grid_shape(int dclass, int plain, int dmax);
void launch_knn_grid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                     int dclass, int plain, int dmax, int* counter, uint32_t* err,
                     DeferEntry* defer, int* defer_count, int num_sms, cudaStream_t st);
void launch_count_grid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                       int plain, int dmax, int* counter, uint32_t* err, DeferEntry* defer,
                       int* defer_count, int num_sms, cudaStream_t st);

// egb_wgrid.cu: warp-level grid kernels (items of WG_QB queries, outliers
// finished in-warp, no deferred pass); kclass <= 8 for kNN.
constexpr int WG_QB = 32;
void launch_knn_wgrid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                      int dclass, int plain, int dmax, int* counter, int num_sms, cudaStream_t st);
// egb_wwalk.cu: FP32-path kNN of warp-grid jobs (K <= 8) by per-lane walks
void launch_knn_walk(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                     int dclass, int* counter, int num_sms, cudaStream_t st);
// egb_wcount.cu: exact key-range ball counts of d = 2 / nested d = 3, 4
// warp-grid jobs (FP32 path; the FP64 comparator keeps launch_count_wgrid)
bool count_keys_supported(int dclass);
void launch_count_keys(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                       int* counter, int num_sms, cudaStream_t st);
void launch_count_wgrid(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int dclass,
                        int plain, int dmax, int* counter, int num_sms, cudaStream_t st);

// egb_wavelet.cu: exact 2-D ball counts in rank space.  A count space of
// columns (a, b) over len points is the permutation S[i] = position in the
// b order of the point at position i of the a order; the ball of a query is
// the rectangle of key ranges [a_lo, a_hi) x [b_lo, b_hi) in those orders, and
// its count is #{i in [a_lo, a_hi) : S[i] in [b_lo, b_hi)}, answered by a
// 4-ary wavelet matrix over S: D levels of 2-bit digits (4^D > len), level
// l holding digit D-1-l of every value in the order of the level (the level
// above stably partitioned by its digit).  Each level is a sequence of
// 32-byte blocks of 64 digits: two bit planes and the counts of digits
// <= 0, <= 1, <= 2 before the block, so a rank is one block read.
constexpr int WM_TILE = 2048;      // values per block of the level passes
constexpr int WM_SUPER = 64;       // tiles per super tile (prefix sums of digits)
constexpr int WM_QBLOCK = 128;     // queries per block of the count kernel
struct WmBlock {                   // 64 digits of one level
  uint32_t hi[2];                  // bit 1 of digit j at bit j % 32 of hi[j / 32]
  uint32_t lo[2];                  // bit 0
  uint32_t le[3];                  // digits <= 0, <= 1, <= 2 before the block
  uint32_t pad;
};
struct WmJob {
  WmBlock* levels;        // [D][nblocks]
  int32_t* bucket;        // [D][4] first position of each digit's run in the
                          // next level (digits below it in the whole level)
  int32_t* seq0;          // [len] the sequence of even levels
  int32_t* seq1;          // [len] the sequence of odd levels
  int32_t* inv_b;         // [len] working offset -> position in the b order
  uint32_t* tcount;       // [D][ntiles][4] digits of each level per tile (zeroed)
  uint32_t* scount;       // [D][nsuper][4] per super tile (zeroed)
  int64_t base_a;         // sorted segment of column a in the key / value buffers
  int64_t base_b;         // sorted segment of column b
  int64_t s1_a, s2_a;     // its samples (egb_search.cuh)
  int64_t s1_b, s2_b;
  int32_t task, slot;
  int32_t len;            // points of the space (= queries)
  int32_t D;              // levels: 4^D > len
  int32_t nblocks;        // (len >> 6) + 1 blocks per level
  int32_t ntiles;         // ceil(len / WM_TILE)
  int32_t nsuper;         // ceil(ntiles / WM_SUPER)
  int32_t tile0;          // first block of the job in the level launches
  int32_t qblk0;          // first block of the job in the count launch
  int32_t seg_begin;      // first working index of the space
  const int2* brange;     // the b order's ball of each query, by working
                          // index, kept by the task's 1-D count of that
                          // column (null: searched here)
};
// Build (after the batch sort): inverse b order, the level-0 sequence, then
// one launch per level for every job at once (max_levels launches).
void launch_wm_build(const WmJob* jobs_d, int njobs, int total_tiles, int max_levels,
                     const int32_t* sorted_vals, cudaStream_t st);
// Counts: one thread per query, in the a order; writes cnt[slot] of the task.
void launch_wm_count(const TaskDev* tasks_d, const WmJob* jobs_d, int njobs, int total_blocks,
                     const KeyIndex& kx, const int32_t* sorted_vals, cudaStream_t st);
// The arrays launch_samples writes: the FP32 copy and the samples of every
// sorted segment (read back through a KeyIndex), after the sort.
struct KeyIndexOut {
  float* fkeys;
  uint64_t* s1;
  uint64_t* s2;
  float* fs1;
  float* fs2;
};
void launch_samples(const SortSeg* segs_d, const int32_t* blk_seg_d, int nblk,
                    const uint64_t* keys, const KeyIndexOut& out, cudaStream_t st);

// egb_discrete.cu: exact group-by of the rows of one column subset of a
// discrete task: the rows equal to each row, into count slot `slot`.
struct GroupJob {
  int32_t* table;               // [2^cap_log2] row + 1 of each slot's owner, 0 = free (zeroed)
  int32_t* count;               // [2^cap_log2] rows per slot (zeroed)
  int32_t* rowslot;             // [n] slot of each row
  unsigned long long* groups;   // distinct rows (zeroed)
  SpaceCols sp;                 // the subset's columns
  int32_t task, slot, n, cap_log2;
  int32_t blk0;                 // first block of the job in the launches
};
void launch_groups(const TaskDev* tasks_d, const GroupJob* jobs_d, int njobs, int total_blocks,
                   uint32_t* err, cudaStream_t st);
// Conditional discrete MI: condition levels with more than a quarter of
// their rows distinct in x (warn[0]) or in y (warn[1]).
struct LevelCheck {
  const int32_t* xz_table;
  const int32_t* xz_rowslot;
  const int32_t* yz_table;
  const int32_t* yz_rowslot;
  const int32_t* z_table;
  const int32_t* z_rowslot;
  const int32_t* z_count;
  int32_t* xd;                 // [z table] distinct x per level (zeroed)
  int32_t* yd;                 // [z table] distinct y per level (zeroed)
  unsigned long long* warn;    // [2] (zeroed)
  int32_t n, pad;
};
void launch_level_checks(const LevelCheck* checks_d, int nchecks, int max_n, cudaStream_t st);

// egb_matrix.cu: the symmetric pairwise matrix (NaN diagonal) of per-pair
// estimates, optionally normalized, and normalize_mi of a value array.
void launch_pairwise_matrix(const double* vals_d, const int32_t* pairs_d, int ntasks, int nvar,
                            int normalize, double* out_d, cudaStream_t st);
void launch_normalize(const double* in_d, int64_t n, double* out_d, cudaStream_t st);

// egb_select.cu: any K (one warp per query, radix select on FP64 bits)
constexpr int SELECT_WARPS = 8;
void launch_knn_select(const JobDev* jobs_d, const WorkItem* items_d, int nitems, uint32_t* err,
                       int num_sms, cudaStream_t st);

}  // namespace egb
