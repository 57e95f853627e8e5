/*
 * ennemi_gb.h -- C ABI of libennemi_gb.so, the GB300 (sm_103a) nearest-
 * neighbour estimator library behind ennemi_gb300.
 *
 * What it replaces.  ennemi's estimators (ennemi/_entropy_estimators.py) do
 * all their neighbour arithmetic through scipy.spatial.cKDTree:
 *
 *   eps = tree.query(pts, k=[k+1], p=inf)[0]           (:39, :108, :142, :194, :240)
 *   n   = tree.query_ball_point(pts, eps - 1e-12, p=inf, return_length=True)
 *                                                      (:109-110, :152-154, :196, :243-245)
 *
 * followed by a digamma combination of the counts (:42, :113, :156, :200,
 * :247).  One call of egb_run_batch() evaluates a whole list of such
 * estimator invocations -- the tasks that ennemi/_driver.py:477-483 and
 * :701-707 fan out to a thread pool (_driver.py:736-785) -- on one GPU and
 * returns one estimate per task, computed with the reference's formulas.
 * egb_knn_eps() and egb_ball_count() are the two cKDTree queries on their own.
 *
 * Semantics kept from the reference (bit for bit):
 *   - distances are max-norm, each coordinate difference rounded to nearest
 *     in IEEE-754 binary64, exactly the value cKDTree compares;
 *   - eps_i is the (k+1)-th smallest such distance from point i to the points
 *     of its search set, the point itself included (distance 0); +inf when
 *     the set has k or fewer points;
 *   - counts are inclusive: #{j : dist(i, j) <= fl64(eps_i - 1e-12)}, the
 *     point itself included when that radius is >= 0;
 *   - a zero count makes the reference's _psi() return a scalar +inf
 *     (_entropy_estimators.py:338-339); the per-slot zero flags reproduce the
 *     resulting -inf / +inf / NaN estimates.
 *
 * Threading: a context is used by one host thread at a time.  All calls
 * return 0 on success or a negative EGB_ERR_* code; egb_last_error() gives a
 * message for the last failure on that context.
 */
#ifndef ENNEMI_GB_H
#define ENNEMI_GB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Estimator kinds; each names the reference function it replaces. */
enum egb_kind {
  EGB_MI = 0,     /* _estimate_single_mi                    _entropy_estimators.py:69-113  */
  EGB_CMI = 1,    /* _estimate_conditional_mi               _entropy_estimators.py:116-156 */
  EGB_SEMI = 2,   /* _estimate_semidiscrete_mi              _entropy_estimators.py:159-200 */
  EGB_CSEMI = 3,  /* _estimate_conditional_semidiscrete_mi  _entropy_estimators.py:203-247 */
  EGB_ENTROPY = 4, /* _estimate_single_entropy              _entropy_estimators.py:21-42   */
  /* Plug-in estimators of discrete variables, from exact counts of equal
   * rows (values compared as doubles, -0 equal to +0; integer data must be
   * exactly representable, |v| < 2^53).  k is not used.                     */
  EGB_DISCRETE_ENTROPY = 5, /* _estimate_discrete_entropy       _entropy_estimators.py:44-56   */
  EGB_DISCRETE_MI = 6,      /* _estimate_discrete_mi            _entropy_estimators.py:257-289 */
  EGB_DISCRETE_CMI = 7      /* _estimate_conditional_discrete_mi _entropy_estimators.py:291-320 */
};

/* Status codes. */
enum egb_status {
  EGB_OK = 0,
  EGB_ERR_ARG = -1,      /* invalid argument (message says which)            */
  EGB_ERR_CUDA = -2,     /* a CUDA runtime call failed                        */
  EGB_ERR_DEVICE = -3,   /* a kernel reported an error (bounded wait gave up,
                            index guard tripped)                               */
  EGB_ERR_NOMEM = -4,    /* device or pinned host allocation failed           */
  EGB_TASK_CONSTANT = 1, /* egb_result.status only: under EGB_RESCALE a column
                            of the task had standard deviation below 1e-20,
                            which the reference rescales differently (no
                            rescale, no noise, a warning); value is NaN and
                            the caller computes the task with its own
                            preprocessing                                     */
  EGB_ERR_STATE = -5     /* call out of order (e.g. fetch before a batch)     */
};

/* Flags for egb_run_batch / egb_knn_eps / egb_ball_count. */
enum egb_flags {
  EGB_INPUT_DEVICE = 1 << 0, /* column pointers are device pointers (else host) */
  EGB_PLAIN_FP64 = 1 << 1,   /* every distance evaluated in FP64 (the plain
                                comparator); default is FP32 distance tiles with
                                an FP64 recheck of every borderline candidate   */
  EGB_TIMING = 1 << 2,       /* record per-phase CUDA-event timings             */
  EGB_FORCE_BRUTE = 1 << 3,  /* never use the sorted (slab / grid) variants for
                                multi-D spaces: brute force over the segment    */
  EGB_KEEP_INTERNALS = 1 << 4, /* keep eps / counts for egb_fetch()             */
  EGB_FORCE_SLAB = 1 << 5,     /* use the sorted-slab variant for every multi-D
                                  space, whatever its size (tests)               */
  EGB_FORCE_GRID = 1 << 6,     /* use the strip (grid) variant for every multi-D
                                  space, whatever its size (tests); the default
                                  picks it for spaces of >= 4096 points          */
  EGB_FORCE_CTA_GRID = 1 << 7, /* grid spaces use the CTA-item kernels, never the
                                  warp-item ones (tests, comparisons)            */
  EGB_GRAPH = 1 << 8,          /* capture the batch's device work (descriptor
                                  upload to read-back) in a CUDA graph and replay
                                  it for later batches with the same signature
                                  (same sizes, pointers and flags); ignored with
                                  EGB_TIMING.  A batch of device-resident columns
                                  without labels that repeats the previous batch
                                  of the context exactly (shapes, column pointers
                                  and strides, flags, stream; the data may have
                                  changed) replays without being planned again  */
  EGB_STAGE_HOST = 1 << 9,     /* copy host columns into device memory before the
                                  gather even where the device reads pageable
                                  host memory directly (by default contiguous
                                  host columns are then read in place)           */
  EGB_RESCALE = 1 << 10,       /* preprocess on the device as the reference's
                                  _rescale_data (_driver.py:871-902) does: every
                                  column of MI, CMI, SEMI and CSEMI tasks becomes
                                  (x - mean) / std + noise, mean and std by
                                  NumPy's pairwise summation (bit-identical), the
                                  noise from the stream set by egb_set_noise at
                                  the reference's positions (x from 0, then y,
                                  then the condition as an n x dz row-major
                                  array).  A condition of two or more columns
                                  is reduced as NumPy reduces axis 0 of such an
                                  array: row by row.  Requires one x column and
                                  at most one y column; ENTROPY tasks are left
                                  as given                                   */
  EGB_FORCE_RANK = 1 << 11     /* every d = 2 ball count uses the rank-space
                                  wavelet-matrix counts, whatever its size
                                  (tests; ignored with EGB_PLAIN_FP64)        */
};

/* One float64 column: sample i at data[i * stride] (stride in elements). */
typedef struct egb_column {
  const double* data;
  int64_t stride;
} egb_column;

/*
 * One estimator invocation.  Columns are listed x first, then y, then z:
 *   EGB_MI       dx >= 1, dy >= 1, dz = 0      (x, y continuous)
 *   EGB_CMI      dx >= 1, dy >= 1, dz >= 1     (cond = z)
 *   EGB_SEMI     dx >= 1, dy = 0,  dz = 0      (discrete y given as labels)
 *   EGB_CSEMI    dx >= 1, dy = 0,  dz >= 1     (discrete y given as labels)
 *   EGB_ENTROPY  dx >= 1, dy = 0,  dz = 0
 *   EGB_DISCRETE_ENTROPY  dx >= 1, dy = 0,  dz = 0
 *   EGB_DISCRETE_MI       dx >= 1, dy >= 1, dz = 0
 *   EGB_DISCRETE_CMI      dx >= 1, dy >= 1, dz >= 1
 * labels (host memory, SEMI/CSEMI only): class index of each sample in
 * [0, nclass); the caller maps the reference's np.unique(y) values to 0..C-1
 * in sorted order.
 */
typedef struct egb_task {
  int32_t kind;
  int32_t k;
  int64_t n;
  int32_t dx, dy, dz;
  int32_t nclass;
  const egb_column* cols;  /* dx + dy + dz entries */
  const int32_t* labels;   /* SEMI / CSEMI: n entries, host memory */
  const int32_t* index;    /* optional (host memory): sample w of every column
                              is data[index[w] * stride] -- the reference's mask
                              subset (_driver.py:834-842) without a copy; NULL =
                              samples 0 .. n-1.  Tasks may share one array.   */
} egb_task;

/*
 * Result of one task.  value is the estimate in nats with the reference
 * formula; term_sum is the sum over samples of the per-sample term
 * (psi(nx)+psi(ny), psi(nxz)+psi(nyz)-psi(nz), psi(n) or log(eps)), and
 * zero_mask has bit s set when count slot s held a zero (for EGB_ENTROPY:
 * bit 0 = some eps was 0).
 */
typedef struct egb_result {
  double value;
  double term_sum;
  uint32_t zero_mask;
  int32_t status;
} egb_result;

typedef struct egb_ctx egb_ctx;

/* Create a context on CUDA device `device` (its own non-blocking stream). */
int egb_create(int device, egb_ctx** out);
void egb_destroy(egb_ctx* ctx);
/* Launch on `stream` (a cudaStream_t, e.g. torch's current stream); NULL
 * restores the context's own stream. */
int egb_set_stream(egb_ctx* ctx, void* stream);
const char* egb_last_error(const egb_ctx* ctx);

/*
 * Evaluate `ntasks` estimator invocations and write one result each.
 * Replaces the per-task calls of _lagged_mi (_driver.py:788-832) and
 * _call_entropy_func (_driver.py:222-226) into the estimators.  Blocks until
 * the results are on the host.
 */
int egb_run_batch(egb_ctx* ctx, const egb_task* tasks, int32_t ntasks, int32_t flags,
                  egb_result* results);

/*
 * Internals of the last batch run with EGB_KEEP_INTERNALS, in the caller's
 * sample order: which = 0 -> eps (double[n]); which = 1 + s -> count slot s
 * (int64[n]); which = 16 + c -> the task's column c as the estimator used it
 * (double[n]: after the index and EGB_RESCALE).  Slots: MI nx, ny; CMI nxz,
 * nyz, nz; SEMI n; CSEMI nxz, nyz, nz; DISCRETE_ENTROPY c_x; DISCRETE_MI
 * c_xy, c_x, c_y; DISCRETE_CMI c_xyz, c_xz, c_yz, c_z (rows equal to each
 * row on those columns).
 */
int egb_fetch(egb_ctx* ctx, int32_t task, int32_t which, void* host_out);

/*
 * cKDTree(points).query(points, k=[k+1], p=inf)[0] for a row-major (n x d)
 * float64 array: eps[i] = (k+1)-th smallest max-norm distance (self
 * included).  points and eps in host memory unless EGB_INPUT_DEVICE.
 */
int egb_knn_eps(egb_ctx* ctx, const double* points, int64_t n, int32_t d, int32_t k,
                int32_t flags, double* eps);

/*
 * cKDTree(points).query_ball_point(points, radius, p=inf, return_length=True):
 * count[i] = #{j : maxnorm(points_j - points_i) <= radius[i]}.
 */
int egb_ball_count(egb_ctx* ctx, const double* points, int64_t n, int32_t d,
                   const double* radius, int32_t flags, int64_t* count);

/*
 * Per-phase device times of the last batch run with EGB_TIMING, in ms:
 * [0] upload, [1] gather+prepare, [2] sort+materialise, [3] kNN, [4] counts,
 * [5] combine+download, [6] whole batch; then the multi-D kernels alone:
 * [7] kNN tile kernels, [8] kNN deferred-query kernels, [9] count tile
 * kernels, [10] count deferred-query kernels; then [11] the radix sort of
 * the batch's columns (part of [2]), [12] the 1-D counts on the sorted
 * columns (part of [4]) and [13] the sort's digit passes alone (part of
 * [11]).  Returns the number written.
 */
int egb_timings(const egb_ctx* ctx, double* ms, int32_t max);

/* Bytes the last batch copied host -> device (inputs, descriptor tables) and
 * device -> host (partial sums, flags); returns 0. */
int egb_last_transfer(const egb_ctx* ctx, int64_t* h2d_bytes, int64_t* d2h_bytes);

/* Work counters of the last batch: [0] kNN candidate-query pairs screened by
 * tile work items, [1] kNN pairs screened for deferred queries, [2] kNN
 * queries deferred, [3..5] the same for the multi-D counts, [6] / [7]
 * algorithmic operations of the kNN / count tile kernels ((2d+1) per pair:
 * d differences, d max-of-abs, one compare), [8] kernels launched, [9] keys
 * and [10] segments of the batch's radix sort, [11] 1 if the batch was
 * planned on the host (0: an EGB_GRAPH replay without planning), [12] 1 if
 * its device work ran as a CUDA graph, [13] the sort's 8-bit digit passes
 * (6: the high 48 bits of the keys, then a repair of the runs tied there; 8:
 * the batch ran again with the full sort because such a run was too long to
 * repair), [14] microseconds of host planning before the first launch and
 * [15] of issuing the launches (or the graph) of a planned batch (0 for a
 * replay without planning).  Returns the number written. */
int egb_last_stats(const egb_ctx* ctx, int64_t* out, int32_t max);

/*
 * Layout policy (the table an autotuner fills; no counterpart in the
 * reference, whose cKDTree has a single layout).  Every multi-dimensional
 * search job of a batch -- a kNN search or a ball count over d >= 2 columns --
 * runs in one of five layouts:
 *   EGB_MODE_BRUTE      tiles of all points against all points
 *   EGB_MODE_SLAB       points sorted by column 0, tiles from a window
 *   EGB_MODE_GRID       equal-count strips, 128-query CTA work items
 *   EGB_MODE_WARP_GRID  equal-count strips, 32-query warp work items
 *                       (kNN only for K = k + 1 <= 8; otherwise GRID)
 *   EGB_MODE_RANK       ball counts of d = 2 only: rank-space rectangle
 *                       counts on a wavelet matrix (otherwise WARP_GRID;
 *                       the all-FP64 comparator keeps WARP_GRID too)
 * Each layout gives the same results bit for bit; only speed differs.  The
 * planner reads the context's table at egb_policy_index(search, d, K, len);
 * EGB_MODE_AUTO (every entry of a new context) selects the built-in rule:
 * brute force below 4096 points, otherwise the rank-space counts for d = 2
 * ball counts and the warp grid for the rest (CTA grid for kNN with
 * 9 <= K <= 32).  K > 32 kNN always uses the select kernel, and the
 * EGB_FORCE_* flags override the table.
 */
#define EGB_MODE_AUTO (-1)
#define EGB_MODE_BRUTE 0
#define EGB_MODE_SLAB 1
#define EGB_MODE_GRID 2
#define EGB_MODE_WARP_GRID 3
#define EGB_MODE_RANK 4
#define EGB_POLICY_SIZE_CLASSES 32 /* floor(log2(len)) */
#define EGB_POLICY_ENTRIES (2 * 4 * 4 * EGB_POLICY_SIZE_CLASSES)

/* search: 0 = kNN, 1 = ball count; d: dimension (>= 2; 5 and up share a
 * class); K: k + 1 for kNN (classes <= 4, <= 8, <= 16, above), ignored for
 * counts; len: points in the job. */
static inline int egb_policy_index(int search, int d, int K, int64_t len) {
  int dc = d <= 2 ? 0 : d == 3 ? 1 : d == 4 ? 2 : 3;
  int kc = search ? 0 : K <= 4 ? 0 : K <= 8 ? 1 : K <= 16 ? 2 : 3;
  int sc = 0;
  while (sc < EGB_POLICY_SIZE_CLASSES - 1 && (len >> (sc + 1)) > 0) ++sc;
  return ((search * 4 + dc) * 4 + kc) * EGB_POLICY_SIZE_CLASSES + sc;
}

/* Replace the context's table with modes[0 .. n) (n == EGB_POLICY_ENTRIES;
 * each entry EGB_MODE_AUTO .. EGB_MODE_RANK).  modes == NULL resets every
 * entry to EGB_MODE_AUTO. */
int egb_set_policy(egb_ctx* ctx, const int8_t* modes, int32_t n);

/* Copy the context's table to modes[0 .. n); returns the number written. */
int egb_get_policy(const egb_ctx* ctx, int8_t* modes, int32_t n);

/* The preprocessing noise stream of EGB_RESCALE batches: noise[p] is the p-th
 * draw of the reference's np.random.default_rng(2_718281828).normal(0.0,
 * 1e-10, ...) (_driver.py:874, :882).  Copied to the device (host memory,
 * len values); kept until replaced.  A batch needs as many values as its
 * largest task draws: n per rescaled column. */
int egb_set_noise(egb_ctx* ctx, const double* noise, int64_t len);

/*
 * egb_knn_eps_noalloc -- egb_knn_eps() for callers that may not allocate
 * device memory.  It has no counterpart in the reference; it exists for
 * callers such as a plugin inside a larger GPU application that owns a fixed,
 * pre-reserved memory pool, a latency-bound loop that cannot accept the
 * implicit device synchronisation of cudaMalloc/cudaFree, or a process near
 * the device's memory limit where an allocation could fail mid-run.
 *
 * points: device pointer to a row-major (n x d) float64 array; eps: device
 * pointer to n float64 outputs, eps[i] = the (k+1)-th smallest max-norm
 * distance from point i (self included), bit-identical to egb_knn_eps().
 * stream: the cudaStream_t to launch on (NULL = the legacy default stream);
 * the call returns after the stream has finished the work.
 *
 * All intermediate data lives in one file-scope __device__ array of
 * EGB_NOALLOC_SCRATCH_BYTES bytes, which every GPU that loads the library
 * keeps until the process exits.  Limits: n <= EGB_NOALLOC_MAX_POINTS,
 * d <= EGB_NOALLOC_MAX_DIM, k + 1 <= 32; anything larger returns EGB_ERR_ARG
 * without launching.  No cudaMalloc, cudaFree or allocating library routine
 * is called.
 *
 * The first call on a device looks up the device address of the scratch
 * array (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  The address is kept for the life of the
 * process: after cudaDeviceReset() on a device, do not call this entry point
 * on that device again.  A CUDA error that the caller left pending before
 * the call stays pending; EGB_ERR_CUDA reports only an error of this call's
 * own launches or copies.  Every call on a device shares the one
 * scratch array: calls that overlap on the GPU (different streams, different
 * host threads) race and must be serialised by the caller.
 */
#define EGB_NOALLOC_MAX_POINTS 16384
#define EGB_NOALLOC_MAX_DIM 8
#define EGB_NOALLOC_SCRATCH_BYTES (1152u * 1024u)
int egb_knn_eps_noalloc(const double* points, int64_t n, int32_t d, int32_t k, double* eps,
                        void* stream);

/*
 * The matrix of pairwise_mi (ennemi/_driver.py:716-721): out[i * nvar + j] =
 * out[j * nvar + i] = values[t] for the pair (i, j) = (pairs[2 t],
 * pairs[2 t + 1]) of each of the ntasks estimates; every other entry (the
 * diagonal included) NaN.  normalize != 0 applies normalize_mi to each value
 * on the way (egb_normalize).  values, pairs and out are host memory, or
 * device memory with EGB_INPUT_DEVICE; out holds nvar * nvar doubles.
 */
int egb_pairwise_matrix(egb_ctx* ctx, const double* values, const int32_t* pairs, int32_t ntasks,
                        int32_t nvar, int32_t normalize, int32_t flags, double* out);

/*
 * normalize_mi (ennemi/_driver.py:60-81): out[i] = sqrt(1 - exp(-2 mi[i]))
 * where mi[i] > 0, otherwise mi[i] unchanged (zero, negative, -inf, NaN).
 * Host memory, or device memory with EGB_INPUT_DEVICE; out may equal mi.
 * The device exp may differ from the host's in the last bit, which the
 * cancellation in 1 - exp(-2 mi) turns into up to 2^-53 / out[i] (1e-14
 * at out = 0.005; negligible for MI values of practical size).
 */
int egb_normalize(egb_ctx* ctx, const double* mi, int64_t n, int32_t flags, double* out);

/*
 * Distinct-value figures of task `task` of the last batch into
 * out[0 .. min(max, 6)); returns the number written.  [0..3]: distinct rows
 * of each count slot (discrete kinds: the distinct values of each column
 * subset, in slot order; 0 for the other kinds); [4], [5]: for
 * EGB_DISCRETE_CMI, the condition levels whose x (y) has more distinct
 * values than a quarter of the level's rows.  The reference warns once for
 * each variable, or each variable of each level, with more than n / 4
 * distinct values (_entropy_estimators.py:249-254, :280-281).
 */
int egb_last_groups(const egb_ctx* ctx, int32_t task, int64_t* out, int32_t max);

/*
 * Test hook for the device-error path: the next egb_run_batch on this context
 * starts with `word` already in its device error word, as though one of its
 * kernels had reported it (bit 0: a bounded wait gave up; bit 1: an index
 * guard tripped).  That batch runs its kernels as usual, without a CUDA
 * graph, and returns EGB_ERR_DEVICE with the message a real report gives;
 * later batches start clean.  No kernel is made to fail.  It has no
 * counterpart in the reference, whose code never runs on a device.
 */
int egb_debug_inject_device_error(egb_ctx* ctx, uint32_t word);

/* Test hook: out[i] = a[i] / b[i] (host arrays) through the device division
 * that the rescale of EGB_RESCALE uses in place of one FP64 divide per
 * sample -- round to nearest even, as IEEE division.  Returns 0. */
int egb_debug_divide(egb_ctx* ctx, const double* a, const double* b, int64_t n, double* out);

/* Name of the context's CUDA device (cudaDeviceProp::name) into name[0 ..
 * len), NUL-terminated; *sms = its multiprocessor count.  Returns 0. */
int egb_device_info(const egb_ctx* ctx, char* name, int32_t len, int32_t* sms);

/* Library version string. */
const char* egb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* ENNEMI_GB_H */
