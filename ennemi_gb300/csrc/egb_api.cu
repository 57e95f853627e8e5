// egb_api.cu -- host planner and C ABI of libennemi_gb.so (include/ennemi_gb.h).
//
// One egb_run_batch() call turns a list of estimator invocations into a fixed
// sequence of batched launches on one stream:
//
//   upload      caller columns (host memory: each distinct address range once)
//               and the descriptor tables (one pinned copy)
//   gather      -> per-task working FP64 columns (class-grouped for the
//               semidiscrete estimators)
//   prepare     column midranges (centres of the FP32 copies)
//   sort        every 1-D space and the first column of every slab job, one
//               segmented LSD radix sort for the whole batch
//   materialise multi-D job blocks (FP64 + centred FP32, working or sorted)
//   kNN         1-D: merge on sorted keys; multi-D: tile kernels (brute force
//               or slab), any-K select for k + 1 > 32
//   radius      rad = eps - 1e-12
//   counts      1-D: gallop + bisect on sorted keys; multi-D: tile kernels
//   combine     per-task term sums (psi table / log) + zero flags
//   download    partial sums, flags, device error word
//
// The spaces each estimator searches follow ennemi/_entropy_estimators.py:
//   MI     kNN (x,y) all;  counts x, y                          (:69-113)
//   CMI    kNN (x,y,z);    counts (x,z), (y,z), z               (:116-156)
//   SEMI   kNN x per class of y;  count x over all samples      (:159-200)
//   CSEMI  kNN (x,z) per class;   counts (x,z) all, z within the
//          class, z all                                          (:203-247)
//   ENT    kNN x                                                 (:21-42)
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "egb_internal.cuh"
#include "egb_search.cuh"
#include "egb_pwtree.h"
#include "ennemi_gb.h"

using namespace egb;

namespace {
std::atomic<long long> g_launches{0};
}  // namespace

void egb::count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {

constexpr int KIND_KNN_ONLY = 100;    // egb_knn_eps
constexpr int KIND_COUNT_ONLY = 101;  // egb_ball_count
constexpr int SLAB_MIN = 4096;        // shorter multi-D segments use brute force
constexpr int NPHASE = 7;
constexpr int NKTIME = 7;   // kNN tile, kNN deferred, count tile, count deferred,
                            // radix sort, 1-D counts, the sort's digit passes
constexpr int NSTATS = 16;
// finish_batch: the batch must run again with the full sort (not a public code)
constexpr int RC_SORT_RETRY = 1;

// Digamma of a positive integer with the reference's formula
// (ennemi/_entropy_estimators.py:341-348): the SciPy constant for psi(1),
// otherwise the asymptotic expansion in the same order of operations.
double psi_int(double y) {
  if (y == 1.0) return -0.5772156649015331;
  return std::log(y) -
         std::pow(y, -6) * (std::pow(y, 2) * (std::pow(y, 2) * (y / 2 + 1.0 / 12) - 1.0 / 120) +
                            1.0 / 252);
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
int64_t round32(int64_t n) { return (n + 31) / 32 * 32; }

struct Layout {
  size_t off = 0;
  size_t take(size_t bytes, size_t align = 256) {
    off = align_up(off, align);
    const size_t o = off;
    off += bytes;
    return o;
  }
};

struct TaskPlan {
  int kind = 0, k = 0, K = 0;
  int64_t n = 0, ld = 0;
  int dx = 0, dy = 0, dz = 0, ncol = 0, nclass = 0, nslot = 0;
  std::vector<int32_t> perm;      // working -> sample index; empty = identity
  std::vector<int32_t> gperm;     // working -> caller position (perm through index), if both
  const int32_t* index = nullptr; // caller's shared sample index (no labels)
  int64_t src_len = 0;            // samples the caller's columns must hold
  size_t tab_index = 0;           // offset of the shared index in the table blob
  std::vector<int64_t> cls_off;   // class segment starts (nclass + 1)
  size_t off_x64 = 0, off_eps = 0, off_rad = 0, off_cnt[4] = {0, 0, 0, 0};
  size_t tab_perm = 0;            // offset of perm inside the table blob
  size_t tab_rad = 0;             // KIND_COUNT_ONLY: caller radii (host input)
  int center0 = 0;                // first column of the task in the centre array
};

// A sort segment: a range of one working column, named by the column's
// identity (equal ids: equal working columns bit for bit, in every task).
struct SegKey {
  int colid;
  int64_t b, e;
  bool operator<(const SegKey& o) const {
    return std::tie(colid, b, e) < std::tie(o.colid, o.b, o.e);
  }
};

struct Space {
  int task;
  int64_t b, e;
  SpaceCols sp;
  int K;     // kNN: k + 1
  int slot;  // counts
};

// What the read-back of a batch needs: enough to replay a captured batch
// without planning it again.
struct GroupStat {
  int is_knn, d;
};
struct ReplayState {
  bool valid = false;
  uint64_t key = 0;
  std::vector<TaskPlan> P;
  std::vector<CombineJob> cjobs;
  std::vector<GroupStat> groups;
  size_t pin_rb = 0, pin_zr = 0, zr_stats = 0, zr_err = 0, zr_zero = 0, zr_groups = 0, zr_warn = 0;
  std::vector<std::pair<int, int>> group_of;  // per group job: (task, slot)
  std::vector<int> warn_of;                   // per level check: its task
  size_t tab_bytes = 0, zr_bytes = 0;
  int nchunks = 0;
  int64_t sort_keys = 0, sort_segs = 0;  // keys and segments of the batch's radix sort
  int64_t sort_passes = 0;                // its 8-bit digit passes
};

}  // namespace

struct egb_ctx {
  int device = 0;
  int num_sms = 1;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // second stream of a batch, with fork / join events: [0] the rank-space
  // matrices build there beside the grid layouts, [1] kNN groups after the
  // first run there beside it, [2] the 1-D counts run there beside the
  // rank-space and multi-D counts
  cudaStream_t side_stream = nullptr;
  cudaEvent_t fork_ev[3] = {}, join_ev[3] = {};
  std::string err;
  void* arena = nullptr;
  size_t arena_cap = 0;
  void* pinned = nullptr;
  size_t pinned_cap = 0;
  double* psi_d = nullptr;
  int64_t psi_len = 0;
  double* noise_d = nullptr;      // preprocessing noise stream (egb_set_noise)
  int64_t noise_len = 0;
  cudaEvent_t ev[NPHASE + 1] = {};
  cudaEvent_t kev[2 * NKTIME] = {};
  double timings[NPHASE + NKTIME] = {};
  int ntimings = 0;
  int64_t h2d_bytes = 0, d2h_bytes = 0;
  // the device reads pageable host memory through the host's page tables
  // (address translation services over a coherent CPU-GPU link)
  bool host_direct = false;
  // CUDA graph of the last batch run with EGB_GRAPH, replayed while the
  // batch signature is unchanged
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_sig = 0;
  long long graph_launches = 0;
  // the last EGB_GRAPH batch of device-resident tasks, kept to replay it
  // without planning while the caller's batch is unchanged (ReplayState)
  ReplayState replay;
  // layout policy: mode per egb_policy_index() (EGB_MODE_AUTO = built-in rule)
  int8_t policy[EGB_POLICY_ENTRIES];
  egb_ctx() { std::memset(policy, EGB_MODE_AUTO, sizeof(policy)); }
  // kNN: tile pairs, deferred pairs, deferred queries; counts: the same;
  // [6] kNN tile ops, [7] count tile ops ((2d+1) per pair); [8] kernels launched
  int64_t stats[NSTATS] = {};
  // egb_debug_inject_device_error: error word the next batch starts with
  uint32_t inject_err = 0;
  // distinct rows per count slot of each task of the last batch (discrete kinds)
  std::vector<std::array<int64_t, 6>> groups;
  // device buffer of the matrix / normalize calls (apart from the batch
  // arena, so that they keep a batch's internals and captured graph intact)
  void* aux = nullptr;
  size_t aux_cap = 0;
  // internals of the last batch (egb_fetch)
  bool kept = false;
  std::vector<TaskPlan> keep;
};

namespace {

int fail(egb_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define EGB_CUDA(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(ctx, EGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int ensure_arena(egb_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->arena_cap) return EGB_OK;
  if (ctx->arena) cudaFree(ctx->arena);
  ctx->arena = nullptr;
  ctx->arena_cap = 0;
  const size_t want = align_up(bytes + bytes / 8, 1 << 20);
  if (cudaMalloc(&ctx->arena, want) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, EGB_ERR_NOMEM, "device allocation of " + std::to_string(want) + " bytes failed");
  }
  ctx->arena_cap = want;
  return EGB_OK;
}

int ensure_pinned(egb_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->pinned_cap) return EGB_OK;
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  ctx->pinned = nullptr;
  ctx->pinned_cap = 0;
  const size_t want = align_up(bytes + bytes / 8, 1 << 16);
  if (cudaMallocHost(&ctx->pinned, want) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, EGB_ERR_NOMEM, "pinned host allocation of " + std::to_string(want) + " bytes failed");
  }
  ctx->pinned_cap = want;
  return EGB_OK;
}

int ensure_psi(egb_ctx* ctx, int64_t need) {
  if (need <= ctx->psi_len) return EGB_OK;
  int64_t len = std::max<int64_t>(need, 1 << 16);
  std::vector<double> tab((size_t)len);
  tab[0] = 0.0;  // placeholder: zero counts are flagged, never looked up
  for (int64_t i = 1; i < len; ++i) tab[(size_t)i] = psi_int((double)i);
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (size_t)len) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, EGB_ERR_NOMEM, "device allocation of the digamma table failed");
  }
  EGB_CUDA(cudaMemcpyAsync(d, tab.data(), sizeof(double) * (size_t)len, cudaMemcpyHostToDevice,
                           ctx->stream));
  EGB_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->psi_d) cudaFree(ctx->psi_d);
  ctx->psi_d = d;
  ctx->psi_len = len;
  return EGB_OK;
}

void set_cols(SpaceCols& sp, std::initializer_list<std::pair<int, int>> ranges) {
  sp.d = 0;
  std::memset(sp.cols, 0, sizeof(sp.cols));
  for (auto r : ranges)
    for (int c = r.first; c < r.first + r.second; ++c) sp.cols[sp.d++] = (int8_t)c;
}

// Work counters, device error word and per-task results of a finished batch
// (pinned read-back region H).
int finish_batch(egb_ctx* ctx, const ReplayState& R, const char* H, int64_t launches,
                 egb_result* results) {
  {
    const unsigned long long* st4 = (const unsigned long long*)(H + R.pin_zr + R.zr_stats);
    for (int i = 0; i < NSTATS; ++i) ctx->stats[i] = 0;
    for (size_t g = 0; g < R.groups.size(); ++g) {
      const int base = R.groups[g].is_knn ? 0 : 3;
      for (int i = 0; i < 3; ++i) ctx->stats[base + i] += (int64_t)st4[4 * g + i];
      ctx->stats[R.groups[g].is_knn ? 6 : 7] += (int64_t)st4[4 * g] * (2 * R.groups[g].d + 1);
    }
    ctx->stats[8] = launches;
    ctx->stats[9] = R.sort_keys;
    ctx->stats[10] = R.sort_segs;
  }
  ctx->stats[13] = R.sort_passes;
  const uint32_t dev_err = *(const uint32_t*)(H + R.pin_zr + R.zr_err);
  if (dev_err == DERR_SORT_TIES) return RC_SORT_RETRY;
  if (dev_err) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "device error word 0x%x (%s)", dev_err,
                  (dev_err & DERR_WAIT_TIMEOUT) ? "bounded wait gave up" : "index guard");
    return fail(ctx, EGB_ERR_DEVICE, buf);
  }

  ctx->groups.assign(R.P.size(), std::array<int64_t, 6>{0, 0, 0, 0, 0, 0});
  {
    const unsigned long long* gz = (const unsigned long long*)(H + R.pin_zr + R.zr_groups);
    for (size_t g = 0; g < R.group_of.size(); ++g)
      ctx->groups[(size_t)R.group_of[g].first][(size_t)R.group_of[g].second] = (int64_t)gz[g];
    const unsigned long long* wz = (const unsigned long long*)(H + R.pin_zr + R.zr_warn);
    for (size_t c = 0; c < R.warn_of.size(); ++c) {
      ctx->groups[(size_t)R.warn_of[c]][4] = (int64_t)wz[2 * c];
      ctx->groups[(size_t)R.warn_of[c]][5] = (int64_t)wz[2 * c + 1];
    }
  }
  const double* partial = (const double*)(H + R.pin_rb);
  const uint32_t* zf = (const uint32_t*)(H + R.pin_zr + R.zr_zero);
  const double INF = HUGE_VAL;
  int ci = 0;
  for (size_t t = 0; t < R.P.size(); ++t) {
    const TaskPlan& p = R.P[t];
    egb_result r{};
    r.status = EGB_OK;
    if (p.kind == KIND_KNN_ONLY || p.kind == KIND_COUNT_ONLY) {
      if (results) results[t] = r;
      continue;
    }
    const CombineJob& c = R.cjobs[(size_t)ci++];
    double S = 0.0;
    for (int i = 0; i < c.nchunk; ++i) S += partial[c.chunk0 + i];
    const uint32_t z = zf[t] & ~RESCALE_CONSTANT;
    if (zf[t] & RESCALE_CONSTANT) {  // the caller preprocesses this task itself
      r.value = NAN;
      r.status = EGB_TASK_CONSTANT;
      if (results) results[t] = r;
      continue;
    }
    const double N = (double)p.n;
    const double mean = S / N;
    double v = 0.0;
    switch (p.kind) {
      case EGB_MI:
        // psi(nx) or psi(ny) is the scalar +inf when it holds a zero
        v = z ? -INF : psi_int(N) + psi_int(p.k) - mean;
        break;
      case EGB_CMI:
      case EGB_CSEMI: {
        const bool a = (z & 3u) != 0, b = (z & 4u) != 0;
        if (a && b) v = NAN;          // inf - inf
        else if (a) v = -INF;         // psi(k) - (+inf)
        else if (b) v = INF;          // psi(k) - (-inf)
        else v = psi_int(p.k) - mean;
        break;
      }
      case EGB_SEMI: {
        double w = 0.0;  // sum over classes of psi(c) * c / N
        for (int cl = 0; cl < p.nclass; ++cl) {
          const double cc = (double)(p.cls_off[(size_t)cl + 1] - p.cls_off[(size_t)cl]);
          w += psi_int(cc) * (cc / N);
        }
        v = z ? -INF : psi_int(N) + psi_int(p.k) - mean - w;
        break;
      }
      case EGB_ENTROPY:
        v = psi_int(N) - psi_int(p.k) + (double)p.ncol * (mean + std::log(2.0));
        break;
      case EGB_DISCRETE_ENTROPY:  // -(1/N) sum_rows log(c / N)
        v = -mean;
        break;
      case EGB_DISCRETE_MI:       // (1/N) sum_rows log(N c_xy / (c_x c_y))
      case EGB_DISCRETE_CMI:      // (1/N) sum_rows log(c_z c_xyz / (c_xz c_yz))
        v = mean;
        break;
    }
    r.value = v;
    r.term_sum = S;
    r.zero_mask = z;
    if (results) results[t] = r;
  }
  return EGB_OK;
}

// Key of a batch for replay: everything the plan depends on when the inputs
// are device-resident and carry no host labels -- task shapes, column
// pointers and strides, flags, stream.  0 = not replayable.
uint64_t replay_key(const egb_ctx* ctx, const egb_task* tasks, int ntasks, int flags,
                    const double* count_radius) {
  if (!(flags & EGB_GRAPH) || !(flags & EGB_INPUT_DEVICE) || (flags & EGB_TIMING) ||
      (flags & EGB_KEEP_INTERNALS) || count_radius)
    return 0;
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int i = 0; i < 8; ++i) h = (h ^ ((v >> (8 * i)) & 0xffu)) * 1099511628211ull;
  };
  mix((uint64_t)ntasks);
  mix((uint64_t)(uint32_t)flags);
  mix((uint64_t)(uintptr_t)ctx->stream);
  for (int t = 0; t < ntasks; ++t) {
    const egb_task& T = tasks[t];
    if (T.labels || T.index || T.kind < EGB_MI || T.kind > EGB_ENTROPY || !T.cols) return 0;
    mix((uint64_t)(uint32_t)T.kind | ((uint64_t)(uint32_t)T.k << 32));
    mix((uint64_t)T.n);
    mix((uint64_t)(uint32_t)T.dx | ((uint64_t)(uint32_t)T.dy << 16) | ((uint64_t)(uint32_t)T.dz << 32));
    const int nc = T.dx + T.dy + T.dz;
    if (T.dx < 0 || T.dy < 0 || T.dz < 0 || nc > 3 * EGB_DMAX) return 0;
    for (int c = 0; c < nc; ++c) {
      mix((uint64_t)(uintptr_t)T.cols[c].data);
      mix((uint64_t)T.cols[c].stride);
    }
  }
  return h ? h : 1;
}

// extra: per-task extras for the internal kinds (radius for KIND_COUNT_ONLY)
// One batch.  sort_first: the first 8-bit key digit the batch sort passes
// over (2: the high 48 bits and a repair of tied runs; 0: all eight).
int run_batch_sorted(egb_ctx* ctx, const egb_task* tasks, int ntasks, int flags,
                     egb_result* results, const double* count_radius, int sort_first) {
  if (!ctx) return EGB_ERR_ARG;
  if (ntasks < 0 || (ntasks > 0 && !tasks)) return fail(ctx, EGB_ERR_ARG, "invalid task list");
  if (ntasks == 0) return EGB_OK;
  using clk = std::chrono::steady_clock;
  const clk::time_point t_entry = clk::now();
  auto us_since = [](clk::time_point t) {
    return (int64_t)std::chrono::duration_cast<std::chrono::microseconds>(clk::now() - t).count();
  };
  const bool dev_in = (flags & EGB_INPUT_DEVICE) != 0;
  const int plain = (flags & EGB_PLAIN_FP64) ? 1 : 0;
  const bool force_brute = (flags & EGB_FORCE_BRUTE) != 0;
  const bool force_slab = (flags & EGB_FORCE_SLAB) != 0 && !force_brute;
  const bool force_grid = (flags & EGB_FORCE_GRID) != 0 && !force_brute && !force_slab;
  const bool cta_grid = (flags & EGB_FORCE_CTA_GRID) != 0;  // grid without the warp form
  const bool force_rank = (flags & EGB_FORCE_RANK) != 0 && !plain;
  const bool timing = (flags & EGB_TIMING) != 0;
  cudaStream_t st = ctx->stream;
  const long long launches0 = g_launches.load();
  // an injected error word (test hook) is consumed by this batch, which is
  // then planned and issued directly, never replayed from a graph
  const uint32_t inject = ctx->inject_err;
  ctx->inject_err = 0;
  // an unchanged device-resident batch replays its graph without planning
  const uint64_t rkey = replay_key(ctx, tasks, ntasks, flags, count_radius);
  if (rkey && !inject && ctx->replay.valid && ctx->replay.key == rkey && ctx->graph_exec) {
    ctx->kept = false;
    ctx->keep.clear();
    EGB_CUDA(cudaGraphLaunch(ctx->graph_exec, st));
    EGB_CUDA(cudaStreamSynchronize(st));
    ctx->h2d_bytes = (int64_t)ctx->replay.tab_bytes;
    ctx->d2h_bytes = (int64_t)(ctx->replay.zr_bytes + sizeof(double) * (size_t)ctx->replay.nchunks);
    const int rc_rep = finish_batch(ctx, ctx->replay, (const char*)ctx->pinned, ctx->graph_launches, results);
    ctx->stats[11] = 0;  // not planned
    ctx->stats[12] = 1;  // graph launched
    return rc_rep;
  }
  ctx->replay.valid = false;  // this batch rewrites the pinned tables
  ctx->kept = false;
  ctx->keep.clear();

  // ------------------------------------------------------------ validate --
  std::vector<TaskPlan> P((size_t)ntasks);
  int64_t max_n = 1, max_ld = 32;
  int ncols_total = 0;
  const bool rescale = (flags & EGB_RESCALE) != 0;
  // shared sample indices, checked once per (array, n): largest entry
  std::map<std::pair<const int32_t*, int64_t>, int64_t> index_max;
  for (int t = 0; t < ntasks; ++t) {
    const egb_task& T = tasks[t];
    TaskPlan& p = P[(size_t)t];
    const std::string who = "task " + std::to_string(t) + ": ";
    p.kind = T.kind;
    p.k = T.k;
    p.n = T.n;
    p.dx = T.dx;
    p.dy = T.dy;
    p.dz = T.dz;
    p.ncol = T.dx + T.dy + T.dz;
    const bool internal = T.kind == KIND_KNN_ONLY || T.kind == KIND_COUNT_ONLY;
    if (!(T.kind >= EGB_MI && T.kind <= EGB_DISCRETE_CMI) && !internal)
      return fail(ctx, EGB_ERR_ARG, who + "unknown estimator kind");
    if (T.n < 1 || T.n > (int64_t)0x3fffffff) return fail(ctx, EGB_ERR_ARG, who + "n out of range");
    if (T.k < 1 && T.kind != KIND_COUNT_ONLY) return fail(ctx, EGB_ERR_ARG, who + "k must be greater than zero");
    if (T.dx < 1 || T.dy < 0 || T.dz < 0 || p.ncol > EGB_DMAX)
      return fail(ctx, EGB_ERR_ARG, who + "column counts out of range (at most 32 columns)");
    const bool needs_y = T.kind == EGB_MI || T.kind == EGB_CMI || T.kind == EGB_DISCRETE_MI ||
                         T.kind == EGB_DISCRETE_CMI;
    const bool needs_z = T.kind == EGB_CMI || T.kind == EGB_CSEMI || T.kind == EGB_DISCRETE_CMI;
    if ((needs_y != (T.dy > 0)) || (needs_z != (T.dz > 0)))
      return fail(ctx, EGB_ERR_ARG, who + "column counts do not match the estimator kind");
    if (!T.cols) return fail(ctx, EGB_ERR_ARG, who + "null column list");
    for (int c = 0; c < p.ncol; ++c)
      if (!T.cols[c].data || T.cols[c].stride < 1)
        return fail(ctx, EGB_ERR_ARG, who + "invalid column " + std::to_string(c));
    p.src_len = T.n;
    if (T.index) {
      if (internal) return fail(ctx, EGB_ERR_ARG, who + "index not supported for this kind");
      auto it = index_max.find({T.index, T.n});
      if (it == index_max.end()) {
        int64_t mx = -1;
        for (int64_t i = 0; i < T.n; ++i) {
          if (T.index[i] < 0) return fail(ctx, EGB_ERR_ARG, who + "negative sample index");
          mx = std::max<int64_t>(mx, T.index[i]);
        }
        it = index_max.emplace(std::make_pair(T.index, T.n), mx).first;
      }
      p.src_len = it->second + 1;
      p.index = T.index;
    }
    if (rescale && T.kind >= EGB_MI && T.kind <= EGB_CSEMI) {
      if (internal) return fail(ctx, EGB_ERR_ARG, who + "EGB_RESCALE applies to estimator tasks only");
      if (T.dx != 1 || T.dy > 1)
        return fail(ctx, EGB_ERR_ARG, who + "EGB_RESCALE needs one x column and at most one y column");
      const int64_t draws = T.n * (int64_t)(T.dx + T.dy + T.dz);
      if (!ctx->noise_d || draws > ctx->noise_len)
        return fail(ctx, EGB_ERR_ARG, who + "EGB_RESCALE needs " + std::to_string(draws) +
                                          " noise values (egb_set_noise)");
    }
    p.K = T.k + 1;
    p.ld = round32(T.n);
    p.center0 = ncols_total;
    ncols_total += p.ncol;
    max_n = std::max(max_n, T.n);
    max_ld = std::max(max_ld, p.ld);
    p.nslot = T.kind == EGB_DISCRETE_ENTROPY ? 1 : T.kind == EGB_DISCRETE_MI ? 3
              : T.kind == EGB_DISCRETE_CMI ? 4
              : T.kind == EGB_MI ? 2 : (T.kind == EGB_CMI || T.kind == EGB_CSEMI) ? 3
              : (T.kind == EGB_SEMI || T.kind == KIND_COUNT_ONLY) ? 1 : 0;
    if (T.kind == EGB_SEMI || T.kind == EGB_CSEMI) {
      if (!T.labels || T.nclass < 1) return fail(ctx, EGB_ERR_ARG, who + "labels required");
      p.nclass = T.nclass;
      std::vector<int64_t> cnt((size_t)T.nclass + 1, 0);
      for (int64_t i = 0; i < T.n; ++i) {
        const int32_t c = T.labels[i];
        if (c < 0 || c >= T.nclass) return fail(ctx, EGB_ERR_ARG, who + "label out of range");
        ++cnt[(size_t)c + 1];
      }
      p.cls_off.assign((size_t)T.nclass + 1, 0);
      for (int c = 0; c < T.nclass; ++c) p.cls_off[(size_t)c + 1] = p.cls_off[(size_t)c] + cnt[(size_t)c + 1];
      std::vector<int64_t> pos(p.cls_off.begin(), p.cls_off.end() - 1);
      p.perm.resize((size_t)T.n);
      for (int64_t i = 0; i < T.n; ++i) p.perm[(size_t)pos[(size_t)T.labels[i]]++] = (int32_t)i;
      if (p.index) {  // class order, then the caller's sample index
        p.gperm.resize(p.perm.size());
        for (size_t w = 0; w < p.perm.size(); ++w) p.gperm[w] = p.index[p.perm[w]];
        p.index = nullptr;
      }
    } else {
      p.nclass = 1;
      p.cls_off = {0, T.n};
    }
  }

  // ------------------------------------------------------------- spaces --
  std::vector<Space> knn, cnt;
  for (int t = 0; t < ntasks; ++t) {
    const TaskPlan& p = P[(size_t)t];
    Space s{};
    s.task = t;
    s.K = p.K;
    const int X = 0, Y = p.dx, Z = p.dx + p.dy;
    switch (p.kind) {
      case EGB_MI:
        s.b = 0; s.e = p.n;
        set_cols(s.sp, {{X, p.dx}, {Y, p.dy}}); knn.push_back(s);
        set_cols(s.sp, {{X, p.dx}}); s.slot = 0; cnt.push_back(s);
        set_cols(s.sp, {{Y, p.dy}}); s.slot = 1; cnt.push_back(s);
        break;
      case EGB_CMI:
        s.b = 0; s.e = p.n;
        set_cols(s.sp, {{X, p.dx}, {Y, p.dy}, {Z, p.dz}}); knn.push_back(s);
        set_cols(s.sp, {{X, p.dx}, {Z, p.dz}}); s.slot = 0; cnt.push_back(s);
        set_cols(s.sp, {{Y, p.dy}, {Z, p.dz}}); s.slot = 1; cnt.push_back(s);
        set_cols(s.sp, {{Z, p.dz}}); s.slot = 2; cnt.push_back(s);
        break;
      case EGB_SEMI:
        set_cols(s.sp, {{X, p.dx}});
        for (int c = 0; c < p.nclass; ++c) {
          s.b = p.cls_off[(size_t)c]; s.e = p.cls_off[(size_t)c + 1];
          if (s.e > s.b) knn.push_back(s);
        }
        s.b = 0; s.e = p.n; s.slot = 0; cnt.push_back(s);
        break;
      case EGB_CSEMI:
        set_cols(s.sp, {{X, p.dx}, {Z, p.dz}});
        for (int c = 0; c < p.nclass; ++c) {
          s.b = p.cls_off[(size_t)c]; s.e = p.cls_off[(size_t)c + 1];
          if (s.e > s.b) knn.push_back(s);
        }
        s.b = 0; s.e = p.n; s.slot = 0; cnt.push_back(s);
        set_cols(s.sp, {{Z, p.dz}}); s.slot = 1;
        for (int c = 0; c < p.nclass; ++c) {
          s.b = p.cls_off[(size_t)c]; s.e = p.cls_off[(size_t)c + 1];
          if (s.e > s.b) cnt.push_back(s);
        }
        s.b = 0; s.e = p.n; s.slot = 2; cnt.push_back(s);
        break;
      case EGB_ENTROPY:
      case KIND_KNN_ONLY:
        s.b = 0; s.e = p.n;
        set_cols(s.sp, {{X, p.dx}}); knn.push_back(s);
        break;
      case KIND_COUNT_ONLY:
        s.b = 0; s.e = p.n;
        set_cols(s.sp, {{X, p.dx}}); s.slot = 0; cnt.push_back(s);
        break;
    }
  }

  // ------------------------------------------------------ sort segments --
  // Working columns of different tasks are the same bits when they come from
  // the same caller column (pointer, stride), the same sample index and
  // length, in sample order (no class order), with the same preprocessing
  // (EGB_RESCALE: the same noise positions; statistics depend on the rest):
  // such columns share one sort segment -- the y column of every task of a
  // lagged estimate_mi, every column of a pairwise_mi, a shared condition.
  std::vector<std::vector<int>> colid((size_t)ntasks);
  {
    std::map<std::tuple<uintptr_t, int64_t, uintptr_t, int64_t, int64_t, int>, int> ids;
    int next_id = 0;
    for (int t = 0; t < ntasks; ++t) {
      const TaskPlan& p = P[(size_t)t];
      colid[(size_t)t].resize((size_t)p.ncol);
      const bool resc = rescale && p.kind >= EGB_MI && p.kind <= EGB_CSEMI;
      for (int c = 0; c < p.ncol; ++c) {
        if (!p.perm.empty()) {  // class-ordered working columns are the task's own
          colid[(size_t)t][(size_t)c] = next_id++;
          continue;
        }
        const int zc = c - p.dx - p.dy;
        const int64_t noise_pos = !resc ? -1 : zc >= 0 ? (int64_t)(p.dx + p.dy) * p.n + zc : (int64_t)c * p.n;
        const int group = !resc ? 0 : (zc >= 0 && p.dz > 1 ? p.dz : 1);
        const auto key = std::make_tuple((uintptr_t)tasks[t].cols[c].data, tasks[t].cols[c].stride,
                                         (uintptr_t)p.index, p.n, noise_pos, group);
        auto it = ids.find(key);
        if (it == ids.end()) it = ids.emplace(key, next_id++).first;
        colid[(size_t)t][(size_t)c] = it->second;
      }
    }
  }
  std::map<SegKey, int> seg_index;
  std::vector<SortSeg> segs;
  auto seg_for = [&](int task, int col, int64_t b, int64_t e) {
    const SegKey key{colid[(size_t)task][(size_t)col], b, e};
    auto it = seg_index.find(key);
    if (it != seg_index.end()) return it->second;
    SortSeg s{};
    s.task = task;
    s.col = col;
    s.src_begin = (int32_t)b;
    s.len = (int32_t)(e - b);
    const int id = (int)segs.size();
    segs.push_back(s);
    seg_index[key] = id;
    return id;
  };

  // kNN: 1-D sorted jobs, multi-D tile jobs, any-K select jobs
  // mode: 0 brute force, 1 slab, 2 grid (CTA items of 128 queries), 3 warp
  // grid (warp items of 32 queries); modes 1-3 carry the two sorted copies
  // (deferred queries, strip bounds), modes 2-3 the strip-ordered copy
  // warp-grid jobs of d >= 3 use nested cells and a third sorted column
  struct MJob {
    Space s; bool is_knn; int slab; int sort_seg; int sel; int sort_seg_b; int mode;
    int sort_seg_c;
  };
  // layout of a multi-D job: EGB_FORCE_* flags, else the context's policy
  // table, else the built-in rule; warp grid kNN needs K <= 8
  // mode 4: rank-space counts (d = 2 ball counts, FP32 path only)
  auto pick_mode = [&](bool is_knn, const Space& s) {
    const int64_t len = s.e - s.b;
    const bool rank_ok = !is_knn && s.sp.d == 2 && !plain;
    int mode;
    if (force_rank && rank_ok) mode = 4;
    else if (force_brute) mode = 0;
    else if (force_slab) mode = 1;
    else if (force_grid || cta_grid) mode = 3;
    else {
      mode = ctx->policy[egb_policy_index(is_knn ? 0 : 1, s.sp.d, s.K, len)];
      if (mode == EGB_MODE_AUTO) mode = len >= SLAB_MIN ? (rank_ok ? 4 : 3) : 0;
    }
    if (mode == 4 && !rank_ok) mode = 3;
    if (mode == 3 && (cta_grid || (is_knn && s.K > 8))) mode = 2;
    return mode;
  };
  struct WmPlan { Space s; int seg_a, seg_b; };
  std::vector<WmPlan> wplans;
  std::vector<std::pair<int, Space>> sorted_knn, sorted_cnt;  // (seg, space)
  std::vector<MJob> mjobs;
  for (const Space& s : knn) {
    if (s.sp.d == 1) {
      sorted_knn.push_back({seg_for(s.task, s.sp.cols[0], s.b, s.e), s});
    } else {
      MJob m{s, true, 0, -1, 0, -1, 0, -1};
      if (s.K > EGB_KREG_MAX) m.sel = 1;
      else m.mode = pick_mode(true, s);
      m.slab = m.mode >= 1 ? 1 : 0;
      if (m.slab) {
        m.sort_seg = seg_for(s.task, s.sp.cols[0], s.b, s.e);
        m.sort_seg_b = seg_for(s.task, s.sp.cols[1], s.b, s.e);
      }
      if (m.mode == 3 && s.sp.d >= 3) m.sort_seg_c = seg_for(s.task, s.sp.cols[2], s.b, s.e);
      mjobs.push_back(m);
    }
  }
  for (const Space& s : cnt) {
    if (s.sp.d == 1) {
      sorted_cnt.push_back({seg_for(s.task, s.sp.cols[0], s.b, s.e), s});
    } else {
      MJob m{s, false, 0, -1, 0, -1, 0, -1};
      m.mode = pick_mode(false, s);
      if (m.mode == 4) {
        wplans.push_back({s, seg_for(s.task, s.sp.cols[0], s.b, s.e),
                          seg_for(s.task, s.sp.cols[1], s.b, s.e)});
        continue;
      }
      m.slab = m.mode >= 1 ? 1 : 0;
      if (m.slab) {
        m.sort_seg = seg_for(s.task, s.sp.cols[0], s.b, s.e);
        m.sort_seg_b = seg_for(s.task, s.sp.cols[1], s.b, s.e);
      }
      if (m.mode == 3 && s.sp.d >= 3) m.sort_seg_c = seg_for(s.task, s.sp.cols[2], s.b, s.e);
      mjobs.push_back(m);
    }
  }
  int64_t sort_total = 0, s1_total = 0, s2_total = 0;
  int nblk_sort = 0, nblk_os = 0;
  for (SortSeg& s : segs) {
    s.out_base = sort_total;
    s.s1_base = s1_total;
    s.s2_base = s2_total;
    s1_total += samples1_of(s.len);
    s2_total += samples2_of(s.len);
    s.blk0 = nblk_sort;
    s.nblk = (s.len + SORT_TILE - 1) / SORT_TILE;
    s.os_blk0 = nblk_os;
    s.os_nblk = (s.len + OS_TILE - 1) / OS_TILE;
    sort_total += s.len;
    nblk_sort += s.nblk;
    nblk_os += s.os_nblk;
  }
  if (sort_total >= ((int64_t)1 << 31)) return fail(ctx, EGB_ERR_ARG, "batch too large for one sort");

  // ------------------------------------------------------------- layout --
  Layout dl;  // device arena
  Layout tl;  // table blob (pinned host, copied to the device as one block)
  // caller data ranges (host input), deduplicated by address range.  Where
  // the device reads pageable host memory directly, the gather kernel reads a
  // range in place when every column in it is contiguous and read in order
  // and the columns together read it about once (one pass over the link, no
  // staging copy); strided columns (re-read once per column), class-permuted
  // ones (scattered reads) and ranges that several columns read (the lagged
  // views of one series, a column shared by many pairs) are staged in the
  // arena with one copy per range.
  struct Range { uintptr_t lo, hi; size_t dev_off; bool stage; uint64_t used; };
  std::vector<Range> ranges;
  const bool direct_ok = !dev_in && ctx->host_direct && !(flags & EGB_STAGE_HOST);
  if (!dev_in) {
    struct Span { uintptr_t lo, hi; bool stage; uint64_t used; };
    std::vector<Span> rs;
    for (int t = 0; t < ntasks; ++t)
      for (int c = 0; c < P[(size_t)t].ncol; ++c) {
        const egb_column& col = tasks[t].cols[c];
        const uintptr_t lo = (uintptr_t)col.data;
        const uintptr_t hi =
            lo + (uintptr_t)(((P[(size_t)t].src_len - 1) * col.stride + 1) * sizeof(double));
        rs.push_back({lo, hi, !direct_ok || col.stride != 1 || !P[(size_t)t].perm.empty(),
                      (uint64_t)(P[(size_t)t].n * (int64_t)sizeof(double))});
      }
    std::sort(rs.begin(), rs.end(), [](const Span& a, const Span& b) {
      return a.lo < b.lo || (a.lo == b.lo && a.hi < b.hi);
    });
    for (const Span& r : rs) {
      if (!ranges.empty() && r.lo <= ranges.back().hi) {
        ranges.back().hi = std::max(ranges.back().hi, r.hi);
        ranges.back().stage = ranges.back().stage || r.stage;
        ranges.back().used += r.used;
      } else {
        ranges.push_back({r.lo, r.hi, 0, r.stage, r.used});
      }
    }
    for (auto& r : ranges) {
      if (2 * r.used > 3 * (uint64_t)(r.hi - r.lo)) r.stage = true;  // read 1.5 times or more
      // keep the element alignment of the source within the 256-byte block
      const size_t mis = r.lo & 255u;
      if (r.stage) r.dev_off = dl.take(r.hi - r.lo + mis) + mis;
    }
  }
  auto dev_col = [&](int t, int c) -> const double* {
    const egb_column& col = tasks[t].cols[c];
    if (dev_in) return col.data;
    const uintptr_t a = (uintptr_t)col.data;
    for (const Range& r : ranges)
      if (a >= r.lo && a < r.hi)
        return r.stage ? (const double*)((char*)ctx->arena + r.dev_off + (a - r.lo)) : col.data;
    return nullptr;
  };

  for (int t = 0; t < ntasks; ++t) {
    TaskPlan& p = P[(size_t)t];
    p.off_x64 = dl.take(sizeof(double) * (size_t)(p.ncol * p.ld));
    p.off_eps = dl.take(sizeof(double) * (size_t)p.ld);
    p.off_rad = dl.take(sizeof(double) * (size_t)p.ld);
    for (int s = 0; s < p.nslot; ++s) p.off_cnt[s] = dl.take(sizeof(int32_t) * (size_t)p.ld);
    const std::vector<int32_t>& gp = p.gperm.empty() ? p.perm : p.gperm;
    if (!gp.empty()) p.tab_perm = tl.take(sizeof(int32_t) * gp.size());
    if (p.kind == KIND_COUNT_ONLY && !dev_in) p.tab_rad = tl.take(sizeof(double) * (size_t)p.n);
  }
  const size_t off_centers = dl.take(sizeof(double) * (size_t)ncols_total);
  const size_t off_minmax = dl.take(sizeof(unsigned long long) * 2 * (size_t)ncols_total);
  const size_t off_keys_a = dl.take(sizeof(uint64_t) * (size_t)std::max<int64_t>(sort_total, 1));
  const size_t off_keys_b = dl.take(sizeof(uint64_t) * (size_t)std::max<int64_t>(sort_total, 1));
  const size_t off_vals_a = dl.take(sizeof(int32_t) * (size_t)std::max<int64_t>(sort_total, 1));
  const size_t off_vals_b = dl.take(sizeof(int32_t) * (size_t)std::max<int64_t>(sort_total, 1));
  const size_t off_s1 = dl.take(sizeof(uint64_t) * (size_t)std::max<int64_t>(s1_total, 1));
  const size_t off_s2 = dl.take(sizeof(uint64_t) * (size_t)std::max<int64_t>(s2_total, 1));
  const size_t off_fk = dl.take(sizeof(float) * (size_t)std::max<int64_t>(sort_total, 1));
  const size_t off_fs1 = dl.take(sizeof(float) * (size_t)std::max<int64_t>(s1_total, 1));
  const size_t off_fs2 = dl.take(sizeof(float) * (size_t)std::max<int64_t>(s2_total, 1));
  const size_t sweep_bytes = sort_sweep_bytes(nblk_os, (int)segs.size());
  const size_t off_sweep = dl.take(sweep_bytes);

  // multi-D job blocks
  std::vector<JobDev> jobs(mjobs.size());
  std::vector<SortSeg> gsegs;        // strip-key sort, one segment per grid job
  std::vector<int32_t> grid_jobs;    // job index of each grid job
  int64_t gsort_total = 0, max_glen = 1;
  bool any_nested = false;
  int64_t max_gkey = 1;  // largest strip / cell key of the grid jobs
  int nblk_grid = 0;
  int64_t max_lds = 32;
  for (size_t j = 0; j < mjobs.size(); ++j) {
    const MJob& m = mjobs[j];
    JobDev& J = jobs[j];
    std::memset(&J, 0, sizeof(J));
    const int64_t len = m.s.e - m.s.b;
    J.lds = round32(len);
    max_lds = std::max(max_lds, J.lds);
    J.task = m.s.task;
    J.seg_begin = (int32_t)m.s.b;
    J.len = (int32_t)len;
    J.K = m.is_knn ? m.s.K : 0;
    // FP32-path warp-grid counts of d = 2, 3 run on keys (egb_wcount.cu)
    J.kform = (m.mode == 3 && !m.is_knn && !plain && count_keys_supported(m.s.sp.d)) ? 1 : 0;
    J.slab = m.slab;
    J.sort_seg = m.sort_seg;
    J.sp = m.s.sp;
    const int d = m.s.sp.d;
    J.sort_seg_b = m.sort_seg_b;
    // warp-grid jobs read only their grid copy: no working-order or sorted
    // copies
    const bool gonly = m.mode == 3;
    if (!gonly) {
      J.c64 = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)(d * J.lds));
      J.c32 = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)(d * J.lds));
      J.idx = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)J.lds);
    }
    J.center = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)d);
    if (m.slab && !gonly) {
      J.c64b = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)(d * J.lds));
      J.c32b = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)(d * J.lds));
      J.idxb = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)J.lds);
    }
    if (m.mode >= 2) {
      J.c64g = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)(d * J.lds));
      J.c32g = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)(d * J.lds));
      J.idxg = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)J.lds);
      J.posg = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)J.lds);
      // strips of at least GRID_MIN_STRIP points: about c * len^(1/dj) of them
      // for warp-grid jobs (GRID_STRIPS_*_C), 256 for the CTA grid
      int64_t want = 256;
      if (m.mode == 3) {
        const TaskPlan& tp = P[(size_t)m.s.task];
        // the radii of a count job come from the task's joint kNN (per class,
        // hence wider balls, for the semidiscrete kinds: one more dimension)
        const int dj = m.is_knn ? d
                       : tp.kind == KIND_COUNT_ONLY ? d + 1
                       : (tp.kind == EGB_SEMI || tp.kind == EGB_CSEMI) ? tp.ncol + 1
                       : std::max(tp.ncol, d + 1);
        const double c = m.is_knn ? GRID_STRIPS_KNN_C : GRID_STRIPS_COUNT_C;
        want = std::min<int64_t>(GRID_STRIPS_MAX, std::llround(c * std::pow((double)len, 1.0 / dj)));
      }
      J.nstrips = (int32_t)std::max<int64_t>(1, std::min<int64_t>(want, len / GRID_MIN_STRIP));
      if (m.sort_seg_c >= 0) {
        // nested: about NEST_CELL_* points per cell, as many strips as cells
        // per strip, every cell at least GRID_MIN_STRIP / 2 points
        const int target = m.is_knn ? (d == 3 ? NEST_CELL_3D : NEST_CELL_4D) : NEST_CELL_COUNT;
        int64_t side = (int64_t)std::lround(std::sqrt((double)len / target));
        const TaskPlan& tq = P[(size_t)m.s.task];
        if (!m.is_knn && tq.kind != EGB_SEMI && tq.kind != EGB_CSEMI) {
          // count jobs of small spaces with wide balls take finer cells: at
          // least NEST_SIDE_C * len^(1/dj) per side, dj as for the strips
          // (the semidiscrete kinds, whose radii come from per-class kNN,
          // measured best with NEST_CELL_COUNT alone)
          const int dj = tq.kind == KIND_COUNT_ONLY ? d + 1 : std::max(tq.ncol, d + 1);
          side = std::max<int64_t>(side, std::llround(NEST_SIDE_C * std::pow((double)len, 1.0 / dj)));
        }
        side = std::max<int64_t>(1, std::min<int64_t>(256, side));
        while (side > 1 && len / (side * side) < GRID_MIN_STRIP / 2) --side;
        J.nstrips = (int32_t)side;
        J.nsub = (int32_t)side;
        J.sort_seg_c = m.sort_seg_c;
        any_nested = true;
        J.czlo = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)(side * side));
        J.czhi = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)(side * side));
        J.czlo32 = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)(side * side));
        J.czhi32 = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)(side * side));
      }
      max_gkey = std::max<int64_t>(max_gkey, (int64_t)J.nstrips * std::max<int32_t>(1, J.nsub));
      J.sylo = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)J.nstrips);
      J.syhi = (double*)(uintptr_t)dl.take(sizeof(double) * (size_t)J.nstrips);
      J.sylo32 = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)J.nstrips);
      J.syhi32 = (float*)(uintptr_t)dl.take(sizeof(float) * (size_t)J.nstrips);
      J.gseg = (int32_t)gsegs.size();
      SortSeg g{};
      g.out_base = gsort_total;
      g.len = (int32_t)len;
      g.blk0 = nblk_grid;
      g.nblk = (int32_t)((len + SORT_TILE - 1) / SORT_TILE);
      g.task = m.s.task;
      gsegs.push_back(g);
      grid_jobs.push_back((int32_t)j);
      gsort_total += len;
      nblk_grid += g.nblk;
      max_glen = std::max(max_glen, len);
    }
  }

  // strip-key sort of the grid jobs (one extra 8-bit radix pass)
  const size_t off_gkeys_a = dl.take(sizeof(uint64_t) * (size_t)std::max<int64_t>(gsort_total, 1));
  const size_t off_gkeys_b = dl.take(sizeof(uint64_t) * (size_t)std::max<int64_t>(gsort_total, 1));
  const size_t off_gvals_a = dl.take(sizeof(int32_t) * (size_t)std::max<int64_t>(gsort_total, 1));
  const size_t off_gvals_b = dl.take(sizeof(int32_t) * (size_t)std::max<int64_t>(gsort_total, 1));
  const size_t off_ginv = dl.take(sizeof(int32_t) * (size_t)std::max<int64_t>(gsort_total, 1));
  const size_t off_gsub = any_nested ? dl.take(sizeof(int32_t) * (size_t)std::max<int64_t>(gsort_total, 1)) : 0;
  const size_t off_ghist = dl.take(sizeof(uint32_t) * 256 * (size_t)std::max(nblk_grid, 1));
  const size_t off_gscan = dl.take(sizeof(uint32_t) * sort_scan_tmp_elems(std::max(nblk_grid, 1)));

  // sorted jobs
  std::vector<SortedJob> sj_knn, sj_cnt;
  int blk_knn = 0, blk_cnt = 0;
  for (auto& pr : sorted_knn) {
    const SortSeg& sg = segs[(size_t)pr.first];
    SortedJob j{};
    j.task = pr.second.task; j.kind = 0; j.slot = 0; j.K = pr.second.K;
    j.base = sg.out_base; j.s1_base = sg.s1_base; j.s2_base = sg.s2_base;
    j.len = sg.len; j.blk0 = blk_knn;
    blk_knn += (sg.len + SORTED_BLOCK - 1) / SORTED_BLOCK;
    sj_knn.push_back(j);
  }
  for (auto& pr : sorted_cnt) {
    const SortSeg& sg = segs[(size_t)pr.first];
    SortedJob j{};
    j.task = pr.second.task; j.kind = 1; j.slot = pr.second.slot; j.K = 0;
    j.base = sg.out_base; j.s1_base = sg.s1_base; j.s2_base = sg.s2_base;
    j.len = sg.len; j.blk0 = blk_cnt;
    blk_cnt += (sg.len + SORTED_BLOCK - 1) / SORTED_BLOCK;
    sj_cnt.push_back(j);
  }

  // rank-space count jobs (wavelet matrices); their tile sums are zeroed
  // by one memset at the start of the batch.  A matrix depends only on its
  // two sort segments: count jobs over the same pair (a condition shared by
  // the tasks of a pairwise_mi) query one matrix, built once (wbuild).
  std::vector<WmJob> wjobs, wbuild;
  std::map<std::pair<int, int>, size_t> build_of;
  int wm_tiles = 0, wm_qblocks = 0, wm_levels = 0;
  size_t wmz_bytes = 0;
  std::vector<size_t> wm_tc_off;  // per build: offset of its sums in the zeroed block
  // The b ball of a rank-space count is the ball of the task's 1-D count
  // over the same sorted segment, when it has one (the condition z of a
  // conditional MI: nz, n_xz and n_yz share it): that count keeps it, by
  // working index, and the rank-space counts read it instead of searching.
  std::vector<size_t> sj_ranges(sj_cnt.size(), 0);  // arena offset per 1-D count job, 0 = none
  auto b_ranges_of = [&](const WmPlan& w) -> const int2* {
    for (size_t k = 0; k < sorted_cnt.size(); ++k) {
      const Space& c = sorted_cnt[k].second;
      if (sorted_cnt[k].first != w.seg_b || c.task != w.s.task || c.b != w.s.b || c.e != w.s.e)
        continue;
      if (!sj_ranges[k])
        sj_ranges[k] = dl.take(sizeof(int2) * (size_t)P[(size_t)w.s.task].ld);
      return (const int2*)(uintptr_t)sj_ranges[k];  // an offset until the arena is known
    }
    return nullptr;
  };
  for (const WmPlan& w : wplans) {
    const auto bkey = std::make_pair(w.seg_a, w.seg_b);
    auto bit = build_of.find(bkey);
    if (bit != build_of.end()) {
      WmJob Q = wbuild[bit->second];
      Q.task = w.s.task;
      Q.slot = w.s.slot;
      Q.brange = b_ranges_of(w);
      Q.qblk0 = wm_qblocks;
      wm_qblocks += (int)((Q.len + WM_QBLOCK - 1) / WM_QBLOCK);
      wjobs.push_back(Q);
      continue;
    }
    WmJob J{};
    const int64_t len = w.s.e - w.s.b;
    J.task = w.s.task;
    J.slot = w.s.slot;
    J.brange = b_ranges_of(w);
    J.len = (int32_t)len;
    int D = 1;
    while (((int64_t)1 << (2 * D)) <= len) ++D;   // 4^D > len
    J.D = D;
    J.nblocks = (int32_t)((len >> 6) + 1);
    J.ntiles = (int32_t)((len + WM_TILE - 1) / WM_TILE);
    J.nsuper = (J.ntiles + WM_SUPER - 1) / WM_SUPER;
    J.tile0 = wm_tiles;
    J.qblk0 = wm_qblocks;
    J.seg_begin = (int32_t)w.s.b;
    const SortSeg& sa = segs[(size_t)w.seg_a];
    const SortSeg& sb = segs[(size_t)w.seg_b];
    J.base_a = sa.out_base;
    J.base_b = sb.out_base;
    J.s1_a = sa.s1_base;
    J.s2_a = sa.s2_base;
    J.s1_b = sb.s1_base;
    J.s2_b = sb.s2_base;
    J.levels = (WmBlock*)(uintptr_t)dl.take(sizeof(WmBlock) * (size_t)D * (size_t)J.nblocks);
    J.bucket = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * 4 * (size_t)D);
    J.seq0 = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)len);
    J.seq1 = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)len);
    J.inv_b = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)len);
    wm_tc_off.push_back(wmz_bytes);
    wmz_bytes += 4 * sizeof(uint32_t) * (size_t)D * (size_t)(J.ntiles + J.nsuper);
    wm_tiles += J.ntiles;
    wm_qblocks += (int)((len + WM_QBLOCK - 1) / WM_QBLOCK);
    wm_levels = std::max(wm_levels, D);
    build_of.emplace(bkey, wbuild.size());
    wbuild.push_back(J);
    wjobs.push_back(J);
  }
  const size_t off_wmz = dl.take(std::max<size_t>(wmz_bytes, 16));

  // discrete tasks: one exact group-by per column subset (egb_discrete.cu);
  // hash tables of twice the rows, zeroed by one memset with the rest
  std::vector<GroupJob> gbjobs;
  std::vector<std::pair<int, int>> gb_owner;  // (task, slot) per group job
  size_t gbz_bytes = 0;
  int gb_blocks = 0;
  for (int t = 0; t < ntasks; ++t) {
    const TaskPlan& p = P[(size_t)t];
    if (p.kind < EGB_DISCRETE_ENTROPY || p.kind > EGB_DISCRETE_CMI) continue;
    const int X = 0, Y = p.dx, Z = p.dx + p.dy;
    std::vector<SpaceCols> subs;
    SpaceCols sc{};
    if (p.kind == EGB_DISCRETE_ENTROPY) {
      set_cols(sc, {{X, p.dx}}); subs.push_back(sc);
    } else if (p.kind == EGB_DISCRETE_MI) {
      set_cols(sc, {{X, p.dx}, {Y, p.dy}}); subs.push_back(sc);
      set_cols(sc, {{X, p.dx}}); subs.push_back(sc);
      set_cols(sc, {{Y, p.dy}}); subs.push_back(sc);
    } else {
      set_cols(sc, {{X, p.dx}, {Y, p.dy}, {Z, p.dz}}); subs.push_back(sc);
      set_cols(sc, {{X, p.dx}, {Z, p.dz}}); subs.push_back(sc);
      set_cols(sc, {{Y, p.dy}, {Z, p.dz}}); subs.push_back(sc);
      set_cols(sc, {{Z, p.dz}}); subs.push_back(sc);
    }
    for (size_t k = 0; k < subs.size(); ++k) {
      GroupJob G{};
      G.sp = subs[k];
      G.task = t;
      G.slot = (int32_t)k;
      G.n = (int32_t)p.n;
      int lg = 6;
      while (((int64_t)1 << lg) < 2 * p.n) ++lg;
      G.cap_log2 = lg;
      G.blk0 = gb_blocks;
      gb_blocks += (int)((p.n + 255) / 256);
      G.table = (int32_t*)(uintptr_t)gbz_bytes;    // offsets in the zeroed block for now
      gbz_bytes += align_up(sizeof(int32_t) * ((size_t)1 << lg), 256);
      G.count = (int32_t*)(uintptr_t)gbz_bytes;
      gbz_bytes += align_up(sizeof(int32_t) * ((size_t)1 << lg), 256);
      G.rowslot = (int32_t*)(uintptr_t)dl.take(sizeof(int32_t) * (size_t)p.n);
      gbjobs.push_back(G);
      gb_owner.push_back({t, (int)k});
    }
  }
  // conditional discrete MI: per-level distinct counts for the warnings
  std::vector<LevelCheck> lchecks;
  std::vector<std::array<int, 4>> lcheck_jobs;   // group jobs xz, yz, z and the task
  for (size_t g = 0; g < gbjobs.size(); ++g) {
    const GroupJob& G = gbjobs[g];
    if (P[(size_t)G.task].kind != EGB_DISCRETE_CMI || G.slot != 3) continue;
    LevelCheck L{};
    L.n = G.n;
    L.xd = (int32_t*)(uintptr_t)gbz_bytes;
    gbz_bytes += align_up(sizeof(int32_t) * ((size_t)1 << G.cap_log2), 256);
    L.yd = (int32_t*)(uintptr_t)gbz_bytes;
    gbz_bytes += align_up(sizeof(int32_t) * ((size_t)1 << G.cap_log2), 256);
    lchecks.push_back(L);
    lcheck_jobs.push_back({(int)g - 2, (int)g - 1, (int)g, G.task});
  }
  const size_t off_gbz = dl.take(std::max<size_t>(gbz_bytes, 16));

  // tile launch groups
  struct Group {
    int is_knn, sel, kclass, dclass, slab, dmax, mode;
    std::vector<WorkItem> items;  // tile groups: items built here
    std::vector<ItemRun> runs;    // grid groups: items built on the device
    std::vector<int32_t> cum;
    int64_t nitems = 0, ncells = 0;
    size_t tab_items = 0, tab_runs = 0, tab_cum = 0, off_items = 0;
    int64_t defer_cap = 0;   // slab groups: every query may be deferred once
    size_t off_defer = 0;
  };
  std::vector<Group> groups;
  std::map<std::tuple<int, int, int, int, int, int>, int> gidx;
  std::vector<size_t> order(mjobs.size());
  for (size_t j = 0; j < order.size(); ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return jobs[a].len > jobs[b].len; });
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const size_t j = order[oi];
    const MJob& m = mjobs[j];
    const int d = m.s.sp.d;
    const int dclass = (d >= 2 && d <= 4) ? d : 0;
    int kclass = 0;
    if (m.is_knn && !m.sel) kclass = m.s.K <= 4 ? 4 : m.s.K <= 8 ? 8 : m.s.K <= 16 ? 16 : 32;
    const auto key = std::make_tuple((int)m.is_knn, m.sel, kclass, dclass, m.slab, m.mode);
    auto it = gidx.find(key);
    int g;
    if (it == gidx.end()) {
      g = (int)groups.size();
      gidx[key] = g;
      Group G;
      G.is_knn = m.is_knn; G.sel = m.sel; G.kclass = kclass; G.dclass = dclass; G.slab = m.slab; G.dmax = d;
      G.mode = m.mode;
      groups.push_back(G);
    } else {
      g = it->second;
    }
    groups[(size_t)g].dmax = std::max(groups[(size_t)g].dmax, d);
  }
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const size_t j = order[oi];
    const MJob& m = mjobs[j];
    const int d = m.s.sp.d;
    const int dclass = (d >= 2 && d <= 4) ? d : 0;
    int kclass = 0;
    if (m.is_knn && !m.sel) kclass = m.s.K <= 4 ? 4 : m.s.K <= 8 ? 8 : m.s.K <= 16 ? 16 : 32;
    Group& G = groups[(size_t)gidx[std::make_tuple((int)m.is_knn, m.sel, kclass, dclass, m.slab, m.mode)]];
    if (G.mode >= 2) {
      // items never straddle a strip (cell); the device writes them
      // (launch_emit_items) from these per-cell offsets
      const int S = jobs[j].nstrips;
      const int S2 = jobs[j].nsub;
      const int64_t len = jobs[j].len;
      const int qb = G.mode == 3 ? WG_QB : GRID_QB;
      ItemRun r{};
      r.job = (int32_t)j;
      r.ncell = S * std::max(S2, 1);
      r.cum0 = (int32_t)G.cum.size();
      r.qb = qb;
      r.cell0 = G.ncells;
      for (int sidx = 0; sidx < S; ++sidx) {
        const int32_t a = strip_start(sidx, len, S), b = strip_start(sidx + 1, len, S);
        for (int c2 = 0; c2 < std::max(S2, 1); ++c2) {
          const int32_t ca = S2 > 0 ? cell_start(a, b - a, c2, S2) : a;
          const int32_t cb = S2 > 0 ? cell_start(a, b - a, c2 + 1, S2) : b;
          G.cum.push_back((int32_t)G.nitems);
          G.nitems += (cb - ca + qb - 1) / qb;
        }
      }
      G.cum.push_back((int32_t)G.nitems);
      G.ncells += r.ncell;
      G.runs.push_back(r);
      if (G.mode == 2) G.defer_cap += len;
      continue;
    }
    int qb;
    if (G.sel) qb = SELECT_WARPS;
    else if (G.is_knn) qb = knn_shape(G.kclass, G.dclass, plain, G.slab, G.dmax).queries();
    else qb = count_shape(G.dclass, plain, G.slab, G.dmax).queries();
    for (int64_t q0 = 0; q0 < jobs[j].len; q0 += qb) G.items.push_back({(int32_t)j, (int32_t)q0, 0, 0});
    G.nitems = (int64_t)G.items.size();
    if (G.slab) G.defer_cap += jobs[j].len;
  }
  for (Group& G : groups)
    if (!G.runs.empty()) G.off_items = dl.take(sizeof(WorkItem) * (size_t)std::max<int64_t>(G.nitems, 1));
  for (Group& G : groups)
    if (G.defer_cap > 0) G.off_defer = dl.take(sizeof(DeferEntry) * (size_t)G.defer_cap);

  std::vector<int> job_group(mjobs.size(), 0);
  for (size_t j = 0; j < mjobs.size(); ++j) {
    const MJob& m = mjobs[j];
    const int d = m.s.sp.d;
    const int dclass = (d >= 2 && d <= 4) ? d : 0;
    int kclass = 0;
    if (m.is_knn && !m.sel) kclass = m.s.K <= 4 ? 4 : m.s.K <= 8 ? 8 : m.s.K <= 16 ? 16 : 32;
    job_group[j] = gidx[std::make_tuple((int)m.is_knn, m.sel, kclass, dclass, m.slab, m.mode)];
  }

  // combine
  std::vector<CombineJob> cjobs;
  std::vector<int32_t> chunk_job;
  for (int t = 0; t < ntasks; ++t) {
    const TaskPlan& p = P[(size_t)t];
    if (p.kind == KIND_KNN_ONLY || p.kind == KIND_COUNT_ONLY) continue;
    CombineJob c{};
    c.task = t;
    c.kind = p.kind;
    c.chunk0 = (int32_t)chunk_job.size();
    c.nchunk = (int32_t)((p.n + COMBINE_CHUNK - 1) / COMBINE_CHUNK);
    for (int i = 0; i < c.nchunk; ++i) chunk_job.push_back((int32_t)cjobs.size());
    cjobs.push_back(c);
  }
  const int nchunks = (int)chunk_job.size();

  // device rescale (EGB_RESCALE): one summation tree per distinct n, every
  // column of MI / CMI / SEMI / CSEMI tasks; noise positions follow the
  // reference's draws (x from 0, then y, then z, n values each)
  std::vector<PwTree> pw_trees;
  std::vector<int2> pw_nodes;
  std::vector<int32_t> pw_levels;
  std::vector<RescaleCol> rcols;
  std::vector<RescaleStat> rstats;        // distinct columns (mean and std once each)
  std::vector<int32_t> rinv;              // inverse class orders, concatenated
  std::vector<size_t> rinv_task;          // per task: offset in rinv, or SIZE_MAX
  size_t off_pw_scratch = 0, off_pw_ms = 0;
  if (rescale) {
    std::map<int64_t, int32_t> tree_of;
    // a column read through the same pointer, stride and sample index (and
    // summed the same way) has the same statistics in every task
    std::map<std::tuple<uintptr_t, int64_t, uintptr_t, int64_t, int>, int32_t> stat_of;
    size_t scratch_elems = 0;
    for (int t = 0; t < ntasks; ++t) {
      const TaskPlan& p = P[(size_t)t];
      if (p.kind != EGB_MI && p.kind != EGB_CMI && p.kind != EGB_SEMI && p.kind != EGB_CSEMI) continue;
      auto it = tree_of.find(p.n);
      if (it == tree_of.end()) it = tree_of.emplace(p.n, pw_build(p.n, pw_trees, pw_nodes, pw_levels)).first;
      // class-ordered tasks sum in sample order through the inverse order
      if (rinv_task.empty()) rinv_task.assign((size_t)ntasks, SIZE_MAX);
      if (!p.perm.empty()) {
        rinv_task[(size_t)t] = rinv.size();
        rinv.resize(rinv.size() + p.perm.size());
        int32_t* inv = rinv.data() + rinv_task[(size_t)t];
        for (size_t w = 0; w < p.perm.size(); ++w) inv[p.perm[w]] = (int32_t)w;
      }
      for (int c = 0; c < p.ncol; ++c) {
        RescaleCol rc{};
        rc.task = t;
        rc.col = c;
        // x from noise position 0, then y, then z (n x dz, row-major)
        const int zc = c - p.dx - p.dy;  // condition column, or negative
        rc.group = zc >= 0 && p.dz > 1 ? p.dz : 1;
        rc.noise_pos = zc >= 0 ? (int64_t)(p.dx + p.dy) * p.n + zc : (int64_t)c * p.n;
        const auto key = std::make_tuple((uintptr_t)tasks[t].cols[c].data, tasks[t].cols[c].stride,
                                         (uintptr_t)p.index, p.n, rc.group);
        const bool ordered = !p.perm.empty();  // its own class order: not shared
        auto f = ordered ? stat_of.end() : stat_of.find(key);
        if (f == stat_of.end()) {
          RescaleStat rs{};
          rs.task = t;
          rs.col = c;
          rs.tree = it->second;
          rs.group = rc.group;
          rs.scratch = (int64_t)scratch_elems;
          if (rs.group == 1) scratch_elems += (size_t)pw_trees[(size_t)it->second].nnode;
          rc.stat = (int32_t)rstats.size();
          rstats.push_back(rs);
          if (!ordered) stat_of.emplace(key, rc.stat);
        } else {
          rc.stat = f->second;
        }
        rcols.push_back(rc);
      }
    }
    off_pw_scratch = dl.take(sizeof(double) * std::max<size_t>(scratch_elems, 1));
    off_pw_ms = dl.take(sizeof(double2) * std::max<size_t>(rstats.size(), 1));
  }

  // tables (pinned blob -> device)
  std::vector<GatherCol> gcols;
  std::vector<int32_t> col_task, col_idx;
  const size_t tab_tasks = tl.take(sizeof(TaskDev) * (size_t)ntasks);
  const size_t tab_gcols = tl.take(sizeof(GatherCol) * (size_t)ncols_total);
  const size_t tab_coltask = tl.take(sizeof(int32_t) * (size_t)ncols_total);
  const size_t tab_colidx = tl.take(sizeof(int32_t) * (size_t)ncols_total);
  const size_t tab_segs = tl.take(sizeof(SortSeg) * std::max<size_t>(segs.size(), 1));
  const size_t tab_blkseg = tl.take(sizeof(int32_t) * (size_t)std::max(nblk_sort, 1));
  const size_t tab_osblkseg = tl.take(sizeof(int32_t) * (size_t)std::max(nblk_os, 1));
  const size_t tab_sjk = tl.take(sizeof(SortedJob) * std::max<size_t>(sj_knn.size(), 1));
  const size_t tab_sjc = tl.take(sizeof(SortedJob) * std::max<size_t>(sj_cnt.size(), 1));
  const size_t tab_jobs = tl.take(sizeof(JobDev) * std::max<size_t>(jobs.size(), 1));
  const size_t tab_gsegs = tl.take(sizeof(SortSeg) * std::max<size_t>(gsegs.size(), 1));
  const size_t tab_blkgseg = tl.take(sizeof(int32_t) * (size_t)std::max(nblk_grid, 1));
  const size_t tab_gridjobs = tl.take(sizeof(int32_t) * std::max<size_t>(grid_jobs.size(), 1));
  const size_t tab_pwtrees = tl.take(sizeof(PwTree) * std::max<size_t>(pw_trees.size(), 1));
  const size_t tab_pwnodes = tl.take(sizeof(int2) * std::max<size_t>(pw_nodes.size(), 1));
  const size_t tab_pwlevels = tl.take(sizeof(int32_t) * std::max<size_t>(pw_levels.size(), 1));
  const size_t tab_rcols = tl.take(sizeof(RescaleCol) * std::max<size_t>(rcols.size(), 1));
  const size_t tab_rstats = tl.take(sizeof(RescaleStat) * std::max<size_t>(rstats.size(), 1));
  const size_t tab_rinv = tl.take(sizeof(int32_t) * std::max<size_t>(rinv.size(), 1));
  // shared sample indices: one copy per (array, n)
  std::map<std::pair<const int32_t*, int64_t>, size_t> index_tab;
  for (TaskPlan& p : P) {
    if (!p.index) continue;
    auto it = index_tab.find({p.index, p.n});
    if (it == index_tab.end())
      it = index_tab.emplace(std::make_pair(p.index, p.n), tl.take(sizeof(int32_t) * (size_t)p.n)).first;
    p.tab_index = it->second;
  }
  std::vector<size_t> tab_sstart(jobs.size(), 0);
  std::vector<size_t> tab_cstart(jobs.size(), 0);
  for (int32_t gj : grid_jobs) {
    const JobDev& J = jobs[(size_t)gj];
    tab_sstart[(size_t)gj] = tl.take(sizeof(int32_t) * (size_t)(J.nstrips + 1));
    if (J.nsub > 0) tab_cstart[(size_t)gj] = tl.take(sizeof(int32_t) * (size_t)(J.nstrips * J.nsub + 1));
  }
  for (Group& G : groups) {
    G.tab_items = tl.take(sizeof(WorkItem) * G.items.size());
    G.tab_runs = tl.take(sizeof(ItemRun) * G.runs.size());
    G.tab_cum = tl.take(sizeof(int32_t) * G.cum.size());
  }
  const size_t tab_wjobs = tl.take(sizeof(WmJob) * std::max<size_t>(wjobs.size(), 1));
  const size_t tab_wbuild = tl.take(sizeof(WmJob) * std::max<size_t>(wbuild.size(), 1));
  const size_t tab_gbjobs = tl.take(sizeof(GroupJob) * std::max<size_t>(gbjobs.size(), 1));
  const size_t tab_lchecks = tl.take(sizeof(LevelCheck) * std::max<size_t>(lchecks.size(), 1));
  const size_t tab_cjobs = tl.take(sizeof(CombineJob) * std::max<size_t>(cjobs.size(), 1));
  const size_t tab_chunkjob = tl.take(sizeof(int32_t) * (size_t)std::max(nchunks, 1));
  const size_t tab_bytes = align_up(tl.off, 256);
  const size_t off_tab = dl.take(tab_bytes);
  // zero-initialised region: counters, job flags, zero flags, error word
  const int ncounters = 2 * (int)groups.size();  // work counter + deferred count
  const size_t zr_stats = 0;  // 4 x u64 per group
  const size_t zr_counters = align_up(zr_stats + 32 * std::max<size_t>(groups.size(), 1), 16);
  const size_t zr_jflags = align_up(zr_counters + sizeof(int) * (size_t)std::max(ncounters, 1), 16);
  const size_t zr_zero = align_up(zr_jflags + sizeof(uint32_t) * std::max<size_t>(jobs.size(), 1), 16);
  const size_t zr_err = align_up(zr_zero + sizeof(uint32_t) * (size_t)ntasks, 16);
  const size_t zr_groups = align_up(zr_err + 16, 16);  // distinct rows per group job
  const size_t zr_warn = zr_groups + sizeof(unsigned long long) * gbjobs.size();  // 2 per check
  const size_t zr_bytes = align_up(zr_warn + 2 * sizeof(unsigned long long) * lchecks.size(), 256);
  const size_t off_zr = dl.take(zr_bytes);
  // readback region: partial sums, then a copy of zero flags + error word
  const size_t off_partial = dl.take(sizeof(double) * (size_t)std::max(nchunks, 1));
  const size_t arena_bytes = align_up(dl.off, 256);

  // pinned: table blob + readback
  const size_t pin_rb = align_up(tab_bytes, 256);
  const size_t pin_bytes = pin_rb + sizeof(double) * (size_t)std::max(nchunks, 1) + zr_bytes;
  int rc = ensure_arena(ctx, arena_bytes);
  if (rc) return rc;
  rc = ensure_pinned(ctx, pin_bytes);
  if (rc) return rc;
  rc = ensure_psi(ctx, max_n + 1);
  if (rc) return rc;
  char* A = (char*)ctx->arena;
  char* H = (char*)ctx->pinned;

  // ------------------------------------------------------- fill tables --
  auto devp = [&](size_t off) { return (void*)(A + off); };
  std::vector<TaskDev> tdev((size_t)ntasks);
  for (int t = 0; t < ntasks; ++t) {
    TaskPlan& p = P[(size_t)t];
    TaskDev& D = tdev[(size_t)t];
    std::memset(&D, 0, sizeof(D));
    D.x64 = (const double*)devp(p.off_x64);
    D.center = (const double*)(A + off_centers) + p.center0;
    D.eps = (double*)devp(p.off_eps);
    D.rad = (double*)devp(p.off_rad);
    for (int s = 0; s < p.nslot; ++s) D.cnt[s] = (int32_t*)devp(p.off_cnt[s]);
    D.ld = p.ld;
    D.n = (int32_t)p.n;
    D.ncol = p.ncol;
    D.rad_given = p.kind == KIND_COUNT_ONLY ? 1 : 0;
    const std::vector<int32_t>& gp = p.gperm.empty() ? p.perm : p.gperm;
    const int32_t* perm_dev = p.index ? (const int32_t*)(A + off_tab + p.tab_index)
                              : gp.empty() ? nullptr : (const int32_t*)(A + off_tab + p.tab_perm);
    if (!gp.empty()) std::memcpy(H + p.tab_perm, gp.data(), sizeof(int32_t) * gp.size());
    if (p.kind == KIND_COUNT_ONLY && !dev_in)
      std::memcpy(H + p.tab_rad, count_radius, sizeof(double) * (size_t)p.n);
    for (int c = 0; c < p.ncol; ++c) {
      GatherCol g{};
      g.src = dev_col(t, c);
      g.stride = tasks[t].cols[c].stride;
      g.perm = perm_dev;
      g.task = t;
      g.col = c;
      gcols.push_back(g);
      col_task.push_back(t);
      col_idx.push_back(c);
    }
  }
  std::memcpy(H + tab_tasks, tdev.data(), sizeof(TaskDev) * tdev.size());
  std::memcpy(H + tab_gcols, gcols.data(), sizeof(GatherCol) * gcols.size());
  for (const auto& e : index_tab)
    std::memcpy(H + e.second, e.first.first, sizeof(int32_t) * (size_t)e.first.second);
  if (!rcols.empty()) {
    std::memcpy(H + tab_pwtrees, pw_trees.data(), sizeof(PwTree) * pw_trees.size());
    std::memcpy(H + tab_pwnodes, pw_nodes.data(), sizeof(int2) * pw_nodes.size());
    std::memcpy(H + tab_pwlevels, pw_levels.data(), sizeof(int32_t) * pw_levels.size());
    auto inv_of = [&](int32_t task) -> const int32_t* {
      const size_t o = rinv_task[(size_t)task];
      return o == SIZE_MAX ? nullptr : (const int32_t*)(A + off_tab + tab_rinv) + o;
    };
    for (RescaleCol& rc : rcols) rc.inv = inv_of(rc.task);
    for (RescaleStat& rs : rstats) rs.inv = inv_of(rs.task);
    std::memcpy(H + tab_rcols, rcols.data(), sizeof(RescaleCol) * rcols.size());
    std::memcpy(H + tab_rstats, rstats.data(), sizeof(RescaleStat) * rstats.size());
    if (!rinv.empty()) std::memcpy(H + tab_rinv, rinv.data(), sizeof(int32_t) * rinv.size());
  }
  std::memcpy(H + tab_coltask, col_task.data(), sizeof(int32_t) * col_task.size());
  std::memcpy(H + tab_colidx, col_idx.data(), sizeof(int32_t) * col_idx.size());
  if (!segs.empty()) std::memcpy(H + tab_segs, segs.data(), sizeof(SortSeg) * segs.size());
  {
    int32_t* bs = (int32_t*)(H + tab_blkseg);
    int32_t* os = (int32_t*)(H + tab_osblkseg);
    for (size_t s = 0; s < segs.size(); ++s) {
      for (int b = 0; b < segs[s].nblk; ++b) bs[segs[s].blk0 + b] = (int32_t)s;
      for (int b = 0; b < segs[s].os_nblk; ++b) os[segs[s].os_blk0 + b] = (int32_t)s;
    }
  }
  if (!gsegs.empty()) std::memcpy(H + tab_gsegs, gsegs.data(), sizeof(SortSeg) * gsegs.size());
  {
    int32_t* bs = (int32_t*)(H + tab_blkgseg);
    for (size_t g = 0; g < gsegs.size(); ++g)
      for (int b = 0; b < gsegs[g].nblk; ++b) bs[gsegs[g].blk0 + b] = (int32_t)g;
  }
  if (!grid_jobs.empty())
    std::memcpy(H + tab_gridjobs, grid_jobs.data(), sizeof(int32_t) * grid_jobs.size());
  if (!sj_knn.empty()) std::memcpy(H + tab_sjk, sj_knn.data(), sizeof(SortedJob) * sj_knn.size());
  for (size_t k = 0; k < sj_cnt.size(); ++k)
    sj_cnt[k].ranges = sj_ranges[k] ? (int2*)(A + sj_ranges[k]) : nullptr;
  if (!sj_cnt.empty()) std::memcpy(H + tab_sjc, sj_cnt.data(), sizeof(SortedJob) * sj_cnt.size());
  for (size_t j = 0; j < jobs.size(); ++j) {
    JobDev J = jobs[j];
    const TaskDev& D = tdev[(size_t)J.task];
    if (J.c64) {
      J.c64 = (double*)(A + (uintptr_t)J.c64);
      J.c32 = (float*)(A + (uintptr_t)J.c32);
      J.idx = (int32_t*)(A + (uintptr_t)J.idx);
    }
    J.center = (double*)(A + (uintptr_t)J.center);
    if (J.c64b) {
      J.c64b = (double*)(A + (uintptr_t)J.c64b);
      J.c32b = (float*)(A + (uintptr_t)J.c32b);
      J.idxb = (int32_t*)(A + (uintptr_t)J.idxb);
    }
    if (J.c64g) {
      J.c64g = (double*)(A + (uintptr_t)J.c64g);
      J.c32g = (float*)(A + (uintptr_t)J.c32g);
      J.idxg = (int32_t*)(A + (uintptr_t)J.idxg);
      J.posg = (int32_t*)(A + (uintptr_t)J.posg);
      J.sylo = (double*)(A + (uintptr_t)J.sylo);
      J.syhi = (double*)(A + (uintptr_t)J.syhi);
      J.sylo32 = (float*)(A + (uintptr_t)J.sylo32);
      J.syhi32 = (float*)(A + (uintptr_t)J.syhi32);
      int32_t* st0 = (int32_t*)(H + tab_sstart[j]);
      for (int s = 0; s <= J.nstrips; ++s) st0[s] = strip_start(s, J.len, J.nstrips);
      J.sstart = (const int32_t*)(A + off_tab + tab_sstart[j]);
      if (J.nsub > 0) {
        J.czlo = (double*)(A + (uintptr_t)J.czlo);
        J.czhi = (double*)(A + (uintptr_t)J.czhi);
        J.czlo32 = (float*)(A + (uintptr_t)J.czlo32);
        J.czhi32 = (float*)(A + (uintptr_t)J.czhi32);
        int32_t* cs0 = (int32_t*)(H + tab_cstart[j]);
        for (int s1 = 0; s1 < J.nstrips; ++s1)
          for (int c2 = 0; c2 < J.nsub; ++c2)
            cs0[s1 * J.nsub + c2] = cell_start(st0[s1], st0[s1 + 1] - st0[s1], c2, J.nsub);
        cs0[J.nstrips * J.nsub] = J.len;
        J.cstart = (const int32_t*)(A + off_tab + tab_cstart[j]);
      }
    }
    J.jflags = (uint32_t*)(A + off_zr + zr_jflags) + j;
    J.stats = (unsigned long long*)(A + off_zr + zr_stats) + 4 * job_group[j];
    J.eps = D.eps;
    J.rad = D.rad;
    J.cnt = mjobs[j].is_knn ? nullptr : D.cnt[mjobs[j].s.slot];
    std::memcpy(H + tab_jobs + sizeof(JobDev) * j, &J, sizeof(JobDev));
  }
  for (Group& G : groups) {
    if (!G.items.empty()) std::memcpy(H + G.tab_items, G.items.data(), sizeof(WorkItem) * G.items.size());
    if (!G.runs.empty()) std::memcpy(H + G.tab_runs, G.runs.data(), sizeof(ItemRun) * G.runs.size());
    if (!G.cum.empty()) std::memcpy(H + G.tab_cum, G.cum.data(), sizeof(int32_t) * G.cum.size());
  }
  {
    // arena offsets -> device pointers; a build's zeroed sums by its index
    std::map<uintptr_t, size_t> build_index;  // levels offset -> build
    for (size_t w = 0; w < wbuild.size(); ++w) build_index[(uintptr_t)wbuild[w].levels] = w;
    auto fix = [&](WmJob J) {
      const size_t bi = build_index.at((uintptr_t)J.levels);
      J.levels = (WmBlock*)(A + (uintptr_t)J.levels);
      J.bucket = (int32_t*)(A + (uintptr_t)J.bucket);
      J.seq0 = (int32_t*)(A + (uintptr_t)J.seq0);
      J.seq1 = (int32_t*)(A + (uintptr_t)J.seq1);
      J.inv_b = (int32_t*)(A + (uintptr_t)J.inv_b);
      if (J.brange) J.brange = (const int2*)(A + (uintptr_t)J.brange);
      J.tcount = (uint32_t*)(A + off_wmz + wm_tc_off[bi]);
      J.scount = J.tcount + 4 * (size_t)J.D * (size_t)J.ntiles;
      return J;
    };
    for (size_t w = 0; w < wjobs.size(); ++w) {
      const WmJob J = fix(wjobs[w]);
      std::memcpy(H + tab_wjobs + sizeof(WmJob) * w, &J, sizeof(WmJob));
    }
    for (size_t w = 0; w < wbuild.size(); ++w) {
      const WmJob J = fix(wbuild[w]);
      std::memcpy(H + tab_wbuild + sizeof(WmJob) * w, &J, sizeof(WmJob));
    }
  }
  for (size_t g = 0; g < gbjobs.size(); ++g) {
    GroupJob G = gbjobs[g];
    G.table = (int32_t*)(A + off_gbz + (uintptr_t)G.table);
    G.count = (int32_t*)(A + off_gbz + (uintptr_t)G.count);
    G.rowslot = (int32_t*)(A + (uintptr_t)G.rowslot);
    G.groups = (unsigned long long*)(A + off_zr + zr_groups) + g;
    std::memcpy(H + tab_gbjobs + sizeof(GroupJob) * g, &G, sizeof(GroupJob));
  }
  int lcheck_max_n = 1;
  for (size_t c = 0; c < lchecks.size(); ++c) {
    LevelCheck L = lchecks[c];
    auto dev_of = [&](const GroupJob& G, bool table) {
      return (const int32_t*)(A + off_gbz + (uintptr_t)(table ? G.table : G.count));
    };
    const GroupJob& Gxz = gbjobs[(size_t)lcheck_jobs[c][0]];
    const GroupJob& Gyz = gbjobs[(size_t)lcheck_jobs[c][1]];
    const GroupJob& Gz = gbjobs[(size_t)lcheck_jobs[c][2]];
    L.xz_table = dev_of(Gxz, true);
    L.yz_table = dev_of(Gyz, true);
    L.z_table = dev_of(Gz, true);
    L.z_count = dev_of(Gz, false);
    L.xz_rowslot = (const int32_t*)(A + (uintptr_t)Gxz.rowslot);
    L.yz_rowslot = (const int32_t*)(A + (uintptr_t)Gyz.rowslot);
    L.z_rowslot = (const int32_t*)(A + (uintptr_t)Gz.rowslot);
    L.xd = (int32_t*)(A + off_gbz + (uintptr_t)L.xd);
    L.yd = (int32_t*)(A + off_gbz + (uintptr_t)L.yd);
    L.warn = (unsigned long long*)(A + off_zr + zr_warn) + 2 * c;
    lcheck_max_n = std::max(lcheck_max_n, L.n);
    std::memcpy(H + tab_lchecks + sizeof(LevelCheck) * c, &L, sizeof(LevelCheck));
  }
  if (!cjobs.empty()) std::memcpy(H + tab_cjobs, cjobs.data(), sizeof(CombineJob) * cjobs.size());
  if (nchunks) std::memcpy(H + tab_chunkjob, chunk_job.data(), sizeof(int32_t) * (size_t)nchunks);

  auto dtab = [&](size_t off) { return (void*)(A + off_tab + off); };
  auto items_of = [&](const Group& G) -> const WorkItem* {
    return G.runs.empty() ? (const WorkItem*)dtab(G.tab_items) : (const WorkItem*)(A + G.off_items);
  };
  const TaskDev* tasks_d = (const TaskDev*)dtab(tab_tasks);
  int* counters = (int*)(A + off_zr + zr_counters);
  uint32_t* zero_d = (uint32_t*)(A + off_zr + zr_zero);
  uint32_t* err_d = (uint32_t*)(A + off_zr + zr_err);

  // ------------------------------------------------------------ launch --
  ctx->h2d_bytes = (int64_t)tab_bytes;
  ctx->d2h_bytes = (int64_t)(zr_bytes + sizeof(double) * (size_t)nchunks);
  if (!dev_in)
    for (const Range& r : ranges) ctx->h2d_bytes += (int64_t)(r.hi - r.lo);
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[0], st));
  if (!dev_in)
    for (const Range& r : ranges)
      if (r.stage)
        EGB_CUDA(cudaMemcpyAsync(A + r.dev_off, (const void*)r.lo, r.hi - r.lo, cudaMemcpyHostToDevice, st));
  const size_t pin_zr = pin_rb + sizeof(double) * (size_t)std::max(nchunks, 1);
  // Everything from the descriptor upload to the read-back: issued directly,
  // or captured once into a CUDA graph and replayed for identical batches.
  auto enqueue = [&]() -> int {
  EGB_CUDA(cudaMemcpyAsync(A + off_tab, H, tab_bytes, cudaMemcpyHostToDevice, st));
  EGB_CUDA(cudaMemsetAsync(A + off_zr, 0, zr_bytes, st));
  if (wmz_bytes) EGB_CUDA(cudaMemsetAsync(A + off_wmz, 0, wmz_bytes, st));
  if (gbz_bytes) EGB_CUDA(cudaMemsetAsync(A + off_gbz, 0, gbz_bytes, st));
  if (nblk_sort) EGB_CUDA(cudaMemsetAsync(A + off_sweep, 0, sweep_bytes, st));
  if (inject)  // the device error word as if a kernel had set these bits
    for (int i = 0; i < 4; ++i)
      EGB_CUDA(cudaMemsetAsync((char*)err_d + i, (int)((inject >> (8 * i)) & 0xffu), 1, st));
  if (dev_in)
    for (int t = 0; t < ntasks; ++t)
      if (P[(size_t)t].kind == KIND_COUNT_ONLY)
        EGB_CUDA(cudaMemcpyAsync(tdev[(size_t)t].rad, count_radius, sizeof(double) * (size_t)P[(size_t)t].n,
                                 cudaMemcpyDeviceToDevice, st));
  if (!dev_in)
    for (int t = 0; t < ntasks; ++t)
      if (P[(size_t)t].kind == KIND_COUNT_ONLY)
        EGB_CUDA(cudaMemcpyAsync(tdev[(size_t)t].rad, A + off_tab + P[(size_t)t].tab_rad,
                                 sizeof(double) * (size_t)P[(size_t)t].n, cudaMemcpyDeviceToDevice, st));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[1], st));

  for (const Group& G : groups)  // grid work items, written on the device
    if (!G.runs.empty())
      launch_emit_items((const JobDev*)dtab(tab_jobs), (const ItemRun*)dtab(G.tab_runs),
                        (int)G.runs.size(), (const int32_t*)dtab(G.tab_cum), G.nitems,
                        (WorkItem*)(A + G.off_items), st);
  launch_gather(tasks_d, (const GatherCol*)dtab(tab_gcols), ncols_total, max_ld, st);
  if (!rcols.empty())
    launch_rescale(tasks_d, (const RescaleStat*)dtab(tab_rstats), (int)rstats.size(),
                   (const RescaleCol*)dtab(tab_rcols), (int)rcols.size(),
                   (const PwTree*)dtab(tab_pwtrees), (const int2*)dtab(tab_pwnodes),
                   (const int32_t*)dtab(tab_pwlevels), (double*)(A + off_pw_scratch),
                   (double2*)(A + off_pw_ms), ctx->noise_d, zero_d, max_n, st);
  launch_prepare(tasks_d, (const int32_t*)dtab(tab_coltask), (const int32_t*)dtab(tab_colidx),
                 ncols_total, max_n, (unsigned long long*)(A + off_minmax), (double*)(A + off_centers),
                 st);
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[2], st));

  uint64_t* keys = (uint64_t*)(A + off_keys_a);
  int32_t* vals = (int32_t*)(A + off_vals_a);
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[8], st));
  launch_sort(tasks_d, (const SortSeg*)dtab(tab_segs), (const int32_t*)dtab(tab_blkseg), nblk_sort,
              (const int32_t*)dtab(tab_osblkseg), nblk_os, (int)segs.size(), keys,
              (uint64_t*)(A + off_keys_b), vals, (int32_t*)(A + off_vals_b), A + off_sweep,
              sort_first, err_d, st, timing ? ctx->kev + 12 : nullptr);
  const KeyIndexOut ko{(float*)(A + off_fk), (uint64_t*)(A + off_s1), (uint64_t*)(A + off_s2),
                       (float*)(A + off_fs1), (float*)(A + off_fs2)};
  const KeyIndex kx{keys, ko.fkeys, ko.s1, ko.s2, ko.fs1, ko.fs2};
  launch_samples((const SortSeg*)dtab(tab_segs), (const int32_t*)dtab(tab_blkseg), nblk_sort, keys,
                 ko, st);
  // the rank-space matrices need only the sorted values: they build on the
  // side stream, joined back before their counts
  const bool fork_wm = !wbuild.empty();
  if (fork_wm) {
    EGB_CUDA(cudaEventRecord(ctx->fork_ev[0], st));
    EGB_CUDA(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev[0], 0));
    launch_wm_build((const WmJob*)dtab(tab_wbuild), (int)wbuild.size(), wm_tiles, wm_levels, vals,
                    ctx->side_stream);
    EGB_CUDA(cudaEventRecord(ctx->join_ev[0], ctx->side_stream));
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[9], st));
  launch_materialize(tasks_d, (const JobDev*)dtab(tab_jobs), (int)jobs.size(), vals,
                     (const SortSeg*)dtab(tab_segs), max_lds, st);
  if (!grid_jobs.empty()) {
    const JobDev* jobs_d = (const JobDev*)dtab(tab_jobs);
    const int32_t* gj_d = (const int32_t*)dtab(tab_gridjobs);
    const int ngrid = (int)grid_jobs.size();
    const SortSeg* gsegs_d = (const SortSeg*)dtab(tab_gsegs);
    const int32_t* blkg_d = (const int32_t*)dtab(tab_blkgseg);
    uint64_t* gka = (uint64_t*)(A + off_gkeys_a);
    uint64_t* gkb = (uint64_t*)(A + off_gkeys_b);
    int32_t* gva = (int32_t*)(A + off_gvals_a);
    int32_t* gvb = (int32_t*)(A + off_gvals_b);
    uint32_t* ghist = (uint32_t*)(A + off_ghist);
    uint32_t* gscan = (uint32_t*)(A + off_gscan);
    int32_t* ginv = (int32_t*)(A + off_ginv);
    int32_t* gsub = any_nested ? (int32_t*)(A + off_gsub) : nullptr;
    launch_grid_inv(jobs_d, gj_d, ngrid, gsegs_d, vals, (const SortSeg*)dtab(tab_segs), ginv, max_glen, st);
    if (any_nested) {
      // strips of the column-2 order -> cell of every point within its strip
      launch_nest_key(jobs_d, gj_d, ngrid, gsegs_d, vals, (const SortSeg*)dtab(tab_segs), ginv, gka,
                      gva, max_glen, st);
      launch_radix_pass(gsegs_d, blkg_d, nblk_grid, gka, gva, gkb, gvb, 0, ghist, gscan, st);
      launch_nest_sub(tasks_d, jobs_d, gj_d, ngrid, gsegs_d, gkb, gvb, gsub, max_glen, st);
    }
    launch_grid_key(jobs_d, gj_d, ngrid, gsegs_d, vals, (const SortSeg*)dtab(tab_segs), ginv, gsub, gka,
                    gva, max_glen, st);
    launch_radix_pass(gsegs_d, blkg_d, nblk_grid, gka, gva, gkb, gvb, 0, ghist, gscan, st);
    if (max_gkey > 256)  // strip / cell keys above 8 bits: second digit
      launch_radix_pass(gsegs_d, blkg_d, nblk_grid, gkb, gvb, gka, gva, 8, ghist, gscan, st);
    launch_materialize_grid(tasks_d, (const JobDev*)dtab(tab_jobs), (const int32_t*)dtab(tab_gridjobs),
                            (int)grid_jobs.size(), vals, (const SortSeg*)dtab(tab_segs),
                            max_gkey > 256 ? gva : gvb, (const SortSeg*)dtab(tab_gsegs),
                            max_lds, st);
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[3], st));

  launch_sorted_jobs(tasks_d, (const SortedJob*)dtab(tab_sjk), (int)sj_knn.size(), blk_knn, kx, vals,
                     st);
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[0], st));
  // kNN groups after the first run on the side stream: each persistent
  // launch fills the GPU, so the next one starts in the previous one's tail
  // (a timed batch keeps them in line)
  int knn_groups = 0;
  for (const Group& G : groups) knn_groups += (G.is_knn && G.nitems > 0) ? 1 : 0;
  const bool fork_knn = !timing && knn_groups > 1;
  if (fork_knn) {
    EGB_CUDA(cudaEventRecord(ctx->fork_ev[1], st));
    EGB_CUDA(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev[1], 0));
  }
  int knn_seen = 0;
  for (size_t g = 0; g < groups.size(); ++g) {
    Group& G = groups[g];
    if (!G.is_knn || G.nitems == 0) continue;
    cudaStream_t gs = (fork_knn && knn_seen++ > 0) ? ctx->side_stream : st;
    if (G.sel)
      launch_knn_select((const JobDev*)dtab(tab_jobs), items_of(G),
                        (int)G.nitems, err_d, ctx->num_sms, gs);
    else if (G.mode == 3)
      launch_knn_wgrid((const JobDev*)dtab(tab_jobs), items_of(G),
                       (int)G.nitems, G.kclass, G.dclass, plain, G.dmax, counters + 2 * g,
                       ctx->num_sms, gs);
    else if (G.mode == 2)
      launch_knn_grid((const JobDev*)dtab(tab_jobs), items_of(G),
                      (int)G.nitems, G.kclass, G.dclass, plain, G.dmax, counters + 2 * g,
                      err_d, (DeferEntry*)(A + G.off_defer), counters + 2 * g + 1, ctx->num_sms, gs);
    else
      launch_knn_tile((const JobDev*)dtab(tab_jobs), items_of(G),
                      (int)G.nitems, G.kclass, G.dclass, plain, G.slab, G.dmax,
                      counters + 2 * g, err_d, (DeferEntry*)(A + G.off_defer),
                      counters + 2 * g + 1, ctx->num_sms, gs);
  }
  if (fork_knn) {
    EGB_CUDA(cudaEventRecord(ctx->join_ev[1], ctx->side_stream));
    EGB_CUDA(cudaStreamWaitEvent(st, ctx->join_ev[1], 0));
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[1], st));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[2], st));
  for (size_t g = 0; g < groups.size(); ++g) {
    Group& G = groups[g];
    if (!G.is_knn || G.sel || !G.slab || G.mode == 3 || G.nitems == 0) continue;
    launch_knn_defer((const JobDev*)dtab(tab_jobs), (const DeferEntry*)(A + G.off_defer),
                     counters + 2 * g + 1, (int)G.defer_cap, G.kclass, G.dclass, plain,
                     ctx->num_sms, st);
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[3], st));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[4], st));

  launch_radius(tasks_d, ntasks, max_ld, st);
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[10], st));
  // the 1-D counts overlap the rank-space and multi-D counts on the side
  // stream (a timed batch keeps them in line, for their own event times)
  bool wm_reads_1d = false;  // rank-space counts that read the 1-D counts' balls
  for (const WmJob& J : wjobs) wm_reads_1d |= J.brange != nullptr;
  const bool fork_1d = !timing && !wm_reads_1d && !sj_cnt.empty() && (!wjobs.empty() || !groups.empty());
  if (fork_1d) {
    EGB_CUDA(cudaEventRecord(ctx->fork_ev[2], st));
    EGB_CUDA(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev[2], 0));
  }
  launch_sorted_jobs(tasks_d, (const SortedJob*)dtab(tab_sjc), (int)sj_cnt.size(), blk_cnt, kx, vals,
                     fork_1d ? ctx->side_stream : st);
  if (fork_1d) EGB_CUDA(cudaEventRecord(ctx->join_ev[2], ctx->side_stream));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[11], st));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[4], st));
  launch_groups(tasks_d, (const GroupJob*)dtab(tab_gbjobs), (int)gbjobs.size(), gb_blocks, err_d, st);
  launch_level_checks((const LevelCheck*)dtab(tab_lchecks), (int)lchecks.size(), lcheck_max_n, st);
  if (fork_wm) EGB_CUDA(cudaStreamWaitEvent(st, ctx->join_ev[0], 0));
  launch_wm_count(tasks_d, (const WmJob*)dtab(tab_wjobs), (int)wjobs.size(), wm_qblocks, kx, vals, st);
  for (size_t g = 0; g < groups.size(); ++g) {
    Group& G = groups[g];
    if (G.is_knn || G.nitems == 0) continue;
    if (G.mode == 3) {
      if (!plain && count_keys_supported(G.dclass))
        launch_count_keys((const JobDev*)dtab(tab_jobs), items_of(G),
                          (int)G.nitems, G.dclass, counters + 2 * g, ctx->num_sms, st);
      else
        launch_count_wgrid((const JobDev*)dtab(tab_jobs), items_of(G),
                           (int)G.nitems, G.dclass, plain, G.dmax, counters + 2 * g,
                           ctx->num_sms, st);
      continue;
    }
    if (G.mode == 2) {
      launch_count_grid((const JobDev*)dtab(tab_jobs), items_of(G),
                        (int)G.nitems, G.dclass, plain, G.dmax, counters + 2 * g, err_d,
                        (DeferEntry*)(A + G.off_defer), counters + 2 * g + 1, ctx->num_sms, st);
      continue;
    }
    launch_count_tile((const JobDev*)dtab(tab_jobs), items_of(G),
                      (int)G.nitems, G.dclass, plain, G.slab, G.dmax, counters + 2 * g,
                      err_d, (DeferEntry*)(A + G.off_defer), counters + 2 * g + 1, ctx->num_sms,
                      st);
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[5], st));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[6], st));
  for (size_t g = 0; g < groups.size(); ++g) {
    Group& G = groups[g];
    if (G.is_knn || !G.slab || G.mode == 3 || G.nitems == 0) continue;
    launch_count_defer((const JobDev*)dtab(tab_jobs), (const DeferEntry*)(A + G.off_defer),
                       counters + 2 * g + 1, (int)G.defer_cap, G.dclass, plain, ctx->num_sms, st);
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->kev[7], st));
  if (fork_1d) EGB_CUDA(cudaStreamWaitEvent(st, ctx->join_ev[2], 0));
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[5], st));

  launch_combine(tasks_d, (const CombineJob*)dtab(tab_cjobs), (const int32_t*)dtab(tab_chunkjob),
                 nchunks, ctx->psi_d, ctx->psi_len, (double*)(A + off_partial), zero_d, err_d, st);
  EGB_CUDA(cudaGetLastError());
  if (nchunks)
    EGB_CUDA(cudaMemcpyAsync(H + pin_rb, A + off_partial, sizeof(double) * (size_t)nchunks,
                             cudaMemcpyDeviceToHost, st));
  EGB_CUDA(cudaMemcpyAsync(H + pin_zr, A + off_zr, zr_bytes, cudaMemcpyDeviceToHost, st));
  return EGB_OK;
  };

  const int64_t plan_us = us_since(t_entry);
  const clk::time_point t_issue = clk::now();
  const bool use_graph = (flags & EGB_GRAPH) != 0 && !timing && !inject;
  if (use_graph) {
    // signature of the batch: the descriptor blob (all device pointers,
    // sizes, job tables) plus the arena, pinned buffer and flags
    uint64_t sig = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
      const unsigned char* b = (const unsigned char*)p;
      for (size_t i = 0; i < n; ++i) sig = (sig ^ b[i]) * 1099511628211ull;
    };
    mix(H, tab_bytes);
    const uintptr_t extra[9] = {(uintptr_t)A, (uintptr_t)H, (uintptr_t)flags, (uintptr_t)zr_bytes,
                                (uintptr_t)nchunks, (uintptr_t)(void*)st, (uintptr_t)ctx->psi_d,
                                (uintptr_t)ctx->psi_len, (uintptr_t)ctx->noise_d};
    mix(extra, sizeof(extra));
    if (!(ctx->graph_exec && ctx->graph_sig == sig)) {
      if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
      ctx->graph_exec = nullptr;
      const long long l0 = g_launches.load();
      EGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const int rc_cap = enqueue();
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      if (rc_cap != EGB_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc_cap;
      }
      if (ce != cudaSuccess) return fail(ctx, EGB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      const cudaError_t ie = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) {
        ctx->graph_exec = nullptr;
        return fail(ctx, EGB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
      }
      ctx->graph_sig = sig;
      ctx->graph_launches = g_launches.load() - l0;
    }
    EGB_CUDA(cudaGraphLaunch(ctx->graph_exec, st));
  } else {
    const int rc_q = enqueue();
    if (rc_q != EGB_OK) return rc_q;
  }
  if (timing) EGB_CUDA(cudaEventRecord(ctx->ev[6], st));
  const int64_t issue_us = us_since(t_issue);
  EGB_CUDA(cudaStreamSynchronize(st));

  if (timing) {
    float ms = 0.f;
    for (int i = 0; i < NPHASE - 1; ++i) {
      cudaEventElapsedTime(&ms, ctx->ev[i], ctx->ev[i + 1]);
      ctx->timings[i] = ms;
    }
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[NPHASE - 1]);
    ctx->timings[NPHASE - 1] = ms;
    for (int i = 0; i < NKTIME; ++i) {
      cudaEventElapsedTime(&ms, ctx->kev[2 * i], ctx->kev[2 * i + 1]);
      ctx->timings[NPHASE + i] = ms;
    }
    ctx->ntimings = NPHASE + NKTIME;
  }

  ReplayState R;
  R.P = std::move(P);
  R.cjobs = std::move(cjobs);
  for (const Group& G : groups) R.groups.push_back({G.is_knn, G.dclass ? G.dclass : G.dmax});
  R.pin_rb = pin_rb;
  R.pin_zr = pin_zr;
  R.zr_stats = zr_stats;
  R.zr_err = zr_err;
  R.zr_groups = zr_groups;
  R.group_of = gb_owner;
  R.zr_warn = zr_warn;
  for (const auto& j : lcheck_jobs) R.warn_of.push_back(j[3]);
  R.zr_zero = zr_zero;
  R.nchunks = nchunks;
  R.tab_bytes = tab_bytes;
  R.zr_bytes = zr_bytes;
  R.sort_keys = sort_total;
  R.sort_segs = (int64_t)segs.size();
  R.sort_passes = 8 - sort_first;
  const int64_t launches =
      use_graph ? (int64_t)ctx->graph_launches : (int64_t)(g_launches.load() - launches0);
  const int rc_fin = finish_batch(ctx, R, H, launches, results);
  ctx->stats[11] = 1;
  ctx->stats[12] = use_graph ? 1 : 0;
  ctx->stats[14] = plan_us;
  ctx->stats[15] = issue_us;
  if (rc_fin != EGB_OK) return rc_fin;
  if (flags & EGB_KEEP_INTERNALS) {
    ctx->keep = std::move(R.P);
    ctx->kept = true;
  } else if (rkey && use_graph) {
    R.key = rkey;
    R.valid = true;
    ctx->replay = std::move(R);
  }
  return EGB_OK;
}

// A batch whose sort met keys tied in their high 48 bits over a run too long
// to repair (finish_batch: RC_SORT_RETRY) runs again with the full sort,
// planned and issued directly.
int run_batch(egb_ctx* ctx, const egb_task* tasks, int ntasks, int flags, egb_result* results,
              const double* count_radius) {
  const int rc = run_batch_sorted(ctx, tasks, ntasks, flags, results, count_radius, 2);
  if (rc != RC_SORT_RETRY) return rc;
  return run_batch_sorted(ctx, tasks, ntasks, flags & ~EGB_GRAPH, results, count_radius, 0);
}

bool create_fork_events(egb_ctx* ctx) {
  for (int i = 0; i < 3; ++i)
    if (cudaEventCreateWithFlags(&ctx->fork_ev[i], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming) != cudaSuccess)
      return false;
  return true;
}

void destroy_fork_events(egb_ctx* ctx) {
  for (int i = 0; i < 3; ++i) {
    if (ctx->fork_ev[i]) cudaEventDestroy(ctx->fork_ev[i]);
    if (ctx->join_ev[i]) cudaEventDestroy(ctx->join_ev[i]);
    ctx->fork_ev[i] = ctx->join_ev[i] = nullptr;
  }
}

}  // namespace

extern "C" {

int egb_create(int device, egb_ctx** out) {
  if (!out) return EGB_ERR_ARG;
  *out = nullptr;
  egb_ctx* ctx = new egb_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || init_sort_kernels() != (int)cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
      !create_fork_events(ctx)) {
    cudaGetLastError();
    destroy_fork_events(ctx);
    if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return EGB_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (ctx->num_sms < 1) ctx->num_sms = 1;
  int pageable = 0, host_tables = 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
  cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
  ctx->host_direct = pageable && host_tables;
  for (auto& e : ctx->ev) cudaEventCreate(&e);
  for (auto& e : ctx->kev) cudaEventCreate(&e);
  *out = ctx;
  return EGB_OK;
}

void egb_destroy(egb_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->psi_d) cudaFree(ctx->psi_d);
  if (ctx->noise_d) cudaFree(ctx->noise_d);
  if (ctx->aux) cudaFree(ctx->aux);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->kev)
    if (e) cudaEventDestroy(e);
  destroy_fork_events(ctx);
  if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

int egb_set_stream(egb_ctx* ctx, void* stream) {
  if (!ctx) return EGB_ERR_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return EGB_OK;
}

const char* egb_last_error(const egb_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int egb_run_batch(egb_ctx* ctx, const egb_task* tasks, int32_t ntasks, int32_t flags,
                  egb_result* results) {
  if (!ctx) return EGB_ERR_ARG;
  cudaSetDevice(ctx->device);
  for (int t = 0; t < ntasks && tasks; ++t)
    if (tasks[t].kind > EGB_DISCRETE_CMI || tasks[t].kind < EGB_MI)
      return fail(ctx, EGB_ERR_ARG, "task " + std::to_string(t) + ": unknown estimator kind");
  return run_batch(ctx, tasks, ntasks, flags, results, nullptr);
}

int egb_fetch(egb_ctx* ctx, int32_t task, int32_t which, void* host_out) {
  if (!ctx || !host_out) return EGB_ERR_ARG;
  if (!ctx->kept) return fail(ctx, EGB_ERR_STATE, "no batch internals kept (run with EGB_KEEP_INTERNALS)");
  if (task < 0 || task >= (int)ctx->keep.size()) return fail(ctx, EGB_ERR_ARG, "task index out of range");
  const TaskPlan& p = ctx->keep[(size_t)task];
  const bool column = which >= 16 && which < 16 + p.ncol;
  if (!column && (which < 0 || which > p.nslot)) return fail(ctx, EGB_ERR_ARG, "no such internal array");
  cudaSetDevice(ctx->device);
  const size_t n = (size_t)p.n;
  std::vector<char> buf(n * 8);
  const char* src = (const char*)ctx->arena +
                    (column ? p.off_x64 + sizeof(double) * (size_t)((which - 16) * p.ld)
                            : which == 0 ? p.off_eps : p.off_cnt[which - 1]);
  const size_t esz = (which == 0 || column) ? 8 : 4;
  EGB_CUDA(cudaMemcpyAsync(buf.data(), src, n * esz, cudaMemcpyDeviceToHost, ctx->stream));
  EGB_CUDA(cudaStreamSynchronize(ctx->stream));
  for (size_t w = 0; w < n; ++w) {
    const size_t i = p.perm.empty() ? w : (size_t)p.perm[w];
    if (esz == 8) ((double*)host_out)[i] = ((const double*)buf.data())[w];
    else ((int64_t*)host_out)[i] = ((const int32_t*)buf.data())[w];
  }
  return EGB_OK;
}

int egb_knn_eps(egb_ctx* ctx, const double* points, int64_t n, int32_t d, int32_t k,
                int32_t flags, double* eps) {
  if (!ctx) return EGB_ERR_ARG;
  if (!points || !eps || n < 1 || d < 1 || d > EGB_DMAX || k < 1)
    return fail(ctx, EGB_ERR_ARG, "egb_knn_eps: invalid arguments");
  cudaSetDevice(ctx->device);
  std::vector<egb_column> cols((size_t)d);
  for (int c = 0; c < d; ++c) cols[(size_t)c] = {points + c, (int64_t)d};
  egb_task t{};
  t.kind = KIND_KNN_ONLY;
  t.k = k;
  t.n = n;
  t.dx = d;
  t.cols = cols.data();
  int rc = run_batch(ctx, &t, 1, flags | EGB_KEEP_INTERNALS, nullptr, nullptr);
  if (rc) return rc;
  const TaskPlan& p = ctx->keep[0];
  const cudaMemcpyKind kind = (flags & EGB_INPUT_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  EGB_CUDA(cudaMemcpyAsync(eps, (const char*)ctx->arena + p.off_eps, sizeof(double) * (size_t)n, kind,
                           ctx->stream));
  EGB_CUDA(cudaStreamSynchronize(ctx->stream));
  return EGB_OK;
}

int egb_ball_count(egb_ctx* ctx, const double* points, int64_t n, int32_t d, const double* radius,
                   int32_t flags, int64_t* count) {
  if (!ctx) return EGB_ERR_ARG;
  if (!points || !radius || !count || n < 1 || d < 1 || d > EGB_DMAX)
    return fail(ctx, EGB_ERR_ARG, "egb_ball_count: invalid arguments");
  cudaSetDevice(ctx->device);
  std::vector<egb_column> cols((size_t)d);
  for (int c = 0; c < d; ++c) cols[(size_t)c] = {points + c, (int64_t)d};
  egb_task t{};
  t.kind = KIND_COUNT_ONLY;
  t.k = 1;
  t.n = n;
  t.dx = d;
  t.cols = cols.data();
  int rc = run_batch(ctx, &t, 1, flags | EGB_KEEP_INTERNALS, nullptr, radius);
  if (rc) return rc;
  if (flags & EGB_INPUT_DEVICE) {
    // widen int32 -> int64 through the host (test-sized path)
    std::vector<int64_t> tmp((size_t)n);
    rc = egb_fetch(ctx, 0, 1, tmp.data());
    if (rc) return rc;
    EGB_CUDA(cudaMemcpy(count, tmp.data(), sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice));
    return EGB_OK;
  }
  return egb_fetch(ctx, 0, 1, count);
}

int egb_set_policy(egb_ctx* ctx, const int8_t* modes, int32_t n) {
  if (!ctx) return EGB_ERR_ARG;
  if (!modes) {
    std::memset(ctx->policy, EGB_MODE_AUTO, sizeof(ctx->policy));
    ctx->replay.valid = false;
    return EGB_OK;
  }
  if (n != EGB_POLICY_ENTRIES) return fail(ctx, EGB_ERR_ARG, "egb_set_policy: table size mismatch");
  for (int i = 0; i < n; ++i)
    if (modes[i] < EGB_MODE_AUTO || modes[i] > EGB_MODE_RANK)
      return fail(ctx, EGB_ERR_ARG, "egb_set_policy: invalid mode at entry " + std::to_string(i));
  std::memcpy(ctx->policy, modes, sizeof(ctx->policy));
  ctx->replay.valid = false;  // the plan of a replayed batch may change
  return EGB_OK;
}

int egb_set_noise(egb_ctx* ctx, const double* noise, int64_t len) {
  if (!ctx) return EGB_ERR_ARG;
  if (len < 0 || (len > 0 && !noise)) return fail(ctx, EGB_ERR_ARG, "invalid noise stream");
  cudaSetDevice(ctx->device);
  EGB_CUDA(cudaStreamSynchronize(ctx->stream));
  // captured graphs hold the stream's address: capture again
  ctx->graph_sig = 0;
  ctx->replay.valid = false;
  if (len > ctx->noise_len || !ctx->noise_d) {
    if (ctx->noise_d) cudaFree(ctx->noise_d);
    ctx->noise_d = nullptr;
    ctx->noise_len = 0;
    if (cudaMalloc(&ctx->noise_d, sizeof(double) * (size_t)std::max<int64_t>(len, 1)) != cudaSuccess) {
      cudaGetLastError();
      ctx->noise_d = nullptr;
      return fail(ctx, EGB_ERR_NOMEM, "noise stream allocation failed");
    }
  }
  if (len > 0) EGB_CUDA(cudaMemcpy(ctx->noise_d, noise, sizeof(double) * (size_t)len, cudaMemcpyHostToDevice));
  ctx->noise_len = len;
  return EGB_OK;
}

int egb_get_policy(const egb_ctx* ctx, int8_t* modes, int32_t n) {
  if (!ctx || !modes) return 0;
  const int m = std::min<int>(n, EGB_POLICY_ENTRIES);
  std::memcpy(modes, ctx->policy, (size_t)m);
  return m;
}

namespace {
int ensure_aux(egb_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->aux_cap) return EGB_OK;
  if (ctx->aux) cudaFree(ctx->aux);
  ctx->aux = nullptr;
  ctx->aux_cap = 0;
  const size_t want = align_up(bytes, 1 << 16);
  if (cudaMalloc(&ctx->aux, want) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, EGB_ERR_NOMEM, "device allocation of " + std::to_string(want) + " bytes failed");
  }
  ctx->aux_cap = want;
  return EGB_OK;
}
}  // namespace

int egb_pairwise_matrix(egb_ctx* ctx, const double* values, const int32_t* pairs, int32_t ntasks,
                        int32_t nvar, int32_t normalize, int32_t flags, double* out) {
  if (!ctx) return EGB_ERR_ARG;
  if (ntasks < 0 || nvar < 0 || (ntasks > 0 && (!values || !pairs)) || (nvar > 0 && !out))
    return fail(ctx, EGB_ERR_ARG, "egb_pairwise_matrix: invalid arguments");
  if ((int64_t)nvar * nvar > ((int64_t)1 << 31))
    return fail(ctx, EGB_ERR_ARG, "egb_pairwise_matrix: nvar too large");
  const bool dev = (flags & EGB_INPUT_DEVICE) != 0;
  if (!dev)
    for (int t = 0; t < ntasks; ++t)
      if (pairs[2 * t] < 0 || pairs[2 * t] >= nvar || pairs[2 * t + 1] < 0 || pairs[2 * t + 1] >= nvar)
        return fail(ctx, EGB_ERR_ARG, "egb_pairwise_matrix: pair " + std::to_string(t) + " out of range");
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const size_t nn = (size_t)nvar * (size_t)nvar;
  const double* vals_d = values;
  const int32_t* pairs_d = pairs;
  double* out_d = out;
  if (!dev) {
    const size_t op = align_up(sizeof(double) * (size_t)ntasks, 256);
    const size_t oo = op + align_up(sizeof(int32_t) * 2 * (size_t)ntasks, 256);
    const int rc = ensure_aux(ctx, oo + sizeof(double) * std::max<size_t>(nn, 1));
    if (rc) return rc;
    char* B = (char*)ctx->aux;
    vals_d = (const double*)B;
    pairs_d = (const int32_t*)(B + op);
    out_d = (double*)(B + oo);
    if (ntasks > 0) {
      EGB_CUDA(cudaMemcpyAsync(B, values, sizeof(double) * (size_t)ntasks, cudaMemcpyHostToDevice, st));
      EGB_CUDA(cudaMemcpyAsync(B + op, pairs, sizeof(int32_t) * 2 * (size_t)ntasks,
                               cudaMemcpyHostToDevice, st));
    }
  }
  launch_pairwise_matrix(vals_d, pairs_d, ntasks, nvar, normalize ? 1 : 0, out_d, st);
  EGB_CUDA(cudaGetLastError());
  if (!dev && nn) EGB_CUDA(cudaMemcpyAsync(out, out_d, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
  EGB_CUDA(cudaStreamSynchronize(st));
  return EGB_OK;
}

int egb_normalize(egb_ctx* ctx, const double* mi, int64_t n, int32_t flags, double* out) {
  if (!ctx) return EGB_ERR_ARG;
  if (n < 0 || (n > 0 && (!mi || !out))) return fail(ctx, EGB_ERR_ARG, "egb_normalize: invalid arguments");
  if (n == 0) return EGB_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const bool dev = (flags & EGB_INPUT_DEVICE) != 0;
  const double* in_d = mi;
  double* out_d = out;
  if (!dev) {
    const size_t half = align_up(sizeof(double) * (size_t)n, 256);
    const int rc = ensure_aux(ctx, 2 * half);
    if (rc) return rc;
    in_d = (const double*)ctx->aux;
    out_d = (double*)((char*)ctx->aux + half);
    EGB_CUDA(cudaMemcpyAsync((void*)in_d, mi, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
  }
  launch_normalize(in_d, n, out_d, st);
  EGB_CUDA(cudaGetLastError());
  if (!dev) EGB_CUDA(cudaMemcpyAsync(out, out_d, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st));
  EGB_CUDA(cudaStreamSynchronize(st));
  return EGB_OK;
}

int egb_debug_divide(egb_ctx* ctx, const double* a, const double* b, int64_t n, double* out) {
  if (!ctx) return EGB_ERR_ARG;
  if (n < 0 || (n > 0 && (!a || !b || !out))) return fail(ctx, EGB_ERR_ARG, "egb_debug_divide: invalid arguments");
  if (n == 0) return EGB_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const size_t part = align_up(sizeof(double) * (size_t)n, 256);
  const int rc = ensure_aux(ctx, 3 * part);
  if (rc) return rc;
  double* a_d = (double*)ctx->aux;
  double* b_d = (double*)((char*)ctx->aux + part);
  double* o_d = (double*)((char*)ctx->aux + 2 * part);
  EGB_CUDA(cudaMemcpyAsync(a_d, a, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
  EGB_CUDA(cudaMemcpyAsync(b_d, b, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
  launch_divide(a_d, b_d, n, o_d, st);
  EGB_CUDA(cudaGetLastError());
  EGB_CUDA(cudaMemcpyAsync(out, o_d, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st));
  EGB_CUDA(cudaStreamSynchronize(st));
  return EGB_OK;
}

int egb_last_groups(const egb_ctx* ctx, int32_t task, int64_t* out, int32_t max) {
  if (!ctx || !out || task < 0 || task >= (int)ctx->groups.size()) return 0;
  const int n = std::min(max, 6);
  for (int i = 0; i < n; ++i) out[i] = ctx->groups[(size_t)task][(size_t)i];
  return n;
}

int egb_debug_inject_device_error(egb_ctx* ctx, uint32_t word) {
  if (!ctx) return EGB_ERR_ARG;
  ctx->inject_err = word;
  return EGB_OK;
}

int egb_timings(const egb_ctx* ctx, double* ms, int32_t max) {
  if (!ctx || !ms) return 0;
  const int n = std::min<int>(max, ctx->ntimings);
  for (int i = 0; i < n; ++i) ms[i] = ctx->timings[i];
  return n;
}

int egb_last_transfer(const egb_ctx* ctx, int64_t* h2d_bytes, int64_t* d2h_bytes) {
  if (!ctx) return EGB_ERR_ARG;
  if (h2d_bytes) *h2d_bytes = ctx->h2d_bytes;
  if (d2h_bytes) *d2h_bytes = ctx->d2h_bytes;
  return EGB_OK;
}

int egb_last_stats(const egb_ctx* ctx, int64_t* out, int32_t max) {
  if (!ctx || !out) return 0;
  const int n = std::min<int>(max, NSTATS);
  for (int i = 0; i < n; ++i) out[i] = ctx->stats[i];
  return n;
}

int egb_device_info(const egb_ctx* ctx, char* name, int32_t len, int32_t* sms) {
  if (!ctx) return EGB_ERR_ARG;
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, ctx->device) != cudaSuccess) {
    cudaGetLastError();
    return EGB_ERR_CUDA;
  }
  if (name && len > 0) {
    std::strncpy(name, prop.name, (size_t)len - 1);
    name[len - 1] = 0;
  }
  if (sms) *sms = prop.multiProcessorCount;
  return EGB_OK;
}

const char* egb_version(void) { return "ennemi_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
