// egb_discrete.cu -- plug-in estimators of discrete variables: an exact
// group-by of rows on the device.
//
// ennemi's discrete estimators (ennemi/_entropy_estimators.py:44-56,
// :257-320) count distinct values with np.unique: the entropy of the rows of
// x, the MI of two discrete variables from the counts of (x, y), x and y, and
// the conditional MI as the count-weighted MI within each condition level.
// Per row, with c_S the number of rows equal to it on the columns S:
//   H(x)       = -(1/N) sum_rows log(c_x / N)
//   I(x; y)    =  (1/N) sum_rows log(N c_xy / (c_x c_y))
//   I(x; y | z) = (1/N) sum_rows log(c_z c_xyz / (c_xz c_yz))
// which are the reference's sums over distinct values, each value counted
// once per row it holds.  The counts come from one open-addressing hash
// table per (task, column subset): a row claims the first free slot of its
// probe sequence or joins the slot whose owner row has the same values
// (compared exactly, -0 equal to +0), so distinct rows never merge whatever
// the hash.  The combine kernel then sums the per-row logarithms.
#include "egb_internal.cuh"

namespace egb {
namespace {

constexpr int GB_THREADS = 256;

// splitmix64's finaliser (Steele, Lea and Flood, 2014) as the mixing step
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ int job_of(const GroupJob* __restrict__ jobs, int njobs, int b) {
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (jobs[m].blk0 <= b) lo = m; else hi = m;
  }
  return lo;
}

__global__ void __launch_bounds__(GB_THREADS)
group_insert_kernel(const TaskDev* __restrict__ tasks, const GroupJob* __restrict__ jobs, int njobs,
                    uint32_t* __restrict__ err) {
  const GroupJob& J = jobs[job_of(jobs, njobs, blockIdx.x)];
  const int row = ((int)blockIdx.x - J.blk0) * GB_THREADS + threadIdx.x;
  if (row >= J.n) return;
  const TaskDev& t = tasks[J.task];
  const int d = J.sp.d;
  uint64_t h = 0x243f6a8885a308d3ull;
  for (int c = 0; c < d; ++c) {
    uint64_t u = (uint64_t)__double_as_longlong(t.x64[(int64_t)J.sp.cols[c] * t.ld + row]);
    u = u == 0x8000000000000000ull ? 0ull : u;  // -0 hashes as +0
    h = mix64(h ^ u);
  }
  const uint32_t mask = (1u << J.cap_log2) - 1u;
  uint32_t slot = (uint32_t)h & mask;
  uint32_t probe = 0;
  for (; probe <= mask; ++probe) {
    int owner = *(volatile int32_t*)(J.table + slot);
    if (owner == 0) {
      owner = atomicCAS(J.table + slot, 0, row + 1);
      if (owner == 0) {  // a new distinct row
        atomicAdd(J.groups, 1ull);
        break;
      }
    }
    bool same = true;
    const int j = owner - 1;
    for (int c = 0; c < d && same; ++c) {
      const double* col = t.x64 + (int64_t)J.sp.cols[c] * t.ld;
      same = col[j] == col[row];
    }
    if (same) break;
    slot = (slot + 1u) & mask;
  }
  if (probe > mask) {  // a table is twice the rows: never full
    atomicOr(err, (uint32_t)DERR_BAD_INDEX);
    J.rowslot[row] = 0;
    return;
  }
  atomicAdd(J.count + slot, 1);
  J.rowslot[row] = (int32_t)slot;
}

// count slot of the task: rows equal to each row on the job's columns
__global__ void __launch_bounds__(GB_THREADS)
group_count_kernel(const TaskDev* __restrict__ tasks, const GroupJob* __restrict__ jobs, int njobs) {
  const GroupJob& J = jobs[job_of(jobs, njobs, blockIdx.x)];
  const int row = ((int)blockIdx.x - J.blk0) * GB_THREADS + threadIdx.x;
  if (row >= J.n) return;
  tasks[J.task].cnt[J.slot][row] = J.count[J.rowslot[row]];
}

// The reference's _verify_not_continuous, applied by the conditional
// discrete MI to each condition level's x and y (:291-320 via :280-281):
// per level, the distinct x (y) values against a quarter of the level's
// rows.  A row that owns its (x, z) slot is one distinct x of its level.
__global__ void __launch_bounds__(GB_THREADS)
level_distinct_kernel(const LevelCheck* __restrict__ checks, int nchecks) {
  const LevelCheck& C = checks[blockIdx.y];
  for (int row = blockIdx.x * GB_THREADS + threadIdx.x; row < C.n; row += gridDim.x * GB_THREADS) {
    const int zs = C.z_rowslot[row];
    const int xs = C.xz_rowslot[row], ys = C.yz_rowslot[row];
    if (C.xz_table[xs] == row + 1) atomicAdd(C.xd + zs, 1);
    if (C.yz_table[ys] == row + 1) atomicAdd(C.yd + zs, 1);
  }
}
__global__ void __launch_bounds__(GB_THREADS)
level_warn_kernel(const LevelCheck* __restrict__ checks, int nchecks) {
  const LevelCheck& C = checks[blockIdx.y];
  for (int row = blockIdx.x * GB_THREADS + threadIdx.x; row < C.n; row += gridDim.x * GB_THREADS) {
    const int zs = C.z_rowslot[row];
    if (C.z_table[zs] != row + 1) continue;  // one row per level
    const long long nz = C.z_count[zs];
    if (4ll * C.xd[zs] > nz) atomicAdd(C.warn + 0, 1ull);
    if (4ll * C.yd[zs] > nz) atomicAdd(C.warn + 1, 1ull);
  }
}

}  // namespace

void launch_level_checks(const LevelCheck* checks_d, int nchecks, int max_n, cudaStream_t st) {
  if (nchecks <= 0) return;
  int gx = (max_n + GB_THREADS - 1) / GB_THREADS;
  gx = gx < 1 ? 1 : gx > 1024 ? 1024 : gx;
  const dim3 grid(gx, nchecks);
  level_distinct_kernel<<<grid, GB_THREADS, 0, st>>>(checks_d, nchecks);
  count_launch();
  level_warn_kernel<<<grid, GB_THREADS, 0, st>>>(checks_d, nchecks);
  count_launch();
}

void launch_groups(const TaskDev* tasks_d, const GroupJob* jobs_d, int njobs, int total_blocks,
                   uint32_t* err, cudaStream_t st) {
  if (njobs <= 0 || total_blocks <= 0) return;
  group_insert_kernel<<<total_blocks, GB_THREADS, 0, st>>>(tasks_d, jobs_d, njobs, err);
  count_launch();
  group_count_kernel<<<total_blocks, GB_THREADS, 0, st>>>(tasks_d, jobs_d, njobs);
  count_launch();
}

}  // namespace egb
