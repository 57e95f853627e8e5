// egb_prep.cu -- data movement around the search kernels.
//
// gather       caller columns (strided, optionally class-permuted) -> the
//              task's working FP64 columns, zero padded up to ld;
// prepare      per working column the midrange centre (min/max over the
//              order-preserving integer keys, so -0.0/+0.0 and any finite
//              values compare exactly);
// materialize  per multi-D job: its columns copied into one SoA block in
//              working or sorted order, with the FP32 centred copy and the
//              job's "FP32 unsafe" flag (a centred value >= 1e37 or not
//              finite: every candidate of that job is then decided in FP64);
// radius       rad = fl64(eps - 1e-12): the reference's count radius
//              (ennemi/_entropy_estimators.py:109-110, :152-154, :196,
//              :243-245);
// combine      per-sample estimator term summed in fixed 4096-sample chunks
//              (deterministic order), plus per-slot "a count was zero" flags.
//              Terms, from ennemi/_entropy_estimators.py:
//                MI     psi(nx) + psi(ny)                       (:113)
//                CMI    psi(nxz) + psi(nyz) - psi(nz)           (:156)
//                SEMI   psi(n)                                  (:200)
//                CSEMI  psi(nxz) + psi(nyz) - psi(nz)           (:247)
//                ENT    log(eps)                                (:42)
//              psi comes from an FP64 table indexed by the integer count.
#include "egb_internal.cuh"
#include "ennemi_gb.h"

namespace egb {

namespace {

constexpr int PREP_THREADS = 256;

int grid_x_for(int64_t n) {
  int64_t b = (n + PREP_THREADS - 1) / PREP_THREADS;
  if (b > 2048) b = 2048;
  return (int)(b < 1 ? 1 : b);
}
int grid_y_for(int n) { return n > 65535 ? 65535 : (n < 1 ? 1 : n); }

// Four loads in flight per thread before its stores: columns read in place
// from host memory cross the CPU-GPU link, where throughput follows the
// requests outstanding.
constexpr int GATHER_UNROLL = 4;
__global__ void gather_kernel(const TaskDev* __restrict__ tasks,
                              const GatherCol* __restrict__ cols, int ncols) {
  for (int g = blockIdx.y; g < ncols; g += gridDim.y) {
    const GatherCol gc = cols[g];
    const TaskDev t = tasks[gc.task];
    double* dst = const_cast<double*>(t.x64) + (int64_t)gc.col * t.ld;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t w0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w0 < t.ld;
         w0 += GATHER_UNROLL * step) {
      double v[GATHER_UNROLL];
#pragma unroll
      for (int u = 0; u < GATHER_UNROLL; ++u) {
        const int64_t w = w0 + u * step;
        v[u] = 0.0;
        if (w < t.n) {
          const int64_t s = gc.perm ? (int64_t)gc.perm[w] : w;
          v[u] = gc.src[s * gc.stride];
        }
      }
#pragma unroll
      for (int u = 0; u < GATHER_UNROLL; ++u) {
        const int64_t w = w0 + u * step;
        if (w < t.ld) dst[w] = v[u];
      }
    }
  }
}

// ----------------------------------------------------------- rescale --
// The reference's _rescale_data (_driver.py:871-902) per column, bit for bit:
// mean = pairwise_sum(x) / n, std = sqrt(pairwise_sum((x - mean)^2) / n),
// x = (x - mean) / std + noise -- every operation one IEEE double rounding
// (explicit _rn intrinsics: no contraction), the sums in NumPy's order.

// Sample i of the column: x[i], or x[inv[i]] for a class-ordered task.
__device__ __forceinline__ double pw_value(const double* a, const int32_t* inv, int i, bool sq,
                                           double m) {
  const double v = inv ? a[inv[i]] : a[i];
  if (!sq) return v;
  const double d = __dsub_rn(v, m);
  return __dmul_rn(d, d);
}

// One leaf of pairwise_sum: fewer than 8 values in order from 0.0; else eight
// running sums over strides of 8, combined ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)),
// then the remaining (len % 8) values in order.
// (a, inv: the column with the leaf's first sample at index 0)
__device__ double pw_leaf(const double* a, const int32_t* inv, int len, bool sq, double m) {
  if (len < 8) {
    double r = 0.0;
    for (int i = 0; i < len; ++i) r = __dadd_rn(r, pw_value(a, inv, i, sq, m));
    return r;
  }
  double r0 = pw_value(a, inv, 0, sq, m), r1 = pw_value(a, inv, 1, sq, m), r2 = pw_value(a, inv, 2, sq, m),
         r3 = pw_value(a, inv, 3, sq, m), r4 = pw_value(a, inv, 4, sq, m), r5 = pw_value(a, inv, 5, sq, m),
         r6 = pw_value(a, inv, 6, sq, m), r7 = pw_value(a, inv, 7, sq, m);
  const int end = len - (len % 8);
  int i = 8;
  for (; i < end; i += 8) {
    r0 = __dadd_rn(r0, pw_value(a, inv, i + 0, sq, m));
    r1 = __dadd_rn(r1, pw_value(a, inv, i + 1, sq, m));
    r2 = __dadd_rn(r2, pw_value(a, inv, i + 2, sq, m));
    r3 = __dadd_rn(r3, pw_value(a, inv, i + 3, sq, m));
    r4 = __dadd_rn(r4, pw_value(a, inv, i + 4, sq, m));
    r5 = __dadd_rn(r5, pw_value(a, inv, i + 5, sq, m));
    r6 = __dadd_rn(r6, pw_value(a, inv, i + 6, sq, m));
    r7 = __dadd_rn(r7, pw_value(a, inv, i + 7, sq, m));
  }
  double res = __dadd_rn(__dadd_rn(__dadd_rn(r0, r1), __dadd_rn(r2, r3)),
                         __dadd_rn(__dadd_rn(r4, r5), __dadd_rn(r6, r7)));
  for (; i < len; ++i) res = __dadd_rn(res, pw_value(a, inv, i, sq, m));
  return res;
}

// The block's pairwise sum of x[0, n) (sq: of (x - m)^2): leaves in parallel,
// then one height at a time; node sums in ns (global, read back through L2).
__device__ double pw_sum(const double* x, const int32_t* inv, const PwTree& tr,
                         const int2* __restrict__ nodes, const int32_t* __restrict__ levels,
                         double* ns, bool sq, double m) {
  for (int i = threadIdx.x; i < tr.nleaf; i += blockDim.x) {
    const int2 L = nodes[tr.node0 + i];
    ns[i] = inv ? pw_leaf(x, inv + L.x, L.y, sq, m) : pw_leaf(x + L.x, nullptr, L.y, sq, m);
  }
  __syncthreads();
  for (int h = 0; h < tr.nlvl; ++h) {
    const int a = levels[tr.lvl0 + h], b = levels[tr.lvl0 + h + 1];
    for (int i = a + threadIdx.x; i < b; i += blockDim.x) {
      const int2 c = nodes[tr.node0 + i];
      ns[i] = __dadd_rn(__ldcg(ns + c.x), __ldcg(ns + c.y));
    }
    __syncthreads();
  }
  return __ldcg(ns + tr.nnode - 1);
}

__global__ void __launch_bounds__(PREP_THREADS)
rescale_stats_kernel(const TaskDev* __restrict__ tasks, const RescaleStat* __restrict__ stats,
                     const PwTree* __restrict__ trees, const int2* __restrict__ nodes,
                     const int32_t* __restrict__ levels, double* __restrict__ scratch,
                     double2* __restrict__ ms) {
  const RescaleStat rs = stats[blockIdx.x];
  const TaskDev t = tasks[rs.task];
  const double* x = t.x64 + (int64_t)rs.col * t.ld;
  const double n = (double)t.n;
  if (rs.group > 1) {  // axis-0 reduction of an (n, group) array: in row order
    if (threadIdx.x == 0) {
      double s = pw_value(x, rs.inv, 0, false, 0.0);
      for (int i = 1; i < t.n; ++i) s = __dadd_rn(s, pw_value(x, rs.inv, i, false, 0.0));
      const double m = __ddiv_rn(s, n);
      double q = pw_value(x, rs.inv, 0, true, m);
      for (int i = 1; i < t.n; ++i) q = __dadd_rn(q, pw_value(x, rs.inv, i, true, m));
      ms[blockIdx.x] = make_double2(m, __dsqrt_rn(__ddiv_rn(q, n)));
    }
    return;
  }
  const PwTree tr = trees[rs.tree];
  double* ns = scratch + rs.scratch;
  const double mean = __ddiv_rn(pw_sum(x, rs.inv, tr, nodes, levels, ns, false, 0.0), n);
  __syncthreads();  // every thread has read the root before the slots are reused
  const double sd = __dsqrt_rn(__ddiv_rn(pw_sum(x, rs.inv, tr, nodes, levels, ns, true, mean), n));
  if (threadIdx.x == 0) ms[blockIdx.x] = make_double2(mean, sd);
}

// RN(a / b) without a division per element.  q = RN(a * rb) (rb = RN(1/b))
// is within two ulps of the quotient; the remainder a - q b from one FMA is
// exact once q is within one ulp (the remainder of a faithful quotient is
// representable: Boldo and Daumas, 2003), and the quotient lies above the
// midpoint between q and its successor exactly when that remainder exceeds
// half an ulp of q times b -- a power-of-two multiple of b, built by integer
// exponent arithmetic.  q steps one ulp at a time until the remainder lies
// between the two midpoints; a remainder equal to one of them is a tie,
// rounded to the even neighbour.  Magnitudes throughout, the sign applied at
// the end (round to nearest is symmetric).  Operands outside the exponent
// range where no step can underflow or overflow take the division itself.
// One FP64 multiply and one or two FMAs per element, against the FP64 pipe's
// few operations per clock per SM.
__device__ __forceinline__ double div_rn(double a, double b, double rb) {
  const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  const uint64_t ma = ua & 0x7fffffffffffffffull, mb = ub & 0x7fffffffffffffffull;
  const int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
  if (ea < 1023 - 900 || ea > 1023 + 900 || eb < 1023 - 900 || eb > 1023 + 900 ||
      abs(ea - eb) > 1000)
    return __ddiv_rn(a, b);
  const double A = __longlong_as_double((long long)ma), B = __longlong_as_double((long long)mb);
  const int64_t half_b = (int64_t)mb - ((int64_t)1 << 52);  // bits of B / 2
  double q = __dmul_rn(A, fabs(rb));
  for (int it = 0; it < 4; ++it) {
    const double e = __fma_rn(-q, B, A);  // A - q B
    const uint64_t uq = (uint64_t)__double_as_longlong(q);
    const int eq = (int)(uq >> 52);
    // half an ulp of q above (and below: half that at a power of two) times B
    const uint64_t h_up = (uint64_t)(half_b + ((int64_t)(eq - 1075) << 52));
    const uint64_t h_dn = (uq & 0xfffffffffffffull) ? h_up : h_up - (1ull << 52);
    const uint64_t ue = (uint64_t)__double_as_longlong(e);
    const uint64_t me = ue & 0x7fffffffffffffffull;
    const bool neg = (ue >> 63) != 0 && me != 0;
    if (!neg && me > h_up) { q = __longlong_as_double((long long)(uq + 1)); continue; }
    if (neg && me > h_dn) { q = __longlong_as_double((long long)(uq - 1)); continue; }
    if (!neg && me == h_up) q = __longlong_as_double((long long)((uq & 1) ? uq + 1 : uq));
    else if (neg && me == h_dn) q = __longlong_as_double((long long)((uq & 1) ? uq - 1 : uq));
    return __longlong_as_double((long long)((uint64_t)__double_as_longlong(q) | sign));
  }
  return __ddiv_rn(a, b);  // not settled in four steps (not met in the fast range)
}

// x = RN(RN(RN(x - mean) / sd) + noise) per sample of a task column (one
// y-row of blocks per column, four samples in flight per thread)
__global__ void __launch_bounds__(PREP_THREADS)
rescale_apply_kernel(const TaskDev* __restrict__ tasks, const RescaleCol* __restrict__ cols,
                     const double2* __restrict__ ms, const double* __restrict__ noise,
                     uint32_t* __restrict__ zero_flags) {
  const RescaleCol rc = cols[blockIdx.y];
  const TaskDev t = tasks[rc.task];
  double* x = const_cast<double*>(t.x64) + (int64_t)rc.col * t.ld;
  const double2 m = ms[rc.stat];
  const double mean = m.x, sd = m.y;
  if (fabs(sd) < 1e-20) {  // np.abs(std) < 1e-20: the reference warns and keeps x
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(zero_flags + rc.task, RESCALE_CONSTANT);
    return;
  }
  __shared__ double rsd_s;  // RN(1 / sd), once per block
  if (threadIdx.x == 0) rsd_s = __ddiv_rn(1.0, sd);
  __syncthreads();
  const double rsd = rsd_s;
  const double* nz = noise + rc.noise_pos;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < t.n; i0 += 4 * step) {
    int w[4];
    double v[4], z[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {  // sample i0 + u * step
      const int64_t i = i0 + u * step;
      w[u] = -1;
      if (i < t.n) {
        w[u] = rc.inv ? rc.inv[i] : (int)i;
        v[u] = x[w[u]];
        z[u] = nz[i * rc.group];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (w[u] >= 0) x[w[u]] = __dadd_rn(div_rn(__dsub_rn(v[u], mean), sd, rsd), z[u]);
  }
}

// egb_debug_divide: div_rn over n pairs (one thread per pair)
__global__ void divide_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                              double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = div_rn(a[i], b[i], __ddiv_rn(1.0, b[i]));
}

__global__ void minmax_kernel(const TaskDev* __restrict__ tasks,
                              const int32_t* __restrict__ col_task,
                              const int32_t* __restrict__ col_idx, int ncols,
                              unsigned long long* __restrict__ minmax) {
  for (int g = blockIdx.y; g < ncols; g += gridDim.y) {
    const TaskDev t = tasks[col_task[g]];
    const double* x = t.x64 + (int64_t)col_idx[g] * t.ld;
    unsigned long long lo = ~0ull, hi = 0ull;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < t.n; i += 4 * stride) {  // four loads in flight
      const double v0 = x[i], v1 = x[i + stride], v2 = x[i + 2 * stride], v3 = x[i + 3 * stride];
      const unsigned long long k0 = key_of(v0), k1 = key_of(v1), k2 = key_of(v2), k3 = key_of(v3);
      lo = min(min(lo, k0), min(k1, min(k2, k3)));
      hi = max(max(hi, k0), max(k1, max(k2, k3)));
    }
    for (; i < t.n; i += stride) {
      const unsigned long long k = key_of(x[i]);
      lo = k < lo ? k : lo;
      hi = k > hi ? k : hi;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o);
      const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi, o);
      lo = a < lo ? a : lo;
      hi = b > hi ? b : hi;
    }
    // one pair of atomics per block (per warp they queue up at the column's
    // two words)
    __shared__ unsigned long long wlo[PREP_THREADS / 32], whi[PREP_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
      wlo[warp] = lo;
      whi[warp] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < PREP_THREADS / 32; ++w) {
        lo = wlo[w] < lo ? wlo[w] : lo;
        hi = whi[w] > hi ? whi[w] : hi;
      }
      atomicMin(&minmax[2 * g], lo);
      atomicMax(&minmax[2 * g + 1], hi);
    }
    __syncthreads();
  }
}

__global__ void center_kernel(const unsigned long long* __restrict__ minmax, int ncols,
                              double* __restrict__ centers) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ncols) return;
  const double lo = value_of(minmax[2 * g]);
  const double hi = value_of(minmax[2 * g + 1]);
  centers[g] = 0.5 * lo + 0.5 * hi;
}

__device__ __forceinline__ bool materialize_copy(const TaskDev& t, const JobDev& J, int d,
                                                 double* c64, float* c32, int32_t* idx,
                                                 const int32_t* sv) {
  bool bad = false;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < J.lds;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (p < J.len) {
      const int32_t w = sv ? sv[p] : J.seg_begin + (int32_t)p;
      idx[p] = w;
      for (int c = 0; c < d; ++c) {
        const int tc = J.sp.cols[c];
        const double v = t.x64[(int64_t)tc * t.ld + w];
        const double cv = v - t.center[tc];
        bad |= !(fabs(cv) < 1e37);
        c64[(int64_t)c * J.lds + p] = v;
        // clamped so that FP32 distances stay finite; a job with a clamped
        // value never trusts its FP32 copy (TF_UNSAFE32)
        c32[(int64_t)c * J.lds + p] = __double2float_rn(fmin(fmax(cv, -1e37), 1e37));
      }
    } else {
      idx[p] = J.seg_begin;
      for (int c = 0; c < d; ++c) {
        c64[(int64_t)c * J.lds + p] = 0.0;
        c32[(int64_t)c * J.lds + p] = 0.0f;
      }
    }
  }
  return bad;
}

__global__ void materialize_kernel(const TaskDev* __restrict__ tasks,
                                   const JobDev* __restrict__ jobs, int njobs,
                                   const int32_t* __restrict__ sorted_vals,
                                   const SortSeg* __restrict__ segs) {
  for (int jb = blockIdx.y; jb < njobs; jb += gridDim.y) {
    const JobDev J = jobs[jb];
    const TaskDev t = tasks[J.task];
    const int d = J.sp.d;
    if (blockIdx.x == 0 && threadIdx.x < d) J.center[threadIdx.x] = t.center[J.sp.cols[threadIdx.x]];
    if (J.c64 == nullptr) continue;  // grid copy only (materialize_grid_kernel)
    const int32_t* sv = J.slab ? sorted_vals + segs[J.sort_seg].out_base : nullptr;
    bool bad = materialize_copy(t, J, d, J.c64, J.c32, J.idx, sv);
    if (J.c64b != nullptr)  // second copy, sorted by column 1 (same values)
      materialize_copy(t, J, d, J.c64b, J.c32b, J.idxb, sorted_vals + segs[J.sort_seg_b].out_base);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(J.jflags, (uint32_t)TF_UNSAFE32);
  }
}

// Grid copy: position p_G of the strip order takes the point at column-0
// position p_A = gvals_sorted[p_G].
__global__ void materialize_grid_kernel(const TaskDev* __restrict__ tasks,
                                        const JobDev* __restrict__ jobs,
                                        const int32_t* __restrict__ grid_jobs, int ngrid,
                                        const int32_t* __restrict__ sorted_vals,
                                        const SortSeg* __restrict__ segs,
                                        const int32_t* __restrict__ gvals_sorted,
                                        const SortSeg* __restrict__ gsegs) {
  for (int g = blockIdx.y; g < ngrid; g += gridDim.y) {
    const JobDev J = jobs[grid_jobs[g]];
    const TaskDev t = tasks[J.task];
    const int d = J.sp.d;
    const int32_t* va = sorted_vals + segs[J.sort_seg].out_base;
    const int32_t* gv = gvals_sorted + gsegs[J.gseg].out_base;
    // column-1 bounds of each strip, from the column-1 sort
    const int32_t* vb = sorted_vals + segs[J.sort_seg_b].out_base;
    const double* x1 = t.x64 + (int64_t)J.sp.cols[1] * t.ld;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < J.nstrips; s += gridDim.x * blockDim.x) {
      const double lo = x1[vb[J.sstart[s]]];
      const double hi = x1[vb[J.sstart[s + 1] - 1]];
      J.sylo[s] = lo;
      J.syhi[s] = hi;
      J.sylo32[s] = __double2float_rd(__dsub_rd(lo, J.center[1]));
      J.syhi32[s] = __double2float_ru(__dsub_ru(hi, J.center[1]));
    }
    bool bad = false;  // a centred value too large for the FP32 copy
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < J.lds;
         p += (int64_t)gridDim.x * blockDim.x) {
      if (p < J.len) {
        const int32_t pa = gv[p];
        const int32_t w = va[pa];
        J.posg[p] = pa;
        J.idxg[p] = w;
        for (int c = 0; c < d; ++c) {
          const int tc = J.sp.cols[c];
          const double v = t.x64[(int64_t)tc * t.ld + w];
          if (J.kform) {
            const uint64_t k = raw_key((uint64_t)__double_as_longlong(v));
            uint32_t* kw = reinterpret_cast<uint32_t*>(J.c64g);
            kw[(int64_t)(2 * c) * J.lds + p] = (uint32_t)(k >> 32);
            kw[(int64_t)(2 * c + 1) * J.lds + p] = (uint32_t)k;
          } else {
            const double cv = v - t.center[tc];
            bad |= !(fabs(cv) < 1e37);
            J.c64g[(int64_t)c * J.lds + p] = v;
            J.c32g[(int64_t)c * J.lds + p] = __double2float_rn(fmin(fmax(cv, -1e37), 1e37));
          }
        }
      } else {
        J.posg[p] = 0;
        J.idxg[p] = J.seg_begin;
        for (int c = 0; c < d; ++c) {
          if (J.kform) {
            uint32_t* kw = reinterpret_cast<uint32_t*>(J.c64g);
            kw[(int64_t)(2 * c) * J.lds + p] = 0u;
            kw[(int64_t)(2 * c + 1) * J.lds + p] = 0u;
          } else {
            J.c64g[(int64_t)c * J.lds + p] = 0.0;
            J.c32g[(int64_t)c * J.lds + p] = 0.0f;
          }
        }
      }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(J.jflags, (uint32_t)TF_UNSAFE32);
  }
}

__global__ void radius_kernel(const TaskDev* __restrict__ tasks, int ntasks) {
  for (int ti = blockIdx.y; ti < ntasks; ti += gridDim.y) {
    const TaskDev t = tasks[ti];
    if (t.rad_given) continue;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < t.n;
         i += (int64_t)gridDim.x * blockDim.x)
      t.rad[i] = t.eps[i] - 1e-12;
  }
}

__device__ __forceinline__ double psi_of(const double* __restrict__ tab, int64_t len, int32_t n,
                                         uint32_t& bad) {
  if (n < 0 || n >= len) {
    bad = 1u;
    return 0.0;
  }
  return tab[n];  // entry 0 is a placeholder; zero counts are flagged
}

__global__ void combine_kernel(const TaskDev* __restrict__ tasks,
                               const CombineJob* __restrict__ jobs,
                               const int32_t* __restrict__ chunk_job,
                               const double* __restrict__ psi_tab, int64_t psi_len,
                               double* __restrict__ partial, uint32_t* __restrict__ zero_flags,
                               uint32_t* __restrict__ err) {
  const int chunk = blockIdx.x;
  const CombineJob jb = jobs[chunk_job[chunk]];
  const TaskDev t = tasks[jb.task];
  const int64_t p0 = (int64_t)(chunk - jb.chunk0) * COMBINE_CHUNK;
  const int64_t p1 = p0 + COMBINE_CHUNK < (int64_t)t.n ? p0 + COMBINE_CHUNK : (int64_t)t.n;
  double acc = 0.0;
  uint32_t zf = 0, bad = 0;
  for (int64_t i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
    double term;
    switch (jb.kind) {
      case EGB_MI: {
        const int32_t a = t.cnt[0][i], b = t.cnt[1][i];
        zf |= (a == 0 ? 1u : 0u) | (b == 0 ? 2u : 0u);
        term = psi_of(psi_tab, psi_len, a, bad) + psi_of(psi_tab, psi_len, b, bad);
        break;
      }
      case EGB_CMI:
      case EGB_CSEMI: {
        const int32_t a = t.cnt[0][i], b = t.cnt[1][i], c = t.cnt[2][i];
        zf |= (a == 0 ? 1u : 0u) | (b == 0 ? 2u : 0u) | (c == 0 ? 4u : 0u);
        term = (psi_of(psi_tab, psi_len, a, bad) + psi_of(psi_tab, psi_len, b, bad)) -
               psi_of(psi_tab, psi_len, c, bad);
        break;
      }
      case EGB_SEMI: {
        const int32_t a = t.cnt[0][i];
        zf |= (a == 0 ? 1u : 0u);
        term = psi_of(psi_tab, psi_len, a, bad);
        break;
      }
      case EGB_DISCRETE_ENTROPY: {   // log(c / N)
        term = log((double)t.cnt[0][i] / (double)t.n);
        break;
      }
      case EGB_DISCRETE_MI: {        // log(N c_xy / (c_x c_y)), integer products exact
        const int64_t num = (int64_t)t.n * t.cnt[0][i];
        const int64_t den = (int64_t)t.cnt[1][i] * t.cnt[2][i];
        term = log((double)num / (double)den);
        break;
      }
      case EGB_DISCRETE_CMI: {       // log(c_z c_xyz / (c_xz c_yz))
        const int64_t num = (int64_t)t.cnt[3][i] * t.cnt[0][i];
        const int64_t den = (int64_t)t.cnt[1][i] * t.cnt[2][i];
        term = log((double)num / (double)den);
        break;
      }
      default: {  // EGB_ENTROPY: log(0) = -inf propagates exactly as in NumPy
        const double e = t.eps[i];
        zf |= (e == 0.0 ? 1u : 0u);
        term = log(e);
        break;
      }
    }
    acc += term;
  }
  // fixed-order block reduction: warp shuffles, then warp 0 over warp sums
  __shared__ double wsum[32];
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  zf = __reduce_or_sync(0xffffffffu, zf);
  bad = __reduce_or_sync(0xffffffffu, bad);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = acc;
  if (lane == 0 && zf) atomicOr(&zero_flags[jb.task], zf);
  if (lane == 0 && bad) atomicOr(err, (uint32_t)DERR_BAD_INDEX);
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    double v = lane < nw ? wsum[lane] : 0.0;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) partial[chunk] = v;
  }
}

}  // namespace

void launch_gather(const TaskDev* tasks_d, const GatherCol* cols_d, int ncols, int64_t max_ld,
                   cudaStream_t st) {
  if (ncols <= 0) return;
  dim3 grid(grid_x_for((max_ld + GATHER_UNROLL - 1) / GATHER_UNROLL), grid_y_for(ncols));
  gather_kernel<<<grid, PREP_THREADS, 0, st>>>(tasks_d, cols_d, ncols);
  count_launch();
}

void launch_rescale(const TaskDev* tasks_d, const RescaleStat* stats_d, int nstats,
                    const RescaleCol* cols_d, int ncols, const PwTree* trees_d,
                    const int2* nodes_d, const int32_t* levels_d, double* scratch, double2* ms,
                    const double* noise, uint32_t* zero_flags, int64_t max_n, cudaStream_t st) {
  if (ncols <= 0 || nstats <= 0) return;
  rescale_stats_kernel<<<nstats, PREP_THREADS, 0, st>>>(tasks_d, stats_d, trees_d, nodes_d, levels_d,
                                                        scratch, ms);
  count_launch();
  const dim3 agrid(grid_x_for((max_n + 3) / 4 / 8), grid_y_for(ncols));  // 32 samples a thread
  rescale_apply_kernel<<<agrid, PREP_THREADS, 0, st>>>(tasks_d, cols_d, ms, noise, zero_flags);
  count_launch();
}

void launch_divide(const double* a_d, const double* b_d, int64_t n, double* out_d, cudaStream_t st) {
  if (n <= 0) return;
  divide_kernel<<<grid_x_for(n), PREP_THREADS, 0, st>>>(a_d, b_d, n, out_d);
  count_launch();
}

void launch_prepare(const TaskDev* tasks_d, const int32_t* col_task_d, const int32_t* col_idx_d,
                    int ncols_total, int64_t max_n, unsigned long long* minmax_d,
                    double* centers_d, cudaStream_t st) {
  if (ncols_total <= 0) return;
  // slot 2g holds the min key (starts all-ones), slot 2g+1 the max key
  // (starts at zero)
  cudaMemsetAsync(minmax_d, 0, sizeof(unsigned long long) * 2 * ncols_total, st);
  cudaMemset2DAsync(minmax_d, 2 * sizeof(unsigned long long), 0xff, sizeof(unsigned long long),
                    ncols_total, st);
  dim3 grid(grid_x_for((max_n + 7) / 8), grid_y_for(ncols_total));  // eight values a thread
  minmax_kernel<<<grid, PREP_THREADS, 0, st>>>(tasks_d, col_task_d, col_idx_d, ncols_total,
                                                minmax_d);
  count_launch();
  center_kernel<<<(ncols_total + 255) / 256, 256, 0, st>>>(minmax_d, ncols_total, centers_d);
  count_launch();
}

void launch_materialize(const TaskDev* tasks_d, const JobDev* jobs_d, int njobs,
                        const int32_t* sorted_vals, const SortSeg* segs_d, int64_t max_lds,
                        cudaStream_t st) {
  if (njobs <= 0) return;
  dim3 grid(grid_x_for(max_lds), grid_y_for(njobs));
  materialize_kernel<<<grid, PREP_THREADS, 0, st>>>(tasks_d, jobs_d, njobs, sorted_vals, segs_d);
  count_launch();
}

namespace {
// One thread per item: its run (the last whose first item is <= it), then
// its cell within the run, both by binary search over the item offsets.
__global__ void emit_items_kernel(const JobDev* __restrict__ jobs, const ItemRun* __restrict__ runs,
                                  int nruns, const int32_t* __restrict__ cum, int64_t nitems,
                                  WorkItem* __restrict__ items) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nitems;
       t += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nruns;
    while (hi - lo > 1) {
      const int m = (lo + hi) >> 1;
      if (cum[runs[m].cum0] <= t) lo = m; else hi = m;
    }
    const ItemRun r = runs[lo];
    int c0 = 0, c1 = r.ncell;  // the last cell whose first item is <= t
    while (c1 - c0 > 1) {
      const int m = (c0 + c1) >> 1;
      if (cum[r.cum0 + m] <= t) c0 = m; else c1 = m;
    }
    const JobDev& J = jobs[r.job];
    int a, b, code;
    if (J.nsub > 0) {
      a = J.cstart[c0];
      b = J.cstart[c0 + 1];
      code = (c0 / J.nsub) | ((c0 % J.nsub) << 16);
    } else {
      a = J.sstart[c0];
      b = J.sstart[c0 + 1];
      code = c0;
    }
    const int q0 = a + (int)(t - cum[r.cum0 + c0]) * r.qb;
    items[t] = WorkItem{r.job, q0, min(q0 + r.qb, b), code};
  }
}
}  // namespace

void launch_emit_items(const JobDev* jobs_d, const ItemRun* runs_d, int nruns, const int32_t* cum_d,
                       int64_t nitems, WorkItem* items_d, cudaStream_t st) {
  if (nruns <= 0 || nitems <= 0) return;
  int grid = (int)((nitems + 255) / 256);
  if (grid > 8192) grid = 8192;
  emit_items_kernel<<<grid, 256, 0, st>>>(jobs_d, runs_d, nruns, cum_d, nitems, items_d);
  count_launch();
}

void launch_materialize_grid(const TaskDev* tasks_d, const JobDev* jobs_d,
                             const int32_t* grid_jobs_d, int ngrid, const int32_t* sorted_vals,
                             const SortSeg* segs_d, const int32_t* gvals_sorted,
                             const SortSeg* gsegs_d, int64_t max_lds, cudaStream_t st) {
  if (ngrid <= 0) return;
  dim3 grid(grid_x_for(max_lds), grid_y_for(ngrid));
  materialize_grid_kernel<<<grid, PREP_THREADS, 0, st>>>(tasks_d, jobs_d, grid_jobs_d, ngrid,
                                                         sorted_vals, segs_d, gvals_sorted, gsegs_d);
  count_launch();
}

void launch_radius(const TaskDev* tasks_d, int ntasks, int64_t max_ld, cudaStream_t st) {
  if (ntasks <= 0) return;
  dim3 grid(grid_x_for(max_ld), grid_y_for(ntasks));
  radius_kernel<<<grid, PREP_THREADS, 0, st>>>(tasks_d, ntasks);
  count_launch();
}

void launch_combine(const TaskDev* tasks_d, const CombineJob* jobs_d, const int32_t* chunk_job_d,
                    int nchunks, const double* psi_tab, int64_t psi_len, double* partial,
                    uint32_t* zero_flags, uint32_t* err, cudaStream_t st) {
  if (nchunks <= 0) return;
  combine_kernel<<<nchunks, 256, 0, st>>>(tasks_d, jobs_d, chunk_job_d, psi_tab, psi_len,
                                          partial, zero_flags, err);
  count_launch();
}

}  // namespace egb
