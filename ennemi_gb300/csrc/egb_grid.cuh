// egb_grid.cuh -- kNN distances and ball counts over the strip layout of a
// multi-D job (the "grid" form of the tile kernels).
//
// Layout (JobDev::c64g/c32g): the job's points split into nstrips
// equal-count strips by their rank in column 1; inside a strip they are
// sorted by column 0.  Strip s covers column-1 values [ylo(s), yhi(s)], read
// exactly from the column-1 sorted copy (c64b).
//
// A work item is up to GRID_QB consecutive positions of one strip.  With
//   xa, xb  = column 0 of its first and last query (sorted),
//   T       = the largest current threshold of its queries (k-th distance
//             so far, or count radius),
// the candidates it must see are, in every strip s that is still open, the
// positions with column 0 in [xa - T, xb + T]: any other point p of strip s
// has |p_0 - q_0| > t_q for every query q (order of column 0 inside the
// strip), hence an FP64 max-norm distance > t_q (rounding is monotone).  A
// strip above the home strip is open while some query has
// fl64(ylo(s) - q_1) <= t_q; once closed for all queries, every strip above
// it is too (strips are ordered in column 1).  Likewise below with yhi.
//
// The window in a strip is found with one round of THREADS evenly spaced
// probes (two __syncthreads_count), giving a range that contains the exact
// one (at most one probe spacing wider at each end).  Ranges of different
// strips are disjoint, so every candidate is seen at most once (counts
// stay exact).  Visiting order: the queries' own positions, the rest of the
// home strip's window, then strips sq+1, sq-1, sq+2, ...
//
// Candidates are staged GRID_TILE at a time with cp.async.bulk from a
// 4-element aligned start (bits outside the range are masked), double
// buffered.  The FP32 screen and FP64 decision are those of the slab kernels
// (egb_knn.cuh, egb_count.cuh).  Beyond the home strip, the window
// half-width T is the largest threshold among queries that are not finished
// yet.  An item stops once at most 1/32 of its threads hold unfinished
// queries (or after SIDE_CAP strips); those queries are deferred, with their
// current threshold, to the warp-per-query kernels.
#pragma once
#include "egb_tile.cuh"

namespace egb {
namespace grid_detail {

constexpr int TS = GRID_TILE + 8;  // shared-memory column stride (elements)
constexpr int GRID_DEFER_FRAC = 32;  // stop once <= 1/32 of the threads are unfinished

template <int U>
__device__ __forceinline__ float pick4(const float4& v) {
  return U == 0 ? v.x : U == 1 ? v.y : U == 2 ? v.z : v.w;
}

__device__ __forceinline__ float thr_from(uint64_t kth_bits, float mq) {
  if (kth_bits >= INF_BITS) return __int_as_float(0x7f800000);
  const float tu = f32_up_of_bits(kth_bits);
  return __fmaf_ru(tu, 1.0f + 0x1p-21f, __fmaf_ru(mq, 0x1p-21f, 0x1p-100f));
}

template <int KMAX>
__device__ __forceinline__ void insert_sorted(uint64_t (&top)[KMAX], uint64_t v) {
  top[KMAX - 1] = v;
#pragma unroll
  for (int s = KMAX - 1; s > 0; --s) {
    const uint64_t a = top[s - 1], b = top[s];
    const bool sw = b < a;
    top[s - 1] = sw ? b : a;
    top[s] = sw ? a : b;
  }
}

// Stage [t0, t1) of column block g (stride lds) into buffer buf (thread 0).
template <typename T>
__device__ __forceinline__ void stage_range(T* tiles, int DM, int buf, const T* g, int64_t lds,
                                            int d, int t0, int t1, uint64_t* bar) {
  const int a = t0 & ~3;
  const int b = (t1 + 3) & ~3;
  const uint32_t bytes = (uint32_t)(b - a) * (uint32_t)sizeof(T);
  fence_proxy_async_smem();
  mbar_expect_tx(bar, bytes * (uint32_t)d);
#pragma unroll 1
  for (int c = 0; c < d; ++c)
    bulk_g2s(tiles + ((size_t)buf * DM + c) * TS, g + (int64_t)c * lds + a, bytes, bar);
}

// Uniform (CTA-wide) schedule of ranges and tiles for one grid item.
struct GridSched {
  int sq, S, len;
  int s0, s1;          // home strip bounds
  int up, dn;          // next strips above / below not yet visited
  bool up_open, dn_open;
  int stage;           // 0 own queries, 1 home left, 2 home right, 3 strips
  bool turn_up;
  int ra, rb, pos;     // current range and next tile start
  int strips_done;     // strips beyond the home strip whose ranges were taken
};

template <int THREADS, bool PLAIN>
struct GridItem {
  // Window [lo, hi) of strip s for column-0 values [xlo, xhi]: one round of
  // THREADS probes.  All threads call it.
  __device__ static void window(const double* x, int s0, int s1, double xlo, double xhi, int& lo,
                                int& hi) {
    const int size = s1 - s0;
    const int tid = threadIdx.x;
    const int p = s0 + (int)((int64_t)tid * size / THREADS);
    const double v = x[p];
    const int cl = __syncthreads_count(v < xlo);
    const int ch = __syncthreads_count(v <= xhi);
    lo = cl == 0 ? s0 : s0 + (int)((int64_t)(cl - 1) * size / THREADS);
    hi = ch == THREADS ? s1 : s0 + (int)((int64_t)ch * size / THREADS);
    if (hi < lo) hi = lo;
  }
};

// Block-wide maximum of a non-negative double given as its bit pattern.
template <int THREADS>
__device__ __forceinline__ double block_max_bits(uint64_t v, uint64_t* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  uint64_t m = 0;
#pragma unroll
  for (int w = 0; w < THREADS / 32; ++w) m = red[w] > m ? red[w] : m;
  return bits_to_double(m);
}

// ------------------------------------------------------------------ kNN --
template <int D, int KMAX, int THREADS, bool PLAIN, bool COUNT>
__global__ void __launch_bounds__(THREADS)
grid_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items, int nitems,
            int* __restrict__ counter, uint32_t* __restrict__ err, int dmax,
            DeferEntry* __restrict__ defer, int* __restrict__ defer_count) {
  using T = CoordT<PLAIN>;
  constexpr int DQ = D ? D : EGB_DMAX;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* tiles = reinterpret_cast<T*>(smem_raw);  // [2][DM][TS]
  const int DM = D ? D : dmax;
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint64_t red[THREADS / 32];
  __shared__ int s_item;
  __shared__ JobDev sj;
  __shared__ WorkItem s_wi;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t issued = 0, consumed = 0;
  int b0t0 = 0, b0t1 = 0, b1t0 = 0, b1t1 = 0;  // tile held by each buffer

  for (;;) {
    if (tid == 0) {
      const int it = atomicAdd(counter, 1);
      s_item = it;
      if (it < nitems) {
        s_wi = items[it];
        sj = jobs[s_wi.job];
      }
    }
    __syncthreads();
    const int item = s_item;
    if (item >= nitems) break;
    const WorkItem wi = s_wi;
    const int d = D ? D : sj.sp.d;
    const int len = sj.len;
    const int64_t lds = sj.lds;
    const double* __restrict__ c64 = sj.c64g;
    const T* gsrc = PLAIN ? reinterpret_cast<const T*>(sj.c64g) : reinterpret_cast<const T*>(sj.c32g);
    const int32_t* __restrict__ sst = sj.sstart;      // strip starts
    const double* __restrict__ ylo_t = sj.sylo;       // strip column-1 bounds
    const double* __restrict__ yhi_t = sj.syhi;
    const int S = sj.nstrips;
    const bool unsafe = !PLAIN && ((*sj.jflags & TF_UNSAFE32) != 0u);

    // ---- the query of this thread
    const int qp = wi.q0 + tid;
    const bool exists = qp < wi.q1;
    T qv[DQ];
    double m = 0.0;
#pragma unroll
    for (int c = 0; c < DQ; ++c) {
      if (D == 0 && c >= d) break;
      qv[c] = exists ? gsrc[(int64_t)c * lds + qp] : T(0);
      if (!PLAIN && exists) {
        const double v = fabs(c64[(int64_t)c * lds + qp] - sj.center[c]);
        m = v > m ? v : m;
      }
    }
    const float mq = __double2float_ru(m);
    const double qy = exists ? c64[lds + qp] : 0.0;

    // kNN state
    uint64_t top[COUNT ? 1 : KMAX];
    float thr = exists ? __int_as_float(0x7f800000) : -1.0f;
    // count state
    double qr = -1.0;
    uint64_t rbits = 0;
    float lo = -1.0f, hi = -1.0f;
    int cntq = 0;
    bool qok = exists;
    if constexpr (COUNT) {
      qr = exists ? sj.rad[sj.idxg[qp]] : -1.0;
      qok = exists && (qr >= 0.0);
      rbits = qok ? (uint64_t)__double_as_longlong(qr) : 0ull;
      if (!PLAIN && qok) {
        if (isinf(qr)) {
          lo = hi = __int_as_float(0x7f800000);
        } else if (unsafe) {
          hi = __int_as_float(0x7f800000);
        } else {
          const double b = band((double)mq, qr);
          lo = __double2float_rd(qr - b);
          hi = __double2float_ru(qr + b);
        }
      }
    } else {
#pragma unroll
      for (int s = 0; s < KMAX; ++s) top[s] = (exists && s >= KMAX - sj.K) ? INF_BITS : 0ull;
    }
    // current threshold of this query as FP64 (kNN: K-th distance so far)
    auto tq = [&]() -> double {
      if constexpr (COUNT) return qr;
      else return bits_to_double(top[KMAX - 1]);
    };
    auto tq_bits = [&]() -> uint64_t {
      if constexpr (COUNT) return qok ? rbits : 0ull;
      else return exists ? top[KMAX - 1] : 0ull;
    };

    auto recheck = [&](int j) {
      uint64_t mm = 0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        const int64_t off = (int64_t)c * lds;
        const uint64_t v = absdiff_bits(c64[off + j], c64[off + qp]);
        mm = v > mm ? v : mm;
      }
      if constexpr (COUNT) {
        cntq += (mm <= rbits) ? 1 : 0;
      } else {
        if (mm < top[KMAX - 1]) {
          insert_sorted<KMAX>(top, mm);
          thr = unsafe ? __int_as_float(0x7f800000) : thr_from(top[KMAX - 1], mq);
        }
      }
    };

    // ---- schedule
    GridSched sc;
    sc.sq = wi.strip;
    sc.S = S;
    sc.len = len;
    sc.s0 = sst[sc.sq];
    sc.s1 = sst[sc.sq + 1];
    sc.up = sc.sq + 1;
    sc.dn = sc.sq - 1;
    sc.up_open = sc.up < S;
    sc.dn_open = sc.dn >= 0;
    sc.stage = 0;
    sc.turn_up = true;
    sc.ra = wi.q0;
    sc.rb = wi.q1;
    sc.pos = wi.q0;
    sc.strips_done = 0;
    const double xa = c64[wi.q0];
    const double xb = c64[wi.q1 - 1];
    bool stop = false;
    int hl = 0, hr = 0;  // home window

    // Is this query finished given the strips not yet visited?
    auto finished = [&]() -> bool {
      if (!qok) return true;
      if (sc.stage < 3) return false;
      const double t = tq();
      const bool u = !sc.up_open || sc.up >= S || (ylo_t[sc.up] - qy > t);
      const bool l = !sc.dn_open || sc.dn < 0 || (qy - yhi_t[sc.dn] > t);
      return u && l;
    };

    // Next tile [t0, t1), t0 = -1 when the item is done, or t0 = -2 when the
    // next range needs the thresholds but a tile is still in flight (plan
    // only on fully processed tiles: a window planned before the item's own
    // tile is consumed would use infinite k-th distances).  All threads call
    // it.
    auto next_tile = [&](int& t0, int& t1, bool can_plan) {
      for (;;) {
        if (sc.pos < sc.rb) {
          t0 = sc.pos;
          t1 = min(sc.pos + GRID_TILE, sc.rb);
          sc.pos = t1;
          return;
        }
        if (stop) {
          t0 = -1;
          return;
        }
        if (!can_plan) {
          t0 = -2;
          return;
        }
        // window half-width: the largest threshold among queries that still
        // need candidates (a finished query needs no further strip)
        const double T = block_max_bits<THREADS>(finished() ? 0ull : tq_bits(), red);
        if (sc.stage == 0) {
          GridItem<THREADS, PLAIN>::window(c64, sc.s0, sc.s1, xa - T, xb + T, hl, hr);
          sc.stage = 1;
          sc.ra = hl;
          sc.rb = min(hr, wi.q0);
          sc.pos = sc.ra;
          continue;
        }
        if (sc.stage == 1) {
          sc.stage = 2;
          sc.ra = max(hl, wi.q1);
          sc.rb = hr;
          sc.pos = sc.ra;
          continue;
        }
        // beyond the home strip: close sides, maybe stop, pick the next strip
        if (sc.stage == 2) sc.stage = 3;
        bool openu = false, opend = false;
        if (qok) {
          const double t = tq();
          if (sc.up_open && sc.up < S) openu = !(ylo_t[sc.up] - qy > t);
          if (sc.dn_open && sc.dn >= 0)
            opend = !(qy - yhi_t[sc.dn] > t);
        }
        sc.up_open = sc.up_open && sc.up < S && __syncthreads_or(openu);
        sc.dn_open = sc.dn_open && sc.dn >= 0 && __syncthreads_or(opend);
        if (!sc.up_open && !sc.dn_open) {
          t0 = -1;
          return;
        }
        if (defer != nullptr) {
          const int nunf = __syncthreads_count(!finished());
          if (nunf > 0 && (nunf * GRID_DEFER_FRAC <= THREADS || sc.strips_done >= SIDE_CAP)) {
            stop = true;
            t0 = -1;
            return;
          }
        }
        int s;
        if ((sc.turn_up && sc.up_open) || !sc.dn_open) {
          s = sc.up++;
          sc.turn_up = false;
        } else {
          s = sc.dn--;
          sc.turn_up = true;
        }
        ++sc.strips_done;
        int wl, wh;
        GridItem<THREADS, PLAIN>::window(c64, sst[s], sst[s + 1],
                                         xa - T, xb + T, wl, wh);
        sc.ra = wl;
        sc.rb = wh;
        sc.pos = wl;
      }
    };

    unsigned long long pairs = 0;
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
      int t0, t1;
      next_tile(t0, t1, issued == consumed);
      if (t0 < 0) break;
      const int buf = issued & 1;
      if (tid == 0) stage_range<T>(tiles, DM, buf, gsrc, lds, d, t0, t1, &bar[buf]);
      if (buf) { b1t0 = t0; b1t1 = t1; } else { b0t0 = t0; b0t1 = t1; }
      ++issued;
    }

    bool failed = false;
    while (consumed < issued) {
      const int buf = consumed & 1;
      const uint32_t par = (consumed >> 1) & 1;
      const int t0 = buf ? b1t0 : b0t0;
      const int t1 = buf ? b1t1 : b0t1;
      const bool ok = mbar_wait(&bar[buf], par);
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      const int a = t0 & ~3;
      const T* tl = tiles + (size_t)buf * DM * TS;
      pairs += (unsigned long long)(t1 - t0);
      for (int g0 = a; g0 < t1; g0 += 4) {
        uint32_t vmask = 0xFu;
        if (g0 < t0) vmask &= ~((1u << (t0 - g0)) - 1u);
        if (g0 + 4 > t1) vmask &= (1u << (t1 - g0)) - 1u;
        uint32_t hits = 0, inside = 0;
        const int o = g0 - a;
        if constexpr (D == 0 || PLAIN) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if constexpr (PLAIN) {
              uint64_t mm = 0;
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (D == 0 && c >= d) break;
                const uint64_t v = absdiff_bits(tl[c * TS + o + u], qv[c]);
                mm = v > mm ? v : mm;
              }
              if constexpr (COUNT) inside |= (qok && mm <= rbits ? 1u : 0u) << u;
              else hits |= (mm < top[KMAX - 1] ? 1u : 0u) << u;
            } else {
              float dist = 0.0f;
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (c >= d) break;
                dist = fmaxf(dist, fabsf(tl[c * TS + o + u] - qv[c]));
              }
              if constexpr (COUNT) {
                inside |= (dist <= lo ? 1u : 0u) << u;
                hits |= ((dist > lo) && (dist <= hi) ? 1u : 0u) << u;
              } else {
                hits |= (dist <= thr ? 1u : 0u) << u;
              }
            }
          }
        } else {
          float4 cv[D];
#pragma unroll
          for (int c = 0; c < D; ++c) cv[c] = *reinterpret_cast<const float4*>(tl + c * TS + o);
#define EGB_GRID_LANE(U)                                                        \
  {                                                                             \
    float dist = fabsf(pick4<U>(cv[0]) - qv[0]);                                \
    _Pragma("unroll") for (int c = 1; c < D; ++c)                               \
        dist = fmaxf(dist, fabsf(pick4<U>(cv[c]) - qv[c]));                     \
    if constexpr (COUNT) {                                                      \
      inside |= (dist <= lo ? 1u : 0u) << U;                                    \
      hits |= ((dist > lo) && (dist <= hi) ? 1u : 0u) << U;                     \
    } else {                                                                    \
      hits |= (dist <= thr ? 1u : 0u) << U;                                     \
    }                                                                           \
  }
          EGB_GRID_LANE(0)
          EGB_GRID_LANE(1)
          EGB_GRID_LANE(2)
          EGB_GRID_LANE(3)
#undef EGB_GRID_LANE
        }
        if constexpr (COUNT) cntq += __popc(inside & vmask);
        hits &= vmask;
        if (__builtin_expect(hits != 0u, 0)) {
          while (hits) {
            const int u = __ffs(hits) - 1;
            hits &= hits - 1u;
            recheck(g0 + u);
          }
        }
      }
      __syncthreads();  // every thread is done with this buffer
      ++consumed;
      int tn0, tn1;
      next_tile(tn0, tn1, issued == consumed);
      if (tn0 >= 0) {
        const int nb = issued & 1;
        if (tid == 0) stage_range<T>(tiles, DM, nb, gsrc, lds, d, tn0, tn1, &bar[nb]);
        if (nb) { b1t0 = tn0; b1t1 = tn1; } else { b0t0 = tn0; b0t1 = tn1; }
        ++issued;
      }
    }
    if (failed) {
      if (tid == 0) {
        atomicOr(err, (uint32_t)DERR_WAIT_TIMEOUT);
        while (consumed < issued) {
          mbar_wait(&bar[consumed & 1], (consumed >> 1) & 1);
          ++consumed;
        }
      }
      __syncthreads();
      return;
    }
    if (exists) {
      const bool fin = !stop || finished();
      if (fin) {
        if constexpr (COUNT) sj.cnt[sj.idxg[qp]] = qok ? cntq : 0;
        else sj.eps[sj.idxg[qp]] = tq();
      } else {
        const int slot = atomicAdd(defer_count, 1);
        atomicAdd(sj.stats + 2, 1ull);
        defer[slot] = DeferEntry{wi.job, sj.posg[qp], tq()};
      }
    }
    if (tid == 0) atomicAdd(sj.stats + 0, pairs * (unsigned long long)(wi.q1 - wi.q0));
    __syncthreads();  // sj, s_wi and s_item are rewritten by the next fetch
  }
}

constexpr int GRID_THREADS = GRID_QB;

template <int D, bool PLAIN>
TileShape grid_shape_t(int dmax) {
  const int DM = D ? D : dmax;
  TileShape s;
  s.threads = GRID_THREADS;
  s.qpt = 1;
  s.tile = GRID_TILE;
  s.smem = 2ull * DM * TS * sizeof(CoordT<PLAIN>);
  return s;
}

template <int D, int KMAX, bool PLAIN, bool COUNT>
void launch_grid_t(const JobDev* jobs, const WorkItem* items, int nitems, int* counter,
                   uint32_t* err, int dmax, DeferEntry* defer, int* defer_count, int num_sms,
                   cudaStream_t st) {
  const TileShape s = grid_shape_t<D, PLAIN>(dmax);
  auto kern = grid_kernel<D, KMAX, GRID_THREADS, PLAIN, COUNT>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GRID_THREADS, s.smem);
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  if (grid > nitems) grid = nitems;
  if (grid < 1) return;
  kern<<<grid, GRID_THREADS, s.smem, st>>>(jobs, items, nitems, counter, err, dmax, defer,
                                            defer_count);
  count_launch();
}

template <bool PLAIN>
struct GridDispatch {
  static TileShape shape(int dclass, int dmax) {
    switch (dclass) {
      case 2: return grid_shape_t<2, PLAIN>(dmax);
      case 3: return grid_shape_t<3, PLAIN>(dmax);
      case 4: return grid_shape_t<4, PLAIN>(dmax);
      default: return grid_shape_t<0, PLAIN>(dmax);
    }
  }
  template <int D>
  static void knn_d(int kclass, const JobDev* jobs, const WorkItem* items, int nitems, int* ctr,
                    uint32_t* err, int dmax, DeferEntry* df, int* dc, int sms, cudaStream_t st) {
    switch (kclass) {
      case 4: launch_grid_t<D, 4, PLAIN, false>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      case 8: launch_grid_t<D, 8, PLAIN, false>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      case 16: launch_grid_t<D, 16, PLAIN, false>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      default: launch_grid_t<D, 32, PLAIN, false>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
    }
  }
  static void knn(int kclass, int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                  int* ctr, uint32_t* err, int dmax, DeferEntry* df, int* dc, int sms,
                  cudaStream_t st) {
    switch (dclass) {
      case 2: knn_d<2>(kclass, jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      case 3: knn_d<3>(kclass, jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      case 4: knn_d<4>(kclass, jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      default: knn_d<0>(kclass, jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
    }
  }
  static void count(int dclass, const JobDev* jobs, const WorkItem* items, int nitems, int* ctr,
                    uint32_t* err, int dmax, DeferEntry* df, int* dc, int sms, cudaStream_t st) {
    switch (dclass) {
      case 2: launch_grid_t<2, 4, PLAIN, true>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      case 3: launch_grid_t<3, 4, PLAIN, true>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      case 4: launch_grid_t<4, 4, PLAIN, true>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
      default: launch_grid_t<0, 4, PLAIN, true>(jobs, items, nitems, ctr, err, dmax, df, dc, sms, st); break;
    }
  }
};

}  // namespace grid_detail
}  // namespace egb
