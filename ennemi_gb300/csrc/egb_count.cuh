// egb_count.cuh -- multi-D ball-count tile kernel, max norm, exact in FP64.
//
// Replaces tree.query_ball_point(pts, r, p=inf, return_length=True) for the
// multi-dimensional marginal spaces of ennemi/_entropy_estimators.py:152-154
// (xz, yz, z of the conditional estimators), :196 (Ross MI with d_x > 1) and
// :243-245, with r = fl64(eps - 1e-12):
//     count_q = #{p : max_c fl64(|p_c - q_c|) <= r_q},  the query included.
//
// FP32 form: per query two FP32 thresholds
//     lo = fl32_down(r - band(M, r)),   hi = fl32_up(r + band(M, r));
// d32 <= lo proves the FP64 distance <= r (counted directly), d32 > hi
// proves it > r; only lo < d32 <= hi goes to FP64 (band() in
// egb_internal.cuh).  The result equals the all-FP64 count exactly.
// Plain form (PLAIN): every distance in FP64.
#pragma once
#include "egb_tile.cuh"

namespace egb {
namespace count_detail {

template <int U>
__device__ __forceinline__ float pick4(const float4& v) {
  return U == 0 ? v.x : U == 1 ? v.y : U == 2 ? v.z : v.w;
}
template <int U>
__device__ __forceinline__ double pick2(const double2& v) {
  return U == 0 ? v.x : v.y;
}

template <int D, int QPT, int THREADS, int TILE, bool PLAIN, bool SLAB>
__global__ void __launch_bounds__(THREADS)
count_tile_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items, int nitems,
                  int* __restrict__ counter, uint32_t* __restrict__ err, int dmax,
                  DeferEntry* __restrict__ defer, int* __restrict__ defer_count) {
  using T = CoordT<PLAIN>;
  constexpr int DQ = D ? D : EGB_DMAX;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* tiles = reinterpret_cast<T*>(smem_raw);  // [2][DM][TILE]
  const int DM = D ? D : dmax;
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_item;
  __shared__ JobDev sj;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t issued = 0, consumed = 0;
  int tile0 = 0, tile1 = 0;

  for (;;) {
    if (tid == 0) {
      const int it = atomicAdd(counter, 1);
      s_item = it;
      if (it < nitems) sj = jobs[items[it].job];
    }
    __syncthreads();
    const int item = s_item;
    if (item >= nitems) break;
    const int q0 = items[item].q0;
    const int job = items[item].job;
    const int d = D ? D : sj.sp.d;
    const int len = sj.len;
    const int64_t lds = sj.lds;
    const double* __restrict__ c64 = sj.c64;
    const T* gsrc = PLAIN ? reinterpret_cast<const T*>(sj.c64) : reinterpret_cast<const T*>(sj.c32);
    const bool unsafe = !PLAIN && ((*sj.jflags & TF_UNSAFE32) != 0u);

    int qp[QPT];
    bool qok[QPT];      // query exists and its radius is >= 0
    T qv[QPT][DQ];
    double qr[QPT];     // FP64 radius
    uint64_t rbits[QPT];
    float lo[QPT], hi[QPT];
    double qx[QPT];
    int cntq[QPT];
#pragma unroll
    for (int q = 0; q < QPT; ++q) {
      qp[q] = q0 + tid + q * THREADS;
      const bool exists = qp[q] < len;
      const double r = exists ? sj.rad[sj.idx[qp[q]]] : -1.0;
      qok[q] = exists && (r >= 0.0);
      qr[q] = r;
      rbits[q] = qok[q] ? (uint64_t)__double_as_longlong(r) : 0ull;
      double m = 0.0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        qv[q][c] = exists ? gsrc[(int64_t)c * lds + qp[q]] : T(0);
        if (!PLAIN && exists) {
          const double v = fabs(c64[(int64_t)c * lds + qp[q]] - sj.center[c]);
          m = v > m ? v : m;
        }
      }
      qx[q] = exists ? c64[qp[q]] : 0.0;
      cntq[q] = 0;
      if (!PLAIN) {
        if (!qok[q]) {
          lo[q] = -1.0f;
          hi[q] = -1.0f;
        } else if (isinf(r)) {  // every candidate is inside (band(M, inf) is inf)
          lo[q] = __int_as_float(0x7f800000);
          hi[q] = lo[q];
        } else if (unsafe) {
          lo[q] = -1.0f;
          hi[q] = __int_as_float(0x7f800000);
        } else {
          const double b = band((double)__double2float_ru(m), r);
          lo[q] = __double2float_rd(r - b);
          hi[q] = __double2float_ru(r + b);
        }
      }
    }

    auto recheck = [&](int q, int j) {
      uint64_t mm = 0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        const int64_t off = (int64_t)c * lds;
        const uint64_t v = absdiff_bits(c64[off + j], c64[off + qp[q]]);
        mm = v > mm ? v : mm;
      }
      cntq[q] += (mm <= rbits[q]) ? 1 : 0;
    };

    TileSched<TILE, SLAB> sc;
    sc.init(len, q0, min(q0 + THREADS * QPT, len));
    const int nhome = sc.h1 - sc.home + 1;
    const int nq_item = min(THREADS * QPT, len - q0);
    unsigned long long pairs = 0;  // thread 0: candidates x queries screened
    int citem = 0;
    bool stop = false;
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
      const int t = sc.next();
      if (t < 0) break;
      const int buf = issued & 1;
      if (tid == 0) stage_tile<T, TILE>(tiles, DM, buf, gsrc, lds, d, len, t, &bar[buf]);
      if (buf) tile1 = t; else tile0 = t;
      ++issued;
    }

    bool failed = false;
    while (consumed < issued) {
      const int buf = consumed & 1;
      const uint32_t par = (consumed >> 1) & 1;
      const int t = buf ? tile1 : tile0;
      const bool ok = mbar_wait(&bar[buf], par);
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      const int A = t * TILE;
      const int cnt = min(TILE, len - A);
      const T* tl = tiles + (size_t)buf * DM * TILE;
      pairs += (unsigned long long)cnt * (unsigned long long)nq_item;
      // Groups of 4 candidates: the FP32 screen counts the sure-inside ones
      // and only marks borderline ones in a bit mask (bit 4q + u); those are
      // decided in FP64 afterwards in a data-dependent loop, which keeps the
      // FP64 work off the hot path (see the kNN kernel).
      for (int g0 = 0; g0 < cnt; g0 += 4) {
        const bool full = g0 + 4 <= cnt;
        uint32_t border = 0;
        if constexpr (D == 0) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool in = g0 + u < cnt;
            const int j = in ? g0 + u : cnt - 1;
#pragma unroll
            for (int q = 0; q < QPT; ++q) {
              if constexpr (!PLAIN) {
                float dist = 0.0f;
#pragma unroll
                for (int c = 0; c < DQ; ++c) {
                  if (c >= d) break;
                  dist = fmaxf(dist, fabsf(tl[c * TILE + j] - qv[q][c]));
                }
                cntq[q] += (in && dist <= lo[q]) ? 1 : 0;
                border |= ((in && dist > lo[q] && dist <= hi[q]) ? 1u : 0u) << (4 * q + u);
              } else {
                uint64_t mm = 0;
#pragma unroll
                for (int c = 0; c < DQ; ++c) {
                  if (c >= d) break;
                  const uint64_t v = absdiff_bits(tl[c * TILE + j], qv[q][c]);
                  mm = v > mm ? v : mm;
                }
                cntq[q] += (in && qok[q] && mm <= rbits[q]) ? 1 : 0;
              }
            }
          }
        } else if constexpr (!PLAIN) {
          float4 cv[D];
#pragma unroll
          for (int c = 0; c < D; ++c) cv[c] = *reinterpret_cast<const float4*>(tl + c * TILE + g0);
          if (full) {
#define EGB_CNT_LANE(U)                                                         \
  _Pragma("unroll") for (int q = 0; q < QPT; ++q) {                             \
    float dist = fabsf(pick4<U>(cv[0]) - qv[q][0]);                             \
    _Pragma("unroll") for (int c = 1; c < D; ++c)                               \
        dist = fmaxf(dist, fabsf(pick4<U>(cv[c]) - qv[q][c]));                  \
    cntq[q] += (dist <= lo[q]) ? 1 : 0;                                         \
    border |= ((dist > lo[q]) && (dist <= hi[q]) ? 1u : 0u) << (4 * q + U);     \
  }
            EGB_CNT_LANE(0)
            EGB_CNT_LANE(1)
            EGB_CNT_LANE(2)
            EGB_CNT_LANE(3)
#undef EGB_CNT_LANE
          } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const bool in = g0 + u < cnt;
#pragma unroll
              for (int q = 0; q < QPT; ++q) {
                float dist = 0.0f;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                  const float cu = u == 0 ? cv[c].x : u == 1 ? cv[c].y : u == 2 ? cv[c].z : cv[c].w;
                  dist = fmaxf(dist, fabsf(cu - qv[q][c]));
                }
                cntq[q] += (in && dist <= lo[q]) ? 1 : 0;
                border |= ((in && dist > lo[q] && dist <= hi[q]) ? 1u : 0u) << (4 * q + u);
              }
            }
          }
        } else {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            double2 cv[D];
#pragma unroll
            for (int c = 0; c < D; ++c)
              cv[c] = *reinterpret_cast<const double2*>(tl + c * TILE + g0 + 2 * h);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const bool in = g0 + 2 * h + u < cnt;
#pragma unroll
              for (int q = 0; q < QPT; ++q) {
                uint64_t mm = 0;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                  const uint64_t v = absdiff_bits(u ? cv[c].y : cv[c].x, qv[q][c]);
                  mm = v > mm ? v : mm;
                }
                cntq[q] += (in && qok[q] && mm <= rbits[q]) ? 1 : 0;
              }
            }
          }
        }
        if (__builtin_expect(border != 0u, 0)) {
#pragma unroll
          for (int q = 0; q < QPT; ++q) {
            uint32_t bq = (border >> (4 * q)) & 0xFu;
            while (bq) {
              const int u = __ffs(bq) - 1;
              bq &= bq - 1u;
              recheck(q, A + g0 + u);
            }
          }
        }
      }
      __syncthreads();
      ++consumed;
      ++citem;
      if constexpr (SLAB) {
        const double XR = sc.doneR ? 0.0 : c64[(int64_t)sc.nextR * TILE];
        const double XL = sc.doneL ? 0.0 : c64[(int64_t)(sc.nextL + 1) * TILE - 1];
        bool allR = true, allL = true, unf = false;
#pragma unroll
        for (int q = 0; q < QPT; ++q) {
          if (!qok[q]) continue;
          const bool r = sc.doneR || (XR - qx[q] > qr[q]);
          const bool l = sc.doneL || (qx[q] - XL > qr[q]);
          allR &= r;
          allL &= l;
          unf |= !(r && l);
        }
        if (!sc.doneR && __syncthreads_and(allR)) sc.doneR = true;
        if (!sc.doneL && __syncthreads_and(allL)) sc.doneL = true;
        if (defer != nullptr && citem >= nhome && !stop) {
          const int nunf = __syncthreads_count(unf);
          if (nunf > 0 && (nunf * DEFER_FRAC <= THREADS || citem - nhome >= SIDE_CAP)) stop = true;
        }
      }
      const int tn = stop ? -1 : sc.next();
      if (tn >= 0) {
        const int nb = issued & 1;
        if (tid == 0) stage_tile<T, TILE>(tiles, DM, nb, gsrc, lds, d, len, tn, &bar[nb]);
        if (nb) tile1 = tn; else tile0 = tn;
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
    {
      const double XR = (!SLAB || sc.doneR) ? 0.0 : c64[(int64_t)sc.nextR * TILE];
      const double XL = (!SLAB || sc.doneL) ? 0.0 : c64[(int64_t)(sc.nextL + 1) * TILE - 1];
#pragma unroll
      for (int q = 0; q < QPT; ++q) {
        if (qp[q] >= len) continue;
        const bool fin = !qok[q] || !SLAB || !stop ||
                         ((sc.doneR || (XR - qx[q] > qr[q])) && (sc.doneL || (qx[q] - XL > qr[q])));
        if (fin) {
          sj.cnt[sj.idx[qp[q]]] = qok[q] ? cntq[q] : 0;
        } else {
          const int slot = atomicAdd(defer_count, 1);
          atomicAdd(sj.stats + 2, 1ull);
          defer[slot] = DeferEntry{job, qp[q], qr[q]};
        }
      }
    }
    if (tid == 0) atomicAdd(sj.stats + 0, pairs);
    __syncthreads();
  }
}

// Deferred slab queries, one warp each: lanes count interleaved positions
// outward from the query until the next unvisited first coordinate on each
// side is beyond the radius; the lane counts are summed.
template <int D, bool PLAIN>
__global__ void __launch_bounds__(256)
count_defer_kernel(const JobDev* __restrict__ jobs, const DeferEntry* __restrict__ list,
                   const int* __restrict__ count_ptr, int cap) {
  using T = CoordT<PLAIN>;
  constexpr int DQ = D ? D : EGB_DMAX;
  const int lane = threadIdx.x & 31;
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  const int count = min(*count_ptr, cap);
  for (int e = gw; e < count; e += nw) {
    const DeferEntry en = list[e];
    const JobDev* J = jobs + en.job;
    const int d = D ? D : J->sp.d;
    const int len = J->len;
    const int64_t lds = J->lds;
    const double* __restrict__ q64 = J->c64;
    const T* qg = PLAIN ? reinterpret_cast<const T*>(J->c64) : reinterpret_cast<const T*>(J->c32);
    const int pos = en.pos;
    const double r = en.tb;  // the radius; deferred queries have r >= 0
    const uint64_t rbits = (uint64_t)__double_as_longlong(r);
    const bool unsafe = !PLAIN && ((*J->jflags & TF_UNSAFE32) != 0u);
    const ScanOrder<T> o = choose_order<T, PLAIN>(J, pos, r);
    const double* __restrict__ c64 = o.c64;
    const T* g = o.g;
    const double* scol = c64 + (int64_t)o.col * lds;
    T qv[DQ];
    double m = 0.0;
#pragma unroll
    for (int c = 0; c < DQ; ++c) {
      if (D == 0 && c >= d) break;
      qv[c] = qg[(int64_t)c * lds + pos];
      if (!PLAIN) {
        const double v = fabs(q64[(int64_t)c * lds + pos] - J->center[c]);
        m = v > m ? v : m;
      }
    }
    float lo = -1.0f, hi = -1.0f;
    if (!PLAIN) {
      if (isinf(r)) {
        lo = hi = __int_as_float(0x7f800000);
      } else if (unsafe) {
        hi = __int_as_float(0x7f800000);
      } else {
        const double b = band((double)__double2float_ru(m), r);
        lo = __double2float_rd(r - b);
        hi = __double2float_ru(r + b);
      }
    }
    int cnt = 0;
    // screen: 0 = outside, 1 = inside, 2 = borderline (FP64 decides)
    auto screen = [&](int j) -> int {
      if constexpr (PLAIN) {
        uint64_t mm = 0;
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          const uint64_t v = absdiff_bits(g[(int64_t)c * lds + j], qv[c]);
          mm = v > mm ? v : mm;
        }
        return mm <= rbits ? 1 : 0;
      } else {
        float dist = 0.0f;
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          dist = fmaxf(dist, fabsf(g[(int64_t)c * lds + j] - qv[c]));
        }
        return dist <= lo ? 1 : (dist <= hi ? 2 : 0);
      }
    };
    auto resolve = [&](int j) {
      uint64_t mm = 0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        const int64_t off = (int64_t)c * lds;
        const uint64_t v = absdiff_bits(c64[off + j], q64[off + pos]);
        mm = v > mm ? v : mm;
      }
      cnt += mm <= rbits ? 1 : 0;
    };
    int nr = o.start, nl = o.start - 1;
    bool doneR = nr >= len, doneL = nl < 0;
    while (!doneR || !doneL) {
      uint32_t border = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int jr = nr + lane + 32 * u;
        const int jl = nl - lane - 32 * u;
        if (!doneR && jr < len) {
          const int sres = screen(jr);
          cnt += sres == 1 ? 1 : 0;
          border |= (sres == 2 ? 1u : 0u) << u;
        }
        if (!doneL && jl >= 0) {
          const int sres = screen(jl);
          cnt += sres == 1 ? 1 : 0;
          border |= (sres == 2 ? 16u : 0u) << u;
        }
      }
      while (border) {
        const int b = __ffs(border) - 1;
        border &= border - 1u;
        resolve(b < 4 ? nr + lane + 32 * b : nl - lane - 32 * (b - 4));
      }
      if (!doneR) {
        nr += 128;
        doneR = nr >= len || (scol[nr] - o.qs > r);
      }
      if (!doneL) {
        nl -= 128;
        doneL = nl < 0 || (o.qs - scol[nl] > r);
      }
    }
    const int total = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0) {
      J->cnt[J->idx[pos]] = total;
      atomicAdd(J->stats + 1, (unsigned long long)(nr - nl - 1));
    }
  }
}

template <int D, bool PLAIN, bool SLAB>
struct CountCfg {
  static constexpr int THREADS = (D == 0 || SLAB) ? 128 : 256;
  static constexpr int QPT = D == 0 ? 1 : 2;
  static constexpr int TILE = D == 0 ? 256 : SLAB ? 512 : (D == 2 ? 2048 : 1024);
};

template <int D, bool PLAIN, bool SLAB>
TileShape count_shape_t(int dmax) {
  using C = CountCfg<D, PLAIN, SLAB>;
  const int DM = D ? D : dmax;
  TileShape s;
  s.threads = C::THREADS;
  s.qpt = C::QPT;
  s.tile = C::TILE;
  s.smem = 2ull * DM * C::TILE * sizeof(CoordT<PLAIN>);
  return s;
}

template <int D, bool PLAIN, bool SLAB>
void launch_count_t(const JobDev* jobs, const WorkItem* items, int nitems, int* counter,
                    uint32_t* err, int dmax, DeferEntry* defer, int* defer_count, int num_sms,
                    cudaStream_t st) {
  using C = CountCfg<D, PLAIN, SLAB>;
  const TileShape s = count_shape_t<D, PLAIN, SLAB>(dmax);
  auto kern = count_tile_kernel<D, C::QPT, C::THREADS, C::TILE, PLAIN, SLAB>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::THREADS, s.smem);
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  if (grid > nitems) grid = nitems;
  if (grid < 1) return;
  kern<<<grid, C::THREADS, s.smem, st>>>(jobs, items, nitems, counter, err, dmax,
                                         SLAB ? defer : nullptr, defer_count);
  count_launch();
}

template <int D, bool PLAIN>
void launch_count_defer_t(const JobDev* jobs, const DeferEntry* list, const int* count, int cap,
                          int num_sms, cudaStream_t st) {
  const int warps_per_block = 8;
  int grid = (cap + warps_per_block - 1) / warps_per_block;
  if (grid > num_sms * 8) grid = num_sms * 8;
  if (grid < 1) return;
  count_defer_kernel<D, PLAIN><<<grid, 32 * warps_per_block, 0, st>>>(jobs, list, count, cap);
  count_launch();
}

template <bool PLAIN, bool SLAB>
struct CountDispatch {
  static TileShape shape(int dclass, int dmax) {
    switch (dclass) {
      case 2: return count_shape_t<2, PLAIN, SLAB>(dmax);
      case 3: return count_shape_t<3, PLAIN, SLAB>(dmax);
      case 4: return count_shape_t<4, PLAIN, SLAB>(dmax);
      default: return count_shape_t<0, PLAIN, SLAB>(dmax);
    }
  }
  static void launch(int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                     int* counter, uint32_t* err, int dmax, DeferEntry* df, int* dc, int num_sms,
                     cudaStream_t st) {
    switch (dclass) {
      case 2: launch_count_t<2, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      case 3: launch_count_t<3, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      case 4: launch_count_t<4, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      default: launch_count_t<0, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
    }
  }
  static void defer(int dclass, const JobDev* jobs, const DeferEntry* list, const int* count,
                    int cap, int num_sms, cudaStream_t st) {
    switch (dclass) {
      case 2: launch_count_defer_t<2, PLAIN>(jobs, list, count, cap, num_sms, st); break;
      case 3: launch_count_defer_t<3, PLAIN>(jobs, list, count, cap, num_sms, st); break;
      case 4: launch_count_defer_t<4, PLAIN>(jobs, list, count, cap, num_sms, st); break;
      default: launch_count_defer_t<0, PLAIN>(jobs, list, count, cap, num_sms, st); break;
    }
  }
};

}  // namespace count_detail
}  // namespace egb
