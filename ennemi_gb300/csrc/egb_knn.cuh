// egb_knn.cuh -- (k+1)-NN distance tile kernel, max norm, exact in FP64.
//
// Replaces cKDTree(pts).query(pts, k=[k+1], p=inf)[0] as used by
// ennemi/_entropy_estimators.py:39, :108, :142, :194, :240: eps of every
// point is the (k+1)-th smallest max-norm distance within its search set,
// the point itself included.
//
// Persistent CTAs pull work items (THREADS*QPT consecutive query positions of
// one job) from a device counter; candidate tiles are staged by egb_tile.cuh.
// Every thread keeps the KMAX smallest FP64 distances of each of its queries
// in registers as bit patterns of non-negative doubles (integer compares,
// sorted insertion), padded so that the last slot is the K-th smallest.
//
// FP32 form: distances are first computed in FP32 from centred coordinates; a
// candidate is evaluated in FP64 only when its FP32 distance passes
//     d32 <= fl32_up(t + band(M, t)),   t = current K-th FP64 distance,
// which every candidate with FP64 distance < t does (band() in
// egb_internal.cuh).  So the list always holds the KMAX smallest FP64
// distances: the same bits as the all-FP64 form and as cKDTree.
// Plain form (PLAIN): every distance in FP64 -- the comparator.
#pragma once
#include "egb_tile.cuh"

namespace egb {
namespace knn_detail {

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

// FP32 screen threshold for K-th distance t (bits) and query magnitude mq:
// an upward-rounded evaluation of t + band(mq, t) = t + 2^-21 (mq + t) + 2^-100
// in FP32 (every operation rounds toward +inf, so the result bounds the exact
// value from above).
__device__ __forceinline__ float thr_from(uint64_t kth_bits, float mq) {
  if (kth_bits >= INF_BITS) return __int_as_float(0x7f800000);
  const float tu = f32_up_of_bits(kth_bits);
  return __fmaf_ru(tu, 1.0f + 0x1p-21f, __fmaf_ru(mq, 0x1p-21f, 0x1p-100f));
}

template <int U>
__device__ __forceinline__ float pick4(const float4& v) {
  return U == 0 ? v.x : U == 1 ? v.y : U == 2 ? v.z : v.w;
}
template <int U>
__device__ __forceinline__ double pick2(const double2& v) {
  return U == 0 ? v.x : v.y;
}

template <int D, int KMAX, int QPT, int THREADS, int TILE, bool PLAIN, bool SLAB>
__global__ void __launch_bounds__(THREADS)
knn_tile_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items, int nitems,
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
  int tile0 = 0, tile1 = 0;  // tile held by buffer 0 / 1

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
    const int K = sj.K;
    const bool unsafe = !PLAIN && ((*sj.jflags & TF_UNSAFE32) != 0u);

    int qp[QPT];
    bool qok[QPT];
    T qv[QPT][DQ];
    uint64_t top[QPT][KMAX];
    float thr[QPT];
    float mq[QPT];
    double qx[QPT];
#pragma unroll
    for (int q = 0; q < QPT; ++q) {
      qp[q] = q0 + tid + q * THREADS;
      qok[q] = qp[q] < len;
      double m = 0.0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        qv[q][c] = qok[q] ? gsrc[(int64_t)c * lds + qp[q]] : T(0);
        if (!PLAIN && qok[q]) {
          const double v = fabs(c64[(int64_t)c * lds + qp[q]] - sj.center[c]);
          m = v > m ? v : m;
        }
      }
      qx[q] = qok[q] ? c64[qp[q]] : 0.0;
      mq[q] = __double2float_ru(m);
#pragma unroll
      for (int s = 0; s < KMAX; ++s) top[q][s] = (qok[q] && s >= KMAX - K) ? INF_BITS : 0ull;
      thr[q] = qok[q] ? __int_as_float(0x7f800000) : -1.0f;
    }

    // FP64 decision for a candidate that passed the FP32 filter.
    auto recheck = [&](int q, int j) {
      uint64_t m = 0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        const int64_t off = (int64_t)c * lds;
        const uint64_t v = absdiff_bits(c64[off + j], c64[off + qp[q]]);
        m = v > m ? v : m;
      }
      if (m < top[q][KMAX - 1]) {
        insert_sorted<KMAX>(top[q], m);
        thr[q] = unsafe ? __int_as_float(0x7f800000) : thr_from(top[q][KMAX - 1], mq[q]);
      }
    };

    TileSched<TILE, SLAB> sc;
    sc.init(len, q0, min(q0 + THREADS * QPT, len));
    const int nhome = sc.h1 - sc.home + 1;
    const int nq_item = min(THREADS * QPT, len - q0);
    unsigned long long pairs = 0;  // thread 0: candidates x queries screened
    int citem = 0;      // tiles consumed by this item
    bool stop = false;  // slab: no further tiles; unfinished queries deferred
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
      // Candidates go in groups of 4.  The FP32 (or FP64) screen of a group
      // only sets bits of a hit mask (bit 4q + u: query q, candidate u); the
      // rare hits are resolved afterwards in a data-dependent loop, so the
      // FP64 recheck and the list insertion stay off the hot path instead
      // of being if-converted into it (the FP64 pipe has 2 lanes per SM).
      for (int g0 = 0; g0 < cnt; g0 += 4) {
        uint32_t hits = 0;
        if constexpr (D == 0) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int j = g0 + u < cnt ? g0 + u : cnt - 1;
#pragma unroll
            for (int q = 0; q < QPT; ++q) {
              if constexpr (!PLAIN) {
                float dist = 0.0f;
#pragma unroll
                for (int c = 0; c < DQ; ++c) {
                  if (c >= d) break;
                  dist = fmaxf(dist, fabsf(tl[c * TILE + j] - qv[q][c]));
                }
                hits |= (dist <= thr[q] ? 1u : 0u) << (4 * q + u);
              } else {
                uint64_t m = 0;
#pragma unroll
                for (int c = 0; c < DQ; ++c) {
                  if (c >= d) break;
                  const uint64_t v = absdiff_bits(tl[c * TILE + j], qv[q][c]);
                  m = v > m ? v : m;
                }
                hits |= (m < top[q][KMAX - 1] ? 1u : 0u) << (4 * q + u);
              }
            }
          }
        } else if constexpr (!PLAIN) {
          float4 cv[D];
#pragma unroll
          for (int c = 0; c < D; ++c) cv[c] = *reinterpret_cast<const float4*>(tl + c * TILE + g0);
#define EGB_KNN_LANE(U)                                                         \
  _Pragma("unroll") for (int q = 0; q < QPT; ++q) {                             \
    float dist = fabsf(pick4<U>(cv[0]) - qv[q][0]);                             \
    _Pragma("unroll") for (int c = 1; c < D; ++c)                               \
        dist = fmaxf(dist, fabsf(pick4<U>(cv[c]) - qv[q][c]));                  \
    hits |= (dist <= thr[q] ? 1u : 0u) << (4 * q + U);                          \
  }
          EGB_KNN_LANE(0)
          EGB_KNN_LANE(1)
          EGB_KNN_LANE(2)
          EGB_KNN_LANE(3)
#undef EGB_KNN_LANE
        } else {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            double2 cv[D];
#pragma unroll
            for (int c = 0; c < D; ++c)
              cv[c] = *reinterpret_cast<const double2*>(tl + c * TILE + g0 + 2 * h);
#define EGB_KNN_LANE64(U)                                                       \
  _Pragma("unroll") for (int q = 0; q < QPT; ++q) {                             \
    uint64_t m = absdiff_bits(pick2<U>(cv[0]), qv[q][0]);                       \
    _Pragma("unroll") for (int c = 1; c < D; ++c) {                             \
      const uint64_t v = absdiff_bits(pick2<U>(cv[c]), qv[q][c]);               \
      m = v > m ? v : m;                                                        \
    }                                                                           \
    hits |= (m < top[q][KMAX - 1] ? 1u : 0u) << (4 * q + 2 * h + U);            \
  }
            EGB_KNN_LANE64(0)
            EGB_KNN_LANE64(1)
#undef EGB_KNN_LANE64
          }
        }
        if (g0 + 4 > cnt) hits &= ((1u << (cnt - g0)) - 1u) * 0x1111u;  // partial group
        if (__builtin_expect(hits != 0u, 0)) {
#pragma unroll
          for (int q = 0; q < QPT; ++q) {
            uint32_t hq = (hits >> (4 * q)) & 0xFu;
            while (hq) {
              const int u = __ffs(hq) - 1;
              hq &= hq - 1u;
              recheck(q, A + g0 + u);
            }
          }
        }
      }
      __syncthreads();  // every thread is done with this buffer
      ++consumed;
      ++citem;
      if constexpr (SLAB) {
        // per query: is every unvisited point on that side beyond its k-th
        // distance?  All true closes the side; few false ends the item.
        const double XR = sc.doneR ? 0.0 : c64[(int64_t)sc.nextR * TILE];
        const double XL = sc.doneL ? 0.0 : c64[(int64_t)(sc.nextL + 1) * TILE - 1];
        bool allR = true, allL = true, unf = false;
#pragma unroll
        for (int q = 0; q < QPT; ++q) {
          if (!qok[q]) continue;
          const double t = bits_to_double(top[q][KMAX - 1]);
          const bool r = sc.doneR || (XR - qx[q] > t);
          const bool l = sc.doneL || (qx[q] - XL > t);
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
        while (consumed < issued) {  // let copies in flight land (bounded)
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
        if (!qok[q]) continue;
        const double t = bits_to_double(top[q][KMAX - 1]);
        const bool fin = !SLAB || !stop ||
                         ((sc.doneR || (XR - qx[q] > t)) && (sc.doneL || (qx[q] - XL > t)));
        if (fin) {
          sj.eps[sj.idx[qp[q]]] = t;
        } else {
          const int slot = atomicAdd(defer_count, 1);
          atomicAdd(sj.stats + 2, 1ull);
          defer[slot] = DeferEntry{job, qp[q], t};
        }
      }
    }
    if (tid == 0) atomicAdd(sj.stats + 0, pairs);
    __syncthreads();  // sj and s_item are rewritten by the next fetch
  }
}

// Deferred slab queries, one warp each.  Lanes take interleaved positions
// outward from the query on both sides (32 per step and side) and keep
// their own KMAX smallest FP64 distances.  The minimum over lanes of the
// lanes' K-th distances bounds the query's K-th distance from above, so it
// both filters candidates (FP32 band as in the tile kernel) and closes a side
// once the next unvisited first coordinate lies beyond it.  The K-th
// smallest of the union of the lane lists is the answer (K-way merge).
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

template <int D, int KMAX, bool PLAIN>
__global__ void __launch_bounds__(256)
knn_defer_kernel(const JobDev* __restrict__ jobs, const DeferEntry* __restrict__ list,
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
    const double* __restrict__ q64 = J->c64;  // query coordinates (first order)
    const T* qg = PLAIN ? reinterpret_cast<const T*>(J->c64) : reinterpret_cast<const T*>(J->c32);
    const int pos = en.pos;
    const int K = J->K;
    const bool unsafe = !PLAIN && ((*J->jflags & TF_UNSAFE32) != 0u);
    const ScanOrder<T> o = choose_order<T, PLAIN>(J, pos, en.tb);
    const double* __restrict__ c64 = o.c64;  // candidates, in the scan order
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
    const float mq = __double2float_ru(m);
    uint64_t top[KMAX];
#pragma unroll
    for (int s = 0; s < KMAX; ++s) top[s] = s >= KMAX - K ? INF_BITS : 0ull;
    // tb bounds the final K-th distance from above: candidates beyond it can
    // neither screen in nor keep a side open
    const uint64_t tb_bits = (uint64_t)__double_as_longlong(en.tb);
    uint64_t tw = tb_bits < INF_BITS ? tb_bits : INF_BITS;
    float thr = (PLAIN || unsafe) ? __int_as_float(0x7f800000) : thr_from(tw, mq);
    // screen of one candidate: FP32 (or FP64 for PLAIN) only
    auto screen = [&](int j) -> bool {
      if constexpr (PLAIN) {
        uint64_t mm = 0;
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          const uint64_t v = absdiff_bits(g[(int64_t)c * lds + j], qv[c]);
          mm = v > mm ? v : mm;
        }
        return mm < top[KMAX - 1] && mm <= tw;
      } else {
        float dist = 0.0f;
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          dist = fmaxf(dist, fabsf(g[(int64_t)c * lds + j] - qv[c]));
        }
        return dist <= thr;
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
      if (mm < top[KMAX - 1]) insert_sorted<KMAX>(top, mm);
    };
    // each step: 4 positions per lane on each open side (128 per side)
    int nr = o.start, nl = o.start - 1;
    bool doneR = nr >= len, doneL = nl < 0;
    while (!doneR || !doneL) {
      uint32_t hits = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int jr = nr + lane + 32 * u;
        const int jl = nl - lane - 32 * u;
        if (!doneR && jr < len && screen(jr)) hits |= 1u << u;
        if (!doneL && jl >= 0 && screen(jl)) hits |= 16u << u;
      }
      while (hits) {
        const int b = __ffs(hits) - 1;
        hits &= hits - 1u;
        resolve(b < 4 ? nr + lane + 32 * b : nl - lane - 32 * (b - 4));
      }
      if (!doneR) nr += 128;
      if (!doneL) nl -= 128;
      const uint64_t lw = warp_min_u64(top[KMAX - 1]);
      tw = lw < tw ? lw : tw;
      if (!PLAIN) thr = unsafe ? __int_as_float(0x7f800000) : thr_from(tw, mq);
      const double tbd = bits_to_double(tw);
      if (!doneR) doneR = nr >= len || (scol[nr] - o.qs > tbd);
      if (!doneL) doneL = nl < 0 || (o.qs - scol[nl] > tbd);
    }
    // K-th smallest of the union of the lane lists
    uint64_t lst[KMAX];
#pragma unroll
    for (int s = 0; s < KMAX; ++s) lst[s] = top[s];
    int h = KMAX - K;
    uint64_t kth = INF_BITS;
    for (int r = 0; r < K; ++r) {
      uint64_t v = h < KMAX ? lst[h] : INF_BITS;
      int who = lane;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const uint64_t ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int ow = __shfl_xor_sync(0xffffffffu, who, o);
        if (ov < v || (ov == v && ow < who)) {
          v = ov;
          who = ow;
        }
      }
      kth = v;
      if (lane == who) ++h;
    }
    if (lane == 0) {
      J->eps[J->idx[pos]] = bits_to_double(kth);
      atomicAdd(J->stats + 1, (unsigned long long)(nr - nl - 1));
    }
  }
}

// Launch shapes.  Brute force: 256 threads, large tiles.  Slab: 128 threads
// and 512-point tiles, so that a work item's candidate window stays close to
// the few thousand points around its queries.
template <int D, int KMAX, bool PLAIN, bool SLAB>
struct KnnCfg {
  static constexpr int THREADS = (D == 0 || SLAB) ? 128 : 256;
  static constexpr int QPT = D == 0 ? 1 : KMAX == 4 ? (SLAB ? 2 : 4) : KMAX == 8 ? 2 : 1;
  static constexpr int TILE = D == 0 ? 256 : SLAB ? 512 : (D == 2 ? 2048 : 1024);
};

template <int D, int KMAX, bool PLAIN, bool SLAB>
TileShape knn_shape_t(int dmax) {
  using C = KnnCfg<D, KMAX, PLAIN, SLAB>;
  const int DM = D ? D : dmax;
  TileShape s;
  s.threads = C::THREADS;
  s.qpt = C::QPT;
  s.tile = C::TILE;
  s.smem = 2ull * DM * C::TILE * sizeof(CoordT<PLAIN>);
  return s;
}

template <int D, int KMAX, bool PLAIN, bool SLAB>
void launch_knn_t(const JobDev* jobs, const WorkItem* items, int nitems, int* counter,
                  uint32_t* err, int dmax, DeferEntry* defer, int* defer_count, int num_sms,
                  cudaStream_t st) {
  using C = KnnCfg<D, KMAX, PLAIN, SLAB>;
  const TileShape s = knn_shape_t<D, KMAX, PLAIN, SLAB>(dmax);
  auto kern = knn_tile_kernel<D, KMAX, C::QPT, C::THREADS, C::TILE, PLAIN, SLAB>;
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

template <int D, int KMAX, bool PLAIN>
void launch_knn_defer_t(const JobDev* jobs, const DeferEntry* list, const int* count, int cap,
                        int num_sms, cudaStream_t st) {
  const int warps_per_block = 8;
  int grid = (cap + warps_per_block - 1) / warps_per_block;
  if (grid > num_sms * 8) grid = num_sms * 8;
  if (grid < 1) return;
  knn_defer_kernel<D, KMAX, PLAIN><<<grid, 32 * warps_per_block, 0, st>>>(jobs, list, count, cap);
  count_launch();
}

// Dispatch over (dclass, kclass) for one (PLAIN, SLAB) pair.
template <bool PLAIN, bool SLAB>
struct KnnDispatch {
  template <int D>
  static TileShape shape_d(int kclass, int dmax) {
    switch (kclass) {
      case 4: return knn_shape_t<D, 4, PLAIN, SLAB>(dmax);
      case 8: return knn_shape_t<D, 8, PLAIN, SLAB>(dmax);
      case 16: return knn_shape_t<D, 16, PLAIN, SLAB>(dmax);
      default: return knn_shape_t<D, 32, PLAIN, SLAB>(dmax);
    }
  }
  static TileShape shape(int kclass, int dclass, int dmax) {
    switch (dclass) {
      case 2: return shape_d<2>(kclass, dmax);
      case 3: return shape_d<3>(kclass, dmax);
      case 4: return shape_d<4>(kclass, dmax);
      default: return shape_d<0>(kclass, dmax);
    }
  }
  template <int D>
  static void launch_d(int kclass, const JobDev* jobs, const WorkItem* items, int nitems,
                       int* counter, uint32_t* err, int dmax, DeferEntry* df, int* dc,
                       int num_sms, cudaStream_t st) {
    switch (kclass) {
      case 4: launch_knn_t<D, 4, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      case 8: launch_knn_t<D, 8, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      case 16: launch_knn_t<D, 16, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      default: launch_knn_t<D, 32, PLAIN, SLAB>(jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
    }
  }
  static void launch(int kclass, int dclass, const JobDev* jobs, const WorkItem* items,
                     int nitems, int* counter, uint32_t* err, int dmax, DeferEntry* df,
                     int* dc, int num_sms, cudaStream_t st) {
    switch (dclass) {
      case 2: launch_d<2>(kclass, jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      case 3: launch_d<3>(kclass, jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      case 4: launch_d<4>(kclass, jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
      default: launch_d<0>(kclass, jobs, items, nitems, counter, err, dmax, df, dc, num_sms, st); break;
    }
  }
  template <int D>
  static void defer_d(int kclass, const JobDev* jobs, const DeferEntry* list, const int* count,
                      int cap, int num_sms, cudaStream_t st) {
    switch (kclass) {
      case 4: launch_knn_defer_t<D, 4, PLAIN>(jobs, list, count, cap, num_sms, st); break;
      case 8: launch_knn_defer_t<D, 8, PLAIN>(jobs, list, count, cap, num_sms, st); break;
      case 16: launch_knn_defer_t<D, 16, PLAIN>(jobs, list, count, cap, num_sms, st); break;
      default: launch_knn_defer_t<D, 32, PLAIN>(jobs, list, count, cap, num_sms, st); break;
    }
  }
  static void defer(int kclass, int dclass, const JobDev* jobs, const DeferEntry* list,
                    const int* count, int cap, int num_sms, cudaStream_t st) {
    switch (dclass) {
      case 2: defer_d<2>(kclass, jobs, list, count, cap, num_sms, st); break;
      case 3: defer_d<3>(kclass, jobs, list, count, cap, num_sms, st); break;
      case 4: defer_d<4>(kclass, jobs, list, count, cap, num_sms, st); break;
      default: defer_d<0>(kclass, jobs, list, count, cap, num_sms, st); break;
    }
  }
};

}  // namespace knn_detail

// One translation unit per (PLAIN, SLAB) pair specialises these
// (EGB_KNN_TU), so the four families compile in parallel.
template <bool PLAIN, bool SLAB>
TileShape knn_shape_v(int kclass, int dclass, int dmax);
template <bool PLAIN, bool SLAB>
void launch_knn_v(int kclass, int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                  int* counter, uint32_t* err, int dmax, DeferEntry* df, int* dc, int num_sms,
                  cudaStream_t st);
template <bool PLAIN>
void launch_knn_defer_v(int kclass, int dclass, const JobDev* jobs, const DeferEntry* list,
                        const int* count, int cap, int num_sms, cudaStream_t st);

}  // namespace egb

#define EGB_KNN_TU(P, S)                                                                  \
  namespace egb {                                                                         \
  template <>                                                                             \
  TileShape knn_shape_v<P, S>(int kclass, int dclass, int dmax) {                         \
    return knn_detail::KnnDispatch<P, S>::shape(kclass, dclass, dmax);                    \
  }                                                                                       \
  template <>                                                                             \
  void launch_knn_v<P, S>(int kclass, int dclass, const JobDev* jobs, const WorkItem* items, \
                          int nitems, int* counter, uint32_t* err, int dmax, DeferEntry* df, \
                          int* dc, int num_sms, cudaStream_t st) {                        \
    knn_detail::KnnDispatch<P, S>::launch(kclass, dclass, jobs, items, nitems, counter, err, \
                                          dmax, df, dc, num_sms, st);                     \
  }                                                                                       \
  }
// The deferred-query kernels live with the slab families.
#define EGB_KNN_DEFER_TU(P)                                                               \
  namespace egb {                                                                         \
  template <>                                                                             \
  void launch_knn_defer_v<P>(int kclass, int dclass, const JobDev* jobs,                 \
                             const DeferEntry* list, const int* count, int cap,          \
                             int num_sms, cudaStream_t st) {                             \
    knn_detail::KnnDispatch<P, true>::defer(kclass, dclass, jobs, list, count, cap,       \
                                            num_sms, st);                                 \
  }                                                                                       \
  }
