// egb_wgrid.cuh -- warp-level form of the grid (strip) kernels.
//
// Same layout and search region as egb_grid.cuh, but every warp works alone:
// it pulls an item of up to 32 consecutive strip positions (one query per
// lane) from the device work counter, plans its windows with ballots and
// shuffles instead of CTA barriers, and reads candidates as float4 broadcasts
// (all lanes load the same 16 bytes) from the job's columns, which stay in
// L1/L2.  Planning therefore never stalls other warps, and each warp's
// windows are narrower (32 queries span a quarter of the x-range of 128).
//
// Schedule of an item: the queries' own positions, the rest of the home
// strip's window [xa - T, xb + T], then strips sq+1, sq-1, sq+2, ... while
// open for some unfinished query, T being the largest threshold among
// unfinished queries.  Window ends are exact (16-ary warp search).  When at
// most OUTLIER_LANES queries are still unfinished, the warp finishes them one
// at a time with all 32 lanes sharing the candidates of the remaining strips
// (window [q0 - t, q0 + t] of that query alone); for kNN each lane keeps its
// own list and the K-th smallest of the union is taken at the end.
//
// Exactness as in the other tile kernels: FP32 screen with the proven band,
// FP64 decision for every candidate the screen cannot settle.
#pragma once
#include "egb_tile.cuh"

namespace egb {
namespace wgrid_detail {

constexpr int WG_WARPS = 4;       // warps per CTA (independent)
constexpr int OUTLIER_LANES = 2;  // switch to cooperative finishing below this

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

__device__ __forceinline__ uint64_t warp_max_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Conservative FP32 planning values.  A grid copy holds, per coordinate,
// f(v) = fl32(clamp(fl64(v - c), +-1e37)), monotone in v.  lo32_of / hi32_of
// bound v - c from below / above; plan_margin(t) >= t (1 + 2^-20), so that a
// candidate skipped because its coordinate gap exceeds plan_margin(t) has an
// FP64 coordinate distance fl64(gap) >= gap (1 - 2^-53) > t.
__device__ __forceinline__ float lo32_of(double v, double c) {
  return __double2float_rd(__dsub_rd(v, c));
}
__device__ __forceinline__ float hi32_of(double v, double c) {
  return __double2float_ru(__dsub_ru(v, c));
}
__device__ __forceinline__ float plan_margin(float t) { return __fmul_ru(t, 1.0f + 0x1p-20f); }

// Exact window of strip [s0, s1) for column-0 values [xlo, xhi]: the lower
// half-warp finds the first position with x >= xlo, the upper half the first
// with x > xhi.
template <typename V>
__device__ __forceinline__ void warp_window(const V* x, int s0, int s1, V xlo, V xhi, int& wlo,
                                            int& whi) {
  const int lane = threadIdx.x & 31;
  const bool upper = lane >= 16;
  const int l16 = lane & 15;
  const unsigned m = upper ? 0xffff0000u : 0x0000ffffu;
  // Both halves run the same loop shape; each keeps its own bracket.
  int lo = s0, hi = s1;
  for (int round = 0; round < 40; ++round) {
    const int n = hi - lo;
    const bool small = n <= 16;
    int p = small ? lo + l16 : lo + (int)((int64_t)(l16 + 1) * n / 17);
    const bool inr = p < hi;
    p = inr ? p : s0;
    const V v = x[p];
    const bool t = inr && (upper ? (v <= xhi) : (v < xlo));
    const unsigned b = __ballot_sync(0xffffffffu, t) & m;
    const int c = __popc(b);
    if (small) {
      lo = lo + c;
      hi = lo;
    } else {
      const int nlo = c == 0 ? lo : lo + (int)((int64_t)c * n / 17) + 1;
      const int nhi = c == 16 ? hi : lo + (int)((int64_t)(c + 1) * n / 17);
      lo = nlo;
      hi = nhi;
    }
    const bool done = hi - lo <= 0;
    if (__all_sync(0xffffffffu, done)) break;
  }
  wlo = __shfl_sync(0xffffffffu, lo, 0);
  whi = __shfl_sync(0xffffffffu, lo, 16);
  if (whi < wlo) whi = wlo;
}

// FP32 threshold bounding from above the FP64 distance of any candidate
// whose FP32 distance is t (t >= 0 finite): t + band(mq, t), rounded up.
__device__ __forceinline__ float up_band32(float t, float mq) {
  if (!(t < __int_as_float(0x7f800000))) return __int_as_float(0x7f800000);
  return __fmaf_ru(t, 1.0f + 0x1p-21f, __fmaf_ru(mq, 0x1p-21f, 0x1p-100f));
}
// FP32 value bounding from below the FP64 distance of a candidate whose FP32
// distance is t (t >= 0 finite).  From |t - D| <= 2^-23 (M + D)(1 + 2^-20)
// + 2^-148 (egb_internal.cuh), D >= (t - 2^-23 M (1 + 2^-20) - 2^-148) /
// (1 + 2^-23 (1 + 2^-20)); with mq >= M and the factors taken four times
// over, (t - 2^-21 mq - 2^-100)(1 - 2^-21) rounded down is below that.
__device__ __forceinline__ float dn_band32(float t, float mq) {
  if (!(t < __int_as_float(0x7f800000))) return 0.0f;
  const float a = __fsub_rd(t, __fmaf_ru(mq, 0x1p-21f, 0x1p-100f));
  return a > 0.0f ? __fmul_rd(a, 1.0f - 0x1p-21f) : 0.0f;
}

template <int KMAX>
__device__ __forceinline__ void insert_sorted_f(float (&l)[KMAX], float v) {
  l[KMAX - 1] = v;
#pragma unroll
  for (int s = KMAX - 1; s > 0; --s) {
    const float a = l[s - 1], b = l[s];
    const bool sw = b < a;
    l[s - 1] = sw ? b : a;
    l[s] = sw ? a : b;
  }
}

// Sorted insert of (v, j) into an FP32 list with candidate indices; returns
// the value pushed out of the last slot.
template <int KMAX>
__device__ __forceinline__ float insert_sorted_fi(float (&l)[KMAX], int (&ix)[KMAX], float v,
                                                  int j) {
  const float out = l[KMAX - 1];
  l[KMAX - 1] = v;
  ix[KMAX - 1] = j;
#pragma unroll
  for (int s = KMAX - 1; s > 0; --s) {
    const float a = l[s - 1], b = l[s];
    const int ia = ix[s - 1], ib = ix[s];
    const bool sw = b < a;
    l[s - 1] = sw ? b : a;
    l[s] = sw ? a : b;
    ix[s - 1] = sw ? ib : ia;
    ix[s] = sw ? ia : ib;
  }
  return out;
}

// K-th smallest of the union of per-lane sorted lists (the first KMAX - K
// entries of each list are padding).  Warp-wide; result in every lane.
template <int KMAX, typename V>
__device__ __forceinline__ V warp_kth_of_lists(const V (&lst_in)[KMAX], int K, V inf) {
  const int lane = threadIdx.x & 31;
  V lst[KMAX];
#pragma unroll
  for (int s = 0; s < KMAX; ++s) lst[s] = lst_in[s];
  int h = KMAX - K;
  V kth = inf;
  for (int r = 0; r < K; ++r) {
    V v = h < KMAX ? lst[h] : inf;
    int who = lane;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const V ov = __shfl_xor_sync(0xffffffffu, v, o);
      const int ow = __shfl_xor_sync(0xffffffffu, who, o);
      if (ov < v || (ov == v && ow < who)) {
        v = ov;
        who = ow;
      }
    }
    kth = v;
    if (lane == who) ++h;
  }
  return kth;
}

// Blocks per SM the register budget of a variant targets: the K <= 4 kNN
// kernels are latency-bound and gain from occupancy more than they lose to
// a few spilled registers outside the candidate loop.
template <int D, int KMAX, bool COUNT>
constexpr int wgrid_min_blocks() {
  return (!COUNT && KMAX == 4) ? (D == 2 ? 5 : 4) : 1;
}

template <int D, int KMAX, bool PLAIN, bool COUNT, bool NEST>
__global__ void __launch_bounds__(WG_WARPS * 32, (wgrid_min_blocks<D, KMAX, COUNT>()))
wgrid_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items, int nitems,
             int* __restrict__ counter, int dmax) {
  using T = CoordT<PLAIN>;
  constexpr int DQ = D ? D : EGB_DMAX;
  // kNN with the FP32 screen: pass 0 finds each query's FP32 k-th distance
  // t32 with an FP32 list of (distance, candidate) and the least FP32
  // distance `rej` of every candidate left out of the list.  Every candidate
  // with FP32 distance <= S = t32 + band + band (the screen bound of an
  // exact pass) is then in the list when rej > S, and the exact k-th
  // distance is the largest exact distance of the K listed candidates -- K
  // FP64 evaluations per query.  Queries without that margin (near ties,
  // unsafe jobs, fewer than K candidates) run pass 1: the schedule again with
  // the fixed bound U = t32 + band >= the exact k-th distance, deciding every
  // candidate with FP32 distance <= S in FP64.  FP64 stays off the hot loop
  // (a 2-lane/clk/SM pipe on GB300).
  constexpr bool TWO_PASS = !PLAIN && !COUNT;
  constexpr float FINF = __builtin_huge_valf();
  const int lane = threadIdx.x & 31;
  (void)dmax;
  // Planning -- window ends, strip and cell tests, thresholds -- is in type
  // T: the FP64 comparator plans on the exact values; the FP32 path plans on
  // centred FP32 values with outward-directed rounding and plan_margin(), so
  // it visits a superset of the candidates exact planning would (GB300
  // issues FP64 at a small fraction of the FP32 rate).

  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const WorkItem wi = items[it];
    const JobDev* __restrict__ J = jobs + wi.job;
    const int d = D ? D : J->sp.d;
    const int len = J->len;
    const int64_t lds = J->lds;
    const double* __restrict__ c64 = J->c64g;
    const T* __restrict__ g = PLAIN ? reinterpret_cast<const T*>(J->c64g)
                                    : reinterpret_cast<const T*>(J->c32g);
    const int32_t* __restrict__ sst = J->sstart;      // strip starts
    const T* __restrict__ wx = g;                     // column 0: window searches
    // strip column-1 bounds and (nested) cell column-2 bounds
    const T* __restrict__ ylo_t = reinterpret_cast<const T*>(PLAIN ? (const void*)J->sylo : (const void*)J->sylo32);
    const T* __restrict__ yhi_t = reinterpret_cast<const T*>(PLAIN ? (const void*)J->syhi : (const void*)J->syhi32);
    const int S = J->nstrips;
    // nested grids: cells of strip s are s * S2 .. s * S2 + S2 - 1
    const int S2 = NEST ? J->nsub : 1;
    const int32_t* __restrict__ cst = J->cstart;
    const T* __restrict__ czlo = reinterpret_cast<const T*>(PLAIN ? (const void*)J->czlo : (const void*)J->czlo32);
    const T* __restrict__ czhi = reinterpret_cast<const T*>(PLAIN ? (const void*)J->czhi : (const void*)J->czhi32);
    const bool unsafe = !PLAIN && ((*J->jflags & TF_UNSAFE32) != 0u);
    const int K = COUNT ? 1 : J->K;

    const int qp = wi.q0 + lane;
    const bool exists = qp < wi.q1;
    const int nq = wi.q1 - wi.q0;
    T qv[DQ];
    double m = 0.0;
#pragma unroll
    for (int c = 0; c < DQ; ++c) {
      if (D == 0 && c >= d) break;
      qv[c] = exists ? g[(int64_t)c * lds + qp] : T(0);
      if (!PLAIN && exists) {
        const double v = fabs(c64[(int64_t)c * lds + qp] - J->center[c]);
        m = v > m ? v : m;
      }
    }
    const float mq = __double2float_ru(m);
    const double qx = exists ? c64[qp] : 0.0;
    const double qy = exists ? c64[lds + qp] : 0.0;
    const double qz = (NEST && exists) ? c64[2 * lds + qp] : 0.0;
    // planning bounds of the query's coordinates 0..2
    T qxl, qxh, qyl, qyh, qzl, qzh;
    if constexpr (PLAIN) {
      qxl = qxh = qx;
      qyl = qyh = qy;
      qzl = qzh = qz;
    } else {
      qxl = exists ? lo32_of(qx, J->center[0]) : 0.0f;
      qxh = exists ? hi32_of(qx, J->center[0]) : 0.0f;
      qyl = exists ? lo32_of(qy, J->center[1]) : 0.0f;
      qyh = exists ? hi32_of(qy, J->center[1]) : 0.0f;
      qzl = (NEST && exists) ? lo32_of(qz, J->center[2]) : 0.0f;
      qzh = (NEST && exists) ? hi32_of(qz, J->center[2]) : 0.0f;
    }

    // ---- per-lane state
    uint64_t top[COUNT ? 1 : KMAX];      // exact list (bit patterns)
    float l32[TWO_PASS ? KMAX : 1];      // FP32 list (pass 0)
    int i32[TWO_PASS ? KMAX : 1];        // its candidates
    float rej = FINF;                    // least FP32 distance left out of the list
    double ufix = 0.0;                    // pass 1: fixed bound of the k-th distance
    float u32fix = 0.0f;                  // the same bound (a float)
    float sfix = 0.0f;                    // pass 1: FP32 screen threshold
    float tcnt = -1.0f;                   // FP32 counts: planning threshold
    double qr = -1.0;
    uint64_t rbits = 0;
    float lo = -1.0f, hi = -1.0f;
    int cntq = 0;
    bool qok = exists;
    int pass = TWO_PASS ? 0 : 1;
    if constexpr (COUNT) {
      qr = exists ? J->rad[J->idxg[qp]] : -1.0;
      qok = exists && (qr >= 0.0);
      rbits = qok ? (uint64_t)__double_as_longlong(qr) : 0ull;
      if (!PLAIN && qok) tcnt = plan_margin(__double2float_ru(qr));
      if (!PLAIN && qok) {
        if (isinf(qr)) {
          lo = hi = FINF;
        } else if (unsafe) {
          hi = FINF;
        } else {
          const double b = band((double)mq, qr);
          lo = __double2float_rd(qr - b);
          hi = __double2float_ru(qr + b);
        }
      }
    } else {
#pragma unroll
      for (int s = 0; s < KMAX; ++s) top[s] = (exists && s >= KMAX - K) ? INF_BITS : 0ull;
      if constexpr (TWO_PASS) {
#pragma unroll
        for (int s = 0; s < KMAX; ++s) {
          l32[s] = (exists && s >= KMAX - K) ? FINF : 0.0f;
          i32[s] = 0;
        }
      }
    }
    // upper bound of what this lane's query still needs (planning threshold)
    auto tq = [&]() -> double {
      if (!qok) return -1.0;
      if constexpr (COUNT) {
        return qr;
      } else if constexpr (TWO_PASS) {
        if (pass == 0) return unsafe ? HUGE_VAL : (double)up_band32(l32[KMAX - 1], mq);
        return ufix;
      } else {
        return bits_to_double(top[KMAX - 1]);
      }
    };
    // the same as a planning value (negative: nothing needed)
    auto tqp = [&]() -> T {
      if constexpr (PLAIN) {
        return tq();
      } else {
        if (!qok) return -1.0f;
        if constexpr (COUNT) return tcnt;
        else return pass == 0 ? (unsafe ? FINF : plan_margin(up_band32(l32[KMAX - 1], mq)))
                              : plan_margin(u32fix);
      }
    };
    // largest planning threshold over the lanes (negative ones count as 0)
    auto wmax = [&](T v) -> T {
      if constexpr (PLAIN) {
        return bits_to_double(warp_max_u64(v >= 0.0 ? (uint64_t)__double_as_longlong(v) : 0ull));
      } else {
        return __uint_as_float(__reduce_max_sync(0xffffffffu, v >= 0.0f ? __float_as_uint(v) : 0u));
      }
    };
    // window ends around [a, b] for threshold t
    auto wlo = [&](T a, T t) -> T {
      if constexpr (PLAIN) return a - t;
      else return fminf(__fsub_rd(a, t), 1e37f);
    };
    auto whi = [&](T b, T t) -> T {
      if constexpr (PLAIN) return b + t;
      else return fmaxf(__fadd_ru(b, t), -1e37f);
    };
    // a range with lower bound lb lies more than t above a query whose
    // upper bound is qh / with upper bound hb more than t below ql
    auto above = [&](T lb, T qh, T t) -> bool {
      if constexpr (PLAIN) return lb - qh > t;
      else return __fsub_rd(lb, qh) > t;
    };
    auto below = [&](T ql, T hb, T t) -> bool {
      if constexpr (PLAIN) return ql - hb > t;
      else return __fsub_rd(ql, hb) > t;
    };
    auto exact_dist = [&](int j, int q) -> uint64_t {
      uint64_t mm = 0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        const int64_t off = (int64_t)c * lds;
        const uint64_t v = absdiff_bits(c64[off + j], c64[off + q]);
        mm = v > mm ? v : mm;
      }
      return mm;
    };

    // Resolve the hits of one group of 4 candidates at g0 (FP32 distances in dst).
    auto resolve = [&](int g0, uint32_t hits, const float (&dst)[4]) {
      while (hits) {
        const int u = __ffs(hits) - 1;
        hits &= hits - 1u;
        const int j = g0 + u;
        if constexpr (TWO_PASS) {
          if (pass == 0) {
            const float dv = u == 0 ? dst[0] : u == 1 ? dst[1] : u == 2 ? dst[2] : dst[3];
            const float out = dv < l32[KMAX - 1] ? insert_sorted_fi<KMAX>(l32, i32, dv, j) : dv;
            rej = fminf(rej, out);
            continue;
          }
        }
        const uint64_t mm = exact_dist(j, qp);
        if constexpr (COUNT) {
          cntq += (mm <= rbits) ? 1 : 0;
        } else if (mm < top[KMAX - 1]) {
          insert_sorted<KMAX>(top, mm);
        }
      }
    };
    // FP32 decision bits of one group (distances in dst, validity in vmask).
    auto decide = [&](int g0, uint32_t vmask, const float (&dst)[4]) {
      uint32_t hits = 0, inside = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if constexpr (COUNT) {
          inside |= (dst[u] <= lo ? 1u : 0u) << u;
          hits |= ((dst[u] > lo) && (dst[u] <= hi) ? 1u : 0u) << u;
        } else if constexpr (TWO_PASS) {
          hits |= ((pass == 0 ? dst[u] < l32[KMAX - 1] : dst[u] <= sfix) ? 1u : 0u) << u;
        }
      }
      if constexpr (COUNT) cntq += __popc(inside & vmask);
      if constexpr (TWO_PASS) {
        if (pass == 0) {
          // the group's least distance, or the list bound when some is a hit
          // (a hit that is left out after all updates rej in resolve)
          float m4;
          if (vmask == 0xFu) {
            m4 = fminf(fminf(dst[0], dst[1]), fminf(dst[2], dst[3]));
          } else {
            m4 = FINF;
#pragma unroll
            for (int u = 0; u < 4; ++u) m4 = fminf(m4, ((vmask >> u) & 1u) ? dst[u] : FINF);
          }
          rej = fminf(rej, fmaxf(m4, l32[KMAX - 1]));
        }
      }
      hits &= vmask;
      if (__builtin_expect(hits != 0u, 0)) resolve(g0, hits, dst);
    };
    // candidates of the group at g0 inside [ra, rb) and outside [ea, eb)
    auto group_mask = [](int g0, int ra, int rb, int ea, int eb) -> uint32_t {
      uint32_t vmask = 0xFu;
      if (g0 < ra) vmask &= ~((1u << (ra - g0)) - 1u);
      if (g0 + 4 > rb) vmask &= (1u << (rb - g0)) - 1u;
      if (g0 + 4 > ea && g0 < eb) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (g0 + u >= ea && g0 + u < eb) vmask &= ~(1u << u);
      }
      return vmask;
    };

    unsigned long long pairs = 0;  // candidate-query pairs screened by this item
    // Screen the candidates [ra, rb) minus [ea, eb) against this lane's query.
    auto scan = [&](int ra, int rb, int ea, int eb) {
      if (rb <= ra) return;
      pairs += (unsigned long long)(rb - ra - max(0, min(rb, eb) - max(ra, ea))) * (unsigned long long)nq;
      if constexpr (D != 0 && !PLAIN) {
        // two groups of 4 per step: both groups' loads are in flight together
        for (int g0 = ra & ~3; g0 < rb; g0 += 8) {
          const bool hasb = g0 + 4 < rb;
          float4 ca[D], cb[D];
#pragma unroll
          for (int c = 0; c < D; ++c) {
            ca[c] = __ldg(reinterpret_cast<const float4*>(g + (int64_t)c * lds + g0));
            cb[c] = hasb ? __ldg(reinterpret_cast<const float4*>(g + (int64_t)c * lds + g0 + 4))
                         : make_float4(0.f, 0.f, 0.f, 0.f);
          }
          float da[4], db[4];
#define EGB_WG_LANE(U)                                                          \
  {                                                                             \
    float x0 = fabsf(pick4<U>(ca[0]) - qv[0]);                                  \
    float x1 = fabsf(pick4<U>(cb[0]) - qv[0]);                                  \
    _Pragma("unroll") for (int c = 1; c < D; ++c) {                             \
      x0 = fmaxf(x0, fabsf(pick4<U>(ca[c]) - qv[c]));                           \
      x1 = fmaxf(x1, fabsf(pick4<U>(cb[c]) - qv[c]));                           \
    }                                                                           \
    da[U] = x0;                                                                 \
    db[U] = x1;                                                                 \
  }
          EGB_WG_LANE(0)
          EGB_WG_LANE(1)
          EGB_WG_LANE(2)
          EGB_WG_LANE(3)
#undef EGB_WG_LANE
          decide(g0, group_mask(g0, ra, rb, ea, eb), da);
          if (hasb) decide(g0 + 4, group_mask(g0 + 4, ra, rb, ea, eb), db);
        }
      } else {
        for (int g0 = ra & ~3; g0 < rb; g0 += 4) {
          const uint32_t vmask = group_mask(g0, ra, rb, ea, eb);
          float dst[4];
          uint32_t hits = 0;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int j = g0 + u < len ? g0 + u : len - 1;
            if constexpr (PLAIN) {
              uint64_t mm = 0;
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (D == 0 && c >= d) break;
                const uint64_t v = absdiff_bits(g[(int64_t)c * lds + j], qv[c]);
                mm = v > mm ? v : mm;
              }
              if constexpr (COUNT) cntq += ((vmask >> u) & 1u) && qok && mm <= rbits ? 1 : 0;
              else hits |= (mm < top[KMAX - 1] ? 1u : 0u) << u;
              dst[u] = 0.0f;
            } else {
              float dist = 0.0f;
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (c >= d) break;
                dist = fmaxf(dist, fabsf(g[(int64_t)c * lds + j] - qv[c]));
              }
              dst[u] = dist;
            }
          }
          if constexpr (PLAIN) {
            hits &= vmask;
            if (hits) resolve(g0, hits, dst);
          } else {
            decide(g0, vmask, dst);
          }
        }
      }
    };

    const int sq = NEST ? (wi.strip & 0xffff) : wi.strip;
    const int hc2 = NEST ? (wi.strip >> 16) : 0;  // home cell within the strip
    const int hs0 = NEST ? cst[sq * S2 + hc2] : sst[sq];
    const int hs1 = NEST ? cst[sq * S2 + hc2 + 1] : sst[sq + 1];
    const T xal = __shfl_sync(0xffffffffu, qxl, 0);        // the item's column-0 range
    const T xbh = __shfl_sync(0xffffffffu, qxh, nq - 1);
    // column-2 centre of the item (nested grids: where other strips start)
    const T zmid = NEST ? __shfl_sync(0xffffffffu, qzl, (nq - 1) >> 1) : T(0);

    // Nested grids: first cell of strip s whose column-2 range reaches z.
    auto start_cell = [&](int s, T z) -> int {
      int c0 = 0;
      for (int b = 0; b < S2; b += 32) {
        const int c = b + lane;
        c0 += __popc(__ballot_sync(0xffffffffu, c < S2 && czhi[s * S2 + c] < z));
      }
      return c0 < S2 ? c0 : S2 - 1;
    };
    // Nested grids: the cells of strip s that some lane still needs, outward
    // in column 2 from cell c0 (cell `skip` already scanned).  A lane needs a
    // cell while the strip's column-1 range and the cell's column-2 range are
    // both within its threshold; cells are ordered by column 2, so each
    // direction ends at the first cell that no lane reaches.
    auto visit_cells = [&](int s, int c0, int skip) {
      const int cb = s * S2;
      int up2 = c0, dn2 = c0 - 1;
      bool tu = true;
      for (;;) {
        const T t = tqp();
        const bool reach = qok && !above(ylo_t[s], qyh, t) && !below(qyl, yhi_t[s], t);
        const bool ou = reach && up2 < S2 && !above(czlo[cb + up2], qzh, t);
        const bool od = reach && dn2 >= 0 && !below(qzl, czhi[cb + dn2], t);
        const bool any_u = __any_sync(0xffffffffu, ou);
        const bool any_d = __any_sync(0xffffffffu, od);
        if (!any_u && !any_d) break;
        int c;
        if ((tu && any_u) || !any_d) {
          c = up2++;
          tu = false;
        } else {
          c = dn2--;
          tu = true;
        }
        if (c == skip) continue;
        const bool nd = reach && !above(czlo[cb + c], qzh, t) && !below(qzl, czhi[cb + c], t);
        if (!__any_sync(0xffffffffu, nd)) continue;
        const T Tw = wmax(nd ? t : T(-1));
        int wl, wh;
        warp_window(wx, cst[cb + c], cst[cb + c + 1], wlo(xal, Tw), whi(xbh, Tw), wl, wh);
        scan(wl, wh, 0, 0);
      }
    };

#pragma unroll 1
    for (; pass < 2; ++pass) {
      if constexpr (TWO_PASS) {
        if (pass == 1) {
          // settle every query whose list holds all candidates within S
          bool need = false;
          const float u32 = unsafe ? FINF : up_band32(l32[KMAX - 1], mq);
          const float s32 = unsafe ? FINF : up_band32(u32, mq);
          if (qok) {
            if (rej > s32) {
              uint64_t mx = 0;
#pragma unroll
              for (int s = 0; s < KMAX; ++s) {
                if (s >= KMAX - K) {
                  const uint64_t e = exact_dist(i32[s], qp);
                  mx = e > mx ? e : mx;
                }
              }
              top[KMAX - 1] = mx;
            } else {
              need = true;
            }
          }
          const unsigned fbm = __ballot_sync(0xffffffffu, need);
          if (fbm == 0u) break;  // every query of the item is settled
          if (lane == 0) atomicAdd(J->stats + 2, (unsigned long long)__popc(fbm));
          // pass 1 for the rest, with the bound fixed from pass 0
          qok = need;
          ufix = need ? (double)u32 : -1.0;
          u32fix = need ? u32 : -1.0f;
          sfix = need ? s32 : -1.0f;
        }
      }
      // ---- own positions (they seed the kNN thresholds), then the rest of
      // the home strip's (cell's) window
      scan(wi.q0, wi.q1, 0, 0);
      {
        const T Tw = wmax(tqp());
        int wl, wh;
        warp_window(wx, hs0, hs1, wlo(xal, Tw), whi(xbh, Tw), wl, wh);
        scan(wl, wh, wi.q0, wi.q1);
      }

      // ---- other strips (nested grids: first the other cells of the home strip)
      int up = sq + 1, dn = sq - 1;
      bool turn_up = true;
      bool home_cells = NEST;
      auto unfinished = [&]() -> bool {
        if (!qok) return false;
        const T t = tqp();
        const bool u = up >= S || above(ylo_t[up], qyh, t);
        const bool l = dn < 0 || below(qyl, yhi_t[dn], t);
        return !(u && l);
      };
      for (;;) {
        if (NEST && home_cells) {
          home_cells = false;
          visit_cells(sq, hc2, hc2);
          continue;
        }
        const bool unf = unfinished();
        const unsigned ub = __ballot_sync(0xffffffffu, unf);
        if (ub == 0u || __popc(ub) <= OUTLIER_LANES) break;
        const T t = tqp();
        const bool ou = unf && up < S && !above(ylo_t[up], qyh, t);
        const bool od = unf && dn >= 0 && !below(qyl, yhi_t[dn], t);
        const bool any_u = __any_sync(0xffffffffu, ou);
        const bool any_d = __any_sync(0xffffffffu, od);
        if (!any_u && !any_d) break;  // an unfinished query always needs a side
        int s;
        if ((turn_up && any_u) || !any_d) {
          s = up++;
          turn_up = false;
        } else {
          s = dn--;
          turn_up = true;
        }
        if constexpr (NEST) {
          visit_cells(s, start_cell(s, zmid), -1);
        } else {
          const T Tw = wmax(unf ? t : T(-1));
          int wl, wh;
          warp_window(wx, sst[s], sst[s + 1], wlo(xal, Tw), whi(xbh, Tw), wl, wh);
          scan(wl, wh, 0, 0);
        }
      }

      // ---- remaining unfinished queries: one at a time, all lanes cooperating
      unsigned rest = __ballot_sync(0xffffffffu, unfinished());
      if (lane == 0 && rest) atomicAdd(J->stats + 1, (unsigned long long)__popc(rest));
      while (rest) {
        const int ol = __ffs(rest) - 1;
        rest &= rest - 1u;
        const T oqxl = __shfl_sync(0xffffffffu, qxl, ol), oqxh = __shfl_sync(0xffffffffu, qxh, ol);
        const T oqyl = __shfl_sync(0xffffffffu, qyl, ol), oqyh = __shfl_sync(0xffffffffu, qyh, ol);
        const T oqzl = __shfl_sync(0xffffffffu, qzl, ol), oqzh = __shfl_sync(0xffffffffu, qzh, ol);
        const float omq = __shfl_sync(0xffffffffu, mq, ol);
        T oqv[DQ];
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          oqv[c] = __shfl_sync(0xffffffffu, qv[c], ol);
        }
        const int oqp = wi.q0 + ol;
        const bool op0 = TWO_PASS && pass == 0;
        uint64_t top2[COUNT ? 1 : KMAX];
        float l2[TWO_PASS ? KMAX : 1];
        int ix2[TWO_PASS ? KMAX : 1];
        float rej2 = FINF;
        int cnt2 = 0;
        float olo = -1.0f, ohi = -1.0f, othr = FINF;
        uint64_t orbits = 0;
        T tb = __shfl_sync(0xffffffffu, tqp(), ol);  // planning bound of what the outlier needs
        if constexpr (COUNT) {
          orbits = __shfl_sync(0xffffffffu, rbits, ol);
          olo = __shfl_sync(0xffffffffu, lo, ol);
          ohi = __shfl_sync(0xffffffffu, hi, ol);
        } else {
#pragma unroll
          for (int s2 = 0; s2 < KMAX; ++s2) top2[s2] = s2 >= KMAX - K ? INF_BITS : 0ull;
          if constexpr (TWO_PASS) {
#pragma unroll
            for (int s2 = 0; s2 < KMAX; ++s2) {
              l2[s2] = s2 >= KMAX - K ? FINF : 0.0f;
              ix2[s2] = 0;
            }
            if (op0) l2[KMAX - 1] = FINF;
            othr = __shfl_sync(0xffffffffu, sfix, ol);
            if (op0) {
              // the owner's current FP32 k-th caps every lane's list
              const float ok32 = __shfl_sync(0xffffffffu, l32[KMAX - 1], ol);
              othr = ok32;
            }
          }
        }
        auto oscan = [&](int ra, int rb) {
          for (int j0 = ra; j0 < rb; j0 += 32) {
            const int j = j0 + lane;
            if (j >= rb) continue;
            bool hit;
            float dist = 0.0f;
            if constexpr (PLAIN) {
              uint64_t mm = 0;
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (D == 0 && c >= d) break;
                const uint64_t v = absdiff_bits(g[(int64_t)c * lds + j], oqv[c]);
                mm = v > mm ? v : mm;
              }
              if constexpr (COUNT) {
                cnt2 += mm <= orbits ? 1 : 0;
                hit = false;
              } else {
                hit = mm < top2[KMAX - 1];
              }
            } else {
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (D == 0 && c >= d) break;
                dist = fmaxf(dist, fabsf(g[(int64_t)c * lds + j] - oqv[c]));
              }
              if constexpr (COUNT) {
                cnt2 += dist <= olo ? 1 : 0;
                hit = dist > olo && dist <= ohi;
              } else if (op0) {
                hit = dist < l2[KMAX - 1] && dist < othr;
              } else {
                hit = dist <= othr;
              }
            }
            if constexpr (TWO_PASS) {
              if (op0) {
                rej2 = fminf(rej2, hit ? insert_sorted_fi<KMAX>(l2, ix2, dist, j) : dist);
                continue;
              }
            }
            if (hit) {
              const uint64_t mm = exact_dist(j, oqp);
              if constexpr (COUNT) cnt2 += mm <= orbits ? 1 : 0;
              else if (mm < top2[KMAX - 1]) insert_sorted<KMAX>(top2, mm);
            }
          }
        };
        int oup = up, odn = dn;
        for (;;) {
          if constexpr (!COUNT) {
            if (op0) {
              // any lane holding K entries bounds the union's FP32 k-th
              float lk = l2[KMAX - 1];
#pragma unroll
              for (int o = 16; o; o >>= 1) lk = fminf(lk, __shfl_xor_sync(0xffffffffu, lk, o));
              if (lk < othr) othr = lk;
              const T nb = unsafe ? T(FINF) : T(plan_margin(up_band32(othr, omq)));
              if (nb < tb) tb = nb;
            } else if constexpr (PLAIN) {
              const double lbd = bits_to_double(warp_min_u64(top2[KMAX - 1]));
              if (lbd < tb) tb = lbd;
            }
          }
          const bool ou = oup < S && !above(ylo_t[oup], oqyh, tb);
          const bool od = odn >= 0 && !below(oqyl, yhi_t[odn], tb);
          if (!ou && !od) break;
          const int s = ou && (!od || (oup - sq) <= (sq - odn)) ? oup++ : odn--;
          int wl, wh;
          if constexpr (NEST) {
            // cells with column-2 range meeting [oqz - tb, oqz + tb]: a run
            int clo = 0, chi = 0;
            for (int b = 0; b < S2; b += 32) {
              const int c = b + lane;
              clo += __popc(__ballot_sync(0xffffffffu, c < S2 && below(oqzl, czhi[s * S2 + c], tb)));
              chi += __popc(__ballot_sync(0xffffffffu, c < S2 && !above(czlo[s * S2 + c], oqzh, tb)));
            }
            for (int c = clo; c < chi; ++c) {
              warp_window(wx, cst[s * S2 + c], cst[s * S2 + c + 1], wlo(oqxl, tb), whi(oqxh, tb), wl, wh);
              pairs += (unsigned long long)(wh > wl ? wh - wl : 0);
              oscan(wl, wh);
            }
          } else {
            warp_window(wx, sst[s], sst[s + 1], wlo(oqxl, tb), whi(oqxh, tb), wl, wh);
            pairs += (unsigned long long)(wh > wl ? wh - wl : 0);
            oscan(wl, wh);
          }
        }
        if constexpr (COUNT) {
          const int add = __reduce_add_sync(0xffffffffu, cnt2);
          if (lane == ol) cntq += add;
        } else {
          bool merged = false;
          if constexpr (TWO_PASS) {
            if (op0) {
              if (lane == ol) {  // the owner's list and left-outs join its lane's
                rej2 = fminf(rej2, rej);
#pragma unroll
                for (int s2 = 0; s2 < KMAX; ++s2) {
                  if (s2 >= KMAX - K) {
                    const float v = l32[s2];
                    rej2 = fminf(rej2, v < l2[KMAX - 1] ? insert_sorted_fi<KMAX>(l2, ix2, v, i32[s2]) : v);
                  }
                }
              }
              // the K smallest of the union, in order, become the owner's list
              float nl[KMAX];
              int ni[KMAX];
#pragma unroll
              for (int s2 = 0; s2 < KMAX; ++s2) {
                nl[s2] = 0.0f;
                ni[s2] = 0;
              }
              int taken = 0;
              for (int r = 0; r < K; ++r) {
                const int hp = KMAX - K + taken;
                float v = FINF;
                int vi = 0;
#pragma unroll
                for (int s2 = 0; s2 < KMAX; ++s2) {
                  if (s2 == hp) {
                    v = l2[s2];
                    vi = ix2[s2];
                  }
                }
                int who = lane;
#pragma unroll
                for (int o = 16; o; o >>= 1) {
                  const float ov = __shfl_xor_sync(0xffffffffu, v, o);
                  const int ow = __shfl_xor_sync(0xffffffffu, who, o);
                  if (ov < v || (ov == v && ow < who)) {
                    v = ov;
                    who = ow;
                  }
                }
                const int bi = __shfl_sync(0xffffffffu, vi, who);
                if (lane == who) ++taken;
                if (lane == ol) {
#pragma unroll
                  for (int s2 = 0; s2 < KMAX - 1; ++s2) {
                    nl[s2] = nl[s2 + 1];
                    ni[s2] = ni[s2 + 1];
                  }
                  nl[KMAX - 1] = v;
                  ni[KMAX - 1] = bi;
                }
              }
              // left out: every lane's next entry and its rejections
              {
                const int hp = KMAX - K + taken;
                float v = FINF;
#pragma unroll
                for (int s2 = 0; s2 < KMAX; ++s2)
                  if (s2 == hp) v = l2[s2];
                float lo2 = fminf(rej2, v);
#pragma unroll
                for (int o = 16; o; o >>= 1) lo2 = fminf(lo2, __shfl_xor_sync(0xffffffffu, lo2, o));
                if (lane == ol) {
#pragma unroll
                  for (int s2 = 0; s2 < KMAX; ++s2) {
                    l32[s2] = nl[s2];
                    i32[s2] = ni[s2];
                  }
                  rej = lo2;
                }
              }
              merged = true;
            }
          }
          if (!merged) {
            if (lane == ol) {
#pragma unroll
              for (int s2 = 0; s2 < KMAX; ++s2)
                if (s2 >= KMAX - K && top[s2] < top2[KMAX - 1]) insert_sorted<KMAX>(top2, top[s2]);
            }
            const uint64_t kth = warp_kth_of_lists<KMAX, uint64_t>(top2, K, INF_BITS);
            if (lane == ol) top[KMAX - 1] = kth;
          }
        }
      }
    }

    if (exists) {
      if constexpr (COUNT) J->cnt[J->idxg[qp]] = qok ? cntq : 0;
      else J->eps[J->idxg[qp]] = bits_to_double(top[KMAX - 1]);
    }
    if (lane == 0) atomicAdd(J->stats + 0, pairs);
  }
}

// d >= 3 (D != 2) runs on nested grids.
template <int D, int KMAX, bool PLAIN, bool COUNT>
void launch_wgrid_t(const JobDev* jobs, const WorkItem* items, int nitems, int* counter, int dmax,
                    int num_sms, cudaStream_t st) {
  auto kern = wgrid_kernel<D, KMAX, PLAIN, COUNT, D != 2>;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WG_WARPS * 32, 0);
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  const int need = (nitems + WG_WARPS - 1) / WG_WARPS;
  if (grid > need) grid = need;
  if (grid < 1) return;
  kern<<<grid, WG_WARPS * 32, 0, st>>>(jobs, items, nitems, counter, dmax);
  count_launch();
}

template <bool PLAIN>
struct WgridDispatch {
  template <int D>
  static void knn_d(int kclass, const JobDev* jobs, const WorkItem* items, int nitems, int* ctr,
                    int dmax, int sms, cudaStream_t st) {
    if (kclass <= 4) launch_wgrid_t<D, 4, PLAIN, false>(jobs, items, nitems, ctr, dmax, sms, st);
    else launch_wgrid_t<D, 8, PLAIN, false>(jobs, items, nitems, ctr, dmax, sms, st);
  }
  static void knn(int kclass, int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                  int* ctr, int dmax, int sms, cudaStream_t st) {
    switch (dclass) {
      case 2: knn_d<2>(kclass, jobs, items, nitems, ctr, dmax, sms, st); break;
      case 3: knn_d<3>(kclass, jobs, items, nitems, ctr, dmax, sms, st); break;
      case 4: knn_d<4>(kclass, jobs, items, nitems, ctr, dmax, sms, st); break;
      default: knn_d<0>(kclass, jobs, items, nitems, ctr, dmax, sms, st); break;
    }
  }
  static void count(int dclass, const JobDev* jobs, const WorkItem* items, int nitems, int* ctr,
                    int dmax, int sms, cudaStream_t st) {
    switch (dclass) {
      case 2: launch_wgrid_t<2, 4, PLAIN, true>(jobs, items, nitems, ctr, dmax, sms, st); break;
      case 3: launch_wgrid_t<3, 4, PLAIN, true>(jobs, items, nitems, ctr, dmax, sms, st); break;
      case 4: launch_wgrid_t<4, 4, PLAIN, true>(jobs, items, nitems, ctr, dmax, sms, st); break;
      default: launch_wgrid_t<0, 4, PLAIN, true>(jobs, items, nitems, ctr, dmax, sms, st); break;
    }
  }
};

}  // namespace wgrid_detail
}  // namespace egb
