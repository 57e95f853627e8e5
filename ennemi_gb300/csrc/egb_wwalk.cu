// egb_wwalk.cu -- kNN distances of warp-grid jobs by per-lane walks.
//
// (k+1)-th smallest max-norm distance per point, self included, over the
// job's grid copy (strips by column 1; nested cells by column 2 for d >= 3;
// column-0 order inside): cKDTree.query(k=[k+1], p=inf)
// (ennemi/_entropy_estimators.py:39, :108, :142, :194, :240).
//
// A warp takes an item of up to 32 consecutive positions of one strip
// (cell), one query per lane.  Every lane walks outward in column 0 from its
// own position -- always to the nearer of the next point on the left and on
// the right -- while that point's column-0 gap is within the lane's current
// screen bound.  Then the warp visits, together, the other cells of the
// strip outward in column 2 and the other strips outward in column 1, while
// some lane's planning bound reaches them; in each one, every lane that it
// reaches walks again from the binary-searched position of its query's
// column 0.  A lane thus screens only the points of its own neighbourhood,
// not the union window of 32 queries, while the control flow of the warp
// stays uniform outside the walks.
//
// Exactness as in egb_wgrid.cuh.  Pass 0 keeps the K smallest FP32 distances
// with their candidates and `rej`, the least FP32 distance of every visited
// candidate left out of the list.  With t32 the FP32 K-th, U = t32 + band
// and S = U + band (band proven in egb_internal.cuh):
//   * a walk stops a direction when the column-0 FP32 gap exceeds S, so every
//     unvisited point of a walked range has FP32 distance > S;
//   * a strip or cell is skipped when its column-1 / column-2 gap exceeds
//     plan_margin(U) on bounds rounded outward, so its points are farther
//     than U in FP64;
//   * if rej > S, every candidate outside the list is farther than U >= the
//     exact K-th, and the exact K-th is the largest exact distance of the K
//     listed candidates.
// Lanes without that margin (near ties, fewer than K candidates, jobs whose
// centred values reach 1e37) walk again with U fixed, deciding in FP64 every
// candidate with FP32 distance <= S.
#include "egb_wgrid.cuh"

namespace egb {
namespace {

using wgrid_detail::insert_sorted;
using wgrid_detail::insert_sorted_fi;
using wgrid_detail::plan_margin;
using wgrid_detail::up_band32;
using wgrid_detail::dn_band32;

constexpr int WW_WARPS = 4;
// A lane whose walks screen more candidates than this in pass 0 leaves its
// query to the cooperative phase (far-out queries of sparse regions).
constexpr int WALK_BUDGET = 192;

// First position of [a, b) with x[p] >= v (x ascending).
__device__ __forceinline__ int lower_bound_f(const float* __restrict__ x, int a, int b, float v) {
  int n = b - a;
  while (n > 0) {
    const int h = n >> 1;
    if (x[a + h] < v) {
      a += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return a;
}

// The same from a guessed position g in [a, b): gallop towards the answer,
// then bisect (exact for any g; a few steps when g is close).
__device__ __forceinline__ int lower_bound_from(const float* __restrict__ x, int a, int b, float v,
                                                int g) {
  if (b <= a) return a;
  g = g < a ? a : (g >= b ? b - 1 : g);
  int lo, hi;  // x[lo - 1] < v <= x[hi] (lo = a, hi = b when absent)
  if (x[g] < v) {
    lo = g + 1;
    int step = 1;
    for (;;) {
      const int t = g + step;
      if (t >= b) { hi = b; break; }
      if (!(x[t] < v)) { hi = t; break; }
      lo = t + 1;
      step <<= 1;
    }
  } else {
    hi = g;
    int step = 1;
    for (;;) {
      const int t = g - step;
      if (t < a) { lo = a; break; }
      if (x[t] < v) { lo = t + 1; break; }
      hi = t;
      step <<= 1;
    }
  }
  return lower_bound_f(x, lo, hi, v);
}

// Resident blocks per SM the register budget is cut for (measured: 2-D at
// six, 3-D with K <= 4 at five; the others keep what they need)
constexpr int walk_min_blocks(int D, int KMAX) { return D == 2 ? 6 : (D == 3 && KMAX == 4 ? 5 : 1); }

template <int D, int KMAX, bool NEST>
__global__ void __launch_bounds__(WW_WARPS * 32, walk_min_blocks(D, KMAX))
wwalk_kernel(const JobDev* __restrict__ jobs, const WorkItem* __restrict__ items, int nitems,
             int* __restrict__ counter) {
  constexpr int DQ = D ? D : EGB_DMAX;
  constexpr float FINF = __builtin_huge_valf();
  const int lane = threadIdx.x & 31;

  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const WorkItem wi = items[it];
    const JobDev* __restrict__ J = jobs + wi.job;
    const int d = D ? D : J->sp.d;
    const int64_t lds = J->lds;
    const double* __restrict__ c64 = J->c64g;
    const float* __restrict__ g = J->c32g;
    const int32_t* __restrict__ sst = J->sstart;
    const float* __restrict__ ylo = J->sylo32;
    const float* __restrict__ yhi = J->syhi32;
    const int S = J->nstrips;
    const int S2 = NEST ? J->nsub : 1;
    const int32_t* __restrict__ cst = J->cstart;
    const float* __restrict__ zlo = J->czlo32;
    const float* __restrict__ zhi = J->czhi32;
    const bool unsafe = (*J->jflags & TF_UNSAFE32) != 0u;
    const int K = J->K;
    const int sq = NEST ? (wi.strip & 0xffff) : wi.strip;
    const int hc2 = NEST ? (wi.strip >> 16) : 0;
    const int nq = wi.q1 - wi.q0;
    const int qp = wi.q0 + lane;
    const bool exists = qp < wi.q1;

    // qv = fl32(fl64(q - c)); for a job without clamped values
    // |fl32(fl64(v)) - v| <= 2^-22 |fl32(..)| + 2^-148 bounds v = q - c,
    // which gives M = max_c |q_c - c| and the planning bounds of columns 1
    // and 2 without FP64 instructions (jobs with clamped values run the FP64
    // pass, whose bounds are infinite)
    float qv[DQ];
    float am = 0.0f;
#pragma unroll
    for (int c = 0; c < DQ; ++c) {
      if (D == 0 && c >= d) break;
      qv[c] = exists ? g[(int64_t)c * lds + qp] : 0.0f;
      am = fmaxf(am, fabsf(qv[c]));
    }
    const float mq = __fmaf_ru(am, 1.0f + 0x1p-22f, 0x1p-148f);
    const float ey = __fmaf_ru(fabsf(qv[1]), 0x1p-22f, 0x1p-148f);
    const float qyl = __fsub_rd(qv[1], ey), qyh = __fadd_ru(qv[1], ey);
    float qzl = 0.0f, qzh = 0.0f;
    if (NEST) {
      const float ez = __fmaf_ru(fabsf(qv[2]), 0x1p-22f, 0x1p-148f);
      qzl = __fsub_rd(qv[2], ez);
      qzh = __fadd_ru(qv[2], ez);
    }
    // column-2 centre of the item: where the cells of other strips start
    const float zmid = NEST ? __shfl_sync(0xffffffffu, qv[NEST ? 2 : 0], (nq - 1) >> 1) : 0.0f;

    float l32[KMAX];     // pass 0: K smallest FP32 distances (padding first)
    int i32[KMAX];       // their candidates
    uint64_t top[KMAX];  // pass 1: K smallest exact distances (bit patterns)
#pragma unroll
    for (int s = 0; s < KMAX; ++s) {
      l32[s] = s >= KMAX - K ? FINF : 0.0f;
      i32[s] = 0;
      top[s] = s >= KMAX - K ? INF_BITS : 0ull;
    }
    float rej = FINF;      // least FP32 distance left out of the list
    bool pass1 = unsafe;   // jobs with clamped values decide everything in FP64
    float ufix = FINF, sfix = FINF;
    bool act = exists;     // this lane searches in the current pass
    bool heavy = false;    // pass 0 gave up: the warp finishes the query together
    unsigned long long visited = 0;

    auto exact_dist = [&](int j) -> uint64_t {
      uint64_t mm = 0;
#pragma unroll
      for (int c = 0; c < DQ; ++c) {
        if (D == 0 && c >= d) break;
        const int64_t off = (int64_t)c * lds;
        const uint64_t v = absdiff_bits(c64[off + j], c64[off + qp]);
        mm = v > mm ? v : mm;
      }
      return mm;
    };
    // screen bound S and planning bound plan_margin(U), kept current as the
    // list changes (refresh); the planning bound is -1 when inactive
    float sb_c = FINF, pb_c = FINF;
    auto refresh = [&]() {
      if (pass1) {
        sb_c = sfix;
        pb_c = plan_margin(ufix);
      } else {
        const float u = up_band32(l32[KMAX - 1], mq);
        sb_c = up_band32(u, mq);
        pb_c = plan_margin(u);
      }
    };
    refresh();
    auto sbound = [&]() -> float { return sb_c; };
    auto pbound = [&]() -> float { return act ? pb_c : -1.0f; };
    auto visit = [&](int j, float dd) {
      ++visited;
      if (!pass1) {
        if (dd < l32[KMAX - 1]) {
          rej = fminf(rej, insert_sorted_fi<KMAX>(l32, i32, dd, j));
          refresh();
        } else {
          rej = fminf(rej, dd);
        }
      } else if (dd <= sfix) {
        const uint64_t mm = exact_dist(j);
        if (mm < top[KMAX - 1]) insert_sorted<KMAX>(top, mm);
      }
    };
    // This lane's walk of [a, b) outward from p0 (the first position whose
    // column 0 is >= the query's): nearer side first, until both sides pass
    // S or end.
    auto walk = [&](int a, int b, int p0) {
      int L = p0 - 1, R = p0;
      float dl = L >= a ? qv[0] - g[L] : FINF;
      float dr = R < b ? g[R] - qv[0] : FINF;
      for (;;) {
        const bool go_l = dl <= dr;
        const float dx = go_l ? dl : dr;
        // both sides exhausted (real gaps are finite: values are clamped to
        // +-1e37), or the nearer side is beyond the screen bound
        if (!(dx < FINF) || !(dx <= sbound())) break;
        if (!pass1 && visited >= (unsigned long long)WALK_BUDGET) {
          heavy = true;  // leave it to the cooperative phase
          act = false;
          break;
        }
        const int j = go_l ? L : R;
        float dd = dx;
#pragma unroll
        for (int c = 1; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          dd = fmaxf(dd, fabsf(g[(int64_t)c * lds + j] - qv[c]));
        }
        visit(j, dd);
        if (go_l) {
          --L;
          dl = L >= a ? qv[0] - g[L] : FINF;
        } else {
          ++R;
          dr = R < b ? g[R] - qv[0] : FINF;
        }
      }
    };
    // the query's relative position in its own strip (cell): where to guess
    // its column 0 in another
    const int ha = NEST ? cst[sq * S2 + hc2] : sst[sq];
    const int hb = NEST ? cst[sq * S2 + hc2 + 1] : sst[sq + 1];
    const float frel = hb > ha ? (float)(qp - ha) / (float)(hb - ha) : 0.0f;
    auto walk_range = [&](int a, int b) {
      walk(a, b, lower_bound_from(g, a, b, qv[0], a + (int)(frel * (float)(b - a))));
    };
    // The warp visits strips and cells together; a lane walks the ones its
    // planning bound reaches.
    auto strip_reach = [&](int s, float t) {
      return act && !(__fsub_rd(ylo[s], qyh) > t) && !(__fsub_rd(qyl, yhi[s]) > t);
    };
    // Nested grids: the cells of strip s outward in column 2 from c0 (cell
    // `skip` already walked); each direction ends at the first cell no lane
    // reaches (cells are ordered by column 2).
    auto cells = [&](int s, int c0, int skip) {
      const int cb = s * S2;
      int up = c0, dn = c0 - 1;
      bool tu = true;
      for (;;) {
        const float t = pbound();
        const bool r = strip_reach(s, t);
        const bool ou = r && up < S2 && !(__fsub_rd(zlo[cb + up], qzh) > t);
        const bool od = r && dn >= 0 && !(__fsub_rd(qzl, zhi[cb + dn]) > t);
        const bool any_u = __any_sync(0xffffffffu, ou);
        const bool any_d = __any_sync(0xffffffffu, od);
        if (!any_u && !any_d) break;
        int c;
        if ((tu && any_u) || !any_d) {
          c = up++;
          tu = false;
        } else {
          c = dn--;
          tu = true;
        }
        if (c == skip) continue;
        const bool need = r && !(__fsub_rd(zlo[cb + c], qzh) > t) && !(__fsub_rd(qzl, zhi[cb + c]) > t);
        if (need) walk_range(cst[cb + c], cst[cb + c + 1]);
      }
    };
    auto start_cell = [&](int s) -> int {
      int c0 = 0;
      for (int b = 0; b < S2; b += 32) {
        const int c = b + lane;
        c0 += __popc(__ballot_sync(0xffffffffu, c < S2 && zhi[s * S2 + c] < zmid));
      }
      return c0 < S2 ? c0 : S2 - 1;
    };
    // the whole search of the current pass (warp-uniform)
    auto search = [&]() {
      if (NEST) {
        const int cb = sq * S2;
        if (act) walk(cst[cb + hc2], cst[cb + hc2 + 1], qp);
        cells(sq, hc2, hc2);
      } else {
        if (act) walk(sst[sq], sst[sq + 1], qp);
      }
      int up = sq + 1, dn = sq - 1;
      bool tu = true;
      for (;;) {
        const float t = pbound();
        const bool ou = act && up < S && !(__fsub_rd(ylo[up], qyh) > t);
        const bool od = act && dn >= 0 && !(__fsub_rd(qyl, yhi[dn]) > t);
        const bool any_u = __any_sync(0xffffffffu, ou);
        const bool any_d = __any_sync(0xffffffffu, od);
        if (!any_u && !any_d) break;
        int s;
        if ((tu && any_u) || !any_d) {
          s = up++;
          tu = false;
        } else {
          s = dn--;
          tu = true;
        }
        if (NEST) {
          cells(s, start_cell(s), -1);
        } else if (strip_reach(s, t)) {
          walk_range(sst[s], sst[s + 1]);
        }
      }
    };

    uint64_t kth = INF_BITS;
    bool again = false;
    if (!unsafe) {
      search();
      // Far-out queries, one at a time with all 32 lanes: a fresh search of
      // every strip and cell within the owner's current planning bound, each
      // lane screening every 32nd candidate of the column-0 windows into its
      // own list; the K smallest of the lists, with their candidates, become
      // the owner's list, and every entry not taken counts as left out.
      unsigned hm = __ballot_sync(0xffffffffu, heavy);
      while (hm) {
        const int ol = __ffs(hm) - 1;
        hm &= hm - 1u;
        float oq[DQ];
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
          if (D == 0 && c >= d) break;
          oq[c] = __shfl_sync(0xffffffffu, qv[c], ol);
        }
        const float omq = __shfl_sync(0xffffffffu, mq, ol);
        const float oyl = __shfl_sync(0xffffffffu, qyl, ol), oyh = __shfl_sync(0xffffffffu, qyh, ol);
        const float ozl = __shfl_sync(0xffffffffu, qzl, ol), ozh = __shfl_sync(0xffffffffu, qzh, ol);
        const float ek = __fmaf_ru(fabsf(oq[0]), 0x1p-22f, 0x1p-148f);
        const float oxl = __fsub_rd(oq[0], ek), oxh = __fadd_ru(oq[0], ek);
        float othr = __shfl_sync(0xffffffffu, l32[KMAX - 1], ol);  // caps every lane's list
        float tb = plan_margin(up_band32(othr, omq));
        float l2[KMAX];
        int ix2[KMAX];
#pragma unroll
        for (int s2 = 0; s2 < KMAX; ++s2) {
          l2[s2] = s2 >= KMAX - K ? FINF : 0.0f;
          ix2[s2] = 0;
        }
        float rej2 = FINF;
        unsigned long long cvis = 0;
        auto crange = [&](int a, int b) {
          int wl, wh;
          wgrid_detail::warp_window<float>(g, a, b, fminf(__fsub_rd(oxl, tb), 1e37f),
                                           fmaxf(__fadd_ru(oxh, tb), -1e37f), wl, wh);
          for (int j0 = wl; j0 < wh; j0 += 32) {
            const int j = j0 + lane;
            if (j < wh) {
              float dd = 0.0f;
#pragma unroll
              for (int c = 0; c < DQ; ++c) {
                if (D == 0 && c >= d) break;
                dd = fmaxf(dd, fabsf(g[(int64_t)c * lds + j] - oq[c]));
              }
              ++cvis;
              // <= : the owner's own K-th candidate lies exactly at the cap
              const bool hit = dd < l2[KMAX - 1] && dd <= othr;
              rej2 = fminf(rej2, hit ? insert_sorted_fi<KMAX>(l2, ix2, dd, j) : dd);
            }
          }
          // any lane holding K entries bounds the union's K-th
          float lk = l2[KMAX - 1];
#pragma unroll
          for (int o = 16; o; o >>= 1) lk = fminf(lk, __shfl_xor_sync(0xffffffffu, lk, o));
          if (lk < othr) othr = lk;
          const float nb = plan_margin(up_band32(othr, omq));
          if (nb < tb) tb = nb;
        };
        auto ccells = [&](int s) {  // nested: the cells of strip s within tb
          int c0 = 0, c1 = 0;
          for (int b = 0; b < S2; b += 32) {
            const int c = b + lane;
            c0 += __popc(__ballot_sync(0xffffffffu, c < S2 && __fsub_rd(ozl, zhi[s * S2 + c]) > tb));
            c1 += __popc(__ballot_sync(0xffffffffu, c < S2 && !(__fsub_rd(zlo[s * S2 + c], ozh) > tb)));
          }
          for (int c = c0; c < c1; ++c) crange(cst[s * S2 + c], cst[s * S2 + c + 1]);
        };
        auto cstrip = [&](int s) {
          if (NEST) ccells(s);
          else crange(sst[s], sst[s + 1]);
        };
        cstrip(sq);
        for (int up = sq + 1, dn = sq - 1;;) {
          const bool ou = up < S && !(__fsub_rd(ylo[up], oyh) > tb);
          const bool od = dn >= 0 && !(__fsub_rd(oyl, yhi[dn]) > tb);
          if (!ou && !od) break;
          const int s = ou && (!od || (up - sq) <= (sq - dn)) ? up++ : dn--;
          cstrip(s);
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
        {
          const int hp = KMAX - K + taken;
          float v = FINF;
#pragma unroll
          for (int s2 = 0; s2 < KMAX; ++s2)
            if (s2 == hp) v = l2[s2];
          float lo2 = fminf(rej2, v);
#pragma unroll
          for (int o = 16; o; o >>= 1) lo2 = fminf(lo2, __shfl_xor_sync(0xffffffffu, lo2, o));
          const unsigned long long cv = __reduce_add_sync(0xffffffffu, (unsigned)cvis);
          if (lane == ol) {
#pragma unroll
            for (int s2 = 0; s2 < KMAX; ++s2) {
              l32[s2] = nl[s2];
              i32[s2] = ni[s2];
            }
            rej = lo2;
            visited += cv;
            refresh();
          }
        }
      }
      if (exists) {
        const float u32 = up_band32(l32[KMAX - 1], mq);
        const float s32 = up_band32(u32, mq);
        if (rej > s32) {
          // every left-out candidate is farther than U >= the exact K-th,
          // which is the largest exact distance of the K listed ones; a
          // listed candidate whose FP32 upper bound does not exceed the last
          // one's FP32 lower bound cannot be larger, so usually only the
          // last is evaluated in FP64
          const float lo_last = dn_band32(l32[KMAX - 1], mq);
          uint64_t mx = 0;
#pragma unroll
          for (int s = 0; s < KMAX; ++s) {
            if (s >= KMAX - K && (s == KMAX - 1 || up_band32(l32[s], mq) > lo_last)) {
              const uint64_t e = exact_dist(i32[s]);
              mx = e > mx ? e : mx;
            }
          }
          kth = mx;
        } else {
          again = true;
          ufix = u32;
          sfix = s32;
        }
      }
      act = again;
      pass1 = true;
      refresh();
    } else {
      again = exists;
      act = exists;
    }
    if (__any_sync(0xffffffffu, act)) {
      search();  // pass 1 for the lanes without the margin
      if (again) kth = top[KMAX - 1];
    }
    if (exists) J->eps[J->idxg[qp]] = bits_to_double(kth);

    const unsigned long long tot = __reduce_add_sync(0xffffffffu, (unsigned)visited);
    const unsigned agm = __ballot_sync(0xffffffffu, again);
    if (lane == 0) {
      atomicAdd(J->stats + 0, tot);
      if (agm) atomicAdd(J->stats + 2, (unsigned long long)__popc(agm));
    }
  }
}

template <int D, int KMAX, bool NEST>
void launch_t(const JobDev* jobs, const WorkItem* items, int nitems, int* counter, int num_sms,
              cudaStream_t st) {
  auto kern = wwalk_kernel<D, KMAX, NEST>;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WW_WARPS * 32, 0);
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  const int need = (nitems + WW_WARPS - 1) / WW_WARPS;
  if (grid > need) grid = need;
  if (grid < 1) return;
  kern<<<grid, WW_WARPS * 32, 0, st>>>(jobs, items, nitems, counter);
  count_launch();
}

template <int KMAX>
void launch_k(int dclass, const JobDev* jobs, const WorkItem* items, int nitems, int* counter,
              int num_sms, cudaStream_t st) {
  switch (dclass) {
    case 2: launch_t<2, KMAX, false>(jobs, items, nitems, counter, num_sms, st); break;
    case 3: launch_t<3, KMAX, true>(jobs, items, nitems, counter, num_sms, st); break;
    case 4: launch_t<4, KMAX, true>(jobs, items, nitems, counter, num_sms, st); break;
    default: launch_t<0, KMAX, true>(jobs, items, nitems, counter, num_sms, st); break;
  }
}

}  // namespace

void launch_knn_walk(const JobDev* jobs_d, const WorkItem* items_d, int nitems, int kclass,
                     int dclass, int* counter, int num_sms, cudaStream_t st) {
  if (nitems <= 0) return;
  if (kclass <= 4) launch_k<4>(dclass, jobs_d, items_d, nitems, counter, num_sms, st);
  else launch_k<8>(dclass, jobs_d, items_d, nitems, counter, num_sms, st);
}

}  // namespace egb
