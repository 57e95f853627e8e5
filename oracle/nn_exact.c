/*
 * nn_exact.c -- CPU oracle for the nearest-neighbour primitives of ennemi.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against; it is never linked into, loaded by or called from the
 * product library.  Only tests/, __graft_entry__.smoke() and the cpu_baseline
 * leg of bench.py may load it.
 *
 * What it restates.  ennemi's estimators (ennemi/_entropy_estimators.py) do all
 * of their neighbour arithmetic inside scipy.spatial.cKDTree (third-party,
 * not vendored in the reference; pinned scipy~=1.10 by setup.py:49, scipy
 * 1.18.1 installed here).  Two calls are used:
 *
 *   tree.query(pts, k=[k+1], p=inf)[0]      (_entropy_estimators.py:39, 108,
 *                                            142, 194, 240)
 *       -> for every point the (k+1)-th smallest max-norm distance to the
 *          points of the tree, the point itself included at distance 0;
 *          +inf when the tree holds fewer than k+1 points.
 *
 *   tree.query_ball_point(pts, r, p=inf, return_length=True)
 *                                           (_entropy_estimators.py:109-110,
 *                                            152-154, 196, 243-245)
 *       -> for every point the number of tree points j with
 *          max_d fl64(|p_jd - q_d|) <= r  (inclusive; 0 when r < 0).
 *
 * Distances are the IEEE-754 double max over dimensions of |a - b| with a - b
 * rounded to nearest; that is the value cKDTree returns bit for bit (pinned by
 * tests/golden, generated from the live reference).  This restatement is a
 * plain brute force: O(n^2) and exact, so it is only used at test sizes.
 *
 * Build: oracle/build_oracle.sh  ->  oracle/_build/libnn_exact.so
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* max-norm distance between row i and row j of a row-major (n x d) array */
static inline double maxnorm(const double *a, const double *b, int d) {
    double m = 0.0;
    for (int t = 0; t < d; ++t) {
        double v = fabs(a[t] - b[t]);
        if (v > m) m = v;
    }
    return m;
}

/* k-th smallest (0-based) of buf[0..n) by quickselect; buf is clobbered */
static double select_kth(double *buf, int64_t n, int64_t kth) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        double pivot = buf[lo + (hi - lo) / 2];
        int64_t i = lo, j = hi;
        while (i <= j) {
            while (buf[i] < pivot) ++i;
            while (buf[j] > pivot) --j;
            if (i <= j) {
                double t = buf[i]; buf[i] = buf[j]; buf[j] = t;
                ++i; --j;
            }
        }
        if (kth <= j) hi = j;
        else if (kth >= i) lo = i;
        else return buf[kth];
    }
    return buf[kth];
}

/*
 * eps[i] = (k+1)-th smallest max-norm distance from query i to the n
 * reference points (query included when it is one of them).
 * queries: (nq x d) row-major, points: (n x d) row-major.
 * Mirrors cKDTree.query(.., k=[k+1], p=inf)[0].
 */
int orc_knn_eps(const double *queries, int64_t nq, const double *points,
                int64_t n, int d, int k, double *eps) {
    if (d <= 0 || k <= 0 || nq < 0 || n < 0) return -1;
    if ((int64_t)k + 1 > n) {
        for (int64_t i = 0; i < nq; ++i) eps[i] = INFINITY;
        return 0;
    }
    int bad = 0;
#pragma omp parallel
    {
        double *buf = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        if (!buf) {
#pragma omp atomic write
            bad = 1;
        } else {
#pragma omp for schedule(dynamic, 16)
            for (int64_t i = 0; i < nq; ++i) {
                const double *q = queries + i * d;
                for (int64_t j = 0; j < n; ++j) buf[j] = maxnorm(points + j * d, q, d);
                eps[i] = select_kth(buf, n, k);
            }
            free(buf);
        }
    }
    return bad ? -2 : 0;
}

/*
 * count[i] = #{ j : maxnorm(points_j - queries_i) <= r[i] }.
 * Mirrors cKDTree.query_ball_point(queries, r, p=inf, return_length=True).
 */
int orc_ball_count(const double *queries, int64_t nq, const double *points,
                   int64_t n, int d, const double *r, int64_t *count) {
    if (d <= 0 || nq < 0 || n < 0) return -1;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < nq; ++i) {
        const double *q = queries + i * d;
        const double ri = r[i];
        int64_t c = 0;
        if (ri >= 0.0) {
            for (int64_t j = 0; j < n; ++j) c += (maxnorm(points + j * d, q, d) <= ri);
        }
        count[i] = c;
    }
    return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
