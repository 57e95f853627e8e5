"""Seeded synthetic workloads with the shapes of the large-sample benchmark
configurations (no dataset involved).  Used by bench.py and the tests.

plain_ksg(n)         one bivariate Gaussian, rho = .6 (the single estimate_mi case)
large_sample(n)      bivariate Gaussians rho in {0, .3, .6, .9} and a trivariate
                     Gaussian (corr(x,y) = .5, corr(x,z) = corr(y,z) = .4)
lagged_ar(length)    16 coupled AR(1) series (phi = .8, coupling .3 from the
                     previous series with a 5-step delay), a mask with ~10 %
                     false in runs of 1-50 samples; estimate_mi of series 0
                     against all 16 at lags 0..48 (784 estimates)
pairwise_mix(n)      64 columns: 16 correlated Gaussians, 16 sin(2x) + .3 noise,
                     16 Student-t(3), 16 log-normal; plus a 2-D Gaussian
                     condition (pairwise_mi: 2,016 pairs)
semidiscrete_mix(n)  x of dimension 1-4 from 3-component Gaussian mixtures,
                     discrete y with 2-50 classes of Dirichlet(.5) sizes; and
                     a 3-D Gaussian mixture for entropy
"""

from __future__ import annotations

import math

import numpy as np
from scipy.signal import lfilter

RHOS = (0.0, 0.3, 0.6, 0.9)
CMI_COV = [[1, 0.5, 0.4], [0.5, 1, 0.4], [0.4, 0.4, 1]]


def _cholesky(cov):
    """Lower Cholesky factor of a small covariance matrix, in Python floats
    (every operation a correctly rounded IEEE-754 one)."""
    d = len(cov)
    L = [[0.0] * d for _ in range(d)]
    for i in range(d):
        for j in range(i + 1):
            s = float(cov[i][j])
            for m in range(j):
                s -= L[i][m] * L[j][m]
            L[i][j] = math.sqrt(s) if i == j else s / L[j][j]
    return L


def gaussian(rng, cov, n: int):
    """n draws of N(0, cov) as a list of contiguous float64 columns.

    Column i is sum_j L[i][j] * z_j over j <= i, left to right, with z the
    generator's standard normals (n x d, row-major) and L the Cholesky factor
    of ``_cholesky``.  Only elementwise products and sums of NumPy arrays
    are used, each rounded once, so the columns are the same bits on every
    IEEE-754 platform (``multivariate_normal`` goes through a LAPACK
    factorisation and a BLAS product, whose last bits differ between x86-64
    and AArch64 builds).
    """
    L = _cholesky(cov)
    z = rng.standard_normal((n, len(cov)))
    cols = []
    for i in range(len(cov)):
        acc = None
        for j in range(i + 1):
            if L[i][j] == 0.0:
                continue
            term = L[i][j] * z[:, j]
            acc = term if acc is None else acc + term
        cols.append(np.ascontiguousarray(acc if acc is not None else np.zeros(n)))
    return cols


def plain_ksg(n: int = 10_000, seed: int = 0, rho: float = 0.6):
    """(x, y): the bivariate Gaussian of the single ``estimate_mi(y, x)`` case."""
    x, y = gaussian(np.random.default_rng(seed), [[1.0, rho], [rho, 1.0]], n)
    return x, y


def large_sample(n: int = 1_000_000, seed: int = 0):
    """[(kind, [columns])]: four 'mi' (x, y) tasks and one 'cmi' (x, y, z)."""
    rng = np.random.default_rng(seed)
    work = []
    for rho in RHOS:
        work.append(("mi", gaussian(rng, [[1.0, rho], [rho, 1.0]], n)))
    work.append(("cmi", gaussian(rng, CMI_COV, n)))
    return work


def lagged_ar(length: int = 200_000, nseries: int = 16, seed: int = 3):
    """(y, x, lags, mask) for estimate_mi(y, x, lags, mask=mask).

    x[:, i](t) = 0.8 x[:, i](t-1) + 0.3 x[:, i-1](t-5) + e_i(t) (series 0 has
    no coupling term), so every series is stationary; y is series 0.
    """
    rng = np.random.default_rng(seed)
    e = rng.normal(size=(length, nseries))
    x = np.empty((length, nseries))
    for i in range(nseries):
        drive = e[:, i].copy()
        if i > 0:
            drive[5:] += 0.3 * x[:-5, i - 1]
        x[:, i] = lfilter([1.0], [1.0, -0.8], drive)
    mask = np.ones(length, dtype=bool)
    target_false = int(0.1 * length)
    while (~mask).sum() < target_false:
        start = int(rng.integers(0, length))
        run = int(rng.integers(1, 51))
        mask[start:start + run] = False
    return x[:, 0].copy(), x, np.arange(49), mask


def with_nan_runs(x: np.ndarray, frac: float = 0.02, seed: int = 9) -> np.ndarray:
    """A copy of x (2-D) with runs of U{1..50} NaNs in every column, about
    `frac` of each column, at different places per column: with
    drop_nan=True every task of a lagged estimate_mi keeps its own rows, so
    the tasks of one call have different lengths."""
    rng = np.random.default_rng(seed)
    out = np.array(x, dtype=np.float64, copy=True)
    n = out.shape[0]
    for c in range(out.shape[1]):
        bad = np.zeros(n, dtype=bool)
        while bad.sum() < int(frac * n):
            start = int(rng.integers(0, n))
            bad[start:start + int(rng.integers(1, 51))] = True
        out[bad, c] = np.nan
    return out


def _random_corr(k: int, rng) -> np.ndarray:
    a = rng.normal(size=(k, k + 2))
    c = a @ a.T
    s = np.sqrt(np.diag(c))
    return c / s[:, None] / s[None, :]


def pairwise_mix(n: int = 50_000, seed: int = 4):
    """(data (n x 64), cond (n x 2))."""
    rng = np.random.default_rng(seed)
    g = rng.multivariate_normal(np.zeros(16), _random_corr(16, rng), size=n)
    base = rng.normal(size=(n, 16))
    s = np.sin(2 * base) + 0.3 * rng.normal(size=(n, 16))
    t = rng.standard_t(3, size=(n, 16))
    ln = np.exp(rng.normal(size=(n, 16)))
    data = np.column_stack((g, s, t, ln))
    cond = rng.multivariate_normal([0, 0], [[1, 0.3], [0.3, 1]], size=n)
    return data, cond


def _mixture(n: int, dim: int, rng) -> np.ndarray:
    comp = rng.integers(0, 3, size=n)
    out = np.empty((n, dim))
    for c in range(3):
        sel = comp == c
        mean = rng.normal(scale=2.0, size=dim)
        cov = _random_corr(dim, rng) * rng.uniform(0.5, 2.0)
        out[sel] = rng.multivariate_normal(mean, cov, size=int(sel.sum()))
    return out


def semidiscrete_mix(n: int = 500_000, seed: int = 5):
    """([(x (n x d), labels)] for d = 1..4 with 2, 10, 25, 50 classes; entropy x (n x 3))."""
    rng = np.random.default_rng(seed)
    cases = []
    for dim, ncls in zip((1, 2, 3, 4), (2, 10, 25, 50)):
        p = rng.dirichlet(np.full(ncls, 0.5))
        y = rng.choice(ncls, p=p, size=n)
        x = _mixture(n, dim, rng) + 0.5 * y[:, None] / ncls
        cases.append((x if dim > 1 else x[:, 0].copy(), y))
    ent = _mixture(n, 3, rng)
    return cases, ent
