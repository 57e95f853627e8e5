"""CPU port of the reference estimators on SciPy's cKDTree (CPU baseline).

TEST INFRASTRUCTURE ONLY.  Used by tests/ as a second, independent checker
and by bench.py as the reference CPU arm / cpu_baseline leg.  The product
package never imports it.

ennemi's estimators (ennemi/_entropy_estimators.py) are thin NumPy wrappers
around scipy.spatial.cKDTree, which holds the whole algorithm.  SciPy is a
third-party dependency that the reference does not vendor (setup.py:49 pins
scipy~=1.10; this image has scipy 1.18.1, and the GPU machine has SciPy as well),
so the faithful CPU implementation of the reference path is: the same tree
builds, the same ``query(.., k=[k+1], p=inf)`` for eps, the same
``query_ball_point(.., eps - 1e-12, p=inf, return_length=True)`` counts, and
the same digamma combination.  Those steps must be alike to measure the same
algorithm; the code around them is written for this project.

``sample_rate`` times a bounded sample: the trees are built over all N points
and only a subset of query points is searched and counted, spread over a
thread pool (cKDTree releases the GIL).  The per-point cost is scaled to the
full task to give estimates per second.
"""

from __future__ import annotations

import concurrent.futures
import os
import time
from typing import Callable, Dict, List, Tuple

import numpy as np
from scipy.spatial import cKDTree

from oracle.oracle import psi, RADIUS_SHRINK


def _cols(*arrs) -> np.ndarray:
    return np.column_stack(tuple(np.asarray(a, dtype=np.float64) for a in arrs))


def _eps(points: np.ndarray, k: int, queries: np.ndarray | None = None) -> np.ndarray:
    tree = cKDTree(points)
    q = points if queries is None else queries
    return tree.query(q, k=[k + 1], p=np.inf)[0].ravel()


def _count(points: np.ndarray, radius: np.ndarray, queries: np.ndarray | None = None) -> np.ndarray:
    tree = cKDTree(points)
    q = points if queries is None else queries
    return tree.query_ball_point(q, radius, p=np.inf, return_length=True)


def ksg_mi(x, y, k: int = 3) -> float:
    """As _estimate_single_mi (_entropy_estimators.py:69-113)."""
    xs, ys = _cols(x), _cols(y)
    r = _eps(_cols(xs, ys), k) - RADIUS_SHRINK
    return float(psi(len(xs)) + psi(k) - np.mean(psi(_count(xs, r)) + psi(_count(ys, r))))


def cmi(x, y, z, k: int = 3) -> float:
    """As _estimate_conditional_mi (_entropy_estimators.py:116-156)."""
    xs, ys, zs = _cols(x), _cols(y), _cols(z)
    r = _eps(_cols(xs, ys, zs), k) - RADIUS_SHRINK
    nxz = _count(_cols(xs, zs), r)
    nyz = _count(_cols(ys, zs), r)
    nz = _count(zs, r)
    return float(psi(k) - np.mean(psi(nxz) + psi(nyz) - psi(nz)))


def entropy(x, k: int = 3) -> float:
    """As _estimate_single_entropy (_entropy_estimators.py:21-42)."""
    xs = _cols(x)
    n, d = xs.shape
    with np.errstate(divide="ignore"):
        return float(psi(n) - psi(k) + d * (np.mean(np.log(_eps(xs, k))) + np.log(2)))


# --------------------------------------------------------------------------
# Bounded-sample timing (bench.py reference arm and cpu_baseline)
# --------------------------------------------------------------------------

def _ksg_point_kernel(xs, ys, k):
    """Trees over all N points; returns a function that processes query rows."""
    joint = _cols(xs, ys)
    tj, tx, ty = cKDTree(joint), cKDTree(_cols(xs)), cKDTree(_cols(ys))

    def run(idx: np.ndarray) -> float:
        r = tj.query(joint[idx], k=[k + 1], p=np.inf)[0].ravel() - RADIUS_SHRINK
        nx = tx.query_ball_point(_cols(xs[idx]), r, p=np.inf, return_length=True)
        ny = ty.query_ball_point(_cols(ys[idx]), r, p=np.inf, return_length=True)
        return float(np.sum(psi(nx) + psi(ny)))
    return run


def _cmi_point_kernel(xs, ys, zs, k):
    joint = _cols(xs, ys, zs)
    xz, yz, z = _cols(xs, zs), _cols(ys, zs), _cols(zs)
    tj, txz, tyz, tz = cKDTree(joint), cKDTree(xz), cKDTree(yz), cKDTree(z)

    def run(idx: np.ndarray) -> float:
        r = tj.query(joint[idx], k=[k + 1], p=np.inf)[0].ravel() - RADIUS_SHRINK
        a = txz.query_ball_point(xz[idx], r, p=np.inf, return_length=True)
        b = tyz.query_ball_point(yz[idx], r, p=np.inf, return_length=True)
        c = tz.query_ball_point(z[idx], r, p=np.inf, return_length=True)
        return float(np.sum(psi(a) + psi(b) - psi(c)))
    return run


def sample_rate(tasks: List[Tuple[str, tuple]], k: int, fraction: float,
                threads: int | None = None, seed: int = 0) -> Dict[str, float]:
    """Time the reference algorithm on a bounded sample of a batch of tasks.

    tasks: list of ("mi", (x, y)) or ("cmi", (x, y, z)) with float64 columns.
    For each task the trees are built over all N points (timed in full) and a
    random ``fraction`` of the query points is searched and counted on a
    thread pool of ``threads`` workers.  Returns the measured seconds and the
    extrapolated seconds for the whole batch (tree builds + queries / fraction).
    """
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    build_s = 0.0
    query_s = 0.0
    sampled = 0
    total = 0
    with concurrent.futures.ThreadPoolExecutor(threads) as pool:
        for kind, cols in tasks:
            n = len(cols[0])
            t0 = time.perf_counter()
            run: Callable[[np.ndarray], float]
            if kind == "mi":
                run = _ksg_point_kernel(cols[0], cols[1], k)
            elif kind == "cmi":
                run = _cmi_point_kernel(cols[0], cols[1], cols[2], k)
            else:
                raise ValueError(kind)
            t1 = time.perf_counter()
            m = max(threads, int(round(n * fraction)))
            idx = np.sort(rng.choice(n, size=min(m, n), replace=False))
            chunks = np.array_split(idx, threads)
            list(pool.map(run, chunks))
            t2 = time.perf_counter()
            build_s += t1 - t0
            query_s += t2 - t1
            sampled += len(idx)
            total += n
    frac = sampled / total
    return {"build_s": build_s, "query_s": query_s, "measured_s": build_s + query_s,
            "extrapolated_s": build_s + query_s / frac, "fraction": frac,
            "threads": threads, "points_sampled": sampled}
