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

``SlicedBatch`` times a batch the way the reference's driver runs it: the
tasks go to a thread pool of ``max_threads`` workers (_driver.py:736-785;
cKDTree releases the GIL), one task per worker, each task single-threaded.
Each task builds its trees over all N points once; its query points are
then processed in ``nslices`` contiguous slices, one slice of every task per
step, so that the steps together search and count every query point exactly
once.  The time of the whole batch is the tree builds plus the sum of the
steps: a measurement, not an extrapolation.  ``sample_rate`` times a few
slices only and scales them to the batch (the bounded CPU baseline).
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
# Timing (bench.py reference arm and cpu_baseline)
# --------------------------------------------------------------------------

def _ksg_point_kernel(xs, ys, k):
    """Trees over all N points; returns a function that processes query rows."""
    joint = _cols(xs, ys)
    tj, tx, ty = cKDTree(joint), cKDTree(_cols(xs)), cKDTree(_cols(ys))
    xc, yc = _cols(xs), _cols(ys)

    def run(lo: int, hi: int) -> float:
        r = tj.query(joint[lo:hi], k=[k + 1], p=np.inf)[0].ravel() - RADIUS_SHRINK
        nx = tx.query_ball_point(xc[lo:hi], r, p=np.inf, return_length=True)
        ny = ty.query_ball_point(yc[lo:hi], r, p=np.inf, return_length=True)
        return float(np.sum(psi(nx) + psi(ny)))
    return run


def _cmi_point_kernel(xs, ys, zs, k):
    joint = _cols(xs, ys, zs)
    xz, yz, z = _cols(xs, zs), _cols(ys, zs), _cols(zs)
    tj, txz, tyz, tz = cKDTree(joint), cKDTree(xz), cKDTree(yz), cKDTree(z)

    def run(lo: int, hi: int) -> float:
        r = tj.query(joint[lo:hi], k=[k + 1], p=np.inf)[0].ravel() - RADIUS_SHRINK
        a = txz.query_ball_point(xz[lo:hi], r, p=np.inf, return_length=True)
        b = tyz.query_ball_point(yz[lo:hi], r, p=np.inf, return_length=True)
        c = tz.query_ball_point(z[lo:hi], r, p=np.inf, return_length=True)
        return float(np.sum(psi(a) + psi(b) - psi(c)))
    return run


def _builder(kind: str, cols, k: int):
    if kind == "mi":
        return lambda: _ksg_point_kernel(cols[0], cols[1], k)
    if kind == "cmi":
        return lambda: _cmi_point_kernel(cols[0], cols[1], cols[2], k)
    raise ValueError(kind)


class SlicedBatch:
    """A batch of ("mi", (x, y)) / ("cmi", (x, y, z)) tasks, timed in steps.

    ``build()`` builds every task's trees on the pool (one task per worker)
    and returns its wall time; ``step(s)`` processes query slice s of every
    task on the pool and returns its wall time.  ``task_seconds`` holds each
    task's own time (its thread's work), whose sum is what the reference's
    max_threads=1 path would take.
    """

    def __init__(self, tasks: List[Tuple[str, tuple]], k: int, nslices: int,
                 threads: int | None = None):
        self.tasks = tasks
        self.k = k
        self.nslices = nslices
        self.threads = threads or os.cpu_count() or 1
        self.pool = concurrent.futures.ThreadPoolExecutor(self.threads)
        self.runs: List[Callable[[int, int], float]] = []
        self.task_seconds = [0.0] * len(tasks)
        self.term_sums = [0.0] * len(tasks)

    def close(self):
        self.pool.shutdown()

    def _timed(self, t: int, fn):
        t0 = time.perf_counter()
        out = fn()
        self.task_seconds[t] += time.perf_counter() - t0
        return out

    def build(self) -> float:
        t0 = time.perf_counter()
        futs = [self.pool.submit(self._timed, t, _builder(kind, cols, self.k))
                for t, (kind, cols) in enumerate(self.tasks)]
        self.runs = [f.result() for f in futs]
        return time.perf_counter() - t0

    def step(self, s: int) -> float:
        t0 = time.perf_counter()
        futs = []
        for t, (kind, cols) in enumerate(self.tasks):
            n = len(cols[0])
            lo, hi = n * s // self.nslices, n * (s + 1) // self.nslices
            futs.append(self.pool.submit(self._timed, t, lambda r=self.runs[t], a=lo, b=hi: r(a, b)))
        for t, f in enumerate(futs):
            self.term_sums[t] += f.result()
        return time.perf_counter() - t0

    def estimates(self) -> List[float]:
        """The estimates once every slice has run (the reference's formulas)."""
        out = []
        for (kind, cols), ts in zip(self.tasks, self.term_sums):
            n = len(cols[0])
            if kind == "mi":
                out.append(float(psi(n) + psi(self.k) - ts / n))
            else:
                out.append(float(psi(self.k) - ts / n))
        return out


def sample_rate(tasks: List[Tuple[str, tuple]], k: int, slices: int, nslices: int,
                threads: int | None = None) -> Dict[str, float]:
    """Time the reference algorithm on a bounded sample of a batch: the tree
    builds in full and ``slices`` of ``nslices`` query slices of every task,
    tasks on a pool as the reference's driver runs them.  Returns the measured
    seconds and the batch time scaled from them (builds + mean step x nslices)."""
    b = SlicedBatch(tasks, k, nslices, threads)
    try:
        build_s = b.build()
        steps = [b.step(s) for s in range(slices)]
    finally:
        b.close()
    return {"build_s": build_s, "step_s": steps, "measured_s": build_s + sum(steps),
            "extrapolated_s": build_s + sum(steps) / len(steps) * nslices,
            "fraction": slices / nslices, "threads": b.threads}
