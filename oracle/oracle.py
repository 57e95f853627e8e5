"""CPU oracle for the ennemi nearest-neighbour estimators.

TEST INFRASTRUCTURE ONLY.  This module is the checker the CUDA path is
compared against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` may import it; the product package
``ennemi_gb300`` never does.

The neighbour primitives come from ``nn_exact.c`` (plain-C brute force that
restates scipy cKDTree's max-norm k-NN and inclusive ball counts, loaded with
ctypes).  The estimator formulas are restated here in NumPy, each citing the
reference function it follows in ``ennemi/_entropy_estimators.py``.  Every
function returns the estimate and, for the parity tests, the internal arrays
(``eps`` and the neighbour counts).

Parity of this oracle with the live reference is pinned by
``tests/golden/*.npz`` (generated by ``tests/golden/make_golden.py`` from the
reference itself) in ``tests/test_oracle_golden.py``.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnn_exact.so")
_lib = None

# Same constant as the reference's radius shrink (_entropy_estimators.py:108-110,
# issue #76 there): counts use radius eps - 1e-12 with an inclusive test.
RADIUS_SHRINK = 1e-12


def build() -> str:
    """Compile nn_exact.c into _build/libnn_exact.so (gcc, OpenMP)."""
    script = os.path.join(_HERE, "build_oracle.sh")
    subprocess.run(["bash", script], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    dp = ctypes.POINTER(ctypes.c_double)
    lp = ctypes.POINTER(ctypes.c_int64)
    lib.orc_knn_eps.argtypes = [dp, ctypes.c_int64, dp, ctypes.c_int64,
                                ctypes.c_int, ctypes.c_int, dp]
    lib.orc_knn_eps.restype = ctypes.c_int
    lib.orc_ball_count.argtypes = [dp, ctypes.c_int64, dp, ctypes.c_int64,
                                   ctypes.c_int, dp, lp]
    lib.orc_ball_count.restype = ctypes.c_int
    lib.orc_num_threads.restype = ctypes.c_int
    _lib = lib
    return lib


def _rows(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    return np.ascontiguousarray(a)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def knn_eps(points: np.ndarray, k: int, queries: np.ndarray | None = None) -> np.ndarray:
    """(k+1)-th smallest max-norm distance, self included (cKDTree.query k=[k+1], p=inf)."""
    lib = _load()
    p = _rows(points)
    q = p if queries is None else _rows(queries)
    out = np.empty(q.shape[0], dtype=np.float64)
    rc = lib.orc_knn_eps(_dptr(q), q.shape[0], _dptr(p), p.shape[0], p.shape[1], int(k), _dptr(out))
    if rc != 0:
        raise RuntimeError(f"orc_knn_eps failed ({rc})")
    return out


def ball_count(points: np.ndarray, radius: np.ndarray, queries: np.ndarray | None = None) -> np.ndarray:
    """#{j : maxnorm(p_j - q_i) <= r_i} (cKDTree.query_ball_point p=inf, return_length)."""
    lib = _load()
    p = _rows(points)
    q = p if queries is None else _rows(queries)
    r = np.ascontiguousarray(radius, dtype=np.float64)
    out = np.empty(q.shape[0], dtype=np.int64)
    rc = lib.orc_ball_count(_dptr(q), q.shape[0], _dptr(p), p.shape[0], p.shape[1], _dptr(r),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc != 0:
        raise RuntimeError(f"orc_ball_count failed ({rc})")
    return out


def psi(x) -> np.ndarray:
    """Digamma of non-negative integers, restating ``_psi`` (_entropy_estimators.py:327-350).

    Same arithmetic as the reference so that every value is bit-identical on
    the same machine: any zero gives the scalar +inf; psi(1) is the SciPy
    constant; larger values use the asymptotic expansion in the same order
    of operations.
    """
    x = np.asarray(x)
    if np.any(x == 0):
        return np.asarray(np.inf)
    out = np.full(x.shape, -0.5772156649015331)
    big = x != 1
    y = np.asarray(x[big], dtype=np.float64)
    out[big] = np.log(y) - np.power(y, -6) * (np.power(y, 2) * (np.power(y, 2) * (y / 2 + 1 / 12) - 1 / 120) + 1 / 252)
    return out


def ksg_mi(x, y, k: int = 3) -> Tuple[float, Dict[str, np.ndarray]]:
    """KSG algorithm 1, following ``_estimate_single_mi`` (_entropy_estimators.py:69-113)."""
    xs, ys = _rows(x), _rows(y)
    n = xs.shape[0]
    joint = np.column_stack((xs, ys))
    eps = knn_eps(joint, k)
    r = eps - RADIUS_SHRINK
    nx = ball_count(xs, r)
    ny = ball_count(ys, r)
    value = psi(n) + psi(k) - np.mean(psi(nx) + psi(ny))
    return float(value), {"eps": eps, "nx": nx, "ny": ny}


def cmi(x, y, z, k: int = 3) -> Tuple[float, Dict[str, np.ndarray]]:
    """Frenzel-Pompe CMI, following ``_estimate_conditional_mi`` (_entropy_estimators.py:116-156)."""
    xs, ys, zs = _rows(x), _rows(y), _rows(z)
    joint = np.column_stack((xs, ys, zs))
    eps = knn_eps(joint, k)
    r = eps - RADIUS_SHRINK
    nxz = ball_count(np.column_stack((xs, zs)), r)
    nyz = ball_count(np.column_stack((ys, zs)), r)
    nz = ball_count(zs, r)
    value = psi(k) - np.mean(psi(nxz) + psi(nyz) - psi(nz))
    return float(value), {"eps": eps, "nxz": nxz, "nyz": nyz, "nz": nz}


def semidiscrete_mi(x, y, k: int = 3) -> Tuple[float, Dict[str, np.ndarray]]:
    """Ross MI, following ``_estimate_semidiscrete_mi`` (_entropy_estimators.py:159-200).

    The k-NN search runs inside each class of ``y``; the count runs over all
    points of ``x``.  eps is +inf for a class of k or fewer points, so every
    point of such a class counts all N points.
    """
    xs = _rows(x)
    n = xs.shape[0]
    y = np.asarray(y)
    values, counts = np.unique(y, return_counts=True)
    eps = np.empty(n)
    n_full = np.empty(n)
    for val in values:
        sel = y == val
        sub = xs[sel]
        e = knn_eps(sub, k)
        eps[sel] = e
        n_full[sel] = ball_count(xs, e - RADIUS_SHRINK, queries=sub)
    weighted = np.sum(np.dot(psi(counts), counts / n))
    value = psi(n) + psi(k) - np.mean(psi(n_full)) - weighted
    return float(value), {"eps": eps, "n": n_full.astype(np.int64)}


def conditional_semidiscrete_mi(x, y, z, k: int = 3) -> Tuple[float, Dict[str, np.ndarray]]:
    """Following ``_estimate_conditional_semidiscrete_mi`` (_entropy_estimators.py:203-247)."""
    xs, zs = _rows(x), _rows(z)
    n = len(y)
    y = np.asarray(y)
    xz = np.column_stack((xs, zs))
    eps = np.empty(n)
    nxz = np.empty(n)
    nyz = np.empty(n)
    nz = np.empty(n)
    for val in np.unique(y):
        sel = y == val
        e = knn_eps(xz[sel], k)
        eps[sel] = e
        r = e - RADIUS_SHRINK
        nxz[sel] = ball_count(xz, r, queries=xz[sel])
        nyz[sel] = ball_count(zs[sel], r)
        nz[sel] = ball_count(zs, r, queries=zs[sel])
    value = psi(k) - np.mean(psi(nxz) + psi(nyz) - psi(nz))
    return float(value), {"eps": eps, "nxz": nxz.astype(np.int64),
                          "nyz": nyz.astype(np.int64), "nz": nz.astype(np.int64)}


def entropy(x, k: int = 3) -> Tuple[float, Dict[str, np.ndarray]]:
    """Kozachenko-Leonenko, following ``_estimate_single_entropy`` (_entropy_estimators.py:21-42)."""
    xs = _rows(x)
    n, d = xs.shape
    eps = knn_eps(xs, k)
    with np.errstate(divide="ignore"):
        value = psi(n) - psi(k) + d * (np.mean(np.log(eps)) + np.log(2))
    return float(value), {"eps": eps}


# --------------------------------------------------------------- discrete --
# Plug-in estimators of discrete variables (_entropy_estimators.py:44-56,
# :257-320), restated with per-row counts of equal rows -- the quantities the
# device's group-by produces -- and the distinct-value figures behind the
# reference's warnings (:249-254).

def _row_counts(cols) -> Tuple[np.ndarray, int]:
    """Per row, the number of rows equal to it on `cols`; and the number of
    distinct rows."""
    a = np.column_stack([np.asarray(c, dtype=np.float64) + 0.0 for c in cols])  # -0 -> +0
    _, inv, cnt = np.unique(a, axis=0, return_inverse=True, return_counts=True)
    return cnt[np.ravel(inv)].astype(np.int64), len(cnt)


def discrete_entropy(x) -> Tuple[float, Dict[str, np.ndarray]]:
    """-sum p log p over the distinct rows of x (_entropy_estimators.py:44-56)."""
    cols = [x] if np.ndim(x) == 1 else list(np.asarray(x).T)
    c, g = _row_counts(cols)
    n = len(c)
    return float(-np.sum(np.log(c / n)) / n), {"c": c, "groups": np.array([g, 0, 0, 0, 0, 0])}


def discrete_mi(x, y) -> Tuple[float, Dict[str, np.ndarray]]:
    """sum over joint values of c log(N c / (cx cy)) / N (_entropy_estimators.py:257-289)."""
    cxy, gxy = _row_counts([x, y])
    cx, gx = _row_counts([x])
    cy, gy = _row_counts([y])
    n = len(cxy)
    v = float(np.sum(np.log((n * cxy).astype(np.float64) / (cx * cy).astype(np.float64))) / n)
    return v, {"cxy": cxy, "cx": cx, "cy": cy, "groups": np.array([gxy, gx, gy, 0, 0, 0])}


def conditional_discrete_mi(x, y, z) -> Tuple[float, Dict[str, np.ndarray]]:
    """Count-weighted discrete MI within each condition level
    (_entropy_estimators.py:291-320)."""
    zc = [z] if np.ndim(z) == 1 else list(np.asarray(z).T)
    cxyz, g0 = _row_counts([x, y] + zc)
    cxz, g1 = _row_counts([x] + zc)
    cyz, g2 = _row_counts([y] + zc)
    cz, g3 = _row_counts(zc)
    n = len(cz)
    v = float(np.sum(np.log((cz * cxyz).astype(np.float64) / (cxz * cyz).astype(np.float64))) / n)
    # levels with more than a quarter of their rows distinct in x (y)
    zrows = np.column_stack([np.asarray(c, dtype=np.float64) + 0.0 for c in zc])
    _, zinv, zcnt = np.unique(zrows, axis=0, return_inverse=True, return_counts=True)
    zinv = np.ravel(zinv)
    wx = wy = 0
    for level in range(len(zcnt)):
        sel = zinv == level
        wx += len(np.unique(np.asarray(x, dtype=np.float64)[sel] + 0.0)) > zcnt[level] / 4
        wy += len(np.unique(np.asarray(y, dtype=np.float64)[sel] + 0.0)) > zcnt[level] / 4
    return v, {"cxyz": cxyz, "cxz": cxz, "cyz": cyz, "cz": cz,
               "groups": np.array([g0, g1, g2, g3, wx, wy])}
