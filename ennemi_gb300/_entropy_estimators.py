"""The estimator functions, with the contracts of ennemi/_entropy_estimators.py.

Each nearest-neighbour estimator keeps the reference's name, argument order,
default ``k=3``, float return value, warnings and non-finite semantics, and
evaluates on the GPU through libennemi_gb.so (``_native.run_tasks``).  The
``*_task`` builders return the same work as a :class:`_native.Task` so that
the driver can evaluate many of them in one batched launch.

The discrete-only estimators (plug-in formulas over ``np.unique`` counts) are
not nearest-neighbour work; they are kept here in NumPy so that the module
offers the reference's full set of functions.
"""

from __future__ import annotations

from typing import Union
from warnings import warn

import numpy as np
import numpy.typing as npt

from . import _native
from ._native import Task

FloatArray = npt.NDArray[np.float64]
IntArray = npt.NDArray[np.int64]

MANY_CLASSES_WARNING = ("The discrete variable has relatively many unique values." +
                        " Did you pass y and x in correct order?")
NOT_CONTINUOUS_WARNING = ("A discrete variable has relatively many unique values." +
                          " Have you set marked the discrete variables in correct order?" +
                          " If both X and Y are discrete, the conditioning variable cannot be continuous" +
                          " (this limitation can be lifted in the future).")
OBJECT_DTYPE_MESSAGE = ("Data type 'object' is not supported." +
                        " Please pass only numeric, boolean, or string data." +
                        " If your data is in a pandas DataFrame, convert string categories" +
                        " to integers (pandas stores strings as objects).")


def _columns(a) -> list:
    """Columns of np.column_stack((a,)) as float64 (cKDTree works in float64)."""
    return _native.as_columns(np.asarray(a, dtype=np.float64))


# ---------------------------------------------------------------- builders --

def entropy_task(x, k: int = 3) -> Task:
    """Kozachenko-Leonenko entropy; _estimate_single_entropy (_entropy_estimators.py:21-42)."""
    cols = _columns(x)
    return Task(_native.ENTROPY, k, cols, n=len(cols[0]))


def mi_task(x, y, k: int = 3) -> Task:
    """KSG algorithm 1; _estimate_single_mi (_entropy_estimators.py:69-113)."""
    xc, yc = _columns(x), _columns(y)
    return Task(_native.MI, k, xc, yc, n=len(xc[0]))


def cmi_task(x, y, cond, k: int = 3) -> Task:
    """Frenzel-Pompe CMI; _estimate_conditional_mi (_entropy_estimators.py:116-156)."""
    xc, yc, zc = _columns(x), _columns(y), _columns(cond)
    return Task(_native.CMI, k, xc, yc, zc, n=len(xc[0]))


def semidiscrete_task(x, y, k: int = 3) -> Task:
    """Ross MI; _estimate_semidiscrete_mi (_entropy_estimators.py:159-200).

    Classes are np.unique(y) in sorted order, as in the reference (:177).
    """
    xc = _columns(x)
    n = len(xc[0])
    values, labels = np.unique(np.asarray(y), return_inverse=True)
    if len(values) > n / 4:
        warn(MANY_CLASSES_WARNING, UserWarning)
    return Task(_native.SEMI, k, xc, labels=np.ravel(labels).astype(np.int32),
                nclass=len(values), n=n)


def conditional_semidiscrete_task(x, y, cond, k: int = 3) -> Task:
    """_estimate_conditional_semidiscrete_mi (_entropy_estimators.py:203-247)."""
    y = np.asarray(y)
    n = len(y)
    xc, zc = _columns(x), _columns(cond)
    values, labels = np.unique(y, return_inverse=True)
    _verify_not_continuous(values, n)
    return Task(_native.CSEMI, k, xc, (), zc, labels=np.ravel(labels).astype(np.int32),
                nclass=len(values), n=n)


def _run_one(task: Task) -> float:
    return float(_native.run_tasks([task])[0])


# -------------------------------------------------------------- estimators --

def _estimate_single_entropy(x: FloatArray, k: int = 3) -> float:
    """Estimate the differential entropy of a d-dimensional variable (nats).

    Same contract as the reference: ``x`` is 1-D or (N x d); the result is
    psi(N) - psi(k) + d (mean(log eps) + log 2) with eps the (k+1)-th
    max-norm neighbour distance.  -inf when duplicates make some eps zero.
    """
    return _run_one(entropy_task(x, k))


def _estimate_single_mi(x: FloatArray, y: FloatArray, k: int = 3) -> float:
    """Mutual information between two continuous variables (nats), KSG-1.

    -inf when duplicate samples make some marginal count zero (the
    reference's _psi(0) = inf semantics).
    """
    return _run_one(mi_task(x, y, k))


def _estimate_conditional_mi(x: FloatArray, y: FloatArray, cond: FloatArray,
                             k: int = 3) -> float:
    """Conditional MI of continuous x, y given continuous cond (Frenzel-Pompe)."""
    return _run_one(cmi_task(x, y, cond, k))


def _estimate_semidiscrete_mi(x: FloatArray, y: FloatArray, k: int = 3) -> float:
    """MI between continuous x and discrete y (Ross 2014)."""
    return _run_one(semidiscrete_task(x, y, k))


def _estimate_conditional_semidiscrete_mi(x: FloatArray, y: FloatArray, cond: FloatArray,
                                          k: int = 3) -> float:
    """Conditional MI between continuous x and discrete y given continuous cond."""
    return _run_one(conditional_semidiscrete_task(x, y, cond, k))


def _verify_not_continuous(values, n: int) -> None:
    """Warning of _entropy_estimators.py:249-254 for too many discrete levels."""
    if len(values) > n / 4:
        warn(NOT_CONTINUOUS_WARNING, UserWarning)


# ------------------------------------------------------------- discrete --

def _assert_not_object(x) -> None:
    if np.asarray(x).dtype.kind == "O":
        raise TypeError(OBJECT_DTYPE_MESSAGE)


def _discrete_on_device(*arrays) -> bool:
    """Numeric data whose values float64 holds exactly goes to the device;
    strings, objects and integers beyond 2^53 keep NumPy's np.unique."""
    for a in arrays:
        a = np.asarray(a)
        if a.dtype.kind not in "biuf" or a.size == 0:
            return False
        if a.dtype.kind in "iu" and np.abs(a.astype(np.float64)).max() >= 2.0 ** 53:
            return False
    return True


def _float_columns(a) -> list:
    a = np.asarray(a)
    a = a.reshape(-1, 1) if a.ndim == 1 else a
    return [np.ascontiguousarray(a[:, c], dtype=np.float64) for c in range(a.shape[1])]


def discrete_entropy_task(x) -> Task:
    """_estimate_discrete_entropy as a device task (rows of x, any width)."""
    cols = _float_columns(x)
    return Task(_native.DISCRETE_ENTROPY, 1, cols, n=len(cols[0]))


def discrete_mi_task(x, y) -> Task:
    """_estimate_discrete_mi as a device task."""
    xs, ys = _float_columns(x), _float_columns(y)
    return Task(_native.DISCRETE_MI, 1, xs, ys, n=len(xs[0]))


def discrete_cmi_task(x, y, cond) -> Task:
    """_estimate_conditional_discrete_mi as a device task."""
    xs, ys, zs = _float_columns(x), _float_columns(y), _float_columns(cond)
    return Task(_native.DISCRETE_CMI, 1, xs, ys, zs, n=len(xs[0]))


def discrete_warnings(task: Task, groups) -> None:
    """The reference's warnings for a discrete task, from the device's
    distinct-value figures (_entropy_estimators.py:249-254, :280-281)."""
    n = task.n
    if task.kind == _native.DISCRETE_MI:
        for g in (groups[1], groups[2]):
            if g > n / 4:
                warn(NOT_CONTINUOUS_WARNING, UserWarning)
    elif task.kind == _native.DISCRETE_CMI:
        for _ in range(groups[4] + groups[5]):
            warn(NOT_CONTINUOUS_WARNING, UserWarning)


def _run_discrete(task: Task) -> float:
    groups = {}
    value = _native.run_tasks([task], groups_out=groups)[0]
    discrete_warnings(task, groups[0])
    return float(value)


def _estimate_discrete_entropy(x) -> float:
    """Plug-in entropy -sum p log p of the distinct rows of x (_entropy_estimators.py:44-56)."""
    x = np.asarray(x)
    _assert_not_object(x)
    if _discrete_on_device(x):
        return _run_discrete(discrete_entropy_task(x))
    _, counts = np.unique(x, axis=0, return_counts=True)
    p = counts / x.shape[0]
    return float(-np.sum(p * np.log(p)))


def _estimate_discrete_mi(x, y) -> float:
    """Plug-in MI of two discrete variables (_entropy_estimators.py:257-289)."""
    data = np.column_stack((x, y))
    _assert_not_object(data)
    if _discrete_on_device(x, y):
        return _run_discrete(discrete_mi_task(x, y))
    n = data.shape[0]
    _, xi, xc = np.unique(data[:, 0], return_inverse=True, return_counts=True)
    _, yi, yc = np.unique(data[:, 1], return_inverse=True, return_counts=True)
    _verify_not_continuous(xc, n)
    _verify_not_continuous(yc, n)
    xi, yi = np.ravel(xi), np.ravel(yi)
    joint = np.zeros((len(xc), len(yc)), dtype=np.int64)
    np.add.at(joint, (xi, yi), 1)
    a, b = np.nonzero(joint)
    j = joint[a, b].astype(np.float64)
    return float(np.sum(j * np.log(n * j / (xc[a] * yc[b]))) / n)


def _estimate_conditional_discrete_mi(x, y, cond) -> float:
    """Discrete CMI as the count-weighted MI within each condition level (:291-320)."""
    n = len(x)
    cond = np.asarray(cond)
    _assert_not_object(cond)
    if _discrete_on_device(x, y, cond):
        return _run_discrete(discrete_cmi_task(x, y, cond))
    _, inv, counts = np.unique(cond, axis=0, return_inverse=True, return_counts=True)
    inv = np.ravel(inv)
    x, y = np.asarray(x), np.asarray(y)
    total = 0.0
    for level in range(len(counts)):
        sel = inv == level
        total += counts[level] * _estimate_discrete_mi(x[sel], y[sel])
    return float(total / n)


# ----------------------------------------------------------------- digamma --

def _psi(x: Union[int, FloatArray, IntArray]) -> FloatArray:
    """Digamma of non-negative integers with the reference's conventions.

    psi(0) is +inf (a scalar, whatever the shape, so that it propagates through
    a mean), psi(1) is SciPy's constant, larger values use the asymptotic
    expansion of _entropy_estimators.py:341-348.
    """
    x = np.asarray(x)
    if np.any(x == 0):
        return np.asarray(np.inf)
    out = np.full(x.shape, -0.5772156649015331)
    big = x != 1
    v = np.asarray(x[big], dtype=np.float64)
    v2 = np.power(v, 2)
    out[big] = np.log(v) - np.power(v, -6) * (v2 * (v2 * (v / 2 + 1 / 12) - 1 / 120) + 1 / 252)
    return out
