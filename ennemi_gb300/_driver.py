"""Public API with the signatures and behaviour of ennemi/_driver.py.

What differs is how the work runs.  The reference hands every (lag, variable)
or (i, j) task to a thread pool, each task building its own cKDTrees
(_driver.py:736-785).  Here every call collects its tasks first -- lagging,
masking, validation and rescaling stay on the host in NumPy, so the inputs
are bit-identical to the reference's -- and then evaluates all of them in one
batched GPU launch sequence (``_native.run_tasks``).  Callbacks fire after
that batch, once per task, in task order.  ``max_threads`` bounds the host
thread pool that prepares the tasks (slicing, masking, rescaling; default
min(16, cpu_count)); the GPU work is one batch whatever its value.  Within a
call, columns shared by several tasks (y, the condition, every column of
pairwise_mi) are prepared once and uploaded once.

Errors and warnings are those of the reference, raised at the same points.
"""

from __future__ import annotations

import os
import sys
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import Callable, List, Optional, Sequence, Tuple, TypeVar, Union
from warnings import warn

import numpy as np
import numpy.typing as npt

from . import _native
from ._entropy_estimators import (
    _assert_not_object, _discrete_on_device, _estimate_conditional_discrete_mi,
    _estimate_discrete_entropy, _estimate_discrete_mi, cmi_task, conditional_semidiscrete_task,
    discrete_cmi_task, discrete_entropy_task, discrete_mi_task, discrete_warnings, entropy_task,
    mi_task, semidiscrete_task)

FloatArray = npt.NDArray[np.float64]
ArrayLike = npt.ArrayLike
GenArrayLike = TypeVar("GenArrayLike", Sequence[float], Sequence[Sequence[float]], FloatArray)

DISCRETE_NORMALIZATION_WARNING = \
    "You have set normalize=True while at least one variable is discrete. " +\
    "The correlation coefficient formula assumes both variables to be continuous, " +\
    "and the results are not comparable across different discrete variables. " +\
    "Compare the raw MI against entropy of the discrete variable instead. " +\
    "If you really want to calculate correlation coefficients, you can suppress " +\
    "this warning by setting normalize=False and calling normalize_mi() on the results."

PREPROCESS_CONSTANT_DATA_WARNING = \
    "A variable not marked as discrete takes only a single value, " +\
    "or values in a very small numerical range. " +\
    "If this is intentional, you can suppress this warning by passing preprocess=False. " +\
    "Note that this disables rescaling on all other variables as well."

NAN_MSG = "input contains NaNs (after applying the mask), pass drop_nan=True to ignore"
K_TOO_LARGE_MSG = "k must be smaller than number of observations (after lag and mask)"
MIXED_COND_MSG = ("Conditioning is not supported with mixed discrete and continuous data. " +
                  "This is a limitation that can be lifted in the future (see " +
                  "https://github.com/polsys/ennemi/issues/87).")

# Seed of the preprocessing noise: digits of e, as in _driver.py:874.
NOISE_SEED = 2_718281828
NOISE_SCALE = 1e-10


# --------------------------------------------------------------- batching --

# Extra egb_run_batch flags for every batch of the public API, e.g.
# _native.PLAIN_FP64 for the all-FP64 comparator or _native.GRAPH to replay
# repeated batches from a CUDA graph.  No flag changes a result.
run_flags = 0


class _Batch:
    """Collects estimator tasks and host-side values; evaluates all GPU work
    in one call and hands back the values in submission order."""

    def __init__(self):
        self.tasks: List[_native.Task] = []
        self.slots: List[Tuple[str, object]] = []

    def add_task(self, task: _native.Task) -> int:
        self.slots.append(("gpu", len(self.tasks)))
        self.tasks.append(task)
        return len(self.slots) - 1

    def add_value(self, value: float) -> int:
        self.slots.append(("host", float(value)))
        return len(self.slots) - 1

    def run(self) -> np.ndarray:
        groups = {}
        gpu = _native.run_tasks(self.tasks, flags=run_flags, groups_out=groups) if self.tasks \
            else np.empty(0)
        for i in sorted(groups):   # the discrete estimators' warnings
            discrete_warnings(self.tasks[i], groups[i])
        out = np.empty(len(self.slots))
        for i, (kind, v) in enumerate(self.slots):
            out[i] = gpu[v] if kind == "gpu" else v
        return out


class _NoiseStream:
    """Standard normals of default_rng(NOISE_SEED), cached and grown on demand.

    The reference draws rng.normal(0, 1e-10, shape) from a fresh generator for
    each task, in the order x, y, z (_driver.py:874-900).  Consecutive draws
    of one generator are consecutive slices of the same stream, and
    normal(0, s) is 0 + s * standard_normal, so slicing this cache gives the
    same doubles bit for bit.
    """

    def __init__(self):
        self._s = np.empty(0)
        self._lock = threading.Lock()

    def take(self, start: int, shape) -> np.ndarray:
        """0 + NOISE_SCALE * z[start : start + prod(shape)] (a read-only view)."""
        count = int(np.prod(shape))
        with self._lock:
            if self._s.size < start + count:
                size = max(start + count, 2 * self._s.size)
                s = 0.0 + NOISE_SCALE * np.random.default_rng(NOISE_SEED).standard_normal(size)
                s.flags.writeable = False
                self._s = s
            s = self._s
        return s[start:start + count].reshape(shape)


_noise = _NoiseStream()


# ------------------------------------------------------------ normalise --

def normalize_mi(mi: Union[float, GenArrayLike]) -> GenArrayLike:
    """Normalize mutual information values to the unit interval.

    Equivalent to passing `normalize=True` to the estimation methods: the
    result is sqrt(1 - exp(-2 MI)), the correlation coefficient of a Gaussian
    pair with that MI.  Non-positive values are returned unchanged.  Pandas
    `DataFrame`/`Series` inputs keep their columns and indices.
    """
    if "pandas" in sys.modules:
        import pandas
        if isinstance(mi, (pandas.DataFrame, pandas.Series)):
            return mi.map(_normalize)
    arr = np.asarray(mi)
    if arr.dtype.kind not in "biuf":   # the reference's error for anything else
        return np.vectorize(_normalize, otypes=[float])(mi)
    return _native.normalize(arr)      # sqrt(1 - exp(-2 mi)) on the device


def _normalize(mi: float) -> float:
    if mi <= 0.0:
        return mi
    return np.sqrt(1 - np.exp(-2 * mi))


# -------------------------------------------------------------- entropy --

def estimate_entropy(x: ArrayLike,
                     *, k: int = 3,
                     multidim: bool = False,
                     discrete: bool = False,
                     mask: Optional[ArrayLike] = None,
                     cond: Optional[ArrayLike] = None,
                     drop_nan: bool = False) -> FloatArray:
    """Estimate the entropy of one or more continuous random variables (nats).

    Same parameters and results as ennemi.estimate_entropy (_driver.py:84-162):
    each column of a 2-D `x` separately, or all columns as one variable with
    `multidim=True`; `mask` selects observations; `cond` gives the conditional
    entropy H(X|Y) = H(X,Y) - H(Y); `discrete=True` uses the plug-in formula;
    `drop_nan=True` drops rows with NaNs.  All continuous estimates of the call
    run in one batched GPU launch.
    """
    x_arr = np.asarray(x)
    if mask is not None:
        mask = np.asarray(mask)
        _validate_mask(mask, x_arr.shape[0])
    if not 1 <= x_arr.ndim <= 2:
        raise ValueError("x must be one- or two-dimensional")
    _validate_k_type(k)

    if cond is None:
        result = _estimate_entropy(x_arr, k, multidim, mask, discrete, drop_nan)
    else:
        cond_arr = np.asarray(cond)
        _validate_cond(cond_arr, x_arr.shape[0])
        result = _estimate_conditional_entropy(x_arr, cond_arr, k, multidim, mask, discrete, drop_nan)

    if not multidim and "pandas" in sys.modules:
        import pandas
        if isinstance(x, pandas.DataFrame):
            return pandas.DataFrame(np.atleast_2d(result), columns=x.columns)
        elif isinstance(x, pandas.Series):
            return pandas.DataFrame(np.atleast_2d(result), columns=[x.name])
    return result


def _entropy_slots(batch: _Batch, x: FloatArray, k: int, multidim: bool,
                   mask, discrete: bool, drop_nan: bool) -> List[int]:
    if multidim or x.ndim == 1:
        xs = _mask_and_validate_entropy(x, mask, drop_nan, discrete, k)
        return [_entropy_slot(batch, xs, k, discrete)]
    return [_entropy_slot(batch, _mask_and_validate_entropy(x[:, i], mask, drop_nan, discrete, k),
                          k, discrete) for i in range(x.shape[1])]


def _estimate_entropy(x: FloatArray, k: int, multidim: bool,
                      mask, discrete: bool, drop_nan: bool) -> FloatArray:
    batch = _Batch()
    slots = _entropy_slots(batch, x, k, multidim, mask, discrete, drop_nan)
    values = batch.run()
    if multidim or x.ndim == 1:
        return np.asarray(values[slots[0]])
    return values[slots]


def _mask_and_validate_entropy(x: FloatArray, mask, drop_nan: bool, discrete: bool,
                               k: int) -> FloatArray:
    if mask is not None:
        x = x[np.asanyarray(mask)]
    if drop_nan and not discrete:
        x = x[~np.max(np.isnan(x), axis=1)] if x.ndim > 1 else x[~np.isnan(x)]
    if k >= x.shape[0]:
        raise ValueError(K_TOO_LARGE_MSG)
    if not discrete and np.any(np.isnan(x)):
        raise ValueError(NAN_MSG)
    return x


def _entropy_slot(batch: _Batch, xs: FloatArray, k: int, discrete: bool) -> int:
    if discrete:
        if _discrete_on_device(xs):
            return batch.add_task(discrete_entropy_task(xs))
        return batch.add_value(_estimate_discrete_entropy(xs))
    return batch.add_task(entropy_task(xs, k))


def _estimate_conditional_entropy(x: FloatArray, cond: FloatArray, k: int, multidim: bool,
                                  mask, discrete: bool, drop_nan: bool) -> FloatArray:
    """H(X|Y) = H(X,Y) - H(Y), both terms in the same batch (_driver.py:202-220)."""
    batch = _Batch()
    marginal = _entropy_slots(batch, cond, k, True, mask, discrete, drop_nan)[0]
    if multidim or x.ndim == 1:
        xs = _mask_and_validate_entropy(np.column_stack((x, cond)), mask, drop_nan, discrete, k)
        joint = [_entropy_slot(batch, xs, k, discrete)]
    else:
        joint = []
        for i in range(x.shape[1]):
            xs = _mask_and_validate_entropy(np.column_stack((x[:, i], cond)), mask, drop_nan,
                                            discrete, k)
            joint.append(_entropy_slot(batch, xs, k, discrete))
    values = batch.run()
    if multidim or x.ndim == 1:
        return np.asarray(values[joint[0]] - values[marginal])
    return values[joint] - values[marginal]


# ------------------------------------------------------------------- MI --

def estimate_mi(y: ArrayLike, x: ArrayLike,
                lag: Union[Sequence[int], ArrayLike, int] = 0,
                *, k: int = 3,
                cond: Optional[ArrayLike] = None,
                cond_lag: Union[Sequence[int], Sequence[Sequence[int]], ArrayLike, int] = 0,
                mask: Optional[ArrayLike] = None,
                discrete_y: bool = False,
                discrete_x: bool = False,
                preprocess: bool = True,
                drop_nan: bool = False,
                normalize: bool = False,
                max_threads: Optional[int] = None,
                callback: Optional[Callable[[int, int], None]] = None) -> FloatArray:
    """Estimate the mutual information between y and each x variable (nats).

    Same parameters and result as ennemi.estimate_mi (_driver.py:229-360): a
    (len(lag), n_x) array; lags follow y(t) ~ x(t - lag) | z(t - cond_lag);
    `cond` selects conditional MI, `discrete_y` / `discrete_x` the Ross
    estimators, `preprocess` the unit-variance rescaling with fixed-seed
    1e-10 noise, `normalize` the correlation scale.  Every (lag, variable)
    task of the call runs in one batched GPU launch; `callback(var, lag)`
    fires once per task after it.  `max_threads` bounds the host preparation threads.
    """
    x_arr = np.asarray(x)
    y_arr = np.asarray(y)
    if cond is not None:
        cond_arr = np.column_stack((np.asarray(cond),))
        ncond = cond_arr.shape[1]
    else:
        cond_arr = None
        ncond = 1
    mask_arr = None if mask is None else np.asarray(mask)

    lag_arr = np.atleast_1d(lag)
    cond_lag_arr = np.broadcast_to(np.column_stack((cond_lag,)), (lag_arr.shape[0], ncond))

    result = _estimate_mi(y_arr, x_arr, lag_arr, k, cond_arr, cond_lag_arr, mask_arr,
                          discrete_x, discrete_y, preprocess, drop_nan, max_threads, callback)

    if normalize:
        if discrete_x or discrete_y:
            warn(DISCRETE_NORMALIZATION_WARNING)
        result = normalize_mi(result)

    if "pandas" in sys.modules:
        import pandas
        if isinstance(x, pandas.DataFrame):
            return pandas.DataFrame(result, index=lag_arr, columns=x.columns)
        elif isinstance(x, pandas.Series):
            return pandas.DataFrame(result, index=lag_arr, columns=[x.name])
    return result


def estimate_corr(y: ArrayLike, x: ArrayLike,
                  lag: Union[Sequence[int], ArrayLike, int] = 0,
                  *, k: int = 3,
                  cond: Optional[ArrayLike] = None,
                  cond_lag: Union[Sequence[int], Sequence[Sequence[int]], ArrayLike, int] = 0,
                  mask: Optional[ArrayLike] = None,
                  preprocess: bool = True,
                  drop_nan: bool = False,
                  max_threads: Optional[int] = None,
                  callback: Optional[Callable[[int, int], None]] = None) -> FloatArray:
    """MI correlation between continuous variables: estimate_mi(..., normalize=True)."""
    return estimate_mi(y, x, lag, k=k, cond=cond, cond_lag=cond_lag, mask=mask,
                       preprocess=preprocess, drop_nan=drop_nan, normalize=True,
                       max_threads=max_threads, callback=callback)


def _estimate_mi(y: FloatArray, x: FloatArray, lag: FloatArray, k: int,
                 cond: Optional[FloatArray], cond_lag: FloatArray,
                 mask: Optional[FloatArray], discrete_x: bool, discrete_y: bool,
                 preprocess: bool, drop_nan: bool, max_threads: Optional[int],
                 callback: Optional[Callable[[int, int], None]]) -> FloatArray:
    _check_parameters(x, y, k, cond, mask)
    min_lag = min(np.min(lag), np.min(cond_lag))
    max_lag = max(np.max(lag), np.max(cond_lag))
    if max_lag - min_lag >= y.size or max_lag >= y.size or min_lag <= -y.size:
        raise ValueError("lag is too large, no observations left")

    nvar = 1 if x.ndim == 1 else x.shape[1]
    indices = [(li, vi) for li in range(len(lag)) for vi in range(nvar)]
    prep = _Prep(mask, min_lag, max_lag)
    jobs = []
    for li, vi in indices:
        xv = x if x.ndim == 1 else x[:, vi]
        jobs.append(_task_job(prep, ("x", vi), xv, ("y",), y, lag[li], max_lag, min_lag, k, mask,
                              cond, cond_lag[li], discrete_x, discrete_y, preprocess, drop_nan,
                              share_x=False))
    if _device_prep_ok((x, y) + (() if cond is None else (cond,)), cond, preprocess, drop_nan,
                       discrete_x or discrete_y, nan_rows_ok=True):
        lo, hi = min(min_lag, 0), max(max_lag, 0)
        n = len(y) - hi + lo if prep.idx is None else len(prep.idx)
        specs = []
        ycol = _native.Col(y[hi:])
        zcols = {}   # condition columns by lag: shared by the tasks of a lag row
        for li, vi in indices:
            xv = x if x.ndim == 1 else x[:, vi]
            zv = None
            if cond is not None:
                zkey = tuple(int(c) for c in cond_lag[li])
                zv = zcols.get(zkey)
                if zv is None:
                    zv = zcols[zkey] = [_native.Col(cond[hi - cond_lag[li][c]:, c])
                                        for c in range(cond.shape[1])]
            specs.append((_native.Col(xv[hi - lag[li]:]), ycol, zv))
        rows = None
        if drop_nan:
            rows = _kept_rows(x, y, cond, lag, cond_lag, indices, hi, len(y) - hi + lo, prep.idx,
                              max_threads)
        values = _run_device_prep(specs, n, k, prep.idx, jobs, max_threads, rows)
    else:
        batch = _Batch()
        slots = [_add_prepared(batch, p) for p in _prepare_all(jobs, max_threads)]
        values = batch.run()[slots]
    result = np.empty((len(lag), nvar))
    for (li, vi), v in zip(indices, values):
        result[li, vi] = v
        if callback is not None:
            callback(vi, lag[li])
    return result


def _check_parameters(x: FloatArray, y: Optional[FloatArray], k: int,
                      cond: Optional[FloatArray], mask: Optional[FloatArray]) -> None:
    _validate_k_type(k)
    if not 1 <= len(x.shape) <= 2:
        raise ValueError("x must be one- or two-dimensional")
    if y is not None:
        if len(y.shape) > 1:
            raise ValueError("y must be one-dimensional")
        if x.shape[0] != y.shape[0]:
            raise ValueError("x and y must have same length")
    if mask is not None:
        _validate_mask(mask, x.shape[0])
    if cond is not None:
        _validate_cond(cond, x.shape[0])


def _validate_k_type(k: int) -> None:
    if not isinstance(k, int):
        raise TypeError("k must be int")
    if k <= 0:
        raise ValueError("k must be greater than zero")


def _validate_mask(mask: FloatArray, input_len: int) -> None:
    if len(mask.shape) > 1:
        raise ValueError("mask must be one-dimensional")
    if len(mask) != input_len:
        raise ValueError("mask length does not match input length")
    if mask.dtype != bool:
        raise TypeError("mask must contain only booleans")


def _validate_cond(cond: FloatArray, input_len: int) -> None:
    if not 1 <= cond.ndim <= 2:
        raise ValueError("cond must be one- or two-dimensional")
    if input_len != len(cond):
        raise ValueError("x and cond must have same length")


# ------------------------------------------------------------- pairwise --

def pairwise_mi(data: ArrayLike,
                *, k: int = 3,
                cond: Optional[ArrayLike] = None,
                mask: Optional[ArrayLike] = None,
                discrete: ArrayLike = False,
                preprocess: bool = True,
                drop_nan: bool = False,
                normalize: bool = False,
                max_threads: Optional[int] = None,
                callback: Optional[Callable[[int, int], None]] = None) -> FloatArray:
    """Pairwise MI between the columns of `data` (nats); NaN diagonal.

    Same parameters and result as ennemi.pairwise_mi (_driver.py:540-623).
    All i < j pairs run in one batched GPU launch; `callback(i, j)` fires once
    per pair after it.  `max_threads` bounds the host preparation threads.
    """
    data_arr = np.asarray(data)
    cond_arr = None if cond is None else np.column_stack((np.asarray(cond),))
    mask_arr = None if mask is None else np.asarray(mask)

    if data_arr.ndim == 1 or data_arr.shape[1] == 1:
        return np.full((1, 1), np.nan)

    discrete_arr = np.broadcast_to(discrete, data_arr.shape[1])
    result = _pairwise_mi(data_arr, k, cond_arr, preprocess, drop_nan, mask_arr, discrete_arr,
                          max_threads, callback)

    if normalize:
        if discrete_arr.any():
            warn(DISCRETE_NORMALIZATION_WARNING)
        result = normalize_mi(result)

    if "pandas" in sys.modules:
        import pandas
        if isinstance(data, pandas.DataFrame):
            return pandas.DataFrame(result, index=data.columns, columns=data.columns)
    return result


def pairwise_corr(data: ArrayLike,
                  *, k: int = 3,
                  cond: Optional[ArrayLike] = None,
                  mask: Optional[ArrayLike] = None,
                  preprocess: bool = True,
                  drop_nan: bool = False,
                  max_threads: Optional[int] = None,
                  callback: Optional[Callable[[int, int], None]] = None) -> FloatArray:
    """Pairwise MI correlation: pairwise_mi(..., normalize=True)."""
    return pairwise_mi(data, k=k, cond=cond, mask=mask, preprocess=preprocess,
                       drop_nan=drop_nan, normalize=True, max_threads=max_threads,
                       callback=callback)


def _pairwise_mi(data: FloatArray, k: int, cond: Optional[FloatArray], preprocess: bool,
                 drop_nan: bool, mask: Optional[FloatArray], discrete: FloatArray,
                 max_threads: Optional[int],
                 callback: Optional[Callable[[int, int], None]]) -> FloatArray:
    _check_parameters(data, None, k, cond, mask)
    if (not (np.all(discrete) or np.all(~discrete))) and (cond is not None):
        raise ValueError(MIXED_COND_MSG)
    nvar = data.shape[1]
    cond_lag = np.full(cond.shape[1], 0) if cond is not None else np.asarray(0)

    prep = _Prep(mask, 0, 0)
    pairs = []
    jobs = []
    for i in range(nvar):
        for j in range(i + 1, nvar):
            pairs.append((i, j))
            jobs.append(_task_job(prep, ("d", i), data[:, i], ("d", j), data[:, j], 0, 0, 0, k, mask,
                                  cond, cond_lag, discrete[i], discrete[j], preprocess, drop_nan,
                                  share_x=True))
    if pairs and _device_prep_ok((data,) + (() if cond is None else (cond,)), cond, preprocess,
                                 drop_nan, bool(np.any(discrete))):
        n = len(data) if prep.idx is None else len(prep.idx)
        cols = [_native.Col(data[:, i]) for i in range(nvar)]
        zv = None if cond is None else [_native.Col(cond[:, c]) for c in range(cond.shape[1])]
        specs = [(cols[i], cols[j], zv) for i, j in pairs]
        values = _run_device_prep(specs, n, k, prep.idx, jobs, max_threads)
    else:
        batch = _Batch()
        slots = [_add_prepared(batch, p) for p in _prepare_all(jobs, max_threads)]
        values = batch.run()[slots] if slots else np.empty(0)
    # the symmetric matrix with a NaN diagonal, assembled on the device
    result = _native.pairwise_matrix(values, pairs, nvar) if pairs else np.full((nvar, nvar), np.nan)
    if callback is not None:
        for i, j in pairs:
            callback(i, j)
    return result


# ------------------------------------------------- device preprocessing --

# Tasks whose variables are all continuous float64 arrays free of NaNs are
# sliced, masked and rescaled on the device (EGB_RESCALE): the library sums a
# variable in NumPy's pairwise order and a condition of two or more columns
# row by row, as NumPy reduces axis 0 of such an array, and
# _numpy_sums_pairwise() confirms once per process that this NumPy sums that
# way, so the preprocessed columns equal the reference's bit for bit.  Any
# other task, and a task with a constant column (which the reference leaves
# unscaled, with a warning), goes through the host preparation below.
device_prep = True   # False: always prepare on the host

_pairwise_checked: Optional[bool] = None


def _pairwise_sum(a) -> float:
    """NumPy's pairwise summation (numpy/_core/src/umath/loops_utils.h.src,
    pairwise_sum) in plain Python, for the run-time check."""
    n = len(a)
    if n < 8:
        r = 0.0
        for v in a:
            r += v
        return r
    if n <= 128:
        r = [float(v) for v in a[:8]]
        i = 8
        while i < n - (n % 8):
            for j in range(8):
                r[j] += a[i + j]
            i += 8
        res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]))
        while i < n:
            res += a[i]
            i += 1
        return res
    n2 = n // 2
    n2 -= n2 % 8
    return _pairwise_sum(a[:n2]) + _pairwise_sum(a[n2:])


def _sequential_sum(a) -> float:
    s = a[0]
    for v in a[1:]:
        s += v
    return s


def _numpy_sums_pairwise() -> bool:
    """True when this NumPy's sum, mean and std of 1-D float64 arrays (and of
    (n, 1) arrays along axis 0) follow _pairwise_sum, and those of (n, 2) and
    (n, 3) arrays along axis 0 add the rows in order (sizes around every
    branch and beyond one 8192-value block)."""
    global _pairwise_checked
    if _pairwise_checked is None:
        rng = np.random.default_rng(12345)
        ok = True
        for n in (1, 5, 8, 9, 100, 128, 129, 136, 1000, 8191, 8193, 16411):
            a = rng.standard_normal(n) * 3.0 + 1.0
            vals = a.tolist()
            s = _pairwise_sum(vals)
            m = s / n
            d = [(v - m) * (v - m) for v in vals]
            sd = float(np.sqrt(_pairwise_sum(d) / n))
            ok = ok and float(np.add.reduce(a)) == s and float(a.mean()) == m and float(a.std()) == sd
            col = a.reshape(n, 1)
            ok = ok and float(col.mean(axis=0)[0]) == m and float(col.std(axis=0)[0]) == sd
        for n in (3, 129, 8193):
            for dz in (2, 3):
                z = rng.standard_normal((n, dz)) * 2.0 - 0.5
                means, sds = z.mean(axis=0), z.std(axis=0)
                for c in range(dz):
                    vals = z[:, c].tolist()
                    m = _sequential_sum(vals) / n
                    sd = float(np.sqrt(_sequential_sum([(v - m) * (v - m) for v in vals]) / n))
                    ok = ok and float(means[c]) == m and float(sds[c]) == sd
        _pairwise_checked = ok
    return _pairwise_checked


def _device_prep_ok(arrays, cond, preprocess: bool, drop_nan: bool, any_discrete: bool,
                    nan_rows_ok: bool = False) -> bool:
    """Whether the call's columns can be prepared on the device: continuous
    float64 data, preprocessing on; NaNs only where the caller drops their rows
    (drop_nan) and the call gives every task its own rows (nan_rows_ok: the
    lagged estimate_mi)."""
    if not (device_prep and preprocess) or any_discrete or (drop_nan and not nan_rows_ok):
        return False
    for a in arrays:
        if a.dtype != np.float64 or (not drop_nan and np.isnan(a).any()):
            return False
    return _numpy_sums_pairwise()


def _kept_rows(x, y, cond, lag, cond_lag, indices, hi: int, n0: int, idx, max_threads):
    """Per task of a lagged estimate_mi with drop_nan: the sample index of
    the rows it keeps -- the masked rows (idx; None: all n0) whose x, y and
    condition values in the task's lagged views are all numbers, the rows
    _apply_masks keeps (_driver.py:834-854) -- or None where that is every
    masked row (such tasks share the call's index)."""
    base = None if idx is None else np.asarray(idx, dtype=np.int32)
    cols = lambda a: [a] if a.ndim == 1 else [a[:, c] for c in range(a.shape[1])]
    fin_x = [~np.isnan(c) for c in cols(x)]
    fin_y = ~np.isnan(y[hi: hi + n0])
    fin_z = [] if cond is None else [~np.isnan(c) for c in cols(cond)]

    def one(li, vi):
        keep = fin_x[vi][hi - lag[li]: hi - lag[li] + n0] & fin_y
        for c, fz in enumerate(fin_z):
            keep &= fz[hi - cond_lag[li][c]: hi - cond_lag[li][c] + n0]
        if base is not None:
            keep = keep[base]
        if keep.all():
            return None
        return base[keep] if base is not None else np.flatnonzero(keep).astype(np.int32)

    jobs = [lambda li=li, vi=vi: one(li, vi) for li, vi in indices]
    return _prepare_all(jobs, max_threads)


def _run_device_prep(specs, n: int, k: int, idx, jobs, max_threads, rows=None) -> np.ndarray:
    """Estimates of the tasks (x, y, condition columns or None): the columns
    are lagged views of the caller's arrays, sample w at view[idx[w]] (idx
    None: the first n), rescaled on the device.  rows: per task, its own
    sample index (drop_nan) or None for idx.  Tasks with a constant column
    are prepared on the host (`jobs`, same order) and run in a second batch."""
    index = None if idx is None else np.ascontiguousarray(idx, dtype=np.int32)
    tasks = []
    for t, (xv, yv, zv) in enumerate(specs):
        own = None if rows is None else rows[t]
        tn, tix = (n, index) if own is None else (len(own), own)
        if tn <= k:  # the first task in order that keeps too few rows raises
            raise ValueError(K_TOO_LARGE_MSG)
        if zv is None:
            tasks.append(_native.Task(_native.MI, k, [xv], [yv], n=tn, index=tix))
        else:
            tasks.append(_native.Task(_native.CMI, k, [xv], [yv], list(zv), n=tn, index=tix))
    res = []
    values = _native.run_tasks(tasks, flags=run_flags | _native.RESCALE, results_out=res,
                               noise=lambda m: _noise.take(0, (m,)))
    redo = [i for i, r in enumerate(res) if r.status == _native.TASK_CONSTANT]
    if redo:
        batch = _Batch()
        slots = [_add_prepared(batch, p) for p in _prepare_all([jobs[i] for i in redo], max_threads)]
        again = batch.run()
        for i, s in zip(redo, slots):
            values[i] = again[s]
    return values


# ------------------------------------------------------- per-task prep --

class _Prep:
    """Host preprocessing of one estimate_mi / pairwise_mi call, memoised per
    column.

    All tasks of a call slice their variables with the same mask, and y, the
    condition and (in pairwise_mi) every data column recur in many tasks.
    A column's sliced values depend only on (variable, offset), and its
    rescaled values on (variable, offset, noise position), where the noise
    position is fixed by the columns before it in the task (x, then y, then
    z; a constant column draws none).  Computing each key once gives the same
    arrays as the reference's per-task code (_driver.py:788-902), bit for bit
    -- the same NumPy operations on the same values and memory layout -- and
    lets the library upload every distinct array once.  With drop_nan the
    rows a task keeps depend on all of its variables, so that case runs the
    unshared per-task path.
    """

    def __init__(self, mask: Optional[FloatArray], min_lag: int, max_lag: int):
        min_lag, max_lag = min(min_lag, 0), max(max_lag, 0)
        self.idx = None if mask is None else np.flatnonzero(mask[max_lag: len(mask) + min_lag])
        self._memo = {}
        self._lock = threading.Lock()

    def _get(self, key, make):
        with self._lock:
            hit = self._memo.get(key)
        if hit is not None:
            return hit
        val = make()
        with self._lock:
            return self._memo.setdefault(key, val)

    def base(self, key, var: FloatArray) -> FloatArray:
        """The variable itself, or a contiguous copy of it when a mask gathers
        from it (same values; gathering from a strided column is slow)."""
        if self.idx is None or var.flags.c_contiguous:
            return var
        return self._get(("c", key), lambda: (np.ascontiguousarray(var),))[0]

    def sliced(self, key, view, share: bool = True):
        """The lagged, masked values of a variable (`view()` gives the lagged slice)."""
        def make():
            v = view()
            return (v if self.idx is None else v[self.idx],)
        return (make() if not share else self._get(("s",) + key, make))[0]

    def has_nan(self, key, values, share: bool = True) -> bool:
        make = lambda: (bool(np.isnan(values).any()),)
        return (make() if not share else self._get(("n",) + key, make))[0]

    def rescaled(self, key, values, pos: int, axis=None, share: bool = True):
        """(values rescaled to zero mean, unit variance, plus noise at `pos`;
        constant) -- a constant column comes back unchanged."""
        def make():
            std = values.std(axis=axis)
            if np.any(np.abs(std) < 1e-20):
                return values, True
            out = (values - values.mean(axis=axis)) / std
            out += _noise.take(pos, out.shape)
            return out, False
        return make() if not share else self._get(("r", pos) + key, make)


def _prepared_task(prep: _Prep, xkey, x: FloatArray, ykey, y: FloatArray, lag: int,
                   max_lag: int, min_lag: int, k: int, cond: Optional[FloatArray],
                   cond_lag: FloatArray, discrete_x: bool, discrete_y: bool,
                   preprocess: bool, share_x: bool):
    """One task of _lagged_mi (_driver.py:788-832) without drop_nan, through
    the per-call memo: ("task", Task) or ("value", float)."""
    min_lag = min(min_lag, 0)
    max_lag = max(max_lag, 0)
    xk = (xkey, max_lag - lag)
    yk = (ykey, max_lag)
    xb, yb = prep.base(xkey, x), prep.base(ykey, y)
    xs = prep.sliced(xk, lambda: xb[max_lag - lag: len(xb) - lag + min_lag], share_x)
    ys = prep.sliced(yk, lambda: yb[max_lag: len(yb) + min_lag])
    zs = None
    if cond is not None:
        zk = ("cond", tuple(int(c) for c in cond_lag))
        zs = prep.sliced(zk, lambda: np.column_stack(
            [cond[max_lag - cond_lag[i]: len(cond) - cond_lag[i] + min_lag, i]
             for i in range(len(cond_lag))]))

    # _validate_masked_data, in the reference's order
    if len(ys) <= k:
        raise ValueError(K_TOO_LARGE_MSG)
    if (not discrete_x or xs.dtype.kind in "iufc") and prep.has_nan(xk, xs, share_x):
        raise ValueError(NAN_MSG)
    if (not discrete_y or ys.dtype.kind in "iufc") and prep.has_nan(yk, ys):
        raise ValueError(NAN_MSG)
    if not (discrete_x and discrete_y) and zs is not None and prep.has_nan(zk, zs):
        raise ValueError(NAN_MSG)

    if preprocess:
        pos = 0
        if not discrete_x:
            xs, const = prep.rescaled(xk, xs, pos, share=share_x)
            if const:
                warn(PREPROCESS_CONSTANT_DATA_WARNING)
            else:
                pos += xs.size
        if not discrete_y:
            ys, const = prep.rescaled(yk, ys, pos)
            if const:
                warn(PREPROCESS_CONSTANT_DATA_WARNING)
            else:
                pos += ys.size
        if zs is not None and not (discrete_x and discrete_y):
            zs, const = prep.rescaled(zk, zs, pos, axis=0)
            if const:
                warn(PREPROCESS_CONSTANT_DATA_WARNING)
    return _task_of(xs, ys, zs, k, discrete_x, discrete_y)


def _task_of(xs, ys, zs, k: int, discrete_x: bool, discrete_y: bool):
    """The estimator a prepared task calls (_driver.py:814-832)."""
    if zs is None:
        if discrete_x and discrete_y:
            if _discrete_on_device(xs, ys):
                _assert_not_object(np.column_stack((xs, ys)))
                return ("task", discrete_mi_task(xs, ys))
            return ("value", _estimate_discrete_mi(xs, ys))
        if discrete_x:
            return ("task", semidiscrete_task(ys, xs, k))
        if discrete_y:
            return ("task", semidiscrete_task(xs, ys, k))
        return ("task", mi_task(xs, ys, k))
    if discrete_x and discrete_y:
        if _discrete_on_device(xs, ys, zs):
            return ("task", discrete_cmi_task(xs, ys, zs))
        return ("value", _estimate_conditional_discrete_mi(xs, ys, zs))
    if discrete_x:
        return ("task", conditional_semidiscrete_task(ys, xs, zs, k))
    if discrete_y:
        return ("task", conditional_semidiscrete_task(xs, ys, zs, k))
    return ("task", cmi_task(xs, ys, zs, k))


def _prepare_all(jobs: List[Callable[[], Tuple[str, object]]], max_threads: Optional[int]):
    """Run the task preparations, on a thread pool when there are several
    (NumPy releases the GIL in its array loops), and return them in order;
    the first failing task in order raises, as in a sequential run."""
    workers = max_threads if max_threads is not None else min(16, os.cpu_count() or 1)
    if len(jobs) < 4 or workers <= 1:
        return [j() for j in jobs]
    with ThreadPoolExecutor(max_workers=min(workers, len(jobs))) as pool:
        futures = [pool.submit(j) for j in jobs]
        return [f.result() for f in futures]


def _add_prepared(batch: _Batch, prepared) -> int:
    kind, v = prepared
    return batch.add_task(v) if kind == "task" else batch.add_value(v)



def _unshared_task(x: FloatArray, y: FloatArray, lag: int, max_lag: int, min_lag: int, k: int,
                   mask: Optional[FloatArray], cond: Optional[FloatArray], cond_lag: FloatArray,
                   discrete_x: bool, discrete_y: bool, preprocess: bool, drop_nan: bool):
    """One task of _lagged_mi (_driver.py:788-832) on its own: slice, mask,
    validate, rescale; ("task", Task) or ("value", float)."""
    min_lag = min(min_lag, 0)
    max_lag = max(max_lag, 0)
    xs = x[max_lag - lag: len(x) - lag + min_lag]
    ys = y[max_lag: len(y) + min_lag]
    if cond is not None:
        zs = np.column_stack([cond[max_lag - cond_lag[i]: len(cond) - cond_lag[i] + min_lag, i]
                              for i in range(len(cond_lag))])
    else:
        zs = None

    xs, ys, zs = _apply_masks(xs, ys, zs, mask, min_lag, max_lag, drop_nan)
    _validate_masked_data(xs, ys, zs, k, discrete_x, discrete_y)
    if preprocess:
        xs, ys, zs = _rescale_data(xs, ys, zs, discrete_x, discrete_y)
    return _task_of(xs, ys, zs, k, discrete_x, discrete_y)


def _task_job(prep: _Prep, xkey, x, ykey, y, lag, max_lag, min_lag, k, mask, cond, cond_lag,
              discrete_x, discrete_y, preprocess, drop_nan, share_x):
    if drop_nan:
        return lambda: _unshared_task(x, y, lag, max_lag, min_lag, k, mask, cond, cond_lag,
                                      discrete_x, discrete_y, preprocess, drop_nan)
    return lambda: _prepared_task(prep, xkey, x, ykey, y, lag, max_lag, min_lag, k, cond,
                                  cond_lag, discrete_x, discrete_y, preprocess, share_x)


def _apply_masks(xs: FloatArray, ys: FloatArray, zs: Optional[FloatArray],
                 mask: Optional[FloatArray], min_lag: int, max_lag: int,
                 drop_nan: bool) -> Tuple[FloatArray, FloatArray, Optional[FloatArray]]:
    """The mask is indexed in y's time frame (_driver.py:834-854)."""
    if mask is not None:
        sub = mask[max_lag: len(mask) + min_lag]
        xs, ys = xs[sub], ys[sub]
        if zs is not None:
            zs = zs[sub]
    if drop_nan:
        keep = ~(np.isnan(xs) | np.isnan(ys))
        if zs is not None:
            keep &= ~np.max(np.isnan(zs), axis=1)
            zs = zs[keep]
        xs, ys = xs[keep], ys[keep]
    return xs, ys, zs


def _validate_masked_data(xs: FloatArray, ys: FloatArray, zs: Optional[FloatArray], k: int,
                          discrete_x: bool, discrete_y: bool) -> None:
    if len(ys) <= k:
        raise ValueError(K_TOO_LARGE_MSG)
    if (not discrete_x or xs.dtype.kind in "iufc") and np.isnan(xs).any():
        raise ValueError(NAN_MSG)
    if (not discrete_y or ys.dtype.kind in "iufc") and np.isnan(ys).any():
        raise ValueError(NAN_MSG)
    if not (discrete_x and discrete_y) and zs is not None and np.isnan(zs).any():
        raise ValueError(NAN_MSG)


def _rescale_data(xs: FloatArray, ys: FloatArray, zs: Optional[FloatArray],
                  discrete_x: bool, discrete_y: bool):
    """Unit variance plus 1e-10 noise, drawn in the order x, y, z from the
    fixed-seed stream (_driver.py:871-902).  Constant data is left as is,
    with a warning, and draws no noise."""
    pos = 0
    if not discrete_x:
        std = xs.std()
        if np.abs(std) < 1e-20:
            warn(PREPROCESS_CONSTANT_DATA_WARNING)
        else:
            xs = (xs - xs.mean()) / std
            xs += _noise.take(pos, xs.shape)
            pos += xs.size
    if not discrete_y:
        std = ys.std()
        if np.abs(std) < 1e-20:
            warn(PREPROCESS_CONSTANT_DATA_WARNING)
        else:
            ys = (ys - ys.mean()) / std
            ys += _noise.take(pos, ys.shape)
            pos += ys.size
    if zs is not None and not (discrete_x and discrete_y):
        std = zs.std(axis=0)
        if np.any(np.abs(std) < 1e-20):
            warn(PREPROCESS_CONSTANT_DATA_WARNING)
        else:
            zs = (zs - zs.mean(axis=0)) / std
            zs += _noise.take(pos, zs.shape)
    return xs, ys, zs
