"""Batched workloads shaped like the lag, pairwise and semidiscrete/entropy
benchmark cases (ennemi_gb300.synthetic), on the GPU.

Full size: the default path (FP32 tiles + FP64 recheck, warp-grid layout)
equals the all-FP64 plain kernels and the CTA-grid variant bit for bit --
counts and distances are exact and the digamma sums run in the same order in
every variant -- and every estimate is finite.  Reduced size: the estimates
match the oracle within 1e-10 nats.
"""

import warnings

import numpy as np
import pytest

import ennemi_gb300 as eg
from ennemi_gb300 import _driver, _native, synthetic
from ennemi_gb300 import _entropy_estimators as ee
from conftest import oracle_run_tasks

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _variants(monkeypatch, fn):
    """fn() under the default flags, PLAIN_FP64 and FORCE_CTA_GRID; asserts equality."""
    out = []
    for flags in (0, _native.PLAIN_FP64, _native.FORCE_CTA_GRID):
        monkeypatch.setattr(_driver, "run_flags", flags)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out.append(np.asarray(fn()))
    monkeypatch.setattr(_driver, "run_flags", 0)
    assert np.array_equal(out[0], out[1], equal_nan=True), np.nanmax(np.abs(out[0] - out[1]))
    assert np.array_equal(out[0], out[2], equal_nan=True), np.nanmax(np.abs(out[0] - out[2]))
    return out[0]


def _gpu_and_oracle(oracle, monkeypatch, fn):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gpu = np.asarray(fn())
        with monkeypatch.context() as m:
            m.setattr(_native, "run_tasks", oracle_run_tasks(oracle))
            ref = np.asarray(fn())
    assert gpu.shape == ref.shape
    assert np.allclose(gpu, ref, rtol=0, atol=TOL, equal_nan=True), np.nanmax(np.abs(gpu - ref))
    return gpu


# ------------------------------------------------------------ batched lags --

def test_lagged_batch_full_size(monkeypatch):
    y, x, lags, mask = synthetic.lagged_ar()
    res = _variants(monkeypatch, lambda: eg.estimate_mi(y, x, lag=lags, mask=mask))
    assert res.shape == (49, 16) and np.all(np.isfinite(res))
    # y is series 0 itself: lag 0 is the largest estimate of that column
    assert np.argmax(res[:, 0]) == 0


def test_lagged_batch_vs_oracle(oracle, monkeypatch):
    y, x, _, mask = synthetic.lagged_ar(length=1500, nseries=4, seed=8)
    lags = np.arange(0, 49, 6)
    res = _gpu_and_oracle(oracle, monkeypatch,
                          lambda: eg.estimate_mi(y, x, lag=lags, mask=mask))
    assert res.shape == (len(lags), 4)
    cond = _gpu_and_oracle(oracle, monkeypatch,
                           lambda: eg.estimate_mi(y, x[:, 1:], lag=lags, mask=mask,
                                                  cond=x[:, 0], cond_lag=lags + 1))
    assert cond.shape == (len(lags), 3)


def test_lagged_batch_nan_runs_full_size(monkeypatch):
    """The lag workload with NaN runs in every x series and drop_nan=True:
    each task keeps its own rows, so the 784 tasks of the batch have
    different lengths."""
    y, x, lags, mask = synthetic.lagged_ar()
    xn = synthetic.with_nan_runs(x)
    res = _variants(monkeypatch, lambda: eg.estimate_mi(y, xn, lag=lags, mask=mask, drop_nan=True))
    assert res.shape == (49, 16) and np.all(np.isfinite(res))
    assert np.argmax(res[:, 0]) == 0


def test_lagged_batch_nan_runs_vs_oracle(oracle, monkeypatch):
    y, x, _, mask = synthetic.lagged_ar(length=1500, nseries=4, seed=8)
    xn = synthetic.with_nan_runs(x, frac=0.05)
    lags = np.arange(0, 49, 6)
    res = _gpu_and_oracle(oracle, monkeypatch,
                          lambda: eg.estimate_mi(y, xn, lag=lags, mask=mask, drop_nan=True))
    assert res.shape == (len(lags), 4) and np.all(np.isfinite(res))


# --------------------------------------------------------- batched pairwise --

def test_pairwise_full_size(monkeypatch):
    data, cond = synthetic.pairwise_mix()
    res = _variants(monkeypatch, lambda: eg.pairwise_mi(data))
    off = ~np.eye(64, dtype=bool)
    assert np.all(np.isfinite(res[off])) and np.all(np.isnan(np.diag(res)))
    assert np.array_equal(res, res.T, equal_nan=True)
    resc = _variants(monkeypatch, lambda: eg.pairwise_mi(data, cond=cond))
    assert np.all(np.isfinite(resc[off]))


def test_pairwise_vs_oracle(oracle, monkeypatch):
    data, cond = synthetic.pairwise_mix(n=1200, seed=9)
    data = data[:, ::8]
    _gpu_and_oracle(oracle, monkeypatch, lambda: eg.pairwise_mi(data))
    _gpu_and_oracle(oracle, monkeypatch, lambda: eg.pairwise_mi(data, cond=cond))


# ------------------------------------------------- semidiscrete and entropy --

def _semidiscrete_tasks(cases, ent):
    tasks = [ee.semidiscrete_task(x, y, 3) for x, y in cases]
    tasks.append(ee.entropy_task(ent, 3))
    tasks.append(ee.conditional_semidiscrete_task(cases[1][0][:, 0], cases[1][1],
                                                  cases[1][0][:, 1], 3))
    return tasks


def test_semidiscrete_batch_full_size():
    cases, ent = synthetic.semidiscrete_mix()
    tasks = _semidiscrete_tasks(cases, ent)
    fast = _native.run_tasks(tasks)
    plain = _native.run_tasks(tasks, flags=_native.PLAIN_FP64)
    cta = _native.run_tasks(tasks, flags=_native.FORCE_CTA_GRID)
    assert np.array_equal(fast, plain) and np.array_equal(fast, cta)
    assert not np.any(np.isnan(fast))
    # one batch of all tasks equals the tasks run one at a time
    single = np.array([_native.run_tasks([t])[0] for t in tasks])
    assert np.array_equal(fast, single)


def test_semidiscrete_batch_vs_oracle(oracle):
    cases, ent = synthetic.semidiscrete_mix(n=2500, seed=10)
    tasks = _semidiscrete_tasks(cases, ent)
    gpu = _native.run_tasks(tasks)
    ref = oracle_run_tasks(oracle)(tasks)
    assert np.allclose(gpu, ref, rtol=0, atol=TOL, equal_nan=True), np.abs(gpu - ref)
