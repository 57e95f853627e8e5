"""Device preprocessing (EGB_RESCALE + sample index) on the GPU.

The working columns the estimators use must equal the reference's
_rescale_data output (_driver.py:871-902) bit for bit: NumPy's mean and std
of the indexed column, then (x - mean) / std + noise at the reference's noise
positions.  The public API must give the same estimates with device and host
preparation.
"""

import numpy as np
import pytest

import ennemi_gb300 as eg
from ennemi_gb300 import _driver
from ennemi_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _noise(m):
    return _driver._noise.take(0, (m,))


def _reference_rescale(col, pos, n):
    return (col - col.mean()) / col.std() + _driver._noise.take(pos, (n,))


@pytest.mark.parametrize("n", [9, 100, 128, 129, 136, 1000, 8193, 20011, 180000])
@pytest.mark.parametrize("indexed", [False, True])
def test_rescaled_columns_equal_numpy(n, indexed):
    rng = np.random.default_rng(n)
    rows = n + 57
    raw = rng.normal(size=(rows, 3)) * [2.0, 0.5, 7.0] + [1.0, -3.0, 0.25]   # strided views
    y = rng.standard_t(3, size=rows)
    idx = np.sort(rng.choice(rows - 5, size=n, replace=False)).astype(np.int32) if indexed else None
    xv, yv, zv = raw[5:, 0], y[5:], raw[5:, 2]
    tasks = [N.Task(N.MI, 3, [xv], [yv], n=n, index=idx),
             N.Task(N.CMI, 3, [xv], [yv], [zv], n=n, index=idx)]
    res = []
    N.run_tasks(tasks, flags=N.RESCALE | N.KEEP_INTERNALS, results_out=res, noise=_noise)
    assert all(r.status == 0 for r in res)
    sel = np.arange(n) if idx is None else idx
    want = [_reference_rescale(c[sel], i * n, n) for i, c in enumerate((xv, yv, zv))]
    for t, ncol in ((0, 2), (1, 3)):
        for c in range(ncol):
            got = N.fetch(t, 16 + c, n)
            assert np.array_equal(got.view(np.uint64), want[c].view(np.uint64)), (t, c)


@pytest.mark.parametrize("n", [9, 129, 8193, 50000])
@pytest.mark.parametrize("dz", [2, 3])
def test_condition_columns_reduce_row_by_row(n, dz):
    """A condition of dz >= 2 columns: NumPy's axis-0 mean / std of the (n, dz)
    array (rows added in order), noise drawn row-major after x and y."""
    rng = np.random.default_rng(100 * n + dz)
    rows = n + 40
    raw = rng.normal(size=(rows, dz + 2)) * 3.0 - 1.0
    idx = np.sort(rng.choice(rows - 3, size=n, replace=False)).astype(np.int32)
    views = [raw[3:, c] for c in range(dz + 2)]
    task = N.Task(N.CMI, 3, [views[0]], [views[1]], views[2:], n=n, index=idx)
    res = []
    N.run_tasks([task], flags=N.RESCALE | N.KEEP_INTERNALS, results_out=res, noise=_noise)
    assert res[0].status == 0
    Z = np.column_stack([v[idx] for v in views[2:]])
    Zr = (Z - Z.mean(axis=0)) / Z.std(axis=0) + _driver._noise.take(2 * n, (n, dz))
    assert np.array_equal(N.fetch(0, 16, n), _reference_rescale(views[0][idx], 0, n))
    assert np.array_equal(N.fetch(0, 17, n), _reference_rescale(views[1][idx], n, n))
    for c in range(dz):
        assert np.array_equal(N.fetch(0, 18 + c, n).view(np.uint64), Zr[:, c].view(np.uint64)), c


def test_semidiscrete_columns_with_index():
    """Labels and an index together: the class order is applied on top of the
    index; the continuous column is rescaled from noise position 0."""
    rng = np.random.default_rng(5)
    rows, n = 30000, 25000
    x = rng.normal(size=rows) * 4 + 2
    z = rng.normal(size=rows)
    idx = np.sort(rng.choice(rows, size=n, replace=False)).astype(np.int32)
    lab = rng.integers(0, 5, size=n).astype(np.int32)
    tasks = [N.Task(N.SEMI, 3, [x], labels=lab, nclass=5, n=n, index=idx),
             N.Task(N.CSEMI, 3, [x], z=[z], labels=lab, nclass=5, n=n, index=idx)]
    N.run_tasks(tasks, flags=N.RESCALE | N.KEEP_INTERNALS, noise=_noise)
    assert np.array_equal(N.fetch(0, 16, n), _reference_rescale(x[idx], 0, n))
    assert np.array_equal(N.fetch(1, 16, n), _reference_rescale(x[idx], 0, n))
    assert np.array_equal(N.fetch(1, 17, n), _reference_rescale(z[idx], n, n))
    # the same tasks prepared on the host
    host = [N.Task(N.SEMI, 3, [_reference_rescale(x[idx], 0, n)], labels=lab, nclass=5),
            N.Task(N.CSEMI, 3, [_reference_rescale(x[idx], 0, n)],
                   z=[_reference_rescale(z[idx], n, n)], labels=lab, nclass=5)]
    assert np.array_equal(N.run_tasks(tasks, flags=N.RESCALE, noise=_noise), N.run_tasks(host))


def test_constant_column_reported():
    rng = np.random.default_rng(2)
    n = 5000
    x = rng.normal(size=n)
    tasks = [N.Task(N.MI, 3, [x], [np.full(n, 3.5)], n=n), N.Task(N.MI, 3, [x], [x[::-1].copy()], n=n)]
    res = []
    v = N.run_tasks(tasks, flags=N.RESCALE, results_out=res, noise=_noise)
    assert res[0].status == N.TASK_CONSTANT and np.isnan(v[0])
    assert res[1].status == 0 and np.isfinite(v[1])


def test_rescale_needs_one_x_and_y_column():
    x = np.random.default_rng(1).normal(size=(500, 2))
    with pytest.raises(RuntimeError, match="one x column"):
        N.run_tasks([N.Task(N.MI, 3, [x[:, 0], x[:, 1]], [x[:, 0]])], flags=N.RESCALE, noise=_noise)


@pytest.mark.parametrize("case", ["lags_mask", "lags_cond", "lags_cond2", "pairwise_mask",
                                  "pairwise_cond2", "constant"])
def test_public_api_same_with_device_and_host_preparation(case, monkeypatch):
    rng = np.random.default_rng(17)
    n = 20000
    x = rng.normal(size=(n, 4))
    x[:, 1] += 0.6 * x[:, 0]
    y = x[:, 0] + rng.normal(size=n)
    z = rng.normal(size=n)
    mask = rng.random(n) > 0.1
    calls = {
        "lags_mask": lambda: eg.estimate_mi(y, x, lag=[0, 1, 7], mask=mask),
        "lags_cond": lambda: eg.estimate_mi(y, x[:, :2], lag=[0, 3], cond=z, cond_lag=2, mask=mask),
        "lags_cond2": lambda: eg.estimate_mi(y, x[:, :2], lag=[0, 3], cond=x[:, 2:],
                                             cond_lag=[[1, 0], [2, 4]], mask=mask),
        "pairwise_mask": lambda: eg.pairwise_mi(x, mask=mask),
        "pairwise_cond2": lambda: eg.pairwise_mi(x[:, :3], cond=np.column_stack((z, y)), mask=mask),
        "constant": lambda: eg.pairwise_mi(np.column_stack((x[:, :2], np.full(n, 2.0)))),
    }
    dev = calls[case]()
    monkeypatch.setattr(_driver, "device_prep", False)
    host = calls[case]()
    assert np.array_equal(dev, host, equal_nan=True)


def _division_cases():
    rng = np.random.default_rng(77)
    n = 400_000
    # random mantissas and signs over the exponents of rescaled data and far beyond
    a = rng.uniform(1, 2, n) * 2.0 ** rng.integers(-60, 60, n) * rng.choice([-1, 1], n)
    b = rng.uniform(1, 2, n) * 2.0 ** rng.integers(-60, 60, n) * rng.choice([-1, 1], n)
    # quotients at and beside binade edges and exact multiples
    k = rng.integers(-8, 9, 50_000)
    bb = rng.uniform(1, 2, 50_000) * 2.0 ** rng.integers(-30, 30, 50_000)
    edge_a = bb * (1.0 + k * 2.0 ** -52)
    edge_a2 = bb * 2.0 ** rng.integers(-5, 5, 50_000)
    ones = np.full(1000, np.nextafter(2.0, 0.0))                      # all-ones mantissa
    # the division's own domain: huge, tiny, subnormal, zeros, inf, nan
    spec = np.array([0.0, -0.0, 1e300, -1e300, 1e-300, 5e-324, -5e-324, np.inf, -np.inf, np.nan,
                     1.0, -1.0, 3.0, 2.0 ** 1000, 2.0 ** -1000, 1e-20, 1e20])
    sa, sb = np.meshgrid(spec, spec)
    return (np.concatenate([a, edge_a, edge_a2, ones * 3.0, ones, sa.ravel()]),
            np.concatenate([b, bb, bb, ones, ones * 3.0, sb.ravel()]))


def test_device_division_is_ieee_division():
    """The rescale divides by the column's standard deviation without an FP64
    divide per sample (reciprocal, exact FMA remainder, midpoint test); it
    must give IEEE division's round-to-nearest-even bits everywhere."""
    a, b = _division_cases()
    got = N.context(0).debug_divide(a, b)
    with np.errstate(all="ignore"):
        want = a / b
    bad = np.flatnonzero(got.view(np.uint64) != want.view(np.uint64))
    nan_both = np.isnan(got[bad]) & np.isnan(want[bad])
    bad = bad[~nan_both]
    assert bad.size == 0, list(zip(a[bad[:5]], b[bad[:5]], got[bad[:5]], want[bad[:5]]))
