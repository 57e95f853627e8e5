"""Host-side logic of the public API, on the CPU.

The GPU evaluation (``_native.run_tasks``) is swapped for the CPU oracle in
these tests only, so that lagging, masking, validation, rescaling, batching
and result assembly can be checked against the reference's own outputs
(tests/golden/golden_driver.npz) without a device.  The product path never
does this: without the CUDA library it raises (last test).
"""

import warnings

import numpy as np
import pytest

import ennemi_gb300 as eg
from ennemi_gb300 import _driver, _native
from conftest import driver_cases, oracle_normalize, oracle_pairwise_matrix, oracle_run_tasks

DCASES = driver_cases()


def _py(v):
    v = np.asarray(v)
    return v.item() if v.ndim == 0 else v


@pytest.fixture
def on_oracle(oracle, monkeypatch):
    calls = []
    monkeypatch.setattr(_native, "run_tasks", oracle_run_tasks(oracle, calls))
    monkeypatch.setattr(_native, "pairwise_matrix", oracle_pairwise_matrix)
    monkeypatch.setattr(_native, "normalize", oracle_normalize)
    return calls


@pytest.mark.parametrize("case", DCASES, ids=[c["name"] for c in DCASES])
def test_driver_matches_reference(on_oracle, case):
    fn = getattr(eg, str(case["func"]))
    args = [_py(case[f"arg{i}"]) for i in range(4) if f"arg{i}" in case]
    kw = {k[3:]: _py(v) for k, v in case.items() if k.startswith("kw_")}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        res = np.asarray(fn(*args, **kw), dtype=np.float64)
    gold = case["result"]
    assert res.shape == gold.shape
    assert np.allclose(res, gold, rtol=0, atol=1e-12, equal_nan=True), (res, gold)
    # every call is one batch
    assert len(on_oracle) <= 1


def test_noise_stream_is_the_reference_draw_sequence():
    for n, dz in [(1, 1), (17, 2), (5000, 3)]:
        rng = np.random.default_rng(_driver.NOISE_SEED)
        a = rng.normal(0.0, 1e-10, n)
        b = rng.normal(0.0, 1e-10, n)
        c = rng.normal(0.0, 1e-10, (n, dz))
        assert np.array_equal(_driver._noise.take(0, (n,)), a)
        assert np.array_equal(_driver._noise.take(n, (n,)), b)
        assert np.array_equal(_driver._noise.take(2 * n, (n, dz)), c)


def test_rescale_matches_reference_formula():
    rng = np.random.default_rng(3)
    x, y, z = rng.normal(5, 3, 300), rng.gamma(2, size=300), rng.normal(size=(300, 2))
    xs, ys, zs = _driver._rescale_data(x, y, z, False, False)
    r = np.random.default_rng(2_718281828)
    ex = (x - x.mean()) / x.std()
    ex += r.normal(0.0, 1e-10, ex.shape)
    ey = (y - y.mean()) / y.std()
    ey += r.normal(0.0, 1e-10, ey.shape)
    ez = (z - z.mean(axis=0)) / z.std(axis=0)
    ez += r.normal(0.0, 1e-10, ez.shape)
    assert np.array_equal(xs, ex) and np.array_equal(ys, ey) and np.array_equal(zs, ez)


def test_constant_variable_warns_and_draws_no_noise():
    x = np.ones(50)
    y = np.arange(50.0)
    with pytest.warns(UserWarning):
        xs, ys, _ = _driver._rescale_data(x, y, None, False, False)
    assert np.array_equal(xs, x)
    r = np.random.default_rng(2_718281828)
    ey = (y - y.mean()) / y.std()
    ey += r.normal(0.0, 1e-10, ey.shape)  # y gets the first draw
    assert np.array_equal(ys, ey)


@pytest.mark.parametrize("call,exc,msg", [
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), k=0), ValueError, "k must be greater than zero"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), k=3.0), TypeError, "k must be int"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(9)), ValueError, "x and y must have same length"),
    (lambda: eg.estimate_mi(np.zeros((10, 2)), np.zeros(10)), ValueError, "y must be one-dimensional"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros((10, 2, 2))), ValueError, "x must be one- or two-dimensional"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), mask=np.ones(9, bool)), ValueError,
     "mask length does not match input length"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), mask=np.ones(10)), TypeError,
     "mask must contain only booleans"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), mask=np.ones((10, 2), bool)), ValueError,
     "mask must be one-dimensional"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), cond=np.zeros(9)), ValueError,
     "x and cond must have same length"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), lag=10), ValueError,
     "lag is too large, no observations left"),
    (lambda: eg.estimate_mi(np.zeros(10), np.zeros(10), k=10), ValueError,
     "k must be smaller than number of observations (after lag and mask)"),
    (lambda: eg.estimate_mi(np.r_[np.nan, np.zeros(9)], np.zeros(10)), ValueError,
     "input contains NaNs (after applying the mask), pass drop_nan=True to ignore"),
    (lambda: eg.estimate_entropy(np.zeros(5), k=5), ValueError,
     "k must be smaller than number of observations (after lag and mask)"),
    (lambda: eg.estimate_entropy(np.zeros((5, 2, 2))), ValueError, "x must be one- or two-dimensional"),
    (lambda: eg.pairwise_mi(np.zeros((10, 3)), cond=np.zeros(10), discrete=[True, False, False]),
     ValueError, "Conditioning is not supported with mixed discrete and continuous data."),
])
def test_validation_messages(call, exc, msg):
    with pytest.raises(exc) as ei:
        call()
    assert str(ei.value).startswith(msg)


def test_callbacks_once_per_task_after_one_batch(on_oracle):
    rng = np.random.default_rng(0)
    x, y = rng.normal(size=(400, 3)), rng.normal(size=400)
    seen = []
    eg.estimate_mi(y, x, [0, 1, 2], callback=lambda v, l: seen.append((v, l)))
    assert sorted(seen) == sorted((v, l) for l in [0, 1, 2] for v in range(3))
    assert on_oracle == [9]
    seen.clear()
    eg.pairwise_mi(x, callback=lambda i, j: seen.append((i, j)))
    assert seen == [(0, 1), (0, 2), (1, 2)]


def test_aliases_exactly_equal(on_oracle):
    rng = np.random.default_rng(1)
    data = rng.normal(size=(300, 3))
    assert np.array_equal(eg.estimate_corr(data[:, 0], data[:, 1:], [0, 1]),
                          eg.estimate_mi(data[:, 0], data[:, 1:], [0, 1], normalize=True))
    assert np.array_equal(eg.pairwise_corr(data), eg.pairwise_mi(data, normalize=True), equal_nan=True)


def test_normalize_mi(monkeypatch):
    """Numeric input goes to the device kernel (here its host stand-in) and
    keeps its shape; anything else raises as the reference does."""
    seen = []

    def fake(values, device=0):
        seen.append(np.shape(values))
        return oracle_normalize(values)
    monkeypatch.setattr(_native, "normalize", fake)
    assert eg.normalize_mi(-0.5) == -0.5
    assert np.isclose(eg.normalize_mi(-0.5 * np.log(1 - 0.36)), 0.6)
    assert eg.normalize_mi([[0.1, 0.0], [np.nan, -np.inf]]).shape == (2, 2)
    assert seen == [(), (), (2, 2)]
    with pytest.raises(TypeError):
        eg.normalize_mi(["a"])


def test_trivial_pairwise():
    assert np.isnan(eg.pairwise_mi(np.zeros(10))).all()


def test_fails_loudly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    x = np.random.default_rng(0).normal(size=100)
    with pytest.raises(RuntimeError):
        eg.estimate_mi(x, x + 1)


def _captured_inputs(monkeypatch, call, unshared):
    """Columns of every task a public call hands to the GPU."""
    seen = []

    def run(tasks, flags=0, device=0, results_out=None, groups_out=None):
        for t in tasks:
            seen.append([np.array(c, copy=True) for c in list(t.x) + list(t.y) + list(t.z)] +
                        ([np.asarray(t.labels).copy()] if t.labels is not None else []))
        return np.zeros(len(tasks))

    with monkeypatch.context() as m:
        m.setattr(_native, "run_tasks", run)
        m.setattr(_native, "pairwise_matrix", oracle_pairwise_matrix)
        m.setattr(_driver, "device_prep", False)   # the host preparation itself
        if unshared:
            m.setattr(_driver, "_task_job",
                      lambda prep, xkey, x, ykey, y, lag, max_lag, min_lag, k, mask, cond,
                      cond_lag, dx, dy, pre, dn, share_x:
                      (lambda: _driver._unshared_task(x, y, lag, max_lag, min_lag, k, mask, cond,
                                                      cond_lag, dx, dy, pre, dn)))
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            call()
    return seen, len(w)


@pytest.mark.parametrize("case", ["lags_mask", "lags_nomask", "lags_cond", "pairwise",
                                  "pairwise_cond_mask", "pairwise_discrete", "constant"])
def test_shared_preparation_is_bit_identical(monkeypatch, case):
    """Columns prepared once per call equal the reference's per-task preparation."""
    rng = np.random.default_rng(7)
    n = 700
    x = rng.normal(size=(n, 3))
    y = x[:, 0] + rng.normal(size=n)
    cond = rng.normal(size=(n, 2))
    mask = rng.random(n) > 0.2
    data = np.column_stack((x, y, rng.integers(0, 3, n)))
    calls = {
        "lags_mask": lambda: eg.estimate_mi(y, x, lag=[0, 1, 5, 1], mask=mask),
        "lags_nomask": lambda: eg.estimate_mi(y, x, lag=[0, 2, -3]),
        "lags_cond": lambda: eg.estimate_mi(y, x, lag=[0, 2], cond=cond, cond_lag=[[1, 0], [3, 2]],
                                            mask=mask),
        "pairwise": lambda: eg.pairwise_mi(data[:, :4]),
        "pairwise_cond_mask": lambda: eg.pairwise_mi(data[:, :4], cond=cond, mask=mask),
        "pairwise_discrete": lambda: eg.pairwise_mi(data, discrete=[False] * 4 + [True]),
        "constant": lambda: eg.pairwise_mi(np.column_stack((x[:, :2], np.ones(n)))),
    }
    a, wa = _captured_inputs(monkeypatch, calls[case], unshared=False)
    b, wb = _captured_inputs(monkeypatch, calls[case], unshared=True)
    assert len(a) == len(b) and wa == wb
    for ta, tb in zip(a, b):
        assert len(ta) == len(tb)
        for ca, cb in zip(ta, tb):
            assert ca.dtype == cb.dtype and ca.shape == cb.shape
            assert np.array_equal(ca.view(np.uint8), cb.view(np.uint8))


@pytest.mark.parametrize("case", ["lags_mask", "lags_nomask", "lags_cond1", "lags_cond2",
                                  "pairwise", "pairwise_cond_mask", "constant", "nan_elsewhere",
                                  "lags_dropnan", "lags_cond_dropnan", "pairwise_dropnan"])
def test_device_preprocessing_matches_host_preparation(oracle, monkeypatch, case):
    """The EGB_RESCALE path (lagged views + shared sample index, rescaled in the
    library) gives what the host preparation gives; the library is stood in for
    by the oracle applying the reference's _rescale_data to the indexed columns."""
    rng = np.random.default_rng(11)
    n = 600
    x = rng.normal(size=(n, 3))
    y = x[:, 0] + rng.normal(size=n)
    cond = rng.normal(size=(n, 2))
    mask = rng.random(n) > 0.2
    xn = x.copy()
    xn[-3:, 1] = np.nan                     # after every lagged slice below (lags 5, 6)
    xd, yd, cd = x.copy(), y.copy(), cond.copy()   # NaN rows dropped per task
    xd[rng.random((n, 3)) < 0.03] = np.nan
    yd[rng.random(n) < 0.03] = np.nan
    cd[rng.random((n, 2)) < 0.03] = np.nan
    calls = {
        "lags_mask": lambda: eg.estimate_mi(y, x, lag=[0, 1, 5, -2], mask=mask),
        "lags_nomask": lambda: eg.estimate_mi(y, x, lag=[0, 2, -3]),
        "lags_cond1": lambda: eg.estimate_mi(y, x, lag=[0, 2], cond=cond[:, 0], cond_lag=[1, 3],
                                             mask=mask),
        "lags_cond2": lambda: eg.estimate_mi(y, x, lag=[0, 2], cond=cond, mask=mask),
        "pairwise": lambda: eg.pairwise_mi(np.column_stack((x, y))),
        "pairwise_cond_mask": lambda: eg.pairwise_mi(x, cond=cond[:, 1], mask=mask),
        "constant": lambda: eg.pairwise_mi(np.column_stack((x[:, :2], np.ones(n)))),
        "nan_elsewhere": lambda: eg.estimate_mi(y, xn, lag=[5, 6]),
        "lags_dropnan": lambda: eg.estimate_mi(yd, xd, lag=[0, 1, 5, -2], mask=mask, drop_nan=True),
        "lags_cond_dropnan": lambda: eg.estimate_mi(yd, xd, lag=[0, 2], cond=cd, cond_lag=[[1, 0], [3, 2]],
                                                    drop_nan=True),
        "pairwise_dropnan": lambda: eg.pairwise_mi(xd, drop_nan=True),
    }
    flags_seen = []
    run = oracle_run_tasks(oracle)

    def recording(tasks, flags=0, **kw):
        flags_seen.append(flags)
        return run(tasks, flags=flags, **kw)

    monkeypatch.setattr(_native, "run_tasks", recording)
    monkeypatch.setattr(_native, "pairwise_matrix", oracle_pairwise_matrix)
    monkeypatch.setattr(_native, "normalize", oracle_normalize)
    with warnings.catch_warnings(record=True) as w_dev:
        warnings.simplefilter("always")
        dev = calls[case]()
    used = any(f & _native.RESCALE for f in flags_seen)
    monkeypatch.setattr(_driver, "device_prep", False)
    with warnings.catch_warnings(record=True) as w_host:
        warnings.simplefilter("always")
        host = calls[case]()
    assert np.array_equal(dev, host, equal_nan=True)
    assert len(w_dev) == len(w_host)
    # the device path is taken exactly where its conditions hold (NaNs: only
    # where the lagged estimate_mi drops their rows per task)
    assert used == (case not in ("nan_elsewhere", "pairwise_dropnan"))


def test_numpy_sums_in_pairwise_order():
    """The run-time check that enables device preprocessing holds for this NumPy,
    and the restatement agrees with np.add.reduce on a longer array."""
    assert _driver._numpy_sums_pairwise()
    a = np.random.default_rng(3).standard_normal(50_001)
    assert _driver._pairwise_sum(a.tolist()) == float(np.add.reduce(a))


@pytest.mark.parametrize("case", ["lags_mask", "lags_nomask", "lags_negative", "lags_cond2",
                                  "pairwise_cond_mask", "lags_mask_dropnan", "lags_cond2_dropnan"])
def test_device_preprocessing_columns_are_the_reference_slices(monkeypatch, case):
    """Every task of the EGB_RESCALE path reads, through its column views and
    shared sample index, exactly the lagged and masked samples the reference's
    _lagged_mi slices (_driver.py:795-806, :834-842), in task order, with n
    and the noise layout (x, y, then the condition) implied by the columns."""
    rng = np.random.default_rng(29)
    n = 500
    x = rng.normal(size=(n, 3))
    y = rng.normal(size=n)
    cond = rng.normal(size=(n, 2))
    mask = rng.random(n) > 0.25
    drop = case.endswith("_dropnan")
    if drop:  # NaNs in every variable; each task keeps its own rows
        x[rng.random((n, 3)) < 0.04] = np.nan
        y[rng.random(n) < 0.04] = np.nan
        cond[rng.random((n, 2)) < 0.04] = np.nan
        case = case[:-len("_dropnan")]
    lags = {"lags_mask": [0, 1, 5], "lags_nomask": [0, 2, 7], "lags_negative": [-2, 0, 3],
            "lags_cond2": [0, 4]}
    seen = []

    def run(tasks, flags=0, device=0, results_out=None, noise=None, groups_out=None):
        assert flags & _native.RESCALE
        for t in tasks:
            ix = np.arange(t.n) if t.index is None else np.asarray(t.index)
            cols = [(c.ref if isinstance(c, _native.Col) else np.asarray(c))[ix]
                    for c in list(t.x) + list(t.y) + list(t.z)]
            seen.append((t.kind, len(t.x), len(t.y), len(t.z), t.n, cols))
        return np.zeros(len(tasks))

    monkeypatch.setattr(_native, "run_tasks", run)
    monkeypatch.setattr(_native, "pairwise_matrix", oracle_pairwise_matrix)
    monkeypatch.setattr(_native, "normalize", oracle_normalize)
    want = []
    if case.startswith("lags"):
        lag = lags[case]
        c2 = case == "lags_cond2"
        cond_lag = [[1, 0], [3, 2]] if c2 else None
        eg.estimate_mi(y, x, lag=lag, mask=None if case == "lags_nomask" else mask,
                       cond=cond if c2 else None, cond_lag=cond_lag if c2 else 0, drop_nan=drop)
        m = None if case == "lags_nomask" else mask
        lo = min(min(lag), 0 if not c2 else min(min(r) for r in cond_lag))
        hi = max(max(lag), 0 if not c2 else max(max(r) for r in cond_lag))
        lo, hi = min(lo, 0), max(hi, 0)
        for li, lg in enumerate(lag):
            for vi in range(3):
                xs = x[hi - lg: n - lg + lo, vi]
                ys = y[hi: n + lo]
                zs = (np.column_stack([cond[hi - cond_lag[li][i]: n - cond_lag[li][i] + lo, i]
                                       for i in range(2)]) if c2 else None)
                xs, ys, zs = _driver._apply_masks(xs, ys, zs, m, lo, hi, drop)
                want.append([xs, ys] + ([zs[:, 0], zs[:, 1]] if c2 else []))
    else:
        eg.pairwise_mi(x, cond=cond, mask=mask)
        for i in range(3):
            for j in range(i + 1, 3):
                xs, ys, zs = _driver._apply_masks(x[:, i], x[:, j], cond, mask, 0, 0, False)
                want.append([xs, ys, zs[:, 0], zs[:, 1]])
    assert len(seen) == len(want)
    for (kind, dx, dy, dz, tn, cols), ref in zip(seen, want):
        assert (dx, dy, dz) == (1, 1, len(ref) - 2) and tn == len(ref[0])
        assert kind == (_native.CMI if dz else _native.MI)
        for got, r in zip(cols, ref):
            assert np.array_equal(got.view(np.uint64), np.ascontiguousarray(r).view(np.uint64))
