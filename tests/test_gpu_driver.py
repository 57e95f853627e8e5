"""The public API on the GPU reproduces the reference's driver outputs
(tests/golden/golden_driver.npz) within 1e-10 nats."""

import warnings

import numpy as np
import pytest

import ennemi_gb300 as eg
from conftest import driver_cases

pytestmark = pytest.mark.gpu
DCASES = driver_cases()


def _py(v):
    v = np.asarray(v)
    return v.item() if v.ndim == 0 else v


@pytest.mark.parametrize("case", DCASES, ids=[c["name"] for c in DCASES])
def test_driver_golden_on_gpu(case):
    fn = getattr(eg, str(case["func"]))
    args = [_py(case[f"arg{i}"]) for i in range(4) if f"arg{i}" in case]
    kw = {k[3:]: _py(v) for k, v in case.items() if k.startswith("kw_")}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        res = np.asarray(fn(*args, **kw), dtype=np.float64)
    gold = case["result"]
    assert res.shape == gold.shape
    assert np.allclose(res, gold, rtol=0, atol=1e-10, equal_nan=True), (res, gold)


def test_normalize_on_device_matches_formula():
    from ennemi_gb300 import _native as N
    rng = np.random.default_rng(3)
    v = np.concatenate([rng.exponential(0.5, size=5000), -rng.exponential(size=100),
                        [0.0, -0.0, np.inf, -np.inf, np.nan, 1e-300, 5e-324, 40.0, 1e300]])
    got = N.normalize(v)
    with np.errstate(invalid="ignore", divide="ignore"):
        ref = np.where(v <= 0.0, v, np.sqrt(1 - np.exp(-2 * v)))
        # device and host exp may differ in the last bit, which the
        # cancellation in 1 - exp(-2 v) turns into 2^-53 / value
        bound = np.where(ref > 0, 2.0 ** -53 / np.maximum(ref, 1e-300), 0.0) + 2e-16
    fin = np.isfinite(ref)
    assert np.all(np.abs(got[fin] - ref[fin]) <= bound[fin])
    assert np.array_equal(got[~fin], ref[~fin], equal_nan=True)
    assert np.array_equal(got[v <= 0], v[v <= 0])          # unchanged, -0.0 and -inf included
    assert np.array_equal(np.signbit(got[v <= 0]), np.signbit(v[v <= 0]))


def test_pairwise_matrix_on_device():
    from ennemi_gb300 import _native as N
    rng = np.random.default_rng(4)
    nvar = 37
    pairs = [(i, j) for i in range(nvar) for j in range(i + 1, nvar)]
    vals = rng.normal(size=len(pairs))
    m = N.pairwise_matrix(vals, pairs, nvar)
    ref = np.full((nvar, nvar), np.nan)
    for (i, j), v in zip(pairs, vals):
        ref[i, j] = ref[j, i] = v
    assert np.array_equal(m, ref, equal_nan=True)
    mn = N.pairwise_matrix(vals, pairs, nvar, normalize=True)
    with np.errstate(invalid="ignore"):
        refn = np.where(ref <= 0.0, ref, np.sqrt(1 - np.exp(-2 * ref)))
    assert np.allclose(mn, refn, rtol=1e-14, atol=1e-15, equal_nan=True)
    with pytest.raises(RuntimeError, match="out of range"):
        N.pairwise_matrix([1.0], [(0, nvar)], nvar)


def test_pairwise_mi_normalized_against_reference_values():
    """pairwise_mi(normalize=True) = normalize_mi of the reference's pairwise
    result (golden), within the estimate tolerance."""
    case = next(c for c in DCASES if str(c["name"]) == "drv_pairwise")
    args = [_py(case[f"arg{i}"]) for i in range(4) if f"arg{i}" in case]
    kw = {k[3:]: _py(v) for k, v in case.items() if k.startswith("kw_")}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        res = eg.pairwise_mi(*args, normalize=True, **kw)
    gold = case["result"]
    with np.errstate(invalid="ignore"):
        ref = np.where(gold <= 0.0, gold, np.sqrt(1 - np.exp(-2 * gold)))
    assert np.allclose(res, ref, rtol=0, atol=1e-10, equal_nan=True)
