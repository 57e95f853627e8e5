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
