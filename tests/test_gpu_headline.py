"""Parity at the two headline configurations, against the live reference.

tests/golden/golden_headline.json was made by tests/golden/make_golden.py
--headline from the reference (ennemi's estimator functions and public
estimate_mi over SciPy's cKDTree) on the same seeded inputs.  It holds the
reference's estimate of every task and SHA-256 digests of the inputs, of eps
and of each neighbour-count array, so the whole N = 1,000,000 batch is pinned
without committing its arrays:

* the single estimate_mi(y, x) of a bivariate Gaussian (rho = 0.6,
  N = 10,000, k = 3) through the public path, preprocessing included
  (_driver.py:229, :871-902 of the reference);
* the large-sample batch -- four KSG MI (rho = 0, .3, .6, .9) and one
  Frenzel-Pompe CMI, N = 1,000,000, k = 3 (_entropy_estimators.py:69-113,
  :116-156) -- on the default FP32-screen path, the all-FP64 comparator and
  the CTA-item grid layout.

The bar: inputs and eps bit for bit, counts exactly, estimates within
1e-10 nats.
"""

import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

HEADLINE = json.load(open(os.path.join(GOLDEN, "golden_headline.json")))
TOL = 1e-10


def digest(arr, dtype) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr, dtype=dtype).tobytes()).hexdigest()


def check_arrays(gold, fetched, label):
    """fetched: {'eps': float64[n], 'nx': int64[n], ...} against the digests."""
    for name, arr in fetched.items():
        if name == "eps":
            assert digest(arr, "<f8") == gold["eps"], (
                f"{label}: eps differs (sum {float(np.sum(arr))!r}, reference {gold['eps_sum']!r})")
        else:
            assert digest(arr, "<i8") == gold[name], (
                f"{label}: {name} differs (sum {int(np.sum(arr))}, reference {gold[name + '_sum']})")


def test_plain_ksg_through_public_api():
    import ennemi_gb300 as eg
    from ennemi_gb300 import _driver, synthetic
    from ennemi_gb300 import _native as N

    c = HEADLINE["plain_ksg"]
    n, k = c["n"], c["k"]
    x, y = synthetic.plain_ksg(n, c["seed"], c["rho"])
    assert digest(x, "<f8") == c["inputs"]["x"] and digest(y, "<f8") == c["inputs"]["y"], \
        "the synthetic generator produced other inputs than the reference saw"
    old = _driver.run_flags
    _driver.run_flags = N.KEEP_INTERNALS
    try:
        value = float(np.asarray(eg.estimate_mi(y, x, k=k)).item())
        prepared = {"x": N.fetch(0, 16, n), "y": N.fetch(0, 17, n)}
        fetched = {"eps": N.fetch(0, 0, n), "nx": N.fetch(0, 1, n), "ny": N.fetch(0, 2, n)}
    finally:
        _driver.run_flags = old
    for name, arr in prepared.items():
        assert digest(arr, "<f8") == c["prepared"][name], f"preprocessed {name} differs"
    check_arrays(c, fetched, "plain KSG")
    assert abs(value - c["value"]) <= TOL, (value, c["value"])
    # the estimator's sanity value: the analytic Gaussian MI
    assert abs(value - c["analytic"]) < 0.05


@pytest.fixture(scope="module")
def large_batch():
    from ennemi_gb300 import synthetic
    g = HEADLINE["large_sample"]
    work = synthetic.large_sample(g["n"], g["seed"])
    for (kind, cols), t in zip(work, g["tasks"]):
        assert kind == t["kind"]
        assert [digest(c, "<f8") for c in cols] == t["inputs"], \
            "the synthetic generator produced other inputs than the reference saw"
    return g, work


@pytest.mark.parametrize("variant", ["default", "plain_fp64", "cta_grid"])
def test_large_sample_batch(large_batch, variant):
    import torch
    from ennemi_gb300 import _native as N

    g, work = large_batch
    k, n = g["k"], g["n"]
    flags = {"default": 0, "plain_fp64": N.PLAIN_FP64, "cta_grid": N.FORCE_CTA_GRID}[variant]
    dcols = [[torch.from_numpy(c).cuda() for c in cols] for _, cols in work]
    tasks = []
    for (kind, _), dc in zip(work, dcols):
        if kind == "mi":
            tasks.append(N.Task(N.MI, k, [dc[0]], [dc[1]], n=n))
        else:
            tasks.append(N.Task(N.CMI, k, [dc[0]], [dc[1]], [dc[2]], n=n))
    values = N.run_tasks(tasks, flags=flags | N.INPUT_DEVICE | N.KEEP_INTERNALS)
    for t, (gold, (kind, _)) in enumerate(zip(g["tasks"], work)):
        slots = ["nx", "ny"] if kind == "mi" else ["nxz", "nyz", "nz"]
        fetched = {"eps": N.fetch(t, 0, n)}
        for s, name in enumerate(slots):
            fetched[name] = N.fetch(t, 1 + s, n)
        check_arrays(gold, fetched, f"{variant} task {t} ({kind})")
        assert abs(values[t] - gold["value"]) <= TOL, (t, values[t], gold["value"])
