"""The CPU oracle reproduces the reference exactly on the golden vectors.

tests/golden/*.npz were generated from the live reference (ennemi +
scipy.spatial.cKDTree) by tests/golden/make_golden.py.  Pinning the oracle to
them makes it a trustworthy checker for the GPU parity tests at sizes that
have no fixture: eps must match bit for bit, neighbour counts exactly and the
estimate to 1e-12 (same formula, same summation in NumPy).
"""

import numpy as np
import pytest
from scipy.special import psi as scipy_psi

from conftest import estimator_cases, inputs_of, outputs_of

CASES = estimator_cases()


def _run(O, kind, k, inp):
    with np.errstate(all="ignore"):
        if kind == "mi":
            return O.ksg_mi(inp["x"], inp["y"], k)
        if kind == "cmi":
            return O.cmi(inp["x"], inp["y"], inp["z"], k)
        if kind == "semi":
            return O.semidiscrete_mi(inp["x"], inp["y"], k)
        if kind == "csemi":
            return O.conditional_semidiscrete_mi(inp["x"], inp["y"], inp["z"], k)
        if kind == "ent":
            return O.entropy(inp["x"], k)
        if kind == "dent":
            return O.discrete_entropy(inp["x"])
        if kind == "dmi":
            return O.discrete_mi(inp["x"], inp["y"])
        if kind == "dcmi":
            return O.conditional_discrete_mi(inp["x"], inp["y"], inp["z"])
    raise ValueError(kind)


def same_value(a, b, tol=1e-12):
    if np.isnan(a) or np.isnan(b):
        return np.isnan(a) and np.isnan(b)
    if np.isinf(a) or np.isinf(b):
        return a == b
    return abs(a - b) <= tol


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference(oracle, case):
    kind, k = str(case["kind"]), int(case["k"])
    value, arrays = _run(oracle, kind, k, inputs_of(case))
    arrays.pop("groups", None)
    gold = outputs_of(case)
    assert set(arrays) == set(gold)
    for key, arr in arrays.items():
        if key == "eps":
            assert np.array_equal(arr.view(np.uint64), gold[key].astype(np.float64).view(np.uint64)), key
        else:
            assert np.array_equal(arr, gold[key]), key
    assert same_value(value, float(case["value"])), (value, float(case["value"]))


def test_oracle_psi_matches_scipy(oracle):
    # the reference's own check (tests/unit/test_entropy_estimators.py:408-422)
    n = np.arange(1, 10000)
    assert np.max(np.abs(oracle.psi(n) - scipy_psi(n))) < 1e-4
    assert np.isinf(oracle.psi(np.array([3, 0, 2])))


def test_golden_cover_edge_cases():
    names = {c["name"] for c in CASES}
    # duplicates (-inf), tiny n, large k, heavy tails, big offsets, lattices,
    # string labels, a class smaller than k + 1, 7-D condition
    for needle in ["duplicates", "n5_k4", "k100", "heavy", "offset", "lattice",
                   "strlabels", "tinyclass", "dz7"]:
        assert any(needle in n for n in names), needle
