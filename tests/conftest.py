"""Shared test set-up: the `gpu` marker, import paths and golden fixtures."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


def load_golden(name):
    """Cases of tests/golden/<name>.npz as a list of dicts."""
    g = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    cases = []
    for case in g["names"]:
        case = str(case)
        d = {"name": case}
        pre = case + "/"
        for key in g.files:
            if key.startswith(pre):
                d[key[len(pre):]] = g[key]
        cases.append(d)
    return cases


def estimator_cases():
    return load_golden("golden_estimators.npz")


def driver_cases():
    return load_golden("golden_driver.npz")


def inputs_of(case):
    return {k[3:]: v for k, v in case.items() if k.startswith("in_")}


def outputs_of(case):
    return {k[4:]: v for k, v in case.items() if k.startswith("out_")}


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
