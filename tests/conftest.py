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


def oracle_run_tasks(O, calls=None):
    """A stand-in for _native.run_tasks that evaluates every task with the
    oracle O (tests only).  Appends the batch size to `calls` if given."""
    from ennemi_gb300 import _native

    class Result:
        def __init__(self, value, status):
            self.value, self.status = value, status

    def run(tasks, flags=0, device=0, results_out=None, noise=None, groups_out=None):
        if calls is not None:
            calls.append(len(tasks))
        out = []
        for ti, t in enumerate(tasks):
            if t.kind in _native.DISCRETE_KINDS:
                cols = [np.asarray(c) for c in list(t.x) + list(t.y) + list(t.z)]
                dx, dy = len(t.x), len(t.y)
                x = np.column_stack(cols[:dx])
                if t.kind == _native.DISCRETE_ENTROPY:
                    v, a = O.discrete_entropy(x)
                elif t.kind == _native.DISCRETE_MI:
                    v, a = O.discrete_mi(cols[0], cols[1])
                else:
                    v, a = O.conditional_discrete_mi(cols[0], cols[1], np.column_stack(cols[dx + dy:]))
                out.append(v)
                if groups_out is not None:
                    groups_out[ti] = [int(g) for g in a["groups"]]
                if results_out is not None:
                    results_out.append(Result(v, 0))
                continue
            n = t.n or (t.x[0].length if isinstance(t.x[0], _native.Col) else len(t.x[0]))
            ix = np.arange(n) if t.index is None else np.asarray(t.index)
            cols = [(c.ref if isinstance(c, _native.Col) else np.asarray(c))[ix]
                    for c in list(t.x) + list(t.y) + list(t.z)]
            if flags & _native.RESCALE and t.kind != _native.ENTROPY:
                # the library's EGB_RESCALE, as the reference's _rescale_data
                # computes it (x from noise position 0, then y, then z)
                nz = noise(n * len(cols))
                if any(np.abs(c.std()) < 1e-20 for c in cols):
                    out.append(np.nan)
                    if results_out is not None:
                        results_out.append(Result(np.nan, _native.TASK_CONSTANT))
                    continue
                nxy = len(t.x) + len(t.y)
                z = np.column_stack(cols[nxy:]) if len(t.z) else None
                cols = [(c - c.mean()) / c.std() + nz[i * n:(i + 1) * n] for i, c in enumerate(cols[:nxy])]
                if z is not None:   # (n, dz) along axis 0, noise row-major
                    z = (z - z.mean(axis=0)) / z.std(axis=0) + nz[nxy * n:].reshape(n, -1)[:, :z.shape[1]]
                    cols += [z[:, j] for j in range(z.shape[1])]
            dx, dy = len(t.x), len(t.y)
            x = np.column_stack(cols[:dx])
            y = np.column_stack(cols[dx:dx + dy]) if dy else None
            z = np.column_stack(cols[dx + dy:]) if len(t.z) else None
            with np.errstate(all="ignore"):
                if t.kind == _native.MI:
                    v = O.ksg_mi(x, y, t.k)[0]
                elif t.kind == _native.CMI:
                    v = O.cmi(x, y, z, t.k)[0]
                elif t.kind == _native.SEMI:
                    v = O.semidiscrete_mi(x, t.labels, t.k)[0]
                elif t.kind == _native.CSEMI:
                    v = O.conditional_semidiscrete_mi(x, t.labels, z, t.k)[0]
                else:
                    v = O.entropy(x, t.k)[0]
            out.append(v)
            if results_out is not None:
                results_out.append(Result(v, 0))
        return np.array(out)

    return run


def oracle_pairwise_matrix(values, pairs, nvar, normalize=False, device=0):
    """Stand-in for _native.pairwise_matrix on the host (tests only): the
    reference's matrix fill (_driver.py:716-721)."""
    out = np.full((nvar, nvar), np.nan)
    for (i, j), v in zip(pairs, values):
        out[i, j] = out[j, i] = oracle_normalize(np.asarray(v))[()] if normalize else v
    return out


def oracle_normalize(values, device=0):
    """Stand-in for _native.normalize on the host (tests only): the
    reference's _normalize (_driver.py:77-81) elementwise."""
    v = np.asarray(values, dtype=np.float64)
    with np.errstate(invalid="ignore"):
        return np.where(v <= 0.0, v, np.sqrt(1 - np.exp(-2 * v)))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
