"""Layout policy on the GPU: every table gives the same results bit for bit,
the tuner picks a measured mode, invalid tables are rejected, and a saved
table is installed when a context is made."""

import numpy as np
import pytest

from ennemi_gb300 import _native as N
from ennemi_gb300 import autotune as A

pytestmark = pytest.mark.gpu


def _tasks(n, seed):
    rng = np.random.default_rng(seed)
    c = [rng.normal(size=n) for _ in range(4)]
    c[1] = c[1] + 0.5 * c[0]
    lab = rng.integers(0, 3, n).astype(np.int32)
    return [N.Task(N.MI, 3, [c[0]], [c[1]], n=n),
            N.Task(N.CMI, 3, [c[0]], [c[1]], [c[2], c[3]], n=n),
            N.Task(N.CMI, 9, [c[0]], [c[1]], [c[2]], n=n),
            N.Task(N.SEMI, 3, [c[0], c[1]], labels=lab, nclass=3, n=n),
            N.Task(N.ENTROPY, 3, [c[0], c[1], c[2]], n=n)]


@pytest.mark.parametrize("n", [3000, 20000])
def test_every_policy_gives_identical_results(n):
    ctx = N.context()
    tasks = _tasks(n, n)
    ctx.set_policy(None)
    base = N.run_tasks(tasks)
    try:
        for mode in (N.MODE_BRUTE, N.MODE_SLAB, N.MODE_GRID, N.MODE_WARP_GRID, N.MODE_RANK):
            ctx.set_policy(np.full(N.POLICY_ENTRIES, mode, dtype=np.int8))
            assert np.array_equal(N.run_tasks(tasks), base), mode
        mixed = np.random.default_rng(1).integers(-1, 5, N.POLICY_ENTRIES).astype(np.int8)
        ctx.set_policy(mixed)
        assert np.array_equal(ctx.get_policy(), mixed)
        assert np.array_equal(N.run_tasks(tasks), base)
    finally:
        ctx.set_policy(None)


def test_invalid_policy_rejected():
    ctx = N.context()
    bad = np.zeros(N.POLICY_ENTRIES, dtype=np.int8)
    bad[3] = 5
    with pytest.raises(RuntimeError, match="invalid mode"):
        ctx.set_policy(bad)
    assert np.all(ctx.get_policy() == N.MODE_AUTO)


def test_tuner_measures_and_installs(tmp_path):
    ctx = N.context()
    report = {}
    tasks = _tasks(6000, 3)
    table = A.autotune(tasks=tasks, save_to=str(tmp_path / "policy.json"), repeats=1,
                       report=report)
    try:
        assert report and np.array_equal(ctx.get_policy(), table)
        for search, d, K, length in A.job_classes(tasks):
            assert table[N.policy_index(search, d, K, length)] in A.MODES
        assert np.array_equal(A.load(str(tmp_path / "policy.json")), table)
        ctx.set_policy(None)
        base = N.run_tasks(tasks)
        ctx.set_policy(table)
        assert np.array_equal(N.run_tasks(tasks), base)
    finally:
        ctx.set_policy(None)


def test_saved_policy_loaded_by_new_context(tmp_path, monkeypatch):
    table = np.full(N.POLICY_ENTRIES, N.MODE_SLAB, dtype=np.int8)
    path = str(tmp_path / "p.json")
    A.save(table, path)
    monkeypatch.setenv(A.CACHE_ENV, path)
    ctx = N.Context(0)
    try:
        assert A.load_cached(ctx)
        assert np.array_equal(ctx.get_policy(), table)
    finally:
        ctx.close()


def test_policy_change_replans_a_replayed_batch():
    torch = pytest.importorskip("torch")
    ctx = N.context()
    rng = np.random.default_rng(4)
    n = 6000
    cols = [torch.from_numpy(rng.normal(size=n)).cuda() for _ in range(2)]
    tasks = [N.Task(N.MI, 3, [cols[0]], [cols[1]], n=n)]
    flags = N.INPUT_DEVICE | N.GRAPH
    try:
        ctx.set_policy(None)
        a = N.run_tasks(tasks, flags=flags)
        b = N.run_tasks(tasks, flags=flags)          # replayed without planning
        grid_pairs = ctx.stats()["knn_tile_pairs"]
        ctx.set_policy(np.full(N.POLICY_ENTRIES, N.MODE_BRUTE, dtype=np.int8))
        c = N.run_tasks(tasks, flags=flags)          # planned again: brute force
        assert ctx.stats()["knn_tile_pairs"] >= n * n > grid_pairs
        assert np.array_equal(a, b) and np.array_equal(a, c)
    finally:
        ctx.set_policy(None)
