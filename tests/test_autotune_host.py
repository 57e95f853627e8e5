"""Host logic of the layout-policy autotuner (no GPU): the job classes a
batch plans, filling of unmeasured size classes, and the policy file."""

import json

import numpy as np

from ennemi_gb300 import _native as N
from ennemi_gb300 import autotune as A


def test_job_classes_follow_the_estimator_spaces():
    x = [np.zeros(100)] * 2
    mi = N.Task(N.MI, 3, x[:1], x[:1], n=100)
    cmi = N.Task(N.CMI, 3, x[:1], x[:1], x, n=100)
    semi = N.Task(N.SEMI, 5, x, labels=np.r_[np.zeros(60, int), np.ones(40, int)], nclass=2, n=100)
    ent = N.Task(N.ENTROPY, 3, x[:1], n=100)
    assert A.job_classes([mi]) == [(0, 2, 4, 100)]
    assert A.job_classes([cmi]) == [(0, 4, 4, 100), (1, 3, 0, 100), (1, 3, 0, 100), (1, 2, 0, 100)]
    assert A.job_classes([semi]) == [(0, 2, 6, 60), (0, 2, 6, 40), (1, 2, 0, 100)]
    assert A.job_classes([ent]) == []


def test_fill_takes_the_nearest_measured_size_class():
    table = np.full(N.POLICY_ENTRIES, N.MODE_AUTO, dtype=np.int8)
    A._fill(table, (0, 3, 4), {10: N.MODE_BRUTE, 14: N.MODE_WARP_GRID})
    get = lambda n: table[N.policy_index(0, 3, 4, n)]
    assert get(2) == N.MODE_BRUTE and get(1 << 11) == N.MODE_BRUTE
    assert get(1 << 12) == N.MODE_BRUTE          # tie: the smaller class
    assert get(1 << 13) == N.MODE_WARP_GRID and get(1 << 30) == N.MODE_WARP_GRID
    # other keys untouched
    assert table[N.policy_index(1, 3, 0, 1 << 13)] == N.MODE_AUTO
    assert table[N.policy_index(0, 3, 8, 1 << 13)] == N.MODE_AUTO


def test_policy_file_round_trip_and_rejects(tmp_path):
    rng = np.random.default_rng(0)
    table = rng.integers(-1, 4, N.POLICY_ENTRIES).astype(np.int8)
    path = str(tmp_path / "p" / "policy.json")
    A.save(table, path, {"note": "test"})
    assert np.array_equal(A.load(path), table)
    doc = json.load(open(path))
    doc["modes"][5] = 7
    json.dump(doc, open(path, "w"))
    assert A.load(path) is None
    json.dump({"entries": 3, "modes": [0, 0, 0]}, open(path, "w"))
    assert A.load(path) is None
    assert A.load(str(tmp_path / "absent.json")) is None


def test_cache_path_honours_environment(monkeypatch, tmp_path):
    monkeypatch.setenv(A.CACHE_ENV, str(tmp_path / "x.json"))
    assert A.cache_path(0) == str(tmp_path / "x.json")
