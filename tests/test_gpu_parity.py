"""GPU parity: eps bit for bit, counts exactly, estimates within 1e-10 nats.

Against (1) the golden vectors made by the live reference (cKDTree) and (2)
the CPU oracle at sizes that have no fixture, for every kernel variant: the
FP32 filter with FP64 recheck (default) and all-FP64 (plain), each as brute
force and as sorted slab.
"""

import numpy as np
import pytest

from ennemi_gb300 import _entropy_estimators as E
from ennemi_gb300 import _native as N
from conftest import estimator_cases, inputs_of, outputs_of

pytestmark = pytest.mark.gpu

CASES = estimator_cases()
VARIANTS = {
    "fp32": 0,
    "fp32-brute": N.FORCE_BRUTE,
    "fp32-slab": N.FORCE_SLAB,
    "fp32-grid": N.FORCE_GRID,
    "fp32-ctagrid": N.FORCE_GRID | N.FORCE_CTA_GRID,
    "fp32-rank": N.FORCE_RANK,
    "fp64-brute": N.PLAIN_FP64 | N.FORCE_BRUTE,
    "fp64-slab": N.PLAIN_FP64 | N.FORCE_SLAB,
    "fp64-grid": N.PLAIN_FP64 | N.FORCE_GRID,
}
SLOTS = {"mi": ["nx", "ny"], "cmi": ["nxz", "nyz", "nz"], "semi": ["n"],
         "csemi": ["nxz", "nyz", "nz"], "ent": [],
         "dent": ["c"], "dmi": ["cxy", "cx", "cy"], "dcmi": ["cxyz", "cxz", "cyz", "cz"]}
TOL = 1e-10  # nats


def make_task(kind, k, inp):
    if kind == "mi":
        return E.mi_task(inp["x"], inp["y"], k)
    if kind == "cmi":
        return E.cmi_task(inp["x"], inp["y"], inp["z"], k)
    if kind == "semi":
        return E.semidiscrete_task(inp["x"], inp["y"], k)
    if kind == "csemi":
        return E.conditional_semidiscrete_task(inp["x"], inp["y"], inp["z"], k)
    if kind == "dent":
        return E.discrete_entropy_task(inp["x"])
    if kind == "dmi":
        return E.discrete_mi_task(inp["x"], inp["y"])
    if kind == "dcmi":
        return E.discrete_cmi_task(inp["x"], inp["y"], inp["z"])
    return E.entropy_task(inp["x"], k)


def same_value(a, b, tol=TOL):
    if np.isnan(a) or np.isnan(b):
        return np.isnan(a) and np.isnan(b)
    if np.isinf(a) or np.isinf(b):
        return a == b
    return abs(a - b) <= tol


def check_internals(i, kind, n, eps_ref, counts_ref):
    if eps_ref is not None:
        eps = N.fetch(i, 0, n)
        assert np.array_equal(eps.view(np.uint64), np.asarray(eps_ref, np.float64).view(np.uint64)), \
            f"eps differs at {np.flatnonzero(eps != eps_ref)[:10]}"
    for s, name in enumerate(SLOTS[kind]):
        c = N.fetch(i, 1 + s, n)
        ref = np.asarray(counts_ref[name]).astype(np.int64)
        assert np.array_equal(c, ref), f"{name} differs at {np.flatnonzero(c != ref)[:10]}"


@pytest.mark.parametrize("variant", list(VARIANTS))
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_golden_estimators(case, variant):
    kind, k = str(case["kind"]), int(case["k"])
    inp = inputs_of(case)
    task = make_task(kind, k, inp)
    vals = N.run_tasks([task], flags=VARIANTS[variant] | N.KEEP_INTERNALS)
    gold = outputs_of(case)
    check_internals(0, kind, task.n, gold.get("eps"), gold)
    assert same_value(vals[0], float(case["value"])), (vals[0], float(case["value"]))


@pytest.mark.parametrize("variant", ["fp32", "fp64-slab", "fp32-grid", "fp32-rank"])
def test_golden_all_in_one_batch(variant):
    tasks = [make_task(str(c["kind"]), int(c["k"]), inputs_of(c)) for c in CASES]
    vals = N.run_tasks(tasks, flags=VARIANTS[variant] | N.KEEP_INTERNALS)
    for i, c in enumerate(CASES):
        gold = outputs_of(c)
        check_internals(i, str(c["kind"]), tasks[i].n, gold.get("eps"), gold)
        assert same_value(vals[i], float(c["value"])), c["name"]


def _oracle_case(O, kind, k, inp):
    with np.errstate(all="ignore"):
        if kind == "mi":
            return O.ksg_mi(inp["x"], inp["y"], k)
        if kind == "cmi":
            return O.cmi(inp["x"], inp["y"], inp["z"], k)
        if kind == "semi":
            return O.semidiscrete_mi(inp["x"], inp["y"], k)
        if kind == "csemi":
            return O.conditional_semidiscrete_mi(inp["x"], inp["y"], inp["z"], k)
        return O.entropy(inp["x"], k)


def _medium_cases():
    rng = np.random.default_rng(2024)
    n = 20000
    g = rng.multivariate_normal([0, 0], [[1, 0.6], [0.6, 1]], size=n)
    yield "mi_gauss_20k", "mi", 3, dict(x=g[:, 0], y=g[:, 1])
    t = rng.standard_t(3, size=n)
    yield "mi_t3_lognormal_20k", "mi", 3, dict(x=t, y=np.exp(rng.normal(size=n)) + 0.1 * t)
    c3 = rng.multivariate_normal([0, 0, 0], [[1, .5, .4], [.5, 1, .4], [.4, .4, 1]], size=n)
    yield "cmi_gauss3_20k", "cmi", 3, dict(x=c3[:, 0], y=c3[:, 1], z=c3[:, 2:])
    c4 = rng.normal(size=(12000, 4))
    yield "cmi_dz2_12k_k5", "cmi", 5, dict(x=c4[:, 0], y=c4[:, 1] + c4[:, 0], z=c4[:, 2:])
    cls = rng.choice(5, p=[0.5, 0.2, 0.2, 0.08, 0.02], size=n)
    yield "semi_x2_5cls_20k", "semi", 3, dict(x=rng.normal(size=(n, 2)) + cls[:, None] * 0.3, y=cls)
    cls2 = (rng.uniform(size=15000) * 3).astype(int)
    yield "csemi_15k", "csemi", 2, dict(x=rng.normal(size=15000) + cls2, y=cls2,
                                          z=rng.normal(size=(15000, 1)))
    yield "ent_3d_20k", "ent", 3, dict(x=rng.normal(size=(n, 3)))
    yield "ent_1d_20k_k40", "ent", 40, dict(x=rng.normal(size=n))
    yield "mi_k40_8k", "mi", 40, dict(x=g[:8000, 0], y=g[:8000, 1])
    yield "mi_rounded_20k", "mi", 3, dict(x=np.round(g[:, 0], 2), y=np.round(g[:, 1], 2))
    yield "ent_9d_3k", "ent", 4, dict(x=rng.normal(size=(3000, 9)))
    big = rng.normal(size=(5000, 2))
    yield "mi_huge_unsafe32_5k", "mi", 3, dict(x=1e300 * big[:, 0], y=big[:, 1])
    # nested-cell grids (d >= 3): generic d, heavy ties, K = 8, 4-D counts
    yield "ent_5d_12k", "ent", 3, dict(x=rng.normal(size=(12000, 5)))
    c3r = np.round(c3, 1)
    yield "cmi_rounded3_20k", "cmi", 3, dict(x=c3r[:, 0], y=c3r[:, 1], z=c3r[:, 2:])
    yield "ent_3d_k7_20k", "ent", 7, dict(x=rng.standard_t(4, size=(n, 3)))
    c6 = rng.normal(size=(10000, 5))
    yield "cmi_dz3_10k", "cmi", 3, dict(x=c6[:, 0], y=c6[:, 1] + 0.5 * c6[:, 2], z=c6[:, 2:])
    # walk kNN / key-range counts: exact duplicates (K-th distance 0, counts
    # with negative radius), K = 8 in 2-D, a job just above the grid size
    dup = rng.integers(0, 40, size=(20000, 2)).astype(np.float64)
    yield "mi_duplicates_20k", "mi", 3, dict(x=dup[:, 0], y=dup[:, 1])
    yield "mi_k7_20k", "mi", 7, dict(x=g[:, 0], y=g[:, 1] ** 3)
    yield "mi_4100", "mi", 3, dict(x=g[:4100, 0], y=g[:4100, 1])
    yield "cmi_dup_z_15k", "cmi", 3, dict(x=c3[:15000, 0], y=c3[:15000, 1],
                                           z=np.round(c3[:15000, 2:], 0))
    # ball ends from FP32 brackets: values far below the FP32 normal range
    # (bracket holds everything -> exact path), scales spread over 40 decades,
    # and balls whose left end crosses zero
    yield "mi_tiny_scales_12k", "mi", 3, dict(x=1e-30 * g[:12000, 0], y=1e-42 * g[:12000, 1])
    spread = 10.0 ** rng.uniform(-20, 20, size=n)
    yield "mi_spread_scales_20k", "mi", 3, dict(x=g[:, 0] * spread, y=g[:, 1])
    near0 = np.concatenate([rng.uniform(-1e-3, 1e-3, size=10000), rng.normal(size=10000)])
    yield "cmi_near_zero_20k", "cmi", 3, dict(x=near0, y=near0[::-1] + 0.1 * g[:, 1],
                                               z=np.abs(near0)[:, None])


MEDIUM = list(_medium_cases())


@pytest.mark.parametrize("variant", ["fp32", "fp32-brute", "fp32-slab", "fp32-ctagrid", "fp64-grid"])
@pytest.mark.parametrize("case", MEDIUM, ids=[c[0] for c in MEDIUM])
def test_medium_against_oracle(oracle, case, variant):
    name, kind, k, inp = case
    ref_value, ref = _oracle_case(oracle, kind, k, inp)
    task = make_task(kind, k, inp)
    vals = N.run_tasks([task], flags=VARIANTS[variant] | N.KEEP_INTERNALS)
    check_internals(0, kind, task.n, ref["eps"], ref)
    assert same_value(vals[0], ref_value), (vals[0], ref_value)


def test_ball_count_radius_on_exact_distances(oracle):
    """Radii equal to exact coordinate distances of dyadic data: every
    boundary is a tie that the inclusive test keeps."""
    rng = np.random.default_rng(11)
    for d in [1, 2]:
        pts = rng.integers(-4000, 4000, size=(9000, d)) / 64.0
        r = rng.integers(0, 200, size=9000) / 64.0
        r[::50] = 0.0
        r[7::50] = -0.0
        cnt = N.ball_count(pts, r)
        assert np.array_equal(cnt, oracle.ball_count(pts, r)), d


def test_primitives_against_oracle(oracle):
    rng = np.random.default_rng(5)
    for d in [1, 2, 3, 6]:
        pts = rng.normal(size=(7000, d))
        for k in [1, 3, 50]:
            eps = N.knn_eps(pts, k)
            assert np.array_equal(eps, oracle.knn_eps(pts, k)), (d, k)
        r = np.abs(rng.normal(0.05, 0.05, size=7000))
        r[::97] = -1e-13
        r[5] = np.inf
        cnt = N.ball_count(pts, r)
        assert np.array_equal(cnt, oracle.ball_count(pts, r)), d


def test_device_input_matches_host_input():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    x = rng.normal(size=30000)
    y = 0.5 * x + rng.normal(size=30000)
    host = N.run_tasks([E.mi_task(x, y, 3)])
    xd = torch.from_numpy(x).cuda()
    yd = torch.from_numpy(y).cuda()
    dev = N.run_tasks([N.Task(N.MI, 3, [xd], [yd], n=30000)], flags=N.INPUT_DEVICE)
    assert host[0] == dev[0]


def test_host_columns_read_in_place_match_staged_copies():
    """Contiguous host columns may be read by the gather kernel in place
    (devices that read pageable memory); strided, shared and class-permuted
    columns are staged.  Every route gives the same bits."""
    rng = np.random.default_rng(23)
    n = 40000
    a = rng.normal(size=n)
    b = 0.6 * a + rng.normal(size=n)
    m = rng.normal(size=(n, 3))                     # strided column views
    m[:, 1] += 0.5 * m[:, 0]
    lab = rng.integers(0, 4, size=n).astype(np.int32)
    s = a + 0.3 * lab
    tasks = [E.mi_task(a, b, 3),
             N.Task(N.MI, 3, [m[:, 0]], [m[:, 1]], n=n),
             N.Task(N.CMI, 3, [a], [m[:, 1]], [b], n=n),
             N.Task(N.CMI, 4, [m[:, 0], m[:, 2]], [b], [a], n=n),
             N.Task(N.SEMI, 3, [s], labels=lab, nclass=4, n=n),
             N.Task(N.ENTROPY, 3, [b, a], n=n)]
    for extra in (0, N.GRAPH):
        staged = N.run_tasks(tasks, flags=N.STAGE_HOST | extra)
        default = N.run_tasks(tasks, flags=extra)
        assert np.array_equal(staged, default), extra
    # odd lengths, and a column 8 bytes off a 16-byte boundary (read one
    # value per request instead of pairs)
    n2 = 40001
    buf = np.empty(n2 + 1)
    off = buf[1:]
    off[:] = rng.normal(size=n2)
    c = rng.normal(size=n2) + 0.4 * off
    assert c.ctypes.data % 16 == 0 and off.ctypes.data % 16 == 8
    odd = [E.mi_task(c, off, 3), E.cmi_task(off, c, c[::-1].copy(), 3), E.entropy_task(c, 3)]
    assert np.array_equal(N.run_tasks(odd, flags=N.STAGE_HOST), N.run_tasks(odd))
    pts = np.ascontiguousarray(m[:, :2])
    r = N.knn_eps(pts, 3)
    assert np.array_equal(r, N.knn_eps(pts, 3, flags=N.STAGE_HOST))
    assert np.array_equal(N.ball_count(pts, r - 1e-12),
                          N.ball_count(pts, r - 1e-12, flags=N.STAGE_HOST))


def test_public_estimators_on_gpu():
    rng = np.random.default_rng(0)
    cov = [[1, 0.6], [0.6, 1]]
    d = rng.multivariate_normal([0, 0], cov, size=4000)
    mi = E._estimate_single_mi(d[:, 0], d[:, 1], 3)
    assert abs(mi - (-0.5 * np.log(1 - 0.36))) < 0.03
    h = E._estimate_single_entropy(d[:, 0])
    assert abs(h - 0.5 * np.log(2 * np.pi * np.e)) < 0.05


def _tie_cases():
    """Columns whose sort keys tie in their high 48 bits (values within a
    relative 2^-36): the six-pass sort repairs short runs in place and sends
    a long run out of order to the full sort; long runs already in order
    (exact duplicates, or ascending input) need neither."""
    rng = np.random.default_rng(31)
    n = 6000
    v = rng.normal(size=n // 3)
    near = np.concatenate([v, np.nextafter(v, np.inf), np.nextafter(np.nextafter(v, -np.inf), -np.inf)])
    yield "short_runs", rng.permutation(near), 6
    yield "long_run_shuffled", 1.0 + rng.permutation(n) * 2.0 ** -52, 8
    yield "long_run_ascending", 1.0 + np.arange(n) * 2.0 ** -52, 6
    yield "duplicates", rng.integers(0, 7, size=n).astype(np.float64), 6
    mixed = rng.normal(size=n)
    mixed[: n // 2] = 3.0 + rng.permutation(n // 2) * 2.0 ** -51
    yield "half_long_run", rng.permutation(mixed), 8


TIES = list(_tie_cases())


@pytest.mark.parametrize("kind", ["mi", "ent", "cmi"])
@pytest.mark.parametrize("case", TIES, ids=[c[0] for c in TIES])
def test_sort_ties_in_high_bits(oracle, case, kind):
    name, x, passes = case
    rng = np.random.default_rng(5)
    n = len(x)
    y = rng.normal(size=n) + 0.5 * np.argsort(np.argsort(x)) / n
    inp = dict(x=x, y=y, z=rng.normal(size=(n, 1)) + x[:, None] * 0)
    if kind == "ent":
        inp = dict(x=x)
    ref_value, ref = _oracle_case(oracle, kind, 3, inp)
    task = make_task(kind, 3, inp)
    ctx = N.context(0)
    vals = N.run_tasks([task], flags=N.KEEP_INTERNALS)
    assert ctx.stats()["sort_passes"] == passes
    check_internals(0, kind, task.n, ref["eps"], ref)
    assert same_value(vals[0], ref_value), (vals[0], ref_value)


def test_graph_replay_matches_direct_launch():
    """The streaming pattern: capture once, then refill the same device
    buffers and replay without planning.  The expected values of both data
    sets are computed first, by direct launches on other buffers, so that no
    other batch runs on the context between the graph calls."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    n = 50000
    host_a = [rng.normal(size=n) for _ in range(3)]
    host_b = [host_a[0], 0.7 * host_a[0] + rng.normal(size=n), host_a[2]]

    def tasks_of(cols):
        return [N.Task(N.MI, 3, [cols[0]], [cols[1]], n=n),
                N.Task(N.CMI, 3, [cols[0]], [cols[1]], [cols[2]], n=n)]
    ctx = N.context(0)
    direct_a = N.run_tasks(tasks_of([torch.from_numpy(c).cuda() for c in host_a]), flags=N.INPUT_DEVICE)
    direct_b = N.run_tasks(tasks_of([torch.from_numpy(c).cuda() for c in host_b]), flags=N.INPUT_DEVICE)
    assert not np.array_equal(direct_a, direct_b)

    cols = [torch.from_numpy(c).cuda() for c in host_a]
    tasks = tasks_of(cols)
    first = N.run_tasks(tasks, flags=N.INPUT_DEVICE | N.GRAPH)   # plans and captures
    st = ctx.stats()
    assert st["planned"] == 1 and st["graph"] == 1
    again = N.run_tasks(tasks, flags=N.INPUT_DEVICE | N.GRAPH)   # replays, no planning
    st = ctx.stats()
    assert st["planned"] == 0 and st["graph"] == 1
    assert np.array_equal(direct_a, first) and np.array_equal(direct_a, again)
    # new data in the same buffers: the replay (still without planning) reads them
    cols[1].copy_(torch.from_numpy(host_b[1]))
    torch.cuda.synchronize()
    replay_b = N.run_tasks(tasks, flags=N.INPUT_DEVICE | N.GRAPH)
    st = ctx.stats()
    assert st["planned"] == 0 and st["graph"] == 1
    assert np.array_equal(direct_b, replay_b)


def test_tasks_sharing_columns_match_tasks_alone():
    """Tasks that read the same caller columns share their sort segments and
    rank-space matrices in one batch; every result equals the task run alone
    (eps bit for bit, counts exactly)."""
    rng = np.random.default_rng(31)
    n = 20000
    a, b, c = rng.normal(size=(3, n))
    b += 0.5 * a
    z = rng.normal(size=(n, 2))
    z1, z2 = np.ascontiguousarray(z[:, 0]), np.ascontiguousarray(z[:, 1])
    tasks = [N.Task(N.MI, 3, [a], [b], n=n), N.Task(N.MI, 3, [a], [c], n=n),
             N.Task(N.MI, 3, [b], [c], n=n), N.Task(N.MI, 3, [c], [a], n=n),
             N.Task(N.CMI, 3, [a], [b], [z1], n=n), N.Task(N.CMI, 3, [a], [c], [z1], n=n),
             N.Task(N.CMI, 3, [a], [b], [z1, z2], n=n), N.Task(N.CMI, 3, [b], [c], [z1, z2], n=n),
             N.Task(N.ENTROPY, 3, [a, z1], n=n)]
    slots = {N.MI: 2, N.CMI: 3, N.ENTROPY: 0}
    together = N.run_tasks(tasks, flags=N.KEEP_INTERNALS)
    kept = [[N.fetch(i, w, n) for w in range(1 + slots[t.kind])] for i, t in enumerate(tasks)]
    for i, t in enumerate(tasks):
        alone = N.run_tasks([t], flags=N.KEEP_INTERNALS)
        assert alone[0] == together[i], i
        for w in range(1 + slots[t.kind]):
            assert np.array_equal(N.fetch(0, w, n), kept[i][w]), (i, w)


@pytest.mark.parametrize("kind", ["dent", "dmi", "dcmi"])
def test_discrete_estimators_and_warnings(oracle, kind):
    """The device group-by against the oracle's counts on data with many
    levels, -0 / +0 and wide values; the reference's too-many-levels
    warnings, counted from the device's distinct-value figures."""
    import warnings
    rng = np.random.default_rng(61)
    n = 30000
    x = rng.integers(-500, 500, size=n).astype(np.float64) * 1e9
    x[::7] = -0.0
    x[3::7] = 0.0
    y = rng.integers(0, 3, size=n).astype(np.float64)
    z = rng.integers(0, 40, size=(n, 2)).astype(np.float64)
    if kind == "dent":
        task, (v_ref, arrs) = E.discrete_entropy_task(np.column_stack((x, y))), \
            oracle.discrete_entropy(np.column_stack((x, y)))
        slots, expect_warn = ["c"], 0
    elif kind == "dmi":
        task, (v_ref, arrs) = E.discrete_mi_task(x, y), oracle.discrete_mi(x, y)
        slots = ["cxy", "cx", "cy"]
        expect_warn = int(arrs["groups"][1] > n / 4) + int(arrs["groups"][2] > n / 4)
    else:
        task, (v_ref, arrs) = E.discrete_cmi_task(x, y, z), oracle.conditional_discrete_mi(x, y, z)
        slots = ["cxyz", "cxz", "cyz", "cz"]
        expect_warn = int(arrs["groups"][4] + arrs["groups"][5])
    groups = {}
    v = N.run_tasks([task], flags=N.KEEP_INTERNALS, groups_out=groups)[0]
    for s, name in enumerate(slots):
        assert np.array_equal(N.fetch(0, 1 + s, n), arrs[name]), name
    assert abs(v - v_ref) <= 1e-10, (v, v_ref)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        E.discrete_warnings(task, groups[0])
    assert len(w) == expect_warn
    assert list(groups[0][:len(slots)]) == [int(g) for g in arrs["groups"][:len(slots)]]
