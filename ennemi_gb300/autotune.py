"""Autotuner of the layout policy: which layout each multi-dimensional search
job runs in (brute-force tiles, slab, CTA grid or warp grid), chosen per
(search kind, dimension, K class, size class) by measurement on this GPU.

The reference has one layout (a cKDTree per space, _entropy_estimators.py);
here every layout returns the same distances and counts bit for bit, so the
policy changes speed only, never a result.

    tune(...)            measure and return a policy table (np.int8 array)
    tune_for_tasks(ts)   measure only the classes a task list uses
    autotune(...)        tune, install in the device's context, save to cache
    load_cached(ctx)     install a saved table (done when a context is made)

A measurement runs seeded Gaussian points through egb_knn_eps (kNN jobs) or
egb_ball_count (count jobs, radii = the k = 3 kNN distances of one more
Gaussian column, as a marginal count of the KSG estimators gets them) with the
table filled with one mode, and takes the device time of the call without the
upload (EGB_TIMING), best of `repeats`.  Size classes outside the measured
range inherit the nearest measured class.  Modes that were more than
`prune` times slower than the best at one size are not tried at larger ones
(brute force and slab work grows faster with the size than grid work).
"""

from __future__ import annotations

import json
import os
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as N

MODES = (N.MODE_BRUTE, N.MODE_SLAB, N.MODE_GRID, N.MODE_WARP_GRID, N.MODE_RANK)
MODE_NAMES = {N.MODE_AUTO: "auto", N.MODE_BRUTE: "brute", N.MODE_SLAB: "slab",
              N.MODE_GRID: "grid", N.MODE_WARP_GRID: "warp_grid", N.MODE_RANK: "rank"}
K_OF_CLASS = (4, 8, 16, 32)   # K = k + 1 measured for each kNN K class
CACHE_ENV = "ENNEMI_GB300_POLICY"

# (search, d, K) -> list of (size class, mode)
Key = Tuple[int, int, int]


def _dim_class_rep(d: int) -> int:
    return min(max(d, 2), 5)


def _k_class_rep(K: int) -> int:
    return 4 if K <= 4 else 8 if K <= 8 else 16 if K <= 16 else 32


def _device_ms(ctx: N.Context) -> float:
    t = ctx.timings()
    return t["total"] - t["upload"]


def _measure(ctx: N.Context, search: int, d: int, K: int, n: int, mode: int,
             repeats: int, rng_seed: int) -> float:
    rng = np.random.default_rng(rng_seed)
    table = np.full(N.POLICY_ENTRIES, mode, dtype=np.int8)
    if search == 0:
        pts = rng.standard_normal((n, d))
    else:
        joint = rng.standard_normal((n, d + 1))
        ctx.set_policy(None)
        radius = N.knn_eps(joint, 3, device=ctx.device) - 1e-12
        pts = np.ascontiguousarray(joint[:, :d])
    ctx.set_policy(table)
    best = np.inf
    for _ in range(repeats + 1):           # first call warms the arena
        if search == 0:
            N.knn_eps(pts, K - 1, flags=N.TIMING, device=ctx.device)
        else:
            N.ball_count(pts, radius, flags=N.TIMING, device=ctx.device)
        best = min(best, _device_ms(ctx))
    return best


def _tune_key(ctx, key: Key, size_classes: Sequence[int], repeats: int,
              prune: float, log) -> Dict[int, Tuple[int, Dict[int, float]]]:
    search, d, K = key
    alive = list(MODES)
    if search == 0 and K > 8:
        alive.remove(N.MODE_WARP_GRID)     # the warp grid runs kNN only for K <= 8
    if search == 0 or d != 2:
        alive.remove(N.MODE_RANK)          # rank-space counts: d = 2 ball counts only
    out = {}
    for sc in sorted(size_classes):
        n = int(round(2 ** (sc + 0.5)))
        if n <= K:
            continue
        times = {m: _measure(ctx, search, d, K, n, m, repeats, 1000 + sc) for m in alive}
        best_mode = min(times, key=times.get)
        out[sc] = (best_mode, times)
        if log:
            log(f"search={'knn' if search == 0 else 'count'} d={d} K={K} n={n}: " +
                " ".join(f"{MODE_NAMES[m]}={t:.3f}ms" for m, t in times.items()) +
                f" -> {MODE_NAMES[best_mode]}")
        alive = [m for m in alive if times[m] <= prune * times[best_mode]]
    return out


def _fill(table: np.ndarray, key: Key, chosen: Dict[int, int]) -> None:
    """Write chosen modes of one key; unmeasured size classes take the nearest."""
    if not chosen:
        return
    search, d, K = key
    measured = sorted(chosen)
    for sc in range(N.POLICY_SIZE_CLASSES):
        near = min(measured, key=lambda m: (abs(m - sc), m))
        table[N.policy_index(search, d, K, 1 << sc)] = chosen[near]


def tune(device: int = 0, searches: Iterable[int] = (0, 1), dims: Iterable[int] = (2, 3, 4, 5),
         ks: Iterable[int] = K_OF_CLASS, size_classes: Iterable[int] = range(8, 21),
         repeats: int = 2, prune: float = 4.0, keys: Optional[Iterable[Key]] = None,
         log=None, report: Optional[dict] = None) -> np.ndarray:
    """Measure the layouts and return a policy table (entries not measured stay
    EGB_MODE_AUTO).  `keys` overrides the (search, d, K) product of searches,
    dims and ks; `report` receives the measured times."""
    ctx = N.context(device)
    old = ctx.get_policy()
    size_classes = list(size_classes)
    if keys is None:
        keys = [(s, d, K) for s in searches for d in dims for K in (ks if s == 0 else (0,))]
    table = np.full(N.POLICY_ENTRIES, N.MODE_AUTO, dtype=np.int8)
    try:
        for key in keys:
            res = _tune_key(ctx, key, size_classes, repeats, prune, log)
            _fill(table, key, {sc: m for sc, (m, _) in res.items()})
            if report is not None:
                report[str(key)] = {int(sc): {MODE_NAMES[m]: t for m, t in times.items()}
                                    for sc, (_, times) in res.items()}
    finally:
        ctx.set_policy(old)
    return table


def job_classes(tasks: Sequence[N.Task]) -> List[Tuple[int, int, int, int]]:
    """(search, d, K, len) of the multi-dimensional jobs a batch plans.

    The spaces follow the estimators (_entropy_estimators.py): MI kNN over
    (x, y), counts over x and y; CMI kNN (x, y, z), counts (x, z), (y, z), z;
    SEMI kNN x within each class, count x over all; CSEMI kNN (x, z) within
    each class, counts (x, z) over all, z within each class and over all;
    entropy kNN x.
    """
    out = []
    for t in tasks:
        n = t.n or len(t.x[0])
        dx, dy, dz, K = len(t.x), len(t.y), len(t.z), t.k + 1
        if t.kind in (N.SEMI, N.CSEMI):
            sizes = np.bincount(np.asarray(t.labels)) if t.labels is not None else [n]
        jobs = []
        if t.kind == N.MI:
            jobs = [(0, dx + dy, n), (1, dx, n), (1, dy, n)]
        elif t.kind == N.CMI:
            jobs = [(0, dx + dy + dz, n), (1, dx + dz, n), (1, dy + dz, n), (1, dz, n)]
        elif t.kind == N.SEMI:
            jobs = [(0, dx, int(c)) for c in sizes if c > 0] + [(1, dx, n)]
        elif t.kind == N.CSEMI:
            jobs = ([(0, dx + dz, int(c)) for c in sizes if c > 0] + [(1, dx + dz, n)] +
                    [(1, dz, int(c)) for c in sizes if c > 0] + [(1, dz, n)])
        elif t.kind == N.ENTROPY:
            jobs = [(0, dx, n)]
        for search, d, length in jobs:
            if d >= 2:
                out.append((search, d, K if search == 0 else 0, length))
    return out


def tune_for_tasks(tasks: Sequence[N.Task], device: int = 0, repeats: int = 2,
                   base: Optional[np.ndarray] = None, log=None,
                   report: Optional[dict] = None) -> np.ndarray:
    """Measure only the (search, d, K, size) classes that `tasks` plan (size
    classes at and one below each job's), on top of `base` (default: all
    EGB_MODE_AUTO)."""
    groups: Dict[Key, set] = {}
    for search, d, K, length in job_classes(tasks):
        key = (search, _dim_class_rep(d), _k_class_rep(K) if search == 0 else 0)
        sc = max(int(length).bit_length() - 1, 0)
        groups.setdefault(key, set()).update({sc})
    table = (np.full(N.POLICY_ENTRIES, N.MODE_AUTO, dtype=np.int8) if base is None
             else np.array(base, dtype=np.int8))
    for key, scs in groups.items():
        part = tune(device, keys=[key], size_classes=sorted(scs), repeats=repeats, log=log,
                    report=report)
        # only the measured size classes of this key are taken over
        search, d, K = key
        for sc in scs:
            i = N.policy_index(search, d, K, 1 << sc)
            table[i] = part[i]
    return table


# ------------------------------------------------------------------ cache --

def cache_path(device: int = 0) -> str:
    """$ENNEMI_GB300_POLICY, else ~/.cache/ennemi_gb300/policy_<gpu>.json."""
    env = os.environ.get(CACHE_ENV)
    if env:
        return env
    name = N.context(device).device_name() if device in N._ctx else f"device{device}"
    tag = "".join(c if c.isalnum() else "_" for c in name)
    return os.path.join(os.path.expanduser("~"), ".cache", "ennemi_gb300", f"policy_{tag}.json")


def save(table: np.ndarray, path: str, meta: Optional[dict] = None) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    doc = {"entries": N.POLICY_ENTRIES, "modes": [int(m) for m in table], "meta": meta or {}}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(doc, f)
    os.replace(tmp, path)


def load(path: str) -> Optional[np.ndarray]:
    """The table saved at `path`, or None if absent or of another layout."""
    try:
        with open(path) as f:
            doc = json.load(f)
    except (OSError, ValueError):
        return None
    if doc.get("entries") != N.POLICY_ENTRIES or len(doc.get("modes", ())) != N.POLICY_ENTRIES:
        return None
    table = np.array(doc["modes"], dtype=np.int8)
    if table.min() < N.MODE_AUTO or table.max() > N.MODE_RANK:
        return None
    return table


def load_cached(ctx: N.Context) -> bool:
    env = os.environ.get(CACHE_ENV)
    tag = "".join(c if c.isalnum() else "_" for c in ctx.device_name())
    path = env or os.path.join(os.path.expanduser("~"), ".cache", "ennemi_gb300", f"policy_{tag}.json")
    table = load(path)
    if table is None:
        return False
    ctx.set_policy(table)
    return True


def autotune(device: int = 0, tasks: Optional[Sequence[N.Task]] = None, save_to: Optional[str] = "",
             log=None, **kw) -> np.ndarray:
    """Tune (all classes, or the classes of `tasks`), install the table in the
    device's context and save it (save_to "" = cache_path(device), None = no
    file).  Returns the table."""
    ctx = N.context(device)
    if tasks is not None:
        table = tune_for_tasks(tasks, device=device, base=ctx.get_policy(), log=log, **kw)
    else:
        table = tune(device, log=log, **kw)
    ctx.set_policy(table)
    if save_to is not None:
        save(table, save_to or cache_path(device), {"version": N.load().egb_version().decode()})
    return table
