"""Generate golden vectors from the live reference (ennemi + scipy cKDTree).

Run in a checkout where the reference package is importable, giving the
directory that holds its ``ennemi`` package:

    python tests/golden/make_golden.py --reference <path to the ennemi checkout>
    python tests/golden/make_golden.py --reference <...> --headline

(or set ENNEMI_REFERENCE instead of passing --reference).

The first form writes ``tests/golden/golden_estimators.npz`` and
``tests/golden/golden_driver.npz``.  Inputs are seeded synthetic arrays; the
outputs are

* the estimate returned by the reference estimator function
  (``ennemi._entropy_estimators._estimate_*``) or public driver function;
* the internal arrays the estimator builds (eps and neighbour counts),
  recomputed with exactly the cKDTree calls the estimator makes
  (the reference does not return them).

The fixtures are small (N <= 3000) so that the CPU oracle and the GPU
parity tests can use them directly.  Nothing at test time reads the
reference: only these committed files.

``--headline`` writes ``tests/golden/golden_headline.json`` for the two
headline configurations, too large to store as arrays:

* the single ``estimate_mi(y, x)`` of a bivariate Gaussian (rho = 0.6,
  N = 10,000, k = 3, seed 0) through the reference's public path with its
  preprocessing;
* the large-sample batch (four bivariate Gaussian KSG MI, rho = 0, .3, .6,
  .9, and one trivariate Gaussian conditional MI; N = 1,000,000, k = 3,
  seed 0) through the reference's estimator functions.

For each task it records the reference's estimate, and SHA-256 digests of
the inputs, of eps (float64 little-endian) and of every neighbour-count
array (int64 little-endian), with a few plain sums for diagnosis.  The
inputs come from ``ennemi_gb300.synthetic``, whose generator gives the same
bits on x86-64 and AArch64, so the digests can be checked on either.
"""

from __future__ import annotations

import argparse
import os
import sys

import numpy as np


def _cases(rng_seed_base: int = 0):
    """Yield (name, kind, k, inputs) for the estimator-level cases."""
    def gauss2(n, rho, seed):
        rng = np.random.default_rng(seed)
        d = rng.multivariate_normal([0, 0], [[1, rho], [rho, 1]], size=n)
        return d[:, 0].copy(), d[:, 1].copy()

    x, y = gauss2(2000, 0.6, 0)
    yield "mi_gauss_rho06_n2000_k3", "mi", 3, dict(x=x, y=y)
    x, y = gauss2(500, -0.9, 1)
    yield "mi_gauss_rhom09_n500_k1", "mi", 1, dict(x=x, y=y)
    x, y = gauss2(1000, 0.0, 2)
    yield "mi_gauss_rho0_n1000_k20", "mi", 20, dict(x=x, y=y)
    x, y = gauss2(1500, 0.8, 3)
    yield "mi_gauss_rho08_n1500_k100", "mi", 100, dict(x=x, y=y)
    x, y = gauss2(40, 0.5, 4)
    yield "mi_gauss_n40_k3", "mi", 3, dict(x=x, y=y)
    x, y = gauss2(5, 0.5, 5)
    yield "mi_gauss_n5_k4", "mi", 4, dict(x=x, y=y)
    # heavy tails: Student-t and log-normal columns, no rescaling
    rng = np.random.default_rng(6)
    t = rng.standard_t(3, size=2500)
    ln = np.exp(0.8 * t / 3 + rng.normal(size=2500))
    yield "mi_heavy_t3_lognormal_n2500_k3", "mi", 3, dict(x=t, y=ln)
    # large offset (preprocess=False style data far from the origin)
    rng = np.random.default_rng(7)
    yield "mi_offset_1e6_n1200_k3", "mi", 3, dict(x=1e6 + rng.normal(size=1200),
                                                   y=-3e5 + 10 * rng.normal(size=1200))
    # duplicates: coarse rounding gives zero eps -> -inf estimate
    rng = np.random.default_rng(8)
    yield "mi_duplicates_n800_k3", "mi", 3, dict(x=np.round(rng.normal(size=800), 1),
                                                 y=np.round(rng.normal(size=800), 1))
    # ties that stay finite: a lattice with jitter-free spacing
    rng = np.random.default_rng(9)
    yield "mi_lattice_n900_k3", "mi", 3, dict(x=np.repeat(np.arange(30.0), 30) * 0.25,
                                              y=np.tile(np.arange(30.0), 30) * 0.5)

    def gauss(n, cov, seed):
        rng = np.random.default_rng(seed)
        return rng.multivariate_normal(np.zeros(len(cov)), cov, size=n)

    d = gauss(2000, [[1, .5, .4], [.5, 1, .4], [.4, .4, 1]], 10)
    yield "cmi_gauss3_n2000_k3", "cmi", 3, dict(x=d[:, 0], y=d[:, 1], z=d[:, 2:3])
    d = gauss(1500, [[1, 0, 2, 1], [0, 6, 1, 2], [2, 1, 5, 2], [1, 2, 2, 2]], 11)
    yield "cmi_gauss4_dz2_n1500_k5", "cmi", 5, dict(x=d[:, 0], y=d[:, 1], z=d[:, 2:])
    rng = np.random.default_rng(12)
    base = rng.normal(size=(800, 9))
    base[:, 1] += 0.5 * base[:, 0]
    yield "cmi_dz7_n800_k3", "cmi", 3, dict(x=base[:, 0], y=base[:, 1], z=base[:, 2:])
    rng = np.random.default_rng(13)
    xx = rng.normal(size=600)
    yield "cmi_cond_equals_y_n600_k4", "cmi", 4, dict(x=xx + 0.3 * rng.normal(size=600), y=xx, z=xx.reshape(-1, 1))

    rng = np.random.default_rng(20)
    cls = rng.choice([0, 1, 2], p=[0.2, 0.5, 0.3], size=2000)
    xs = rng.normal(0.3 * cls, 1.0)
    yield "semi_3class_n2000_k3", "semi", 3, dict(x=xs, y=cls)
    rng = np.random.default_rng(21)
    cls = rng.choice([0, 1, 2, 3], p=[0.3, 0.3, 0.398, 0.002], size=1500)
    xs = rng.normal(size=(1500, 2)) + cls[:, None] * 0.2
    yield "semi_x2d_tinyclass_n1500_k3", "semi", 3, dict(x=xs, y=cls)
    rng = np.random.default_rng(22)
    cls = rng.choice(["a", "b"], size=700)
    xs = rng.uniform(size=(700, 3))
    yield "semi_x3d_strlabels_n700_k2", "semi", 2, dict(x=xs, y=cls)

    rng = np.random.default_rng(30)
    xx = rng.normal(size=1500)
    cls = np.sign(xx + 0.5 * rng.normal(size=1500))
    zz = rng.normal(size=1500)
    yield "csemi_n1500_k3", "csemi", 3, dict(x=xx, y=cls, z=zz.reshape(-1, 1))
    rng = np.random.default_rng(31)
    xx = rng.gamma(1.5, size=1200)
    cls = np.zeros(1200)
    cls[xx < 0.5] = 1e-4
    cls[xx > 2.0] = 4
    zz = rng.normal(size=(1200, 2))
    yield "csemi_3level_dz2_n1200_k1", "csemi", 1, dict(x=xx + zz[:, 0], y=cls, z=zz)

    rng = np.random.default_rng(40)
    yield "ent_1d_n2000_k3", "ent", 3, dict(x=rng.normal(size=2000))
    rng = np.random.default_rng(41)
    yield "ent_3d_n2000_k3", "ent", 3, dict(x=rng.normal(size=(2000, 3)))
    rng = np.random.default_rng(42)
    yield "ent_2d_n1000_k30", "ent", 30, dict(x=rng.uniform(size=(1000, 2)))
    rng = np.random.default_rng(43)
    yield "ent_dup_n300_k2", "ent", 2, dict(x=np.round(rng.normal(size=300), 1))
    rng = np.random.default_rng(44)
    yield "ent_5d_n700_k4", "ent", 4, dict(x=rng.normal(size=(700, 5)))

    # discrete plug-in estimators (k unused)
    rng = np.random.default_rng(50)
    yield "dent_1d_n3000", "dent", 1, dict(x=rng.integers(0, 12, size=3000).astype(np.float64))
    rng = np.random.default_rng(51)
    yield "dent_2d_n2000", "dent", 1, dict(x=np.column_stack((rng.integers(0, 5, size=2000),
                                                              rng.choice([-0.5, 0.0, 2.5], size=2000))))
    rng = np.random.default_rng(52)
    dx = rng.integers(0, 6, size=2500)
    dy = (dx + rng.integers(0, 3, size=2500)) % 7
    yield "dmi_n2500", "dmi", 1, dict(x=dx.astype(np.float64), y=dy.astype(np.float64))
    rng = np.random.default_rng(53)
    yield "dmi_manylevels_n400", "dmi", 1, dict(x=rng.integers(0, 300, size=400).astype(np.float64),
                                                 y=rng.integers(0, 2, size=400).astype(np.float64))
    rng = np.random.default_rng(54)
    dz = rng.integers(0, 4, size=3000)
    ddx = (dz + rng.integers(0, 3, size=3000)) % 5
    ddy = (ddx + dz + rng.integers(0, 2, size=3000)) % 4
    yield "dcmi_n3000", "dcmi", 1, dict(x=ddx.astype(np.float64), y=ddy.astype(np.float64),
                                        z=dz.astype(np.float64).reshape(-1, 1))
    rng = np.random.default_rng(55)
    dz2 = rng.integers(0, 3, size=(1500, 2))
    yield "dcmi_dz2_n1500", "dcmi", 1, dict(x=rng.integers(0, 4, size=1500).astype(np.float64),
                                            y=(dz2[:, 0] + rng.integers(0, 2, size=1500)).astype(np.float64),
                                            z=dz2.astype(np.float64))


def _internals(kind, k, inp, cKDTree):
    """Recompute the estimator's internal arrays with its own cKDTree calls."""
    cs = np.column_stack
    if kind == "mi":
        x, y = cs((inp["x"],)), cs((inp["y"],))
        xy = cs((x, y))
        eps = cKDTree(xy).query(xy, k=[k + 1], p=np.inf)[0].flatten()
        nx = cKDTree(x).query_ball_point(x, eps - 1e-12, p=np.inf, return_length=True)
        ny = cKDTree(y).query_ball_point(y, eps - 1e-12, p=np.inf, return_length=True)
        return dict(eps=eps, nx=nx, ny=ny)
    if kind == "cmi":
        x, y, z = cs((inp["x"],)), cs((inp["y"],)), cs((inp["z"],))
        xyz = cs((x, y, z))
        eps = cKDTree(xyz).query(xyz, k=[k + 1], p=np.inf)[0].flatten()
        xz, yz = cs((x, z)), cs((y, z))
        r = eps - 1e-12
        return dict(eps=eps,
                    nxz=cKDTree(xz).query_ball_point(xz, r, p=np.inf, return_length=True),
                    nyz=cKDTree(yz).query_ball_point(yz, r, p=np.inf, return_length=True),
                    nz=cKDTree(z).query_ball_point(z, r, p=np.inf, return_length=True))
    if kind == "semi":
        x = cs((inp["x"],))
        y = inp["y"]
        n = len(y)
        eps = np.empty(n)
        cnt = np.empty(n, dtype=np.int64)
        xt = cKDTree(x)
        for val in np.unique(y):
            sel = y == val
            e = cKDTree(x[sel]).query(x[sel], k=[k + 1], p=np.inf)[0].flatten()
            eps[sel] = e
            cnt[sel] = xt.query_ball_point(x[sel], e - 1e-12, p=np.inf, return_length=True)
        return dict(eps=eps, n=cnt)
    if kind == "csemi":
        x, z = cs((inp["x"],)), cs((inp["z"],))
        y = inp["y"]
        n = len(y)
        xz = cs((x, z))
        eps = np.empty(n)
        nxz = np.empty(n, dtype=np.int64)
        nyz = np.empty(n, dtype=np.int64)
        nz = np.empty(n, dtype=np.int64)
        for val in np.unique(y):
            sel = y == val
            e = cKDTree(xz[sel]).query(xz[sel], k=[k + 1], p=np.inf)[0].flatten()
            r = e - 1e-12
            eps[sel] = e
            nxz[sel] = cKDTree(xz).query_ball_point(xz[sel], r, p=np.inf, return_length=True)
            nyz[sel] = cKDTree(z[sel]).query_ball_point(z[sel], r, p=np.inf, return_length=True)
            nz[sel] = cKDTree(z).query_ball_point(z[sel], r, p=np.inf, return_length=True)
        return dict(eps=eps, nxz=nxz, nyz=nyz, nz=nz)
    if kind == "ent":
        x = inp["x"]
        if x.ndim == 1:
            x = x.reshape(-1, 1)
        eps = cKDTree(x).query(x, k=[k + 1], p=np.inf)[0].flatten()
        return dict(eps=eps)
    if kind in ("dent", "dmi", "dcmi"):
        # rows equal to each row on each column subset, with np.unique as the
        # reference counts them
        def counts(*arrs):
            rows = np.column_stack(arrs)
            _, inv, cnt = np.unique(rows, axis=0, return_inverse=True, return_counts=True)
            return cnt[np.ravel(inv)].astype(np.int64)
        if kind == "dent":
            return dict(c=counts(inp["x"]))
        if kind == "dmi":
            return dict(cxy=counts(inp["x"], inp["y"]), cx=counts(inp["x"]), cy=counts(inp["y"]))
        return dict(cxyz=counts(inp["x"], inp["y"], inp["z"]), cxz=counts(inp["x"], inp["z"]),
                    cyz=counts(inp["y"], inp["z"]), cz=counts(inp["z"]))
    raise ValueError(kind)


def _driver_cases():
    """Public-API cases: (name, function, args, kwargs)."""
    rng = np.random.default_rng(100)
    n = 1200
    ar = np.zeros((n, 3))
    for t in range(1, n):
        ar[t] = 0.7 * ar[t - 1] + rng.normal(size=3)
        ar[t, 1] += 0.4 * ar[t - 3, 0] if t >= 3 else 0.0
    mask = rng.uniform(size=n) > 0.1
    yield "drv_lags_mask", "estimate_mi", (ar[:, 1], ar[:, [0, 2]], [-2, 0, 1, 3, 5]), dict(mask=mask, k=3)
    yield "drv_cond_lag", "estimate_mi", (ar[:, 1], ar[:, 0], [0, 2, 4]), dict(cond=ar[:, 2], cond_lag=[1, 2, 3])
    yield "drv_normalize", "estimate_mi", (ar[:, 1], ar[:, :3], 0), dict(normalize=True)
    yield "drv_nopreprocess", "estimate_mi", (ar[:, 1], ar[:, 0], [0, 1]), dict(preprocess=False)
    yield "drv_pairwise", "pairwise_mi", (ar,), dict(k=2)
    yield "drv_pairwise_cond", "pairwise_mi", (ar[:, :2],), dict(cond=ar[:, 2])
    data = ar.copy()
    data[::37, 0] = np.nan
    yield "drv_dropnan", "estimate_mi", (data[:, 1], data[:, 0], [0, 1]), dict(drop_nan=True)
    cls = (ar[:, 0] > 0.5).astype(int) + (ar[:, 0] > -0.5).astype(int)
    yield "drv_discrete_y", "estimate_mi", (cls, ar[:, [1, 2]], [0, 1]), dict(discrete_y=True)
    yield "drv_discrete_x", "estimate_mi", (ar[:, 1], cls, [0, 2]), dict(discrete_x=True)
    yield "drv_discrete_y_cond", "estimate_mi", (cls, ar[:, 1]), dict(discrete_y=True, cond=ar[:, 2])
    yield "drv_entropy_cols", "estimate_entropy", (ar,), dict(k=3)
    yield "drv_entropy_multidim", "estimate_entropy", (ar[:, :2],), dict(multidim=True, k=4)
    yield "drv_entropy_cond", "estimate_entropy", (ar[:, :2],), dict(cond=ar[:, 2], k=3)
    yield "drv_entropy_mask", "estimate_entropy", (ar[:, 0],), dict(mask=mask)
    lv = np.round(ar * 0.8).astype(int)
    yield "drv_discrete_both", "estimate_mi", (lv[:, 1], lv[:, [0, 2]], [0, 1, 2]), \
        dict(discrete_x=True, discrete_y=True)
    yield "drv_discrete_both_cond", "estimate_mi", (lv[:, 1], lv[:, 0]), \
        dict(discrete_x=True, discrete_y=True, cond=lv[:, 2])
    yield "drv_discrete_entropy", "estimate_entropy", (lv,), dict(discrete=True)
    yield "drv_discrete_entropy_multidim", "estimate_entropy", (lv[:, :2],), \
        dict(discrete=True, multidim=True)
    yield "drv_discrete_pairwise", "pairwise_mi", (lv,), dict(discrete=True)


def digest(arr, dtype) -> str:
    """SHA-256 of the array's values as little-endian `dtype` bytes."""
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(arr, dtype=dtype).tobytes()).hexdigest()


def _summary(name, arr):
    a = np.asarray(arr)
    if name == "eps":
        return {"eps": digest(a, "<f8"), "eps_sum": float(np.sum(a))}
    return {name: digest(a, "<i8"), name + "_sum": int(np.sum(a.astype(np.int64)))}


def headline(args) -> None:
    """golden_headline.json: the two headline configurations (see the module
    docstring)."""
    import concurrent.futures
    import json
    import warnings
    root = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, root)
    import ennemi
    from ennemi import _driver as rd
    from ennemi import _entropy_estimators as ee
    from scipy.spatial import cKDTree
    from ennemi_gb300 import synthetic

    out = {"generator": "ennemi_gb300.synthetic (plain_ksg, large_sample)",
           "reference": f"ennemi {getattr(ennemi, '__version__', '?')} with scipy cKDTree "
                        f"{__import__('scipy').__version__}, numpy {np.__version__}"}

    # the single estimate_mi(y, x) through the public path
    n1, k = 10_000, 3
    x, y = synthetic.plain_ksg(n1, 0, 0.6)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        value = float(np.asarray(ennemi.estimate_mi(y, x, k=k)).item())
        xs, ys, _ = rd._rescale_data(x, y, None, False, False)
    inter = _internals("mi", k, dict(x=xs, y=ys), cKDTree)
    c1 = {"n": n1, "k": k, "rho": 0.6, "seed": 0, "call": "estimate_mi(y, x, k=3)",
          "value": value, "analytic": -0.5 * float(np.log(1 - 0.36)),
          "inputs": {"x": digest(x, "<f8"), "y": digest(y, "<f8")},
          "prepared": {"x": digest(xs, "<f8"), "y": digest(ys, "<f8")}}
    for key, arr in inter.items():
        c1.update(_summary(key, arr))
    out["plain_ksg"] = c1
    print("plain_ksg", value)

    # the large-sample batch through the estimator functions
    n2 = 1_000_000
    work = synthetic.large_sample(n2, 0)

    def one(item):
        kind, cols = item
        if kind == "mi":
            val = float(ee._estimate_single_mi(cols[0], cols[1], k))
            inter = _internals("mi", k, dict(x=cols[0], y=cols[1]), cKDTree)
        else:
            val = float(ee._estimate_conditional_mi(cols[0], cols[1], cols[2], k))
            inter = _internals("cmi", k, dict(x=cols[0], y=cols[1], z=cols[2]), cKDTree)
        rec = {"kind": kind, "value": val, "inputs": [digest(c, "<f8") for c in cols]}
        for key, arr in inter.items():
            rec.update(_summary(key, arr))
        return rec

    with concurrent.futures.ThreadPoolExecutor(len(work)) as pool:
        tasks = list(pool.map(one, work))
    for rho, t in zip(synthetic.RHOS, tasks):
        t["rho"] = rho
    tasks[-1]["cov"] = synthetic.CMI_COV
    out["large_sample"] = {"n": n2, "k": k, "seed": 0, "tasks": tasks}
    print("large_sample", [t["value"] for t in tasks])
    path = os.path.join(args.out, "golden_headline.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")
    print("wrote", path)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("ENNEMI_REFERENCE"),
                    help="directory holding the reference's ennemi package "
                         "(default: $ENNEMI_REFERENCE)")
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    ap.add_argument("--headline", action="store_true",
                    help="write golden_headline.json (the two headline configurations)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or ENNEMI_REFERENCE) is required")
    sys.path.insert(0, args.reference)
    if args.headline:
        headline(args)
        return
    import ennemi
    from ennemi import _entropy_estimators as ee
    from scipy.spatial import cKDTree

    funcs = {"mi": lambda i, k: ee._estimate_single_mi(i["x"], i["y"], k),
             "cmi": lambda i, k: ee._estimate_conditional_mi(i["x"], i["y"], i["z"], k),
             "semi": lambda i, k: ee._estimate_semidiscrete_mi(i["x"], i["y"], k),
             "csemi": lambda i, k: ee._estimate_conditional_semidiscrete_mi(i["x"], i["y"], i["z"], k),
             "ent": lambda i, k: ee._estimate_single_entropy(i["x"], k),
             "dent": lambda i, k: ee._estimate_discrete_entropy(i["x"]),
             "dmi": lambda i, k: ee._estimate_discrete_mi(i["x"], i["y"]),
             "dcmi": lambda i, k: ee._estimate_conditional_discrete_mi(i["x"], i["y"], i["z"])}
    out = {}
    names = []
    import warnings
    for name, kind, k, inp in _cases():
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            value = funcs[kind](inp, k)
        names.append(name)
        out[f"{name}/kind"] = np.asarray(kind)
        out[f"{name}/k"] = np.asarray(k)
        out[f"{name}/value"] = np.asarray(value, dtype=np.float64)
        for key, arr in inp.items():
            out[f"{name}/in_{key}"] = np.asarray(arr)
        for key, arr in _internals(kind, k, inp, cKDTree).items():
            out[f"{name}/out_{key}"] = np.asarray(arr)
    out["names"] = np.asarray(names)
    np.savez_compressed(os.path.join(args.out, "golden_estimators.npz"), **out)

    dout = {}
    dnames = []
    for name, fname, fargs, kw in _driver_cases():
        fn = getattr(ennemi, fname)
        with warnings.catch_warnings(), np.errstate(all="ignore"):
            warnings.simplefilter("ignore")
            res = np.asarray(fn(*fargs, **kw), dtype=np.float64)
        dnames.append(name)
        dout[f"{name}/func"] = np.asarray(fname)
        dout[f"{name}/result"] = res
        for i, a in enumerate(fargs):
            dout[f"{name}/arg{i}"] = np.asarray(a)
        for key, v in kw.items():
            dout[f"{name}/kw_{key}"] = np.asarray(v)
    dout["names"] = np.asarray(dnames)
    np.savez_compressed(os.path.join(args.out, "golden_driver.npz"), **dout)
    print(f"wrote {len(names)} estimator cases and {len(dnames)} driver cases")


if __name__ == "__main__":
    main()
