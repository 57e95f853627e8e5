"""ctypes binding of libennemi_gb.so (include/ennemi_gb.h).

This is the only way the package reaches the GPU: there is no CPU fallback.
If the library is missing or no CUDA device is visible, every estimator call
raises ``RuntimeError``.

``run_tasks`` evaluates a list of :class:`Task` in one ``egb_run_batch`` call.
Columns may be NumPy arrays (host memory; uploaded by the library, each
distinct address range once) or CUDA tensors exposing ``data_ptr()`` (device
memory, used in place); one batch uses one kind.
"""

from __future__ import annotations

import ctypes
import os
import threading
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _build

MI, CMI, SEMI, CSEMI, ENTROPY = 0, 1, 2, 3, 4
DISCRETE_ENTROPY, DISCRETE_MI, DISCRETE_CMI = 5, 6, 7
DISCRETE_KINDS = (DISCRETE_ENTROPY, DISCRETE_MI, DISCRETE_CMI)

INPUT_DEVICE = 1 << 0
PLAIN_FP64 = 1 << 1
TIMING = 1 << 2
FORCE_BRUTE = 1 << 3
KEEP_INTERNALS = 1 << 4
FORCE_SLAB = 1 << 5
FORCE_GRID = 1 << 6
FORCE_CTA_GRID = 1 << 7
GRAPH = 1 << 8
STAGE_HOST = 1 << 9
RESCALE = 1 << 10
FORCE_RANK = 1 << 11
TASK_CONSTANT = 1        # egb_result.status: constant column under RESCALE

# layout policy (include/ennemi_gb.h)
MODE_AUTO, MODE_BRUTE, MODE_SLAB, MODE_GRID, MODE_WARP_GRID, MODE_RANK = -1, 0, 1, 2, 3, 4
POLICY_SIZE_CLASSES = 32
POLICY_ENTRIES = 2 * 4 * 4 * POLICY_SIZE_CLASSES


def policy_index(search: int, d: int, K: int, length: int) -> int:
    """egb_policy_index(): search 0 = kNN, 1 = ball count; K = k + 1."""
    dc = 0 if d <= 2 else 1 if d == 3 else 2 if d == 4 else 3
    kc = 0 if search else (0 if K <= 4 else 1 if K <= 8 else 2 if K <= 16 else 3)
    sc = min(max(int(length).bit_length() - 1, 0), POLICY_SIZE_CLASSES - 1)
    return ((search * 4 + dc) * 4 + kc) * POLICY_SIZE_CLASSES + sc


PHASES = ("upload", "prepare", "sort", "knn", "counts", "combine", "total",
          "knn_tile", "knn_defer", "count_tile", "count_defer", "sort_radix", "count_1d",
          "sort_passes")


class EgbColumn(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("stride", ctypes.c_int64)]


class EgbTask(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("k", ctypes.c_int32), ("n", ctypes.c_int64),
                ("dx", ctypes.c_int32), ("dy", ctypes.c_int32), ("dz", ctypes.c_int32),
                ("nclass", ctypes.c_int32), ("cols", ctypes.POINTER(EgbColumn)),
                ("labels", ctypes.POINTER(ctypes.c_int32)),
                ("index", ctypes.POINTER(ctypes.c_int32))]


class EgbResult(ctypes.Structure):
    _fields_ = [("value", ctypes.c_double), ("term_sum", ctypes.c_double),
                ("zero_mask", ctypes.c_uint32), ("status", ctypes.c_int32)]


_lib = None
_lib_lock = threading.Lock()
_ctx = {}


def lib_path() -> str:
    return _build.LIB_PATH


def load():
    """Load libennemi_gb.so (building it first if the sources are newer)."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        if _build.needs_build():
            _build.build()
        lib = ctypes.CDLL(_build.LIB_PATH)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        dp = ctypes.POINTER(ctypes.c_double)
        lib.egb_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        lib.egb_create.restype = ctypes.c_int
        lib.egb_destroy.argtypes = [vp]
        lib.egb_destroy.restype = None
        lib.egb_set_stream.argtypes = [vp, vp]
        lib.egb_set_stream.restype = ctypes.c_int
        lib.egb_last_error.argtypes = [vp]
        lib.egb_last_error.restype = ctypes.c_char_p
        lib.egb_run_batch.argtypes = [vp, ctypes.POINTER(EgbTask), i32, i32, ctypes.POINTER(EgbResult)]
        lib.egb_run_batch.restype = ctypes.c_int
        lib.egb_fetch.argtypes = [vp, i32, i32, vp]
        lib.egb_fetch.restype = ctypes.c_int
        lib.egb_knn_eps.argtypes = [vp, vp, i64, i32, i32, i32, vp]
        lib.egb_knn_eps.restype = ctypes.c_int
        lib.egb_ball_count.argtypes = [vp, vp, i64, i32, vp, i32, vp]
        lib.egb_ball_count.restype = ctypes.c_int
        lib.egb_timings.argtypes = [vp, dp, i32]
        lib.egb_timings.restype = ctypes.c_int
        lib.egb_last_transfer.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i64)]
        lib.egb_last_transfer.restype = ctypes.c_int
        lib.egb_last_stats.argtypes = [vp, ctypes.POINTER(i64), i32]
        lib.egb_last_stats.restype = ctypes.c_int
        lib.egb_set_policy.argtypes = [vp, ctypes.POINTER(ctypes.c_int8), i32]
        lib.egb_set_policy.restype = ctypes.c_int
        lib.egb_set_noise.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
        lib.egb_set_noise.restype = ctypes.c_int
        lib.egb_get_policy.argtypes = [vp, ctypes.POINTER(ctypes.c_int8), i32]
        lib.egb_get_policy.restype = ctypes.c_int
        lib.egb_device_info.argtypes = [vp, ctypes.c_char_p, i32, ctypes.POINTER(i32)]
        lib.egb_device_info.restype = ctypes.c_int
        lib.egb_last_groups.argtypes = [vp, i32, ctypes.POINTER(i64), i32]
        lib.egb_last_groups.restype = ctypes.c_int
        lib.egb_pairwise_matrix.argtypes = [vp, vp, vp, i32, i32, i32, i32, vp]
        lib.egb_pairwise_matrix.restype = ctypes.c_int
        lib.egb_normalize.argtypes = [vp, vp, i64, i32, vp]
        lib.egb_normalize.restype = ctypes.c_int
        lib.egb_debug_inject_device_error.argtypes = [vp, ctypes.c_uint32]
        lib.egb_debug_inject_device_error.restype = ctypes.c_int
        lib.egb_debug_divide.argtypes = [vp, vp, vp, ctypes.c_int64, vp]
        lib.egb_debug_divide.restype = ctypes.c_int
        lib.egb_version.argtypes = []
        lib.egb_version.restype = ctypes.c_char_p
        _lib = lib
        return lib


class Context:
    """One library context (device, stream, arena).  Calls are serialised."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.device = device
        h = ctypes.c_void_p()
        rc = self.lib.egb_create(device, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"egb_create(device={device}) failed ({rc}): no usable CUDA device")
        self.h = h
        self.lock = threading.Lock()
        self.noise_len = 0      # values of the RESCALE noise stream on the device

    def close(self):
        if self.h:
            self.lib.egb_destroy(self.h)
            self.h = ctypes.c_void_p()

    def error(self) -> str:
        return self.lib.egb_last_error(self.h).decode()

    def check(self, rc: int, what: str):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc}): {self.error()}")

    def set_stream(self, stream_handle: int | None):
        self.check(self.lib.egb_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)), "egb_set_stream")

    def transfer_bytes(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self.lib.egb_last_transfer(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def stats(self) -> dict:
        names = ("knn_tile_pairs", "knn_defer_pairs", "knn_deferred",
                 "count_tile_pairs", "count_defer_pairs", "count_deferred",
                 "knn_tile_ops", "count_tile_ops", "kernel_launches", "sort_keys", "sort_segments",
                 "planned", "graph", "sort_passes", "plan_us", "issue_us")
        buf = (ctypes.c_int64 * len(names))()
        n = self.lib.egb_last_stats(self.h, buf, len(names))
        return {names[i]: int(buf[i]) for i in range(n)}

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        sms = ctypes.c_int32()
        self.check(self.lib.egb_device_info(self.h, buf, 256, ctypes.byref(sms)), "egb_device_info")
        return f"{buf.value.decode()}_{sms.value}sm"

    def set_policy(self, modes) -> None:
        """Install a layout policy table (POLICY_ENTRIES modes); None resets it."""
        if modes is None:
            self.check(self.lib.egb_set_policy(self.h, None, 0), "egb_set_policy")
            return
        m = np.ascontiguousarray(modes, dtype=np.int8)
        if m.shape != (POLICY_ENTRIES,):
            raise ValueError(f"policy table must have {POLICY_ENTRIES} entries")
        self.check(self.lib.egb_set_policy(
            self.h, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), POLICY_ENTRIES), "egb_set_policy")

    def set_noise(self, values) -> None:
        """The RESCALE noise stream: values[p] = p-th draw of the reference's
        default_rng(2_718281828).normal(0.0, 1e-10, ...)."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        with self.lock:
            self.check(self.lib.egb_set_noise(
                self.h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(v)), "egb_set_noise")
            self.noise_len = len(v)

    def inject_device_error(self, word: int) -> None:
        """Test hook: the next batch starts with `word` in its device error
        word and reports it (egb_debug_inject_device_error)."""
        with self.lock:
            self.check(self.lib.egb_debug_inject_device_error(self.h, int(word)),
                       "egb_debug_inject_device_error")

    def debug_divide(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        """Test hook: a / b through the device division of the rescale
        (egb_debug_divide)."""
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        out = np.empty_like(a)
        with self.lock:
            self.check(self.lib.egb_debug_divide(self.h, a.ctypes.data, b.ctypes.data, a.size,
                                                 out.ctypes.data), "egb_debug_divide")
        return out

    def get_policy(self) -> np.ndarray:
        m = np.empty(POLICY_ENTRIES, dtype=np.int8)
        self.lib.egb_get_policy(self.h, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), POLICY_ENTRIES)
        return m

    def timings(self) -> dict:
        buf = (ctypes.c_double * len(PHASES))()
        n = self.lib.egb_timings(self.h, buf, len(PHASES))
        return {PHASES[i]: buf[i] for i in range(n)}


def context(device: int = 0) -> Context:
    ctx = _ctx.get(device)
    if ctx is None:
        ctx = Context(device)
        from . import autotune
        autotune.load_cached(ctx)   # a saved layout policy for this device, if any
        _ctx[device] = ctx
    return ctx


@dataclass
class Task:
    """One estimator invocation: columns are x first, then y, then z."""
    kind: int
    k: int
    x: Sequence
    y: Sequence = ()
    z: Sequence = ()
    labels: Optional[np.ndarray] = None   # int32 class index per sample (SEMI/CSEMI)
    nclass: int = 0
    index: Optional[np.ndarray] = None    # int32 sample positions in the columns (shareable)
    n: int = 0
    keep: List = field(default_factory=list)


def as_columns(a) -> list:
    """Split a float64 array (1-D or n x d) into a list of 1-D column views."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return [a]
    return [a[:, c] for c in range(a.shape[1])]


def _col_struct(col, device: bool):
    if device:
        stride = col.stride(0) if col.dim() == 1 else col.stride(0)
        return EgbColumn(col.data_ptr(), int(stride)), col
    c = np.asarray(col, dtype=np.float64)
    if c.ndim != 1:
        raise ValueError("columns must be one-dimensional")
    s = c.strides[0]
    if s <= 0 or s % 8 != 0 or not c.flags.aligned:
        c = np.ascontiguousarray(c)
        s = 8
    return EgbColumn(c.ctypes.data, s // 8), c


class Col:
    """A column resolved once and shared by many tasks: its address, stride
    (elements) and length, and the array that keeps the memory alive."""

    __slots__ = ("ptr", "stride", "length", "ref")

    def __init__(self, col, device: bool = False):
        s, ref = _col_struct(col, device)
        self.ptr, self.stride, self.ref = s.data, s.stride, ref
        self.length = int(ref.shape[0])


def _length(col) -> int:
    return col.length if type(col) is Col else len(col)


def run_tasks(tasks: List[Task], flags: int = 0, device: int = 0,
              results_out: Optional[list] = None, noise=None,
              groups_out: Optional[dict] = None) -> np.ndarray:
    """Evaluate the tasks in one batched call; returns the estimates.

    groups_out (a dict) receives, for each task of a discrete kind, the six
    distinct-value figures of egb_last_groups under the task's index.

    With RESCALE, `noise(m)` returns the first m values (at least) of the
    preprocessing noise stream; the device copy is extended when a batch needs
    more values than it holds."""
    if not tasks:
        return np.empty(0)
    ctx = context(device)
    if flags & RESCALE:
        need = max((t.n or _length(t.x[0])) * (len(t.x) + len(t.y) + len(t.z)) for t in tasks)
        if ctx.noise_len < need:
            if noise is None:
                raise ValueError("RESCALE needs the noise stream")
            ctx.set_noise(noise(max(need, 2 * ctx.noise_len)))
    is_dev = bool(flags & INPUT_DEVICE)
    ctasks = (EgbTask * len(tasks))()
    keep = []
    index_ptr = {}   # one int32 copy per index array shared by tasks
    # every task's columns in one array
    allcols = (EgbColumn * sum(len(t.x) + len(t.y) + len(t.z) for t in tasks))()
    base, csize = ctypes.addressof(allcols), ctypes.sizeof(EgbColumn)
    colp = ctypes.POINTER(EgbColumn)
    off = 0
    for i, t in enumerate(tasks):
        first = off
        n0 = None
        for col in (*t.x, *t.y, *t.z):
            e = allcols[off]
            if type(col) is Col:
                e.data, e.stride = col.ptr, col.stride
                length = col.length
            else:
                st, ref = _col_struct(col, is_dev)
                e.data, e.stride = st.data, st.stride
                keep.append(ref)
                length = ref.shape[0]
            if n0 is None:
                n0 = length
            off += 1
        ct = ctasks[i]
        ct.kind, ct.k, ct.n = t.kind, int(t.k), int(t.n or n0)
        ct.dx, ct.dy, ct.dz = len(t.x), len(t.y), len(t.z)
        ct.cols = ctypes.cast(base + first * csize, colp)
        if t.labels is not None:
            lab = np.ascontiguousarray(t.labels, dtype=np.int32)
            keep.append(lab)
            ct.labels = lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            ct.nclass = int(t.nclass)
        if t.index is not None:
            ptr = index_ptr.get(id(t.index))
            if ptr is None:
                ix = np.ascontiguousarray(t.index, dtype=np.int32)
                keep.append(ix)
                ptr = index_ptr[id(t.index)] = ix.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            ct.index = ptr
    keep.append(allcols)
    res = (EgbResult * len(tasks))()
    with ctx.lock:
        rc = ctx.lib.egb_run_batch(ctx.h, ctasks, len(tasks), flags, res)
        ctx.check(rc, "egb_run_batch")
        if groups_out is not None:
            buf = (ctypes.c_int64 * 6)()
            for i, t in enumerate(tasks):
                if t.kind in DISCRETE_KINDS:
                    ctx.lib.egb_last_groups(ctx.h, i, buf, 6)
                    groups_out[i] = [int(v) for v in buf]
    if results_out is not None:
        results_out.extend(res)
    return np.array([r.value for r in res], dtype=np.float64)


def fetch(task_index: int, which: int, n: int, device: int = 0) -> np.ndarray:
    """eps (which=0), count slot which-1, or working column which-16 of the
    last batch run with KEEP_INTERNALS."""
    ctx = context(device)
    out = np.empty(n, dtype=np.float64 if which == 0 or which >= 16 else np.int64)
    with ctx.lock:
        ctx.check(ctx.lib.egb_fetch(ctx.h, task_index, which, out.ctypes.data), "egb_fetch")
    return out


def knn_eps(points, k: int, flags: int = 0, device: int = 0) -> np.ndarray:
    """cKDTree(points).query(points, k=[k+1], p=inf)[0].ravel() on the GPU."""
    ctx = context(device)
    p = np.ascontiguousarray(points, dtype=np.float64)
    if p.ndim == 1:
        p = p.reshape(-1, 1)
    out = np.empty(p.shape[0])
    with ctx.lock:
        ctx.check(ctx.lib.egb_knn_eps(ctx.h, p.ctypes.data, p.shape[0], p.shape[1], int(k),
                                      flags & ~INPUT_DEVICE, out.ctypes.data), "egb_knn_eps")
    return out


def ball_count(points, radius, flags: int = 0, device: int = 0) -> np.ndarray:
    """cKDTree(points).query_ball_point(points, radius, p=inf, return_length=True)."""
    ctx = context(device)
    p = np.ascontiguousarray(points, dtype=np.float64)
    if p.ndim == 1:
        p = p.reshape(-1, 1)
    r = np.ascontiguousarray(np.broadcast_to(np.asarray(radius, dtype=np.float64), (p.shape[0],)))
    out = np.empty(p.shape[0], dtype=np.int64)
    with ctx.lock:
        ctx.check(ctx.lib.egb_ball_count(ctx.h, p.ctypes.data, p.shape[0], p.shape[1], r.ctypes.data,
                                         flags & ~INPUT_DEVICE, out.ctypes.data), "egb_ball_count")
    return out


def pairwise_matrix(values, pairs, nvar: int, normalize: bool = False, device: int = 0) -> np.ndarray:
    """The symmetric nvar x nvar matrix of per-pair estimates with a NaN
    diagonal, assembled on the device (egb_pairwise_matrix); `normalize`
    applies normalize_mi to the values."""
    ctx = context(device)
    v = np.ascontiguousarray(values, dtype=np.float64)
    p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    if len(v) != len(p):
        raise ValueError("one pair per value")
    out = np.empty((nvar, nvar), dtype=np.float64)
    with ctx.lock:
        ctx.check(ctx.lib.egb_pairwise_matrix(ctx.h, v.ctypes.data, p.ctypes.data, len(v), int(nvar),
                                              1 if normalize else 0, 0, out.ctypes.data),
                  "egb_pairwise_matrix")
    return out


def normalize(values, device: int = 0) -> np.ndarray:
    """normalize_mi of a float64 array on the device (egb_normalize); the
    result has the shape of `values`."""
    ctx = context(device)
    v = np.ascontiguousarray(values, dtype=np.float64)
    out = np.empty_like(v)
    with ctx.lock:
        ctx.check(ctx.lib.egb_normalize(ctx.h, v.ctypes.data, v.size, 0, out.ctypes.data),
                  "egb_normalize")
    return out
