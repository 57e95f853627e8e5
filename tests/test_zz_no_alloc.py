"""egb_knn_eps_noalloc: the kNN-distance query for callers that cannot
allocate device memory (a plugin with a fixed memory pool, a latency-bound
loop that cannot afford cudaMalloc's synchronisation).  Its scratch is a
fixed file-scope device array, so two calls in a row must not see each
other's leftovers.  Collected last (file name), so that a run stopping at
the first failure has run every other test before it.
"""

import ctypes

import numpy as np
import pytest

from ennemi_gb300 import _native as N

pytestmark = pytest.mark.gpu

MAX_POINTS = 16384


def _lib():
    lib = N.load()
    lib.egb_knn_eps_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    lib.egb_knn_eps_noalloc.restype = ctypes.c_int
    return lib


def test_noalloc_matches_knn_eps_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = _lib()
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    # the second call is smaller and of lower dimension: any stale state of
    # the first call left in the shared scratch would show up
    for n, d, k in [(12000, 3, 3), (9000, 2, 5)]:
        pts = rng.normal(size=(n, d))
        ref = N.knn_eps(pts, k)  # the allocating entry point
        dp = torch.from_numpy(pts).cuda()
        out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.egb_knn_eps_noalloc(dp.data_ptr(), n, d, k, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        # bit-exact, the tolerance of every eps comparison in this suite
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_noalloc_rejects_sizes_beyond_its_limits():
    torch = pytest.importorskip("torch")
    lib = _lib()
    buf = torch.zeros(2 * (MAX_POINTS + 1), dtype=torch.float64, device="cuda")
    out = torch.zeros(MAX_POINTS + 1, dtype=torch.float64, device="cuda")
    assert lib.egb_knn_eps_noalloc(buf.data_ptr(), MAX_POINTS + 1, 2, 3, out.data_ptr(), None) == -1
    assert lib.egb_knn_eps_noalloc(buf.data_ptr(), 100, 9, 3, out.data_ptr(), None) == -1
    assert lib.egb_knn_eps_noalloc(buf.data_ptr(), 100, 2, 32, out.data_ptr(), None) == -1
