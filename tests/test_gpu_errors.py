"""The device-error path, driven from the host.

Kernels report failures (a bounded wait that gave up, an index guard that
tripped) through one device error word per batch, which egb_run_batch turns
into EGB_ERR_DEVICE.  No kernel here is made to fail: the test hook
egb_debug_inject_device_error() presets that word for the next batch, which
then runs its kernels as usual.  The tests check the status and message the
caller sees, and that the same context runs the next batch bit for bit as
before -- plain, with kept internals and as a CUDA graph.
"""

import numpy as np
import pytest

from ennemi_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _tasks(n=6000, seed=3):
    rng = np.random.default_rng(seed)
    a, b, c = (rng.normal(size=n) for _ in range(3))
    return [N.Task(N.MI, 3, [a], [0.5 * a + b], n=n),
            N.Task(N.CMI, 3, [a], [b + 0.3 * c], [c], n=n)], n


@pytest.mark.parametrize("word, text", [(1, "bounded wait gave up"), (2, "index guard")])
def test_injected_device_error_is_reported_and_context_recovers(word, text):
    tasks, n = _tasks()
    ctx = N.context(0)
    base = N.run_tasks(tasks, flags=N.KEEP_INTERNALS)
    base_eps = N.fetch(0, 0, n)
    ctx.inject_device_error(word)
    with pytest.raises(RuntimeError, match=text) as err:
        N.run_tasks(tasks)
    assert "(-3)" in str(err.value)     # EGB_ERR_DEVICE
    # the next batch on the same context starts clean
    again = N.run_tasks(tasks, flags=N.KEEP_INTERNALS)
    assert np.array_equal(base, again)
    assert np.array_equal(base_eps, N.fetch(0, 0, n))


def test_injected_error_bypasses_graph_replay():
    torch = pytest.importorskip("torch")
    tasks, n = _tasks(20000, 4)
    dev = [N.Task(t.kind, t.k, [torch.from_numpy(np.asarray(c)).cuda() for c in t.x],
                  [torch.from_numpy(np.asarray(c)).cuda() for c in t.y],
                  [torch.from_numpy(np.asarray(c)).cuda() for c in t.z], n=n) for t in tasks]
    ctx = N.context(0)
    first = N.run_tasks(dev, flags=N.INPUT_DEVICE | N.GRAPH)
    ctx.inject_device_error(2)
    with pytest.raises(RuntimeError, match="index guard"):
        N.run_tasks(dev, flags=N.INPUT_DEVICE | N.GRAPH)
    st = ctx.stats()
    assert st["planned"] == 1 and st["graph"] == 0
    # capture and replay work again afterwards
    again = N.run_tasks(dev, flags=N.INPUT_DEVICE | N.GRAPH)
    replay = N.run_tasks(dev, flags=N.INPUT_DEVICE | N.GRAPH)
    assert ctx.stats()["planned"] == 0
    assert np.array_equal(first, again) and np.array_equal(first, replay)


def test_sort_tie_report_reruns_batch_with_full_sort():
    """DERR_SORT_TIES (a run of keys tied in their high 48 bits too long for
    the in-kernel repair) is not an error: the batch runs again, planned and
    without a graph, with all eight digit passes, and returns the same
    results as the six-pass sort."""
    tasks, n = _tasks()
    ctx = N.context(0)
    base = N.run_tasks(tasks, flags=N.KEEP_INTERNALS)
    base_eps = N.fetch(0, 0, n)
    assert ctx.stats()["sort_passes"] == 6
    ctx.inject_device_error(4)
    again = N.run_tasks(tasks, flags=N.KEEP_INTERNALS)
    st = ctx.stats()
    assert st["sort_passes"] == 8 and st["planned"] == 1 and st["graph"] == 0
    assert np.array_equal(base, again)
    assert np.array_equal(base_eps, N.fetch(0, 0, n))
