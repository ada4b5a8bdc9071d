"""Pipelined host-vector calls (SpB_mxv_host_async_ext / SpB_VNEC_host_wait_ext):
a stream of independent right-hand sides enqueued without waiting gives the
same y, bit for bit, as one synchronous SpB_mxv_host_ext call per vector, for
every plan kind, with pageable and page-locked host buffers."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = ["L", "S", "S_fp32", "D", "HYBRID", "AUTO"]


def _plan(kind, m):
    from vnec_gb300 import api

    kw = {"L": dict(kernel=api.KERNEL_L), "S": dict(kernel=api.KERNEL_S),
          "S_fp32": dict(kernel=api.KERNEL_S, precision=api.PREC_FP32), "D": dict(kernel=api.KERNEL_D),
          "HYBRID": dict(kernel=api.KERNEL_HYBRID), "AUTO": dict()}[kind]
    return api.Plan(m, **kw)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
def test_async_host_calls_match_sync(built, kind, pinned):
    import torch

    from vnec_gb300 import generators as G

    m = G.lognormal(60000, sigma=1.2, cap=2000, seed=11)
    p = _plan(kind, m)
    n = 5
    xs = [G.vector(m.n_cols, seed=20 + i) for i in range(n)]
    want = [p.mxv_host(x) for x in xs]
    if pinned:
        hx = [torch.from_numpy(x).pin_memory().numpy() for x in xs]
        hy = [torch.empty(m.n_rows, dtype=torch.float64).pin_memory().numpy() for _ in range(n)]
    else:
        hx = xs
        hy = [np.full(m.n_rows, np.nan) for _ in range(n)]
    for rep in range(2):  # the second round reuses both buffer slots
        for i in range(n):
            p.mxv_host_async(hx[i], hy[i])
        p.host_wait()
        for i in range(n):
            assert hy[i].tobytes() == want[i].tobytes(), (rep, i)
    # a synchronous call while pipelined ones are in flight (it waits for
    # their SpMVs: they share the plan's scratch)
    for i in range(2, n):
        hy[i].fill(np.nan)
        p.mxv_host_async(hx[i], hy[i])
    assert p.mxv_host(xs[1]).tobytes() == want[1].tobytes()
    p.host_wait()
    for i in range(2, n):
        assert hy[i].tobytes() == want[i].tobytes(), i
    p.free()


def test_async_host_calls_batch_plan(built):
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    mats = [G.lognormal(300 + 37 * i, sigma=1.0, cap=200, seed=i) for i in range(12)]
    for k, prec in ((1, api.PREC_FP64), (8, api.PREC_FP64), (8, api.PREC_FP32)):
        bp = api.BatchPlan(mats, k, precision=prec)
        n_rows, n_cols = sum(m.n_rows for m in mats), sum(m.n_cols for m in mats)
        xs = [np.random.default_rng(i).uniform(-1, 1, size=n_cols * k) for i in range(4)]
        want = [bp.mxv_host(x).reshape(-1) for x in xs]
        ys = [np.empty(n_rows * k) for _ in xs]
        for x, y in zip(xs, ys):
            bp.mxv_host_async(x, y)
        bp.host_wait()
        for y, w in zip(ys, want):
            assert y.tobytes() == w.tobytes()
        bp.free()


def test_host_calls_reject_bad_arrays(built):
    """Wrong dtype, wrong size or read-only y is refused before anything is
    enqueued (a short host buffer would be overrun by the copies)."""
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    m = G.uniform_k(1000, 5, seed=1)
    p = api.Plan(m, kernel=api.KERNEL_S)
    x, y = np.zeros(m.n_cols), np.zeros(m.n_rows)
    ro = np.zeros(m.n_rows)
    ro.flags.writeable = False
    bad = [(np.zeros(m.n_cols, dtype=np.float32), y), (x[:-1], y), (x, y[:-1]), (x, ro)]
    for bx, by in bad:
        with pytest.raises(ValueError):
            p.mxv_host_async(bx, by)
    with pytest.raises(ValueError):
        p.mxv_host(x[:-1])
    with pytest.raises(ValueError):
        p.mxv_host(x, y[:-1])
    p.host_wait()  # nothing enqueued
    assert p.mxv_host(x, y) is y
    p.free()


@pytest.mark.parametrize("kind", ["S", "L", "HYBRID"])
def test_host_calls_from_many_threads(built, kind):
    """Host-vector calls on one plan from several host threads (ctypes releases
    the GIL, so the calls overlap in the library): each thread's results equal
    the single-threaded ones bit for bit."""
    import threading

    from vnec_gb300 import generators as G

    m = G.lognormal(50000, sigma=1.3, cap=3000, seed=12)
    p = _plan(kind, m)
    xs = [G.vector(m.n_cols, seed=40 + i) for i in range(8)]
    want = [p.mxv_host(x) for x in xs]
    errors = []

    def worker(t):
        try:
            for rep in range(6):
                i = (t + rep) % len(xs)
                if rep % 3 == 2:
                    y = np.empty(m.n_rows)
                    p.mxv_host_async(xs[i], y)
                    p.host_wait()
                else:
                    y = p.mxv_host(xs[i])
                if y.tobytes() != want[i].tobytes():
                    errors.append((t, rep, i))
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append((t, repr(e)))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    p.free()
    assert not errors, errors
