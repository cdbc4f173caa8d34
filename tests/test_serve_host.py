"""Server scheduling logic (the native nglod_serve_* scheduler, driven through
its callback executor) on the CPU with a simulated executor."""
import time

import numpy as np
import pytest
import torch

from nglod_gb300 import serve


class FakeExecutor:
    """Each request 'runs' for units * us_per_unit microseconds after launch."""

    def __init__(self, us_per_unit=0.002, num_streams=4):
        self.streams = [None] * num_streams
        self.us = us_per_unit
        self.launched = []

    def launch(self, tk, si):
        tk.handle = time.monotonic() + tk.request.units() * self.us * 1e-6
        self.launched.append(tk.rid)

    def done(self, tk):
        return time.monotonic() >= tk.handle

    def wait(self, tk, timeout):
        left = tk.handle - time.monotonic()
        if left > timeout:
            time.sleep(timeout)
            return False
        time.sleep(max(0.0, left))
        return True


def _render(w, h, model=0):
    return serve.RenderRequest(model, w, h, 2)


def test_budget_is_never_exceeded_and_order_is_fifo():
    ex = FakeExecutor(us_per_unit=0.05)
    budget = _render(256, 256).nbytes() * 2 + 100
    s = serve.Server(ex, budget)
    tks = [s.submit(_render(256, 256)) for _ in range(7)]
    assert s.drain(timeout=30)
    assert s.peak_used <= budget
    assert s.max_concurrent == 2
    assert ex.launched == [t.rid for t in tks]
    assert all(t.t_done >= t.t_admit >= t.t_arrival for t in tks)


def test_requests_overlap_when_budget_allows():
    ex = FakeExecutor(us_per_unit=0.05, num_streams=8)
    s = serve.Server(ex, 1 << 34)
    for _ in range(6):
        s.submit(_render(128, 128))
    s.poll()
    assert s.info()["running"] == 6
    assert s.drain(timeout=30)
    st = s.stats()
    assert st["requests"] == 6 and st["max_concurrent"] == 6


def test_oversized_request_is_refused():
    s = serve.Server(FakeExecutor(), 1000)
    with pytest.raises(ValueError):
        s.submit(_render(64, 64))


def test_bounded_stop_reports_unfinished():
    ex = FakeExecutor(us_per_unit=1000.0)  # 1 ms per pixel: far longer than the stop timeout
    s = serve.Server(ex, 1 << 30, num_streams=1)
    s.submit(_render(64, 64))
    s.submit(_render(64, 64))
    s.poll()
    t0 = time.monotonic()
    finished, running, dropped = s.stop(timeout=0.2)
    assert time.monotonic() - t0 < 2.0
    assert (finished, running, dropped) == (0, 1, 1)


def test_poisson_workload_is_seeded_and_mixed():
    a = serve.poisson_workload(5.0, 200.0, 8, seed=3)
    b = serve.poisson_workload(5.0, 200.0, 8, seed=3)
    assert a == b
    assert 850 < len(a) < 1150
    kinds = {spec["kind"] for _, spec in a}
    assert kinds == {"render", "query"}
    sizes = {(s["width"], s["height"]) for _, s in a if s["kind"] == "render"}
    assert sizes == {(256, 256), (512, 512), (1280, 720), (1920, 1080)}
    ns = [s["n"] for _, s in a if s["kind"] == "query"]
    assert min(ns) >= 1e4 and max(ns) <= 1e6
    assert all(0 <= s["model"] < 8 for _, s in a)


def test_stats_percentiles():
    ex = FakeExecutor(us_per_unit=0.01)
    s = serve.Server(ex, 1 << 34)
    wl = serve.poisson_workload(0.3, 200.0, 2, seed=1, sizes=((64, 64),), query_range=(100, 1000))
    st = serve.run_workload(s, wl, lambda spec: torch.zeros(spec["n"], 3))
    assert st["requests"] == len(wl)
    assert st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]


class RegionCheckingExecutor(FakeExecutor):
    """Checks that the regions of requests running together never overlap and
    stay inside the pool; fails the launches of chosen requests."""

    def __init__(self, budget, fail=(), **kw):
        super().__init__(**kw)
        self.budget = budget
        self.fail = set(fail)
        self.live = {}
        self.max_end = 0

    def launch(self, tk, si):
        if tk.rid in self.fail:
            raise RuntimeError("planted launch failure")
        off, nb = tk.region
        assert off % 256 == 0 and off + nb <= self.budget
        for o2, n2 in self.live.values():
            assert off + nb <= o2 or o2 + n2 <= off, "overlapping regions"
        self.live[tk.rid] = (off, nb)
        self.max_end = max(self.max_end, off + nb)
        super().launch(tk, si)

    def done(self, tk):
        fin = super().done(tk)
        if fin:
            self.live.pop(tk.rid, None)
        return fin


def test_pool_regions_are_disjoint_and_reused():
    sizes = [(64, 64), (200, 100), (32, 32), (128, 96), (256, 256), (16, 16)]
    budget = serve.RenderRequest(0, 256, 256).nbytes() + serve.RenderRequest(0, 200, 100).nbytes()
    ex = RegionCheckingExecutor(budget, us_per_unit=0.02, num_streams=4)
    s = serve.Server(ex, budget)
    rng = np.random.default_rng(0)
    tks = [s.submit(_render(*sizes[int(rng.integers(len(sizes)))])) for _ in range(60)]
    assert s.drain(timeout=60)
    assert all(t.status == 0 for t in tks)
    info = s.info()
    assert info["used_bytes"] == 0 and info["held"] == 0 and info["completed"] == 60
    assert info["peak_used_bytes"] <= budget and ex.max_end <= budget


def test_failed_launch_is_reported_and_serving_continues():
    ex = RegionCheckingExecutor(1 << 30, fail={1, 3}, us_per_unit=0.01)
    s = serve.Server(ex, 1 << 30)
    tks = [s.submit(_render(32, 32)) for _ in range(5)]
    assert s.drain(timeout=30)
    assert [t.status for t in tks] == [0, -1, 0, -1, 0]
    assert tks[1].error == "invalid argument" and tks[0].error is None
    assert s.info()["used_bytes"] == 0


def test_native_api_errors():
    import ctypes
    from nglod_gb300 import _lib
    lib = _lib.load()
    s = serve.Server(FakeExecutor(), 1 << 20)
    assert lib.nglod_serve_release(s._h, 12345, 0, None) == -1
    assert b"not a polled" in lib.nglod_last_error()
    bad = serve.RenderRequest(0, 0, 10).native()
    assert lib.nglod_serve_request_bytes(ctypes.byref(bad)) == 0
    rid = ctypes.c_int64()
    assert lib.nglod_serve_submit(s._h, ctypes.byref(bad), -1.0, ctypes.byref(rid)) == -1
    cfg = _lib.ServeConfig(1 << 20, 0, 0)
    h = ctypes.c_void_p()
    assert lib.nglod_serve_start(ctypes.byref(cfg), ctypes.byref(h)) == -1  # num_slots 0: rejected before CUDA
    s.stop(0.1)
    with pytest.raises(RuntimeError, match="stopped"):
        s.submit(_render(8, 8))
    s.close()
