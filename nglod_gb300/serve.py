"""Continuous-batching request server for resident neural SDFs.

The reference has no serving layer (its GLUT viewer renders one frame at a
time, sol-renderer/sdfRenderer.cpp:217-242).  ``Server`` keeps several
models resident on the GPU and serves two request kinds as they arrive:

    RenderRequest   a width x height pinhole render (camera rays generated on
                    the device, BF16 or float32 persistent sphere tracer) ->
                    RenderBuffer (x, depth, hit, normal) on the device
    QueryRequest    SDF values of a point batch at a LOD -> [N, 1]

Scheduling.  Requests wait in arrival order until (a) their device memory
(ray state and outputs, counted in bytes) fits under the HBM budget next to
the requests already running and (b) a stream is free.  Each admitted
request is enqueued on its own CUDA stream, so requests of different models,
resolutions and LODs run on the GPU at the same time; a request that arrives
while others are on the GPU is admitted as soon as budget and a stream free
up.  Completion is detected by polling CUDA events, never by blocking the
device.  Results are bit-identical to serving the same request alone: every
kernel computes each ray / point independently of the others in its launch.

``stats()`` reports p50 / p99 latency (arrival to completion, host
monotonic clock) beside rays/s and queries/s.  ``stop(timeout)`` waits for
running work with a bounded wait and reports what did not finish.
"""
import collections
import dataclasses
import itertools
import math
import time
from typing import Optional

import numpy as np
import torch

RENDER_BYTES_PER_RAY = 12 + 12 + 12 + 4 + 1 + 12  # org, dir, x, t, hit, normal
QUERY_BYTES_PER_POINT = 12 + 4


@dataclasses.dataclass
class RenderRequest:
    model: int
    width: int
    height: int
    lod: Optional[int] = None
    eye: tuple = (0.0, 0.0, 4.0)
    at: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    fov: float = 30.0
    num_steps: int = 64

    def nbytes(self):
        return self.width * self.height * RENDER_BYTES_PER_RAY + 64

    def units(self):
        return self.width * self.height


@dataclasses.dataclass
class QueryRequest:
    model: int
    points: torch.Tensor
    lod: Optional[int] = None

    def nbytes(self):
        return self.points.shape[0] * QUERY_BYTES_PER_POINT + 64

    def units(self):
        return self.points.shape[0]


@dataclasses.dataclass
class Ticket:
    rid: int
    request: object
    t_arrival: float
    t_admit: float = math.nan
    t_done: float = math.nan
    stream: object = None
    handle: object = None
    result: object = None

    @property
    def latency_ms(self):
        return (self.t_done - self.t_arrival) * 1e3


class CudaExecutor:
    """Launches requests on CUDA streams with the nglod_gb300 kernels."""

    def __init__(self, models, device, num_streams, tracer_args=None):
        from .options import default_args
        from .tracer import SphereTracer
        self.models = models
        self.device = device
        self.streams = [torch.cuda.Stream(device=device) for _ in range(num_streams)]
        self.tracer_args = tracer_args or default_args()

        self._tracer_cls = SphereTracer

    def launch(self, ticket, stream_index):
        from . import _lib
        req = ticket.request
        s = self.streams[stream_index]
        model = self.models[req.model]
        with torch.cuda.stream(s):
            if isinstance(req, RenderRequest):
                n = req.width * req.height
                org = torch.empty(n, 3, device=self.device)
                dr = torch.empty(n, 3, device=self.device)
                e = np.asarray(req.eye, np.float32)
                a = np.asarray(req.at, np.float32)
                u = np.asarray(req.up, np.float32)
                _lib.check(_lib.load().nglod_camera_rays(e.ctypes.data_as(_lib.ctypes.c_void_p),
                                                         a.ctypes.data_as(_lib.ctypes.c_void_p),
                                                         u.ctypes.data_as(_lib.ctypes.c_void_p), req.fov, req.width,
                                                         req.height, _lib.ptr(org), _lib.ptr(dr),
                                                         _lib.ctypes.c_void_p(s.cuda_stream)), "nglod_camera_rays")
                tracer = self._tracer_cls(self.tracer_args, num_steps=req.num_steps)
                old = model.lod
                model.lod = req.lod
                rb = tracer(model, org, dr)
                model.lod = old
                ticket.result = rb
            else:
                pts = req.points
                if not pts.is_cuda:
                    pts = pts.to(self.device, non_blocking=True)
                if hasattr(model, "tiles"):  # BF16 form
                    out = model.sdf(pts, lod=req.lod)
                else:
                    with torch.no_grad():
                        out = model.sdf(pts, lod=req.lod)
                ticket.result = out
            ev = torch.cuda.Event()
            ev.record(s)
        ticket.handle = ev

    def done(self, ticket):
        return ticket.handle.query()

    def wait(self, ticket, timeout):
        t0 = time.monotonic()
        while not ticket.handle.query():
            if time.monotonic() - t0 > timeout:
                return False
            time.sleep(1e-4)
        return True


class Server:
    def __init__(self, executor, hbm_budget_bytes, num_streams=None):
        self.ex = executor
        self.budget = int(hbm_budget_bytes)
        self.num_streams = num_streams or len(getattr(executor, "streams", [None] * 8))
        self.pending = collections.deque()
        self.running = {}
        self.free_streams = list(range(self.num_streams))
        self.finished = []
        self.used = 0
        self.peak_used = 0
        self.max_concurrent = 0
        self._ids = itertools.count()
        self._t_first = None
        self._t_last = None

    # -- submission -------------------------------------------------------------
    def submit(self, request, t_arrival=None):
        if request.nbytes() > self.budget:
            raise ValueError(f"request needs {request.nbytes()} B, more than the whole budget {self.budget} B")
        t = time.monotonic() if t_arrival is None else t_arrival
        tk = Ticket(next(self._ids), request, t)
        self.pending.append(tk)
        if self._t_first is None:
            self._t_first = t
        return tk

    # -- progress ---------------------------------------------------------------
    def poll(self):
        """Retire finished requests, admit waiting ones; returns newly finished tickets."""
        now = time.monotonic()
        done = []
        for rid, (tk, si) in list(self.running.items()):
            if self.ex.done(tk):
                tk.t_done = now
                self.used -= tk.request.nbytes()
                self.free_streams.append(si)
                del self.running[rid]
                done.append(tk)
                self.finished.append(tk)
                self._t_last = now
        while self.pending and self.free_streams:
            tk = self.pending[0]
            need = tk.request.nbytes()
            if self.used + need > self.budget:
                break
            self.pending.popleft()
            si = self.free_streams.pop(0)
            tk.t_admit = time.monotonic()
            self.used += need
            self.peak_used = max(self.peak_used, self.used)
            self.ex.launch(tk, si)
            self.running[tk.rid] = (tk, si)
            self.max_concurrent = max(self.max_concurrent, len(self.running))
        return done

    def idle(self):
        return not self.pending and not self.running

    def drain(self, timeout=60.0):
        t0 = time.monotonic()
        while not self.idle():
            self.poll()
            if time.monotonic() - t0 > timeout:
                return False
            time.sleep(5e-5)
        return True

    def stop(self, timeout=10.0):
        """Bounded shutdown: waits up to `timeout` for running requests, drops
        the waiting ones, returns (finished, unfinished_running, dropped)."""
        dropped = list(self.pending)
        self.pending.clear()
        t0 = time.monotonic()
        for rid, (tk, _) in list(self.running.items()):
            left = max(0.0, timeout - (time.monotonic() - t0))
            self.ex.wait(tk, left)
        self.poll()
        return len(self.finished), len(self.running), len(dropped)

    # -- statistics -------------------------------------------------------------
    def stats(self):
        lat = np.array([t.latency_ms for t in self.finished]) if self.finished else np.zeros(0)
        span = (self._t_last - self._t_first) if self.finished else float("nan")
        rays = sum(t.request.units() for t in self.finished if isinstance(t.request, RenderRequest))
        pts = sum(t.request.units() for t in self.finished if isinstance(t.request, QueryRequest))
        by_kind = {}
        for t in self.finished:
            r = t.request
            key = f"render_{r.width}x{r.height}" if isinstance(r, RenderRequest) else "query"
            by_kind.setdefault(key, []).append(t.latency_ms)
        pct = lambda a, q: float(np.percentile(a, q)) if len(a) else None
        return {
            "requests": len(self.finished),
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": float(lat.max()) if len(lat) else None,
            "rays_per_s": rays / span if span > 0 else None, "queries_per_s": pts / span if span > 0 else None,
            "span_s": span, "peak_budget_bytes": self.peak_used, "budget_bytes": self.budget,
            "max_concurrent": self.max_concurrent,
            "by_kind": {k: {"n": len(v), "p50_ms": pct(v, 50), "p99_ms": pct(v, 99)} for k, v in by_kind.items()},
        }


def poisson_workload(duration_s, rate_hz, num_models, seed=0, sizes=((256, 256), (512, 512), (1280, 720), (1920, 1080)),
                     lods=(0, 1, 2, 3, 4), query_range=(1e4, 1e6), render_fraction=0.5):
    """Seeded request stream: (arrival offset s, request spec dict) list.

    Arrivals are a Poisson process; half the requests (by default) are renders
    of a uniformly chosen size at a uniformly chosen LOD, the rest point
    queries of log-uniform size.  Points are generated lazily by the driver.
    """
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        model = int(rng.integers(num_models))
        lod = int(rng.choice(lods))
        if rng.random() < render_fraction:
            w, h = sizes[int(rng.integers(len(sizes)))]
            out.append((t, {"kind": "render", "model": model, "width": w, "height": h, "lod": lod}))
        else:
            n = int(round(math.exp(rng.uniform(math.log(query_range[0]), math.log(query_range[1])))))
            out.append((t, {"kind": "query", "model": model, "n": n, "lod": lod, "seed": int(rng.integers(1 << 30))}))
    return out


def run_workload(server, workload, make_points, poll_sleep=5e-5):
    """Submits each request at its arrival time (relative to now) and polls
    until everything has finished; returns the server's stats."""
    t0 = time.monotonic()
    i = 0
    while i < len(workload) or not server.idle():
        now = time.monotonic() - t0
        while i < len(workload) and workload[i][0] <= now:
            off, spec = workload[i]
            if spec["kind"] == "render":
                req = RenderRequest(spec["model"], spec["width"], spec["height"], spec["lod"])
            else:
                req = QueryRequest(spec["model"], make_points(spec), spec["lod"])
            server.submit(req, t_arrival=t0 + off)
            i += 1
        server.poll()
        time.sleep(poll_sleep)
    return server.stats()
