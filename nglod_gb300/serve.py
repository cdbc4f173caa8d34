"""Continuous-batching request server for resident neural SDFs.

The reference has no serving layer (its GLUT viewer renders one frame at a
time, sol-renderer/sdfRenderer.cpp:217-242).  ``Server`` keeps several
models resident on the GPU and serves two request kinds as they arrive:

    RenderRequest   a width x height pinhole render (camera rays generated on
                    the device, BF16 or float32 persistent sphere tracer) ->
                    RenderBuffer (x, depth, hit, normal) on the device
    QueryRequest    SDF values of a point batch at a LOD -> [N, 1]

Scheduling is native (``nglod_serve_*``, csrc/serve.cu): requests wait in
arrival order until (a) their device state (ray state and results, counted
in bytes) fits in the server's pool of ``hbm_budget_bytes`` next to the
requests already there and (b) a slot (one CUDA stream each) is free.
Admitted requests of different models, resolutions and LODs run on the GPU
at the same time; a request that arrives while others run is admitted as
soon as memory and a slot free up.  Completion is detected by polling CUDA
events, never by blocking the device.  Results are bit-identical to serving
the same request alone: every kernel computes each ray / point
independently of the others in its launch.

``stats()`` reports p50 / p99 latency (arrival to completion, host
monotonic clock) beside rays/s and queries/s.  ``stop(timeout)`` waits for
running work with a bounded wait and reports what did not finish.

Executors: ``CudaExecutor`` (resident models on one device) runs requests
with the library's kernels.  Any other object with ``launch(ticket, slot)``
and ``done(ticket)`` methods is driven through the same native scheduler by
callbacks (used to test the scheduling on hosts without a GPU).
"""
import ctypes
import dataclasses
import math
import time
from typing import Optional

import numpy as np
import torch

from . import _lib


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

    def native(self, trace_params=None):
        r = _lib.ServeRequest()
        r.kind = _lib.SERVE_RENDER
        r.model = self.model
        r.lod = -1 if self.lod is None else int(self.lod)
        r.width, r.height = self.width, self.height
        r.eye[:], r.at[:], r.up[:] = [float(v) for v in self.eye], [float(v) for v in self.at], \
            [float(v) for v in self.up]
        r.fov_deg = float(self.fov)
        if trace_params is not None:
            r.trace = trace_params
        r.trace.num_steps = int(self.num_steps)
        return r

    def nbytes(self):
        """Device bytes the server's pool holds for this request."""
        return int(_lib.load().nglod_serve_request_bytes(ctypes.byref(self.native())))

    def units(self):
        return self.width * self.height


@dataclasses.dataclass
class QueryRequest:
    model: int
    points: torch.Tensor
    lod: Optional[int] = None

    def native(self, points_ptr=None):
        r = _lib.ServeRequest()
        r.kind = _lib.SERVE_QUERY
        r.model = self.model
        r.lod = -1 if self.lod is None else int(self.lod)
        r.n = int(self.points.shape[0])
        # any non-null address sizes the request; submit passes the real one
        r.points = points_ptr if points_ptr is not None else (self.points.data_ptr() or 16)
        return r

    def nbytes(self):
        return int(_lib.load().nglod_serve_request_bytes(ctypes.byref(self.native())))

    def units(self):
        return self.points.shape[0]


@dataclasses.dataclass
class Ticket:
    rid: int
    request: object
    t_arrival: float
    t_admit: float = math.nan
    t_done: float = math.nan
    status: int = 0
    error: Optional[str] = None
    handle: object = None
    result: object = None
    inputs: object = None
    region: Optional[tuple] = None  # (offset, bytes) of its pool region while admitted

    @property
    def latency_ms(self):
        return (self.t_done - self.t_arrival) * 1e3


class _DeviceArray:
    """__cuda_array_interface__ view of a finished result in the server's pool."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None, "stream": None}


def _pool_tensor(ptr, shape, typestr, device):
    return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device=device).clone()


class CudaExecutor:
    """Resident models (``OctreeSDF`` float32 or ``Bf16OctreeSDF``) on one
    device, run by the library's kernels; ``num_streams`` slots."""

    def __init__(self, models, device, num_streams, tracer_args=None):
        from .options import default_args
        self.models = models
        self.device = torch.device(device)
        self.streams = [None] * num_streams
        self.tracer_args = tracer_args or default_args()

    def trace_params(self):
        a = self.tracer_args
        p = _lib.TraceParams()
        p.num_steps = int(a.num_steps)
        p.min_dis = float(np.float32(a.min_dis))
        p.osc_dis = float(np.float32(a.min_dis * 3))
        p.step_size = float(np.float32(a.step_size))
        p.far_clip = float(np.float32(a.camera_clamp[1]))
        p.lod = -1
        p.want_normals = 1
        return p

    def start(self, config):
        from .bf16 import Bf16OctreeSDF
        lib = _lib.load()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.nglod_serve_start(ctypes.byref(config), ctypes.byref(h)), "nglod_serve_start")
        keep = []
        for m in self.models:
            mid = ctypes.c_int32()
            if isinstance(m, Bf16OctreeSDF):
                st = lib.nglod_serve_add_model_bf16(h, ctypes.byref(m._m), ctypes.byref(mid))
            else:
                dm = m.dense_model()
                keep.append(dm)
                st = lib.nglod_serve_add_model_f32(h, ctypes.byref(dm), ctypes.byref(mid))
            if st != 0:
                lib.nglod_serve_destroy(h)
                _lib.check(st, "nglod_serve_add_model")
        return h, keep

    def prepare(self, request):
        """(native request, tensors to keep alive until completion)."""
        if isinstance(request, RenderRequest):
            return request.native(self.trace_params()), None
        pts = request.points
        if not pts.is_cuda or pts.device != self.device:
            pts = pts.to(self.device, non_blocking=True)
        pts = pts.detach().float().contiguous()
        r = request.native(pts.data_ptr() or 16)
        r.has_ready_stream = 1
        r.ready_stream = torch.cuda.current_stream(self.device).cuda_stream
        return r, pts

    def collect(self, res, request):
        n, dev = res.units, self.device
        if isinstance(request, RenderRequest):
            from .tracer import RenderBuffer
            return RenderBuffer(x=_pool_tensor(res.x, (n, 3), "<f4", dev),
                                depth=_pool_tensor(res.t, (n, 1), "<f4", dev),
                                hit=_pool_tensor(res.hit, (n,), "|u1", dev).view(torch.bool),
                                normal=_pool_tensor(res.normal, (n, 3), "<f4", dev))
        if n == 0:
            return torch.empty(0, 1, device=dev)
        return _pool_tensor(res.sdf, (n, 1), "<f4", dev)

    def release_stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream


class Server:
    def __init__(self, executor, hbm_budget_bytes, num_streams=None):
        self.ex = executor
        self.budget = int(hbm_budget_bytes)
        self.num_streams = num_streams or len(getattr(executor, "streams", [None] * 8))
        self.finished = []
        self._live = {}       # native ticket -> Ticket, submitted and not yet polled
        self._incoming = None  # the Ticket being submitted (launch callbacks may see it first)
        self._t_first = None
        self._t_last = None
        self._lib = _lib.load()
        cfg = _lib.ServeConfig(self.budget, self.num_streams, 0)
        self._native = isinstance(executor, CudaExecutor)
        self._keep = []
        if self._native:
            self._h, self._keep = executor.start(cfg)
        else:
            self._h = ctypes.c_void_p()
            self._cb = (_lib.SERVE_LAUNCH_FN(self._launch_cb), _lib.SERVE_QUERY_FN(self._query_cb))
            exs = _lib.ServeExecutor(None, *self._cb)
            _lib.check(self._lib.nglod_serve_start_custom(ctypes.byref(cfg), ctypes.byref(exs), ctypes.byref(self._h)),
                       "nglod_serve_start_custom")

    # -- callbacks of a non-CUDA executor ----------------------------------------
    def _ticket(self, rid):
        tk = self._live.get(rid)
        if tk is None:
            tk = self._incoming
            tk.rid = rid
        return tk

    def _launch_cb(self, ctx, rid, slot, req, region, nbytes):
        try:
            tk = self._ticket(rid)
            tk.region = (region, nbytes)
            self.ex.launch(tk, slot)
            return 0
        except Exception:  # noqa: BLE001 - reported as a failed request
            return -1

    def _query_cb(self, ctx, rid, slot):
        try:
            return 1 if self.ex.done(self._ticket(rid)) else 0
        except Exception:  # noqa: BLE001
            return -1

    # -- submission -------------------------------------------------------------
    def submit(self, request, t_arrival=None):
        t = time.monotonic() if t_arrival is None else t_arrival
        if self._native:
            req, inputs = self.ex.prepare(request)
        else:
            req, inputs = request.native(), None
        tk = Ticket(-1, request, t, inputs=inputs)
        rid = ctypes.c_int64(-1)
        self._incoming = tk
        try:
            st = self._lib.nglod_serve_submit(self._h, ctypes.byref(req), float(t), ctypes.byref(rid))
        finally:
            self._incoming = None
        if st == -4:
            raise ValueError(f"request needs {request.nbytes()} B, more than the whole budget {self.budget} B")
        _lib.check(st, "nglod_serve_submit")
        tk.rid = rid.value
        self._live[tk.rid] = tk
        if self._t_first is None:
            self._t_first = t
        return tk

    # -- progress ---------------------------------------------------------------
    def poll(self):
        """Retire finished requests, admit waiting ones; returns newly finished tickets."""
        done = []
        buf = (_lib.ServeResult * 64)()
        cnt = ctypes.c_int32()
        while True:
            _lib.check(self._lib.nglod_serve_poll(self._h, buf, 64, ctypes.byref(cnt)), "nglod_serve_poll")
            for res in buf[:cnt.value]:
                tk = self._live.pop(res.ticket)
                tk.t_admit, tk.t_done, tk.status = res.t_admit, res.t_done, res.status
                if res.status == 0:
                    if self._native:
                        tk.result = self.ex.collect(res, tk.request)
                else:
                    tk.error = _lib.STATUS.get(res.status, str(res.status))
                tk.inputs = None
                if self._native:
                    st = self._lib.nglod_serve_release(self._h, res.ticket, 1,
                                                       ctypes.c_void_p(self.ex.release_stream()))
                else:
                    st = self._lib.nglod_serve_release(self._h, res.ticket, 0, None)
                _lib.check(st, "nglod_serve_release")
                done.append(tk)
                self.finished.append(tk)
                self._t_last = tk.t_done
            if cnt.value < 64:
                return done

    def info(self):
        i = _lib.ServeInfo()
        _lib.check(self._lib.nglod_serve_get_info(self._h, ctypes.byref(i)), "nglod_serve_get_info")
        return {f[0]: getattr(i, f[0]) for f in i._fields_}

    @property
    def peak_used(self):
        return self.info()["peak_used_bytes"]

    @property
    def max_concurrent(self):
        return self.info()["max_concurrent"]

    def idle(self):
        return not self._live

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
        unfinished, dropped = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self._lib.nglod_serve_stop(self._h, float(timeout), ctypes.byref(unfinished), ctypes.byref(dropped)),
                   "nglod_serve_stop")
        self.poll()
        return len(self.finished), unfinished.value, dropped.value

    def close(self):
        """Waits for the server's streams and frees its pool (nglod_serve_destroy)."""
        if getattr(self, "_h", None) and self._h.value:
            h, self._h = self._h, ctypes.c_void_p()
            _lib.check(self._lib.nglod_serve_destroy(h), "nglod_serve_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

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
        info = self.info()
        return {
            "requests": len(self.finished),
            "failed": sum(1 for t in self.finished if t.status != 0),
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": float(lat.max()) if len(lat) else None,
            "rays_per_s": rays / span if span > 0 else None, "queries_per_s": pts / span if span > 0 else None,
            "span_s": span, "peak_budget_bytes": info["peak_used_bytes"], "budget_bytes": self.budget,
            "max_concurrent": info["max_concurrent"],
            "by_kind": {k: {"n": len(v), "p50_ms": pct(v, 50), "p99_ms": pct(v, 99)} for k, v in by_kind.items()},
        }


def poisson_workload(duration_s, rate_hz, num_models, seed=0, sizes=((256, 256), (512, 512), (1280, 720), (1920, 1080)),
                     lods=(0, 1, 2, 3, 4), query_range=(1e4, 1e6), render_fraction=0.5):
    """Seeded request stream: (arrival offset s, request spec dict) list.

    Arrivals are a Poisson process; half the requests (by default) are renders
    of a uniformly chosen size at a uniformly chosen LOD, the rest point
    queries of log-uniform size.  run_workload makes the points when it
    submits each query.
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
