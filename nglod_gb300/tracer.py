"""Drop-in ``SphereTracer`` / ``BaseTracer`` / ``RenderBuffer``.

Mirrors sdf-net/lib/tracer/BaseTracer.py:26-52, SphereTracer.py:39-132 and
RenderBuffer.py:28-137.  ``SphereTracer.forward(net, ray_o, ray_d)`` runs the
whole march (aabb prologue, march loop, AABB cull, finite-difference normals)
in one persistent kernel launch (``nglod_trace``) with no host
synchronisation.  ``PlainSphereTracer`` keeps the reference's host-driven loop
structure (per-step masks, compaction and a ``cond.any()`` sync) on the GPU,
calling the fused sdf kernel once per step; it is the plain float32 GPU form
that the persistent tracers are compared against.
"""
from dataclasses import astuple, dataclass, fields
from typing import Union

import numpy as np
import torch
import torch.nn.functional as F

from . import _lib
from .octree_sdf import OctreeSDF, setparam
from .sol_nglod import aabb


@dataclass
class RenderBuffer:
    x: Union[torch.Tensor, None] = None
    min_x: Union[torch.Tensor, None] = None
    hit: Union[torch.Tensor, None] = None
    depth: Union[torch.Tensor, None] = None
    relative_depth: Union[torch.Tensor, None] = None
    normal: Union[torch.Tensor, None] = None
    rgb: Union[torch.Tensor, None] = None
    shadow: Union[torch.Tensor, None] = None
    ao: Union[torch.Tensor, None] = None
    view: Union[torch.Tensor, None] = None
    err: Union[torch.Tensor, None] = None
    albedo: Union[torch.Tensor, None] = None

    def __iter__(self):
        return iter(astuple(self))

    def __add__(self, other):
        def cat(pair):
            a, b = pair
            if a is not None and b is not None:
                return torch.cat(pair)
            return a if a is not None else b
        return self.__class__(*map(cat, zip(self, other)))

    def _apply(self, fn):
        return self.__class__(**{f.name: (None if getattr(self, f.name) is None else fn(getattr(self, f.name)))
                                 for f in fields(self)})

    def cuda(self):
        return self._apply(lambda t: t.cuda())

    def cpu(self):
        return self._apply(lambda t: t.cpu())

    def detach(self):
        return self._apply(lambda t: t.detach())

    def byte(self):
        return self._apply(lambda t: t.byte())

    def float(self):
        return self._apply(lambda t: t.float())

    def reshape(self, *dims):
        return self._apply(lambda t: t.reshape(*dims))

    def transpose(self):
        """[W, H, C] images -> [H, W, C] (RenderBuffer.py:86-88)."""
        return self._apply(lambda t: t.permute(1, 0, 2))

    def numpy(self):
        return self._apply(lambda t: t.numpy())

    def exrdict(self):
        """The set fields, rgb renamed 'default' (RenderBuffer.py:98-104)."""
        d = {f.name: getattr(self, f.name) for f in fields(self) if getattr(self, f.name) is not None}
        if "rgb" in d:
            d["default"] = d.pop("rgb")
        return d


class BaseTracer(object):
    """BaseTracer.py:26-52: settings come from ``args`` unless passed."""

    def __init__(self, args=None, camera_clamp=None, step_size=None, grad_method=None, num_steps=None,
                 min_dis=None):
        self.args = args
        self.camera_clamp = setparam(args, camera_clamp, "camera_clamp")
        self.step_size = setparam(args, step_size, "step_size")
        self.grad_method = setparam(args, grad_method, "grad_method")
        self.num_steps = setparam(args, num_steps, "num_steps")
        self.min_dis = setparam(args, min_dis, "min_dis")
        self.inv_num_steps = 1.0 / self.num_steps
        self.diagonal = np.sqrt(3) * 2.0

    def __call__(self, *args, **kwargs):
        return self.forward(*args, **kwargs)

    def forward(self, net, ray_o, ray_d):
        raise NotImplementedError

    def trace_params(self, net):
        p = _lib.TraceParams()
        p.num_steps = int(self.num_steps)
        # Thresholds as the reference compares them: Python floats against
        # float32 tensors, i.e. rounded to float32 (SphereTracer.py:84-90).
        p.min_dis = float(np.float32(self.min_dis))
        p.osc_dis = float(np.float32(self.min_dis * 3))
        p.step_size = float(np.float32(self.step_size))
        p.far_clip = float(np.float32(self.camera_clamp[1]))
        p.lod = -1 if net.lod is None else int(net.lod)
        p.want_normals = 1
        return p


def _check_net(net, grad_method):
    from .bf16 import Bf16OctreeSDF
    if not isinstance(net, (OctreeSDF, Bf16OctreeSDF)):
        raise TypeError("nglod_gb300.SphereTracer traces nglod_gb300.OctreeSDF / Bf16OctreeSDF networks")
    if grad_method != "finitediff":
        raise NotImplementedError(f"grad_method={grad_method!r}: the fused tracer computes 'finitediff' normals")


def _sdf_fn(net):
    """The network's sdf at its current lod through the library's query
    kernels (the reference calls ``net(x)``)."""
    if isinstance(net, OctreeSDF):
        lod = net.lod if net.lod is not None and 0 <= net.lod < net.num_lods else None
        return lambda p: net._sdf_infer(p, lod, False)
    return lambda p: net(p)


def get_min(tracer, net, ray_o, ray_d):
    """SphereTracer.get_min (sdf-net/lib/tracer/SphereTracer.py:134-218): the
    march of ``forward`` with the reference's get_min rules, and per ray the
    point of the smallest sdf seen (``min_x``).  Its rules, kept as they are:
    every ray marches from the start (``cond`` is recomputed each step from
    |d|, the oscillation test and |t| < far, not carried over), including rays
    that miss the box (they start at their origin, t = 0); ``min_x`` takes the
    point the step just moved to wherever the previous step's d is below the
    running minimum; hit rays get the finite-difference gradient, not
    normalised.  Each step's evaluations go through the library's sdf kernel
    on the compacted active points.  The reference builds its result with
    ``RenderBuffer(..., minx=minx)``, a keyword its RenderBuffer does not have
    (the field is ``min_x``), so as shipped it raises TypeError on its last
    line; this returns the buffer with ``min_x`` set."""
    _check_net(net, tracer.grad_method)
    f = _sdf_fn(net)
    x, t, hit = aabb(ray_o, ray_d)
    normal = torch.zeros_like(x)
    with torch.no_grad():
        d = f(x)
        dprev = d.clone()
        mind = d.clone()
        minx = x.clone()
        for _ in range(tracer.num_steps):
            hit = (torch.abs(t) < tracer.camera_clamp[1])[:, 0]
            cond = (torch.abs(d) > tracer.min_dis)[:, 0]
            cond = cond & (torch.abs((d + dprev) / 2.0) > tracer.min_dis * 3)[:, 0]
            cond = cond & hit
            if not cond.any():
                break
            x = torch.where(cond.view(-1, 1), torch.addcmul(ray_o, ray_d, t), x)
            new_mins = (d < mind)[..., 0]
            mind[new_mins] = d[new_mins]
            minx[new_mins] = x[new_mins]
            dprev = torch.where(cond.unsqueeze(1), d, dprev)
            d[cond] = f(x[cond]) * tracer.step_size
            t = torch.where(cond.view(-1, 1), t + d, t)
        hit = hit & ~(torch.abs(x) > 1.0).any(dim=-1)
        xh = x[hit]
        h = 1.0 / (64.0 * 3.0)
        eps = torch.eye(3, device=x.device) * h
        normal[hit] = torch.cat([f(xh + eps[k]) - f(xh - eps[k]) for k in range(3)], dim=-1) / (h * 2.0)
    return RenderBuffer(x=x, depth=t, hit=hit, normal=normal, min_x=minx)


class SphereTracer(BaseTracer):
    """Persistent fused sphere tracer (one kernel launch per call).

    A float32 ``OctreeSDF`` is traced by ``nglod_trace``; a ``Bf16OctreeSDF``
    (the BF16 form) by ``nglod_trace_bf16``, which evaluates 128 rays per
    block on the tensor cores.
    """

    def get_min(self, net, ray_o, ray_d):
        return get_min(self, net, ray_o, ray_d)

    def forward(self, net, ray_o, ray_d):
        _check_net(net, self.grad_method)
        from .bf16 import Bf16OctreeSDF
        if isinstance(net, Bf16OctreeSDF):
            return self._forward_bf16(net, ray_o, ray_d)
        _lib.require_cuda(ray_o, ray_d)
        ray_o = ray_o.detach().float().contiguous()
        ray_d = ray_d.detach().float().contiguous()
        n = ray_o.shape[0]
        dev = ray_o.device
        x = torch.empty(n, 3, device=dev, dtype=torch.float32)
        t = torch.empty(n, 1, device=dev, dtype=torch.float32)
        hit = torch.empty(n, device=dev, dtype=torch.bool)
        normal = torch.empty(n, 3, device=dev, dtype=torch.float32)
        counter = torch.empty(1, device=dev, dtype=torch.int64)
        m = net.dense_model()
        p = self.trace_params(net)
        _lib.check(_lib.load().nglod_trace(m, p, _lib.ptr(ray_o), _lib.ptr(ray_d), n, _lib.ptr(x), _lib.ptr(t),
                                           _lib.ptr(hit), _lib.ptr(normal), _lib.ptr(counter),
                                           _lib.stream_ptr(dev)), "nglod_trace")
        return RenderBuffer(x=x, depth=t, hit=hit, normal=normal)

    def _forward_bf16(self, net, ray_o, ray_d):
        _lib.require_cuda(ray_o, ray_d)
        ray_o = ray_o.detach().float().contiguous()
        ray_d = ray_d.detach().float().contiguous()
        n = ray_o.shape[0]
        dev = ray_o.device
        x = torch.empty(n, 3, device=dev, dtype=torch.float32)
        t = torch.empty(n, 1, device=dev, dtype=torch.float32)
        hit = torch.empty(n, device=dev, dtype=torch.bool)
        normal = torch.empty(n, 3, device=dev, dtype=torch.float32)
        counter = torch.empty(1, device=dev, dtype=torch.int64)
        p = self.trace_params(net)
        _lib.check(_lib.load().nglod_trace_bf16(net._m, p, _lib.ptr(ray_o), _lib.ptr(ray_d), n, _lib.ptr(x),
                                                _lib.ptr(t), _lib.ptr(hit), _lib.ptr(normal), _lib.ptr(counter),
                                                _lib.ptr(net._status), _lib.stream_ptr(dev)), "nglod_trace_bf16")
        return RenderBuffer(x=x, depth=t, hit=hit, normal=normal)


class PlainSphereTracer(BaseTracer):
    """The reference's host-driven march (SphereTracer.py:41-132) on the GPU.

    Every step builds the active mask, synchronises on ``cond.any()``,
    compacts the active points and calls the float32 sdf kernel on them
    (nglod_sdf_fwd), whose arithmetic the fused float32 tracer shares, so
    that the two march identically.

    ``last_evaluations`` (a device int64 tensor) counts the sdf evaluations of
    the last frame: the first one of every ray, one per ray and march step,
    and the six finite-difference taps of every hit ray.  The fused tracers
    march by the same rules, so it is the frame's algorithmic work for them
    too.
    """

    last_evaluations = None

    def get_min(self, net, ray_o, ray_d):
        return get_min(self, net, ray_o, ray_d)

    def forward(self, net, ray_o, ray_d):
        _check_net(net, self.grad_method)
        x, t, cond = aabb(ray_o, ray_d)
        normal = torch.zeros_like(x)
        evals = torch.full((), x.shape[0], dtype=torch.int64, device=x.device)
        dense = isinstance(net, OctreeSDF)
        lod = net.lod if dense and net.lod is not None and 0 <= net.lod < net.num_lods else None

        def f(p):
            return net._sdf_infer(p, lod, False) if dense else net(p)

        with torch.no_grad():
            d = f(x)
            dprev = d.clone()
            hit = torch.zeros_like(d).bool()[:, 0]
            for _ in range(self.num_steps):
                hit = (torch.abs(t) < self.camera_clamp[1])[:, 0]
                cond = cond & (torch.abs(d) > self.min_dis)[:, 0]
                cond = cond & (torch.abs((d + dprev) / 2.0) > self.min_dis * 3)[:, 0]
                cond = cond & hit
                if not cond.any():
                    break
                evals += cond.sum()
                x = torch.where(cond.view(-1, 1), torch.addcmul(ray_o, ray_d, t), x)
                dprev = torch.where(cond.unsqueeze(1), d, dprev)
                d[cond] = f(x[cond]) * self.step_size
                t = torch.where(cond.view(-1, 1), t + d, t)
            hit = hit & ~(torch.abs(x) > 1.0).any(dim=-1)
            xh = x[hit]
            evals += 6 * xh.shape[0]
            h = 1.0 / (64.0 * 3.0)
            eps = torch.eye(3, device=x.device) * h
            grad = torch.cat([f(xh + eps[k]) - f(xh - eps[k]) for k in range(3)], dim=-1) / (h * 2.0)
            normal[hit] = F.normalize(grad, p=2, dim=-1, eps=1e-5)
        self.last_evaluations = evals
        return RenderBuffer(x=x, depth=t, hit=hit, normal=normal)
