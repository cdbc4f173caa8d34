"""Surface samples and octrees from a network.

    sample_surface(n, net)         SphereTracer.sample_surface (sdf-net/lib/tracer/
                                   SphereTracer.py:220-245): rays with origins uniform
                                   in [-1, 1]^3 and directions uniform on the sphere,
                                   traced until n hits are collected
    voxel_sparsify(n, net, lod)    renderutils.voxel_sparsify (sdf-net/lib/renderutils.py:
                                   56-73): the occupied voxels of levels 2 .. lod+2
                                   under n surface samples
    trace_surface_points(n, net)   surface points from rays that start outside the box
    octree_from_sdf(net, level)    SPC of the voxels within one voxel diagonal of the
                                   network's zero set (what SOL_NGLOD.py:50 builds with
                                   voxel_sparsify), on the GPU

The reference's tracer counts a ray whose origin lies inside [-1, 1]^3 as a
hit at depth 0 (its aabb prologue skips such rays and its march starts with
|t| < far, SphereTracer.py:53-90), and SphereTracer.sample_surface's origins
are inside: its samples are the origins themselves.  sample_surface and
voxel_sparsify keep that behaviour (they are drop-ins);
trace_surface_points starts its rays on a sphere of radius 2 around the box,
so they march onto the surface, and voxel_sparsify(points=...) takes such
points.  (renderutils.sample_surface itself raises: it passes ``sol=`` to a
tracer constructor that has no such argument.)
"""
import ctypes
import math

import torch

from . import _lib
from .spc import SPC


def _tracer(tracer, num_steps=256):
    if tracer is not None:
        return tracer
    from .options import default_args
    from .tracer import SphereTracer
    return SphereTracer(default_args(num_steps=num_steps))


def _unif_sphere(n, device, generator=None):
    """sample_unif_sphere (geoutils.py:31-40) on the device: z = 1 - 2u,
    r = sqrt(1 - z^2), phi = 2 pi v."""
    u = torch.rand(2, n, device=device, generator=generator)
    z = 1 - 2 * u[0]
    r = torch.sqrt(torch.clamp(1 - z * z, min=0))
    phi = 2 * math.pi * u[1]
    return torch.stack([r * torch.cos(phi), r * torch.sin(phi), z], dim=1)


def _collect(n, net, tracer, make_rays, max_rounds):
    got, total = [], 0
    with torch.no_grad():
        for _ in range(max_rounds):
            ro, rd = make_rays()
            rb = tracer(net, ro, rd)
            pts = rb.x[rb.hit]
            got.append(pts)
            total += pts.shape[0]
            if total >= n:
                break
    return torch.cat(got) if got else torch.zeros(0, 3)


def sample_surface(n, net, tracer=None, device="cuda", generator=None, max_rounds=1000):
    """SphereTracer.sample_surface(n, net): hit positions of random rays
    (origins uniform in the box, directions uniform) until n are collected."""
    tr = _tracer(tracer)
    return _collect(n, net, tr, lambda: (torch.rand(n, 3, device=device, generator=generator) * 2 - 1,
                                         _unif_sphere(n, device, generator)), max_rounds)


def trace_surface_points(n, net, tracer=None, device="cuda", generator=None, max_rounds=1000):
    """Surface points: rays from uniform points on the sphere of radius 2
    towards uniform points in the box, traced; at least n hit positions."""
    tr = _tracer(tracer)

    def rays():
        o = _unif_sphere(n, device, generator) * 2.0
        target = torch.rand(n, 3, device=device, generator=generator) * 2 - 1
        d = target - o
        return o, d / d.norm(dim=1, keepdim=True)
    return _collect(n, net, tr, rays, max_rounds)


def voxel_sparsify(n, net, lod, tracer=None, points=None, device="cuda"):
    """renderutils.voxel_sparsify: [unique voxels of level i + 2 under the
    surface samples, i = 0 .. lod], each sorted lexicographically as
    torch.unique sorts.  Samples: sample_surface(n, net) (net.lod = lod while
    tracing), or ``points``."""
    if points is None:
        old = net.lod
        net.lod = lod
        try:
            points = sample_surface(n, net, tracer, device)[:n]
        finally:
            net.lod = old
    points = points.to(device).float()
    L = lod + 2
    res = 2 ** L
    v = (((points + 1.0) / 2.0) * res).floor().long()
    # voxels on the far faces (sample == 1.0) lie outside the grid and are
    # kept apart: the octree covers [0, res)
    inside = ((v >= 0) & (v < res)).all(dim=1)
    s = SPC.from_voxels(v[inside].int(), L)
    out = []
    for i in range(lod + 1):
        lv = i + 2
        pts = s.GetLevelPoints(lv)[:, :3].long()
        extra = v[~inside] >> (L - lv)
        if extra.numel():
            pts = torch.cat([pts, extra])
            pts = torch.unique(pts, dim=0)
        key = (pts[:, 0] * (2 ** lv) + pts[:, 1]) * (2 ** lv) + pts[:, 2]
        out.append(pts[torch.argsort(key)])
    return out


def octree_from_sdf(net, level, band=None, lod=None, chunk=1 << 21, device=None):
    """SPC of the voxels of the 2^level grid whose centre's |sdf| (network
    net at lod) is at most ``band`` (default: one voxel diagonal,
    sqrt(3) * 2 / 2^level), built on the GPU."""
    if device is None:
        p = net.grids[0] if hasattr(net, "grids") else net.features[0].fm
        device = p.device
    res = 2 ** level
    band = math.sqrt(3) * 2.0 / res if band is None else float(band)
    total = res ** 3
    lib = _lib.load()
    st = _lib.stream_ptr(device)
    cap = min(total, 1 << 26)
    voxels = torch.empty(cap, 3, dtype=torch.int16, device=device)
    centres = torch.empty(min(chunk, total), 3, device=device)
    parts = torch.empty(min(chunk, total) // 1024 + 2, dtype=torch.int32, device=device)
    ctrl = torch.empty(3, dtype=torch.int64, device=device)
    got = 0
    for start in range(0, total, chunk):
        cnt = min(chunk, total - start)
        _lib.check(lib.nglod_voxel_centres(level, start, cnt, _lib.ptr(centres), st), "nglod_voxel_centres")
        if hasattr(net, "tiles"):
            d = net.sdf(centres[:cnt], lod=lod)
        else:
            with torch.no_grad():
                d = net.sdf(centres[:cnt], lod=lod)
        d = d.contiguous()
        sel = ctypes.c_int64()
        _lib.check(lib.nglod_select_band(_lib.ptr(d), cnt, band, level, start, _lib.ptr(voxels), got, cap,
                                         _lib.ptr(parts), _lib.ptr(ctrl), ctypes.byref(sel), st), "nglod_select_band")
        got += sel.value
    if got == 0:
        raise RuntimeError(f"octree_from_sdf: no voxel of the 2^{level} grid lies within {band:g} of the surface")
    return SPC.from_voxels(voxels[:got].int(), level)
