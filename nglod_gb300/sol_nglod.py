"""Drop-in for the reference's ``sol_nglod`` CUDA extension.

``aabb(ray_o, ray_d) -> [x, t, hit]`` mirrors
sdf-net/lib/extensions/sol_nglod/sol_nglod_kernel.cu:161-192: x [N, 3] is the
entry point into [-1, 1]^3 (ray_o where the ray misses or starts inside the
box), t [N, 1] the entry distance (0 where not hit), hit [N] bool.  Launches
on torch's current stream (the reference used the legacy default stream).
"""
import torch

from . import _lib


def aabb(ray_o, ray_d):
    _lib.require_cuda(ray_o, ray_d)
    if ray_o.dtype != torch.float32 or ray_d.dtype != torch.float32:
        raise RuntimeError("aabb: float32 rays required")
    ray_o = ray_o.contiguous()
    ray_d = ray_d.contiguous()
    n = ray_o.shape[0]
    x = torch.empty_like(ray_o)
    t = torch.empty(n, 1, device=ray_o.device, dtype=torch.float32)
    hit = torch.empty(n, device=ray_o.device, dtype=torch.bool)
    _lib.check(_lib.load().nglod_aabb(_lib.ptr(ray_o), _lib.ptr(ray_d), n, _lib.ptr(x), _lib.ptr(t), _lib.ptr(hit),
                                      _lib.stream_ptr(ray_o.device)), "nglod_aabb")
    return [x, t, hit]
