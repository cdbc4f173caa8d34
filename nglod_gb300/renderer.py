"""Renderer: sphere tracing plus the shading passes, on the GPU.

Drop-in for sdf-net/lib/renderer.py's ``Renderer`` (renderer.py:39-345):

    render(net, ray_o, ray_d)          renderer.py:118-223: trace, ground plane
                                       and shadow rays, relative depth,
                                       ambient occlusion -> RenderBuffer [W, H, .]
    render_lookat(net, f, t, fov, ...) renderer.py:98-116
    shade_tensor(net, f, t, fov, mm)   renderer.py:255-290: matcap colour,
                                       segmentation, blurred shadow map, AO
    shade_images(net, f, t, fov, aa)   renderer.py:292-331: the same on the CPU,
                                       transposed to [H, W, .]

Every pass runs as a kernel of the library (nglod_shade_*, csrc/shade.cu);
tracing and the AO's 40 sdf taps per shaded ray use the network's own entry
points (float32 OctreeSDF or the BF16 form).  Deviations, all for lack of a
file or a device-side RNG of the reference: the matcap texture is an array
(``matcap=``, or a ``.npy`` path; by default a procedural green sphere,
nglod_gb300.synthetic.matcap_texture) since the reference's
data/matcap/green.png is not distributed; without ``ground_height`` the
ground plane sits at the lowest hit point of the frame (the reference takes
the lowest point of 10^6 surface samples); the shadow rays' N(0, 0.01^2)
noise comes from torch's generator on the device, or ``shadow_noise=``.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .octree_sdf import setparam
from .tracer import RenderBuffer

LIGHT = (-1.5, 4.5, -1.5)


def _u(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Renderer:
    def __init__(self, tracer, args=None, render_res=None, camera_clamp=None, camera_proj=None, render_batch=None,
                 shading_mode=None, matcap_path=None, shadow=None, ao=None, perf=None, device=None, matcap=None,
                 ground_height=None):
        self.args = args
        self.camera_clamp = tracer.camera_clamp
        self.render_res = setparam(args, render_res, "render_res")
        self.camera_proj = setparam(args, camera_proj, "camera_proj")
        self.render_batch = setparam(args, render_batch, "render_batch")
        self.shading_mode = setparam(args, shading_mode, "shading_mode")
        self.matcap_path = setparam(args, matcap_path, "matcap_path")
        self.shadow = bool(setparam(args, shadow, "shadow"))
        self.ao = bool(setparam(args, ao, "ao"))
        self.perf = setparam(args, perf, "perf")
        self.device = setparam(args, device, "device") or "cuda"
        self.ground_height = setparam(args, ground_height, "ground_height")
        self.width, self.height = self.render_res
        self.tracer = tracer
        if matcap is None:
            if self.matcap_path is not None and str(self.matcap_path).endswith(".npy"):
                matcap = np.load(self.matcap_path)
            else:
                from .synthetic import matcap_texture
                matcap = matcap_texture()
        tex = np.asarray(matcap)[..., :3].transpose(1, 0, 2).astype(np.float32)  # (width, height, 3) as the sampler
        self._texture = torch.from_numpy(np.ascontiguousarray(tex))
        self._tex_dev = {}

    # -- passes -------------------------------------------------------------------
    def _texture_on(self, dev):
        key = str(dev)
        if key not in self._tex_dev:
            self._tex_dev[key] = self._texture.to(dev)
        return self._tex_dev[key]

    def _min_hit_y(self, rb):
        key = torch.empty(1, dtype=torch.int32, device=rb.x.device)
        _lib.check(_lib.load().nglod_shade_min_hit_y(_u(rb.x), _u(rb.hit), rb.x.shape[0], _u(key),
                                                     _lib.stream_ptr(rb.x.device)), "nglod_shade_min_hit_y")
        k = int(key.item()) & 0xFFFFFFFF
        if k == 0xFFFFFFFF:
            return -1.0
        bits = (k & 0x7FFFFFFF) if k & 0x80000000 else (~k & 0xFFFFFFFF)
        return float(np.array([bits], np.uint32).view(np.float32)[0])

    def _sdf(self, net, pts):
        from .bf16 import Bf16OctreeSDF
        if isinstance(net, Bf16OctreeSDF):
            return net.sdf(pts)
        with torch.no_grad():
            return net.sdf(pts)

    def render(self, net, ray_o, ray_d, shadow_noise=None):
        """RenderBuffer reshaped to [W, H, .] (renderer.py:118-223)."""
        rb = self._render_flat(net, ray_o, ray_d, shadow_noise)
        out = RenderBuffer(x=rb.x, hit=rb.hit[:, None], depth=rb.depth, relative_depth=rb.relative_depth,
                           normal=rb.normal, shadow=None if rb.shadow is None else rb.shadow[:, None], ao=rb.ao,
                           view=rb.view)
        return out.reshape(self.width, self.height, -1)

    def _render_flat(self, net, ray_o, ray_d, shadow_noise=None):
        _lib.require_cuda(ray_o, ray_d)
        lib = _lib.load()
        dev = ray_o.device
        st = _lib.stream_ptr(dev)
        ray_o = ray_o.detach().float().contiguous()
        ray_d = ray_d.detach().float().contiguous()
        n = ray_o.shape[0]
        with torch.no_grad():
            if self.render_batch and self.render_batch > 0:
                rb = RenderBuffer()
                for o, d in zip(torch.split(ray_o, self.render_batch), torch.split(ray_d, self.render_batch)):
                    rb = rb + self.tracer(net, o, d)
            else:
                rb = self.tracer(net, ray_o, ray_d)
        hit = rb.hit.contiguous()
        plane_hit = None
        if self.shadow:
            min_y = self.ground_height if self.ground_height is not None else self._min_hit_y(rb)
            plane_hit = torch.empty(n, dtype=torch.bool, device=dev)
            _lib.check(lib.nglod_shade_ground(_u(ray_o), _u(ray_d), n, float(min_y), _u(rb.x), _u(rb.depth),
                                              _u(hit), _u(rb.normal), _u(plane_hit), st), "nglod_shade_ground")
            if shadow_noise is None:
                shadow_noise = torch.zeros_like(rb.x).normal_(0.0, 0.01)
            noise = shadow_noise.to(dev).float().contiguous()
            so = torch.empty_like(rb.x)
            sd = torch.empty_like(rb.x)
            light_hit = torch.empty(n, dtype=torch.bool, device=dev)
            light = np.asarray(LIGHT, np.float32)
            _lib.check(lib.nglod_shade_shadow_rays(_u(rb.x), _u(rb.normal), _u(noise), n,
                                                   light.ctypes.data_as(ctypes.c_void_p), _u(so), _u(sd),
                                                   _u(light_hit), st), "nglod_shade_shadow_rays")
            with torch.no_grad():
                srb = self.tracer(net, so, sd)
            rb.shadow = srb.hit.contiguous()
            rb.light_hit = light_hit
        rb.hit = hit
        rb.relative_depth = torch.empty_like(rb.depth)
        _lib.check(lib.nglod_shade_compose(None, n, None, None, _u(rb.depth), float(self.camera_clamp[1]),
                                           _u(rb.relative_depth), st), "nglod_shade_compose")
        if self.ao:
            rb.ao = self._ambient_occlusion(net, rb, plane_hit)
        rb.view = ray_d
        rb._plane_hit = plane_hit
        return rb

    def _ambient_occlusion(self, net, rb, plane_hit):
        lib = _lib.load()
        dev = rb.x.device
        st = _lib.stream_ptr(dev)
        n = rb.x.shape[0]
        idx = torch.empty(n, dtype=torch.int32, device=dev)
        parts = torch.empty(n // 1024 + 2, dtype=torch.int32, device=dev)
        ctrl = torch.empty(2, dtype=torch.int64, device=dev)
        m = ctypes.c_int64()
        _lib.check(lib.nglod_shade_ao_select(_u(rb.hit), _u(plane_hit), n, _u(idx), _u(parts), _u(ctrl),
                                             ctypes.byref(m), st), "nglod_shade_ao_select")
        m = m.value
        ao = torch.empty(n, 1, device=dev)
        r = None
        if m > 0:
            taps = torch.empty(m * 40, 3, device=dev)
            _lib.check(lib.nglod_shade_ao_taps(_u(rb.x), _u(rb.normal), _u(idx), m, _u(taps), st),
                       "nglod_shade_ao_taps")
            r = self._sdf(net, taps).contiguous()
        _lib.check(lib.nglod_shade_ao_reduce(_u(r), _u(idx), m, _u(plane_hit), n, _u(ao), st),
                   "nglod_shade_ao_reduce")
        return ao

    def render_lookat(self, net, f=(0, 0, 1), t=(0, 0, 0), fov=30.0, camera_proj="persp", device="cuda", mm=None,
                      shadow_noise=None):
        """Pinhole rays from f towards t (look_at, geoutils.py:180-206, without
        the pixel jitter), rotated by the model matrix mm, rendered (flat
        buffers, as shade_tensor consumes them)."""
        if camera_proj != "persp":
            raise NotImplementedError("camera_proj='ortho' is not built")
        W, H = self.width, self.height
        org = torch.empty(W * H, 3, device=device)
        dr = torch.empty(W * H, 3, device=device)
        e, a, u = (np.asarray(v, np.float32) for v in (f, t, (0, 1, 0)))
        _lib.check(_lib.load().nglod_camera_rays(e.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                                                 u.ctypes.data_as(ctypes.c_void_p), float(fov), W, H, _u(org),
                                                 _u(dr), _lib.stream_ptr(org.device)), "nglod_camera_rays")
        if mm is not None:
            mm = mm.to(org.device).float()
            org = torch.mm(org, mm)
            dr = torch.mm(dr, mm)
        return self._render_flat(net, org, dr, shadow_noise=shadow_noise)

    def shade_tensor(self, net, f=(0, 0, 1), t=(0, 0, 0), fov=30.0, mm=None, shadow_noise=None):
        """Shaded RenderBuffer [W, H, .] (renderer.py:255-290)."""
        if self.shading_mode != "matcap":
            raise NotImplementedError(f"shading_mode={self.shading_mode!r}: only 'matcap' is built "
                                      "(OctreeSDF has no 'rb' colour head)")
        if mm is not None and not torch.equal(mm.float().cpu(), torch.eye(3)):
            raise NotImplementedError("shade_tensor: model matrices other than the identity are not built")
        return self.shade_buffer(self.render_lookat(net, f=f, t=t, fov=fov, shadow_noise=shadow_noise))

    def shade_buffer(self, rb):
        """shade_tensor's passes on a rendered buffer (flat rays)."""
        lib = _lib.load()
        dev = rb.x.device
        st = _lib.stream_ptr(dev)
        n = rb.x.shape[0]
        W, H = self.width, self.height
        tex = self._texture_on(dev)
        rgb = torch.empty(n, 3, device=dev)
        _lib.check(lib.nglod_shade_matcap(_u(rb.view), _u(rb.normal), _u(rb.hit), n, _u(tex), tex.shape[0],
                                          tex.shape[1], _u(rgb), st), "nglod_shade_matcap")
        rb.normal = torch.where(rb.hit[:, None], rb.normal, torch.ones_like(rb.normal))
        smap = None
        if self.shadow:
            smap = torch.empty(n, device=dev)
            scratch = torch.empty(n, device=dev)
            shadow = torch.empty(n, dtype=torch.bool, device=dev)
            _lib.check(lib.nglod_shade_shadow_map(_u(rb.shadow), _u(rb.light_hit), W, H, 2.0, _u(smap), _u(scratch),
                                                  _u(shadow), st), "nglod_shade_shadow_map")
            rb.shadow = shadow
        _lib.check(lib.nglod_shade_compose(_u(rgb), n, _u(smap), _u(rb.ao), None, float(self.camera_clamp[1]),
                                           None, st), "nglod_shade_compose")
        rb.rgb = rgb
        out = RenderBuffer(x=rb.x, hit=rb.hit[:, None], depth=rb.depth, relative_depth=rb.relative_depth,
                           normal=rb.normal, rgb=rb.rgb, shadow=None if rb.shadow is None else rb.shadow[:, None],
                           ao=rb.ao, view=rb.view)
        return out.reshape(W, H, -1)

    def shade_images(self, net, f=(0, 0, 1), t=(0, 0, 0), fov=30.0, aa=1, mm=None):
        """shade_tensor on the CPU, transposed to [H, W, .] (renderer.py:292-331);
        aa > 1 averages aa renders (identical here: the rays carry no jitter)."""
        from dataclasses import fields
        rbs = [self.shade_tensor(net, f=f, t=t, fov=fov, mm=mm) for _ in range(max(1, aa))]
        rb = rbs[0]
        if aa > 1:
            rb = RenderBuffer(**{fl.name: (None if getattr(rb, fl.name) is None else
                                           sum(getattr(r, fl.name).float() for r in rbs) / aa) for fl in fields(rb)})
        return rb.cpu().transpose()
