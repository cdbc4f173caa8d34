"""numpy restatement of the reference Renderer's shading (test
infrastructure: only the tests use it, as the checker of
nglod_gb300.renderer).

Follows sdf-net/lib/renderer.py:118-223 (render: ground plane and shadow
rays 131-161, relative depth 167, ambient occlusion 184-208; shade_tensor:
matcap 262-279, segmentation 280-281, shadow map 283-286, AO 288-289) and
sdf-net/lib/geoutils.py:237-276 (matcap_sampler, spherical_envmap), in
float32 one torch operation at a time.  The two third-party calls are
scipy's, as in the reference: RegularGridInterpolator for the matcap and
ndimage.gaussian_filter for the shadow map.
"""
import numpy as np
from scipy.interpolate import RegularGridInterpolator
from scipy.ndimage import gaussian_filter

from oracle import dense

f32 = np.float32
LIGHT = np.array([-1.5, 4.5, -1.5], f32)
AO_TAPS = 40


def ground(ro, rd, min_y, x, t, hit, normal):
    """renderer.py:131-150 -> (x, t, hit, normal, plane_hit), new arrays."""
    x, t, hit, normal = x.copy(), t.copy(), hit.copy(), normal.copy()
    rate = (-rd[:, 1]).astype(f32)
    delta = (ro[:, 1] - f32(min_y)).astype(f32)
    with np.errstate(divide="ignore", invalid="ignore"):
        pt = (delta / rate).astype(f32)
        ph = (pt > 0) & (pt < 500) & (pt < t[:, 0])
    hit = hit & ~ph
    t[ph, 0] = pt[ph]
    x[ph] = (ro[ph] + (rd[ph] * pt[ph, None]).astype(f32)).astype(f32)
    normal[ph] = 0
    normal[ph, 1] = 1
    return x, t, hit, normal, ph


def shadow_rays(x, normal, noise, light=LIGHT):
    """renderer.py:152-158 -> (origins, directions, light_hit)."""
    so = (x + (f32(0.1) * normal).astype(f32)).astype(f32)
    sd = ((noise + light[None]).astype(f32) - so).astype(f32)
    nrm = np.sqrt((sd * sd).sum(1, dtype=f32)).astype(f32)
    sd = (sd / np.maximum(nrm, f32(1e-12))[:, None]).astype(f32)
    light_hit = (sd * normal).sum(1, dtype=f32) > 0
    return so, sd, light_hit


def ao_distances():
    # the reference's Python floats, used against float32 tensors
    return [f32(0.1 * 0.25 * (float(i + 1) / float(AO_TAPS + 1)) ** 1.6) for i in range(AO_TAPS)]


def ambient_occlusion(sdf_fn, x, normal, hit, plane_hit=None):
    """renderer.py:184-208: ao [n] (1 where neither hit nor plane_hit)."""
    acc = np.zeros(x.shape[0], f32)
    sel = hit | (plane_hit if plane_hit is not None else False)
    for d in ao_distances():
        q = (x + (normal * d).astype(f32)).astype(f32)
        r = np.zeros(x.shape[0], f32)
        if sel.any():
            r[sel] = sdf_fn(q[sel])
        if plane_hit is not None:
            r[plane_hit] = np.minimum(r[plane_hit], d)
        e = ((d - r).astype(f32) - f32(0.0015)).astype(f32)
        acc[sel] = (acc[sel] + (f32(3.5) * np.maximum(e[sel], 0)).astype(f32)).astype(f32)
    ao = np.clip((f32(1) - acc).astype(f32), f32(0.1), f32(1))
    return (ao * ao).astype(f32)


def spherical_envmap(view, normal):
    """geoutils.py:253-276 (float32)."""
    rds = view.astype(f32).copy()
    rds[:, 2] *= -1
    dot = (normal * rds).sum(1, keepdims=True, dtype=f32)
    r = (rds - ((f32(2) * dot).astype(f32) * normal).astype(f32)).astype(f32)
    r[:, 2] -= f32(1)
    m = (f32(2) * np.sqrt((r * r).sum(1, keepdims=True, dtype=f32))).astype(f32)
    with np.errstate(divide="ignore", invalid="ignore"):
        vn = ((r[:, :2] / m).astype(f32) + f32(0.5)).astype(f32)
    vn = (f32(1) - vn).astype(f32)
    vn = np.clip(vn, 0, 1)
    vn[np.isnan(vn)] = 0
    return vn


def matcap_rgb(texture_image, view, normal, hit):
    """shade_tensor's matcap branch and segmentation: rgb [n, 3] in [0, 1]."""
    tex = np.asarray(texture_image).transpose(1, 0, 2)
    interp = RegularGridInterpolator((np.linspace(0, 1, tex.shape[0]), np.linspace(0, 1, tex.shape[1])), tex)
    rgb = (interp(spherical_envmap(view, normal))[:, :3].astype(f32) / f32(255)).astype(f32)
    rgb[~hit] = 1
    return rgb


def shadow_map(shadow, width, height, sigma=2):
    """renderer.py:283-285: [W*H] shadow flags -> blurred map [W*H]."""
    m = np.clip((f32(1) - shadow.astype(f32) + f32(0.9)).astype(f32), 0, 1).reshape(width, height)
    return gaussian_filter(m, sigma=sigma).reshape(-1)


def shade(model, ro, rd, noise, texture_image, ground_height, width, height, num_steps=64, lod=None):
    """The whole Renderer.shade_tensor with shadow and ao on: dict of flat
    [W*H, ...] arrays (x, depth, hit, normal, rgb, shadow, ao,
    relative_depth), for a float32 oracle model."""
    from oracle import cref

    def aabb_fn(o, d):
        return cref.aabb(o.astype(f32), d.astype(f32))

    x, t, hit, normal = dense.sphere_trace(model, ro, rd, lod=lod, num_steps=num_steps, aabb_fn=aabb_fn)
    x, t, hit, normal, ph = ground(ro, rd, ground_height, x, t, hit, normal)
    so, sd, light_hit = shadow_rays(x, normal, noise)
    _, _, shit, _ = dense.sphere_trace(model, so, sd, lod=lod, num_steps=num_steps, aabb_fn=aabb_fn)
    shadow = shit & light_hit
    rel = (np.clip(t, 0, f32(10)) / f32(10)).astype(f32)
    ao = ambient_occlusion(lambda q: dense.sdf(model, q, lod=lod)[:, 0].astype(f32), x, normal, hit, ph)
    normal = normal.copy()
    normal[~hit] = 1
    rgb = matcap_rgb(texture_image, rd, normal, hit)
    rgb = (rgb * shadow_map(shadow, width, height)[:, None]).astype(f32)
    rgb = (rgb * ao[:, None]).astype(f32)
    return {"x": x, "depth": t, "hit": hit, "normal": normal, "rgb": rgb, "shadow": shadow, "ao": ao,
            "relative_depth": rel}
