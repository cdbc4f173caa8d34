"""Seeded synthetic inputs for the neural-SDF path.

The reference trains on meshes (sdf-net/lib/datasets/MeshDataset.py) that are
not available here; every workload instead uses an analytic SDF: the union of
16 spheres with centres U[-0.6, 0.6]^3 and radii U[0.1, 0.3] drawn from a
seeded ``torch.Generator``.  Point batches follow the reference's sampler mix
(sdf-net/lib/torchgp/sample_uniform.py, sample_near_surface.py): a third
uniform in [-1, 1]^3 and two thirds on the surface perturbed by N(0, 0.01^2).
Cameras follow ``look_at`` (sdf-net/lib/geoutils.py:180-206) without the
random pixel jitter of ``normalized_grid`` (geoutils.py:149-152).
"""
import math

import numpy as np
import torch


def sphere_union(seed=1, n=16):
    """Centres [n, 3] and radii [n] (float64 numpy) of the seeded sphere union."""
    g = torch.Generator().manual_seed(seed)
    c = torch.rand((n, 3), generator=g, dtype=torch.float64) * 1.2 - 0.6
    r = torch.rand((n,), generator=g, dtype=torch.float64) * 0.2 + 0.1
    return c.numpy(), r.numpy()


def sphere_union_sdf(p, centres, radii):
    """min_k(|p - c_k| - r_k) for numpy or torch points [N, 3]; returns [N]."""
    if isinstance(p, torch.Tensor):
        c = torch.as_tensor(centres, dtype=p.dtype, device=p.device)
        r = torch.as_tensor(radii, dtype=p.dtype, device=p.device)
        return (torch.cdist(p, c) - r).min(dim=1).values
    p = np.asarray(p, dtype=np.float64)
    d = np.sqrt(((p[:, None, :] - centres[None]) ** 2).sum(-1)) - radii[None]
    return d.min(axis=1)


def uniform_points(n, seed=0, lo=-1.0, hi=1.0):
    """[n, 3] float32 points U[lo, hi]^3 from a seeded generator."""
    g = torch.Generator().manual_seed(seed)
    return torch.rand((n, 3), generator=g) * (hi - lo) + lo


def surface_points(n, centres, radii, seed=0):
    """[n, 3] float64 points on the boundary of the sphere union.

    A sphere is chosen with probability proportional to its area, a point is
    drawn uniformly on it, and points that lie inside another sphere (so not
    on the union's boundary) are rejected and redrawn.
    """
    g = torch.Generator().manual_seed(seed)
    area = radii ** 2
    prob = torch.as_tensor(area / area.sum())
    out = []
    have = 0
    c = torch.as_tensor(centres)
    r = torch.as_tensor(radii)
    while have < n:
        m = max(2 * (n - have), 1024)
        k = torch.multinomial(prob, m, replacement=True, generator=g)
        v = torch.randn((m, 3), generator=g, dtype=torch.float64)
        v = v / v.norm(dim=1, keepdim=True)
        p = c[k] + v * r[k, None]
        dist = torch.cdist(p, c) - r[None]
        dist[torch.arange(m), k] = 1.0
        keep = (dist >= 0).all(dim=1)
        p = p[keep]
        out.append(p)
        have += p.shape[0]
    return torch.cat(out)[:n].numpy()


def training_batch(n, centres, radii, seed=0, sigma=0.01):
    """Points [n, 3] float32 and ground-truth SDF [n, 1] float32.

    One third uniform in [-1, 1]^3, two thirds surface samples perturbed by
    N(0, sigma^2) per axis; ground truth is the analytic SDF.
    """
    g = torch.Generator().manual_seed(seed + 7919)
    nu = n // 3
    ns = n - nu
    pu = torch.rand((nu, 3), generator=g, dtype=torch.float64) * 2 - 1
    ps = torch.as_tensor(surface_points(ns, centres, radii, seed=seed))
    ps = ps + torch.randn((ns, 3), generator=g, dtype=torch.float64) * sigma
    p = torch.cat([pu, ps])
    p = p[torch.randperm(n, generator=g)]
    gt = sphere_union_sdf(p.numpy(), centres, radii)
    return p.float(), torch.as_tensor(gt, dtype=torch.float32)[:, None]


def near_surface_query(n, centres, radii, seed=0, band=0.02):
    """[n, 3] float32: half uniform in [-1, 1]^3, half within ``band`` of the surface."""
    g = torch.Generator().manual_seed(seed + 104729)
    nu = n // 2
    ns = n - nu
    pu = torch.rand((nu, 3), generator=g, dtype=torch.float64) * 2 - 1
    ps = torch.as_tensor(surface_points(ns, centres, radii, seed=seed + 1))
    dirn = torch.randn((ns, 3), generator=g, dtype=torch.float64)
    dirn = dirn / dirn.norm(dim=1, keepdim=True)
    ps = ps + dirn * (torch.rand((ns, 1), generator=g, dtype=torch.float64) * 2 - 1) * band
    return torch.cat([pu, ps]).float()


def look_at_rays(eye=(0.0, 0.0, 4.0), at=(0.0, 0.0, 0.0), width=128, height=128, fov=30.0,
                 up=(0.0, 1.0, 0.0)):
    """Perspective pinhole rays (origins [W*H, 3], unit directions [W*H, 3]) float32.

    Pixel order follows the reference: ``torch.meshgrid(window_x, window_y)``
    with x major, window_x = linspace(-1, 1, W) * W/H and window_y =
    linspace(1, -1, H).
    """
    eye = np.asarray(eye, np.float64)
    at = np.asarray(at, np.float64)
    up = np.asarray(up, np.float64)
    view = at - eye
    view /= np.linalg.norm(view)
    right = np.cross(view, up)
    right /= np.linalg.norm(right)
    cup = np.cross(right, view)
    cup /= np.linalg.norm(cup)
    wx = np.linspace(-1, 1, width) * (width / height)
    wy = np.linspace(1, -1, height)
    gx, gy = np.meshgrid(wx, wy, indexing="ij")
    tanh = math.tan(math.radians(fov / 2))
    pix = right * gx[..., None] * tanh + cup * gy[..., None] * tanh + eye + view
    pix = pix.reshape(-1, 3)
    d = pix - eye
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    o = np.broadcast_to(eye, d.shape).copy()
    return torch.from_numpy(o).float(), torch.from_numpy(d).float()


def matcap_texture(size=64):
    """uint8 [size, size, 3] matcap image (rows = image y, as an image file
    decodes): a lit green sphere filling the square, standing in for the
    reference's data/matcap/green.png, which is not distributed with it."""
    u = (np.arange(size) + 0.5) / size * 2 - 1
    xx, yy = np.meshgrid(u, -u)  # image rows run top to bottom
    rr = xx * xx + yy * yy
    nz = np.sqrt(np.clip(1 - rr, 0, 1))
    light = np.array([-0.4, 0.5, 0.77])
    light = light / np.linalg.norm(light)
    lam = np.clip(xx * light[0] + yy * light[1] + nz * light[2], 0, 1)
    spec = lam ** 24
    base = np.array([0.18, 0.62, 0.32])
    col = base[None, None, :] * (0.15 + 0.85 * lam[..., None]) + 0.5 * spec[..., None]
    col = np.where((rr <= 1)[..., None], col, base[None, None, :] * 0.15)
    return np.clip(np.round(col * 255), 0, 255).astype(np.uint8)


def icosphere(subdivisions=3, radius=1.0, centre=(0.0, 0.0, 0.0)):
    """Closed triangle mesh of a sphere: [V float64 [#V, 3], F int64 [#F, 3]],
    an icosahedron subdivided `subdivisions` times (each face into four,
    new vertices pushed onto the sphere), faces wound outward."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, float) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]
        nf = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    V = np.array(V) * radius + np.asarray(centre, float)
    return V, np.array(F, dtype=np.int64)


def torus(R=0.6, r=0.25, n_major=48, n_minor=24):
    """Closed triangle mesh of a torus around the y axis: [V, F]."""
    u = np.arange(n_major) * 2 * np.pi / n_major
    v = np.arange(n_minor) * 2 * np.pi / n_minor
    uu, vv = np.meshgrid(u, v, indexing="ij")
    x = (R + r * np.cos(vv)) * np.cos(uu)
    z = (R + r * np.cos(vv)) * np.sin(uu)
    y = r * np.sin(vv)
    V = np.stack([x, y, z], -1).reshape(-1, 3)
    F = []
    for i in range(n_major):
        for j in range(n_minor):
            a = i * n_minor + j
            b = ((i + 1) % n_major) * n_minor + j
            c = ((i + 1) % n_major) * n_minor + (j + 1) % n_minor
            d = i * n_minor + (j + 1) % n_minor
            F += [(a, d, b), (b, d, c)]
    return V, np.array(F, dtype=np.int64)
