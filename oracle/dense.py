"""numpy restatement of NGLOD's dense neural-SDF path (test infrastructure).

Every function runs in the dtype of its inputs, so the same code is the
float32 mirror of the reference and the float64 oracle the error reports use.

A model is a plain dict::

    {"num_lods": int, "base_lod": int,
     "fms": [ndarray [C, s, s, s]] * num_lods,      # FeatureVolume.fm[0]
     "w0": [[H, 3+C]], "b0": [[H]], "w1": [[1, H]], "b1": [[1]]}

which is exactly the reference's state_dict (``features.{i}.fm``,
``louts.{i}.{0,2}.{weight,bias}``) with the leading batch axis of fm dropped.
"""
import numpy as np


def model_from_state_dict(sd, num_lods, base_lod, dtype=np.float64):
    """Build an oracle model from an OctreeSDF state_dict (torch or numpy)."""
    def a(v):
        v = v.detach().cpu().numpy() if hasattr(v, "detach") else np.asarray(v)
        return v.astype(dtype)
    m = {"num_lods": num_lods, "base_lod": base_lod, "fms": [], "w0": [], "b0": [], "w1": [], "b1": []}
    for i in range(num_lods):
        m["fms"].append(a(sd[f"features.{i}.fm"])[0])
        m["w0"].append(a(sd[f"louts.{i}.0.weight"]))
        m["b0"].append(a(sd[f"louts.{i}.0.bias"]))
        m["w1"].append(a(sd[f"louts.{i}.2.weight"]))
        m["b1"].append(a(sd[f"louts.{i}.2.bias"]))
    return m


def feature_volume(fm, x):
    """Trilinear ``F.grid_sample(fm, x, align_corners=True, padding_mode='border')``.

    Follows sdf-net/lib/models/OctreeSDF.py:46-57 (FeatureVolume.forward).
    x[:, 0] indexes the W axis, x[:, 1] H and x[:, 2] D.  The unnormalised
    coordinate is u = (x + 1) / 2 * (size - 1), clamped to [0, size - 1]; the
    corner weights are the products of distances to the opposite corner, as
    in PyTorch's 3-D grid sampler.  Returns [N, C].
    """
    C, D, H, W = fm.shape
    dt = fm.dtype
    one = dt.type(1)
    two = dt.type(2)

    def src(c, size):
        u = ((c + one) / two) * dt.type(size - 1)
        return np.minimum(dt.type(size - 1), np.maximum(u, dt.type(0)))

    ix = src(x[:, 0].astype(dt), W)
    iy = src(x[:, 1].astype(dt), H)
    iz = src(x[:, 2].astype(dt), D)
    x0 = np.floor(ix)
    y0 = np.floor(iy)
    z0 = np.floor(iz)
    x1, y1, z1 = x0 + one, y0 + one, z0 + one
    fcl = np.ascontiguousarray(fm.transpose(1, 2, 3, 0))  # [D, H, W, C]
    out = np.zeros((x.shape[0], C), dtype=dt)
    for cz, wz in ((z0, z1 - iz), (z1, iz - z0)):
        for cy, wy in ((y0, y1 - iy), (y1, iy - y0)):
            for cx, wx in ((x0, x1 - ix), (x1, ix - x0)):
                w = wx * wy * wz
                ok = (cx >= 0) & (cx < W) & (cy >= 0) & (cy < H) & (cz >= 0) & (cz < D)
                xi = np.clip(cx, 0, W - 1).astype(np.int64)
                yi = np.clip(cy, 0, H - 1).astype(np.int64)
                zi = np.clip(cz, 0, D - 1).astype(np.int64)
                v = fcl[zi, yi, xi]
                out += np.where(ok[:, None], v * w[:, None], dt.type(0))
    return out


def decoder(m, i, ex):
    """``louts[i]``: Linear(3+C, H) -> ReLU -> Linear(H, 1) (OctreeSDF.py:81-88)."""
    h = np.maximum(ex @ m["w0"][i].T + m["b0"][i], 0)
    return h @ m["w1"][i].T + m["b1"][i]


def summed_volume(m, lod):
    """LOD-summed volume ``lod`` [C, s, s, s] in the model's dtype: at every
    vertex of LOD lod's grid, the running feature sum of ``sdf``
    (OctreeSDF.py:109-110) there, i.e. the sum over LODs i <= lod of volume
    i's trilinear sample.  Grid spacings halve from LOD to LOD, so each cell
    of LOD lod lies inside one cell of every coarser grid, and a trilinear
    function restricted to a sub-box is trilinear: ``feature_volume`` of this
    volume gives the running sum at any point up to rounding (the border
    clamp is the same for every LOD).  The restatement of
    nglod_build_summed_volume, which computes it on the device in float64."""
    s = m["fms"][lod].shape[-1]
    t = np.linspace(-1.0, 1.0, s).astype(m["fms"][lod].dtype)
    z, y, x = np.meshgrid(t, t, t, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)  # x -> W, y -> H, z -> D
    acc = 0
    for i in range(lod + 1):
        acc = acc + feature_volume(m["fms"][i], pts)
    return np.ascontiguousarray(acc.T.reshape(-1, s, s, s))


def sdf(m, x, lod=None, return_lst=False):
    """``OctreeSDF.sdf(x, lod, return_lst)`` (OctreeSDF.py:94-155).

    Running sum of the per-LOD features, ``cat([x, sum])`` and the LOD's own
    decoder; returns at ``lod`` when ``0 <= lod < num_lods``, else the finest
    prediction (or the list of all of them with ``return_lst``).
    """
    x = np.asarray(x)
    dt = m["fms"][0].dtype
    x = x.astype(dt)
    acc = None
    outs = []
    for i in range(m["num_lods"]):
        f = feature_volume(m["fms"][i], x)
        acc = f if acc is None else acc + f
        d = decoder(m, i, np.concatenate([x, acc], axis=1))
        if lod is not None and lod == i:
            return d
        outs.append(d)
    return outs if return_lst else outs[-1]


def aabb(ray_o, ray_d):
    """Ray vs the [-1, 1]^3 box, vectorised restatement of the sol_nglod kernel.

    sdf-net/lib/extensions/sol_nglod/sol_nglod_kernel.cu:77-188.  Rays whose
    origin is inside the box are skipped (x = ray_o, t = 0, hit = False); a
    miss also leaves x = ray_o, t = 0.  Runs in the inputs' dtype (the
    bit-exact float32 form is ``oracle.spc.aabb``).
    """
    o = np.asarray(ray_o)
    d = np.asarray(ray_d)
    dt = o.dtype
    n = o.shape[0]
    x = o.copy()
    t = np.zeros((n, 1), dtype=dt)
    hit = np.zeros(n, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = (1.0 / d.astype(np.float64)).astype(dt)
        sgn = np.where(np.signbit(d), dt.type(1), dt.type(-1))
        cmax = np.abs(o).max(axis=1)
        outside = ~(cmax < 1)
        dd = (sgn - o) * inv  # winding = +1 for rays starting outside
        tests = []
        for a, (b, c) in enumerate(((1, 2), (0, 2), (0, 1))):
            lb = d[:, b] * dd[:, a] + o[:, b]
            lc = d[:, c] * dd[:, a] + o[:, c]
            tests.append((dd[:, a] >= 0) & (np.abs(lb) < 1) & (np.abs(lc) < 1))
        dist = np.where(tests[0], dd[:, 0], np.where(tests[1], dd[:, 1], np.where(tests[2], dd[:, 2], 0)))
        anyhit = (tests[0] | tests[1] | tests[2]) & outside & (dist < 500)
    hit[anyhit] = True
    t[anyhit, 0] = dist[anyhit]
    x[anyhit] = d[anyhit] * dist[anyhit, None] + o[anyhit]
    return x, t, hit


def finitediff_gradient(f, x):
    """Central differences with h = 1/192 (sdf-net/lib/diffutils.py:61-70)."""
    dt = x.dtype
    h = dt.type(1.0 / (64.0 * 3.0))
    cols = []
    for k in range(3):
        e = np.zeros(3, dtype=dt)
        e[k] = h
        cols.append(f(x + e) - f(x - e))
    return np.concatenate(cols, axis=-1) / (h * dt.type(2))


def normalize(v, eps=1e-5):
    """``F.normalize(v, p=2, dim=-1, eps)``: v / max(||v||, eps)."""
    n = np.sqrt((v * v).sum(axis=-1, keepdims=True))
    return v / np.maximum(n, v.dtype.type(eps))


def get_min(m, ray_o, ray_d, lod=None, num_steps=128, min_dis=3e-4, step_size=1.0, camera_clamp=(-5.0, 10.0),
            aabb_fn=aabb):
    """``SphereTracer.get_min(net, ray_o, ray_d)`` (tracer/SphereTracer.py:134-218).

    Returns (x, t, hit, normal, min_x).  Its rules: ``cond`` is recomputed
    every step (|d|, oscillation, |t| < far) without the aabb mask, so rays
    that miss the box march from their origins; before each step's update,
    min_x takes the new point wherever the previous d is below the running
    minimum; normals are the finite-difference gradient, not normalised.
    """
    dt = m["fms"][0].dtype
    o = np.asarray(ray_o).astype(dt)
    dr = np.asarray(ray_d).astype(dt)
    net = lambda p: sdf(m, p, lod=lod)
    x, t, _ = aabb_fn(o, dr)
    x = x.astype(dt)
    t = t.astype(dt)
    normal = np.zeros_like(x)
    d = net(x)
    dprev = d.copy()
    mind = d.copy()
    minx = x.copy()
    hit = np.zeros(o.shape[0], dtype=bool)
    far = dt.type(camera_clamp[1])
    md = dt.type(min_dis)
    for _ in range(num_steps):
        hit = np.abs(t[:, 0]) < far
        cond = np.abs(d[:, 0]) > md
        cond = cond & (np.abs((d[:, 0] + dprev[:, 0]) / dt.type(2)) > md * dt.type(3))
        cond = cond & hit
        if not cond.any():
            break
        x = np.where(cond[:, None], o + dr * t, x)
        new = d[:, 0] < mind[:, 0]
        mind[new] = d[new]
        minx[new] = x[new]
        dprev = np.where(cond[:, None], d, dprev)
        d[cond] = net(x[cond]) * dt.type(step_size)
        t = np.where(cond[:, None], t + d, t)
    hit = hit & ~(np.abs(x) > 1).any(axis=-1)
    if hit.any():
        normal[hit] = finitediff_gradient(net, x[hit])
    return x, t, hit, normal, minx


def sphere_trace(m, ray_o, ray_d, lod=None, num_steps=128, min_dis=3e-4, step_size=1.0,
                 camera_clamp=(-5.0, 10.0), aabb_fn=aabb):
    """``SphereTracer.forward(net, ray_o, ray_d)`` (tracer/SphereTracer.py:41-132).

    Returns (x [N,3], t [N,1], hit [N] bool, normal [N,3]).  Keeps the
    reference's quirks: x is the last evaluated point while t has already
    been advanced by the last d; ``hit`` is |t| < far as evaluated at the
    start of the last executed iteration, then culled to |x| <= 1; normals
    are finite differences of the same network (``grad_method='finitediff'``).
    """
    dt = m["fms"][0].dtype
    o = np.asarray(ray_o).astype(dt)
    dr = np.asarray(ray_d).astype(dt)
    net = lambda p: sdf(m, p, lod=lod)
    x, t, cond = aabb_fn(o, dr)
    x = x.astype(dt)
    t = t.astype(dt)
    n = o.shape[0]
    normal = np.zeros_like(x)
    d = net(x)
    dprev = d.copy()
    hit = np.zeros(n, dtype=bool)
    far = dt.type(camera_clamp[1])
    md = dt.type(min_dis)
    for _ in range(num_steps):
        hit = np.abs(t[:, 0]) < far
        cond = cond & (np.abs(d[:, 0]) > md)
        cond = cond & (np.abs((d[:, 0] + dprev[:, 0]) / dt.type(2)) > md * dt.type(3))
        cond = cond & hit
        if not cond.any():
            break
        x = np.where(cond[:, None], o + dr * t, x)
        dprev = np.where(cond[:, None], d, dprev)
        d[cond] = net(x[cond]) * dt.type(step_size)
        t = np.where(cond[:, None], t + d, t)
    hit = hit & ~(np.abs(x) > 1).any(axis=-1)
    if hit.any():
        g = finitediff_gradient(net, x[hit])
        normal[hit] = normalize(g)
    return x, t, hit, normal

