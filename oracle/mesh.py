"""numpy restatement of the mesh signed distance (test infrastructure: only
the tests use it, as the checker of nglod_mesh_sdf).

Follows the algorithm of sdf-net/lib/extensions/mesh2sdf_cuda/
mesh2sdf_kernel.cu:307-617 (kernel_mesh2sdf_quad + kernel_quad_aggr, the
function compute_sdf calls): per triangle the squared distance to the plane
when the three edge half-space signs (copysign) sum to 2 or more, else to
the nearest clamped edge point; the minimum over triangles; negative when
each of 13 fixed lines through the point (|det| >= 1e-8) crosses the mesh
at t >= 0 and at t < 0.  Vectorised over points x triangles in float32.
"""
import numpy as np

f32 = np.float32
S2, S3 = f32(0.707106781), f32(0.577350269)
DIRS = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, S2, S2], [S2, 0, S2], [S2, S2, 0], [0, S2, -S2], [S2, 0, -S2],
                 [S2, -S2, 0], [S3, S3, S3], [-S3, S3, S3], [S3, -S3, S3], [S3, S3, -S3]], f32)


def _dot(a, b):
    return (a * b).sum(-1, dtype=f32)


def mesh_sdf(triangles, points, chunk=512):
    """triangles [m, 3, 3], points [n, 3] -> signed distances [n]."""
    tri = np.asarray(triangles, f32)
    pts = np.asarray(points, f32)
    v0, v1, v2 = tri[:, 0], tri[:, 1], tri[:, 2]
    v10, v21, v02 = v1 - v0, v2 - v1, v0 - v2
    nor = np.cross(v10, v02).astype(f32)
    c10, c21, c02 = (np.cross(e, nor).astype(f32) for e in (v10, v21, v02))
    inv = [(f32(1) / _dot(e, e)).astype(f32) for e in (v10, v21, v02, nor)]
    e2 = -v02
    degenerate = (nor == 0).all(-1)
    out = np.empty(pts.shape[0], f32)
    for s in range(0, pts.shape[0], chunk):
        p = pts[s:s + chunk, None, :]
        p0, p1, p2 = p - v0, p - v1, p - v2
        sg = (np.copysign(f32(1), _dot(c10, p0)) + np.copysign(f32(1), _dot(c21, p1)) +
              np.copysign(f32(1), _dot(c02, p2)))

        def edge(e, q, i):
            x = np.clip(_dot(e, q) * i, 0, 1).astype(f32)
            d = (e * x[..., None] - q).astype(f32)
            return _dot(d, d)
        ed = np.minimum(edge(v10, p0, inv[0]), np.minimum(edge(v21, p1, inv[1]), edge(v02, p2, inv[2])))
        fd = (_dot(nor, p0) ** 2 * inv[3]).astype(f32)
        d2 = np.maximum(np.where(sg < 2, ed, fd), 0)
        d2 = np.where(degenerate, np.inf, d2).min(1)
        qvec = np.cross(p0, v10).astype(f32)
        pos = np.zeros((p.shape[0], 13), bool)
        neg = np.zeros((p.shape[0], 13), bool)
        for k, dr in enumerate(DIRS):
            pvec = np.cross(np.broadcast_to(dr, e2.shape), e2).astype(f32)
            det = _dot(v10, pvec)
            ok = ~((det > -1e-8) & (det < 1e-8))
            with np.errstate(divide="ignore", invalid="ignore"):
                idet = np.where(ok, f32(1) / det, 0).astype(f32)
            u = (_dot(p0, pvec) * idet).astype(f32)
            v = (_dot(np.broadcast_to(dr, qvec.shape), qvec) * idet).astype(f32)
            t = (_dot(e2, qvec) * idet).astype(f32)
            hit = ok & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1)
            pos[:, k] = (hit & (t >= 0)).any(1)
            neg[:, k] = (hit & (t < 0)).any(1)
        inside = (pos & neg).all(1)
        dist = np.sqrt(d2).astype(f32)
        out[s:s + chunk] = np.where(inside, -dist, dist)
    return out
