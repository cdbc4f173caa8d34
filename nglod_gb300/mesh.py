"""Mesh data path: reading and normalising meshes, sampling points on and
near them, and their signed distance on the GPU.

Drop-ins for sdf-net/lib/torchgp (load_obj, normalize, per_face_normals,
area_weighted_distribution, random_face, sample_surface,
sample_near_surface, sample_uniform, point_sample, compute_sdf) and
sdf-net/lib/datasets/MeshDataset.py.  ``compute_sdf`` runs the library's
mesh-distance kernels (nglod_mesh_prepare / nglod_mesh_sdf); the samplers
are torch code on the mesh's device, as the reference's are.  ``load_obj``
parses Wavefront .obj text itself (vertices, faces triangulated as fans;
materials are not read), the reference's tinyobjloader being absent.
"""
import os

import numpy as np
import torch

from . import _lib
from .octree_sdf import setparam


def load_obj(fname, load_materials=False):
    """[V [#V, 3] float32, F [#F, 3] int64] of a Wavefront .obj file
    (load_obj.py:60-87); polygons are split into fans (v0, vi, vi+1)."""
    if load_materials:
        raise NotImplementedError("load_obj: materials are not read")
    if fname is None or not os.path.exists(fname):
        raise FileNotFoundError(f"Invalid file path and/or format, must be an existing Wavefront .obj: {fname}")
    verts, faces = [], []
    with open(fname) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v":
                verts.append([float(v) for v in parts[1:4]])
            elif parts[0] == "f":
                idx = []
                for tok in parts[1:]:
                    i = int(tok.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                for k in range(1, len(idx) - 1):
                    faces.append([idx[0], idx[k], idx[k + 1]])
    return [torch.tensor(verts, dtype=torch.float32).reshape(-1, 3),
            torch.tensor(faces, dtype=torch.int64).reshape(-1, 3)]


def save_obj(fname, V, F):
    with open(fname, "w") as fh:
        for v in np.asarray(V, dtype=np.float64):
            fh.write(f"v {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}\n")
        for f in np.asarray(F, dtype=np.int64):
            fh.write(f"f {f[0] + 1} {f[1] + 1} {f[2] + 1}\n")


def normalize(V, F):
    """Centre the bounding box at the origin, scale the farthest vertex to
    distance 1 (normalize.py:24-38)."""
    V_max, _ = torch.max(V, dim=0)
    V_min, _ = torch.min(V, dim=0)
    V = V - (V_max + V_min) / 2.0
    max_dist = torch.sqrt(torch.max(torch.sum(V ** 2, dim=-1)))
    return V * (1.0 / max_dist), F


def per_face_normals(V, F):
    mesh = V[F]
    return torch.cross(mesh[:, 0] - mesh[:, 1], mesh[:, 1] - mesh[:, 2], dim=-1)


def area_weighted_distribution(V, F, normals=None):
    if normals is None:
        normals = per_face_normals(V, F)
    areas = torch.norm(normals, p=2, dim=1) * 0.5
    areas /= torch.sum(areas) + 1e-10
    return torch.distributions.Categorical(areas.view(-1))


def random_face(V, F, num_samples, distrib=None):
    if distrib is None:
        distrib = area_weighted_distribution(V, F)
    normals = per_face_normals(V, F)
    idx = distrib.sample([num_samples])
    return F[idx], normals[idx]


def sample_surface(V, F, num_samples, distrib=None):
    """[points, face normals] sampled area-weighted on the surface
    (sample_surface.py:24-47)."""
    if distrib is None:
        distrib = area_weighted_distribution(V, F)
    fidx, normals = random_face(V, F, num_samples, distrib)
    f = V[fidx]
    u = torch.sqrt(torch.rand(num_samples)).to(V.device).unsqueeze(-1)
    v = torch.rand(num_samples).to(V.device).unsqueeze(-1)
    samples = (1 - u) * f[:, 0, :] + (u * (1 - v)) * f[:, 1, :] + u * v * f[:, 2, :]
    return samples, normals


def sample_near_surface(V, F, num_samples, variance=0.01, distrib=None):
    if distrib is None:
        distrib = area_weighted_distribution(V, F)
    samples = sample_surface(V, F, num_samples, distrib)[0]
    samples += torch.randn_like(samples) * variance
    return samples


def sample_uniform(num_samples):
    return torch.rand(num_samples, 3) * 2.0 - 1.0


def point_sample(V, F, techniques, num_samples):
    """point_sample.py:29-57: techniques among 'trace', 'near', 'rand'."""
    distrib = area_weighted_distribution(V, F) if ("trace" in techniques or "near" in techniques) else None
    samples = []
    for technique in techniques:
        if technique == "trace":
            samples.append(sample_surface(V, F, num_samples, distrib=distrib)[0])
        elif technique == "near":
            samples.append(sample_near_surface(V, F, num_samples, distrib=distrib))
        elif technique == "rand":
            samples.append(sample_uniform(num_samples).to(V.device))
    return torch.cat(samples, dim=0)


def triangle_records(V, F):
    """Device records of the mesh's triangles for mesh_sdf (nglod_mesh_prepare)."""
    _lib.require_cuda(V)
    tri = V[F].float().contiguous()
    m = tri.shape[0]
    lib = _lib.load()
    rec = torch.empty(max(m, 1), int(lib.nglod_mesh_record_floats()), device=V.device)
    _lib.check(lib.nglod_mesh_prepare(_lib.ptr(tri), m, _lib.ptr(rec), _lib.stream_ptr(V.device)),
               "nglod_mesh_prepare")
    return rec[:m]


def mesh_sdf(records, points):
    """Signed distances [n] of points [n, 3] to the mesh of `records`."""
    _lib.require_cuda(records, points)
    points = points.float().contiguous()
    out = torch.empty(points.shape[0], device=points.device)
    _lib.check(_lib.load().nglod_mesh_sdf(_lib.ptr(records), records.shape[0], _lib.ptr(points), points.shape[0],
                                          _lib.ptr(out), _lib.stream_ptr(points.device)), "nglod_mesh_sdf")
    return out


def compute_sdf(V, F, points):
    """compute_sdf.py:26-40 on the GPU: [n] signed distances (negative inside)."""
    return mesh_sdf(triangle_records(V, F), points)


class MeshDataset(torch.utils.data.Dataset):
    """MeshDataset.py:34-109: SDF samples of a single normalised mesh."""

    def __init__(self, args=None, dataset_path=None, raw_obj_path=None, sample_mode=None, get_normals=None,
                 seed=None, num_samples=None, trim=None, sample_tex=None, mesh=None, device="cuda"):
        self.args = args
        self.dataset_path = setparam(args, dataset_path, "dataset_path")
        self.sample_mode = setparam(args, sample_mode, "sample_mode") or ["rand", "near", "near", "trace", "trace"]
        self.get_normals = bool(setparam(args, get_normals, "get_normals"))
        self.num_samples = setparam(args, num_samples, "num_samples") or 100000
        self.sample_tex = bool(setparam(args, sample_tex, "sample_tex"))
        if self.sample_tex:
            raise NotImplementedError("MeshDataset: texture sampling is not built")
        if mesh is not None:
            V, F = mesh
        else:
            V, F = load_obj(self.dataset_path)
        self.V, self.F = normalize(V.to(device).float(), F.to(device))
        self.mesh = self.V[self.F]
        self._records = triangle_records(self.V, self.F)
        self.resample()

    def resample(self):
        self.nrm = None
        if self.get_normals:
            self.pts, self.nrm = sample_surface(self.V, self.F, self.num_samples * 5)
            self.nrm = self.nrm.cpu()
        else:
            self.pts = point_sample(self.V, self.F, self.sample_mode, self.num_samples)
        self.d = mesh_sdf(self._records, self.pts)[..., None].cpu()
        self.pts = self.pts.cpu()

    def __getitem__(self, idx):
        if self.get_normals:
            return self.pts[idx], self.d[idx], self.nrm[idx]
        return self.pts[idx], self.d[idx]

    def __len__(self):
        return self.pts.size()[0]

    def num_shapes(self):
        return 1
