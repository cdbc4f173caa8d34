"""Mesh data path on the CPU: the samplers against the reference's own
torchgp output (tests/golden/mesh_small.npz), the mesh-distance oracle
against analytic shapes, and .obj reading."""
import numpy as np
import torch

from nglod_gb300 import mesh, synthetic
from oracle import mesh as omesh


def test_normalize_normals_and_point_sample_match_reference(golden):
    z = golden("mesh_small")
    V = torch.from_numpy(z["V"])
    F = torch.from_numpy(z["F"])
    Vn, Fn = mesh.normalize(V, F)
    assert torch.equal(Vn, torch.from_numpy(z["V_normalized"]))
    assert torch.equal(mesh.per_face_normals(Vn, Fn), torch.from_numpy(z["face_normals"]))
    torch.manual_seed(3)
    pts = mesh.point_sample(Vn, Fn, ["trace", "near", "rand"], 300)
    assert torch.equal(pts, torch.from_numpy(z["point_sample"]))


def test_oracle_distance_against_analytic_shapes():
    rng = np.random.default_rng(0)
    p = rng.uniform(-1.5, 1.5, (1500, 3)).astype(np.float32)
    V, F = synthetic.icosphere(3)
    d = omesh.mesh_sdf(V[F], p)
    ref = np.linalg.norm(p, axis=1) - 1
    # the inscribed polyhedron lies within 1 - cos(edge angle / 2) of the sphere
    assert np.abs(d - ref).max() < 5e-3
    far = np.abs(ref) > 5e-3
    assert (np.sign(d[far]) == np.sign(ref[far])).all()
    V, F = synthetic.torus()
    d = omesh.mesh_sdf(V[F], p)
    q = np.sqrt(p[:, 0] ** 2 + p[:, 2] ** 2) - 0.6
    ref = np.sqrt(q ** 2 + p[:, 1] ** 2) - 0.25
    assert np.abs(d - ref).max() < 5e-3
    far = np.abs(ref) > 5e-3
    assert (np.sign(d[far]) == np.sign(ref[far])).all()


def test_obj_round_trip(tmp_path):
    V, F = synthetic.torus(n_major=12, n_minor=6)
    path = tmp_path / "t.obj"
    mesh.save_obj(path, V, F)
    with open(path, "a") as fh:  # a quad is split into a fan of two triangles
        fh.write("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf -4 -3/1 -2//2 -1\n")
    V2, F2 = mesh.load_obj(str(path))
    n = V.shape[0]
    assert np.allclose(V2[:n].numpy(), V, atol=1e-6)
    assert np.array_equal(F2[:F.shape[0]].numpy(), F)
    assert F2[F.shape[0]:].tolist() == [[n, n + 1, n + 2], [n, n + 2, n + 3]]
