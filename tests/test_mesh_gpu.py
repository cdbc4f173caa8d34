"""Mesh signed distance on the GPU (nglod_mesh_prepare / nglod_mesh_sdf)
against the numpy restatement, and MeshDataset + training on a mesh."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import mesh, synthetic, trainer
from nglod_gb300.options import default_args
from oracle import mesh as omesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", ["icosphere", "torus"])
def test_mesh_sdf_matches_oracle(cuda, shape):
    V, F = synthetic.icosphere(3) if shape == "icosphere" else synthetic.torus()
    rng = np.random.default_rng(1)
    p = rng.uniform(-1.3, 1.3, (20000, 3)).astype(np.float32)
    Vd = torch.from_numpy(V).float().to(cuda)
    Fd = torch.from_numpy(F).to(cuda)
    got = mesh.compute_sdf(Vd, Fd, torch.from_numpy(p).to(cuda)).cpu().numpy()
    want = omesh.mesh_sdf(V[F].astype(np.float32), p)
    np.testing.assert_allclose(np.abs(got), np.abs(want), atol=2e-6, rtol=1e-5)
    # the crossing tests may differ only for points on a face or edge plane
    assert (np.sign(got) == np.sign(want)).mean() > 0.9995


def test_mesh_sdf_edge_cases(cuda):
    V, F = synthetic.icosphere(1)
    Vd = torch.from_numpy(V).float().to(cuda)
    Fd = torch.from_numpy(F).to(cuda)
    rec = mesh.triangle_records(Vd, Fd)
    assert mesh.mesh_sdf(rec, torch.zeros(0, 3, device=cuda)).shape == (0,)
    p = torch.tensor([[0.0, 0.0, 0.0], [3.0, 0.0, 0.0], [0.0, 0.0, -2.0]], device=cuda)
    d = mesh.mesh_sdf(rec, p).cpu().numpy()
    want = omesh.mesh_sdf(V[F].astype(np.float32), p.cpu().numpy())
    assert d[0] < 0 and d[1] > 0 and d[2] > 0
    np.testing.assert_allclose(d, want, atol=2e-6)
    # a degenerate (zero-area) triangle adds no distance and no crossing
    Vz = torch.cat([Vd, torch.tensor([[5.0, 5.0, 5.0]], device=cuda)])
    Fz = torch.cat([Fd, torch.tensor([[Vd.shape[0], Vd.shape[0], Vd.shape[0]]], device=cuda)])
    assert torch.equal(mesh.compute_sdf(Vz, Fz, p), mesh.mesh_sdf(rec, p))


def test_mesh_dataset_trains(cuda):
    V, F = synthetic.torus()
    ds = mesh.MeshDataset(mesh=(torch.from_numpy(V), torch.from_numpy(F)), num_samples=40000,
                          sample_mode=["rand", "near", "near", "trace"], device=cuda)
    assert len(ds) == 160000
    pts, d = ds[0:5]
    assert pts.shape == (5, 3) and d.shape == (5, 1)
    sub = slice(0, 4000)
    want = omesh.mesh_sdf(ds.mesh.cpu().numpy(), ds.pts[sub].numpy())
    np.testing.assert_allclose(np.abs(ds.d[sub, 0].numpy()), np.abs(want), atol=2e-6, rtol=1e-5)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=3, base_lod=2)).to(cuda)
    batches = [(ds.pts[i:i + 40000].to(cuda), ds.d[i:i + 40000].to(cuda)) for i in range(0, 160000, 40000)]
    _, losses = trainer.fit(net, batches, 300, lr=1e-3, log_every=100)
    assert losses[-1] < 0.2 * losses[0], losses
