"""Surface samples and octrees from a network (nglod_gb300.surface) on the
GPU, against numpy on the same inputs and the octree oracle."""
import math

import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import surface, synthetic
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.options import default_args
from oracle import dense
from oracle import spc as ospc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def net(cuda):
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    m = ng.OctreeSDF(default_args(num_lods=4, base_lod=2))
    init_from_sdf(m, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=4)
    return m.to(cuda).eval()


def test_octree_from_sdf_matches_numpy_band(net, cuda):
    level = 5
    res = 2 ** level
    s = surface.octree_from_sdf(net, level, chunk=10000)  # several chunks
    got = {tuple(p) for p in s.GetLevelPoints(level)[:, :3].cpu().numpy().tolist()}
    v = np.arange(res ** 3)
    xyz = np.stack([v // (res * res), (v // res) % res, v % res], 1)
    inv = np.float32(2.0 / res)
    centres = ((xyz.astype(np.float32) + np.float32(0.5)) * inv - np.float32(1)).astype(np.float32)
    m32 = dense.model_from_state_dict(net.state_dict(), 4, 2, np.float32)
    d = dense.sdf(m32, centres)[:, 0]
    band = np.float32(math.sqrt(3) * 2.0 / res)
    want = {tuple(p) for p in xyz[np.abs(d) <= band].tolist()}
    assert len(want) > 500
    diff = got ^ want
    dd = {tuple(p): abs(abs(x) - band) for p, x in zip(xyz.tolist(), d)}
    assert all(dd[p] < 1e-5 for p in diff), [dd[p] for p in diff][:5]
    # the octree of the selected voxels is the spc3d octree of the same set
    vox = np.array(sorted(got), dtype=np.uint16)
    octree, _ = ospc.points_to_octree(vox, level)
    assert np.array_equal(s.GetOctree().cpu().numpy(), octree)


def test_voxel_sparsify_levels_match_numpy(net, cuda):
    pts = surface.trace_surface_points(20000, net, generator=torch.Generator(device=cuda).manual_seed(3))[:20000]
    assert pts.shape[0] == 20000
    lod = 3
    vs = surface.voxel_sparsify(20000, net, lod, points=pts)
    p = pts.cpu().numpy().astype(np.float32)
    for i in range(lod + 1):
        res = 2 ** (i + 2)
        want = np.unique(np.floor(((p + 1.0) / 2.0) * res).astype(np.int64), axis=0)
        assert np.array_equal(vs[i].cpu().numpy(), want), i


def test_surface_points_lie_on_the_surface_and_reference_samples_keep_origins(net, cuda):
    c, r = synthetic.sphere_union(1)
    gen = torch.Generator(device=cuda).manual_seed(5)
    pts = surface.trace_surface_points(5000, net, generator=gen)
    assert pts.shape[0] >= 5000
    # on the network's zero set within the tracer's stopping distances
    # (3e-4, oscillation 9e-4), and near the analytic surface it encodes
    with torch.no_grad():
        dn = net.sdf(pts).abs()
    assert torch.quantile(dn[:, 0], 0.99).item() < 2e-3
    d = synthetic.sphere_union_sdf(pts.double().cpu().numpy(), c, r)
    assert np.median(np.abs(d)) < 1e-2
    # SphereTracer.sample_surface: origins inside the box are hits at depth 0
    s = surface.sample_surface(3000, net, generator=torch.Generator(device=cuda).manual_seed(6))
    assert s.shape[0] >= 3000 and (s.abs() <= 1).all()
