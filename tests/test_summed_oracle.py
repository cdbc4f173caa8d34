"""The LOD-summed volume identity on the CPU (float64 oracle): sampling
summed volume L alone gives OctreeSDF.sdf's running feature sum at LOD L,
inside and outside the box, so the decoders see the same input."""
import numpy as np
import pytest
import torch

from oracle import dense
from tests.helpers import oracle_model, seeded_model


@pytest.mark.parametrize("base_lod", [2, 3])
def test_summed_volume_sample_equals_running_sum(base_lod):
    net = seeded_model(num_lods=4, base_lod=base_lod, seed=17)
    with torch.no_grad():
        for fv in net.features:
            fv.fm.normal_(0.0, 0.05)
    m = oracle_model(net, np.float64)
    rng = np.random.default_rng(base_lod)
    x = rng.uniform(-1.3, 1.3, (4000, 3))
    x[:50] = np.array([1.0, -1.0, 0.25])  # on the box faces
    for lod in range(4):
        sv = dense.summed_volume(m, lod)
        assert sv.shape == m["fms"][lod].shape
        want = sum(dense.feature_volume(m["fms"][i], x) for i in range(lod + 1))
        got = dense.feature_volume(sv, x)
        assert np.abs(got - want).max() <= 1e-14 * max(1.0, np.abs(want).max()), lod
        # the decoder at lod sees the same input: the same prediction as sdf()
        pred = dense.decoder(m, lod, np.concatenate([x, got], axis=1))
        np.testing.assert_allclose(pred, dense.sdf(m, x, lod=lod), rtol=0, atol=1e-13)


def test_summed_volume_of_lod0_is_the_volume():
    net = seeded_model(num_lods=3, base_lod=2, seed=3)
    m = oracle_model(net, np.float64)
    np.testing.assert_array_equal(dense.summed_volume(m, 0), m["fms"][0])


def test_sparse_summed_features_equal_the_per_level_sum():
    """Sparse path: corner features built from the LOD-summed volumes and
    sampled in the query voxel alone give the reference's sum over the
    ancestors' samples (sparse_grid_sample.cuh:52-107), float32 restatement."""
    from nglod_gb300 import synthetic
    from oracle import sparse as osparse
    from oracle import spc as ospc
    c, r = synthetic.sphere_union(1)
    net = seeded_model(num_lods=4, base_lod=2, seed=5)
    with torch.no_grad():
        for fv in net.features:
            fv.fm.normal_(0.0, 0.05)
    m64 = oracle_model(net, np.float64)
    level = 5
    vox = ospc.voxels_near_surface(lambda p: synthetic.sphere_union_sdf(p, c, r), level)
    octree, _ = ospc.points_to_octree(vox, level)
    pts, pyr, _ = ospc.set_geometry(octree)
    fms32 = [f.astype(np.float32) for f in m64["fms"]]
    per_level = osparse.build(fms32, pts, pyr, 4)
    summed = osparse.build([dense.summed_volume(m64, l).astype(np.float32) for l in range(4)], pts, pyr, 4)
    x = synthetic.near_surface_query(6000, c, r, seed=6).numpy().astype(np.float32)
    for lod in (0, 2, 3):
        lv = lod + 2
        a, b = int(pyr[1, lv]), int(pyr[1, lv + 1])
        index = {tuple(p): a + k for k, p in enumerate(pts[a:b, :3].astype(np.int64))}
        v = np.clip(np.floor((x.astype(np.float64) + 1) / 2 * 2 ** lv), 0, 2 ** lv - 1).astype(np.int64)
        g = np.array([index.get(tuple(p), -1) for p in v])
        inside = g >= 0
        assert inside.mean() > 0.3
        want = osparse.features(per_level, lod, g[inside], x[inside])
        got = osparse.features(summed, lod, g[inside], x[inside], summed=True)
        assert np.abs(got - want).max() < 1e-5, lod
