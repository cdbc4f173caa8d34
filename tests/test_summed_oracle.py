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
