"""Pins the CPU oracle against golden vectors produced by the reference's own
code (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import cref, dense
from tests.helpers import model_from_fixture, oracle_model

# The reference ran in float32 on the CPU; the oracle at float64 must agree to
# within float32 rounding of the reference's own sums.
SDF_TOL = 1e-5
DEPTH_TOL = 1e-4


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sdf_matches_reference(golden, dtype):
    fx = golden("dense_small")
    net = model_from_fixture(fx, 3, 1)
    m = oracle_model(net, dtype)
    x = fx["points"]
    for lod in [0, 1, 2]:
        np.testing.assert_allclose(dense.sdf(m, x, lod=lod), fx[f"sdf_lod{lod}"], atol=SDF_TOL, rtol=0)
    np.testing.assert_allclose(dense.sdf(m, x), fx["sdf_lodNone"], atol=SDF_TOL, rtol=0)
    np.testing.assert_allclose(dense.sdf(m, x, lod=7), fx["sdf_lod7"], atol=SDF_TOL, rtol=0)
    np.testing.assert_allclose(np.stack(dense.sdf(m, x, return_lst=True)), fx["sdf_lst"], atol=SDF_TOL, rtol=0)
    # BaseLOD.forward ignores its lod argument and uses net.lod (here 1).
    np.testing.assert_allclose(dense.sdf(m, x, lod=1), fx["forward_lod1"], atol=SDF_TOL, rtol=0)


def test_feature_volume_matches_torch_grid_sample(golden):
    import torch
    import torch.nn.functional as F
    fx = golden("dense_small")
    fm = fx["param/features.2.fm"]
    x = fx["points"]
    ref = F.grid_sample(torch.from_numpy(fm).double(), torch.from_numpy(x).double().reshape(1, -1, 1, 1, 3),
                        align_corners=True, padding_mode="border")[0, :, :, 0, 0].T.numpy()
    np.testing.assert_allclose(dense.feature_volume(fm[0].astype(np.float64), x), ref, atol=1e-12, rtol=0)


def test_aabb_oracles_agree_and_edge_cases():
    rng = np.random.default_rng(3)
    o = rng.uniform(-3, 3, (4000, 3)).astype(np.float32)
    d = rng.normal(size=(4000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:50, 0] = 0.0  # axis-parallel rays: infinite reciprocals
    o[50:60] = [0.1, 0.2, 0.3]  # origins inside the box are skipped
    xc, tc, hc = cref.aabb(o, d)
    xn, tn, hn = dense.aabb(o.astype(np.float64), d.astype(np.float64))
    assert (hc == hn).mean() > 0.999
    both = hc & hn
    np.testing.assert_allclose(tc[both], tn[both], atol=1e-5, rtol=0)
    assert not hc[50:60].any() and (tc[50:60] == 0).all() and (xc[50:60] == o[50:60]).all()
    miss = ~hc
    assert (xc[miss] == o[miss]).all() and (tc[miss] == 0).all()


def test_get_min_matches_reference(golden):
    """The oracle's get_min against the reference's own SphereTracer.get_min
    (tests/golden/get_min_small.npz) on trace_small's network."""
    fx = golden("get_min_small")
    net = model_from_fixture(golden("trace_small"), 2, 3)
    m = oracle_model(net, np.float32)
    x, t, hit, normal, minx = dense.get_min(m, fx["ray_o"], fx["ray_d"], num_steps=int(fx["num_steps"]),
                                            aabb_fn=cref.aabb)
    assert (hit == fx["hit"]).mean() >= 0.9999
    both = hit & fx["hit"]
    for got, want in [(t, fx["depth"]), (x, fx["x"]), (minx, fx["min_x"])]:
        np.testing.assert_allclose(got[both], want[both], atol=DEPTH_TOL, rtol=0)
        np.testing.assert_allclose(got[~both], want[~both], atol=DEPTH_TOL, rtol=1e-4)
    np.testing.assert_allclose(normal[both], fx["normal"][both], atol=1e-3, rtol=0)
    # rays that miss the box march from their origins under get_min's rules
    _, _, in_box = cref.aabb(fx["ray_o"], fx["ray_d"])
    moved = np.abs(fx["x"] - fx["ray_o"]).max(axis=1) > 0
    assert (~in_box).sum() > 0 and moved[~in_box].all()


@pytest.mark.parametrize("name,lod", [("lodNone", None), ("lod0", 0)])
def test_sphere_trace_matches_reference(golden, name, lod):
    fx = golden("trace_small")
    net = model_from_fixture(fx, 2, 3)
    m = oracle_model(net, np.float32)
    x, t, hit, normal = dense.sphere_trace(m, fx["ray_o"], fx["ray_d"], lod=lod, num_steps=int(fx["trace/num_steps"]),
                                           aabb_fn=cref.aabb)
    assert (hit == fx[f"{name}/hit"]).mean() >= 0.9999
    both = hit & fx[f"{name}/hit"]
    # Depth bar on rays that hit; rays that run out past the far clip carry
    # ~60 steps of float32 rounding, bounded relatively.
    np.testing.assert_allclose(t[both], fx[f"{name}/depth"][both], atol=DEPTH_TOL, rtol=0)
    np.testing.assert_allclose(t[~both], fx[f"{name}/depth"][~both], atol=DEPTH_TOL, rtol=1e-4)
    np.testing.assert_allclose(normal[both], fx[f"{name}/normal"][both], atol=1e-3, rtol=0)
    # The reference's quirk: rays that start inside the box are never marched
    # but count as hits at depth 0 (SphereTracer.py:84,119).
    assert fx[f"{name}/hit"][-7] and fx[f"{name}/depth"][-7, 0] == 0


def test_torch_port_matches_reference(golden):
    """The CPU-baseline port reproduces the reference's outputs."""
    import torch
    from oracle import torch_port
    fx = golden("dense_small")
    sd = {k[len("param/"):]: torch.from_numpy(v) for k, v in fx.items() if k.startswith("param/")}
    net = torch_port.RefOctreeSDF(sd, 3)
    x = torch.from_numpy(fx["points"])
    with torch.no_grad():
        for lod in [0, 1, 2]:
            np.testing.assert_allclose(net.sdf(x, lod=lod).numpy(), fx[f"sdf_lod{lod}"], atol=1e-6, rtol=0)
    tx = golden("trace_small")
    sd = {k[len("param/"):]: torch.from_numpy(v) for k, v in tx.items() if k.startswith("param/")}
    tnet = torch_port.RefOctreeSDF(sd, 2)
    x, t, hit, normal = torch_port.sphere_trace(tnet, torch.from_numpy(tx["ray_o"]), torch.from_numpy(tx["ray_d"]),
                                                num_steps=int(tx["trace/num_steps"]))
    assert (hit.numpy() == tx["lodNone/hit"]).mean() >= 0.9999
    both = hit.numpy() & tx["lodNone/hit"]
    np.testing.assert_allclose(t.numpy()[both], tx["lodNone/depth"][both], atol=DEPTH_TOL, rtol=0)
