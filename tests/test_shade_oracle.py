"""The shading oracle (oracle/shade.py) against the reference Renderer's own
output (tests/golden/shade_small.npz: Renderer.shade_tensor with a ground
plane, shadow rays, ambient occlusion and matcap shading)."""
import numpy as np

from oracle import dense, shade


def _model(golden):
    tr = golden("trace_small")
    sd = {k[len("param/"):]: tr[k] for k in tr if k.startswith("param/")}
    return dense.model_from_state_dict(sd, 2, 3, np.float32)


def test_shade_oracle_matches_reference_renderer(golden):
    z = golden("shade_small")
    W, H = int(z["width"]), int(z["height"])
    o = shade.shade(_model(golden), z["ray_o"], z["ray_d"], z["noise"], z["matcap"], float(z["ground_height"]), W, H)
    flat = lambda a: np.asarray(a).reshape(W * H, -1)
    assert np.array_equal(flat(o["hit"]), flat(z["hit"]))
    assert np.array_equal(flat(o["shadow"]), flat(z["shadow"]))
    assert flat(z["hit"]).sum() > 100 and flat(z["shadow"]).sum() > 100
    tol = {"x": 1e-5, "depth": 1e-5, "relative_depth": 1e-6, "normal": 5e-5, "ao": 1e-4, "rgb": 5e-4}
    for k, t in tol.items():
        np.testing.assert_allclose(flat(o[k]), flat(z[k]), atol=t, rtol=0, err_msg=k)


def test_ground_plane_and_ao_edge_cases():
    # a ray parallel to the plane, one pointing away, one hitting the plane in front of the surface
    ro = np.array([[0, 0.5, 3], [0, 0.5, 3], [0, 0.5, 3]], np.float32)
    rd = np.array([[0, 0, -1], [0, 1, 0], [0, -0.6, -0.8]], np.float32)
    x = ro.copy()
    t = np.full((3, 1), 5.0, np.float32)
    hit = np.array([True, False, True])
    normal = np.zeros((3, 3), np.float32)
    x2, t2, hit2, n2, ph = shade.ground(ro, rd, -0.5, x, t, hit, normal)
    assert ph.tolist() == [False, False, True]
    assert hit2.tolist() == [True, False, False] and n2[2].tolist() == [0, 1, 0]
    assert abs(t2[2, 0] - 1.0 / 0.6) < 1e-6
    # AO of an unoccluded point is 1; a point inside a wall is darkened to the floor 0.1^2
    ao_free = shade.ambient_occlusion(lambda q: np.full(q.shape[0], 10.0, np.float32), x2[:1], np.array(
        [[0, 1, 0]], np.float32), np.array([True]))
    ao_wall = shade.ambient_occlusion(lambda q: np.full(q.shape[0], -1.0, np.float32), x2[:1], np.array(
        [[0, 1, 0]], np.float32), np.array([True]))
    assert ao_free[0] == 1.0 and abs(ao_wall[0] - 0.01) < 1e-7
