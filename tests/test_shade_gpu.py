"""Shading passes on the GPU (nglod_shade_*, nglod_gb300.renderer.Renderer)
against the reference Renderer's own output (tests/golden/shade_small.npz)
and, stage by stage on the same inputs, against the oracle (oracle/shade.py)."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300.options import default_args
from nglod_gb300.renderer import Renderer
from oracle import dense, shade
from tests.helpers import model_from_fixture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(golden, cuda):
    z = golden("shade_small")
    net = model_from_fixture(golden("trace_small"), 2, 3, cuda)
    W, H = int(z["width"]), int(z["height"])
    tracer = ng.SphereTracer(default_args(num_steps=64, min_dis=0.0003, step_size=1.0, camera_clamp=[-5, 10]))
    r = Renderer(tracer, args=default_args(render_res=[W, H], shadow=True, ao=True, ground_height=-0.7),
                 matcap=z["matcap"])
    return z, net, r, (W, H)


def test_renderer_matches_reference_renderer(setup, cuda):
    z, net, r, (W, H) = setup
    ro = torch.from_numpy(z["ray_o"]).to(cuda)
    rd = torch.from_numpy(z["ray_d"]).to(cuda)
    rb = r.shade_buffer(r._render_flat(net, ro, rd, shadow_noise=torch.from_numpy(z["noise"])))
    got = {k: getattr(rb, k).reshape(W * H, -1).cpu().numpy() for k in
           ("x", "depth", "hit", "normal", "rgb", "shadow", "ao", "relative_depth")}
    want = {k: z[k].reshape(W * H, -1) for k in got}
    assert (got["hit"] == want["hit"]).mean() >= 0.999
    assert (got["shadow"] == want["shadow"]).mean() >= 0.995
    same = (got["hit"] == want["hit"])[:, 0]
    for k, tol in {"x": 1e-4, "depth": 1e-4, "relative_depth": 1e-5, "normal": 2e-3, "ao": 2e-3}.items():
        np.testing.assert_allclose(got[k][same], want[k][same], atol=tol, rtol=0, err_msg=k)
    # colour: blurred shadows spread a flipped shadow ray over a few pixels
    d = np.abs(got["rgb"] - want["rgb"])
    assert np.percentile(d, 99) < 2e-3 and d.mean() < 5e-4, (np.percentile(d, 99), d.mean())


def test_stages_match_oracle_on_same_inputs(setup, cuda):
    z, net, r, (W, H) = setup
    lib = ng._lib.load()
    u = lambda t: ng._lib.ptr(t)
    st = ng._lib.stream_ptr(cuda)
    rng = np.random.default_rng(3)
    n = W * H
    ro, rd = z["ray_o"], z["ray_d"]
    x = z["x"].astype(np.float32)
    t = (z["depth"] + rng.uniform(0, 3, (n, 1))).astype(np.float32)
    hit = z["hit"][:, 0].copy()
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    # ground plane (every device input is held by a name for as long as the
    # kernels reading it may run)
    dx, dt, dh, dn = (torch.from_numpy(a.copy()).to(cuda) for a in (x, t, hit, nrm))
    dro, drd = torch.from_numpy(ro).to(cuda), torch.from_numpy(rd).to(cuda)
    ph = torch.empty(n, dtype=torch.bool, device=cuda)
    ng._lib.check(lib.nglod_shade_ground(u(dro), u(drd), n, -0.7, u(dx), u(dt), u(dh), u(dn), u(ph), st), "ground")
    ox, ot, oh, on, oph = shade.ground(ro, rd, -0.7, x, t, hit, nrm)
    assert oph.sum() > 50
    for a, b in ((dx, ox), (dt, ot), (dh, oh), (dn, on), (ph, oph)):
        assert np.array_equal(a.cpu().numpy(), b)
    # shadow rays
    noise = z["noise"]
    so, sd = torch.empty(n, 3, device=cuda), torch.empty(n, 3, device=cuda)
    lh = torch.empty(n, dtype=torch.bool, device=cuda)
    light = np.asarray(shade.LIGHT, np.float32)
    dnoise = torch.from_numpy(noise).to(cuda)
    ng._lib.check(lib.nglod_shade_shadow_rays(u(dx), u(dn), u(dnoise), n, light.ctypes.data_as(ng._lib.ctypes.c_void_p),
                                              u(so), u(sd), u(lh), st), "shadow rays")
    oso, osd, olh = shade.shadow_rays(ox, on, noise)
    assert np.array_equal(so.cpu().numpy(), oso)
    np.testing.assert_allclose(sd.cpu().numpy(), osd, atol=1e-6, rtol=0)
    assert (lh.cpu().numpy() == olh).mean() > 0.999
    # ambient occlusion with the oracle's float32 sdf at the GPU's own taps
    m32 = dense.model_from_state_dict(net.state_dict(), 2, 3, np.float32)
    rb = ng.RenderBuffer(x=dx, hit=dh, normal=dn)
    ao = r._ambient_occlusion(net, rb, ph).cpu().numpy()[:, 0]
    oao = shade.ambient_occlusion(lambda q: dense.sdf(m32, q)[:, 0].astype(np.float32), ox, on, oh, oph)
    np.testing.assert_allclose(ao, oao, atol=1e-5, rtol=0)
    assert (oao < 0.999).sum() > 20
    # matcap and shadow map
    tex = r._texture_on(cuda)
    rgb = torch.empty(n, 3, device=cuda)
    ng._lib.check(lib.nglod_shade_matcap(u(drd), u(dn), u(dh), n, u(tex), tex.shape[0], tex.shape[1], u(rgb), st),
                  "matcap")
    np.testing.assert_allclose(rgb.cpu().numpy(), shade.matcap_rgb(z["matcap"], rd, on, oh), atol=1e-5, rtol=0)
    sh = torch.from_numpy(rng.random(n) < 0.3).to(cuda)
    smap, scratch = torch.empty(n, device=cuda), torch.empty(n, device=cuda)
    sflag = torch.empty(n, dtype=torch.bool, device=cuda)
    ng._lib.check(lib.nglod_shade_shadow_map(u(sh), u(lh), W, H, 2.0, u(smap), u(scratch), u(sflag), st),
                  "shadow map")
    want = shade.shadow_map(sh.cpu().numpy() & lh.cpu().numpy(), W, H)
    np.testing.assert_allclose(smap.cpu().numpy(), want, atol=1e-7, rtol=0)


def test_shade_tensor_and_images(setup, cuda):
    z, net, r, (W, H) = setup
    rb = r.shade_tensor(net, f=(1.2, 1.6, 3.2), t=(0.0, -0.2, 0.0), fov=40.0)
    assert rb.rgb.shape == (W, H, 3) and rb.hit.shape == (W, H, 1) and rb.ao.shape == (W, H, 1)
    assert 0.0 <= rb.rgb.min().item() and rb.rgb.max().item() <= 1.0
    assert (rb.rgb[~rb.hit[..., 0]] <= 1.0).all()
    img = r.shade_images(net, f=(1.2, 1.6, 3.2), t=(0.0, -0.2, 0.0), fov=40.0)
    assert img.rgb.shape == (H, W, 3) and img.rgb.device.type == "cpu"
    # the BF16 form renders the same picture within its precision
    from nglod_gb300.bf16 import Bf16OctreeSDF
    b = Bf16OctreeSDF(net)
    torch.manual_seed(1)
    rb32 = r.shade_tensor(net, f=(1.2, 1.6, 3.2), t=(0.0, -0.2, 0.0), fov=40.0)
    torch.manual_seed(1)
    rb16 = r.shade_tensor(b, f=(1.2, 1.6, 3.2), t=(0.0, -0.2, 0.0), fov=40.0)
    b.check_status()
    assert (rb16.hit == rb32.hit).float().mean().item() > 0.99
    assert (rb16.rgb - rb32.rgb).abs().mean().item() < 0.02
