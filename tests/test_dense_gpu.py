"""Parity of the dense float32 CUDA path with the oracle and the reference's
golden vectors.  Tolerances follow the spec bar: 1e-5 abs on SDF
values, 1e-4 on depth of hit rays, >= 99.99 % hit-mask agreement."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

import nglod_gb300 as ng
from nglod_gb300 import synthetic
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.options import default_args
from oracle import cref, dense
from tests.helpers import model_from_fixture, oracle_model, seeded_model

pytestmark = pytest.mark.gpu

SDF_TOL = 1e-5
DEPTH_TOL = 1e-4


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-3, 3, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:64, 1] = 0.0
    d[64:96, :2] = 0.0
    o[96:160] = rng.uniform(-0.9, 0.9, (64, 3))
    o[160:200, 0] = 1.0
    return o, d


def test_aabb_bit_exact(cuda):
    o, d = _rays(200_000, 1)
    x, t, hit = ng.sol_nglod.aabb(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda))
    xo, to, ho = cref.aabb(o, d)
    assert np.array_equal(hit.cpu().numpy(), ho)
    assert np.array_equal(t.cpu().numpy().view(np.uint32), to.view(np.uint32))
    assert np.array_equal(x.cpu().numpy().view(np.uint32), xo.view(np.uint32))


def test_volume_sample_matches_grid_sample(cuda):
    net = seeded_model(num_lods=3, seed=2).to(cuda)
    x = torch.rand(50_000, 3, device=cuda) * 2.4 - 1.2
    for fv in net.features:
        got = fv(x)
        ref = F.grid_sample(fv.fm.detach().double(), x.double().reshape(1, -1, 1, 1, 3), align_corners=True,
                            padding_mode="border")[0, :, :, 0, 0].T
        assert (got.double() - ref).abs().max().item() < 1e-6


def test_sdf_matches_reference_golden(golden, cuda):
    fx = golden("dense_small")
    net = model_from_fixture(fx, 3, 1, device=cuda)
    x = torch.from_numpy(fx["points"]).to(cuda)
    with torch.no_grad():
        for lod in [0, 1, 2]:
            np.testing.assert_allclose(net.sdf(x, lod=lod).cpu().numpy(), fx[f"sdf_lod{lod}"], atol=SDF_TOL, rtol=0)
        np.testing.assert_allclose(net.sdf(x).cpu().numpy(), fx["sdf_lodNone"], atol=SDF_TOL, rtol=0)
        np.testing.assert_allclose(net.sdf(x, lod=7).cpu().numpy(), fx["sdf_lod7"], atol=SDF_TOL, rtol=0)
        lst = net.sdf(x, return_lst=True)
        np.testing.assert_allclose(torch.stack(lst).cpu().numpy(), fx["sdf_lst"], atol=SDF_TOL, rtol=0)
        net.lod = 1
        np.testing.assert_allclose(net(x, lod=0).cpu().numpy(), fx["forward_lod1"], atol=SDF_TOL, rtol=0)


def test_sdf_full_architecture_vs_fp64_oracle(cuda):
    """Config: 5 LODs (5^3..65^3), C=32, H=128, seed 0, 262,144 points U[-1,1]^3."""
    net = seeded_model(num_lods=5, base_lod=2, seed=0).to(cuda)
    x = synthetic.uniform_points(262_144, seed=0)
    m = oracle_model(net.cpu(), np.float64)
    net = net.to(cuda)
    with torch.no_grad():
        got = net.sdf(x.to(cuda), lod=4).cpu().numpy()
    ref = dense.sdf(m, x.numpy(), lod=4)
    assert np.abs(got - ref).max() < SDF_TOL
    sub = x[:8192]
    with torch.no_grad():
        lst = [t.cpu().numpy() for t in net.sdf(sub.to(cuda), return_lst=True)]
    ref_lst = dense.sdf(m, sub.numpy(), return_lst=True)
    for lod in range(5):
        assert np.abs(lst[lod] - ref_lst[lod]).max() < SDF_TOL


def test_sdf_training_mode_keeps_loss_preds(cuda):
    net = seeded_model(num_lods=3, seed=4).to(cuda)
    net.train()
    x = torch.rand(1000, 3, device=cuda) * 2 - 1
    with torch.no_grad():
        out = net.sdf(x)
        assert isinstance(net.loss_preds, list) and len(net.loss_preds) == 3
        assert torch.equal(out, net.loss_preds[-1])
        net.loss_preds = None
        net.sdf(x, lod=1)
        assert net.loss_preds is None


def test_empty_and_ragged_inputs(cuda):
    net = seeded_model(num_lods=2, seed=1).to(cuda)
    with torch.no_grad():
        assert net.sdf(torch.zeros(0, 3, device=cuda)).shape == (0, 1)
        for n in [1, 31, 33, 257, 1023]:
            x = torch.rand(n, 3, device=cuda) * 2 - 1
            got = net.sdf(x).cpu().numpy()
            ref = dense.sdf(oracle_model(net.cpu()), x.cpu().numpy())
            net.to(cuda)
            assert np.abs(got - ref).max() < SDF_TOL
    rb = ng.SphereTracer(default_args(num_steps=16))(net, torch.zeros(0, 3, device=cuda), torch.zeros(0, 3, device=cuda))
    assert rb.x.shape == (0, 3)


def _check_trace(rb, x, t, hit, normal):
    h = rb.hit.cpu().numpy()
    assert (h == hit).mean() >= 0.9999
    both = h & hit
    tt = rb.depth.cpu().numpy()
    np.testing.assert_allclose(tt[both], t[both], atol=DEPTH_TOL, rtol=0)
    np.testing.assert_allclose(tt[~both], t[~both], atol=DEPTH_TOL, rtol=1e-4)
    np.testing.assert_allclose(rb.normal.cpu().numpy()[both], normal[both], atol=1e-3, rtol=0)
    assert (rb.normal.cpu().numpy()[~h] == 0).all()


@pytest.mark.parametrize("name,lod", [("lodNone", None), ("lod0", 0)])
@pytest.mark.parametrize("tracer_cls", [ng.SphereTracer, ng.PlainSphereTracer])
def test_trace_matches_reference_golden(golden, cuda, name, lod, tracer_cls):
    fx = golden("trace_small")
    net = model_from_fixture(fx, 2, 3, device=cuda)
    net.lod = lod
    tracer = tracer_cls(default_args(num_steps=int(fx["trace/num_steps"])))
    rb = tracer(net, torch.from_numpy(fx["ray_o"]).to(cuda), torch.from_numpy(fx["ray_d"]).to(cuda))
    _check_trace(rb, None, fx[f"{name}/depth"], fx[f"{name}/hit"], fx[f"{name}/normal"])
    assert rb.hit[-7].item() and rb.depth[-7, 0].item() == 0.0


@pytest.mark.parametrize("tracer_cls", [ng.SphereTracer, ng.PlainSphereTracer])
def test_get_min_matches_reference_golden(golden, cuda, tracer_cls):
    """SphereTracer.get_min against the reference's own get_min on
    trace_small's network (tests/golden/get_min_small.npz): hit mask, depth
    and final point at the trace tolerances, the unnormalised finite-difference
    normals at 1e-3, and the minimum-sdf points min_x at the depth tolerance."""
    fx = golden("get_min_small")
    tr = golden("trace_small")
    net = model_from_fixture(tr, 2, 3, device=cuda)
    net.lod = None
    tracer = tracer_cls(default_args(num_steps=int(fx["num_steps"])))
    rb = tracer.get_min(net, torch.from_numpy(fx["ray_o"]).to(cuda), torch.from_numpy(fx["ray_d"]).to(cuda))
    h = rb.hit.cpu().numpy()
    assert (h == fx["hit"]).mean() >= 0.9999
    both = h & fx["hit"]
    # hit rays at the depth bar; rays that march out to the far clip carry
    # their steps' float32 rounding, bounded relatively (as for forward)
    for got, want in [(rb.depth, fx["depth"]), (rb.x, fx["x"]), (rb.min_x, fx["min_x"])]:
        got = got.cpu().numpy()
        np.testing.assert_allclose(got[both], want[both], atol=DEPTH_TOL, rtol=0)
        np.testing.assert_allclose(got[~both], want[~both], atol=DEPTH_TOL, rtol=1e-4)
    np.testing.assert_allclose(rb.normal.cpu().numpy()[both], fx["normal"][both], atol=1e-3, rtol=0)
    assert (rb.normal.cpu().numpy()[~h] == 0).all()


def test_trace_full_model_vs_oracle(cuda):
    """5-LOD network holding the seed-1 sphere union; 96x96 camera, 128 steps."""
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=2)
    m = oracle_model(net, np.float32)
    net = net.to(cuda).eval()
    ro, rd = synthetic.look_at_rays(width=96, height=96)
    rb = ng.SphereTracer(default_args(num_steps=128))(net, ro.to(cuda), rd.to(cuda))
    x, t, hit, normal = dense.sphere_trace(m, ro.numpy(), rd.numpy(), num_steps=128, aabb_fn=cref.aabb)
    assert hit.sum() > 1000
    _check_trace(rb, x, t, hit, normal)
    both = rb.hit.cpu().numpy() & hit
    assert np.abs(rb.x.cpu().numpy()[both] - x[both]).max() < DEPTH_TOL


def test_trace_matches_plain_tracer_at_scale(cuda):
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=2)
    net = net.to(cuda).eval()
    ro, rd = synthetic.look_at_rays(width=640, height=360)
    a = default_args(num_steps=64)
    fused = ng.SphereTracer(a)(net, ro.to(cuda), rd.to(cuda))
    plain = ng.PlainSphereTracer(a)(net, ro.to(cuda), rd.to(cuda))
    _check_trace(fused, None, plain.depth.cpu().numpy(), plain.hit.cpu().numpy(), plain.normal.cpu().numpy())


def test_frame_size_traces_vs_oracle_on_sampled_rays(cuda):
    """The bench's 1920x1080 frame (64 steps) traced by the fused float32
    and BF16 tracers; rays are independent, so a random sample of 6,000 of
    them is checked against the oracle traced alone: float32 against the
    float32 oracle at the drop-in's tolerances, BF16 against the FP64 oracle
    at the BF16 bar (hit agreement >= 99 %, mean |depth| <= 1e-3)."""
    from nglod_gb300.bf16 import Bf16OctreeSDF
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=2)
    m32, m64 = oracle_model(net, np.float32), oracle_model(net, np.float64)
    net = net.to(cuda).eval()
    ro, rd = synthetic.look_at_rays(width=1920, height=1080)
    a = default_args(num_steps=64)
    f32 = ng.SphereTracer(a)(net, ro.to(cuda), rd.to(cuda))
    b16 = ng.SphereTracer(a)(Bf16OctreeSDF(net), ro.to(cuda), rd.to(cuda))
    rng = np.random.default_rng(7)
    hits = np.flatnonzero(f32.hit.cpu().numpy().reshape(-1))
    pick = np.concatenate([rng.choice(hits, 4000, replace=False), rng.integers(0, ro.shape[0], 2000)])
    so, sd = ro.numpy()[pick], rd.numpy()[pick]
    x, t, hit, normal = dense.sphere_trace(m32, so, sd, num_steps=64, aabb_fn=cref.aabb)
    sub = lambda rb: ng.tracer.RenderBuffer(x=rb.x[pick], depth=rb.depth[pick], hit=rb.hit[pick],
                                            normal=rb.normal[pick])
    _check_trace(sub(f32), x, t, hit, normal)
    x6, t6, h6, _ = dense.sphere_trace(m64, so.astype(np.float64), sd.astype(np.float64), num_steps=64,
                                       aabb_fn=lambda o, d: tuple(v.astype(np.float64) if v.dtype != bool else v
                                                                  for v in cref.aabb(o.astype(np.float32),
                                                                                     d.astype(np.float32))))
    hb = b16.hit.cpu().numpy()[pick]
    assert (hb == h6).mean() >= 0.99
    both = hb & h6
    assert np.abs(b16.depth.cpu().numpy()[pick][both, 0] - t6[both, 0]).mean() <= 1e-3


@pytest.fixture(scope="module")
def full_net(cuda):
    """The full architecture (5 LODs, 5^3..65^3 volumes, C=32, H=128) holding
    the sphere-union SDF, and 262,144 query points of the headline's
    distribution."""
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=2)
    x = synthetic.near_surface_query(262_144, c, r, seed=1)
    return net.to(cuda).eval(), x.to(cuda)


def _simt(net, x, lod):
    from nglod_gb300 import _lib
    out = torch.empty(x.shape[0], 1, device=x.device)
    _lib.check(_lib.load().nglod_sdf_fwd_simt(net.dense_model(), _lib.ptr(x), x.shape[0], lod, 0, _lib.ptr(out),
                                              _lib.stream_ptr(x.device)), "nglod_sdf_fwd_simt")
    return out


@pytest.mark.parametrize("lod", [0, 2, 4])
def test_tensor_core_f32_query_within_float32_bounds(full_net, lod):
    """The float32 query's tensor-core form (split-TF32 decoder) against
    float64 and against the per-thread float32 decoder on 262,144 points: both
    forms stay within 1e-5 of float64, and within 2e-6 of each other."""
    net, x = full_net
    with torch.no_grad():
        tc = net.sdf(x, lod=lod)
    net.check_status()
    simt = _simt(net, x, lod)
    m64 = oracle_model(net, np.float64)
    want = dense.sdf(m64, x.cpu().numpy().astype(np.float64), lod=lod)
    e_tc = np.abs(tc.cpu().numpy().astype(np.float64) - want).max()
    e_simt = np.abs(simt.cpu().numpy().astype(np.float64) - want).max()
    assert e_tc < SDF_TOL and e_simt < SDF_TOL, (e_tc, e_simt)
    assert (tc - simt).abs().max().item() < 2e-6


@pytest.mark.parametrize("base_lod,num_lods,lod", [(1, 4, 3), (2, 2, 1), (3, 3, 2), (2, 5, 0), (4, 2, 1)])
def test_tensor_core_f32_query_staging_variants(cuda, base_lod, num_lods, lod):
    """The persistent float32 query stages the leading volumes that fit in
    shared memory beside its tiles: three levels at base_lod 1 (3^3, 5^3,
    9^3), two at base_lod 2, one at base_lod 3 (9^3; 17^3 does not fit), none
    at base_lod 4, only LOD 0 when lod = 0.  Each variant against the
    per-thread float32 decoder and float64, on ragged sizes (partial last
    tile, fewer tiles than groups, points outside the box)."""
    net = seeded_model(num_lods=num_lods, base_lod=base_lod, seed=base_lod).to(cuda)
    m64 = oracle_model(net.cpu(), np.float64)
    net.to(cuda)
    gen = torch.Generator().manual_seed(11 + base_lod)
    for n in [1, 127, 129, 513, 70_001]:
        x = (torch.rand(n, 3, generator=gen) * 2.4 - 1.2).to(cuda)
        with torch.no_grad():
            tc = net.sdf(x, lod=lod)
        net.check_status()
        simt = _simt(net, x, lod)
        want = dense.sdf(m64, x.cpu().numpy().astype(np.float64), lod=lod)
        assert np.abs(tc.cpu().numpy().astype(np.float64) - want).max() < SDF_TOL, n
        assert (tc - simt).abs().max().item() < 2e-6, n


def test_tensor_core_f32_wait_timeout_reports_status_and_recovers(full_net):
    """The error path of the float32 query's bounded tensor-core wait,
    without a GPU fault: with the wait cut to one non-blocking test the call
    reports a timeout through nglod_dense_status, and the next call with the
    default bound gives the same values as before."""
    from nglod_gb300 import _lib
    net, x = full_net
    lib = _lib.load()
    with torch.no_grad():
        good = net.sdf(x, lod=4)
    net.check_status()
    try:
        _lib.check(lib.nglod_debug_mma_wait_polls(0), "nglod_debug_mma_wait_polls")
        with torch.no_grad():
            net.sdf(x, lod=4)
        with pytest.raises(RuntimeError, match="timed out"):
            net.check_status()
    finally:
        _lib.check(lib.nglod_debug_mma_wait_polls(-1), "nglod_debug_mma_wait_polls")
    with torch.no_grad():
        again = net.sdf(x, lod=4)
    net.check_status()
    assert torch.equal(again, good)
