"""Sparse SDF (sol-renderer's SDF class) on the GPU against the numpy
restatement of SDF::sphereTrace and against the dense model."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import spc, synthetic
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.options import default_args
from nglod_gb300.sparse_sdf import SparseSDF
from oracle import sparse as osparse
from oracle import spc as ospc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(cuda):
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=4, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=3)
    level = 5  # LODs 0..3 on octree levels 2..5
    vox = ospc.voxels_near_surface(lambda p: synthetic.sphere_union_sdf(p, c, r), level)
    s = spc.SPC.from_voxels(torch.from_numpy(vox.astype(np.int32)).to(cuda), level)
    net = net.to(cuda).eval()
    return net, s, (c, r)


def _oracle_model(net, s, num_lods):
    pts = s.GetPoints().cpu().numpy()
    pyr = s.GetPyramid().numpy()
    fms = [fv.fm.detach().cpu().numpy()[0].astype(np.float16).astype(np.float32) for fv in net.features]
    m = osparse.build(fms, pts, pyr, num_lods)
    decs = [tuple(t.detach().cpu().numpy().astype(np.float16).astype(np.float32).reshape(t.shape)
                  for t in (d[0].weight, d[0].bias, d[2].weight, d[2].bias)) for d in net.louts]
    return m, decs


def test_build_matches_oracle(scene):
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s)
    m, _ = _oracle_model(net, s, 4)
    assert sp.corner_counts == m["counts"]
    np.testing.assert_array_equal(sp.corner_feats.cpu().numpy(), m["cf"])
    pyr = s.GetPyramid().numpy()
    a = pyr[1, 2]
    np.testing.assert_array_equal(sp.corner_idx.cpu().numpy()[a:], m["trink"][a:])
    np.testing.assert_array_equal(sp.parent.cpu().numpy()[a:], m["parent"][a:])


@pytest.mark.parametrize("lod", [0, 3])
def test_query_equals_dense_inside_voxels(scene, lod):
    """With float32 features and weights the sparse SDF equals the dense one
    at points inside occupied voxels; outside it is NaN."""
    net, s, (c, r) = scene
    sp = SparseSDF.from_dense(net, s, precision="f32", half_weights=False)
    x = synthetic.near_surface_query(20000, c, r, seed=4).to(s.GetOctree().device)
    got = sp.forward(x, lod)
    with torch.no_grad():
        want = net.sdf(x, lod=lod)
    inside = ~torch.isnan(got[:, 0])
    assert inside.float().mean() > 0.3
    assert (got[inside] - want[inside]).abs().max().item() < 1e-5
    # NaN exactly where the point's voxel at octree level lod+2 is unoccupied
    res = 2 ** (lod + 2)
    vox = ((x + 1) / 2 * res).floor().long().clamp(0, res - 1)
    occ = torch.zeros(res, res, res, dtype=torch.bool, device=x.device)
    lp = s.GetLevelPoints(lod + 2)[:, :3].long()
    occ[lp[:, 0], lp[:, 1], lp[:, 2]] = True
    assert torch.equal(inside, occ[vox[:, 0], vox[:, 1], vox[:, 2]])
    assert torch.isnan(sp.forward(torch.tensor([[2.0, 0.0, 0.0]], device=x.device), lod)).all()


@pytest.mark.parametrize("precision,decoder", [("fp16", "f32"), ("bf16", "f32"), ("bf16", "tc")])
def test_sparse_trace_matches_oracle(scene, precision, decoder):
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s, precision=precision, decoder=decoder)
    ro, rd = synthetic.look_at_rays(width=96, height=72)
    dev = s.GetOctree().device
    (x, t, hit, normal), nug = sp.render(ro.to(dev), rd.to(dev), lod=3, num_steps=50)
    sp.check_status()
    m, decs = _oracle_model(net, s, 4)
    if precision == "bf16":
        m["cf"] = sp.corner_feats.float().cpu().numpy()
    dfn = osparse.decode_bf16_tile if decoder == "tc" else osparse.decode
    xo, to, ho, no = osparse.sphere_trace(m, decs, 3, ro.numpy(), rd.numpy(), nug.cpu().numpy(), num_steps=50,
                                          decoder=dfn)
    h = hit.cpu().numpy()
    assert h.sum() > 500
    assert (h == ho).mean() >= 0.999
    both = h & ho
    if decoder == "f32":
        np.testing.assert_allclose(t.cpu().numpy()[both], to[both], atol=1e-4, rtol=0)
        np.testing.assert_allclose(normal.cpu().numpy()[both], no[both], atol=2e-3, rtol=0)
    else:
        # fp32 tensor-core sums against the float64 restatement: a step can
        # land on the other side of a hit threshold for a few rays
        err = np.abs(t.cpu().numpy()[both] - to[both])[:, 0]
        assert np.percentile(err, 99) < 1e-4 and err.max() < 5e-3, (np.percentile(err, 99), err.max())
        cosang = (normal.cpu().numpy()[both] * no[both]).sum(-1)
        assert np.percentile(cosang, 1) > 0.999
    nh = ~h & ~ho
    assert (normal.cpu().numpy()[nh] == 1).all()


def test_sparse_tc_trace_against_fp64_dense_oracle(scene):
    """Error of the tensor-core sparse trace (bf16 features and decoder)
    against the FP64 dense oracle trace of the same network, stated."""
    from oracle import cref, dense
    from tests.helpers import oracle_model
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s, precision="bf16", decoder="tc", half_weights=False)
    ro, rd = synthetic.look_at_rays(width=96, height=72)
    dev = s.GetOctree().device
    (x, t, hit, normal), _ = sp.render(ro.to(dev), rd.to(dev), lod=3, num_steps=64)
    sp.check_status()
    m64 = oracle_model(net, np.float64)
    xo, to, ho, no = dense.sphere_trace(m64, ro.numpy().astype(np.float64), rd.numpy().astype(np.float64),
                                        num_steps=128, lod=3, aabb_fn=lambda o, d: tuple(
                                            v.astype(np.float64) if v.dtype != bool else v
                                            for v in cref.aabb(o.astype(np.float32), d.astype(np.float32))))
    h = hit.cpu().numpy()
    both = h & ho
    assert both.sum() > 500 and (h == ho).mean() > 0.99
    err = np.abs(t.cpu().numpy()[both, 0] - to[both, 0])
    print(f"sparse tc trace depth vs fp64 dense: mean {err.mean():.2e} median {np.median(err):.2e} "
          f"p99 {np.percentile(err, 99):.2e}")
    assert np.median(err) < 1e-3


def test_sparse_tc_trace_corner_chains_are_identical(scene):
    """The tensor-core sparse trace reading each voxel's corner_chain row
    gives bit-identical x, t, hit and normals to the same trace walking the
    parent links, and the chain rows hold the ancestors' corner indices."""
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s, precision="bf16", decoder="tc")
    assert len(sp.chains) == sp.num_lods
    pyr = s.GetPyramid()
    lod = 3
    start, cnt = int(pyr[1, lod + 2]), int(pyr[1, lod + 3] - pyr[1, lod + 2])
    ci, par = sp.corner_idx.cpu().numpy().reshape(-1, 8), sp.parent.cpu().numpy()
    ch = sp.chains[lod].cpu().numpy()
    rng = np.random.default_rng(0)
    for v in rng.integers(0, cnt, 50):
        g = start + int(v)
        for k in range(lod + 1):
            assert np.array_equal(ch[v, k], ci[g]), (v, k)
            g = par[g]
    ro, rd = synthetic.look_at_rays(width=96, height=72)
    dev = s.GetOctree().device
    a, _ = sp.render(ro.to(dev), rd.to(dev), lod=lod, num_steps=64)
    for i in range(sp.num_lods):
        sp._m.corner_chain[i] = None
    b, _ = sp.render(ro.to(dev), rd.to(dev), lod=lod, num_steps=64)
    sp.check_status()
    assert a[2].sum().item() > 500
    for u, w in zip(a, b):
        assert torch.equal(u, w)


def test_sparse_vs_dense_tracer(scene):
    """The sparse trace (fp16 export, 50 steps) against the dense float32
    tracer on the same network: same surface within a voxel's reach."""
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s)
    ro, rd = synthetic.look_at_rays(width=128, height=96)
    dev = s.GetOctree().device
    net.lod = 3
    (x, t, hit, normal), _ = sp.render(ro.to(dev), rd.to(dev), lod=3, num_steps=50)
    rb = ng.SphereTracer(default_args(num_steps=128))(net, ro.to(dev), rd.to(dev))
    net.lod = None
    both = hit & rb.hit
    agree = (hit == rb.hit).float().mean().item()
    assert agree > 0.98, agree
    assert (t[both] - rb.depth[both]).abs().median().item() < 2e-3
    cosang = (normal[both] * rb.normal[both]).sum(-1)
    assert cosang.median().item() > 0.99


def test_npz_round_trip(scene, tmp_path):
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s)
    path = tmp_path / "model.npz"
    sp.save_npz(str(path))
    z = np.load(str(path))
    assert set(z.files) == {"octree", "cc", "cf", "w0", "b0", "w1", "b1", "pyramid"}
    assert z["cc"].dtype == np.uint8 and z["cf"].dtype == np.float16 and z["w0"].shape == (4, 128, 35)
    sp2 = SparseSDF.from_npz(str(path))
    assert torch.equal(sp2.corner_idx, sp.corner_idx) and torch.equal(sp2.corner_feats, sp.corner_feats)
    ro, rd = synthetic.look_at_rays(width=64, height=48)
    dev = s.GetOctree().device
    a, _ = sp.render(ro.to(dev), rd.to(dev), lod=3)
    b, _ = sp2.render(ro.to(dev), rd.to(dev), lod=3)
    assert torch.equal(a[1], b[1]) and torch.equal(a[2], b[2])


@pytest.mark.parametrize("lod", [0, 3])
def test_summed_query_equals_dense_inside_voxels(scene, lod):
    """LOD-summed corner features (float32): one voxel's corners per query
    give the dense float32 SDF within rounding at points inside occupied
    voxels, and NaN at the same points as the per-level form."""
    net, s, (c, r) = scene
    sp = SparseSDF.from_dense(net, s, precision="f32", half_weights=False, summed=True)
    ref = SparseSDF.from_dense(net, s, precision="f32", half_weights=False)
    assert sp.summed and not sp.chains
    x = synthetic.near_surface_query(20000, c, r, seed=5).to(s.GetOctree().device)
    got = sp.forward(x, lod)
    with torch.no_grad():
        want = net.sdf(x, lod=lod)
    inside = ~torch.isnan(got[:, 0])
    assert torch.equal(inside, ~torch.isnan(ref.forward(x, lod)[:, 0]))
    assert inside.float().mean() > 0.3
    assert (got[inside] - want[inside]).abs().max().item() < 1e-5
    with pytest.raises(ValueError, match="npz"):
        sp.save_npz("/dev/null")


def test_summed_tc_trace_against_fp64_dense_oracle(scene):
    """The tensor-core sparse trace over LOD-summed bf16 corner features: the
    same bound against the FP64 dense oracle as the per-level trace, and the
    per-level trace's hit mask on all but a few rays."""
    from oracle import cref, dense
    from tests.helpers import oracle_model
    net, s, _ = scene
    sp = SparseSDF.from_dense(net, s, precision="bf16", decoder="tc", half_weights=False, summed=True)
    per_level = SparseSDF.from_dense(net, s, precision="bf16", decoder="tc", half_weights=False)
    ro, rd = synthetic.look_at_rays(width=96, height=72)
    dev = s.GetOctree().device
    (x, t, hit, normal), _ = sp.render(ro.to(dev), rd.to(dev), lod=3, num_steps=64)
    (_, t2, hit2, _), _ = per_level.render(ro.to(dev), rd.to(dev), lod=3, num_steps=64)
    sp.check_status()
    per_level.check_status()
    m64 = oracle_model(net, np.float64)
    xo, to, ho, no = dense.sphere_trace(m64, ro.numpy().astype(np.float64), rd.numpy().astype(np.float64),
                                        num_steps=128, lod=3, aabb_fn=lambda o, d: tuple(
                                            v.astype(np.float64) if v.dtype != bool else v
                                            for v in cref.aabb(o.astype(np.float32), d.astype(np.float32))))
    h = hit.cpu().numpy()
    both = h & ho
    assert both.sum() > 500 and (h == ho).mean() > 0.99
    err = np.abs(t.cpu().numpy()[both, 0] - to[both, 0])
    print(f"summed sparse tc trace depth vs fp64 dense: mean {err.mean():.2e} median {np.median(err):.2e} "
          f"p99 {np.percentile(err, 99):.2e}")
    assert np.median(err) < 1e-3
    assert (hit == hit2).float().mean().item() > 0.995


def test_summed_f32_decoder_trace_matches_per_level(scene):
    """The float32-decoder sparse trace over LOD-summed float32 corner
    features against the per-level one: same hits on all but a few rays,
    depths within 1e-4 where both hit."""
    net, s, _ = scene
    kw = dict(precision="f32", half_weights=False, decoder="f32")
    sp = SparseSDF.from_dense(net, s, summed=True, **kw)
    ref = SparseSDF.from_dense(net, s, **kw)
    ro, rd = synthetic.look_at_rays(width=96, height=72)
    dev = s.GetOctree().device
    (_, t, hit, _), _ = sp.render(ro.to(dev), rd.to(dev), lod=3, num_steps=50)
    (_, t2, hit2, _), _ = ref.render(ro.to(dev), rd.to(dev), lod=3, num_steps=50)
    both = hit & hit2
    assert both.sum().item() > 500
    assert (hit == hit2).float().mean().item() > 0.999
    assert np.percentile((t[both] - t2[both]).abs().cpu().numpy(), 99) < 1e-4
