"""BF16 form (bf16 volumes, tcgen05 decoder) against a numpy emulation of the
same bf16 arithmetic (tight), the FP64 oracle (error per LOD, reported and
bounded) and the float32 CUDA path."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import synthetic
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.bf16 import Bf16OctreeSDF
from nglod_gb300.options import default_args
from oracle import dense
from tests.helpers import seeded_model, oracle_model

pytestmark = pytest.mark.gpu

# BF16 error bounds against the FP64 oracle, per LOD 0..4, about twice the
# errors measured on the GB300 (analytic-init network with noise 1e-2,
# 65,536 near-surface points): per-LOD volumes max 6.2e-3 / mean 3.6e-4 at
# LOD 0 down to 5.3e-3 / 3.2e-4; LOD-summed volumes max 7.2e-3 / mean 4.3e-4.
PER_LOD_MAX = (1.3e-2, 1.2e-2, 1.1e-2, 1.1e-2, 1.1e-2)
PER_LOD_MEAN = (7.5e-4, 7.0e-4, 6.6e-4, 6.6e-4, 6.6e-4)
SUMMED_MAX = (1.45e-2, 1.3e-2, 1.4e-2, 1.4e-2, 1.3e-2)
SUMMED_MEAN = (8.6e-4, 6.8e-4, 6.2e-4, 7.2e-4, 7.6e-4)


def _bf16(a):
    """Round float32 array to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def emulate(m, x, lod, rounded=False):
    """The BF16 form's arithmetic in numpy: bf16 volumes, fp32 LOD sum rounded
    to bf16, positions and b0 as bf16 hi + lo, bf16 first-layer weights,
    products accumulated in float64, ReLU / second layer in float32.
    rounded: m's volumes already hold bf16 values."""
    x = x.astype(np.float32)
    acc = np.zeros((x.shape[0], 32), np.float32)
    for i in range(lod + 1):
        fm = m["fms"][i] if rounded else _bf16(m["fms"][i])
        acc += dense.feature_volume(fm.astype(np.float32), x)
    f = _bf16(acc)
    hi = _bf16(x)
    lo = _bf16(x - hi)
    w0 = _bf16(m["w0"][lod].astype(np.float32)).astype(np.float64)
    b0 = m["b0"][lod].astype(np.float32)
    b0h = _bf16(b0)
    b0l = _bf16(b0 - b0h)
    h = f.astype(np.float64) @ w0[:, 3:].T + hi.astype(np.float64) @ w0[:, :3].T + lo.astype(np.float64) @ w0[:, :3].T
    h = np.maximum((h + b0h + b0l).astype(np.float32), 0)
    return (h @ m["w1"][lod].astype(np.float32).T + m["b1"][lod].astype(np.float32))


def emulate_summed(m, x, lod):
    """emulate() for Bf16OctreeSDF(summed=True): volume lod = the LOD-summed
    volume rounded once to bf16, sampled alone."""
    x = x.astype(np.float32)
    sv = _bf16(dense.summed_volume(m, lod).astype(np.float32))
    one = {"fms": [sv], "w0": [m["w0"][lod]], "b0": [m["b0"][lod]], "w1": [m["w1"][lod]], "b1": [m["b1"][lod]]}
    return emulate(one, x, 0, rounded=True)


@pytest.fixture(scope="module")
def nets(cuda):
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-2, seed=1)
    m32 = oracle_model(net, np.float32)
    m64 = oracle_model(net, np.float64)
    net = net.to(cuda).eval()
    return net, Bf16OctreeSDF(net), m32, m64, (c, r)


def test_bf16_matches_emulation_and_reports_error(nets):
    net, bnet, m32, m64, (c, r) = nets
    x = synthetic.near_surface_query(65536, c, r, seed=2)
    dev = net.features[0].fm.device
    report = {}
    for lod in range(5):
        got = bnet.sdf(x.to(dev), lod=lod).cpu().numpy()
        emu = emulate(m32, x.numpy(), lod)
        np.testing.assert_allclose(got, emu, atol=2e-4, rtol=0)
        ref = dense.sdf(m64, x.numpy().astype(np.float64), lod=lod)
        err = np.abs(got - ref)
        report[lod] = (err.max(), err.mean())
        assert err.max() < PER_LOD_MAX[lod] and err.mean() < PER_LOD_MEAN[lod], (lod, err.max(), err.mean())
    bnet.check_status()
    print("bf16 error vs fp64 oracle per lod (max, mean):", report)


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 4097])
def test_bf16_ragged_sizes(nets, n):
    net, bnet, m32, _, _ = nets
    x = torch.rand(n, 3) * 2.2 - 1.1
    got = bnet.sdf(x.to(net.features[0].fm.device), lod=3).cpu().numpy()
    np.testing.assert_allclose(got, emulate(m32, x.numpy(), 3), atol=2e-4, rtol=0)


def test_bf16_full_size_against_float32_path(nets):
    net, bnet, _, _, (c, r) = nets
    dev = net.features[0].fm.device
    x = synthetic.near_surface_query(4_194_304, c, r, seed=1).to(dev)
    got = bnet.sdf(x, lod=4)
    with torch.no_grad():
        ref = net.sdf(x, lod=4)
    assert torch.isfinite(got).all()
    d = (got - ref).abs()
    print(f"bf16 vs float32 on 4M points at lod 4: max {d.max().item():.2e} mean {d.mean().item():.2e}")
    assert d.max().item() < 2e-2 and d.mean().item() < PER_LOD_MEAN[4]
    bnet.check_status()
    assert bnet.sdf(torch.zeros(0, 3, device=dev)).shape == (0, 1)


def test_bf16_trace_against_fp64_oracle(nets):
    """BF16 served tracer vs the FP64 oracle trace: hit masks and depth."""
    from oracle import cref
    net, bnet, m32, m64, _ = nets
    dev = net.features[0].fm.device
    ro, rd = synthetic.look_at_rays(width=96, height=96)
    tr = ng.SphereTracer(default_args(num_steps=128))
    rb = tr(bnet, ro.to(dev), rd.to(dev))
    bnet.check_status()
    x, t, hit, normal = dense.sphere_trace(m64, ro.numpy().astype(np.float64), rd.numpy().astype(np.float64),
                                           num_steps=128, aabb_fn=lambda o, d: tuple(
                                               v.astype(np.float64) if v.dtype != bool else v
                                               for v in cref.aabb(o.astype(np.float32), d.astype(np.float32))))
    h = rb.hit.cpu().numpy()
    assert hit.sum() > 1500
    assert (h == hit).mean() > 0.995
    both = h & hit
    err = np.abs(rb.depth.cpu().numpy()[both] - t[both])
    print(f"bf16 trace depth error vs fp64: mean {err.mean():.2e} p99 {np.percentile(err, 99):.2e} max {err.max():.2e}")
    assert err.mean() < 1e-3 and np.percentile(err, 99) < 5e-3
    cosang = (rb.normal.cpu().numpy()[both] * normal[both]).sum(-1)
    assert np.median(cosang) > 0.999


def test_bf16_trace_matches_fp32_trace_semantics(nets):
    """Same rules as the float32 tracer: rays that start inside the box are
    hits at depth 0, misses keep x = ray_o, normals of non-hits are 0."""
    net, bnet, _, _, _ = nets
    dev = net.features[0].fm.device
    ro = torch.tensor([[0.0, 0.0, 0.0], [3.0, 3.0, 3.0], [0.0, 0.0, 4.0]], device=dev)
    rd = torch.tensor([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, -1.0]], device=dev)
    a = ng.SphereTracer(default_args(num_steps=64))
    r16 = a(bnet, ro, rd)
    r32 = a(net, ro, rd)
    assert torch.equal(r16.hit, r32.hit)
    assert r16.depth[0, 0].item() == 0.0 and torch.equal(r16.x[1], ro[1])
    assert (r16.normal[~r16.hit] == 0).all()
    assert abs(r16.depth[2, 0].item() - r32.depth[2, 0].item()) < 5e-3


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("n,chunk", [(0, 1000), (1, 1000), (9999, 1000), (300_001, 65_536), (1_048_576, 1 << 20)])
def test_host_memory_queries_equal_device_queries(nets, n, chunk, pinned):
    """sdf_host gives bitwise the device path's values, BF16 and float32
    forms: with pinned host buffers the query kernel reads and writes them
    itself; with pageable ones they go in chunks pipelined on three streams."""
    net, bnet, _, _, _ = nets
    dev = net.features[0].fm.device
    x = torch.rand(n, 3) * 2.2 - 1.1
    if pinned:
        x = x.pin_memory()
    out16 = torch.empty(n, 1, pin_memory=pinned)
    out32 = torch.empty(n, 1, pin_memory=pinned)
    got16 = bnet.sdf_host(x, lod=4, chunk=chunk, out=out16)
    got32 = net.sdf_host(x, lod=3, chunk=chunk, out=out32)
    torch.cuda.synchronize()
    bnet.check_status()
    assert got16.shape == (n, 1) and got32.shape == (n, 1)
    assert torch.equal(got16, bnet.sdf(x.to(dev), lod=4).cpu())
    with torch.no_grad():
        assert torch.equal(got32, net.sdf(x.to(dev), lod=3).cpu())
    if n:
        with pytest.raises(RuntimeError, match="CPU tensor"):
            bnet.sdf_host(x.to(dev))


def test_pair_volumes_are_built_and_give_identical_results(nets):
    """nglod_bf16_build_pairs against a torch construction of the pair layout,
    and queries through pair volumes equal to queries through the vertex
    volumes bit for bit (same corner order), including points outside the
    box (border clamp) and exactly on the last vertex plane (x0 = s - 1)."""
    net, bnet, m32, _, _ = nets
    dev = net.features[0].fm.device
    assert len(bnet.pairs) == bnet.num_lods
    for g, pv in zip(bnet.grids, bnet.pairs):
        s = g.shape[-1]
        v = g[0].permute(1, 2, 3, 0)  # [z][y][x][32]
        nx = torch.cat([v[:, :, 1:], v[:, :, -1:]], dim=2)
        want = torch.stack([v.reshape(s, s, s, 4, 8), nx.reshape(s, s, s, 4, 8)], dim=4)  # [.., unit, x, 8]
        assert torch.equal(pv.reshape(s, s, s, 4, 2, 8), want)
    plain = Bf16OctreeSDF(net, pairs=False)
    assert not plain.pairs
    gen = torch.Generator().manual_seed(9)
    x = torch.rand(70001, 3, generator=gen) * 2.4 - 1.2
    x[:300] = torch.tensor([1.0, 1.0, 1.0])
    x[300:600, 0] = 1.0
    x[600:900, 1] = -1.0
    x = x.to(dev)
    for lod in range(bnet.num_lods):
        a = bnet.sdf(x, lod=lod)
        b = plain.sdf(x, lod=lod)
        assert torch.equal(a, b), (lod, (a - b).abs().max().item())
    np.testing.assert_allclose(a.cpu().numpy(), emulate(m32, x.cpu().numpy(), bnet.num_lods - 1), atol=2e-4, rtol=0)
    bnet.check_status()
    plain.check_status()


@pytest.mark.parametrize("base_lod,num_lods", [(1, 4), (3, 3), (4, 2)])
def test_staged_query_variants_equal_the_vertex_kernel(cuda, base_lod, num_lods):
    """The persistent BF16 query stages the leading vertex volumes that fit
    in shared memory (three at base_lod 1: 3^3, 5^3, 9^3; one at base_lod 3;
    none at base_lod 4) and reads the rest as pair lines; at every lod its
    results equal the vertex-volume kernel's bit for bit (same corner order
    and weights), on ragged sizes and points outside the box."""
    net = seeded_model(num_lods=num_lods, base_lod=base_lod, seed=base_lod).to(cuda)
    staged = Bf16OctreeSDF(net)
    plain = Bf16OctreeSDF(net, pairs=False)
    assert staged.pairs and not plain.pairs
    gen = torch.Generator().manual_seed(5 + base_lod)
    for n in [1, 127, 129, 513, 40_001]:
        x = (torch.rand(n, 3, generator=gen) * 2.4 - 1.2).to(cuda)
        for lod in range(num_lods):
            a = staged.sdf(x, lod=lod)
            b = plain.sdf(x, lod=lod)
            assert torch.equal(a, b), (n, lod, (a - b).abs().max().item())
    staged.check_status()
    plain.check_status()


def test_tensor_core_wait_timeout_reports_status_and_recovers(nets):
    """The error path of the bounded tensor-core wait, without a GPU fault:
    with the wait cut to a single non-blocking test (nglod_debug_mma_wait_polls
    (0)) the first product of every block is still running when tested, so
    the call reports a timeout through its status and stops after letting
    the issued product finish; the next call with the default bound runs
    normally on the same context and gives the same values as before."""
    from nglod_gb300 import _lib
    net, bnet, _, _, _ = nets
    dev = net.features[0].fm.device
    lib = _lib.load()
    x = (torch.rand(100_000, 3, generator=torch.Generator().manual_seed(4)) * 2 - 1).to(dev)
    good = bnet.sdf(x, lod=2)
    bnet.check_status()
    try:
        _lib.check(lib.nglod_debug_mma_wait_polls(0), "nglod_debug_mma_wait_polls")
        bnet.sdf(x, lod=2)
        with pytest.raises(RuntimeError, match="timed out"):
            bnet.check_status()
    finally:
        _lib.check(lib.nglod_debug_mma_wait_polls(-1), "nglod_debug_mma_wait_polls")
    again = bnet.sdf(x, lod=2)
    bnet.check_status()
    assert torch.equal(again, good)


@pytest.fixture(scope="module")
def summed(nets):
    net = nets[0]
    return Bf16OctreeSDF(net, summed=True)


def test_summed_volumes_are_the_float64_sums_rounded_once(nets, summed):
    """nglod_bf16_build_summed: every value is the float64 LOD sum at that
    vertex rounded to the nearest bf16 (within half a bf16 ulp, ties either
    way); the pair volumes are built from the summed volumes."""
    _, _, _, m64, _ = nets
    assert summed.summed and len(summed.pairs) == summed.num_lods
    for lod in range(summed.num_lods):
        want = dense.summed_volume(m64, lod)
        got = summed.grids[lod][0].float().cpu().numpy().astype(np.float64)
        assert got.shape == want.shape
        ulp = 2.0 ** (np.floor(np.log2(np.maximum(np.abs(want), 1e-30))) - 7)
        assert (np.abs(got - want) <= 0.5 * ulp * (1 + 1e-9)).all(), lod
        if lod == 0:  # LOD 0 alone: the bf16 rounding of the volume itself
            assert torch.equal(summed.grids[0], nets[1].grids[0])


@pytest.mark.parametrize("n", [1, 129, 65_536])
def test_summed_form_matches_emulation_and_fp64(nets, summed, n):
    """Queries through LOD-summed volumes (one gather per query) against
    their numpy emulation (tight) and the FP64 oracle (the per-LOD form's
    bounds), every LOD, near-surface points plus points outside the box."""
    net, bnet, m32, m64, (c, r) = nets
    dev = net.features[0].fm.device
    x = synthetic.near_surface_query(n, c, r, seed=3)
    x[: n // 8] *= 1.3
    report = {}
    for lod in range(summed.num_lods):
        got = summed.sdf(x.to(dev), lod=lod).cpu().numpy()
        np.testing.assert_allclose(got, emulate_summed(m64, x.numpy(), lod), atol=2e-4, rtol=0)
        err = np.abs(got - dense.sdf(m64, x.numpy().astype(np.float64), lod=lod))
        report[lod] = (err.max(), err.mean())
        assert err.max() < SUMMED_MAX[lod] and err.mean() < SUMMED_MEAN[lod], (lod, err.max(), err.mean())
    summed.check_status()
    print("summed bf16 error vs fp64 oracle per lod (max, mean):", report)


def test_summed_form_trace_against_fp64_oracle(nets, summed):
    """The BF16 tracer over LOD-summed volumes: same bounds against the FP64
    oracle trace as the per-LOD form."""
    from oracle import cref
    net, _, _, m64, _ = nets
    dev = net.features[0].fm.device
    ro, rd = synthetic.look_at_rays(width=96, height=96)
    rb = ng.SphereTracer(default_args(num_steps=128))(summed, ro.to(dev), rd.to(dev))
    summed.check_status()
    x, t, hit, normal = dense.sphere_trace(m64, ro.numpy().astype(np.float64), rd.numpy().astype(np.float64),
                                           num_steps=128, aabb_fn=lambda o, d: tuple(
                                               v.astype(np.float64) if v.dtype != bool else v
                                               for v in cref.aabb(o.astype(np.float32), d.astype(np.float32))))
    h = rb.hit.cpu().numpy()
    assert (h == hit).mean() > 0.995
    both = h & hit
    err = np.abs(rb.depth.cpu().numpy()[both] - t[both])
    assert err.mean() < 1e-3 and np.percentile(err, 99) < 5e-3
