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
from tests.helpers import oracle_model

pytestmark = pytest.mark.gpu


def _bf16(a):
    """Round float32 array to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def emulate(m, x, lod):
    """The BF16 form's arithmetic in numpy: bf16 volumes, fp32 LOD sum rounded
    to bf16, positions as bf16 hi + lo, bf16 first-layer weights, products
    accumulated in float64, b0 / ReLU / second layer in float32."""
    x = x.astype(np.float32)
    acc = np.zeros((x.shape[0], 32), np.float32)
    for i in range(lod + 1):
        acc += dense.feature_volume(_bf16(m["fms"][i]).astype(np.float32), x)
    f = _bf16(acc)
    hi = _bf16(x)
    lo = _bf16(x - hi)
    w0 = _bf16(m["w0"][lod].astype(np.float32)).astype(np.float64)
    h = f.astype(np.float64) @ w0[:, 3:].T + hi.astype(np.float64) @ w0[:, :3].T + lo.astype(np.float64) @ w0[:, :3].T
    h = np.maximum(h.astype(np.float32) + m["b0"][lod].astype(np.float32), 0)
    return (h @ m["w1"][lod].astype(np.float32).T + m["b1"][lod].astype(np.float32))


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
        assert err.max() < 2e-2 and err.mean() < 2e-3, (lod, err.max(), err.mean())
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
    assert d.max().item() < 2e-2 and d.mean().item() < 2e-3
    bnet.check_status()
    assert bnet.sdf(torch.zeros(0, 3, device=dev)).shape == (0, 1)
