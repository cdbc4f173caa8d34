"""nglod_sdf_bwd_noalloc against nglod_sdf_bwd, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device
memory (a plugin whose GPU memory belongs to its host application, a process
whose allocator is locked after start-up): it takes its per-point scratch
from an array built into the library.  These tests check that it produces the
same gradients as the entry point with caller-provided scratch, on two calls
in a row with different inputs (the built-in array keeps the first call's
contents when the second starts), and that batches beyond the array's
capacity are refused.  The file name sorts last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from nglod_gb300 import _lib
from tests.helpers import seeded_model

pytestmark = pytest.mark.gpu

# Same bar as the other backward tests: max |difference| / max |gradient| (the
# two calls differ only in the order of their floating-point atomic adds).
REL_TOL = 1e-5


def _forward(net, n, mask, seed, dev):
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = (torch.rand(n, 3, generator=g) * 2.2 - 1.1).to(dev)
    L = mask.bit_length() - 1
    m = net.dense_model()
    preds = torch.zeros(L + 1, n, device=dev)
    feats = torch.empty(L + 1, n, 32, device=dev)
    relu = torch.empty(L + 1, n, 4, device=dev, dtype=torch.int32)
    lib = _lib.load()
    _lib.check(lib.nglod_sdf_fwd_train(m, _lib.ptr(x), n, mask, _lib.ptr(preds), _lib.ptr(feats), _lib.ptr(relu),
                                       _lib.stream_ptr(dev)), "nglod_sdf_fwd_train")
    gp = (torch.randn(L + 1, n, generator=g) * 1e-2).to(dev)
    return x, m, preds, feats, relu, gp


def _grad_buffers(net, mask):
    L = mask.bit_length() - 1
    g = _lib.DenseGrads()
    bufs = {}
    for i in range(L + 1):
        bufs[f"fm{i}"] = torch.zeros_like(net.features[i].fm, memory_format=torch.channels_last_3d)
        g.grid[i] = bufs[f"fm{i}"].data_ptr()
        if (mask >> i) & 1:
            lin0, lin1 = net.louts[i][0], net.louts[i][2]
            for key, p in (("w0", lin0.weight), ("b0", lin0.bias), ("w1", lin1.weight), ("b1", lin1.bias)):
                bufs[f"{key}{i}"] = torch.zeros_like(p)
                getattr(g, key)[i] = bufs[f"{key}{i}"].data_ptr()
    return g, bufs


def _run(net, x, m, feats, relu, gp, mask, noalloc):
    dev = x.device
    n = x.shape[0]
    g, bufs = _grad_buffers(net, mask)
    gx = torch.zeros(n, 3, device=dev)
    lib = _lib.load()
    if noalloc:
        st = lib.nglod_sdf_bwd_noalloc(m, _lib.ptr(x), n, mask, _lib.ptr(gp), _lib.ptr(feats), _lib.ptr(relu), g,
                                       _lib.ptr(gx), _lib.stream_ptr(dev))
    else:
        scratch = torch.empty_like(feats)
        st = lib.nglod_sdf_bwd(m, _lib.ptr(x), n, mask, _lib.ptr(gp), _lib.ptr(feats), _lib.ptr(relu),
                               _lib.ptr(scratch), g, _lib.ptr(gx), _lib.stream_ptr(dev))
    _lib.check(st, "nglod_sdf_bwd_noalloc" if noalloc else "nglod_sdf_bwd")
    torch.cuda.synchronize()
    # a bounded tensor-core wait that gave up would leave the gradients
    # incomplete: report that as such, not as a parity mismatch
    status = ctypes.c_int32(-1)
    _lib.check(lib.nglod_train_status(ctypes.byref(status)), "nglod_train_status")
    assert status.value == 0, "a tensor-core wait of the backward gave up"
    bufs["x"] = gx
    return {k: v.cpu().numpy() for k, v in bufs.items()}


@pytest.mark.parametrize("with_masks", [True, False])
def test_noalloc_backward_matches_allocating_backward_twice(cuda, with_masks):
    """with_masks: the tensor-core decoder backward (forward ReLU masks);
    without: the float32 one."""
    net = seeded_model(num_lods=5, base_lod=2, seed=21).to(cuda)
    # Two calls in a row: a large 5-LOD batch, then a smaller 3-LOD batch on
    # other points, so the second call starts from the first call's scratch.
    for n, mask, seed in [(20_000, 0b11111, 1), (7_001, 0b00111, 2)]:
        x, m, preds, feats, relu, gp = _forward(net, n, mask, seed, cuda)
        if not with_masks:
            relu = None
        want = _run(net, x, m, feats, relu, gp, mask, noalloc=False)
        got = _run(net, x, m, feats, relu, gp, mask, noalloc=True)
        assert set(got) == set(want)
        gpn = gp.cpu().numpy()
        for k in want:
            scale = np.abs(want[k]).max()
            assert scale > 0, k
            if k.startswith("b1"):
                # db1 = sum of n random-sign dLoss/dpred values: the total is
                # about sqrt(n) times smaller than the sum of its terms, so the
                # atomic-order bound is taken against the sum of |terms|
                scale = np.abs(gpn[int(k[2:])]).sum()
            err = np.abs(got[k] - want[k]).max() / scale
            assert err < REL_TOL, (n, k, err)


def test_noalloc_refuses_batches_beyond_its_array(cuda):
    net = seeded_model(num_lods=5, base_lod=2, seed=21).to(cuda)
    lib = _lib.load()
    m = net.dense_model()
    g, _ = _grad_buffers(net, 0b11111)
    n = (16 << 20) // (5 * 32 * 4) + 1  # one point more than 5 LODs x 32 floats fit in 16 MiB
    dummy = torch.zeros(4, device=cuda)
    st = lib.nglod_sdf_bwd_noalloc(m, _lib.ptr(dummy), n, 0b11111, _lib.ptr(dummy), _lib.ptr(dummy), None, g, None,
                                   _lib.stream_ptr(cuda))
    assert st == -4
    msg = lib.nglod_last_error().decode()
    assert f"at most {n - 1} points" in msg, msg
    assert isinstance(ctypes.sizeof(_lib.DenseGrads), int)
