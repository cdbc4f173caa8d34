"""Hand-written backward and Adam against the reference's autograd gradients,
FP64 central finite differences and torch.optim.Adam."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import synthetic, trainer
from nglod_gb300.autograd import check_backward_status
from oracle import dense
from tests.helpers import model_from_fixture, oracle_model, seeded_model

pytestmark = pytest.mark.gpu


def _grads(net):
    return {k: p.grad.detach().cpu().numpy() for k, p in net.named_parameters() if p.grad is not None}


def test_backward_matches_reference_autograd(golden, cuda):
    """Same loss as the fixture (Trainer.step_geometry over lods 0, 1, 2 with
    separate sdf calls); gradients vs the reference's autograd on the CPU."""
    fx = golden("dense_small")
    net = model_from_fixture(fx, 3, 1, device=cuda).train()
    x = torch.from_numpy(fx["points"]).to(cuda)
    gts = torch.from_numpy(fx["train/gts"]).to(cuda)
    net.zero_grad()
    loss = 0
    for lod in [0, 1, 2]:
        loss = loss + ((net.sdf(x, lod=lod) - gts) ** 2).sum()
    loss = loss / x.shape[0]
    loss.backward()
    assert abs(loss.item() - float(fx["train/loss"])) < 1e-5 * max(1.0, abs(float(fx["train/loss"])))
    got = _grads(net)
    for k, g in got.items():
        ref = fx["grad/" + k]
        scale = np.abs(ref).max() + 1e-12
        err = np.abs(g - ref).max() / scale
        assert err < 1e-4, (k, err)
    assert set(got) == {k[len("grad/"):] for k in fx if k.startswith("grad/")}
    check_backward_status()


def test_return_lst_backward_equals_separate_calls(cuda):
    net = seeded_model(num_lods=4, base_lod=2, seed=3).to(cuda).train()
    x = torch.rand(3000, 3, device=cuda) * 2.2 - 1.1
    gts = torch.rand(3000, 1, device=cuda) * 0.2 - 0.1
    net.zero_grad()
    preds = net.sdf(x, return_lst=True)
    trainer.l2_loss(preds, gts, [0, 1, 2, 3], x.shape[0]).backward()
    a = _grads(net)
    net.zero_grad()
    loss = sum(((net.sdf(x, lod=l) - gts) ** 2).sum() for l in range(4)) / x.shape[0]
    loss.backward()
    b = _grads(net)
    for k in a:
        scale = np.abs(b[k]).max() + 1e-12
        assert np.abs(a[k] - b[k]).max() / scale < 1e-5, k


def _fd_check(net, x, gts, lods, picks, h=1e-3):
    """Gradient entries vs FP64 central differences of the oracle loss."""
    m = oracle_model(net.cpu(), np.float64)
    xn = x.cpu().numpy().astype(np.float64)
    gn = gts.cpu().numpy().astype(np.float64)

    def loss_of(mm):
        return sum(((dense.sdf(mm, xn, lod=l) - gn) ** 2).sum() for l in lods) / xn.shape[0]

    out = []
    for name, idx in picks:
        kind, i = name.split(":")
        i = int(i)
        arr = {"fm": m["fms"], "w0": m["w0"], "b0": m["b0"], "w1": m["w1"], "b1": m["b1"]}[kind][i]
        base = arr[idx]
        arr[idx] = base + h
        lp = loss_of(m)
        arr[idx] = base - h
        lm = loss_of(m)
        arr[idx] = base
        out.append((lp - lm) / (2 * h))
    return np.array(out)


def test_backward_vs_fp64_finite_differences(cuda):
    """Gradient entries vs FP64 central differences of the oracle loss.

    With the configuration's step h = 1e-3 (10 % of a feature value) the
    stencil crosses ReLU kinks, so the difference quotient itself is off by
    up to ~2e-3 per entry; the bar there is the vector relative error
    ||g - fd|| / ||fd|| <= 1e-3.  With h = 1e-5 the FP64 quotient matches the
    exact gradient to ~1e-9 and each entry must agree to 1e-3.
    """
    net = seeded_model(num_lods=2, base_lod=2, seed=7)
    c, r = synthetic.sphere_union(1)
    x, gts = synthetic.training_batch(512, c, r, seed=3)
    net = net.to(cuda).train()
    xd, gd = x.to(cuda), gts.to(cuda)
    net.zero_grad()
    trainer.l2_loss(net.sdf(xd, return_lst=True), gd, [0, 1], 512).backward()
    grads = {"fm:0": net.features[0].fm.grad[0].cpu().numpy(), "fm:1": net.features[1].fm.grad[0].cpu().numpy(),
             "w0:1": net.louts[1][0].weight.grad.cpu().numpy(), "b0:0": net.louts[0][0].bias.grad.cpu().numpy(),
             "w1:1": net.louts[1][2].weight.grad.cpu().numpy(), "b1:0": net.louts[0][2].bias.grad.cpu().numpy()}
    rng = np.random.default_rng(0)
    picks = []
    for name, g in grads.items():
        flat = np.argsort(-np.abs(g).ravel())[:3]  # the largest entries
        for f in list(flat) + [rng.integers(g.size)]:
            picks.append((name, np.unravel_index(f, g.shape)))
    got = np.array([grads[n][i] for n, i in picks])
    fd3 = _fd_check(net, x, gts, [0, 1], picks, h=1e-3)
    assert np.linalg.norm(got - fd3) / np.linalg.norm(fd3) < 1e-3
    fd5 = _fd_check(net.to(cuda), x, gts, [0, 1], picks, h=1e-5)
    big = np.abs(fd5) > 1e-6
    assert big.sum() >= 12
    rel = np.abs(got - fd5)[big] / np.abs(fd5)[big]
    assert rel.max() < 1e-3, rel.max()
    assert np.abs(got - fd5)[~big].max(initial=0) < 1e-7


def test_grad_x_vs_finite_differences(cuda):
    net = seeded_model(num_lods=3, base_lod=2, seed=9).to(cuda).eval()
    x = (torch.rand(256, 3, device=cuda) * 1.8 - 0.9).requires_grad_(True)
    y = net.sdf(x, lod=2)
    (gx,) = torch.autograd.grad(y.sum(), x)
    m = oracle_model(net.cpu(), np.float64)
    xn = x.detach().cpu().numpy().astype(np.float64)
    # h = 1e-6 in FP64: a stencil rarely straddles a grid-cell face or a ReLU
    # kink, where the one-sided analytic derivative and the quotient differ.
    h = 1e-6
    fd = np.zeros_like(xn)
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        fd[:, k] = (dense.sdf(m, xn + e, lod=2) - dense.sdf(m, xn - e, lod=2))[:, 0] / (2 * h)
    g = gx.cpu().numpy()
    close = np.abs(g - fd) <= 2e-4 + 1e-3 * np.abs(fd)
    assert close.mean() >= 0.995, close.mean()
    assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-2


def test_fused_adam_matches_torch_adam(cuda):
    torch.manual_seed(0)
    p1 = torch.randn(1000, 37, device=cuda)
    p2 = p1.clone()
    q1 = torch.randn(5, 32, 9, 9, 9, device=cuda).contiguous(memory_format=torch.channels_last_3d)
    q2 = q1.clone()
    # a length that is not a multiple of 4, and a tensor 4 bytes off a
    # 16-byte boundary: the kernel's one-element path
    r1 = torch.randn(1001, 3, device=cuda)
    r2 = r1.clone()
    u1 = torch.randn(4001, device=cuda)[1:]
    u2 = u1.clone()
    assert u1.data_ptr() % 16 != 0
    a = trainer.FusedAdam([p1, q1, r1, u1], lr=1e-3)
    b = torch.optim.Adam([p2, q2, r2, u2], lr=1e-3, foreach=False)
    for p in (p1, p2, q1, q2, r1, r2, u1, u2):
        p.requires_grad_(True)
    for s in range(5):
        for x1, x2 in ((p1, p2), (q1, q2), (r1, r2), (u1, u2)):
            g = torch.randn_like(x1)
            x1.grad, x2.grad = g.clone(), g.clone()
        a.step()
        b.step()
    for x1, x2 in ((p1, p2), (q1, q2), (r1, r2), (u1, u2)):
        assert (x1 - x2).abs().max().item() < 1e-6


def test_training_reduces_loss(cuda):
    c, r = synthetic.sphere_union(1)
    net = seeded_model(num_lods=5, base_lod=2, seed=0).to(cuda).train()
    opt = trainer.FusedAdam(net.parameters(), lr=1e-3)
    losses = []
    for it in range(60):
        x, g = synthetic.training_batch(16384, c, r, seed=100 + it)
        losses.append(trainer.step_geometry(net, opt, x.to(cuda), g.to(cuda)).item())
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.5 * losses[0], losses[::10]


def _torch_reference_grads(net, x, gts, lods):
    """Plain PyTorch fp32 on the GPU (grid_sample + Linear + autograd, TF32
    off) of the same loss: sum over `lods` of ((sdf_l - gts)^2).sum() / n."""
    import torch.nn.functional as F
    assert not torch.backends.cuda.matmul.allow_tf32
    fms = [fv.fm.detach().clone().contiguous().requires_grad_(True) for fv in net.features]
    decs = [[p.detach().clone().requires_grad_(True) for p in (d[0].weight, d[0].bias, d[2].weight, d[2].bias)]
            for d in net.louts]
    n = x.shape[0]
    acc, loss = None, 0.0
    for i in range(max(lods) + 1):
        s = F.grid_sample(fms[i], x.reshape(1, n, 1, 1, 3), align_corners=True,
                          padding_mode="border")[0, :, :, 0, 0].transpose(0, 1)
        acc = s if acc is None else acc + s
        if i in lods:
            w0, b0, w1, b1 = decs[i]
            d = F.linear(F.relu(F.linear(torch.cat([x, acc], -1), w0, b0)), w1, b1)
            loss = loss + ((d - gts) ** 2).sum()
    (loss / n).backward()
    out = {f"features.{i}.fm": fms[i].grad for i in range(len(fms))}
    for i, d in enumerate(decs):
        for name, p in zip(("0.weight", "0.bias", "2.weight", "2.bias"), d):
            out[f"louts.{i}.{name}"] = p.grad
    return out


@pytest.mark.parametrize("hidden,lods,n", [(128, [0, 1, 2, 3, 4], 100_003), (128, [1, 3], 40_000),
                                           (128, [4], 131), (64, [0, 2, 4], 30_001)])
def test_backward_matches_torch_fp32_at_size(cuda, hidden, lods, n):
    """The backward (tensor-core decoder part at hidden 128, float32 tile
    reductions otherwise) against PyTorch fp32 autograd on the GPU, with many
    tiles per block, a ragged last tile and LOD masks with gaps.  Bar: max
    |g - ref| / max |ref| < 1e-4 per tensor (the bf16 hi / lo products are
    good to about 2^-16 relative)."""
    from nglod_gb300.options import default_args
    torch.manual_seed(5)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2, hidden_dim=hidden)).to(cuda).train()
    with torch.no_grad():
        for fv in net.features:
            fv.fm.normal_(0.0, 0.05)
    c, r = synthetic.sphere_union(1)
    x, gts = synthetic.training_batch(n, c, r, seed=11)
    x, gts = x.to(cuda), gts.to(cuda)
    ref = _torch_reference_grads(net, x, gts, lods)
    net.zero_grad()
    preds = net.sdf(x, return_lst=True)
    trainer.l2_loss(preds, gts, lods, n).backward()
    check_backward_status()
    params = dict(net.named_parameters())
    for k, want in ref.items():
        got = params[k].grad
        scale = 0.0 if want is None else want.abs().max().item()
        if scale == 0.0:
            assert got is None or got.abs().max().item() == 0.0, k
            continue
        err = (got - want).abs().max().item() / scale
        assert err < 1e-4, (k, err)


def test_fused_l2_loss_matches_autograd_loss(cuda):
    """nglod_l2_loss: the loss of l2_loss in float64 and the gradient that
    l2_loss(...).backward() gives its predictions, for a LOD subset."""
    torch.manual_seed(3)
    n = 70_001
    preds = torch.randn(5, n, 1, device=cuda, dtype=torch.float32) * 0.1
    gts = torch.randn(n, 1, device=cuda, dtype=torch.float32) * 0.1
    lods = [0, 2, 4]
    loss, grad = trainer.fused_l2_loss(preds, gts, lods)
    p = preds.clone().requires_grad_(True)
    ref = trainer.l2_loss([p[i] for i in range(5)], gts, lods, n)
    ref.backward()
    want = sum(((preds[l].double() - gts.double()) ** 2).sum() for l in lods).item() / n
    assert abs(loss.item() - want) <= 1e-12 * max(1.0, abs(want))
    assert abs(loss.item() - ref.item()) <= 1e-5 * abs(want)
    np.testing.assert_allclose(grad.cpu().numpy(), p.grad.cpu().numpy(), rtol=1e-6, atol=1e-12)
    assert (grad[1] == 0).all() and (grad[3] == 0).all()


@pytest.mark.parametrize("n,mask", [(20_001, 0b11111), (4_099, 0b10101), (77, 0b01000)])
def test_tensor_core_forward_against_fp64_decode(cuda, n, mask):
    """The training forward at hidden 128 with ReLU masks (split-TF32 products
    on tcgen05) against a float64 decode of the feature sums it saves: the
    predictions within 1e-5 of the prediction scale, and every ReLU bit equal
    to the sign of the float64 pre-activation wherever that lies beyond 1e-6
    of zero (units nearer zero are settled by a float32 evaluation, whose
    rounding may differ from float64's)."""
    from nglod_gb300 import _lib
    net = seeded_model(num_lods=5, base_lod=2, seed=8).to(cuda)
    with torch.no_grad():
        for fv in net.features:
            fv.fm.normal_(0.0, 0.05)
    g = torch.Generator(device="cpu").manual_seed(n)
    x = (torch.rand(n, 3, generator=g) * 2.2 - 1.1).to(cuda)
    L = mask.bit_length() - 1
    preds = torch.zeros(L + 1, n, device=cuda)
    feats = torch.empty(L + 1, n, 32, device=cuda)
    relu = torch.empty(L + 1, n, 4, device=cuda, dtype=torch.int32)
    lib = _lib.load()
    _lib.check(lib.nglod_sdf_fwd_train(net.dense_model(), _lib.ptr(x), n, mask, _lib.ptr(preds), _lib.ptr(feats),
                                       _lib.ptr(relu), _lib.stream_ptr(cuda)), "nglod_sdf_fwd_train")
    torch.cuda.synchronize()
    check_backward_status()
    xn = x.cpu().double().numpy()
    fn = feats.cpu().double().numpy()
    bits = relu.cpu().numpy().view(np.uint32)
    for l in range(L + 1):
        if not (mask >> l) & 1:
            continue
        lin0, lin1 = net.louts[l][0], net.louts[l][2]
        w0 = lin0.weight.detach().cpu().double().numpy()
        b0 = lin0.bias.detach().cpu().double().numpy()
        w1 = lin1.weight.detach().cpu().double().numpy()[0]
        b1 = lin1.bias.detach().cpu().double().numpy()[0]
        pre = np.concatenate([xn, fn[l]], axis=1) @ w0.T + b0
        want = np.maximum(pre, 0.0) @ w1 + b1
        got = preds[l].cpu().double().numpy()
        assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max(), l
        on = ((bits[l][:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(n, 128).astype(bool)
        settled = np.abs(pre) > 1e-6
        assert ((on == (pre > 0)) | ~settled).all(), l
        assert settled.mean() > 0.99
