"""Host-side behaviour of the drop-in API, on the CPU (no kernels launched)."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300.options import default_args
from tests.helpers import seeded_model


def test_seeded_construction_equals_reference(golden):
    """Same constructor call order as the reference, so the same seed gives the
    reference's initial weights bit for bit (OctreeSDF.py:60-88)."""
    fx = golden("dense_small")
    net = seeded_model(num_lods=3, base_lod=1, seed=0)
    sd = net.state_dict()
    ref_keys = sorted(k[len("param/"):] for k in fx if k.startswith("param/"))
    assert sorted(sd) == ref_keys
    for k in ref_keys:
        np.testing.assert_array_equal(sd[k].numpy(), fx["param/" + k])


def test_full_architecture_parameters():
    net = seeded_model()
    assert sum(p.numel() for p in net.parameters()) == 10_146_213
    for i, fv in enumerate(net.features):
        s = 2 ** (i + 2) + 1
        assert fv.fm.shape == (1, 32, s, s, s)
        assert fv.fm.is_contiguous(memory_format=torch.channels_last_3d)
    assert net.louts[4][0].weight.shape == (128, 35)


def test_training_parameter_list_and_model_descriptor():
    """The training path's parameter list (read from the modules' parameter
    tables) is the reference's parameters, in the order the autograd function
    takes them, and the kernels' model descriptor holds their addresses."""
    from nglod_gb300 import autograd
    net = seeded_model(num_lods=5, base_lod=2, seed=0)
    ps = autograd.train_params(net)
    want = [fv.fm for fv in net.features]
    for dec in net.louts:
        want += [dec[0].weight, dec[0].bias, dec[2].weight, dec[2].bias]
    assert len(ps) == len(want) == 25 and all(a is b for a, b in zip(ps, want))
    assert [id(p) for p in ps] == [id(p) for p in net.parameters()]
    fms, decs = ps[:5], [tuple(ps[5 + 4 * i: 9 + 4 * i]) for i in range(5)]
    m = autograd._model_from_params(net, fms, decs)
    assert (m.num_lods, m.base_lod, m.feature_dim, m.hidden_dim) == (5, 2, 32, 128)
    for i in range(5):
        assert m.grid[i] == fms[i].data_ptr()
        assert (m.w0[i], m.b0[i], m.w1[i], m.b1[i]) == tuple(t.data_ptr() for t in decs[i])
    for i in range(5, len(m.grid)):
        assert not m.grid[i] and not m.w0[i] and not m.b1[i]


def test_dense_model_descriptor():
    """OctreeSDF.dense_model: the volumes' and decoders' addresses per LOD, and
    contiguous copies (kept alive by the descriptor) of parameters that are
    not in the kernels' layout."""
    net = seeded_model(num_lods=3, base_lod=2, seed=1)
    w = net.louts[1][0].weight
    w.data = w.data.t().contiguous().t()  # same values, transposed strides
    fm = net.features[2].fm
    fm.data = fm.data.contiguous()  # channel-first instead of channels_last_3d
    m = net.dense_model()
    assert (m.num_lods, m.base_lod, m.feature_dim, m.hidden_dim) == (3, 2, 32, 128)
    assert len(m._keep) == 2
    wc = next(t for t in m._keep if t.dim() == 2)
    fc = next(t for t in m._keep if t.dim() == 5)
    assert torch.equal(wc, w) and wc.is_contiguous()
    assert torch.equal(fc, fm) and fc.is_contiguous(memory_format=torch.channels_last_3d)
    for i in range(3):
        dec = net.louts[i]
        assert m.grid[i] == (fc if i == 2 else net.features[i].fm).data_ptr()
        assert m.w0[i] == (wc if i == 1 else dec[0].weight).data_ptr()
        assert (m.b0[i], m.w1[i], m.b1[i]) == (dec[0].bias.data_ptr(), dec[2].weight.data_ptr(),
                                               dec[2].bias.data_ptr())
    assert not m.grid[3] and not m.w0[3]


def test_cpu_tensors_are_rejected():
    net = seeded_model(num_lods=2)
    with torch.no_grad(), pytest.raises(RuntimeError, match="CUDA tensors only"):
        net.sdf(torch.zeros(4, 3))
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        ng.sol_nglod.aabb(torch.zeros(4, 3), torch.ones(4, 3))


@pytest.mark.parametrize("opt", [dict(pos_enc=True), dict(ff_dim=8), dict(pos_invariant=True),
                                 dict(joint_decoder=True), dict(interpolate=0.5)])
def test_out_of_path_options_raise(opt):
    with pytest.raises(NotImplementedError):
        ng.OctreeSDF(default_args(num_lods=2, **opt))


def test_tracer_settings_from_args():
    a = default_args(num_steps=64, min_dis=1e-3, camera_clamp=[-5, 7])
    tr = ng.SphereTracer(a)
    assert tr.num_steps == 64 and tr.min_dis == 1e-3 and tr.camera_clamp == [-5, 7]
    tr2 = ng.SphereTracer(a, num_steps=8)
    assert tr2.num_steps == 8
    net = seeded_model(num_lods=2)
    net.lod = 1
    p = tr.trace_params(net)
    assert p.lod == 1 and p.num_steps == 64
    assert p.osc_dis == pytest.approx(3e-3, rel=1e-6)
    assert p.far_clip == 7.0
    with pytest.raises(TypeError):
        tr(torch.nn.Linear(3, 1), torch.zeros(1, 3), torch.ones(1, 3))
    with pytest.raises(NotImplementedError):
        ng.SphereTracer(a, grad_method="autodiff")(net, torch.zeros(1, 3), torch.ones(1, 3))


def test_render_buffer_concat():
    a = ng.RenderBuffer(x=torch.zeros(2, 3), hit=torch.ones(2, dtype=torch.bool))
    b = ng.RenderBuffer(x=torch.ones(3, 3), depth=torch.ones(3, 1))
    c = a + b
    assert c.x.shape == (5, 3) and c.hit.shape == (2,) and c.depth.shape == (3, 1)
    assert c.normal is None


def test_default_args_rejects_unknown():
    with pytest.raises(KeyError):
        default_args(not_an_option=1)
