"""torch.autograd.Function over the hand-written training kernels.

``sdf_train(net, x, lod, all_lods)`` is what ``OctreeSDF.sdf`` calls when
autograd needs gradients: forward ``nglod_sdf_fwd_train`` saves the per-LOD
feature sums, backward ``nglod_sdf_bwd`` produces the gradients of every
volume and decoder that the requested predictions depend on (and of x when x
requires grad), replacing autograd through F.grid_sample and nn.Linear
(sdf-net/lib/models/OctreeSDF.py:94-155).
"""
import ctypes

import torch

from . import _lib
from .octree_sdf import CL3D, _as_cl3d, param_list


def _model_from_params(net, fms, decs):
    m = _lib.DenseModel()
    m.num_lods = net.num_lods
    m.base_lod = net.base_lod
    m.feature_dim = net.fdim
    m.hidden_dim = net.hidden_dim
    m.grid_dtype = _lib.F32
    m.grid[:len(fms)] = [fm.data_ptr() for fm in fms]
    k = len(decs)
    m.w0[:k] = [d[0].data_ptr() for d in decs]
    m.b0[:k] = [d[1].data_ptr() for d in decs]
    m.w1[:k] = [d[2].data_ptr() for d in decs]
    m.b1[:k] = [d[3].data_ptr() for d in decs]
    return m


class _SdfTrain(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, mask, net, *params):
        nl = net.num_lods
        L = mask.bit_length() - 1
        # grad mode is off here: the parameters are used and saved as they are
        fms = [_as_cl3d(p) for p in params[:nl]]
        decs = [tuple(p.contiguous() for p in params[nl + 4 * i: nl + 4 * i + 4]) for i in range(nl)]
        xd = x.detach().float().contiguous()
        n = xd.shape[0]
        dev = xd.device
        # the forward writes every row in the mask; rows outside it stay zero
        alloc = torch.empty if mask == (1 << (L + 1)) - 1 else torch.zeros
        preds = alloc(L + 1, n, 1, device=dev, dtype=torch.float32)
        feats = torch.empty(L + 1, n, net.fdim, device=dev, dtype=torch.float32)
        # ReLU masks of the forward: the tensor-core backward (hidden_dim 128) takes them as the
        # ReLU derivative; other widths recompute the hidden layer
        relu = (torch.empty(L + 1, n, net.hidden_dim // 32, device=dev, dtype=torch.int32)
                if net.hidden_dim == 128 else None)
        m = _model_from_params(net, fms, decs)
        _lib.check(_lib.load().nglod_sdf_fwd_train(m, _lib.ptr(xd), n, mask, _lib.ptr(preds), _lib.ptr(feats),
                                                   _lib.ptr(relu), _lib.stream_ptr(dev)), "nglod_sdf_fwd_train")
        ctx.relu = relu
        ctx.save_for_backward(xd, feats, *fms, *[p for d in decs for p in d])
        ctx.mask = mask
        ctx.net = net
        ctx.L = L
        ctx.x_needs_grad = x.requires_grad
        return preds

    @staticmethod
    def backward(ctx, grad_preds):
        net = ctx.net
        nl = net.num_lods
        L = ctx.L
        saved = ctx.saved_tensors
        xd, feats = saved[0], saved[1]
        fms = saved[2:2 + nl]
        flat = saved[2 + nl:]
        decs = [tuple(flat[4 * i: 4 * i + 4]) for i in range(nl)]
        n = xd.shape[0]
        dev = xd.device
        gp = grad_preds.detach().float().contiguous()
        m = _model_from_params(net, fms, decs)
        g = _lib.DenseGrads()
        gfm = [None] * nl
        gdec = [[None] * 4 for _ in range(nl)]
        for i in range(L + 1):
            gfm[i] = torch.empty_like(fms[i], memory_format=CL3D)
            g.grid[i] = gfm[i].data_ptr()
            if (ctx.mask >> i) & 1:
                gdec[i] = [torch.empty_like(p) for p in decs[i]]
                g.w0[i], g.b0[i], g.w1[i], g.b1[i] = [t.data_ptr() for t in gdec[i]]
        dfeat = torch.empty_like(feats)
        gx = torch.empty(n, 3, device=dev, dtype=torch.float32) if ctx.x_needs_grad else None
        # the kernels add into the gradient buffers: zero them in a few multi-tensor launches
        torch._foreach_zero_([t for t in gfm[:L + 1]] + [t for d in gdec for t in d if t is not None] +
                             ([gx] if gx is not None else []))
        _lib.check(_lib.load().nglod_sdf_bwd(m, _lib.ptr(xd), n, ctx.mask, _lib.ptr(gp), _lib.ptr(feats),
                                             _lib.ptr(ctx.relu), _lib.ptr(dfeat), g, _lib.ptr(gx),
                                             _lib.stream_ptr(dev)), "nglod_sdf_bwd")
        ctx.relu = None
        out = [gx, None, None] + gfm + [t for d in gdec for t in d]
        return tuple(out)


def train_params(net):
    """The parameters the training kernels take, in their order
    (octree_sdf.param_list)."""
    return param_list(net)


def sdf_train_stacked(net, x):
    """Differentiable predictions of every LOD as one [num_lods, N, 1] tensor
    (the rows sdf_train(net, x, None, True) returns as a list)."""
    _lib.require_cuda(x, net.features[0].fm)
    if x.dim() != 2 or x.shape[1] != 3:
        raise NotImplementedError("OctreeSDF.sdf: only [N, 3] query points are supported")
    return _SdfTrain.apply(x, (1 << net.num_lods) - 1, net, *train_params(net))


def sdf_train(net, x, lod, all_lods):
    """Differentiable predictions: [N, 1] at `lod` (finest if None), or the
    list of every LOD's [N, 1] when all_lods."""
    _lib.require_cuda(x, net.features[0].fm)
    if x.dim() != 2 or x.shape[1] != 3:
        raise NotImplementedError("OctreeSDF.sdf: only [N, 3] query points are supported")
    L = net.num_lods - 1 if lod is None else lod
    mask = ((1 << (L + 1)) - 1) if all_lods else (1 << L)
    preds = _SdfTrain.apply(x, mask, net, *train_params(net))
    if all_lods:
        return [preds[i] for i in range(L + 1)]
    return preds[L]


def check_backward_status():
    """Raises if a bounded tensor-core wait of the training forward or
    backward since the last check gave up (its predictions or gradients
    would be incomplete).  Synchronises the device (nglod_train_status)."""
    v = ctypes.c_int32(0)
    _lib.check(_lib.load().nglod_train_status(ctypes.byref(v)), "nglod_train_status")
    if v.value:
        raise RuntimeError("nglod_sdf_fwd_train / nglod_sdf_bwd: a bounded tensor-core wait timed out; "
                           "results are incomplete")
