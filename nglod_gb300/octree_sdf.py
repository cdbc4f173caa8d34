"""Drop-in ``OctreeSDF`` / ``FeatureVolume`` backed by the nglod_gb300 kernels.

Mirrors sdf-net/lib/models/OctreeSDF.py:38-155, BaseLOD.py:31-46 and
BaseSDF.py:32-73: same constructor (``OctreeSDF(args)``), same attributes
(``lod``, ``num_lods``, ``features[i].fm``, ``louts[i]``, ``loss_preds``),
same state_dict keys and shapes (``features.{i}.fm`` [1, C, s, s, s],
``louts.{i}.{0,2}.{weight,bias}``) and the same random initialisation order,
so a seeded construction gives the reference's weights.

Differences that are layout only: every ``fm`` Parameter is stored
``torch.channels_last_3d`` (its shape is unchanged), so the 32 channels of a
grid vertex are contiguous for the gather kernels.  Options the reference
implements outside the hot path (positional / Fourier encoding,
``pos_invariant``, ``joint_decoder``, ``interpolate`` -- whose reference path
raises NameError at OctreeSDF.py:138) raise NotImplementedError.
"""
import ctypes

import torch
import torch.nn as nn

from . import _lib

CL3D = torch.channels_last_3d


def setparam(args, param, paramstr):
    """Argument bridge of sdf-net/lib/utils.py:33-38."""
    argsparam = getattr(args, paramstr, None)
    if param is not None or argsparam is None:
        return param
    return argsparam


def _as_cl3d(t):
    return t if t.is_contiguous(memory_format=CL3D) else t.contiguous(memory_format=CL3D)


def param_list(net):
    """features.{i}.fm, then louts.{i}.{0,2}.{weight,bias} of every LOD, read
    from the modules' parameter tables (nn.Sequential indexing and
    Module.__getattr__ cost more host time than the rest of a call's launch
    path)."""
    ps = [fv._parameters["fm"] for fv in net.features._modules.values()]
    for dec in net.louts._modules.values():
        l0, l2 = dec._modules["0"]._parameters, dec._modules["2"]._parameters
        ps += [l0["weight"], l0["bias"], l2["weight"], l2["bias"]]
    return ps


class FeatureVolume(nn.Module):
    """Feature grid of (fsize+1)^3 vertices x fdim channels (OctreeSDF.py:38-57)."""

    def __init__(self, fdim, fsize):
        super().__init__()
        self.fsize = fsize
        self.fdim = fdim
        fm = torch.randn(1, fdim, fsize + 1, fsize + 1, fsize + 1) * 0.01
        self.fm = nn.Parameter(fm.contiguous(memory_format=CL3D))
        self.sparse = None

    def forward(self, x):
        """Trilinear sample at x [N, 3]: [N, fdim] (grid_sample, border, align_corners)."""
        _lib.require_cuda(x, self.fm)
        if x.dim() != 2 or x.shape[1] != 3:
            raise NotImplementedError("FeatureVolume: only [N, 3] query points are supported")
        x = x.detach().float().contiguous()
        fm = _as_cl3d(self.fm.detach())
        out = torch.empty(x.shape[0], self.fdim, device=x.device, dtype=torch.float32)
        _lib.check(_lib.load().nglod_volume_sample(_lib.ptr(fm), self.fsize + 1, self.fdim, _lib.ptr(x),
                                                   x.shape[0], _lib.ptr(out), _lib.stream_ptr(x.device)),
                   "nglod_volume_sample")
        return out


class OctreeSDF(nn.Module):
    """Neural SDF with a pyramid of feature volumes and one decoder per LOD."""

    def __init__(self, args, init=None):
        super().__init__()
        # BaseSDF.__init__ (BaseSDF.py:33-58)
        self.args = args
        self.pos_enc = setparam(args, None, "pos_enc")
        self.ff_dim = setparam(args, None, "ff_dim")
        self.ff_width = setparam(args, None, "ff_width")
        self.input_dim = 3
        self.out_dim = 1
        if self.ff_dim is not None and self.ff_dim > 0:
            raise NotImplementedError("Fourier-feature encoding is outside the nglod_gb300 path")
        if self.pos_enc:
            raise NotImplementedError("positional encoding is outside the nglod_gb300 path")
        # BaseLOD.__init__ (BaseLOD.py:33-35)
        self.num_lods = args.num_lods
        self.lod = None
        # OctreeSDF.__init__ (OctreeSDF.py:60-88)
        self.fdim = args.feature_dim
        self.fsize = getattr(args, "feature_size", 4)
        self.hidden_dim = args.hidden_dim
        self.pos_invariant = getattr(args, "pos_invariant", False)
        if self.pos_invariant:
            raise NotImplementedError("pos_invariant decoders are outside the nglod_gb300 path")
        self.base_lod = args.base_lod
        self.features = nn.ModuleList([FeatureVolume(self.fdim, 2 ** (i + self.base_lod))
                                       for i in range(self.num_lods)])
        self.interpolate = getattr(args, "interpolate", None)
        if self.interpolate is not None:
            raise NotImplementedError("LOD interpolation is outside the nglod_gb300 path "
                                      "(the reference's own path raises NameError, OctreeSDF.py:138)")
        self.sdf_input_dim = self.fdim + self.input_dim
        if getattr(args, "joint_decoder", False):
            raise NotImplementedError("joint_decoder is outside the nglod_gb300 path")
        self.num_decoder = self.num_lods
        self.louts = nn.ModuleList([
            nn.Sequential(nn.Linear(self.sdf_input_dim, self.hidden_dim, bias=True), nn.ReLU(),
                          nn.Linear(self.hidden_dim, 1, bias=True))
            for _ in range(self.num_decoder)])
        self.loss_preds = None

    # -- reference API --------------------------------------------------------
    def encode(self, x):
        return x

    def forward(self, x, lod=None):
        """BaseLOD.forward (BaseLOD.py:37-41): the ``lod`` argument is ignored,
        ``self.lod`` selects the LOD."""
        if lod is None:
            lod = self.lod
        x = self.encode(x)
        return self.sdf(x)

    def freeze(self):
        for _, v in self.named_parameters():
            v.requires_grad_(False)

    def sdf(self, x, lod=None, return_lst=False):
        """OctreeSDF.sdf (OctreeSDF.py:94-155) on the fused CUDA kernels.

        Returns [N, 1] at ``lod`` (0 <= lod < num_lods); otherwise the finest
        prediction, or the list of every LOD's [N, 1] with ``return_lst``.
        Differentiable in the features and decoder weights when autograd
        needs it.  Both forms gather and sum the features in float32 and, at
        hidden width 128, run the decoder's first layer on the tensor cores as
        split-TF32 products (relative error about 2^-21, float32's own size);
        the training form takes its ReLU decisions near zero in float32.
        ``check_status()`` reports a bounded tensor-core wait that gave up.
        """
        if lod is None:
            lod = self.lod
        in_range = lod is not None and 0 <= lod < self.num_lods
        # The reference returns at `lod` before the list is complete; otherwise
        # it evaluates every LOD, keeps the list in training mode and returns
        # the list or its last entry.
        all_lods = (not in_range) and (return_lst or self.training)
        need_grad = torch.is_grad_enabled() and (
            any(p.requires_grad for p in self.parameters()) or x.requires_grad)
        if need_grad:
            from .autograd import sdf_train
            preds = sdf_train(self, x, lod if in_range else None, all_lods)
        else:
            preds = self._sdf_infer(x, lod if in_range else None, all_lods)
        if not all_lods:
            return preds
        if self.training:
            self.loss_preds = preds
        return preds if return_lst else preds[-1]

    @torch.no_grad()
    def sdf_host(self, x_host, lod=None, out=None, chunk=1 << 19):
        """Inference sdf of points in host memory ([n, 3] float32) into host
        memory ([n, 1], returned; pinned when allocated here) through
        nglod_sdf_fwd_host: pinned points and results are read and written by
        the query kernel itself over the host link, other host memory goes
        in chunks pipelined on three streams joined into the current one.
        The result is complete once the current stream's work is."""
        if lod is None:
            lod = self.lod
        if x_host.is_cuda or x_host.dtype != torch.float32 or not x_host.is_contiguous():
            raise RuntimeError("sdf_host takes a contiguous float32 CPU tensor (use sdf for device tensors)")
        n = x_host.shape[0]
        if out is None:
            out = torch.empty(n, 1, pin_memory=True)
        dev = self.features[0].fm.device
        _lib.require_cuda(self.features[0].fm)
        nbytes = int(_lib.load().nglod_host_query_scratch_bytes(chunk))
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        m = self.dense_model()
        in_range = lod is not None and 0 <= lod < self.num_lods
        _lib.check(_lib.load().nglod_sdf_fwd_host(m, _lib.ptr(x_host), n, lod if in_range else -1, _lib.ptr(out), chunk,
                                                  _lib.ptr(scratch), _lib.stream_ptr(dev)), "nglod_sdf_fwd_host")
        return out

    # -- kernel plumbing ------------------------------------------------------
    def dense_model(self):
        """The ``nglod_dense_model`` descriptor of the current parameters."""
        m = _lib.DenseModel()
        m.num_lods = self.num_lods
        m.base_lod = self.base_lod
        m.feature_dim = self.fdim
        m.hidden_dim = self.hidden_dim
        m.grid_dtype = _lib.F32
        keep = []
        nl = self.num_lods
        ps = param_list(self)
        grids = []
        for fm in ps[:nl]:
            if fm.dtype != torch.float32:
                raise RuntimeError("nglod_gb300 float32 path: parameters must be float32")
            if not fm.is_contiguous(memory_format=CL3D):
                fm = _as_cl3d(fm.detach())
                keep.append(fm)
            grids.append(fm.data_ptr())
        ws = []
        for w in ps[nl:]:
            if not w.is_contiguous():
                w = w.detach().contiguous()
                keep.append(w)
            ws.append(w.data_ptr())
        m.grid[:nl] = grids
        m.w0[:nl] = ws[0::4]
        m.b0[:nl] = ws[1::4]
        m.w1[:nl] = ws[2::4]
        m.b1[:nl] = ws[3::4]
        m._keep = keep
        return m

    def check_status(self):
        """Raises if a bounded tensor-core wait of an inference call since the
        last check gave up (nglod_dense_status; reading it synchronises)."""
        st = ctypes.c_int32(0)
        _lib.check(_lib.load().nglod_dense_status(ctypes.byref(st)), "nglod_dense_status")
        if st.value != 0:
            raise RuntimeError("nglod_sdf_fwd: a bounded tensor-core wait timed out")

    def _sdf_infer(self, x, lod, all_lods, simt=False):
        """Forward kernel without autograd: [N, 1], or [num_lods] list of [N, 1].
        simt: the per-thread float32 decoder even where the tensor-core form
        applies (nglod_sdf_fwd_simt)."""
        _lib.require_cuda(x, self.features[0].fm)
        if x.dim() != 2 or x.shape[1] != 3:
            raise NotImplementedError("OctreeSDF.sdf: only [N, 3] query points are supported")
        x = x.detach().float().contiguous()
        n = x.shape[0]
        m = self.dense_model()
        if all_lods:
            out = torch.empty(self.num_lods, n, 1, device=x.device, dtype=torch.float32)
        else:
            out = torch.empty(n, 1, device=x.device, dtype=torch.float32)
        fn = _lib.load().nglod_sdf_fwd_simt if simt else _lib.load().nglod_sdf_fwd
        _lib.check(fn(m, _lib.ptr(x), n, -1 if lod is None else lod, 1 if all_lods else 0, _lib.ptr(out),
                      _lib.stream_ptr(x.device)), "nglod_sdf_fwd")
        return list(out.unbind(0)) if all_lods else out
