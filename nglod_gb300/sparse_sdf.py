"""Sparse neural SDF on an SPC octree: sol-renderer's ``SDF`` class.

    SparseSDF.from_dense(net, spc)   SOL_NGLOD export (sdf-net/lib/models/SOL_NGLOD.py:31-75)
                                     + SDF::loadWeights/initTrinkets (sol-renderer/SDF.cu:65-216)
    SparseSDF.from_npz(path)         SDF::loadWeights from the reference's .npz
    SparseSDF.save_npz(path)         SOL_NGLOD.save (SOL_NGLOD.py:80-100), same keys
    SparseSDF.forward(x, lod)        SDF::forward (declared in SDF.h:52-54, never defined there)
    SparseSDF.sphereTrace(...)       SDF::sphereTrace (SDF.cu:297-472) incl. getNormal (218-295)
    SparseSDF.render(ray_o, ray_d, lod)   the headless frame of sdfRenderer.cpp:217-229:
                                     spc_raytrace -> first-nugget flags -> sphereTrace

LOD i lives on octree level i + 2.  Corner features are stored float32
(``precision='fp16'`` rounds them through float16 as the reference's export
does, ``'f32'`` keeps the dense values) or bfloat16 (``'bf16'``).  Decoder
weights are rounded through float16 by default, like the export.  With
bfloat16 features the sphere trace decodes on the tensor cores by default
(``decoder='tc'``: the BF16 decoder tile of the dense BF16 form,
nglod_sparse_trace_tc); ``decoder='f32'`` keeps the reference's float32
decoder arithmetic.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .spc import SPC, mark_first, spc_raytrace

MAX_LEVELS = 16
SparseModel = _lib.SparseModel


def _u(t):
    return ctypes.c_void_p(t.data_ptr())


class SparseSDF:
    def __init__(self, spc, corner_feats, corner_idx, parent, corner_counts, decoders, feat_dtype, decoder=None,
                 chains=True, summed=False):
        """chains (tensor-core decoder): also keep, per lod, every level-(lod+2)
        voxel's corner indices of all its ancestors in one row
        (nglod_sparse_build_chain), which the tensor-core trace reads instead
        of walking the parent links; results are identical.

        summed: corner_feats hold LOD-summed features (from_dense(summed=
        True)), and a query at lod samples its level-(lod+2) voxel alone."""
        if decoder is None:
            decoder = "tc" if feat_dtype == _lib.BF16 else "f32"
        if decoder not in ("tc", "f32") or (decoder == "tc" and feat_dtype != _lib.BF16):
            raise ValueError("decoder must be 'f32', or 'tc' with bf16 corner features")
        self.decoder = decoder
        self.spc = spc
        self.corner_feats = corner_feats
        self.corner_idx = corner_idx
        self.parent = parent
        self.corner_counts = list(corner_counts)
        self.decoders = decoders  # list of (w0 [H,35], b0 [H], w1 [1,H], b1 [1]) float32 on device
        self.feat_dtype = feat_dtype
        self.summed = bool(summed)
        self.num_lods = len(decoders)
        self.hidden_dim = decoders[0][0].shape[0]
        self.tiles = []
        if decoder == "tc":
            from .bf16 import pack_decoder_tile
            dev = corner_feats.device
            self.tiles = [pack_decoder_tile(w0, b0).to(dev) for w0, b0, _, _ in decoders]
        self._status = torch.zeros(1, dtype=torch.int32, device=corner_feats.device)
        self._m = self._descriptor()
        self.chains = []
        if decoder == "tc" and chains and not self.summed:
            self._build_chains()

    def _build_chains(self):
        dev = self.corner_feats.device
        pyr = self.spc.GetPyramid()
        lib = _lib.load()
        for lod in range(self.num_lods):
            cnt = int(pyr[1, lod + 3] - pyr[1, lod + 2])
            ch = torch.empty(max(cnt, 1), lod + 1, 8, dtype=torch.int32, device=dev)
            _lib.check(lib.nglod_sparse_build_chain(self._m, lod, cnt, _u(ch), _lib.stream_ptr(dev)),
                       "nglod_sparse_build_chain")
            self.chains.append(ch)
            self._m.corner_chain[lod] = ch.data_ptr()

    # -- construction ----------------------------------------------------------
    @classmethod
    def from_dense(cls, net, spc, precision="fp16", half_weights=True, decoder=None, summed=False):
        """Corner features of every occupied voxel of octree levels 2..num_lods+1
        taken from net's feature volumes, and net's decoders.

        summed: take them from net's LOD-summed volumes instead
        (nglod_build_summed_volume: the sum of the samples of volumes 0..l at
        LOD l's vertices, float64, one float32 rounding), so that a query at
        lod samples the corners of its level-(lod+2) voxel alone: each
        ancestor voxel contains the point, so the ancestors' samples that the
        reference adds (sparse_grid_sample.cuh:52-107) are already in the
        corner values, up to rounding."""
        if precision not in ("fp16", "f32", "bf16"):
            raise ValueError("precision must be 'fp16', 'f32' or 'bf16'")
        dev = spc.GetOctree().device
        vols = []
        dm = net.dense_model() if summed else None
        for i, fv in enumerate(net.features):
            if summed:
                _lib.require_cuda(fv.fm)
                v = torch.empty_like(fv.fm, dtype=torch.float32, memory_format=torch.channels_last_3d)
                _lib.check(_lib.load().nglod_build_summed_volume(dm, i, _lib.F32, v.data_ptr(),
                                                                 _lib.stream_ptr(fv.fm.device)),
                           "nglod_build_summed_volume")
                v = v.to(dev)
            else:
                v = fv.fm.detach().to(dev).float()
            if precision == "fp16":
                v = v.half().float()
            vols.append(v.contiguous(memory_format=torch.channels_last_3d))
        decs = []
        for dec in net.louts:
            ws = [dec[0].weight, dec[0].bias, dec[2].weight, dec[2].bias]
            ws = [w.detach().to(dev).float() for w in ws]
            if half_weights:
                ws = [w.half().float() for w in ws]
            decs.append(tuple(w.contiguous() for w in ws))
        return cls._build(spc, vols, decs, net.base_lod, _lib.BF16 if precision == "bf16" else _lib.F32, decoder,
                          summed)

    @classmethod
    def _build(cls, spc, vols, decs, base_lod, feat_dtype, decoder=None, summed=False):
        nl = len(vols)
        dev = spc.GetOctree().device
        level = spc.GetLevel()
        if level < nl + 1:
            raise ValueError(f"octree of level {level} cannot hold {nl} LODs (needs level >= {nl + 1})")
        dm = _lib.DenseModel()
        dm.num_lods, dm.base_lod, dm.feature_dim, dm.hidden_dim = nl, base_lod, vols[0].shape[1], decs[0][0].shape[0]
        dm.grid_dtype = _lib.F32
        for i, v in enumerate(vols):
            dm.grid[i] = v.data_ptr()
            dm.w0[i], dm.b0[i], dm.w1[i], dm.b1[i] = [t.data_ptr() for t in decs[i]]
        psize = spc.GetPoints().shape[0]
        pyr = spc.GetPyramid()
        npts = int(pyr[1, nl + 2]) - int(pyr[1, 2])
        cap = 8 * npts + 64
        elem = 4 if feat_dtype == _lib.F32 else 2
        feats = torch.empty(cap * 32 * elem // 4 + 4, dtype=torch.float32, device=dev)
        corner_idx = torch.full((psize, 8), -1, dtype=torch.int32, device=dev)
        parent = torch.full((psize,), -1, dtype=torch.int32, device=dev)
        lib = _lib.load()
        nbytes = lib.nglod_sparse_build_scratch_bytes(nl + 1)
        scratch = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        off = (-scratch.data_ptr()) % 256
        counts = (ctypes.c_int64 * nl)()
        pyr_np = np.ascontiguousarray(pyr.numpy(), dtype=np.int32)
        _lib.check(lib.nglod_sparse_build(dm, _u(spc.GetPoints()), pyr_np.ctypes.data_as(ctypes.c_void_p), level,
                                          feat_dtype, _u(feats), cap, _u(corner_idx), _u(parent), counts,
                                          ctypes.c_void_p(scratch.data_ptr() + off), _lib.stream_ptr(dev)),
                   "nglod_sparse_build")
        total = sum(counts)
        if feat_dtype == _lib.F32:
            cf = feats[:total * 32].view(total, 32).clone()
        else:
            cf = feats.view(torch.bfloat16)[:total * 32].view(total, 32).clone()
        return cls(spc, cf, corner_idx, parent, list(counts), decs, feat_dtype, decoder, summed=summed)

    @classmethod
    def from_npz(cls, path, device="cuda", precision="f32", decoder=None):
        """Load the reference's export (keys octree, cc, cf, w0, b0, w1, b1, pyramid)."""
        z = np.load(path)
        spc = SPC(torch.from_numpy(np.ascontiguousarray(z["octree"], dtype=np.uint8)).to(device))
        cc = torch.from_numpy(z["cc"].astype(np.int64)).to(device)
        cf = torch.from_numpy(z["cf"].astype(np.float32)).to(device)
        counts = [int(c) for c in z["pyramid"]]
        vols = []
        o = 0
        for i, c in enumerate(counts):
            s = 2 ** (i + 2) + 1
            v = torch.zeros(1, cf.shape[1], s, s, s, device=device)
            idx = cc[o:o + c]
            v[0, :, idx[:, 2], idx[:, 1], idx[:, 0]] = cf[o:o + c].T
            vols.append(v.contiguous(memory_format=torch.channels_last_3d))
            o += c
        decs = []
        for i in range(len(counts)):
            ws = [torch.from_numpy(z[k][i].astype(np.float32)).to(device) for k in ("w0", "b0", "w1", "b1")]
            ws[1] = ws[1].reshape(-1)
            ws[3] = ws[3].reshape(-1)
            decs.append(tuple(w.contiguous() for w in ws))
        return cls._build(spc, vols, decs, 2, _lib.BF16 if precision == "bf16" else _lib.F32, decoder)

    def corner_coords(self, lod):
        """[count, 3] corner coordinates of LOD lod, in their stored order."""
        pts = self.spc.GetLevelPoints(lod + 2)[:, :3].long()
        offs = torch.tensor([[(j >> 2) & 1, (j >> 1) & 1, j & 1] for j in range(8)], device=pts.device)
        return torch.unique((pts[:, None, :] + offs[None]).reshape(-1, 3), dim=0)

    def save_npz(self, path):
        """The reference's export format (SOL_NGLOD.save, SOL_NGLOD.py:80-100)."""
        if self.summed:
            raise ValueError("LOD-summed corner features have no place in the reference's npz format")
        cc = torch.cat([self.corner_coords(i) for i in range(self.num_lods)]).cpu().numpy().astype(np.uint8)
        cf = self.corner_feats.float().cpu().numpy().astype(np.float16)
        stack = lambda k: np.stack([self.decoders[i][k].cpu().numpy().astype(np.float16) for i in range(self.num_lods)])
        np.savez_compressed(path, octree=self.spc.GetOctree().cpu().numpy(), cc=cc, cf=cf, w0=stack(0),
                            b0=stack(1), w1=stack(2), b1=stack(3), pyramid=np.array(self.corner_counts))

    def _descriptor(self):
        m = SparseModel()
        m.num_lods = self.num_lods
        m.feature_dim = self.corner_feats.shape[1]
        m.hidden_dim = self.hidden_dim
        m.feat_dtype = self.feat_dtype
        m.corner_feats = self.corner_feats.data_ptr()
        m.corner_idx = self.corner_idx.data_ptr()
        m.parent = self.parent.data_ptr()
        m.points = self.spc.GetPoints().data_ptr()
        pyr = self.spc.GetPyramid()
        for l in range(min(pyr.shape[1], MAX_LEVELS)):
            m.level_start[l] = int(pyr[1, l])
        for i, (w0, b0, w1, b1) in enumerate(self.decoders):
            m.w0[i], m.b0[i], m.w1[i], m.b1[i] = w0.data_ptr(), b0.data_ptr(), w1.data_ptr(), b1.data_ptr()
        for i, tile in enumerate(self.tiles):
            m.w0_tile[i] = tile.data_ptr()
        m.summed = int(self.summed)
        return m

    def check_status(self):
        """Raises if a bounded tensor-core wait of the tensor-core trace gave up."""
        if int(self._status.item()) != 0:
            raise RuntimeError("nglod_sparse_trace_tc: a bounded tensor-core wait timed out")

    # -- evaluation ---------------------------------------------------------------
    def forward(self, x, lod):
        """Sparse SDF [N, 1] at lod; NaN where x lies in no occupied voxel."""
        _lib.require_cuda(x)
        x = x.float().contiguous()
        out = torch.empty(x.shape[0], 1, device=x.device)
        _lib.check(_lib.load().nglod_sparse_query(self._m, _u(self.spc.GetOctree()), _u(self.spc.GetPrefix()), lod,
                                                  _u(x), x.shape[0], _u(out), _lib.stream_ptr(x.device)),
                   "nglod_sparse_query")
        return out

    def sphereTrace(self, ray_o, ray_d, nuggets, points=None, info=None, lod=None, num_steps=50):
        """[x, t, hit, normal] (SDF.cu:297-472).  ``points`` and ``info`` are
        accepted for signature compatibility; the voxel table and the first
        nugget of each ray are derived from the model and the nuggets."""
        if lod is None:
            lod = self.num_lods - 1
        _lib.require_cuda(ray_o, ray_d, nuggets)
        ray_o = ray_o.float().contiguous()
        ray_d = ray_d.float().contiguous()
        nuggets = nuggets.to(torch.int32).contiguous()
        n = ray_o.shape[0]
        dev = ray_o.device
        x = torch.empty(n, 3, device=dev)
        t = torch.empty(n, 1, device=dev)
        hit = torch.empty(n, dtype=torch.bool, device=dev)
        normal = torch.empty(n, 3, device=dev)
        first = torch.empty(n, dtype=torch.int32, device=dev)
        counter = torch.empty(1, dtype=torch.int64, device=dev)
        if self.decoder == "tc":
            _lib.check(_lib.load().nglod_sparse_trace_tc(self._m, lod, num_steps, _u(ray_o), _u(ray_d), n,
                                                         _u(nuggets), nuggets.shape[0], _u(first), _u(x), _u(t),
                                                         _u(hit), _u(normal), _u(counter), _u(self._status),
                                                         _lib.stream_ptr(dev)), "nglod_sparse_trace_tc")
        else:
            _lib.check(_lib.load().nglod_sparse_trace(self._m, lod, num_steps, _u(ray_o), _u(ray_d), n, _u(nuggets),
                                                      nuggets.shape[0], _u(first), _u(x), _u(t), _u(hit), _u(normal),
                                                      _u(counter), _lib.stream_ptr(dev)), "nglod_sparse_trace")
        return [x, t, hit, normal]

    def render(self, ray_o, ray_d, lod=None, num_steps=50):
        """spc_raytrace to level lod+2, then sphereTrace (sdfRenderer.cpp:227-229,
        sdfRenderer.cu:208-224)."""
        if lod is None:
            lod = self.num_lods - 1
        s = self.spc
        nug = spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), ray_o, ray_d, lod + 2, prefix=s.GetPrefix())
        info = mark_first(nug)
        return self.sphereTrace(ray_o, ray_d, nug, None, info, lod, num_steps), nug
