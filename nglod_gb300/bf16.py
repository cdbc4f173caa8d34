"""BF16 form of the dense OctreeSDF: bf16 feature volumes, tcgen05 decoder.

``Bf16OctreeSDF(net)`` snapshots a float32 ``OctreeSDF`` for inference:
volumes converted to bf16 (channel-last), each decoder's first layer packed
once into the bf16 tensor-core tile layout (``nglod_bf16_pack_decoder``),
b0 / w1 / b1 kept in float32.  ``sdf(x, lod)`` has the semantics of
OctreeSDF.sdf(x, lod) (sdf-net/lib/models/OctreeSDF.py:94-146) with bf16
storage and bf16 x bf16 -> fp32 products (b0 enters the product as a bf16
hi + lo pair); its error against the FP64 oracle
is measured per LOD by tests/test_bf16_gpu.py and bench.py.  Point queries
read pair volumes (every vertex beside its +x neighbour, 128-byte lines;
``pairs=False`` keeps only the vertex volumes), with identical results.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def pack_decoder_tile(w0, b0):
    """w0 [128, 35], b0 [128] float32 -> uint8 [12288] tile (host pack through the C ABI)."""
    w = np.ascontiguousarray(w0.detach().cpu().numpy(), dtype=np.float32)
    b = np.ascontiguousarray(b0.detach().cpu().numpy(), dtype=np.float32)
    out = np.zeros(_lib.BF16_TILE_BYTES, dtype=np.uint8)
    _lib.check(_lib.load().nglod_bf16_pack_decoder(w.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                                                   w.shape[0], w.shape[1], out.ctypes.data_as(ctypes.c_void_p)),
               "nglod_bf16_pack_decoder")
    return torch.from_numpy(out)


class Bf16OctreeSDF:
    """pairs: also keep each volume as a pair volume (every vertex beside
    its +x neighbour, nglod_bf16_build_pairs; twice the volume bytes), which
    point queries read with whole 128-byte lines; results are identical.

    summed: keep LOD-summed volumes instead of the per-LOD ones
    (nglod_build_summed_volume): volume l holds, at each of LOD l's vertices,
    the sum of the trilinear samples of volumes 0..l there, in float64
    rounded once to bf16.  Each cell of LOD l lies inside one cell of every
    coarser grid, so sampling volume l alone gives the running feature sum
    up to rounding, and a query at lod L gathers one volume instead of
    L + 1.  Same memory as the per-LOD volumes; a different bf16 rounding of
    the same features (one rounding of the sum instead of one per LOD)."""

    def __init__(self, net, pairs=True, summed=False):
        _lib.require_cuda(net.features[0].fm)
        dev = net.features[0].fm.device
        self.num_lods = net.num_lods
        self.base_lod = net.base_lod
        self.lod = net.lod
        self.summed = bool(summed)
        if self.summed:
            dm = net.dense_model()
            self.grids = []
            for i, fv in enumerate(net.features):
                g = torch.empty_like(fv.fm, dtype=torch.bfloat16, memory_format=torch.channels_last_3d)
                _lib.check(_lib.load().nglod_build_summed_volume(dm, i, _lib.BF16, g.data_ptr(),
                                                                 _lib.stream_ptr(dev)), "nglod_build_summed_volume")
                self.grids.append(g)
        else:
            self.grids = [fv.fm.detach().to(torch.bfloat16).contiguous(memory_format=torch.channels_last_3d)
                          for fv in net.features]
        self.tiles, self.b0, self.w1, self.b1 = [], [], [], []
        for dec in net.louts:
            self.tiles.append(pack_decoder_tile(dec[0].weight, dec[0].bias).to(dev))
            self.b0.append(dec[0].bias.detach().float().contiguous())
            self.w1.append(dec[2].weight.detach().float().reshape(-1).contiguous())
            self.b1.append(dec[2].bias.detach().float().contiguous())
        m = _lib.Bf16Model()
        m.num_lods, m.base_lod, m.feature_dim, m.hidden_dim = self.num_lods, self.base_lod, net.fdim, net.hidden_dim
        for i in range(self.num_lods):
            m.grid[i] = self.grids[i].data_ptr()
            m.w0_tile[i] = self.tiles[i].data_ptr()
            m.b0[i], m.w1[i], m.b1[i] = self.b0[i].data_ptr(), self.w1[i].data_ptr(), self.b1[i].data_ptr()
        self.pairs = []
        if pairs:
            lib = _lib.load()
            for i, g in enumerate(self.grids):
                s = g.shape[-1]
                pv = torch.empty(s, s, s, 2, g.shape[1], dtype=torch.bfloat16, device=dev)
                _lib.check(lib.nglod_bf16_build_pairs(g.data_ptr(), s, pv.data_ptr(), _lib.stream_ptr(dev)),
                           "nglod_bf16_build_pairs")
                self.pairs.append(pv)
                m.grid_pairs[i] = pv.data_ptr()
        m.summed = int(self.summed)
        self._m = m
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)

    def sdf(self, x, lod=None):
        if lod is None:
            lod = self.lod
        _lib.require_cuda(x)
        x = x.detach().float().contiguous()
        out = torch.empty(x.shape[0], 1, device=x.device)
        _lib.check(_lib.load().nglod_sdf_fwd_bf16(self._m, _lib.ptr(x), x.shape[0], -1 if lod is None else lod,
                                                  _lib.ptr(out), _lib.ptr(self._status), _lib.stream_ptr(x.device)),
                   "nglod_sdf_fwd_bf16")
        return out

    def sdf_host(self, x_host, lod=None, out=None, chunk=1 << 19):
        """sdf of points in host memory ([n, 3] float32) into host memory
        ([n, 1] float32, returned) through nglod_sdf_fwd_bf16_host: pinned
        points and results are read and written by the query kernel itself
        over the host link; other host memory is copied in, evaluated and
        copied out in chunks on three streams joined into the current one.
        The result is complete once the current stream's work is (e.g. after
        torch.cuda.synchronize())."""
        if lod is None:
            lod = self.lod
        if x_host.is_cuda or x_host.dtype != torch.float32 or not x_host.is_contiguous():
            raise RuntimeError("sdf_host takes a contiguous float32 CPU tensor (use sdf for device tensors)")
        n = x_host.shape[0]
        if out is None:
            out = torch.empty(n, 1, pin_memory=True)
        dev = self._status.device
        scratch = self._host_scratch(chunk, dev)
        _lib.check(_lib.load().nglod_sdf_fwd_bf16_host(self._m, _lib.ptr(x_host), n, -1 if lod is None else lod,
                                                       _lib.ptr(out), chunk, _lib.ptr(scratch), _lib.ptr(self._status),
                                                       _lib.stream_ptr(dev)), "nglod_sdf_fwd_bf16_host")
        return out

    def _host_scratch(self, chunk, dev):
        nbytes = int(_lib.load().nglod_host_query_scratch_bytes(chunk))
        cur = getattr(self, "_scratch", None)
        if cur is None or cur.numel() < nbytes:
            self._scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        return self._scratch

    def check_status(self):
        """Raises if a tensor-core wait of the last launches gave up."""
        if int(self._status.item()) != 0:
            raise RuntimeError("nglod_sdf_fwd_bf16: a bounded tensor-core wait timed out")

    __call__ = sdf
