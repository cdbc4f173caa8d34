"""Structured point cloud (SPC) octrees on the GPU.

Drop-ins for sol-renderer's octree layer:

    SPC                         include/spc/spc/SPC.h:100-138, SPC.cu:46-238
    spc_raytrace                include/spc/spc/spc_raytrace_cuda.cpp:141-199
    spc_generate_primary_rays   spc_raytrace_cuda.cpp:65-121
    mark_first (d_MarkUniqueRays)  sol-renderer/sdfRenderer.cu:108-120

Formats are the reference's: octree = child-occupancy bytes of levels
0..L-1 (Morton order within a level); points int16 [psize, 4]; pyramid int32
[2, L+2] on the CPU (counts, exclusive sums).  ``SPC.from_voxels`` builds the
octree on the GPU from leaf voxels (the reference does this on the CPU in
sdf-net/lib/spc3d.py:224-255).
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib

CTRL_WORDS = 20
MAX_LEVELS = 15
MAX_TOTAL_POINTS = 1 << 28


def _u(t):
    return ctypes.c_void_p(t.data_ptr())


def octree_prefix(octree):
    """uint32 (as int32 storage) [osize+1]: exclusive sums of child counts."""
    _lib.require_cuda(octree)
    osize = octree.numel()
    dev = octree.device
    prefix = torch.empty(osize + 1, dtype=torch.int32, device=dev)
    partials = torch.empty(osize // 1024 + 3, dtype=torch.int32, device=dev)
    ctrl = torch.empty(2, dtype=torch.int64, device=dev)
    _lib.check(_lib.load().nglod_spc_prefix(_u(octree), osize, _u(prefix), _u(partials), _u(ctrl),
                                            _lib.stream_ptr(dev)), "nglod_spc_prefix")
    return prefix


class SPC:
    """An octree with its decoded points (SPC::SetGeometry)."""

    def __init__(self, octree=None):
        self.m_Octree = None
        self.m_Points = None
        self.m_Pyramid = None
        self.m_Prefix = None
        self.m_Level = 0
        self.m_Psize = 0
        self.m_Osize = 0
        if octree is not None:
            self.SetGeometry(octree)

    @classmethod
    def from_voxels(cls, voxels, level):
        """Octree of the given leaf voxels [n, 3] (any order, duplicates allowed)."""
        _lib.require_cuda(voxels)
        v = voxels.to(torch.int32).clamp_(min=0).to(torch.int16).contiguous()
        n = v.shape[0]
        dev = v.device
        lib = _lib.load()
        nbytes = lib.nglod_spc_build_scratch_bytes(level)
        if nbytes < 0:
            raise RuntimeError(f"SPC.from_voxels: level {level} outside [1, 9]")
        scratch = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        off = (-scratch.data_ptr()) % 256
        cap = min(n, 1 << 30) * level + 16
        octree = torch.empty(cap, dtype=torch.uint8, device=dev)
        osize = ctypes.c_int64(0)
        pyr = np.zeros((2, level + 2), dtype=np.int32)
        _lib.check(lib.nglod_spc_build(_u(v), n, level, _u(octree), cap, ctypes.byref(osize),
                                       pyr.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(scratch.data_ptr() + off),
                                       _lib.stream_ptr(dev)), "nglod_spc_build")
        return cls(octree[:osize.value].clone())

    def SetGeometry(self, octree):
        _lib.require_cuda(octree)
        if octree.dtype != torch.uint8:
            raise RuntimeError("octree must be a uint8 tensor")
        octree = octree.contiguous()
        osize = octree.numel()
        dev = octree.device
        # An octree of L levels has at most 8 * osize + 1 points.
        cap = 8 * osize + 64
        points = torch.empty(cap, 4, dtype=torch.int16, device=dev)
        prefix = torch.empty(osize + 1, dtype=torch.int32, device=dev)
        pyr = np.zeros(2 * (MAX_LEVELS + 2), dtype=np.int32)
        level = ctypes.c_int32(0)
        _lib.check(_lib.load().nglod_spc_decode(_u(octree), osize, _u(points), cap, _u(prefix),
                                                pyr.ctypes.data_as(ctypes.c_void_p), ctypes.byref(level),
                                                _lib.stream_ptr(dev)), "nglod_spc_decode")
        L = level.value
        pyramid = torch.from_numpy(pyr[:2 * (L + 2)].reshape(2, L + 2).copy())
        psize = int(pyramid[1, L + 1])
        self.m_Octree = octree
        self.m_Points = points[:psize].clone()
        self.m_Pyramid = pyramid
        self.m_Prefix = prefix
        self.m_Level = L
        self.m_Psize = int(pyramid[0, L])
        self.m_Osize = osize
        return [self.m_Points, self.m_Pyramid]

    def LoadNPZ(self, filename, device="cuda"):
        octree = np.load(filename)["octree"]
        self.SetGeometry(torch.from_numpy(np.ascontiguousarray(octree, dtype=np.uint8)).to(device))

    def SaveNPZ(self, filename):
        np.savez(filename, octree=self.m_Octree.cpu().numpy())

    def GetOctree(self):
        return self.m_Octree

    def GetPoints(self, l=None):
        """All points, or the points from level l's first onward (SPC.cu:126-132)."""
        if l is None:
            return self.m_Points
        return self.m_Points[int(self.m_Pyramid[1, l]):]

    def GetLevelPoints(self, l):
        a, b = int(self.m_Pyramid[1, l]), int(self.m_Pyramid[1, l + 1])
        return self.m_Points[a:b]

    def GetPyramid(self):
        return self.m_Pyramid

    def GetPrefix(self):
        return self.m_Prefix

    def GetPSize(self):
        return self.m_Psize

    def GetOSize(self):
        return self.m_Osize

    def GetLevel(self):
        return self.m_Level


def spc_raytrace(octree, points, pyramid, Org, Dir, targetLevel, prefix=None, capacity=None):
    """Nuggets int32 [count, 2] = (ray index, voxel index within targetLevel)
    for every voxel at targetLevel that each ray's line passes through, per
    ray front to back.  Same checks as spc_raytrace_cuda.cpp:149-160."""
    if octree.dtype != torch.uint8:
        raise RuntimeError("input is not Byte")
    if points.dtype != torch.int16 or points.dim() != 2 or points.shape[1] != 4 or not points.is_contiguous():
        raise RuntimeError("points: input is not a contiguous Nx4 Short tensor")
    if pyramid.is_cuda or pyramid.dtype != torch.int32 or not pyramid.is_contiguous():
        raise RuntimeError("pyramid must be a contiguous int32 CPU tensor")
    if pyramid.dim() != 2 or pyramid.shape[0] != 2:
        raise RuntimeError("bad spc table")
    level = pyramid.shape[1] - 2
    if level >= MAX_LEVELS:
        raise RuntimeError("bad spc table")
    h = pyramid.numpy().reshape(-1)
    if octree.numel() != int(h[2 * level + 2]):
        raise RuntimeError("bad spc octree size")
    if points.shape[0] != int(h[2 * level + 3]):
        raise RuntimeError("bad spc points size")
    if int(h[level + 1]) != 0 or int(h[level + 2]) != 0:
        raise RuntimeError("bad spc table")
    _lib.require_cuda(octree, points, Org, Dir)
    Org = Org.float().contiguous()
    Dir = Dir.float().contiguous()
    n = Org.shape[0]
    dev = Org.device
    if prefix is None:
        prefix = octree_prefix(octree)
    if capacity is None:
        # four nuggets per ray covers typical frames in one pass (a frame of
        # 1920x1080 rays against a level-7 sphere-union octree needs ~2.5 per
        # ray at level 6); a larger count costs one retry with 4x the buffers.
        capacity = max(4 * n, 1 << 22)
    capacity = max(capacity, n)
    lib = _lib.load()
    while True:
        a = torch.empty(capacity, 2, dtype=torch.int32, device=dev)
        b = torch.empty(capacity, 2, dtype=torch.int32, device=dev)
        info = torch.empty(max(capacity, 1024), dtype=torch.int32, device=dev)
        partials = torch.empty(capacity // 1024 + 2, dtype=torch.int32, device=dev)
        ctrl = torch.empty(CTRL_WORDS, dtype=torch.int64, device=dev)
        count = ctypes.c_int64(0)
        which = ctypes.c_int32(0)
        st = lib.nglod_spc_raytrace(_u(octree), _u(points), _u(prefix), pyramid.numpy().ctypes.data_as(ctypes.c_void_p),
                                    level, targetLevel, _u(Org), _u(Dir), n, _u(a), _u(b), capacity, _u(info),
                                    _u(partials), _u(ctrl), ctypes.byref(count), ctypes.byref(which),
                                    _lib.stream_ptr(dev))
        if st == -4 and capacity < MAX_TOTAL_POINTS:
            capacity = min(capacity * 4, MAX_TOTAL_POINTS)
            continue
        _lib.check(st, "nglod_spc_raytrace")
        return (a if which.value == 0 else b)[:count.value]


def mark_first(nuggets):
    """int32 [n]: 1 where a nugget is the first of its ray (d_MarkUniqueRays)."""
    _lib.require_cuda(nuggets)
    nuggets = nuggets.contiguous()
    info = torch.empty(nuggets.shape[0], dtype=torch.int32, device=nuggets.device)
    _lib.check(_lib.load().nglod_spc_mark_first(_u(nuggets), nuggets.shape[0], _u(info),
                                                _lib.stream_ptr(nuggets.device)), "nglod_spc_mark_first")
    return info


def inverse_view_projection(eye, at, up, width, height, fov, world=None):
    """4x4 float32 row-major matrix of spc_raytrace_cuda.cpp:80-103 (row-vector convention)."""
    f = np.float32
    eye, at, up = (np.asarray(v, dtype=f) for v in (eye, at, up))
    world = np.eye(4, dtype=f) if world is None else np.asarray(world, dtype=f).reshape(4, 4)
    world_inv = world.T
    ar = f(width) / f(height)
    rad = f(0.01745329) * f(fov)
    t = f(math.tan(f(0.5) * rad))
    pvp = np.array([[f(2) * ar * t / f(width), 0, 0, 0],
                    [0, f(2) * t / f(height), 0, 0],
                    [0, 0, 0, 1],
                    [ar * t * (f(1) - f(width)) / f(width), t * (f(1) - f(height)) / f(height), -1, 0]], dtype=f)
    z = at - eye
    z = z / np.sqrt((z * z).sum())
    x = np.cross(z, up).astype(f)
    x = x / np.sqrt((x * x).sum())
    y = np.cross(x, z).astype(f)
    view = np.array([[x[0], x[1], x[2], 0], [y[0], y[1], y[2], 0], [-z[0], -z[1], -z[2], 0],
                     [eye[0], eye[1], eye[2], 1]], dtype=f)
    return (pvp @ view @ world_inv).astype(f)


def spc_generate_primary_rays(Eye, At, Up, imageW, imageH, fov, World=None, device="cuda"):
    """[Org, Dir] float32 [W*H, 3] pinhole rays, pixel i = (i % W, i // W);
    directions are not normalised (as in the reference)."""
    to_np = (lambda v: v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v)
    M = inverse_view_projection(to_np(Eye), to_np(At), to_np(Up), imageW, imageH, fov,
                                None if World is None else to_np(World))
    n = imageW * imageH
    org = torch.empty(n, 3, device=device)
    dr = torch.empty(n, 3, device=device)
    Mc = np.ascontiguousarray(M, dtype=np.float32)
    _lib.check(_lib.load().nglod_spc_generate_rays(Mc.ctypes.data_as(ctypes.c_void_p), imageW, imageH, _u(org),
                                                   _u(dr), _lib.stream_ptr(org.device)), "nglod_spc_generate_rays")
    return [org, dr]
