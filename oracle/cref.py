"""ctypes front end of the C oracle ``oracle/nglod_oracle.c`` (test infrastructure).

``build()`` compiles it with gcc into oracle/_build/libnglod_oracle.so.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nglod_oracle.c")
OUT = os.path.join(HERE, "_build", "libnglod_oracle.so")
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]

_LIB = None


def build(force=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        cmd = ["gcc", *CFLAGS, SRC, "-o", OUT, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return OUT


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        _LIB.oracle_aabb.argtypes = [vp, vp, i64, vp, vp, vp]
        _LIB.oracle_aabb.restype = None
        _LIB.oracle_child_order_table.argtypes = [vp]
        _LIB.oracle_child_order_table.restype = None
        _LIB.oracle_spc_raytrace.argtypes = [vp, vp, vp, vp, ctypes.c_int, ctypes.c_int, vp, vp, i64, vp, i64]
        _LIB.oracle_spc_raytrace.restype = i64
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def aabb(ray_o, ray_d):
    """Bit-exact float32 restatement of sol_nglod.aabb: (x [N,3], t [N,1], hit [N] bool)."""
    o = np.ascontiguousarray(ray_o, dtype=np.float32)
    d = np.ascontiguousarray(ray_d, dtype=np.float32)
    n = o.shape[0]
    x = np.empty((n, 3), np.float32)
    t = np.empty((n, 1), np.float32)
    hit = np.empty(n, np.uint8)
    lib().oracle_aabb(_p(o), _p(d), n, _p(x), _p(t), _p(hit))
    return x, t, hit.astype(bool)


def child_order_table():
    t = np.zeros(64, np.uint8)
    lib().oracle_child_order_table(_p(t))
    return t.reshape(8, 8)


def spc_raytrace(octree, points, prefix, pyramid, level, target, org, dir, cap=1 << 26):
    """C restatement of spc_raytrace: nuggets int32 [count, 2] (ray, voxel at target)."""
    octree = np.ascontiguousarray(octree, np.uint8)
    points = np.ascontiguousarray(points, np.int16)
    prefix = np.ascontiguousarray(prefix, np.uint32)
    pyramid = np.ascontiguousarray(pyramid, np.int32)
    org = np.ascontiguousarray(org, np.float32)
    dir = np.ascontiguousarray(dir, np.float32)
    out = np.empty((cap, 2), np.int32)
    cnt = lib().oracle_spc_raytrace(_p(octree), _p(points), _p(prefix), _p(pyramid), level, target, _p(org),
                                    _p(dir), org.shape[0], _p(out), cap)
    if cnt < 0:
        raise RuntimeError("capacity exceeded")
    return out[:cnt].copy()
