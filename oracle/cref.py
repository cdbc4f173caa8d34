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
