"""The C-ABI library loads, exports every entry point include/nglod_gb300.h
declares, and its structs match the ctypes mirrors.  No CUDA work is issued:
only argument-validation paths that return before touching the device."""
import ctypes
import os
import re
import subprocess

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "nglod_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nglod_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ["nglod_aabb", "nglod_sdf_fwd", "nglod_trace", "nglod_volume_sample", "nglod_last_error"]:
        assert required in names


def test_library_exports_every_declared_symbol(built_library):
    lib = ctypes.CDLL(built_library)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    from nglod_gb300 import _lib
    assert set(_lib.SIGNATURES) <= set(declared_functions())
    assert set(declared_functions()) <= set(_lib.SIGNATURES), "every declared symbol has a Python binding"


def _c_layout(tmp_path, structs):
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "nglod_gb300.h"', "int main(void) {"]
    for s, fields in structs.items():
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f in fields:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (ln.split() for ln in out.strip().splitlines())}


def test_struct_layouts_match_ctypes(tmp_path):
    from nglod_gb300 import _lib
    mirrors = {"nglod_dense_model": _lib.DenseModel, "nglod_trace_params": _lib.TraceParams}
    mirrors.update({k: v for k, v in _lib.STRUCTS.items()} if hasattr(_lib, "STRUCTS") else {})
    structs = {name: [f[0] for f in cls._fields_] for name, cls in mirrors.items()}
    lay = _c_layout(tmp_path, structs)
    for name, cls in mirrors.items():
        assert lay[name] == ctypes.sizeof(cls), name
        for f in cls._fields_:
            assert lay[f"{name}.{f[0]}"] == getattr(cls, f[0]).offset, (name, f[0])


def test_validation_errors_without_device(built_library):
    from nglod_gb300 import _lib
    lib = _lib.load()
    assert lib.nglod_sdf_fwd(None, None, 0, 0, 0, None, None) == -1
    assert b"model is null" in lib.nglod_last_error()
    m = _lib.DenseModel()
    m.num_lods, m.base_lod, m.feature_dim, m.hidden_dim = 2, 2, 16, 128
    assert lib.nglod_sdf_fwd(m, None, 0, 0, 0, None, None) == -2
    assert b"feature_dim=16" in lib.nglod_last_error()
    m.feature_dim = 32
    assert lib.nglod_sdf_fwd(m, None, 0, 0, 0, None, None) == -1  # null volume pointers
    assert lib.nglod_aabb(None, None, 0, None, None, None, None) == 0  # empty input: no work
    assert lib.nglod_aabb(None, None, -1, None, None, None, None) == -1
    assert lib.nglod_trace(None, None, None, None, 0, None, None, None, None, None, None) == -1
    p = _lib.TraceParams()
    p.num_steps = -1
    m.grid[0] = m.grid[1] = 256
    for k in ("w0", "b0", "w1", "b1"):
        getattr(m, k)[0] = getattr(m, k)[1] = 256
    assert lib.nglod_trace(m, p, None, None, 0, None, None, None, None, None, None) == -1
    assert b"num_steps" in lib.nglod_last_error()
    # traversal capacity: below 2^29, so that a level's count fits the 32-bit chunk states
    import ctypes
    pyr = (ctypes.c_int32 * 32)()
    cnt, rb = ctypes.c_int64(0), ctypes.c_int32(0)

    def raytrace(capacity):
        return lib.nglod_spc_raytrace(None, None, None, pyr, 7, 7, None, None, 10, None, None, capacity, None, None,
                                      None, ctypes.byref(cnt), ctypes.byref(rb), None)
    assert raytrace(1 << 29) == -4
    assert b"2^29" in lib.nglod_last_error()
    assert raytrace((1 << 29) - 1) == -1  # past the capacity check: the null octree
    assert raytrace(5) == -4  # fewer nuggets than rays


def test_python_shim_raises_on_status():
    from nglod_gb300 import _lib
    with pytest.raises(RuntimeError, match="invalid argument"):
        _lib.check(_lib.load().nglod_aabb(None, None, -5, None, None, None, None), "nglod_aabb")


def test_bf16_and_training_validation_without_device(built_library):
    """Argument checks of the pair-volume, loss and training entry points
    that run before any CUDA call (fake device addresses, no GPU)."""
    from nglod_gb300 import _lib
    lib = _lib.load()
    b = _lib.Bf16Model()
    b.num_lods, b.base_lod, b.feature_dim, b.hidden_dim = 2, 2, 32, 128
    for i in range(2):
        b.grid[i] = b.w0_tile[i] = b.b0[i] = b.w1[i] = b.b1[i] = 4096 * (i + 1)
    b.grid_pairs[0] = 4096
    b.grid_pairs[1] = 4096 + 16  # 16-byte but not 32-byte aligned
    fake = ctypes.c_void_p(1 << 20)
    assert lib.nglod_sdf_fwd_bf16(b, fake, 10, 1, fake, fake, None) == -5
    assert b"pair volume 1" in lib.nglod_last_error()
    assert lib.nglod_bf16_build_pairs(fake, 1, fake, None) == -1  # s < 2
    assert lib.nglod_bf16_build_pairs(ctypes.c_void_p(4096 + 8), 5, fake, None) == -5
    assert lib.nglod_l2_loss(fake, fake, 10, 0, 1, fake, fake, None) == -1  # rows = 0
    assert lib.nglod_l2_loss(fake, fake, 10, 1, 1, None, fake, None) == -1  # no loss_out
    m = _lib.DenseModel()
    m.num_lods, m.base_lod, m.feature_dim, m.hidden_dim = 2, 2, 32, 128
    for i in range(2):
        m.grid[i] = m.w0[i] = m.b0[i] = m.w1[i] = m.b1[i] = 4096 * (i + 1)
    mis = ctypes.c_void_p((1 << 20) + 4)  # not 16-byte aligned
    assert lib.nglod_sdf_fwd_train(m, fake, 10, 0b11, fake, fake, mis, None) == -5
    assert b"relu_masks" in lib.nglod_last_error()
    g = _lib.DenseGrads()
    for i in range(2):
        g.grid[i] = g.w0[i] = g.b0[i] = g.w1[i] = g.b1[i] = 4096 * (i + 1)
    assert lib.nglod_sdf_bwd(m, fake, 10, 0b11, fake, fake, mis, fake, g, None, None) == -5


def test_summed_volume_validation_without_device(built_library):
    """Argument checks of nglod_build_summed_volume, before any CUDA call."""
    from nglod_gb300 import _lib
    lib = _lib.load()
    m = _lib.DenseModel()
    m.num_lods, m.base_lod, m.feature_dim, m.hidden_dim = 3, 2, 32, 128
    for i in range(3):
        m.grid[i] = 4096 * (i + 1)
    out = ctypes.c_void_p(1 << 20)
    assert lib.nglod_build_summed_volume(m, 3, _lib.F32, out, None) == -1  # lod beyond num_lods - 1
    assert b"lod=3" in lib.nglod_last_error()
    assert lib.nglod_build_summed_volume(m, 1, 7, out, None) == -1  # dtype
    assert lib.nglod_build_summed_volume(m, 1, _lib.BF16, ctypes.c_void_p((1 << 20) + 8), None) == -5
    assert lib.nglod_build_summed_volume(m, 0, _lib.BF16, None, None) == -1
    m.grid[1] = None
    assert lib.nglod_build_summed_volume(m, 2, _lib.F32, out, None) == -1
    assert b"volume 1" in lib.nglod_last_error()
    m.grid[1] = 8192
    m.feature_dim = 16
    assert lib.nglod_build_summed_volume(m, 1, _lib.F32, out, None) == -1


def test_line_read_probe_validation_without_device(built_library):
    """Argument checks of nglod_measure_line_reads, before any CUDA call."""
    from nglod_gb300 import _lib
    lib = _lib.load()
    buf, sink = ctypes.c_void_p(1 << 20), ctypes.c_void_p(1 << 21)
    assert lib.nglod_measure_line_reads(None, 10, 4, 1, sink, None) == -1
    assert lib.nglod_measure_line_reads(ctypes.c_void_p((1 << 20) + 16), 10, 4, 1, sink, None) == -5
    assert lib.nglod_measure_line_reads(buf, 0, 4, 1, sink, None) == -1
    assert lib.nglod_measure_line_reads(buf, 1 << 33, 4, 1, sink, None) == -1
    assert lib.nglod_measure_line_reads(buf, 10, 0, 1, sink, None) == -1


def test_fma_probe_validation_without_device(built_library):
    """Argument checks of nglod_measure_fma and nglod_measure_smem_reads,
    before any CUDA call."""
    from nglod_gb300 import _lib
    lib = _lib.load()
    sink = ctypes.c_void_p(1 << 21)
    assert lib.nglod_measure_fma(16, 1, None, None) == -1
    assert lib.nglod_measure_fma(0, 1, sink, None) == -1
    assert lib.nglod_measure_fma(16, 0, sink, None) == -1
    assert lib.nglod_measure_smem_reads(16, 1, None, None) == -1
    assert lib.nglod_measure_smem_reads(0, 1, sink, None) == -1
    assert lib.nglod_measure_smem_reads(16, 0, sink, None) == -1
