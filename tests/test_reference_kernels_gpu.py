"""Parity of the native rows against the reference's OWN CUDA kernels.

The kernels of ``sol_nglod_kernel.cu``, ``spc_raytrace_cuda_kernel.cu`` and
``sol-renderer/SDF.cu`` are compiled unchanged for sm_103a (oracle/ref_build.py)
and launched on this GPU by ``oracle/refkern.py``, which restates the
reference's host code around them.  Integer results (nugget lists) and the
aabb kernel's float results must be bit-identical; the sparse sphere trace,
whose reference decodes with cuBLAS, is held to the drop-in's tolerances:
hit agreement >= 99.99 %, and depth within 1e-4 (normals 1e-3) on all but
0.01 % of the rays both hit.
"""
import os
import tempfile

import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import spc, synthetic
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.options import default_args
from nglod_gb300.sol_nglod import aabb
from nglod_gb300.sparse_sdf import SparseSDF
from oracle import refkern
from oracle import spc as ospc

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref(cuda):
    if not refkern.available():
        pytest.fail("oracle/_ref cubins missing: build them with oracle.ref_build where the reference is present")
    return refkern


def _ms(fn, reps=3):
    """Median CUDA-event time of fn() on the current stream, after one warm-up call."""
    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return sorted(times)[len(times) // 2]


def _bits(t):
    return t.contiguous().view(torch.int32) if t.dtype == torch.float32 else t


def _edge_rays(n, seed):
    """Random rays plus the aabb kernel's edge cases: origins inside the box,
    on its faces, zero and negative-zero direction components, rays parallel
    to faces, grazing rays and far origins."""
    g = np.random.default_rng(seed)
    o = g.uniform(-3, 3, (n, 3)).astype(np.float32)
    d = g.normal(size=(n, 3)).astype(np.float32)
    k = n // 16
    o[:k] = g.uniform(-0.99, 0.99, (k, 3))                       # inside: skipped by the kernel
    o[k:2 * k, 0] = 1.0                                             # on the +x face
    d[2 * k:3 * k, 1] = 0.0                                         # zero component
    d[3 * k:4 * k, 2] = -0.0                                        # negative zero
    d[4 * k:5 * k, 1:] = 0.0                                        # axis-parallel
    o[5 * k:6 * k, 1] = np.float32(1.0)                             # grazing the y = 1 plane
    d[5 * k:6 * k, 1] = 0.0
    o[6 * k:7 * k] *= 1e3                                           # far away (t can pass 500)
    d[7 * k:8 * k] = -o[7 * k:8 * k] + g.uniform(-0.5, 0.5, (k, 3))  # aimed at the box
    return o, d


def test_aabb_bit_exact_with_reference_kernel(ref, cuda):
    """nglod_aabb against the reference aabb_kernel on 2,073,600 camera rays
    and 2M edge-case rays: x, t and hit bit for bit."""
    ros, rds = [], []
    for eye in ((0.0, 0.0, 4.0), (2.5, 1.7, -2.9), (-1.0, 3.5, 0.2)):
        o, d = synthetic.look_at_rays(eye=eye, width=1920, height=1080)
        ros.append(o)
        rds.append(d)
    o, d = _edge_rays(2_000_000, seed=5)
    ros.append(torch.from_numpy(o))
    rds.append(torch.from_numpy(d))
    ro = torch.cat(ros).to(cuda).contiguous()
    rd = torch.cat(rds).to(cuda).contiguous()
    x, t, hit = aabb(ro, rd)
    xr, tr, hr = ref.aabb(ro, rd)
    assert hr.sum().item() > 1_000_000
    assert torch.equal(hit, hr)
    assert torch.equal(_bits(x), _bits(xr))
    assert torch.equal(_bits(t), _bits(tr))


def _band_spc(level, cuda, seed=1):
    c, r = synthetic.sphere_union(seed)
    vox = ospc.voxels_near_surface(lambda p: synthetic.sphere_union_sdf(p, c, r), level)
    return spc.SPC.from_voxels(torch.from_numpy(vox.astype(np.int32)).to(cuda), level)


def _mixed_rays(cuda):
    ro, rd = synthetic.look_at_rays(eye=(1.9, 1.2, 3.1), width=64, height=48, fov=40.0)
    o, d = _edge_rays(20_000, seed=9)
    return (torch.cat([ro, torch.from_numpy(o)]).to(cuda).contiguous(),
            torch.cat([rd, torch.from_numpy(d)]).to(cuda).contiguous())


@pytest.mark.parametrize("level,targets", [(3, [0, 1, 3]), (5, [0, 2, 4, 5])])
def test_spc_raytrace_bit_exact_with_reference_kernels(ref, cuda, level, targets):
    s = _band_spc(level, cuda)
    o, d = _mixed_rays(cuda)
    for target in targets:
        got = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, target)
        want = ref.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, target)
        assert want.shape[0] > 0
        assert got.shape == want.shape, (target, got.shape, want.shape)
        assert torch.equal(got, want), target


@pytest.mark.parametrize("target", [6, 7])
def test_spc_raytrace_bit_exact_with_reference_kernels_at_frame_size(ref, cuda, target):
    """1920x1080 rays into the level-7 octree of the sphere-union surface
    band, to levels 6 and 7: every nugget, in the same order."""
    s = _band_spc(7, cuda)
    o, d = synthetic.look_at_rays(width=1920, height=1080)
    o, d = o.to(cuda), d.to(cuda)
    got = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, target)
    want = ref.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, target)
    assert want.shape[0] > 1_000_000
    assert got.shape == want.shape
    assert torch.equal(got, want)
    # first-nugget flags of the frame (d_MarkUniqueRays, sdfRenderer.cu:108-120)
    first = spc.mark_first(got)
    assert torch.equal(first, ref.mark_unique_rays(want))
    assert int(first.sum()) == int(torch.unique(want[:, 0]).numel())
    t_ours = _ms(lambda: spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, target,
                                          prefix=s.GetPrefix()))
    t_ref = _ms(lambda: ref.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, target))
    print(f"traversal 1920x1080 to level {target}: ours {t_ours:.3f} ms, reference kernels {t_ref:.3f} ms")


def test_generate_rays_bit_exact_with_reference_kernel(ref, cuda):
    """nglod_spc_generate_rays against d_generate_rays on the same matrix."""
    W, H = 1920, 1080
    M = spc.inverse_view_projection([0.3, 0.5, 4.0], [0, 0, 0], [0, 1, 0], W, H, 30.0)
    import ctypes
    from nglod_gb300 import _lib
    org = torch.empty(W * H, 3, device=cuda)
    dr = torch.empty(W * H, 3, device=cuda)
    Mc = np.ascontiguousarray(M, dtype=np.float32)
    _lib.check(_lib.load().nglod_spc_generate_rays(Mc.ctypes.data_as(ctypes.c_void_p), W, H, _lib.ptr(org),
                                                   _lib.ptr(dr), _lib.stream_ptr(cuda)), "nglod_spc_generate_rays")
    org_r, dr_r = ref.generate_rays(Mc, W, H)
    assert torch.equal(_bits(org), _bits(org_r))
    assert torch.equal(_bits(dr), _bits(dr_r))


def _sparse_scene(cuda, num_lods, seed=1):
    c, r = synthetic.sphere_union(seed)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=num_lods, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=3)
    s = _band_spc(num_lods + 1, cuda, seed)
    return net.to(cuda).eval(), s


def _compare_sparse_trace(ref, cuda, num_lods, width, height, lod):
    net, s = _sparse_scene(cuda, num_lods)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "model.npz")
        SparseSDF.from_dense(net, s).save_npz(path)  # the reference export format, float16 arrays
        z = dict(np.load(path))
        ours = SparseSDF.from_npz(path, device=cuda, precision="f32", decoder="f32")
    return _trace_against_reference(ref, cuda, ours, z, width, height, lod)


def _trace_against_reference(ref, cuda, ours, z, width, height, lod):
    s2 = ours.spc
    sdf_ref = ref.SdfRef(z, s2.GetPoints(), s2.GetPyramid(), device=cuda)
    eye, at, up = [0.4, 0.9, 3.8], [0, 0, 0], [0, 1, 0]
    org, dr = spc.spc_generate_primary_rays(torch.tensor(eye), torch.tensor(at), torch.tensor(up), width, height, 30.0,
                                            device=cuda)
    target = lod + 2
    nug = ref.spc_raytrace(s2.GetOctree(), s2.GetPoints(), s2.GetPyramid(), org, dr, target)
    info = ref.mark_unique_rays(nug)
    pyr = s2.GetPyramid()
    pts = s2.GetPoints()[int(pyr[1, target]):, :3].contiguous()
    xr, tr, hr, nr = sdf_ref.sphere_trace(org, dr, nug, pts, info, lod)
    x, t, hit, normal = ours.sphereTrace(org, dr, nug, None, None, lod)
    t_ref = _ms(lambda: sdf_ref.sphere_trace(org, dr, nug, pts, info, lod))
    t_ours = _ms(lambda: ours.sphereTrace(org, dr, nug, None, None, lod))
    print(f"sparse trace {width}x{height} lod {lod} (float32 decoder): ours {t_ours:.3f} ms, "
          f"reference kernels + cuBLAS {t_ref:.3f} ms")
    agree = (hit == hr).float().mean().item()
    both = hit & hr
    assert both.sum().item() > 0.05 * hit.numel()
    dt = (t[both] - tr[both]).abs()[:, 0]
    close = dt < 1e-4
    # A ray whose last step lands within rounding of the hit or oscillation
    # threshold (step.cuh:63-65) can stop one step earlier on one side; such
    # rays must stay below 0.01 % and differ by at most a few such steps.
    far = 1.0 - close.float().mean().item()
    derr = dt.max().item()
    xerr = (x[both] - xr[both]).abs()[close].max().item()
    nerr = (normal[both] - nr[both]).abs()[close].max().item()
    assert agree >= 0.9999, agree
    assert far <= 1e-4, far
    assert derr < 5e-3, derr
    assert xerr < 1e-4, xerr
    assert nerr < 1e-3, nerr
    # rays that hit neither keep the reference's constant normal
    neither = ~hit & ~hr
    assert torch.equal(normal[neither], nr[neither])
    print(f"hit agreement {agree:.6f}, depth beyond 1e-4 on {far:.2e} of hits (max {derr:.2e}), normal {nerr:.2e}")
    return agree, derr, nerr


def test_sparse_trace_matches_reference_sdf_kernels(ref, cuda):
    """SparseSDF.sphereTrace (float32 decoder) against SDF::sphereTrace on the
    reference's kernels and cuBLAS, from the same reference-format npz: 4 LODs
    on a level-5 octree, lod 3, 320x240 renderer rays."""
    _compare_sparse_trace(ref, cuda, num_lods=4, width=320, height=240, lod=3)


def test_sparse_trace_matches_reference_sdf_kernels_at_frame_size(ref, cuda):
    """The same at 1920x1080, 5 LODs on a level-6 octree, lod 4 (the
    reference's SDF class holds as many LODs as the octree has levels below
    level 2, so a 5-LOD model is traced on a level-6 octree)."""
    _compare_sparse_trace(ref, cuda, num_lods=5, width=1920, height=1080, lod=4)


def test_reference_export_round_trip(cuda, golden):
    """SparseSDF.from_npz reads the npz that the reference's own exporter
    wrote (SOL_NGLOD.save, tests/golden/sol_export_small.npz), and save_npz
    writes it back array for array: same keys, dtypes, shapes and values."""
    z = golden("sol_export_small")
    sp = SparseSDF.from_npz(os.path.join(GOLDEN, "sol_export_small.npz"), device=cuda)
    assert sp.corner_counts == [int(v) for v in z["pyramid"]]
    assert sp.spc.GetLevel() == len(z["pyramid"]) + 1
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "again.npz")
        sp.save_npz(path)
        w = dict(np.load(path))
    assert sorted(w) == sorted(z)
    for k in z:
        assert w[k].dtype == z[k].dtype and w[k].shape == z[k].shape, k
        assert np.array_equal(w[k], z[k]), k


@pytest.mark.parametrize("lod", [1, 2])
def test_reference_export_traces_like_reference(ref, cuda, golden, lod):
    """The reference-exported model traced by SparseSDF.sphereTrace and by
    SDF::sphereTrace on the reference kernels: 320x240 renderer rays."""
    z = golden("sol_export_small")
    ours = SparseSDF.from_npz(os.path.join(GOLDEN, "sol_export_small.npz"), device=cuda, precision="f32",
                              decoder="f32")
    _trace_against_reference(ref, cuda, ours, z, 320, 240, lod)
