"""SPC octree on the GPU: build and decode bit-exact with the reference's
spc3d / SetGeometry, traversal bit-exact with the C restatement of
spc_raytrace."""
import numpy as np
import pytest
import torch

from nglod_gb300 import _lib, spc, synthetic
from oracle import cref
from oracle import spc as ospc

pytestmark = pytest.mark.gpu


def _sphere_octree(level, seed=1):
    c, r = synthetic.sphere_union(seed)
    vox = ospc.voxels_near_surface(lambda p: synthetic.sphere_union_sdf(p, c, r), level)
    return vox


def test_build_matches_spc3d_golden(golden, cuda):
    fx = golden("spc_small")
    level = int(fx["level"])
    s = spc.SPC.from_voxels(torch.from_numpy(fx["voxels"].astype(np.int32)).to(cuda), level)
    assert np.array_equal(s.GetOctree().cpu().numpy(), fx["octree"])
    pyr = s.GetPyramid().numpy()
    assert np.array_equal(pyr[0, :level + 1], fx["pyramid"])
    leaves = s.GetLevelPoints(level)[:, :3].cpu().numpy().astype(np.uint16)
    assert np.array_equal(leaves, fx["decoded_leaf_points"])


@pytest.mark.parametrize("level", [3, 6, 7])
def test_decode_matches_oracle(cuda, level):
    vox = _sphere_octree(level)
    octree, counts = ospc.points_to_octree(vox, level)
    s = spc.SPC(torch.from_numpy(octree).to(cuda))
    pts, pyr, prefix = ospc.set_geometry(octree)
    assert s.GetLevel() == level
    assert np.array_equal(s.GetPyramid().numpy(), pyr)
    assert np.array_equal(s.GetPoints().cpu().numpy(), pts)
    assert np.array_equal(s.GetPrefix().cpu().numpy().view(np.uint32), prefix)
    assert np.array_equal(spc.octree_prefix(s.GetOctree()).cpu().numpy().view(np.uint32), prefix)
    # GPU build from the same voxels (shuffled, with duplicates) gives the same bytes
    rng = np.random.default_rng(level)
    v = np.concatenate([vox, vox[: len(vox) // 3]])[rng.permutation(len(vox) + len(vox) // 3)]
    b = spc.SPC.from_voxels(torch.from_numpy(v.astype(np.int32)).to(cuda), level)
    assert np.array_equal(b.GetOctree().cpu().numpy(), octree)


def _rays(n_img=(64, 48), seed=0):
    ro, rd = synthetic.look_at_rays(eye=(1.9, 1.2, 3.1), width=n_img[0], height=n_img[1], fov=40.0)
    rng = np.random.default_rng(seed)
    o2 = rng.uniform(-2.5, 2.5, (2000, 3)).astype(np.float32)
    o2[:300] = rng.uniform(-0.8, 0.8, (300, 3))  # origins inside the volume
    d2 = rng.normal(size=(2000, 3)).astype(np.float32)
    d2[:100, 0] = 0.0  # axis-parallel components
    d2[100:150, 1:] = 0.0
    ro = np.concatenate([ro.numpy(), o2])
    rd = np.concatenate([rd.numpy(), d2])
    return ro, rd


@pytest.mark.parametrize("level,targets", [(5, [0, 2, 5]), (7, [3, 6, 7])])
def test_raytrace_bit_exact(cuda, level, targets):
    vox = _sphere_octree(level)
    s = spc.SPC.from_voxels(torch.from_numpy(vox.astype(np.int32)).to(cuda), level)
    pts = s.GetPoints().cpu().numpy()
    pyr = s.GetPyramid().numpy()
    prefix = s.GetPrefix().cpu().numpy().view(np.uint32)
    octree = s.GetOctree().cpu().numpy()
    ro, rd = _rays()
    for target in targets:
        got = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), torch.from_numpy(ro).to(cuda),
                               torch.from_numpy(rd).to(cuda), target).cpu().numpy()
        want = cref.spc_raytrace(octree, pts, prefix, pyr, level, target, ro, rd)
        assert got.shape == want.shape, (target, got.shape, want.shape)
        assert np.array_equal(got, want), target


def test_raytrace_bit_exact_at_frame_size(cuda):
    """The sparse bench's traversal at full size -- 1920x1080 rays into the
    level-7 octree of the sphere-union surface band, to level 6 (lod 4 + 2,
    5.1M nuggets) -- bit-exact with the C restatement: every nugget, in the
    same order."""
    level = 7
    vox = _sphere_octree(level)
    s = spc.SPC.from_voxels(torch.from_numpy(vox.astype(np.int32)).to(cuda), level)
    pts = s.GetPoints().cpu().numpy()
    pyr = s.GetPyramid().numpy()
    prefix = s.GetPrefix().cpu().numpy().view(np.uint32)
    octree = s.GetOctree().cpu().numpy()
    ro, rd = synthetic.look_at_rays(width=1920, height=1080)
    for target in (6,):
        got = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), ro.to(cuda), rd.to(cuda),
                               target).cpu().numpy()
        want = cref.spc_raytrace(octree, pts, prefix, pyr, level, target, ro.numpy(), rd.numpy())
        assert got.shape[0] > 1_000_000
        assert np.array_equal(got, want), target


def test_raytrace_capacity_and_empty(cuda):
    level = 5
    s = spc.SPC.from_voxels(torch.from_numpy(_sphere_octree(level).astype(np.int32)).to(cuda), level)
    ro, rd = _rays()
    o = torch.from_numpy(ro).to(cuda)
    d = torch.from_numpy(rd).to(cuda)
    full = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, level)
    # a capacity below the nugget count grows transparently in Python ...
    small = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), o, d, level, capacity=o.shape[0])
    assert torch.equal(full, small)
    # ... and is an error code (not silent truncation) at the C ABI
    lib = _lib.load()
    cap = o.shape[0]
    bufs = [torch.empty(cap, 2, dtype=torch.int32, device=cuda) for _ in range(2)]
    info = torch.empty(max(cap, 1024), dtype=torch.int32, device=cuda)
    parts = torch.empty(cap // 1024 + 2, dtype=torch.int32, device=cuda)
    ctrl = torch.empty(spc.CTRL_WORDS, dtype=torch.int64, device=cuda)
    import ctypes
    cnt, which = ctypes.c_int64(0), ctypes.c_int32(0)
    pyr = s.GetPyramid().numpy()
    st = lib.nglod_spc_raytrace(spc._u(s.GetOctree()), spc._u(s.GetPoints()), spc._u(s.GetPrefix()),
                                pyr.ctypes.data_as(ctypes.c_void_p), level, level, spc._u(o), spc._u(d), o.shape[0],
                                spc._u(bufs[0]), spc._u(bufs[1]), cap, spc._u(info), spc._u(parts), spc._u(ctrl),
                                ctypes.byref(cnt), ctypes.byref(which), _lib.stream_ptr(cuda))
    assert full.shape[0] > cap and st == -4
    # rays that miss the volume give an empty list
    miss = spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(),
                            torch.tensor([[5.0, 5.0, 5.0]], device=cuda), torch.tensor([[1.0, 0.0, 0.0]], device=cuda),
                            level)
    assert miss.shape == (0, 2)


def test_mark_first(cuda):
    nug = torch.tensor([[0, 3], [0, 4], [2, 1], [5, 0], [5, 2], [5, 9]], dtype=torch.int32, device=cuda)
    assert spc.mark_first(nug).cpu().tolist() == [1, 0, 1, 1, 0, 0]


def test_generate_primary_rays(cuda):
    W, H = 64, 48
    org, dr = spc.spc_generate_primary_rays(torch.tensor([0.0, 0.0, 4.0]), torch.zeros(3), torch.tensor([0.0, 1.0, 0.0]),
                                            W, H, 30.0)
    M = spc.inverse_view_projection([0, 0, 4], [0, 0, 0], [0, 1, 0], W, H, 30.0).astype(np.float64)
    i = np.arange(W * H)
    b = np.stack([i % W, i // W, np.zeros_like(i), np.ones_like(i)], 1).astype(np.float64) @ M
    a = np.array([0, 0, 1, 0], np.float64) @ M
    np.testing.assert_allclose(dr.cpu().numpy(), b[:, :3], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(org.cpu().numpy(), np.broadcast_to(a[:3], (W * H, 3)), rtol=1e-5, atol=1e-6)
    # the centre pixel looks at the target
    c = dr[(H // 2) * W + W // 2].cpu().numpy()
    assert c[2] < 0 and abs(c[0]) < 0.05 and abs(c[1]) < 0.05
