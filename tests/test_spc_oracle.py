"""SPC octree oracle: codec pinned to the reference's spc3d outputs, child order
pinned to the reference's table, traversal checked against exact geometry."""
import numpy as np

from nglod_gb300 import synthetic
from oracle import cref, spc


def test_child_order_matches_reference_table(golden):
    fx = golden("spc_small")
    assert np.array_equal(cref.child_order_table(), fx["order_table"])


def test_morton_codec_matches_spc3d(golden):
    fx = golden("spc_small")
    m = spc.to_morton(fx["voxels"])
    assert np.array_equal(np.sort(m), fx["morton"])
    assert np.array_equal(spc.to_point(fx["morton"]), fx["points_sorted"])


def test_points_to_octree_matches_spc3d(golden):
    fx = golden("spc_small")
    level = int(fx["level"])
    octree, counts = spc.points_to_octree(fx["voxels"], level)
    assert np.array_equal(octree, fx["octree"])
    assert np.array_equal(counts, fx["pyramid"])
    assert np.array_equal(np.cumsum(counts), fx["pyramid_sum"])
    # duplicates and order do not matter
    v = np.concatenate([fx["voxels"][::-1], fx["voxels"][:100]])
    assert np.array_equal(spc.points_to_octree(v, level)[0], fx["octree"])


def test_set_geometry_matches_spc3d_decode(golden):
    fx = golden("spc_small")
    pts, pyr, prefix = spc.set_geometry(fx["octree"])
    level = int(fx["level"])
    assert pyr.shape == (2, level + 2)
    assert np.array_equal(pyr[0, :level + 1], fx["decoded_pyramid"])
    assert pyr[0, level + 1] == 0 and pyr[1, 0] == 0
    leaves = pts[pyr[1, level]:pyr[1, level + 1], :3]
    assert np.array_equal(leaves.astype(np.uint16), fx["decoded_leaf_points"])
    assert prefix[-1] == pts.shape[0] - 1
    # every node's children are its Morton children
    for l in range(level):
        a, b = pyr[1, l], pyr[1, l + 1]
        parents = spc.to_morton(pts[a:b, :3].astype(np.uint16))
        kids = spc.to_morton(pts[b:pyr[1, l + 2], :3].astype(np.uint16))
        assert np.array_equal(np.unique(kids >> np.uint64(3)), parents)


def _line_hits_box(o, d, lo, hi):
    """FP64 slab test of the infinite line o + t d against [lo, hi]^3."""
    tmin, tmax = -np.inf, np.inf
    for k in range(3):
        if d[k] == 0:
            if o[k] < lo[k] or o[k] > hi[k]:
                return False
            continue
        a, b = (lo[k] - o[k]) / d[k], (hi[k] - o[k]) / d[k]
        tmin, tmax = max(tmin, min(a, b)), min(tmax, max(a, b))
    return tmin <= tmax


def test_traversal_visits_exactly_the_crossed_voxels_front_to_back(golden):
    fx = golden("spc_small")
    pts, pyr, prefix = spc.set_geometry(fx["octree"])
    level = int(fx["level"])
    ro, rd = synthetic.look_at_rays(eye=(1.7, 1.1, 3.0), width=24, height=18, fov=35.0)
    ro, rd = ro.numpy(), rd.numpy()
    for target in (2, level):
        nug = cref.spc_raytrace(fx["octree"], pts, prefix, pyr, level, target, ro, rd)
        vox = pts[pyr[1, target]:pyr[1, target + 1], :3].astype(np.float64)
        s = 2.0 ** -target
        mismatch = 0
        for r in range(ro.shape[0]):
            o = 0.5 * ro[r].astype(np.float64) + 0.5
            d = 0.5 * rd[r].astype(np.float64)
            want = {i for i in range(vox.shape[0]) if _line_hits_box(o, d, vox[i] * s, (vox[i] + 1) * s)}
            got = nug[nug[:, 0] == r, 1]
            assert len(set(got.tolist())) == len(got)
            mismatch += len(want.symmetric_difference(set(got.tolist())))
            if len(got) > 1:  # front to back: entry distances non-decreasing
                c = (vox[got] + 0.5) * s
                t = ((c - o) @ d) / (d @ d)
                assert np.all(np.diff(t) > -1.5 * s), (r, t)
        assert mismatch <= 2, mismatch
        assert nug.shape[0] > 0


def test_sparse_corner_export_matches_reference_unique_corners(golden):
    """oracle.sparse.build's corners and features equal geoutils.unique_corners
    of the reference on the coded volumes of the fixture."""
    from oracle import sparse
    fx = golden("spc_small")
    pts, pyr, prefix = spc.set_geometry(fx["octree"])
    level = int(fx["level"])
    fms = []
    for lv in range(2, level + 1):
        s = 2 ** lv + 1
        c = np.arange(2).reshape(2, 1, 1, 1)
        z = np.arange(s).reshape(1, s, 1, 1)
        y = np.arange(s).reshape(1, 1, s, 1)
        x = np.arange(s).reshape(1, 1, 1, s)
        fms.append((c * 1e6 + z * 1e4 + y * 1e2 + x).astype(np.float64))
    m = sparse.build(fms, pts, pyr, level - 1, corner_dtype=np.float64)
    o = 0
    for i, lv in enumerate(range(2, level + 1)):
        n = m["counts"][i]
        assert np.array_equal(m["cc"][o:o + n], fx[f"corners/{lv}/cc"])
        assert np.array_equal(m["cf"][o:o + n].astype(np.float64), fx[f"corners/{lv}/cf"].astype(np.float32))
        o += n
    # trinket corners really are the voxel's corners, parents contain their children
    for lv in range(2, level + 1):
        a, b = pyr[1, lv], pyr[1, lv + 1]
        vox = pts[a:b, :3].astype(np.int64)
        for j in range(8):
            off = np.array([(j >> 2) & 1, (j >> 1) & 1, j & 1])
            assert np.array_equal(m["cc"][m["trink"][a:b, j]], vox + off)
        if lv > 2:
            assert np.array_equal(pts[m["parent"][a:b], :3].astype(np.int64), vox >> 1)
        else:
            assert (m["parent"][a:b] == -1).all()
