"""numpy restatement of the SPC octree codec (test infrastructure).

Follows sdf-net/lib/spc3d.py (to_morton 24-31, to_point 33-40,
points_to_nodes 224-255, nodes_to_points 273-304) and sol-renderer's
SPC::SetGeometry (include/spc/spc/SPC.cu:148-238), vectorised.  Integer only,
so results are exact.
"""
import numpy as np


def to_morton(p):
    """Morton codes of [n, 3] integer points: bit 3i+2 = x_i, 3i+1 = y_i, 3i = z_i."""
    p = np.asarray(p, dtype=np.uint64)
    m = np.zeros(p.shape[0], dtype=np.uint64)
    for i in range(16):
        b = np.uint64(i)
        one = np.uint64(1)
        m |= ((p[:, 2] >> b) & one) << (np.uint64(3) * b)
        m |= ((p[:, 1] >> b) & one) << (np.uint64(3) * b + one)
        m |= ((p[:, 0] >> b) & one) << (np.uint64(3) * b + np.uint64(2))
    return m


def to_point(m):
    m = np.asarray(m, dtype=np.uint64)
    out = np.zeros((m.shape[0], 3), dtype=np.uint16)
    for i in range(16):
        b = np.uint64(i)
        one = np.uint64(1)
        out[:, 0] |= (((m >> (np.uint64(3) * b + np.uint64(2))) & one) << b).astype(np.uint16)
        out[:, 1] |= (((m >> (np.uint64(3) * b + one)) & one) << b).astype(np.uint16)
        out[:, 2] |= (((m >> (np.uint64(3) * b)) & one) << b).astype(np.uint16)
    return out


def points_to_octree(voxels, level):
    """Octree bytes and per-level counts from leaf voxels [n, 3] at `level`.

    Leaves are Morton-sorted and deduplicated; each level's byte for a node is
    the OR of 1 << (child Morton & 7) over its children (spc3d.py:200-222).
    Returns (octree uint8 [osize], counts int64 [level + 1]).
    """
    m = np.unique(to_morton(voxels))
    counts = [0] * (level + 1)
    counts[level] = m.size
    levels = []
    for l in range(level, 0, -1):
        parent = m >> np.uint64(3)
        child = (m & np.uint64(7)).astype(np.uint32)
        up, inv = np.unique(parent, return_inverse=True)
        byte = np.zeros(up.size, dtype=np.uint32)
        np.bitwise_or.at(byte, inv, (np.uint32(1) << child))
        levels.append(byte.astype(np.uint8))
        counts[l - 1] = up.size
        m = up
    octree = np.concatenate(levels[::-1]) if levels else np.zeros(0, np.uint8)
    return octree, np.array(counts, dtype=np.int64)


def set_geometry(octree):
    """SPC::SetGeometry: (points int16 [psize, 4], pyramid int32 [2, L+2],
    prefix uint32 [osize+1]) where prefix is the exclusive scan of child
    counts (popcounts) over all octree bytes."""
    octree = np.asarray(octree, dtype=np.uint8)
    osize = octree.size
    pc = np.unpackbits(octree[:, None], axis=1).sum(axis=1).astype(np.uint64)
    prefix = np.zeros(osize + 1, dtype=np.uint64)
    prefix[1:] = np.cumsum(pc)
    counts = [1]
    codes = [np.zeros(1, dtype=np.uint64)]
    start = 0
    while start < osize:
        cnt = counts[-1]
        m = codes[-1]
        bytes_ = octree[start:start + cnt]
        kids = []
        for j in range(8):
            has = (bytes_ >> j) & 1
            kids.append(np.where(has == 1, np.uint64(8) * m + np.uint64(j), np.uint64(0xFFFFFFFFFFFFFFFF)))
        kids = np.stack(kids, axis=1).reshape(-1)
        kids = kids[kids != np.uint64(0xFFFFFFFFFFFFFFFF)]
        codes.append(kids)
        counts.append(kids.size)
        start += cnt
    if start != osize:
        raise ValueError("octree bytes do not describe a complete tree")
    L = len(counts) - 1
    allcodes = np.concatenate(codes)
    pts = np.zeros((allcodes.size, 4), dtype=np.int16)
    pts[:, :3] = to_point(allcodes).astype(np.int16)
    pyr = np.zeros((2, L + 2), dtype=np.int32)
    pyr[0, :L + 1] = counts
    pyr[1, 1:] = np.cumsum(counts)
    return pts, pyr, prefix.astype(np.uint32)


def voxels_near_surface(sdf_fn, level, band=None):
    """Leaf voxels [n, 3] uint16 whose centre lies within `band` (default one
    voxel diagonal) of the zero set of sdf_fn (float64 [N,3] -> [N])."""
    res = 2 ** level
    if band is None:
        band = np.sqrt(3) * (2.0 / res)
    idx = np.stack(np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing="ij"), -1).reshape(-1, 3)
    centres = (idx + 0.5) / res * 2 - 1
    keep = np.abs(sdf_fn(centres)) <= band
    return idx[keep].astype(np.uint16)
