"""numpy restatement of sol-renderer's sparse SDF (test infrastructure).

Construction follows SOL_NGLOD (sdf-net/lib/models/SOL_NGLOD.py:68-75:
unique corners per level in lexicographic order, features fm[:, z, y, x])
and SDF::initTrinkets / index_trinket_kernel (sol-renderer/SDF.cu:141-216,
solr/sdf/index_trinket.cuh:48-97).  Evaluation follows
sparse_grid_sample_kernel (solr/sdf/sparse_grid_sample.cuh:52-107), the
decoder addmm/relu/addmm (SDF.cu:420-421), step_kernel (solr/sdf/step.cuh:
48-85), ray_aabb / ray_aabb_kernel (solr/gfx/ray_aabb.cuh:42-192),
getNormal + normalize_kernel (SDF.cu:218-295, solr/common/normalize.cuh) and
the host loop of SDF::sphereTrace (SDF.cu:297-472), vectorised over rays in
float32 (fused multiply-adds evaluated in float64 and rounded once more).
"""
import numpy as np

f32 = np.float32


def _fma(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(f32)


def build(fms, pts, pyr, num_lods, corner_dtype=np.float32):
    """fms: per-LOD dense volumes [C, s, s, s] (LOD i: s = 2^(i+2)+1);
    pts/pyr from oracle.spc.set_geometry.  Returns a dict model."""
    psize = pts.shape[0]
    cc_all, cf_all, counts = [], [], []
    trink = np.full((psize, 8), -1, np.int64)
    parent = np.full(psize, -1, np.int64)
    offset = 0
    for i in range(num_lods):
        lv = i + 2
        a, b = pyr[1, lv], pyr[1, lv + 1]
        vox = pts[a:b, :3].astype(np.int64)
        offs = np.array([[(j >> 2) & 1, (j >> 1) & 1, j & 1] for j in range(8)])
        corners = np.unique((vox[:, None, :] + offs[None]).reshape(-1, 3), axis=0)
        fm = fms[i]
        cf = fm[:, corners[:, 2], corners[:, 1], corners[:, 0]].T.astype(corner_dtype)
        s = 2 ** lv + 1
        key = (corners[:, 0] * s + corners[:, 1]) * s + corners[:, 2]
        for j in range(8):
            c = vox + offs[j]
            k = (c[:, 0] * s + c[:, 1]) * s + c[:, 2]
            trink[a:b, j] = offset + np.searchsorted(key, k)
        if lv > 2:
            pa, pb = pyr[1, lv - 1], pyr[1, lv]
            ppts = pts[pa:pb, :3].astype(np.int64)
            ps = 2 ** (lv - 1)
            pkey = (ppts[:, 0] * ps + ppts[:, 1]) * ps + ppts[:, 2]
            order = np.argsort(pkey)
            q = vox >> 1
            qk = (q[:, 0] * ps + q[:, 1]) * ps + q[:, 2]
            parent[a:b] = pa + order[np.searchsorted(pkey[order], qk)]
        cc_all.append(corners)
        cf_all.append(cf)
        counts.append(corners.shape[0])
        offset += corners.shape[0]
    return {"cc": np.concatenate(cc_all), "cf": np.concatenate(cf_all).astype(np.float32), "counts": counts,
            "trink": trink, "parent": parent, "pts": pts, "pyr": pyr}


def features(m, lod, g, x, summed=False):
    """sparse_grid_sample_kernel: [n, C] feature sums starting in voxels g (global).

    summed: m's corner features come from LOD-summed volumes
    (dense.summed_volume), and the sum stops after the query level (the
    summed form of nglod_sparse_model)."""
    n = x.shape[0]
    C = m["cf"].shape[1]
    out = np.zeros((n, C), f32)
    nx = _fma(x[:, 0], 0.5, 0.5)
    ny = _fma(x[:, 1], 0.5, 0.5)
    nz = _fma(x[:, 2], 0.5, 0.5)
    g = g.copy()
    cc = m["cc"].astype(f32)
    last = lod + 2 if summed else 2
    for lv in range(lod + 2, last - 1, -1):
        if lv != lod + 2:
            g = m["parent"][g]
        res = f32(2 ** lv)
        iz, iy, ix = nx * res, ny * res, nz * res  # the reference's naming: iz holds x
        v = m["trink"][g]  # [n, 8], v[j] with j = 4*dx + 2*dy + dz
        # corner order of the accumulation: x fastest, then y, then z
        for k in range(8):
            bx, by, bz = k & 1, (k >> 1) & 1, k >> 2
            j = 4 * bx + 2 * by + bz
            opp = m["trink"][g][:, 4 * (1 - bx) + 2 * (1 - by) + (1 - bz)]
            wz = (ix - cc[opp, 2]) if bz else (cc[opp, 2] - ix)
            wy = (iy - cc[opp, 1]) if by else (cc[opp, 1] - iy)
            wx = (iz - cc[opp, 0]) if bx else (cc[opp, 0] - iz)
            w = ((wz * wy) * wx).astype(f32)
            out = (out + m["cf"][v[:, j]] * w[:, None]).astype(f32)
    return out


def decode(dec, x, feats):
    w0, b0, w1, b1 = dec
    ex = np.concatenate([x, feats], axis=1).astype(f32)
    h = np.maximum(ex @ w0.T + b0, 0).astype(f32)
    return (h @ w1.T + b1).astype(f32)[:, 0]


def _bf16(a):
    """float32 -> bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=f32)
    u = a.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(f32)


def decode_bf16_tile(dec, x, feats):
    """The BF16 decoder tile of the tensor-core trace (not a reference
    computation; it restates the tile's arithmetic to check the kernel):
    features and first-layer weights rounded to bf16, positions and b0 as
    bf16 hi + lo, products summed in float64 (the tensor core sums in fp32),
    ReLU and the second layer in float32."""
    w0, b0, w1, b1 = dec
    x = x.astype(f32)
    f = _bf16(feats).astype(np.float64)
    hi = _bf16(x)
    lo = _bf16(x - hi)
    wb = _bf16(w0).astype(np.float64)
    b0h = _bf16(b0)
    b0l = _bf16(b0 - b0h)
    h = f @ wb[:, 3:].T + hi.astype(np.float64) @ wb[:, :3].T + lo.astype(np.float64) @ wb[:, :3].T
    h = np.maximum((h + b0h.astype(np.float64) + b0l.astype(np.float64)).astype(f32), 0)
    return (h @ w1.astype(f32).T + b1.astype(f32)).astype(f32)[:, 0]


def _voxel_entry(q, d, inv, sgn, vc, r):
    o = (q - vc).astype(f32)
    cmax = np.abs(o).max(axis=1)
    wind = np.where(cmax < r, f32(-1), f32(1)) * f32(r)
    dd = [(_fma(wind, sgn[:, k], -o[:, k]) * inv[:, k]).astype(f32) for k in range(3)]
    tests = []
    for a, (b, c) in enumerate(((1, 2), (0, 2), (0, 1))):
        tests.append((dd[a] >= 0) & (np.abs(_fma(d[:, b], dd[a], o[:, b])) < r) &
                     (np.abs(_fma(d[:, c], dd[a], o[:, c])) < r))
    dist = np.where(tests[0], dd[0], np.where(tests[1], dd[1], np.where(tests[2], dd[2], f32(0))))
    return np.where(wind < 0, wind, dist).astype(f32)


def sphere_trace(m, decs, lod, ray_o, ray_d, nuggets, num_steps=50, decoder=decode):
    """SDF::sphereTrace: (x [n,3], t [n,1], hit [n], normal [n,3]).
    ``decoder``: decode (the reference's float32 decoder) or
    decode_bf16_tile."""
    decode_fn = decoder
    o = ray_o.astype(f32)
    dr = ray_d.astype(f32)
    n = o.shape[0]
    lv = lod + 2
    lstart = m["pyr"][1, lv]
    r = f32(1.0 / 2 ** lv)
    x = o.copy()
    t = np.zeros(n, f32)
    dprev = np.zeros(n, f32)
    cond = np.zeros(n, bool)
    hit = np.zeros(n, bool)
    pidx = np.full(n, -1, np.int64)
    inv = (f32(1) / dr).astype(f32)
    sgn = np.where(np.signbit(dr), f32(1), f32(-1))
    # per-ray nugget lists
    nug = nuggets.astype(np.int64)
    heads = np.flatnonzero(np.r_[True, nug[1:, 0] != nug[:-1, 0]]) if len(nug) else np.zeros(0, np.int64)
    lens = np.diff(np.r_[heads, len(nug)])
    rays = nug[heads, 0] if len(nug) else np.zeros(0, np.int64)
    K = int(lens.max()) if len(lens) else 0
    lists = np.full((n, max(K, 1)), -1, np.int64)
    for k in range(K):
        sel = lens > k
        lists[rays[sel], k] = nug[heads[sel] + k, 1]
    has = np.zeros(n, bool)
    has[rays] = True
    vox = m["pts"][:, :3].astype(f32)

    def walk(active, q):
        found = np.zeros(n, bool)
        for k in range(K):
            cand = active & ~found & (lists[:, k] >= 0)
            if not cand.any():
                break
            idx = np.flatnonzero(cand)
            pid = lists[idx, k]
            p = vox[lstart + pid]
            vc = _fma(r, _fma(2.0, p, 1.0), -1.0)
            dd = _voxel_entry(q[idx], dr[idx], inv[idx], sgn[idx], vc, r)
            ok = dd != 0
            sel = idx[ok]
            found[sel] = True
            pidx[sel] = lstart + pid[ok]
            cond[sel] = True
            ahead = sel[dd[ok] > 0]
            t[ahead] = (t[ahead] + dd[ok][dd[ok] > 0]).astype(f32)
            x[ahead] = _fma(dr[ahead], t[ahead, None], o[ahead])
        miss = active & ~found
        cond[miss] = False
        t[miss] = 100
        x[miss] = _fma(dr[miss], t[miss, None], o[miss])

    walk(has, o)
    for _ in range(num_steps):
        act = np.flatnonzero(cond)
        if act.size == 0:
            break
        d = decode_fn(decs[lod], x[act], features(m, lod, pidx[act], x[act]))
        t[act] = (t[act] + d).astype(f32)
        h = (np.abs(d).astype(np.float64) < 0.0003) | (np.abs((d + dprev[act]).astype(f32)).astype(np.float64) * 0.5
                                                       < 0.0015)
        hit[act] = h
        cond[act] = (t[act].astype(np.float64) < 5.0) & ~h
        x[act] = _fma(dr[act], t[act, None], o[act])
        dprev[act] = d
        walk(cond.copy(), x)
    normal = np.ones((n, 3), f32)
    hi = np.flatnonzero(hit)
    if hi.size:
        for k in range(3):
            e = np.zeros(3, f32)
            e[k] = f32(0.001)
            xf = (x[hi] + e).astype(f32)
            xb = (x[hi] - e).astype(f32)
            df = decode_fn(decs[lod], xf, features(m, lod, pidx[hi], xf))
            db = decode_fn(decs[lod], xb, features(m, lod, pidx[hi], xb))
            normal[hi, k] = (df - db).astype(f32)
        nrm = np.sqrt((normal[hi].astype(np.float64) ** 2).sum(1)).astype(f32)
        normal[hi] = (normal[hi] / nrm[:, None]).astype(f32)
    return x, t[:, None], hit, normal
