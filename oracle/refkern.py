"""The reference's own CUDA kernels, run on the GPU as the oracle of the native rows
(TEST INFRASTRUCTURE ONLY: used by tests/ and never by the nglod_gb300 package).

The cubins in ``oracle/_ref/`` are the reference sources compiled unchanged
(``oracle/ref_build.py``).  This module loads them with the CUDA driver API
(``cuModuleLoad`` into the context torch made current) and launches their
kernels on torch's current stream with the reference's own grid shapes.  The
reference's HOST code needs libtorch, CUB and (for the viewer) GL, none of
which can be linked here, so the host steps around the kernels are restated
below, each citing the lines it follows.  Where the reference calls CUB's
DeviceScan, an integer ``torch.cumsum`` computes the same prefix sums; where
it calls ``torch::addmm``, ``torch.addmm`` is the same cuBLAS call.

    aabb(ray_o, ray_d)                          sol_nglod.aabb (sol_nglod_kernel.cu:155-188)
    spc_raytrace(octree, points, pyramid, ...)  spc_raytrace (spc_raytrace_cuda.cpp:141-199,
                                                spc_raytrace_cuda_kernel.cu:194-265)
    generate_rays(M, W, H)                      generate_primary_rays_cuda (spc_raytrace_cuda_kernel.cu:271-296)
    SdfRef(npz, octree points, pyramid)         SDF::loadWeights / initTrinkets / sphereTrace /
                                                getNormal (sol-renderer/SDF.cu:65-472)

Bounds are checked here, on the host, before each launch: every index a
kernel forms stays inside the buffers it is given (the one place the
reference reads past a buffer, ``d_Decide``'s ``D[offset + pidx]`` at the
octree's leaf level, gets a buffer padded to the point count; the value read
there is unused).
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import ref_build

# Mangled entry names, as ptxas reported them for the reference sources.
AABB_F32 = "_Z11aabb_kernelIfEvPKT_S2_PS0_S3_Pbi"
SCAN_NODES = "_Z12d_ScanNodesAjPKhPj"
INIT_NUGGETS = "_Z13d_InitNuggetsjP5uint2"
DECIDE = "_Z8d_DecidejP6short4P6float3S2_P5uint2PjS5_jjj"
SUBDIVIDE = "_Z11d_SubdividejP5uint2S0_P6float3P6short4PhPjS6_S6_jjj"
COMPACTIFY = "_Z12d_CompactifyjP5uint2S0_PjS1_"
GENERATE_RAYS = "_Z15d_generate_raysjjj8float4x4P6float3S1_"
INDEX_TRINKET = "_ZN4solr20index_trinket_kernelEPK7ushort4PKiPKfPNS_7TrinketEiiiiiii"
SPARSE_SAMPLE = "_ZN4solr25sparse_grid_sample_kernelEPKfPKiS3_PKNS_7TrinketES1_PKjS8_PfiiiiiS3_"
STEP = "_ZN4solr11step_kernelEPKfS1_PKiS1_PfS4_S4_S4_PbS5_i"
RAY_AABB_NUGGETS = "_ZN4solr15ray_aabb_kernelEPKfS1_S1_S1_PK5uint2PKsPKiS8_fbPfS9_PbPiii"
NORMALIZE = "_ZN4solr16normalize_kernelEPKiPfi"

MAX_LEVELS = 15  # spc_math.h:31
TRINKET_WORDS = 9  # solr::Trinket {uint v[8]; int parent;} (util_structs.cuh:33-37)


class _Float4x4(ctypes.Structure):
    _fields_ = [("m", ctypes.c_float * 16)]


class _Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        vp, u32 = ctypes.c_void_p, ctypes.c_uint
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [vp, u32, u32, u32, u32, u32, u32, u32, vp, ctypes.POINTER(vp), vp]
        self.cu.cuCtxGetCurrent.argtypes = [ctypes.POINTER(vp)]
        self.cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        self.modules = {}
        self.functions = {}

    def check(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else '?'})")

    def function(self, module, name):
        key = (module, name)
        if key in self.functions:
            return self.functions[key]
        torch.zeros(1, device="cuda")  # torch's context is created and current
        ctx = ctypes.c_void_p()
        self.check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context for the reference kernels")
        if module not in self.modules:
            path = ref_build.cubin_path(module)
            if not os.path.exists(path):
                raise RuntimeError(f"reference cubin {path} missing: run oracle.ref_build where the reference "
                                   "checkout is present")
            mod = ctypes.c_void_p()
            self.check(self.cu.cuModuleLoad(ctypes.byref(mod), path.encode()), f"cuModuleLoad {module}")
            self.modules[module] = mod
        fn = ctypes.c_void_p()
        self.check(self.cu.cuModuleGetFunction(ctypes.byref(fn), self.modules[module], name.encode()),
                   f"cuModuleGetFunction {name}")
        self.functions[key] = fn
        return fn

    def launch(self, module, name, grid, block, args):
        """args: ctypes scalars / structures, kept alive for the call."""
        if grid <= 0:
            return
        fn = self.function(module, name)
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.check(self.cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, stream, ptrs, None), f"launch {name}")


_DRV = None


def driver():
    global _DRV
    if _DRV is None:
        _DRV = _Driver()
    return _DRV


def available():
    return ref_build.available()


def entries():
    with open(ref_build.manifest_path()) as f:
        return json.load(f)["kernels"]


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _u32(v):
    return ctypes.c_uint(int(v))


def _i32(v):
    return ctypes.c_int(int(v))


def _dev(*ts):
    for t in ts:
        if not (t.is_cuda and t.is_contiguous()):
            raise ValueError("reference kernels take contiguous CUDA tensors")


# ---------------------------------------------------------------------------------------------
# sol_nglod.aabb


def aabb(ray_o, ray_d):
    """f_aabb (sol_nglod_kernel.cu:155-188): x = ray_o.clone(), t = 0 [N,1],
    hit = False, then aabb_kernel<float> with 256-thread blocks."""
    _dev(ray_o, ray_d)
    assert ray_o.dtype == torch.float32 and ray_o.shape == ray_d.shape and ray_o.shape[1] == 3
    n = ray_o.shape[0]
    x = ray_o.clone()
    hit = torch.zeros(n, dtype=torch.bool, device=ray_o.device)
    t = torch.zeros(n, 1, dtype=torch.float32, device=ray_o.device)
    driver().launch("sol_nglod", AABB_F32, (n + 255) // 256, 256,
                    [_p(ray_o), _p(ray_d), _p(x), _p(t), _p(hit), _i32(n)])
    return x, t, hit


# ---------------------------------------------------------------------------------------------
# spc_raytrace


def spc_raytrace(octree, points, pyramid, org, dir, target_level, capacity=1 << 26):
    """spc_raytrace (spc_raytrace_cuda.cpp:141-199) around the reference's
    traversal kernels (spc_raytrace_cuda_kernel.cu:194-265).  ``capacity``
    stands for MAX_TOTAL_POINTS (2^27 nuggets per buffer in the reference);
    a level whose nugget count exceeds it raises instead of truncating."""
    _dev(octree, points, org, dir)
    assert octree.dtype == torch.uint8 and points.dtype == torch.int16 and points.shape[1] == 4
    pyr = pyramid.cpu().to(torch.int32).contiguous()
    assert pyr.dim() == 2 and pyr.shape[0] == 2
    level = pyr.shape[1] - 2
    assert level < MAX_LEVELS
    h = pyr.flatten().numpy().astype(np.int64)
    psum = h[level + 2:]
    osize, psize = int(h[2 * level + 2]), int(h[2 * level + 3])
    if octree.shape[0] != osize or points.shape[0] != psize:
        raise ValueError("bad spc octree or points size")
    if not (0 <= target_level <= level):
        raise ValueError("target level outside the octree")
    dev = octree.device
    num = org.shape[0]
    if num > capacity:
        raise ValueError("more rays than nugget capacity")
    # D (popcounts) and S (their exclusive sum): osize entries in the reference; padded to psize so
    # that d_Decide's read of D[PyramidSum[Level] + pidx] at the leaf level stays inside the buffer.
    D = torch.zeros(psize, dtype=torch.int32, device=dev)
    S = torch.zeros(psize, dtype=torch.int32, device=dev)
    nug = torch.zeros(2, capacity, 2, dtype=torch.int32, device=dev)
    info = torch.zeros(capacity, dtype=torch.int32, device=dev)
    prefix = torch.zeros(capacity + 1, dtype=torch.int32, device=dev)
    drv = driver()
    drv.launch("spc_raytrace", SCAN_NODES, (osize + 1023) // 1024, 1024, [_u32(osize), _p(octree), _p(D)])
    S[:osize] = torch.cumsum(D[:osize], 0, dtype=torch.int64).to(torch.int32) - D[:osize]
    drv.launch("spc_raytrace", INIT_NUGGETS, (num + 1023) // 1024, 1024, [_u32(num), _p(nug[0])])
    buf = 0
    cnt = 0
    pbase = points.data_ptr()
    for l in range(target_level + 1):
        proot = ctypes.c_void_p(pbase + int(psum[l]) * 8)
        drv.launch("spc_raytrace", DECIDE, (num + 1023) // 1024, 1024,
                   [_u32(num), proot, _p(org), _p(dir), _p(nug[buf]), _p(info), _p(D), _u32(l), _u32(psum[l]),
                    _u32(target_level - l)])
        prefix[1:num + 1] = torch.cumsum(info[:num], 0, dtype=torch.int64).to(torch.int32)
        cnt = int(prefix[num].item())
        if cnt == 0:
            return torch.zeros(0, 2, dtype=torch.int32, device=dev)
        if cnt > capacity:
            raise RuntimeError(f"level {l}: {cnt} nuggets exceed the capacity {capacity}")
        if l < target_level:
            drv.launch("spc_raytrace", SUBDIVIDE, (num + 1023) // 1024, 1024,
                       [_u32(num), _p(nug[buf]), _p(nug[1 - buf]), _p(org), proot, _p(octree), _p(S), _p(info),
                        _p(prefix), _u32(l), _u32(psum[l]), _u32(psum[l + 1])])
        else:
            drv.launch("spc_raytrace", COMPACTIFY, (num + 1023) // 1024, 1024,
                       [_u32(num), _p(nug[buf]), _p(nug[1 - buf]), _p(info), _p(prefix)])
        buf = 1 - buf
        num = cnt
    return nug[buf, :cnt].clone()


def generate_rays(M, width, height, device="cuda"):
    """generate_primary_rays_cuda (spc_raytrace_cuda_kernel.cu:271-296): the
    reference kernel d_generate_rays on a given float32 4x4 matrix (row-major,
    row-vector convention); returns [Org, Dir] float32 [W*H, 3]."""
    n = width * height
    org = torch.zeros(n, 3, device=device)
    dr = torch.zeros(n, 3, device=device)
    m = _Float4x4()
    for i, v in enumerate(np.asarray(M, dtype=np.float32).reshape(16)):
        m.m[i] = float(v)
    driver().launch("spc_raytrace", GENERATE_RAYS, (n + 1023) // 1024, 1024,
                    [_u32(n), _u32(width), _u32(height), m, _p(org), _p(dr)])
    return org, dr


def mark_unique_rays(nuggets):
    """d_MarkUniqueRays (sol-renderer/sdfRenderer.cu:108-120), restated in
    torch ops: info[0] = 1, info[i] = nuggets[i-1].x != nuggets[i].x.  The
    source file also includes the GL viewer's headers, so it is not compiled."""
    n = nuggets.shape[0]
    info = torch.zeros(n, dtype=torch.int32, device=nuggets.device)
    if n:
        info[0] = 1
        info[1:] = (nuggets[1:, 0] != nuggets[:-1, 0]).to(torch.int32)
    return info


# ---------------------------------------------------------------------------------------------
# sol-renderer's SDF class


class SdfRef:
    """sol-renderer's SDF class on the reference kernels.

    npz: the reference export's arrays (keys cc, cf, w0, b0, w1, b1, pyramid;
    SOL_NGLOD.save, sdf-net/lib/models/SOL_NGLOD.py:80-100).  points / pyramid:
    the SPC of the npz's octree (SPC::SetGeometry's output; any exact decode)."""

    def __init__(self, npz, points, pyramid, device="cuda"):
        self.dev = torch.device(device)
        # SDF::loadWeights (SDF.cu:65-141): float16 arrays -> float32 on the device; weights transposed
        h = lambda k: torch.from_numpy(np.asarray(npz[k]).astype(np.float16).astype(np.float32))
        w0, b0, w1, b1 = h("w0"), h("b0"), h("w1"), h("b1")
        self.w0 = [w0[i].to(self.dev).t() for i in range(w0.shape[0])]
        self.b0 = [b0[i].to(self.dev) for i in range(b0.shape[0])]
        self.w1 = [w1[i].to(self.dev).t() for i in range(w1.shape[0])]
        self.b1 = [b1[i].to(self.dev) for i in range(b1.shape[0])]
        self.cc = torch.from_numpy(np.asarray(npz["cc"]).astype(np.uint8).astype(np.int32)).to(self.dev).contiguous()
        self.cf = h("cf").to(self.dev).contiguous()
        self.pyramid_cf = [int(v) for v in np.asarray(npz["pyramid"]).reshape(-1)[: w0.shape[0]]]
        self.nl = len(self.w0)
        self._init_trinkets(points, pyramid)

    def _init_trinkets(self, points, pyramid):
        """SDF::initTrinkets (SDF.cu:143-216) with the arguments sdfRenderer.cpp:396-398 passes:
        the SPC's point count, level, per-level counts and points."""
        _dev(points)
        pyr = pyramid.cpu().to(torch.int64)
        level = pyr.shape[1] - 2
        if level != self.nl + 1:
            # initTrinkets reads pyramid_cf_cpu[level - 2] for every level >= 2
            raise ValueError(f"octree level {level} does not match {self.nl} LODs (needs {self.nl + 1})")
        counts = [int(v) for v in pyr[0, : level + 1]]
        psize = int(points.shape[0])
        self.points = points
        self.m_pyramid = torch.tensor(np.cumsum(counts), dtype=torch.int32, device=self.dev)  # [i] = PyramidSum[i+1]
        self.m_res = torch.tensor([4 * 2 ** i for i in range(level - 1)], dtype=torch.int32, device=self.dev)
        self.trinkets = torch.zeros(psize, TRINKET_WORDS, dtype=torch.int32, device=self.dev)
        mp = self.m_pyramid.cpu().numpy()
        offset_cf = 0
        for i in range(2, level + 1):
            parent_i = max(i - 1, 2)
            parent_offset = int(mp[parent_i - 1])
            offset = int(mp[i - 1])
            n = counts[i]
            assert offset + n <= psize and offset_cf + self.pyramid_cf[i - 2] <= self.cc.shape[0]
            driver().launch("sdf", INDEX_TRINKET, (n + 1023) // 1024, 1024,
                            [_p(points), _p(self.cc), _p(self.cf), _p(self.trinkets), _i32(self.pyramid_cf[i - 2]),
                             _i32(offset_cf), _i32(n), _i32(offset), _i32(counts[parent_i]), _i32(parent_offset),
                             _i32(i)])
            offset_cf += self.pyramid_cf[i - 2]

    def _sample(self, x, pidx, idxes, n, lod):
        xs = torch.zeros(n, self.cf.shape[1] + 3, device=self.dev)
        driver().launch("sdf", SPARSE_SAMPLE, (n + 127) // 128, 128,
                        [_p(x), _p(pidx), _p(idxes), _p(self.trinkets), _p(self.cf), _p(self.m_pyramid),
                         _p(self.m_res), _p(xs), _i32(n), _i32(self.cf.shape[0]), _i32(self.cf.shape[1]),
                         _i32(self.nl), _i32(lod), _p(self.cc)])
        return xs

    def _decode(self, xs, lod):
        xsw0 = torch.relu(torch.addmm(self.b0[lod], xs, self.w0[lod]))
        return torch.addmm(self.b1[lod], xsw0, self.w1[lod])

    def get_normal(self, x, pidx, hit, lod):
        """SDF::getNormal (SDF.cu:218-295)."""
        nr = x.shape[0]
        active = torch.nonzero(hit).to(torch.int32).contiguous()
        n = active.shape[0]
        normal = torch.ones(nr, 3, device=self.dev)
        eps = [torch.tensor(v, dtype=torch.float32, device=self.dev)
               for v in ([0.001, 0.0, 0.0], [0.0, 0.001, 0.0], [0.0, 0.0, 0.001])]
        for i in range(3):
            xf = (x + eps[i]).contiguous()
            xb = (x - eps[i]).contiguous()
            d = self._decode(self._sample(xf, pidx, active, n, lod), lod) - \
                self._decode(self._sample(xb, pidx, active, n, lod), lod)
            normal[hit, i] = d[:, 0]
        driver().launch("sdf", NORMALIZE, (n + 127) // 128, 128, [_p(active), _p(normal), _i32(n)])
        return normal

    def sphere_trace(self, ray_o, ray_d, nuggets, points, info, lod, march_iter=50):
        """SDF::sphereTrace (SDF.cu:297-472): [x, t, hit, normal].  points:
        int16 [P, 3] level-(lod+2) voxel coordinates (sdfRenderer.cu:220-222);
        info: first-nugget flags."""
        _dev(ray_o, ray_d, nuggets, points, info)
        assert points.dtype == torch.int16 and points.shape[1] == 3 and info.dtype == torch.int32
        nn = nuggets.shape[0]
        nr = ray_o.shape[0]
        x = ray_o.clone()
        t = torch.zeros(nr, 1, device=self.dev)
        d = torch.zeros(nr, 1, device=self.dev)
        dprev = torch.zeros(nr, 1, device=self.dev)
        ray_inv = (1.0 / ray_d).contiguous()
        pidx = torch.zeros(nr, 1, dtype=torch.int32, device=self.dev) - 1
        info_idxes = torch.nonzero(info)[:, 0].to(torch.int32).contiguous()
        n_iidx = info_idxes.shape[0]
        voxel_res = 2 ** (lod + 2)
        voxel_radius = ctypes.c_float(1.0 / voxel_res)
        cond = torch.zeros(nr, dtype=torch.bool, device=self.dev)
        hit = torch.zeros(nr, dtype=torch.bool, device=self.dev)
        if nn:
            assert int(nuggets[:, 0].max()) < nr and int(nuggets[:, 1].max()) < points.shape[0]
        drv = driver()

        def aabb(init, query, blocks):
            drv.launch("sdf", RAY_AABB_NUGGETS, (n_iidx + blocks - 1) // blocks, blocks,
                       [_p(ray_o), _p(ray_d), _p(ray_inv), _p(query), _p(nuggets), _p(points), _p(info),
                        _p(info_idxes), voxel_radius, ctypes.c_bool(init), _p(x), _p(t), _p(cond), _p(pidx),
                        _i32(nn), _i32(n_iidx)])

        aabb(True, ray_o, 256)
        for _ in range(march_iter):
            active = torch.nonzero(cond)[:, 0].to(torch.int32).contiguous()
            n_active = active.shape[0]
            if n_active == 0:
                break
            _d = self._decode(self._sample(x, pidx, active, n_active, lod), lod).contiguous()
            drv.launch("sdf", STEP, (n_active + 127) // 128, 128,
                       [_p(ray_o), _p(ray_d), _p(active), _p(_d), _p(x), _p(t), _p(d), _p(dprev), _p(cond), _p(hit),
                        _i32(n_active)])
            aabb(False, x, 128)
        normal = self.get_normal(x, pidx, hit, lod)
        return x, t, hit, normal
