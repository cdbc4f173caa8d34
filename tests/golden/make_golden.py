"""Generates the golden fixtures in tests/golden/ by running the reference's own
Python code (sdf-net/lib) on seeded synthetic inputs, on the CPU.

    python tests/golden/make_golden.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to /root/reference (the read-only checkout of
nv-tlabs/nglod).  Modules the reference imports but the hot path does not use
(mesh2sdf, polyscope, PIL, cv2, tinyobjloader) are stubbed; the CUDA-only
``sol_nglod.aabb`` is replaced by the bit-exact C restatement in
oracle/nglod_oracle.c, and ``PerfTimer`` (which creates CUDA events) by a
no-op.  Everything else -- OctreeSDF.sdf, SphereTracer.forward,
diffutils.gradient, autograd through grid_sample, spc3d.SPC3D,
geoutils.unique_corners -- is the reference's code.

Fixtures:
  dense_small.npz  OctreeSDF(num_lods=3, base_lod=1, C=32, H=128, seed 0):
                   sdf at every lod, lod=None, lod >= num_lods, return_lst;
                   parameter gradients of the 3-LOD L2 training loss.
  trace_small.npz  OctreeSDF(num_lods=2, base_lod=3) set to a sphere-union SDF
                   plus noise; SphereTracer.forward on 40x40 camera rays and
                   edge-case rays, lod None and 0.
  spc_small.npz    SPC3D octree of level 5 built from the voxels near the
                   sphere-union surface: Morton codes, octree bytes, pyramid,
                   decoded points; unique_corners of levels 2..5.
  mesh_small.npz   torchgp.normalize, per_face_normals and point_sample
                   (['trace', 'near', 'rand'], torch seed 3) on a procedural
                   icosphere.
  sol_export_small.npz  SOL_NGLOD(net).save() (sdf-net/lib/models/SOL_NGLOD.py:31-100)
                   on trace_small's construction at num_lods=3, base_lod=2: the
                   reference's own sparse export (octree, cc, cf, w0, b0, w1,
                   b1, pyramid), which sol-renderer's SDF::loadWeights reads.
                   As shipped, SOL_NGLOD's voxel_sparsify -> sample_surface
                   builds SphereTracer(device, sol=sol) (renderutils.py:33),
                   which raises TypeError (BaseTracer has no ``sol``
                   argument); the generator gives renderutils a factory that
                   builds the reference SphereTracer from parsed options
                   instead, and runs sample_surface on the CPU.  Everything
                   else in the export runs unchanged.
  get_min_small.npz  SphereTracer.get_min on trace_small's network and rays
                   (lod None): x, depth, hit, unnormalised normals and min_x.
                   As shipped, get_min's last line passes ``minx=`` to
                   RenderBuffer, whose field is ``min_x``, and raises
                   TypeError; the generator maps the keyword.
  shade_small.npz  Renderer.shade_tensor with a ground plane, shadow rays and
                   ambient occlusion on trace_small's network, 48x40 rays,
                   matcap shading with nglod_gb300.synthetic.matcap_texture
                   (served through the stubbed PIL.Image.open), shadow-ray
                   noise from torch.manual_seed(7); torch.Tensor.cuda is made
                   a no-op for the call (the reference moves its images to the
                   GPU).
"""
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from nglod_gb300 import synthetic  # noqa: E402
from nglod_gb300.analytic_init import init_from_sdf  # noqa: E402
from nglod_gb300.octree_sdf import OctreeSDF as DropIn  # noqa: E402
from nglod_gb300.options import default_args  # noqa: E402
from oracle import cref  # noqa: E402


class _NoTimer:
    def __init__(self, *a, **k):
        pass

    def check(self, *a, **k):
        return None

    def reset(self):
        pass


def _cpu_aabb(ray_o, ray_d):
    x, t, hit = cref.aabb(ray_o.detach().float().numpy(), ray_d.detach().float().numpy())
    dt = ray_o.dtype
    return [torch.from_numpy(x).to(dt), torch.from_numpy(t).to(dt), torch.from_numpy(hit)]


def import_reference(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "sdf-net"))
    for name in ["mesh2sdf", "polyscope", "cv2", "tinyobjloader"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    pil = types.ModuleType("PIL")
    pil.Image = types.ModuleType("PIL.Image")
    sys.modules["PIL"] = pil
    sys.modules["PIL.Image"] = pil.Image
    sol = types.ModuleType("sol_nglod")
    sol.aabb = _cpu_aabb
    sys.modules["sol_nglod"] = sol
    import lib.utils
    lib.utils.PerfTimer = _NoTimer
    from lib.models.OctreeSDF import OctreeSDF
    import lib.tracer.SphereTracer  # noqa: F401
    ST = sys.modules["lib.tracer.SphereTracer"]
    ST.PerfTimer = _NoTimer
    from lib.options import parse_options
    from lib import spc3d, geoutils
    return OctreeSDF, ST.SphereTracer, parse_options, spc3d, geoutils


def ref_args(parse_options, **kw):
    argv = ["--net", "OctreeSDF"]
    for k, v in kw.items():
        flag = "--" + k.replace("_", "-")
        if isinstance(v, bool):
            if v:
                argv.append(flag)
        elif isinstance(v, (list, tuple)):
            argv += [flag] + [str(u) for u in v]
        else:
            argv += [flag, str(v)]
    return parse_options(return_parser=True).parse_args(argv)


def dense_small(OctreeSDF, parse_options):
    args = ref_args(parse_options, num_lods=3, base_lod=1, feature_dim=32, hidden_dim=128)
    torch.manual_seed(0)
    net = OctreeSDF(args)
    g = torch.Generator().manual_seed(11)
    pts = torch.rand((600, 3), generator=g) * 2.2 - 1.1
    special = torch.tensor([[-1, -1, -1], [1, 1, 1], [0, 0, 0], [1, -1, 0.5], [-1.5, 0.25, 2.0],
                            [0.5, 0.5, 0.5], [-0.5, 1.0, -0.25], [0.999999, -0.999999, 1e-7]], dtype=torch.float32)
    pts = torch.cat([pts, special])
    out = {"points": pts.numpy()}
    net.eval()
    with torch.no_grad():
        for lod in [0, 1, 2]:
            out[f"sdf_lod{lod}"] = net.sdf(pts, lod=lod).numpy()
        out["sdf_lodNone"] = net.sdf(pts).numpy()
        out["sdf_lod7"] = net.sdf(pts, lod=7).numpy()
        out["sdf_lst"] = np.stack([t.numpy() for t in net.sdf(pts, return_lst=True)])
        net.lod = 1
        out["forward_lod1"] = net(pts).numpy()
        net.lod = None
    for k, v in net.state_dict().items():
        out["param/" + k] = v.numpy()
    # Training loss of Trainer.step_geometry (trainer.py:317-339) over all LODs.
    c, r = synthetic.sphere_union(1)
    gts = torch.from_numpy(synthetic.sphere_union_sdf(pts.numpy(), c, r)).float()[:, None]
    net.train()
    net.zero_grad()
    loss = 0
    for lod in [0, 1, 2]:
        loss = loss + ((net.sdf(pts, lod=lod) - gts) ** 2).sum()
    loss = loss / pts.shape[0]
    loss.backward()
    out["train/gts"] = gts.numpy()
    out["train/loss"] = np.array(loss.item())
    for k, p in net.named_parameters():
        out["grad/" + k] = p.grad.numpy()
    np.savez_compressed(os.path.join(HERE, "dense_small.npz"), **out)


def trace_small_net(OctreeSDF, parse_options, **extra):
    args = ref_args(parse_options, num_lods=2, base_lod=3, feature_dim=32, hidden_dim=128, num_steps=64,
                    min_dis=0.0003, step_size=1.0, camera_clamp=[-5, 10], grad_method="finitediff", **extra)
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    dropin = DropIn(default_args(num_lods=2, base_lod=3))
    init_from_sdf(dropin, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=2e-3,
                  seed=5)
    with torch.no_grad():
        for fv in dropin.features:
            fv.fm[:, 4:] = 0  # keep the fixtures small: noise in channels 1-3 only
    net = OctreeSDF(args)
    net.load_state_dict(dropin.state_dict())
    return net.eval(), args


def trace_small(OctreeSDF, SphereTracer, parse_options):
    net, args = trace_small_net(OctreeSDF, parse_options)
    ro, rd = synthetic.look_at_rays(width=40, height=40)
    extra_o = torch.tensor([[0, 0, 0], [0.5, 0.2, -0.3], [3, 3, 3], [0, 0, 4], [1, 0, 0], [0, 2, 0],
                            [-0.2, 0.1, 1.0]], dtype=torch.float32)
    extra_d = torch.tensor([[1, 0, 0], [0, 0, 1], [1, 0, 0], [0, 0, -1], [-1, 0, 0], [0, -1, 0],
                            [0, 0, -1]], dtype=torch.float32)
    ro = torch.cat([ro, extra_o])
    rd = torch.cat([rd, extra_d])
    out = {"ray_o": ro.numpy(), "ray_d": rd.numpy()}
    tracer = SphereTracer(args)
    for name, lod in [("lodNone", None), ("lod0", 0)]:
        net.lod = lod
        rb = tracer(net, ro, rd)
        out[f"{name}/x"] = rb.x.detach().numpy()
        out[f"{name}/depth"] = rb.depth.detach().numpy()
        out[f"{name}/hit"] = rb.hit.numpy()
        out[f"{name}/normal"] = rb.normal.detach().numpy()
    net.lod = None
    for k, v in net.state_dict().items():
        out["param/" + k] = v.numpy()
    out["trace/num_steps"] = np.array(64)
    np.savez_compressed(os.path.join(HERE, "trace_small.npz"), **out)


def get_min_small(OctreeSDF, SphereTracer, parse_options):
    """SphereTracer.get_min on trace_small's network and rays (lod None).  As
    shipped, get_min ends with RenderBuffer(..., minx=minx), a keyword the
    reference's RenderBuffer does not have (its field is min_x), and raises
    TypeError; the generator gives the tracer module a RenderBuffer factory
    that takes ``minx`` as ``min_x``.  The march itself runs unchanged."""
    ST = sys.modules["lib.tracer.SphereTracer"]
    RB = ST.RenderBuffer
    net, args = trace_small_net(OctreeSDF, parse_options)
    ro, rd = synthetic.look_at_rays(width=40, height=40)
    extra_o = torch.tensor([[0, 0, 0], [0.5, 0.2, -0.3], [3, 3, 3], [0, 0, 4], [1, 0, 0], [0, 2, 0],
                            [-0.2, 0.1, 1.0]], dtype=torch.float32)
    extra_d = torch.tensor([[1, 0, 0], [0, 0, 1], [1, 0, 0], [0, 0, -1], [-1, 0, 0], [0, -1, 0],
                            [0, 0, -1]], dtype=torch.float32)
    ro = torch.cat([ro, extra_o])
    rd = torch.cat([rd, extra_d])
    ST.RenderBuffer = lambda minx=None, **k: RB(min_x=minx, **k)
    try:
        rb = SphereTracer(args).get_min(net, ro, rd)
    finally:
        ST.RenderBuffer = RB
    out = {"ray_o": ro.numpy(), "ray_d": rd.numpy(), "x": rb.x.detach().numpy(),
           "depth": rb.depth.detach().numpy(), "hit": rb.hit.numpy(), "normal": rb.normal.detach().numpy(),
           "min_x": rb.min_x.detach().numpy(), "num_steps": np.array(int(args.num_steps))}
    np.savez_compressed(os.path.join(HERE, "get_min_small.npz"), **out)


def shade_small(OctreeSDF, SphereTracer, parse_options):
    import lib.renderer as R
    W, H = 48, 40
    net, args = trace_small_net(OctreeSDF, parse_options, render_res=[W, H], shadow=True, ao=True,
                                ground_height=-0.7, shading_mode="matcap", matcap_path="synthetic")
    tex = synthetic.matcap_texture(64)
    sys.modules["PIL.Image"].open = lambda path: tex
    R.PerfTimer = _NoTimer
    ro, rd = synthetic.look_at_rays(eye=(1.2, 1.6, 3.2), at=(0.0, -0.2, 0.0), width=W, height=H, fov=40.0)
    tracer = SphereTracer(args)
    renderer = R.Renderer(tracer, args=args)
    renderer.render_lookat = lambda net_, f=None, t=None, fov=None, camera_proj=None, device=None, mm=None: \
        renderer.render(net_, ro, rd)
    cuda = torch.Tensor.cuda
    torch.Tensor.cuda = lambda self, *a, **k: self
    try:
        torch.manual_seed(7)
        rb = renderer.shade_tensor(net)
    finally:
        torch.Tensor.cuda = cuda
    torch.manual_seed(7)
    noise = torch.zeros(W * H, 3).normal_(0.0, 0.01)
    out = {"ray_o": ro.numpy(), "ray_d": rd.numpy(), "noise": noise.numpy(), "matcap": tex,
           "ground_height": np.array(-0.7, np.float32), "width": np.array(W), "height": np.array(H)}
    for k in ("x", "depth", "hit", "normal", "rgb", "shadow", "ao", "relative_depth"):
        v = getattr(rb, k)
        out[k] = v.detach().numpy().reshape(W * H, -1)
    # the network's parameters are trace_small.npz's (same construction)
    np.savez_compressed(os.path.join(HERE, "shade_small.npz"), **out)


def mesh_small():
    """The reference's torchgp normalize, per_face_normals and point_sample on
    a procedural icosphere (the reference's meshes are not distributed)."""
    from lib.torchgp import normalize, per_face_normals, point_sample
    V, F = synthetic.icosphere(2, radius=0.8, centre=(0.1, -0.05, 0.2))
    V = torch.from_numpy(V).float()
    F = torch.from_numpy(F)
    Vn, Fn = normalize(V, F)
    torch.manual_seed(3)
    pts = point_sample(Vn, Fn, ["trace", "near", "rand"], 300)
    out = {"V": V.numpy(), "F": F.numpy(), "V_normalized": Vn.numpy(), "face_normals": per_face_normals(Vn, Fn).numpy(),
           "point_sample": pts.numpy()}
    np.savez_compressed(os.path.join(HERE, "mesh_small.npz"), **out)


def sol_export_small(OctreeSDF, SphereTracer, parse_options):
    """SOL_NGLOD(net).save() of a 3-LOD network (base_lod 2) holding the
    sphere-union SDF, run on the CPU."""
    import lib.renderutils as RU
    from lib.models.SOL_NGLOD import SOL_NGLOD
    targs = ref_args(parse_options, num_lods=3, base_lod=2, num_steps=64, min_dis=0.0003, step_size=1.0,
                     camera_clamp=[-5, 10], grad_method="finitediff")
    RU.SphereTracer = lambda device, sol=False: SphereTracer(targs)
    RU.sample_surface.__defaults__ = (False, "cpu")
    RU.voxel_sparsify.__defaults__ = (False, "cpu")
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    dropin = DropIn(default_args(num_lods=3, base_lod=2))
    init_from_sdf(dropin, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=2e-3,
                  seed=6)
    with torch.no_grad():
        for fv in dropin.features:
            fv.fm[:, 4:] = 0  # keep the fixture small: noise in channels 1-3 only
    net = OctreeSDF(targs)
    net.load_state_dict(dropin.state_dict())
    net.eval()
    torch.manual_seed(13)  # sample_surface's random rays
    sol = SOL_NGLOD(net)
    sol.save(os.path.join(HERE, "sol_export_small.npz"))


def coded_volume(s, channels=2):
    c = torch.arange(channels, dtype=torch.float64).view(channels, 1, 1, 1)
    z = torch.arange(s, dtype=torch.float64).view(1, s, 1, 1)
    y = torch.arange(s, dtype=torch.float64).view(1, 1, s, 1)
    x = torch.arange(s, dtype=torch.float64).view(1, 1, 1, s)
    return (c * 1e6 + z * 1e4 + y * 1e2 + x)[None]


def order_table(ref_root):
    """The Order[8][8] child-order table of spc_raytrace_cuda_kernel.cu, read
    from the source text."""
    import re
    path = os.path.join(ref_root, "sol-renderer", "include", "spc", "spc", "spc_raytrace_cuda_kernel.cu")
    text = open(path).read()
    body = text[text.index("Order[8][8]"):]
    body = body[body.index("{") + 1:body.index("};")]
    rows = re.findall(r"\{([^{}]*)\}", body)
    return np.array([[int(v) for v in r.split(",")] for r in rows], dtype=np.uint8)


def spc_small(spc3d, geoutils, ref_root):
    level = 5
    res = 2 ** level
    c, r = synthetic.sphere_union(1)
    idx = np.stack(np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing="ij"), -1).reshape(-1, 3)
    centres = (idx + 0.5) / res * 2 - 1
    keep = np.abs(synthetic.sphere_union_sdf(centres, c, r)) <= np.sqrt(3) * (2.0 / res)
    vox = idx[keep].astype(np.uint16)
    spc = spc3d.SPC3D(level)
    for i in range(vox.shape[0]):
        spc.mdata[i] = spc3d.to_morton(vox[i])
        spc.psize += 1
    spc.mdata[:spc.psize] = np.sort(spc.mdata[:spc.psize])
    morton = spc.mdata[:spc.psize].copy()
    spc.morton_to_point(spc.psize, spc.mdata, spc.pdata)
    points_sorted = spc.pdata[:spc.psize].copy()
    osize = spc.points_to_nodes()
    octree = spc.oroot[:osize].copy()
    pyramid = spc.pyramid[:level + 1].copy()
    pyramid_sum = spc.pyramid_sum[:level + 1].copy()
    dec = spc3d.SPC3D(level, nodebytes=octree.copy())
    npts = dec.nodes_to_points()
    out = {"order_table": order_table(ref_root),
           "voxels": vox, "morton": morton, "points_sorted": points_sorted, "octree": octree,
           "pyramid": pyramid, "pyramid_sum": pyramid_sum, "decoded_leaf_points": dec.pdata[:npts].copy(),
           "decoded_pyramid": dec.pyramid[:level + 1].copy(), "level": np.array(level)}
    # unique_corners of each octree level's voxels (geoutils.py:60-77).  The
    # feature volume encodes its own index, fm[0, c, z, y, x] =
    # c*1e6 + z*1e4 + y*1e2 + x, so cf pins the gather order exactly.
    for lv in range(2, level + 1):
        shift = level - lv
        vs = torch.unique(torch.from_numpy(points_sorted.astype(np.int64)) >> shift, dim=0)
        out[f"corners/{lv}/voxels"] = vs.numpy()
        corners, feats = geoutils.unique_corners(vs, coded_volume(2 ** lv + 1))
        out[f"corners/{lv}/cc"] = corners.numpy()
        out[f"corners/{lv}/cf"] = feats.numpy()
    np.savez_compressed(os.path.join(HERE, "spc_small.npz"), **out)


def main():
    """make_golden.py [REFERENCE_ROOT [FIXTURE ...]]: all fixtures, or only the
    named ones (e.g. get_min_small)."""
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    only = set(sys.argv[2:])
    OctreeSDF, SphereTracer, parse_options, spc3d, geoutils = import_reference(ref_root)
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    jobs = [("dense_small", lambda: dense_small(OctreeSDF, parse_options)),
            ("trace_small", lambda: trace_small(OctreeSDF, SphereTracer, parse_options)),
            ("get_min_small", lambda: get_min_small(OctreeSDF, SphereTracer, parse_options)),
            ("spc_small", lambda: spc_small(spc3d, geoutils, ref_root)),
            ("shade_small", lambda: shade_small(OctreeSDF, SphereTracer, parse_options)),
            ("mesh_small", mesh_small),
            ("sol_export_small", lambda: sol_export_small(OctreeSDF, SphereTracer, parse_options))]
    for name, job in jobs:
        if not only or name in only:
            job()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
