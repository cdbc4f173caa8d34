"""Serving on the GPU: results in a concurrent mix equal the same requests
run alone (bitwise), HBM budget respected, requests overlap."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import serve, synthetic
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.bf16 import Bf16OctreeSDF
from nglod_gb300.options import default_args

pytestmark = pytest.mark.gpu


def _model(seed, dev):
    c, r = synthetic.sphere_union(seed)
    torch.manual_seed(seed)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=seed)
    return net.to(dev).eval()


def test_mixed_requests_equal_alone(cuda):
    f32 = _model(2, cuda)
    # a per-LOD BF16 model, a LOD-summed BF16 model and a float32 model
    models = [Bf16OctreeSDF(f32), Bf16OctreeSDF(_model(3, cuda), summed=True), f32]
    ex = serve.CudaExecutor(models, cuda, num_streams=4)
    budget = serve.RenderRequest(0, 160, 120).nbytes() * 3
    srv = serve.Server(ex, budget)
    reqs = []
    rng = np.random.default_rng(0)
    for i in range(18):
        m = i % 3
        if i % 2 == 0:
            w, h = [(96, 64), (160, 120), (64, 64)][i % 3]
            reqs.append(serve.RenderRequest(m, w, h, lod=int(rng.integers(5)), eye=(0.3 * (i % 4), 0.2, 4.0)))
        else:
            pts = torch.rand(int(rng.integers(1000, 60000)), 3, device=cuda) * 2 - 1
            reqs.append(serve.QueryRequest(m, pts, lod=int(rng.integers(5))))
    tks = [srv.submit(r) for r in reqs]
    assert srv.drain(timeout=120)
    assert srv.peak_used <= budget
    assert srv.max_concurrent >= 2
    for tk in tks:
        r = tk.request
        model = models[r.model]
        if isinstance(r, serve.RenderRequest):
            alone = serve.Server(serve.CudaExecutor(models, cuda, num_streams=1), 1 << 28)
            t2 = alone.submit(serve.RenderRequest(r.model, r.width, r.height, r.lod, eye=r.eye))
            assert alone.drain(timeout=60)
            alone.close()
            for k in ("x", "depth", "hit", "normal"):
                assert torch.equal(getattr(tk.result, k), getattr(t2.result, k)), k
            assert tk.result.hit.any()
        else:
            with torch.no_grad():  # the inference kernels, as the server runs them
                ref = model.sdf(r.points, lod=r.lod)
            assert torch.equal(tk.result, ref)
    st = srv.stats()
    assert st["requests"] == len(reqs) and st["p99_ms"] is not None and st["failed"] == 0
    info = srv.info()
    assert info["used_bytes"] == 0 or info["held"] == 0
    srv.close()


def test_native_server_through_the_c_abi(cuda):
    """The nglod_serve_* calls used directly, as a C caller would: submit a
    render and a query, poll until both finish, read results in the pool,
    release, destroy; the results equal the direct kernel calls."""
    import ctypes
    from nglod_gb300 import _lib
    lib = _lib.load()
    net = _model(4, cuda)
    b = Bf16OctreeSDF(net)
    h = ctypes.c_void_p()
    cfg = _lib.ServeConfig(64 << 20, 2, 0)
    _lib.check(lib.nglod_serve_start(ctypes.byref(cfg), ctypes.byref(h)), "start")
    mid = ctypes.c_int32()
    _lib.check(lib.nglod_serve_add_model_bf16(h, ctypes.byref(b._m), ctypes.byref(mid)), "add")
    ex = serve.CudaExecutor([b], cuda, 2)
    rr = serve.RenderRequest(mid.value, 64, 48, lod=3).native(ex.trace_params())
    pts = torch.rand(5000, 3, device=cuda) * 2 - 1
    qr = serve.QueryRequest(mid.value, pts, lod=2).native(pts.data_ptr())
    qr.has_ready_stream = 1
    qr.ready_stream = torch.cuda.current_stream().cuda_stream
    ids = [ctypes.c_int64(), ctypes.c_int64()]
    _lib.check(lib.nglod_serve_submit(h, ctypes.byref(rr), -1.0, ctypes.byref(ids[0])), "submit")
    _lib.check(lib.nglod_serve_submit(h, ctypes.byref(qr), -1.0, ctypes.byref(ids[1])), "submit")
    out = {}
    res = (_lib.ServeResult * 4)()
    cnt = ctypes.c_int32()
    import time
    t0 = time.monotonic()
    while len(out) < 2 and time.monotonic() - t0 < 30:
        _lib.check(lib.nglod_serve_poll(h, res, 4, ctypes.byref(cnt)), "poll")
        for r in res[:cnt.value]:
            assert r.status == 0 and r.t_submit <= r.t_admit <= r.t_done
            if r.kind == _lib.SERVE_QUERY:
                out["q"] = serve._pool_tensor(r.sdf, (r.units, 1), "<f4", cuda)
            else:
                out["t"] = serve._pool_tensor(r.t, (r.units, 1), "<f4", cuda)
            _lib.check(lib.nglod_serve_release(h, r.ticket, 1, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                       "release")
    assert len(out) == 2
    assert torch.equal(out["q"], b.sdf(pts, lod=2))
    ro, rd = torch.empty(64 * 48, 3, device=cuda), torch.empty(64 * 48, 3, device=cuda)
    e, a, u = (np.asarray(v, np.float32) for v in ((0, 0, 4), (0, 0, 0), (0, 1, 0)))
    _lib.check(lib.nglod_camera_rays(e.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                                     u.ctypes.data_as(ctypes.c_void_p), 30.0, 64, 48, _lib.ptr(ro), _lib.ptr(rd),
                                     _lib.stream_ptr(cuda)), "rays")
    b.lod = 3
    import nglod_gb300 as ng2
    direct = ng2.SphereTracer(ex.tracer_args, num_steps=64)(b, ro, rd)
    b.lod = None
    assert torch.equal(out["t"], direct.depth)
    unfinished, dropped = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(lib.nglod_serve_stop(h, 1.0, ctypes.byref(unfinished), ctypes.byref(dropped)), "stop")
    assert unfinished.value == 0 and dropped.value == 0
    _lib.check(lib.nglod_serve_destroy(h), "destroy")


def test_camera_rays_match_look_at(cuda):
    from nglod_gb300 import _lib
    import ctypes
    W, H = 37, 21
    org = torch.empty(W * H, 3, device=cuda)
    dr = torch.empty(W * H, 3, device=cuda)
    e = np.array([0.5, 1.0, 3.5], np.float32)
    a = np.zeros(3, np.float32)
    u = np.array([0, 1, 0], np.float32)
    _lib.check(_lib.load().nglod_camera_rays(e.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                                             u.ctypes.data_as(ctypes.c_void_p), 35.0, W, H, _lib.ptr(org),
                                             _lib.ptr(dr), _lib.stream_ptr(cuda)), "nglod_camera_rays")
    ro, rd = synthetic.look_at_rays(eye=tuple(e), width=W, height=H, fov=35.0)
    assert (dr.cpu() - rd).abs().max().item() < 1e-5
    assert (org.cpu() - ro).abs().max().item() == 0
