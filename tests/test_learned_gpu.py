"""What training buys: the network trained on the GPU by the project's own
forward/backward kernels, against the random-init network (floor) and the
non-learned method of equal memory (the same five volumes holding samples of
the ground-truth SDF, no learned decoder), on SDF error and traced depth."""
import numpy as np
import pytest
import torch

import nglod_gb300 as ng
from nglod_gb300 import synthetic, trainer
from nglod_gb300.analytic_init import init_from_sdf
from nglod_gb300.options import default_args

pytestmark = pytest.mark.gpu


def _analytic_depth(ro, rd, c, r):
    """Exact first intersection of rays with the sphere union (inf if none)."""
    oc = ro[:, None, :] - c[None]
    b = (oc * rd[:, None, :]).sum(-1)
    cc = (oc * oc).sum(-1) - r[None] ** 2
    disc = b * b - cc
    t = -b - np.sqrt(np.maximum(disc, 0))
    t = np.where((disc >= 0) & (t > 0), t, np.inf)
    return t.min(axis=1)


def test_training_beats_floor_and_reports_nonlearned(cuda):
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(1)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2)).to(cuda).train()
    floor = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    floor.load_state_dict(net.state_dict())
    floor = floor.to(cuda).eval()
    opt = trainer.FusedAdam(net.parameters(), lr=1e-3)
    batches = [synthetic.training_batch(65536, c, r, seed=200 + k) for k in range(6)]
    batches = [(a.to(cuda), b.to(cuda)) for a, b in batches]
    losses = []
    for it in range(600):
        xb, gb = batches[it % len(batches)]
        losses.append(trainer.step_geometry(net, opt, xb, gb).item())
    net.eval()
    assert losses[-1] < 0.05 * losses[0], (losses[0], losses[-1])

    grid = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(grid, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=0.0)
    grid = grid.to(cuda).eval()

    q = synthetic.near_surface_query(65536, c, r, seed=9).to(cuda)
    gt = torch.from_numpy(synthetic.sphere_union_sdf(q.cpu().double().numpy(), c, r)).float().to(cuda)[:, None]
    with torch.no_grad():
        l1 = {name: (m.sdf(q, lod=4) - gt).abs().mean().item() for name, m in
              (("trained", net), ("random_init", floor), ("nonlearned_grid", grid))}
    ro, rd = synthetic.look_at_rays(width=96, height=96)
    truth = _analytic_depth(ro.numpy().astype(np.float64), rd.numpy().astype(np.float64), c, r)
    depth = {}
    for name, m in (("trained", net), ("random_init", floor), ("nonlearned_grid", grid)):
        rb = ng.SphereTracer(default_args(num_steps=128))(m, ro.to(cuda), rd.to(cuda))
        h = rb.hit.cpu().numpy() & np.isfinite(truth)
        err = np.abs(rb.depth.cpu().numpy()[:, 0] - truth)[h]
        depth[name] = (float(np.median(err)) if h.any() else float("inf"),
                       float((rb.hit.cpu().numpy() == np.isfinite(truth)).mean()))
    print("SDF L1 vs analytic:", l1, "| depth median error, hit agreement:", depth)
    assert l1["trained"] < 0.2 * l1["random_init"]
    assert depth["trained"][1] > 0.97 and depth["trained"][0] < 1e-2
    assert depth["random_init"][1] < depth["trained"][1]
