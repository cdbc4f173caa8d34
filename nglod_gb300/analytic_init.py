"""Weights that make an ``OctreeSDF`` reproduce a given SDF without training.

Channel 0 of feature volume i holds the residual S(v) - sum_{j<i} f_j(v) at
volume i's vertices v, where f_j is the trilinear interpolant of volume j's
channel 0; decoder i computes relu(f0) - relu(-f0) = f0.  So ``sdf(x, lod=i)``
is the trilinear interpolant of S on LOD i's grid.  With ``noise > 0`` the
other channels and weights get N(0, noise^2) values (a perturbation of order
noise^2 on the output).  Used to give traces a real surface in tests and as
the non-learned baseline of equal memory: the same grids holding samples of
the ground-truth SDF, no learned decoder.
"""
import torch
import torch.nn.functional as F


def vertex_grid(s, dtype=torch.float64):
    """[s^3, 3] vertex positions in [-1, 1]^3, ordered as fm[:, z, y, x] (x fastest)."""
    lin = torch.linspace(-1, 1, s, dtype=dtype)
    zz, yy, xx = torch.meshgrid(lin, lin, lin, indexing="ij")
    return torch.stack([xx, yy, zz], -1).reshape(-1, 3)


def _sample(vol, pts):
    """Trilinear sample of vol [s, s, s] at pts [N, 3] (grid_sample, align_corners)."""
    g = pts.reshape(1, -1, 1, 1, 3).to(vol.dtype)
    return F.grid_sample(vol[None, None], g, align_corners=True, padding_mode="border").reshape(-1)


@torch.no_grad()
def init_from_sdf(net, sdf_fn, noise=0.0, seed=0):
    """Overwrite net's volumes and decoders (see module docstring).

    sdf_fn maps float64 points [N, 3] (torch) to [N] distances.
    """
    g = torch.Generator().manual_seed(seed)
    levels = []
    for fv in net.features:
        s = fv.fsize + 1
        pts = vertex_grid(s)
        target = sdf_fn(pts).reshape(-1).to(torch.float64)
        prev = torch.zeros_like(target)
        for vol in levels:
            prev += _sample(vol, pts)
        res = (target - prev).reshape(s, s, s)
        levels.append(res)
        fm = torch.randn(1, fv.fdim, s, s, s, generator=g, dtype=torch.float64) * noise
        fm[0, 0] = res
        fv.fm.copy_(fm.to(fv.fm.dtype))
    for dec in net.louts:
        lin0, lin1 = dec[0], dec[2]
        w0 = torch.randn(lin0.weight.shape, generator=g, dtype=torch.float64) * noise
        w0[0:2] = 0
        w0[0, 3] = 1.0
        w0[1, 3] = -1.0
        w1 = torch.randn(lin1.weight.shape, generator=g, dtype=torch.float64) * noise
        w1[0, 0] = 1.0
        w1[0, 1] = -1.0
        lin0.weight.copy_(w0.to(lin0.weight.dtype))
        lin0.bias.zero_()
        lin1.weight.copy_(w1.to(lin1.weight.dtype))
        lin1.bias.zero_()
    return net
