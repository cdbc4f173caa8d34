"""Restatement of the reference's CPU torch path, used as the timed CPU baseline
(``bench.py --impl reference`` and the ``cpu_baseline`` leg).  Test and
CPU-baseline infrastructure only.

The reference itself cannot be imported where the benchmark runs, so this
module re-expresses its computation with the same torch operators it calls:

    FeatureVolume.forward   F.grid_sample(fm, x, align_corners=True,
                            padding_mode='border')      OctreeSDF.py:46-57
    OctreeSDF.sdf           running sum, cat([x, sum]), Linear-ReLU-Linear,
                            decoder evaluated twice per LOD, early return at
                            ``lod``                         OctreeSDF.py:94-155
    SphereTracer.forward    masked march with cond.any() per step, then
                            finite-difference normals      SphereTracer.py:41-132

Weights come from an OctreeSDF state_dict (the drop-in's or the reference's).
"""
import torch
import torch.nn.functional as F


class RefOctreeSDF:
    def __init__(self, state_dict, num_lods, dtype=torch.float32):
        self.num_lods = num_lods
        self.fms = [state_dict[f"features.{i}.fm"].detach().cpu().to(dtype).contiguous() for i in range(num_lods)]
        self.dec = []
        for i in range(num_lods):
            self.dec.append(tuple(state_dict[f"louts.{i}.{j}.{w}"].detach().cpu().to(dtype)
                                  for j in (0, 2) for w in ("weight", "bias")))
        self.lod = None

    def _decode(self, i, ex):
        w0, b0, w1, b1 = self.dec[i]
        return F.linear(F.relu(F.linear(ex, w0, b0)), w1, b1)

    def sdf(self, x, lod=None, return_lst=False):
        if lod is None:
            lod = self.lod
        l = []
        samples = []
        n = x.shape[0]
        for i in range(self.num_lods):
            s = F.grid_sample(self.fms[i], x.reshape(1, n, 1, 1, 3), align_corners=True,
                              padding_mode="border")[0, :, :, 0, 0].transpose(0, 1)
            samples.append(s)
            if i > 0:
                samples[i] += samples[i - 1]
            ex = torch.cat([x, samples[i]], dim=-1)
            d = self._decode(i, ex)
            d = self._decode(i, ex)  # the reference evaluates each decoder twice (OctreeSDF.py:124,142)
            if lod is not None and lod == i:
                return d
            l.append(d)
        return l if return_lst else l[-1]

    def __call__(self, x):
        return self.sdf(x)


def aabb(ray_o, ray_d):
    """Vectorised sol_nglod.aabb (sol_nglod_kernel.cu:92-150) in torch."""
    n = ray_o.shape[0]
    x = ray_o.clone()
    t = torch.zeros(n, 1, dtype=ray_o.dtype)
    hit = torch.zeros(n, dtype=torch.bool)
    inv = (1.0 / ray_d.double()).to(ray_o.dtype)
    sgn = torch.where(torch.signbit(ray_d), 1.0, -1.0).to(ray_o.dtype)
    outside = ~(ray_o.abs().amax(dim=1) < 1)
    dd = (sgn - ray_o) * inv
    tests = []
    for a, (b, c) in enumerate(((1, 2), (0, 2), (0, 1))):
        lb = torch.addcmul(ray_o[:, b], ray_d[:, b], dd[:, a])
        lc = torch.addcmul(ray_o[:, c], ray_d[:, c], dd[:, a])
        tests.append((dd[:, a] >= 0) & (lb.abs() < 1) & (lc.abs() < 1))
    dist = torch.where(tests[0], dd[:, 0], torch.where(tests[1], dd[:, 1], torch.where(tests[2], dd[:, 2], 0.0)))
    ok = (tests[0] | tests[1] | tests[2]) & outside & (dist < 500)
    hit[ok] = True
    t[ok, 0] = dist[ok]
    x[ok] = torch.addcmul(ray_o[ok], ray_d[ok], dist[ok, None])
    return x, t, hit


@torch.no_grad()
def sphere_trace(net, ray_o, ray_d, num_steps=128, min_dis=3e-4, step_size=1.0, camera_clamp=(-5.0, 10.0)):
    x, t, cond = aabb(ray_o, ray_d)
    normal = torch.zeros_like(x)
    d = net(x)
    dprev = d.clone()
    hit = torch.zeros_like(d).bool()[:, 0]
    for _ in range(num_steps):
        hit = (torch.abs(t) < camera_clamp[1])[:, 0]
        cond = cond & (torch.abs(d) > min_dis)[:, 0]
        cond = cond & (torch.abs((d + dprev) / 2.0) > min_dis * 3)[:, 0]
        cond = cond & hit
        if not cond.any():
            break
        x = torch.where(cond.view(-1, 1), torch.addcmul(ray_o, ray_d, t), x)
        dprev = torch.where(cond.unsqueeze(1), d, dprev)
        d[cond] = net(x[cond]) * step_size
        t = torch.where(cond.view(-1, 1), t + d, t)
    hit = hit & ~(torch.abs(x) > 1.0).any(dim=-1)
    xh = x[hit]
    h = 1.0 / (64.0 * 3.0)
    eps = torch.eye(3, dtype=x.dtype) * h
    grad = torch.cat([net(xh + eps[k]) - net(xh - eps[k]) for k in range(3)], dim=-1) / (h * 2.0)
    normal[hit] = F.normalize(grad, p=2, dim=-1, eps=1e-5)
    return x, t, hit, normal
