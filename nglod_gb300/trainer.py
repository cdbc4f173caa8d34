"""Training step of the dense model on the nglod_gb300 kernels.

``FusedAdam`` is a torch.optim.Optimizer whose step is one multi-tensor
kernel launch (``nglod_adam_step``) with torch.optim.Adam's update rule.
``step_geometry`` is Trainer.step_geometry (sdf-net/lib/trainer.py:294-340):
L2 loss summed over the loss LODs and divided by the batch size, backward,
optimizer step.  The loss is reduced in float64 on the GPU.
"""
import ctypes

import torch

from . import _lib
from .autograd import check_backward_status, sdf_train_stacked


class FusedAdam(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=0.0):
        super().__init__(params, dict(lr=lr, betas=betas, eps=eps, weight_decay=weight_decay))
        # step tables go host -> device asynchronously through a ring of pinned
        # buffers; an event per slot marks when its copy has been consumed
        self._ring = []
        self._ring_pos = 0

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        for group in self.param_groups:
            entries = []
            dev = None
            step_no = None
            for p in group["params"]:
                if p.grad is None:
                    continue
                _lib.require_cuda(p)
                if p.dtype != torch.float32 or p.grad.dtype != torch.float32:
                    raise RuntimeError("FusedAdam: float32 parameters and gradients required")
                st = self.state[p]
                if not st:
                    st["step"] = 0
                    st["exp_avg"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                    st["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                st["step"] += 1
                step_no = st["step"] if step_no is None else step_no
                if st["step"] != step_no:
                    raise RuntimeError("FusedAdam: parameters of a group must share their step count")
                g = p.grad
                if g.stride() != p.stride():
                    g = _like(p, g)
                    p.grad = g
                entries.append((p, g, st["exp_avg"], st["exp_avg_sq"]))
                dev = p.device
            if not entries:
                continue
            tab = (_lib.AdamTensor * len(entries))()
            for i, (p, g, m, v) in enumerate(entries):
                tab[i].param, tab[i].grad = p.data_ptr(), g.data_ptr()
                tab[i].exp_avg, tab[i].exp_avg_sq = m.data_ptr(), v.data_ptr()
                tab[i].numel = p.numel()
            dtab = self._upload(tab, dev)
            b1, b2 = group["betas"]
            _lib.check(_lib.load().nglod_adam_step(ctypes.c_void_p(dtab.data_ptr()), len(entries),
                                                   max(p.numel() for p, *_ in entries), group["lr"], b1, b2,
                                                   group["eps"], group["weight_decay"], step_no,
                                                   _lib.stream_ptr(dev)), "nglod_adam_step")
            self._ring[self._ring_pos - 1][2].record(torch.cuda.current_stream(dev))
        return loss

    def _upload(self, tab, dev, slots=4):
        """Device copy of the step table through the next pinned ring slot
        (non-blocking; waits only if that slot's previous step has not run)."""
        nbytes = ctypes.sizeof(tab)
        if len(self._ring) < slots:
            self._ring.append([None, None, torch.cuda.Event()])
        slot = self._ring[self._ring_pos % len(self._ring)]
        self._ring_pos = self._ring_pos % len(self._ring) + 1
        slot[2].synchronize()
        if slot[0] is None or slot[0].numel() < nbytes or slot[1].device != dev:
            slot[0] = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
            slot[1] = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        ctypes.memmove(slot[0].data_ptr(), ctypes.addressof(tab), nbytes)
        slot[1][:nbytes].copy_(slot[0][:nbytes], non_blocking=True)
        return slot[1]


def _like(p, g):
    """g copied into a tensor with p's strides (dense, same memory format)."""
    out = torch.empty_like(p, memory_format=torch.preserve_format)
    out.copy_(g)
    return out


def l2_loss(preds, gts, loss_lods, batch_size):
    """sum over loss LODs of ((pred - gt)^2).sum() / batch_size (trainer.py:325-336)."""
    loss = 0
    for l in loss_lods:
        loss = loss + ((preds[l] - gts) ** 2).sum()
    return loss / batch_size


def fused_l2_loss(preds, gts, loss_lods):
    """l2_loss over stacked predictions [rows, n, 1] in one launch
    (nglod_l2_loss): returns the loss (float64, 0-dim, on the device) and
    its gradient with respect to preds."""
    preds = preds.detach().contiguous()
    gts = gts.detach().float().contiguous()
    n = preds.shape[1]
    mask = 0
    for l in loss_lods:
        mask |= 1 << l
    loss = torch.empty((), dtype=torch.float64, device=preds.device)
    grad = torch.empty_like(preds)
    _lib.check(_lib.load().nglod_l2_loss(_lib.ptr(preds), _lib.ptr(gts), n, preds.shape[0], mask, _lib.ptr(loss),
                                         _lib.ptr(grad), _lib.stream_ptr(preds.device)), "nglod_l2_loss")
    return loss, grad


def step_geometry(net, optimizer, pts, gts, loss_lods=None):
    """One training step; returns the loss (float64, reduced on the GPU).
    The loss and its gradient come from one kernel (fused_l2_loss) and
    enter the backward as the gradient of the stacked predictions, with the
    same values as l2_loss(...).backward()."""
    if loss_lods is None:
        loss_lods = list(range(net.num_lods))
    preds = sdf_train_stacked(net, pts)
    # after the forward's launch (which reads no gradient), so that the
    # device starts on the step sooner
    net.zero_grad()
    loss, grad = fused_l2_loss(preds, gts, loss_lods)
    preds.backward(grad)
    optimizer.step()
    return loss


def fit(net, batches, steps, lr=1e-3, loss_lods=None, seed=0, log_every=500):
    """``steps`` calls of step_geometry with a FusedAdam(lr) optimizer,
    cycling through ``batches`` (device (pts, gts) pairs), each batch in a
    fresh random order (a device permutation from ``seed``).  Returns the
    optimizer and the losses of every ``log_every``-th and of the last step."""
    net.train()
    opt = FusedAdam(net.parameters(), lr=lr)
    dev = batches[0][0].device
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    losses = []
    for it in range(steps):
        xb, gb = batches[it % len(batches)]
        perm = torch.randperm(xb.shape[0], device=dev, generator=gen)
        l = step_geometry(net, opt, xb[perm], gb[perm], loss_lods)
        if it % log_every == 0 or it == steps - 1:
            losses.append(float(l.item()))
    check_backward_status()
    return opt, losses
