"""Shared builders for the tests (models from fixtures, seeded models)."""
import numpy as np
import torch

from nglod_gb300 import OctreeSDF
from nglod_gb300.options import default_args
from oracle import dense


def model_from_fixture(fx, num_lods, base_lod, device="cpu"):
    """Drop-in OctreeSDF loaded with the fixture's reference state_dict."""
    net = OctreeSDF(default_args(num_lods=num_lods, base_lod=base_lod))
    sd = {k[len("param/"):]: torch.from_numpy(v) for k, v in fx.items() if k.startswith("param/")}
    net.load_state_dict(sd)
    return net.to(device).eval()


def oracle_model(net, dtype=np.float64):
    return dense.model_from_state_dict(net.state_dict(), net.num_lods, net.base_lod, dtype)


def seeded_model(num_lods=5, base_lod=2, seed=0, device="cpu"):
    torch.manual_seed(seed)
    return OctreeSDF(default_args(num_lods=num_lods, base_lod=base_lod)).to(device).eval()
