"""Argument namespaces with the reference's defaults.

``OctreeSDF(args)`` and ``SphereTracer(args)`` read their settings from an
``argparse.Namespace`` produced by sdf-net/lib/options.py:parse_options.
``default_args(**overrides)`` builds one with that parser's defaults for every
field this path reads (options.py:60-221), so callers without the reference's
CLI get the same behaviour.
"""
import argparse

DEFAULTS = dict(
    # net (options.py:58-92)
    net="OctreeSDF", pos_enc=False, feature_dim=32, feature_size=4, joint_feature=False, num_layers=1,
    num_lods=1, base_lod=2, ff_dim=-1, ff_width=16.0, hidden_dim=128, pretrained=None, periodic=False,
    skip=None, freeze=-1, pos_invariant=False, joint_decoder=False, feat_sum=False, jit=False,
    # optimizer (options.py:141-149)
    optimizer="adam", lr=0.001, loss=["l2_loss"], grad_method="finitediff",
    # trainer (options.py:152-188)
    epochs=250, batch_size=512, only_last=False, return_lst=False, growth_strategy="increase",
    # renderer (options.py:191-232)
    sol=False, render_res=[512, 512], render_batch=0, camera_origin=[-2.8, 2.8, -2.8], camera_lookat=[0, 0, 0],
    camera_fov=30, camera_proj="persp", camera_clamp=[-5, 10], lod=None, interpolate=None, render_every=1,
    num_steps=256, step_size=1.0, min_dis=0.0003, tracer="SphereTracer", matcap_path="data/matcap/green.png",
    ground_height=None, ao=False, shadow=False, shading_mode="matcap", perf=False,
)


def default_args(**overrides):
    d = dict(DEFAULTS)
    unknown = set(overrides) - set(d)
    if unknown:
        raise KeyError(f"unknown option(s): {sorted(unknown)}")
    d.update(overrides)
    return argparse.Namespace(**d)
