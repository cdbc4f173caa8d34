"""GB300-native (sm_103a) NGLOD neural-SDF hot path.

Drop-ins for the reference's hot-path API:

    OctreeSDF(args)            sdf-net/lib/models/OctreeSDF.py
    SphereTracer(args)         sdf-net/lib/tracer/SphereTracer.py
    RenderBuffer               sdf-net/lib/tracer/RenderBuffer.py
    sol_nglod.aabb             sdf-net/lib/extensions/sol_nglod

all backed by the C-ABI library ``nglod_gb300/_build/libnglod_gb300.so``
(include/nglod_gb300.h).  There is no CPU fallback: calls with CPU tensors or
without the built library raise RuntimeError.
"""
from . import autograd, sol_nglod, trainer
from ._lib import load as load_library
from .octree_sdf import FeatureVolume, OctreeSDF, setparam
from .tracer import BaseTracer, PlainSphereTracer, RenderBuffer, SphereTracer
from .renderer import Renderer

__all__ = ["OctreeSDF", "FeatureVolume", "SphereTracer", "PlainSphereTracer", "BaseTracer", "RenderBuffer", "Renderer",
           "sol_nglod", "setparam", "load_library", "trainer", "autograd"]
