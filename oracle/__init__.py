"""CPU oracle for the NGLOD neural-SDF hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``nglod_gb300`` imports this package;
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use it, and only as the checker or the timed CPU baseline.

Contents
--------
dense       numpy restatement (float32 or float64) of the dense path:
            FeatureVolume / OctreeSDF.sdf / SphereTracer.forward /
            finite-difference normals / the sol_nglod ``aabb`` kernel.
torch_port  restatement of the same path written with the torch CPU ops the
            reference calls (grid_sample, Linear, where); it is the CPU
            baseline that ``bench.py --impl reference`` times.
spc         ctypes front end of ``nglod_oracle.c``: bit-exact C restatements of
            the sol_nglod ``aabb`` kernel and of the SPC octree codec and
            ray/octree traversal.
analytic    the analytic 16-sphere SDF and the seeded synthetic generators.

Parity pins: ``tests/golden/make_golden.py`` runs the reference's own Python
(``OctreeSDF``, ``SphereTracer``, ``spc3d.SPC3D``) on seeded inputs and commits
the outputs as fixtures; ``tests/test_oracle_golden.py`` checks this package
against them.
"""
