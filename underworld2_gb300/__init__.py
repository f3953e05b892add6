"""underworld2_gb300 -- GB300-native particle-in-cell Stokes path of Underworld2.

A drop-in for ``uw.systems.Stokes``, ``uw.systems.Solver`` and
``uw.systems.SwarmAdvector`` on regular Cartesian Q1/dQ0 meshes, computed by
hand-written sm_103a CUDA kernels behind the C ABI in ``include/uwg.h``::

    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (64, 64), (0., 0.), (1., 1.))
    ...
"""
__version__ = "0.1.0"

from . import conditions, container, function, mesh, swarm, systems, utils  # noqa: E402,F401
