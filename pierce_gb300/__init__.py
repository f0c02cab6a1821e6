"""pierce_gb300 — GB300-native mesh spatial joins (overlap, intersection,
containment) over preprocessed triangle-mesh datasets.

Host-side mirror of the Pierce query path.  The compute path is the CUDA
library ``libpierce_gb300.so`` (sm_103a) reached through its C ABI
(``include/pierce_capi.h``); the `.pre` format, edge extraction and the
seeded generators live in ``libpierce_host.so`` (``include/pierce_host.h``).
"""
from .geometry import (Geometry, icospheres, ellipsoid_pair, tubes, instances, expand_instances,  # noqa: F401
                       SPHERES, ELLIPSOIDS)

__all__ = ["Geometry", "icospheres", "ellipsoid_pair", "tubes", "instances", "expand_instances", "SPHERES",
           "ELLIPSOIDS"]
