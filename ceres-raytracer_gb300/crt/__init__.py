"""crt: drop-in Python API of the CERES ray tracer backed by the GB300 ray-query library.

Same modules, classes, functions and signatures as the reference package (crt/__init__.py,
body_fixed.py, rendering.py, cameras.py, lights.py, lidars.py, rigid_body.py, entity.py,
rotations.py); the extension module `_crt` sits beside this package and runs every ray query on
the GPU.  SPICE helpers import `spiceypy` only when called.
"""
from .rigid_body import RigidBody
from .entity import Entity
from .body_fixed import BodyFixedGroup, BodyFixedEntity

__all__ = ["Entity", "RigidBody", "BodyFixedGroup", "BodyFixedEntity"]
