"""RigidBody: pose (position, rotation), scale and SPICE pose helpers (reference crt/rigid_body.py).

The rotation is a 3x3 matrix R; the extension applies R to entity geometry and R^T to camera and
lidar boresights, exactly as the reference's C++ side does.
"""
from typing import Union

import numpy as np
from numpy.typing import ArrayLike

from ._validate_values import validate_position, validate_rotation, validate_scale


def _spice():
    try:
        import spiceypy
    except ImportError as e:   # the reference imports spiceypy at module load; here only when used
        raise ImportError("spiceypy is required for SPICE-driven poses") from e
    return spiceypy


class RigidBody:
    """Position, rotation and scale of a body, with optional NAIF/SPICE identifiers."""

    def __init__(self, position: ArrayLike = np.zeros(3), rotation: ArrayLike = np.eye(3),
                 scale: Union[float, int] = 1, name: Union[str, None] = None, frame: Union[str, None] = None,
                 origin: str = "SSB", ref: Union[str, None] = "J2000", abcorr: Union[str, None] = "NONE"):
        self.scale = validate_scale(scale)
        self.position = validate_position(position)
        self.rotation = validate_rotation(rotation)
        self.name = name
        self.frame = frame
        self.origin = origin
        self.ref = ref
        self.abcorr = abcorr

    def set_scale(self, scale: float):
        self.scale = validate_scale(scale)
        self._cpp.set_scale(self.scale)

    def set_position(self, position: ArrayLike):
        self.position = validate_position(position)
        self._cpp.set_position(self.position)

    def set_rotation(self, rotation: ArrayLike):
        self.rotation = validate_rotation(rotation)
        self._cpp.set_rotation(self.rotation)

    def set_pose(self, position: ArrayLike, rotation: ArrayLike):
        self.position = validate_position(position)
        self.rotation = validate_rotation(rotation)
        self._cpp.set_pose(self.position, self.rotation)

    def spice_position(self, et: float):
        position, _ = _spice().spkpos(self.name, et, self.ref, self.abcorr, self.origin)
        self.set_position(position)

    def spice_rotation(self, et: float):
        self.set_rotation(_spice().pxform(self.ref, self.frame, et))

    def spice_pose(self, et: float):
        sp = _spice()
        position, _ = sp.spkpos(self.name, et, self.ref, self.abcorr, self.origin)
        rotation = sp.pxform(self.ref, self.frame, et)
        self.set_pose(position, rotation)
