"""Lights (reference crt/lights.py)."""
from abc import ABC

import numpy as np
from numpy.typing import ArrayLike

import _crt
from .rigid_body import RigidBody


class Light(ABC):
    intensity: float


class PointLight(RigidBody, Light):
    """Point light: intensity / d^2, capped at 1e4 (lights/point_light.hpp:37-39)."""

    def __init__(self, intensity: float, **kwargs):
        super().__init__(**kwargs)
        self.intensity = intensity
        self._cpp = _crt.PointLight(self.intensity)
        self.set_pose(self.position, np.eye(3))


class AreaLight(RigidBody, Light):
    """Rectangular light of the given side lengths, sampled uniformly (lights/area_light.hpp:54-72)."""

    def __init__(self, intensity: float, size: ArrayLike, **kwargs):
        super().__init__(**kwargs)
        self.intensity = intensity
        self.size = size
        self._cpp = _crt.AreaLight(self.intensity, list(self.size))
        self.set_pose(self.position, self.rotation)
