"""Cameras (reference crt/cameras.py)."""
from abc import ABC, abstractmethod

import numpy as np
from numpy.typing import ArrayLike

import _crt
from .rigid_body import RigidBody


class Camera(ABC):
    @abstractmethod
    def get_fov(self, degrees=True):
        return


class SimpleCamera(RigidBody, Camera):
    """Pinhole camera: focal length, resolution [W, H], sensor size; boresight -z unless z_positive."""

    def __init__(self, focal_length: float, resolution: ArrayLike, sensor_size: ArrayLike, z_positive: bool = False,
                 **kwargs):
        super().__init__(**kwargs)
        self.focal_length = focal_length
        self.resolution = resolution
        self.sensor_size = sensor_size
        self._cpp = _crt.SimpleCamera(focal_length, list(resolution), list(sensor_size), z_positive)
        self.set_pose(self.position, self.rotation)

    def get_fov(self, degrees: bool = True) -> np.ndarray:
        # same expression as the reference (crt/cameras.py:64-69)
        half = np.arctan2(np.asarray(self.sensor_size) / 2, 2 * self.focal_length)
        return np.rad2deg(2 * half) if degrees else 2 * half
