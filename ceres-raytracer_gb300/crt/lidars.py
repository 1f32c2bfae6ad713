"""LiDARs (reference crt/lidars.py)."""
from abc import ABC

import numpy as np
from numpy.typing import ArrayLike

import _crt
from ._validate_values import validate_position, validate_rotation
from .rigid_body import RigidBody, _spice


class Lidar(ABC):
    def batch_set_pose(self, batch_positions: ArrayLike, batch_rotations: ArrayLike):
        """Set up to 100 000 poses: positions [n, 3], rotations [3, 3, n] (reference lidars.py:17-30)."""
        batch_positions = np.asarray(batch_positions, dtype=np.float64)
        batch_rotations = np.asarray(batch_rotations, dtype=np.float64)
        n = batch_positions.shape[0]
        if n > 100000:
            raise ValueError("No more than 100,000 poses can be batch set")
        self.batch_positions = np.zeros(batch_positions.shape)
        for idx in range(n):
            self.batch_positions[idx, :] = validate_position(batch_positions[idx, :])
        self.batch_rotations = batch_rotations
        pad = np.zeros((3, 3, 100000))
        pad[:, :, :batch_rotations.shape[2]] = batch_rotations
        self._cpp.batch_set_pose(np.ascontiguousarray(self.batch_positions), pad, n)

    def batch_spice_pose(self, ets: np.ndarray):
        sp = _spice()
        positions, _ = sp.spkpos(self.name, ets, self.ref, self.abcorr, self.origin)
        rotations = np.zeros((3, 3, ets.size))
        for idx, et in enumerate(ets):
            rotations[:, :, idx] = validate_rotation(sp.pxform(self.ref, self.frame, et))
        self.batch_set_pose(np.array(positions, dtype=np.float64), rotations)


class SimpleLidar(RigidBody, Lidar):
    """Single-beam LiDAR along the boresight (-z unless z_positive).  Extension: set_beam_grid()
    gives it an nx x ny grid of beams for BodyFixedGroup.lidar_scan()."""

    def __init__(self, z_positive: bool = False, **kwargs):
        super().__init__(**kwargs)
        self.z_positive = z_positive
        self._cpp = _crt.SimpleLidar(z_positive)
        self.set_pose(self.position, self.rotation)

    def set_beam_grid(self, nx: int, ny: int, half_angle_x: float, half_angle_y: float):
        """Beams at angles uniform over [-half, half] (radians) on both axes of the sensor frame."""
        self._cpp.set_beam_grid(int(nx), int(ny), float(half_angle_x), float(half_angle_y))
