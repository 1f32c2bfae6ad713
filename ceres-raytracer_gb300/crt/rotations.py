"""Elementary frame rotations and Euler sequences (reference crt/rotations.py)."""
import numpy as np


def rotation_1(rot):
    c, s = np.cos(rot), np.sin(rot)
    return np.array([[1, 0, 0], [0, c, s], [0, -s, c]])


def rotation_2(rot):
    c, s = np.cos(rot), np.sin(rot)
    return np.array([[c, 0, -s], [0, 1, 0], [s, 0, c]])


def rotation_3(rot):
    c, s = np.cos(rot), np.sin(rot)
    return np.array([[c, s, 0], [-s, c, 0], [0, 0, 1]])


_AXES = {"1": rotation_1, "2": rotation_2, "3": rotation_3}


def euler_to_rotmat(sequence, angles, degrees=False):
    """Product of frame rotations about axes '1', '2', '3' applied left to right."""
    if degrees:
        angles = np.deg2rad(angles)
    rotmat = np.eye(3)
    for idx, axis in enumerate(sequence):
        if axis not in _AXES:
            raise Exception("Not a valid euler angle sequence!")
        rotmat = rotmat @ _AXES[axis](angles[idx])
    return rotmat
