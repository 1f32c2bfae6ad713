"""Argument normalisation for poses and scales (reference: crt/_validate_values.py).

The reference's checks are `assert (cond, msg)` on a tuple, which never fails; it accepts any
value and converts positions and rotations to float64 numpy arrays.  The same conversions are done
here; malformed shapes raise ValueError instead of crashing later in the extension module.
"""
import numpy as np


def sanitize_array(array):
    return np.array(array, dtype=np.float64, copy=True)


def validate_scale(scale):
    return scale


def validate_position(position):
    p = np.asarray(position, dtype=np.float64).squeeze()
    if p.size != 3:
        raise ValueError("positions must have 3 components")
    return sanitize_array(p.reshape(3))


def validate_rotation(rotation):
    r = np.asarray(rotation, dtype=np.float64)
    if r.shape != (3, 3):
        raise ValueError("rotations must be 3x3 arrays")
    return sanitize_array(r)
