"""Entity: a mesh with colour, shading mode and pose (reference crt/entity.py)."""
from numpy.typing import ArrayLike

import _crt
from .rigid_body import RigidBody


class Entity(RigidBody):
    """Mesh loaded from `geometry_path` (Wavefront OBJ) with a Lambertian colour."""

    def __init__(self, geometry_path: str, color: ArrayLike = [1, 1, 1], geometry_type: str = "obj",
                 smooth_shading: bool = False, **kwargs):
        super().__init__(**kwargs)
        self.geometry_path = geometry_path
        self.geometry_type = geometry_type
        self.color = color
        self.smooth_shading = smooth_shading
        self._cpp = _crt.Entity(self.geometry_path, self.geometry_type, self.smooth_shading, list(self.color))
        self.set_pose(self.position, self.rotation)
        self.set_scale(self.scale)

    def set_reflectivity(self, specular: float, diffuse: float):
        """Extension: specular / diffuse reflectivity used by the radiation-pressure integrator."""
        self.specular, self.diffuse = float(specular), float(diffuse)
        self._cpp.set_reflectivity(self.specular, self.diffuse)
