"""Body-fixed groups: entities whose BVH is built once and kept resident on the GPU
(reference crt/body_fixed.py and src/crt/rendering_body_fixed/body_fixed_group.hpp).

Cameras, lights and LiDARs are expressed in the group's body frame before each query; like the
reference, render() and the passes update the pose of the camera / lights passed in.
"""
from typing import List, Tuple, Union

import numpy as np
from numpy.typing import ArrayLike

import _crt
from .cameras import Camera
from .lidars import Lidar
from .lights import Light
from .rigid_body import RigidBody


class BodyFixedEntity(RigidBody):
    """Mesh, colour and pose of one member of a BodyFixedGroup."""

    def __init__(self, geometry_path: str, color: ArrayLike = [1, 1, 1], geometry_type: str = "obj",
                 smooth_shading: bool = False, **kwargs):
        super().__init__(**kwargs)
        self.geometry_path = geometry_path
        self.geometry_type = geometry_type
        self.color = color
        self.smooth_shading = smooth_shading
        self._cpp = _crt.BodyFixedEntity(self.geometry_path, self.geometry_type, self.smooth_shading, list(self.color))
        self.set_pose(self.position, self.rotation)
        self.set_scale(self.scale)

    def set_reflectivity(self, specular: float, diffuse: float):
        """Extension: specular / diffuse reflectivity for the radiation-pressure integrator."""
        self.specular, self.diffuse = float(specular), float(diffuse)
        self._cpp.set_reflectivity(self.specular, self.diffuse)


def _as_list(x):
    return list(x) if isinstance(x, (list, tuple)) else [x]


class BodyFixedGroup(RigidBody):
    """Group of BodyFixedEntity rendered in the body frame with a cached (device-resident) BVH."""

    def __init__(self, entities: Union[BodyFixedEntity, List[BodyFixedEntity], Tuple[BodyFixedEntity, ...]],
                 **kwargs):
        super().__init__(**kwargs)
        self._cpp = _crt.BodyFixedGroup([e._cpp for e in _as_list(entities)])

    def transform_to_body(self, position: ArrayLike, rotation: ArrayLike) -> Tuple[np.ndarray, np.ndarray]:
        """Position and rotation in the body frame: p_b = s R (p - p_g), R_b = (R R_in^T)^T."""
        relative_position = self.scale * np.matmul(self.rotation, np.asarray(position) - self.position)
        relative_rotation = np.matmul(self.rotation, np.asarray(rotation).T).T
        return relative_position, relative_rotation

    def _to_body(self, body):
        p, r = self.transform_to_body(body.position, body.rotation)
        body.set_pose(p, r)

    def render(self, camera: Camera, lights: Union[Light, List[Light], Tuple[Light, ...]], min_samples: int = 1,
               max_samples: int = 1, noise_threshold: float = 1., num_bounces: int = 1, *, seed: int = 0,
               return_radiance: bool = False):
        """uint8 RGBA image [H, W, 4]; with return_radiance=True also the float RGBA radiance."""
        self._to_body(camera)
        lights = _as_list(lights)
        for light in lights:
            self._to_body(light)
        return self._cpp.render(camera._cpp, [l._cpp for l in lights], min_samples, max_samples, noise_threshold,
                                num_bounces, seed=seed, return_radiance=return_radiance)

    def simulate_lidar(self, lidar: Lidar, num_rays: int = 1):
        self._to_body(lidar)
        return self._cpp.simulate_lidar(lidar._cpp, num_rays)

    def batch_simulate_lidar(self, lidar: Lidar, num_rays: int = 1):
        positions = np.asarray(lidar.batch_positions, dtype=np.float64)
        rotations = np.asarray(lidar.batch_rotations, dtype=np.float64)
        rel_pos = self.scale * (positions - self.position) @ self.rotation.T
        rel_rot = np.einsum("ijn,kj->ikn", rotations, self.rotation)   # (R R_n^T)^T = R_n R^T
        lidar.batch_set_pose(rel_pos, rel_rot)
        return self._cpp.batch_simulate_lidar(lidar._cpp, num_rays)

    def lidar_scan(self, lidar: Lidar):
        """Extension: (range [ny, nx] float64, triangle index [ny, nx] uint32, 0xFFFFFFFF on a miss)
        for a LiDAR with a beam grid (SimpleLidar.set_beam_grid)."""
        self._to_body(lidar)
        return self._cpp.lidar_scan(lidar._cpp)

    def srp(self, sun_direction: ArrayLike, quaternions: ArrayLike, grid: int, num_bounces: int = 2,
            flux: float = 1361.0, c: float = 299792458.0, center_of_mass: ArrayLike = (0.0, 0.0, 0.0),
            facet_power: bool = False):
        """Extension: solar radiation force / torque (body frame) for each attitude quaternion (w, x, y, z,
        body -> inertial), optionally with per-triangle absorbed power."""
        q = np.ascontiguousarray(quaternions, dtype=np.float64).reshape(-1, 4)
        return self._cpp.srp(np.asarray(sun_direction, dtype=np.float64), q, int(grid), int(num_bounces), float(flux),
                             float(c), np.asarray(center_of_mass, dtype=np.float64), facet_power)

    def normal_pass(self, camera: Camera, return_image: bool = False):
        self._to_body(camera)
        normals = self._cpp.normal_pass(camera._cpp)
        if return_image:
            return normals, 255 * np.abs(normals)
        return normals

    def intersection_pass(self, camera: Camera, return_image: bool = False):
        self._to_body(camera)
        intersections = self._cpp.intersection_pass(camera._cpp)
        if return_image:
            return intersections, _depth_image(intersections)
        return intersections

    def instance_pass(self, camera: Camera, return_image: bool = False):
        self._to_body(camera)
        instances = self._cpp.instance_pass(camera._cpp)
        if return_image:
            return instances, _instance_image(instances)
        return instances


def _depth_image(points):
    image = np.sqrt((points ** 2).sum(-1))
    image = image - np.min(image)
    return 255 * image / np.max(image)


def _instance_image(instances):
    unique_ids = np.unique(instances)
    colors = np.random.randint(0, high=255, size=(3, unique_ids.size))
    image = np.zeros((instances.shape[0], instances.shape[1], 3))
    for idx, i in enumerate(unique_ids):
        image[instances == i, :] = colors[:, idx]
    return image
