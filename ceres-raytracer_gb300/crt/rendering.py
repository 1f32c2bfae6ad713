"""Dynamic-scene queries: the BVH is rebuilt on the GPU for every call (reference crt/rendering.py,
src/crt/rendering_dynamic/render.hpp and passes.hpp)."""
from typing import List, Tuple, Union

import numpy as np

import _crt
from .body_fixed import _depth_image, _instance_image
from .cameras import Camera
from .entity import Entity
from .lidars import Lidar
from .lights import Light
from ._pybind_convert import validate_entities, validate_lights


def render(camera: Camera, lights: Union[Light, List[Light], Tuple[Light, ...]],
           entities: Union[Entity, List[Entity], Tuple[Entity, ...]], min_samples: int = 1, max_samples: int = 1,
           noise_threshold: float = 1., num_bounces: int = 1, *, seed: int = 0, return_radiance: bool = False):
    return _crt.render(camera._cpp, validate_lights(lights), validate_entities(entities), min_samples, max_samples,
                       noise_threshold, num_bounces, seed=seed, return_radiance=return_radiance)


def simulate_lidar(lidar: Lidar, entities: Union[Entity, List[Entity], Tuple[Entity, ...]], num_rays: int = 1):
    return _crt.simulate_lidar(lidar._cpp, validate_entities(entities), num_rays)


def normal_pass(camera: Camera, entities, return_image: bool = False):
    normals = _crt.normal_pass(camera._cpp, [e._cpp for e in entities])
    if return_image:
        return normals, 255 * np.abs(normals)
    return normals


def intersection_pass(camera: Camera, entities, return_image: bool = False):
    intersections = _crt.intersection_pass(camera._cpp, [e._cpp for e in entities])
    if return_image:
        return intersections, _depth_image(intersections)
    return intersections


def instance_pass(camera: Camera, entities, return_image: bool = False):
    instances = _crt.instance_pass(camera._cpp, [e._cpp for e in entities])
    if return_image:
        return instances, _instance_image(instances)
    return instances
