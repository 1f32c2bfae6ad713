"""List normalisation for the extension module (reference crt/_pybind_convert.py)."""
from .entity import Entity
from .lights import AreaLight, PointLight


def valid_light(light):
    return isinstance(light, (PointLight, AreaLight))


def validate_lights(lights):
    lights = list(lights) if isinstance(lights, (list, tuple)) else [lights]
    return [l._cpp for l in lights]


def validate_entities(entities):
    entities = list(entities) if isinstance(entities, (list, tuple)) else [entities]
    return [e._cpp for e in entities]
