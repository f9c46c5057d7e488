"""Headless frames of a simulation (the reference's Renderer, web/js/main.js:130-272).

The camera is the reference's orbit camera (main.js:23-32: angles theta,
phi, distance, target) with its projection (fov pi/4, near 0.02, far 50)
and light (0.5, 0.9, 0.35) (main.js:232-243). Frames are rendered by
xpbi_render into an RGBA8 image; write_ppm stores one as a binary PPM.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi

DEFAULT_ORBIT = dict(theta=0.5, phi=0.32, dist=2.1, target=[0.5, 0.28, 0.5])  # scenes.js:90


def orbit_eye(theta: float, phi: float, dist: float, target) -> list[float]:
    """camEye (main.js:24-32)."""
    ct, st = math.cos(theta), math.sin(theta)
    cp, sp = math.cos(phi), math.sin(phi)
    return [target[0] + dist * cp * st, target[1] + dist * sp, target[2] + dist * cp * ct]


def camera(orbit: dict | None = None, particle_radius: float = 0.0, draw_ground: bool = True,
           draw_box: bool = True, fov_y: float = math.pi / 4, near_z: float = 0.02, far_z: float = 50.0,
           light_dir=(0.5, 0.9, 0.35)) -> _abi.Camera:
    """The reference's camera for an orbit (a scene's `camera` entry)."""
    o = dict(DEFAULT_ORBIT)
    if orbit:
        o.update(orbit)
    c = _abi.Camera()
    eye = orbit_eye(o["theta"], o["phi"], o["dist"], o["target"])
    for k in range(3):
        c.eye[k] = eye[k]
        c.target[k] = float(o["target"][k])
        c.light_dir[k] = float(light_dir[k])
    c.fov_y, c.near_z, c.far_z = fov_y, near_z, far_z
    c.particle_radius = particle_radius
    c.draw_ground = 1 if draw_ground else 0
    c.draw_box = 1 if draw_box else 0
    return c


def render(sim, scene: int = 0, cam: _abi.Camera | None = None, width: int = 960, height: int = 540) -> np.ndarray:
    """One frame of scene `scene` as an (height, width, 4) uint8 array."""
    if cam is None:
        cam = camera(sim.scenes[scene].get("camera"))
    img = np.empty((height, width, 4), np.uint8)
    _abi.check(_abi.lib().xpbi_render(sim._h, scene, C.byref(cam), width, height,
                                      img.ctypes.data_as(C.POINTER(C.c_uint8)), None))
    return img


def write_ppm(path: str, img: np.ndarray) -> None:
    """Binary PPM (P6) of the RGB channels."""
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(img[:, :, :3]).tobytes())
