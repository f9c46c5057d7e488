"""GB300-native XPBI substep behind the reference's ``Simulation`` surface.

The compute path is libxpbi.so (hand-written sm_103a CUDA, C ABI in
include/xpbi.h); this package is its host-side mirror of web/js/sim.js and
web/js/scenes.js.
"""
from . import render, scenes
from ._abi import XpbiError, lib
from .sim import Simulation, make_params, pack_uniforms, params_for

__all__ = ["Simulation", "XpbiError", "lib", "make_params", "pack_uniforms", "params_for", "render", "scenes"]
