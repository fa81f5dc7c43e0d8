"""Python binding of the REFERENCE's own render path -- TEST INFRASTRUCTURE.

Loads ``oracle/_ref/libumbreon_ref.so``: CueMol/umbreon's src/umbreon compiled
unmodified against the Embree / oneTBB stand-ins of ``oracle/shim`` by
``oracle/build_ref.py`` (needs the reference sources; absent elsewhere).
``render(scene, opt)`` runs the reference's ``umbreon::render`` on a scene
described for this library and returns its colour, depth and view-z planes.
Only tests and fixture scripts use this module, as the checker.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from umbreon_gb300 import abi
from umbreon_gb300.api import RenderOptions, Scene, make_render_desc

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libumbreon_ref.so"
_L = None


def available() -> bool:
    return LIB.exists()


def lib():
    global _L
    if _L is None:
        L = C.CDLL(str(LIB))
        L.ref_render.restype = C.c_int
        L.ref_render.argtypes = [C.POINTER(abi.SceneDesc), C.POINTER(abi.RenderDesc), C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.POINTER(C.c_double)]
        _L = L
    return _L


def render(scene: Scene, opt: RenderOptions):
    """(color (H, W, 4), depth (Hss, Wss), viewZ (Hss, Wss), renderSeconds)."""
    sd, keep_s = scene.to_desc()
    rd, keep_r = make_render_desc(scene, opt)
    ss = max(1, opt.supersample)
    color = np.zeros((opt.height, opt.width, 4), np.float32)
    depth = np.zeros((opt.height * ss, opt.width * ss), np.float32)
    vz = np.zeros_like(depth)
    secs = C.c_double(0.0)
    st = lib().ref_render(C.byref(sd), C.byref(rd), color.ctypes.data, depth.ctypes.data, vz.ctypes.data,
                          C.byref(secs))
    if st != 0:
        raise RuntimeError("the reference's render threw")
    return color, depth, vz, secs.value
