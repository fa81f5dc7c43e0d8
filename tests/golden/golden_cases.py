"""Seeded scenes of the golden fixtures (one small case per workload family).

Each case returns (Scene, RenderOptions) from the project's seeded scene
generators at sizes the oracle renders in seconds.  `digest` fingerprints a
scene's inputs so a fixture can tell whether it is compared against the very
same inputs (bit-exact comparison) or against inputs that differ in the last
bits (a platform whose libm rounds exp / sin differently: parity bars).
"""
import dataclasses
import hashlib

import numpy as np

from umbreon_gb300 import scenes


def space_filling_160x120():
    return scenes.space_filling(width=160, height=120)


def ball_and_stick_160x90_ss2_ao8():
    return scenes.ball_and_stick(n=2000, width=160, height=90, supersample=2, ao_samples=8)


def molecular_surface_96_ao8_4layers():
    return scenes.molecular_surface(n_atoms=600, box=16.0, n_spheres=300, width=96, height=96, ao_samples=8,
                                    layers=4)


def spheres_5k_128_enhanced_ao_fog():
    return scenes.differentiable(n=5000, res=128, ao_samples=8)


def perspective_transparent_160x120():
    sc, opt = scenes.space_filling(n=600, width=160, height=120)
    sc.sphere_color[:, 3] = 0.5
    sc.camera.orthographic = False
    sc.camera.fovy = 40.0
    sc.camera.position = (20.0, 20.0, 110.0)
    opt.maxTransparentLayers = 6
    return sc, opt


def pt2_defaults_ball_and_stick_96x54_ss2():
    """pt2 GI, the reference's default integrator, every option at its default
    (reduced gather grid, denoise, upsample, edge patch)."""
    sc, opt = scenes.ball_and_stick(n=1500, width=96, height=54, supersample=2, ao_samples=4)
    opt.gi, opt.giIntegrator = True, 2
    return sc, opt


def pt2_restir_two_rounds_64x48():
    """pt2 with two ReSTIR spatial rounds on the render grid, unbiased."""
    sc, opt = scenes.ball_and_stick(n=800, width=64, height=48, supersample=1, ao_samples=4)
    opt.gi, opt.giIntegrator, opt.pt1Spp = True, 2, 4
    opt.pt2Rounds, opt.pt2Unbiased = 2, True
    return sc, opt


# name -> (generator, uses AO or soft shadows: sample directions come from
# sin / cos, whose last bit differs between CUDA and the host libm; "gi":
# path-traced GI, whose gather paths take those directions too)
CASES = {
    "space_filling_160x120": (space_filling_160x120, False),
    "ball_and_stick_160x90_ss2_ao8": (ball_and_stick_160x90_ss2_ao8, True),
    "molecular_surface_96_ao8_4layers": (molecular_surface_96_ao8_4layers, True),
    "spheres_5k_128_enhanced_ao_fog": (spheres_5k_128_enhanced_ao_fog, True),
    "perspective_transparent_160x120": (perspective_transparent_160x120, False),
    "pt2_defaults_ball_and_stick_96x54_ss2": (pt2_defaults_ball_and_stick_96x54_ss2, "gi"),
    "pt2_restir_two_rounds_64x48": (pt2_restir_two_rounds_64x48, "gi"),
}


def _feed(h, v):
    if isinstance(v, np.ndarray):
        h.update(str(v.dtype).encode())
        h.update(str(v.shape).encode())
        h.update(np.ascontiguousarray(v).tobytes())
    elif dataclasses.is_dataclass(v):
        for f in dataclasses.fields(v):
            h.update(f.name.encode())
            _feed(h, getattr(v, f.name))
    elif isinstance(v, (list, tuple)):
        for x in v:
            _feed(h, x)
    else:
        h.update(repr(v).encode())


def digest(sc, opt) -> str:
    """sha1 over every field of the scene and the options."""
    h = hashlib.sha1()
    _feed(h, sc)
    _feed(h, opt)
    return h.hexdigest()
