"""The oracle's a-trous restatement (denoise_atrous.cpp:27-220) on
properties the reference's design states: background pixels and pixels
without a normal guide are untouched, the filter lowers the pixel-to-pixel
noise of a flat AO-lit region, zero iterations is the identity, and without
the AOV guides nothing changes."""
import copy

import numpy as np

from oracle import oracle
from umbreon_gb300 import abi, scenes
from umbreon_gb300.api import RenderOptions, Scene


def _floor():
    """A large ambient-only floor under a partial occluder: noisy legacy AO."""
    q = 8.0
    pos = np.array([(-q, -q, 0), (q, -q, 0), (q, q, 0), (-q, -q, 0), (q, q, 0), (-q, q, 0),
                    (0.5, -q, 0.6), (q, -q, 0.6), (q, q, 0.6), (0.5, -q, 0.6), (q, q, 0.6), (0.5, q, 0.6)],
                   np.float32)
    nrm = np.array([(0, 0, 1)] * 6 + [(0, 0, -1)] * 6, np.float32)
    col = np.array([(0.8, 0.8, 0.8, 1)] * 6 + [(0.2, 0.2, 0.2, 1)] * 6, np.float32)
    sc = Scene(mesh_positions=pos, mesh_normals=nrm, mesh_colors=col,
               mesh_material=abi.material(ambient=1.0, diffuse=0.0))
    sc.camera = scenes.ortho_cam()
    sc.background = (0.3, 0.3, 0.3)
    return sc


def _opt(**kw):
    return RenderOptions(width=48, height=48, aoSamples=4, aoDistance=4.0, aoWriteAov=True, **kw)


def test_denoise_smooths_flat_region():
    sc = _floor()
    raw = oracle.render(sc, _opt())
    dn = oracle.render(sc, _opt(denoiser=1))
    region = (slice(10, 38), slice(2, 20))  # open floor, x < 0
    rough = lambda c: float(np.mean(np.abs(np.diff(c[region][..., 0], axis=1))))
    assert rough(dn.color) < 0.5 * rough(raw.color)


def test_background_and_unguided_pixels_untouched():
    sc = _floor()
    sc.mesh_positions = sc.mesh_positions * np.array([0.15, 0.15, 1.0], np.float32)
    raw = oracle.render(sc, _opt())
    dn = oracle.render(sc, _opt(denoiser=1))
    bg = raw.hit_geom == 0xFFFFFFFF
    assert bg.any() and np.array_equal(dn.color[bg], raw.color[bg])


def test_zero_iterations_and_no_guides_are_identity():
    sc = _floor()
    raw = oracle.render(sc, _opt())
    assert np.array_equal(oracle.render(sc, _opt(denoiser=1, denoiseIters=0)).color, raw.color)
    o = _opt()
    o.aoWriteAov = False
    plain = oracle.render(sc, o)
    o2 = copy.copy(o)
    o2.denoiser = 1
    assert np.array_equal(oracle.render(sc, o2).color, plain.color)
