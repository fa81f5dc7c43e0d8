"""Coarse-grid AO (RenderOptions::aoResDiv > 1) on the GPU against the oracle.

The reference (embree_renderer.cpp:527-553, ao/ao_coarse.hpp,
hit_shader.hpp:129-145) gathers AO once per cell of the hi-res grid divided by
aoResDiv and lets every hit interpolate it with normal / depth guides, falling
back to its own AO rays where the guides reject.  The lookup weights use
pow / exp, whose last bits differ between CUDA and the host's libm, so a hit
on the 0.3 weight-sum threshold may fall back on one side only: the fallback
mask must agree on >= 99.5% of first hits; the image is held to the grid
parity bars (hit-id agreement >= 99.9%, PSNR >= 45 dB, |error| <= 1e-3 at the
99.9th percentile of pixels whose subpixels agree on the first hit).
"""
import copy

import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_linear, psnr_srgb
from umbreon_gb300 import scenes

pytestmark = pytest.mark.gpu
AO_QUANTILE = 0.999


def _render(gpu_ctx, sc, opt):
    b = gpu_ctx.build(sc)
    try:
        return gpu_ctx.render(b, sc, opt)
    finally:
        b.release()


def _case(name):
    sc, opt = scenes.molecular_surface(n_atoms=600, box=16.0, n_spheres=300, width=96, height=96,
                                       ao_samples=8, layers=2)
    opt.aoResDebug = True
    if name == "div2_ss1":
        opt.aoResDiv = 2
    elif name == "out_ss2":
        opt.supersample, opt.aoResDiv = 2, -1
    elif name == "div3_enhanced_aov":
        opt.aoResDiv = 3
        opt.aoFalloffPower, opt.aoMultiScale, opt.aoBentNormal = 1.0, True, True
        opt.aoWriteAov = True
    elif name == "out_ss2_adaptive":
        opt.supersample, opt.aoResDiv, opt.aaMode = 2, -1, 1
    else:
        raise KeyError(name)
    return sc, opt


@pytest.mark.parametrize("name", ["div2_ss1", "out_ss2", "div3_enhanced_aov", "out_ss2_adaptive"])
def test_coarse_ao_matches_oracle(gpu_ctx, oracle_lib, name):
    sc, opt = _case(name)
    g = _render(gpu_ctx, sc, opt)
    o = oracle_lib.render(sc, opt)
    assert g.aoPatchMask is not None and g.aoPatchMask.shape == o.aoPatchMask.shape
    patched = float(np.mean(o.aoPatchMask > 0))
    assert 0.0 < patched < 0.9, patched
    mask_agree = float(np.mean(g.aoPatchMask == o.aoPatchMask))
    assert mask_agree >= 0.995, (mask_agree, patched)
    ss = max(1, opt.supersample)
    agree = id_agreement(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim)
    m = agree_mask_final(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim, ss)
    diff = np.abs(g.color - o.color)[m]
    info = dict(name=name, patched=patched, mask_agree=mask_agree, agree=agree,
                err=float(np.quantile(diff, AO_QUANTILE)), psnr_lin=psnr_linear(g.color, o.color),
                psnr_srgb=psnr_srgb(g.color, o.color))
    assert agree >= 0.999, info
    assert info["psnr_lin"] >= 45.0 and info["psnr_srgb"] >= 45.0, info
    assert info["err"] <= 1e-3, info
    if opt.aoWriteAov:
        for k in ("contactAo", "shapeAo", "avgHitDist"):
            d = np.abs(getattr(g, k) - getattr(o, k))[m]
            assert float(np.quantile(d, 0.99)) <= 1e-3, (k, float(d.max()))


def test_coarse_ao_cuts_ao_rays(gpu_ctx):
    """The AO rays of the grid plus the fallback hits replace one gather per
    hit (one opaque layer, no shadow rays: every occlusion ray is an AO ray)."""
    sc, opt = _case("div2_ss1")
    opt.aoResDebug = False
    opt.shadows, opt.transparency = False, False
    inline = copy.copy(opt)
    inline.aoResDiv = 0
    g = _render(gpu_ctx, sc, opt)
    f = _render(gpu_ctx, sc, inline)
    assert g.stats["rays_occlusion"] < 0.5 * f.stats["rays_occlusion"], (g.stats, f.stats)


def test_coarse_ao_frames_in_a_batch(gpu_ctx):
    """A batch runs coarse-AO items as their own passes: each equals the frame
    rendered alone."""
    sc, opt = _case("div2_ss1")
    opt.aoResDebug = False
    inline = copy.copy(opt)
    inline.aoResDiv = 0
    b = gpu_ctx.build(sc)
    try:
        frames, stats = gpu_ctx.render_batch([(b, sc, opt), (b, sc, inline)])
        alone = gpu_ctx.render(b, sc, opt)
        alone_i = gpu_ctx.render(b, sc, inline)
    finally:
        b.release()
    assert np.array_equal(frames[0].color, alone.color)
    assert np.array_equal(frames[1].color, alone_i.color)
