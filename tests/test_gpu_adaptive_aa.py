"""Adaptive antialiasing (RenderOptions::aaMode = 1) on the GPU.

The reference (embree_renderer.cpp:1379-1670, render/adaptive_aa.hpp) shades
the centre subpixel of every output pixel, flags pixels whose 4-neighbour
centre pairs differ (geomID / section, colour contrast > aaThreshold, normal,
depth crack), dilates the mask once, shades every subpixel of flagged blocks
and replicates a centre re-shaded with ss^2 AO / soft-shadow samples into the
other blocks.  Bars: the refinement mask agrees with the oracle's on >= 99%
of output pixels (a colour contrast at the threshold may tip either way);
the image meets the grid parity bars (hit-id agreement >= 99.9%, PSNR >=
45 dB, max |error| <= 1e-3 on pixels whose subpixels agree on the first hit
and whose masks agree); flagged pixels are bitwise equal to the full-grid
render, as the reference promises.
"""
import copy

import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_linear, psnr_srgb
from umbreon_gb300 import scenes
from umbreon_gb300.abi import UbrError

pytestmark = pytest.mark.gpu

# AO and soft shadows: the same per-pixel sample streams as the oracle, with
# rare sample-level flips where a ray grazes an occluder
AO_QUANTILE = 0.999


def _adaptive(opt, threshold=None):
    a = copy.copy(opt)
    a.aaMode, a.aaDebug = 1, True
    if threshold is not None:
        a.aaThreshold = threshold
    return a


def _case(name):
    if name == "space_filling_soft_shadows":
        sc, opt = scenes.space_filling(n=600, width=128, height=96)
        opt.supersample = 2
        opt.shadows, opt.lightRadius, opt.shadowSamples = True, 4.0, 2
    elif name == "molecular_surface_ss3_ao":
        sc, opt = scenes.molecular_surface(n_atoms=600, box=16.0, n_spheres=300, width=96, height=96,
                                           ao_samples=8, layers=2)
        opt.supersample = 3
    elif name == "perspective_transparent":
        sc, opt = scenes.space_filling(n=600, width=120, height=90)
        sc.sphere_color[:, 3] = 0.5
        sc.camera.orthographic = False
        sc.camera.fovy = 40.0
        sc.camera.position = (20.0, 20.0, 110.0)
        opt.supersample = 2
        opt.maxTransparentLayers = 6
    elif name == "ball_and_stick_ss4":
        sc, opt = scenes.ball_and_stick(n=400, width=96, height=64, supersample=4, ao_samples=4)
    else:
        raise KeyError(name)
    return sc, opt


def _render(gpu_ctx, sc, opt):
    b = gpu_ctx.build(sc)
    try:
        return gpu_ctx.render(b, sc, opt)
    finally:
        b.release()


@pytest.mark.parametrize("case", ["space_filling_soft_shadows", "molecular_surface_ss3_ao",
                                  "perspective_transparent", "ball_and_stick_ss4"])
def test_adaptive_matches_oracle(gpu_ctx, oracle_lib, case):
    sc, opt = _case(case)
    a = _adaptive(opt)
    g = _render(gpu_ctx, sc, a)
    o = oracle_lib.render(sc, a)
    assert g.aaMask is not None and g.aaMask.shape == (opt.height, opt.width)
    mask_agree = float(np.mean(g.aaMask == o.aaMask))
    flagged = float(np.mean(o.aaMask > 0))
    assert 0.02 < flagged < 0.98, flagged  # both kinds of block are exercised
    assert mask_agree >= 0.99, (mask_agree, flagged)
    ss = opt.supersample
    agree = id_agreement(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim)
    m = agree_mask_final(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim, ss) & (g.aaMask == o.aaMask)
    diff = np.abs(g.color - o.color)[m]
    err = float(np.quantile(diff, AO_QUANTILE))
    pl, ps = psnr_linear(g.color, o.color), psnr_srgb(g.color, o.color)
    info = dict(case=case, mask_agree=mask_agree, flagged=flagged, agree=agree, err=err, worst=float(diff.max()),
                psnr_linear=pl, psnr_srgb=ps)
    assert agree >= 0.999, info
    assert pl >= 45.0 and ps >= 45.0, info
    assert err <= 1e-3, info


@pytest.mark.parametrize("case", ["molecular_surface_ss3_ao", "perspective_transparent"])
def test_adaptive_flagged_pixels_equal_grid(gpu_ctx, case):
    """Flagged blocks shade every subpixel at its own seed: bitwise the grid."""
    sc, opt = _case(case)
    grid = _render(gpu_ctx, sc, opt)
    ad = _render(gpu_ctx, sc, _adaptive(opt))
    m = ad.aaMask > 0
    assert m.any() and (~m).any()
    assert np.array_equal(ad.color[m], grid.color[m])
    ss = opt.supersample
    H, W = opt.height, opt.width
    blk = np.repeat(np.repeat(m, ss, 0), ss, 1)
    assert np.array_equal(ad.hit_prim[blk], grid.hit_prim[blk])
    assert np.array_equal(ad.depth[blk], grid.depth[blk])


def test_adaptive_unflagged_blocks_replicate_centre(gpu_ctx):
    """Without stochastic effects the centre is not re-shaded: every subpixel
    of an unflagged block carries the centre's first hit and depth."""
    sc, opt = _case("space_filling_soft_shadows")
    opt.shadowSamples = 1  # hard shadows: nothing to boost
    ad = _render(gpu_ctx, sc, _adaptive(opt))
    ss, H, W = opt.supersample, opt.height, opt.width
    m = ad.aaMask > 0
    c = ss // 2
    for plane in (ad.hit_prim, ad.hit_geom, ad.depth, ad.viewZ):
        blocks = plane.reshape(H, ss, W, ss)
        centre = blocks[:, c:c + 1, :, c:c + 1]
        same = (blocks == centre).all(axis=(1, 3))
        assert same[~m].all()


def test_adaptive_threshold_zero_flags_more(gpu_ctx):
    sc, opt = _case("space_filling_soft_shadows")
    lo = _render(gpu_ctx, sc, _adaptive(opt, threshold=0.0)).aaMask
    hi = _render(gpu_ctx, sc, _adaptive(opt, threshold=10.0)).aaMask
    assert lo.sum() >= hi.sum()
    assert np.all(lo >= hi)


def test_adaptive_frames_in_a_batch(gpu_ctx):
    """A batch runs adaptive-AA items as their own passes: each equals the
    frame rendered alone."""
    sc, opt = _case("space_filling_soft_shadows")
    b = gpu_ctx.build(sc)
    try:
        a = _adaptive(opt)
        grid = copy.copy(opt)
        frames, stats = gpu_ctx.render_batch([(b, sc, a), (b, sc, grid), (b, sc, a)])
        alone_a = gpu_ctx.render(b, sc, a)
        alone_g = gpu_ctx.render(b, sc, grid)
    finally:
        b.release()
    assert np.array_equal(frames[0].color, alone_a.color) and np.array_equal(frames[2].color, alone_a.color)
    assert np.array_equal(frames[1].color, alone_g.color)


@pytest.mark.parametrize("ss,depth", [(1, 2), (2, 3), (2, 4)])
def test_adaptive_fine_lattice_matches_oracle(gpu_ctx, oracle_lib, ss, depth):
    """aaDepth > ss: each flagged cell is the box average of k^2 samples of
    the (W k) x (H k) lattice, k = ceil(aaDepth / ss)."""
    sc, opt = _case("molecular_surface_ss3_ao")
    opt.width = opt.height = 64
    opt.supersample = ss
    a = _adaptive(opt)
    a.aaDepth = depth
    g = _render(gpu_ctx, sc, a)
    o = oracle_lib.render(sc, a)
    mask_agree = float(np.mean(g.aaMask == o.aaMask))
    assert mask_agree >= 0.99, mask_agree
    agree = id_agreement(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim)
    m = agree_mask_final(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim, ss) & (g.aaMask == o.aaMask)
    diff = np.abs(g.color - o.color)[m]
    info = dict(agree=agree, err=float(np.quantile(diff, AO_QUANTILE)), psnr=psnr_srgb(g.color, o.color))
    assert agree >= 0.999, info
    assert info["err"] <= 1e-3 and info["psnr"] >= 45.0, info


def test_fine_lattice_at_ss1_equals_ss2_grid(gpu_ctx):
    """At ss 1 with aaDepth 2 the fine lattice is the ss 2 grid's lattice
    with the same seeds: flagged pixels equal the ss 2 grid render."""
    sc, opt = _case("molecular_surface_ss3_ao")
    opt.width = opt.height = 64
    opt.supersample = 1
    a = _adaptive(opt)
    a.aaDepth = 2
    ad = _render(gpu_ctx, sc, a)
    g2 = copy.copy(opt)
    g2.supersample = 2
    grid2 = _render(gpu_ctx, sc, g2)
    grid1 = _render(gpu_ctx, sc, opt)
    m = ad.aaMask > 0
    assert m.any() and (~m).any()
    assert np.array_equal(ad.color[m], grid2.color[m])
    assert np.array_equal(ad.color[~m], grid1.color[~m])


def test_boosted_centres_reuse_centre_ao(gpu_ctx):
    """Opaque frames with the tea2 AO stream: the boosted centre copies its
    first aoSamples AO results from the centre pass instead of tracing them.
    Same image as the persistent occlusion kernel (which traces them all),
    with fewer occlusion rays."""
    from umbreon_gb300.api import Context
    sc, opt = scenes.molecular_surface(n_atoms=600, box=16.0, n_spheres=300, width=96, height=96,
                                       ao_samples=8, layers=2)
    sc.mesh_colors = sc.mesh_colors.copy()
    sc.mesh_colors[:, 3] = 1.0  # opaque: one layer
    opt.supersample = 2
    a = _adaptive(opt)
    traced = Context(0, trace_mode=2)
    try:
        full = _render(traced, sc, a)
    finally:
        traced.close()
    reused = _render(gpu_ctx, sc, a)
    assert np.array_equal(reused.color, full.color)
    assert reused.stats["rays_occlusion"] < full.stats["rays_occlusion"]
