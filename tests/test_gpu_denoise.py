"""The a-trous denoiser (RenderOptions::denoiser, pipeline.cpp:224-252,
denoise_atrous.cpp) on the GPU against the oracle: the final-resolution
linear colour filtered with the AO AOV normal and albedo guides before the
gamma.  Bars as the grid parity tests (PSNR >= 45 dB, |error| <= 1e-3 at the
99.9th percentile on pixels whose subpixels agree on the first hit): the
edge-stop weights use powf / expf, whose last bits may differ from the host
libm."""
import copy

import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_linear, psnr_srgb
from umbreon_gb300 import scenes

pytestmark = pytest.mark.gpu


def _render(gpu_ctx, sc, opt):
    b = gpu_ctx.build(sc)
    try:
        return gpu_ctx.render(b, sc, opt)
    finally:
        b.release()


def _scene(ss=1):
    sc, opt = scenes.molecular_surface(n_atoms=600, box=16.0, n_spheres=300, width=96, height=96,
                                       ao_samples=8, layers=2)
    opt.supersample = ss
    opt.aoWriteAov = True
    sc.assumedGamma = 2.2
    return sc, opt


@pytest.mark.parametrize("ss,backend,demod", [(1, 1, True), (2, 1, True), (2, 2, False)])
def test_denoise_matches_oracle(gpu_ctx, oracle_lib, ss, backend, demod):
    sc, opt = _scene(ss)
    opt.denoiser, opt.denoiseDemodulateAlbedo = backend, demod
    g = _render(gpu_ctx, sc, opt)
    o = oracle_lib.render(sc, opt)
    agree = id_agreement(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim)
    m = agree_mask_final(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim, ss)
    diff = np.abs(g.color - o.color)[m]
    info = dict(agree=agree, err=float(np.quantile(diff, 0.999)), psnr_lin=psnr_linear(g.color, o.color),
                psnr_srgb=psnr_srgb(g.color, o.color))
    assert agree >= 0.999, info
    assert info["psnr_lin"] >= 45.0 and info["psnr_srgb"] >= 45.0, info
    assert info["err"] <= 1e-3, info
    # the filter did something: the denoised frame differs from the raw one
    raw = copy.copy(opt)
    raw.denoiser = 0
    assert not np.array_equal(_render(gpu_ctx, sc, raw).color, g.color)


def test_denoise_without_guides_is_a_no_op(gpu_ctx):
    """Without aoWriteAov (and without GI) the reference has no edge guide and
    leaves the frame as rendered."""
    sc, opt = _scene()
    opt.aoWriteAov = False
    plain = _render(gpu_ctx, sc, opt)
    opt.denoiser = 1
    assert np.array_equal(_render(gpu_ctx, sc, opt).color, plain.color)
