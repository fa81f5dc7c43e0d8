"""Principled materials (Material::model == Principled, the direct pass of
shading/principled.hpp) on the GPU against the oracle.

A ball-and-stick scene whose atoms and bonds mix POV, isotropic principled
(dielectric and metal, several roughnesses) and anisotropic principled
materials, with AO, hard or area-light soft shadows (the per-sample
visibility x BRDF estimator on the 'PBRD' stream) and a molecular surface
with principled mesh materials.  Bars as the grid parity tests: hit-id
agreement >= 99.9%, PSNR >= 45 dB, |error| <= 1e-3 at the 99.9th percentile
of pixels whose subpixels agree on the first hit (the anisotropy rotation
uses cosf / sinf, whose last bits may differ from the host's libm).
"""
import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_linear, psnr_srgb
from umbreon_gb300 import abi, scenes

pytestmark = pytest.mark.gpu
QUANTILE = 0.999


def _pbr_mats(n, seed):
    rng = np.random.default_rng(seed)
    m = np.full(n, scenes.pov_material(), abi.MATERIAL_DTYPE)
    kind = rng.integers(0, 4, n)  # 0 POV, 1 dielectric, 2 metal, 3 anisotropic metal
    pbr = kind > 0
    m["model"][pbr] = 1
    m["pbr_roughness"][pbr] = rng.uniform(0.05, 0.8, int(pbr.sum())).astype(np.float32)
    m["pbr_specular"][pbr] = 0.5
    m["pbr_metallic"][kind >= 2] = 1.0
    an = kind == 3
    m["pbr_anisotropy"][an] = rng.uniform(-0.9, 0.9, int(an.sum())).astype(np.float32)
    m["pbr_anisotropy_rotation"][an] = rng.uniform(0.0, 0.5, int(an.sum())).astype(np.float32)
    return m


def _ball_and_stick(soft):
    sc, opt = scenes.ball_and_stick(n=1500, width=192, height=108, supersample=2, ao_samples=8)
    sc.sphere_material = _pbr_mats(sc.sphere_count(), 11)
    sc.cyl_material = _pbr_mats(len(sc.cyl_radius), 12)
    if soft:
        opt.shadowSamples, opt.lightRadius = 4, 3.0
    return sc, opt


def _compare(gpu_ctx, oracle_lib, sc, opt):
    b = gpu_ctx.build(sc)
    try:
        g = gpu_ctx.render(b, sc, opt)
    finally:
        b.release()
    o = oracle_lib.render(sc, opt)
    ss = max(1, opt.supersample)
    agree = id_agreement(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim)
    m = agree_mask_final(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim, ss)
    diff = np.abs(g.color - o.color)[m]
    info = dict(agree=agree, err=float(np.quantile(diff, QUANTILE)), worst=float(diff.max()),
                psnr_lin=psnr_linear(g.color, o.color), psnr_srgb=psnr_srgb(g.color, o.color))
    assert agree >= 0.999, info
    assert info["psnr_lin"] >= 45.0 and info["psnr_srgb"] >= 45.0, info
    assert info["err"] <= 1e-3, info
    return g, o


@pytest.mark.parametrize("soft", [False, True])
def test_principled_ball_and_stick(gpu_ctx, oracle_lib, soft):
    sc, opt = _ball_and_stick(soft)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_principled_molecular_surface(gpu_ctx, oracle_lib):
    sc, opt = scenes.molecular_surface(n_atoms=600, box=16.0, n_spheres=300, width=96, height=96,
                                       ao_samples=8, layers=2)
    mm = np.array(sc.mesh_material, abi.MATERIAL_DTYPE, copy=True)
    mm["model"], mm["pbr_metallic"], mm["pbr_roughness"], mm["pbr_specular"] = 1, 0.3, 0.4, 0.5
    sc.mesh_material = mm
    sc.sphere_material = _pbr_mats(sc.sphere_count(), 13)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_principled_adjoint_rejected(gpu_ctx):
    from umbreon_gb300.abi import UbrError
    sc, opt = scenes.differentiable(n=200, res=32, ao_samples=0)
    m = np.array(sc.sphere_material, abi.MATERIAL_DTYPE, copy=True)
    m["model"] = 1
    sc.sphere_material = m
    b = gpu_ctx.build(sc)
    try:
        with pytest.raises(UbrError):
            gpu_ctx.adjoint(b, sc, opt, np.zeros((opt.height, opt.width, 4), np.float32))
    finally:
        b.release()
