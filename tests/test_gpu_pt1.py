"""The pt1 GI pass (integrator/pt1/: the gather on the render grid or on a
reduced grid with its own primary rays, the denoise of E, the joint-bilateral
upsample, the silhouette edge patch, and the [E] composite of
render/embree_renderer.cpp:560-934) on the GPU against the oracle.

Both sides draw the same per-pixel sample streams (hashU32(pix ^
hashU32(pt1Seed)), tea2, Hammersley + Cranley-Patterson when pt1Ld), so the
frames agree up to traversal float order: a gather ray that grazes a
silhouette can hit on one side and escape on the other, moving that pixel by
one sample's share.  Bars: first-hit id agreement >= 99.9%, linear PSNR >=
45 dB, |error| <= 1e-3 at the 99th percentile of pixels whose first hits
agree; the lone-sphere known answer (every gather ray sees the white sky)
is exact to float rounding.
"""
import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_linear
from umbreon_gb300 import scenes
from umbreon_gb300.api import RenderOptions

pytestmark = pytest.mark.gpu
KINVALID = 0xFFFFFFFF


def _gi(opt, **kw):
    opt.gi, opt.giIntegrator, opt.pt1Denoise, opt.pt1GatherDiv = True, 1, False, 1
    for k, v in kw.items():
        setattr(opt, k, v)
    return opt


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
    info = dict(agree=agree, err=float(np.quantile(diff, 0.99)), worst=float(diff.max()),
                psnr=psnr_linear(g.color, o.color))
    assert agree >= 0.999, info
    assert info["psnr"] >= 45.0, info
    assert info["err"] <= 1e-3, info
    return g, o


def test_lone_sphere_known_answer(gpu_ctx):
    mat = scenes.pov_material()
    sc = scenes.material_sphere_scene((0.6, 0.4, 0.2, 1.0), mat, (0.0, 0.0, 0.0))
    sc.lights = []
    opt = _gi(RenderOptions(width=48, height=48, supersample=1), pt1Spp=8, giBounces=2, giIntensity=0.5,
              giEnvIntensity=2.0)
    b = gpu_ctx.build(sc)
    try:
        g = gpu_ctx.render(b, sc, opt)
    finally:
        b.release()
    hit = g.hit_geom.reshape(48, 48) != KINVALID
    col = g.color.reshape(48, 48, 4)[..., :3]
    want = 0.5 * float(mat["diffuse"]) * np.array([0.6, 0.4, 0.2], np.float32) * 2.0
    assert int(hit.sum()) > 100
    np.testing.assert_allclose(col[hit], np.broadcast_to(want, col[hit].shape), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("integrator", [1, 2])
def test_enclosed_sphere_known_answers(gpu_ctx, integrator):
    """The closed-form answers of the sphere inside a shadowing shell (every
    gather path ends on the shell, whose NEE is shadowed: E = 0; with
    giMaxDistance short of the shell: E = the sky), on the GPU."""
    from test_oracle_pt1 import enclosed_known_answers

    def render(sc, opt):
        b = gpu_ctx.build(sc)
        try:
            g = gpu_ctx.render(b, sc, opt)
        finally:
            b.release()
        prim = np.where(g.hit_geom.reshape(32, 32) == KINVALID, -1, g.hit_prim.reshape(32, 32).astype(np.int64))
        return g.color.reshape(32, 32, 4)[..., :3], prim
    enclosed_known_answers(render, rtol=1e-5, integrator=integrator)


@pytest.mark.parametrize("case", ["one_bounce_ld", "three_bounces_tea2"])
def test_space_filling_gi(gpu_ctx, oracle_lib, case):
    sc, opt = scenes.space_filling(n=600, width=96, height=72)
    opt.shadows = True
    if case == "one_bounce_ld":
        _gi(opt, pt1Spp=8, giBounces=1, pt1Ld=True)
    else:
        _gi(opt, pt1Spp=4, giBounces=3, pt1Ld=False, pt1Clamp=2.0, pt1SkyMode=1, pt1Seed=7,
            pt1SkyRadiance=(0.9, 0.95, 1.1), giMaxDistance=25.0)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_ball_and_stick_gi_with_ao_and_fog(gpu_ctx, oracle_lib):
    sc, opt = scenes.ball_and_stick(n=800, width=80, height=48, supersample=2, ao_samples=4)
    _gi(opt, pt1Spp=4, giBounces=2)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_molecular_surface_gi_transparent(gpu_ctx, oracle_lib):
    sc, opt = scenes.molecular_surface(n_atoms=300, box=14.0, n_spheres=60, width=72, height=72, ao_samples=4,
                                       layers=2)
    _gi(opt, pt1Spp=4, giBounces=2, supersample=1)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def _defaults(opt, **kw):
    """GI on with every pt1 option at the reference's default (gather grid =
    the supersample factor, a-trous denoise of E, upsample, edge patch)."""
    opt.gi, opt.giIntegrator = True, 1
    for k, v in kw.items():
        setattr(opt, k, v)
    return opt


def test_lone_sphere_known_answer_reduced_grid(gpu_ctx):
    mat = scenes.pov_material()
    sc = scenes.material_sphere_scene((0.6, 0.4, 0.2, 1.0), mat, (0.0, 0.0, 0.0))
    sc.lights = []
    for ss, div in ((2, -1), (1, 3)):
        opt = _defaults(RenderOptions(width=48, height=48, supersample=ss), pt1Spp=4, giIntensity=0.5,
                        giEnvIntensity=2.0, pt1GatherDiv=div)
        b = gpu_ctx.build(sc)
        try:
            g = gpu_ctx.render(b, sc, opt)
        finally:
            b.release()
        hit = (g.hit_geom != KINVALID).reshape(48 * ss, 48, ss).all(-1).reshape(48, ss, 48).all(1)
        col = g.color[..., :3]
        want = 0.5 * float(mat["diffuse"]) * np.array([0.6, 0.4, 0.2], np.float32) * 2.0
        assert int(hit.sum()) > 100
        np.testing.assert_allclose(col[hit], np.broadcast_to(want, col[hit].shape), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("ss,div,denoise,patch", [(2, -1, True, True), (1, 2, True, True), (1, 3, True, True),
                                                  (2, 1, True, False), (1, 2, False, True)])
def test_ball_and_stick_default_pipeline(gpu_ctx, oracle_lib, ss, div, denoise, patch):
    """The reference's default pt1 pipeline: reduced gather grid with its own
    primary rays, the a-trous denoise of E, the joint-bilateral upsample and
    the silhouette edge patch, against the oracle's restatement of each."""
    sc, opt = scenes.ball_and_stick(n=800, width=80, height=48, supersample=ss, ao_samples=4)
    _defaults(opt, pt1Spp=4, giBounces=2, pt1GatherDiv=div, pt1Denoise=denoise, pt1EdgePatch=patch)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_molecular_surface_default_pipeline(gpu_ctx, oracle_lib):
    sc, opt = scenes.molecular_surface(n_atoms=300, box=14.0, n_spheres=60, width=72, height=72, ao_samples=4,
                                       layers=2)
    _defaults(opt, pt1Spp=4, supersample=2)
    _compare(gpu_ctx, oracle_lib, sc, opt)


def _pt2_materials(sc, mesh=False):
    """Mix pt2's features into a scene: emissive spheres and bonds, mirror
    and glossy POV finishes, principled metal and dielectric, an area light."""
    from umbreon_gb300 import abi
    n = sc.sphere_count()
    mats = np.array(sc.sphere_material, abi.MATERIAL_DTYPE).copy()
    idx = np.arange(n)
    mats["emission"][idx % 9 == 0] = 3.0
    mats["reflection"][idx % 7 == 1] = 0.4                    # mirror (specular 0 -> no lobe)
    mats["specular"][idx % 7 == 1] = 0.0
    mats["reflection"][idx % 11 == 2] = 0.3                   # glossy (reflection + highlight)
    pr = idx % 13 == 3
    mats["model"][pr] = 1
    mats["pbr_metallic"][pr] = 1.0
    mats["pbr_roughness"][pr] = 0.4
    die = idx % 17 == 4
    mats["model"][die] = 1
    mats["pbr_specular"][die] = 0.5
    mats["pbr_roughness"][die] = 0.05                          # below the glossy cut: a mirror lobe
    sc.sphere_material = mats
    if sc.cylinder_count():
        cm = np.array(sc.cyl_material, abi.MATERIAL_DTYPE).copy()
        cm["emission"][np.arange(len(cm)) % 10 == 5] = 2.0
        sc.cyl_material = cm
    if mesh:
        m = np.array(sc.mesh_material, abi.MATERIAL_DTYPE).copy()
        m["emission"] = 0.5
        sc.mesh_material = m
    sc.lights[0].angularRadius = 0.05
    return sc


@pytest.mark.parametrize("ss,pattern,adaptive", [(1, 1, False), (2, 1, False), (1, 0, True), (2, 1, True)])
def test_pt2_ball_and_stick(gpu_ctx, oracle_lib, ss, pattern, adaptive):
    """pt2 at its defaults (blue-noise Sobol first bounce, emission with the
    emissive NEE and MIS, traced mirror and glossy reflection with the glossy
    denoise, area-light NEE jitter) on a mixed-material scene, GPU vs oracle;
    the per-pixel Sobol pattern and adaptive spp as variants."""
    sc, opt = scenes.ball_and_stick(n=600, width=64, height=48, supersample=ss, ao_samples=4)
    _pt2_materials(sc)
    opt.gi, opt.giIntegrator, opt.pt1Spp = True, 2, 4
    opt.pt2Pattern, opt.pt2Adaptive, opt.pt2GlossySpp = pattern, adaptive, 4
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_pt2_molecular_surface_emissive_mesh(gpu_ctx, oracle_lib):
    sc, opt = scenes.molecular_surface(n_atoms=300, box=14.0, n_spheres=60, width=64, height=64, ao_samples=4,
                                       layers=2)
    _pt2_materials(sc, mesh=True)
    opt.gi, opt.giIntegrator, opt.pt1Spp, opt.pt2GlossySpp = True, 2, 4, 4
    _compare(gpu_ctx, oracle_lib, sc, opt)


@pytest.mark.parametrize("ss,rounds,unbiased,grid", [(2, 2, False, -1), (1, 1, True, 1), (1, 3, False, 2),
                                                     (2, 2, True, -1)])
def test_pt2_restir_rounds(gpu_ctx, oracle_lib, ss, rounds, unbiased, grid):
    """pt2's ReSTIR spatial rounds (pt2Rounds > 0, integrator/pt2/
    pt2_reservoir.hpp, pt2_spatial.hpp): the gather streams every sample
    into the point's reservoir, the rounds resample neighbours' reservoirs
    (with `unbiased`, one visibility ray per contributor) and the last one
    writes E; on the reduced grid of the defaults and on the render grid,
    GPU vs oracle.  The oracle equals the reference's code bit for bit on
    these options (tests/test_ref_pin.py)."""
    sc, opt = scenes.ball_and_stick(n=600, width=64, height=48, supersample=ss, ao_samples=4)
    _pt2_materials(sc)
    opt.gi, opt.giIntegrator, opt.pt1Spp, opt.pt2GlossySpp = True, 2, 4, 4
    opt.pt2Rounds, opt.pt2Unbiased, opt.pt1GatherDiv = rounds, unbiased, grid
    if rounds == 3:
        opt.pt2Radius, opt.pt2WClamp, opt.pt2MCap, opt.pt2Adaptive = 6.0, 4.0, 20.0, True  # adaptive is ignored
    _compare(gpu_ctx, oracle_lib, sc, opt)


def test_pt2_restir_changes_only_the_gi_term(gpu_ctx):
    """ReSTIR moves E but nothing else: with gi_intensity 0 the frames with
    and without rounds are identical, and with GI on they differ."""
    sc, opt = scenes.ball_and_stick(n=600, width=64, height=48, supersample=2, ao_samples=4)
    opt.gi, opt.giIntegrator, opt.pt1Spp = True, 2, 4
    b = gpu_ctx.build(sc)
    try:
        import copy
        on = copy.copy(opt)
        on.pt2Rounds = 2
        assert not np.array_equal(gpu_ctx.render(b, sc, opt).color, gpu_ctx.render(b, sc, on).color)
        opt.giIntensity = on.giIntensity = 0.0
        assert np.array_equal(gpu_ctx.render(b, sc, opt).color, gpu_ctx.render(b, sc, on).color)
    finally:
        b.release()
