"""The pt1 GI gather in the oracle (integrator/pt1/pt1_gather.hpp, the
[E] composite of render/embree_renderer.cpp:908-927) and the host-side
checks of the GI settings this library builds.

Known answer: a lone convex sphere lit only by the uniform white gather sky
sees the sky in every cosine-hemisphere direction, so E_stored = mean(L) is
exactly the sky radiance (ambient x giEnvIntensity) and, with no lights, a
hit pixel is exactly giIntensity x kd x pigment x E (the constant ambient is
dropped under GI, hit_shader.hpp:221-242).
"""
import numpy as np
import pytest

from umbreon_gb300 import api, scenes
from umbreon_gb300.api import RenderOptions

KINVALID = 0xFFFFFFFF


def _lone_sphere(**kw):
    mat = scenes.pov_material()
    sc = scenes.material_sphere_scene((0.6, 0.4, 0.2, 1.0), mat, (0.0, 0.0, 0.0))
    sc.lights = []
    kw.setdefault("giIntegrator", 1)
    opt = RenderOptions(width=32, height=32, supersample=1, gi=True, pt1Denoise=False, pt1GatherDiv=1, **kw)
    return sc, opt, float(mat["diffuse"])


@pytest.mark.parametrize("ld", [True, False])
@pytest.mark.parametrize("gain,env", [(1.0, 1.0), (0.5, 2.0)])
def test_lone_sphere_sees_the_whole_sky(oracle_lib, ld, gain, env):
    sc, opt, kd = _lone_sphere(pt1Ld=ld, giIntensity=gain, giEnvIntensity=env, pt1Spp=6, giBounces=2)
    o = oracle_lib.render(sc, opt)
    hit = o.hit_geom.reshape(32, 32) != KINVALID
    assert 50 < int(hit.sum()) < 32 * 32
    col = o.color.reshape(32, 32, 4)[..., :3]
    want = gain * kd * np.array([0.6, 0.4, 0.2], np.float32) * env
    np.testing.assert_allclose(col[hit], np.broadcast_to(want, col[hit].shape), rtol=1e-6, atol=1e-7)
    assert np.all(col[~hit] == 0.0)


def test_gi_off_keeps_the_ambient(oracle_lib):
    sc, opt, kd = _lone_sphere()
    opt.gi = False
    o = oracle_lib.render(sc, opt)
    hit = o.hit_geom.reshape(32, 32) != KINVALID
    col = o.color.reshape(32, 32, 4)[..., :3]
    amb = float(scenes.pov_material()["ambient"])
    np.testing.assert_allclose(col[hit][0], amb * np.array([0.6, 0.4, 0.2]), rtol=1e-6)


def test_occluder_darkens_the_gather(oracle_lib):
    # a second sphere beside the first blocks part of its sky
    sc, opt, _ = _lone_sphere(pt1Spp=16)
    a = oracle_lib.render(sc, opt).color.reshape(32, 32, 4)[..., :3].sum()
    sc.sphere_center_radius = np.array([[0, 0, 0, 1], [1.6, 0, -0.5, 0.8]], np.float32)
    sc.sphere_color = np.array([[0.6, 0.4, 0.2, 1.0]] * 2, np.float32)
    sc.sphere_material = np.concatenate([sc.sphere_material] * 2)
    o = oracle_lib.render(sc, opt)
    g = o.hit_geom.reshape(32, 32)
    p = o.hit_prim.reshape(32, 32)
    first = (g != KINVALID) & (p == 0)
    col = o.color.reshape(32, 32, 4)[..., :3]
    want = float(scenes.pov_material()["diffuse"]) * np.array([0.6, 0.4, 0.2])
    assert np.all(col[first] <= want * (1 + 1e-6))
    assert np.any(col[first].sum(-1) < 0.95 * want.sum())
    assert a > 0


def test_only_the_cache_integrator_is_refused():
    opt = RenderOptions(width=8, height=8, gi=True, giIntegrator=0)
    with pytest.raises(ValueError, match="irradiance-cache"):
        api.check_gi(opt)
    for integ in (1, 2):
        opt.giIntegrator = integ
        api.check_gi(opt)


@pytest.mark.parametrize("integrator", [1, 2])
@pytest.mark.parametrize("ss,div", [(1, 2), (2, -1), (2, 1), (3, -1), (1, 3)])
@pytest.mark.parametrize("denoise,patch", [(True, True), (False, True), (True, False)])
def test_default_pipeline_known_answer(oracle_lib, ss, div, denoise, patch, integrator):
    """The whole pt1 pipeline at the reference's defaults (gather grid =
    the supersample factor, a-trous denoise of E, joint-bilateral upsample,
    edge patch) keeps the lone sphere's constant E = sky exactly: every stage
    is a normalised weighted mean of that constant."""
    sc, opt, kd = _lone_sphere(pt1Spp=4, giIntensity=0.5, giEnvIntensity=2.0)
    opt.supersample, opt.pt1GatherDiv, opt.pt1Denoise, opt.pt1EdgePatch = ss, div, denoise, patch
    opt.giIntegrator = integrator
    o = oracle_lib.render(sc, opt)
    hit = (o.hit_geom != KINVALID).reshape(32 * ss, 32, ss).all(-1).reshape(32, ss, 32).all(1)
    col = o.color[..., :3]
    want = 0.5 * kd * np.array([0.6, 0.4, 0.2], np.float32) * 2.0
    assert 50 < int(hit.sum()) < 32 * 32
    np.testing.assert_allclose(col[hit], np.broadcast_to(want, col[hit].shape), rtol=2e-6, atol=1e-7)


def _closed_box():
    """A closed box, floor z = 0 to ceiling z = 1, walls at x, y = +-1, all
    faces' vertex normals pointing inward, seen from inside by a camera
    looking down at the floor's middle.  No gather ray escapes to the sky;
    the light travels straight down, so the floor's shadow rays hit the
    ceiling, the ceiling faces away from it and the walls are edge-on."""
    from umbreon_gb300.api import Camera, DistantLight, Scene
    c = [(x, y, z) for z in (0.0, 1.0) for y in (-1.0, 1.0) for x in (-1.0, 1.0)]
    quads = [((0, 1, 3, 2), (0, 0, 1)), ((4, 6, 7, 5), (0, 0, -1)), ((0, 4, 5, 1), (0, 1, 0)),
             ((2, 3, 7, 6), (0, -1, 0)), ((0, 2, 6, 4), (1, 0, 0)), ((1, 5, 7, 3), (-1, 0, 0))]
    pos, nrm = [], []
    for (a, b, cc, d), n in quads:
        for i in (a, b, cc, a, cc, d):
            pos.append(c[i])
            nrm.append(n)
    col = np.tile(np.array([0.8, 0.7, 0.6, 1.0], np.float32), (len(pos), 1))
    sc = Scene(mesh_positions=np.array(pos, np.float32), mesh_normals=np.array(nrm, np.float32), mesh_colors=col)
    sc.camera = Camera(position=(0.0, 0.0, 0.5), direction=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0),
                       orthographic=True, height=0.5)
    sc.lights = [DistantLight(direction=(0.0, 0.0, -1.0), intensity=1.0)]
    return sc


@pytest.mark.parametrize("bounces", [1, 3])
def test_closed_room_gathers_nothing(oracle_lib, bounces):
    """No sky is visible and every gather vertex's light is occluded (ceiling
    vertices' shadow rays hit the floor; floor vertices face away from the
    light), so E = 0.  The floor's own light is shadowed by the ceiling and
    GI drops the constant ambient: the GI frame is black, the frame without
    GI is the ambient term alone."""
    sc = _closed_box()
    opt = RenderOptions(width=16, height=16, gi=True, giIntegrator=1, pt1Spp=8, giBounces=bounces, shadows=True)
    o = oracle_lib.render(sc, opt)
    assert np.all(o.hit_geom != KINVALID)
    assert np.all(o.color[..., :3] == 0.0)
    opt.gi = False
    d = oracle_lib.render(sc, opt)
    want = 0.2 * np.array([0.8, 0.7, 0.6], np.float32)
    np.testing.assert_allclose(d.color[..., :3], np.broadcast_to(want, d.color[..., :3].shape), rtol=1e-6)


def test_gather_distance_cut_sees_only_sky(oracle_lib):
    """giMaxDistance below the distance to any wall or the ceiling: every
    gather ray ends short and counts as a miss, so E = the uniform sky
    exactly."""
    sc = _closed_box()
    opt = RenderOptions(width=16, height=16, gi=True, giIntegrator=1, pt1Spp=8, giMaxDistance=0.5, giEnvIntensity=1.5)
    o = oracle_lib.render(sc, opt)
    opt.giMaxDistance = 0.0
    closed = oracle_lib.render(sc, opt)
    # the same frame with the cut: E = sky = ambient (1, 1, 1) x 1.5 on top of the closed room's frame
    kd = 0.8  # Mesh::material default diffuse
    diff = o.color[..., :3] - closed.color[..., :3]
    want = kd * np.array([0.8, 0.7, 0.6], np.float32) * 1.5
    np.testing.assert_allclose(diff, np.broadcast_to(want, diff.shape), rtol=1e-5, atol=1e-6)


def test_gather_div_resolution():
    o = RenderOptions(width=8, height=8, supersample=2)
    assert api.gi_gather_div(o) == 2            # -1 = the supersample factor
    o.pt1GatherDiv, o.pt1HalfRes = 0, False
    assert api.gi_gather_div(o) == 1
    o.supersample, o.pt1GatherDiv = 1, -1
    assert api.gi_gather_div(o) == 1


def _pt2_sphere(reflection=0.0, specular=0.0, emission=0.0, **kw):
    from umbreon_gb300 import abi
    mat = abi.material(ambient=0.2, diffuse=0.6, specular=specular, reflection=reflection, emission=emission)
    sc = scenes.material_sphere_scene((0.6, 0.4, 0.2, 1.0), mat, (0.3, 0.3, 0.3))
    sc.lights = []
    kw.setdefault("pt1Spp", 4)
    opt = RenderOptions(width=32, height=32, supersample=1, gi=True, giIntegrator=2, **kw)
    return sc, opt


def test_pt2_mirror_sphere_reflects_the_sky(oracle_lib):
    """pt2's traced mirror owns the reflection term: a lone mirror-finish
    sphere's reflected rays all escape, so each hit pixel is the diffuse GI
    (sky) plus reflection x sky, and the fake reflection x background term
    is gone."""
    sc, opt = _pt2_sphere(reflection=0.5, giEnvIntensity=1.5)
    o = oracle_lib.render(sc, opt)
    hit = o.hit_geom.reshape(32, 32) != KINVALID
    col = o.color.reshape(32, 32, 4)[..., :3]
    want = 0.6 * np.array([0.6, 0.4, 0.2], np.float32) * 1.5 + 0.5 * 1.5
    np.testing.assert_allclose(col[hit], np.broadcast_to(want, col[hit].shape), rtol=2e-6)
    opt.pt2Reflect = False  # the fake term returns: + reflection x background
    f = oracle_lib.render(sc, opt).color.reshape(32, 32, 4)[..., :3]
    want = 0.6 * np.array([0.6, 0.4, 0.2], np.float32) * 1.5 + 0.5 * 0.3
    np.testing.assert_allclose(f[hit], np.broadcast_to(want, f[hit].shape), rtol=2e-6)


def test_pt2_glossy_lobe_sees_only_sky(oracle_lib):
    """A glossy finish (reflection with a highlight) samples a GGX lobe; on a
    lone sphere every sample escapes to the uniform sky, so the traced term is
    reflection x sky x the mean VNDF weight, which lies in (0, 1]."""
    sc, opt = _pt2_sphere(reflection=0.5, specular=0.3, pt2GlossySpp=8)
    o = oracle_lib.render(sc, opt)
    hit = o.hit_geom.reshape(32, 32) != KINVALID
    col = o.color.reshape(32, 32, 4)[..., :3]
    diffuse = 0.6 * np.array([0.6, 0.4, 0.2], np.float32)
    spec = col[hit] - diffuse
    assert np.all(spec > 0.0) and np.all(spec <= 0.5 * (1 + 1e-5))
    np.testing.assert_allclose(spec[:, 0], spec[:, 1], rtol=1e-5)  # grey: the sky, weighted


def test_pt2_emitter_lights_a_neighbour(oracle_lib):
    """pt2 transports emission: an emissive sphere beside a receiver brightens
    it through the gather (emission at vertices, MIS-weighted against the
    emissive NEE draw); pt1 and pt2 with emission off do not."""
    from umbreon_gb300 import abi
    sc, opt = _pt2_sphere(pt1Spp=16, giEnvIntensity=0.0)
    em = abi.material(ambient=0.2, diffuse=0.6, emission=4.0)
    sc.sphere_center_radius = np.array([[0, 0, 0, 1], [2.2, 0, 0.3, 0.8]], np.float32)
    sc.sphere_color = np.array([[0.6, 0.4, 0.2, 1.0], [1.0, 1.0, 1.0, 1.0]], np.float32)
    sc.sphere_material = np.array([sc.sphere_material[0], em], abi.MATERIAL_DTYPE)
    on = oracle_lib.render(sc, opt)
    opt.pt2Emissive = False
    off = oracle_lib.render(sc, opt)
    opt.pt2Emissive, opt.pt2EmissiveNee = True, False
    bsdf_only = oracle_lib.render(sc, opt)
    rec = (on.hit_geom.reshape(32, 32) != KINVALID) & (on.hit_prim.reshape(32, 32) == 0)
    a = on.color.reshape(32, 32, 4)[..., :3][rec].sum()
    b = off.color.reshape(32, 32, 4)[..., :3][rec].sum()
    c = bsdf_only.color.reshape(32, 32, 4)[..., :3][rec].sum()
    assert b == 0.0 and a > 0.0 and c > 0.0
    # both estimators are unbiased: their means agree within Monte-Carlo noise
    assert abs(a - c) < 0.15 * a


def _enclosed_sphere(**kw):
    """The lone sphere inside a closed spherical shell (radius 50, camera
    inside it), lit by the key light with shadows: every gather ray ends on
    the shell, and every shadow ray (the primary one and the NEE one at a
    shell vertex) is blocked by the shell."""
    sc, opt, kd = _lone_sphere(shadows=True, **kw)
    sc.sphere_center_radius = np.array([[0, 0, 0, 1], [0, 0, 0, 50]], np.float32)
    sc.sphere_color = np.array([[0.6, 0.4, 0.2, 1.0], [0.9, 0.9, 0.9, 1.0]], np.float32)
    sc.sphere_material = np.concatenate([sc.sphere_material] * 2)
    from umbreon_gb300.scenes import key_light
    sc.lights = [key_light()]
    return sc, opt, kd


def enclosed_known_answers(render, rtol=1e-6, integrator=1):
    """Closed-form pt1 answers on the enclosed sphere (pt1_gather.hpp:336-420,
    pt1EvalVertex :117-220): (1) every gather path ends on the shell, whose
    vertices' NEE is shadowed, so E = 0 and the inner sphere's pixels are
    exactly 0 at any bounce count; (2) with giMaxDistance below the gap to
    the shell every gather ray misses, so E is the sky exactly, as for the
    lone sphere.  The same holds for pt2 (`integrator` 2), whose extensions
    add no light here (no emitters, no glossy lobe, a point-like light).
    `render(scene, options)` returns (colour HxWx3, hit prim)."""
    for bounces in (1, 2, 3):
        sc, opt, kd = _enclosed_sphere(pt1Spp=8, giBounces=bounces, giIntegrator=integrator)
        col, prim = render(sc, opt)
        inner = prim == 0
        assert int(inner.sum()) > 50
        assert np.all(col[inner] == 0.0), (bounces, float(np.abs(col[inner]).max()))
    sc, opt, kd = _enclosed_sphere(pt1Spp=8, giBounces=2, giMaxDistance=10.0, giIntegrator=integrator)
    col, prim = render(sc, opt)
    inner = prim == 0
    want = kd * np.array([0.6, 0.4, 0.2], np.float32)
    np.testing.assert_allclose(col[inner], np.broadcast_to(want, col[inner].shape), rtol=rtol, atol=rtol / 10)


@pytest.mark.parametrize("integrator", [1, 2])
def test_enclosed_sphere_known_answers(oracle_lib, integrator):
    def render(sc, opt):
        o = oracle_lib.render(sc, opt)
        prim = np.where(o.hit_geom.reshape(32, 32) == KINVALID, -1, o.hit_prim.reshape(32, 32).astype(np.int64))
        return o.color.reshape(32, 32, 4)[..., :3], prim
    enclosed_known_answers(render, integrator=integrator)
