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
    opt = RenderOptions(width=32, height=32, supersample=1, gi=True, giIntegrator=1, pt1Denoise=False,
                        pt1GatherDiv=1, **kw)
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


@pytest.mark.parametrize("bad,msg", [(dict(giIntegrator=2), "pt1"), (dict(pt1Denoise=True), "denoise"),
                                     (dict(supersample=2, pt1GatherDiv=-1), "full-resolution"),
                                     (dict(pt1GatherDiv=0, pt1HalfRes=True), "full-resolution")])
def test_unbuilt_gi_settings_raise(bad, msg):
    opt = RenderOptions(width=8, height=8, gi=True, giIntegrator=1, pt1Denoise=False, pt1GatherDiv=1)
    for k, v in bad.items():
        setattr(opt, k, v)
    with pytest.raises(ValueError, match=msg):
        api.check_gi(opt)


def test_gather_div_resolution():
    o = RenderOptions(width=8, height=8, supersample=2)
    assert api.gi_gather_div(o) == 2            # -1 = the supersample factor
    o.pt1GatherDiv, o.pt1HalfRes = 0, False
    assert api.gi_gather_div(o) == 1
    o.supersample, o.pt1GatherDiv = 1, -1
    assert api.gi_gather_div(o) == 1
