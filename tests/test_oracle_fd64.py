"""The float64 restatement used to check the adjoint by finite differences
(oracle/fd64.py) against the float oracle, on the CPU."""
import numpy as np
import pytest

from umbreon_gb300 import scenes


@pytest.fixture(scope="module")
def small():
    from oracle import fd64
    sc, opt = scenes.differentiable(n=300, res=48)
    f = fd64.Fd64Frame(sc, opt, threads=4)
    img = f.record()
    return sc, opt, f, img


def test_fd64_matches_float_oracle(small):
    """Same frame as the float restatement of the path (pinned on the
    reference's known-answer tests): same first hits, colours within float
    rounding."""
    from oracle import oracle
    sc, opt, f, img = small
    fr = oracle.OracleScene(sc).render(sc, opt, threads=4)
    oid = np.where(fr.hit_geom == 0xFFFFFFFF, -1, fr.hit_prim.astype(np.int64))
    assert (f.primary_ids() == oid).mean() >= 0.999
    agree = f.primary_ids() == oid
    d = np.abs(fr.color[..., :3] - img[..., :3])[agree]
    assert d.max() <= 5e-5, d.max()


def test_frozen_visibility_reproduces_record(small):
    sc, opt, f, img = small
    assert np.array_equal(f.frozen(), img)


def test_finite_differences_converge(small):
    """With visibility held fixed the loss is smooth (up to the kinks of the
    clamps, e.g. an AO hit at the AO distance): steps 1e-4 and 2e-4 agree."""
    sc, opt, f, img = small
    rng = np.random.default_rng(3)
    target = img + 0.05 * rng.standard_normal(img.shape)
    w = np.ones(img.shape[:2])
    ids = f.primary_ids()
    k = int(np.bincount(ids[ids >= 0]).argmax())
    for name, idx in [("diffuse", ()), ("phong_size", ()), ("light_direction", (0, 1)), ("fog_end", ()),
                      ("ao_distance", ()), ("sphere_center", (k, 0)), ("sphere_radius", (k,))]:
        a = f.fd(name, idx, target, w, h=1e-4)
        b = f.fd(name, idx, target, w, h=2e-4)
        assert abs(a - b) <= 1e-3 * max(abs(a), 1e-6) + 1e-9, (name, a, b)
