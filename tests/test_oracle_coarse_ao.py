"""Coarse-grid AO (RenderOptions::aoResDiv) in the oracle, pinned on the
reference's own tests (tests/test_ao_coarse.cpp): the bilateral lookup on
hand-built grids (:97-204)."""

import numpy as np

from oracle import oracle
from umbreon_gb300.api import RenderOptions

UP = (0.0, 0.0, 1.0)


def grid(w, h, depth, openness):
    """Eligible flat cells: normal +z, constant depth (test_ao_coarse.cpp:22-35)."""
    n = np.zeros((h, w, 3), np.float32)
    n[..., 2] = 1.0
    return dict(openness=np.asarray(openness, np.float32).reshape(h, w), normal=n,
                depth=np.full((h, w), depth, np.float32), hit=np.ones((h, w), np.uint8))


def look(g, lattice, px, py, N=UP, z=10.0, **q):
    return oracle.coarse_ao_lookup(g["openness"], g["normal"], g["depth"], g["hit"], lattice, px, py, N, z, **q)


def test_bilinear_interior():
    g = grid(2, 2, 10.0, [0, 1, 0, 1])
    a, b = look(g, (8, 8), 3, 3), look(g, (8, 8), 4, 3)
    assert a is not None and b is not None
    assert abs(0.5 * (a[0] + b[0]) - 0.5) <= 1e-5
    assert a[0] < 0.5 < b[0]
    c = look(g, (8, 8), 1, 1)
    assert c is not None and c[0] < 0.4


def test_depth_rejection():
    g = grid(2, 2, 10.0, [0.5] * 4)
    assert look(g, (8, 8), 4, 4, z=10.0) is not None
    assert look(g, (8, 8), 4, 4, z=20.0) is None


def test_normal_rejection():
    g = grid(2, 2, 10.0, [0.5] * 4)
    assert look(g, (8, 8), 4, 4, N=(1.0, 0.0, 0.0)) is None
    mild = np.array([0.2, 0.0, 1.0], np.float32)
    mild /= np.linalg.norm(mild)
    assert look(g, (8, 8), 4, 4, N=mild) is not None


def test_all_miss_quad():
    g = grid(2, 2, 10.0, [0.5] * 4)
    g["hit"][:] = 0
    assert look(g, (8, 8), 4, 4) is None


def test_quality_channels():
    g = grid(2, 2, 10.0, [0.5] * 4)
    bent = np.zeros((2, 2, 3), np.float32)
    bent[..., 2] = 1.0
    r = look(g, (8, 8), 4, 4, bent=bent, contact=np.full((2, 2), 0.25, np.float32),
             shape=np.full((2, 2), 0.75, np.float32), avg=np.full((2, 2), 2.0, np.float32))
    assert r is not None
    assert abs(r[1][2] - 1.0) <= 1e-5 and abs(r[1][0]) <= 1e-5
    assert abs(r[2] - 0.25) <= 1e-5 and abs(r[3] - 0.75) <= 1e-5
    legacy = look(grid(2, 2, 10.0, [0.5] * 4), (8, 8), 4, 4)
    assert legacy is not None and legacy[2] == 1.0 and legacy[3] == 1.0
    assert legacy[1][0] == 0.0 and legacy[1][2] == 0.0


def test_border_clamp():
    g = grid(3, 3, 10.0, [0.5] * 9)
    for p in (0, 8):
        assert look(g, (9, 9), p, 0) is not None
        assert look(g, (9, 9), 0, p) is not None
        assert look(g, (9, 9), p, p) is not None


# The renderer cases (test_ao_coarse.cpp:210-384) are known-answer cases in
# kat_cases.py, run on the oracle and on the GPU; thread-count invariance is
# the oracle's own property.

def test_determinism_and_threads():
    from kat_cases import ao_coarse_scene
    sc = ao_coarse_scene()
    o = RenderOptions(width=12, height=12, supersample=2, aoSamples=16, aoDistance=100.0, aoResDiv=-1)
    a = oracle.OracleScene(sc).render(sc, o, threads=1)
    b = oracle.render(sc, o)
    assert np.array_equal(a.color, b.color)
