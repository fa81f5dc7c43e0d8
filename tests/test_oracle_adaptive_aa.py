"""The oracle's adaptive-AA restatement (embree_renderer.cpp:1379-1670,
render/adaptive_aa.hpp) against properties the reference states for it:
flagged blocks are bitwise the full-grid render, a fine lattice at ss 1 with
aaDepth 2 samples the ss 2 grid's points with its seeds, the mask is a
dilated (3x3) set, and a zero threshold flags at least as much."""
import copy

import numpy as np
import pytest

from umbreon_gb300 import scenes


def _scene(ss, ao=8):
    sc, opt = scenes.molecular_surface(n_atoms=300, box=12.0, n_spheres=150, width=48, height=48,
                                       ao_samples=ao, layers=2)
    opt.supersample = ss
    return sc, opt


def _adaptive(opt, **kw):
    a = copy.copy(opt)
    a.aaMode, a.aaDebug = 1, True
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def test_flagged_blocks_equal_grid(oracle_lib):
    sc, opt = _scene(2)
    grid = oracle_lib.render(sc, opt)
    ad = oracle_lib.render(sc, _adaptive(opt))
    m = ad.aaMask > 0
    assert 0.05 < m.mean() < 0.95
    assert np.array_equal(ad.color[m], grid.color[m])
    # AO on mesh hits: replicated blocks carry a re-shaded centre, not the grid
    assert not np.array_equal(ad.color[~m], grid.color[~m])


def test_fine_lattice_ss1_is_ss2_grid(oracle_lib):
    sc, opt = _scene(1)
    ad = oracle_lib.render(sc, _adaptive(opt, aaDepth=2))
    g2 = copy.copy(opt)
    g2.supersample = 2
    grid2 = oracle_lib.render(sc, g2)
    grid1 = oracle_lib.render(sc, opt)
    m = ad.aaMask > 0
    assert m.any() and (~m).any()
    assert np.array_equal(ad.color[m], grid2.color[m])
    assert np.array_equal(ad.color[~m], grid1.color[~m])


def test_mask_is_dilated(oracle_lib):
    sc, opt = _scene(2, ao=0)
    m = oracle_lib.render(sc, _adaptive(opt)).aaMask > 0
    # every flagged pixel has a flagged 4- or 8-neighbour (one dilation ring
    # around raw pairs, which always flag two pixels)
    pad = np.pad(m, 1)
    nb = sum(np.roll(np.roll(pad, dy, 0), dx, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)
             if (dy, dx) != (0, 0))[1:-1, 1:-1]
    assert np.all(nb[m] > 0)


@pytest.mark.parametrize("thr", [0.0, 0.05])
def test_lower_threshold_flags_superset(oracle_lib, thr):
    sc, opt = _scene(2, ao=0)
    lo = oracle_lib.render(sc, _adaptive(opt, aaThreshold=thr)).aaMask
    hi = oracle_lib.render(sc, _adaptive(opt, aaThreshold=0.5)).aaMask
    assert np.all(lo >= hi)
