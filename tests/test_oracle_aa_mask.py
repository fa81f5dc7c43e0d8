"""The refinement-mask predicates of the reference's adaptive-AA tests
(tests/test_adaptive_aa.cpp:233-316), restated on hand-built centre records
and run through the oracle's mask builder (adaptive_aa.hpp:65-190)."""
import numpy as np

from oracle import oracle

INVALID = 0xFFFFFFFF
PX_WORLD = 0.1  # output-pixel world size stand-in (test_adaptive_aa.cpp:233)


def flat(Wf, Hf):
    """Identical flat-surface centres (test_adaptive_aa.cpp:72-84): colour
    0.5, alpha 1, geomID 1, section 0, view z 10, normal +z."""
    rgba = np.tile(np.array([0.5, 0.5, 0.5, 1.0], np.float32), (Hf, Wf, 1))
    vz = np.full((Hf, Wf), 10.0, np.float32)
    geom = np.ones((Hf, Wf), np.uint32)
    group = np.zeros((Hf, Wf), np.int32)
    nrm = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (Hf, Wf, 1))
    return dict(rgba=rgba, view_z=vz, geom=geom, group=group, normal=nrm)


def mask(c):
    return oracle.aa_mask(pixel_world_size=PX_WORLD, **c)


def test_flat_grid_empty():
    assert mask(flat(8, 8)).sum() == 0


def test_geom_boundary_pair_plus_ring():
    c = flat(8, 8)
    c["geom"][:, 4:] = 2
    m = mask(c)
    expect = np.zeros((8, 8), np.uint8)
    expect[:, 2:6] = 1  # pair {3, 4} + one-ring dilation
    assert np.array_equal(m, expect)


def test_section_boundary_fires():
    c = flat(8, 8)
    c["group"][:, 4:] = 3
    assert mask(c).sum() > 0


def test_colour_contrast_threshold():
    c = flat(8, 1)
    c["rgba"][0, 4, 1] += np.float32(0.09)
    assert mask(c).sum() == 0
    c["rgba"][0, 4, 1] += np.float32(0.02)
    assert mask(c).sum() > 0
    c2 = flat(8, 1)
    c2["rgba"][0, 4, 3] = 0.7
    assert mask(c2).sum() > 0


def test_normal_delta():
    c = flat(8, 1)
    c["normal"][0, 4:] = (0.6, 0.0, 0.8)  # 1 - cos = 0.2
    assert mask(c).sum() == 0
    c["normal"][0, 4:] = (1.0, 0.0, 0.0)  # 1 - cos = 1
    assert mask(c).sum() > 0


def test_depth_crack_and_slope_compensation():
    c = flat(8, 1)
    c["view_z"][0] = 10.0 + 3.0 * np.arange(8, dtype=np.float32)
    assert mask(c).sum() == 0
    c = flat(8, 1)
    c["view_z"][0, 4:] = 13.0
    assert mask(c).sum() > 0


def test_background_pairs_quiet_but_hit_miss_fires():
    c = flat(8, 1)
    c["geom"][:] = INVALID
    c["group"][:] = -1
    c["normal"][:] = 0.0
    c["view_z"][:] = 0.0
    assert mask(c).sum() == 0
    c["geom"][0, :4] = 1
    c["group"][0, :4] = 0
    assert mask(c).sum() > 0


def test_perspective_scales_the_absolute_floor():
    c = flat(8, 1)
    c["view_z"][0, 4:] = 10.5  # step 0.5 > 12 * 0.1 * ... only without the |z| scale
    c["view_z"][0, :4] = 10.0
    # orthographic floor 1.2 > 0.5: quiet; perspective floor 1.2 * 10 = 12: quiet
    assert mask(c).sum() == 0
    c["view_z"][0, 4:] = 11.5  # step 1.5: above 1.2, below 12
    assert oracle.aa_mask(pixel_world_size=PX_WORLD, perspective=False, **c).sum() > 0
    assert oracle.aa_mask(pixel_world_size=PX_WORLD, perspective=True, **c).sum() == 0
