"""The stroke-edge pass's first-hit G-buffer (ubr_render_desc.edge_gbuffer)
on the GPU against the oracle: (section << 2) | kind object ids and global
material ids (exact), shading normals and surface opacity (1e-5), on pixels
whose first hit agrees; the clip-cut planes under view clipping."""
import copy

import numpy as np
import pytest

from umbreon_gb300 import abi, scenes
from umbreon_gb300.abi import UbrError

pytestmark = pytest.mark.gpu


def _render(gpu_ctx, sc, opt):
    b = gpu_ctx.build(sc)
    try:
        return gpu_ctx.render(b, sc, opt)
    finally:
        b.release()


def _check(g, o):
    agree = (g.hit_geom == o.hit_geom) & (g.hit_prim == o.hit_prim)
    assert agree.mean() >= 0.999
    assert np.array_equal(g.objectId[agree], o.objectId[agree])
    assert np.array_equal(g.materialId[agree], o.materialId[agree])
    assert float(np.abs(g.gbNormal - o.gbNormal)[agree].max()) <= 1e-5
    assert float(np.abs(g.surfAlpha - o.surfAlpha)[agree].max()) <= 1e-5
    assert np.array_equal(g.clipCut[agree], o.clipCut[agree])
    for k in ("clipNearVz", "clipFarVz"):
        assert float(np.abs(getattr(g, k) - getattr(o, k))[agree].max()) <= 1e-4


def _sections_and_materials(sc, seed):
    rng = np.random.default_rng(seed)
    if sc.sphere_center_radius is not None:
        sc.sphere_group = rng.integers(0, 5, sc.sphere_count()).astype(np.uint16)
    if sc.cyl_radius is not None:
        n = len(sc.cyl_radius)
        sc.cyl_group = rng.integers(0, 5, n).astype(np.uint16)
        sc.cyl_open = (rng.random(n) < 0.5).astype(np.uint8)
    return sc


@pytest.mark.parametrize("clip", [False, True])
def test_edge_gbuffer_ball_and_stick(gpu_ctx, oracle_lib, clip):
    sc, opt = scenes.ball_and_stick(n=800, width=96, height=64, supersample=2, ao_samples=0)
    sc = _sections_and_materials(sc, 3)
    sc.sphere_color[::3, 3] = 0.5
    if clip:
        z = float(sc.camera.position[2])
        sc.clipNear, sc.clipFar = z - 10.0, z + 2.0
    opt.edgeGBuffer = True
    _check(_render(gpu_ctx, sc, opt), oracle_lib.render(sc, opt))


def test_edge_gbuffer_mesh_instances(gpu_ctx, oracle_lib):
    sc, opt = scenes.molecular_surface(n_atoms=300, box=12.0, n_spheres=100, width=64, height=64,
                                       ao_samples=0, layers=2)
    nt = sc.triangle_count()
    rng = np.random.default_rng(5)
    sc.mesh_materials = np.full(3, scenes.pov_material(), abi.MATERIAL_DTYPE)
    sc.mesh_tri_material = rng.integers(0, 3, nt).astype(np.uint8)
    sc.mesh_tri_group = rng.integers(0, 4, nt).astype(np.uint16)
    sc.instance_offsets = np.array([[0, 0, 0], [2.0, 0.0, -30.0]], np.float32)
    opt.edgeGBuffer = True
    _check(_render(gpu_ctx, sc, opt), oracle_lib.render(sc, opt))


def test_edge_gbuffer_rejects_adaptive(gpu_ctx):
    sc, opt = scenes.space_filling(n=50, width=16, height=16)
    opt.supersample, opt.aaMode, opt.edgeGBuffer = 2, 1, True
    with pytest.raises(UbrError):
        _render(gpu_ctx, sc, opt)
