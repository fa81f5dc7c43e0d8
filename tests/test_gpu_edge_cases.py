"""Edge cases of the C-ABI path on the GPU: empty and single-kind scenes,
ragged frame sizes, degenerate primitives, argument errors and the size
guard, cancellation, empty batches and queries.  Where an image is produced
it is compared with the oracle under the grid parity bars."""
import copy

import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_srgb
from umbreon_gb300 import abi, scenes
from umbreon_gb300.abi import UbrError
from umbreon_gb300.api import RenderOptions, Scene

pytestmark = pytest.mark.gpu


def _render(gpu_ctx, sc, opt, **kw):
    b = gpu_ctx.build(sc)
    try:
        return gpu_ctx.render(b, sc, opt, **kw)
    finally:
        b.release()


def _close_to_oracle(gpu_ctx, oracle_lib, sc, opt):
    g = _render(gpu_ctx, sc, opt)
    o = oracle_lib.render(sc, opt)
    ss = max(1, opt.supersample)
    assert id_agreement(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim) >= 0.999
    m = agree_mask_final(g.hit_geom, g.hit_prim, o.hit_geom, o.hit_prim, ss)
    assert float(np.abs(g.color - o.color)[m].max(initial=0.0)) <= 1e-3
    assert psnr_srgb(g.color, o.color) >= 45.0
    return g, o


def test_empty_scene_is_background(gpu_ctx):
    sc = Scene()
    sc.camera = scenes.ortho_cam()
    sc.background = (0.25, 0.5, 0.75)
    f = _render(gpu_ctx, sc, RenderOptions(width=7, height=5, supersample=2, aoSamples=4, shadows=True))
    assert np.allclose(f.color[..., :3], (0.25, 0.5, 0.75)) and np.all(f.color[..., 3] == 1.0)
    assert np.all(f.depth == 0.0) and np.all(f.hit_geom == 0xFFFFFFFF)


@pytest.mark.parametrize("w,h,ss", [(1, 1, 1), (1, 1, 3), (7, 5, 3), (13, 1, 2), (1, 9, 4)])
def test_ragged_frames(gpu_ctx, oracle_lib, w, h, ss):
    sc, opt = scenes.space_filling(n=300, width=w, height=h)
    opt.supersample = ss
    opt.aoSamples = 0
    _close_to_oracle(gpu_ctx, oracle_lib, sc, opt)


def test_degenerate_primitives(gpu_ctx, oracle_lib):
    """Zero-radius spheres, zero-length and zero-radius cylinders, collinear
    and zero-area triangles render finite pixels that match the oracle."""
    sc, opt = scenes.space_filling(n=200, width=48, height=36)
    cr = sc.sphere_center_radius.copy()
    cr[::7, 3] = 0.0
    sc.sphere_center_radius = cr
    p0 = cr[:20, :3].copy()
    p1 = p0.copy()
    p1[10:] += np.float32(2.0)
    sc.cyl_p0, sc.cyl_p1 = p0, p1
    sc.cyl_radius = np.where(np.arange(20) % 3 == 0, 0.0, 0.3).astype(np.float32)
    sc.cyl_color = np.ones((20, 4), np.float32)
    sc.cyl_material = np.full(20, scenes.pov_material(), abi.MATERIAL_DTYPE)
    sc.cyl_open = (np.arange(20) % 2).astype(np.uint8)
    tri = np.array([[0, 0, 0], [1, 1, 1], [2, 2, 2],      # collinear
                    [5, 5, 5], [5, 5, 5], [5, 5, 5],      # a point
                    [3, 0, 0], [3, 4, 0], [0, 4, 0]], np.float32) + cr[0, :3]
    sc.mesh_positions = tri
    sc.mesh_normals = np.tile([0, 0, 1], (9, 1)).astype(np.float32)
    sc.mesh_colors = np.ones((9, 4), np.float32)
    g, o = _close_to_oracle(gpu_ctx, oracle_lib, sc, opt)
    assert np.all(np.isfinite(g.color))


def test_argument_errors(gpu_ctx):
    sc, opt = scenes.space_filling(n=50, width=8, height=8)
    import ctypes as C
    from umbreon_gb300.api import make_render_desc
    b = gpu_ctx.build(sc)
    try:
        # bad sizes and sample counts, and a supersampled frame of 2^31
        # pixels or more, are refused before any allocation (no output
        # buffers are passed)
        for bad in (dict(width=0), dict(height=-1), dict(aoSamples=-1),
                    dict(width=23171, height=23171, supersample=2)):
            o = copy.copy(opt)
            for k, v in bad.items():
                setattr(o, k, v)
            rd, keep = make_render_desc(sc, o)
            fr = abi.Frame()
            st = gpu_ctx._L.ubr_render(gpu_ctx.handle, b.handle, C.byref(rd), C.byref(fr), None, None)
            assert st == abi.UBR_INVALID_ARGUMENT, bad
        # the context stays usable
        assert gpu_ctx.render(b, sc, opt).color.shape == (8, 8, 4)
    finally:
        b.release()


def test_cancel_before_start(gpu_ctx):
    sc, opt = scenes.space_filling(n=50, width=8, height=8)
    flag = np.ones(1, np.int32)
    with pytest.raises(UbrError) as e:
        _render(gpu_ctx, sc, opt, cancel=flag)
    assert e.value.status == abi.UBR_CANCELLED
    flag[0] = 0
    assert _render(gpu_ctx, sc, opt, cancel=flag).color.shape == (8, 8, 4)


def test_empty_batch_and_queries(gpu_ctx):
    frames, stats = gpu_ctx.render_batch([])
    assert frames == []
    sc, opt = scenes.space_filling(n=50, width=8, height=8)
    b = gpu_ctx.build(sc)
    try:
        out = gpu_ctx.occluded(b, np.zeros((0, 6), np.float32), 1e-4)
        assert out.shape == (0,)
    finally:
        b.release()


def test_arena_cap_reports_out_of_memory(gpu_ctx):
    """A context whose device arena cap is too small for the frame refuses
    with UBR_OUT_OF_MEMORY and stays usable for smaller work."""
    from umbreon_gb300.api import Context
    sc, opt = scenes.space_filling(n=200, width=64, height=48)
    small = Context(0, arena_bytes=4 << 20)
    try:
        b = small.build(sc)
        try:
            big = copy.copy(opt)
            big.width, big.height, big.supersample = 1024, 1024, 2
            with pytest.raises(UbrError) as e:
                small.render(b, sc, big, want_ids=False)
            assert e.value.status == abi.UBR_OUT_OF_MEMORY
            tiny = copy.copy(opt)
            tiny.width, tiny.height = 16, 12
            assert small.render(b, sc, tiny).color.shape == (12, 16, 4)
        finally:
            b.release()
    finally:
        small.close()
