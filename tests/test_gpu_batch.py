"""Batched rendering (ubr_render_batch) and CUDA-graph replay.

A batch runs every stage once over the pixels and rays of all its frames, so
each frame of a batch must be bit-identical to the same frame rendered alone
(per-pixel work does not depend on which other pixels share a launch)."""
import numpy as np
import pytest

from umbreon_gb300 import scenes

pytestmark = pytest.mark.gpu


def _items(gpu_ctx):
    a_sc, a_opt = scenes.space_filling(n=700, width=96, height=72)
    b_sc, b_opt = scenes.ball_and_stick(n=1500, width=80, height=48, supersample=2, ao_samples=8)
    c_sc, c_opt = scenes.space_filling(n=400, width=64, height=64)
    c_opt.aoSamples, c_opt.aoDistance, c_opt.aoFalloffPower = 6, 4.0, 1.0   # enhanced AO, other stride
    c_opt.shadows = True
    d_sc, d_opt = scenes.molecular_surface(n_atoms=300, box=12.0, n_spheres=100, width=72, height=72,
                                           ao_samples=4, layers=3)                # transparent: several rounds
    items = []
    for sc, opt in ((a_sc, a_opt), (b_sc, b_opt), (c_sc, c_opt), (d_sc, d_opt), (a_sc, a_opt)):
        items.append((gpu_ctx.build(sc), sc, opt))
    return items


def test_batch_equals_single_frames(gpu_ctx):
    items = _items(gpu_ctx)
    try:
        batch, stats = gpu_ctx.render_batch(items)
        assert stats["layers"] >= 2  # the transparent frame forces the multi-round path
        for (built, sc, opt), got in zip(items, batch):
            ref = gpu_ctx.render(built, sc, opt)
            assert np.array_equal(got.color, ref.color)
            assert np.array_equal(got.depth, ref.depth)
            assert np.array_equal(got.hit_prim, ref.hit_prim)
        # opaque frames only: one round, replayed from the captured graph
        opaque = [items[0], items[1], items[2]]
        first, s1 = gpu_ctx.render_batch(opaque)
        again, s2 = gpu_ctx.render_batch(opaque)
        assert s1["layers"] == 1 and s2["layers"] == 1
        for x, y in zip(first, again):
            assert np.array_equal(x.color, y.color)
    finally:
        for built, _, _ in items:
            built.release()


def test_single_frame_graph_replay(gpu_ctx):
    sc, opt = scenes.ball_and_stick(n=2000, width=128, height=72, supersample=2, ao_samples=8)
    built = gpu_ctx.build(sc)
    try:
        frames = [gpu_ctx.render(built, sc, opt) for _ in range(3)]
        for f in frames[1:]:
            assert np.array_equal(f.color, frames[0].color)
            assert np.array_equal(f.hit_prim, frames[0].hit_prim)
        opt2 = scenes.ball_and_stick(n=2000, width=128, height=72, supersample=2, ao_samples=4)[1]
        g = gpu_ctx.render(built, sc, opt2)      # parameters change: graph re-captured / updated
        assert not np.array_equal(g.color, frames[0].color)
        h = gpu_ctx.render(built, sc, opt)
        assert np.array_equal(h.color, frames[0].color)
    finally:
        built.release()


def test_batch_frames_of_ragged_sizes(gpu_ctx):
    """Frames whose hi-res grids are not multiples of the 8 x 4 pixel tiles
    of a first round (a right strip and a bottom band outside the tiles)
    render in a batch exactly as alone."""
    a_sc, a_opt = scenes.space_filling(n=500, width=67, height=45)
    b_sc, b_opt = scenes.ball_and_stick(n=1200, width=53, height=37, supersample=3, ao_samples=4)
    c_sc, c_opt = scenes.space_filling(n=300, width=13, height=7)
    items = [(gpu_ctx.build(sc), sc, opt) for sc, opt in ((a_sc, a_opt), (b_sc, b_opt), (c_sc, c_opt))]
    try:
        batch, _ = gpu_ctx.render_batch(items)
        for (built, sc, opt), got in zip(items, batch):
            ref = gpu_ctx.render(built, sc, opt)
            assert np.array_equal(got.color, ref.color)
            assert np.array_equal(got.depth, ref.depth)
            assert np.array_equal(got.hit_prim, ref.hit_prim)
            assert np.isfinite(ref.color).all()
    finally:
        for built, _, _ in items:
            built.release()
