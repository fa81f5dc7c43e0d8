"""The BVH builders (Karras radix tree, PLOC clustering) and collapses
(greedy, SAH-optimal) give the same frames: hits do not depend on the tree
(ties resolve to the lowest ids)."""
import numpy as np
import pytest

from umbreon_gb300 import scenes

pytestmark = pytest.mark.gpu

CASES = {
    "ball_and_stick": lambda: scenes.ball_and_stick(n=3000, width=160, height=90, supersample=2, ao_samples=8),
    "space_filling": lambda: scenes.space_filling(width=160, height=120),
    "molecular_surface": lambda: scenes.molecular_surface(n_atoms=600, n_spheres=200, box=16.0, width=96,
                                                          height=96, ao_samples=8),
    "differentiable": lambda: scenes.differentiable(n=2000, res=96),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_builders_render_identically(name):
    from umbreon_gb300.api import Context
    sc, opt = CASES[name]()
    out = {}
    for key in ((1, 1), (2, 1), (1, 2), (2, 2)):  # (builder, collapse)
        ctx = Context(0, bvh_builder=key[0], bvh_collapse=key[1])
        b = ctx.build(sc)
        fr = ctx.render(b, sc, opt)
        out[key] = (fr.color.copy(), fr.hit_prim.copy(), b.info()["bvh_nodes"])
        b.release()
        ctx.close()
    for key in out:
        assert np.array_equal(out[(1, 1)][1], out[key][1]), key
        assert np.array_equal(out[(1, 1)][0], out[key][0]), key


@pytest.mark.parametrize("name", sorted(CASES))
def test_occlusion_kernels_render_identically(name):
    """The four occlusion kernels (one thread per ray, persistent refill,
    resident grid with shared-memory top levels, interleaved node / primitive
    steps) give the same frame."""
    from umbreon_gb300.api import Context
    sc, opt = CASES[name]()
    out = {}
    for mode in (1, 2, 3, 4):
        ctx = Context(0, trace_mode=mode)
        b = ctx.build(sc)
        out[mode] = ctx.render(b, sc, opt).color.copy()
        b.release()
        ctx.close()
    for mode in (2, 3, 4):
        assert np.array_equal(out[1], out[mode]), mode

