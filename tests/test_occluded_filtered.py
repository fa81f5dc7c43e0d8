"""Filtered segment visibility of the stroke-edge pass (EmbreeRenderer::occluded
with excludeFaceFilter, embree_renderer.cpp:76-133, 294-357): known answers on
the oracle (CPU) and GPU == oracle on random segments (GPU)."""
import numpy as np
import pytest

from umbreon_gb300 import abi, scenes
from umbreon_gb300.api import Scene


def _quad_and_sphere(instances=None):
    pos, nrm, col = scenes.quad_mesh()
    sc = Scene(mesh_positions=pos, mesh_normals=nrm, mesh_colors=col,
               sphere_center_radius=np.array([[0.0, 0.0, 5.0, 1.0]], np.float32),
               sphere_color=np.array([[1, 1, 1, 1]], np.float32),
               sphere_material=np.full(1, abi.material(), abi.MATERIAL_DTYPE))
    if instances is not None:
        sc.instance_offsets = np.asarray(instances, np.float32)
    return sc


def _seg(a, b):
    return np.array([list(a) + list(b)], np.float32)


@pytest.fixture(scope="module")
def osc():
    from oracle import oracle
    return oracle.OracleScene(_quad_and_sphere())


def test_plain_hit_and_face_exclusion(osc):
    s = _seg((0.5, -0.5, 1.0), (0.5, -0.5, -1.0))   # crosses triangle 0 of the quad
    assert osc.occluded_filtered(s, 1e-4)[0] == 1
    assert osc.occluded_filtered(s, 1e-4, exclude_faces=[[0]])[0] == 0
    assert osc.occluded_filtered(s, 1e-4, exclude_faces=[[1]])[0] == 1
    assert osc.occluded_filtered(s, 1e-4, exclude_faces=[[1, 0]])[0] == 0


def test_grazing_face_is_not_an_occluder(osc):
    # 0.5 degrees off the quad's plane: |cos| = sin(0.5 deg) = 0.0087
    ang = np.radians(0.5)
    d = np.array([np.cos(ang), 0.0, -np.sin(ang)])
    a = np.array([-1.0, 0.3, 0.0]) - d * 1.0
    s = _seg(a, a + 2.0 * d)
    assert osc.occluded_filtered(s, 1e-4)[0] == 1
    assert osc.occluded_filtered(s, 1e-4, graze_cos_eps=0.01)[0] == 0
    assert osc.occluded_filtered(s, 1e-4, graze_cos_eps=0.005)[0] == 1


def test_coincident_plane_is_not_an_occluder(osc):
    # starts 2e-4 above the quad, leaves through it: perpendicular distance 2e-4
    s = _seg((0.3, 0.2, 2e-4), (0.3, 0.2, -1.0))
    assert osc.occluded_filtered(s, 1e-6)[0] == 1
    assert osc.occluded_filtered(s, 1e-6, coplanar_eps=1e-3)[0] == 0
    assert osc.occluded_filtered(s, 1e-6, coplanar_eps=1e-4)[0] == 1


def test_sphere_exit_point_still_occludes(osc):
    # starts just above the sphere's top (tangent plane within 1e-3): the entry
    # is coincident, the exit point on the far side is a real occluder
    s = _seg((0.0, 0.0, 6.0 + 2e-4), (0.0, 0.0, 3.0))
    assert osc.occluded_filtered(s, 1e-6, coplanar_eps=1e-3)[0] == 1
    assert osc.occluded_filtered(_seg((0.0, 0.0, 6.0 + 2e-4), (0.0, 0.0, 5.0)), 1e-6, coplanar_eps=1e-3)[0] == 0


def test_instanced_faces_compare_modulo_base_triangles():
    from oracle import oracle
    o = oracle.OracleScene(_quad_and_sphere(instances=[[0, 0, 0], [10, 0, 0]]))
    s = _seg((10.5, -0.5, 1.0), (10.5, -0.5, -1.0))  # triangle 2 = copy of triangle 0
    assert o.occluded_filtered(s, 1e-4)[0] == 1
    assert o.occluded_filtered(s, 1e-4, exclude_faces=[[0]])[0] == 0


def _random_queries(sc, n, seed):
    """Segments that start on mesh triangles (their own face excluded, as the
    edge pass does) or in free space, with random exclusions."""
    rng = np.random.default_rng(seed)
    pos = np.asarray(sc.mesh_positions, np.float32)
    idx = np.asarray(sc.mesh_index, np.int64).reshape(-1, 3)
    t = rng.integers(0, len(idx), n)
    w = rng.dirichlet([1, 1, 1], n)
    a = np.einsum("nk,nkd->nd", w, pos[idx[t]])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    b = a + d * rng.uniform(0.5, 8.0, (n, 1))
    free = rng.random(n) < 0.3
    a[free] += rng.normal(scale=3.0, size=(int(free.sum()), 3))
    segs = np.concatenate([a, b], 1).astype(np.float32)
    faces = [[int(t[i])] + list(rng.integers(0, len(idx), rng.integers(0, 3))) for i in range(n)]
    return segs, faces


@pytest.mark.gpu
@pytest.mark.parametrize("graze,coplanar", [(0.0, 0.0), (0.05, 0.0), (0.0, 1e-3), (0.05, 1e-3)])
def test_gpu_matches_oracle(graze, coplanar):
    from oracle import oracle
    from umbreon_gb300.api import Context
    sc, _ = scenes.molecular_surface(n_atoms=400, n_spheres=150, box=14.0, width=32, height=32, ao_samples=0)
    segs, faces = _random_queries(sc, 20000, seed=int(graze * 100 + coplanar * 1e4))
    ref = oracle.OracleScene(sc).occluded_filtered(segs, 1e-4, graze, coplanar, faces)
    ctx = Context(0)
    built = ctx.build(sc)
    got = ctx.occluded_filtered(built, segs, 1e-4, graze, coplanar, faces)
    plain = ctx.occluded(built, segs, 1e-4)
    built.release()
    ctx.close()
    assert (got == ref).mean() >= 0.999
    assert ref.sum() > 1000 and (ref == 0).sum() > 1000
    # filtering only removes occluders
    assert np.all(got <= plain)


@pytest.mark.gpu
@pytest.mark.parametrize("workload", ["ball_and_stick", "molecular_surface"])
def test_gpu_plain_segments_match_oracle(workload):
    """ubr_occluded_batch (the plain any-hit branch, embree_renderer.cpp:
    294-315) against the oracle's test of the same trimmed open segments, on
    spheres + capped cylinders and on a mesh + spheres."""
    from oracle import oracle
    from umbreon_gb300.api import Context
    if workload == "ball_and_stick":
        sc, _ = scenes.ball_and_stick(n=4000, width=32, height=32, supersample=1)
        rng = np.random.default_rng(11)
        pos = sc.sphere_center_radius[:, :3]
        a = rng.uniform(pos.min(0) - 1.0, pos.max(0) + 1.0, size=(50000, 3))
        segs = np.concatenate([a, a + rng.normal(scale=3.0, size=(50000, 3))], 1).astype(np.float32)
    else:
        sc, _ = scenes.molecular_surface(n_atoms=400, n_spheres=150, box=14.0, width=32, height=32, ao_samples=0)
        segs, _ = _random_queries(sc, 50000, seed=5)
    ref = oracle.OracleScene(sc).occluded_filtered(segs, 1e-4)
    ctx = Context(0)
    built = ctx.build(sc)
    got = ctx.occluded(built, segs, 1e-4)
    built.release()
    ctx.close()
    assert (got == ref).mean() >= 0.9995, int((got != ref).sum())
    assert ref.sum() > 1000 and (ref == 0).sum() > 1000
