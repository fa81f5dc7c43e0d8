"""Known-answer cases of the reference's own tests, restated as data.

Each case builds a small scene the way the reference test does and lists the
analytic values the reference asserts, with the reference's tolerances:
  tests/test_render_shading.cpp:20-241, tests/test_render_transparency.cpp:230-301,
  tests/test_render_shadows_gi.cpp:30-157, tests/test_render_ao.cpp:20-170.
A case is (name, builder) where builder() returns a list of renders to make
[(scene, opt), ...] and a check(frames) -> list of (label, ok) pairs.
"""
import numpy as np
import sys, os
sys.path.insert(0, os.path.dirname(__file__))

from umbreon_gb300 import abi, scenes
from umbreon_gb300.api import Camera, DistantLight, RenderOptions, Scene

C = (2, 2)  # centre pixel of a 5x5 image


def approx(a, b, eps):
    return abs(float(a) - float(b)) <= eps


def o5(**kw):
    return RenderOptions(width=5, height=5, **kw)


def centre(f):
    return f.color[C[0], C[1]]


def case_mesh_lambert():
    sc = scenes.quad_scene()
    def check(fs):
        c = centre(fs[0])
        return [("mesh R=0.30", approx(c[0], 0.30, 1e-4)), ("mesh G=0.36", approx(c[1], 0.36, 1e-4)),
                ("mesh B=0.42", approx(c[2], 0.42, 1e-4)), ("mesh alpha=1", approx(c[3], 1.0, 1e-6)),
                ("mesh depth=10", approx(fs[0].depth[2, 2], 10.0, 1e-3))]
    return [(sc, o5())], check


def case_background():
    sc = scenes.quad_scene()
    sc.mesh_positions = None
    def check(fs):
        c = centre(fs[0])
        return [("bg R", approx(c[0], 0.4, 1e-6)), ("bg G", approx(c[1], 0.1, 1e-6)),
                ("bg B", approx(c[2], 0.2, 1e-6)), ("bg depth 0", approx(fs[0].depth[2, 2], 0.0, 1e-6))]
    return [(sc, o5())], check


def case_outline_sphere():
    sc = scenes.material_sphere_scene((0.3, 0.4, 0.5, 1.0), abi.flat_outline(), (0.4, 0.1, 0.2))
    def check(fs):
        c = centre(fs[0])
        return [("outline R", approx(c[0], 0.3, 1e-4)), ("outline G", approx(c[1], 0.4, 1e-4)),
                ("outline B", approx(c[2], 0.5, 1e-4))]
    return [(sc, o5())], check


def case_gamma():
    sc = scenes.quad_scene(bg=(0, 0, 0))
    sc.assumedGamma = 2.0
    def check(fs):
        c = centre(fs[0])
        return [("gamma R", approx(c[0], 0.09, 1e-4)), ("gamma G", approx(c[1], 0.36 * 0.36, 1e-4)),
                ("gamma alpha", approx(c[3], 1.0, 1e-6))]
    return [(sc, o5())], check


def case_supersample():
    sc = scenes.quad_scene(bg=(0, 0, 0))
    def check(fs):
        f = fs[0]
        return [("ss width", f.color.shape[1] == 5), ("ss height", f.color.shape[0] == 5),
                ("ss value", approx(centre(f)[0], 0.30, 1e-4))]
    return [(sc, o5(supersample=2))], check


def _mat_sphere(color, bg, **m):
    return scenes.material_sphere_scene(color, abi.material(**m), bg)


def case_matte():
    sc = _mat_sphere((0.6, 0.4, 0.2, 1.0), (0, 0, 0), ambient=0.0, diffuse=0.8, brilliance=0.0)
    def check(fs):
        c = centre(fs[0])
        return [("matte R", approx(c[0], 0.24, 1e-4)), ("matte G", approx(c[1], 0.16, 1e-4)),
                ("matte B", approx(c[2], 0.08, 1e-4))]
    return [(sc, o5())], check


def case_metallic():
    kw = dict(ambient=0.35, diffuse=0.3, brilliance=2.0, specular=0.8, roughness=1.0 / 20.0, metallic=True,
              reflection=0.10)
    a = _mat_sphere((0.6, 0.4, 0.2, 1.0), (0, 0, 0), **kw)
    b = _mat_sphere((0.6, 0.4, 0.2, 1.0), (1, 1, 1), **kw)
    def check(fs):
        c, d = centre(fs[0]), centre(fs[1])
        return [("metallic R", approx(c[0], 0.54, 1e-3)), ("metallic G", approx(c[1], 0.36, 1e-3)),
                ("metallic B", approx(c[2], 0.18, 1e-3)), ("reflection R", approx(d[0], 0.64, 1e-3)),
                ("reflection G", approx(d[1], 0.46, 1e-3))]
    return [(a, o5()), (b, o5())], check


def case_phong():
    sc = _mat_sphere((0.2, 0.4, 0.6, 1.0), (0, 0, 0), ambient=0.3, diffuse=0.5, brilliance=0.0, phong=10000.0,
                     phong_size=50.0)
    def check(fs):
        c = centre(fs[0])
        lr, lg, lb = c[0] - 0.11, c[1] - 0.22, c[2] - 0.33
        return [("phong lift 5000", approx(lr, 5000.0, 1.0)), ("phong achromatic RG", approx(lr, lg, 1e-4)),
                ("phong achromatic GB", approx(lg, lb, 1e-4))]
    return [(sc, o5())], check


def case_fill_light():
    kw = dict(ambient=0.0, diffuse=0.0, brilliance=1.0, specular=0.5, roughness=0.05)
    a = _mat_sphere((0.6, 0.4, 0.2, 1.0), (0, 0, 0), **kw)
    b = _mat_sphere((0.6, 0.4, 0.2, 1.0), (0, 0, 0), **kw)
    b.lights[0].castsHighlight = False
    def check(fs):
        return [("highlight R=0.25", approx(centre(fs[0])[0], 0.25, 1e-3)),
                ("fill R=0", approx(centre(fs[1])[0], 0.0, 1e-4)),
                ("fill G=0", approx(centre(fs[1])[1], 0.0, 1e-4))]
    return [(a, o5()), (b, o5())], check


def case_metallic_fresnel():
    sc = scenes.quad_scene(color=(1.0, 0.0, 0.0, 1.0), bg=(0, 0, 0))
    sc.mesh_material = abi.material(ambient=0.0, diffuse=0.0, specular=1.0, roughness=0.5, metallic=True)
    sc.lights = [DistantLight(direction=(-0.8660254, 0.0, -0.5), intensity=1.0)]
    def check(fs):
        c = centre(fs[0])
        return [("fresnel R", approx(c[0], 0.75, 2e-3)), ("fresnel G", approx(c[1], 0.04445, 2e-3)),
                ("fresnel G==B", approx(c[1], c[2], 1e-5))]
    return [(sc, o5())], check


# --- transparency (test_render_transparency.cpp F1-F4) ---

def _quads(spec, bg):
    """spec = [(rgba, z, group)] -> flat-material scene of stacked quads."""
    pos, col, grp = [], [], []
    for rgba, z, g in spec:
        for p in [(-2, -2, z), (2, -2, z), (2, 2, z), (-2, -2, z), (2, 2, z), (-2, 2, z)]:
            pos.append(p)
            col.append(rgba)
        grp += [g, g]
    pos = np.array(pos, np.float32)
    sc = Scene(mesh_positions=pos, mesh_normals=np.tile([0, 0, 1], (len(pos), 1)).astype(np.float32),
               mesh_colors=np.array(col, np.float32), mesh_material=abi.flat_outline(),
               mesh_tri_group=np.array(grp, np.uint16))
    sc.camera = scenes.ortho_cam()
    sc.background = bg
    sc.ambientColor = (1, 1, 1)
    return sc


def case_over_f1():
    sc = _quads([((1, 0, 0, 1.0), 0.0, 0), ((0, 0, 1, 0.6), 1.0, 1)], (0, 0, 0))
    def check(fs):
        c = centre(fs[0])
        return [("F1 R=0.4", approx(c[0], 0.4, 1e-4)), ("F1 B=0.6", approx(c[2], 0.6, 1e-4)),
                ("F1 alpha", approx(c[3], 1.0, 1e-6))]
    return [(sc, o5())], check


def case_over_f2():
    a = _quads([((1, 0, 0, 1.0), 0.0, 0), ((0, 0, 1, 0.5), 0.5, 2), ((0, 1, 0, 0.5), 1.0, 1)], (0, 0, 0))
    b = _quads([((1, 0, 0, 1.0), 0.0, 0), ((0, 1, 0, 0.5), 0.5, 1), ((0, 0, 1, 0.5), 1.0, 2)], (0, 0, 0))
    def check(fs):
        c, d = centre(fs[0]), centre(fs[1])
        return [("F2 green-front G", approx(c[1], 0.5, 1e-4)), ("F2 green-front B", approx(c[2], 0.25, 1e-4)),
                ("F2 blue-front B", approx(d[2], 0.5, 1e-4)), ("F2 blue-front G", approx(d[1], 0.25, 1e-4))]
    return [(a, o5()), (b, o5())], check


def case_over_f3():
    sc = _quads([((1, 0, 0, 1.0), 0.0, 0), ((0, 0, 1, 0.5), 0.5, 1), ((0, 0, 1, 0.5), 1.0, 1)], (0, 0, 0))
    def check(fs):
        c = centre(fs[0])
        return [("F3 B=0.75", approx(c[2], 0.75, 1e-4)), ("F3 R=0.25", approx(c[0], 0.25, 1e-4))]
    return [(sc, o5())], check


def case_over_f4():
    sc = _quads([((0, 0, 1, 0.6), 1.0, 1)], (0.2, 0.2, 0.2))
    def check(fs):
        c = centre(fs[0])
        return [("F4 B=0.6", approx(c[2], 0.6, 1e-4)), ("F4 R=0", approx(c[0], 0.0, 1e-4)),
                ("F4 alpha=0.6", approx(c[3], 0.6, 1e-4))]
    return [(sc, o5(transparentBackground=True))], check


# --- shadows (test_render_shadows_gi.cpp:30-157) ---

def _floor_slab(floor_rgba=(1, 1, 1, 1), slab=True, ambient=0.2, diffuse=0.8):
    pos, nrm, col = [], [], []
    for p in [(-2, -2, 0), (2, -2, 0), (2, 2, 0), (-2, -2, 0), (2, 2, 0), (-2, 2, 0)]:
        pos.append(p); nrm.append((0, 0, 1)); col.append(floor_rgba)
    if slab:
        z = 0.4
        for p in [(0.1, -2, z), (4, -2, z), (4, 2, z), (0.1, -2, z), (4, 2, z), (0.1, 2, z)]:
            pos.append(p); nrm.append((0, 0, -1)); col.append((0, 0, 0, 1))
    sc = Scene(mesh_positions=np.array(pos, np.float32), mesh_normals=np.array(nrm, np.float32),
               mesh_colors=np.array(col, np.float32), mesh_material=abi.material(ambient=ambient, diffuse=diffuse))
    sc.camera = scenes.ortho_cam()
    sc.ambientColor = (1, 1, 1)
    sc.background = (0, 0, 0)
    return sc


def case_hard_shadow():
    sc = _floor_slab()
    sc.lights = [DistantLight(direction=(-0.6, 0.0, -0.8), intensity=1.0)]
    def check(fs):
        off, on = centre(fs[0])[0], centre(fs[1])[0]
        return [("shadow off ~0.84", approx(off, 0.84, 0.03)), ("shadow on ~0.2", approx(on, 0.2, 0.03)),
                ("on darker", on + 0.2 < off)]
    return [(sc, o5(shadows=False)), (sc, o5(shadows=True))], check


def case_soft_shadow():
    pos, nrm, col = scenes.quad_mesh((1, 1, 1, 1))
    sc = Scene(mesh_positions=pos, mesh_normals=nrm, mesh_colors=col,
               mesh_material=abi.material(ambient=0.2, diffuse=0.8),
               sphere_center_radius=np.array([[0.9, 0.0, 1.2, 0.45]], np.float32),
               sphere_color=np.array([[0, 0, 0, 1]], np.float32),
               sphere_material=np.array([abi.flat_outline()], abi.MATERIAL_DTYPE))
    sc.camera = scenes.ortho_cam()
    sc.background = (0, 0, 0)
    sc.lights = [DistantLight(direction=(-0.6, 0.0, -0.8), intensity=1.0)]
    soft = o5(shadows=True, lightRadius=22.0, shadowSamples=64)
    def check(fs):
        lit, hard, s1, s2 = (centre(f)[0] for f in fs)
        return [("hard ~0.2", approx(hard, 0.2, 0.03)), ("lit ~0.84", approx(lit, 0.84, 0.03)),
                ("penumbra between", hard + 0.05 < s1 and s1 + 0.05 < lit),
                ("soft deterministic", np.array_equal(fs[2].color, fs[3].color))]
    return [(sc, o5(shadows=False)), (sc, o5(shadows=True)), (sc, soft), (sc, soft)], check


def case_acne_guard():
    q = 100.0
    pos = np.array([(-q, -q, 0), (q, -q, 0), (q, q, 0), (-q, -q, 0), (q, q, 0), (-q, q, 0)], np.float32)
    sc = Scene(mesh_positions=pos, mesh_normals=np.tile([0, 0, 1], (6, 1)).astype(np.float32),
               mesh_colors=np.ones((6, 4), np.float32), mesh_material=abi.material(ambient=0.2, diffuse=0.8))
    sc.camera = Camera(position=(0.0, 1200.0, 1600.0), direction=(0.0, -0.6, -0.8), up=(0.0, 1.0, 0.0),
                       orthographic=True, height=6.0)
    sc.lights = [scenes.key_light()]
    sc.background = (0, 0, 0)
    def check(fs):
        return [("acne guard min > 0.5", float(fs[0].color[..., 0].min()) > 0.5)]
    return [(sc, o5(shadows=True))], check


# --- ambient occlusion (test_render_ao.cpp:20-170) ---

def case_ao_open():
    sc = scenes.quad_scene(bg=(0, 0, 0))
    def check(fs):
        c = centre(fs[0])
        return [("AO open R~0.30", approx(c[0], 0.30, 0.02)), ("AO open G~0.36", approx(c[1], 0.36, 0.02))]
    return [(sc, o5(aoSamples=64, aoDistance=100.0))], check


def case_ao_occlusion():
    a = _floor_slab(slab=False, ambient=1.0, diffuse=0.0)
    b = _floor_slab(slab=True, ambient=1.0, diffuse=0.0)
    o = o5(aoSamples=128, aoDistance=10.0)
    def check(fs):
        op, oc = centre(fs[0])[0], centre(fs[1])[0]
        return [("AO open floor ~1", approx(op, 1.0, 0.03)), ("AO slab darkens", oc + 0.05 < op),
                ("AO not black", oc > 0.05)]
    return [(a, o), (b, o)], check


def case_ao_outline_gate():
    def sph(probe_from_edge):
        flat = abi.material(ambient=1.0, diffuse=0.0)
        sc = Scene(sphere_center_radius=np.array([[0, 0, 0, 1.0], [0, 2.2, 0, 2.0]], np.float32),
                   sphere_color=np.array([[1, 1, 1, 1], [0, 0, 0, 1]], np.float32),
                   sphere_material=np.array([flat, flat], abi.MATERIAL_DTYPE),
                   sphere_from_edge=np.array([1 if probe_from_edge else 0, 1], np.uint8))
        sc.camera = scenes.ortho_cam()
        sc.background = (0, 0, 0)
        return sc
    off = o5(aoSamples=0)
    on = o5(aoSamples=128, aoDistance=10.0)
    def check(fs):
        diff = float(np.abs(fs[1].color - fs[0].color).sum())
        return [("AO darkens real sphere", diff > 0.05),
                ("AO outline gate identical", np.array_equal(fs[2].color, fs[3].color))]
    return [(sph(False), off), (sph(False), on), (sph(True), off), (sph(True), on)], check


def case_ao_determinism():
    sc = scenes.quad_scene(bg=(0, 0, 0))
    o = o5(aoSamples=32, aoDistance=100.0)
    def check(fs):
        return [("AO bit-identical", np.array_equal(fs[0].color, fs[1].color))]
    return [(sc, o), (sc, o)], check


# --- adaptive antialiasing (test_adaptive_aa.cpp:89-125 fixtures, :333-606) ---

def _scene_x(x0, x1):
    """Quad over [x0, x1] x [-2, 2] at z = 0 facing +Z, colour (0.5, 0.6,
    0.7), material 0.2 / 0.8, the ortho rig, one 0.5 key light, background 0.1."""
    pos = np.array([(x0, -2, 0), (x1, -2, 0), (x1, 2, 0), (x0, -2, 0), (x1, 2, 0), (x0, 2, 0)], np.float32)
    sc = Scene(mesh_positions=pos, mesh_normals=np.tile([0, 0, 1], (6, 1)).astype(np.float32),
               mesh_colors=np.tile(np.array([0.5, 0.6, 0.7, 1.0], np.float32), (6, 1)),
               mesh_material=abi.material(ambient=0.2, diffuse=0.8))
    sc.camera = scenes.ortho_cam()
    sc.lights = [scenes.key_light()]
    sc.background = (0.1, 0.1, 0.1)
    return sc


def _close(a, b, eps):
    return a.color.shape == b.color.shape and float(np.abs(a.color - b.color).max()) <= eps


def _equal(a, b):
    return np.array_equal(a.color, b.color) and np.array_equal(a.depth, b.depth)


def case_aa_uniform():
    sc = _scene_x(-2.0, 2.0)
    grid = RenderOptions(width=6, height=6, supersample=2)
    adap = RenderOptions(width=6, height=6, supersample=2, aaMode=1)
    def check(fs):
        return [("uniform: adaptive == grid within 1e-6", _close(fs[0], fs[1], 1e-6)),
                ("uniform: final size 6x6", fs[1].color.shape[:2] == (6, 6))]
    return [(sc, grid), (sc, adap)], check


def case_aa_silhouette():
    sc = _scene_x(-2.0, 0.0)
    grid = RenderOptions(width=9, height=9, supersample=3)
    adap = RenderOptions(width=9, height=9, supersample=3, aaMode=1, aaDebug=True)
    def check(fs):
        a, b = fs
        m = b.aaMask > 0
        return [("silhouette: adaptive == grid within 1e-6", _close(a, b, 1e-6)),
                ("silhouette: flagged pixels bitwise grid", m.any() and np.array_equal(a.color[m], b.color[m])),
                ("mask sized 9x9", b.aaMask.shape == (9, 9)),
                ("silhouette column 4 flagged", bool(np.all(b.aaMask[:, 4] > 0))),
                ("far columns quiet", bool(np.all(b.aaMask[:, 0] == 0) and np.all(b.aaMask[:, 8] == 0)))]
    return [(sc, grid), (sc, adap)], check


def case_aa_determinism():
    sc = _scene_x(-2.0, 0.0)
    adap = RenderOptions(width=9, height=9, supersample=3, aaMode=1, aoSamples=8, aoDistance=100.0,
                         shadows=True, shadowSamples=4, lightRadius=2.0)
    def check(fs):
        return [("adaptive + AO + soft shadows deterministic (bitwise)", _equal(fs[0], fs[1]))]
    return [(sc, adap), (sc, adap)], check


def case_aa_ao_compensation():
    sc = _scene_x(-2.0, 2.0)
    z = 0.4
    slab = np.array([(0.2, -2, z), (4, -2, z), (4, 2, z), (0.2, -2, z), (4, 2, z), (0.2, 2, z)], np.float32)
    sc.mesh_positions = np.concatenate([sc.mesh_positions, slab])
    sc.mesh_normals = np.concatenate([sc.mesh_normals, np.tile([0, 0, -1], (6, 1)).astype(np.float32)])
    sc.mesh_colors = np.concatenate([sc.mesh_colors, np.tile([0, 0, 0, 1], (6, 1)).astype(np.float32)])
    sc.mesh_material = abi.material(ambient=1.0, diffuse=0.0)
    sc.lights = []
    grid = RenderOptions(width=8, height=8, supersample=2, aoSamples=16, aoDistance=100.0)
    adap = RenderOptions(width=8, height=8, supersample=2, aoSamples=16, aoDistance=100.0, aaMode=1)
    def check(fs):
        a, b = fs[0].color[4, 6, 0], fs[1].color[4, 6, 0]
        return [("AO compensation: unflagged pixel within 0.05 of the grid", abs(float(a) - float(b)) < 0.05)]
    return [(sc, grid), (sc, adap)], check


def case_aa_depth_equal_ss():
    sc = _scene_x(-2.0, 0.0)
    o1 = RenderOptions(width=9, height=9, supersample=3, aaMode=1)
    o2 = RenderOptions(width=9, height=9, supersample=3, aaMode=1, aaDepth=3)
    def check(fs):
        return [("aa-depth == ss: bitwise aa-depth 0", _equal(fs[0], fs[1]))]
    return [(sc, o1), (sc, o2)], check


def case_aa_depth_ss1():
    sc = _scene_x(-2.0, 0.0)
    grid = RenderOptions(width=9, height=9)
    adap = RenderOptions(width=9, height=9, aaMode=1, aaDepth=2, aaDebug=True)
    def check(fs):
        a, b = fs
        m = b.aaMask > 0
        same = (a.color == b.color).all(-1)
        return [("aa-depth ss=1: mask 9x9", b.aaMask.shape == (9, 9)),
                ("aa-depth ss=1: unflagged bitwise 1-sample grid", bool(np.all(same[~m]))),
                ("aa-depth ss=1: some flagged pixels refined", bool(np.any(~same[m])))]
    return [(sc, grid), (sc, adap)], check


# --- coarse-grid AO (test_ao_coarse.cpp:40-76 rig, :210-384) ---

def ao_coarse_scene(slab=True):
    """Ambient-only white floor with a black slab over the +x half, the ortho
    rig, no lights, background 0.1."""
    pos = [(-2, -2, 0), (2, -2, 0), (2, 2, 0), (-2, -2, 0), (2, 2, 0), (-2, 2, 0)]
    nrm = [(0, 0, 1)] * 6
    col = [(1, 1, 1, 1)] * 6
    if slab:
        z = 0.4
        pos += [(0.2, -2, z), (4, -2, z), (4, 2, z), (0.2, -2, z), (4, 2, z), (0.2, 2, z)]
        nrm += [(0, 0, -1)] * 6
        col += [(0, 0, 0, 1)] * 6
    sc = Scene(mesh_positions=np.array(pos, np.float32), mesh_normals=np.array(nrm, np.float32),
               mesh_colors=np.array(col, np.float32), mesh_material=abi.material(ambient=1.0, diffuse=0.0))
    sc.camera = scenes.ortho_cam()
    sc.lights = []
    sc.background = (0.1, 0.1, 0.1)
    return sc


def _with(opt, **kw):
    o = RenderOptions(**{k: getattr(opt, k) for k in opt.__dataclass_fields__})
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def case_ao_coarse_inline_neutrality():
    sc = ao_coarse_scene()
    o0 = RenderOptions(width=8, height=8, supersample=2, aoSamples=16, aoDistance=100.0)
    e0 = _with(o0, aoMultiScale=True, aoMultibounce=True)
    def check(fs):
        return [("legacy: div 0 == div 1 bitwise", np.array_equal(fs[0].color, fs[1].color)),
                ("enhanced: div 0 == div 1 bitwise", np.array_equal(fs[2].color, fs[3].color))]
    return [(sc, o0), (sc, _with(o0, aoResDiv=1)), (sc, e0), (sc, _with(e0, aoResDiv=1))], check


def case_ao_coarse_close_to_inline():
    sc = ao_coarse_scene()
    full = RenderOptions(width=16, height=16, supersample=3, aoSamples=256, aoDistance=100.0, aoLowDiscrepancy=True)
    f32 = _with(full, aoSamples=32, aoLowDiscrepancy=False)
    def check(fs):
        return [("coarse vs inline within 0.05 (256 spp + LD)", _close(fs[0], fs[1], 0.05)),
                ("coarse vs inline mean |diff| < 0.02 (32 spp)",
                 float(np.mean(np.abs(fs[2].color - fs[3].color))) < 0.02)]
    return [(sc, full), (sc, _with(full, aoResDiv=-1)), (sc, f32), (sc, _with(f32, aoResDiv=-1))], check


def case_ao_coarse_fallback_exact():
    sc = ao_coarse_scene()
    full = RenderOptions(width=24, height=24, aoSamples=16, aoDistance=100.0)
    def check(fs):
        a, b = fs
        ok = b.aoPatchMask is not None and b.aoPatchMask.shape == (24, 24)
        m = b.aoPatchMask > 0 if ok else None
        return [("patch mask at render resolution", ok),
                ("patch mask fires somewhere, not everywhere", ok and 0 < int(m.sum()) < 24 * 24),
                ("patched pixels bitwise the inline render", ok and np.array_equal(a.color[m], b.color[m]))]
    return [(sc, full), (sc, _with(full, aoResDiv=2, aoResDebug=True))], check


def case_ao_coarse_determinism():
    sc = ao_coarse_scene()
    o = RenderOptions(width=12, height=12, supersample=2, aoSamples=16, aoDistance=100.0, aoResDiv=-1)
    def check(fs):
        return [("coarse AO deterministic (bitwise)", np.array_equal(fs[0].color, fs[1].color))]
    return [(sc, o), (sc, o)], check


def case_ao_coarse_adaptive():
    sc = ao_coarse_scene()
    g = RenderOptions(width=12, height=12, supersample=3, aoSamples=16, aoDistance=100.0, aoResDiv=-1)
    a = _with(g, aaMode=1)
    def check(fs):
        return [("adaptive + coarse deterministic", np.array_equal(fs[1].color, fs[2].color)),
                ("adaptive + coarse within 0.05 of grid + coarse", _close(fs[0], fs[1], 0.05))]
    return [(sc, g), (sc, a), (sc, a)], check


def case_ao_coarse_transparency():
    sc = ao_coarse_scene()
    z = 1.0
    shell = np.array([(-2, -2, z), (2, -2, z), (2, 2, z), (-2, -2, z), (2, 2, z), (-2, 2, z)], np.float32)
    sc.mesh_positions = np.concatenate([sc.mesh_positions, shell])
    sc.mesh_normals = np.concatenate([sc.mesh_normals, np.tile([0, 0, 1], (6, 1)).astype(np.float32)])
    sc.mesh_colors = np.concatenate([sc.mesh_colors, np.tile([0.5, 0.7, 0.9, 0.4], (6, 1)).astype(np.float32)])
    full = RenderOptions(width=12, height=12, supersample=2, aoSamples=16, aoDistance=100.0)
    def check(fs):
        return [("transparent shell: coarse within 0.05 of inline", _close(fs[0], fs[1], 0.05))]
    return [(sc, full), (sc, _with(full, aoResDiv=-1))], check


# --- principled materials, direct pass (test_principled.cpp:33-161 rig) ---

def _pov_diffuse():
    return abi.material(ambient=0.2, diffuse=0.8, specular=0.0, phong=0.0, brilliance=1.0, reflection=0.0)


def _pbr(metallic, roughness, specular, anisotropy=0.0, rotation=0.0):
    m = _pov_diffuse()
    m["model"] = 1
    m["pbr_metallic"], m["pbr_roughness"], m["pbr_specular"] = metallic, roughness, specular
    m["pbr_anisotropy"], m["pbr_anisotropy_rotation"] = anisotropy, rotation
    return m


def _unit(v):
    v = np.asarray(v, np.float64)
    return tuple(float(x) for x in v / np.linalg.norm(v))


def pbr_scene(floor_mat, sphere_mat, fill=False, bond_mat=None):
    """Floor quad (y = 0, 8 x 8) + unit sphere at (0, 1, 0), perspective
    camera, one distant light; optional capped bond along x (addBond)."""
    c = [(-4, 0, -4), (4, 0, -4), (4, 0, 4), (-4, 0, -4), (4, 0, 4), (-4, 0, 4)]
    sc = Scene(mesh_positions=np.array(c, np.float32),
               mesh_normals=np.tile([0, 1, 0], (6, 1)).astype(np.float32),
               mesh_colors=np.tile([0.7, 0.7, 0.7, 1.0], (6, 1)).astype(np.float32), mesh_material=floor_mat,
               sphere_center_radius=np.array([[0, 1, 0, 1]], np.float32),
               sphere_color=np.array([[0.8, 0.3, 0.3, 1.0]], np.float32),
               sphere_material=np.array([sphere_mat], abi.MATERIAL_DTYPE))
    if bond_mat is not None:
        sc.cyl_p0 = np.array([[-2.0, 1.4, 1.0]], np.float32)
        sc.cyl_p1 = np.array([[2.0, 1.4, 1.0]], np.float32)
        sc.cyl_radius = np.array([0.5], np.float32)
        sc.cyl_color = np.array([[0.85, 0.7, 0.3, 1.0]], np.float32)
        sc.cyl_material = np.array([bond_mat], abi.MATERIAL_DTYPE)
        sc.cyl_open = np.zeros(1, np.uint8)
    sc.camera = Camera(position=(0.0, 3.0, 8.0), direction=_unit((0, -0.35, -1)), up=(0.0, 1.0, 0.0),
                       orthographic=False, fovy=40.0)
    sc.lights = [DistantLight(direction=_unit((-0.4, -1.0, -0.3)), color=(1.0, 1.0, 1.0), intensity=0.8,
                              castsHighlight=not fill)]
    sc.background = (0.9, 0.9, 0.95)
    sc.ambientColor = (0.5, 0.5, 0.5)
    return sc


def _opts(**kw):
    return RenderOptions(width=48, height=36, **kw)


def _lum(f):
    c = f.color.astype(np.float64)
    return float(np.mean(0.2126 * c[..., 0] + 0.7152 * c[..., 1] + 0.0722 * c[..., 2]))


def case_pbr_diffuse_parity():
    pov = pbr_scene(_pov_diffuse(), _pov_diffuse())
    pbr = pbr_scene(_pbr(0.0, 0.5, 0.0), _pbr(0.0, 0.5, 0.0))
    def check(fs):
        return [("diffuse parity, shadows off (bitwise)", np.array_equal(fs[0].color, fs[1].color)),
                ("diffuse parity, hard shadows (bitwise)", np.array_equal(fs[2].color, fs[3].color))]
    return [(pov, _opts()), (pbr, _opts()), (pov, _opts(shadows=True)), (pbr, _opts(shadows=True))], check


def case_pbr_determinism_and_area_light():
    m = _pbr(0.6, 0.25, 0.5)
    sc = pbr_scene(m, m)
    hard = _opts(shadows=True)
    area = _opts(shadows=True, shadowSamples=4, lightRadius=8.6)
    def check(fs):
        return [("principled render run-to-run bit-exact", np.array_equal(fs[0].color, fs[1].color)),
                ("area-light path run-to-run bit-exact", np.array_equal(fs[2].color, fs[3].color)),
                ("area light changes the principled render", not np.array_equal(fs[0].color, fs[2].color))]
    return [(sc, hard), (sc, hard), (sc, area), (sc, area)], check


def case_pbr_fill_light_roughness_inert():
    r1, r2 = _pbr(0.8, 0.1, 0.5), _pbr(0.8, 0.7, 0.5)
    def check(fs):
        return [("fill light: roughness does not enter (bitwise)", np.array_equal(fs[0].color, fs[1].color))]
    return [(pbr_scene(r1, r1, fill=True), _opts()), (pbr_scene(r2, r2, fill=True), _opts())], check


def case_pbr_roughness_and_metal():
    r1, r2, metal = _pbr(1.0, 0.15, 0.5), _pbr(1.0, 0.6, 0.5), _pbr(1.0, 0.3, 0.5)
    def check(fs):
        return [("roughness changes the principled render", not np.array_equal(fs[0].color, fs[1].color)),
                ("metal visible in basic mode", _lum(fs[2]) > 0.05),
                ("metal visible in AO mode", _lum(fs[3]) > 0.05),
                ("AO-mode principled render bit-exact", np.array_equal(fs[3].color, fs[4].color))]
    ao = _opts(aoSamples=8)
    return [(pbr_scene(r1, r1), _opts()), (pbr_scene(r2, r2), _opts()), (pbr_scene(metal, metal), _opts()),
            (pbr_scene(metal, metal), ao), (pbr_scene(metal, metal), ao)], check


def case_pbr_anisotropy():
    iso = _pbr(1.0, 0.35, 0.5)
    mesh_aniso = _pbr(1.0, 0.35, 0.5, anisotropy=0.8)
    diffuse = _pbr(0.0, 0.5, 0.0)
    an, rot = _pbr(1.0, 0.35, 0.5, 0.8, 0.0), _pbr(1.0, 0.35, 0.5, 0.8, 0.25)
    def check(fs):
        return [("mesh anisotropy is bitwise inert", np.array_equal(fs[0].color, fs[1].color)),
                ("anisotropy changes the direct highlight (primitives)", not np.array_equal(fs[2].color, fs[3].color)),
                ("anisotropic render finite", bool(np.all(np.isfinite(fs[2].color)))),
                ("anisotropyRotation reorients the lobe", not np.array_equal(fs[2].color, fs[4].color)),
                ("anisotropic render run-to-run bit-exact", np.array_equal(fs[4].color, fs[5].color))]
    return [(pbr_scene(mesh_aniso, diffuse), _opts()), (pbr_scene(iso, diffuse), _opts()),
            (pbr_scene(_pov_diffuse(), an, bond_mat=an), _opts()),
            (pbr_scene(_pov_diffuse(), iso, bond_mat=iso), _opts()),
            (pbr_scene(_pov_diffuse(), rot, bond_mat=rot), _opts()),
            (pbr_scene(_pov_diffuse(), rot, bond_mat=rot), _opts())], check


# --- fog (test_fog.cpp:30-97), restated through a render: the quad at view
# z 10 of the ortho rig, mesh Lambert colour (0.30, 0.36, 0.42) ---

def _fogged(start, end, color=(1.0, 1.0, 1.0), bg=(0.4, 0.1, 0.2)):
    from umbreon_gb300.api import Fog
    sc = scenes.quad_scene(bg=bg)
    sc.fog = Fog(enabled=True, color=color, start=start, end=end)
    return sc


def case_fog_linear():
    def check(fs):
        mid, before, after, bgf = centre(fs[0]), centre(fs[1]), centre(fs[2]), fs[0].color[0, 0]
        return [("f = 0.5: R = mix(1, 0.30, 0.5)", approx(mid[0], 0.65, 1e-4)),
                ("f = 0.5: B = mix(1, 0.42, 0.5)", approx(mid[2], 0.71, 1e-4)),
                ("opaque: alpha untouched", approx(mid[3], 1.0, 1e-6)),
                ("before start: unfogged", approx(before[0], 0.30, 1e-4)),
                ("after end: full fog colour", approx(after[0], 1.0, 1e-6)),
                ("background (view z 0) skipped", approx(bgf[0], 0.4, 1e-6) and approx(bgf[2], 0.2, 1e-6))]
    sc = _fogged(5.0, 15.0)
    sc.mesh_positions = sc.mesh_positions * np.array([0.5, 0.5, 1.0], np.float32)  # leave background corners
    return [(sc, o5()), (_fogged(12.0, 20.0), o5()), (_fogged(2.0, 8.0), o5())], check


def case_fog_degenerate_slab():
    def check(fs):
        return [("degenerate slab: near side unfogged", approx(centre(fs[0])[0], 0.30, 1e-4)),
                ("degenerate slab: far side full fog", approx(centre(fs[1])[0], 1.0, 1e-6))]
    return [(_fogged(12.0, 12.0), o5()), (_fogged(8.0, 8.0), o5())], check


def case_fog_transparent_background():
    fog = (0.7, 0.8, 0.9)
    def check(fs):
        op, tr = centre(fs[0]), centre(fs[1])
        f = 0.625  # (15 - 10) / (15 - 7)
        over = [tr[k] * tr[3] + fog[k] * (1.0 - tr[3]) for k in range(3)]
        return [("transparent: RGB unchanged", approx(tr[0], 0.30, 1e-4)),
                ("transparent: alpha faded by f", approx(tr[3], f, 1e-5)),
                ("transparent over fog colour == opaque",
                 all(approx(over[k], op[k], 1e-5) for k in range(3)))]
    return [(_fogged(7.0, 15.0, fog), o5()), (_fogged(7.0, 15.0, fog), o5(transparentBackground=True))], check


# --- clip planes (test_clip_planes.cpp:14-70): unit sphere at the origin,
# ortho camera at z 10, blue background ---

def _clip_scene(near=None, far=None):
    sc = scenes.material_sphere_scene((1.0, 0.0, 0.0, 1.0), abi.material(ambient=0.2, diffuse=0.8), (0.0, 0.0, 1.0))
    if near is not None:
        sc.clipNear = near
    if far is not None:
        sc.clipFar = far
    return sc


def case_clip_planes():
    def check(fs):
        c0, cf, cn, cc = (centre(f) for f in fs)
        return [("no clip: centre hits the sphere", c0[0] > 0.3 and c0[2] < 0.5),
                ("clipFar 8: background", approx(cf[2], 1.0, 1e-4) and cf[0] < 1e-4),
                ("clipNear 12: background", cn[0] < 1e-4),
                ("clipNear 10: interior back wall at view z 11", 10.5 < float(fs[3].viewZ[2, 2]) < 11.5)]
    return [(_clip_scene(), o5()), (_clip_scene(far=8.0), o5()), (_clip_scene(near=12.0), o5()),
            (_clip_scene(near=10.0), o5())], check


def case_clip_cut_gbuffer():
    """test_clip_planes.cpp:52-96 with the edge G-buffer on."""
    def check(fs):
        near10, far8, near12 = fs
        return [("clipNear 10: interior back wall flagged clip-cut", int(near10.clipCut[2, 2]) == 1),
                ("clipNear 10: corner miss ray unflagged", int(near10.clipCut[0, 0]) == 0),
                ("clipNear 10: corner records no removed hit",
                 near10.clipNearVz[0, 0] == 0.0 and near10.clipFarVz[0, 0] == 0.0),
                ("clipFar 8: removed hit (view z 9) beyond the plane", approx(far8.clipFarVz[2, 2], 9.0, 1e-2)),
                ("clipFar 8: nothing recorded in front of a near plane", far8.clipNearVz[2, 2] == 0.0),
                ("clipNear 12: removed hit in front of the plane", approx(near12.clipNearVz[2, 2], 9.0, 1e-2))]
    g = o5(edgeGBuffer=True)
    return [(_clip_scene(near=10.0), g), (_clip_scene(far=8.0), g), (_clip_scene(near=12.0), g)], check


# --- indexed mesh (test_mesh_indexed.cpp:23-93) ---

def case_mesh_indexed_equals_deindexed():
    pos = np.array([(-2, -2, 0), (2, -2, 0), (2, 2, 0), (-2, 2, 0)], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    col = np.tile(np.array([0.5, 0.6, 0.7, 1.0], np.float32), (4, 1))
    nrm = np.tile(np.array([0, 0, 1], np.float32), (4, 1))
    def mk(p, n, c, i):
        sc = Scene(mesh_positions=p, mesh_normals=n, mesh_colors=c, mesh_index=i,
                   mesh_material=abi.material(ambient=0.2, diffuse=0.8))
        sc.camera = scenes.ortho_cam()
        sc.background = (0.1, 0.2, 0.3)
        sc.lights = [DistantLight(direction=(0.0, 0.0, -1.0), intensity=0.5)]
        return sc
    flat = idx.reshape(-1)
    de = mk(pos[flat], nrm[flat], col[flat], None)
    opt = RenderOptions(width=24, height=24, supersample=2)
    def check(fs):
        return [("indexed vs de-indexed render bit-identical", np.array_equal(fs[0].color, fs[1].color))]
    return [(mk(pos, nrm, col, idx), opt), (de, opt)], check


CASES = {k[5:]: v for k, v in globals().items() if k.startswith("case_")}


def run_case(builder, render_fn):
    renders, check = builder()
    frames = [render_fn(sc, opt) for sc, opt in renders]
    return check(frames)
