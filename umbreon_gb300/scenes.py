"""Seeded synthetic scenes for the five benchmark workloads.

The reference's real scenes are LFS pointers that are not present, so every
workload is generated here from a named PRNG: PCG32 (O'Neill 2014, the
"pcg32_random_r" output function with pcg32_srandom_r seeding), one stream per
element index so generation is vectorised and order independent.  Seeds are
20261203 + workload index.

  ball_and_stick(...) and friends return (Scene, RenderOptions).
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .api import Camera, DistantLight, Fog, RenderOptions, Scene

BASE_SEED = 20261203
_MULT = np.uint64(6364136223846793005)
RADII = np.array([1.2, 1.5, 1.7, 1.8, 2.0], np.float32)
RADIUS_P = np.array([0.5, 0.2, 0.15, 0.1, 0.05])


def pcg32(seed: int, n: int, k: int) -> np.ndarray:
    """(n, k) uint32: k successive outputs of PCG32 stream i (initseq = i)."""
    with np.errstate(over="ignore"):
        inc = (np.arange(n, dtype=np.uint64) << np.uint64(1)) | np.uint64(1)
        state = np.zeros(n, np.uint64)
        state = state * _MULT + inc
        state = state + np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        state = state * _MULT + inc
        out = np.empty((n, k), np.uint32)
        for j in range(k):
            old = state
            state = old * _MULT + inc
            xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)) & np.uint64(0xFFFFFFFF)
            rot = (old >> np.uint64(59)).astype(np.uint64)
            r = ((xs >> rot) | (xs << ((np.uint64(32) - rot) & np.uint64(31)))) & np.uint64(0xFFFFFFFF)
            out[:, j] = r.astype(np.uint32)
    return out


def uniform(seed: int, n: int, k: int) -> np.ndarray:
    """(n, k) float64 in [0, 1) from pcg32."""
    return pcg32(seed, n, k).astype(np.float64) * (1.0 / 4294967296.0)


def pov_material():
    """The workloads' POV finish: ambient 0.2, diffuse 0.7, specular 0.3
    (Blinn, roughness 0.02 => exponent 50), phong 0, phong_size 40."""
    return abi.material(ambient=0.2, diffuse=0.7, specular=0.3, roughness=0.02, brilliance=1.0,
                        phong=0.0, phong_size=40.0)


def sample_radii(u: np.ndarray) -> np.ndarray:
    cdf = np.cumsum(RADIUS_P)
    idx = np.searchsorted(cdf, u, side="right")
    return RADII[np.minimum(idx, len(RADII) - 1)]


def random_spheres(n: int, box: float, seed: int, material=None):
    """Centres U[0,box)^3, radii from {1.2..2.0} with p {.5,.2,.15,.1,.05},
    rgb U[0.2,1], alpha 1."""
    u = uniform(seed, n, 7)
    cr = np.empty((n, 4), np.float32)
    cr[:, :3] = (u[:, :3] * box).astype(np.float32)
    cr[:, 3] = sample_radii(u[:, 3])
    col = np.ones((n, 4), np.float32)
    col[:, :3] = (0.2 + 0.8 * u[:, 4:7]).astype(np.float32)
    mat = np.full(n, pov_material() if material is None else material, abi.MATERIAL_DTYPE)
    return cr, col, mat


def space_filling(seed: int = BASE_SEED + 0, n: int = 2000, width: int = 640, height: int = 480,
                  phong_variant: bool = False):
    """Workload 0: 2,000 spheres in a 40 A cube, one light + ambient, POV finish,
    640x480, 1 spp, no AO / shadows / fog."""
    mat = pov_material()
    if phong_variant:
        mat = abi.material(ambient=0.2, diffuse=0.7, specular=0.0, phong=0.3, phong_size=40.0)
    cr, col, mats = random_spheres(n, 40.0, seed, mat)
    sc = Scene(sphere_center_radius=cr, sphere_color=col, sphere_material=mats)
    sc.camera = Camera(position=(20.0, 20.0, 120.0), direction=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0),
                       orthographic=True, height=48.0)
    sc.lights = [DistantLight(direction=(0.0, -0.3, -1.0), intensity=1.0)]
    sc.ambientColor = (1.0, 1.0, 1.0)
    sc.background = (0.0, 0.0, 0.0)
    opt = RenderOptions(width=width, height=height, supersample=1)
    return sc, opt


ELEMENT_RGB = np.array([[0.55, 0.55, 0.55], [0.2, 0.3, 1.0], [1.0, 0.15, 0.1], [1.0, 0.85, 0.2]], np.float32)
ELEMENT_P = np.array([0.5, 0.2, 0.2, 0.1])


def _frame_ortho(sc: Scene, lo: np.ndarray, hi: np.ndarray, width: int, height: int, margin: float = 1.08):
    c = 0.5 * (lo + hi)
    R = 0.5 * float(np.linalg.norm(hi - lo))
    dist = R + 10.0
    sc.camera = Camera(position=(float(c[0]), float(c[1]), float(c[2] + dist)), direction=(0.0, 0.0, -1.0),
                       up=(0.0, 1.0, 0.0), orthographic=True,
                       height=float(margin * max(hi[1] - lo[1], (hi[0] - lo[0]) * height / width)))
    return c, R, dist


def ball_and_stick(seed: int = BASE_SEED + 1, n: int = 20000, width: int = 1920, height: int = 1080,
                   supersample: int = 2, ao_samples: int = 16):
    """Workload 1: 20,000 spheres (r 0.4) on a random walk with 1.5 A steps and
    the 19,999 capped cylinders (r 0.2) joining consecutive atoms; 2 lights
    with hard shadows, 16 AO rays at distance 6, 1920x1080 ss2, linear fog
    from the bounding sphere's near point + {0.6, 1.0} x diameter."""
    u = uniform(seed, n, 3)
    z = 2.0 * u[:, 0] - 1.0
    phi = 2.0 * math.pi * u[:, 1]
    rxy = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    steps = np.stack([rxy * np.cos(phi), rxy * np.sin(phi), z], 1) * 1.5
    steps[0] = 0.0
    pos = np.cumsum(steps, 0).astype(np.float32)
    elem = np.minimum(np.searchsorted(np.cumsum(ELEMENT_P), u[:, 2], side="right"), 3)
    cr = np.empty((n, 4), np.float32)
    cr[:, :3] = pos
    cr[:, 3] = 0.4
    col = np.ones((n, 4), np.float32)
    col[:, :3] = ELEMENT_RGB[elem]
    mat = pov_material()
    sc = Scene(sphere_center_radius=cr, sphere_color=col,
               sphere_material=np.full(n, mat, abi.MATERIAL_DTYPE))
    sc.cyl_p0 = pos[:-1].copy()
    sc.cyl_p1 = pos[1:].copy()
    sc.cyl_radius = np.full(n - 1, 0.2, np.float32)
    sc.cyl_color = col[:-1].copy()
    sc.cyl_material = np.full(n - 1, mat, abi.MATERIAL_DTYPE)
    sc.cyl_open = np.zeros(n - 1, np.uint8)
    lo = pos.min(0) - 0.4
    hi = pos.max(0) + 0.4
    c, R, dist = _frame_ortho(sc, lo, hi, width, height)
    sc.lights = [DistantLight(direction=(-0.5, -0.6, -1.0), intensity=0.8),
                 DistantLight(direction=(0.7, -0.2, -1.0), intensity=0.4)]
    sc.background = (1.0, 1.0, 1.0)
    near = dist - R
    sc.fog = Fog(enabled=True, color=(1.0, 1.0, 1.0), start=float(near + 0.6 * 2 * R),
                 end=float(near + 1.0 * 2 * R))
    opt = RenderOptions(width=width, height=height, supersample=supersample, aoSamples=ao_samples,
                        aoDistance=6.0, shadows=True)
    return sc, opt


# --- small known-answer scenes (the reference's own test fixtures, restated:
# tests/render_test_util.hpp:14-71) ---

def quad_mesh(color=(0.5, 0.6, 0.7, 1.0)):
    """A 4x4 quad at z=0 facing +Z, two de-indexed triangles, material 0.2/0.8."""
    p00, p10, p11, p01 = (-2, -2, 0), (2, -2, 0), (2, 2, 0), (-2, 2, 0)
    pos = np.array([p00, p10, p11, p00, p11, p01], np.float32)
    nrm = np.tile(np.array([0, 0, 1], np.float32), (6, 1))
    col = np.tile(np.array(color, np.float32), (6, 1))
    return pos, nrm, col


def ortho_cam():
    return Camera(position=(0.0, 0.0, 10.0), direction=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0),
                  orthographic=True, height=4.0)


def key_light():
    return DistantLight(direction=(0.0, 0.0, -1.0), color=(1.0, 1.0, 1.0), intensity=0.5)


def quad_scene(color=(0.5, 0.6, 0.7, 1.0), bg=(0.4, 0.1, 0.2)):
    pos, nrm, col = quad_mesh(color)
    sc = Scene(mesh_positions=pos, mesh_normals=nrm, mesh_colors=col,
               mesh_material=abi.material(ambient=0.2, diffuse=0.8))
    sc.camera = ortho_cam()
    sc.lights = [key_light()]
    sc.background = bg
    return sc


def material_sphere_scene(color, mat, bg):
    sc = Scene(sphere_center_radius=np.array([[0, 0, 0, 1]], np.float32),
               sphere_color=np.array([color], np.float32),
               sphere_material=np.array([mat], abi.MATERIAL_DTYPE))
    sc.camera = ortho_cam()
    sc.lights = [key_light()]
    sc.background = bg
    return sc
