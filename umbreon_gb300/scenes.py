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


# --- molecular surface: iso-surface of a sum of Gaussians -------------------

# Freudenthal split of a cube into 6 tetrahedra around the (0,0,0)-(1,1,1)
# diagonal; neighbouring cubes split shared faces along the same diagonal, so
# the extracted surface is crack-free.  Corner c has offset (c&1, c>>1&1, c>>2&1).
_TETS = np.array([[0, 7, 1, 3], [0, 7, 3, 2], [0, 7, 2, 6], [0, 7, 6, 4], [0, 7, 4, 5], [0, 7, 5, 1]])
_TET_EDGES = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]])


def gaussian_density(atoms: np.ndarray, sigma: float, h: float, lo: np.ndarray, shape, cutoff: float = 3.0):
    """sum_i exp(-|x - a_i|^2 / sigma^2) on a grid (origin lo, spacing h),
    each atom splatted within cutoff*sigma."""
    nx, ny, nz = shape
    field = np.zeros(nx * ny * nz, np.float64)
    r = int(math.ceil(cutoff * sigma / h))
    base = np.floor((atoms - lo) / h).astype(np.int64)
    offs = np.stack(np.meshgrid(*(np.arange(-r, r + 2),) * 3, indexing="ij"), -1).reshape(-1, 3)
    inv2 = 1.0 / (sigma * sigma)
    for chunk in np.array_split(offs, max(1, len(offs) // 256)):
        g = base[None, :, :] + chunk[:, None, :]                  # (c, n, 3)
        ok = np.all((g >= 0) & (g < np.array(shape)), axis=-1)
        p = lo + g * h
        d2 = np.sum((p - atoms[None]) ** 2, axis=-1)
        w = np.exp(-d2 * inv2) * ok * (d2 <= (cutoff * sigma) ** 2)
        flat = (g[..., 0] * ny + g[..., 1]) * nz + g[..., 2]
        field += np.bincount(np.where(ok, flat, 0).ravel(), weights=w.ravel(), minlength=field.size)
    return field.reshape(shape)


def marching_tetrahedra(field: np.ndarray, iso: float, lo: np.ndarray, h: float):
    """Indexed iso-surface of `field` at `iso`: (positions, normals, index).
    Triangles wind counter-clockwise seen from the low-field side, and vertex
    normals point down the gradient (outward for a density)."""
    nx, ny, nz = field.shape
    f = field.ravel()
    gx, gy, gz = np.gradient(field, h)
    grad = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], 1)
    ci, cj, ck = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")
    cube0 = ((ci * ny + cj) * nz + ck).ravel()
    corner = np.array([((c & 1) * ny + ((c >> 1) & 1)) * nz + ((c >> 2) & 1) for c in range(8)])
    inside_c = f[cube0[:, None] + corner[None, :]] > iso
    keep = inside_c.any(1) & ~inside_c.all(1)
    cube0 = cube0[keep]
    tris = []
    for t in _TETS:
        vid = cube0[:, None] + corner[t][None, :]                 # (m, 4) grid ids
        ins = f[vid] > iso
        case = ins[:, 0] * 1 + ins[:, 1] * 2 + ins[:, 2] * 4 + ins[:, 3] * 8
        for cs in range(1, 15):
            sel = case == cs
            if not sel.any():
                continue
            v = vid[sel]
            inside = [(cs >> q) & 1 for q in range(4)]
            n_in = sum(inside)
            # edges crossing the surface, in a cyclic order around the tet
            if n_in == 1 or n_in == 3:
                a = inside.index(1) if n_in == 1 else inside.index(0)
                others = [q for q in range(4) if q != a]
                polys = [[(a, others[0]), (a, others[1]), (a, others[2])]]
            else:
                ia = [q for q in range(4) if inside[q]]
                oa = [q for q in range(4) if not inside[q]]
                polys = [[(ia[0], oa[0]), (ia[0], oa[1]), (ia[1], oa[1]), (ia[1], oa[0])]]
            for poly in polys:
                ge = np.stack([np.stack([np.minimum(v[:, p], v[:, q]), np.maximum(v[:, p], v[:, q])], 1)
                               for (p, q) in poly], 1)           # (m, k, 2) sorted edge keys
                tris.append(ge[:, [0, 1, 2]])
                if len(poly) == 4:
                    tris.append(ge[:, [0, 2, 3]])
    E = np.concatenate(tris, 0)                                   # (T, 3, 2)
    keys = E[..., 0].astype(np.int64) * f.size + E[..., 1]
    uk, inv = np.unique(keys.ravel(), return_inverse=True)
    a_id, b_id = uk // f.size, uk % f.size
    fa, fb = f[a_id], f[b_id]
    w = np.clip((iso - fa) / np.where(fb != fa, fb - fa, 1.0), 0.0, 1.0)[:, None]

    def gpos(g):
        k = g % nz
        j = (g // nz) % ny
        i = g // (ny * nz)
        return lo + np.stack([i, j, k], 1) * h

    pos = gpos(a_id) * (1 - w) + gpos(b_id) * w
    gv = grad[a_id] * (1 - w) + grad[b_id] * w
    nrm = -gv / np.maximum(np.linalg.norm(gv, axis=1, keepdims=True), 1e-12)
    idx = inv.reshape(-1, 3)
    # orient: geometric normal along the outward (down-gradient) normal
    p0, p1, p2 = pos[idx[:, 0]], pos[idx[:, 1]], pos[idx[:, 2]]
    ng = np.cross(p1 - p0, p2 - p0)
    flip = np.sum(ng * (nrm[idx[:, 0]] + nrm[idx[:, 1]] + nrm[idx[:, 2]]), 1) < 0
    idx[flip] = idx[flip][:, [0, 2, 1]]
    area2 = np.linalg.norm(ng, axis=1)
    idx = idx[area2 > 1e-12]
    return pos.astype(np.float32), nrm.astype(np.float32), idx.astype(np.uint32)


def molecular_surface(seed: int = BASE_SEED + 2, n_atoms: int = 10000, box: float = 60.0, grid: float = 0.5,
                      sigma: float = 1.5, iso: float = 1.35, n_spheres: int = 5000, width: int = 2048,
                      height: int = 2048, ao_samples: int = 32, layers: int = 4):
    """Workload 2: iso-surface (0.5 A grid) of a sum of Gaussians over 10,000
    random atoms in a 60 A box, vertex alpha 0.5, plus 5,000 opaque sphere
    atoms; up to 4 transparent layers, 32 AO rays, 2 shadowed lights, 2048^2."""
    u = uniform(seed, n_atoms, 6)
    atoms = u[:, :3] * box
    margin = 3.0 * sigma
    lo = np.full(3, -margin)
    shape = tuple([int(math.ceil((box + 2 * margin) / grid)) + 1] * 3)
    field = gaussian_density(atoms, sigma, grid, lo, shape)
    pos, nrm, idx = marching_tetrahedra(field, iso, lo, grid)
    col = np.empty((len(pos), 4), np.float32)
    col[:, 0] = 0.35 + 0.5 * (pos[:, 0] / box).clip(0, 1)
    col[:, 1] = 0.55
    col[:, 2] = 0.85 - 0.5 * (pos[:, 2] / box).clip(0, 1)
    col[:, 3] = 0.5
    sc = Scene(mesh_positions=pos, mesh_normals=nrm, mesh_colors=col, mesh_index=idx, mesh_material=pov_material())
    ns = min(n_spheres, n_atoms)
    cr = np.empty((ns, 4), np.float32)
    cr[:, :3] = atoms[:ns]
    cr[:, 3] = 0.6
    sc.sphere_center_radius = cr
    scol = np.ones((ns, 4), np.float32)
    scol[:, :3] = (0.3 + 0.7 * u[:ns, 3:6]).astype(np.float32)
    sc.sphere_color = scol
    sc.sphere_material = np.full(ns, pov_material(), abi.MATERIAL_DTYPE)
    blo, bhi = pos.min(0), pos.max(0)
    _frame_ortho(sc, blo, bhi, width, height, margin=1.02)
    sc.lights = [DistantLight(direction=(-0.4, -0.5, -1.0), intensity=0.8),
                 DistantLight(direction=(0.6, 0.3, -1.0), intensity=0.4)]
    sc.background = (1.0, 1.0, 1.0)
    opt = RenderOptions(width=width, height=height, supersample=1, aoSamples=ao_samples, aoDistance=4.0,
                        shadows=True, maxTransparentLayers=layers)
    return sc, opt


# --- batched turntable workload ---------------------------------------------

def turntable_batch(seed: int = BASE_SEED + 3, n_items: int = 64, n_scenes: int = 8, ao_samples: int = 8,
                    resolutions=(256, 512, 1024, 2048), max_spheres: int = 200000, min_spheres: int = 5000):
    """Workload 3: n_items (scene, turntable angle, resolution) frames.  Scenes
    hold log-uniform 5k..200k spheres with workload 0's radius distribution in
    a cube sized to keep workload 0's density (40 A for 2,000 spheres); each
    item picks one of 36 turntable angles (10 degree steps, perspective
    fovy 40) and a square resolution from `resolutions`; 8 AO rays, two
    shadowed lights.  Returns (scenes, items) with items = [(scene index,
    Scene, RenderOptions)] sharing the geometry of their scene."""
    us = uniform(seed, n_scenes, 1)[:, 0]
    counts = np.exp(np.log(min_spheres) + us * (np.log(max_spheres) - np.log(min_spheres))).astype(int)
    bases = []
    for i, n in enumerate(counts):
        box = 40.0 * (n / 2000.0) ** (1.0 / 3.0)
        cr, col, mats = random_spheres(int(n), box, seed * 131 + i)
        bases.append((Scene(sphere_center_radius=cr, sphere_color=col, sphere_material=mats), box))
    ui = uniform(seed + 7, n_items, 3)
    items = []
    for k in range(n_items):
        si = min(int(ui[k, 0] * n_scenes), n_scenes - 1)
        angle = 10.0 * min(int(ui[k, 1] * 36), 35)
        res = resolutions[min(int(ui[k, 2] * len(resolutions)), len(resolutions) - 1)]
        base, box = bases[si]
        c = np.full(3, 0.5 * box)
        radius = 0.5 * np.sqrt(3.0) * box
        dist = radius / math.sin(math.radians(20.0)) * 1.05
        a = math.radians(angle)
        pos = c + dist * np.array([math.sin(a), 0.0, math.cos(a)])
        sc = Scene(sphere_center_radius=base.sphere_center_radius, sphere_color=base.sphere_color,
                   sphere_material=base.sphere_material)
        sc.camera = Camera(position=tuple(float(x) for x in pos), direction=tuple(float(x) for x in (c - pos)),
                           up=(0.0, 1.0, 0.0), fovy=40.0, orthographic=False)
        sc.lights = [DistantLight(direction=(-0.4, -0.6, -0.7), intensity=0.8),
                     DistantLight(direction=(0.6, -0.2, -0.8), intensity=0.4)]
        sc.background = (0.0, 0.0, 0.0)
        opt = RenderOptions(width=res, height=res, supersample=1, aoSamples=ao_samples,
                            aoDistance=0.1 * box, shadows=True)
        items.append((si, sc, opt))
    return [b for b, _ in bases], items


def differentiable(seed: int = BASE_SEED + 4, n: int = 100000, res: int = 1024, ao_samples: int = 16,
                   box: float | None = None):
    """Workload 4: n spheres with workload 0's radius and colour distribution
    in a cube of 120 A at 100,000 spheres (the side scales with n^(1/3) to
    keep the density), POV finish with Blinn specular 0.3 (roughness 0.02)
    and Phong 0.3 (size 40), res x res orthographic view along -z, one
    shadowed light, enhanced AO (16 rays, linear falloff: power 1) at
    distance 4 A, linear fog across the cube's depth."""
    if box is None:
        box = 120.0 * (n / 100000.0) ** (1.0 / 3.0)
    mat = abi.material(ambient=0.2, diffuse=0.7, specular=0.3, roughness=0.02, brilliance=1.0,
                       phong=0.3, phong_size=40.0)
    cr, col, mats = random_spheres(n, box, seed, mat)
    sc = Scene(sphere_center_radius=cr, sphere_color=col, sphere_material=mats)
    c = 0.5 * box
    dist = 1.5 * box + 10.0
    sc.camera = Camera(position=(c, c, c + dist), direction=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0),
                       orthographic=True, height=1.02 * box)
    sc.lights = [DistantLight(direction=(-0.35, -0.45, -0.8), intensity=0.9)]
    sc.ambientColor = (1.0, 1.0, 1.0)
    sc.background = (0.05, 0.05, 0.1)
    # view-z of the cube's front face is dist - box / 2
    sc.fog = Fog(enabled=True, color=(0.6, 0.65, 0.7), start=dist - 0.5 * box + 0.1 * box,
                 end=dist - 0.5 * box + 1.4 * box)
    opt = RenderOptions(width=res, height=res, supersample=1, aoSamples=ao_samples, aoDistance=4.0,
                        aoFalloffPower=1.0, shadows=True)
    return sc, opt


def differentiable_target(sc: Scene, opt: RenderOptions, seed: int = BASE_SEED + 40):
    """The target of workload 4's loss: the same scene with perturbed diffuse,
    specular and phong size, light direction turned by up to 10 degrees and
    intensity scaled by up to +/-20%, fog range, AO distance, per-sphere
    colours (+/-0.05) and centres (+/-0.1 A)."""
    import copy
    u = uniform(seed, 8, 1)[:, 0]
    t = copy.deepcopy(sc)
    o = copy.deepcopy(opt)
    m = np.array(t.sphere_material, abi.MATERIAL_DTYPE, copy=True)
    m["diffuse"] *= 1.0 + 0.2 * (u[0] - 0.5)
    m["specular"] *= 1.0 + 0.2 * (u[1] - 0.5)
    m["phong_size"] *= 1.0 + 0.2 * (u[2] - 0.5)
    t.sphere_material = m
    L = t.lights[0]
    d = np.asarray(L.direction, np.float64)
    d = d / np.linalg.norm(d)
    axis = np.cross(d, [0.0, 1.0, 0.0])
    axis /= np.linalg.norm(axis)
    ang = math.radians(10.0 * (2.0 * u[3] - 1.0))
    d2 = d * math.cos(ang) + np.cross(axis, d) * math.sin(ang) + axis * np.dot(axis, d) * (1 - math.cos(ang))
    t.lights = [DistantLight(direction=tuple(float(x) for x in d2), intensity=L.intensity * (1.0 + 0.4 * (u[4] - 0.5)),
                             color=L.color, castsHighlight=L.castsHighlight)]
    span = t.fog.end - t.fog.start
    t.fog = Fog(enabled=True, color=t.fog.color, start=t.fog.start + 0.1 * span * (u[5] - 0.5),
                end=t.fog.end + 0.1 * span * (u[5] - 0.5))
    o.aoDistance = opt.aoDistance * (1.0 + 0.3 * (u[6] - 0.5))
    n = sc.sphere_count()
    up = uniform(seed + 1, n, 6)
    col = np.array(t.sphere_color, np.float32, copy=True)
    col[:, :3] = np.clip(col[:, :3] + 0.1 * (up[:, :3] - 0.5), 0.0, 1.0)
    cr = np.array(t.sphere_center_radius, np.float32, copy=True)
    cr[:, :3] += (0.2 * (up[:, 3:6] - 0.5)).astype(np.float32)
    t.sphere_color = col
    t.sphere_center_radius = cr
    return t, o
