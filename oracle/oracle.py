"""Python binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the C++ restatement in ``oracle/src``) and
renders a ``umbreon_gb300.api.Scene`` on the host cores.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use this
module, and only as the checker or the timed CPU reference -- never as the
product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from umbreon_gb300 import abi
from umbreon_gb300.api import FrameResult, RenderOptions, Scene, attach_aovs, make_render_desc

HERE = Path(__file__).resolve().parent
_L = None


def lib():
    global _L
    if _L is None:
        p = HERE / "liboracle.so"
        if not p.exists():
            from umbreon_gb300 import build
            build.build_oracle()
        L = C.CDLL(str(p))
        L.oracle_scene_create.restype = C.c_void_p
        L.oracle_scene_create.argtypes = [C.POINTER(abi.SceneDesc)]
        L.oracle_scene_destroy.argtypes = [C.c_void_p]
        L.oracle_scene_bvh_nodes.restype = C.c_uint64
        L.oracle_scene_bvh_nodes.argtypes = [C.c_void_p]
        L.oracle_scene_geom_id.restype = C.c_uint32
        L.oracle_scene_geom_id.argtypes = [C.c_void_p, C.c_int]
        L.oracle_render.restype = C.c_int
        L.oracle_render.argtypes = [C.c_void_p, C.POINTER(abi.RenderDesc), C.POINTER(abi.Frame), C.c_int]
        L.oracle_render_rows.restype = C.c_int
        L.oracle_render_rows.argtypes = [C.c_void_p, C.POINTER(abi.RenderDesc), C.POINTER(abi.Frame), C.c_int,
                                         C.c_int, C.c_int]
        L.oracle_intersect.restype = C.c_int
        L.oracle_intersect.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64] + [C.c_void_p] * 6
        L.oracle_occluded.restype = C.c_int
        L.oracle_occluded.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        L.oracle_occluded_filtered.restype = C.c_int
        L.oracle_occluded_filtered.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_float, C.c_float,
                                               C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_coarse_ao_lookup.restype = C.c_int
        L.oracle_coarse_ao_lookup.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 8 + [
            C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_void_p, C.c_float, C.c_void_p]
        L.oracle_aa_mask.restype = C.c_int
        L.oracle_aa_mask.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 5 + [C.c_float, C.c_float, C.c_int,
                                                                              C.c_void_p]
        _L = L
    return _L


def coarse_ao_lookup(openness, normal, depth, hit, lattice, px, py, N, z, bent=None, contact=None, shape=None,
                     avg=None):
    """One coarse-grid AO lookup on a hand-built (h, w) grid; returns None when
    the guides reject, else (openness, bent (3,), contact, shape, avgHitDist)."""
    op = np.ascontiguousarray(openness, np.float32)
    h, w = op.shape
    arrs = [op, np.ascontiguousarray(normal, np.float32), np.ascontiguousarray(depth, np.float32),
            np.ascontiguousarray(hit, np.uint8)]
    q = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (bent, contact, shape, avg)]
    n = np.ascontiguousarray(N, np.float32)
    out = np.zeros(7, np.float32)
    ok = lib().oracle_coarse_ao_lookup(w, h, *[a.ctypes.data for a in arrs],
                                       *[None if a is None else a.ctypes.data for a in q],
                                       lattice[0], lattice[1], px, py, n.ctypes.data, z, out.ctypes.data)
    if not ok:
        return None
    return float(out[0]), out[1:4].copy(), float(out[4]), float(out[5]), float(out[6])


def aa_mask(rgba, view_z, geom, group, normal, threshold=0.1, pixel_world_size=0.1, perspective=False):
    """Adaptive-AA refinement mask (Hf, Wf) of hand-built centre records:
    rgba (Hf, Wf, 4), view_z (Hf, Wf), geom / group (Hf, Wf), normal (Hf, Wf, 3)."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    Hf, Wf = rgba.shape[:2]
    vz = np.ascontiguousarray(view_z, np.float32)
    g = np.ascontiguousarray(geom, np.uint32)
    gr = np.ascontiguousarray(group, np.int32)
    nr = np.ascontiguousarray(normal, np.float32)
    out = np.zeros((Hf, Wf), np.uint8)
    st = lib().oracle_aa_mask(Wf, Hf, rgba.ctypes.data, vz.ctypes.data, g.ctypes.data, gr.ctypes.data,
                              nr.ctypes.data, threshold, pixel_world_size, int(perspective), out.ctypes.data)
    if st != 0:
        raise ValueError("aa_mask: empty grid")
    return out


class OracleScene:
    def __init__(self, scene: Scene):
        d, self._keep = scene.to_desc()
        self.h = lib().oracle_scene_create(C.byref(d))
        if not self.h:
            raise RuntimeError("oracle_scene_create failed")

    def geom_id(self, kind: int) -> int:
        return int(lib().oracle_scene_geom_id(self.h, kind))

    def intersect(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        t = np.zeros(n, np.float32)
        g = np.zeros(n, np.uint32)
        p = np.zeros(n, np.uint32)
        u = np.zeros(n, np.float32)
        v = np.zeros(n, np.float32)
        ng = np.zeros((n, 3), np.float32)
        lib().oracle_intersect(self.h, rays.ctypes.data, n, t.ctypes.data, g.ctypes.data, p.ctypes.data,
                               u.ctypes.data, v.ctypes.data, ng.ctypes.data)
        return t, g, p, u, v, ng

    def occluded(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        out = np.zeros(len(rays), np.uint8)
        lib().oracle_occluded(self.h, rays.ctypes.data, len(rays), out.ctypes.data)
        return out

    def occluded_filtered(self, segs: np.ndarray, eps: float, graze_cos_eps: float = 0.0, coplanar_eps: float = 0.0,
                          exclude_faces=None) -> np.ndarray:
        segs = np.ascontiguousarray(segs, np.float32).reshape(-1, 6)
        n = len(segs)
        out = np.zeros(n, np.uint8)
        offs = faces = None
        if exclude_faces is not None:
            offs = np.zeros(n + 1, np.uint32)
            np.cumsum([len(f) for f in exclude_faces], out=offs[1:])
            faces = np.ascontiguousarray(np.concatenate([np.asarray(f, np.int32) for f in exclude_faces] +
                                                        [np.zeros(1, np.int32)]), np.int32)
        lib().oracle_occluded_filtered(self.h, segs.ctypes.data, n, eps, graze_cos_eps, coplanar_eps,
                                       offs.ctypes.data if offs is not None else None,
                                       faces.ctypes.data if faces is not None else None, out.ctypes.data)
        return out

    def render(self, scene: Scene, opt: RenderOptions, threads: int = 0, rows: tuple | None = None) -> FrameResult:
        rd, keep = make_render_desc(scene, opt)
        ss = max(1, opt.supersample)
        W, H = opt.width * ss, opt.height * ss
        color = np.zeros((opt.height, opt.width, 4), np.float32)
        depth = np.zeros((H, W), np.float32)
        vz = np.zeros((H, W), np.float32)
        hg = np.zeros((H, W), np.uint32)
        hp = np.zeros((H, W), np.uint32)
        fr = abi.Frame()
        fr.color = abi.ptr(color)
        fr.depth = abi.ptr(depth)
        fr.view_z = abi.ptr(vz)
        fr.hit_geom = abi.ptr(hg, C.c_uint32)
        fr.hit_prim = abi.ptr(hp, C.c_uint32)
        aovs = attach_aovs(fr, opt)
        r0, r1 = rows if rows else (0, 0)
        st = lib().oracle_render_rows(self.h, C.byref(rd), C.byref(fr), threads, r0, r1)
        if st != 0:
            raise RuntimeError("oracle: unsupported request (adaptive AA with the edge G-buffer)")
        stats = dict(render_ms=fr.render_ms, rays_primary=fr.rays_primary, rays_occlusion=fr.rays_occlusion,
                     capped_rays=fr.capped_rays)
        return FrameResult(opt.width, opt.height, color, depth, vz, hg, hp, fr.render_ms / 1e3, stats, **aovs)

    def __del__(self):
        try:
            if self.h:
                lib().oracle_scene_destroy(self.h)
                self.h = None
        except Exception:
            pass


def render(scene: Scene, opt: RenderOptions, threads: int = 0) -> FrameResult:
    return OracleScene(scene).render(scene, opt, threads)
