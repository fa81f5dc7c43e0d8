"""Float64 finite differences of the single-layer sphere frame -- TEST
INFRASTRUCTURE ONLY (the checker of ``ubr_adjoint``).

Binds ``oracle_fd64_render`` (``oracle/src/oracle_fd64.cpp``): the frame
restated in double with a visibility record.  ``Fd64Frame.record()`` traces
the unperturbed frame and stores which sphere every ray hits;
``Fd64Frame.fd()`` then takes central differences of an L2 image loss with
that visibility held fixed, the derivative the adjoint computes.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os

import numpy as np

from umbreon_gb300 import abi
from umbreon_gb300.api import RenderOptions, Scene, make_render_desc

from .oracle import lib

D3 = C.c_double * 3


class Fd64Desc(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("ss", C.c_int32), ("ortho", C.c_int32),
        ("cam_pos", D3), ("cam_dir", D3), ("cam_up", D3),
        ("cam_height", C.c_double), ("cam_fovy", C.c_double),
        ("clip_near", C.c_double), ("clip_far", C.c_double),
        ("ambient_color", D3), ("background", D3),
        ("n_lights", C.c_int32), ("shadows", C.c_int32), ("ao_samples", C.c_int32), ("ao_multiscale", C.c_int32),
        ("light_dir", D3 * 4), ("light_color", D3 * 4), ("light_intensity", C.c_double * 4),
        ("light_highlight", C.c_int32 * 4),
        ("ao_distance", C.c_double), ("ao_intensity", C.c_double), ("ao_falloff_power", C.c_double),
        ("ao_diffuse_factor", C.c_double),
        ("ao_low_discrepancy", C.c_int32), ("ao_enhanced", C.c_int32), ("fog_on", C.c_int32),
        ("transparent_bg", C.c_int32),
        ("fog_start", C.c_double), ("fog_end", C.c_double), ("fog_color", D3),
        ("gamma", C.c_double), ("specular_scale", C.c_double),
        ("mat", C.c_double * 9),
        ("metallic", C.c_int32), ("pad", C.c_int32),
        ("seed_x0", C.c_int32), ("seed_y0", C.c_int32), ("seed_w", C.c_int32), ("pad2", C.c_int32),
    ]


def _bind():
    L = lib()
    if not getattr(L, "_fd64_bound", False):
        L.oracle_fd64_render.restype = C.c_int
        L.oracle_fd64_render.argtypes = [C.POINTER(Fd64Desc), C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                         C.c_int, C.c_void_p, C.c_int]
        L.oracle_fd64_vis_stride.restype = C.c_int32
        L.oracle_fd64_vis_stride.argtypes = [C.c_int32]
        L._fd64_bound = True
    return L


# global parameter name -> (field, index getter)
_MAT = {name: k for k, name in enumerate(abi.MATERIAL_GRAD_FIELDS)}


class Fd64Frame:
    """The frame of (scene, opt) in double; spheres only, one shared material."""

    def __init__(self, scene: Scene, opt: RenderOptions, threads: int | None = None, seed_window=None):
        """seed_window = (x0, y0, W): the frame is the window at (x0, y0) of a
        W-wide frame, whose pixel coordinates seed the sample streams."""
        rd, _ = make_render_desc(scene, opt)
        d = Fd64Desc()
        if seed_window is not None:
            d.seed_x0, d.seed_y0, d.seed_w = seed_window
        d.width, d.height, d.ss = opt.width, opt.height, max(1, opt.supersample)
        d.ortho = int(rd.cam_orthographic)
        for k in range(3):
            d.cam_pos[k], d.cam_dir[k], d.cam_up[k] = rd.cam_position[k], rd.cam_direction[k], rd.cam_up[k]
            d.ambient_color[k], d.background[k] = scene.ambientColor[k], scene.background[k]
            d.fog_color[k] = scene.fog.color[k]
        d.cam_height, d.cam_fovy = rd.cam_height, rd.cam_fovy
        d.clip_near, d.clip_far = scene.clipNear, scene.clipFar
        if len(scene.lights) > 4:
            raise ValueError("at most 4 lights")
        d.n_lights = len(scene.lights)
        for l, li in enumerate(scene.lights):
            for k in range(3):
                d.light_dir[l][k] = li.direction[k]
                d.light_color[l][k] = li.color[k]
            d.light_intensity[l] = li.intensity
            d.light_highlight[l] = int(li.castsHighlight)
        d.shadows = int(opt.shadows)
        d.ao_samples = opt.aoSamples
        d.ao_multiscale = int(opt.aoMultiScale)
        d.ao_distance, d.ao_intensity = opt.aoDistance, opt.aoIntensity
        d.ao_falloff_power, d.ao_diffuse_factor = opt.aoFalloffPower, opt.aoDiffuseFactor
        d.ao_low_discrepancy = int(opt.aoLowDiscrepancy)
        d.ao_enhanced = int(opt.aoEnhanced())
        d.fog_on = int(scene.fog.enabled)
        d.fog_start, d.fog_end = scene.fog.start, scene.fog.end
        d.transparent_bg = int(opt.transparentBackground)
        d.gamma, d.specular_scale = scene.assumedGamma, opt.specularScale
        mats = np.asarray(scene.sphere_material, abi.MATERIAL_DTYPE).reshape(-1)
        m0 = mats[0]
        if not all(mats[i].tobytes() == m0.tobytes() for i in range(len(mats))):
            raise ValueError("the float64 frame takes one material shared by every sphere")
        for k, name in enumerate(abi.MATERIAL_GRAD_FIELDS):
            d.mat[k] = float(m0[name])
        d.metallic = int(m0["metallic"])
        self.d = d
        cr = np.asarray(scene.sphere_center_radius, np.float32).reshape(-1, 4)
        self.sph = np.ascontiguousarray(cr.astype(np.float64))
        self.col = np.ascontiguousarray(np.asarray(scene.sphere_color, np.float32).reshape(-1, 4)[:, :3]
                                        .astype(np.float64))
        self.threads = threads or min(16, os.cpu_count() or 1)
        L = _bind()
        self._L = L
        ss = d.ss
        self.stride = int(L.oracle_fd64_vis_stride(d.ao_samples))
        self.vis = np.zeros((d.height * ss, d.width * ss, self.stride), np.int32)

    def _render(self, record: bool) -> np.ndarray:
        out = np.zeros((self.d.height, self.d.width, 4), np.float64)
        st = self._L.oracle_fd64_render(C.byref(self.d), self.sph.ctypes.data, self.col.ctypes.data,
                                        len(self.sph), self.vis.ctypes.data, int(record), out.ctypes.data,
                                        self.threads)
        if st != 0:
            raise RuntimeError("oracle_fd64_render failed")
        return out

    def record(self) -> np.ndarray:
        """Trace the frame (brute force, double) and keep its visibility."""
        return self._render(True)

    def frozen(self) -> np.ndarray:
        """The image with the recorded visibility held fixed."""
        return self._render(False)

    def primary_ids(self) -> np.ndarray:
        """Recorded primary sphere per hi-res sample (-1 = background)."""
        v = self.vis[..., 0]
        return np.where(v < 0, -1, v >> 1)

    # -- parameter access -------------------------------------------------
    @contextlib.contextmanager
    def shifted(self, name: str, index=(), delta: float = 0.0):
        """Temporarily add delta to one parameter."""
        idx = index if isinstance(index, tuple) else (index,)
        d = self.d
        if name in _MAT:
            arr, j = d.mat, (_MAT[name],)
        elif name in ("light_direction", "light_color"):
            arr = d.light_dir if name == "light_direction" else d.light_color
            arr, j = arr[idx[0]], (idx[1],)
        elif name == "light_intensity":
            arr, j = d.light_intensity, (idx[0],)
        elif name in ("ambient_color", "background", "fog_color"):
            arr, j = getattr(d, name), (idx[0],)
        elif name in ("fog_start", "fog_end", "ao_distance", "ao_intensity", "specular_scale"):
            old = getattr(d, name)
            setattr(d, name, old + delta)
            try:
                yield
            finally:
                setattr(d, name, old)
            return
        elif name == "sphere_color":
            arr, j = self.col, (idx[0], idx[1])
        elif name == "sphere_center":
            arr, j = self.sph, (idx[0], idx[1])
        elif name == "sphere_radius":
            arr, j = self.sph, (idx[0], 3)
        else:
            raise KeyError(name)
        if isinstance(arr, np.ndarray):
            old = arr[j]
            arr[j] = old + delta
            try:
                yield
            finally:
                arr[j] = old
        else:
            old = arr[j[0]]
            arr[j[0]] = old + delta
            try:
                yield
            finally:
                arr[j[0]] = old

    def loss(self, img: np.ndarray, target: np.ndarray, weight: np.ndarray) -> float:
        diff = img[..., :3] - target[..., :3]
        return float(np.sum(weight[..., None] * diff * diff))

    def fd(self, name: str, index, target: np.ndarray, weight: np.ndarray, h: float = 1e-4) -> float:
        """Central difference of loss() at visibility held fixed."""
        with self.shifted(name, index, +h):
            lp = self.loss(self.frozen(), target, weight)
        with self.shifted(name, index, -h):
            lm = self.loss(self.frozen(), target, weight)
        return (lp - lm) / (2.0 * h)


def interior_mask(ids: np.ndarray) -> np.ndarray:
    """Samples whose 3x3 neighbourhood (inside the image) shows one id."""
    H, W = ids.shape
    ok = np.ones((H, W), bool)
    pad = np.pad(ids, 1, mode="edge")
    valid = np.pad(np.ones((H, W), bool), 1, constant_values=False)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            nb = pad[1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
            nv = valid[1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
            ok &= ~nv | (nb == ids)
    return ok
