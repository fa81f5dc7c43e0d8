"""Python host mirror of the umbreon public API over the C-ABI.

``Scene`` / ``RenderOptions`` / ``render()`` carry the same names, fields,
defaults and meaning as ``umbreon::Scene`` (scene.hpp:430-479),
``umbreon::RenderOptions`` (render/render_options.hpp:14-328, the fields this
path honours) and ``umbreon::render`` (umbreon.hpp:29).  Geometry is held as
numpy structure-of-arrays instead of vectors of structs; ``render`` returns a
``FrameResult`` with the reference's field names and sizes.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

INF = float("inf")


@dataclass
class Camera:
    position: tuple = (0.0, 0.0, 1.0)
    direction: tuple = (0.0, 0.0, -1.0)
    up: tuple = (0.0, 1.0, 0.0)
    fovy: float = 40.0
    orthographic: bool = False
    height: float = 1.0


@dataclass
class DistantLight:
    direction: tuple = (0.0, -0.3, -1.0)
    color: tuple = (1.0, 1.0, 1.0)
    intensity: float = 1.0
    castsHighlight: bool = True
    angularRadius: float = 0.0


@dataclass
class Fog:
    enabled: bool = False
    color: tuple = (0.0, 0.0, 0.0)
    start: float = 0.0
    end: float = 0.0


def _f32(a, cols=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if cols is not None:
        a = a.reshape(-1, cols)
    return a


@dataclass
class Scene:
    """umbreon::Scene as structure-of-arrays (scene.hpp:430-479)."""
    # mesh
    mesh_positions: np.ndarray = None   # (V,3)
    mesh_normals: np.ndarray = None     # (V,3)
    mesh_colors: np.ndarray = None      # (V,4)
    mesh_index: np.ndarray = None       # (T,3) uint32 or None (de-indexed)
    mesh_material: np.ndarray = field(default_factory=lambda: abi.material())
    mesh_materials: np.ndarray = None   # (M,) MATERIAL_DTYPE
    mesh_tri_material: np.ndarray = None  # (T,) uint8
    mesh_tri_group: np.ndarray = None     # (T,) uint16
    # spheres
    sphere_center_radius: np.ndarray = None  # (N,4)
    sphere_color: np.ndarray = None          # (N,4)
    sphere_material: np.ndarray = None       # (N,) MATERIAL_DTYPE
    sphere_group: np.ndarray = None
    sphere_from_edge: np.ndarray = None
    # cylinders
    cyl_p0: np.ndarray = None
    cyl_p1: np.ndarray = None
    cyl_radius: np.ndarray = None
    cyl_color: np.ndarray = None
    cyl_opacity1: np.ndarray = None
    cyl_material: np.ndarray = None
    cyl_group: np.ndarray = None
    cyl_open: np.ndarray = None
    cyl_from_edge: np.ndarray = None
    instance_offsets: np.ndarray = None
    camera: Camera = field(default_factory=Camera)
    lights: list = field(default_factory=list)
    ambientIntensity: float = 0.25
    ambientColor: tuple = (1.0, 1.0, 1.0)
    background: tuple = (0.0, 0.0, 0.0)
    fog: Fog = field(default_factory=Fog)
    aoDistance: float = 1.0e20
    assumedGamma: float = 1.0
    clipNear: float = -INF
    clipFar: float = INF

    def triangle_count(self) -> int:
        if self.mesh_positions is None:
            return 0
        if self.mesh_index is not None:
            return int(np.asarray(self.mesh_index).size // 3)
        return int(len(self.mesh_positions) // 3)

    def sphere_count(self) -> int:
        return 0 if self.sphere_center_radius is None else int(len(self.sphere_center_radius))

    def cylinder_count(self) -> int:
        return 0 if self.cyl_p0 is None else int(len(self.cyl_p0))

    def to_desc(self):
        """Build a ubr_scene_desc; returns (desc, keepalive)."""
        keep = []

        def P(a, dtype=np.float32, ctype=C.c_float):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ctype))

        def M(a):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=abi.MATERIAL_DTYPE)).reshape(-1)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(abi.Material))

        d = abi.SceneDesc()
        d.abi_version = abi.ABI_VERSION
        if self.mesh_positions is not None:
            pos = _f32(self.mesh_positions, 3)
            d.mesh_vertex_count = len(pos)
            d.mesh_positions = P(pos)
            d.mesh_normals = P(_f32(self.mesh_normals, 3)) if self.mesh_normals is not None else None
            d.mesh_colors = P(_f32(self.mesh_colors, 4)) if self.mesh_colors is not None else None
            d.mesh_triangle_count = self.triangle_count()
            d.mesh_index = P(self.mesh_index, np.uint32, C.c_uint32) if self.mesh_index is not None else None
            mm = np.asarray(self.mesh_material, dtype=abi.MATERIAL_DTYPE).reshape(())
            d.mesh_material = abi.Material.from_buffer_copy(mm.tobytes())
            if self.mesh_materials is not None:
                d.mesh_materials = M(self.mesh_materials)
                d.mesh_material_count = len(np.asarray(self.mesh_materials).reshape(-1))
            d.mesh_tri_material = P(self.mesh_tri_material, np.uint8, C.c_uint8)
            d.mesh_tri_group = P(self.mesh_tri_group, np.uint16, C.c_uint16)
        n = self.sphere_count()
        if n:
            d.sphere_count = n
            d.sphere_center_radius = P(_f32(self.sphere_center_radius, 4))
            d.sphere_color = P(_f32(self.sphere_color, 4))
            mats = self.sphere_material
            if mats is None:
                mats = np.full(n, abi.flat_outline(), abi.MATERIAL_DTYPE)
            d.sphere_material = M(np.broadcast_to(np.asarray(mats, abi.MATERIAL_DTYPE), (n,)))
            d.sphere_group = P(self.sphere_group, np.uint16, C.c_uint16)
            d.sphere_from_edge = P(self.sphere_from_edge, np.uint8, C.c_uint8)
        n = self.cylinder_count()
        if n:
            d.cylinder_count = n
            d.cyl_p0 = P(_f32(self.cyl_p0, 3))
            d.cyl_p1 = P(_f32(self.cyl_p1, 3))
            d.cyl_radius = P(_f32(self.cyl_radius))
            d.cyl_color = P(_f32(self.cyl_color, 4))
            d.cyl_opacity1 = P(_f32(self.cyl_opacity1)) if self.cyl_opacity1 is not None else None
            mats = self.cyl_material
            if mats is None:
                mats = np.full(n, abi.flat_outline(), abi.MATERIAL_DTYPE)
            d.cyl_material = M(np.broadcast_to(np.asarray(mats, abi.MATERIAL_DTYPE), (n,)))
            d.cyl_group = P(self.cyl_group, np.uint16, C.c_uint16)
            d.cyl_open = P(self.cyl_open, np.uint8, C.c_uint8)
            d.cyl_from_edge = P(self.cyl_from_edge, np.uint8, C.c_uint8)
        if self.instance_offsets is not None and len(self.instance_offsets):
            offs = _f32(self.instance_offsets, 3)
            d.instance_count = len(offs)
            d.instance_offsets = P(offs)
        return d, keep


@dataclass
class RenderOptions:
    """The umbreon::RenderOptions fields of the ray-cast + shade path, with
    the reference defaults (render_options.hpp:14-328)."""
    width: int = 1024
    height: int = 768
    supersample: int = 1
    aoSamples: int = 0
    aoDistance: float = 1.0e20
    aoIntensity: float = 1.0
    aoFalloffPower: float = 0.0
    aoMultiScale: bool = False
    aoBentNormal: bool = False
    aoSkyColor: tuple = (1.0, 1.0, 1.0)
    aoGroundColor: tuple = (1.0, 1.0, 1.0)
    aoUseCameraUp: bool = True
    aoUp: tuple = (0.0, 1.0, 0.0)
    aoMultibounce: bool = False
    aoLowDiscrepancy: bool = False
    aoDiffuseFactor: float = 0.0
    shadows: bool = False
    shadowSamples: int = 1
    lightRadius: float = 0.0
    envLights: int = 0
    envIntensity: float = 1.0
    envKeyScale: float = 0.0
    envAngle: float = 90.0
    specularScale: float = 1.0
    transparency: bool = True
    transparentBackground: bool = False
    maxTransparentLayers: int = 256
    giIntegrator: int = 2
    aoWriteAov: bool = False
    aaMode: int = 0
    aaThreshold: float = 0.1
    aaDepth: int = 0
    aaDebug: bool = False
    aoResDiv: int = 0        # coarse-grid AO divisor (-1 = supersample factor; 0 / 1 = per hit)
    aoResDebug: bool = False  # return the coarse-AO fallback mask
    edgeGBuffer: bool = False  # return the stroke-edge pass's first-hit G-buffer (hi-res)
    denoiser: int = 0          # 0 none, 1 a-trous, 2 OIDN (runs the a-trous); needs aoWriteAov guides
    denoiseIters: int = 5
    denoiseSigmaZ: float = 1.0
    denoiseSigmaN: float = 128.0
    denoiseSigmaL: float = 4.0
    denoiseDemodulateAlbedo: bool = True
    # GI (render_options.hpp:85-252): the pt1 / pt2 path-traced gather
    gi: bool = False
    pt1Spp: int = 8
    giBounces: int = 1
    giMaxDistance: float = 0.0
    giIntensity: float = 1.0
    giEnvIntensity: float = 1.0
    pt1Seed: int = 0
    pt1SkyMode: int = 0
    pt1SkyRadiance: tuple = (1.0, 1.0, 1.0)
    pt1Ld: bool = True
    pt1Clamp: float = 0.0
    pt1GatherDiv: int = -1
    pt1HalfRes: bool = True
    pt1Denoise: bool = True
    pt1UpsampleNormalPow: float = 32.0
    pt1UpsampleDepthScale: float = 0.02
    pt1EdgePatch: bool = True
    pt1EdgePatchSppMul: int = 4
    pt1EdgePatchThresh: float = 0.3
    pt2Pattern: int = 1
    pt2Emissive: bool = True
    pt2Rounds: int = 0
    pt2Radius: float = 16.0
    pt2Unbiased: bool = False
    pt2MCap: float = 100.0
    pt2WClamp: float = 0.0
    pt2Adaptive: bool = False
    pt2AdaptiveThresh: float = 0.15
    pt2AdaptiveMul: int = 4
    pt2EmissiveNee: bool = True
    pt2Reflect: bool = True
    pt2Glossy: bool = True
    pt2GlossySpp: int = 8
    pt2GlossyDenoise: bool = True

    def aoEnhanced(self) -> bool:
        return (self.aoFalloffPower > 0.0 or self.aoMultiScale or self.aoBentNormal or self.aoMultibounce
                or self.aoLowDiscrepancy or self.aoDiffuseFactor > 0.0)


def make_render_desc(scene: Scene, opt: RenderOptions):
    """Flatten scene constants + options into a ubr_render_desc."""
    keep = []
    d = abi.RenderDesc()
    d.abi_version = abi.ABI_VERSION
    d.width, d.height, d.supersample = opt.width, opt.height, opt.supersample
    cam = scene.camera
    d.cam_position[:] = cam.position
    d.cam_direction[:] = cam.direction
    d.cam_up[:] = cam.up
    d.cam_fovy = cam.fovy
    d.cam_orthographic = int(cam.orthographic)
    d.cam_height = cam.height
    n = len(scene.lights)
    if n:
        arr = (abi.Light * n)()
        for i, l in enumerate(scene.lights):
            arr[i].direction[:] = l.direction
            arr[i].color[:] = l.color
            arr[i].intensity = l.intensity
            arr[i].casts_highlight = int(l.castsHighlight)
            arr[i].angular_radius = l.angularRadius
        keep.append(arr)
        d.lights = C.cast(arr, C.POINTER(abi.Light))
    d.light_count = n
    d.ambient_color[:] = scene.ambientColor
    d.background[:] = scene.background
    d.fog_enabled = int(scene.fog.enabled)
    d.fog_color[:] = scene.fog.color
    d.fog_start, d.fog_end = scene.fog.start, scene.fog.end
    d.clip_near, d.clip_far = scene.clipNear, scene.clipFar
    d.assumed_gamma = scene.assumedGamma
    d.ao_samples = opt.aoSamples
    d.ao_distance = opt.aoDistance
    d.ao_intensity = opt.aoIntensity
    d.ao_falloff_power = opt.aoFalloffPower
    d.ao_multiscale = int(opt.aoMultiScale)
    d.ao_bent_normal = int(opt.aoBentNormal)
    d.ao_sky_color[:] = opt.aoSkyColor
    d.ao_ground_color[:] = opt.aoGroundColor
    d.ao_use_camera_up = int(opt.aoUseCameraUp)
    d.ao_up[:] = opt.aoUp
    d.ao_multibounce = int(opt.aoMultibounce)
    d.ao_low_discrepancy = int(opt.aoLowDiscrepancy)
    d.ao_diffuse_factor = opt.aoDiffuseFactor
    d.shadows = int(opt.shadows)
    d.shadow_samples = opt.shadowSamples
    d.light_radius_deg = opt.lightRadius
    d.env_lights = opt.envLights
    d.env_intensity = opt.envIntensity
    d.env_key_scale = opt.envKeyScale
    d.env_angle = opt.envAngle
    d.specular_scale = opt.specularScale
    d.transparency = int(opt.transparency)
    d.transparent_background = int(opt.transparentBackground)
    d.max_transparent_layers = opt.maxTransparentLayers
    d.gi_integrator = opt.giIntegrator
    d.ao_write_aov = int(opt.aoWriteAov)
    d.aa_mode, d.aa_threshold, d.aa_depth = opt.aaMode, opt.aaThreshold, opt.aaDepth
    d.ao_res_div = opt.aoResDiv
    d.edge_gbuffer = int(opt.edgeGBuffer)
    d.denoiser, d.denoise_iters = opt.denoiser, opt.denoiseIters
    d.denoise_sigma_z, d.denoise_sigma_n, d.denoise_sigma_l = opt.denoiseSigmaZ, opt.denoiseSigmaN, opt.denoiseSigmaL
    d.denoise_demodulate_albedo = int(opt.denoiseDemodulateAlbedo)
    if opt.gi:
        check_gi(opt)
        # pipeline.cpp:60-78: adaptive AA and coarse-grid AO fall back to the
        # grid and per-hit AO under GI
        if d.aa_mode == 1:
            d.aa_mode = 0
        if (max(1, opt.supersample) if opt.aoResDiv < 0 else opt.aoResDiv) > 1:
            d.ao_res_div = 0
        d.gi = 1
        d.pt1_spp, d.gi_bounces = opt.pt1Spp, opt.giBounces
        d.gi_max_distance, d.gi_intensity, d.gi_env_intensity = opt.giMaxDistance, opt.giIntensity, opt.giEnvIntensity
        d.pt1_seed, d.pt1_sky_mode = opt.pt1Seed & 0xFFFFFFFF, opt.pt1SkyMode
        for k in range(3):
            d.pt1_sky_radiance[k] = opt.pt1SkyRadiance[k]
        d.pt1_ld, d.pt1_clamp = int(opt.pt1Ld), opt.pt1Clamp
        d.pt1_gather_div, d.pt1_half_res, d.pt1_denoise = opt.pt1GatherDiv, int(opt.pt1HalfRes), int(opt.pt1Denoise)
        d.pt1_upsample_normal_pow, d.pt1_upsample_depth_scale = opt.pt1UpsampleNormalPow, opt.pt1UpsampleDepthScale
        d.pt1_edge_patch, d.pt1_edge_patch_spp_mul = int(opt.pt1EdgePatch), opt.pt1EdgePatchSppMul
        d.pt1_edge_patch_thresh = opt.pt1EdgePatchThresh
        d.pt2_pattern, d.pt2_emissive, d.pt2_rounds = opt.pt2Pattern, int(opt.pt2Emissive), opt.pt2Rounds
        d.pt2_radius, d.pt2_unbiased, d.pt2_m_cap = opt.pt2Radius, int(opt.pt2Unbiased), opt.pt2MCap
        d.pt2_w_clamp, d.pt2_adaptive = opt.pt2WClamp, int(opt.pt2Adaptive)
        d.pt2_adaptive_thresh, d.pt2_adaptive_mul = opt.pt2AdaptiveThresh, opt.pt2AdaptiveMul
        d.pt2_emissive_nee, d.pt2_reflect, d.pt2_glossy = int(opt.pt2EmissiveNee), int(opt.pt2Reflect), int(opt.pt2Glossy)
        d.pt2_glossy_spp, d.pt2_glossy_denoise = opt.pt2GlossySpp, int(opt.pt2GlossyDenoise)
    return d, keep


def gi_gather_div(opt) -> int:
    """The pt1 gather grid divisor the reference resolves (pipeline.cpp
    resolves -1 to the supersample factor; embree_renderer.cpp:717-719 maps 0
    to 2 or 1 through pt1HalfRes)."""
    div = opt.pt1GatherDiv
    if div < 0:
        div = max(1, opt.supersample)
    if div == 0:
        div = 2 if opt.pt1HalfRes else 1
    return max(1, div)


def check_gi(opt) -> None:
    """Raise ValueError for the GI settings this library does not build."""
    if opt.giIntegrator not in (1, 2):
        raise ValueError("gi: the irradiance-cache integrator (giIntegrator 0) is not part of this library")


@dataclass
class FrameResult:
    """umbreon::FrameResult subset (frame_result.hpp:43-124) plus hit ids."""
    width: int
    height: int
    color: np.ndarray        # (H, W, 4) final
    depth: np.ndarray        # (Hss, Wss) hi-res
    viewZ: np.ndarray        # (Hss, Wss) hi-res
    hit_geom: np.ndarray     # (Hss, Wss)
    hit_prim: np.ndarray
    renderSeconds: float = 0.0
    stats: dict = field(default_factory=dict)
    # AO AOVs (RenderOptions.aoWriteAov), output resolution
    albedo: np.ndarray = None      # (H, W, 3)
    normal: np.ndarray = None      # (H, W, 3)
    bentNormal: np.ndarray = None  # (H, W, 3)
    contactAo: np.ndarray = None   # (H, W)
    shapeAo: np.ndarray = None     # (H, W)
    avgHitDist: np.ndarray = None  # (H, W)
    aaMask: np.ndarray = None      # (H, W) adaptive-AA refinement mask (aaDebug)
    aoPatchMask: np.ndarray = None  # (Hss, Wss) coarse-AO fallback mask (aoResDebug)
    objectId: np.ndarray = None     # (Hss, Wss) edge G-buffer (edgeGBuffer): (section << 2) | kind
    materialId: np.ndarray = None   # (Hss, Wss) global material index
    gbNormal: np.ndarray = None     # (Hss, Wss, 3) first-hit shading normal
    surfAlpha: np.ndarray = None    # (Hss, Wss) first-hit opacity
    clipCut: np.ndarray = None      # (Hss, Wss) uint8
    clipNearVz: np.ndarray = None   # (Hss, Wss)
    clipFarVz: np.ndarray = None    # (Hss, Wss)


AOV_FIELDS = (("albedo", "albedo", 3), ("normal", "normal", 3), ("bentNormal", "bent_normal", 3),
              ("contactAo", "contact_ao", 1), ("shapeAo", "shape_ao", 1), ("avgHitDist", "avg_hit_dist", 1))


def attach_aovs(fr, opt) -> dict:
    """Allocate the AO AOV planes of a frame when opt.aoWriteAov asks for
    them, the adaptive-AA mask when opt.aaDebug does, and the coarse-AO
    fallback mask when opt.aoResDebug does."""
    out = {}
    ss = max(1, opt.supersample)
    div = ss if opt.aoResDiv < 0 else opt.aoResDiv
    if opt.aoResDebug and div > 1 and opt.aoSamples > 0:
        out["aoPatchMask"] = np.zeros((opt.height * ss, opt.width * ss), np.float32)
        fr.ao_patch_mask = abi.ptr(out["aoPatchMask"])
    if opt.edgeGBuffer:
        hw = (opt.height * ss, opt.width * ss)
        planes = (("objectId", "gb_object_id", np.uint32, ()), ("materialId", "gb_material_id", np.uint32, ()),
                  ("gbNormal", "gb_normal", np.float32, (3,)), ("surfAlpha", "gb_surf_alpha", np.float32, ()),
                  ("clipCut", "gb_clip_cut", np.uint8, ()), ("clipNearVz", "gb_clip_near_vz", np.float32, ()),
                  ("clipFarVz", "gb_clip_far_vz", np.float32, ()))
        for name, cname, dt, tail in planes:
            a = np.zeros(hw + tail, dt)
            out[name] = a
            ctype = {np.uint32: C.c_uint32, np.uint8: C.c_uint8}.get(dt, C.c_float)
            setattr(fr, cname, a.ctypes.data_as(C.POINTER(ctype)))
    if opt.aaMode == 1 and opt.aaDebug:
        out["aaMask"] = np.zeros((opt.height, opt.width), np.float32)
        fr.aa_mask = abi.ptr(out["aaMask"])
    if opt.aoWriteAov:
        for name, cname, ch in AOV_FIELDS:
            a = np.zeros((opt.height, opt.width, ch) if ch > 1 else (opt.height, opt.width), np.float32)
            out[name] = a
            setattr(fr, cname, abi.ptr(a))
    return out


class Context:
    """One GPU, one stream (ubr_context)."""

    def __init__(self, device: int = 0, arena_bytes: int = 0, stream: int | None = None, bvh_leaf_max: int = 0,
                 trace_mode: int = 0, graphs: bool = True, bvh_builder: int = 0, bvh_collapse: int = 0,
                 sah_prim_scale: float = 0.0):
        L = abi.lib()
        self._L = L
        h = C.c_void_p()
        cd = abi.ContextDesc(abi.ABI_VERSION, device, arena_bytes, stream, bvh_leaf_max, trace_mode,
                             0 if graphs else 1, bvh_builder, bvh_collapse, sah_prim_scale)
        st = L.ubr_context_create(C.byref(h), C.byref(cd))
        if st != abi.UBR_OK:
            raise abi.UbrError(st, "ubr_context_create failed")
        self.handle = h

    def _check(self, st):
        if st != abi.UBR_OK:
            raise abi.UbrError(st, self._L.ubr_context_last_error(self.handle).decode())

    def build(self, scene: Scene) -> "BuiltScene":
        d, keep = scene.to_desc()
        h = C.c_void_p()
        self._check(self._L.ubr_scene_build(self.handle, C.byref(d), C.byref(h)))
        return BuiltScene(self, h)

    def render(self, built: "BuiltScene", scene: Scene, opt: RenderOptions, want_ids: bool = True,
               cancel: np.ndarray | None = None) -> FrameResult:
        rd, keep = make_render_desc(scene, opt)
        ss = max(1, opt.supersample)
        W, H = opt.width * ss, opt.height * ss
        color = np.zeros((opt.height, opt.width, 4), np.float32)
        depth = np.zeros((H, W), np.float32)
        vz = np.zeros((H, W), np.float32)
        hg = np.zeros((H, W), np.uint32) if want_ids else None
        hp = np.zeros((H, W), np.uint32) if want_ids else None
        fr = abi.Frame()
        fr.memory = abi.MEMORY_HOST
        fr.color = abi.ptr(color)
        fr.depth = abi.ptr(depth)
        fr.view_z = abi.ptr(vz)
        fr.hit_geom = abi.ptr(hg, C.c_uint32)
        fr.hit_prim = abi.ptr(hp, C.c_uint32)
        aovs = attach_aovs(fr, opt)
        cptr = cancel.ctypes.data_as(C.POINTER(C.c_int32)) if cancel is not None else None
        st = self._L.ubr_render(self.handle, built.handle, C.byref(rd), C.byref(fr), cptr, None)
        stats = dict(render_ms=fr.render_ms, total_ms=fr.total_ms, rays_primary=fr.rays_primary,
                     rays_occlusion=fr.rays_occlusion, capped_rays=fr.capped_rays,
                     stack_overflows=fr.stack_overflows, layers=fr.layers, kernels=fr.kernels)
        if st not in (abi.UBR_OK,):
            self._check(st)
        return FrameResult(opt.width, opt.height, color, depth, vz, hg, hp, fr.render_ms / 1e3, stats, **aovs)

    def render_batch(self, items, want_ids: bool = True, flags: int = 0):
        """Render [(built, scene, opt), ...] in one launch sequence
        (ubr_render_batch); returns ([FrameResult], batch stats)."""
        n = len(items)
        keep, results = [], []
        arr = (abi.BatchItem * n)()
        frames = []
        for i, (built, scene, opt) in enumerate(items):
            rd, k = make_render_desc(scene, opt)
            keep += [rd, k]
            ss = max(1, opt.supersample)
            W, H = opt.width * ss, opt.height * ss
            res = FrameResult(opt.width, opt.height, np.zeros((opt.height, opt.width, 4), np.float32),
                              np.zeros((H, W), np.float32), np.zeros((H, W), np.float32),
                              np.zeros((H, W), np.uint32) if want_ids else None,
                              np.zeros((H, W), np.uint32) if want_ids else None)
            fr = abi.Frame()
            fr.memory = abi.MEMORY_HOST
            fr.color = abi.ptr(res.color)
            fr.depth = abi.ptr(res.depth)
            fr.view_z = abi.ptr(res.viewZ)
            fr.hit_geom = abi.ptr(res.hit_geom, C.c_uint32)
            fr.hit_prim = abi.ptr(res.hit_prim, C.c_uint32)
            frames.append(fr)
            results.append(res)
            arr[i].scene = built.handle
            arr[i].desc = C.pointer(rd)
            arr[i].frame = C.pointer(fr)
        total = abi.Frame()
        total.flags = flags
        self._check(self._L.ubr_render_batch(self.handle, n, arr, C.byref(total)))
        stats = dict(render_ms=total.render_ms, total_ms=total.total_ms, rays_primary=total.rays_primary,
                     rays_occlusion=total.rays_occlusion, kernels=total.kernels, layers=total.layers,
                     phase_ms=list(total.phase_ms))
        return results, stats

    def adjoint(self, built: "BuiltScene", scene: Scene, opt: RenderOptions, d_color: np.ndarray,
                interior_only: bool = False, spheres: bool = True) -> dict:
        """Gradients of a loss L given dL/d(colour) (H, W, 4) (ubr_adjoint):
        per-sphere colour / centre / radius arrays and the global parameters."""
        rd, keep = make_render_desc(scene, opt)
        dc = np.ascontiguousarray(d_color, np.float32).reshape(opt.height, opt.width, 4)
        n = scene.sphere_count()
        g = abi.Grads()
        g.memory = abi.MEMORY_HOST
        g.flags = abi.ADJOINT_INTERIOR_ONLY if interior_only else 0
        out = {}
        if spheres:
            out["sphere_color"] = np.zeros((n, 3), np.float32)
            out["sphere_center"] = np.zeros((n, 3), np.float32)
            out["sphere_radius"] = np.zeros(n, np.float32)
            g.sphere_color = abi.ptr(out["sphere_color"])
            g.sphere_center = abi.ptr(out["sphere_center"])
            g.sphere_radius = abi.ptr(out["sphere_radius"])
        self._check(self._L.ubr_adjoint(self.handle, built.handle, C.byref(rd), dc.ctypes.data, C.byref(g)))
        for k, name in enumerate(abi.MATERIAL_GRAD_FIELDS):
            out[name] = float(g.material[k])
        nl = min(len(scene.lights), abi.ADJOINT_MAX_LIGHTS)
        out["light_direction"] = np.array([list(g.light_direction[l]) for l in range(nl)], np.float64).reshape(nl, 3)
        out["light_color"] = np.array([list(g.light_color[l]) for l in range(nl)], np.float64).reshape(nl, 3)
        out["light_intensity"] = np.array([g.light_intensity[l] for l in range(nl)], np.float64)
        out["ambient_color"] = np.array(list(g.ambient_color))
        out["background"] = np.array(list(g.background))
        out["fog_start"], out["fog_end"] = float(g.fog_start), float(g.fog_end)
        out["fog_color"] = np.array(list(g.fog_color))
        out["ao_distance"], out["ao_intensity"] = float(g.ao_distance), float(g.ao_intensity)
        out["specular_scale"] = float(g.specular_scale)
        out["stats"] = dict(samples=int(g.samples), rays=int(g.rays), adjoint_ms=float(g.adjoint_ms))
        return out

    def occluded(self, built: "BuiltScene", segs: np.ndarray, eps: float) -> np.ndarray:
        segs = np.ascontiguousarray(segs, np.float32).reshape(-1, 6)
        out = np.zeros(len(segs), np.uint8)
        self._check(self._L.ubr_occluded_batch(self.handle, built.handle, segs.ctypes.data, len(segs),
                                               eps, out.ctypes.data, abi.MEMORY_HOST))
        return out

    def occluded_filtered(self, built: "BuiltScene", segs: np.ndarray, eps: float, graze_cos_eps: float = 0.0,
                          coplanar_eps: float = 0.0, exclude_faces=None) -> np.ndarray:
        """Filtered segment visibility (ubr_occluded_filtered_batch);
        exclude_faces: one sequence of base-triangle ids per segment, or None."""
        segs = np.ascontiguousarray(segs, np.float32).reshape(-1, 6)
        n = len(segs)
        out = np.zeros(n, np.uint8)
        offs = faces = None
        if exclude_faces is not None:
            lens = np.array([len(f) for f in exclude_faces], np.uint32)
            offs = np.zeros(n + 1, np.uint32)
            np.cumsum(lens, out=offs[1:])
            faces = np.ascontiguousarray(np.concatenate([np.asarray(f, np.int32) for f in exclude_faces])
                                         if n else np.zeros(0, np.int32), np.int32)
            if faces.size == 0:
                faces = np.zeros(1, np.int32)
        self._check(self._L.ubr_occluded_filtered_batch(
            self.handle, built.handle, segs.ctypes.data, n, eps, graze_cos_eps, coplanar_eps,
            offs.ctypes.data if offs is not None else None, faces.ctypes.data if faces is not None else None,
            out.ctypes.data, abi.MEMORY_HOST))
        return out

    def close(self):
        if getattr(self, "handle", None):
            self._L.ubr_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BuiltScene:
    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    def info(self) -> dict:
        i = abi.SceneInfo()
        self.ctx._check(self.ctx._L.ubr_scene_get_info(self.handle, C.byref(i)))
        return dict(prim_count=list(i.prim_count), geom_id=list(i.geom_id), bvh_nodes=i.bvh_nodes,
                    device_bytes=i.device_bytes, build_ms=i.build_ms, bounds_lo=list(i.bounds_lo),
                    bounds_hi=list(i.bounds_hi), flatten_ms=i.flatten_ms, upload_ms=i.upload_ms)

    def release(self):
        if self.handle:
            self.ctx._L.ubr_scene_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


_DEFAULT_CTX = None


def render(scene: Scene, opt: RenderOptions) -> FrameResult:
    """umbreon::render (umbreon.hpp:29): build, render, release, on GPU 0."""
    global _DEFAULT_CTX
    if _DEFAULT_CTX is None:
        _DEFAULT_CTX = Context(0)
    b = _DEFAULT_CTX.build(scene)
    try:
        return _DEFAULT_CTX.render(b, scene, opt)
    finally:
        b.release()
