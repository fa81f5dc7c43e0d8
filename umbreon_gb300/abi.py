"""ctypes mirror of include/ubr.h and the loader for libubr.so.

The CUDA path is the only path: if ``libubr.so`` is missing or fails to load,
:func:`lib` raises -- there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = Path(__file__).resolve().parent / "lib"

ABI_VERSION = 2
INVALID_ID = 0xFFFFFFFF

STATUS = {
    0: "UBR_OK", 1: "UBR_INVALID_ARGUMENT", 2: "UBR_OUT_OF_MEMORY", 3: "UBR_CUDA_ERROR",
    4: "UBR_CANCELLED", 5: "UBR_TRAVERSAL_LIMIT", 6: "UBR_NO_DEVICE", 7: "UBR_INTERNAL",
}
UBR_OK, UBR_INVALID_ARGUMENT, UBR_OUT_OF_MEMORY, UBR_CUDA_ERROR = 0, 1, 2, 3
UBR_CANCELLED, UBR_TRAVERSAL_LIMIT, UBR_NO_DEVICE, UBR_INTERNAL = 4, 5, 6, 7
MEMORY_HOST, MEMORY_DEVICE = 0, 1

f32p = C.POINTER(C.c_float)
u32p = C.POINTER(C.c_uint32)
u16p = C.POINTER(C.c_uint16)
u8p = C.POINTER(C.c_uint8)


class Material(C.Structure):
    _fields_ = [
        ("ambient", C.c_float), ("diffuse", C.c_float), ("specular", C.c_float),
        ("roughness", C.c_float), ("brilliance", C.c_float), ("phong", C.c_float),
        ("phong_size", C.c_float), ("metallic", C.c_uint32), ("reflection", C.c_float),
        ("emission", C.c_float), ("model", C.c_uint32), ("pbr_metallic", C.c_float),
        ("pbr_roughness", C.c_float), ("pbr_specular", C.c_float),
        ("pbr_anisotropy", C.c_float), ("pbr_anisotropy_rotation", C.c_float),
    ]


MATERIAL_DTYPE = np.dtype([(n, np.float32 if t is C.c_float else np.uint32)
                           for n, t in Material._fields_])
assert MATERIAL_DTYPE.itemsize == C.sizeof(Material)


def material(ambient=0.2, diffuse=0.8, specular=0.0, roughness=0.02, brilliance=1.0, phong=0.0,
             phong_size=40.0, metallic=False, reflection=0.0, emission=0.0, model=0):
    """umbreon::Material defaults (scene.hpp:130-141)."""
    m = np.zeros((), MATERIAL_DTYPE)
    m["ambient"], m["diffuse"], m["specular"], m["roughness"] = ambient, diffuse, specular, roughness
    m["brilliance"], m["phong"], m["phong_size"], m["metallic"] = brilliance, phong, phong_size, int(metallic)
    m["reflection"], m["emission"], m["model"] = reflection, emission, model
    m["pbr_roughness"], m["pbr_specular"] = 0.5, 0.5
    return m


def flat_outline():
    """Material::flatOutline (scene.hpp:206-219): out = pigment."""
    return material(ambient=1.0, diffuse=0.0, specular=0.0)


class SceneDesc(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32),
        ("mesh_vertex_count", C.c_uint64), ("mesh_positions", f32p), ("mesh_normals", f32p),
        ("mesh_colors", f32p), ("mesh_triangle_count", C.c_uint64), ("mesh_index", u32p),
        ("mesh_material", Material), ("mesh_materials", C.POINTER(Material)),
        ("mesh_material_count", C.c_uint32), ("mesh_tri_material", u8p), ("mesh_tri_group", u16p),
        ("sphere_count", C.c_uint64), ("sphere_center_radius", f32p), ("sphere_color", f32p),
        ("sphere_material", C.POINTER(Material)), ("sphere_group", u16p), ("sphere_from_edge", u8p),
        ("cylinder_count", C.c_uint64), ("cyl_p0", f32p), ("cyl_p1", f32p), ("cyl_radius", f32p),
        ("cyl_color", f32p), ("cyl_opacity1", f32p), ("cyl_material", C.POINTER(Material)),
        ("cyl_group", u16p), ("cyl_open", u8p), ("cyl_from_edge", u8p),
        ("instance_count", C.c_uint64), ("instance_offsets", f32p),
    ]


class Light(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("color", C.c_float * 3), ("intensity", C.c_float),
                ("casts_highlight", C.c_uint32), ("angular_radius", C.c_float)]


class RenderDesc(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32), ("width", C.c_int32), ("height", C.c_int32),
        ("supersample", C.c_int32),
        ("cam_position", C.c_float * 3), ("cam_direction", C.c_float * 3), ("cam_up", C.c_float * 3),
        ("cam_fovy", C.c_float), ("cam_orthographic", C.c_uint32), ("cam_height", C.c_float),
        ("lights", C.POINTER(Light)), ("light_count", C.c_uint32),
        ("ambient_color", C.c_float * 3), ("background", C.c_float * 3),
        ("fog_enabled", C.c_uint32), ("fog_color", C.c_float * 3), ("fog_start", C.c_float),
        ("fog_end", C.c_float), ("clip_near", C.c_float), ("clip_far", C.c_float),
        ("assumed_gamma", C.c_float),
        ("ao_samples", C.c_int32), ("ao_distance", C.c_float), ("ao_intensity", C.c_float),
        ("ao_falloff_power", C.c_float), ("ao_multiscale", C.c_uint32), ("ao_bent_normal", C.c_uint32),
        ("ao_sky_color", C.c_float * 3), ("ao_ground_color", C.c_float * 3),
        ("ao_use_camera_up", C.c_uint32), ("ao_up", C.c_float * 3), ("ao_multibounce", C.c_uint32),
        ("ao_low_discrepancy", C.c_uint32), ("ao_diffuse_factor", C.c_float),
        ("shadows", C.c_uint32), ("shadow_samples", C.c_int32), ("light_radius_deg", C.c_float),
        ("env_lights", C.c_int32), ("env_intensity", C.c_float), ("env_key_scale", C.c_float),
        ("env_angle", C.c_float), ("specular_scale", C.c_float), ("transparency", C.c_uint32),
        ("transparent_background", C.c_uint32), ("max_transparent_layers", C.c_int32),
        ("gi_integrator", C.c_int32), ("ao_write_aov", C.c_uint32), ("aa_mode", C.c_int32),
        ("aa_threshold", C.c_float), ("aa_depth", C.c_int32), ("ao_res_div", C.c_int32),
        ("edge_gbuffer", C.c_uint32), ("denoiser", C.c_int32), ("denoise_iters", C.c_int32),
        ("denoise_sigma_z", C.c_float), ("denoise_sigma_n", C.c_float), ("denoise_sigma_l", C.c_float),
        ("denoise_demodulate_albedo", C.c_uint32),
        ("gi", C.c_uint32), ("pt1_spp", C.c_int32), ("gi_bounces", C.c_int32), ("gi_max_distance", C.c_float),
        ("gi_intensity", C.c_float), ("gi_env_intensity", C.c_float), ("pt1_seed", C.c_uint32),
        ("pt1_sky_mode", C.c_int32), ("pt1_sky_radiance", C.c_float * 3), ("pt1_ld", C.c_uint32),
        ("pt1_clamp", C.c_float),
        ("pt1_gather_div", C.c_int32), ("pt1_half_res", C.c_uint32), ("pt1_denoise", C.c_uint32),
        ("pt1_upsample_normal_pow", C.c_float), ("pt1_upsample_depth_scale", C.c_float),
        ("pt1_edge_patch", C.c_uint32), ("pt1_edge_patch_spp_mul", C.c_int32), ("pt1_edge_patch_thresh", C.c_float),
        ("pt2_pattern", C.c_int32), ("pt2_emissive", C.c_uint32), ("pt2_rounds", C.c_int32),
        ("pt2_radius", C.c_float), ("pt2_unbiased", C.c_uint32), ("pt2_m_cap", C.c_float),
        ("pt2_w_clamp", C.c_float), ("pt2_adaptive", C.c_uint32), ("pt2_adaptive_thresh", C.c_float),
        ("pt2_adaptive_mul", C.c_int32), ("pt2_emissive_nee", C.c_uint32), ("pt2_reflect", C.c_uint32),
        ("pt2_glossy", C.c_uint32), ("pt2_glossy_spp", C.c_int32), ("pt2_glossy_denoise", C.c_uint32),
    ]


class Frame(C.Structure):
    _fields_ = [
        ("memory", C.c_int32), ("flags", C.c_uint32), ("color", f32p), ("depth", f32p), ("view_z", f32p),
        ("hit_geom", u32p), ("hit_prim", u32p),
        ("render_ms", C.c_double), ("total_ms", C.c_double), ("rays_primary", C.c_uint64),
        ("rays_occlusion", C.c_uint64), ("capped_rays", C.c_uint64), ("stack_overflows", C.c_uint64),
        ("layers", C.c_uint32), ("kernels", C.c_uint32), ("phase_ms", C.c_double * 5),
        ("node_bytes", C.c_uint64 * 2), ("prim_bytes", C.c_uint64 * 2), ("nodes_visited", C.c_uint64 * 2),
        ("albedo", f32p), ("normal", f32p), ("bent_normal", f32p), ("contact_ao", f32p), ("shape_ao", f32p),
        ("avg_hit_dist", f32p), ("aa_mask", f32p), ("ao_patch_mask", f32p),
        ("gb_object_id", u32p), ("gb_material_id", u32p), ("gb_normal", f32p), ("gb_surf_alpha", f32p),
        ("gb_clip_cut", C.POINTER(C.c_uint8)), ("gb_clip_near_vz", f32p), ("gb_clip_far_vz", f32p),
        ("gi_ms", C.c_double * 6), ("gi_gather_rays", C.c_uint64), ("gi_nee_rays", C.c_uint64),
        ("gi_gbuffer_rays", C.c_uint64), ("gi_patched_pixels", C.c_uint64),
    ]


FRAME_PROFILE = 1
FRAME_COUNT = 2


class ContextDesc(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("device", C.c_int32), ("arena_bytes", C.c_uint64),
                ("stream", C.c_void_p), ("bvh_leaf_max", C.c_uint32), ("trace_mode", C.c_uint32),
                ("disable_graphs", C.c_uint32), ("bvh_builder", C.c_uint32),
                ("bvh_collapse", C.c_uint32), ("bvh_sah_prim_scale", C.c_float), ("reserved", C.c_uint32 * 2)]


class SceneInfo(C.Structure):
    _fields_ = [("prim_count", C.c_uint64 * 4), ("geom_id", C.c_uint32 * 4), ("bvh_nodes", C.c_uint64),
                ("device_bytes", C.c_uint64), ("build_ms", C.c_double), ("bounds_lo", C.c_float * 3),
                ("bounds_hi", C.c_float * 3), ("flatten_ms", C.c_double), ("upload_ms", C.c_double)]


class BatchItem(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("desc", C.POINTER(RenderDesc)), ("frame", C.POINTER(Frame))]


# Every symbol include/ubr.h declares, with its ctypes signature.
ADJOINT_MAX_LIGHTS = 4
ADJOINT_INTERIOR_ONLY = 1


class Grads(C.Structure):
    """ubr_grads (include/ubr.h)."""
    _fields_ = [
        ("memory", C.c_int32), ("flags", C.c_uint32),
        ("sphere_color", f32p), ("sphere_center", f32p), ("sphere_radius", f32p),
        ("material", C.c_float * 9),
        ("light_direction", (C.c_float * 3) * ADJOINT_MAX_LIGHTS),
        ("light_color", (C.c_float * 3) * ADJOINT_MAX_LIGHTS),
        ("light_intensity", C.c_float * ADJOINT_MAX_LIGHTS),
        ("ambient_color", C.c_float * 3), ("background", C.c_float * 3),
        ("fog_start", C.c_float), ("fog_end", C.c_float), ("fog_color", C.c_float * 3),
        ("ao_distance", C.c_float), ("ao_intensity", C.c_float), ("specular_scale", C.c_float),
        ("samples", C.c_uint64), ("rays", C.c_uint64), ("adjoint_ms", C.c_float),
        ("reserved_f", C.c_float * 3), ("reserved", C.c_uint64 * 4),
    ]


MATERIAL_GRAD_FIELDS = ("ambient", "diffuse", "specular", "roughness", "brilliance", "phong", "phong_size",
                        "reflection", "emission")

SIGNATURES = {
    "ubr_status_string": (C.c_char_p, [C.c_int]),
    "ubr_abi_version": (C.c_uint32, []),
    "ubr_context_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(ContextDesc)]),
    "ubr_context_destroy": (C.c_int, [C.c_void_p]),
    "ubr_context_last_error": (C.c_char_p, [C.c_void_p]),
    "ubr_scene_build": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    "ubr_scene_release": (C.c_int, [C.c_void_p]),
    "ubr_scene_get_info": (C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    "ubr_render": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RenderDesc), C.POINTER(Frame),
                             C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]),
    "ubr_render_batch": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(BatchItem), C.POINTER(Frame)]),
    "ubr_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RenderDesc), C.c_void_p, C.POINTER(Grads)]),
    "ubr_occluded_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_float,
                                     C.c_void_p, C.c_int32]),
    "ubr_occluded_filtered_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_float, C.c_float,
                                              C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "ubr_occluded_batch_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_float,
                                             C.c_void_p]),
}

_LIB = None


def lib_path() -> Path:
    """libubr.so of this package, or the file named by UBR_LIBRARY."""
    import os
    return Path(os.environ.get("UBR_LIBRARY") or (LIBDIR / "libubr.so"))


def lib():
    """Load libubr.so; raise if it is not built (no fallback exists)."""
    global _LIB
    if _LIB is None:
        p = lib_path()
        if not p.exists():
            raise RuntimeError(f"{p} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def ptr(a, ctype=C.c_float):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


class UbrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
