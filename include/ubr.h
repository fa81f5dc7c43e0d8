/*
 * ubr.h -- C-ABI of the GB300 ray-cast + shade library (libubr.so).
 *
 * This is the device boundary of the umbreon renderer.  The reference runs the
 * whole pixel loop on the CPU through Embree and TBB; here the C++ host layer
 * (umbreon::render, same public API) flattens Scene/RenderOptions into the
 * plain structs below and calls these entry points, which run everything on
 * one GPU.  Only plain pointers, sizes and POD structs cross the boundary: no
 * C++ types, no torch types, no exceptions.  Every entry returns ubr_status.
 *
 * Reference interfaces replaced (paths inside the CueMol/umbreon project):
 *   ubr_context_*        the RTCDevice the renderer creates per frame or
 *                        shares across group-alpha passes
 *                        (src/umbreon/render/embree_renderer.cpp:1267-1274,
 *                         src/umbreon/umbreon.cpp:21-40)
 *   ubr_scene_build      detail::buildEmbreeScene (render/scene_build.hpp:126,
 *                        scene_build.cpp:133-170, curve_build.cpp:41-267)
 *   ubr_render           EmbreeRenderer::render + the finishing steps of
 *                        renderFrame (render/embree_renderer.cpp:1260-1745,
 *                        render/pipeline.cpp:44-50,126-129,182-223,254)
 *   ubr_occluded_batch   EmbreeRenderer::occluded (embree_renderer.cpp:294-357),
 *   ubr_occluded_filtered_batch   plain and filtered branches
 *   ubr_render_batch     no reference counterpart (many frames per launch)
 *   ubr_adjoint          no reference counterpart (image-loss gradients)
 */
#ifndef UBR_H_
#define UBR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UBR_ABI_VERSION 2u

/* Status codes.  The reference throws std::runtime_error on device/BVH
 * failure (scene_build.cpp:164-168, embree_renderer.cpp:1271-1286); the host
 * layer maps every non-OK status to that exception, except UBR_CANCELLED
 * which becomes FrameResult::cancelled = true (embree_renderer.cpp:1743). */
typedef enum ubr_status {
  UBR_OK = 0,
  UBR_INVALID_ARGUMENT = 1,
  UBR_OUT_OF_MEMORY = 2,
  UBR_CUDA_ERROR = 3,
  UBR_CANCELLED = 4,
  UBR_TRAVERSAL_LIMIT = 5, /* a traversal stack overflowed; frame still written */
  UBR_NO_DEVICE = 6,
  UBR_INTERNAL = 7
} ubr_status;

/* Primitive kinds, in the geomID attach order of the reference
 * (scene_build.cpp:159-161: mesh, spheres, open cylinders, capped cylinders).
 * The geomID of a kind is its rank among the kinds present in the scene. */
typedef enum ubr_kind {
  UBR_KIND_MESH = 0,
  UBR_KIND_SPHERE = 1,
  UBR_KIND_CYLINDER_OPEN = 2,   /* ROUND_LINEAR_CURVE, chained */
  UBR_KIND_CYLINDER_CAPPED = 3  /* CONE_LINEAR_CURVE, flat caps */
} ubr_kind;

#define UBR_INVALID_ID 0xFFFFFFFFu

/* POV finish, field-for-field umbreon::Material (scene.hpp:130-224). */
typedef struct ubr_material {
  float ambient;
  float diffuse;
  float specular;
  float roughness;
  float brilliance;
  float phong;
  float phong_size;
  uint32_t metallic;       /* bool */
  float reflection;
  float emission;
  uint32_t model;          /* 0 Pov, 1 Principled (GGX direct pass, the
                            * pbr_* fields; anisotropy on spheres and
                            * cylinders), 2 Toon (shaded as Pov) */
  float pbr_metallic;
  float pbr_roughness;
  float pbr_specular;
  float pbr_anisotropy;
  float pbr_anisotropy_rotation;
} ubr_material;

/* Scene geometry, structure of arrays, HOST memory.  Mirrors umbreon::Scene's
 * Mesh / Sphere / Cylinder vectors (scene.hpp:233-356) and instanceOffsets.
 * NULL optional arrays take the reference's empty-vector meaning. */
typedef struct ubr_scene_desc {
  uint32_t abi_version;            /* UBR_ABI_VERSION */
  /* mesh */
  uint64_t mesh_vertex_count;
  const float* mesh_positions;     /* 3 * vertex_count */
  const float* mesh_normals;       /* 3 * vertex_count */
  const float* mesh_colors;        /* 4 * vertex_count (rgb + opacity) */
  uint64_t mesh_triangle_count;
  const uint32_t* mesh_index;      /* 3 * triangle_count, NULL = de-indexed */
  ubr_material mesh_material;      /* Mesh::material */
  const ubr_material* mesh_materials; /* Mesh::materials (may be NULL) */
  uint32_t mesh_material_count;
  const uint8_t* mesh_tri_material;   /* triangle_count or NULL */
  const uint16_t* mesh_tri_group;     /* triangle_count or NULL */
  /* spheres */
  uint64_t sphere_count;
  const float* sphere_center_radius;  /* 4 * n: x y z r */
  const float* sphere_color;          /* 4 * n */
  const ubr_material* sphere_material;/* n */
  const uint16_t* sphere_group;       /* n or NULL */
  const uint8_t* sphere_from_edge;    /* n or NULL */
  /* cylinders */
  uint64_t cylinder_count;
  const float* cyl_p0;                /* 3 * n */
  const float* cyl_p1;                /* 3 * n */
  const float* cyl_radius;            /* n */
  const float* cyl_color;             /* 4 * n */
  const float* cyl_opacity1;          /* n or NULL (NULL = all < 0) */
  const ubr_material* cyl_material;   /* n */
  const uint16_t* cyl_group;          /* n or NULL */
  const uint8_t* cyl_open;            /* n or NULL (NULL = all capped) */
  const uint8_t* cyl_from_edge;       /* n or NULL */
  /* grid instances (offsets baked into the geometry, scene_build.cpp:150-152) */
  uint64_t instance_count;
  const float* instance_offsets;      /* 3 * n or NULL */
} ubr_scene_desc;

/* One distant light, umbreon::DistantLight (scene.hpp:390-405). */
typedef struct ubr_light {
  float direction[3];   /* direction the light travels */
  float color[3];
  float intensity;
  uint32_t casts_highlight;
  float angular_radius;
} ubr_light;

/* Flattened render request: the RenderOptions fields this path honours
 * (render_options.hpp:14-328) plus Scene's camera, lights, ambient,
 * background, fog, clip planes and assumed gamma (scene.hpp:380-479). */
typedef struct ubr_render_desc {
  uint32_t abi_version;
  int32_t width;          /* FINAL output size */
  int32_t height;
  int32_t supersample;
  /* camera */
  float cam_position[3];
  float cam_direction[3];
  float cam_up[3];
  float cam_fovy;
  uint32_t cam_orthographic;
  float cam_height;
  /* lights and scene constants */
  const ubr_light* lights;
  uint32_t light_count;
  float ambient_color[3];
  float background[3];
  uint32_t fog_enabled;
  float fog_color[3];
  float fog_start;
  float fog_end;
  float clip_near;        /* -inf = off */
  float clip_far;         /* +inf = off */
  float assumed_gamma;
  /* ambient occlusion */
  int32_t ao_samples;
  float ao_distance;
  float ao_intensity;
  float ao_falloff_power;
  uint32_t ao_multiscale;
  uint32_t ao_bent_normal;
  float ao_sky_color[3];
  float ao_ground_color[3];
  uint32_t ao_use_camera_up;
  float ao_up[3];
  uint32_t ao_multibounce;
  uint32_t ao_low_discrepancy;
  float ao_diffuse_factor;
  /* shadows */
  uint32_t shadows;
  int32_t shadow_samples;
  float light_radius_deg;
  /* environment dome */
  int32_t env_lights;
  float env_intensity;
  float env_key_scale;
  float env_angle;
  /* shading / transparency */
  float specular_scale;
  uint32_t transparency;
  uint32_t transparent_background;
  int32_t max_transparent_layers;
  /* giIntegrator selects the soft-shadow radius rule
   * (embree_renderer.cpp:452-454) and, with gi (below), the integrator:
   * only 1 (pt1) is built here */
  int32_t gi_integrator;
  /* RenderOptions::aoWriteAov (render_options.hpp:62): fill the AO AOV
   * outputs of ubr_frame */
  uint32_t ao_write_aov;
  /* RenderOptions::aaMode / aaThreshold / aaDepth (render_options.hpp:26-39):
   * 1 = adaptive AA (centre sample per output pixel, refinement mask,
   * flagged blocks shaded per subpixel, the others replicate a centre
   * re-shaded with ss^2 AO / soft-shadow samples); aaDepth above the
   * supersample factor shades each flagged cell as the box average of
   * ceil(aaDepth / ss)^2 samples of a finer lattice; other aa_mode values
   * render the full grid */
  int32_t aa_mode;
  float aa_threshold;
  int32_t aa_depth;
  /* RenderOptions::aoResDiv (render_options.hpp:64-74): > 1 gathers the AO
   * once per cell of the hi-res grid divided by this factor (on the first
   * hits of that coarse grid) and lets each shaded hit interpolate it with
   * normal / depth guides, falling back to its own AO rays where the guides
   * reject; -1 = the supersample factor; 0 or 1 = AO rays at every hit */
  int32_t ao_res_div;
  /* the stroke-edge pass's first-hit G-buffer (RenderOptions::strokeEdges
   * enables it in the reference, transparency.hpp:394-428, 470-481): fills
   * the gb_* planes of ubr_frame; the edge pass itself is the caller's.
   * Not with adaptive AA (UBR_INVALID_ARGUMENT). */
  uint32_t edge_gbuffer;
  /* RenderOptions::denoiser / denoiseIters / denoiseSigmaZ / denoiseSigmaN /
   * denoiseSigmaL / denoiseDemodulateAlbedo (render_options.hpp:255-268):
   * 1 (a-trous) or 2 (OIDN, absent here: the a-trous runs, as the reference
   * does without OIDN) filters the final-resolution linear colour before the
   * gamma (pipeline.cpp:224-252), guided by the AO AOV normal and albedo; it
   * runs only when ao_write_aov provides them, as in the reference without
   * GI. */
  int32_t denoiser;
  int32_t denoise_iters;
  float denoise_sigma_z;
  float denoise_sigma_n;
  float denoise_sigma_l;
  uint32_t denoise_demodulate_albedo;
  /* GI: RenderOptions::gi with the path-traced gather (pt1, the
   * reference's frozen anchor, giIntegrator = 1; pt2, its default, = 2),
   * pt1Spp, giBounces, giMaxDistance (0 = unbounded), giIntensity,
   * giEnvIntensity, pt1Seed, pt1SkyMode / pt1SkyRadiance (the gather's miss
   * term; mode 1 takes ao_ground_color as the ground tint), pt1Ld and
   * pt1Clamp (render_options.hpp:85-151).  gi != 0 needs gi_integrator 1
   * or 2, pt1_spp >= 1, gi_bounces >= 1, no adaptive AA and no coarse-grid
   * AO (the reference turns those two off under GI, pipeline.cpp:60-78), and
   * one frame per call (not ubr_render_batch); otherwise
   * UBR_INVALID_ARGUMENT.  The irradiance cache (giIntegrator 0) is not part
   * of this library. */
  uint32_t gi;
  int32_t pt1_spp;
  int32_t gi_bounces;
  float gi_max_distance;
  float gi_intensity;
  float gi_env_intensity;
  uint32_t pt1_seed;
  int32_t pt1_sky_mode;
  float pt1_sky_radiance[3];
  uint32_t pt1_ld;
  float pt1_clamp;
  /* the gather grid and what follows it (render_options.hpp:130-176):
   * pt1GatherDiv (-1 = the supersample factor, 0 = pt1HalfRes ? 2 : 1,
   * k >= 1 = a ceil(W/k) x ceil(H/k) grid with its own primary rays),
   * pt1HalfRes, pt1Denoise (the a-trous filter on E at gather resolution:
   * OIDN is absent, as in a reference build without it), the joint-bilateral
   * upsample's pt1UpsampleNormalPow / pt1UpsampleDepthScale, and the
   * silhouette edge patch pt1EdgePatch / pt1EdgePatchSppMul /
   * pt1EdgePatchThresh.  The denoise takes denoise_iters / denoise_sigma_*
   * above. */
  int32_t pt1_gather_div;
  uint32_t pt1_half_res;
  uint32_t pt1_denoise;
  float pt1_upsample_normal_pow;
  float pt1_upsample_depth_scale;
  uint32_t pt1_edge_patch;
  int32_t pt1_edge_patch_spp_mul;
  float pt1_edge_patch_thresh;
  /* pt2 (gi_integrator = 2, render_options.hpp:178-252): first-bounce
   * pattern (0 Owen-scrambled Sobol per pixel, 1 blue noise), emission at
   * gather vertices, ReSTIR rounds / radius / unbiased / M cap / W clamp,
   * adaptive spp (threshold, multiplier), emissive-triangle NEE, traced
   * mirror reflection, glossy reflection (spp, denoise). */
  int32_t pt2_pattern;
  uint32_t pt2_emissive;
  int32_t pt2_rounds;
  float pt2_radius;
  uint32_t pt2_unbiased;
  float pt2_m_cap;
  float pt2_w_clamp;
  uint32_t pt2_adaptive;
  float pt2_adaptive_thresh;
  int32_t pt2_adaptive_mul;
  uint32_t pt2_emissive_nee;
  uint32_t pt2_reflect;
  uint32_t pt2_glossy;
  int32_t pt2_glossy_spp;
  uint32_t pt2_glossy_denoise;
} ubr_render_desc;

/* Where a frame's buffers live. */
typedef enum ubr_memory {
  UBR_MEMORY_HOST = 0,    /* pageable or pinned host memory; copied at the end */
  UBR_MEMORY_DEVICE = 1   /* device pointers on the context's GPU */
} ubr_memory;

/* Caller-owned output buffers.  NULL pointers are skipped.  Sizes follow
 * FrameResult (frame_result.hpp:43-124) as renderFrame leaves it:
 *   color   : W*H*4 final (downsampled, fogged, gamma'd) linear RGBA
 *   depth   : Wss*Hss  hi-res first-hit ray distance (renderFrame does not
 *             downsample depth, pipeline.cpp:182-228)
 *   view_z  : Wss*Hss  hi-res plane eye-z of the first hit
 *   hit_geom, hit_prim : Wss*Hss first-hit (geomID, primID); UBR_INVALID_ID
 *             on a miss (parity evidence, not a FrameResult field)
 * Statistics are written back into the struct. */
#define UBR_FRAME_PROFILE 1u  /* time each kernel phase with CUDA events */
#define UBR_FRAME_COUNT 2u    /* count BVH node / primitive bytes fetched */

typedef struct ubr_frame {
  int32_t memory;         /* ubr_memory */
  uint32_t flags;         /* UBR_FRAME_PROFILE | UBR_FRAME_COUNT */
  float* color;
  float* depth;
  float* view_z;
  uint32_t* hit_geom;
  uint32_t* hit_prim;
  /* out: statistics */
  double render_ms;       /* device time of the pixel loop (renderSeconds) */
  double total_ms;        /* device time of the whole ubr_render call */
  uint64_t rays_primary;  /* closest-hit rays traced (all layers) */
  uint64_t rays_occlusion;/* AO + shadow any-hit rays traced */
  uint64_t capped_rays;   /* rays that reached the transparent-layer cap */
  uint64_t stack_overflows;
  uint32_t layers;        /* transparency rounds executed */
  uint32_t kernels;       /* kernels launched by this call */
  /* with UBR_FRAME_PROFILE: device ms per phase
   * [0] closest-hit trace, [1] surface prep, [2] AO + shadow rays,
   * [3] shade + composite, [4] fog/downsample/gamma */
  double phase_ms[5];
  /* with UBR_FRAME_COUNT: bytes of BVH nodes and of primitive records
   * fetched, [0] closest-hit rays, [1] occlusion rays */
  uint64_t node_bytes[2];
  uint64_t prim_bytes[2];
  uint64_t nodes_visited[2];
  /* AO AOVs of the first hit, output resolution (box-averaged like the
   * colour), written when the desc sets ao_write_aov (FrameResult::albedo,
   * normal, bentNormal, contactAo, shapeAo, avgHitDist; frame_result.hpp:48-79,
   * filled by storeShadingChannels, embree_renderer.cpp:213-233): mesh hits
   * give the vertex colour, shading normal and the AO estimator's bent
   * normal / contact / shape openness / mean occluder distance; primitive
   * hits and background keep the neutral values (0, 0, 0, 1, 1, 0). */
  float* albedo;          /* 3 per pixel */
  float* normal;          /* 3 per pixel */
  float* bent_normal;     /* 3 per pixel */
  float* contact_ao;      /* 1 per pixel */
  float* shape_ao;        /* 1 per pixel */
  float* avg_hit_dist;    /* 1 per pixel */
  /* adaptive AA refinement mask, output resolution, 1 = refined
   * (FrameResult::aaMask with aaDebug); written when aa_mode = 1 */
  float* aa_mask;
  /* coarse-grid AO fallback mask, hi-res, 1 = the first hit gathered its own
   * AO (FrameResult::aoPatchMask with aoResDebug); written when the coarse
   * grid is active */
  float* ao_patch_mask;
  /* edge G-buffer, hi-res, written when edge_gbuffer = 1 (FrameResult::
   * objectId / materialId / normal / surfAlpha / clipCut / clipNearVz /
   * clipFarVz): (section << 2) | kind and the global material index of the
   * first hit (0xFFFFFFFF on background), its shading normal (3 per pixel)
   * and opacity; with clip planes set, 1 where a backface first hit has its
   * clipped-away front confirmed, and on background pixels the view z of
   * the first surface removed in front of the near / beyond the far plane */
  uint32_t* gb_object_id;
  uint32_t* gb_material_id;
  float* gb_normal;
  float* gb_surf_alpha;
  uint8_t* gb_clip_cut;
  float* gb_clip_near_vz;
  float* gb_clip_far_vz;
  /* GI statistics (FrameResult::pt1Timing, pt1Rays; frame_result.hpp): the
   * device ms of the gather G-buffer, the gather (with pt2's adaptive
   * refinement), the denoise of E, the upsample, the edge patch, and pt2's
   * traced mirror + glossy reflection; the gather rays (all bounces and the
   * reflection rays), the NEE shadow rays, the G-buffer primary rays, and
   * the number of pixels the edge patch re-gathered */
  double gi_ms[6];
  uint64_t gi_gather_rays;
  uint64_t gi_nee_rays;
  uint64_t gi_gbuffer_rays;
  uint64_t gi_patched_pixels;
} ubr_frame;

/* Context: one GPU, one CUDA stream, one device arena.  Scenes and frame
 * scratch are allocated stream-ordered from the context's own memory pool;
 * memory released by ubr_scene_release or scratch growth stays in that pool
 * for reuse until ubr_context_destroy. */
typedef struct ubr_context ubr_context;
typedef struct ubr_scene ubr_scene;

typedef struct ubr_context_desc {
  uint32_t abi_version;
  int32_t device;              /* CUDA ordinal */
  uint64_t arena_bytes;        /* 0 = grow on demand; >0 = hard cap */
  void* stream;                /* cudaStream_t to run on, NULL = own stream */
  /* BVH tuning (0 = library default): the most primitives a wide-BVH leaf
   * holds (1..3); smaller leaves mean more nodes and fewer primitive tests */
  uint32_t bvh_leaf_max;
  /* occlusion-ray kernel (0 = library default): 1 = one thread per ray,
   * 2 = persistent warps that refill idle lanes with new rays, 3 = resident
   * grid striding over the rays with the top BVH levels in shared memory,
   * 4 = one thread per ray with node visits and primitive tests interleaved
   * one per step */
  uint32_t trace_mode;
  /* 1 = launch every kernel on its own instead of replaying single-layer
   * frames from a captured CUDA graph (0 = graphs, the default) */
  uint32_t disable_graphs;
  /* BVH builder (0 = library default): 1 = Karras radix tree over Morton
   * codes, 2 = locally-ordered clustering (PLOC) over the same Morton order;
   * leaf sizes above 1 always use the radix tree */
  uint32_t bvh_builder;
  /* binary -> 8-wide collapse (0 = library default): 1 = greedy (open the
   * largest child, leaves of bvh_leaf_max primitives), 2 = SAH-optimal
   * dynamic programme choosing every node's children and leaves of 1..3
   * primitives */
  uint32_t bvh_collapse;
  /* SAH collapse: weight of a primitive test against a node visit, as a
   * multiple of the library's per-kind weights (0 = 1) */
  float bvh_sah_prim_scale;
  uint32_t reserved[2];
} ubr_context_desc;

const char* ubr_status_string(ubr_status s);
uint32_t ubr_abi_version(void);

ubr_status ubr_context_create(ubr_context** out, const ubr_context_desc* desc);
ubr_status ubr_context_destroy(ubr_context* ctx);
/* Message of the last failure on this context (never NULL). */
const char* ubr_context_last_error(const ubr_context* ctx);

/* Upload the scene, build the side tables and the LBVH on the GPU.
 * primIDs follow the reference order (scene_build.cpp:46-71,99-121,
 * curve_build.cpp:95-175,221-247) so (geomID, primID) can be compared. */
ubr_status ubr_scene_build(ubr_context* ctx, const ubr_scene_desc* desc,
                           ubr_scene** out);
/* Frees the scene's device memory.  Destroying a context releases the device
 * memory of the scenes still alive on it; their handles then stay valid for
 * ubr_scene_release only. */
ubr_status ubr_scene_release(ubr_scene* scene);
/* Scene facts: primitive counts per kind, BVH node count, build time. */
typedef struct ubr_scene_info {
  uint64_t prim_count[4];
  uint32_t geom_id[4];     /* UBR_INVALID_ID when the kind is absent */
  uint64_t bvh_nodes;
  uint64_t device_bytes;
  double build_ms;         /* host wall time of ubr_scene_build */
  float bounds_lo[3];
  float bounds_hi[3];
  double flatten_ms;       /* of which: host flattening (primID order, chains, materials) */
  double upload_ms;        /*           allocations + host-to-device copies queued */
} ubr_scene_info;
ubr_status ubr_scene_get_info(const ubr_scene* scene, ubr_scene_info* info);

/* Render one frame: primary rays, closest hits through the transparency walk,
 * POV shading with AO and shadow rays, fog, box downsample, gamma.
 * cancel_flag (host memory, may be NULL) is polled between kernel rounds;
 * a set flag returns UBR_CANCELLED with a partial frame.
 * progress_units (may be NULL) counts finished transparency rounds. */
ubr_status ubr_render(ubr_context* ctx, const ubr_scene* scene,
                      const ubr_render_desc* desc, ubr_frame* frame,
                      const volatile int32_t* cancel_flag,
                      uint64_t* progress_units);

/* Many frames in one launch sequence: every stage runs once over the pixels
 * and rays of all items (a global ray queue), and single-layer batches are
 * replayed from a CUDA graph.  Items may use different scenes, cameras,
 * resolutions and options; each item's outputs go to its own frame buffers.
 * `total` (may be NULL) receives the batch's statistics; its `flags` select
 * profiling as for ubr_render.  Items whose passes depend on per-frame host
 * decisions (adaptive AA, the coarse AO grid, the edge G-buffer) run as their
 * own launch sequences after the batched rest; `total` then sums the
 * statistics.  No reference counterpart (the reference renders one frame per
 * call). */
typedef struct ubr_batch_item {
  const ubr_scene* scene;
  const ubr_render_desc* desc;
  ubr_frame* frame;
} ubr_batch_item;

ubr_status ubr_render_batch(ubr_context* ctx, uint32_t n, const ubr_batch_item* items,
                            ubr_frame* total);

/* Adjoint of ubr_render: gradients of a scalar image loss L with respect to
 * scene and render parameters, given dL/d(colour) of the frame.  No
 * reference counterpart (the reference renders forward only).
 *
 * Scope: sphere scenes rendered in one opaque layer (every sphere opaque, or
 * transparency off); distant lights with hard shadows (at most
 * UBR_ADJOINT_MAX_LIGHTS, no env dome, no soft shadows); legacy or enhanced AO
 * without bent normal or multibounce; POV shading; fog; box downsample;
 * assumed gamma.  Other descriptions return UBR_INVALID_ARGUMENT.
 *
 * Visibility is held fixed: the primary hit, each AO sample's occluder and
 * each shadow bit are recomputed by re-traversal and enter as constants.
 * Gradients flow through hit distances, normals, AO sample directions and
 * occluder distances, and every shading, fog, downsample and gamma term, but
 * not through visibility changes (silhouette / edge terms are excluded).  With
 * UBR_ADJOINT_INTERIOR_ONLY only hi-res samples whose 3x3 neighbourhood shows
 * one primitive (or only background) contribute. */
#define UBR_ADJOINT_MAX_LIGHTS 4
#define UBR_ADJOINT_INTERIOR_ONLY 1u

typedef struct ubr_grads {
  int32_t memory;             /* UBR_MEMORY_*: d_color and the per-sphere arrays */
  uint32_t flags;             /* UBR_ADJOINT_INTERIOR_ONLY */
  /* per input sphere (n = sphere_count of the scene desc, instances summed);
   * each may be NULL */
  float* sphere_color;        /* 3n: d/d(r, g, b) */
  float* sphere_center;       /* 3n */
  float* sphere_radius;       /* n */
  /* global parameters (written) */
  float material[9];          /* d/d ambient, diffuse, specular, roughness, brilliance,
                                 phong, phong_size, reflection, emission, each moved
                                 together in every sphere's material */
  float light_direction[UBR_ADJOINT_MAX_LIGHTS][3];  /* d/d ubr_light.direction */
  float light_color[UBR_ADJOINT_MAX_LIGHTS][3];
  float light_intensity[UBR_ADJOINT_MAX_LIGHTS];
  float ambient_color[3];
  float background[3];
  float fog_start, fog_end;
  float fog_color[3];
  float ao_distance, ao_intensity;
  float specular_scale;
  /* statistics (written) */
  uint64_t samples;           /* hi-res samples that contributed */
  uint64_t rays;              /* rays re-traced */
  float adjoint_ms;           /* device time of the adjoint launches */
  float reserved_f[3];
  uint64_t reserved[4];
} ubr_grads;

/* d_color: dL/d(frame colour), width x height x 4 floats (r g b a) in
 * grads->memory.  Per-sphere arrays are overwritten (not accumulated). */
ubr_status ubr_adjoint(ubr_context* ctx, const ubr_scene* scene, const ubr_render_desc* desc,
                       const float* d_color, ubr_grads* grads);

/* Segment occlusion for the stroke-edge pass: out[i] = 1 when any geometry
 * lies strictly inside segment (p[i], q[i]) trimmed by eps
 * (embree_renderer.cpp:294-315 plain any-hit branch).  segs = 6*n floats
 * (px py pz qx qy qz), in the memory space given by `memory`.  Returns
 * UBR_TRAVERSAL_LIMIT (answers still written) when a traversal ran out of
 * stack, since its answer may have missed an occluder. */
ubr_status ubr_occluded_batch(ubr_context* ctx, const ubr_scene* scene,
                              const float* segs, uint64_t n, float eps,
                              uint8_t* out, int32_t memory);

/* Filtered segment occlusion for the stroke-edge pass's visibility rays:
 * EmbreeRenderer::occluded with its argument filter (embree_renderer.cpp:
 * 76-133, 294-357).  Same trimmed open segment as ubr_occluded_batch, but a
 * candidate hit is not an occluder when it lies on one of segment i's own
 * mesh faces exclude_faces[exclude_offsets[i] .. exclude_offsets[i+1])
 * (base-triangle ids, compared modulo the base triangle count of an instanced
 * mesh), when the ray meets its face at |cos| <= graze_cos_eps, or when the
 * face's plane passes within coplanar_eps of the segment start (<= 0 disables
 * either test).  exclude_offsets (n + 1 entries, starting at 0) and
 * exclude_faces may both be NULL.  All arrays in the memory space `memory`.
 * Traversal overflow: UBR_TRAVERSAL_LIMIT, as ubr_occluded_batch. */
ubr_status ubr_occluded_filtered_batch(ubr_context* ctx, const ubr_scene* scene,
                                       const float* segs, uint64_t n, float eps,
                                       float graze_cos_eps, float coplanar_eps,
                                       const uint32_t* exclude_offsets,
                                       const int32_t* exclude_faces,
                                       uint8_t* out, int32_t memory);

/* Segment occlusion that allocates nothing.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory when
 * they query -- a host with its own strict GPU memory budget, a plugin
 * sandbox whose host owns every device allocation, or a per-frame loop that
 * must not risk an allocation failure or the synchronisation that
 * cudaMalloc/cudaFree can cause.  Same answers and status as
 * ubr_occluded_batch on HOST buffers (segs = 6*n floats, out = n bytes),
 * staged through one fixed device array compiled into the library (about
 * 12.5 MiB, held by every GPU that loads the library until the process
 * exits).
 *   - n may be at most 524,288; larger n returns UBR_INVALID_ARGUMENT.
 *   - The first call on a context resolves the array's device address on
 *     the context's device; make that first call before any stream capture.
 *   - Every call on a device shares the one array: calls whose GPU work
 *     overlaps (other threads, other contexts on the same device) race. */
ubr_status ubr_occluded_batch_noalloc(ubr_context* ctx, const ubr_scene* scene,
                                      const float* segs, uint64_t n, float eps,
                                      uint8_t* out);

#ifdef __cplusplus
}
#endif

#endif /* UBR_H_ */
