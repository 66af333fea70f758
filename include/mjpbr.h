/*
 * mjpbr.h — C ABI of the GB300-native batched PBR render path (libmjpbr.so).
 *
 * The library renders thousands of MuJoCo worlds per launch on one sm_103a GPU. Every entry
 * point takes a plain-old-data scene descriptor (MjpbrScene) that holds device pointers to the
 * model, data and render-context arrays plus the render settings, and a CUDA stream
 * (cudaStream_t passed as void*). Entry points return an int status (MJPBR_OK = 0); on failure
 * mjpbr_last_error() returns a message for the calling thread. No C++ exception crosses the ABI,
 * no entry point allocates device memory unless its comment says so, and none synchronises the
 * stream, so calls can be captured into a CUDA graph.
 *
 * Arrays follow MuJoCo Warp's batching convention: a table whose leading dimension is a batch
 * dimension (an mjpbr_f32b / mjpbr_i32b) is indexed with worldid % nbatch, so nbatch is 1 (one
 * value shared by every world) or nworld (one per world). Matrices are row-major 3x3 (MuJoCo's
 * xmat). Vectors are packed float triples.
 *
 * Reference interfaces replaced (julien-blanchon/mujoco_warp_pbr, paths inside that project):
 *   mjpbr_refit_bvh        mujoco_warp.refit_bvh(m, d, rc.base)          (called at tests/conftest.py:44,
 *                                                                          benchmarks/bench.py:184-186)
 *   mjpbr_render           mujoco_warp_pbr.render(m, d, rc, seed)        (mujoco_warp_pbr/_src/render.py:431-460)
 *   mjpbr_get_rgb          mujoco_warp_pbr.get_rgb(rc, cam, out)         (mujoco_warp_pbr/_src/output.py:34-38)
 *   mjpbr_get_depth        mujoco_warp_pbr.get_depth(rc, cam, s, out)    (mujoco_warp_pbr/_src/output.py:41-45)
 *   mjpbr_get_segmentation mujoco_warp_pbr.get_segmentation(...)         (mujoco_warp_pbr/_src/output.py:48-52)
 *   mjpbr_get_image        get_hdr / get_albedo / get_normal             (mujoco_warp_pbr/_src/output.py:55-152)
 *   mjpbr_dfg_lut          ibl.dfg_lut_array                              (mujoco_warp_pbr/_src/ibl.py:62-101)
 *   mjpbr_build_mips       mip chains of texture.upload_textures / EnvironmentMap
 *                                                                         (mujoco_warp_pbr/_src/texture.py:63-101,
 *                                                                          mujoco_warp_pbr/_src/envmap.py:330-340)
 *   mjpbr_prefilter_env    envmap._prefilter                              (mujoco_warp_pbr/_src/envmap.py:171-221)
 *   mjpbr_env_sh9          envmap._sh9_irradiance                         (mujoco_warp_pbr/_src/envmap.py:224-249)
 *   mjpbr_env_sampling_tables  envmap.sampling_distribution               (mujoco_warp_pbr/_src/envmap.py:409-430)
 *   mjpbr_denoise_atrous   denoise.denoise                                (mujoco_warp_pbr/_src/denoise.py:214-248)
 *   mjpbr_build_scene_bvh  scene BVH build of mujoco_warp.create_render_context (third party; called at
 *                                                                          mujoco_warp_pbr/_src/io.py:511-528)
 *   mjpbr_build_mesh_bvh   per-mesh BVH build (warp.Mesh, mujoco_warp_pbr/_src/io.py:164-179,198-203)
 *   mjpbr_build_mesh_bvh_device  GPU mesh BVH builds of warp.Mesh (mujoco_warp_pbr/_src/io.py:164-179)
 *   mjpbr_newton_sync_poses   newton_pbr ScenePoses.sync                  (newton-pbr/newton_pbr/_render.py:31-131)
 *   mjpbr_newton_images       newton_pbr SensorPbrCamera output copy      (newton-pbr/newton_pbr/sensor.py:45-86,247-265)
 */
#ifndef MJPBR_H_
#define MJPBR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MJPBR_ABI_VERSION 3

/* Most rendering cameras of one context (the per-camera tables below are inline). */
#define MJPBR_MAX_RENDER 16
/* MuJoCo's texture roles (mjNTEXROLE). */
#define MJPBR_NTEXROLE 10
/* Levels of a mip chain (16384² textures at most). */
#define MJPBR_MAX_MIPS 15

enum MjpbrStatus {
  MJPBR_OK = 0,
  MJPBR_ERR_ARG = 1,         /* invalid argument (message in mjpbr_last_error) */
  MJPBR_ERR_CUDA = 2,        /* a CUDA call failed */
  MJPBR_ERR_DEVICE = 3,      /* a kernel reported an error through the scene's error word */
  MJPBR_ERR_UNSUPPORTED = 4  /* feature not built into this library */
};

/* MuJoCo enums used by the arrays (mjtGeom, mjtLightType, mjtProjection, mjtTextureRole). */
enum MjpbrGeomType {
  MJPBR_GEOM_PLANE = 0, MJPBR_GEOM_HFIELD = 1, MJPBR_GEOM_SPHERE = 2, MJPBR_GEOM_CAPSULE = 3,
  MJPBR_GEOM_ELLIPSOID = 4, MJPBR_GEOM_CYLINDER = 5, MJPBR_GEOM_BOX = 6, MJPBR_GEOM_MESH = 7,
  MJPBR_GEOM_SDF = 8
};
enum MjpbrLightType { MJPBR_LIGHT_SPOT = 0, MJPBR_LIGHT_DIRECTIONAL = 1, MJPBR_LIGHT_POINT = 2, MJPBR_LIGHT_IMAGE = 3 };
enum MjpbrProjection { MJPBR_PROJ_PERSPECTIVE = 0, MJPBR_PROJ_ORTHOGRAPHIC = 1 };
enum MjpbrTexRole {
  MJPBR_ROLE_USER = 0, MJPBR_ROLE_RGB = 1, MJPBR_ROLE_OCCLUSION = 2, MJPBR_ROLE_ROUGHNESS = 3,
  MJPBR_ROLE_METALLIC = 4, MJPBR_ROLE_NORMAL = 5, MJPBR_ROLE_OPACITY = 6, MJPBR_ROLE_EMISSIVE = 7,
  MJPBR_ROLE_RGBA = 8, MJPBR_ROLE_ORM = 9
};
/* Tone mappers, light models, tiers and thread orders (mujoco_warp_pbr/_src/types.py:29-103). */
enum MjpbrToneMapper { MJPBR_TONE_PBR_NEUTRAL = 0, MJPBR_TONE_ACES = 1, MJPBR_TONE_CLAMP = 2 };
enum MjpbrLightModel { MJPBR_LIGHT_MODEL_PHYSICAL = 0, MJPBR_LIGHT_MODEL_MUJOCO = 1 };
enum MjpbrTier { MJPBR_TIER_REALTIME = 0, MJPBR_TIER_PATH = 1 };
enum MjpbrRenderOrder { MJPBR_ORDER_ROW = 0, MJPBR_ORDER_TILED = 1, MJPBR_ORDER_WORLD = 2 };
/* Schedules. Real-time tier: one CTA per (camera tile, world); a persistent launch whose warps
 * pull work items (settings.queue_item pixels of one camera image of one world) from a device
 * counter (scene.work_counter[1]); or a staged wavefront (primary rays, surfaces, mirror rays,
 * shadow rays and shading as separate kernels over compacted ray queues, chunks of worlds at a
 * time in scene.wave_scratch; translucent layers render with the grid schedule). Path tier: GRID
 * and QUEUE select the persistent path kernel, WAVEFRONT the staged bounce loop (extend, shade,
 * shadow, next-event kernels over compacted path queues in scene.wave_scratch). Every schedule of
 * a tier renders identical images. */
enum MjpbrSchedule { MJPBR_SCHEDULE_GRID = 0, MJPBR_SCHEDULE_QUEUE = 1, MJPBR_SCHEDULE_WAVEFRONT = 2 };
/* Texel formats of MjpbrTexture. */
enum MjpbrTexFormat { MJPBR_TEX_RGBA8 = 0, MJPBR_TEX_RGBA16F = 1 };

/* A batched table: nbatch rows (1 or nworld), row r used by worlds with worldid % nbatch == r. */
typedef struct mjpbr_f32b { const float* ptr; int32_t nbatch; int32_t pad_; } mjpbr_f32b;
typedef struct mjpbr_i32b { const int32_t* ptr; int32_t nbatch; int32_t pad_; } mjpbr_i32b;

/* One 3x3 convolution layer of the learned denoiser (stride 1, zero padding), NHWC BF16
 * activations, FP32 accumulation on the tensor cores. Input channels are `in` (c_in of them)
 * followed, when c_in2 > 0, by `in2`: (nimg, height, width, c_in2) when in2_full, else
 * (nimg, height / 2, width / 2, c_in2) upsampled x2 (nearest) while staging: the U-Net's skip
 * concatenation (mjpbr_upsample2_bf16 makes the full-resolution copy). weight: (c_out, 9, c_in + c_in2), taps row-major (dy, dx).
 * Epilogue: + bias, ReLU if relu, zeroed where mask <= 0 if mask (a ReLU derivative), stored as
 * BF16 to out and/or FP32 to out_f32. Channel counts are multiples of 16, c_out <= 256; width is
 * a power-of-two multiple of 16 up to 128 or a multiple of 128, height * width a multiple of 128
 * (128 / min(width, 128) rows per 128-pixel tile). */
typedef struct MjpbrConv {
  const uint16_t* in;
  const uint16_t* in2;
  const uint16_t* weight;
  const float* bias;
  uint16_t* out;
  float* out_f32;
  const uint16_t* mask;
  int32_t* error_word;
  int32_t nimg, height, width, c_in, c_in2, c_out;
  int32_t relu;
  int32_t in2_full; /* 1: in2 has the output resolution; 0: half of it, upsampled x2 */
} MjpbrConv;

/* Weights of the learned denoiser's U-Net (mujoco_warp_pbr_gb300.kpcn), layers in the order e0a
 * e0b e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b d0a d0b head: BF16 weight (c_out, 9, c_in + c_in2)
 * as raw 16-bit values and FP32 bias (c_out), device pointers. */
#define MJPBR_KPCN_LAYERS 15
typedef struct MjpbrKpcnWeights {
  const uint16_t* weight[MJPBR_KPCN_LAYERS];
  const float* bias[MJPBR_KPCN_LAYERS];
} MjpbrKpcnWeights;

/* Weight and bias gradients of a 3x3 convolution layer (same tensors and constraints as
 * MjpbrConv): grad_weight (c_out, 9, c_in + c_in2) += sum over pixels of grad_out (x) the shifted
 * input, grad_bias (c_out) += sum of grad_out; FP32, accumulated into the existing values. */
typedef struct MjpbrConvGrad {
  const uint16_t* in;
  const uint16_t* in2;
  const uint16_t* grad_out;
  float* grad_weight;
  float* grad_bias;
  int32_t* error_word;
  int32_t nimg, height, width, c_in, c_in2, c_out;
  int32_t tiles_per_cta; /* 128-pixel tiles each CTA accumulates before its atomic reduction (0: 64) */
  int32_t in2_full;      /* 1: in2 has the output resolution; 0: half of it, upsampled x2 */
} MjpbrConvGrad;

/* One mipmapped 2D texture inside MjpbrScene.tex_data (RGBA, row-major levels). */
typedef struct MjpbrTexture {
  int32_t format;   /* MjpbrTexFormat */
  int32_t width;    /* level 0 */
  int32_t height;
  int32_t nlevel;
  int64_t level_offset[MJPBR_MAX_MIPS]; /* byte offset of each level in tex_data */
  int32_t pad_[2];
} MjpbrTexture;

/* Render settings (mujoco_warp_pbr/_src/kernel_inputs.py:47-116 plus the path-tier and denoiser
 * parameters of PbrRenderContext, mujoco_warp_pbr/_src/types.py:123-322). Booleans are 0 / 1. */
typedef struct MjpbrSettings {
  int32_t tier;
  int32_t render_order;
  int32_t samples_per_axis;  /* real-time supersampling per axis (N x N rays) */
  int32_t tone_mapper;
  int32_t render_hdr;
  int32_t render_guides;
  int32_t light_model;
  int32_t use_shadows;
  int32_t shadow_samples;    /* > 1: soft shadows from bulbradius */
  int32_t headlight_active;
  int32_t has_env;           /* an environment map lights the scene */
  int32_t env_background;    /* missed rays show the environment map */
  int32_t textures;          /* any texture role is sampled */
  int32_t base_color_map;
  int32_t normal_map;
  int32_t orm_map;
  int32_t emissive_map;
  int32_t opacity_map;
  int32_t specular_aa;
  int32_t vertex_normals;
  int32_t has_reflection;    /* MuJoCo reflectance adds a mirror ray */
  int32_t has_transparency;
  int32_t max_layers;
  int32_t cull_backfaces;
  int32_t path_samples;      /* path tier: samples per pixel */
  int32_t max_depth;         /* path tier: bounces */
  int32_t rr_depth;          /* path tier: Russian roulette start */
  int32_t denoise;           /* path tier: write denoiser features instead of RGB */
  int32_t schedule;          /* real-time tier: MjpbrSchedule */
  int32_t queue_item;        /* queue schedule: pixels per work item (32, 64 or 128) */
  int32_t stack_depth;       /* traversal stack entries per ray: 0 (32) or 8..32; the scene BVH's
                                inner levels + the deepest mesh BVH's + 1 always suffice */
  float znear;
  float zfar;                /* <= 0: unbounded */
  float shadow_light_fraction;
  float headlight_intensity; /* illuminance times exposure (physical model) */
  float headlight_diffuse[3];
  float headlight_specular[3];
  float background[3];       /* linear display colour of missed rays */
  float inv_texel_angle;     /* inverse angular size of a radiance texel (env background LOD) */
  float denoise_sigma_color;
  float denoise_sigma_normal;
  float denoise_sigma_depth;
  float denoise_sigma_albedo;
} MjpbrSettings;

/* Everything one render reads and writes. Device pointers unless stated otherwise. Pointers of
 * features the settings switch off may be NULL. */
typedef struct MjpbrScene {
  int32_t abi_version;       /* MJPBR_ABI_VERSION */
  int32_t nworld;            /* 1 .. 2^24 */
  int32_t ngeom;
  int32_t nmat;
  int32_t nlight;
  int32_t ncam;              /* model cameras */
  int32_t nmesh;
  int32_t ntex;
  int32_t nenv;

  /* ---- Model (mujoco_warp.Model fields) ---- */
  const int32_t* geom_type;        /* (ngeom,) MjpbrGeomType */
  mjpbr_i32b geom_dataid;          /* (*, ngeom) mesh id of mesh geoms, height-field id of height fields */
  mjpbr_i32b geom_matid;           /* (*, ngeom) */
  mjpbr_f32b geom_size;            /* (*, ngeom, 3) */
  mjpbr_f32b geom_rgba;            /* (*, ngeom, 4) */
  mjpbr_f32b mat_rgba;             /* (*, nmat, 4) */
  mjpbr_f32b mat_emission;         /* (*, nmat) */
  mjpbr_i32b mat_texid;            /* (*, nmat, MJPBR_NTEXROLE) */
  mjpbr_f32b mat_texrepeat;        /* (*, nmat, 2) */
  mjpbr_i32b mat_texuniform;       /* (*, nmat) */
  mjpbr_i32b light_type;           /* (*, nlight) */
  mjpbr_i32b light_castshadow;     /* (*, nlight) */
  mjpbr_i32b light_active;         /* (*, nlight) */
  mjpbr_f32b light_attenuation;    /* (*, nlight, 3) */
  mjpbr_f32b light_cutoff;         /* (*, nlight) degrees */
  mjpbr_f32b light_exponent;       /* (*, nlight) */
  mjpbr_f32b light_diffuse;        /* (*, nlight, 3) */
  mjpbr_f32b light_specular;       /* (*, nlight, 3) */
  const int32_t* cam_projection;   /* (ncam,) MjpbrProjection */
  mjpbr_f32b cam_fovy;             /* (*, ncam) degrees (orthographic: frustum height) */
  const float* cam_sensorsize;     /* (ncam, 2); 0: use fovy */
  mjpbr_f32b cam_intrinsic;        /* (*, ncam, 4) fx, fy, cx, cy in sensor units */
  const int32_t* mesh_vertadr;     /* (nmesh,) */
  const int32_t* mesh_faceadr;     /* (nmesh,) */
  const int32_t* mesh_normaladr;   /* (nmesh,) */
  const int32_t* mesh_texcoordadr; /* (nmesh,) first texcoord, -1: no UVs */
  const float* mesh_vert;          /* (nvert, 3) mesh frame */
  const int32_t* mesh_face;        /* (nface, 3) */
  const float* mesh_normal;        /* (nnormal, 3) */
  const int32_t* mesh_facenormal;  /* (nface, 3) */
  const float* mesh_texcoord;      /* (ntexcoord, 2) */
  const int32_t* mesh_facetexcoord;/* (nface, 3) */

  /* ---- Data (mujoco_warp.Data fields) ---- */
  const float* geom_xpos;          /* (nworld, ngeom, 3) */
  const float* geom_xmat;          /* (nworld, ngeom, 9) */
  const float* cam_xpos;           /* (nworld, ncam, 3) */
  const float* cam_xmat;           /* (nworld, ncam, 9) */
  const float* light_xpos;         /* (nworld, nlight, 3) */
  const float* light_xdir;         /* (nworld, nlight, 3) */

  /* ---- Render context: cameras and outputs (mujoco_warp.RenderContext) ---- */
  int32_t nrender;                               /* rendering cameras */
  int32_t total_rays;                            /* sum of W*H over rendering cameras */
  int32_t cam_id_map[MJPBR_MAX_RENDER];          /* rendering camera -> model camera */
  int32_t cam_res[MJPBR_MAX_RENDER][2];          /* width, height */
  int32_t render_rgb[MJPBR_MAX_RENDER];
  int32_t render_depth[MJPBR_MAX_RENDER];
  int32_t render_seg[MJPBR_MAX_RENDER];
  int32_t ray_adr[MJPBR_MAX_RENDER];             /* first pixel of each camera among total_rays */
  int32_t rgb_adr[MJPBR_MAX_RENDER];             /* -1: camera renders no RGB */
  int32_t depth_adr[MJPBR_MAX_RENDER];
  int32_t seg_adr[MJPBR_MAX_RENDER];
  int32_t rgb_stride;                            /* pixels per world of rgb_data, hdr, guides */
  int32_t depth_stride;
  int32_t seg_stride;
  int32_t pad0_;
  uint32_t* rgb_data;                            /* (nworld, rgb_stride) RGBA8, R in the low byte */
  float* depth_data;                             /* (nworld, depth_stride) */
  int32_t* seg_data;                             /* (nworld, seg_stride, 2) (id, type) */
  float* hdr_data;                               /* (nworld, rgb_stride, 3) linear, pre-exposure */
  float* guide_albedo;                           /* (nworld, rgb_stride, 3) */
  float* guide_normal;                           /* (nworld, rgb_stride, 3) */

  /* ---- Render context: per-world material, light and exposure tables ---- */
  mjpbr_f32b geom_metallic;        /* (*, ngeom) */
  mjpbr_f32b geom_roughness;       /* (*, ngeom) perceptual */
  mjpbr_f32b geom_reflectance;     /* (*, ngeom) dielectric F0 = 0.16 r^2 */
  mjpbr_f32b mat_reflectance;      /* (*, nmat) MuJoCo mirror reflectance */
  mjpbr_f32b light_intensity;      /* (*, nlight) lux or candela */
  mjpbr_f32b light_range;          /* (*, nlight) */
  mjpbr_f32b light_bulbradius;     /* (*, nlight) */
  mjpbr_f32b exposure;             /* (*) */
  mjpbr_f32b ambient_radiance;     /* (*, 3) */
  mjpbr_i32b env_id;               /* (*) */
  mjpbr_f32b env_intensity;        /* (*) */
  mjpbr_f32b env_yaw;              /* (*) radians */

  /* ---- Scene BVH: one binary tree per world over the enabled geoms ---- */
  int32_t nbvh_geom;               /* enabled geoms (slots) per world */
  int32_t nnode;                   /* inner nodes per world (nbvh_geom - 1, at least 1) */
  const int32_t* enabled_geom_ids; /* (nbvh_geom,) slot -> geom id */
  mjpbr_i32b tlas_child;           /* (*, nnode, 2) child refs: >= 0 inner node, < 0 leaf slot ~ref */
  const float* mesh_bounds;        /* (nmesh + nhfield, 6) local AABB of each triangle BVH (lower, upper) */
  float* world_blocks;             /* (nworld, world_block_floats) written by mjpbr_refit_bvh */
  int32_t world_block_floats;      /* per-world block size in floats (a multiple of 4) */
  int32_t nhfield;                 /* height fields; their triangle BVHs follow the meshes' */

  /* ---- Triangle BVHs, shared by every world: one per mesh (index = mesh id), then one per
   *      height field (index = nmesh + height-field id, its grid triangulated as a closed prism) */
  const float* blas_nodes;         /* (nblasnode, 16) child-bounds nodes, see mjpbr_build_mesh_bvh */
  const float* blas_tris;          /* (nblastri, 12) v0, v1, v2 (xyz + face id bits in w of v0) */
  const int32_t* blas_root;        /* (nmesh + nhfield,) first node of each BVH */
  const int32_t* blas_tri_base;    /* (nmesh + nhfield,) first triangle of each BVH */

  /* ---- Textures ---- */
  const MjpbrTexture* textures;    /* (ntex,) device copy */
  const uint8_t* tex_data;

  /* ---- Environment maps (image-based lighting) ---- */
  const float* dfg_lut;            /* (dfg_size, dfg_size, 2) rows: perceptual roughness, cols: NoV */
  int32_t dfg_size;
  int32_t prefilter_levels;        /* depth of the GGX-prefiltered stack */
  int32_t prefilter_width;
  int32_t prefilter_height;
  const uint16_t* env_prefiltered; /* (nenv, levels, height, width, 4) float16 */
  const MjpbrTexture* env_radiance;/* (nenv,) mipmapped radiance, formats RGBA16F, into env_data */
  const uint8_t* env_data;
  const float* env_sh;             /* (nenv, 9, 3) SH9 Lambertian radiance */
  int32_t cdf_width;
  int32_t cdf_height;
  const float* env_prob;           /* (nenv, h, w) */
  const float* env_marginal;       /* (nenv, h + 1) */
  const float* env_conditional;    /* (nenv, h, w + 1) */

  /* ---- Per-pixel camera rays (set_camera_rays), NULL for pinhole cameras ---- */
  const float* ray_origin;         /* (total_rays, 3) camera frame */
  const float* ray_direction;      /* (total_rays, 3) camera frame, zero: no ray */
  int32_t bundle_res[MJPBR_MAX_RENDER][2];

  /* ---- Path-tier denoiser features (nworld, rgb_stride) ---- */
  uint32_t* aov_guide;             /* (.., 4) first-hit guide of the filter: words 0-2 hold the
                                      normal xyz then the albedo xyz as IEEE half floats (low half
                                      first), word 3 the depth (float bits) */
  float* aov_emission;             /* (.., 3) exposed first-hit emission, kept out of filtering */
  float* denoise_buffers[2];       /* (.., 4) demodulated radiance and its variance; the path
                                      tracer writes [0], the filter passes ping-pong */
  int32_t denoise_iterations;
  int32_t pad2_;

  /* ---- Status and scratch ---- */
  int32_t* error_word;             /* device int32, kernels OR error bits into it (may be NULL) */
  int32_t* work_counter;           /* device int32[4] scratch of the persistent kernels' work queues
                                      (the library zeroes it on the stream before each use) */
  void* wave_scratch;              /* wavefront schedule: device scratch, 256-byte aligned (NULL otherwise) */
  int64_t wave_scratch_bytes;      /* its size; mjpbr_wave_scratch_bytes gives the size for a chunk of worlds */

  MjpbrSettings settings;
} MjpbrScene;

/* ABI version this library was built with (MJPBR_ABI_VERSION). */
int mjpbr_abi_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* mjpbr_last_error(void);

/* Layout check for bindings written in other languages: out[0..7] = sizeof(MjpbrScene),
 * sizeof(MjpbrSettings), sizeof(MjpbrTexture), offsetof(MjpbrScene, nrender),
 * offsetof(MjpbrScene, world_blocks), offsetof(MjpbrScene, env_prefiltered),
 * offsetof(MjpbrScene, error_word), offsetof(MjpbrScene, settings). */
void mjpbr_struct_layout(int64_t out[8]);

/* Size in floats of one world's block for a scene with these counts (used to size world_blocks). */
int32_t mjpbr_world_block_floats(int32_t nbvh_geom, int32_t nnode, int32_t nlight, int32_t nrender);

/* Bytes of wave_scratch the wavefront schedule needs to render `worlds` worlds per chunk of
 * this scene (more scratch, fewer chunks; the whole frame in one chunk with worlds = nworld),
 * or -1. Host only; reads the scene's counts and settings, no device pointer. New with the
 * wavefront schedule (the reference renders every world in one megakernel launch). */
int64_t mjpbr_wave_scratch_bytes(const MjpbrScene* scene, int32_t worlds);

/* Stage profile of the wavefront schedule, for tools: after mjpbr_wave_profile_begin, every
 * wavefront render issued from this host thread records CUDA events (the library's own, reused) on
 * the render stream at each stage boundary of each chunk of worlds; mjpbr_wave_profile_end waits
 * for the last one, writes the milliseconds of the primary, surface, mirror, mirror-surface,
 * shadow and resolve stages summed over the chunks into stage_ms[6] and the number of chunks into
 * *chunks, and stops recording. Not for use inside a stream capture. No counterpart in the
 * reference (its megakernel is a single launch). */
int mjpbr_wave_profile_begin(void);
int mjpbr_wave_profile_end(double* stage_ms, int32_t* chunks);

/* Per-geom world AABBs from the current poses, bottom-up refit of every world's scene BVH, and the
 * per-world blocks (geom, light, camera records and BVH nodes) the render kernels stage into
 * shared memory. Replaces mujoco_warp.refit_bvh(m, d, rc.base). Launches one kernel. */
int mjpbr_refit_bvh(const MjpbrScene* scene, void* stream);

/* Renders the frame into the output buffers (real-time or path-traced tier per settings.tier;
 * with settings.denoise the path tier writes features and the caller runs mjpbr_denoise_atrous).
 * Replaces mujoco_warp_pbr.render (mujoco_warp_pbr/_src/render.py:431-460). Call
 * mjpbr_refit_bvh first whenever geometry or cameras moved. */
int mjpbr_render(const MjpbrScene* scene, uint32_t seed, void* stream);

/* BF16 tensor-core GEMM: d (m x n, FP32, row-major) = a (m x k, BF16 bits, row-major) times the
 * transpose of b (n x k, BF16 bits, row-major), FP32 accumulation. m a multiple of 128, n a
 * multiple of 16 in [16, 256], k a multiple of 16; 16-byte aligned device pointers. A bounded
 * wait that gives up ORs bit 4 into *error_word (may be NULL). Building block of the learned
 * denoiser; no counterpart in the reference. */
int mjpbr_gemm_bf16(const uint16_t* a, const uint16_t* b, float* d, int32_t m, int32_t n, int32_t k, int32_t* error_word,
                    void* stream);

/* Forward 3x3 convolution (see MjpbrConv); also the input-gradient pass with the flipped,
 * transposed weights. No counterpart in the reference (its denoiser is the a-trous filter). */
int mjpbr_conv3x3_bf16(const MjpbrConv* conv, void* stream);

/* Bytes of the workspace mjpbr_denoise_learned needs for chunks of nimg worlds of a camera of
 * width x height (-1: a size the network's tiles do not cover). */
int64_t mjpbr_kpcn_workspace_bytes(int32_t nimg, int32_t height, int32_t width);

/* The learned denoiser on a path-traced frame rendered with denoising (settings.denoise, the
 * render's denoise_buffers[0] and aov_guide): per RGB camera, chunk worlds at a time, the network
 * input, the U-Net, the per-pixel 5 x 5 kernels into denoise_buffers[1], then the a-trous filter's
 * finish pass without filtering into the outputs. The same launches as kpcn.KPCN.denoise; no
 * counterpart in the reference (its denoiser is the a-trous filter, mjpbr_denoise_atrous). */
int mjpbr_denoise_learned(const MjpbrScene* scene, const MjpbrKpcnWeights* weights, void* workspace, int64_t workspace_bytes,
                          int32_t chunk, void* stream);

/* Weight / bias gradients of a 3x3 convolution (see MjpbrConvGrad), on the tensor cores. */
int mjpbr_conv3x3_wgrad_bf16(const MjpbrConvGrad* grad, void* stream);

/* ---- Learned denoiser building blocks (no counterpart in the reference). NHWC layouts, one
 * image per world of camera `cam`; BF16 as raw 16-bit values. ---- */
/* Network input (nw, H, W, 16) BF16 of worlds [w0, w0 + nw): log(1 + demodulated radiance),
 * albedo, normal, log(1 + depth), log(1 + standard deviation of the mean's luminance), zeros;
 * from denoise_buffers[0] and aov_guide written by a denoising render. */
int mjpbr_kpcn_features(const MjpbrScene* scene, int32_t cam, int32_t w0, int32_t nw, uint16_t* x0, void* stream);
/* Demodulated training target (nworld, H, W, 4) FP32 from the FP64 sum of converged HDR frames
 * (laid out like hdr_data) times inv_n, with the denoising render's albedo and emission. */
int mjpbr_kpcn_target(const MjpbrScene* scene, int32_t cam, const double* hdr_sum, double inv_n, float* target, void* stream);
/* acc[i] += src[i] in FP64. */
int mjpbr_accumulate_f64(const float* src, double* acc, int64_t n, void* stream);
/* 2 x 2 average pooling of BF16 (nimg, h, w, c). */
int mjpbr_avgpool2_bf16(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, void* stream);
/* x2 nearest upsampling of BF16 (nimg, h, w, c) to (nimg, 2 h, 2 w, c); c a multiple of 8. */
int mjpbr_upsample2_bf16(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, void* stream);
/* Softmax of 25 of the 32 FP32 logits per pixel, the 5 x 5 kernel applied to the radiance (float4
 * records); weights (nimg, h, w, 25) may be NULL (inference); out (nimg, h, w, 4), w = 0. */
int mjpbr_kpcn_apply(const float* logits, const float* radiance, float* weights, float* out, int32_t nimg, int32_t h, int32_t w,
                     void* stream);
/* Relative L1 (|d| / sqrt(t^2 + 0.01)) and relative-MSE loss of out against target (float4
 * records): gradient, and the two sums
 * added to sums[0..1]. With scale and offset (float4 records, see mjpbr_kpcn_remod; may be NULL)
 * both are first mapped to HDR as offset + x * scale. */
int mjpbr_kpcn_loss(const float* out, const float* target, const float* scale, const float* offset, float* grad, float* sums,
                    int64_t npix, float w_l1, float w_rel, void* stream);
/* The per-pixel HDR mapping of the demodulated radiance of camera `cam` (nworld, H, W, 4) each:
 * scale = max(albedo, 0.01) / exposure, offset = exposed first-hit emission / exposure. */
int mjpbr_kpcn_remod(const MjpbrScene* scene, int32_t cam, float* scale, float* offset, void* stream);
/* Backward of mjpbr_kpcn_apply: BF16 logit gradients (nimg, h, w, 32). */
int mjpbr_kpcn_apply_grad(const float* grad, const float* weights, const float* radiance, uint16_t* grad_logits, int32_t nimg,
                          int32_t h, int32_t w, void* stream);
/* Gradient of a skip concatenation (FP32 (nimg, h, w, c1 + c2)): skip part to dskip (FP32), the
 * upsampled part pooled (sum of 2 x 2) and masked by low > 0 into dlow (BF16, half resolution). */
int mjpbr_split_concat_grad(const float* dcat, const uint16_t* low, float* dskip, uint16_t* dlow, int32_t nimg, int32_t h, int32_t w,
                            int32_t c1, int32_t c2, void* stream);
/* dact = (dskip + average-pool gradient of dpool) masked by act > 0 (dskip may be NULL). */
int mjpbr_unpool_add_grad(const float* dskip, const float* dpool, const uint16_t* act, uint16_t* dact, int32_t nimg, int32_t h,
                          int32_t w, int32_t c, void* stream);
/* Adam step on FP32 parameters (gradient zeroed); refreshes the BF16 copy and, if flip, the
 * (c_in, 9, c_out) tap-reversed copy of a convolution weight. */
int mjpbr_adam(float* param, float* grad, float* m, float* v, uint16_t* copy, uint16_t* flip, int64_t n, int32_t cout, int32_t cin,
               float lr, float beta1, float beta2, float eps, int32_t step, void* stream);

/* mjpbr_refit_bvh + mjpbr_render in one call that allocates nothing and takes no scratch from the
 * caller: the per-world blocks and the path tracer's work counter live in static device memory of
 * the library (scene->world_blocks, scene->work_counter and scene->wave_scratch are ignored; the
 * wavefront schedule renders as the grid schedule / the persistent path kernel, with the same images). For hosts that cannot
 * give the library device memory after start-up (a fixed device-memory arena, a plugin host that
 * owns every allocation). Limit: nworld * world_block_floats <= 4,194,304 (16 MiB), else
 * MJPBR_ERR_ARG. Calls overlapping in time share the static memory and race. The memory belongs
 * to the current device: a stream of another device is rejected with MJPBR_ERR_ARG. The first
 * call on a device (and the first after its context was re-created) looks the memory up; make it
 * before any stream capture. No counterpart in the reference. */
int mjpbr_refit_render_static(const MjpbrScene* scene, uint32_t seed, void* stream);

/* Display RGB in [0, 1] of rendering camera `cam` into out (nworld_out, H, W, 3) float32.
 * mujoco_warp_pbr/_src/output.py:34-38. */
int mjpbr_get_rgb(const MjpbrScene* scene, int32_t cam, float* out, int32_t nworld_out, void* stream);

/* Planar depth / depth_scale clamped to [0, 1] into out (nworld_out, H, W) float32.
 * mujoco_warp_pbr/_src/output.py:41-45. */
int mjpbr_get_depth(const MjpbrScene* scene, int32_t cam, float depth_scale, float* out, int32_t nworld_out,
                    void* stream);

/* (object id, object type) per pixel into out (nworld_out, H, W, 2) int32; background (-1, -1).
 * mujoco_warp_pbr/_src/output.py:48-52. */
int mjpbr_get_segmentation(const MjpbrScene* scene, int32_t cam, int32_t* out, int32_t nworld_out, void* stream);

/* One camera's image of a per-RGB-pixel vec3 buffer: which = 0 hdr_data, 1 guide_albedo,
 * 2 guide_normal, into out (nworld_out, H, W, 3). mujoco_warp_pbr/_src/output.py:55-152. */
int mjpbr_get_image(const MjpbrScene* scene, int32_t which, int32_t cam, float* out, int32_t nworld_out,
                    void* stream);

/* Newton sensor adapter, pose step: the geom poses (geom_xpos (nworld, ngeom, 3), geom_xmat
 * (nworld, ngeom, 9)) and camera `cam`'s pose (cam_xpos (nworld, ncam, 3), cam_xmat (nworld, ncam, 9))
 * of every render world from a Newton model's transforms. Transforms are Newton's transformf:
 * position, then a unit quaternion (x, y, z, w), 7 floats. Geom g of world w shows shape
 * s = geom_shape[w or 0][g] (geom_shape_rows 1 or nworld): pose = body_q[shape_body[s]] (if >= 0)
 * * shape_transform[s] * geom_offset[g]; world w's camera takes camera_transforms[w] (both look
 * along local -Z with +Y up). A shape index outside [0, nshape) or a body index >= nbody is
 * skipped and ORs 8 into *error_word (device int32). All arrays device memory.
 * newton-pbr/newton_pbr/_render.py:31-77 (the pose kernel) and :96-131 (ScenePoses.sync). */
int mjpbr_newton_sync_poses(const float* body_q, int32_t nbody, const int32_t* shape_body, const float* shape_transform,
                            int32_t nshape, const int32_t* geom_shape, int32_t geom_shape_rows, const float* geom_offset,
                            const float* camera_transforms, int32_t nworld, int32_t ngeom, int32_t ncam, int32_t cam,
                            float* geom_xpos, float* geom_xmat, float* cam_xpos, float* cam_xmat, int32_t* error_word,
                            void* stream);

/* Newton sensor adapter, output step: rendering camera `cam`'s outputs, every world, in Newton's
 * formats, each (nworld, H, W[, 3]) device memory or NULL when not wanted: color packed
 * 0xAABBGGRR; depth the ray distance (planar depth * ray_scale[pixel], ray_scale (H, W)) and
 * forward_depth the planar depth, both -1 where nothing is hit; shape_index the Newton shape
 * geom_shape[w or 0][geom] of a geom hit, else 0xFFFFFFFF; hdr linear radiance before exposure.
 * newton-pbr/newton_pbr/sensor.py:45-86 (_copy_outputs) called at :247-265. */
int mjpbr_newton_images(const MjpbrScene* scene, int32_t cam, const int32_t* geom_shape, int32_t geom_shape_rows,
                        const float* ray_scale, uint32_t* color, float* depth, float* forward_depth, uint32_t* shape_index,
                        float* hdr, void* stream);

/* Split-sum DFG table (size, size, 2) float32 into lut (device), nsample Hammersley samples per
 * texel. mujoco_warp_pbr/_src/ibl.py:62-101. */
int mjpbr_dfg_lut(float* lut, int32_t size, int32_t nsample, void* stream);

/* Box-filters level 0 of a texture (tex: host description, data: device bytes at
 * tex->level_offset) into its further levels
 * (2x2 average per level, odd sizes truncate). The mip chains of texture uploads and environment
 * maps, mujoco_warp_pbr/_src/texture.py:91-99 and mujoco_warp_pbr/_src/envmap.py:330-337. */
int mjpbr_build_mips(const MjpbrTexture* tex, uint8_t* data, void* stream);

/* GGX-prefiltered stack (levels, height, width, 4) float16 of one environment map (radiance: host
 * description of a RGBA16F mipmapped texture in device bytes data), nsample importance samples per texel with filtered importance
 * sampling. mujoco_warp_pbr/_src/envmap.py:171-221. */
int mjpbr_prefilter_env(const MjpbrTexture* radiance, const uint8_t* data, int32_t levels, int32_t height,
                        int32_t width, int32_t nsample, uint16_t* stack, void* stream);

/* SH9 coefficients (9, 3) float32 of the Lambertian radiance of an equirect image (height, width, 3)
 * float32 (device), projected in double precision; rows: device scratch of height * 27 doubles.
 * mujoco_warp_pbr/_src/envmap.py:224-249 (there host NumPy at context creation). */
int mjpbr_env_sh9(const float* image, int32_t height, int32_t width, double* rows, float* sh, void* stream);

/* Importance-sampling tables of an equirect image (height, width, 3) float64 (device, at most 4096
 * rows): cell probabilities prob (height, width), marginal row CDF (height + 1) and conditional
 * column CDFs (height, width + 1), float32, distribution proportional to luminance * sin(theta).
 * mujoco_warp_pbr/_src/envmap.py:409-430 (there host NumPy at context creation). */
int mjpbr_env_sampling_tables(const double* image, int32_t height, int32_t width, float* prob, float* marginal,
                              float* conditional, void* stream);

/* Failure-detection check of the library's bounded device waits (the mbarrier waits of the
 * tensor-core kernels): one CTA whose roles wait on mbarriers that nothing completes, each wait
 * bounded by `polls` (1 .. 2^20); the first to give up raises the CTA's abort flag, which releases
 * the other roles, and kErrWaitTimeout (4) is ORed into *error_word (device int32); each of
 * the three roles adds 1 to *roles_done (device int32) when it returns. The context stays usable.
 * No counterpart in the reference (its kernels have no device waits). */
int mjpbr_wait_probe(uint32_t polls, int32_t* error_word, int32_t* roles_done, void* stream);

/* Edge-avoiding à-trous filter of the path tier's noisy HDR into rgb_data (and hdr_data with
 * render_hdr): demodulation, denoise_iterations 5x5 passes, remodulation and tone mapping.
 * mujoco_warp_pbr/_src/denoise.py:214-248. Uses scene.denoise_buffers as scratch. */
int mjpbr_denoise_atrous(const MjpbrScene* scene, void* stream);

/* Host: number of nodes of a binary BVH over nprim primitives (nprim - 1, at least 1). */
int32_t mjpbr_bvh_node_count(int32_t nprim);

/* Host: SAH-built binary BVH over nprim boxes (lower/upper (nprim, 3) host arrays), one primitive
 * per leaf. child_out (nnode, 2) receives the child refs in the MjpbrScene.tlas_child encoding
 * (>= 0 inner node, < 0 ~slot); children always come after their parent, so a reverse sweep
 * refits bottom-up. Stands in for the scene BVH build of mujoco_warp.create_render_context. */
int mjpbr_build_scene_bvh(const float* lower, const float* upper, int32_t nprim, int32_t* child_out);

/* Host: SAH-built BVH of one triangle mesh (vert (nvert, 3), face (nface, 3) host arrays) with at
 * most leaf_size triangles per leaf. nodes_out (mjpbr_bvh_node_count(nface), 16) floats and
 * tris_out (nface, 12) floats receive the node and triangle records the render kernels read;
 * bounds_out (6) the mesh AABB. Stands in for the warp.Mesh BVH of mujoco_warp's render context.
 * Returns the number of nodes written in *nnode_out. */
int mjpbr_build_mesh_bvh(const float* vert, int32_t nvert, const int32_t* face, int32_t nface, int32_t leaf_size,
                         float* nodes_out, float* tris_out, float* bounds_out, int32_t* nnode_out);

/* Device scratch bytes of mjpbr_build_mesh_bvh_device for nsrc sources of nface faces in all
 * (-1 for nsrc < 1 or nface < nsrc). */
int64_t mjpbr_mesh_bvh_device_scratch_bytes(int32_t nsrc, int32_t nface);

/* Device: linear BVHs (Morton-ordered radix trees, subtrees of at most leaf_size triangles as
 * leaves) of nsrc triangle meshes at once, in the records of mjpbr_build_mesh_bvh. Sources are
 * concatenated: source s has faces [face_base[s], face_base[s + 1]) of face (nface, 3), whose
 * vertex indices are local (< vert_num[s]) to the vertices from vert_base[s] of vert (*, 3);
 * every source needs at least one face. Source s's nodes go to nodes from row node_base[s]
 * (capacity mjpbr_bvh_node_count(its faces)), its triangles to tris rows [face_base[s],
 * face_base[s + 1]) in leaf order (leaf refs are relative to face_base[s]), its AABB to
 * bounds[s] (6), its node count to nnode[s]. All arrays (and scratch) device memory; a face
 * naming a vertex out of range is clamped and ORs 16 into *error_word. Stands in for the GPU
 * mesh BVH builds of Warp (wp.Mesh bvh_constructor "lbvh" / "cubql",
 * mujoco_warp_pbr/_src/io.py:164-179). */
int mjpbr_build_mesh_bvh_device(const float* vert, const int32_t* face, const int32_t* vert_base, const int32_t* vert_num,
                                const int32_t* face_base, const int32_t* node_base, int32_t nsrc, int32_t nface, int32_t leaf_size,
                                float* nodes, float* tris, float* bounds, int32_t* nnode, void* scratch, int64_t scratch_bytes,
                                int32_t* error_word, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MJPBR_H_ */
