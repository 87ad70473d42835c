/*
 * mypbr_gpu.h — the C ABI of the GB300 path-tracing backend.
 *
 * This is the drop-in boundary for mypbr's per-pixel path-tracing loop,
 *   frame camera::render(const hittable& world, const hittable_list& lights,
 *                        int save_every, const pass_callback& on_pass)
 * (include/camera.h:79-105 of the reference). The reference passes a virtual
 * C++ object graph (hittable / material / texture / light_list,
 * include/hittable.h:34-60, include/material.h:22-72, include/texture.h:17-22,
 * include/light_list.h:33-134), which cannot cross a C ABI. Here the same
 * scene travels as plain arrays (mypbr_flat_scene), built on the host from the
 * same .scene / OBJ files by mypbr_scene_load (the counterpart of load_scene,
 * include/scene.h:244), with the BVH already built on the host by the same
 * binned-SAH rules as include/bvh.h:110-205.
 *
 * Everything in the flat scene is FP64 on the host, as the reference stores it
 * (include/vec3.h:11); the device copy made by mypbr_gpu_scene_create is FP32
 * apart from the film accumulators, which stay FP64.
 *
 * Conventions
 *   - every function returns a mypbr_status (0 = MYPBR_OK) unless noted;
 *   - output images are row-major from the top-left pixel, like the reference's
 *     frame (include/camera.h:71-76, include/denoiser.h:11-20), and hold
 *     averages over the samples, not sums;
 *   - buffers passed in are owned by the caller; the library owns device memory
 *     and the handles it returns;
 *   - one render per scene handle at a time; functions are not re-entrant on the
 *     same handle.
 */
#ifndef MYPBR_GPU_H
#define MYPBR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MYPBR_ABI_VERSION 2

/* ------------------------------------------------------------------ status */

typedef enum mypbr_status {
    MYPBR_OK = 0,
    MYPBR_ERR_CUDA = 1,             /* a CUDA call failed (message via mypbr_last_error) */
    MYPBR_ERR_UNSUPPORTED = 2,      /* a scene feature this backend does not implement */
    MYPBR_ERR_QUEUE_OVERFLOW = 3,   /* a device queue ran out of capacity */
    MYPBR_ERR_DEVICE_TIMEOUT = 4,   /* a bounded device wait gave up */
    MYPBR_ERR_INVALID_ARGUMENT = 5, /* null pointer, bad size or bad index */
    MYPBR_ERR_OUT_OF_MEMORY = 6,    /* device or host allocation failed */
    MYPBR_ERR_BAD_SCENE = 7,        /* the scene text or a referenced file is malformed */
    MYPBR_ERR_IO = 8,               /* a file could not be opened or read */
    MYPBR_ERR_NO_DEVICE = 9,        /* no CUDA device is visible */
    MYPBR_ERR_DEVICE_CHECK = 10     /* a device-side bounds check fired (index recorded) */
} mypbr_status;

/* Human-readable name of a status code. Never NULL. */
const char* mypbr_gpu_status_string(int status);

/* The message of the last failure on the calling thread ("" if none). Like the
 * reference's "path:line: message" on std::cerr (include/scene.h:255-258). */
const char* mypbr_last_error(void);

/* ------------------------------------------------------------ flat scene */

/* Primitive kinds, as stored in mypbr_prim_ref.kind and light members. */
enum {
    MYPBR_PRIM_SPHERE = 0,   /* include/sphere.h:23-52 */
    MYPBR_PRIM_QUAD = 1,     /* include/quad.h:30-81 */
    MYPBR_PRIM_TRIANGLE = 2, /* include/mesh.h:47-108 */
    MYPBR_PRIM_MEDIUM = 3,   /* include/medium.h:60-88 */
    MYPBR_PRIM_VOXEL_BLOCK = 4 /* include/voxel.h:193-268 */
};

/* Voxel kinds (include/voxel.h:21): a surface lies where neighbouring cells
 * differ in kind, opaque cells showing faces towards empty and transparent
 * ones, transparent cells towards empty ones only. */
enum { MYPBR_VOXEL_EMPTY = 0, MYPBR_VOXEL_OPAQUE = 1, MYPBR_VOXEL_TRANSPARENT = 2 };

/* One palette entry of a voxel model: the material of that palette index and
 * its kind. A model's palette is 256 consecutive entries. */
typedef struct mypbr_voxel_entry {
    int32_t material;
    int32_t kind;
} mypbr_voxel_entry;

/* A placed voxel model (include/voxel.h:164-268): nx*ny*nz palette indices at
 * `cells` in voxel_cells (x fastest, then y, then z; cell (x, y, z) covers
 * [x, x+1] x [y, y+1] x [z, z+1] in model space), placed in the world by
 * transform `xform` (model -> world). Instances of one model share cells.
 * edge_material >= 0 draws the outlines of the shapes edge_width wide
 * (voxel.h:313-331). */
typedef struct mypbr_voxel_model {
    int32_t nx, ny, nz;
    int32_t xform;
    int64_t cells;
    int32_t palette;       /* first of 256 entries in voxel_palettes */
    int32_t edge_material;
    double edge_width;
} mypbr_voxel_model;

/* A block of a model, cells [lo, hi), walked by a 3D DDA (voxel.h:356-382);
 * blocks are the BVH primitives of voxel models. */
typedef struct mypbr_voxel_block {
    int32_t model;
    int32_t lo[3], hi[3];
    int32_t reserved;
} mypbr_voxel_block;

/* An affine map p -> M p + t with its inverse, as the reference's transform
 * (include/transform.h:72-173). */
typedef struct mypbr_xform {
    double m[3][3];
    double t[3];
    double inv_m[3][3];
    double inv_t[3];
} mypbr_xform;

/* A sphere; a negative radius flips the normal inwards (include/sphere.h:9-16).
 * xform >= 0 places the sphere through that transform: the ray is moved into
 * the sphere's own space, as instance::hit does (include/instance.h:29-41). */
typedef struct mypbr_sphere {
    double center[3];
    double radius;
    int32_t material;
    int32_t xform;
} mypbr_sphere;

/* A parallelogram Q + a u + b v, a, b in [0, 1], in world space (transforms
 * are baked in). normal is the unit outward normal (include/quad.h:11-18 for an
 * untransformed quad; the inverse-transpose image for a transformed one). */
typedef struct mypbr_quad {
    double q[3], u[3], v[3];
    double normal[3];
    int32_t material;
    int32_t reserved;
} mypbr_quad;

/* Triangle flags. */
enum {
    MYPBR_TRI_FLIP_NORMAL = 1, /* geometric normal is -normalize(e1 x e2) (mirroring transform) */
    MYPBR_TRI_ALPHA_MASK = 2   /* the mesh's alpha_mask cuts holes in this triangle (include/mesh.h:23-26) */
};

/* One triangle of a mesh by vertex indices (include/mesh.h:28-44); normal and
 * uv indices are -1 when absent. Positions are in world space. */
typedef struct mypbr_triangle {
    int32_t v[3];
    int32_t n[3];
    int32_t t[3];
    int32_t material;
    int32_t flags;
    int32_t mesh; /* index into mypbr_flat_scene.meshes (-1: none) */
} mypbr_triangle;

/* A mesh = a contiguous range of triangles with one area CDF, used when the
 * mesh is a light (include/mesh.h:175-216). */
typedef struct mypbr_mesh {
    int64_t first_triangle;
    int64_t triangle_count;
    int32_t material;
    /* Image texture whose coverage masks the mesh's triangles that carry
     * MYPBR_TRI_ALPHA_MASK (include/mesh.h:81-86): a ray hits where the
     * coverage is a with probability a. Read only for those triangles. */
    int32_t alpha_mask;
} mypbr_mesh;

/* A homogeneous medium of the given density (collisions per unit length) in
 * a convex boundary (include/medium.h:289-331). shape 0: sphere (a = centre,
 * b[0] = radius); shape 1: box (a = min corner, b = max corner). xform >= 0
 * moves the boundary (the medium keeps world-space distances). */
typedef struct mypbr_medium {
    int32_t shape;
    int32_t xform;
    int32_t material;
    int32_t reserved;
    double density;
    double a[3], b[3];
} mypbr_medium;

/* Objects without a finite bounding box, tested beside the BVH
 * (scene::unbounded, include/scene.h:34-36): the infinite ground
 * (include/plane.h:17-34) and exponential height fog (include/medium.h:347-390). */
enum { MYPBR_UNBOUNDED_GROUND = 0, MYPBR_UNBOUNDED_HEIGHT_FOG = 1 };
typedef struct mypbr_unbounded {
    int32_t kind;
    int32_t material;
    double height;       /* ground: plane y = height; fog: base */
    double density;      /* fog only */
    double scale_height; /* fog only */
} mypbr_unbounded;

/* One node of the host-built BVH, in the reference's depth-first layout
 * (include/bvh.h:93-98): the left child is the next node; interior nodes keep
 * the right child's index in offset; leaves keep the first primitive reference
 * in offset and count > 0. */
typedef struct mypbr_bvh_node {
    double bmin[3], bmax[3];
    int32_t offset;
    int32_t count;
    int32_t axis;
    int32_t reserved;
} mypbr_bvh_node;

/* A BVH leaf entry: which primitive (kind, index into that kind's array). */
typedef struct mypbr_prim_ref {
    int32_t kind;
    int32_t index;
} mypbr_prim_ref;

/* ---------------------------------------------------------- appearance */

enum {
    MYPBR_TEX_SOLID = 0,   /* p[0..2] = colour (include/texture.h:24-36) */
    MYPBR_TEX_CHECKER = 1, /* p[0] = 1/scale, a = even texture, b = odd (texture.h:38-56) */
    MYPBR_TEX_IMAGE = 2,   /* width x height texels at offset (texture.h:67-209) */
    /* Wrappers of texture a (a < this texture's index, chains at most 6 deep): */
    MYPBR_TEX_SCALED = 3,       /* p[0..2] x a (scaled_texture, texture.h:212-225) */
    MYPBR_TEX_CHANNEL = 4,      /* grey p[0] x channel b (0 red, 1 green, 2 blue) of a (texture.h:228-245) */
    MYPBR_TEX_UV_TRANSFORM = 5, /* a at moved (u, v): offset p[0..1], rotation p[2] radians, scale p[3..4]
                                   (KHR_texture_transform, uv_transform_texture, texture.h:248-267) */
    MYPBR_TEX_NORMAL_SCALE = 6  /* encoded normal of a with its tilt times p[0] (texture.h:270-282) */
};
enum {
    MYPBR_TEXF_HDR = 1,    /* texels are RGB float in texels_hdr, else RGBA8 in texels_ldr */
    MYPBR_TEXF_LINEAR = 2, /* 8-bit values are data (k / 255), not sRGB */
    MYPBR_TEXF_REPEAT = 4, /* wrap (u, v) instead of clamping */
    MYPBR_TEXF_GREY_MASK = 8 /* no alpha channel: as a mask, the grey level (red byte) is the coverage */
};
typedef struct mypbr_texture {
    int32_t type;
    int32_t a, b;
    int32_t width, height;
    int32_t flags;
    int64_t offset; /* first texel (ldr: byte offset / 4 per texel; hdr: float offset / 3) */
    double p[6];
} mypbr_texture;

enum {
    MYPBR_MAT_LAMBERTIAN = 0,      /* include/material.h:74-101 */
    MYPBR_MAT_METAL = 1,           /* include/material.h:109-173 */
    MYPBR_MAT_DIELECTRIC = 2,      /* include/material.h:184-264 */
    MYPBR_MAT_THIN_DIELECTRIC = 3, /* include/material.h:683-707 */
    MYPBR_MAT_PRINCIPLED = 4,      /* include/material.h:346-552 */
    MYPBR_MAT_DIFFUSE_LIGHT = 5,   /* include/material.h:568-615 */
    MYPBR_MAT_PHASE = 6            /* include/medium.h:248-274 */
};

/* Material flags. */
enum {
    MYPBR_MATF_MEASURED = 1,   /* metal / principled conductor uses the complex IOR (microfacet.h:98-142) */
    MYPBR_MATF_COAT = 2,       /* principled has a clear coat (material.h:366-371) */
    MYPBR_MATF_COAT_TINT = 4   /* principled coat tint differs from white (material.h:379) */
};

/*
 * A material. Texture slots hold texture indices (-1 = none). Parameter slots
 * by type:
 *   LAMBERTIAN      tex[0] albedo
 *   METAL           p[0..2] albedo (Schlick f0), p[3] roughness (clamped [0,1]),
 *                   p[4..6] eta, p[7..9] k (measured), p[10..12] f_avg
 *   DIELECTRIC      p[0] ior, p[1] roughness, p[2..4] sigma_a
 *   THIN_DIELECTRIC p[0] ior, p[2..4] tint
 *   PRINCIPLED      tex[0] base, tex[1] metallic, tex[2] roughness, tex[3] base normal map,
 *                   tex[4] coat weight, tex[5] coat roughness, tex[6] coat normal map,
 *                   p[0] dielectric f0, p[4..6] eta, p[7..9] k, p[10..12] conductor f_avg,
 *                   p[13..15] coat tint
 *   DIFFUSE_LIGHT   p[0..2] emission, p[3] spread (degrees), p[4] tan(spread/2) (inf = none),
 *                   p[5] cosine share
 *   PHASE           p[0..2] albedo, p[3] g
 * Wrappers, any type:
 *   normal_map  >= 0: normal_mapped wrapper (material.h:631-674) with that texture
 *   emission_tex >= 0: emissive_surface wrapper (material.h:714-741)
 */
typedef struct mypbr_material {
    int32_t type;
    int32_t flags;
    int32_t tex[8];
    int32_t normal_map;
    int32_t emission_tex;
    double p[16];
} mypbr_material;

/* --------------------------------------------------------------- lights */

enum {
    MYPBR_LIGHT_GROUP = 0,       /* a primitive, a box (6 quads) or a mesh */
    MYPBR_LIGHT_ENVIRONMENT = 1, /* include/environment.h:163-349 */
    MYPBR_LIGHT_SUN = 2          /* include/sun.h:23-83 */
};

/* A light of the light list (include/light_list.h:33-134). Its members are
 * light_members[first_member .. first_member + member_count): it is sampled by
 * picking a member by member_cdf and a direction towards that member; its pdf
 * is the member-weighted sum (hittable_list.h:107-124, mesh.h:197-216).
 * probability is the power-based selection probability p_k
 * (light_list.h:45-96), and the lights' CDF is the running sum. */
typedef struct mypbr_light {
    int32_t kind;
    int32_t first_member;
    int32_t member_count;
    int32_t reserved;
    double probability;
} mypbr_light;

typedef struct mypbr_light_member {
    int32_t prim_kind;
    int32_t prim_index;
    double weight; /* selection probability within the light */
} mypbr_light_member;

/* An equirectangular environment (include/environment.h:163-349): width x
 * height RGB floats, row 0 at +y. width == 0 means none. */
typedef struct mypbr_environment {
    int32_t width, height;
    const float* pixels;
    double intensity;
    double rotation; /* in turns */
} mypbr_environment;

/* A sun (include/sun.h:23-83). enabled == 0 means none. */
typedef struct mypbr_sun {
    int32_t enabled;
    int32_t disk_visible;
    double direction[3]; /* unit, towards the sun */
    double angular_diameter; /* degrees */
    double irradiance[3];
} mypbr_sun;

/* The whole scene as plain arrays. */
typedef struct mypbr_flat_scene {
    uint32_t abi_version;
    uint32_t reserved0;

    const mypbr_sphere* spheres;       int64_t sphere_count;
    const mypbr_quad* quads;           int64_t quad_count;
    const double* positions;           int64_t position_count; /* xyz triples */
    const double* normals;             int64_t normal_count;   /* xyz triples */
    const double* uvs;                 int64_t uv_count;       /* uv pairs */
    const mypbr_triangle* triangles;   int64_t triangle_count;
    const mypbr_mesh* meshes;          int64_t mesh_count;
    const mypbr_medium* media;         int64_t medium_count;
    const mypbr_xform* xforms;         int64_t xform_count;
    const mypbr_unbounded* unbounded;  int64_t unbounded_count;

    const mypbr_bvh_node* bvh_nodes;   int64_t bvh_node_count;
    const mypbr_prim_ref* bvh_prims;   int64_t bvh_prim_count;

    const mypbr_material* materials;   int64_t material_count;
    const mypbr_texture* textures;     int64_t texture_count;
    const uint8_t* texels_ldr;         int64_t texels_ldr_bytes;
    const float* texels_hdr;           int64_t texels_hdr_count;

    const mypbr_light* lights;               int64_t light_count;
    const mypbr_light_member* light_members; int64_t light_member_count;
    mypbr_environment environment;
    mypbr_sun sun;

    /* The sky seen by escaping rays when there is no environment
     * (include/camera.h:41-42, :515-529): the gradient, or a constant. */
    int32_t use_sky;
    int32_t reserved1;
    double background[3];

    /* Voxel models (MYPBR_PRIM_VOXEL_BLOCK primitives index voxel_blocks). */
    const mypbr_voxel_model* voxel_models;   int64_t voxel_model_count;
    const mypbr_voxel_block* voxel_blocks;   int64_t voxel_block_count;
    const mypbr_voxel_entry* voxel_palettes; int64_t voxel_palette_count;
    const uint8_t* voxel_cells;              int64_t voxel_cell_bytes;
} mypbr_flat_scene;

/* --------------------------------------------------------------- camera */

/* The reference camera's public settings (include/camera.h:20-56) that shape
 * rays. image_height is int(image_width / aspect_ratio), at least 1
 * (camera.h:143-144); mypbr_camera_init fills it. */
typedef struct mypbr_camera {
    int32_t image_width;
    int32_t image_height;
    double aspect_ratio;
    double vfov;
    double lookfrom[3], lookat[3], vup[3];
    double defocus_angle;
    double focus_dist;
    double ortho_height;
    int32_t blades;
    int32_t reserved;
    double blade_rotation;
} mypbr_camera;

/* The reference camera's defaults (camera.h:20-56). */
void mypbr_camera_init(mypbr_camera* cam);

/* Render settings: the integrator knobs of camera.h:23-34 plus this backend's. */
typedef struct mypbr_render_opts {
    int32_t samples_per_pixel;   /* camera.h:23 */
    int32_t max_depth;           /* camera.h:24 */
    int32_t max_diffuse;         /* camera.h:27, 0 = no cap */
    int32_t max_specular;        /* camera.h:28 */
    int32_t max_scatter;         /* camera.h:29 */
    int32_t transparent_shadows; /* camera.h:34 */
    int32_t collect_features;    /* camera.h:56: also fill albedo, normal, variance */
    int32_t guided;              /* path guiding: 0 off; 1 on (8 hidden layers); 2, 4 or 8 hidden
                                    layers. The scene handle keeps the network between renders. */
    uint64_t seed;               /* seeds the counter-based random numbers */
    int32_t samples_per_wave;    /* passes traced together (0 = automatic) */
    int32_t timing;              /* 1: time each kernel kind with CUDA events (stats) */
    int32_t first_row;           /* render only rows [first_row, first_row + row_count) */
    int32_t row_count;           /* 0 = every row; other rows of the outputs are left as they are */
} mypbr_render_opts;

void mypbr_render_opts_init(mypbr_render_opts* opts);

/* ------------------------------------------------------------ host layer */

typedef struct mypbr_host_scene mypbr_host_scene;

/* Parses a .scene file (grammar of include/scene.h:44-243) with its OBJ meshes
 * and .hdr environment, builds the SAH BVH and the light list, and returns the
 * flat scene plus the camera and render settings the file gives. On failure,
 * *out is NULL and mypbr_last_error() holds "path:line: message". */
int mypbr_scene_load(const char* path, mypbr_host_scene** out);

/* The same from text in memory; relative paths resolve against base_dir. */
int mypbr_scene_parse(const char* text, const char* base_dir, mypbr_host_scene** out);

const mypbr_flat_scene* mypbr_scene_flat(const mypbr_host_scene* s);
const mypbr_camera* mypbr_scene_camera(const mypbr_host_scene* s);
const mypbr_render_opts* mypbr_scene_render_opts(const mypbr_host_scene* s);
void mypbr_scene_free(mypbr_host_scene* s);

/* The Kulla-Conty tables E[32][32] (row = roughness, column = mu) then
 * E_avg[32], built on the host by the reference's deterministic VNDF
 * quadrature (include/microfacet.h:299-337). out must hold 1056 doubles. */
int mypbr_ggx_albedo_table(double* out);

/* ---------------------------------------------------------- device layer */

typedef struct mypbr_gpu_scene mypbr_gpu_scene;

/* Copies the flat scene to HBM (FP32 geometry, compact BVH) on the current
 * CUDA device. The flat scene may be freed afterwards. */
int mypbr_gpu_scene_create(const mypbr_flat_scene* scene, mypbr_gpu_scene** out);
void mypbr_gpu_scene_destroy(mypbr_gpu_scene* scene);

/* Called between passes with the number of samples per pixel done; the output
 * buffers then hold the running average (camera.h:95-102). */
typedef void (*mypbr_pass_callback)(int done, void* user);

/* Renders the scene: the replacement for camera::render (camera.h:79-105).
 * radiance: W*H*3 doubles (required). albedo, normal: W*H*3, variance: W*H;
 * filled when opts->collect_features, otherwise may be NULL. The call is
 * synchronous. If save_every > 0, on_pass is called every save_every passes
 * (not after the last one). */
int mypbr_gpu_render(mypbr_gpu_scene* scene, const mypbr_camera* cam, const mypbr_render_opts* opts,
                     double* radiance, double* albedo, double* normal, double* variance,
                     int save_every, mypbr_pass_callback on_pass, void* user);

/* The same, with outputs left in device memory (each a device pointer of the
 * sizes above, NULL allowed as for mypbr_gpu_render) and work issued on the
 * given CUDA stream (NULL = the legacy default stream). Returns once the
 * work is queued; stats (optional) are filled after a stream sync. */
typedef struct mypbr_render_stats {
    uint64_t paths;            /* camera rays traced */
    uint64_t extension_rays;   /* closest-hit rays traced for path continuation */
    uint64_t shadow_rays;      /* shadow rays traced */
    uint64_t kernel_launches;  /* kernels this call launched */
    /* with opts->timing: summed CUDA-event time per kernel kind, milliseconds */
    double ms_generate, ms_extend, ms_shade, ms_shadow, ms_other;
    uint64_t launches_extend, launches_shade, launches_shadow;
} mypbr_render_stats;

int mypbr_gpu_render_device(mypbr_gpu_scene* scene, const mypbr_camera* cam, const mypbr_render_opts* opts,
                            double* d_radiance, double* d_albedo, double* d_normal, double* d_variance,
                            void* cuda_stream, mypbr_render_stats* stats);

/* mypbr_gpu_render with, in addition, the per-channel variance of the mean
 * radiance (W*H*3 doubles, may be NULL) from the per-sample second moments,
 * and render statistics (may be NULL). */
int mypbr_gpu_render_ex(mypbr_gpu_scene* scene, const mypbr_camera* cam, const mypbr_render_opts* opts,
                        double* radiance, double* albedo, double* normal, double* variance,
                        double* channel_variance, int save_every, mypbr_pass_callback on_pass, void* user,
                        mypbr_render_stats* stats);

/* The render with no device allocation, for callers that may not allocate
 * device memory while they render (a host that gives this library a fixed
 * device-memory budget up front, or a per-frame callback where the
 * synchronisation an allocation can cause would stall the frame). It has no
 * counterpart in the reference. Every scratch buffer comes from one static
 * 18 MiB device array in the library, present on every GPU that loads it until
 * the library is unloaded; the scene comes from mypbr_gpu_scene_create and the
 * outputs are caller-provided device buffers as for mypbr_gpu_render_device.
 * Limits: at most 65,536 pixels in the rendered rows (width x row_count:
 * 256 x 256, say, or a 34-row band of a 1920-wide frame), bounce caps at most
 * 255 and max_depth <= 1024; larger requests fail with
 * MYPBR_ERR_INVALID_ARGUMENT. Guided rendering is not supported here
 * (MYPBR_ERR_UNSUPPORTED). The outputs are indexed over the whole image, as
 * for mypbr_gpu_render_device: only the band's rows are written. Calls share
 * the array: it is cleared at the start of each call, and calls that overlap
 * on the GPU race, so issue one at a time. The first call on a device looks up
 * the array's address with that device current and keeps it: make that first
 * call before any stream capture begins, and do not reset the device while
 * the library is loaded. Synchronous: returns when the frame is done. */
int mypbr_gpu_render_noalloc(mypbr_gpu_scene* scene, const mypbr_camera* cam, const mypbr_render_opts* opts,
                             double* d_radiance, double* d_albedo, double* d_normal, double* d_variance,
                             void* cuda_stream);

/* Self-intersection probe (no counterpart in the reference, whose rays skip
 * t < 0.001): for n rays (n x 8 as for mypbr_gpu_trace) the closest hit, then
 * a reflected ray and a ray going on through the surface, both started as
 * the renderer starts them (hit point moved off the surface by its FP32
 * error bound). out (n x 8 words): kind of the first hit (-1 none), 1 where
 * the reflected / the continued ray met the surface it left, kind of the
 * reflected ray's hit (-1 none), then as float bits for the first spawned ray
 * that met its surface (else the reflected one) its t, its origin's offset,
 * the cosine of its direction to the normal and its walk's t_min. */
int mypbr_gpu_test_spawn(mypbr_gpu_scene* scene, const float* rays, int64_t n, int32_t* out);

/* Ray batch query: closest hit of n rays against the scene, the reference's
 * world.hit (hittable_list.h:25-37 over bvh.h:45-86 and scene::unbounded)
 * without media (media are stochastic). rays: n x 8 floats (ox oy oz dx dy dz
 * tmin tmax), device or host memory as `on_device` says. hits: n x 8 floats
 * (t, nx, ny, nz, u, v, front_face, material) and prim: n x 2 int32 (kind,
 * index; kind -1 on a miss; a voxel face reports its block; the ground plane
 * reports kind 5). The walk is the one the handle's traversal setting names
 * (mypbr_gpu_set_launch: 2, 3 or 5 where the tree allows it), else the plain
 * binary walk. */
int mypbr_gpu_trace(mypbr_gpu_scene* scene, const float* rays, int64_t n, float* hits, int32_t* prim,
                    int on_device);

/* Pointwise BSDF query, for parity checks of eval / pdf (material.h:35-44 and
 * the scatter() pdf): for each of n records evaluates material `material` at a
 * surface point. rec: n x 16 floats (p xyz, normal xyz, front_face, u, v,
 * dpdu xyz, dpdv xyz, unused), r_in: n x 3 floats (incoming direction),
 * wi: n x 3 floats (outgoing direction). out: n x 4 floats (eval rgb, pdf).
 * Host memory. */
int mypbr_gpu_bsdf_eval(mypbr_gpu_scene* scene, int32_t material, const float* rec, const float* r_in,
                        const float* wi, int64_t n, float* out);

/* ------------------------------------------------------------- denoiser */

/* The settings of the reference's denoiser (include/denoiser.h:39-43). */
typedef struct mypbr_denoise_opts {
    int32_t iterations;       /* a-trous passes, taps 2^i apart (5) */
    int32_t reserved;
    double sigma_luminance;   /* in standard deviations of the noise (4) */
    double sigma_normal;      /* distance between normals (0.1) */
    double sigma_albedo;      /* distance between albedos (0.1) */
} mypbr_denoise_opts;

void mypbr_denoise_opts_init(mypbr_denoise_opts* opts);

/* denoiser::run (include/denoiser.h:45-75): filters a frame's radiance with
 * its albedo, normal and variance guides (W*H*3, W*H*3, W*H*3, W*H doubles,
 * rows from the top left) into out (W*H*3). opts may be NULL (defaults).
 * Pointers are device memory if on_device, else host memory. Synchronous. */
int mypbr_gpu_denoise(const double* radiance, const double* albedo, const double* normal, const double* variance,
                      int32_t width, int32_t height, const mypbr_denoise_opts* opts, double* out, int on_device);

/* ------------------------------------------------------ device BVH build */

enum { MYPBR_BVH_LBVH = 1 };

/* What a device BVH build did: primitives, interior nodes, depth (interior
 * nodes on the deepest path), build time on the device, and the SAH cost
 * (node visits 0.125, primitive tests 1, relative to the root's area) of the
 * new tree and of the one it replaced. */
typedef struct mypbr_bvh_report {
    int64_t primitives;
    int64_t nodes;
    int32_t depth;
    int32_t reserved;
    double build_ms;
    double sah_cost;
    double sah_cost_before;
} mypbr_bvh_report;

/* Rebuilds the scene handle's BVH on the device (MYPBR_BVH_LBVH: a linear BVH
 * over Morton-sorted primitive centroids, Karras 2012) and uses it for later
 * renders and queries. No counterpart in the reference, whose host SAH build
 * (bvh.h:110-205, built here by mypbr_gpu_scene_create) stays the default
 * and the quality reference. */
int mypbr_gpu_scene_rebuild_bvh(mypbr_gpu_scene* scene, int32_t method, mypbr_bvh_report* report);

/* ------------------------------------------------------------ sky bake */

/* atmosphere_settings (include/atmosphere.h:39-46): densities relative to
 * Earth's, the haze's forward scattering, the overall radiance scale. */
typedef struct mypbr_sky_settings {
    double rayleigh, mie, mie_g, ozone, intensity;
} mypbr_sky_settings;

void mypbr_sky_settings_init(mypbr_sky_settings* settings);

/* atmosphere::bake and sun_transmittance (atmosphere.h:53-108): the
 * single-scattering sky for a sun in sun_direction of irradiance
 * sun_irradiance, as a width x height equirectangular image (rgb, 3 doubles
 * per pixel, host memory), and (if not NULL) the sun's transmittance through
 * the air (3 doubles). on_gpu: bake on the device, else on the host. The
 * scene loader bakes `sky atmosphere` skies the same way (256 x 128). */
int mypbr_sky_bake(const mypbr_sky_settings* settings, const double sun_direction[3], const double sun_irradiance[3],
                   int32_t width, int32_t height, double* rgb, double* sun_transmittance, int on_gpu);

/* ------------------------------------------------------------ batches */

/* One render of a batch: device output buffers as for mypbr_gpu_render_device
 * (albedo / normal / variance may be NULL unless opts->collect_features). */
typedef struct mypbr_batch_job {
    mypbr_gpu_scene* scene;
    const mypbr_camera* camera;
    const mypbr_render_opts* opts;
    double* radiance;
    double* albedo;
    double* normal;
    double* variance;
    int32_t status;   /* out: this job's status */
    int32_t reserved;
} mypbr_batch_job;

/* Renders every job (many scenes or frames of different sizes and spp): jobs
 * on different scene handles run concurrently on the handles' own streams,
 * one wave of each in turn, waves replayed from captured CUDA graphs; jobs on
 * one handle run in order. Returns when all are done: the first failing
 * job's status, or MYPBR_OK. No counterpart in the reference (its renders
 * are one at a time, camera.h:79-105). */
int mypbr_gpu_render_batch(mypbr_batch_job* jobs, int32_t n);

/* The autotuner's choice for a scene handle and view: threads per block of
 * the bounce kernels, paths per wave and the traversal scheme (1: lanes take
 * new rays as theirs finish; 2: each lane walks its ray to the end over the
 * tree collapsed to 4 children per node; 3: the binary tree with leaves
 * postponed until the warp's lanes all hold one; 4: the plain binary walk;
 * 5: each lane walks the tree collapsed to 8 children per node with
 * quantised boxes; 0, the default, is 4 for trees whose leaves are mostly
 * spheres and 3 otherwise), with the Mpaths/s of each of the 40 trials
 * (traversal 1 to 5; within each, block 128 then 256; within each, 16M,
 * 32M, 64M, 128M paths; 0 for trials skipped because the scene's tree does
 * not allow that walk). */
typedef struct mypbr_tune_result {
    int32_t block;
    int32_t traversal;
    int64_t wave_paths;
    double mpaths_per_s;
    double trial_mpaths[40];  /* traversal 1..5 x block 128, 256 x 16, 32, 64, 128 M paths per wave */
} mypbr_tune_result;

/* Sets the launch settings the autotuner would set (0 keeps a setting's
 * default: block 256, 128M paths per wave for plain renders and 32M for
 * guided ones, traversal 0). Traversal: 0 the
 * scene's default, 1 lanes that take new rays, 2 the 4-wide tree, 3 postponed
 * leaves, 4 the plain binary walk, 5 the 8-wide tree with quantised boxes. A
 * traversal the scene's tree does not allow (2 or 5 without that tree, 3 or
 * 5 with leaves of 16 or more references) walks the plain binary tree. */
int mypbr_gpu_set_launch(mypbr_gpu_scene* scene, int32_t block, int64_t wave_paths, int32_t traversal);

/* Times short renders of the view with each setting and keeps the fastest on
 * the handle: later renders use it unless opts->samples_per_wave is set. */
int mypbr_gpu_autotune(mypbr_gpu_scene* scene, const mypbr_camera* camera, const mypbr_render_opts* opts,
                       mypbr_tune_result* out);

/* ------------------------------------------------ display and images */

/* Tonemappers of display_settings (include/tonemap.h:10). */
enum { MYPBR_TONEMAP_NONE = 0, MYPBR_TONEMAP_REINHARD = 1, MYPBR_TONEMAP_ACES = 2 };

/* display_settings + post_settings (include/tonemap.h:12-18,
 * include/postprocess.h:13-21). */
typedef struct mypbr_display_opts {
    double exposure;        /* stops: radiance x 2^exposure */
    int32_t tonemap;        /* MYPBR_TONEMAP_* */
    int32_t reserved;
    double bloom;           /* strength, 0 = off */
    double bloom_threshold; /* luminance above which pixels glow */
    double bloom_radius;    /* reach of the glow, fraction of the image width */
    double vignette;        /* corner darkening, 0 = off */
} mypbr_display_opts;

void mypbr_display_opts_init(mypbr_display_opts* opts);

/* postprocess (include/postprocess.h:104-151) of a radiance image (W*H*3
 * doubles, rows from the top left) on the GPU: into `linear` (W*H*3 doubles,
 * may be NULL) the bloomed and vignetted radiance; into `rgb8` (W*H*3 bytes,
 * may be NULL) the display image after exposure, tonemapping and the sRGB
 * curve (display_settings::apply + to_byte, tonemap.h:28-37, color3.h:33-36).
 * Pointers are device memory if on_device, else host memory. */
int mypbr_gpu_display(const double* radiance, int32_t width, int32_t height, const mypbr_display_opts* opts,
                      double* linear, uint8_t* rgb8, int on_device);

/* Decodes an 8-bit image file (PNG of any color type and depth, interlaced
 * or not, with tRNS; TGA types 1, 2, 3 and their run-length forms; baseline
 * and progressive JPEG; BMP of 1, 4, 8, 16, 24 and 32 bits; GIF, first frame;
 * binary PGM / PPM of 8 and 16 bits) to RGBA bytes, rows from the top, as image_texture loads one
 * (stbi_load with 4 channels, include/texture.h:67-98). *channels is the
 * file's own count as stb_image reports it (1 grey, 2 grey + alpha, 3 RGB,
 * 4 RGBA). With rgba NULL only the size is returned; else rgba holds
 * capacity >= w * h * 4 bytes. Arithmetic-coded or lossless JPEG and
 * run-length BMP files give MYPBR_ERR_UNSUPPORTED. */
int mypbr_image_read(const char* path, int32_t* width, int32_t* height, int32_t* channels, uint8_t* rgba,
                     int64_t capacity);

/* The environment's sampling tables for an equirectangular image (W*H*3
 * floats, rows from the top): texel_pdf (W*H floats) = p * W * H with p
 * proportional to luminance x sin(theta) (environment.h:147-176; a black
 * image: rows by sin(theta)), and alias (W*H pairs of floats: probability,
 * alias index as int bits) an alias table holding the same distribution.
 * on_gpu: built on the device (the way mypbr_gpu_scene_create builds them),
 * else on the host with Vose's method. Host pointers. */
int mypbr_env_distribution(const float* rgb, int32_t width, int32_t height, float* texel_pdf, float* alias,
                           int on_gpu);

/* write_image (include/image_io.h:84-106): the format follows the extension;
 * .png and .ppm are display images (post-processed on the GPU), .hdr and .pfm
 * the raw radiance; an empty path writes PPM to stdout. */
int mypbr_write_image(const char* path, const double* radiance, int32_t width, int32_t height,
                      const mypbr_display_opts* opts, int on_device);

/* The failure path of the device's bounded waits, without a fault: one CTA
 * waits on an mbarrier phase that nothing completes, gives up after about a
 * second, and this returns MYPBR_ERR_DEVICE_TIMEOUT; the context stays
 * usable. For tests. */
int mypbr_gpu_test_wait_timeout(void);

/* ----------------------------------------------------- path guiding
 *
 * No counterpart in the reference: a learned sampling proposal, used by
 * mypbr_gpu_render* when opts->guided != 0. An MLP maps a surface vertex
 * (position in the scene box, normal, outgoing direction; one-blob encoded
 * into 128 inputs) through `hidden` ReLU layers of 64 units to 64 outputs,
 * the first 40 of which are 8 von Mises-Fisher lobes (mean xyz, log kappa,
 * logit). BF16 weights and activations, FP32 accumulation on the tensor
 * cores. Weights are passed as FP32, matrix after matrix, each [64 out][in]
 * row-major (in = 128 for the first, 64 after): 64*128 + hidden*64*64 values.
 * These entry points expose the kernels to the parity tests. Synchronous. */

/* Puts the scene handle's guiding network back to its initial (untrained)
 * weights, keeping its buffers: the next guided render starts from scratch. */
int mypbr_guide_reset(mypbr_gpu_scene* scene);

/* How guided renders of this scene handle sample: at the first `depths`
 * bounces of a path (1..4096; default 4), a direction comes from the learned
 * mixture with probability `alpha` (0 < alpha < 1; default 0.5) at the first
 * bounce and `alpha_deep` at the later ones (0 <= alpha_deep < 1, or below 0
 * for alpha itself; default), else from the BSDF, and the density used is the
 * mixture of both (one-sample MIS), so the estimate stays unbiased whatever
 * the network outputs: the BSDF proposal keeps every direction the BSDF can
 * scatter into reachable. The setting applies from the next render. */
int mypbr_guide_configure(mypbr_gpu_scene* scene, float alpha, int32_t depths, float alpha_deep);

/* How the guiding network of this scene handle trains (no counterpart in the
 * reference): Adam steps after each of the first 8 waves of a guided render
 * (small waves, every path recorded; default 16), after each later wave
 * (default 4), the total after which recording and training stop (default
 * 1500), the steps taken before the mixture is sampled at all (default
 * 128, the end of the first recorded waves; until then guided renders sample
 * as plain ones), and the cap on one training record's weight as a multiple
 * of its batch's mean weight (default 256; 0 for no cap, else 1 to 1e6), so
 * that a few very bright paths cannot take over the fit. Applies from the
 * next wave. */
int mypbr_guide_schedule(mypbr_gpu_scene* scene, int32_t steps_early, int32_t steps_late, int32_t max_steps,
                         int32_t use_after, float weight_cap);

/* the network's encoded inputs (n x 128, BF16 values as floats) of n
 * vertices given by their 7 scalars in [0, 1] (n x 7). */
int mypbr_guide_test_encode(const float* scalars, int64_t n, float* out);
/* outputs (n x 64) of the network for encoded inputs (n x 128). */
int mypbr_guide_test_forward(int hidden, const float* weights, const float* inputs, int64_t n, float* out);
/* weight gradients (same layout as weights) of sum_i dout_i . out_i. */
int mypbr_guide_test_backward(int hidden, const float* weights, const float* inputs, const float* dout, int64_t n,
                              float* grads);
/* the training loss -c log q(dir) of mixtures given by raw outputs (n x 64)
 * and its gradient with respect to those outputs (n x 64). */
int mypbr_guide_test_loss(const float* raw, const float* dirs, const float* c, int64_t n, float* grad, float* loss);
/* mixture sampling with uniforms u (n x 3): samples (n x 3), the density at
 * each sample and at the given directions dirs (n x 3). */
int mypbr_guide_test_mixture(const float* raw, const float* u, const float* dirs, int64_t n, float* samples,
                             float* pdf_sample, float* pdf_dir);

#ifdef __cplusplus
}
#endif

#endif /* MYPBR_GPU_H */
