/*
 * polyred_cuda.h — C ABI of libpolyred_cuda.so, the GB300 (sm_103a) render path
 * behind polyred's `render.CUDA(dev)` option.
 *
 * The library replaces, as one device frame, the CPU passes that
 * render.(*Renderer).Render runs (render/raster.go:155-199):
 *   shadow passes   render/shadow.go:92-228   (passShadows / drawDepth)
 *   forward raster  render/raster.go:226-273, 380-572 (cpuForwardPass / draw /
 *                   drawClipped) with render/cull.go and render/clipping.go
 *   deferred shade  render/raster.go:275-359 (passDeferred / shade) with
 *                   shader/blinn_cpu.go:24-106, render/shadow.go:230-283,
 *                   material/ao.go:20-73
 *   gamma           render/raster.go:361-378, shader/gamma.go:13-18,
 *                   color/srgb.go:15-33
 * Results follow the reference's single-worker order (render.Workers(1)):
 * triangle-ID and depth buffers are bit-exact with it.
 *
 * Every entry point takes plain integers and pointers (no struct by value, no
 * callbacks, no varargs) so that a purego binding (gpu/backend_vk.go:209-232
 * style SyscallN) can call it. Descriptor structs are passed by pointer and
 * start with a `size` field (sizeof the struct the caller was compiled with).
 *
 * Threading: one pr_ctx owns one CUDA stream and its device buffers. Calls on
 * one context must be serialised by the caller (the Go renderer holds a
 * mutex, as render/options.go:125-141 waits for an in-flight frame). Distinct
 * contexts may be used concurrently.
 *
 * Errors: every function returns a status (PR_OK or a negative PR_ERR_*).
 * pr_last_error() gives a thread-local detail string for the last failure on
 * the calling thread. There is no silent CPU fallback.
 */
#ifndef POLYRED_CUDA_H
#define POLYRED_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PR_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------- */
#define PR_OK                 0
#define PR_ERR_INVALID_ARG   -1
#define PR_ERR_OOM           -2
#define PR_ERR_CUDA          -3
#define PR_ERR_OVERFLOW      -4  /* an internal capacity was exceeded after retry */
#define PR_ERR_TIMEOUT       -5  /* a bounded device wait gave up */
#define PR_ERR_UNIMPLEMENTED -6
#define PR_ERR_NO_SCENE      -7
#define PR_ERR_UNSUPPORTED   -8  /* e.g. a non-uniform texture, MSAA in a batch */
#define PR_ERR_NO_DEVICE     -9
#define PR_ERR_SINGULAR     -10  /* Mat4.Inv of a zero determinant; the
                                    reference panics (math/mat4.go:261-263) */
#define PR_ERR_FATAL        -11  /* input the reference rejects with a panic
                                    rather than an error (pr_obj_parse) */

/* ---- flags ------------------------------------------------------------ */
/* material.Standard flags (material/material.go:23-29) */
#define PR_MAT_FLAT_SHADING    1u
#define PR_MAT_AO              2u
#define PR_MAT_RECEIVE_SHADOW  4u
#define PR_MAT_MIPMAP          8u  /* buffer.Texture.UseMipmap() (buffer/texture.go:56-59) */

#define PR_LIGHT_POINT         0   /* light/point.go */
#define PR_LIGHT_DIRECTIONAL   1   /* light/directional.go */

#define PR_FRAME_PERSPECTIVE   1u  /* option.Perspect (render/options.go:49-56) */
#define PR_FRAME_SHADOWMAP     2u  /* render.ShadowMap(true) */
#define PR_FRAME_GAMMA         4u  /* render.GammaCorrection(true) */

#define PR_SCENE_DEVICE_PTRS   1u  /* triangle arrays are device pointers */
#define PR_OUT_DEVICE_PTRS     1u  /* output arrays are device pointers */

#define PR_TRI_NONE 0xFFFFFFFFu    /* tri_id of a pixel no triangle covers */

/* ---- scene ------------------------------------------------------------ */

/* One geometry in scene traversal order (scene/core.go:86-200). Its
 * triangles are [first_tri, first_tri + n_tris) of the soup. `model` is the
 * composed model matrix that cpuForwardPass builds as
 * modelMatrix.MulM(g.ModelMatrix()) (render/raster.go:242), row-major
 * X00 X01 X02 X03 X10 ... X33. `mat_base` is the offset of this geometry's
 * materials in the flat material table (render/raster.go:252-262). */
typedef struct pr_object {
    uint32_t first_tri;
    uint32_t n_tris;
    int32_t  mat_base;
    uint32_t reserved;
    float    model[16];
} pr_object;

/* material.BlinnPhong (material/material.go:43-51) with a uniform (1x1)
 * texture (buffer/texture.go:16-24). Colours are RGBA8 as stored by the
 * reference (color.FromValue rounds half away from zero). */
typedef struct pr_material {
    uint8_t  diffuse[4];
    uint8_t  specular[4];
    uint8_t  texture[4];    /* the texel of a uniform (1x1) texture */
    float    shininess;
    uint32_t flags;         /* PR_MAT_* */
    int32_t  texture_size;  /* Texture.Size(): 1 for a uniform texture; ignored
                               when pr_scene_desc.textures gives an image */
} pr_material;

/* An image texture, buffer.NewTexture(TextureImage(img)) (buffer/texture.go:
 * 35-67): the library builds its mipmap (each level imageutil.Resize of the
 * image) when the material has PR_MAT_MIPMAP. Host memory. */
typedef struct pr_texture {
    int32_t width, height;   /* 1..16384 */
    const uint8_t* rgba;     /* [height][width][4] image.RGBA pixels, rows top-down; NULL: no image */
} pr_texture;

/* The triangle soup: per triangle three vertices (primitive.Vertex,
 * geometry/primitive/vertex.go:14-20). Arrays are host pointers unless
 * flags has PR_SCENE_DEVICE_PTRS. */
typedef struct pr_scene_desc {
    uint32_t size;
    uint32_t flags;
    uint32_t n_tris;
    uint32_t n_objects;
    uint32_t n_materials;
    uint32_t reserved;
    const float*   pos;      /* [n_tris][3][4]  Vertex.Pos (x,y,z,w) */
    const float*   nor;      /* [n_tris][3][4]  Vertex.Nor (x,y,z,w) */
    const float*   uv;       /* [n_tris][3][2]  Vertex.UV */
    const uint8_t* col;      /* [n_tris][3][4]  Vertex.Col RGBA8 */
    const int32_t* mat_id;   /* [n_tris] Triangle.MaterialID, geometry-local; <0 = vertex colour */
    const pr_object*   objects;    /* [n_objects] (host memory) */
    const pr_material* materials;  /* [n_materials] flat table (host memory) */
    /* [n_materials] or NULL (host memory): the image texture of each
     * material, sampled by Texture.Query (buffer/texture.go:83-187) at the
     * FragmentShader's level of detail (shader/blinn_cpu.go:28-35); entries
     * with rgba NULL keep the material's uniform texel. The mipmaps are
     * built on the host at every pr_scene_upload / pr_frame_submit that
     * carries the images. Not available in batches and the adjoint
     * (PR_ERR_UNSUPPORTED). */
    const pr_texture*  textures;
} pr_scene_desc;
#define PR_SCENE_DESC_SIZE_V1 80u  /* pr_scene_desc up to materials */

/* ---- frame ------------------------------------------------------------ */

/* A light source (light.Source) in scene.Lights() order. For a light with
 * cast_shadow set and PR_FRAME_SHADOWMAP on, shadow_view/shadow_proj are the
 * light camera initShadowMaps builds (render/shadow.go:41-85); see
 * pr_shadow_camera. */
typedef struct pr_light {
    int32_t type;            /* PR_LIGHT_* */
    int32_t cast_shadow;
    float   pos[3];          /* point: Position() */
    float   dir[3];          /* directional: Dir() (already normalised) */
    float   intensity;
    uint8_t color[4];
    float   shadow_view[16];
    float   shadow_proj[16];
} pr_light;

typedef struct pr_frame_desc {
    uint32_t size;           /* sizeof(pr_frame_desc); PR_FRAME_DESC_SIZE_V1 (no msaa field) is accepted */
    uint32_t flags;          /* PR_FRAME_* */
    int32_t  width, height;  /* render.Size: the image Render() returns */
    float    view[16];       /* Camera.ViewMatrix() */
    float    proj[16];       /* Camera.ProjMatrix() */
    float    cam_pos[3];     /* Camera.Position() */
    uint8_t  background[4];  /* render.Background */
    uint32_t n_lights;
    uint32_t n_ambient;
    const pr_light* lights;  /* [n_lights] */
    const float*    ambient; /* [n_ambient] light.Environment intensities, traversal order */
    int32_t  shadow_width;   /* 0 = framebuffer size (the reference's only mode) */
    int32_t  shadow_height;
    /* render.MSAA(n) (render/options.go:66-68), 1..16; 0 counts as 1. The
     * frame renders into a framebuffer of (n*width) x (n*height)
     * (render/raster.go:147-151) whose viewport test and clipping use n times
     * the framebuffer size, as the reference's draw and cullViewFrustum do
     * (render/raster.go:414-441, render/cull.go:15-23); the shadow maps
     * default to the framebuffer size. passAntialiasing's imageutil.Resize
     * (internal/imageutil/resize.go:16-66) then scales the RGBA image to
     * width x height. With n > 1 pr_outputs.rgba is [height][width][4] and
     * every other output is [n*height][n*width] (the framebuffer). Not
     * available in batches and the adjoint (PR_ERR_UNSUPPORTED). */
    int32_t  msaa;
    int32_t  reserved;
} pr_frame_desc;
#define PR_FRAME_DESC_SIZE_V1 192u  /* pr_frame_desc up to shadow_height */

/* ---- outputs ------------------------------------------------------------
 * Every array is optional (NULL = not wanted). Rows are top-down: row r holds
 * raster row y = height-1-r, the order of buffer.FragmentBuffer storage
 * (buffer/buffer.go:209-213) and of Render()'s *image.RGBA. */
typedef struct pr_outputs {
    uint32_t size;
    uint32_t flags;          /* PR_OUT_DEVICE_PTRS */
    uint8_t*  rgba;          /* [H][W][4] final image (after gamma when enabled) */
    uint32_t* tri_id;        /* [H][W] winning input triangle index, PR_TRI_NONE if empty */
    float*    depth;         /* [H][W] Fragment.Depth (0 where empty) */
    float*    nor;           /* [H][W][4] Fragment.Nor */
    float*    face_nor;      /* [H][W][4] Fragment.FaceNor */
    float*    world_pos;     /* [H][W][4] Fragment.WordPos */
    float*    uvd;           /* [H][W][4] Fragment.U, V, Du, Dv */
    uint8_t*  vcol;          /* [H][W][4] Fragment.Col (interpolated vertex colour) */
    int32_t*  mat_id;        /* [H][W] flat Fragment.MaterialID (-1 where empty) */
    float*    shadow_maps;   /* [n_lights][SH][SW] shadow depth maps after the frame
                                (rows bottom-up, index x + y*SW as render/shadow.go:213) */
} pr_outputs;

/* Per-frame counters (optional, pr_frame_stats). */
typedef struct pr_stats {
    uint32_t size;
    uint32_t n_tris_in;
    uint32_t n_raster_tris;    /* after cull/clip, main view */
    uint32_t n_clipped_tris;   /* input triangles that went through clipTriangle */
    uint32_t n_raster_tasks;   /* raster work items (pixel-box chunks of <= 32 px), all passes */
    uint32_t n_nan_fragments;  /* fragments with NaN depth (degenerate triangles) */
    uint32_t n_kernel_launches;
    uint32_t reserved;
    float    ms_shadow, ms_setup, ms_raster, ms_shade, ms_total;
    float    ms_ao;            /* ambient occlusion part of ms_shade */
    uint32_t n_ao_pixels;
} pr_stats;

/* ---- entry points ------------------------------------------------------ */

int         pr_abi_version(void);
const char* pr_error_string(int status);
const char* pr_last_error(void);

/* Create a context on CUDA device `device` (a caller-chosen ordinal). The
 * context never resets or closes the device (cf. render/raster.go:57-60: a
 * caller-supplied device is not closed by the renderer). */
int pr_create(int device, void** out_ctx);
int pr_destroy(void* ctx);

/* Copy a scene to the device (replacing the previous one). Host arrays may
 * be freed after the call returns. Also clears the shadow maps, as
 * initShadowMaps allocates them zeroed (render/shadow.go:87). */
int pr_scene_upload(void* ctx, const pr_scene_desc* scene);

/* Zero the persistent shadow maps (initShadowMaps on NewRenderer/Options:
 * render/raster.go:135-140, render/options.go:135-140). Render() itself never
 * clears them (render/shadow.go:221-228). */
int pr_shadow_reset(void* ctx);

/* Render one frame: shadows, forward raster, deferred shading, gamma
 * (render/raster.go:155-199), then copy the requested outputs. Blocks until
 * the outputs are complete. */
int pr_render(void* ctx, const pr_frame_desc* frame, pr_outputs* out);

/* Render without synchronising; outputs must be device pointers
 * (PR_OUT_DEVICE_PTRS). pr_sync waits for the context's stream. */
int pr_render_async(void* ctx, const pr_frame_desc* frame, pr_outputs* out);
int pr_sync(void* ctx);

/* pr_scene_upload + pr_render in one call that does not wait: the scene is
 * copied on a stream of its own into the context's second set of scene
 * buffers while the previous frame is still computing, the frame is queued
 * behind it, and host outputs are copied back on a third stream while the
 * next frame computes. The scene's arrays and host outputs must stay valid
 * and unchanged until pr_sync (page-locked memory from pr_host_alloc moves
 * at the link's full rate); outputs may also be device pointers
 * (PR_OUT_DEVICE_PTRS). Like pr_scene_upload it starts the shadow maps from
 * zero; shadow_maps output is not available. Capacities are not grown here:
 * size them with one synchronous pr_render of a similar scene first;
 * pr_sync reports a frame that overflowed. The reference walks the scene
 * anew in every Render() (render/raster.go:241-271), so a frame loop that
 * changes its scene every frame maps to this call. */
int pr_frame_submit(void* ctx, const pr_scene_desc* scene, const pr_frame_desc* frame, pr_outputs* out);

/* Counters of the last frame rendered on this context. */
int pr_frame_stats(void* ctx, pr_stats* out);

/* The CUDA stream (cudaStream_t) the context launches on, for callers that
 * time or order work around it. */
int pr_stream(void* ctx, void** out_stream);

/* Page-locked host memory (cudaHostAlloc) for scene arrays and frame
 * outputs: copies from and to it run at the link's full rate instead of
 * through the driver's staging buffers. bytes > 0; free with pr_host_free.
 * (The reference keeps its frame buffers in ordinary Go memory,
 * render/raster.go:99-118; a Go host passes these instead.) */
int pr_host_alloc(size_t bytes, void** out_ptr);
int pr_host_free(void* ptr);

/* Device memory for outputs kept on the GPU (PR_OUT_DEVICE_PTRS) by hosts
 * that have no device allocator of their own: the frame's fragments stay
 * device-resident, as the reference's deferred seam wants them
 * (render/gpudeferred.go:110-187), and the host reads what it needs.
 * pr_device_alloc / pr_device_free: cudaMalloc / cudaFree on the context's
 * GPU. pr_device_read copies `bytes` from device address `src` to host
 * memory `dst` after every frame already issued on the context (it waits
 * for them), and returns when the copy is done. */
int pr_device_alloc(void* ctx, size_t bytes, void** out_ptr);
int pr_device_free(void* ctx, void* ptr);
int pr_device_read(void* ctx, const void* src, size_t bytes, void* dst);

/* ---- host math helpers --------------------------------------------------
 * f32 arithmetic exactly as the reference's Go (amd64) evaluates it, so a
 * host that is not Go can build the same matrices. Matrices are row-major. */

/* camera.ViewMatrix(pos, target, up)  (camera/camera.go:42-53) */
int pr_view_matrix(const float pos[3], const float target[3], const float up[3], float out[16]);
/* (*camera.Perspective).ProjMatrix (camera/perspective.go:100-111); fov in degrees */
int pr_perspective_matrix(float fov, float aspect, float near, float far, float out[16]);
/* (*camera.Orthographic).ProjMatrix (camera/orthographic.go:106-119) */
int pr_orthographic_matrix(float left, float right, float bottom, float top,
                           float near, float far, float out[16]);
/* Mat4.MulM (math/mat4.go:201-220): out = a * b */
int pr_mat4_mul(const float a[16], const float b[16], float out[16]);
/* Mat4.Inv (math/mat4.go:259-283); PR_ERR_SINGULAR on a zero determinant */
int pr_mat4_inv(const float m[16], float out[16]);
/* The orthographic light camera initShadowMaps fits around the main camera
 * frustum (render/shadow.go:41-85): writes its view and projection. */
int pr_shadow_camera(const float light_pos[3], const float scene_center[3],
                     const float cam_view[16], const float cam_proj[16],
                     float out_view[16], float out_proj[16]);

/* ---- allocation-free depth map ------------------------------------------
 * No counterpart in the reference.
 *
 * For callers that cannot allocate device memory: a host whose device memory
 * is all owned by another allocator (for example a framework's fixed caching
 * pool), or a frame loop that cannot pay for cudaMalloc/cudaFree (cudaFree
 * synchronises the whole device). It runs the shadow-map raster — the
 * drawDepth pass of render/shadow.go, the same kernels pr_render uses for
 * shadow maps — on the caller's device triangles into the caller's device
 * depth map, which is read and then updated like the reference's persistent
 * maps: a texel changes only where a fragment is stored into it, and a
 * texel no fragment replaces keeps its bits (a -0 or a NaN payload
 * included). It allocates nothing: all scratch lives in one static 16 MiB
 * device array of the library, which every GPU that loads the library keeps
 * until the process exits; the driver commits it when the library's kernels
 * are first loaded on a device (with lazy module loading, that can be inside
 * the first call that launches one of them, this one or another).
 *
 * Limits (larger inputs are rejected with PR_ERR_INVALID_ARG, or
 * PR_ERR_OVERFLOW for the task count, leaving the map unchanged):
 * n_tris <= PR_NOALLOC_MAX_TRIS, n_objects <= PR_NOALLOC_MAX_OBJECTS,
 * width*height <= PR_NOALLOC_MAX_TEXELS, raster tasks (1024-pixel chunks of
 * the triangles' pixel boxes) <= PR_NOALLOC_MAX_TASKS.
 *
 * The first call on a device looks up the array's device address. Every
 * call uses the same array: calls
 * whose work overlaps on the GPU (other streams, other host threads) race and
 * corrupt each other. The call returns when its work on `stream` is done.
 */
#define PR_NOALLOC_MAX_TRIS    65536
#define PR_NOALLOC_MAX_OBJECTS 256
#define PR_NOALLOC_MAX_TEXELS  1048576
#define PR_NOALLOC_MAX_TASKS   262144

typedef struct pr_depth_map_desc {
    uint32_t size;
    uint32_t n_tris;
    uint32_t n_objects;
    int32_t  width, height;
    uint32_t reserved;
    const float*     pos;      /* DEVICE [n_tris][3][4] Vertex.Pos */
    const pr_object* objects;  /* HOST [n_objects]: first_tri, n_tris, model */
    float view[16];            /* light camera View (row-major) */
    float proj[16];            /* light camera Proj */
    float* depth;              /* DEVICE [height][width] map, texel x + y*width */
    void*  stream;             /* cudaStream_t; NULL = the default stream */
} pr_depth_map_desc;

int pr_depth_map_noalloc(const pr_depth_map_desc* desc);

/* ---- batched rendering ------------------------------------------------------
 * No counterpart in the reference, where one Renderer renders one view at a
 * time: many views, each with its own scene (uploaded once to the batch),
 * camera, lights and outputs, rendered as one GPU job. Every view is the
 * first Render() of a fresh renderer: its shadow maps start zeroed. Results
 * are those pr_render gives for the view on a fresh context, bit for bit.
 *
 * The work runs as a fixed sequence of multi-view launches, captured once
 * per batch shape in a CUDA graph and relaunched: triangle setup of every
 * shadow pass (one per view and casting light) and of every view, then one
 * persistent raster launch over a global queue of (pass, 32-task) work
 * items, then resolve, shading and AO of every view. pr_batch_tune times the
 * raster task size and the persistent grid over candidates and keeps the
 * fastest, and sizes the record and task capacities from the needs it saw.
 * Each view's outputs must be device pointers (PR_OUT_DEVICE_PTRS) with rgba
 * set; shadow_maps output is not supported in a batch. */
typedef struct pr_batch_view {
    uint32_t scene;            /* index from pr_batch_add_scene */
    uint32_t reserved;
    const pr_frame_desc* frame;
    pr_outputs* out;
} pr_batch_view;

typedef struct pr_batch_stats {
    uint32_t size;
    uint32_t n_views;
    uint32_t n_passes;           /* raster passes: views + casting lights of each */
    uint32_t n_kernel_launches;  /* kernels in the batch's sequence */
    uint32_t graph_reused;       /* 1: the last batch relaunched a captured graph */
    uint32_t n_fallback_views;   /* views re-rendered alone (NaN depth in a shadow pass) */
    uint32_t n_retries;          /* re-runs after a capacity grew */
    uint32_t task_px;            /* pixels per raster task */
    uint32_t raster_blocks;      /* persistent raster grid */
    uint32_t reserved;
    double   ms_total;           /* device time of the last batch (CUDA events) */
    uint64_t device_bytes;       /* device memory held by the batch's work buffers */
} pr_batch_stats;

int pr_batch_create(int device, void** out_batch);
int pr_batch_destroy(void* batch);
int pr_batch_add_scene(void* batch, const pr_scene_desc* scene, uint32_t* out_index);
int pr_batch_render(void* batch, uint32_t n_views, const pr_batch_view* views);
/* Renders the batch under each candidate setting and keeps the fastest;
 * writes a JSON report (timings per candidate, chosen setting, capacities)
 * into report[report_cap] when report is not NULL. */
int pr_batch_tune(void* batch, uint32_t n_views, const pr_batch_view* views, char* report, size_t report_cap);
int pr_batch_get_stats(void* batch, pr_batch_stats* out);

/* ---- differentiable deferred shading --------------------------------------
 * No counterpart in the reference (which has no gradients): an adjoint of
 * the deferred-shading pass, shade + FragmentShader (render/raster.go:320-356,
 * shader/blinn_cpu.go:24-106), with visibility held fixed.
 *
 * pr_diff_forward renders a frame exactly as pr_render does (shadow maps,
 * raster, G-buffer, AO) and, from it, a float "radiance" image and a
 * per-pixel differentiation G-buffer (PR_DGB_FLOATS floats a pixel: the
 * triangle, its material, the screen barycentric weights of the pixel centre
 * in the input triangle, the world position, the face normal and the fixed
 * factor w_shadow * w_ao). Radiance, per pixel and channel c:
 *   material pixels: fac * clamp(La_c + kd_c Ld_c + ks_c Ls_c, 0, 255), the
 *     pre-Round value of FragmentShader with kd/ks = Diffuse/255,
 *     Specular/255 as floats and the interpolated normal n = unit(sum_k b_k N_k)
 *     (N_k = NormalMatrix * vertex normal), or face normal when flat;
 *     fac = 0.5^visibles (shadows) * float32(Pow(T, 10000)) (AO);
 *   material-less pixels: 255 * sum_k p_k C_k, the perspective-correct
 *     interpolation of the vertex colours C_k (in [0,1]);
 *   background: the background colour.
 * pr_diff_backward takes dL/d(radiance) and that G-buffer, recomputes every
 * interpolated attribute and per-light term from it (nothing per light is
 * stored), and returns dL/d of: vertex colours and normals, kd, ks,
 * shininess, light positions and intensities, ambient intensities. */
#define PR_DGB_FLOATS 16

typedef struct pr_diff_params {
    uint32_t size;
    uint32_t n_materials;        /* entries of kd/ks/shininess (= the scene's) */
    const float* vertex_color;   /* DEVICE [n_tris][3][4] RGBA in [0,1]; NULL: scene RGBA8 / 255 */
    const float* vertex_normal;  /* DEVICE [n_tris][3][4] object-space normals; NULL: the scene's */
    const float* kd;             /* HOST [n_materials][3] in [0,1]; NULL: scene Diffuse / 255 */
    const float* ks;             /* HOST [n_materials][3]; NULL: scene Specular / 255 */
    const float* shininess;      /* HOST [n_materials]; NULL: the scene's */
} pr_diff_params;

typedef struct pr_diff_grads {
    uint32_t size;
    uint32_t reserved;
    float*  vertex_color;        /* DEVICE [n_tris][3][4], overwritten; NULL: not wanted */
    float*  vertex_normal;       /* DEVICE [n_tris][3][4] (w = 0), overwritten; NULL: not wanted */
    double* kd;                  /* HOST [n_materials][3] */
    double* ks;                  /* HOST [n_materials][3] */
    double* shininess;           /* HOST [n_materials] */
    double* light_pos;           /* HOST [n_lights][3] (0 for directional lights) */
    double* light_intensity;     /* HOST [n_lights] */
    double* ambient;             /* HOST [n_ambient] */
} pr_diff_grads;

/* radiance: DEVICE [H][W][4] (alpha = the frame's alpha); gbuf: DEVICE
 * [H][W][PR_DGB_FLOATS]; out: optional further outputs (device pointers,
 * PR_OUT_DEVICE_PTRS), as pr_render. Rows top-down. Returns when done. */
int pr_diff_forward(void* ctx, const pr_frame_desc* frame, const pr_diff_params* params, float* radiance,
                    float* gbuf, pr_outputs* out);
/* frame and params as given to the pr_diff_forward that produced gbuf;
 * grad_radiance: DEVICE [H][W][4] (alpha ignored). Returns when done. */
int pr_diff_backward(void* ctx, const pr_frame_desc* frame, const pr_diff_params* params, const float* gbuf,
                     const float* grad_radiance, pr_diff_grads* grads);

/* ---- OBJ / MTL parsing ------------------------------------------------
 * Replaces model/obj/obj.go: obj.Load's line parsers (File.parse,
 * parseObjLine, parseMtlLine, obj.go:139-611) as one pass over a text
 * buffer; the host keeps the file handling of obj.Load (obj.go:78-137: which
 * .mtl to read, the fallback to <name>.mtl, default materials when the .mtl
 * fails) and model.Load's mesh assembly (model/load.go:40-152). Host only:
 * no CUDA call, no device needed.
 *
 * A handle holds one obj.File's state. Feed it the .obj text, then the .mtl
 * text, in the reference's order: the current material carries over from
 * the .obj into the .mtl as it does in the reference. Numbers parse as Go's
 * strconv.ParseFloat(s, 32) / ParseInt(s, 10, 32) / ParseUint(s, 10, 32).
 *
 * pr_obj_parse returns PR_ERR_INVALID_ARG where obj.go returns an error
 * (message in pr_last_error(): "<what> in line:<n>" or strconv's text), and
 * PR_ERR_FATAL where the reference panics (an .mtl property before any
 * material, a colour outside [0, 1]). Lines before the failing one stay
 * parsed. */
#define PR_OBJ_TEXT_OBJ  0
#define PR_OBJ_TEXT_MTL  1
#define PR_OBJ_NO_INDEX  4294967295LL  /* obj.go's invINDEX: corner without vt / vn */

typedef struct pr_obj_material {  /* obj.Material (obj.go:57-68) */
    int32_t name;          /* offset of the name in pr_obj_info.strings */
    int32_t map_kd;        /* offset of map_Kd's file name; -1: none */
    int32_t illum;
    float   opacity;       /* d */
    float   refraction;    /* Ni */
    float   shininess;     /* Ns */
    uint8_t ambient[4];    /* Ka, Kd, Ks, Ke through color.FromValue; alpha 255 */
    uint8_t diffuse[4];
    uint8_t specular[4];
    uint8_t emissive[4];
} pr_obj_material;

typedef struct pr_obj_info {     /* views into the handle, valid until its next parse or destroy */
    uint32_t size;               /* sizeof(pr_obj_info), set by the caller */
    uint32_t reserved;
    const float* vertices;  int64_t n_vertices;   /* [n][3], 'v' with w divided in */
    const float* normals;   int64_t n_normals;    /* [n][3] */
    const float* uvs;       int64_t n_uvs;        /* [n][2] */
    int64_t n_faces;
    int64_t n_corners;
    const int64_t* face_start;      /* [n_faces + 1]: corners of face i are [face_start[i], face_start[i+1]) */
    const int64_t* corner_v;        /* [n_corners] 0-based; relative indices resolved (may be out of range) */
    const int64_t* corner_vt;       /* [n_corners]; PR_OBJ_NO_INDEX when absent */
    const int64_t* corner_vn;       /* [n_corners]; PR_OBJ_NO_INDEX when absent */
    const int32_t* face_object;     /* [n_faces] object of each face */
    const int32_t* face_material;   /* [n_faces] material index; -1: obj.go's "polyred_default" */
    const uint8_t* face_smooth;     /* [n_faces] */
    int64_t n_objects;               /* 'o' / 'g' lines and implicit "unnamed<line>" objects */
    const int32_t* object_name;      /* [n_objects] string offsets */
    const int64_t* object_mat_start; /* [n_objects + 1] ranges of object_mat */
    const int32_t* object_mat;       /* Object.Materials as material indices */
    int64_t n_materials;             /* in order of first mention */
    const pr_obj_material* materials;
    int64_t n_warnings;
    const int32_t* warnings;         /* string offsets, File.Warnings */
    /* string entries: a native-endian uint32 length n, n bytes (which may
     * hold NUL, as Go strings may), a NUL */
    const char* strings;  int64_t strings_len;
    int32_t matlib;                  /* last mtllib file name; -1: none */
    int32_t current_material;        /* matCurrent; -1: none */
    int64_t line;                    /* File.line after the last parse */
    const char* error;  int64_t error_len;  /* the last parse's error message, all its bytes; empty: none */
} pr_obj_info;

int pr_obj_create(void** out);
int pr_obj_destroy(void* obj);
/* kind: PR_OBJ_TEXT_OBJ or PR_OBJ_TEXT_MTL; text need not be NUL-terminated */
int pr_obj_parse(void* obj, int kind, const char* text, size_t len);
int pr_obj_get(void* obj, pr_obj_info* out);

/* ---- image helpers for texture loading --------------------------------
 * imageutil.LoadImage (internal/imageutil/image.go:47-106) decodes an image
 * file, converts it to image.RGBA and, with GammaCorrect(true), maps R, G, B
 * from sRGB to linear. Host only. */
/* The byte map of that gamma correction: out[b] = uint8(FromsRGB2Linear(
 * float32(b)/0xff)*0xff + 0.5) (color/srgb.go:35-75). */
int pr_srgb_decode_table(uint8_t out[256]);
/* PNG scanline reconstruction (the five filter types of the PNG
 * specification, as Go's image/png undoes them): `in` holds height rows of
 * a filter byte and row_bytes bytes, bpp = bytes per complete pixel (at
 * least 1); writes height rows of row_bytes bytes to out. PR_ERR_INVALID_ARG
 * for an unknown filter type. */
int pr_png_unfilter(const uint8_t* in, int height, size_t row_bytes, int bpp, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif /* POLYRED_CUDA_H */
