// oracle.h — C API of the CPU oracle (liboracle.so).
//
// TEST INFRASTRUCTURE: loaded only by tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg, to compare with. It shares the scene/frame/
// output descriptors of include/polyred_cuda.h so both sides read the same
// inputs.
#pragma once

#include "../include/polyred_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_stats {
    uint32_t n_clipped;  // input triangles that went through clipTriangle
} orc_stats;

// One Render() of the reference in single-worker order. shadow_state is the
// persistent [n_lights][SH][SW] shadow-map storage (read, then updated), or
// NULL for zeroed maps. threads > 1 splits rows (same result, see oracle.cpp).
/* imageutil.Resize (internal/imageutil/resize.go:16-181) of a dx x dy RGBA
 * image, rows top-down, to w x h */
int orc_resize(const uint8_t* img, int dx, int dy, int w, int h, uint8_t* out);
/* NewTexture's levels and Texture.Query (buffer/texture.go:35-187), for tests */
long long orc_texture_build(int w, int h, const uint8_t* rgba, int mipmap, uint8_t* out, size_t cap, int32_t* desc);
int orc_texture_query(int w, int h, const uint8_t* rgba, int mipmap, int n, const float* lod, const float* du,
                      const float* dv, const float* u, const float* v, uint8_t* out);
int orc_render(const pr_scene_desc* scene, const pr_frame_desc* frame, float* shadow_state, int threads,
               pr_outputs* out, orc_stats* stats);

// The 8 AO march directions of material/ao.go:28 (float32 angle accumulation).
void orc_ao_directions(float cosv[8], float sinv[8], int* n);

// Building blocks, for the known-answer tests.
void orc_barycoord(const float p[2], const float t1[2], const float t2[2], const float t3[2], float out[3]);
void orc_view_matrix(const float pos[3], const float target[3], const float up[3], float out[16]);
void orc_perspective_matrix(float fov, float aspect, float n, float f, float out[16]);
void orc_ortho_matrix(float l, float r, float b, float t, float n, float f, float out[16]);
void orc_mat4_mul(const float a[16], const float b[16], float out[16]);
int orc_mat4_inv(const float m[16], float out[16]);
int orc_aabb_intersect(const float a_min[3], const float a_max[3], const float b_min[3], const float b_max[3]);
int orc_aabb_contains(const float a_min[3], const float a_max[3], const float* pts, int n);
void orc_new_aabb(const float* pts, int n, float out_min[3], float out_max[3]);
int orc_tri_is_valid(const float p1[4], const float p2[4], const float p3[4]);
void orc_tri_face_normal(const float p1[4], const float p2[4], const float p3[4], float out[4]);
void orc_fragment_shader(const pr_material* m, const float nor[4], const float face_nor[4], const float wpos[4],
                         const float cam[3], const pr_light* lights, int n_lights, const float* ambient,
                         int n_ambient, uint8_t out[4]);
void orc_interp_world_pos(const float bc[3], const float m1[4], const float m2[4], const float m3[4], float out[4]);
void orc_gamma_table(uint8_t out[256]);
float orc_from_linear_srgb(float v);
double orc_go_pow(double x, double y);
double orc_go_atan(double x);
float orc_fma32(float x, float y, float z);
int64_t orc_go_f2i(float x);
uint8_t orc_go_f2u8(float x);
int orc_shadow_camera(const float light_pos[3], const float center[3], const float cam_view[16],
                      const float cam_proj[16], float out_view[16], float out_proj[16]);

#ifdef __cplusplus
}
#endif
