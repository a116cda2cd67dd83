// pr_hostmath.h — host-side float32 matrix math with the reference's exact
// evaluation order (math/mat4.go, camera/*.go, math/vec3.go). Compiled with
// -ffp-contract=off so no multiply-add is fused, as Go amd64 evaluates it.
#pragma once

#include <cstdint>

namespace prh {

struct M4 {
    float m[16];
};

M4 mulm(const M4& a, const M4& b);                       // Mat4.MulM (math/mat4.go:201-220)
bool inv(const M4& a, M4* out);                          // Mat4.Inv (math/mat4.go:259-283)
M4 transpose(const M4& a);                               // Mat4.T (math/mat4.go:249-256)
M4 viewport(float w, float h);                           // math.ViewportMatrix (math/math.go:270-277)
M4 view_matrix(const float pos[3], const float target[3], const float up[3]);  // camera/camera.go:42-53
M4 perspective(float fov, float aspect, float n, float f);                      // camera/perspective.go:100-111
M4 ortho(float l, float r, float b, float t, float n, float f);                 // camera/orthographic.go:106-119
bool shadow_camera(const float light_pos[3], const float center[3], const M4& cam_view, const M4& cam_proj,
                   M4* out_view, M4* out_proj);          // render/shadow.go:41-85
void gamma_table(uint8_t out[256]);                      // shader/gamma.go:13-18 + color/srgb.go
void srgb_decode_table(uint8_t out[256]);                // LoadImage's GammaCorrect map (color/srgb.go)
void ao_directions(float cosv[8], float sinv[8], int* n); // material/ao.go:28
// Which AO directions may use the device's tap offset table on a W x H frame
// (fast[k]), and which component is tiny and negative (tiny[k]: 0, 1 = x, 2 = y).
// Returns half an ulp of float32 at max(W, H) + 100, which bounds the
// rounding of every tap coordinate.
float ao_classify(const float cosv[8], const float sinv[8], int n, int W, int H, int8_t fast[8], int8_t tiny[8]);

}  // namespace prh
