/* A plain C host of libpolyred_cuda.so: everything below goes through
 * include/polyred_cuda.h alone, as a C or C++ program (or a cgo / JNI /
 * N-API shim) would use the library. Prints one "key value..." line per
 * check; tests/test_c_host.py compiles it, runs it and compares the values
 * with the Python host's.
 *
 *   pr_c_host            host-only entry points; pr_create must report
 *                        PR_ERR_NO_DEVICE when no GPU is visible
 *   pr_c_host --render   also renders a one-triangle scene at 64x64 on GPU 0
 */
#include <stdio.h>
#include <stdint.h>
#include <string.h>

#include "polyred_cuda.h"

#define CHECK(call)                                                                    \
    do {                                                                               \
        int rc_ = (call);                                                              \
        if (rc_ != PR_OK) {                                                            \
            printf("fail %s %d %s\n", #call, rc_, pr_last_error());                   \
            return 1;                                                                  \
        }                                                                              \
    } while (0)

static uint32_t bits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

static void print_matrix(const char* name, const float m[16]) {
    printf("%s", name);
    for (int i = 0; i < 16; i++) printf(" %08x", bits(m[i]));
    printf("\n");
}

static int render_triangle(void) {
    void* ctx = NULL;
    CHECK(pr_create(0, &ctx));
    /* one triangle facing the camera, material 0 */
    const float pos[3][4] = {{-1, -1, 0, 1}, {1, -1, 0, 1}, {0, 1, 0, 1}};
    const float nor[3][4] = {{0, 0, 1, 0}, {0, 0, 1, 0}, {0, 0, 1, 0}};
    const float uv[3][2] = {{0, 0}, {1, 0}, {0, 1}};
    const uint8_t col[3][4] = {{255, 255, 255, 255}, {255, 255, 255, 255}, {255, 255, 255, 255}};
    const int32_t mat_id[1] = {0};
    pr_object obj;
    memset(&obj, 0, sizeof obj);
    obj.first_tri = 0;
    obj.n_tris = 1;
    obj.mat_base = 0;
    for (int i = 0; i < 16; i++) obj.model[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    pr_material mat;
    memset(&mat, 0, sizeof mat);
    const uint8_t kd[4] = {204, 77, 51, 255}, ks[4] = {128, 128, 128, 255}, tex[4] = {255, 255, 255, 255};
    memcpy(mat.diffuse, kd, 4);
    memcpy(mat.specular, ks, 4);
    memcpy(mat.texture, tex, 4);
    mat.shininess = 32;
    mat.flags = PR_MAT_MIPMAP;
    mat.texture_size = 1;
    pr_scene_desc scene;
    memset(&scene, 0, sizeof scene);
    scene.size = sizeof scene;
    scene.n_tris = 1;
    scene.n_objects = 1;
    scene.n_materials = 1;
    scene.pos = &pos[0][0];
    scene.nor = &nor[0][0];
    scene.uv = &uv[0][0];
    scene.col = &col[0][0];
    scene.mat_id = mat_id;
    scene.objects = &obj;
    scene.materials = &mat;
    CHECK(pr_scene_upload(ctx, &scene));

    pr_frame_desc f;
    memset(&f, 0, sizeof f);
    f.size = sizeof f;
    f.flags = PR_FRAME_PERSPECTIVE | PR_FRAME_GAMMA;
    f.width = 64;
    f.height = 64;
    const float eye[3] = {0, 0, 4}, target[3] = {0, 0, 0}, up[3] = {0, 1, 0};
    CHECK(pr_view_matrix(eye, target, up, f.view));
    CHECK(pr_perspective_matrix(45.0f, 1.0f, 0.1f, 100.0f, f.proj));
    memcpy(f.cam_pos, eye, sizeof eye);
    pr_light light;
    memset(&light, 0, sizeof light);
    light.type = PR_LIGHT_POINT;
    light.pos[0] = 2;
    light.pos[1] = 2;
    light.pos[2] = 4;
    light.intensity = 1;
    memset(light.color, 255, 4);
    const float ambient[1] = {0.1f};
    f.n_lights = 1;
    f.lights = &light;
    f.n_ambient = 1;
    f.ambient = ambient;
    f.msaa = 1;

    static uint8_t rgba[64 * 64 * 4];
    static uint32_t tri_id[64 * 64];
    pr_outputs out;
    memset(&out, 0, sizeof out);
    out.size = sizeof out;
    out.rgba = rgba;
    out.tri_id = tri_id;
    CHECK(pr_render(ctx, &f, &out));
    int covered = 0, lit = 0;
    for (int i = 0; i < 64 * 64; i++) {
        if (tri_id[i] == 0) covered++;
        else if (tri_id[i] != PR_TRI_NONE) {
            printf("fail tri_id %u at %d\n", tri_id[i], i);
            return 1;
        }
        if (tri_id[i] == 0 && (rgba[4 * i] | rgba[4 * i + 1] | rgba[4 * i + 2])) lit++;
    }
    printf("render covered %d lit %d\n", covered, lit);
    CHECK(pr_destroy(ctx));
    return 0;
}

int main(int argc, char** argv) {
    const int render = argc > 1 && strcmp(argv[1], "--render") == 0;
    printf("abi %d %d\n", pr_abi_version(), PR_ABI_VERSION);

    /* host matrices, as the reference's camera package builds them */
    float view[16], proj[16], pv[16], inv[16];
    const float eye[3] = {0, 1.5f, 4}, target[3] = {0, 0, 0}, up[3] = {0, 1, 0};
    CHECK(pr_view_matrix(eye, target, up, view));
    CHECK(pr_perspective_matrix(45.0f, 1.6f, 0.1f, 100.0f, proj));
    CHECK(pr_mat4_mul(proj, view, pv));
    CHECK(pr_mat4_inv(pv, inv));
    print_matrix("view", view);
    print_matrix("proj", proj);
    print_matrix("pv", pv);
    print_matrix("inv", inv);
    const float zero[16] = {0};
    printf("singular %d\n", pr_mat4_inv(zero, inv));

    /* OBJ parsing, and an error with obj.go's message */
    const char* text = "o tri\nv 0 0 0\nv 1 0 0\nv 0 1 0 2\nvt 0 0\nf 1/1 2/1 3/1\nf -3 -2 -1\n";
    void* h = NULL;
    CHECK(pr_obj_create(&h));
    CHECK(pr_obj_parse(h, PR_OBJ_TEXT_OBJ, text, strlen(text)));
    pr_obj_info info;
    memset(&info, 0, sizeof info);
    info.size = sizeof info;
    CHECK(pr_obj_get(h, &info));
    printf("obj %lld %lld %lld %lld %08x %lld\n", (long long)info.n_vertices, (long long)info.n_faces,
           (long long)info.n_objects, (long long)info.corner_vt[3], bits(info.vertices[7]),
           (long long)info.corner_v[5]);
    const char* bad = "v 1 2\n";
    const int bad_rc = pr_obj_parse(h, PR_OBJ_TEXT_OBJ, bad, strlen(bad));  /* before reading its message */
    printf("obj_error %d %s\n", bad_rc, pr_last_error());
    CHECK(pr_obj_destroy(h));

    /* texture image helpers */
    uint8_t table[256];
    CHECK(pr_srgb_decode_table(table));
    printf("srgb %d %d %d\n", table[64], table[128], table[200]);
    const uint8_t filtered[2 * 7] = {1, 10, 20, 30, 1, 1, 1, 2, 5, 5, 5, 5, 5, 5};
    uint8_t row[2 * 6];
    CHECK(pr_png_unfilter(filtered, 2, 6, 3, row));
    printf("unfilter");
    for (int i = 0; i < 12; i++) printf(" %d", row[i]);
    printf("\n");

    /* a device context */
    void* ctx = NULL;
    const int rc = pr_create(0, &ctx);
    printf("create %d\n", rc);
    if (rc == PR_OK) CHECK(pr_destroy(ctx));
    if (render) return render_triangle();
    return 0;
}
