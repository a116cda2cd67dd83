// Material textures on the host: buffer.NewTexture's mipmap (buffer/texture.go:35-67),
// each level imageutil.Resize of the image (internal/imageutil/resize.go:16-181),
// packed for the shade kernel; and the host instance of the texture query
// (pr_texture.h) behind two test entry points.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/polyred_cuda.h"
#include "../../include/polyred_cuda_testing.h"
#include "pr_texture.h"

namespace prk {
int set_last_error(int status, const char* msg);
}

namespace prh {

namespace {

struct Img {
    int w = 0, h = 0;
    std::vector<uint32_t> px;  // packed RGBA8, rows top-down
};

// linear() of resize.go
float linear_kernel(float in) {
    in = std::fabs(in);
    if (in <= 1) return 1 - in;
    return 0;
}

// createWeights8 (resize.go:161-181) with filterLength 2 and linear():
// int16 taps (x256, truncated) and the first input index of every output.
int weights8(int dy, float scale, std::vector<int16_t>& coeffs, std::vector<int>& start) {
    const int len = 2 * (int)(float)prt::go_max(-DBL_MAX, prt::go_max((double)std::ceil(scale), 1.0));
    const float factor = std::min(1.0f / scale, 1.0f);
    coeffs.assign((size_t)dy * len, 0);
    start.assign(dy, 0);
    for (int y = 0; y < dy; y++) {
        float interp = scale * ((float)y + 0.5f) - 0.5f;
        start[y] = (int)interp - len / 2 + 1;
        interp -= (float)start[y];
        for (int i = 0; i < len; i++) coeffs[(size_t)y * len + i] = (int16_t)(linear_kernel((interp - (float)i) * factor) * 256);
    }
    return len;
}

// resizeRGBA (resize.go:79-121): output row y, column x from input row x
// (each pass transposes).
void resize_pass(const Img& in, Img& out, const std::vector<int16_t>& coeffs, const std::vector<int>& start, int len) {
    const int maxX = in.w - 1;
    for (int x = 0; x < out.w; x++) {
        const uint32_t* row = in.px.data() + (size_t)x * in.w;
        for (int y = 0; y < out.h; y++) {
            int32_t acc[4] = {0, 0, 0, 0}, sum = 0;
            for (int i = 0; i < len; i++) {
                const int32_t c = coeffs[(size_t)y * len + i];
                if (c == 0) continue;
                int xi = start[y] + i;
                xi = (unsigned)xi < (unsigned)maxX ? xi : (xi >= maxX ? maxX : 0);
                const uint32_t p = row[xi];
                for (int k = 0; k < 4; k++) acc[k] += c * (int32_t)((p >> (8 * k)) & 0xffu);
                sum += c;
            }
            uint32_t o = 0;
            for (int k = 0; k < 4; k++) {
                const int v = acc[k] / sum;
                o |= (uint32_t)std::min(std::max(v, 0), 255) << (8 * k);
            }
            out.px[(size_t)y * out.w + x] = o;
        }
    }
}

// imageutil.Resize(width, height, img); a zero width or height follows the
// other's scale (calcFactors, resize.go:124-144).
Img go_resize(int width, int height, const Img& img) {
    const float ow = (float)img.w, oh = (float)img.h;
    float sx, sy;
    if (width == 0) {
        if (height == 0) {
            sx = sy = 1.0f;
        } else {
            sy = oh / (float)height;
            sx = sy;
        }
    } else {
        sx = ow / (float)width;
        sy = height == 0 ? sx : oh / (float)height;
    }
    if (width == 0) width = (int)(0.7f + ow / sx);
    if (height == 0) height = (int)(0.7f + oh / sy);
    if (width == img.w && height == img.h) return img;
    if (img.w <= 0 || img.h <= 0) return img;
    Img temp, out;
    temp.w = img.h;
    temp.h = width;
    temp.px.assign((size_t)temp.w * temp.h, 0);
    out.w = width;
    out.h = height;
    out.px.assign((size_t)out.w * out.h, 0);
    std::vector<int16_t> coeffs;
    std::vector<int> start;
    int len = weights8(temp.h, sx, coeffs, start);
    resize_pass(img, temp, coeffs, start, len);
    len = weights8(out.h, sy, coeffs, start);
    resize_pass(temp, out, coeffs, start, len);
    return out;
}

}  // namespace

// The texture of one material: level 0 the image, then (with mipmaps)
// NewTexture's levels, each a Resize of the image to dx/2^i x dy/2^i.
// Appends the texels and fills the descriptor.
int build_texture(int w, int h, const uint8_t* rgba, bool mipmap, std::vector<uint32_t>& texels, prt::TexDesc& d) {
    if (w < 1 || h < 1 || w > 16384 || h > 16384 || !rgba) return -1;
    Img img;
    img.w = w;
    img.h = h;
    img.px.resize((size_t)w * h);
    std::memcpy(img.px.data(), rgba, img.px.size() * 4);
    std::memset(&d, 0, sizeof(d));
    d.use_mipmap = mipmap ? 1 : 0;
    d.size = w;
    int L = 1;
    if (mipmap && !(w == 1 && h == 1)) L = (int)(float)prt::go_log2((double)std::max((float)w, (float)h)) + 1;
    if (L > prt::kMaxTexLevels) return -1;
    d.n_levels = L;
    for (int i = 0; i < L; i++) {
        Img lv;
        const Img* src = &img;
        if (i > 0) {
            lv = go_resize(w / (1 << i), h / (1 << i), img);
            src = &lv;
        }
        d.w[i] = src->w;
        d.h[i] = src->h;
        d.off[i] = (uint32_t)texels.size();
        texels.insert(texels.end(), src->px.begin(), src->px.end());
    }
    return 0;
}

}  // namespace prh

// ---- host image helpers (ABI) ----

namespace prh {
void srgb_decode_table(uint8_t out[256]);
}

extern "C" {

int pr_srgb_decode_table(uint8_t out[256]) {
    if (!out) return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_srgb_decode_table: NULL argument");
    prh::srgb_decode_table(out);
    return PR_OK;
}

int pr_png_unfilter(const uint8_t* in, int height, size_t row_bytes, int bpp, uint8_t* out) {
    if ((!in || !out) && height > 0) return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_png_unfilter: NULL argument");
    if (height < 0 || bpp < 1 || bpp > 8) return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_png_unfilter: bad size");
    const uint8_t* prev = nullptr;
    for (int y = 0; y < height; y++) {
        const uint8_t* src = in + (size_t)y * (row_bytes + 1);
        const uint8_t f = src[0];
        src++;
        uint8_t* cur = out + (size_t)y * row_bytes;
        switch (f) {
            case 0:  // None
                std::memcpy(cur, src, row_bytes);
                break;
            case 1:  // Sub
                for (size_t i = 0; i < row_bytes; i++) cur[i] = (uint8_t)(src[i] + (i >= (size_t)bpp ? cur[i - bpp] : 0));
                break;
            case 2:  // Up
                for (size_t i = 0; i < row_bytes; i++) cur[i] = (uint8_t)(src[i] + (prev ? prev[i] : 0));
                break;
            case 3:  // Average
                for (size_t i = 0; i < row_bytes; i++) {
                    const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
                    cur[i] = (uint8_t)(src[i] + ((a + b) >> 1));
                }
                break;
            case 4:  // Paeth
                for (size_t i = 0; i < row_bytes; i++) {
                    const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
                    const int c = (i >= (size_t)bpp && prev) ? prev[i - bpp] : 0;
                    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                    const int pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    cur[i] = (uint8_t)(src[i] + pred);
                }
                break;
            default:
                return prk::set_last_error(PR_ERR_INVALID_ARG, "png: invalid format: bad filter type");
        }
        prev = cur;
    }
    return PR_OK;
}

}  // extern "C"

// ---- test entry points (include/polyred_cuda_testing.h) ----

extern "C" {

// The levels build_texture makes: texels into `out` (capacity `cap`
// texels), levels as [n, w0, h0, off0, w1, h1, off1, ...] into `desc`
// (1 + 3 * 16 ints). Returns the texel count, or a negative status.
long long pr_debug_texture_build(int w, int h, const uint8_t* rgba, int mipmap, uint32_t* out, size_t cap,
                                 int32_t* desc) {
    std::vector<uint32_t> tx;
    prt::TexDesc d;
    if (prh::build_texture(w, h, rgba, mipmap != 0, tx, d)) return PR_ERR_INVALID_ARG;
    if (out && tx.size() <= cap) std::memcpy(out, tx.data(), tx.size() * 4);
    if (desc) {
        desc[0] = d.n_levels;
        for (int i = 0; i < prt::kMaxTexLevels; i++) {
            desc[1 + 3 * i] = d.w[i];
            desc[2 + 3 * i] = d.h[i];
            desc[3 + 3 * i] = (int32_t)d.off[i];
        }
    }
    return (long long)tx.size();
}

// Texture.Query of n (lod, u, v) triples on that texture, and when du / dv
// are given, the FragmentShader lod of (du[k], dv[k]) in place of lod[k].
int pr_debug_texture_query(int w, int h, const uint8_t* rgba, int mipmap, int n, const float* lod, const float* du,
                           const float* dv, const float* u, const float* v, uint8_t* out) {
    std::vector<uint32_t> tx;
    prt::TexDesc d;
    if (prh::build_texture(w, h, rgba, mipmap != 0, tx, d) || n < 0 || !u || !v || !out || (!lod && !(du && dv)))
        return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_debug_texture_query: bad arguments");
    for (int k = 0; k < n; k++) {
        const float l = (du && dv) ? prt::tex_lod(d, du[k], dv[k]) : lod[k];
        const uint32_t c = prt::tex_query(d, tx.data(), l, u[k], v[k]);
        std::memcpy(out + 4 * k, &c, 4);
    }
    return PR_OK;
}

}  // extern "C"
