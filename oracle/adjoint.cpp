// FP64 reference for differentiable deferred shading (TEST INFRASTRUCTURE).
//
// The float radiance of the shade pass with visibility fixed by a
// differentiation G-buffer, and its adjoint, both in float64. It restates the
// same model as the device (pre-Round values of FragmentShader,
// shader/blinn_cpu.go:24-106, times the fixed shadow / AO factor of
// render/raster.go:339-356 and material/ao.go:34-37; material-less pixels show
// the perspective-correct interpolation of vertex colours,
// render/raster.go:324-334, 546-549). The tests compare the GPU radiance,
// the GPU gradients and (through orc_diff_forward64) central finite
// differences with it.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct D3 { double x, y, z; };
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double nrm(D3 a) { return std::sqrt(dot(a, a)); }

const uint32_t kLit = 1u, kFlat = 2u, kConst = 4u, kUnlit = 8u;
// orc_diff_in.flags: the backward accumulates majorants instead of the
// gradients: per pixel its terms with every factor and sum replaced by
// magnitudes (majorants()), which bound the rounding error of a float32
// evaluation of the gradient.
const int32_t kAbs = 1;

}  // namespace

extern "C" {

typedef struct orc_diff_in {
    int32_t W, H;
    const float* gbuf;          // [H*W][16]
    uint32_t n_tris;
    uint32_t n_objects;
    const double* vcol;         // [n_tris*3][4] in [0,1]
    const double* vnor;         // [n_tris*3][4] object space
    const uint32_t* obj_first;  // [n_objects]
    const float* obj_normal;    // [n_objects][16]
    int32_t n_mats;
    int32_t n_lights;
    const double* kd;           // [n_mats][3]
    const double* ks;           // [n_mats][3]
    const double* shin;         // [n_mats]
    const uint8_t* tex;         // [n_mats][4]
    const int32_t* ltype;       // [n_lights] 0 point, 1 directional
    const double* lpos;         // [n_lights][3]
    const float* ldir;          // [n_lights][3]
    const double* lint;         // [n_lights]
    const uint8_t* lcol;        // [n_lights][4]
    int32_t n_amb;
    int32_t only_tri;           // >= 0: only pixels of this triangle
    const double* amb;          // [n_amb]
    double cam[3];
    double bg[4];
    int32_t only_mat;           // >= 0: only pixels of this material
    int32_t flags;              // kAbs: accumulate |contribution| of every pixel
} orc_diff_in;

typedef struct orc_diff_out {
    double* vcol;   // [n_tris*3][4]
    double* vnor;   // [n_tris*3][4]
    double* kd;     // [n_mats][3]
    double* ks;     // [n_mats][3]
    double* shin;   // [n_mats]
    double* lpos;   // [n_lights][3]
    double* lint;   // [n_lights]
    double* amb;    // [n_amb]
} orc_diff_out;

}  // extern "C"

namespace {

uint32_t find_obj(const orc_diff_in* in, uint32_t t) {
    uint32_t lo = 0, hi = in->n_objects - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (in->obj_first[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Per light of one pixel: direction, half vector, intensity, distance and
// the clamped diffuse and specular terms.
struct LT { D3 L, H; double I, dist, hlen, nd, nh, ld, ls; };

inline D3 absv(D3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }

// The absolute mode's contribution of one lit pixel: the backward's terms
// with every factor replaced by its magnitude and every sum by a sum of
// magnitudes (the projections of the unit-vector derivatives included), so
// that it bounds every intermediate a float32 evaluation of the pixel's
// gradient forms, before any cancellation: the scale of its rounding error.
void majorants(const orc_diff_in* in, orc_diff_out* out, uint32_t t, int32_t m, double fac, const double* pre,
               const double* g, const double* col, const double* kd, const double* ks, double s, bool flat, D3 n,
               double mlen, const float* M, const float* d, const std::vector<LT>& lt) {
    double ag[3];
    for (int c = 0; c < 3; c++) ag[c] = (pre[c] > 0.0 && pre[c] < 255.0) ? std::fabs(g[c] * fac) : 0.0;
    D3 Ld = {0, 0, 0}, Ls = {0, 0, 0};
    for (int l = 0; l < in->n_lights; l++) {
        Ld = Ld + (lt[l].ld * lt[l].I) * D3{col[0], col[1], col[2]};
        Ls = Ls + (lt[l].ls * lt[l].I) * D3{(double)in->lcol[4 * l], (double)in->lcol[4 * l + 1], (double)in->lcol[4 * l + 2]};
    }
    const double LdA[3] = {Ld.x, Ld.y, Ld.z}, LsA[3] = {Ls.x, Ls.y, Ls.z};
    for (int c = 0; c < 3; c++) {
        if (out->kd) out->kd[3 * m + c] += ag[c] * LdA[c];
        if (out->ks) out->ks[3 * m + c] += ag[c] * LsA[c];
    }
    const double gcol = ag[0] * col[0] + ag[1] * col[1] + ag[2] * col[2];
    for (int e = 0; e < in->n_amb; e++)
        if (out->amb) out->amb[e] += gcol;
    D3 gnA = {0, 0, 0};
    const D3 nA = absv(n);
    for (int l = 0; l < in->n_lights; l++) {
        const LT& q = lt[l];
        const double A = ag[0] * std::fabs(kd[0]) * col[0] + ag[1] * std::fabs(kd[1]) * col[1] + ag[2] * std::fabs(kd[2]) * col[2];
        const double B = ag[0] * std::fabs(ks[0]) * in->lcol[4 * l] + ag[1] * std::fabs(ks[1]) * in->lcol[4 * l + 1] +
                         ag[2] * std::fabs(ks[2]) * in->lcol[4 * l + 2];
        const double invd = in->ltype[l] == 0 ? 1.0 / q.dist : 1.0;
        if (out->lint) out->lint[l] += (A * q.ld + B * q.ls) * invd;
        const double nhc = std::fmin(std::fmax(q.nh, 0.0), 1.0);
        if (q.ls > 0.0 && nhc < 1.0 && out->shin) out->shin[m] += B * q.I * q.ls * std::fabs(std::log(nhc));
        const double gnd = (q.nd > 0.0 && q.nd < 1.0) ? A * q.I : 0.0;
        const double gnh = (q.nh > 0.0 && q.nh < 1.0) ? B * q.I * std::fabs(s) * std::pow(nhc, s - 1.0) : 0.0;
        const D3 LA = absv(q.L), HA = absv(q.H);
        gnA = gnA + gnd * LA + gnh * HA;
        if (in->ltype[l] == 0 && out->lpos) {
            const D3 gLA = gnd * nA + (gnh / q.hlen) * (nA + std::fabs(q.nh) * HA);
            const D3 gDA = (1.0 / q.dist) * (gLA + dot(LA, gLA) * LA) + ((A * q.ld + B * q.ls) * q.I / q.dist) * LA;
            out->lpos[3 * l] += gDA.x;
            out->lpos[3 * l + 1] += gDA.y;
            out->lpos[3 * l + 2] += gDA.z;
        }
    }
    if (!flat && out->vnor) {
        const D3 gmA = (1.0 / mlen) * (gnA + dot(nA, gnA) * nA);
        for (int k = 0; k < 3; k++) {
            const D3 gNA = std::fabs((double)d[4 + k]) * gmA;
            double* gv = out->vnor + 4 * (3 * (size_t)t + k);
            for (int j = 0; j < 3; j++)
                gv[j] += std::fabs(M[j]) * gNA.x + std::fabs(M[4 + j]) * gNA.y + std::fabs(M[8 + j]) * gNA.z;
        }
    }
}

// One pixel: radiance R[3]; with g != null also accumulates dL/d(params).
void pixel(const orc_diff_in* in, size_t i, double R[3], const double* g, orc_diff_out* out) {
    const bool absm = (in->flags & kAbs) != 0;
    auto acc = [absm](double& dst, double v) { dst += absm ? std::fabs(v) : v; };  // dst += v, or |v|
    const float* d = in->gbuf + 16 * i;
    uint32_t t, fl;
    int32_t m;
    std::memcpy(&t, d + 0, 4);
    std::memcpy(&m, d + 1, 4);
    std::memcpy(&fl, d + 2, 4);
    const double fac = d[3];
    R[0] = R[1] = R[2] = 0.0;
    if (t == 0xFFFFFFFFu) {
        for (int c = 0; c < 3; c++) R[c] = in->bg[c];
        return;
    }
    if (fl & kUnlit) {
        for (int k = 0; k < 3; k++) {
            const double p = d[4 + k];
            const double* C = in->vcol + 4 * (3 * (size_t)t + k);
            for (int c = 0; c < 3; c++) {
                R[c] += 255.0 * p * C[c];
                if (g && out->vcol) acc(out->vcol[4 * (3 * (size_t)t + k) + c], g[c] * 255.0 * p);
            }
        }
        return;
    }
    if (!(fl & (kLit | kConst)) || m < 0 || m >= in->n_mats) return;
    const uint8_t* tx = in->tex + 4 * m;
    const double col[3] = {(double)tx[0], (double)tx[1], (double)tx[2]};
    if (fl & kConst) {
        for (int c = 0; c < 3; c++) R[c] = fac * col[c];
        return;
    }
    const double* kd = in->kd + 3 * m;
    const double* ks = in->ks + 3 * m;
    const double s = in->shin[m];
    const D3 x = {d[8], d[9], d[10]};
    const bool flat = (fl & kFlat) != 0;
    D3 n, mv = {0, 0, 0};
    double mlen = 1.0;
    const float* M = nullptr;
    if (flat) {
        n = {d[12], d[13], d[14]};
    } else {
        M = in->obj_normal + 16 * (size_t)find_obj(in, t);
        for (int k = 0; k < 3; k++) {
            const double* v = in->vnor + 4 * (3 * (size_t)t + k);
            D3 N = {M[0] * v[0] + M[1] * v[1] + M[2] * v[2] + M[3] * v[3],
                    M[4] * v[0] + M[5] * v[1] + M[6] * v[2] + M[7] * v[3],
                    M[8] * v[0] + M[9] * v[1] + M[10] * v[2] + M[11] * v[3]};
            mv = mv + (double)d[4 + k] * N;
        }
        mlen = nrm(mv);
        n = (1.0 / mlen) * mv;
    }
    double La[3] = {0, 0, 0}, Ld[3] = {0, 0, 0}, Ls[3] = {0, 0, 0};
    for (int e = 0; e < in->n_amb; e++)
        for (int c = 0; c < 3; c++) La[c] += in->amb[e] * col[c];
    const D3 Vd = D3{in->cam[0], in->cam[1], in->cam[2]} - x;
    const D3 V = (1.0 / nrm(Vd)) * Vd;
    std::vector<LT> lt(in->n_lights);
    for (int l = 0; l < in->n_lights; l++) {
        LT& q = lt[l];
        if (in->ltype[l] == 0) {
            const D3 D = D3{in->lpos[3 * l], in->lpos[3 * l + 1], in->lpos[3 * l + 2]} - x;
            q.dist = nrm(D);
            q.L = (1.0 / q.dist) * D;
            q.I = in->lint[l] / q.dist;
        } else {
            q.L = {-(double)in->ldir[3 * l], -(double)in->ldir[3 * l + 1], -(double)in->ldir[3 * l + 2]};
            q.dist = 1.0;
            q.I = in->lint[l];
        }
        const D3 Hv = q.L + V;
        q.hlen = nrm(Hv);
        q.H = (1.0 / q.hlen) * Hv;
        q.nd = dot(n, q.L);
        q.nh = dot(n, q.H);
        q.ld = std::fmin(std::fmax(q.nd, 0.0), 1.0);
        const double nhc = std::fmin(std::fmax(q.nh, 0.0), 1.0);
        q.ls = nhc > 0.0 ? std::pow(nhc, s) : 0.0;
        for (int c = 0; c < 3; c++) {
            Ld[c] += q.ld * col[c] * q.I;
            Ls[c] += q.ls * in->lcol[4 * l + c] * q.I;
        }
    }
    double pre[3];
    for (int c = 0; c < 3; c++) {
        pre[c] = La[c] + kd[c] * Ld[c] + ks[c] * Ls[c];
        R[c] = fac * std::fmin(std::fmax(pre[c], 0.0), 255.0);
    }
    if (!g) return;
    if (absm) {
        majorants(in, out, t, m, fac, pre, g, col, kd, ks, s, flat, n, mlen, M, d, lt);
        return;
    }
    double gg[3];
    for (int c = 0; c < 3; c++) gg[c] = (pre[c] > 0.0 && pre[c] < 255.0) ? g[c] * fac : 0.0;
    for (int c = 0; c < 3; c++) {
        if (out->kd) acc(out->kd[3 * m + c], gg[c] * Ld[c]);
        if (out->ks) acc(out->ks[3 * m + c], gg[c] * Ls[c]);
    }
    const double gcol = gg[0] * col[0] + gg[1] * col[1] + gg[2] * col[2];
    for (int e = 0; e < in->n_amb; e++)
        if (out->amb) acc(out->amb[e], gcol);
    D3 gn = {0, 0, 0};
    for (int l = 0; l < in->n_lights; l++) {
        const LT& q = lt[l];
        const double A = gg[0] * kd[0] * col[0] + gg[1] * kd[1] * col[1] + gg[2] * kd[2] * col[2];
        const double B = gg[0] * ks[0] * in->lcol[4 * l] + gg[1] * ks[1] * in->lcol[4 * l + 1] +
                         gg[2] * ks[2] * in->lcol[4 * l + 2];
        if (out->lint) acc(out->lint[l], (A * q.ld + B * q.ls) * (in->ltype[l] == 0 ? 1.0 / q.dist : 1.0));
        const double nhc = std::fmin(std::fmax(q.nh, 0.0), 1.0);
        if (q.ls > 0.0 && nhc < 1.0 && out->shin) acc(out->shin[m], B * q.I * q.ls * std::log(nhc));
        const double gnd = (q.nd > 0.0 && q.nd < 1.0) ? A * q.I : 0.0;
        const double gnh = (q.nh > 0.0 && q.nh < 1.0) ? B * q.I * s * std::pow(nhc, s - 1.0) : 0.0;
        gn = gn + gnd * q.L + gnh * q.H;
        if (in->ltype[l] == 0 && out->lpos) {
            const D3 gL = gnd * n + (gnh / q.hlen) * (n - q.nh * q.H);
            const D3 gD = (1.0 / q.dist) * (gL - dot(q.L, gL) * q.L) + (-(A * q.ld + B * q.ls) * q.I / q.dist) * q.L;
            acc(out->lpos[3 * l], gD.x);
            acc(out->lpos[3 * l + 1], gD.y);
            acc(out->lpos[3 * l + 2], gD.z);
        }
    }
    if (!flat && out->vnor) {
        const D3 gm = (1.0 / mlen) * (gn - dot(n, gn) * n);
        for (int k = 0; k < 3; k++) {
            const D3 gN = (double)d[4 + k] * gm;
            double* gv = out->vnor + 4 * (3 * (size_t)t + k);
            for (int j = 0; j < 3; j++) acc(gv[j], M[j] * gN.x + M[4 + j] * gN.y + M[8 + j] * gN.z);
        }
    }
}

bool selected(const orc_diff_in* in, size_t i) {
    if (in->only_tri < 0 && in->only_mat < 0) return true;
    const float* d = in->gbuf + 16 * i;
    uint32_t t;
    int32_t m;
    std::memcpy(&t, d + 0, 4);
    std::memcpy(&m, d + 1, 4);
    if (in->only_tri >= 0 && t != (uint32_t)in->only_tri) return false;
    if (in->only_mat >= 0 && m != in->only_mat) return false;
    return true;
}

}  // namespace

extern "C" {

// Radiance [H*W][4] (alpha from the G-buffer) where radiance != NULL; returns
// sum over the selected pixels of sum_rgb (R - target)^2 (target NULL: 0).
double orc_diff_forward64(const orc_diff_in* in, double* radiance, const float* target) {
    const size_t npx = (size_t)in->W * in->H;
    double loss = 0.0;
    for (size_t i = 0; i < npx; i++) {
        if (!selected(in, i)) continue;
        double R[3];
        pixel(in, i, R, nullptr, nullptr);
        if (radiance) {
            for (int c = 0; c < 3; c++) radiance[4 * i + c] = R[c];
            radiance[4 * i + 3] = in->gbuf[16 * i + 7];
        }
        if (target)
            for (int c = 0; c < 3; c++) {
                const double e = R[c] - target[4 * i + c];
                loss += e * e;
            }
    }
    return loss;
}

// Accumulates into out (zero it first) the gradients of sum_i grad_i . R_i.
void orc_diff_backward64(const orc_diff_in* in, const double* grad, orc_diff_out* out) {
    const size_t npx = (size_t)in->W * in->H;
    for (size_t i = 0; i < npx; i++) {
        double R[3];
        pixel(in, i, R, grad + 4 * i, out);
    }
}

}  // extern "C"
