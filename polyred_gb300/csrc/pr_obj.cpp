// Wavefront OBJ / MTL parser for the host loader: the line grammar and parse
// state of the reference's model/obj/obj.go (File.parse, parseObjLine,
// parseMtlLine and their field parsers, obj.go:139-611), written as one
// pass over a text buffer that appends to flat arrays.
//
// Numbers follow Go's strconv: ParseFloat(s, 32) (decimal and hexadecimal
// forms, inf/infinity/nan, '_' digit separators, correctly rounded to
// float32, an error past the float32 range), ParseInt(s, 10, 32) and
// ParseUint(s, 10, 32). Lines split on '\n' only and fields on Go's
// unicode.IsSpace (strings.Fields), so files with '\r\n' ends or non-ASCII
// spaces give the reference's fields.
//
// Error behaviour mirrors obj.go: a malformed line stops the parse with the
// reference's message (formatError's "<what> in line:<n>", or strconv's);
// what was parsed before it stays in the state, as in the reference's File.
// Inputs on which the reference panics instead (an MTL property before any
// material, a colour outside [0, 1]) return PR_ERR_FATAL.
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <climits>
#include <new>
#include <stdexcept>
#include <string>
#include <system_error>
#include <unordered_map>
#include <vector>

#include "../../include/polyred_cuda.h"

namespace prk {
int set_last_error(int status, const char* msg);
}

namespace {

struct Span {
    const char* p;
    size_t n;
    bool eq(const char* s) const { return strlen(s) == n && memcmp(p, s, n) == 0; }
    std::string str() const { return std::string(p, n); }
};

struct Material {
    int32_t name;
    int32_t map_kd = -1;
    int32_t illum = 0;
    float opacity = 0, refraction = 0, shininess = 0;
    uint8_t ambient[4] = {0, 0, 0, 0}, diffuse[4] = {0, 0, 0, 0}, specular[4] = {0, 0, 0, 0},
            emissive[4] = {0, 0, 0, 0};
};

struct ObjState {
    std::vector<float> vertices, normals, uvs;
    std::vector<int64_t> face_start{0};
    std::vector<int64_t> cv, cvt, cvn;
    std::vector<int32_t> face_object, face_material;
    std::vector<uint8_t> face_smooth;
    std::vector<int32_t> object_name;
    std::vector<int64_t> object_mat_start{0};
    std::vector<int32_t> object_mat;
    std::vector<Material> materials;
    std::vector<pr_obj_material> mat_out;
    std::unordered_map<std::string, int32_t> mat_index;
    std::vector<int32_t> warnings;
    std::string strings;
    int32_t matlib = -1;
    int32_t mat_current = -1;
    bool smooth = false;
    int64_t line = 1;
    std::string error;

    // entries: a native-endian uint32 length, the bytes (Go strings may hold
    // NUL), a NUL
    int32_t intern(const char* p, size_t n) {
        if (strings.size() + n + 5 > (size_t)INT32_MAX) throw std::length_error("string table exceeds 2 GiB");
        int32_t off = (int32_t)strings.size();
        const uint32_t len = (uint32_t)n;
        strings.append((const char*)&len, 4);
        strings.append(p, n);
        strings.push_back('\0');
        return off;
    }
    int32_t intern(const std::string& s) { return intern(s.data(), s.size()); }
};

// Outcome of one line: ok, an error the reference returns, or a panic.
enum LineStatus { L_OK = 0, L_ERROR = 1, L_FATAL = 2 };

// ---------------------------------------------------------------- fields

// Byte classes: 1 = ASCII white space (\t \n \v \f \r ' '), 2 = a lead byte
// of a non-ASCII white-space rune (C2, E1, E2, E3), 0 = anything else.
struct ByteClass {
    unsigned char c[256];
    ByteClass() {
        memset(c, 0, sizeof(c));
        for (int b : {' ', '\t', '\n', '\v', '\f', '\r'}) c[b] = 1;
        for (int b : {0xC2, 0xE1, 0xE2, 0xE3}) c[b] = 2;
    }
};
const ByteClass kClass;

// Width of the unicode.IsSpace rune starting at p (0 if none). Non-ASCII
// white space is U+0085, U+00A0, U+1680, U+2000..U+200A, U+2028, U+2029,
// U+202F, U+205F and U+3000; their lead bytes (C2, E1, E2, E3) never
// continue another sequence, so they mark rune boundaries whatever precedes.
inline size_t space_width(const unsigned char* p, const unsigned char* end) {
    unsigned char k = kClass.c[*p];
    if (k != 2) return k;
    size_t left = (size_t)(end - p);
    if (p[0] == 0xC2 && left >= 2 && (p[1] == 0x85 || p[1] == 0xA0)) return 2;
    if (left >= 3) {
        if (p[0] == 0xE1 && p[1] == 0x9A && p[2] == 0x80) return 3;
        if (p[0] == 0xE2 && p[1] == 0x80 && ((p[2] >= 0x80 && p[2] <= 0x8A) || p[2] == 0xA8 || p[2] == 0xA9 || p[2] == 0xAF))
            return 3;
        if (p[0] == 0xE2 && p[1] == 0x81 && p[2] == 0x9F) return 3;
        if (p[0] == 0xE3 && p[1] == 0x80 && p[2] == 0x80) return 3;
    }
    return 0;
}

// strings.Fields of one line.
void split_fields(const char* p, size_t n, std::vector<Span>& out) {
    out.clear();
    const unsigned char* s = (const unsigned char*)p;
    const unsigned char* end = s + n;
    while (s < end) {
        size_t w;
        while (s < end && (w = space_width(s, end)) != 0) s += w;
        if (s >= end) break;
        const unsigned char* b = s;
        while (s < end && space_width(s, end) == 0) s++;
        out.push_back({(const char*)b, (size_t)(s - b)});
    }
}

// ---------------------------------------------------------------- strconv

std::string go_quote(Span s) {
    std::string q = "\"";
    for (size_t i = 0; i < s.n; i++) {
        unsigned char c = (unsigned char)s.p[i];
        char buf[8];
        switch (c) {
            case '"': q += "\\\""; break;
            case '\\': q += "\\\\"; break;
            case '\a': q += "\\a"; break;
            case '\b': q += "\\b"; break;
            case '\f': q += "\\f"; break;
            case '\n': q += "\\n"; break;
            case '\r': q += "\\r"; break;
            case '\t': q += "\\t"; break;
            case '\v': q += "\\v"; break;
            default:
                if (c < 0x20 || c >= 0x7F) {
                    snprintf(buf, sizeof(buf), "\\x%02x", c);
                    q += buf;
                } else {
                    q.push_back((char)c);
                }
        }
    }
    return q + "\"";
}

std::string num_error(const char* fn, Span s, bool range) {
    return std::string("strconv.") + fn + ": parsing " + go_quote(s) + (range ? ": value out of range" : ": invalid syntax");
}

char lower(char c) { return (char)(c | 0x20); }
bool is_dec(char c) { return c >= '0' && c <= '9'; }
bool is_hex(char c) { return is_dec(c) || (lower(c) >= 'a' && lower(c) <= 'f'); }

// strconv's underscoreOK: '_' only between digits, or between a base prefix
// and a digit.
bool underscore_ok(const char* s, size_t n) {
    char saw = '^';
    size_t i = 0;
    if (n >= 1 && (s[0] == '-' || s[0] == '+')) {
        s++;
        n--;
    }
    bool hex = false;
    if (n >= 2 && s[0] == '0' && (lower(s[1]) == 'b' || lower(s[1]) == 'o' || lower(s[1]) == 'x')) {
        i = 2;
        saw = '0';
        hex = lower(s[1]) == 'x';
    }
    for (; i < n; i++) {
        if (is_dec(s[i]) || (hex && lower(s[i]) >= 'a' && lower(s[i]) <= 'f')) {
            saw = '0';
            continue;
        }
        if (s[i] == '_') {
            if (saw != '0') return false;
            saw = '_';
            continue;
        }
        if (saw == '_') return false;
        saw = '!';
    }
    return saw != '_';
}

size_t common_prefix_ci(const char* s, size_t n, const char* word) {
    size_t i = 0;
    while (i < n && word[i] && lower(s[i]) == word[i]) i++;
    return i;
}

// Clinger's fast path (W. D. Clinger, "How to Read Floating Point Numbers
// Accurately", PLDI 1990): when the decimal digits form an integer
// M <= 2^24 and the power of ten k has |k| <= 10, both M and 10^|k| are
// exact floats, so one IEEE multiply or divide rounds the exact value
// correctly. `m` is a well-formed unsigned decimal without '_'. Returns
// false when the text is outside the fast path.
bool clinger_fast(const char* m, size_t n, float* out) {
    static const float kPow10[11] = {1e0f, 1e1f, 1e2f, 1e3f, 1e4f, 1e5f, 1e6f, 1e7f, 1e8f, 1e9f, 1e10f};
    uint64_t mant = 0;
    int digits = 0, frac = 0;
    bool dot = false;
    size_t i = 0;
    for (; i < n; i++) {
        char c = m[i];
        if (c == '.') {
            dot = true;
            continue;
        }
        if (!is_dec(c)) break;
        if (mant == 0 && c == '0') {  // leading zeros carry no digits
            if (dot) frac++;
            continue;
        }
        if (++digits > 8) return false;
        mant = mant * 10 + (uint64_t)(c - '0');
        if (dot) frac++;
    }
    int exp = 0;
    if (i < n) {  // 'e' / 'E' [sign] digits
        i++;
        bool eneg = false;
        if (m[i] == '+' || m[i] == '-') eneg = m[i++] == '-';
        for (; i < n; i++) {
            exp = exp * 10 + (m[i] - '0');
            if (exp > 100) return false;
        }
        if (eneg) exp = -exp;
    }
    if (mant > (1u << 24)) return false;
    int k = exp - frac;
    if (mant == 0) {
        *out = 0.0f;
        return true;
    }
    if (k < -10 || k > 10) return false;
    float f = (float)mant;
    *out = k < 0 ? f / kPow10[-k] : f * kPow10[k];
    return true;
}

// strconv.ParseFloat(s, 32). Returns false with *msg set on error.
bool parse_f32(Span sp, float* out, std::string* msg) {
    const char* s = sp.p;
    size_t n = sp.n;
    if (n == 0) {
        *msg = num_error("ParseFloat", sp, false);
        return false;
    }
    // special(): [+-]inf / [+-]infinity / nan, any case
    {
        size_t i = 0;
        bool neg = false, sign = false;
        if (s[0] == '+' || s[0] == '-') {
            neg = s[0] == '-';
            sign = true;
            i = 1;
        }
        if (i < n && lower(s[i]) == 'i') {
            size_t k = common_prefix_ci(s + i, n - i, "infinity");
            if (k > 3 && k < 8) k = 3;
            if (k == 3 || k == 8) {
                if (i + k != n) {
                    *msg = num_error("ParseFloat", sp, false);
                    return false;
                }
                *out = neg ? -INFINITY : INFINITY;
                return true;
            }
        } else if (!sign && lower(s[0]) == 'n') {
            if (common_prefix_ci(s, n, "nan") == 3) {
                if (n != 3) {
                    *msg = num_error("ParseFloat", sp, false);
                    return false;
                }
                *out = NAN;
                return true;
            }
        }
    }
    // readFloat's grammar
    size_t i = 0;
    bool neg = false, underscores = false;
    if (s[i] == '+') {
        i++;
    } else if (s[i] == '-') {
        neg = true;
        i++;
    }
    bool hex = false;
    if (i + 2 < n && s[i] == '0' && lower(s[i + 1]) == 'x') {
        hex = true;
        i += 2;
    }
    size_t mant_begin = i;
    bool sawdot = false, sawdigits = false;
    for (; i < n; i++) {
        char c = s[i];
        if (c == '_') {
            underscores = true;
            continue;
        }
        if (c == '.') {
            if (sawdot) break;
            sawdot = true;
            continue;
        }
        if (is_dec(c) || (hex && is_hex(c))) {
            sawdigits = true;
            continue;
        }
        break;
    }
    bool ok = sawdigits;
    if (ok) {
        char exp_char = hex ? 'p' : 'e';
        if (i < n && lower(s[i]) == exp_char) {
            i++;
            if (i < n && (s[i] == '+' || s[i] == '-')) i++;
            if (i >= n || !is_dec(s[i])) {
                ok = false;
            } else {
                for (; i < n && (is_dec(s[i]) || s[i] == '_'); i++)
                    if (s[i] == '_') underscores = true;
            }
        } else if (hex) {
            ok = false;
        }
    }
    if (ok && underscores && !underscore_ok(s, i)) ok = false;
    if (!ok || i != n) {
        *msg = num_error("ParseFloat", sp, false);
        return false;
    }
    // The text is well formed: convert the magnitude, correctly rounded.
    std::string clean;
    const char* m = s + mant_begin;
    size_t mn = n - mant_begin;
    if (underscores) {
        for (size_t k = 0; k < mn; k++)
            if (m[k] != '_') clean.push_back(m[k]);
        m = clean.data();
        mn = clean.size();
    }
    float v = 0;
    bool range = false;
    if (!hex && !underscores && clinger_fast(m, mn, &v)) {
        *out = neg ? -v : v;
        return true;
    }
    if (!hex) {
        auto r = std::from_chars(m, m + mn, v, std::chars_format::general);
        if (r.ec == std::errc::result_out_of_range || r.ptr != m + mn) {
            // from_chars leaves underflow and overflow to strtof, which
            // returns the rounded value (0, a subnormal or infinity).
            std::string tmp(m, mn);
            v = strtof(tmp.c_str(), nullptr);
            range = std::isinf(v);
        } else if (r.ec != std::errc()) {
            *msg = num_error("ParseFloat", sp, false);
            return false;
        }
    } else {
        std::string tmp = "0x" + std::string(m, mn);
        v = strtof(tmp.c_str(), nullptr);
        range = std::isinf(v);
    }
    if (range) {
        *msg = num_error("ParseFloat", sp, true);
        return false;
    }
    *out = neg ? -v : v;
    return true;
}

// strconv.ParseUint(s, 10, bits) on the unsigned part; range flag on overflow.
bool parse_udec(const char* s, size_t n, uint64_t limit, uint64_t* out, bool* range) {
    *range = false;
    if (n == 0) return false;
    uint64_t v = 0;
    for (size_t i = 0; i < n; i++) {
        if (!is_dec(s[i])) return false;
        if (!*range) {
            v = v * 10 + (uint64_t)(s[i] - '0');
            if (v > limit) *range = true;
        }
    }
    *out = v;
    return true;
}

// strconv.ParseInt(s, 10, 32)
bool parse_i32(Span sp, int64_t* out, std::string* msg) {
    const char* s = sp.p;
    size_t n = sp.n;
    bool neg = false;
    if (n > 0 && (s[0] == '+' || s[0] == '-')) {
        neg = s[0] == '-';
        s++;
        n--;
    }
    uint64_t u;
    bool range;
    if (!parse_udec(s, n, (uint64_t)1 << 32, &u, &range)) {
        *msg = num_error("ParseInt", sp, false);
        return false;
    }
    const uint64_t cutoff = (uint64_t)1 << 31;
    if (range || (!neg && u >= cutoff) || (neg && u > cutoff)) {
        *msg = num_error("ParseInt", sp, true);
        return false;
    }
    *out = neg ? -(int64_t)u : (int64_t)u;
    return true;
}

// strconv.ParseUint(s, 10, 32)
bool parse_u32(Span sp, uint64_t* out) {
    bool range;
    return parse_udec(sp.p, sp.n, 0xFFFFFFFFull, out, &range) && !range;
}

// color.FromValue[float32](r, g, b, 1) (color/color.go:33-44): false when a
// component is outside [0, 1], where the reference panics.
bool color_from_value(const float c[3], uint8_t out[4]) {
    for (int k = 0; k < 3; k++)
        if (c[k] < 0.0f || c[k] > 1.0f) return false;
    for (int k = 0; k < 3; k++) {
        float x = c[k] * 255.0f;  // float32 product
        double r = std::round((double)x);
        out[k] = std::isnan(r) ? 0 : (uint8_t)r;
    }
    out[3] = 255;  // 1 * 255
    return true;
}

// ---------------------------------------------------------------- OBJ lines

struct Parser {
    ObjState& st;
    std::vector<Span> f;
    std::string msg;

    LineStatus fail(const std::string& what) {
        msg = what + " in line:" + std::to_string(st.line);
        return L_ERROR;
    }
    LineStatus raw(const std::string& m) {
        msg = m;
        return L_ERROR;
    }
    void warn(const char* type, const std::string& m) {
        st.warnings.push_back(st.intern(std::string(type) + "(" + std::to_string(st.line) + "): " + m));
    }

    void new_object(const std::string& name) {
        st.object_name.push_back(st.intern(name));
        st.object_mat_start.push_back(st.object_mat_start.back());
    }
    bool have_object() const { return !st.object_name.empty(); }
    int64_t current_object_mats() const {
        return st.object_mat_start.back() - st.object_mat_start[st.object_mat_start.size() - 2];
    }
    void object_add_material(int32_t m) {
        st.object_mat.push_back(m);
        st.object_mat_start.back()++;
    }
    int32_t material_named(Span name) {
        std::string key = name.str();
        auto it = st.mat_index.find(key);
        if (it != st.mat_index.end()) return it->second;
        Material m;
        m.name = st.intern(key);
        int32_t idx = (int32_t)st.materials.size();
        st.materials.push_back(m);
        st.mat_index.emplace(key, idx);
        return idx;
    }

    LineStatus obj_line() {
        if (f.empty() || f[0].p[0] == '#') return L_OK;
        Span t = f[0];
        size_t nf = f.size() - 1;
        if (t.eq("mtllib")) {
            if (nf < 1) return fail("Material library (mtllib) with no fields");
            st.matlib = st.intern(f[1].p, f[1].n);
        } else if (t.eq("o") || t.eq("g")) {
            if (nf < 1) return fail("obj line (o) with no fields");
            new_object(f[1].str());
        } else if (t.eq("v")) {
            if (nf < 3) return fail("vertex has less than 3 vertices in 'v' line: " + go_list(1));
            float w = 1.0f;
            if (nf == 4) {
                float v;
                if (!parse_f32(f[4], &v, &msg)) return L_ERROR;
                w = 1.0f / v;
            }
            for (int k = 1; k <= 3; k++) {
                float v;
                if (!parse_f32(f[k], &v, &msg)) return L_ERROR;
                st.vertices.push_back(w == 1.0f ? v : v * w);
            }
        } else if (t.eq("vn")) {
            if (nf < 3) return fail("normal has less than 3 vertices in 'vn' line: " + go_list(1));
            for (int k = 1; k <= 3; k++) {
                float v;
                if (!parse_f32(f[k], &v, &msg)) return L_ERROR;
                st.normals.push_back(v);
            }
        } else if (t.eq("vt")) {
            if (nf < 2) return fail("Less than 2 texture coords. in 'vt' line");
            for (int k = 1; k <= 2; k++) {
                float v;
                if (!parse_f32(f[k], &v, &msg)) return L_ERROR;
                st.uvs.push_back(v);
            }
        } else if (t.eq("f")) {
            return face();
        } else if (t.eq("usemtl")) {
            if (nf < 1) return fail("Usemtl with no fields");
            if (!have_object()) new_object("unnamed" + std::to_string(st.line));
            int32_t m = material_named(f[1]);
            object_add_material(m);
            st.mat_current = m;
        } else if (t.eq("s")) {
            if (nf < 1) return fail("'s' with no fields");
            st.smooth = !(f[1].eq("0") || f[1].eq("off"));
        } else {
            warn("obj", "unsupported field: " + t.str());
        }
        return L_OK;
    }

    // fmt's %v of the fields after the line type: [a b c]
    std::string go_list(size_t from) const {
        std::string s = "[";
        for (size_t k = from; k < f.size(); k++) {
            if (k > from) s += " ";
            s += f[k].str();
        }
        return s + "]";
    }

    // One index of a face corner: 1-based absolute, or negative relative to
    // the count parsed so far; zero is an error.
    LineStatus corner_index(Span s, int64_t count, const char* zero_msg, int64_t* out) {
        int64_t v;
        if (!parse_i32(s, &v, &msg)) return L_ERROR;
        if (v > 0) {
            *out = v - 1;
        } else if (v < 0) {
            *out = (count - 1) + v + 1;
        } else {
            return fail(zero_msg);
        }
        return L_OK;
    }

    LineStatus face() {
        if (!have_object()) new_object("unnamed" + std::to_string(st.line));
        if (current_object_mats() == 0 && st.mat_current >= 0) object_add_material(st.mat_current);
        size_t nf = f.size() - 1;
        if (nf < 3) return fail("face line with less 3 fields");
        size_t start = st.cv.size();
        LineStatus ls = L_OK;
        for (size_t k = 1; k <= nf && ls == L_OK; k++) {
            // strings.Split(field, "/")
            Span parts[3];
            size_t np = 0;
            const char* p = f[k].p;
            const char* e = p + f[k].n;
            const char* b = p;
            for (; p <= e; p++) {
                if (p == e || *p == '/') {
                    if (np < 3) parts[np] = {b, (size_t)(p - b)};
                    np++;
                    b = p + 1;
                }
            }
            int64_t vi = 0, ti = PR_OBJ_NO_INDEX, ni = PR_OBJ_NO_INDEX;
            ls = corner_index(parts[0], (int64_t)(st.vertices.size() / 3), "face vertex index value equal to 0", &vi);
            if (ls == L_OK && np > 1 && parts[1].n > 0)
                ls = corner_index(parts[1], (int64_t)(st.uvs.size() / 2), "face uv index value equal to 0", &ti);
            if (ls == L_OK && np >= 3)
                ls = corner_index(parts[2], (int64_t)(st.normals.size() / 3), "face normal index value equal to 0", &ni);
            if (ls == L_OK) {
                st.cv.push_back(vi);
                st.cvt.push_back(ti);
                st.cvn.push_back(ni);
            }
        }
        if (ls != L_OK) {
            st.cv.resize(start);
            st.cvt.resize(start);
            st.cvn.resize(start);
            return ls;
        }
        st.face_start.push_back((int64_t)st.cv.size());
        st.face_object.push_back((int32_t)st.object_name.size() - 1);
        st.face_material.push_back(st.mat_current);
        st.face_smooth.push_back(st.smooth ? 1 : 0);
        return L_OK;
    }

    // ------------------------------------------------------------ MTL lines

    LineStatus mtl_color(uint8_t out[4]) {
        float c[3];
        for (int k = 0; k < 3; k++)
            if (!parse_f32(f[k + 1], &c[k], &msg)) return L_ERROR;
        if (!color_from_value(c, out)) {
            char buf[160];
            snprintf(buf, sizeof(buf), "out of range [0, 1], got (%g, %g, %g, 1)", c[0], c[1], c[2]);
            msg = buf;
            return L_FATAL;
        }
        return L_OK;
    }

    Material* current() { return st.mat_current >= 0 ? &st.materials[st.mat_current] : nullptr; }

    LineStatus mtl_line() {
        if (f.empty() || f[0].p[0] == '#') return L_OK;
        Span t = f[0];
        size_t nf = f.size() - 1;
        if (t.eq("newmtl")) {
            if (nf < 1) return fail("newmtl with no fields");
            st.mat_current = material_named(f[1]);
            return L_OK;
        }
        bool known = t.eq("d") || t.eq("Ka") || t.eq("Kd") || t.eq("Ke") || t.eq("Ks") || t.eq("Ni") ||
                     t.eq("Ns") || t.eq("illum") || t.eq("map_Kd");
        if (!known) {
            warn("mtl", "field not supported: " + t.str());
            return L_OK;
        }
        bool colour = t.eq("Ka") || t.eq("Kd") || t.eq("Ke") || t.eq("Ks");
        if (colour ? nf < 3 : nf < 1) {
            if (colour) return fail("'" + t.str() + "' with less than 3 fields");
            if (t.eq("map_Kd")) return fail("No fields");
            return fail("'" + t.str() + "' with no fields");
        }
        // The property is parsed first, then stored through the current
        // material, which the reference dereferences without a check.
        Material tmp;
        Material* m = current();
        Material* dst = m ? m : &tmp;
        LineStatus ls = L_OK;
        if (colour) {
            uint8_t* c = t.eq("Ka") ? dst->ambient : t.eq("Kd") ? dst->diffuse : t.eq("Ke") ? dst->emissive : dst->specular;
            uint8_t v[4];
            ls = mtl_color(v);
            if (ls == L_OK) memcpy(c, v, 4);
        } else if (t.eq("illum")) {
            uint64_t u;
            if (!parse_u32(f[1], &u)) return fail("'d' parse int error");
            dst->illum = (int32_t)(uint32_t)u;
        } else if (t.eq("map_Kd")) {
            if (m) dst->map_kd = st.intern(f[1].p, f[1].n);
        } else {
            float v;
            if (!parse_f32(f[1], &v, &msg)) return fail("'d' parse float error");
            (t.eq("d") ? dst->opacity : t.eq("Ni") ? dst->refraction : dst->shininess) = v;
        }
        if (ls != L_OK) return ls;
        if (!m) {
            msg = "mtl property '" + t.str() + "' before any material (line " + std::to_string(st.line) + ")";
            return L_FATAL;
        }
        return L_OK;
    }
};

}  // namespace

// ---------------------------------------------------------------- C ABI

extern "C" {

int pr_obj_create(void** out) {
    if (!out) {
        return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_obj_create: NULL argument");
    }
    ObjState* st = new (std::nothrow) ObjState();
    if (!st) return prk::set_last_error(PR_ERR_OOM, "pr_obj_create: out of host memory");
    *out = st;
    return PR_OK;
}

int pr_obj_destroy(void* h) {
    if (!h) {
        return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_obj_destroy: NULL handle");
    }
    delete (ObjState*)h;
    return PR_OK;
}

int pr_obj_parse(void* h, int kind, const char* text, size_t len) {
    if (!h || (!text && len) || (kind != PR_OBJ_TEXT_OBJ && kind != PR_OBJ_TEXT_MTL)) {
        return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_obj_parse: NULL handle or text, or unknown kind");
    }
    ObjState& st = *(ObjState*)h;
    Parser ps{st, {}, {}};
    try {
        // File.parse: each '\n'-terminated line (and the unterminated tail)
        // is parsed; the counter starts at 1 and advances after every line
        // but the last.
        st.line = 1;
        st.error.clear();
        size_t pos = 0;
        for (;;) {
            const char* nl = len > pos ? (const char*)memchr(text + pos, '\n', len - pos) : nullptr;
            size_t end = nl ? (size_t)(nl - text) : len;
            split_fields(text + pos, end - pos, ps.f);
            LineStatus ls = kind == PR_OBJ_TEXT_OBJ ? ps.obj_line() : ps.mtl_line();
            if (ls != L_OK) {
                st.error = ps.msg;
                return prk::set_last_error(ls == L_FATAL ? PR_ERR_FATAL : PR_ERR_INVALID_ARG, ps.msg.c_str());
            }
            if (!nl) break;
            pos = end + 1;
            st.line++;
        }
    } catch (const std::bad_alloc&) {
        return prk::set_last_error(PR_ERR_OOM, "pr_obj_parse: out of host memory");
    } catch (const std::length_error&) {
        return prk::set_last_error(PR_ERR_OVERFLOW, "pr_obj_parse: names and warnings exceed 2 GiB");
    }
    return PR_OK;
}

int pr_obj_get(void* h, pr_obj_info* out) {
    if (!h || !out) {
        return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_obj_get: NULL argument");
    }
    if (out->size != sizeof(pr_obj_info)) {
        return prk::set_last_error(PR_ERR_INVALID_ARG, "pr_obj_get: pr_obj_info.size mismatch");
    }
    ObjState& st = *(ObjState*)h;
    st.mat_out.resize(st.materials.size());
    for (size_t i = 0; i < st.materials.size(); i++) {
        const Material& m = st.materials[i];
        pr_obj_material& o = st.mat_out[i];
        o.name = m.name;
        o.map_kd = m.map_kd;
        o.illum = m.illum;
        o.opacity = m.opacity;
        o.refraction = m.refraction;
        o.shininess = m.shininess;
        memcpy(o.ambient, m.ambient, 4);
        memcpy(o.diffuse, m.diffuse, 4);
        memcpy(o.specular, m.specular, 4);
        memcpy(o.emissive, m.emissive, 4);
    }
    out->vertices = st.vertices.data();
    out->n_vertices = (int64_t)st.vertices.size() / 3;
    out->normals = st.normals.data();
    out->n_normals = (int64_t)st.normals.size() / 3;
    out->uvs = st.uvs.data();
    out->n_uvs = (int64_t)st.uvs.size() / 2;
    out->n_faces = (int64_t)st.face_object.size();
    out->n_corners = (int64_t)st.cv.size();
    out->face_start = st.face_start.data();
    out->corner_v = st.cv.data();
    out->corner_vt = st.cvt.data();
    out->corner_vn = st.cvn.data();
    out->face_object = st.face_object.data();
    out->face_material = st.face_material.data();
    out->face_smooth = st.face_smooth.data();
    out->n_objects = (int64_t)st.object_name.size();
    out->object_name = st.object_name.data();
    out->object_mat_start = st.object_mat_start.data();
    out->object_mat = st.object_mat.data();
    out->n_materials = (int64_t)st.materials.size();
    out->materials = st.mat_out.data();
    out->n_warnings = (int64_t)st.warnings.size();
    out->warnings = st.warnings.data();
    out->strings = st.strings.data();
    out->strings_len = (int64_t)st.strings.size();
    out->matlib = st.matlib;
    out->current_material = st.mat_current;
    out->line = st.line;
    out->error = st.error.data();
    out->error_len = (int64_t)st.error.size();
    return PR_OK;
}

}  // extern "C"
