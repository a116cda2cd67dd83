"""Extract the render path's known-answer vectors from the reference's Go
tests (read as text) into reference_kats.json.

Run where the reference tree is available:
    python tests/golden/extract_kats.py /path/to/polyred
The JSON it writes is committed; the tests read only the JSON.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def floats(s):
    return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?(?:e[-+]?\d+)?", s)]


def block(text, start_pat, end_pat):
    m = re.search(start_pat, text, re.S)
    assert m, start_pat
    rest = text[m.end():]
    e = re.search(end_pat, rest, re.S)
    return rest[:e.start()]


def main(ref):
    out = {"source": "reference Go tests, extracted as text by tests/golden/extract_kats.py"}

    t = open(os.path.join(ref, "camera/camera_test.go")).read()
    # TestViewMatrix (camera/camera_test.go:106-145)
    vm = block(t, r"func TestViewMatrix.*?want := math\.NewMat4\[float32\]\(", r"\)\n")
    pos = floats(re.search(r"func TestViewMatrix.*?pos := math\.NewVec3\[float32\]\(([^)]*)\)", t, re.S).group(1))
    look = floats(re.search(r"func TestViewMatrix.*?lookAt := math\.NewVec3\[float32\]\(([^)]*)\)", t, re.S).group(1))
    up = floats(re.search(r"func TestViewMatrix.*?up := math\.NewVec3\[float32\]\(([^)]*)\)", t, re.S).group(1))
    out["view_matrix"] = {"cite": "camera/camera_test.go:106-145", "pos": pos, "target": look, "up": up,
                          "want": floats(vm)}
    # TestProjMatrix (camera/camera_test.go:147-194)
    pj = t[t.index("func TestProjMatrix"):t.index("func BenchmarkCamera")]
    fov = floats(re.search(r"fov := float32\(([^)]*)\)", pj).group(1))[0]
    aspect = floats(re.search(r"aspect := float32\(([^)]*)\)", pj).group(1))[0]
    near = floats(re.search(r"near := float32\(([^)]*)\)", pj).group(1))[0]
    far = floats(re.search(r"far := float32\(([^)]*)\)", pj).group(1))[0]
    wants = re.findall(r"want (?::=|=) math\.NewMat4\[float32\]\((.*?)\)\n", pj, re.S)
    l = floats(re.search(r"left := float32\(([^)]*)\)", pj).group(1))[0]
    r = floats(re.search(r"right := float32\(([^)]*)\)", pj).group(1))[0]
    top = floats(re.search(r"top := float32\(([^)]*)\)", pj).group(1))[0]
    bot = floats(re.search(r"bottom := float32\(([^)]*)\)", pj).group(1))[0]
    n2 = floats(re.search(r"near = float32\(([^)]*)\)", pj).group(1))[0]
    f2 = floats(re.search(r"far = float32\(([^)]*)\)", pj).group(1))[0]
    out["perspective_matrix"] = {"cite": "camera/camera_test.go:147-171", "fov": fov, "aspect": aspect,
                                 "near": near, "far": far, "want": floats(wants[0])}
    out["ortho_matrix"] = {"cite": "camera/camera_test.go:173-193", "left": l, "right": r, "bottom": bot, "top": top,
                           "near": n2, "far": f2, "want": floats(wants[1])}

    t = open(os.path.join(ref, "math/interpolate_test.go")).read()
    b = t[t.index("func TestBarycoord"):t.index("func BenchmarkBarycoord")]
    p = floats(re.search(r"p := math\.Vec2\[float32\]\{([^}]*)\}", b).group(1))
    vs = [floats(x) for x in re.findall(r"math\.NewVec2\[float32\]\(([^)]*)\)", b)]
    want = floats(re.search(r"barycoords\[0\] != ([\d.]+) \|\| barycoords\[1\] != ([\d.]+) \|\| barycoords\[2\] != ([\d.]+)",
                            b).group(0).replace("barycoords[0]", "").replace("barycoords[1]", "").replace("barycoords[2]", ""))
    out["barycoord"] = {"cite": "math/interpolate_test.go:104-115", "p": p, "v": vs, "want": want}

    t = open(os.path.join(ref, "geometry/primitive/box_test.go")).read()
    out["aabb"] = {"cite": "geometry/primitive/box_test.go:14-110",
                   "a": [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
                   "b_disjoint": [[-1, -0.5, -0.5], [-0.5, -1, -0.5], [-0.5, -0.5, -1]],
                   "c_inside": [[0.5, 0, 0], [0, 0.5, 0], [0, 0, 0.5]],
                   "d_touch": [[-1, 0, 0], [0, -1, 0], [0, 0, -1]],
                   "outside_point": [-1, -1, -1],
                   "expect": {"a_b": False, "a_c": True, "a_d": True}}
    assert "aabb1.Intersect(aabb2)" in t and "aabb1.Intersect(aabb4)" in t

    t = open(os.path.join(ref, "geometry/primitive/triangle_test.go")).read()
    iv = t[t.index("func TestTriangle_IsValid"):t.index("func TestTriangle_Area")]
    poss = [floats(x) for x in re.findall(r"math\.NewVec4\[float32\]\(([^)]*)\)", iv)]
    out["tri_is_valid"] = {"cite": "geometry/primitive/triangle_test.go:29-52",
                           "cases": [{"p": poss[0:3], "valid": False}, {"p": poss[3:6], "valid": True}]}

    t = open(os.path.join(ref, "render/worldpos_test.go")).read()
    out["interp_world_pos"] = {"cite": "render/worldpos_test.go:17-32",
                               "m": [[10, 0, 0, 0], [0, 10, 0, 0], [0, 0, 10, 0]],
                               "centroid_sum_range": [9.99, 10.01]}
    assert "1.0 / 3" in t

    t = open(os.path.join(ref, "render/shading_equiv_test.go")).read()
    norms = [floats(x) for x in re.findall(r"\{([-\d., ]+)\}", t[t.index("norms := "):t.index("poss := ")])]
    poss = [floats(x) for x in re.findall(r"\{([-\d., ]+)\}", t[t.index("poss := "):t.index("// Mirror")])]
    out["shading_equivalence"] = {
        "cite": "render/shading_equiv_test.go:33-105",
        "texture": [200, 150, 100, 255], "diffuse": [220, 180, 160, 255], "specular": [255, 255, 255, 255],
        "shininess": 32, "cam": [0, 1.5, 3],
        "point": {"intensity": 3, "color": [255, 240, 220, 255], "position": [-2, 3, 4]},
        "directional": {"intensity": 1, "color": [180, 200, 255, 255], "direction": [0, -1, -1]},
        "ambient": 0.4, "norms": norms, "poss": poss, "tolerance_lsb": 1}
    assert "light.Intensity(3)" in t and "light.Intensity(0.4)" in t and "material.Shininess(32)" in t

    t = open(os.path.join(ref, "gpu/shader/gpumath/kernels/srgb_test.go")).read()
    vals = floats(re.search(r"range \[\]float64\{([^}]*)\}", t).group(1))
    out["srgb"] = {"cite": "gpu/shader/gpumath/kernels/srgb_test.go:13-28", "values": vals, "tolerance": 1e-6,
                   "exponent": 0.4166666666}

    t = open(os.path.join(ref, "color/color_test.go")).read()
    out["srgb_roundtrip"] = {"cite": "color/color_test.go:33-56", "orig": 0.5, "eps": 1e-7,
                             "fixed": [[0, 0], [1, 1]]}
    assert "FromLinear2sRGB[float32](0) != 0" in t

    t = open(os.path.join(ref, "render/material_table_test.go")).read()
    out["mat_at"] = {"cite": "render/material_table_test.go:17-34", "table_len": 2,
                     "cases": [[-1, None], [0, 0], [1, 1], [2, None], [1 << 30, None]]}
    assert "matAt(table, 1<<30)" in t

    out["color_from_value"] = {"cite": "color/color.go:33-44 (used by material.Diffuse/Specular)",
                               "cases": [[[0.8, 0.3, 0.2, 1.0], [204, 77, 51, 255]],
                                         [[0.5, 0.5, 0.5, 1.0], [128, 128, 128, 255]]]}
    # TestQuery (buffer/texture_test.go:25-166): Texture.Query(lod, u, v)
    t = open(os.path.join(ref, "buffer/texture_test.go")).read()
    pix = [int(v) for v in floats(re.search(r"Pix: \[\]uint8\{(.*?)\}", t, re.S).group(1))]
    rect = [int(v) for v in floats(re.search(r"Rect:\s*image\.Rect\(([^)]*)\)", t).group(1))]
    cases = []
    pat = (r'\{\s*"([^"]+)",\s*(.*?),\s*(-?[\d.]+),\s*(-?[\d.]+),\s*(-?[\d.]+),\s*'
           r"color\.RGBA\{R:\s*(\d+),\s*G:\s*(\d+),\s*B:\s*(\d+),\s*A:\s*(\d+)\}")
    for m in re.finditer(pat, t[t.index("tests = []struct"):t.index("func TestQuery")], re.S):
        name, tex = m.group(1), m.group(2)
        if "TextureImage(data)" in tex:
            kind = {"image": "data", "mipmap": "TextureIsoMipmap(true)" in tex}
        elif "mustLoadTexture" in tex:
            kind = {"asset": os.path.basename(re.search(r'"([^"]+)"', tex).group(1)), "mipmap": True,
                    "gamma_correct": False}
        else:
            kind = {"default": True}
        cases.append({"name": name, "texture": kind, "u": float(m.group(3)), "v": float(m.group(4)),
                      "lod": float(m.group(5)), "want": [int(m.group(k)) for k in range(6, 10)]})
    out["texture_query"] = {"cite": "buffer/texture_test.go:25-166 (TestQuery)", "data_pix": pix,
                            "data_rect": rect, "cases": cases}
    json.dump(out, open(os.path.join(HERE, "reference_kats.json"), "w"), indent=1)
    print("wrote", os.path.join(HERE, "reference_kats.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: extract_kats.py <reference checkout>")
    main(sys.argv[1])
