"""The Go purego binding (polyred_gb300/go/cuda/*.go) against the C header,
without a Go toolchain: every struct the binding mirrors has the C layout
(field offsets and sizes under Go's 64-bit size and alignment rules, against
the C compiler's offsetof/sizeof), every bound symbol is declared in
include/polyred_cuda.h with the same number of parameters, and the Go
constants equal the header's."""
import os
import re
import subprocess

import pytest

from polyred_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GO_DIR = os.path.join(ROOT, "polyred_gb300", "go", "cuda")
HEADER = os.path.join(ROOT, "include", "polyred_cuda.h")

MIRRORS = {"Object": "pr_object", "Material": "pr_material", "Texture": "pr_texture", "SceneDesc": "pr_scene_desc",
           "Light": "pr_light", "FrameDesc": "pr_frame_desc", "Outputs": "pr_outputs",
           "DiffParams": "pr_diff_params", "DiffGrads": "pr_diff_grads"}

CONSTANTS = {"OK": "PR_OK", "ErrInvalidArg": "PR_ERR_INVALID_ARG", "ErrOOM": "PR_ERR_OOM", "ErrCUDA": "PR_ERR_CUDA",
             "ErrOverflow": "PR_ERR_OVERFLOW", "ErrTimeout": "PR_ERR_TIMEOUT", "ErrUnimpl": "PR_ERR_UNIMPLEMENTED",
             "ErrNoScene": "PR_ERR_NO_SCENE", "ErrUnsupported": "PR_ERR_UNSUPPORTED",
             "ErrNoDevice": "PR_ERR_NO_DEVICE", "ErrSingular": "PR_ERR_SINGULAR", "ErrFatal": "PR_ERR_FATAL",
             "MatFlatShading": "PR_MAT_FLAT_SHADING", "MatAO": "PR_MAT_AO",
             "MatReceiveShadow": "PR_MAT_RECEIVE_SHADOW", "MatMipmap": "PR_MAT_MIPMAP",
             "LightPoint": "PR_LIGHT_POINT", "LightDirectional": "PR_LIGHT_DIRECTIONAL",
             "FramePerspective": "PR_FRAME_PERSPECTIVE", "FrameShadowMap": "PR_FRAME_SHADOWMAP",
             "FrameGamma": "PR_FRAME_GAMMA", "TriNone": "PR_TRI_NONE", "DGBFloats": "PR_DGB_FLOATS"}

# Go's sizes and alignments on 64-bit targets (amd64, arm64)
BASIC = {"bool": 1, "uint8": 1, "int8": 1, "byte": 1, "int16": 2, "uint16": 2, "int32": 4, "uint32": 4,
         "float32": 4, "rune": 4, "int64": 8, "uint64": 8, "float64": 8, "int": 8, "uint": 8, "uintptr": 8,
         "unsafe.Pointer": 8}


def go_sources():
    return {f: open(os.path.join(GO_DIR, f)).read() for f in sorted(os.listdir(GO_DIR)) if f.endswith(".go")}


def strip_comments(src):
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def go_structs():
    """{name: [(field, type), ...]} of every struct type in the binding."""
    out = {}
    for src in go_sources().values():
        for m in re.finditer(r"^type (\w+) struct \{(.*?)^\}", strip_comments(src), flags=re.S | re.M):
            fields = []
            for line in m.group(2).splitlines():
                line = line.strip()
                if not line:
                    continue
                toks = line.split()
                typ = toks[-1]
                names = [n.strip() for n in " ".join(toks[:-1]).split(",")]
                fields += [(n, typ) for n in names]
            out[m.group(1)] = fields
    return out


def go_layout(typ, structs):
    """(size, align) of a Go type."""
    if typ in BASIC:
        return BASIC[typ], BASIC[typ]
    if typ.startswith("*"):
        return 8, 8
    m = re.fullmatch(r"\[(\d+)\](.+)", typ)
    if m:
        s, a = go_layout(m.group(2), structs)
        return int(m.group(1)) * s, a
    if typ in structs:
        offs, size, align = go_struct_offsets(typ, structs)
        return size, align
    raise ValueError(f"unsupported Go type {typ}")


def go_struct_offsets(name, structs):
    off, align, offs = 0, 1, []
    for fname, typ in structs[name]:
        s, a = go_layout(typ, structs)
        off = (off + a - 1) // a * a
        offs.append((fname, off, s))
        off += s
        align = max(align, a)
    return offs, (off + align - 1) // align * align, align


@pytest.fixture(scope="module")
def c_layouts(tmp_path_factory):
    """{c_struct: (sizeof, [(field, offsetof, sizeof field)])} and the header
    constants, from a probe compiled against the header."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){"]
    for cname in MIRRORS.values():
        st = getattr(_abi, cname)
        lines.append(f'printf("S {cname} %zu\\n", sizeof({cname}));')
        for f, _ in st._fields_:
            lines.append(f'printf("F {cname} {f} %zu %zu\\n", offsetof({cname}, {f}), sizeof((({cname}*)0)->{f}));')
    for c in CONSTANTS.values():
        lines.append(f'printf("C {c} %lld\\n", (long long)({c}));')
    lines.append("return 0;}")
    d = tmp_path_factory.mktemp("go_probe")
    src = d / "probe.c"
    src.write_text("\n".join(lines))
    exe = d / "probe"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    sizes, fields, consts = {}, {}, {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        t = ln.split()
        if t[0] == "S":
            sizes[t[1]] = int(t[2])
        elif t[0] == "F":
            fields.setdefault(t[1], []).append((t[2], int(t[3]), int(t[4])))
        else:
            consts[t[1]] = int(t[2])
    return sizes, fields, consts


def test_every_mirror_is_in_the_binding():
    structs = go_structs()
    for g in MIRRORS:
        assert g in structs, g


@pytest.mark.parametrize("go_name", sorted(MIRRORS))
def test_struct_layout_matches_the_header(go_name, c_layouts):
    sizes, fields, _ = c_layouts
    structs = go_structs()
    cname = MIRRORS[go_name]
    offs, size, _ = go_struct_offsets(go_name, structs)
    cf = fields[cname]
    assert len(offs) == len(cf), (go_name, [f for f, _, _ in offs], [f for f, _, _ in cf])
    for (gf, go_off, go_sz), (cfname, c_off, c_sz) in zip(offs, cf):
        assert (go_off, go_sz) == (c_off, c_sz), (go_name, gf, cfname, go_off, go_sz, c_off, c_sz)
    assert size == sizes[cname], (go_name, size, sizes[cname])


def test_go_constants_match_the_header(c_layouts):
    _, _, consts = c_layouts
    src = strip_comments("\n".join(go_sources().values()))
    for go, c in CONSTANTS.items():
        m = re.search(rf"^\s*(?:const\s+)?{go}\s*=\s*(-?(?:0x[0-9A-Fa-f]+|\d+))\s*$", src, flags=re.M)
        assert m, go
        assert int(m.group(1), 0) == consts[c], (go, c)


def _c_prototypes():
    text = strip_comments(open(HEADER).read())
    protos = {}
    for m in re.finditer(r"\b(pr_\w+)\s*\(([^()]*)\)\s*;", text):
        params = m.group(2).strip()
        protos[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return protos


def test_bound_symbols_are_declared_with_their_arity():
    protos = _c_prototypes()
    src = strip_comments("\n".join(go_sources().values()))
    decls = {m.group(1): m.group(2) for m in re.finditer(r"^\s*(pr\w+)\s+func\(([^)]*)\)", src, flags=re.M)}
    binds = re.findall(r"(?:RegisterLibFunc|register)\(&(\w+),\s*lib,\s*\"(\w+)\"\)", src)
    assert len(binds) >= 17
    for var, sym in binds:
        assert sym in protos, sym
        params = decls[var].strip()
        n = 0 if not params else len(params.split(","))
        assert n == protos[sym], (var, sym, n, protos[sym])
