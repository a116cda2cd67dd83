"""Make tests/golden/obj_assets.json from the reference's own OBJ test assets
(internal/testdata/*.obj, the files its loader tests read:
model/obj/obj_test.go:14-26, model/load_test.go:19-31).

For every asset the oracle (oracle/objparse.py) parses the .obj and its
.mtl, and this script checks what it read against a separate scan of the
text: line counts per record type, the first and last vertex, normal and
UV written out with Python's float(), face corner counts, the material
names. It then records digests of the parsed arrays, which
tests/test_objload_cpu.py compares with the native parser when the assets
are present.

Usage: python tests/golden/make_obj_fixtures.py [TESTDATA_DIR]
"""
import glob
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import objparse  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "obj_assets.json")


def testdata_dir(reference_root):
    """The reference's test assets (internal/testdata of its checkout)."""
    return os.path.join(reference_root, "internal", "testdata")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def oracle_record(path):
    f = objparse.load_file(path)
    faces = [fc for ob in f.Objs for fc in ob.Faces]
    starts = np.cumsum([0] + [len(fc.Vertices) for fc in faces]).astype(np.int64)
    cv = np.array([v for fc in faces for v in fc.Vertices], np.int64)
    cvt = np.array([v for fc in faces for v in fc.Uvs], np.int64)
    cvn = np.array([v for fc in faces for v in fc.Normals], np.int64)
    mats = {k: (None if m is None else {"Illum": m.Illum, "Diffuse": list(m.Diffuse), "Specular": list(m.Specular),
                                         "Shininess": float(m.Shininess), "MapKd": m.MapKd})
            for k, m in sorted(f.Materials.items())}
    return f, {
        "n_vertices": len(f.Vertices) // 3, "n_normals": len(f.Normals) // 3, "n_uvs": len(f.Uvs) // 2,
        "n_faces": len(faces), "objects": [ob.Name for ob in f.Objs], "matlib": f.Matlib,
        "vertices": digest(np.array(f.Vertices, np.float32)), "normals": digest(np.array(f.Normals, np.float32)),
        "uvs": digest(np.array(f.Uvs, np.float32)), "face_start": digest(starts), "corner_v": digest(cv),
        "corner_vt": digest(cvt), "corner_vn": digest(cvn),
        "face_material": [fc.Material for fc in faces[:1]] + [fc.Material for fc in faces[-1:]],
        "materials": mats, "warnings": f.Warnings,
    }


def text_scan(path):
    """Counts and end values read from the text with str.split()."""
    rows = {"v": [], "vn": [], "vt": [], "f": [], "o": [], "g": []}
    with open(path, "rb") as fh:
        for line in fh.read().decode().splitlines():
            parts = line.split()
            if parts and parts[0] in rows:
                rows[parts[0]].append(parts[1:])
    return rows


def check(path, f, rec):
    rows = text_scan(path)
    assert rec["n_vertices"] == len(rows["v"]), path
    assert rec["n_normals"] == len(rows["vn"]), path
    assert rec["n_uvs"] == len(rows["vt"]), path
    assert rec["n_faces"] == len(rows["f"]), path
    assert rec["objects"] == [r[0] for r in rows["o"] + rows["g"]] or len(rows["g"]) > 0, path
    for key, arr, k in (("v", f.Vertices, 3), ("vn", f.Normals, 3), ("vt", f.Uvs, 2)):
        if rows[key]:
            first = [np.float32(float(x)) for x in rows[key][0][:k]]
            last = [np.float32(float(x)) for x in rows[key][-1][:k]]
            assert [np.float32(x) for x in arr[:k]] == first, (path, key)
            assert [np.float32(x) for x in arr[-k:]] == last, (path, key)
    faces = [fc for ob in f.Objs for fc in ob.Faces]
    assert [len(fc.Vertices) for fc in faces] == [len(r) for r in rows["f"]], path
    if rows["f"]:
        first = rows["f"][0][0].split("/")
        assert faces[0].Vertices[0] == int(first[0]) - 1, path


def main(reference_root):
    d = testdata_dir(reference_root)
    if not os.path.isdir(d):
        sys.exit(f"no test assets at {d}")
    out = {}
    for path in sorted(glob.glob(os.path.join(d, "*.obj"))):
        f, rec = oracle_record(path)
        check(path, f, rec)
        out[os.path.basename(path)] = rec
        print(f"{os.path.basename(path)}: {rec['n_vertices']} v, {rec['n_normals']} vn, {rec['n_uvs']} vt, "
              f"{rec['n_faces']} f, objects {len(rec['objects'])}, materials {len(rec['materials'])}")
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_obj_fixtures.py <reference checkout>")
    main(sys.argv[1])
