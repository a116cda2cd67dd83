"""Texture image loading (polyred_gb300.imageload: imageutil.LoadImage for
PNG) against the oracle's per-pixel restatement of Go's image/png reader
and draw.Draw: PNGs made here with every colour type and bit depth, all
five filters, Adam7, tRNS, out-of-range palette indices; the GammaCorrect
byte map; malformed files; an OBJ whose map_Kd is a PNG. No GPU."""
import os
import struct
import zlib

import numpy as np
import pytest

from oracle import imageparse as ip
from polyred_gb300 import imageload, objload

ADAM7 = [(8, 8, 0, 0), (8, 8, 4, 0), (4, 8, 0, 4), (4, 4, 2, 0), (2, 4, 0, 2), (2, 2, 1, 0), (1, 2, 0, 1)]
NCH = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


@pytest.fixture(autouse=True)
def _lib(native_lib):
    return native_lib


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _pack_row(s, depth):
    """samples (w, nch) -> PNG row bytes."""
    flat = s.reshape(-1)
    if depth == 16:
        return b"".join(struct.pack(">H", int(v)) for v in flat)
    if depth == 8:
        return bytes(int(v) for v in flat)
    per = 8 // depth
    out = bytearray((len(flat) * depth + 7) // 8)
    for i, v in enumerate(flat):
        out[i // per] |= int(v) << (8 - depth - (i % per) * depth)
    return bytes(out)


def _filter(row, prev, f, bpp):
    out = bytearray(len(row))
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        pred = [0, a, b, (a + b) // 2, ip._paeth(a, b, c)][f]
        out[i] = (row[i] - pred) & 0xFF
    return bytes([f]) + bytes(out)


def encode_png(samples, depth, ctype, plte=None, trns=None, interlace=False, seed=0):
    h, w, nch = samples.shape
    rng = np.random.default_rng(seed)
    bpp = max(1, depth * nch // 8)
    raw = b""
    for dx, dy, x0, y0 in (ADAM7 if interlace else [(1, 1, 0, 0)]):
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prev = bytes(len(_pack_row(sub[0], depth)))
        for r in range(sub.shape[0]):
            row = _pack_row(sub[r], depth)
            raw += _filter(row, prev, int(rng.integers(0, 5)), bpp)
            prev = row
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if plte is not None:
        data += _chunk(b"PLTE", bytes(np.asarray(plte, np.uint8).reshape(-1)))
    if trns is not None:
        data += _chunk(b"tRNS", bytes(trns))
    data += _chunk(b"IDAT", zlib.compress(raw)[:7]) + _chunk(b"IDAT", zlib.compress(raw)[7:])
    return data + _chunk(b"IEND", b"")


CASES = [(ct, d) for ct, ds in imageload.DEPTHS.items() for d in ds]


@pytest.mark.parametrize("ctype,depth", CASES)
@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("with_trns", [False, True])
def test_png_decode_matches_oracle(ctype, depth, interlace, with_trns):
    if with_trns and ctype in (4, 6):
        pytest.skip("tRNS is not used with an alpha channel")
    seed = ctype * 1000 + depth * 10 + interlace * 3 + with_trns
    rng = np.random.default_rng(seed)
    h, w = (13, 17) if interlace else (7, 9)
    top = (1 << depth) - 1
    samples = rng.integers(0, top + 1, (h, w, NCH[ctype]))
    plte = trns = None
    if ctype == 3:
        n = min(top + 1, 5)
        plte = rng.integers(0, 256, (n, 3))
        if depth >= 4:
            samples[0, :3, 0] = [n, n + 1, top]  # indices past the palette: opaque black
        if with_trns:
            trns = list(rng.integers(0, 256, min(n + 1, top + 1)))
    elif with_trns:
        pick = samples[1, 1]  # a colour that occurs
        if depth == 16:
            trns = [b for v in (pick if ctype == 2 else pick[:1]) for b in (int(v) >> 8, int(v) & 0xFF)]
        else:
            trns = [b for v in (pick if ctype == 2 else pick[:1]) for b in (0, int(v))]
    data = encode_png(samples, depth, ctype, plte, trns, interlace, seed)
    got = imageload.decode_png(data)
    want = ip.decode(data)
    assert got.shape == (h, w, 4)
    assert np.array_equal(got, want)


def test_gamma_table_matches_oracle():
    assert imageload.srgb_decode_table().tolist() == ip.srgb_decode_table()
    t = imageload.srgb_decode_table()
    assert t[0] == 0 and t[255] == 255 and (np.diff(t.astype(int)) >= 0).all()


def test_load_image_gamma(tmp_path):
    rng = np.random.default_rng(5)
    samples = rng.integers(0, 256, (20, 30, 4))
    p = tmp_path / "t.png"
    p.write_bytes(encode_png(samples, 8, 6, seed=5))
    for g in (False, True):
        assert np.array_equal(imageload.load_image(str(p), gamma_correct=g), ip.load_image(str(p), gamma_correct=g))


def test_malformed_pngs(tmp_path):
    good = encode_png(np.zeros((3, 3, 3), int), 8, 2)
    bad_crc = good[:-5] + bytes([good[-5] ^ 1]) + good[-4:]
    with pytest.raises(ValueError, match="checksum"):
        imageload.decode_png(bad_crc)
    with pytest.raises(ValueError):
        imageload.decode_png(good[:40])
    raw = zlib.compress(b"\x07" + bytes(9) + b"\x00" + bytes(9) + b"\x00" + bytes(9))  # filter type 7
    bad_filter = good[:33] + _chunk(b"IDAT", raw) + _chunk(b"IEND", b"")
    with pytest.raises(ValueError, match="filter"):
        imageload.decode_png(bad_filter)
    p = tmp_path / "x.jpg"
    p.write_bytes(b"\xff\xd8\xff\xe0" + bytes(20))
    with pytest.raises(NotImplementedError):
        imageload.load_image(str(p))


def test_reference_png_assets():
    """The reference's small PNG test assets, when present, decode alike."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from helpers import reference_testdata
    d = reference_testdata()
    if not os.path.isdir(d):
        pytest.skip("reference assets not present")
    names = [n for n in sorted(os.listdir(d)) if n.endswith(".png") and os.path.getsize(os.path.join(d, n)) < 40000]
    assert names
    for n in names:
        path = os.path.join(d, n)
        assert np.array_equal(imageload.load_image(path, True), ip.load_image(path, True)), n


def test_obj_map_kd_png(tmp_path):
    """model.Load of an OBJ whose material has a PNG map_Kd: the material's
    texture is the gamma-corrected image, mipmapped."""
    rng = np.random.default_rng(9)
    samples = rng.integers(0, 256, (16, 8, 3))
    (tmp_path / "tex.png").write_bytes(encode_png(samples, 8, 2, seed=9))
    (tmp_path / "m.mtl").write_text("newmtl a\nKd 1 1 1\nKs 0.5 0.5 0.5\nNs 10\nillum 2\nmap_Kd tex.png\n")
    (tmp_path / "m.obj").write_text("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 0 1\n"
                                    "f 1/1 2/2 3/3\n")
    g = objload.load(str(tmp_path / "m.obj"))
    tex = g.objects[0].materials[0].texture
    assert tex.mipmap and tex.size() == 8
    assert np.array_equal(tex.rgba, ip.load_image(str(tmp_path / "tex.png"), gamma_correct=True))
    g2 = objload.load(str(tmp_path / "m.obj"), image_textures="ignore")
    assert g2.objects[0].materials[0].texture == (0, 0, 255, 255)


def _reassemble(chunks):
    return b"\x89PNG\r\n\x1a\n" + b"".join(_chunk(k, bytes(b)) for k, b in chunks)


def _split(data):
    pos, out = 8, []
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        out.append([kind, bytearray(data[pos + 8:pos + 8 + n])])
        pos += 12 + n
    return out


@pytest.mark.parametrize("seed", range(120))
def test_mutated_pngs_match_oracle(seed):
    """Seeded damage with valid CRCs (scanline bytes, IHDR fields, a tRNS of
    any length, chunk order): both decoders give the same image or both
    reject the file."""
    import random
    rng = random.Random(0x9A1 + seed)
    ctype, depth = rng.choice(CASES)
    h, w = rng.randrange(1, 12), rng.randrange(1, 12)
    top = (1 << depth) - 1
    s = np.random.default_rng(seed).integers(0, top + 1, (h, w, NCH[ctype]))
    plte = np.random.default_rng(seed).integers(0, 256, (min(top + 1, 6), 3)) if ctype == 3 else None
    cs = _split(encode_png(s, depth, ctype, plte, None, rng.random() < 0.5, seed))
    k = rng.randrange(4)
    if k == 0:
        raw = bytearray(zlib.decompress(b"".join(bytes(b) for kind, b in cs if kind == b"IDAT")))
        for _ in range(rng.randrange(1, 4)):
            if raw and rng.random() < 0.5:
                raw[rng.randrange(len(raw))] = rng.randrange(256)
            elif raw and rng.random() < 0.5:
                del raw[rng.randrange(len(raw))]
            else:
                raw.insert(rng.randrange(len(raw) + 1), rng.randrange(256))
        cs = [c for c in cs if c[0] != b"IDAT"]
        cs.insert(-1, [b"IDAT", bytearray(zlib.compress(bytes(raw)))])
    elif k == 1:
        cs[0][1][rng.choice([8, 9, 12])] = rng.choice([0, 1, 2, 3, 4, 6, 8, 16, 7])
    elif k == 2:
        cs.insert(rng.randrange(1, len(cs)), [b"tRNS", bytearray(rng.randrange(256) for _ in range(rng.choice([2, 3, 6, 9])))])
    data = _reassemble(cs)
    try:
        want = ip.decode(data)
    except ValueError:
        with pytest.raises(ValueError):
            imageload.decode_png(data)
        return
    assert np.array_equal(imageload.decode_png(data), want)


def test_reference_load_image_golden():
    """TestLoadImage (internal/imageutil/image_test.go:16-41): ground.png
    loaded with GammaCorrect(true) equals golden.png pixel for pixel."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from helpers import reference_testdata
    d = reference_testdata()
    ground, golden = os.path.join(d, "ground.png"), os.path.join(d, "golden.png")
    if not (os.path.exists(ground) and os.path.exists(golden)):
        pytest.skip("reference test assets not present")
    got = imageload.load_image(ground, gamma_correct=True)
    want = imageload.load_image(golden, gamma_correct=False)
    assert got.shape == want.shape
    assert np.array_equal(got, want)
