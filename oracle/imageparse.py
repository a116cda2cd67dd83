"""PNG loading oracle (TEST INFRASTRUCTURE).

A pure-Python restatement of what imageutil.LoadImage (internal/imageutil/
image.go:47-106) does to a PNG: Go's image/png reader (chunks, tRNS,
Adam7, the five scanline filters, the image type per colour type and
depth), draw.Draw to *image.RGBA, and the GammaCorrect byte map built from
color/srgb.go's tables. Per-pixel loops: small images only. Used by tests/
to check polyred_gb300.imageload; never by the product.
"""
import math
import struct
import zlib

import numpy as np

F32 = np.float32


def _go_pow(x, y):
    """math.Pow for finite x > 0, y > 0 (Go math/pow.go)."""
    if y == 0 or x == 1:
        return 1.0
    if y == 1:
        return x
    yi, yf = float(int(y)), y - int(y)
    a1, ae = 1.0, 0
    if yf != 0:
        if yf > 0.5:
            yf -= 1
            yi += 1
        a1 = math.exp(yf * math.log(x))
    x1, xe = math.frexp(x)
    i = int(yi)
    while i != 0:
        if xe < -(1 << 12) or (1 << 12) < xe:
            ae += xe
            break
        if i & 1 == 1:
            a1 *= x1
            ae += xe
        x1 *= x1
        xe <<= 1
        if x1 < 0.5:
            x1 += x1
            xe -= 1
        i >>= 1
    return math.ldexp(a1, max(-4096, min(4096, ae)))


def srgb_decode_table():
    """uint8(FromsRGB2Linear(float32(b)/0xff)*0xff + 0.5) for every byte b."""
    lut = []
    for i in range(1024):
        v = i / 1024
        lut.append(v / 12.92 if v <= 0.04045 else _go_pow((v + 0.055) / 1.055, 2.4))
    lut.append(lut[1023])
    out = []
    for b in range(256):
        v = F32(F32(b) / F32(255))
        if v <= 0:
            s = F32(0)
        elif v >= 1:
            s = F32(1)
        else:
            i = F32(v * F32(1024))
            fl = int(i) & 1023
            v0, v1 = F32(lut[fl]), F32(lut[fl + 1])
            i = F32(i - F32(fl))
            s = F32(F32(v0 * F32(F32(1) - i)) + F32(v1 * i))
        q = F32(F32(s * F32(255)) + F32(0.5))
        out.append(int(q) & 0xFF)
    return out


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    if pb <= pc:
        return b
    return c


def _unfilter(raw, pos, rows, row_bytes, bpp):
    out, prev = [], [0] * row_bytes
    for _ in range(rows):
        f = raw[pos]
        cur = list(raw[pos + 1:pos + 1 + row_bytes])
        pos += 1 + row_bytes
        for i in range(row_bytes):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if f == 0:
                d = 0
            elif f == 1:
                d = a
            elif f == 2:
                d = b
            elif f == 3:
                d = (a + b) // 2
            elif f == 4:
                d = _paeth(a, b, c)
            else:
                raise ValueError("png: invalid format: bad filter type")
            cur[i] = (cur[i] + d) & 0xFF
        out.append(cur)
        prev = cur
    return out, pos


def _nrgba(r, g, b, a):
    """color.NRGBA -> draw.Draw into image.RGBA."""
    sa = a * 0x101
    return [(r * sa // 0xFF) >> 8, (g * sa // 0xFF) >> 8, (b * sa // 0xFF) >> 8, sa >> 8]


def _nrgba64(r, g, b, a):
    return [(r * a // 0xFFFF) >> 8, (g * a // 0xFFFF) >> 8, (b * a // 0xFFFF) >> 8, a >> 8]


def decode(data):
    """PNG bytes -> (H, W, 4) uint8 as LoadImage holds it before gamma."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos = 8
    ihdr, plte, trns, idat = None, None, None, b""
    allowed = {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if len(body) != n or len(data[pos + 8 + n:pos + 12 + n]) != 4:
            raise ValueError("png: unexpected EOF")
        if zlib.crc32(kind + body) & 0xFFFFFFFF != struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]:
            raise ValueError("png: invalid format: invalid checksum")
        if ihdr is None and kind != b"IHDR":
            raise ValueError("png: invalid format: chunk out of order")
        if kind == b"IHDR":  # parseIHDR's checks
            if n != 13:
                raise ValueError("png: invalid format: bad IHDR length")
            ihdr = struct.unpack(">IIBBBBB", body)
            w_, h_, d_, c_, comp, filt, inter_ = ihdr
            if comp != 0 or filt != 0 or inter_ not in (0, 1):
                raise ValueError("png: unsupported feature: compression, filter or interlace method")
            if c_ not in allowed or d_ not in allowed[c_]:
                raise ValueError("png: unsupported feature: bit depth / color type")
            if w_ <= 0 or h_ <= 0 or w_ >= 1 << 31 or h_ >= 1 << 31:
                raise ValueError("png: invalid format: invalid dimension")
        elif kind == b"PLTE":
            if idat or n % 3 or n == 0 or n // 3 > 256 or (ihdr[3] == 3 and n // 3 > 1 << ihdr[2]):
                raise ValueError("png: invalid format: bad PLTE")
            plte = [tuple(body[3 * i:3 * i + 3]) + (0xFF,) for i in range(n // 3)]
        elif kind == b"tRNS":
            c_ = ihdr[3]
            if c_ in (4, 6) or idat or (c_ == 3 and plte is None) or (c_ == 0 and n != 2) or (c_ == 2 and n != 6) \
                    or n > 256:
                raise ValueError("png: invalid format: bad tRNS")
            trns = body
        elif kind == b"IDAT":
            if ihdr[3] == 3 and plte is None:
                raise ValueError("png: invalid format: chunk out of order")
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + n
    if ihdr is None or not idat:
        raise ValueError("png: invalid format: missing IDAT")
    w, h, depth, ctype, _, _, inter = ihdr
    raw = zlib.decompress(idat)
    nch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = depth * nch
    bpp = max(1, bits // 8)
    palette = None
    if ctype == 3:
        palette = [("rgba", c) for c in plte] + [("rgba", (0, 0, 0, 0xFF))] * (256 - len(plte))
        if trns is not None:
            for i in range(len(trns)):
                palette[i] = ("nrgba", palette[i][1][:3] + (trns[i],))
    img = np.zeros((h, w, 4), np.uint8)
    passes = [(8, 8, 0, 0), (8, 8, 4, 0), (4, 8, 0, 4), (4, 4, 2, 0), (2, 4, 0, 2), (2, 2, 1, 0), (1, 2, 0, 1)] \
        if inter else [(1, 1, 0, 0)]
    pos = 0
    for dx, dy, x0, y0 in passes:
        pw, ph = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
        if pw <= 0 or ph <= 0:
            continue
        row_bytes = (pw * bits + 7) // 8
        if pos + ph * (row_bytes + 1) > len(raw):
            raise ValueError("png: invalid format: not enough pixel data")
        rows, pos = _unfilter(raw, pos, ph, row_bytes, bpp)
        for ry, row in enumerate(rows):
            for rx in range(pw):
                if depth < 8:
                    bit = rx * depth
                    s = [(row[bit // 8] >> (8 - depth - bit % 8)) & ((1 << depth) - 1)]
                elif depth == 8:
                    s = row[rx * nch:(rx + 1) * nch]
                else:
                    s = [(row[2 * (rx * nch + k)] << 8) | row[2 * (rx * nch + k) + 1] for k in range(nch)]
                if ctype == 0:
                    y = s[0] * (0xFF // ((1 << depth) - 1)) if depth < 8 else s[0]
                    if trns is not None:
                        if depth == 16:
                            t = (trns[0] << 8) | trns[1]
                            px = _nrgba64(y, y, y, 0 if y == t else 0xFFFF)
                        else:
                            t = (trns[1] * (0xFF // ((1 << depth) - 1))) & 0xFF
                            px = _nrgba(y, y, y, 0 if y == t else 0xFF)
                    else:
                        px = [y >> 8] * 3 + [0xFF] if depth == 16 else [y] * 3 + [0xFF]
                elif ctype == 2:
                    if trns is not None:
                        if depth == 16:
                            t = [(trns[2 * k] << 8) | trns[2 * k + 1] for k in range(3)]
                            px = _nrgba64(*s, 0 if list(s) == t else 0xFFFF)
                        else:
                            t = [trns[1], trns[3], trns[5]]
                            px = _nrgba(*s, 0 if list(s) == t else 0xFF)
                    else:
                        px = [v >> 8 for v in s] + [0xFF] if depth == 16 else list(s) + [0xFF]
                elif ctype == 3:
                    kind, c = palette[s[0]]
                    px = list(c) if kind == "rgba" else _nrgba(*c)
                elif ctype == 4:
                    px = _nrgba64(s[0], s[0], s[0], s[1]) if depth == 16 else _nrgba(s[0], s[0], s[0], s[1])
                else:
                    px = _nrgba64(*s) if depth == 16 else _nrgba(*s)
                img[y0 + ry * dy, x0 + rx * dx] = px
    if pos != len(raw):
        raise ValueError("png: invalid format: too much pixel data")
    return img


def load_image(path, gamma_correct=False):
    with open(path, "rb") as fh:
        img = decode(fh.read())
    if gamma_correct:
        t = np.array(srgb_decode_table(), np.uint8)
        img[..., :3] = t[img[..., :3]]
    return img
