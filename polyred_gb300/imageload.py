"""Image files for textures: imageutil.LoadImage (internal/imageutil/
image.go:47-106) for PNG.

  load_image(path, gamma_correct=False) -> (H, W, 4) uint8, rows top-down

LoadImage decodes the file (image.Decode), converts it to *image.RGBA with
draw.Draw(..., draw.Src) and, with GammaCorrect(true), maps R, G and B of
every pixel from sRGB to linear (pr_srgb_decode_table). Here the PNG
decoder follows Go's image/png: every colour type and bit depth, tRNS,
Adam7 interlacing, CRC checks; the scanline filters are undone natively
(pr_png_unfilter). The conversion to RGBA is Go's: non-premultiplied
colours (NRGBA, with tRNS or an alpha channel) become (c * a*0x101 / 0xff)
>> 8, 16-bit samples keep their high byte, palette indices past the palette
are opaque black. JPEG and other formats raise NotImplementedError.
"""
import struct
import zlib

import numpy as np

from . import native

PNG_SIG = b"\x89PNG\r\n\x1a\n"

# (dx, dy, x0, y0) of the seven Adam7 passes
ADAM7 = [(8, 8, 0, 0), (8, 8, 4, 0), (4, 8, 0, 4), (4, 4, 2, 0), (2, 4, 0, 2), (2, 2, 1, 0), (1, 2, 0, 1)]

# channels per colour type: 0 gray, 2 RGB, 3 palette, 4 gray+alpha, 6 RGBA
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
DEPTHS = {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}


class PNGError(ValueError):
    """image/png's FormatError / UnsupportedError."""


_TABLE = None


def srgb_decode_table():
    """LoadImage's gamma map for one byte (pr_srgb_decode_table)."""
    global _TABLE
    if _TABLE is None:
        t = np.zeros(256, np.uint8)
        native.check(native.load().pr_srgb_decode_table(t.ctypes.data))
        _TABLE = t
    return _TABLE


def _chunks(data):
    if data[:8] != PNG_SIG:
        raise PNGError("png: invalid format: not a PNG file")
    pos = 8
    while True:
        if pos + 8 > len(data):
            raise PNGError("png: invalid format: unexpected EOF")
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        crc = data[pos + 8 + n:pos + 12 + n]
        if len(body) != n or len(crc) != 4:
            raise PNGError("png: invalid format: unexpected EOF")
        if zlib.crc32(kind + body) & 0xFFFFFFFF != struct.unpack(">I", crc)[0]:
            raise PNGError("png: invalid format: invalid checksum")
        yield kind, body
        if kind == b"IEND":
            return
        pos += 12 + n


def _unfilter(raw, height, row_bytes, bpp):
    out = np.zeros(height * row_bytes, np.uint8)
    if height == 0 or row_bytes == 0:
        return out.reshape(height, row_bytes)
    src = np.frombuffer(raw, np.uint8)
    st = native.load().pr_png_unfilter(src.ctypes.data, height, row_bytes, bpp, out.ctypes.data)
    if st != 0:
        raise PNGError("png: invalid format: bad filter type")
    return out.reshape(height, row_bytes)


def _samples(rows, width, depth, nch):
    """Unfiltered rows -> (h, width, nch) integer samples."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :width * nch].reshape(h, width, nch).astype(np.uint16)
    if depth == 16:
        b = rows[:, :width * nch * 2].reshape(h, width * nch, 2).astype(np.uint16)
        return ((b[..., 0] << 8) | b[..., 1]).reshape(h, width, nch)
    per = 8 // depth  # sub-byte samples (nch == 1), most significant first
    shifts = np.arange(per - 1, -1, -1, dtype=np.uint16) * depth
    v = (rows[:, :, None].astype(np.uint16) >> shifts) & ((1 << depth) - 1)
    return v.reshape(h, -1)[:, :width].reshape(h, width, 1)


def _premultiply(rgb, a, full):
    """NRGBA(64) -> RGBA bytes as draw.Draw does: 8-bit c*a*0x101/0xff >> 8,
    16-bit c*a/0xffff >> 8."""
    rgb = rgb.astype(np.uint64)
    a = a.astype(np.uint64)
    if full == 0xFF:
        return ((rgb * (a * 0x101)[..., None]) // 0xFF) >> 8, (a * 0x101) >> 8
    return ((rgb * a[..., None]) // 0xFFFF) >> 8, a >> 8


def decode_png(data):
    """image/png Decode + draw.Draw to *image.RGBA: (H, W, 4) uint8."""
    ihdr = None
    palette = None
    n_plte = 0
    trns = None
    idat = []
    for kind, body in _chunks(bytes(data)):
        if ihdr is None and kind != b"IHDR":
            raise PNGError("png: invalid format: missing IHDR")
        if kind == b"IHDR":
            if len(body) != 13:
                raise PNGError("png: invalid format: bad IHDR length")
            w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", body)
            if ctype not in DEPTHS or depth not in DEPTHS[ctype]:
                raise PNGError(f"png: unsupported feature: bit depth {depth}, color type {ctype}")
            if comp != 0 or filt != 0 or inter > 1:
                raise PNGError("png: unsupported feature: compression, filter or interlace method")
            if w <= 0 or h <= 0 or w >= 1 << 31 or h >= 1 << 31:
                raise PNGError("png: invalid format: non-positive dimension")
            ihdr = (w, h, depth, ctype, inter)
        elif kind == b"PLTE":
            if idat:
                raise PNGError("png: invalid format: chunk out of order")
            if len(body) % 3 or len(body) // 3 > 256 or len(body) == 0:
                raise PNGError("png: invalid format: bad PLTE length")
            n = n_plte = len(body) // 3
            palette = np.zeros((256, 4), np.uint16)
            palette[:, 3] = 0xFF  # entries past the palette: opaque black
            palette[:n, :3] = np.frombuffer(body, np.uint8).reshape(n, 3)
        elif kind == b"tRNS":
            if ihdr[3] in (4, 6):
                raise PNGError("png: invalid format: tRNS, color type mismatch")
            if idat or (ihdr[3] == 3 and palette is None):
                raise PNGError("png: invalid format: chunk out of order")
            trns = body
        elif kind == b"IDAT":
            if ihdr[3] == 3 and palette is None:
                raise PNGError("png: invalid format: chunk out of order")
            idat.append(body)
    if ihdr is None or not idat:
        raise PNGError("png: invalid format: missing IDAT")
    w, h, depth, ctype, inter = ihdr
    if ctype == 3 and palette is None:
        raise PNGError("png: invalid format: missing palette")
    if ctype == 3 and n_plte > 1 << depth:
        raise PNGError("png: invalid format: bad PLTE length")
    nch = CHANNELS[ctype]
    bits = depth * nch
    bpp = max(1, bits // 8)
    try:
        raw = zlib.decompress(b"".join(idat))
    except zlib.error as e:
        raise PNGError(f"png: invalid format: {e}") from None

    passes = ADAM7 if inter else [(1, 1, 0, 0)]
    samples = np.zeros((h, w, nch), np.uint16)
    pos = 0
    for dx, dy, x0, y0 in passes:
        pw, ph = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
        if pw <= 0 or ph <= 0:
            continue
        row_bytes = (pw * bits + 7) // 8
        n = ph * (row_bytes + 1)
        if pos + n > len(raw):
            raise PNGError("png: invalid format: not enough pixel data")
        rows = _unfilter(raw[pos:pos + n], ph, row_bytes, bpp)
        pos += n
        samples[y0::dy, x0::dx] = _samples(rows, pw, depth, nch)
    if pos != len(raw):
        raise PNGError("png: invalid format: too much pixel data")

    out = np.zeros((h, w, 4), np.uint8)
    full = 0xFFFF if depth == 16 else 0xFF
    hi = (lambda v: v >> 8) if depth == 16 else (lambda v: v)
    if ctype == 0:  # gray
        y = samples[..., 0]
        if depth < 8:
            y = y * (0xFF // ((1 << depth) - 1))
        if trns is not None:
            if len(trns) != 2:
                raise PNGError("png: invalid format: bad tRNS length")
            t = (trns[0] << 8) | trns[1] if depth == 16 else trns[1] * (0xFF // ((1 << depth) - 1)) % 256
            a = np.where(y == t, 0, full)
            c, aa = _premultiply(np.stack([y, y, y], -1), a, full)
            out[..., :3], out[..., 3] = c, aa
        else:
            out[..., :3] = hi(y)[..., None]
            out[..., 3] = 0xFF
    elif ctype == 2:  # RGB
        rgb = samples
        if trns is not None:
            if len(trns) != 6:
                raise PNGError("png: invalid format: bad tRNS length")
            t = [(trns[2 * k] << 8) | trns[2 * k + 1] if depth == 16 else trns[2 * k + 1] for k in range(3)]
            a = np.where((rgb[..., 0] == t[0]) & (rgb[..., 1] == t[1]) & (rgb[..., 2] == t[2]), 0, full)
            c, aa = _premultiply(rgb, a, full)
            out[..., :3], out[..., 3] = c, aa
        else:
            out[..., :3] = hi(rgb)
            out[..., 3] = 0xFF
    elif ctype == 3:  # palette
        pal = palette.copy()
        nrgba = np.zeros(256, bool)
        if trns is not None:  # entries become color.NRGBA, past the PLTE too
            if len(trns) > 256:
                raise PNGError("png: invalid format: bad tRNS length")
            pal[:len(trns), 3] = np.frombuffer(trns, np.uint8)
            nrgba[:len(trns)] = True
        idx = samples[..., 0].astype(np.intp)
        rgb, a = pal[idx, :3], pal[idx, 3]
        c, aa = _premultiply(rgb, a, 0xFF)
        keep = ~nrgba[idx]  # color.RGBA entries pass through
        out[..., :3] = np.where(keep[..., None], rgb, c)
        out[..., 3] = np.where(keep, a, aa)
    else:  # gray + alpha, RGBA: NRGBA / NRGBA64
        color = samples[..., :1].repeat(3, -1) if ctype == 4 else samples[..., :3]
        c, aa = _premultiply(color, samples[..., -1], full)
        out[..., :3], out[..., 3] = c, aa
    return out


def load_image(path, gamma_correct=False):
    """imageutil.LoadImage(path, GammaCorrect(gamma_correct))."""
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:8] != PNG_SIG:
        raise NotImplementedError(f"{path}: only PNG images are decoded (image.Decode's other formats are not)")
    img = decode_png(data)
    if gamma_correct:
        img[..., :3] = srgb_decode_table()[img[..., :3]]
    return img
