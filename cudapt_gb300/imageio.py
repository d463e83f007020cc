"""Image files of the RMSE experiments and result export.

CudaPT writes its results as 8-bit PNG (libpng, RGBA, `NPGLHelper::saveRGBImagePNG`,
src/glhelper.cpp:192-262) and BMP (SOIL, `saveRGBImageBMP`, :62-66), and reads
Radiance RGBE (.hdr) environment images (`NPHDRHelper`, src/hdrhelper.cpp,
used by src/glhelper.cpp:94-113).  This module writes and reads those formats
from their published specifications (PNG: ISO/IEC 15948; BMP: the Windows
BITMAPINFOHEADER layout; RGBE: G. Ward, "Real Pixels", Graphics Gems II) with
the standard library only.

Float images use the renderer's layout: W*H*3 floats, row 0 at the bottom.
The 8-bit conversions themselves (clamp, exposure, gamma, byte truncation)
run on the GPU in ``gbpt_tonemap_rgba8``; see ``tonemap``.
"""
import struct
import zlib

import numpy as np


# ---- PNG -------------------------------------------------------------------
def _chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def write_png(path, rgba, width, height):
    """8-bit RGBA, rows top first (filter type 0 on every row)."""
    a = np.ascontiguousarray(rgba, np.uint8).reshape(height, width, 4)
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(height))
    ihdr = struct.pack(">IIBBBBB", width, height, 8, 6, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw, 6)) +
                _chunk(b"IEND", b""))


def _unfilter(ft, line, prev, bpp):
    out = bytearray(line)
    for i in range(len(out)):
        a = out[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        if ft == 1:
            out[i] = (out[i] + a) & 0xFF
        elif ft == 2:
            out[i] = (out[i] + b) & 0xFF
        elif ft == 3:
            out[i] = (out[i] + ((a + b) >> 1)) & 0xFF
        elif ft == 4:
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[i] = (out[i] + pr) & 0xFF
    return bytes(out)


def read_png(path):
    """8-bit RGB or RGBA, non-interlaced PNG -> (uint8 array H x W x C, width, height)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, w = 8, [], None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if zlib.crc32(kind + body) & 0xFFFFFFFF != struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]:
            raise ValueError(f"{path}: bad CRC in {kind!r}")
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body)
            if depth != 8 or ctype not in (2, 6) or inter:
                raise ValueError(f"{path}: only 8-bit RGB/RGBA non-interlaced PNG is supported")
            ch = 4 if ctype == 6 else 3
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + n
    raw = zlib.decompress(b"".join(idat))
    stride = w * ch
    rows, prev = [], bytes(stride)
    for y in range(h):
        line = raw[y * (stride + 1):(y + 1) * (stride + 1)]
        prev = _unfilter(line[0], line[1:], prev, ch)
        rows.append(prev)
    return np.frombuffer(b"".join(rows), np.uint8).reshape(h, w, ch), w, h


# ---- BMP -------------------------------------------------------------------
def write_bmp(path, rgb8, width, height):
    """24-bit BMP from 8-bit RGB rows top first (BMP stores them bottom first, BGR, 4-byte row padding)."""
    a = np.ascontiguousarray(rgb8, np.uint8).reshape(height, width, -1)[:, :, :3]
    pad = (4 - (width * 3) % 4) % 4
    rows = b"".join(a[y, :, ::-1].tobytes() + b"\x00" * pad for y in range(height - 1, -1, -1))
    header = struct.pack("<2sIHHI", b"BM", 54 + len(rows), 0, 0, 54)
    info = struct.pack("<IiiHHIIiiII", 40, width, height, 1, 24, 0, len(rows), 2835, 2835, 0, 0)
    with open(path, "wb") as f:
        f.write(header + info + rows)


def read_bmp(path):
    """24-bit uncompressed BMP -> (uint8 RGB rows top first, width, height)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:2] != b"BM":
        raise ValueError(f"{path}: not a BMP file")
    off = struct.unpack("<I", data[10:14])[0]
    w, h, _, bpp, comp = struct.unpack("<iiHHI", data[18:34])
    if bpp != 24 or comp != 0:
        raise ValueError(f"{path}: only 24-bit uncompressed BMP is supported")
    stride = (w * 3 + 3) & ~3
    flip = h > 0
    h = abs(h)
    rows = [np.frombuffer(data[off + y * stride:off + y * stride + w * 3], np.uint8).reshape(w, 3)[:, ::-1]
            for y in range(h)]
    a = np.stack(rows[::-1] if flip else rows)
    return a, w, h


# ---- Radiance RGBE (.hdr) --------------------------------------------------
def float_to_rgbe(rgb):
    """(N,3) float -> (N,4) uint8: mantissas scaled by 256/2^e of the largest channel, e + 128."""
    rgb = np.asarray(rgb, np.float32).reshape(-1, 3)
    v = rgb.max(axis=1)
    out = np.zeros((len(rgb), 4), np.uint8)
    ok = v >= 1e-32
    m, e = np.frexp(v[ok])  # v = m * 2^e, m in [0.5, 1)
    scale = (m * 256.0 / v[ok]).astype(np.float64)
    out[ok, :3] = np.floor(rgb[ok] * scale[:, None]).clip(0, 255).astype(np.uint8)
    out[ok, 3] = (e + 128).astype(np.uint8)
    return out


def rgbe_to_float(rgbe):
    """(N,4) uint8 -> (N,3) float32: (mantissa + 0.5) * 2^(e - 136) when e != 0."""
    q = np.asarray(rgbe, np.uint8).reshape(-1, 4)
    out = np.zeros((len(q), 3), np.float32)
    nz = q[:, 3] != 0
    f = np.ldexp(1.0, q[nz, 3].astype(np.int32) - (128 + 8))
    out[nz] = ((q[nz, :3].astype(np.float64) + 0.5) * f[:, None]).astype(np.float32)
    return out


def write_rgbe(path, rgb, width, height, rle=True):
    """Radiance .hdr of a float W*H*3 image with row 0 at the bottom ("-Y H +X W": top row first in the file)."""
    img = np.asarray(rgb, np.float32).reshape(height, width, 3)[::-1]
    px = float_to_rgbe(img.reshape(-1, 3)).reshape(height, width, 4)
    head = f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {height} +X {width}\n".encode()
    body = bytearray()
    for y in range(height):
        line = px[y]
        if not rle or width < 8 or width > 0x7FFF:
            body += line.tobytes()
            continue
        body += bytes([2, 2, width >> 8, width & 0xFF])
        for c in range(4):
            body += _rle_channel(line[:, c])
    with open(path, "wb") as f:
        f.write(head + bytes(body))


def _rle_channel(v):
    """New-style run-length encoding of one channel of a scanline: runs of >= 3 equal bytes
    as (128 + n, value), the rest as (n, bytes...), n <= 127."""
    out = bytearray()
    n, i = len(v), 0
    while i < n:
        j = i
        while j < n and j - i < 127 and v[j] == v[i]:
            j += 1
        if j - i >= 3:
            out += bytes([128 + (j - i), int(v[i])])
            i = j
            continue
        k = i
        while k < n and k - i < 127:
            if k + 2 < n and v[k] == v[k + 1] == v[k + 2]:
                break
            k += 1
        out += bytes([k - i]) + bytes(v[i:k].tolist())
        i = k
    return bytes(out)


def read_rgbe(path):
    """Radiance .hdr (flat or new-style RLE scanlines, "-Y H +X W") -> (float W*H*3 with row 0 at the bottom, W, H)."""
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    fmt = None
    if not data.startswith(b"#?"):
        raise ValueError(f"{path}: missing #? header")
    while True:
        end = data.index(b"\n", pos)
        line = data[pos:end].decode("ascii", "replace")
        pos = end + 1
        if line == "":
            break
        if line.startswith("FORMAT="):
            fmt = line[7:]
    if fmt not in (None, "32-bit_rle_rgbe"):
        raise ValueError(f"{path}: unsupported format {fmt}")
    end = data.index(b"\n", pos)
    dims = data[pos:end].decode().split()
    pos = end + 1
    if len(dims) != 4 or dims[0] != "-Y" or dims[2] != "+X":
        raise ValueError(f"{path}: unsupported orientation {' '.join(dims)}")
    h, w = int(dims[1]), int(dims[3])
    px = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w <= 0x7FFF and data[pos] == 2 and data[pos + 1] == 2 and not (data[pos + 2] & 0x80):
            if (data[pos + 2] << 8 | data[pos + 3]) != w:
                raise ValueError(f"{path}: scanline width mismatch")
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        n -= 128
                        px[y, x:x + n, c] = data[pos]
                        pos += 1
                    else:
                        if n == 0 or x + n > w:
                            raise ValueError(f"{path}: bad run length")
                        px[y, x:x + n, c] = np.frombuffer(data[pos:pos + n], np.uint8)
                        pos += n
                    x += n
        else:
            px[y] = np.frombuffer(data[pos:pos + 4 * w], np.uint8).reshape(w, 4)
            pos += 4 * w
    rgb = rgbe_to_float(px.reshape(-1, 4)).reshape(h, w, 3)[::-1]
    return np.ascontiguousarray(rgb).reshape(-1), w, h


# ---- conversions on the GPU --------------------------------------------------
TONEMAP_RESULT, TONEMAP_MSE, TONEMAP_CLAMP = 0, 1, 2


def tonemap(rgb, width, height, exposure=1.0, kind=TONEMAP_RESULT, ref=None):
    """8-bit RGBA (rows top first) of a float image, computed by ``gbpt_tonemap_rgba8``."""
    import ctypes

    from ._native import check, load, ptr
    a = np.ascontiguousarray(rgb, np.float32).reshape(-1)
    r = None if ref is None else np.ascontiguousarray(ref, np.float32).reshape(-1)
    out = np.zeros((height, width, 4), np.uint8)
    check(load().gbpt_tonemap_rgba8(ptr(a), ptr(r) if r is not None else None, width, height,
                                     ctypes.c_float(exposure), kind, ptr(out), 0))
    return out


def save_result_png(path, rgb, width, height, exposure=1.0):
    """CUDAPTWindow::BrowseAndSaveResult (src/cudapt.cpp:482-522)."""
    write_png(path, tonemap(rgb, width, height, exposure, TONEMAP_RESULT), width, height)


def save_mse_png(path, rgb, converged, width, height):
    """CUDAPTWindow::BrowseAndSaveMSEResult (src/cudapt.cpp:553-586)."""
    write_png(path, tonemap(rgb, width, height, 1.0, TONEMAP_MSE, converged), width, height)


def save_converged_bmp(path, converged, width, height):
    """CUDAPTWindow::ExportConvergedResult (src/cudapt.cpp:867-896)."""
    write_bmp(path, tonemap(converged, width, height, 1.0, TONEMAP_CLAMP)[:, :, :3], width, height)


def rmse(a, b):
    """sqrt(mean((a - b)^2)) on the GPU (``gbpt_rmse``, double accumulation)."""
    import ctypes

    from ._native import check, load, ptr
    x = np.ascontiguousarray(a, np.float32).reshape(-1)
    y = np.ascontiguousarray(b, np.float32).reshape(-1)
    if x.size != y.size:
        raise ValueError("images differ in size")
    out = ctypes.c_double()
    check(load().gbpt_rmse(ptr(x), ptr(y), x.size, 0, ctypes.addressof(out)))
    return out.value

