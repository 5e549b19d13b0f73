"""Image files: PNG for screenshots (8-bit RGB, as ScreenShot.cpp's crop; the reference encodes
JPEG or AVIF through third-party encoders, ScreenShot.cpp:18-205), PFM (portable float map) for
linear HDR dumps, and the texture inputs: PNG images of glTF materials (8-bit, any colour type,
every filter, not interlaced) and Radiance RGBE (.hdr) skies, decoded as the reference's loader
decodes them (stbi_loadf: channel m of a pixel with exponent byte e is m 2^(e - 136), 0 when e
is 0, alpha 1; GlobalTexturePool::LoadHDRTexture, src/Assets/Texture.cpp:275, 432-446).
Standard library and numpy only."""
import struct
import zlib

import numpy as np


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def encode_png(rgb: np.ndarray) -> bytes:
    """(h, w, 3) or (h, w, 4) uint8 -> PNG bytes (8-bit RGB / RGBA, no filtering)."""
    a = np.ascontiguousarray(rgb, np.uint8)
    if a.ndim != 3 or a.shape[2] not in (3, 4):
        raise ValueError("expected an (h, w, 3|4) uint8 image")
    h, w, c = a.shape
    raw = np.concatenate([np.zeros((h, 1), np.uint8), a.reshape(h, w * c)], axis=1).tobytes()
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 2 if c == 3 else 6, 0, 0, 0)
    return b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b"")


_PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}   # colour type -> samples per pixel


def _unfilter(raw: np.ndarray, h: int, stride: int, bpp: int) -> np.ndarray:
    """PNG scanline filters 0-4 (None, Sub, Up, Average, Paeth) undone row by row."""
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft = raw[y, 0]
        line = raw[y, 1:].astype(np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft in (1, 3, 4):
            cur = np.zeros(stride, np.int32)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                if ft == 1:
                    p = a
                elif ft == 3:
                    p = (a + b) >> 1
                else:
                    c = prev[x - bpp] if x >= bpp else 0
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 0xFF
        else:
            raise ValueError(f"unknown PNG filter {ft}")
        out[y] = cur
        prev = cur
    return out


def decode_png(data: bytes, rgba: bool = False) -> np.ndarray:
    """PNG bytes (8-bit samples, colour types 0, 2, 3, 4, 6, no interlacing) -> (h, w, c) uint8:
    RGB and RGBA images as stored (c = 3, 4) unless rgba is set; grey, grey-alpha and palette
    images, and every image with rgba set, as RGBA (grey expanded, the palette through PLTE and
    tRNS, missing alpha 255)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr, plte, trns = 8, b"", None, None, None
    while pos + 8 <= len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body[:13])
        elif tag == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
        pos += 12 + n
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or ctype not in _PNG_CHANNELS or interlace != 0:
        raise ValueError("only non-interlaced 8-bit PNG images are read")
    c = _PNG_CHANNELS[ctype]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)
    if raw.size != h * (1 + w * c):
        raise ValueError("PNG image data of the wrong size")
    px = _unfilter(raw.reshape(h, 1 + w * c), h, w * c, c).reshape(h, w, c)
    if ctype in (2, 6) and not rgba:
        return px.copy()
    out = np.full((h, w, 4), 255, np.uint8)
    if ctype == 3:
        if plte is None:
            raise ValueError("palette image without PLTE")
        i = px[..., 0]
        out[..., :3] = plte[np.minimum(i, plte.shape[0] - 1)]
        if trns is not None:
            alpha = np.full(256, 255, np.uint8)
            alpha[:trns.size] = trns[:256]
            out[..., 3] = alpha[i]
    elif ctype in (0, 4):
        out[..., :3] = px[..., :1]
        if ctype == 4:
            out[..., 3] = px[..., 1]
    else:
        out[..., :c] = px
    return out


def decode_hdr(data: bytes) -> np.ndarray:
    """Radiance RGBE (.hdr) bytes -> (h, w, 4) float32 RGBA, rows top to bottom: flat and
    new-style run-length scanlines, "-Y h +X w" orientation; each channel m 2^(e - 136)
    (0 when e is 0) and alpha 1, as stbi_loadf returns them."""
    pos = 0
    lines = []
    while True:
        end = data.index(b"\n", pos)
        line = data[pos:end].decode("latin-1").strip()
        pos = end + 1
        if line == "":
            if lines:
                break
            continue
        lines.append(line)
        if len(lines) > 64:
            raise ValueError("RGBE header too long")
    if not lines[0].startswith("#?"):
        raise ValueError("not a Radiance RGBE file")
    if not any(l.startswith("FORMAT=32-bit_rle_rgbe") for l in lines):
        raise ValueError("unsupported RGBE format")
    end = data.index(b"\n", pos)
    res = data[pos:end].decode("latin-1").split()
    pos = end + 1
    if len(res) != 4 or res[0] != "-Y" or res[2] != "+X":
        raise ValueError("only -Y h +X w RGBE images are read")
    h, w = int(res[1]), int(res[3])
    buf = np.frombuffer(data, np.uint8)
    rgbe = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if w < 8 or w > 0x7FFF or not (buf[pos] == 2 and buf[pos + 1] == 2 and buf[pos + 2] < 128):
            rgbe[y] = buf[pos:pos + 4 * w].reshape(w, 4)   # flat scanline
            pos += 4 * w
            continue
        if (int(buf[pos + 2]) << 8 | int(buf[pos + 3])) != w:
            raise ValueError("RGBE scanline width mismatch")
        pos += 4
        for ch in range(4):
            x = 0
            while x < w:
                n = int(buf[pos])
                pos += 1
                if n > 128:
                    n -= 128
                    if x + n > w:
                        raise ValueError("RGBE run overflows its scanline")
                    rgbe[y, x:x + n, ch] = buf[pos]
                    pos += 1
                else:
                    if n == 0 or x + n > w:
                        raise ValueError("RGBE run overflows its scanline")
                    rgbe[y, x:x + n, ch] = buf[pos:pos + n]
                    pos += n
                x += n
    e = rgbe[..., 3].astype(np.int32)
    scale = np.where(e > 0, np.ldexp(np.float32(1.0), e - 136), np.float32(0.0)).astype(np.float32)
    out = np.ones((h, w, 4), np.float32)
    out[..., :3] = rgbe[..., :3].astype(np.float32) * scale[..., None]
    return out


def load_hdr(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        return decode_hdr(f.read())


def encode_hdr(rgbe: np.ndarray, rle: bool = False) -> bytes:
    """(h, w, 4) uint8 RGBE pixels -> a Radiance file, flat or with run-length scanlines (runs
    of equal bytes as 128 + n, others as literal runs)."""
    h, w = rgbe.shape[:2]
    a = np.ascontiguousarray(rgbe, np.uint8)
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (h, w))
    if not rle:
        return bytes(out) + a.tobytes()
    for y in range(h):
        out += bytes([2, 2, w >> 8, w & 0xFF])
        for ch in range(4):
            row = a[y, :, ch].tolist()
            x = 0
            while x < w:
                r = 1
                while x + r < w and r < 127 and row[x + r] == row[x]:
                    r += 1
                if r >= 3:
                    out += bytes([128 + r, row[x]])
                    x += r
                    continue
                s = x
                while x < w and x - s < 128 and not (x + 2 < w and row[x] == row[x + 1] == row[x + 2]):
                    x += 1
                out += bytes([x - s]) + bytes(row[s:x])
    return bytes(out)


# The reference's sky textures, in the order the engine loads them into the texture pool
# (NextEngine::OnRendererDeviceSet, src/Runtime/Engine.cpp:853-870): SkyIdx i is file i.
REFERENCE_SKIES = ("river_road_2.hdr", "canary_wharf_1k.hdr", "kloppenheim_01_puresky_1k.hdr",
                   "kloppenheim_07_1k.hdr", "std_env.hdr", "rainforest_trail_1k.hdr", "studio_small_03_1k.hdr",
                   "studio_small_09_1k.hdr", "sunset_fairway_1k.hdr", "umhlanga_sunrise_1k.hdr",
                   "shanghai_bund_1k.hdr")


def write_png(path: str, rgb: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(encode_png(rgb))


def write_pfm(path: str, img: np.ndarray) -> None:
    """(h, w, 3|4) float image -> colour PFM (little-endian, rows bottom to top; alpha dropped)."""
    a = np.asarray(img, np.float32)[..., :3]
    h, w = a.shape[:2]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(a[::-1]).astype("<f4").tobytes())


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        if f.readline().strip() != b"PF":
            raise ValueError("not a colour PFM file")
        w, h = (int(v) for v in f.readline().split())
        scale = float(f.readline())
        dt = "<f4" if scale < 0 else ">f4"
        a = np.frombuffer(f.read(w * h * 12), dt).reshape(h, w, 3)
    return a[::-1].astype(np.float32)
