"""Image files for the output stage: PNG for screenshots (8-bit RGB, as ScreenShot.cpp's crop;
the reference encodes JPEG or AVIF through third-party encoders, ScreenShot.cpp:18-205) and PFM
(portable float map) for linear HDR dumps. Standard library and numpy only."""
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


def decode_png(data: bytes) -> np.ndarray:
    """PNG bytes written by encode_png (8-bit, filter 0 rows) -> (h, w, c) uint8."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if depth != 8 or ctype not in (2, 6):
                raise ValueError("only 8-bit RGB / RGBA")
            c = 3 if ctype == 2 else 4
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    rows = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * c)
    if (rows[:, 0] != 0).any():
        raise ValueError("filtered rows are not supported")
    return rows[:, 1:].reshape(h, w, c).copy()


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
