"""Checkpoints of the learned denoiser: parameters and Adam's state, so training resumes where
it stopped. The reference has no checkpoints; its nearest relative is the cooked CPU-BVH cache
keyed by a hash of its input (CPUAccelerationStructure.cpp:207-222).

File layout (little-endian): magic b"GKRTUNET", u32 version (1), u32 parameter count n, u64 Adam
step, 32-byte SHA-256 of the payload, then the payload: n float32 parameters, n float32 first
moments, n float32 second moments. Loading checks magic, version, count, size and hash."""
import hashlib
import struct

import numpy as np

MAGIC = b"GKRTUNET"
VERSION = 1
_HEAD = struct.Struct("<8sIIQ32s")


class CheckpointError(ValueError):
    pass


def encode(params: np.ndarray, m: np.ndarray, v: np.ndarray, step: int) -> bytes:
    p, m, v = (np.ascontiguousarray(a, "<f4").reshape(-1) for a in (params, m, v))
    if not (p.size == m.size == v.size):
        raise ValueError("parameters and moments differ in size")
    payload = p.tobytes() + m.tobytes() + v.tobytes()
    return _HEAD.pack(MAGIC, VERSION, p.size, int(step), hashlib.sha256(payload).digest()) + payload


def decode(data: bytes, expect_count: int | None = None):
    """-> (params, m, v, step); raises CheckpointError on any mismatch."""
    if len(data) < _HEAD.size:
        raise CheckpointError("file shorter than the header")
    magic, version, n, step, digest = _HEAD.unpack_from(data)
    if magic != MAGIC:
        raise CheckpointError("not a denoiser checkpoint")
    if version != VERSION:
        raise CheckpointError(f"checkpoint version {version}, expected {VERSION}")
    if expect_count is not None and n != expect_count:
        raise CheckpointError(f"checkpoint holds {n} parameters, the network has {expect_count}")
    payload = data[_HEAD.size:]
    if len(payload) != 12 * n:
        raise CheckpointError("payload size does not match the parameter count")
    if hashlib.sha256(payload).digest() != digest:
        raise CheckpointError("payload hash mismatch (corrupted file)")
    a = np.frombuffer(payload, "<f4").astype(np.float32)
    return a[:n].copy(), a[n:2 * n].copy(), a[2 * n:].copy(), step


def save(path: str, params, m, v, step: int) -> None:
    with open(path, "wb") as f:
        f.write(encode(params, m, v, step))


def load(path: str, expect_count: int | None = None):
    with open(path, "rb") as f:
        return decode(f.read(), expect_count)
