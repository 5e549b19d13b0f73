"""Denoiser checkpoint files: exact round trip, and every corruption refused."""
import numpy as np
import pytest

from gknextengine_gb300 import checkpoint as ck


def sample(n=1000, seed=0):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=n).astype(np.float32), rng.normal(size=n).astype(np.float32) * 1e-3,
            np.abs(rng.normal(size=n)).astype(np.float32) * 1e-6, 1234)


def test_round_trip_is_exact(tmp_path):
    p, m, v, step = sample()
    path = str(tmp_path / "net.ckpt")
    ck.save(path, p, m, v, step)
    p2, m2, v2, s2 = ck.load(path, p.size)
    assert s2 == step
    for a, b in ((p, p2), (m, m2), (v, v2)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("what", ["magic", "version", "count", "truncated", "payload"])
def test_corruptions_are_refused(what):
    p, m, v, step = sample(64)
    data = bytearray(ck.encode(p, m, v, step))
    if what == "magic":
        data[0:8] = b"NOTACKPT"
    elif what == "version":
        data[8] = 9
    elif what == "count":
        pass
    elif what == "truncated":
        data = data[:-4]
    else:
        data[-1] ^= 0x01
    with pytest.raises(ck.CheckpointError):
        ck.decode(bytes(data), expect_count=65 if what == "count" else 64)


def test_sizes_must_agree():
    p, m, v, step = sample(16)
    with pytest.raises(ValueError):
        ck.encode(p, m[:8], v, step)
