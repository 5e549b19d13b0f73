"""Generates the committed fixtures under tests/golden/ (run from the repo root).

* rng_kat.json — PCG4D known answers (assets/shaders/common/Const_Func.slang:227-258)
  computed by the pure-Python restatement below, independent of the C++ oracle.
* cornell_32.npz — a 32 x 32 oracle render of the Cornell workload (regression pin of the
  oracle's shading path; the reference publishes no images or vectors for this path).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

M = 0xFFFFFFFF


def pcg4d_py(v):
    v = [(x * 1664525 + 1013904223) & M for x in v]
    v[0] = (v[0] + v[1] * v[3]) & M
    v[1] = (v[1] + v[2] * v[0]) & M
    v[2] = (v[2] + v[0] * v[1]) & M
    v[3] = (v[3] + v[1] * v[2]) & M
    v = [x ^ (x >> 16) for x in v]
    v[0] = (v[0] + v[1] * v[3]) & M
    v[1] = (v[1] + v[2] * v[0]) & M
    v[2] = (v[2] + v[0] * v[1]) & M
    v[3] = (v[3] + v[1] * v[2]) & M
    return v


def u2f_py(x):
    f = struct.unpack("<f", struct.pack("<I", 0x3F800000 | (x >> 9)))[0]
    return float(np.float32(np.float32(f) - np.float32(1.0)))


def rng_kat():
    seeds = [[0, 0, 0, 0], [1, 2, 3, 0], [255, 17, 9, 0], [1919, 1079, 119, 0]]
    out = []
    for s in seeds:
        v = list(s)
        seq = []
        for _ in range(8):
            v = pcg4d_py(v)
            seq.append({"state": list(v), "float": u2f_py(v[0])})
        out.append({"seed": s, "sequence": seq})
    return out


def main():
    with open(os.path.join(HERE, "rng_kat.json"), "w") as f:
        json.dump(rng_kat(), f, indent=1)
    from gknextengine_gb300 import abi, camera, scenes
    from oracle import oracle as O
    sc, cam, st = scenes.cornell()
    W = H = 32
    fb = camera.FrameBuilder(W, H, st)
    fc = fb.build(cam, 0)
    im = O.new_images(W, H)
    osc = O.OracleScene(sc)
    rays = osc.trace_pass(fc, W, H, im)
    np.savez_compressed(os.path.join(HERE, "cornell_32.npz"),
                        diffuse=im[abi.IMG_SINGLE_DIFFUSE], specular=im[abi.IMG_SINGLE_SPECULAR],
                        albedo=im[abi.IMG_ALBEDO], normal=im[abi.IMG_NORMAL],
                        object_id=im[abi.IMG_OBJECT_ID], hit_inst=im[abi.IMG_HIT_INST],
                        hit_prim=im[abi.IMG_HIT_PRIM], rays=np.array([rays], np.uint64))
    print("wrote golden fixtures; rays", rays)


if __name__ == "__main__":
    main()
