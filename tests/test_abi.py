"""CPU tests of the C ABI: the library loads, exports every declared symbol, its struct
layouts match the ctypes mirror, and host-only entry points work without a GPU."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from gknextengine_gb300 import abi, native, scenes

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "gkrt.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gkrt_\w+)\s*\(", src, re.M)))


def test_header_declarations_are_bound():
    assert set(declared_functions()) == set(native.EXPORTED)


def test_library_exports_every_declared_symbol(gkrt_lib):
    L = C.CDLL(gkrt_lib)
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_abi_version(gkrt_lib):
    assert native.load().gkrt_abi_version() == 2


def test_struct_layouts_match_c(tmp_path):
    """Compile a probe against gkrt.h with gcc and compare sizeof/offsetof to ctypes."""
    probe = tmp_path / "probe.c"
    fields = {
        "GkrtSceneDesc": [f for f, _ in abi.GkrtSceneDesc._fields_],
        "GkrtFrameConstants": [f for f, _ in abi.GkrtFrameConstants._fields_],
        "GkrtImageView": [f for f, _ in abi.GkrtImageView._fields_],
        "GkrtStats": [f for f, _ in abi.GkrtStats._fields_],
        "GkrtDeviceDesc": [f for f, _ in abi.GkrtDeviceDesc._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for s, fl in fields.items():
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f in fl:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    for s in ("GkrtMaterial", "GkrtLight", "GkrtMesh", "GkrtInstance", "GkrtRay", "GkrtHit"):
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
    lines.append("return 0;}")
    probe.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", str(probe), "-o", str(exe)])
    out = dict(l.rsplit(" ", 1) for l in subprocess.check_output([str(exe)], text=True).splitlines())
    for s in fields:
        ct = getattr(abi, s)
        assert int(out[s]) == C.sizeof(ct), s
        for f in fields[s]:
            assert int(out[f"{s}.{f}"]) == getattr(ct, f).offset, f"{s}.{f}"
    assert int(out["GkrtMaterial"]) == abi.MATERIAL_DTYPE.itemsize
    assert int(out["GkrtLight"]) == abi.LIGHT_DTYPE.itemsize
    assert int(out["GkrtMesh"]) == abi.MESH_DTYPE.itemsize
    assert int(out["GkrtInstance"]) == abi.INSTANCE_DTYPE.itemsize
    assert int(out["GkrtRay"]) == abi.RAY_DTYPE.itemsize
    assert int(out["GkrtHit"]) == abi.HIT_DTYPE.itemsize


def test_affine_inverse_host_only(gkrt_lib):
    L = native.load()
    w = scenes.trs((1.0, -2.0, 3.0), rot_y_deg=33.0, scale=(0.5, 2.0, 1.5)).astype(np.float32)
    out = np.zeros(12, np.float32)
    rc = L.gkrt_affine_inverse(w.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == abi.GKRT_OK
    np.testing.assert_allclose(out, scenes.affine_inverse(w), rtol=1e-5, atol=1e-6)
    sing = np.zeros(12, np.float32)
    assert L.gkrt_affine_inverse(sing.ctypes.data_as(C.POINTER(C.c_float)),
                                 out.ctypes.data_as(C.POINTER(C.c_float))) == abi.GKRT_ERR_INVALID_ARG


def test_null_arguments_are_rejected(gkrt_lib):
    L = native.load()
    assert L.gkrt_context_create(None, None) == abi.GKRT_ERR_INVALID_ARG
    assert L.gkrt_resize(None, 4, 4) == abi.GKRT_ERR_INVALID_ARG
    assert L.gkrt_scene_upload(None, None) == abi.GKRT_ERR_INVALID_ARG
    assert L.gkrt_context_destroy(None) == abi.GKRT_ERR_INVALID_ARG


def test_no_device_is_reported(gkrt_lib):
    """Without a GPU the context cannot be created and the call says so."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = native.load()
    h = C.c_void_p()
    rc = L.gkrt_context_create(None, C.byref(h))
    assert rc == abi.GKRT_ERR_NO_DEVICE and not h.value


def test_scene_sizes():
    sc, _, _ = scenes.cornell()
    assert sc.triangle_count == 36
    b, _, st = scenes.bricks()
    assert b.meshes[0]["index_count"] // 3 == 252
    assert 1_000_000 < b.triangle_count < 1_100_000
    w = b.instances["world"].reshape(-1, 3, 4)
    wi = b.instances["world_inv"].reshape(-1, 3, 4)
    m = np.einsum("nij,njk->nik", w[:, :, :3], wi[:, :, :3])
    assert np.allclose(m, np.eye(3), atol=1e-5)
