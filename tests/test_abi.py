"""The C ABI: the library loads, exports every entry point the header
declares, and its host-only logic works without a GPU."""
import os
import re
import zlib

import numpy as np
import pytest

from conftest import ROOT, golden
import kagayaki_gb300 as kg
from kagayaki_gb300 import _lib, api
from oracle import orc


def header_functions():
    src = open(os.path.join(ROOT, "include", "kagayaki.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kgk_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    L = kg.lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.PROTOTYPES)


def test_version_and_status_strings():
    L = kg.lib()
    assert b"sm_103a" in L.kgk_version()
    assert L.kgk_status_string(0) == b"KGK_OK"
    assert L.kgk_status_string(8) == b"KGK_ERR_DEVICE_CHECK"


def test_invalid_arguments_are_rejected_before_any_device_work():
    import ctypes
    L = kg.lib()
    h = ctypes.c_void_p()
    assert L.kgk_scene_create(None, 0, None, 0, None, 0, None, ctypes.byref(h)) == 1
    assert "no triangles" in kg.last_error()
    assert L.kgk_build_bvh(None, None) == 1
    assert L.kgk_trace_closest(None, None, 0, None, None, None) == 1
    assert L.kgk_camera_setup(_lib.KgkVec(0, 0, 0, 0), 28.0, 0, 0, 0, 0, None) == 1


def test_camera_setup_matches_reference_host_math():
    g = golden("camera_ref.npz")
    for k in range(len(g["org"])):
        cam = api.camera_setup(g["org"][k], float(g["dist"][k]), g["rot"][k], 1080)
        assert np.array_equal(api.camera_array(cam), g["cams"][k])


def test_tonemap_matches_oracle():
    rng = np.random.default_rng(0)
    img = rng.uniform(-0.5, 3.0, (17, 23, 4)).astype(np.float32)
    ours = api.tonemap(img)
    ref = orc.tonemap(img.reshape(-1, 4)).reshape(17, 23, 4)
    assert np.array_equal(ours, ref)


def test_png_is_decodable(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.uniform(0, 1, (9, 13, 4)).astype(np.float32)
    p = str(tmp_path / "x.png")
    api.save_png(img, p)
    data = open(p, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    # walk chunks, check CRCs, inflate IDAT
    pos, idat = 8, b""
    while pos < len(data):
        n = int.from_bytes(data[pos:pos + 4], "big")
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = int.from_bytes(data[pos + 8 + n:pos + 12 + n], "big")
        assert zlib.crc32(typ + body) == crc
        if typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(9, 1 + 13 * 4)
    assert (rows[:, 0] == 0).all()
    assert np.array_equal(rows[:, 1:].reshape(9, 13, 4), api.tonemap(img))


def test_png_write_failure_is_reported():
    img = np.zeros((2, 2, 4), np.float32)
    with pytest.raises(kg.KgkError) as e:
        api.save_png(img, "/nonexistent-dir/x.png")
    assert e.value.status == 5
