"""OpenEXR output (kgk_save_exr), read back by a reader written here from the
OpenEXR file layout (magic, version, attribute header, scanline offset
table, channel-planar scanlines).  The reference writes PNG only, so there is
no reference output to pin against; the bar is the file layout and the pixel
values: FP32 channels bit-exact, FP16 channels equal to numpy's
round-to-nearest-even conversion (NaN stays NaN).  Host-only."""
import struct

import numpy as np
import pytest

from kagayaki_gb300 import KgkError, save_exr


def read_exr(path):
    b = open(path, "rb").read()
    assert b[:4] == bytes([0x76, 0x2f, 0x31, 0x01])
    assert struct.unpack_from("<I", b, 4)[0] == 2  # version 2, single-part scanline
    pos, attrs = 8, {}
    while b[pos] != 0:
        e = b.index(b"\0", pos)
        name = b[pos:e].decode()
        pos = e + 1
        e = b.index(b"\0", pos)
        typ = b[pos:e].decode()
        pos = e + 1
        size = struct.unpack_from("<i", b, pos)[0]
        attrs[name] = (typ, b[pos + 4:pos + 4 + size])
        pos += 4 + size
    pos += 1
    chans, cpos, raw = [], 0, attrs["channels"][1]
    while raw[cpos] != 0:
        e = raw.index(b"\0", cpos)
        nm = raw[cpos:e].decode()
        ptype, _, xs, ys = struct.unpack_from("<iI ii".replace(" ", ""), raw, e + 1)
        chans.append((nm, ptype))
        assert (xs, ys) == (1, 1)
        cpos = e + 1 + 16
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    assert attrs["compression"] == ("compression", b"\0")
    offsets = struct.unpack_from(f"<{h}Q", b, pos)
    img = {nm: np.zeros((h, w), np.float32) for nm, _ in chans}
    for y, off in enumerate(offsets):
        yy, size = struct.unpack_from("<ii", b, off)
        assert yy == y
        p = off + 8
        for nm, ptype in chans:
            dt = np.dtype("<f2") if ptype == 1 else np.dtype("<f4")
            img[nm][y] = np.frombuffer(b, dt, w, p).astype(np.float32)
            p += w * dt.itemsize
        assert p == off + 8 + size
    return attrs, chans, img


def _image(h, w, seed=1):
    rng = np.random.default_rng(seed)
    img = np.zeros((h, w, 4), np.float32)
    img[..., :3] = rng.lognormal(0, 3, (h, w, 3)).astype(np.float32) * rng.choice([-1, 1], (h, w, 3))
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 65504.0, 65519.9, 65520.0, 1e-8, 2.0 ** -24,
                        2.0 ** -25, 3 * 2.0 ** -26, 6.1e-5, 1e30, -1e-30], np.float32)
    img.reshape(-1, 4)[:len(special), 0] = special
    img.reshape(-1, 4)[:len(special), 2] = special[::-1]
    return img


@pytest.mark.parametrize("half", [False, True])
def test_exr_layout_and_values(tmp_path, half):
    img = _image(13, 17)
    path = tmp_path / "out.exr"
    save_exr(img, path, half=half)
    attrs, chans, got = read_exr(path)
    assert [c[0] for c in chans] == ["B", "G", "R"]
    assert {c[1] for c in chans} == {1 if half else 2}
    for k in ["displayWindow", "lineOrder", "pixelAspectRatio", "screenWindowCenter", "screenWindowWidth"]:
        assert k in attrs
    for nm, c in (("R", 0), ("G", 1), ("B", 2)):
        want = img[..., c]
        if half:
            want = want.astype(np.float16).astype(np.float32)
        nan = np.isnan(want)
        assert np.array_equal(np.isnan(got[nm]), nan), nm
        assert np.array_equal(got[nm][~nan].view(np.uint32), want[~nan].view(np.uint32)), nm


def test_exr_half_rounding_exhaustive_neighbourhoods(tmp_path):
    # every FP16 boundary region: floats around each half value's midpoints
    halves = np.arange(0, 0x7c00, 7, dtype=np.uint16).view(np.float16).astype(np.float32)
    mids = (halves[:-1].astype(np.float64) + halves[1:].astype(np.float64)) / 2
    vals = np.concatenate([halves, np.nextafter(mids.astype(np.float32), 0), mids.astype(np.float32),
                           np.nextafter(mids.astype(np.float32), np.inf)])
    vals = np.concatenate([vals, -vals])
    n = (len(vals) + 2) // 3 * 3
    vals = np.resize(vals, n)
    img = np.zeros((1, n // 3, 4), np.float32)
    img[0, :, :3] = vals.reshape(-1, 3)
    path = tmp_path / "h.exr"
    save_exr(img, path, half=True)
    _, _, got = read_exr(path)
    for nm, c in (("R", 0), ("G", 1), ("B", 2)):
        want = img[0, :, c].astype(np.float16).astype(np.float32)
        assert np.array_equal(got[nm][0].view(np.uint32), want.view(np.uint32)), nm


def test_exr_errors(tmp_path):
    with pytest.raises(KgkError, match="cannot open"):
        save_exr(np.ones((2, 2, 4), np.float32), tmp_path / "missing_dir" / "x.exr")
    with pytest.raises(KgkError, match="empty"):
        save_exr(np.zeros((0, 3, 4), np.float32), tmp_path / "e.exr")
