"""save_png (FileIO/IO_save_png.cuh:34-56) against the reference's own code:
the library's tone mapping (kgk_tonemap_rgba8: powf(x, 1/2.2f), clamp to
[0, 1], x255 truncated, alpha 255) and the oracle's restatement give the bytes
the reference's save_png writes, for every step of the byte function +-8 ulp,
special values (zeros, denormals, infinities, negatives, NaN) and seeded random
values (tests/golden/tonemap_ref.npz, made by running save_png and reading its
PNG back).  No GPU: the host function; the device one is checked against the
same fixture in tests/test_output_gpu.py."""
import numpy as np

from conftest import golden
from kagayaki_gb300 import tonemap
from oracle import orc


def _image(vals):
    img = np.zeros((1, len(vals), 4), np.float32)
    img[0, :, :3] = vals
    return img


def test_host_tonemap_equals_reference_save_png():
    g = golden("tonemap_ref.npz")
    ours = tonemap(_image(g["inputs"]))[0]
    assert np.array_equal(ours, g["rgba"])
    # every byte value occurs, and the special values are in the set
    assert len(np.unique(g["rgba"][:, :3])) == 256
    v = g["inputs"]
    assert np.isnan(v).any() and np.isinf(v).any() and (v < 0).any()


def test_oracle_tonemap_equals_reference_save_png():
    g = golden("tonemap_ref.npz")
    assert np.array_equal(orc.tonemap(_image(g["inputs"])[0]), g["rgba"])
