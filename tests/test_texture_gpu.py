"""Textures: RGBA8 storage and bilinear filtering.

A textured Lambert quad faces the camera under a constant environment L = 1
(a flat surface never sees itself), so the expected radiance of a pixel is
the texture's albedo at the pixel's uv.
  * RGBA8 texels decode to (v/255)^2.2 + 1e-4, the float the reference's
    loader gives the same byte: with nearest filtering an RGBA8 texture and
    the float texture of those values render bit-identical frames;
  * bilinear filtering reproduces a linear colour ramp exactly (up to the
    Monte Carlo noise of the estimator, 3 sigma of the FP64 accumulator).
"""
import numpy as np
import pytest

from kagayaki_gb300 import ESTIMATOR_UNBIASED, Scene, camera_setup, scenes, structs

pytestmark = pytest.mark.gpu


def quad_scene(tex_id=0):
    """Square [-1,1]^2 at z = 0 facing +z, uv (0,0) at (-1,-1) to (1,1) at (1,1)."""
    tris = np.zeros(2, structs.TRIANGLE)
    P = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    for t, (a, b, c) in enumerate([(0, 1, 2), (0, 2, 3)]):
        for k, i in enumerate((a, b, c)):
            tris["verts"][t, k, :3] = P[i]
            tris["verts"][t, 3 + k, :3] = (0, 0, 1)
            tris["verts"][t, 6 + k, :2] = UV[i]
    mat = structs.make_material(structs.LAMBERT, (0.5, 0.5, 0.5), tex=tex_id)
    return scenes.canonical(tris), np.stack([mat])


def decode(v):
    return ((np.float32(v) / np.float32(255.0)) ** np.float32(2.2)).astype(np.float64) + 1e-4


def test_rgba8_nearest_equals_float_texture():
    rng = np.random.default_rng(3)
    t8 = rng.integers(0, 256, (16, 16, 4), np.uint8)
    tris, mats = quad_scene()
    env = np.ones((16, 32, 3), np.float32)
    cam = camera_setup((0.0, 0.0, 3.0), 28.0, (0.0, 0.0, 0.0), 32)
    # the float texture the reference's loader would produce for these bytes
    lut = np.array([np.float32(np.float64(np.float32(np.float32(v) / np.float32(255.0)) ** np.float32(2.2)) + 1e-4)
                    for v in range(256)], np.float32)
    placeholder = [np.zeros((1, 1, 3), np.float32)]  # replaced below
    with Scene(tris, mats, textures=placeholder, env=env) as s:
        s.build_bvh()
        s.set_textures_rgba8([t8])
        a, _ = s.render(cam, 32, 32, spp=8, estimator=ESTIMATOR_UNBIASED, seed=5, max_depth=3)
        a = a.copy()
    tf = lut[t8[..., :3]].astype(np.float32)
    with Scene(tris, mats, textures=[tf], env=env) as s:
        s.build_bvh()
        b, _ = s.render(cam, 32, 32, spp=8, estimator=ESTIMATOR_UNBIASED, seed=5, max_depth=3)
    # identical up to the last bit of the decode table (host powf vs numpy pow)
    np.testing.assert_allclose(a, b, rtol=2e-6, atol=0)


def test_bilinear_reproduces_a_linear_ramp():
    W = H = 32
    tw, th = 8, 8
    # texel centres at u = (i + 0.5) / tw: albedo linear in u (red) and v (green)
    u = (np.arange(tw) + 0.5) / tw
    v = 1.0 - (np.arange(th) + 0.5) / th  # row 0 is the top (v = 1)
    tex = np.zeros((th, tw, 3), np.float32)
    tex[..., 0] = 0.2 + 0.6 * u[None, :]
    tex[..., 1] = 0.1 + 0.7 * v[:, None]
    tex[..., 2] = 0.5
    tris, mats = quad_scene()
    env = np.ones((16, 32, 3), np.float32)
    cam = camera_setup((0.0, 0.0, 3.0), 28.0, (0.0, 0.0, 0.0), H)
    with Scene(tris, mats, textures=[tex], env=env) as s:
        s.build_bvh()
        s.accum_reset(W, H)
        for k in range(8):
            s.render(cam, W, H, spp=256, estimator=ESTIMATOR_UNBIASED, seed=9, frame_index=k, accumulate=True,
                     max_depth=3, texture_filter=1)
        mean, var, n = s.accum_read(W, H)
    from kagayaki_gb300 import camera_array
    c = camera_array(cam).astype(np.float64)
    checked = 0
    for y in range(10, 23, 3):
        for x in range(10, 23, 3):
            d = c[4:7] * c[8] + c[9:12] * ((x - W / 2) * c[17]) + c[13:16] * ((H / 2 - y) * c[17])
            d /= np.linalg.norm(d)
            t = -c[2] / d[2]
            p = c[0:3] + t * d
            uu, vv = (p[0] + 1) / 2, (p[1] + 1) / 2
            if not (0.5 / tw < uu < 1 - 0.5 / tw and 0.5 / th < vv < 1 - 0.5 / th):
                continue  # the ramp wraps around outside the texel-centre range
            exp = np.array([0.2 + 0.6 * uu, 0.1 + 0.7 * vv, 0.5])
            got, sig = mean[y, x], np.sqrt(var[y, x])
            assert np.all(np.abs(got - exp) <= 3 * sig + 2e-3), (x, y, got, exp, sig)
            checked += 1
    assert checked >= 9


def test_scene_load_obj_renders_like_the_host_arrays(tmp_path):
    """kgk_scene_load_obj (OBJ/MTL/PNG straight to the device) equals
    kgk_load_obj + kgk_scene_create of the same files, frame for frame."""
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import scene_files
    from kagayaki_gb300 import ESTIMATOR_COMPAT, load_obj
    path = scene_files.write_obj_scene(str(tmp_path))
    scene_files.write_images(str(tmp_path))
    hdr = str(tmp_path / "rle.hdr")
    cam = camera_setup((0.5, 1.5, 14.0), 28.0, (0.0, 0.0, 0.0), 24)
    with Scene.from_obj(path, hdr) as s:
        s.build_bvh()
        a, _ = s.render(cam, 24, 24, spp=4, estimator=ESTIMATOR_COMPAT, max_depth=4)
        a = a.copy()
    tris, mats, texs, env = load_obj(path, hdr)
    with Scene(tris, mats, textures=texs, env=env) as s:
        s.build_bvh()
        b, _ = s.render(cam, 24, 24, spp=4, estimator=ESTIMATOR_COMPAT, max_depth=4)
    assert np.array_equal(a, b)
    assert a[..., :3].max() > 0
