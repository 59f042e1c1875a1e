"""Frames from the wavefront tracer.

compat estimator: per-sample comparison with the reference's own render of
the Cornell box (golden frames: same xorshift stream, so most samples follow
the same path and agree to FP32 rounding; the bars are in tests/conftest.py)
and a 3-sigma test of the per-pixel mean against the reference's 256-sample
statistics.
unbiased estimator: analytic furnace scenes (closed emissive box,
constant-environment convex object)."""
import numpy as np
import pytest

from conftest import BAR_CLOSE, BAR_CLOSE_FRAME0, golden, sample_stats
from kagayaki_gb300 import ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED, Scene, scenes, structs
from kagayaki_gb300.structs import KgkCamera

pytestmark = pytest.mark.gpu


def cam_from_array(a):
    c = KgkCamera.from_buffer_copy(np.ascontiguousarray(a, np.float32).tobytes())
    return c


@pytest.fixture(scope="module")
def cornell():
    tris, mats, cam = scenes.cornell_box()
    s = Scene(tris, mats)
    s.build_bvh()
    yield s
    s.close()


def test_compat_samples_follow_the_reference(cornell):
    g = golden("c1_render_ref.npz")
    W, H = int(g["width"]), int(g["height"])
    cam = cam_from_array(g["camera"])
    ref = g["frames"]
    ours = []
    for f in range(ref.shape[0]):
        img, st = cornell.render(cam, W, H, spp=1, estimator=ESTIMATOR_COMPAT, frame_index=f)
        assert st["traversal_overflows"] == 0
        ours.append(img.reshape(-1, 4)[:, :3])
    # per sample within 1e-4 relative (the bars and what explains the rest:
    # tests/conftest.py)
    st = sample_stats(np.stack(ours), ref)
    print("Cornell 48x48 x 8 frames", st)
    assert st["close_frame0"] > BAR_CLOSE_FRAME0, st
    assert st["close"] > BAR_CLOSE, st
    assert st["chains_in_step"] > 0.9, st


def test_compat_mean_within_3_sigma_of_reference(cornell):
    g = golden("c1_render_ref.npz")
    n = int(g["n32"])
    cam = cam_from_array(g["camera32"])
    img, st = cornell.render(cam, 32, 32, spp=n, estimator=ESTIMATOR_COMPAT, frame_index=0)
    mean = img.reshape(-1, 4)[1:, :3]
    ref_mean, ref_var = g["mean32"][1:], g["var32"][1:]
    sigma = np.sqrt(2.0 * ref_var / n) + 1e-6
    frac = (np.abs(mean - ref_mean) > 3 * sigma).mean()
    assert frac < 0.01, frac
    assert st["rays_closest"] > 0 and st["rays_shadow"] > 0


def test_compat_chain_equals_multi_sample_call(cornell):
    """spp=4 in one call == four chained frames (the persistent seed chain)."""
    tris, mats, c = scenes.cornell_box()
    from kagayaki_gb300 import camera_setup
    cam = camera_setup(c["origin"], c["dist"], c["rot"], 24)
    one, _ = cornell.render(cam, 24, 24, spp=4, estimator=ESTIMATOR_COMPAT, frame_index=0)
    acc = np.zeros_like(one)
    for f in range(4):
        img, _ = cornell.render(cam, 24, 24, spp=1, estimator=ESTIMATOR_COMPAT, frame_index=f)
        acc += img
    np.testing.assert_allclose(one[..., :3], (acc / 4)[..., :3], rtol=1e-5, atol=1e-6)


def closed_box(albedo, emission):
    """A closed cube of emissive Lambert walls (inward normals)."""
    m = np.stack([structs.make_material(structs.LAMBERT, (albedo,) * 3, emission=(emission,) * 3)])
    q = scenes._quad
    x0, x1 = -1.0, 1.0
    parts = [q((x0, x0, x1), (x1, x0, x1), (x1, x0, x0), (x0, x0, x0), 0, 0),
             q((x0, x1, x0), (x1, x1, x0), (x1, x1, x1), (x0, x1, x1), 0, 1),
             q((x0, x0, x0), (x1, x0, x0), (x1, x1, x0), (x0, x1, x0), 0, 2),
             q((x0, x0, x1), (x0, x0, x0), (x0, x1, x0), (x0, x1, x1), 0, 3),
             q((x1, x0, x0), (x1, x0, x1), (x1, x1, x1), (x1, x1, x0), 0, 4),
             q((x0, x0, x1), (x0, x1, x1), (x1, x1, x1), (x1, x0, x1), 0, 5)]
    return scenes.canonical(np.concatenate(parts)), m


def test_unbiased_white_furnace():
    """Closed box, albedo 0.5, emission 1: radiance 1 / (1 - 0.5) = 2 everywhere."""
    from kagayaki_gb300 import camera_setup
    tris, mats = closed_box(0.5, 1.0)
    with Scene(tris, mats) as s:
        s.build_bvh()
        cam = camera_setup((0.1, 0.05, 0.2), 28.0, (0.0, 0.0, 0.0), 32)
        img, st = s.render(cam, 32, 32, spp=512, estimator=ESTIMATOR_UNBIASED, rr_start_depth=2, seed=7)
    m = img[..., :3].mean()
    assert abs(m - 2.0) < 0.02, m
    assert st["rays_shadow"] > 0


def test_unbiased_constant_environment_on_convex_object():
    """A convex diffuse object under a constant environment L=1 reflects
    albedo * 1 everywhere it is seen (no self-shadowing); background = 1."""
    from kagayaki_gb300 import camera_setup
    v, f = scenes.icosphere(3)
    nrm = v.astype(np.float32)
    uv = np.zeros((len(v), 2), np.float32)
    tris = scenes.canonical(scenes._tris_from_indexed(v.astype(np.float32), nrm, uv, f.astype(np.int64), 0, False, 0))
    mats = np.stack([structs.make_material(structs.LAMBERT, (0.6, 0.6, 0.6))])
    env = np.ones((64, 128, 3), np.float32)
    with Scene(tris, mats, env=env) as s:
        s.build_bvh()
        cam = camera_setup((0.0, 0.0, 4.0), 28.0, (0.0, 0.0, 0.0), 32)
        img, st = s.render(cam, 32, 32, spp=256, estimator=ESTIMATOR_UNBIASED, seed=3, max_depth=8)
    c = img[..., :3]
    center = c[12:20, 12:20].mean()
    corner = c[:3, :3].mean()
    assert abs(center - 0.6) < 0.01, center
    assert abs(corner - 1.0) < 1e-4, corner


def test_accumulator_fp64_matches_frames(cornell):
    from kagayaki_gb300 import camera_setup
    tris, mats, c = scenes.cornell_box()
    cam = camera_setup(c["origin"], c["dist"], c["rot"], 16)
    cornell.accum_reset(16, 16)
    acc = np.zeros((16, 16, 3))
    for f in range(3):
        img, _ = cornell.render(cam, 16, 16, spp=8, estimator=ESTIMATOR_UNBIASED, frame_index=f,
                                accumulate=True)
        acc += img[..., :3]
    mean, var, n = cornell.accum_read(16, 16)
    assert n == 24
    np.testing.assert_allclose(mean, acc / 3, rtol=1e-4, atol=1e-5)
    assert (var >= 0).all()


def test_unbiased_tail_matches_wavefront(cornell):
    """The unbiased estimator draws each path's random numbers from (seed,
    frame, sample, pixel), so a frame rendered as one wave (wavefront bounces,
    then the tail kernel) and as tail-only waves traces the same paths.  The
    tail defers its face-light and environment shadow rays to a parallel pass
    and adds the visible contributions in slot order, so the two frames agree
    up to the order of the radiance sums (rtol 1e-4)."""
    from kagayaki_gb300 import camera_setup
    tris, mats, c = scenes.cornell_box()
    W = H = 256
    cam = camera_setup(c["origin"], c["dist"], c["rot"], H)
    kw = dict(spp=4, estimator=ESTIMATOR_UNBIASED, seed=3, max_depth=8)
    a, sa = cornell.render(cam, W, H, **kw)                     # one wave of 262,144 paths
    b, sb = cornell.render(cam, W, H, wave_paths=65536, **kw)   # four waves of 65,536: tail only
    assert a[..., :3].mean() > 0.05
    np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=1e-4, atol=1e-6)
    # every shadow ray is counted once, traced inline or deferred
    assert sa["rays_shadow"] == sb["rays_shadow"] and sa["rays_closest"] == sb["rays_closest"]
