"""The learned radiance cache inside the wavefront renderer
(kgk_render with use_cache=1, unbiased estimator).

The cache has no counterpart in the reference.  What is checked:
  * argument rules (needs kgk_nrc_init, needs the unbiased estimator);
  * bias: in a closed white-furnace box (albedo 0.5, emission 1) radiance is
    2 everywhere; after online training the cached frames stay within 3 %;
  * gain: on the Cornell box at equal samples per pixel, frames that end
    their paths in the trained cache are closer (relative MSE) to a converged
    plain render than plain frames are, and take less device time.
"""
import numpy as np
import pytest

from kagayaki_gb300 import ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED, KgkError, Scene, camera_setup, scenes

from test_render_gpu import closed_box

pytestmark = pytest.mark.gpu


def rel_mse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_cache_needs_init_and_unbiased_estimator():
    tris, mats, c = scenes.cornell_box()
    with Scene(tris, mats) as s:
        s.build_bvh()
        cam = camera_setup(c["origin"], c["dist"], c["rot"], 16)
        with pytest.raises(KgkError):
            s.render(cam, 16, 16, estimator=ESTIMATOR_UNBIASED, use_cache=True)
        s.cache_init()
        with pytest.raises(KgkError):
            s.render(cam, 16, 16, estimator=ESTIMATOR_COMPAT, use_cache=True)
        img, st = s.render(cam, 16, 16, estimator=ESTIMATOR_UNBIASED, use_cache=True)
        assert np.isfinite(img).all()


def test_cache_white_furnace_bias():
    tris, mats = closed_box(0.5, 1.0)
    W = H = 64
    with Scene(tris, mats) as s:
        s.build_bvh()
        s.cache_init(train_paths=1024, seed=5)
        cam = camera_setup((0.1, 0.05, 0.2), 28.0, (0.0, 0.0, 0.0), H)
        for f in range(40):
            s.render(cam, W, H, spp=1, estimator=ESTIMATOR_UNBIASED, rr_start_depth=2, seed=11,
                     frame_index=f, use_cache=True)
        means = []
        for f in range(40, 48):
            img, _ = s.render(cam, W, H, spp=4, estimator=ESTIMATOR_UNBIASED, rr_start_depth=2, seed=11,
                              frame_index=f, use_cache=True)
            means.append(img[..., :3].mean())
    m = float(np.mean(means))
    assert abs(m - 2.0) < 0.06, m


def test_cache_beats_plain_at_equal_spp_on_cornell():
    tris, mats, c = scenes.cornell_box()
    W = H = 128
    cam = camera_setup(c["origin"], c["dist"], c["rot"], H)
    with Scene(tris, mats) as s:
        s.build_bvh()
        ref, _ = s.render(cam, W, H, spp=4096, estimator=ESTIMATOR_UNBIASED, seed=99, max_depth=32)
        ref = ref[..., :3].astype(np.float64)
        s.cache_init(train_paths=2048, seed=3)
        for f in range(60):
            s.render(cam, W, H, spp=1, estimator=ESTIMATOR_UNBIASED, seed=5, frame_index=f,
                     use_cache=True, max_depth=32)
        e_cache, e_plain, t_cache, t_plain = [], [], 0.0, 0.0
        for f in range(60, 68):
            a, sa = s.render(cam, W, H, spp=4, estimator=ESTIMATOR_UNBIASED, seed=5, frame_index=f,
                             use_cache=True, max_depth=32)
            b, sb = s.render(cam, W, H, spp=4, estimator=ESTIMATOR_UNBIASED, seed=5, frame_index=f,
                             max_depth=32)
            e_cache.append(rel_mse(a[..., :3], ref))
            e_plain.append(rel_mse(b[..., :3], ref))
            t_cache += sa["ms_device"]
            t_plain += sb["ms_device"]
            assert sa["rays_closest"] < sb["rays_closest"]
    ec, ep = float(np.mean(e_cache)), float(np.mean(e_plain))
    print(f"relMSE cache {ec:.5f} ({t_cache:.2f} ms) plain {ep:.5f} ({t_plain:.2f} ms)")
    assert ec < ep, (ec, ep)
