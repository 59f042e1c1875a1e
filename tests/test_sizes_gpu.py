"""Image sizes the tiled paths treat at their edges, on the GPU: frames whose
sides are not multiples of the 8 x 4 slot tiles (scanline order then) or of
the SVGF tiles and row segments, down to the smallest each entry point
accepts.  Every frame must come back finite, with the rays counted and no
traversal overflow; the compat estimator's frames must equal the oracle's on
nearly every sample (the per-sample bar of the parity tests)."""
import ctypes

import numpy as np
import pytest

from conftest import BAR_CLOSE_FRAME0
from kagayaki_gb300 import ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED, Scene, camera_setup, scenes
from kagayaki_gb300._lib import check, lib
from kagayaki_gb300.structs import KgkSvgfConfig

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (7, 3), (33, 17), (64, 36), (130, 4)]


@pytest.mark.parametrize("W,H", SIZES)
def test_render_sizes(W, H):
    from oracle import orc
    tris, mats, c = scenes.cornell_box()
    with Scene(tris, mats) as s:
        s.build_bvh()
        cam = camera_setup(c["origin"], c["dist"], c["rot"], H)
        for est in (ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED):
            img, st = s.render(cam, W, H, spp=2, estimator=est, frame_index=0, max_depth=8)
            assert img.shape == (H, W, 4)
            assert np.isfinite(img[..., :3]).all(), (W, H, est)
            assert st["rays_closest"] > 0 and st["traversal_overflows"] == 0
        # one compat sample against the oracle's (pixel 0 is NaN there: the
        # reference's seed divides by zero)
        one, _ = s.render(cam, W, H, spp=1, estimator=ESTIMATOR_COMPAT, frame_index=0)
    if W * H > 1:
        ref, _ = orc.render_compat(tris, mats, orc.camera_setup(c["origin"], c["dist"], c["rot"], H), W, H, 1)
        a = one.reshape(-1, 4)[1:, :3].astype(np.float64)
        b = ref[0][1:].astype(np.float64)
        close = (np.abs(a - b) <= 1e-3 * np.maximum(np.abs(b), 1e-3)).all(-1)
        assert close.mean() >= min(BAR_CLOSE_FRAME0, 1.0 - 1.5 / len(close)), (W, H, close.mean())


@pytest.mark.parametrize("W,H", [(2, 2), (7, 3), (33, 17), (130, 4)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_svgf_sizes(W, H, mode):
    tris, mats, c = scenes.cornell_box()
    with Scene(tris, mats) as s:
        s.build_bvh()
        cfg = KgkSvgfConfig(mode=mode, width=W, height=H, frame_index=0, atrous_iterations=5, alpha=0.2,
                            sigma_z=1.0, sigma_n=128.0, sigma_l=4.0)
        for f in range(3):
            cam = camera_setup((c["origin"][0] + 0.05 * f, c["origin"][1], c["origin"][2]), c["dist"], c["rot"], H)
            noisy, _ = s.render(cam, W, H, spp=1, estimator=ESTIMATOR_UNBIASED, frame_index=f, write_gbuffer=True,
                                max_depth=8)
            cfg.frame_index = f
            out = np.empty_like(noisy)
            check(lib().kgk_svgf(s._h, ctypes.byref(cfg), ctypes.c_void_p(noisy.ctypes.data),
                                 ctypes.c_void_p(out.ctypes.data)))
            assert np.isfinite(out[..., :3]).all(), (W, H, mode, f)
