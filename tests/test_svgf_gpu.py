"""SVGF on the GPU: the drop-in ApplySVGF (kgk_svgf_apply) against the
reference's own filter (golden, race-free reading) and the standard filter's
error reduction on rendered frames."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from kagayaki_gb300 import ESTIMATOR_UNBIASED, Scene, camera_setup, scenes
from kagayaki_gb300._lib import check, lib
from kagayaki_gb300.structs import KgkSvgfConfig

pytestmark = pytest.mark.gpu

# FP32 with the device's expf and contracted multiply-adds against the host
# build: per-pixel relative error bound, and the fraction of pixels that may
# leave it (a flipped threshold in the 0.2-blend chain).
SVGF_RTOL = 1e-4


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _run_apply(res, filt, prev, cur, W, H, frame):
    check(lib().kgk_svgf_apply(_p(res), _p(filt), _p(prev), _p(cur), W, H, frame))


def _close(a, b):
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-3)
    return (rel <= SVGF_RTOL).all(-1)


def test_svgf_apply_matches_reference_two_frames():
    g = golden("svgf_ref.npz")
    W, H = int(g["width"]), int(g["height"])
    npx = W * H
    prev = np.zeros(npx * 112, np.uint8)
    cur = g["gbuf"].copy()
    r0, f0 = g["res0"].copy(), np.zeros_like(g["res0"])
    _run_apply(r0, f0, prev, cur, W, H, 0)
    ok0 = _close(f0[:, :3], g["out_filtered0"][:, :3])
    assert ok0.mean() > 0.995, ok0.mean()
    assert _close(r0[:, :3], g["out_result0"][:, :3]).mean() > 0.995
    prev1, cur1 = cur.copy(), g["gbuf"].copy()
    r1, f1 = g["res1"].copy(), np.zeros_like(g["res1"])
    _run_apply(r1, f1, prev1, cur1, W, H, 1)
    ok1 = _close(f1[:, :3], g["out_filtered1"][:, :3])
    assert ok1.mean() > 0.995, ok1.mean()
    # integer state (object / material ids, flags) identical
    rec = np.dtype([("f", "<f4", (16,)), ("ids", "<i4", (2,)), ("pi", "<i4", (2,)), ("pf", "<f4", (2,)),
                    ("n", "<i4"), ("m", "<f4", (4,)), ("fl", "u1", (2,)), ("pad", "u1", (2,))])
    a, b = cur1.view(rec), g["out_cur1"].view(rec)
    assert np.array_equal(a["ids"], b["ids"])
    assert (a["fl"] == b["fl"]).mean() > 0.995


def test_svgf_apply_rejects_bad_sizes():
    r = np.zeros((4, 4), np.float32)
    b = np.zeros(4 * 112, np.uint8)
    assert lib().kgk_svgf_apply(_p(r), _p(r), _p(b), _p(b), 1, 4, 0) == 1


def test_svgf_standard_reduces_error_over_an_orbit():
    tris, mats, c = scenes.cornell_box()
    W = H = 64
    with Scene(tris, mats) as s:
        s.build_bvh()
        cfg = KgkSvgfConfig(mode=1, width=W, height=H, frame_index=0, atrous_iterations=5, alpha=0.2,
                            sigma_z=1.0, sigma_n=128.0, sigma_l=4.0)
        errs_noisy, errs_filt = [], []
        for f in range(8):
            org = (c["origin"][0] + 0.02 * f, c["origin"][1], c["origin"][2])
            cam = camera_setup(org, c["dist"], c["rot"], H)
            ref, _ = s.render(cam, W, H, spp=1024, estimator=ESTIMATOR_UNBIASED, seed=99, frame_index=1000 + f,
                              max_depth=8)
            noisy, _ = s.render(cam, W, H, spp=1, estimator=ESTIMATOR_UNBIASED, seed=5, frame_index=f,
                                write_gbuffer=True, max_depth=8)
            cfg.frame_index = f
            out = np.empty_like(noisy)
            check(lib().kgk_svgf(s._h, ctypes.byref(cfg), _p(noisy), _p(out)))
            rr = ref[..., :3]
            def relmse(x):
                return float(np.mean((x[..., :3] - rr) ** 2 / (rr ** 2 + 1e-2)))
            errs_noisy.append(relmse(noisy))
            errs_filt.append(relmse(out))
    assert all(np.isfinite(errs_filt))
    # every filtered frame at most half the relative MSE of its 1-spp input,
    # and the history never makes a later frame worse than the first
    assert all(f < 0.5 * n for f, n in zip(errs_filt, errs_noisy)), (errs_noisy, errs_filt)
    assert max(errs_filt[2:]) <= 1.5 * errs_filt[0], errs_filt
