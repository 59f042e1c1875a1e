"""SVGF on the GPU: the drop-in ApplySVGF (kgk_svgf_apply) against the
reference's own filter (golden, race-free reading) and the standard filter's
error reduction on rendered frames."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from kagayaki_gb300 import ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED, Scene, camera_setup, scenes
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


def test_svgf_apply_follows_the_reference_over_an_orbit():
    """Config C3's comparison, frame by frame: kgk_svgf_apply (ApplySVGF,
    SVGF.cuh:495-522) over a 16-frame camera orbit of the Cornell box at
    256 x 256 against the oracle's race-free restatement of the reference's
    filter (orc.svgf_compat, bit-exact with the reference's own code on the
    golden frames, tests/test_oracle.py).  Both take the same inputs each
    frame - the compat frame and render()'s SVGFBuffer records
    (kgk_gbuffer_records) - and carry their own state from frame to frame
    as main.cu does (prev = this frame's records after filtering)."""
    from oracle import orc
    tris, mats, c = scenes.cornell_box()
    W = H = 256
    npx = W * H
    prev_g = np.zeros(npx * 112, np.uint8)
    prev_o = np.zeros(npx * 112, np.uint8)
    worst = 1.0
    with Scene(tris, mats) as s:
        s.build_bvh()
        for f in range(16):
            # 0.25 degrees of yaw and 0.1 units of sideways motion per frame
            org = (c["origin"][0] + 0.1 * f, c["origin"][1], c["origin"][2])
            cam = camera_setup(org, c["dist"], (c["rot"][0], c["rot"][1] + 0.25 * f, c["rot"][2]), H)
            noisy, _ = s.render(cam, W, H, spp=1, estimator=ESTIMATOR_COMPAT, frame_index=f, write_gbuffer=True)
            recs = s.gbuffer_records(W, H).view(np.uint8)
            res = np.ascontiguousarray(noisy.reshape(-1, 4))
            res[:, 3] = 0.0
            r_g, f_g, cur_g = res.copy(), np.zeros_like(res), recs.copy()
            r_o, f_o, cur_o = res.copy(), np.zeros_like(res), recs.copy()
            _run_apply(r_g, f_g, prev_g, cur_g, W, H, f)
            orc.svgf_compat(W, H, r_o, f_o, prev_o, cur_o, f)
            ok = _close(f_g[1:, :3], f_o[1:, :3])
            worst = min(worst, float(ok.mean()))
            assert ok.mean() > 0.995, (f, ok.mean())
            prev_g, prev_o = cur_g, cur_o
    print("SVGF orbit 256x256 x 16 frames: worst frame within 1e-4 of the race-free reference", worst)


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


@pytest.mark.parametrize("W,H,mode", [(72, 56, 1), (70, 53, 1), (70, 53, 2)])
def test_svgf_standard_matches_restatement(W, H, mode):
    """kgk_svgf (standard) pixel by pixel against its numpy restatement
    (tests/svgf_standard_ref.py) over six frames of a still camera: frame 0
    runs the 7 x 7 spatial variance everywhere, frames 4 and 5 the temporal
    moments; tile edges fall inside the image (W not a multiple of 32, H of
    8 in the second case).  The frames come from the compat estimator, whose
    primary rays pass through the pixel centres (the unbiased one jitters
    them), so the G-buffer is the same every frame and each pixel reprojects
    onto itself, as the restatement assumes.  The device's weights use ex2 / lg2
    approximations (~2^-22 relative, x sigma_n = 128 in the exponent), so a
    pixel agrees within 2e-3 relative; where the blurred variance is tiny the
    luminance weight's exponent |l - lq| / sigma_l sqrt(var) magnifies FP32
    rounding of l, so up to 2 % of pixels may leave that bound.  mode 2
    (KGK_SVGF_TEMPORAL) is the same reprojection and history with no spatial
    pass, and isolated outliers clamped before they enter the history."""
    from svgf_standard_ref import StandardSVGF
    tris, mats, c = scenes.cornell_box()
    ref = StandardSVGF(W, H, iterations=5 if mode == 1 else 0, firefly=mode == 2)
    cam = camera_setup(c["origin"], c["dist"], c["rot"], H)
    cfg = KgkSvgfConfig(mode=mode, width=W, height=H, frame_index=0, atrous_iterations=5, alpha=0.2,
                        sigma_z=1.0, sigma_n=128.0, sigma_l=4.0)
    worst = 1.0
    with Scene(tris, mats) as s:
        s.build_bvh()
        for f in range(6):
            noisy, _ = s.render(cam, W, H, spp=1, estimator=ESTIMATOR_COMPAT, frame_index=f, write_gbuffer=True)
            recs = s.gbuffer_records(W, H)
            cfg.frame_index = f
            out = np.empty_like(noisy)
            check(lib().kgk_svgf(s._h, ctypes.byref(cfg), _p(noisy), _p(out)))
            n = recs["Normal"][:, :3].reshape(H, W, 3)
            alb = recs["Albedo"][:, :3].reshape(H, W, 3)
            mat = np.where(recs["ObjectID"] >= 0, np.maximum(recs["MaterialID"], 0), -1).reshape(H, W)
            exp = ref.frame(noisy[..., :3], n, recs["Depth"].reshape(H, W), mat, alb)
            got = out[..., :3].astype(np.float64)
            rel = np.abs(got - exp) / np.maximum(np.abs(exp), 1e-3)
            ok = (rel <= 2e-3).all(-1)
            worst = min(worst, float(ok.mean()))
            assert np.isfinite(got).all()
            assert ok.mean() > 0.98, (f, ok.mean(), float(rel.max()))
    print(f"SVGF mode {mode} {W}x{H} x 6 frames vs restatement: worst frame within 2e-3", worst)
