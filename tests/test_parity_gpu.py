"""The device's compat estimator (the reference's own RayTrace, quirks
included) against the reference's render of the same scenes, on the GPU.

Scenes (kagayaki_gb300.scenes.parity_scene): Disney boxes in the Cornell box,
a textured Cornell box, and displaced Disney icospheres under an HDR sky
(environment NEE, IBL on misses, MIS between them).  Fixtures come from the
reference's own source compiled for the host (tests/golden/make_golden.py);
the oracle (oracle/orc.c) is pinned to them on the CPU (tests/test_oracle.py)
and stands in for the reference at sizes whose fixtures would be too large.

Per-sample agreement.  The device follows the reference's random stream, so
a sample takes the same path as the reference's until a discrete decision
(Russian roulette, lobe or light choice, a shadow ray's verdict, which
triangle a ray hits at an edge) comes out differently.  Such flips come from
rounding: the device's sinf / cosf / acosf / powf / logf differ from glibc's
by an ulp or two, and nvcc contracts multiply-adds that the reference's host
build rounds separately.  After a flip the pixel's seed chain is out of step
for the rest of the frames (render.cuh:29,42), so per-sample agreement is
measured per frame and per chain; image agreement is the per-pixel 3-sigma
test.
"""
import numpy as np
import pytest

from conftest import BAR_CLOSE, BAR_CLOSE_FRAME0, golden, sample_stats
from kagayaki_gb300 import ESTIMATOR_COMPAT, Scene, scenes
from kagayaki_gb300._lib import check, lib
from kagayaki_gb300.structs import SVGF_BUFFER, KgkCamera

pytestmark = pytest.mark.gpu

KINDS = ["disney", "textured", "env"]


def cam_from_array(a):
    return KgkCamera.from_buffer_copy(np.ascontiguousarray(a, np.float32).tobytes())


def scene_of(kind):
    tris, mats, c, tex, env = scenes.parity_scene(kind)
    s = Scene(tris, mats, textures=tex or None, env=env)
    s.build_bvh()
    return s, c


def render_frames(s, cam, W, H, frames):
    """frames one-sample compat frames in a chain: (frames, W*H, 3)."""
    out = []
    for f in range(frames):
        img, st = s.render(cam, W, H, spp=1, estimator=ESTIMATOR_COMPAT, frame_index=f)
        assert st["traversal_overflows"] == 0
        out.append(img.reshape(-1, 4)[:, :3].copy())
    return np.stack(out)


@pytest.mark.parametrize("kind", KINDS)
def test_compat_scene_samples_follow_the_reference(kind):
    g = golden("parity_scenes_ref.npz")
    ref = g[f"{kind}_frames"]
    s, _ = scene_of(kind)
    with s:
        ours = render_frames(s, cam_from_array(g[f"{kind}_camera"]), 48, 48, ref.shape[0])
    st = sample_stats(ours, ref)
    print(kind, st)
    assert st["close_frame0"] > BAR_CLOSE_FRAME0, st
    assert st["close"] > BAR_CLOSE, st
    assert st["chains_in_step"] > 0.9, st


@pytest.mark.parametrize("kind", KINDS)
def test_compat_scene_mean_within_3_sigma_of_reference(kind):
    g = golden("parity_scenes_ref.npz")
    n = int(g[f"{kind}_n32"])
    s, _ = scene_of(kind)
    with s:
        img, st = s.render(cam_from_array(g[f"{kind}_camera32"]), 32, 32, spp=n, estimator=ESTIMATOR_COMPAT)
    mean = img.reshape(-1, 4)[1:, :3]
    ref_mean, ref_var = g[f"{kind}_mean32"][1:], g[f"{kind}_var32"][1:]
    sigma = np.sqrt(2.0 * ref_var / n) + 1e-6
    frac = float((np.abs(mean - ref_mean) > 3 * sigma).mean())
    print(kind, "outside 3 sigma", frac)
    assert frac < 0.01, frac
    assert st["rays_closest"] > 0 and st["rays_shadow"] > 0


def record_fields_equal(ours, ref):
    """Field-wise comparison of SVGFBuffer records: returns the fraction of
    records whose integer fields are equal and whose float fields agree
    within 1e-6 relative."""
    ok = np.ones(len(ours), bool)
    for f in ("ObjectID", "MaterialID", "PosLastFrameI", "sampleNum", "willApplyATrousFilter",
              "willApplyTemporalAccumulation"):
        eq = ours[f] == ref[f]
        ok &= eq.reshape(len(ours), -1).all(1)
    for f in ("Albedo", "Emission", "Normal", "ColorHistory", "PosLastFrameF", "MomentOne", "MomentTwo",
              "Variance", "Depth"):
        a = ours[f].reshape(len(ours), -1).astype(np.float64)
        b = ref[f].reshape(len(ours), -1).astype(np.float64)
        ok &= (np.abs(a - b) <= 1e-6 * np.maximum(np.abs(b), 1.0)).all(1)
    return ok


@pytest.mark.parametrize("kind", KINDS)
def test_gbuffer_records_match_reference(kind):
    """render()'s SVGFBuffer fill (render.cuh:28, RayTrace.cuh:66-82): our
    G-buffer written as the reference's records (kgk_gbuffer_records)."""
    g = golden("parity_scenes_ref.npz")
    ref = np.frombuffer(g[f"{kind}_gbuf32"].tobytes(), SVGF_BUFFER)
    s, _ = scene_of(kind)
    with s:
        s.render(cam_from_array(g[f"{kind}_camera32"]), 32, 32, spp=1, estimator=ESTIMATOR_COMPAT,
                 write_gbuffer=True)
        ours = s.gbuffer_records(32, 32)
    ok = record_fields_equal(ours, ref)
    print(kind, "records equal", ok.mean())
    assert ok[1:].mean() > 0.99, ok.mean()
    hit = ref["ObjectID"] >= 0
    assert hit.any() and (kind != "env" or (~hit).any())


def test_gbuffer_records_match_reference_cornell():
    """The same on the Cornell box fixture of the SVGF test (40 x 24)."""
    g = golden("svgf_ref.npz")
    W, H = int(g["width"]), int(g["height"])
    ref = np.frombuffer(g["gbuf"].tobytes(), SVGF_BUFFER)
    tris, mats, c = scenes.cornell_box()
    from oracle import orc
    cam = cam_from_array(orc.camera_setup(c["origin"], c["dist"], c["rot"], H))
    with Scene(tris, mats) as s:
        s.build_bvh()
        s.render(cam, W, H, spp=1, estimator=ESTIMATOR_COMPAT, write_gbuffer=True)
        ours = s.gbuffer_records(W, H)
    ok = record_fields_equal(ours, ref)
    print("cornell records equal", ok.mean())
    assert ok.mean() > 0.99


def test_device_disney_brdf_matches_reference():
    """evaluate_Disney_BRDF / _pdf on the device (kgk_disney_eval) against the
    reference's own values (disney_ref.npz: eight materials, 256 direction
    pairs each)."""
    g = golden("disney_ref.npz")
    worst_b, worst_p = 0.0, 0.0
    for k in range(len(g["mats"])):
        m = np.ascontiguousarray(g["mats"][k])
        wo, wi, n = (np.ascontiguousarray(g[x][k], np.float32) for x in ("wo", "wi", "n"))
        b = np.empty_like(wo)
        p = np.empty(len(wo), np.float32)
        check(lib().kgk_disney_eval(m.ctypes.data, len(wo), wo.ctypes.data, wi.ctypes.data, n.ctypes.data,
                                    b.ctypes.data, p.ctypes.data))
        rb = g["brdf"][k].astype(np.float64)
        rp = g["pdf"][k].astype(np.float64)
        eb = np.abs(b - rb) / np.maximum(np.abs(rb), 1e-3)
        ep = np.abs(p - rp) / np.maximum(np.abs(rp), 1e-3)
        worst_b, worst_p = max(worst_b, float(eb.max())), max(worst_p, float(ep.max()))
    print("disney device vs reference: max rel brdf", worst_b, "pdf", worst_p)
    assert worst_b < 1e-4 and worst_p < 1e-4


def test_c1_image_within_3_sigma_of_reference():
    """Config C1 as written: the Cornell box at 256 x 256, 16 samples per
    pixel in one call, the reference's estimator.  Every pixel's mean is
    compared with the reference's 16-sample mean; sigma is the reference's
    per-sample standard deviation (256 samples) scaled to the difference of
    two 16-sample means."""
    g = golden("c1_image_ref.npz")
    tris, mats, _ = scenes.cornell_box()
    spp = int(g["spp"])
    with Scene(tris, mats) as s:
        s.build_bvh()
        img, st = s.render(cam_from_array(g["camera"]), 256, 256, spp=spp, estimator=ESTIMATOR_COMPAT)
    mean = img.reshape(-1, 4)[1:, :3]
    ref = g["mean16"][1:].astype(np.float32)
    sigma = g["std1"][1:].astype(np.float32) * np.sqrt(2.0 / spp) + 1e-4
    out = np.abs(mean - ref) > 3 * sigma
    px_out = float(out.any(-1).mean())
    same = float((np.abs(mean - ref) <= 1e-3 * np.maximum(ref, 1e-2)).all(-1).mean())
    print("C1 256x256x16: pixels outside 3 sigma", px_out, "pixels within 1e-3", same,
          "rays", st["rays_closest"] + st["rays_shadow"], "reference traversals", int(g["rays16"]))
    assert px_out < 0.005, px_out


def test_c1_samples_follow_the_reference():
    """Config C1's 16 chained frames at 256 x 256, sample by sample, against
    the reference's own samples of 2048 seeded pixels (c1_image_ref.npz)."""
    g = golden("c1_image_ref.npz")
    tris, mats, _ = scenes.cornell_box()
    with Scene(tris, mats) as s:
        s.build_bvh()
        ours = render_frames(s, cam_from_array(g["camera"]), 256, 256, 16)
    px = g["px_sample"]
    # sample_stats drops its first pixel column: prepend a dummy one
    a = np.concatenate([np.zeros((16, 1, 3), np.float32), ours[:, px]], 1)
    b = np.concatenate([np.zeros((16, 1, 3), np.float32), g["samples16"]], 1)
    st = sample_stats(a, b)
    print("C1 per sample", st)
    assert st["close_frame0"] > BAR_CLOSE_FRAME0, st
    assert st["close"] > BAR_CLOSE, st
    assert st["chains_in_step"] > 0.85, st
