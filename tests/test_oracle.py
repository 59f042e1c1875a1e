"""The CPU oracle against the golden fixtures made by the reference's own
source (tests/golden/make_golden.py).  No GPU."""
import hashlib

import numpy as np
import pytest

from conftest import C1_HI, C1_LO, golden
from kagayaki_gb300 import scenes
from oracle import orc


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_scene_and_rays_are_the_golden_inputs():
    g = golden("c1_trace_ref.npz")
    tris, _, _ = scenes.cornell_box()
    rays = scenes.parity_rays(1 << 20, C1_LO, C1_HI, seed=1)
    assert digest(tris) == str(g["tri_digest"])
    assert digest(rays) == str(g["ray_digest"])


def test_c1_closest_hits_bit_exact_with_reference():
    g = golden("c1_trace_ref.npz")
    tris, _, _ = scenes.cornell_box()
    rays = scenes.parity_rays(1 << 20, C1_LO, C1_HI, seed=1)
    ids, t = orc.closest_brute(tris, rays)
    ref_ids = g["ids"].astype(np.int32)
    assert np.array_equal(ids, ref_ids)
    assert np.array_equal(t[:1 << 16], g["t_head"])
    # the reference reports every Cornell ray (no table overflow)
    assert g["ok"][ref_ids >= 0].all()


def test_exact_intersection_agrees_with_reference_test_away_from_edges():
    """orc.exact_hit (exact rational arithmetic) gives the reference test's
    answer wherever the float barycentrics are clear of the edges."""
    tris, _, _ = scenes.cornell_box()
    rays = scenes.parity_rays(64, C1_LO, C1_HI, seed=5)
    checked = 0
    for i in range(len(rays)):
        r = rays[i:i + 1]
        for k in range(0, len(tris), 3):
            t, u, v = (np.zeros(1, np.float32) for _ in range(3))
            hit = orc.orc().orc_intersect_ref(tris[k:k + 1].ctypes.data, r.ctypes.data, t.ctypes.data,
                                              u.ctypes.data, v.ctypes.data)
            if min(abs(u[0]), abs(v[0]), abs(1 - u[0] - v[0])) < 1e-3 or abs(t[0]) < 1e-3:
                continue
            ehit, et, eu, ev = orc.exact_hit(tris[k], r[0])
            assert bool(hit) == ehit
            if ehit:
                assert abs(float(et) - t[0]) <= 1e-5 * abs(t[0])
            checked += 1
    assert checked > 500


def test_oracle_bvh_equals_brute_force():
    tris, _, info = scenes.icosphere_field(n_meshes=2, subdiv=3, seed=5, box=6.0)
    rays = scenes.parity_rays(1 << 14, info["lo"], info["hi"], seed=9)
    a_ids, a_t = orc.closest_brute(tris, rays)
    b_ids, b_t = orc.closest_bvh(tris, rays)
    assert np.array_equal(a_ids, b_ids)
    assert np.array_equal(a_t, b_t)


def test_icosphere_closest_hits_match_reference():
    g = golden("ico_trace_ref.npz")
    tris, _, info = scenes.icosphere_field(n_meshes=2, subdiv=3, seed=5, box=6.0)
    rays = scenes.parity_rays(1 << 16, info["lo"], info["hi"], seed=3)
    assert digest(tris) == str(g["tri_digest"])
    ids, t = orc.closest_bvh(tris, rays)
    # the reference's return value is "found a hit"; at 2,562 triangles its
    # 5000-entry table never overflows, so every miss is a real miss
    assert np.array_equal(g["ok"] == 1, g["ids"] >= 0)
    flags = orc.classify(tris, rays, ids, t)
    sel = flags == 0
    assert sel.mean() > 0.999
    assert np.array_equal(ids[sel], g["ids"][sel])
    hit = sel & (ids >= 0)
    assert np.array_equal(t[hit], g["t"][hit])


def test_compat_render_per_sample_matches_reference():
    g = golden("c1_render_ref.npz")
    tris, mats, _ = scenes.cornell_box()
    W, H = int(g["width"]), int(g["height"])
    frames = g["frames"]
    out, nrays = orc.render_compat(tris, mats, g["camera"], W, H, frames.shape[0])
    a, b = out[:, 1:], frames[:, 1:]
    same = (a == b).all(-1)
    assert same.mean() > 0.999, same.mean()
    assert abs(nrays - int(g["rays"])) <= 0.001 * int(g["rays"])


def test_compat_render_mean_within_3_sigma_of_reference():
    g = golden("c1_render_ref.npz")
    tris, mats, _ = scenes.cornell_box()
    n = int(g["n32"])
    out, _ = orc.render_compat(tris, mats, g["camera32"], 32, 32, n)
    mean = out[:, 1:].mean(0)
    ref_mean, ref_var = g["mean32"][1:], g["var32"][1:]
    sigma = np.sqrt(2.0 * ref_var / n) + 1e-6
    frac_out = (np.abs(mean - ref_mean) > 3 * sigma).mean()
    assert frac_out < 0.01, frac_out


@pytest.mark.parametrize("kind", ["disney", "textured", "env"])
def test_compat_scene_per_sample_matches_reference(kind):
    """Disney materials, textures and the environment light (HDR NEE, IBL,
    MIS with both) in the reference's own estimator: every sample of the
    oracle equals the reference's bit for bit, apart from the samples of the
    rare pixels where the two traversals (the oracle's brute force, the
    reference's BVH) break a closest-hit tie differently: two pixels of the
    2,303 over six frames (1677 at frame 0, 330 at frame 5)."""
    g = golden("parity_scenes_ref.npz")
    tris, mats, _, tex, env = scenes.parity_scene(kind)
    frames = g[f"{kind}_frames"]
    out, nrays = orc.render_compat(tris, mats, g[f"{kind}_camera"], 48, 48, frames.shape[0], env=env,
                                   textures=tex)
    a, b = out[:, 1:], frames[:, 1:]
    same = (a == b).all(-1)
    assert same.mean() > 0.999, same.mean()
    assert len(np.unique(np.nonzero(~same)[1])) <= 2
    if kind == "env":
        # no face light: the reference still traces its face-light shadow ray
        # toward Objects[-1] (ChooseLightSource returns -1,
        # NextEventEstimation_FaceLight.cuh:25,61), a ray that can never count,
        # which the oracle does not trace
        assert nrays < int(g[f"{kind}_rays"])
    else:
        assert nrays == int(g[f"{kind}_rays"])


@pytest.mark.parametrize("kind", ["disney", "textured", "env"])
def test_compat_scene_mean_within_3_sigma_of_reference(kind):
    g = golden("parity_scenes_ref.npz")
    tris, mats, _, tex, env = scenes.parity_scene(kind)
    n = int(g[f"{kind}_n32"])
    out, _ = orc.render_compat(tris, mats, g[f"{kind}_camera32"], 32, 32, n, env=env, textures=tex)
    mean = out[:, 1:].mean(0)
    ref_mean, ref_var = g[f"{kind}_mean32"][1:], g[f"{kind}_var32"][1:]
    sigma = np.sqrt(2.0 * ref_var / n) + 1e-6
    assert (np.abs(mean - ref_mean) > 3 * sigma).mean() < 0.01


def test_c1_image_matches_reference():
    """The Cornell box at config C1's size (256 x 256, 16 samples per pixel):
    the oracle's per-pixel means equal the reference's (stored as float16)."""
    g = golden("c1_image_ref.npz")
    tris, mats, _ = scenes.cornell_box()
    out, nrays = orc.render_compat(tris, mats, g["camera"], 256, 256, int(g["spp"]))
    mean = out[:, 1:].mean(0).astype(np.float16).astype(np.float32)
    ref = g["mean16"][1:].astype(np.float32)
    same = (mean == ref).all(-1)
    assert same.mean() > 0.999, same.mean()
    assert abs(nrays - int(g["rays16"])) <= 1e-4 * int(g["rays16"])
    # every sample of the 2048 stored pixels over the 16 chained frames
    px = g["px_sample"]
    same_s = (out[:, px] == g["samples16"]).all(-1)
    assert same_s.mean() > 0.999, same_s.mean()


def test_reference_build_is_deterministic_on_disney():
    """With the reference's uninitialised lobe-sum array read as zeros
    (oracle/Makefile builds it with -ftrivial-auto-var-init=zero), repeated
    reference renders of a Disney scene agree bit for bit."""
    if not orc.ref_available():
        pytest.skip("the reference build (oracle/_ref) is not here")
    tris, mats, c, tex, env = scenes.parity_scene("disney")
    cam = orc.camera_setup(c["origin"], c["dist"], c["rot"], 24)
    a, _ = orc.ref_render(tris, mats, cam, 24, 24, 1)
    b, _ = orc.ref_render(tris, mats, cam, 24, 24, 3)
    assert np.array_equal(a[0, 1:], b[0, 1:])


def test_disney_brdf_bit_exact_with_reference():
    g = golden("disney_ref.npz")
    for k in range(len(g["mats"])):
        b, p = orc.disney_eval(g["mats"][k], g["wo"][k], g["wi"][k], g["n"][k])
        assert np.array_equal(b, g["brdf"][k])
        assert np.array_equal(p, g["pdf"][k])


def test_camera_setup_matches_reference():
    g = golden("camera_ref.npz")
    for k in range(len(g["org"])):
        c = orc.camera_setup(g["org"][k], float(g["dist"][k]), g["rot"][k], 1080)
        assert np.array_equal(c, g["cams"][k])


def test_light_and_env_cdfs_match_reference():
    g = golden("cdf_ref.npz")
    tris, mats, _ = scenes.cornell_box()
    assert np.array_equal(orc.light_cdf(tris, mats), g["light"])
    assert np.array_equal(orc.env_cdf(g["env"]), g["env_cdf"])


def test_tonemap_rule():
    img = np.array([[0.0, 0.5, 1.0, 0], [2.0, -1.0, 0.25, 0], [1e-4, 0.999, 0.218, 0]], np.float32)
    out = orc.tonemap(img)
    exp = np.clip(np.power(img[:, :3], np.float32(1 / 2.2)), 0, 1)
    exp = np.nan_to_num(exp, nan=0.0)
    assert np.array_equal(out[:, :3], (exp * 255).astype(np.uint8))
    assert (out[:, 3] == 255).all()


def test_svgf_restatement_bit_exact_with_reference():
    g = golden("svgf_ref.npz")
    W, H = int(g["width"]), int(g["height"])
    npx = W * H
    prev = np.zeros(npx * 112, np.uint8)
    cur = g["gbuf"].copy()
    r0, f0 = g["res0"].copy(), np.zeros_like(g["res0"])
    orc.svgf_compat(W, H, r0, f0, prev, cur, 0)
    assert np.array_equal(f0, g["out_filtered0"])
    assert np.array_equal(r0, g["out_result0"])
    assert np.array_equal(cur, g["out_cur0"])
    prev1, cur1 = cur.copy(), g["gbuf"].copy()
    r1, f1 = g["res1"].copy(), np.zeros_like(g["res1"])
    orc.svgf_compat(W, H, r1, f1, prev1, cur1, 1)
    assert np.array_equal(f1, g["out_filtered1"])
    assert np.array_equal(cur1, g["out_cur1"])


def test_mlp_oracle_gradients_match_finite_differences():
    """The FP64 MLP oracle's backward pass, checked by central differences of
    the relative-L2 loss with its stop-gradient denominator held at the base
    point."""
    from oracle import mlp_oracle as mo
    rng = np.random.default_rng(0)
    w = [rng.uniform(-1, 1, (64, 64)) * 0.3 for _ in range(5)] + [rng.uniform(-1, 1, (3, 64)) * 0.3]
    raw = rng.uniform(0, 1, (64, 13))
    t = rng.uniform(0, 1, (64, 3))
    _, g, y0 = mo.gradients(w, raw, t, quantize=False)
    den0 = y0 * y0 + mo.EPS_REL

    def frozen_loss(ws):
        y, _, _ = mo.forward(ws, raw, quantize=False)
        return np.sum((y - t) ** 2 / den0) / y.size

    eps = 1e-6
    for (l, i, j) in [(0, 3, 40), (2, 5, 7), (4, 63, 0), (5, 1, 17)]:
        wp = [x.copy() for x in w]
        wp[l][i, j] += eps
        wm = [x.copy() for x in w]
        wm[l][i, j] -= eps
        fd = (frozen_loss(wp) - frozen_loss(wm)) / (2 * eps)
        assert abs(fd - g[l][i, j]) <= 1e-6 + 1e-5 * abs(fd), (l, i, j, fd, g[l][i, j])


def test_reference_arm_svgf_input_matches_reference_records():
    """The records the reference arm feeds the reference's own ApplySVGF
    (oracle/ref_gpu.py cornell_svgf_inputs: RayTrace.cuh:66-82 restated over
    the oracle's primary hits) against the records the reference's render()
    fills for the same Cornell-box view (svgf_ref.npz, its host build)."""
    from oracle import ref_gpu
    g = golden("svgf_ref.npz")
    W, H = int(g["width"]), int(g["height"])
    res, rec = ref_gpu.cornell_svgf_inputs(W, H)
    a, b = rec.view(ref_gpu._SVGF_REC), g["gbuf"].view(ref_gpu._SVGF_REC)
    same = (a["ObjectID"] == b["ObjectID"]) & (a["MaterialID"] == b["MaterialID"]) & (a["Depth"] == b["Depth"])
    same &= (np.abs(a["Normal"] - b["Normal"]) <= 1e-6).all(-1) & (a["Albedo"] == b["Albedo"]).all(-1)
    same &= (a["PosLastFrameI"] == b["PosLastFrameI"]).all(-1) & (a["MomentOne"] == b["MomentOne"])
    assert same.mean() >= 1.0 - 1.5 / len(same), same.mean()  # one record may differ (a tie at an edge)
    assert res.shape == (W * H, 4) and np.isfinite(res).all()
