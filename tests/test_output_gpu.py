"""Frame output on the device: save_png's tone mapping (IO_save_png.cuh:34-56)
computed on the GPU, fused into SVGF's last pass, and the frame loop's
asynchronous RGBA8 copies.

  * the device tone mapping gives the host function's bytes exactly (bit for
    bit, including every step of the byte function, +-8 ulp around each, and
    NaN / infinities / negative / denormal inputs);
  * kgk_svgf_output from the frame kgk_render kept on the device gives the
    same filtered frame as kgk_svgf from host buffers, and RGBA8 bytes equal
    to the host tone mapping of that frame, in both filter modes;
  * asynchronous RGBA8 copies into pinned buffers, overlapping the next
    frames, equal the synchronous results frame for frame.
"""
import numpy as np
import pytest

from kagayaki_gb300 import ESTIMATOR_UNBIASED, Scene, camera_setup, scenes, tonemap
from kagayaki_gb300.api import PinnedBuffer
from kagayaki_gb300.structs import KgkSvgfConfig

pytestmark = pytest.mark.gpu


def _host_byte(x):
    return int(tonemap(np.array([[[x, 0, 0, 0]]], np.float32))[0, 0, 0])


def _steps():
    """Bit patterns where the host byte function steps up (binary search)."""
    out = []
    for k in range(1, 256):
        lo, hi = 0, 0x7f800000
        while lo < hi:
            mid = (lo + hi) // 2
            if _host_byte(np.uint32(mid).view(np.float32)) >= k:
                hi = mid
            else:
                lo = mid + 1
        out.append(lo)
    return np.array(out, np.int64)


def test_device_tonemap_matches_host_bytes():
    torch = pytest.importorskip("torch")
    steps = _steps()
    around = (steps[:, None] + np.arange(-8, 9)[None, :]).ravel()
    around = around[(around >= 0) & (around <= 0x7f800000)].astype(np.uint32).view(np.float32)
    rng = np.random.default_rng(2)
    special = np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, -1e-30, 1e-45, 1e-38, -3.0, 1.0, 1e30],
                       np.float32)
    vals = np.concatenate([around, special, rng.uniform(-1, 4, 100_000).astype(np.float32),
                           np.exp(rng.uniform(-60, 10, 100_000)).astype(np.float32)])
    n = len(vals) // 3 * 3
    img = np.zeros((1, n // 3, 4), np.float32)
    img[0, :, :3] = vals[:n].reshape(-1, 3)
    host = tonemap(img)
    dev_in = torch.from_numpy(img).cuda()
    dev_out = torch.zeros((1, n // 3, 4), dtype=torch.uint8, device="cuda")
    from kagayaki_gb300._lib import check, lib
    import ctypes
    # device image to a host buffer, and device image to a device buffer
    got = np.empty_like(host)
    check(lib().kgk_tonemap_rgba8(ctypes.c_void_p(dev_in.data_ptr()), n // 3, 1, ctypes.c_void_p(got.ctypes.data)))
    check(lib().kgk_tonemap_rgba8(ctypes.c_void_p(dev_in.data_ptr()), n // 3, 1,
                                  ctypes.c_void_p(dev_out.data_ptr())))
    torch.cuda.synchronize()
    assert np.array_equal(got, host)
    assert np.array_equal(dev_out.cpu().numpy(), host)
    # the steps themselves: every byte value is reached
    assert len(np.unique(host[..., :3])) == 256


def test_device_tonemap_equals_reference_save_png():
    """The device tone mapping against the bytes of the reference's own
    save_png (tests/golden/tonemap_ref.npz)."""
    torch = pytest.importorskip("torch")
    import ctypes
    from conftest import golden
    from kagayaki_gb300._lib import check, lib
    g = golden("tonemap_ref.npz")
    img = np.zeros((1, len(g["inputs"]), 4), np.float32)
    img[0, :, :3] = g["inputs"]
    dev_in = torch.from_numpy(img).cuda()
    dev_out = torch.zeros((1, len(g["inputs"]), 4), dtype=torch.uint8, device="cuda")
    check(lib().kgk_tonemap_rgba8(ctypes.c_void_p(dev_in.data_ptr()), len(g["inputs"]), 1,
                                  ctypes.c_void_p(dev_out.data_ptr())))
    torch.cuda.synchronize()
    assert np.array_equal(dev_out.cpu().numpy()[0], g["rgba"])


def _scene_and_cams(H):
    tris, mats, c = scenes.cornell_box()
    cams = [camera_setup((c["origin"][0] + 0.03 * f, c["origin"][1], c["origin"][2]), c["dist"], c["rot"], H)
            for f in range(6)]
    return tris, mats, cams


@pytest.mark.parametrize("mode", [0, 1])
def test_svgf_output_from_the_kept_frame(mode):
    W, H = 96, 64
    tris, mats, cams = _scene_and_cams(H)
    kw = dict(spp=2, estimator=ESTIMATOR_UNBIASED, seed=4, write_gbuffer=True, max_depth=6)
    cfg = KgkSvgfConfig(mode=mode, width=W, height=H, atrous_iterations=5, atrous_repeats=5, alpha=0.2,
                        sigma_z=1.0, sigma_n=128.0, sigma_l=4.0)
    # host buffers through kgk_svgf
    ref = []
    with Scene(tris, mats) as s:
        s.build_bvh()
        for f, cam in enumerate(cams[:3]):
            noisy, _ = s.render(cam, W, H, frame_index=f, **kw)
            cfg.frame_index = f
            filt = np.empty((H, W, 4), np.float32)
            s.svgf_output(cfg, noisy=noisy, filtered=filt)
            ref.append(filt)
    # the kept frame, float and RGBA8 outputs
    with Scene(tris, mats) as s:
        s.build_bvh()
        for f, cam in enumerate(cams[:3]):
            img, _ = s.render(cam, W, H, frame_index=f, keep_on_device=True, **kw)
            assert img is None
            cfg.frame_index = f
            filt = np.empty((H, W, 4), np.float32)
            rgba = np.empty((H, W, 4), np.uint8)
            s.svgf_output(cfg, filtered=filt, rgba8=rgba)
            assert np.array_equal(filt[..., :3], ref[f][..., :3]), f
            assert np.array_equal(rgba, tonemap(filt)), f


def test_async_rgba8_copies_equal_the_synchronous_results():
    W, H = 128, 96
    tris, mats, cams = _scene_and_cams(H)
    kw = dict(spp=1, estimator=ESTIMATOR_UNBIASED, seed=8, write_gbuffer=True, max_depth=6)
    cfg = KgkSvgfConfig(mode=1, width=W, height=H, atrous_iterations=5, alpha=0.2, sigma_z=1.0, sigma_n=128.0,
                        sigma_l=4.0)
    sync_bytes = []
    with Scene(tris, mats) as s:
        s.build_bvh()
        for f, cam in enumerate(cams):
            s.render(cam, W, H, frame_index=f, keep_on_device=True, **kw)
            cfg.frame_index = f
            rgba = np.empty((H, W, 4), np.uint8)
            s.svgf_output(cfg, rgba8=rgba)
            sync_bytes.append(rgba)
    bufs = [PinnedBuffer((H, W, 4), np.uint8) for _ in cams]
    try:
        with Scene(tris, mats) as s:
            s.build_bvh()
            for f, cam in enumerate(cams):
                # the copy of frame f-1 runs while frame f renders
                s.render(cam, W, H, frame_index=f, keep_on_device=True, **kw)
                cfg.frame_index = f
                s.svgf_output(cfg, rgba8=bufs[f].array, async_=True)
            s.sync()
            for f in range(len(cams)):
                assert np.array_equal(bufs[f].array, sync_bytes[f]), f
    finally:
        for b in bufs:
            b.free()


def test_svgf_output_needs_a_kept_frame():
    from kagayaki_gb300 import KgkError
    W, H = 32, 32
    tris, mats, cams = _scene_and_cams(H)
    cfg = KgkSvgfConfig(mode=1, width=W, height=H, atrous_iterations=5, alpha=0.2, sigma_z=1.0, sigma_n=128.0,
                        sigma_l=4.0)
    with Scene(tris, mats) as s:
        s.build_bvh()
        s.render(cams[0], W, H, spp=1, estimator=ESTIMATOR_UNBIASED, write_gbuffer=True)  # host output
        with pytest.raises(KgkError, match="keep its frame"):
            s.svgf_output(cfg, rgba8=np.empty((H, W, 4), np.uint8))
        with pytest.raises(KgkError, match="no output"):
            s.svgf_output(cfg)


def test_exr_from_device_memory_equals_host(tmp_path):
    """kgk_save_exr from a device image writes the same file as from the host copy."""
    torch = pytest.importorskip("torch")
    import ctypes
    from kagayaki_gb300 import save_exr
    from kagayaki_gb300._lib import check, lib
    rng = np.random.default_rng(5)
    img = rng.lognormal(0, 2, (24, 31, 4)).astype(np.float32)
    dev = torch.from_numpy(img).cuda()
    for half in (0, 1):
        save_exr(img, tmp_path / "host.exr", half=bool(half))
        check(lib().kgk_save_exr(ctypes.c_void_p(dev.data_ptr()), 31, 24, half, str(tmp_path / "dev.exr").encode()))
        assert (tmp_path / "host.exr").read_bytes() == (tmp_path / "dev.exr").read_bytes()
