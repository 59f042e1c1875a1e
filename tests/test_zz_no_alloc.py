"""kgk_svgf_apply_noalloc: the denoiser entry point for callers that cannot
allocate device memory (their allocator owns all of it, or their frame loop
must not call cudaMalloc / cudaFree, which synchronise the device).  It must
give the same result as kgk_svgf_apply, call after call, while taking its
scratch from the library's fixed device array.

This file sorts last so that a run stopping at the first failure has run
every other test before it."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from kagayaki_gb300._lib import check, last_error, lib

pytestmark = pytest.mark.gpu


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def test_noalloc_matches_kgk_svgf_apply_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = golden("svgf_ref.npz")
    W, H = int(g["width"]), int(g["height"])
    npx = W * H
    dev = torch.device("cuda", 0)

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    def vp(t):
        return ctypes.c_void_p(t.data_ptr())

    # existing entry point, host buffers
    prev_h = np.zeros(npx * 112, np.uint8)
    # allocation-free entry point, device buffers owned by the caller
    prev_d = d(np.zeros(npx * 112, np.uint8))
    for frame, res in ((0, g["res0"]), (1, g["res1"])):
        cur_h = g["gbuf"].copy()
        r_h, f_h = res.copy(), np.zeros_like(res)
        check(lib().kgk_svgf_apply(_p(r_h), _p(f_h), _p(prev_h), _p(cur_h), W, H, frame))
        cur_d = d(g["gbuf"])
        r_d, f_d = d(res), d(np.zeros_like(res))
        st = lib().kgk_svgf_apply_noalloc(vp(r_d), vp(f_d), vp(prev_d), vp(cur_d), W, H, frame, None)
        assert st == 0, last_error()
        # both entry points launch the same kernels on the same scratch layout,
        # so the outputs agree bit for bit (a scratch overlap would show here)
        np.testing.assert_array_equal(f_d.cpu().numpy(), f_h)
        np.testing.assert_array_equal(r_d.cpu().numpy(), r_h)
        np.testing.assert_array_equal(cur_d.cpu().numpy(), cur_h)
        # the next call filters the next frame against this one's state
        prev_h = cur_h
        prev_d = cur_d


def test_noalloc_rejects_oversize_and_host_buffers():
    W, H = 1024, 1024  # 2^20 pixels > KGK_SVGF_NOALLOC_MAX_PIXELS
    tiny = np.zeros(16, np.float32)
    st = lib().kgk_svgf_apply_noalloc(_p(tiny), _p(tiny), _p(tiny), _p(tiny), W, H, 0, None)
    assert st == 1 and "maximum" in last_error()
    r = np.zeros((4, 4), np.float32)
    b = np.zeros(4 * 112, np.uint8)
    st = lib().kgk_svgf_apply_noalloc(_p(r), _p(r), _p(b), _p(b), 2, 2, 0, None)
    assert st == 1 and "device memory" in last_error()
