"""Radiance-cache MLP kernels against the FP64 oracle (oracle/mlp_oracle.py),
at hidden width 64 and 128.

Tolerances: the device runs BF16 weights/activations with FP32 accumulation;
the oracle replays the same BF16 rounding of weights, encoded inputs and
activations in FP64, so the remaining differences are accumulation order
and BF16 rounding of gradients inside backpropagation.
  forward:   |y_gpu - y_ref| <= 2e-2 * (|y_ref| + 0.05)
  gradients: per-layer relative L2 error <= 3e-2
"""
import ctypes

import numpy as np
import pytest

from kagayaki_gb300 import Scene, scenes
from kagayaki_gb300._lib import check, lib
from kagayaki_gb300.structs import KgkNrcConfig
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

FWD_TOL = 2e-2
GRAD_TOL = 3e-2


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def n_params(width):
    return width * 64 + 4 * width * width + 3 * width


def init(s, width):
    cfg = KgkNrcConfig(width=width)
    check(lib().kgk_nrc_init(s._h, ctypes.byref(cfg)))


@pytest.fixture(scope="module", params=[64, 128], ids=["w64", "w128"])
def cache_scene(request):
    tris, mats, _ = scenes.cornell_box()
    s = Scene(tris, mats)
    s.width = request.param
    init(s, s.width)
    yield s
    s.close()


def split(w, width):
    """Flat master weights -> [(width, 64), 4 x (width, width), (3, width)]."""
    out, o = [], 0
    for fan_in in [64, width, width, width, width]:
        out.append(w[o:o + width * fan_in].reshape(width, fan_in))
        o += width * fan_in
    out.append(w[o:o + 3 * width].reshape(3, width))
    assert o + 3 * width == w.size
    return out


def rand_weights(seed, width, scale=1.0):
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-1, 1, m.size) * scale * np.sqrt(6.0 / m.shape[1])
             for m in split(np.zeros(n_params(width)), width)]
    return np.concatenate(parts).astype(np.float32)


def rand_raw(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.uniform(0, 1, (n, 3))
    nr = rng.normal(size=(n, 3))
    nr /= np.linalg.norm(nr, axis=1, keepdims=True)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    r = rng.uniform(0, 1, (n, 1))
    a = rng.uniform(0, 1, (n, 3))
    return np.concatenate([p, nr, v, r, a], 1).astype(np.float32)


def set_w(s, w):
    check(lib().kgk_nrc_set_weights(s._h, _p(w), w.size))


def test_weights_roundtrip(cache_scene):
    w = rand_weights(1, cache_scene.width)
    set_w(cache_scene, w)
    back = np.empty_like(w)
    check(lib().kgk_nrc_get_weights(cache_scene._h, _p(back), back.size))
    assert np.array_equal(w, back)


def test_wrong_weight_count_is_rejected(cache_scene):
    from kagayaki_gb300 import KgkError
    w = rand_weights(1, 192 - cache_scene.width)
    with pytest.raises(KgkError, match="expected"):
        set_w(cache_scene, w)


def test_unsupported_width_is_rejected():
    from kagayaki_gb300 import KgkError
    tris, mats, _ = scenes.cornell_box()
    with Scene(tris, mats) as s:
        with pytest.raises(KgkError, match="width 64 or 128"):
            init(s, 96)


def test_forward_matches_oracle(cache_scene):
    W = cache_scene.width
    w = rand_weights(2, W)
    set_w(cache_scene, w)
    raw = rand_raw(1000, 3)
    out = np.empty((1000, 3), np.float32)
    check(lib().kgk_nrc_infer(cache_scene._h, _p(raw), 1000, _p(out)))
    y, _, _ = mo.forward(split(w.astype(np.float64), W), raw.astype(np.float64))
    err = np.abs(out - y) / (np.abs(y) + 0.05)
    assert err.max() <= FWD_TOL, err.max()


def test_gradients_match_oracle(cache_scene):
    W = cache_scene.width
    w = rand_weights(4, W)
    set_w(cache_scene, w)
    n = 4096
    raw = rand_raw(n, 5)
    tgt = np.random.default_rng(6).uniform(0, 2, (n, 3)).astype(np.float32)
    g = np.empty(n_params(W), np.float32)
    loss = np.zeros(1, np.float32)
    check(lib().kgk_nrc_gradients(cache_scene._h, _p(raw), _p(tgt), n, _p(g), _p(loss)))
    ref_loss, ref_g, _ = mo.gradients(split(w.astype(np.float64), W), raw.astype(np.float64),
                                      tgt.astype(np.float64))
    assert abs(loss[0] - ref_loss) <= 1e-2 * abs(ref_loss), (loss[0], ref_loss)
    for l, (gg, rg) in enumerate(zip(split(g.astype(np.float64), W), ref_g)):
        rel = np.linalg.norm(gg - rg) / np.linalg.norm(rg)
        assert rel <= GRAD_TOL, (l, rel)


def test_adam_step_matches_oracle(cache_scene):
    W = cache_scene.width
    w = rand_weights(7, W)
    set_w(cache_scene, w)
    init(cache_scene, W)  # fresh Adam state
    set_w(cache_scene, w)
    n = 2048
    raw = rand_raw(n, 8)
    tgt = np.random.default_rng(9).uniform(0, 2, (n, 3)).astype(np.float32)
    g = np.empty(n_params(W), np.float32)
    check(lib().kgk_nrc_gradients(cache_scene._h, _p(raw), _p(tgt), n, _p(g), None))
    loss = np.zeros(1, np.float32)
    check(lib().kgk_nrc_train(cache_scene._h, _p(raw), _p(tgt), n, 1, _p(loss)))
    after = np.empty_like(w)
    check(lib().kgk_nrc_get_weights(cache_scene._h, _p(after), after.size))
    m = [np.zeros_like(x) for x in split(w.astype(np.float64), W)]
    v = [np.zeros_like(x) for x in split(w.astype(np.float64), W)]
    exp = mo.adam(split(w.astype(np.float64), W), split(g.astype(np.float64), W), m, v, 1)
    # a first Adam step moves every weight by about lr * sign(g)
    np.testing.assert_allclose(after, np.concatenate([e.ravel() for e in exp]), rtol=0, atol=2e-4)


def test_training_fits_a_radiance_field(cache_scene):
    init(cache_scene, cache_scene.width)
    n = 16384
    raw = rand_raw(n, 10)
    p = raw[:, :3]
    tgt = np.stack([0.5 + 0.4 * np.sin(2 * np.pi * p[:, 0]), 0.6 + 0.3 * np.cos(2 * np.pi * p[:, 1]),
                    0.3 + 0.2 * p[:, 2] * raw[:, 12]], 1).astype(np.float32)
    l0 = np.zeros(1, np.float32)
    check(lib().kgk_nrc_train(cache_scene._h, _p(raw), _p(tgt), n, 1, _p(l0)))
    l1 = np.zeros(1, np.float32)
    check(lib().kgk_nrc_train(cache_scene._h, _p(raw), _p(tgt), n, 400, _p(l1)))
    assert l1[0] < 0.05 * l0[0], (l0, l1)
    test = rand_raw(2048, 11)
    out = np.empty((2048, 3), np.float32)
    check(lib().kgk_nrc_infer(cache_scene._h, _p(test), 2048, _p(out)))
    pt = test[:, :3]
    exp = np.stack([0.5 + 0.4 * np.sin(2 * np.pi * pt[:, 0]), 0.6 + 0.3 * np.cos(2 * np.pi * pt[:, 1]),
                    0.3 + 0.2 * pt[:, 2] * test[:, 12]], 1)
    assert np.mean(np.abs(out - exp)) < 0.05
    sc = np.zeros(1, np.float32)
    check(lib().kgk_nrc_loss_scale(cache_scene._h, _p(sc)))
    assert sc[0] >= 1.0
