"""FP64 CPU oracle of the radiance-cache MLP.  TEST INFRASTRUCTURE ONLY:
used by tests/ to check the GPU kernels' encoding, forward pass, gradients
and Adam steps.  The cache has no counterpart in the reference; this file
restates the network the library implements.

Network: 64 inputs -> `depth` hidden layers of `width` (ReLU, no biases) ->
3 outputs (linear).  Weights W[l] are (out, in) matrices.
Encoding of a query (13 raw floats: position normalised to [0,1]^3, normal,
view direction, roughness, albedo) into 64 inputs:
  [0, 36)  per axis a, octave k = 0..5: sin(2^k pi p_a), cos(2^k pi p_a)
  [36, 39) normal, [39, 42) view direction
  [42, 48) per component: sin(pi n_c), cos(pi n_c)
  [48, 54) per component: sin(pi v_c), cos(pi v_c)
  54 roughness, [55, 58) albedo, [58, 64) 1 (bias inputs)
Loss: relative L2, mean over samples and channels of
  (y - t)^2 / (stopgrad(y)^2 + 0.01).
"""
import numpy as np

N_IN = 64
N_RAW = 13
EPS_REL = 0.01


def encode(raw):
    raw = np.asarray(raw, np.float64)
    n = raw.shape[0]
    p, nr, v, r, a = raw[:, 0:3], raw[:, 3:6], raw[:, 6:9], raw[:, 9], raw[:, 10:13]
    x = np.zeros((n, N_IN))
    for ax in range(3):
        for k in range(6):
            x[:, ax * 12 + 2 * k] = np.sin(np.pi * (2.0 ** k) * p[:, ax])
            x[:, ax * 12 + 2 * k + 1] = np.cos(np.pi * (2.0 ** k) * p[:, ax])
    x[:, 36:39] = nr
    x[:, 39:42] = v
    for c in range(3):
        x[:, 42 + 2 * c] = np.sin(np.pi * nr[:, c])
        x[:, 42 + 2 * c + 1] = np.cos(np.pi * nr[:, c])
        x[:, 48 + 2 * c] = np.sin(np.pi * v[:, c])
        x[:, 48 + 2 * c + 1] = np.cos(np.pi * v[:, c])
    x[:, 54] = r
    x[:, 55:58] = a
    x[:, 58:64] = 1.0
    return x


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(weights, raw, quantize=True):
    """Returns (y, activations list [x, h1, ..., hL], pre-activations)."""
    q = bf16 if quantize else (lambda z: np.asarray(z, np.float64))
    x = q(encode(raw))
    acts = [x]
    pres = []
    h = x
    for W in weights[:-1]:
        z = h @ q(W).T
        pres.append(z)
        h = q(np.maximum(z, 0.0))
        acts.append(h)
    y = h @ q(weights[-1]).T
    return y, acts, pres


def loss_and_grad_y(y, t):
    d = y - t
    den = y * y + EPS_REL
    n = y.size
    loss = np.sum(d * d / den) / n
    dy = 2.0 * d / den / n
    return loss, dy


def gradients(weights, raw, target, quantize=True):
    """Gradients of the relative-L2 loss w.r.t. every W (FP64, through the
    same bf16-rounded weights / activations as the device when quantize)."""
    q = bf16 if quantize else (lambda z: np.asarray(z, np.float64))
    y, acts, pres = forward(weights, raw, quantize)
    loss, dy = loss_and_grad_y(y, np.asarray(target, np.float64))
    grads = [None] * len(weights)
    dz = dy
    for l in range(len(weights) - 1, -1, -1):
        grads[l] = dz.T @ acts[l]
        if l > 0:
            da = dz @ q(weights[l])
            dz = da * (pres[l - 1] > 0)
    return loss, grads, y


def adam(weights, grads, m, v, step, lr=1e-2, b1=0.9, b2=0.99, eps=1e-10):
    out = []
    for l, (W, g) in enumerate(zip(weights, grads)):
        m[l] = b1 * m[l] + (1 - b1) * g
        v[l] = b2 * v[l] + (1 - b2) * g * g
        mh = m[l] / (1 - b1 ** step)
        vh = v[l] / (1 - b2 ** step)
        out.append(W - lr * mh / (np.sqrt(vh) + eps))
    return out
