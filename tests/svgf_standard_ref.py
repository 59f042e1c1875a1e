"""A numpy restatement of the standard SVGF filter (kgk_svgf, mode
KGK_SVGF_STANDARD) for the parity test of its CUDA kernels.  The reference
has no such filter (its ApplySVGF is the compat filter, restated in
oracle/orc.c); this is the specification of this library's own: temporal
integration of demodulated colour and luminance moments, the variance from
moments or a 7 x 7 spatial estimate, a-trous passes at steps 1, 2, 4, ...
with the 3 x 3 blurred variance, the first pass fed back into the history,
and re-modulation by the albedo.

Reprojection is restated only for a camera that does not move: every pixel
reprojects onto itself (the kernel's bilinear taps put all but rounding-level
weight there).  Computes in float64; the device's weights use the hardware
ex2 / lg2 approximations (relative error ~2^-22).
"""
import numpy as np

KS = 1e-4
LOG2E = 1.4426950408889634
FIREFLY = 4.0
KG = np.array([0.25, 0.5, 0.25])
KW1 = np.array([1, 4, 6, 4, 1]) / 16.0


def lum(c):
    return 0.2126 * c[..., 0] + 0.7152 * c[..., 1] + 0.0722 * c[..., 2]


def shifted(a, ox, oy, fill):
    """a[y + oy, x + ox] for every (y, x), `fill` outside the image."""
    H, W = a.shape[:2]
    out = np.full_like(a, fill)
    ys, yd = (slice(oy, H), slice(0, H - oy)) if oy >= 0 else (slice(0, H + oy), slice(-oy, H))
    xs, xd = (slice(ox, W), slice(0, W - ox)) if ox >= 0 else (slice(0, W + ox), slice(-ox, W))
    out[yd, xd] = a[ys, xs]
    return out


def inside(H, W, ox, oy):
    y, x = np.mgrid[0:H, 0:W]
    return (x + ox >= 0) & (x + ox < W) & (y + oy >= 0) & (y + oy < H)


def depth_gradient(d, sz, step):
    """sigma_z * |grad d| * step, the gradient as max of the central
    differences (one-sided at the border)."""
    H, W = d.shape
    y, x = np.mgrid[0:H, 0:W]
    dxp = np.where(x + 1 < W, shifted(d, 1, 0, 0.0), d)
    dxm = np.where(x > 0, shifted(d, -1, 0, 0.0), d)
    dyp = np.where(y + 1 < H, shifted(d, 0, 1, 0.0), d)
    dym = np.where(y > 0, shifted(d, 0, -1, 0.0), d)
    return sz * 0.5 * np.maximum(np.abs(dxp - dxm), np.abs(dyp - dym)) * step


class StandardSVGF:
    def __init__(self, W, H, alpha=0.2, sz=1.0, sn=128.0, sl=4.0, iterations=5, firefly=False):
        self.W, self.H = W, H
        self.alpha, self.sz, self.sn, self.sl, self.iters = alpha, sz, sn, sl, iterations
        self.firefly = firefly  # the temporal mode's outlier clamp
        self.prev = None  # (hist, mom, normal, depth, mat)

    def frame(self, noisy, normal, depth, mat, albedo):
        """noisy, normal, albedo: (H, W, 3); depth (H, W); mat (H, W) int,
        -1 for no hit.  Returns the filtered frame (H, W, 3)."""
        H, W = self.H, self.W
        noisy, normal, albedo, depth = (np.asarray(a, np.float64) for a in (noisy, normal, albedo, depth))
        hit = mat >= 0
        dl = noisy / (albedo + KS)
        l = lum(dl)
        if self.firefly:
            # 4x the brightest of the eight neighbours that hit (+ 1e-3)
            lmax = np.zeros((H, W))
            anyn = np.zeros((H, W), bool)
            for oy in (-1, 0, 1):
                for ox in (-1, 0, 1):
                    if ox == 0 and oy == 0:
                        continue
                    qh = shifted(hit, ox, oy, False)
                    ql = shifted(l, ox, oy, 0.0)
                    lmax = np.where(qh, np.maximum(lmax, ql), lmax)
                    anyn |= qh
            cap = FIREFLY * lmax + 1e-3
            clamp = hit & anyn & (l > cap)
            scale = np.where(clamp, cap / np.where(clamp, l, 1.0), 1.0)
            dl0 = dl
            dl = dl * scale[..., None]
            l = np.where(clamp, cap, l)
            # the 3 x 3 colour box (neighbours that hit, unclamped; the pixel
            # itself clamped) that the history is clamped to
            bmin, bmax = dl.copy(), dl.copy()
            for oy in (-1, 0, 1):
                for ox in (-1, 0, 1):
                    if ox == 0 and oy == 0:
                        continue
                    qh = shifted(hit, ox, oy, False)[..., None]
                    qd = shifted(dl0, ox, oy, 0.0)
                    bmin = np.where(qh, np.minimum(bmin, qd), bmin)
                    bmax = np.where(qh, np.maximum(bmax, qd), bmax)
        hist = np.zeros((H, W, 4))
        mom = np.zeros((H, W, 2))
        c = dl.copy()
        m = np.stack([l, l * l], -1)
        length = np.ones((H, W))
        if self.prev is not None:
            ph, pm, pn, pd, pmat = self.prev
            ok = hit & (pmat == mat) & ((pn * normal).sum(-1) >= 0.9) & (np.abs(pd - depth) <= 0.05 * depth + 1e-3)
            length = np.where(ok, np.minimum(ph[..., 3] + 1.0, 64.0), 1.0)
            ac = np.maximum(self.alpha, 1.0 / length)
            hc = np.clip(ph[..., :3], bmin, bmax) if self.firefly else ph[..., :3]
            c = np.where(ok[..., None], hc * (1 - ac[..., None]) + dl * ac[..., None], dl)
            m = np.where(ok[..., None], np.stack([pm[..., 0] * (1 - ac) + l * ac, pm[..., 1] * (1 - ac) + l * l * ac], -1),
                         m)
        hist[..., :3] = np.where(hit[..., None], c, noisy)
        hist[..., 3] = np.where(hit, length, 0.0)
        mom[:] = np.where(hit[..., None], m, 0.0)
        col = np.zeros((H, W, 4))
        col[..., :3] = hist[..., :3]
        col[..., 3] = self._variance(hist, mom, normal, depth, mat)
        src = col
        for i in range(self.iters):
            src = self._atrous(src, normal, depth, mat, 1 << i)
            if i == 0:
                hist[..., :3] = np.where(hit[..., None], src[..., :3], hist[..., :3])
        out = np.where(hit[..., None], src[..., :3] * (albedo + KS), src[..., :3])
        self.prev = (hist, mom, normal, depth, np.where(hit, mat, -1))
        return out

    def _variance(self, hist, mom, normal, depth, mat):
        H, W = self.H, self.W
        hit = mat >= 0
        length = hist[..., 3]
        temporal = np.maximum(0.0, mom[..., 1] - mom[..., 0] ** 2)
        kz = depth_gradient(depth, self.sz, 1)
        s1 = np.zeros((H, W))
        s2 = np.zeros((H, W))
        sw = np.zeros((H, W))
        with np.errstate(divide="ignore"):
            for ky in range(-3, 4):
                for kx in range(-3, 4):
                    qm = shifted(mat, kx, ky, -2)
                    qn = shifted(normal, kx, ky, 0.0)
                    qd = shifted(depth, kx, ky, 0.0)
                    qmo = shifted(mom, kx, ky, 0.0)
                    rz = LOG2E / (kz * np.sqrt(kx * kx + ky * ky) + 1e-3)
                    e = self.sn * np.log2(np.maximum(0.0, (normal * qn).sum(-1))) - np.abs(depth - qd) * rz
                    w = np.where(qm == mat, np.exp2(e), 0.0)
                    s1 += w * qmo[..., 0]
                    s2 += w * qmo[..., 1]
                    sw += w
        with np.errstate(invalid="ignore", divide="ignore"):
            spatial = np.where(sw > 0, np.maximum(0.0, s2 / sw - (s1 / sw) ** 2), 0.0) * 4.0 / length
        return np.where(hit, np.where(length >= 4.0, temporal, spatial), 0.0)

    def _atrous(self, col, normal, depth, mat, step):
        H, W = self.H, self.W
        hit = mat >= 0
        gs = np.zeros((H, W))
        gw = np.zeros((H, W))
        for ky in (-1, 0, 1):
            for kx in (-1, 0, 1):
                k = KG[kx + 1] * KG[ky + 1]
                ins = inside(H, W, kx, ky)
                gs += np.where(ins, k * shifted(col[..., 3], kx, ky, 0.0), 0.0)
                gw += np.where(ins, k, 0.0)
        gvar = gs / gw
        kz = depth_gradient(depth, self.sz, step)
        l = lum(col[..., :3])
        rl = LOG2E / (self.sl * np.sqrt(np.maximum(gvar, 0.0)) + 1e-6)
        k0 = KW1[2] * KW1[2]
        sc = col[..., :3] * k0
        sv = k0 * k0 * col[..., 3]
        sw = np.full((H, W), k0)
        with np.errstate(divide="ignore"):
            for oy in range(-2, 3):
                for ox in range(-2, 3):
                    if ox == 0 and oy == 0:
                        continue
                    qm = shifted(mat, ox * step, oy * step, -2)
                    qn = shifted(normal, ox * step, oy * step, 0.0)
                    qd = shifted(depth, ox * step, oy * step, 0.0)
                    qc = shifted(col, ox * step, oy * step, 0.0)
                    rz = LOG2E / (kz * np.sqrt(ox * ox + oy * oy) + 1e-3)
                    e = (self.sn * np.log2(np.maximum(0.0, (normal * qn).sum(-1))) - np.abs(depth - qd) * rz -
                         np.abs(l - lum(qc[..., :3])) * rl)
                    w = np.where(qm == mat, KW1[ox + 2] * KW1[oy + 2] * np.exp2(e), 0.0)
                    sc += qc[..., :3] * w[..., None]
                    sv += w * w * qc[..., 3]
                    sw += w
        out = np.concatenate([sc / sw[..., None], (sv / (sw * sw))[..., None]], -1)
        return np.where(hit[..., None], out, col)
