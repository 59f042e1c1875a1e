"""Unbiased estimator with Disney materials: a smooth-shaded sphere under a
constant environment L = 1.  A convex object never sees itself, so the
expected radiance of a visible point is the BRDF's directional albedo
A(wo) = integral of f(wi, wo) cos(wi) dwi, which this test integrates by
quadrature with an fp64 numpy statement of the BRDF the unbiased estimator
uses (Disney lobes as evaluated by the reference, specular shadowing by
height-correlated Smith GGX in the shading frame).  The renderer's per-pixel
means must match A(wo) within 3 sigma of the FP64 accumulator's estimate
(plus 0.5 % for the quadrature and the normal interpolation) — which checks
that the lobe sampling, its pdf and the MIS weights are consistent — and the
per-sample variance must stay bounded (no unbounded sampling weights).
"""
import numpy as np
import pytest

from kagayaki_gb300 import ESTIMATOR_UNBIASED, Scene, camera_setup, scenes, structs

pytestmark = pytest.mark.gpu


def disney_albedo(m, n, wo, n_theta=768, n_phi=1536):
    """A(wo) per channel for an isotropic Disney material (fp64 quadrature)."""
    base = np.array(m["diffuse"][:3], np.float64)
    rough, metal, spec = float(m["roughness"]), float(m["metallic"]), float(m["specular"])
    stint, cc, ccg = float(m["specularTint"]), float(m["clearcoat"]), float(m["cloearcoatGloss"])
    a = max(0.001, rough * rough)
    ac = (1 - ccg) * 0.1 + ccg * 0.001
    wt0 = 1 - metal
    # quadrature over the hemisphere around n: theta midpoints, phi midpoints
    th = (np.arange(n_theta) + 0.5) * (np.pi / 2) / n_theta
    ph = (np.arange(n_phi) + 0.5) * (2 * np.pi) / n_phi
    T, P = np.meshgrid(th, ph, indexing="ij")
    t = np.cross([0.0, 1.0, 0.0] if abs(n[0]) > 1e-4 else [1.0, 0.0, 0.0], n)
    t /= np.linalg.norm(t)
    b = np.cross(n, t)
    wi = (np.sin(T)[..., None] * (np.cos(P)[..., None] * t + np.sin(P)[..., None] * b) +
          np.cos(T)[..., None] * n)
    dw = np.sin(T) * (np.pi / 2 / n_theta) * (2 * np.pi / n_phi)
    ndl = np.cos(T)
    ndv = float(np.dot(n, wo))
    h = wi + wo
    h /= np.linalg.norm(h, axis=-1, keepdims=True)
    ldh = np.einsum("ijk,k->ij", h, wo)  # = wi.h
    ndh = h @ n
    sch = lambda x: (1 - x) ** 5  # noqa: E731
    FL, FV = sch(ndl), sch(ndv)
    fd90 = 0.5 + 2 * rough * ldh ** 2
    fd = ((1 - FL) + FL * fd90) * ((1 - FV) + FV * fd90)
    f = (base / np.pi)[None, None, :] * (fd * wt0)[..., None]
    nd = base / np.linalg.norm(base)
    rho = (1 - stint) + nd * stint
    f0 = rho * ((1 - metal) * 0.08 * spec) + base * metal
    fw = sch(ndh)
    F = f0[None, None, :] + (1 - f0)[None, None, :] * fw[..., None]
    q = (1 - ndh ** 2) / (a * a) + ndh ** 2
    D = 1 / (np.pi * a * a * q * q)

    def lam(c):
        return 0.5 * (-1 + np.sqrt(1 + a * a * (1 - c * c) / (c * c)))
    G = 1 / (1 + lam(ndv) + lam(ndl))
    f = f + F * (D * G / (4 * ndv * ndl))[..., None]
    if cc > 0:
        a2 = max(min(ac, 0.9999), 0.0001) ** 2
        Dc = ((a2 - 1) / (2 * np.pi * np.log(np.sqrt(a2)))) / ((a2 - 1) * ndh ** 2 + 1)
        Fc = 0.04 + 0.96 * fw

        def sg(c):
            return 1 / (c + np.sqrt(0.0625 + c * c - 0.0625 * c * c))
        f = f + (0.25 * cc * Fc * Dc * sg(ndv) * sg(ndl))[..., None]
    return (f * (ndl * dw)[..., None]).sum(axis=(0, 1))


@pytest.mark.parametrize("mat", [
    dict(diffuse=(0.8, 0.5, 0.3), roughness=0.5, specular=0.5),
    dict(diffuse=(0.9, 0.7, 0.2), roughness=0.35, metallic=1.0, specular=0.5),
    dict(diffuse=(0.2, 0.4, 0.8), roughness=0.6, specular=0.5, clearcoat=1.0, cloearcoatGloss=0.5),
])
def test_disney_sphere_under_constant_environment(mat):
    m = structs.make_material(structs.DISNEY, **mat)
    v, f = scenes.icosphere(5)
    v = v.astype(np.float32)
    uv = np.zeros((len(v), 2), np.float32)
    tris = scenes.canonical(scenes._tris_from_indexed(v, v, uv, f.astype(np.int64), 0, True, 0))
    env = np.ones((64, 128, 3), np.float32)
    W = H = 48
    with Scene(tris, np.stack([m]), env=env) as s:
        s.build_bvh()
        cam = camera_setup((0.0, 0.0, 3.2), 28.0, (0.0, 0.0, 0.0), H)
        s.accum_reset(W, H)
        for k in range(64):
            s.render(cam, W, H, spp=256, estimator=ESTIMATOR_UNBIASED, seed=11, frame_index=k,
                     accumulate=True, max_depth=6)
        mean, var, n = s.accum_read(W, H)
        # shading normal and view direction at a few pixels along a radius
        from kagayaki_gb300 import camera_array
        c = camera_array(cam)
        org = c[0:3]
        rays, pix = [], []
        for x in range(24, 37):
            y = 24
            d = (c[4:7] * c[8] + c[9:12] * ((x - W / 2) * c[17]) + c[13:16] * ((H / 2 - y) * c[17]))
            d /= np.linalg.norm(d)
            r = np.zeros((), structs.RAY)
            r["dir"][:3] = d
            r["org"][:3] = org
            rays.append(r)
            pix.append((y, x))
        rays = np.stack(rays)
        ids, t = s.trace_closest(rays)
    checked = 0
    for (y, x), r, i, tt in zip(pix, rays, ids, t):
        if i < 0:
            continue
        d = np.array(r["dir"][:3], np.float64)
        p = np.array(org, np.float64) + tt * d
        tv = tris["verts"][i].astype(np.float64)
        v0, v1, v2 = tv[0, :3], tv[1, :3], tv[2, :3]
        # barycentric weights of p, then the interpolated (smooth) normal
        e1, e2, ep = v1 - v0, v2 - v0, p - v0
        d11, d12, d22 = e1 @ e1, e1 @ e2, e2 @ e2
        dp1, dp2 = ep @ e1, ep @ e2
        den = d11 * d22 - d12 * d12
        b1 = (d22 * dp1 - d12 * dp2) / den
        b2 = (d11 * dp2 - d12 * dp1) / den
        nrm = (1 - b1 - b2) * tv[3, :3] + b1 * tv[4, :3] + b2 * tv[5, :3]
        nrm /= np.linalg.norm(nrm)
        wo = -d
        if nrm @ wo < 0.3:  # the radiance changes fast across a pixel near the silhouette
            continue
        A = disney_albedo(m, nrm, wo)
        got = mean[y, x]
        sig = np.sqrt(var[y, x])
        tol = 3 * sig + 0.005 * A + 1e-4
        assert np.all(np.abs(got - A) <= tol), (x, y, got, A, sig)
        # bounded weights: per-sample standard deviation (sigma of the mean * sqrt(n))
        assert np.all(sig * np.sqrt(n) < 5.0 * np.maximum(A, 0.05)), (x, y, sig * np.sqrt(n), A)
        checked += 1
    assert checked >= 8


def env_irradiance_lambert(env, n, albedo, n_lat=1024, n_lon=2048):
    """(albedo / pi) * integral of L(w) max(0, n.w) dw for the lat-long map
    `env` (row 0 = +z, column c at u = 1 - c / W), fp64 quadrature."""
    h, w, _ = env.shape
    lat = (np.arange(n_lat) + 0.5) / n_lat * np.pi - np.pi / 2
    lon = (np.arange(n_lon) + 0.5) / n_lon * 2 * np.pi - np.pi
    LA, LO = np.meshgrid(lat, lon, indexing="ij")
    d = np.stack([np.cos(LA) * np.cos(LO), np.cos(LA) * np.sin(LO), np.sin(LA)], -1)
    v = LA / np.pi + 0.5
    u = LO / (2 * np.pi) + 0.5
    row = np.clip(((1 - v) * h).astype(int), 0, h - 1)
    col = np.clip(((1 - u) * w).astype(int), 0, w - 1)
    L = env[row, col].astype(np.float64)
    dw = np.cos(LA) * (np.pi / n_lat) * (2 * np.pi / n_lon)
    c = np.maximum(0.0, d @ n)
    return np.asarray(albedo) / np.pi * (L * (c * dw)[..., None]).sum(axis=(0, 1))


def test_lambert_sphere_under_structured_environment():
    """Environment importance sampling (alias table), its pdf and the MIS
    weights: a Lambert sphere lit by a lat-long map with a bright lobe."""
    rng = np.random.default_rng(4)
    h, w = 32, 64
    env = rng.uniform(0.2, 1.0, (h, w, 3)).astype(np.float32)
    env[6:9, 40:44] = (60.0, 50.0, 30.0)  # a small bright patch
    m = structs.make_material(structs.LAMBERT, (0.7, 0.5, 0.3))
    v, f = scenes.icosphere(5)
    v = v.astype(np.float32)
    uv = np.zeros((len(v), 2), np.float32)
    tris = scenes.canonical(scenes._tris_from_indexed(v, v, uv, f.astype(np.int64), 0, True, 0))
    W = H = 48
    with Scene(tris, np.stack([m]), env=env) as s:
        s.build_bvh()
        cam = camera_setup((0.0, 0.0, 3.2), 28.0, (0.0, 0.0, 0.0), H)
        s.accum_reset(W, H)
        for k in range(32):
            s.render(cam, W, H, spp=256, estimator=ESTIMATOR_UNBIASED, seed=17, frame_index=k,
                     accumulate=True, max_depth=6)
        mean, var, n = s.accum_read(W, H)
    from kagayaki_gb300 import camera_array
    c = camera_array(cam)
    org = np.array(c[0:3], np.float64)
    checked = 0
    for (y, x) in [(24, 24), (24, 28), (24, 32), (20, 24), (28, 24), (18, 30), (30, 18), (26, 21)]:
        d = (c[4:7] * c[8] + c[9:12] * ((x - W / 2) * c[17]) + c[13:16] * ((H / 2 - y) * c[17])).astype(np.float64)
        d /= np.linalg.norm(d)
        # analytic unit-sphere hit (the 20,480-triangle icosphere is within 2e-4 of it)
        b = org @ d
        disc = b * b - (org @ org - 1.0)
        if disc <= 0:
            continue
        p = org + (-b - np.sqrt(disc)) * d
        nrm = p / np.linalg.norm(p)
        if nrm @ -d < 0.4:
            continue
        E = env_irradiance_lambert(env, nrm, (0.7, 0.5, 0.3))
        got, sig = mean[y, x], np.sqrt(var[y, x])
        assert np.all(np.abs(got - E) <= 3 * sig + 0.01 * E), (x, y, got, E, sig)
        checked += 1
    assert checked >= 6
