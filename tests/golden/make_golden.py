"""Generates the golden fixtures in tests/golden/ by running the reference's
own render-path source compiled for the host (oracle/_ref, built from the
reference checkout by `make -C oracle ref`).  Run in a container that has the
reference checkout:

    python tests/golden/make_golden.py

Fixtures:
  c1_trace_ref.npz      reference closest hits of the 2^20 Cornell parity rays
                        (ids for all rays, t for the first 2^16), ray digest
  ico_trace_ref.npz     the same for a 2-icosphere scene (2,562 triangles)
  c1_render_ref.npz     per-sample compat renders (render.cuh:21-49) of the
                        Cornell box, 48x48, 8 chained frames, plus 256-frame
                        mean/variance at 32x32
  disney_ref.npz        evaluate_Disney_BRDF / _pdf on seeded directions
  camera_ref.npz        Camera_SetUpCamera for a few poses
  cdf_ref.npz           calculate_Lss / calculate_Lss_HDR for small inputs
  svgf_ref.npz          ApplySVGF (race-free reading) on two frames
  parity_scenes_ref.npz per-sample compat renders of the Disney, textured and
                        environment scenes of scenes.parity_scene (48x48, 6
                        chained frames), their 256-frame mean/variance at
                        32x32, and render()'s SVGFBuffer records at 32x32
  c1_image_ref.npz      the Cornell box at config C1's size (256x256): the
                        16-sample per-pixel mean and the per-pixel standard
                        deviation of one sample (from 256 samples), float16,
                        and all 16 samples of 2048 seeded pixels (float32)
  tonemap_ref.npz       save_png's bytes (the reference's gamma, clamp and
                        truncation, through its PNG writer and read back)
                        for every step of the byte function +-8 ulp, special
                        and random values
  loader_ref.npz        load_object + load_Textures on the seeded OBJ scene of
                        tests/golden/scene_files.py, and stbi_loadf on its
                        seeded PNG / PNM / .hdr images

    python tests/golden/make_golden.py --only loader   # just loader_ref.npz
    python tests/golden/make_golden.py --only parity   # the two files above
    python tests/golden/make_golden.py --only tonemap  # tonemap_ref.npz

The reference's sample_BXDF (sampling.cuh:15-19) adds into an uninitialised
array, so its Disney lobe choice depends on stack contents; oracle/Makefile
builds the reference with -ftrivial-auto-var-init=zero, which gives that
array its zero-initialised reading and makes the renders reproducible.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from kagayaki_gb300 import scenes, structs  # noqa: E402
from oracle import orc  # noqa: E402

C1_LO, C1_HI = (-4.99, 0.01, -4.99), (4.99, 9.99, 4.99)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ico_scene():
    tris, mats, info = scenes.icosphere_field(n_meshes=2, subdiv=3, seed=5, box=6.0)
    return tris, mats, info


def make_loader_golden():
    """Reference loader outputs for the seeded files of scene_files.py."""
    import tempfile
    sys.path.insert(0, HERE)
    import scene_files
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name in scene_files.write_images(d):
            img = orc.ref_load_image(os.path.join(d, name))
            assert img is not None, name
            out["img_" + name] = img
        scene_files.write_obj_scene(d)
        tris, mats, texs = orc.ref_load_obj(d)
    out["obj_tris"] = scenes.canonical(tris)
    out["obj_mats"] = mats
    for i, t in enumerate(texs):
        out[f"obj_tex{i}"] = t
    out["obj_ntex"] = np.int32(len(texs))
    np.savez_compressed(os.path.join(HERE, "loader_ref.npz"), **out)


PARITY_KINDS = ("disney", "textured", "env")
# samples per pixel of the 32x32 statistics.  The environment scene stops at
# 128: further on, a direction whose z rounds beyond 1 makes asin return NaN,
# clamp passes it on and (int)NaN indexes the environment CDF far out of
# bounds (ImageBasedLighting.cuh:6-31,85-90), which crashes the host build.
PARITY_N32 = {"disney": 256, "textured": 256, "env": 128}


def make_parity_golden():
    """Reference renders of scenes.parity_scene's Disney, textured and
    environment scenes, and of the Cornell box at C1's size."""
    out = {}
    for kind in PARITY_KINDS:
        tris, mats, c, tex, env = scenes.parity_scene(kind)
        cam = orc.camera_setup(c["origin"], c["dist"], c["rot"], 48)
        frames, nrays = orc.ref_render(tris, mats, cam, 48, 48, 6, env=env, textures=tex)
        cam32 = orc.camera_setup(c["origin"], c["dist"], c["rot"], 32)
        many, _, gb = orc.ref_render(tris, mats, cam32, 32, 32, PARITY_N32[kind], env=env, textures=tex,
                                     gbuf=True)
        out[f"{kind}_frames"] = frames
        out[f"{kind}_camera"] = cam
        out[f"{kind}_rays"] = np.int64(nrays)
        out[f"{kind}_mean32"] = np.nanmean(many, axis=0)
        out[f"{kind}_var32"] = np.nanvar(many, axis=0, ddof=1)
        out[f"{kind}_camera32"] = cam32
        out[f"{kind}_gbuf32"] = gb
        out[f"{kind}_n32"] = np.int32(PARITY_N32[kind])
    np.savez_compressed(os.path.join(HERE, "parity_scenes_ref.npz"), **out)

    tris, mats, c = scenes.cornell_box()
    cam = orc.camera_setup(c["origin"], c["dist"], c["rot"], 256)
    sixteen, rays16 = orc.ref_render(tris, mats, cam, 256, 256, 16)
    many, _ = orc.ref_render(tris, mats, cam, 256, 256, 256)
    # every sample of 2048 seeded pixels (1..65535) over the 16 chained frames
    px = np.sort(np.random.default_rng(41).choice(np.arange(1, 256 * 256), 2048, replace=False)).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "c1_image_ref.npz"), camera=cam, spp=np.int32(16),
                        rays16=np.int64(rays16), mean16=np.nanmean(sixteen, axis=0).astype(np.float16),
                        std1=np.nanstd(many, axis=0, ddof=1).astype(np.float16), n_std=np.int32(256),
                        px_sample=px, samples16=sixteen[:, px])


def tonemap_inputs():
    """Inputs of the tone-map fixture: every step of the byte function (found
    with the oracle's restatement) +-8 ulp, special values and seeded random
    values, as (n, 3) float32."""
    import ctypes

    def byte(x):
        img = np.zeros((1, 4), np.float32)
        img[0, 0] = x
        return int(orc.tonemap(img)[0, 0])
    steps = []
    for k in range(1, 256):
        lo, hi = 0, 0x7f800000
        while lo < hi:
            mid = (lo + hi) // 2
            if byte(np.uint32(mid).view(np.float32)) >= k:
                hi = mid
            else:
                lo = mid + 1
        steps.append(lo)
    around = (np.array(steps, np.int64)[:, None] + np.arange(-8, 9)[None, :]).ravel()
    around = around[(around >= 0) & (around <= 0x7f800000)].astype(np.uint32).view(np.float32)
    rng = np.random.default_rng(12)
    special = np.array([0.0, -0.0, 1e-45, 1e-38, 1.0, 1.0000001, 2.0, 1e30, np.inf, -1e-30, -3.0, -np.inf, np.nan],
                       np.float32)
    vals = np.concatenate([around, special, rng.uniform(0, 1.3, 12000).astype(np.float32),
                           np.exp(rng.uniform(-20, 1, 4000)).astype(np.float32)])
    vals = np.concatenate([vals, np.zeros((-len(vals)) % 3, np.float32)])
    return vals.reshape(-1, 3)


def make_tonemap_golden():
    """save_png's bytes (FileIO/IO_save_png.cuh:34-56, the reference's own
    code, its PNG read back) for the inputs of tonemap_inputs()."""
    import ctypes
    import tempfile
    w, h = ctypes.c_int(), ctypes.c_int()
    orc.ref().ref_image_size(ctypes.byref(w), ctypes.byref(h))
    vals = tonemap_inputs()
    img = np.zeros((w.value * h.value, 4), np.float32)
    img[:len(vals), :3] = vals
    out = np.zeros((w.value * h.value, 4), np.uint8)
    with tempfile.TemporaryDirectory() as d:
        rc = orc.ref().ref_save_png_bytes(img.ctypes.data, os.path.join(d, "ref").encode(), out.ctypes.data)
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "tonemap_ref.npz"), inputs=vals, rgba=out[:len(vals)])


def main():
    orc.build(ref=True)
    assert orc.ref_available(), "oracle/_ref was not built (needs the reference checkout)"
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only == "loader":
        make_loader_golden()
        print("loader fixture written to", HERE)
        return
    if only == "parity":
        make_parity_golden()
        print("parity fixtures written to", HERE)
        return
    if only == "tonemap":
        make_tonemap_golden()
        print("tone-map fixture written to", HERE)
        return
    make_tonemap_golden()
    make_loader_golden()
    make_parity_golden()
    assert orc.ref_available(), "oracle/_ref was not built (needs the reference checkout)"

    # --- closest hits, Cornell box ---
    tris, mats, cam = scenes.cornell_box()
    rays = scenes.parity_rays(1 << 20, C1_LO, C1_HI, seed=1)
    ids, t, ok, nodes, _ = orc.ref_trace(tris, rays)
    np.savez_compressed(os.path.join(HERE, "c1_trace_ref.npz"), ids=ids.astype(np.int8), ok=ok,
                        t_head=t[:1 << 16], ray_digest=digest(rays), tri_digest=digest(tris),
                        ref_nodes=nodes)

    # --- closest hits, small displaced icospheres ---
    it, im, info = ico_scene()
    irays = scenes.parity_rays(1 << 16, info["lo"], info["hi"], seed=3)
    iids, itt, iok, inodes, _ = orc.ref_trace(it, irays)
    np.savez_compressed(os.path.join(HERE, "ico_trace_ref.npz"), ids=iids, t=itt, ok=iok,
                        ray_digest=digest(irays), tri_digest=digest(it), ref_nodes=inodes)

    # --- compat renders ---
    W = H = 48
    c = orc.camera_setup(cam["origin"], cam["dist"], cam["rot"], H)
    frames, nrays = orc.ref_render(tris, mats, c, W, H, 8)
    W2 = H2 = 32
    c2 = orc.camera_setup(cam["origin"], cam["dist"], cam["rot"], H2)
    many, nrays2 = orc.ref_render(tris, mats, c2, W2, H2, 256)
    np.savez_compressed(os.path.join(HERE, "c1_render_ref.npz"), frames=frames, width=W, height=H,
                        camera=c, rays=nrays, mean32=np.nanmean(many, axis=0),
                        var32=np.nanvar(many, axis=0, ddof=1), n32=256, camera32=c2,
                        rays32=nrays2)

    # --- Disney BRDF ---
    rng = scenes.CounterRng(11)
    mlist, wo_l, wi_l, n_l, b_l, p_l = [], [], [], [], [], []
    for k in range(8):
        m = structs.make_material(structs.DISNEY, tuple(rng.uniform(3, 0.05, 0.95)),
                                  metallic=float(rng.uniform(1)[0] < 0.3),
                                  roughness=float(rng.uniform(1, 0.05, 1.0)[0]), specular=0.5,
                                  clearcoat=float(rng.uniform(1)[0]),
                                  subsurface=float(rng.uniform(1)[0] * (k % 2)),
                                  sheen=float(rng.uniform(1)[0] * (k % 3 == 0)),
                                  sheenTint=0.5, specularTint=0.3,
                                  anisotropic=float(rng.uniform(1)[0] * (k % 2)),
                                  cloearcoatGloss=float(rng.uniform(1)[0]))
        n = 256
        nrm = np.zeros((n, 3), np.float32)
        nrm[:, 2] = 1.0
        def hemi(count):
            u1, u2 = rng.uniform(count), rng.uniform(count)
            z = u1
            r = np.sqrt(np.maximum(0, 1 - z * z))
            return np.stack([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2), z], 1).astype(np.float32)
        wo, wi = hemi(n), hemi(n)
        brdf = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        L = orc.ref()
        L.ref_disney_eval(m.ctypes.data, n, wo.ctypes.data, wi.ctypes.data, nrm.ctypes.data,
                          brdf.ctypes.data, pdf.ctypes.data)
        mlist.append(m)
        wo_l.append(wo); wi_l.append(wi); n_l.append(nrm); b_l.append(brdf); p_l.append(pdf)
    np.savez_compressed(os.path.join(HERE, "disney_ref.npz"), mats=np.stack(mlist), wo=np.stack(wo_l),
                        wi=np.stack(wi_l), n=np.stack(n_l), brdf=np.stack(b_l), pdf=np.stack(p_l))

    # --- camera ---
    poses = [((15.8153, 0.908405, 0.704717), 28.0, (103.426, 0.0, 95.9501)),
             ((0.0173, 5.0131, 13.6), 28.0, (0.0, 0.0, 0.0)),
             ((25.0, 0.0, 5.0), 28.0, (90.0, 0.0, 90.0)),
             ((-3.0, 7.0, 1.0), 35.0, (12.5, -40.0, 7.0))]
    cams = []
    for org, dist, rot in poses:
        out = np.zeros(18, np.float32)
        o = np.asarray(org, np.float32)
        orc.ref().ref_camera_setup(o.ctypes.data, dist, rot[0], rot[1], rot[2], out.ctypes.data)
        cams.append(out)
    np.savez_compressed(os.path.join(HERE, "camera_ref.npz"),
                        org=np.array([p[0] for p in poses], np.float32),
                        dist=np.array([p[1] for p in poses], np.float32),
                        rot=np.array([p[2] for p in poses], np.float32), cams=np.stack(cams))

    # --- CDFs ---
    lcdf = np.zeros(len(tris), np.float32)
    orc.ref().ref_light_cdf(tris.ctypes.data, len(tris), mats.ctypes.data, len(mats), lcdf.ctypes.data)
    env, _ = scenes.sky_environment(64, 32, sun_peak=100.0, seed=3)
    env = np.ascontiguousarray(env)
    ecdf = np.zeros(64 * 32, np.float32)
    orc.ref().ref_env_cdf(env.ctypes.data, 64, 32, 3, ecdf.ctypes.data)
    np.savez_compressed(os.path.join(HERE, "cdf_ref.npz"), light=lcdf, env=env, env_cdf=ecdf)
    # --- SVGF: ApplySVGF over a reference-rendered G-buffer, two frames ---
    SW, SH = 40, 24
    cs = orc.camera_setup(cam["origin"], cam["dist"], cam["rot"], SH)
    frames2, _, gb = orc.ref_render(tris, mats, cs, SW, SH, 2, gbuf=True)
    sz = orc.ref().ref_sizeof_svgfbuffer()
    npx = SW * SH
    def vec(img):
        v = np.zeros((npx, 4), np.float32)
        v[:, :3] = np.nan_to_num(img, nan=0.0)
        return v
    res0, res1 = vec(frames2[0]), vec(frames2[1])
    prev = np.zeros(npx * sz, np.uint8)
    cur = gb.copy()
    r0, f0 = res0.copy(), np.zeros_like(res0)
    assert orc.ref().ref_svgf(SW, SH, r0.ctypes.data, f0.ctypes.data, prev.ctypes.data, cur.ctypes.data, 0) == 0
    cur0 = cur.copy()
    prev1 = cur0.copy()
    cur1 = gb.copy()
    r1, f1 = res1.copy(), np.zeros_like(res1)
    assert orc.ref().ref_svgf(SW, SH, r1.ctypes.data, f1.ctypes.data, prev1.ctypes.data, cur1.ctypes.data, 1) == 0
    np.savez_compressed(os.path.join(HERE, "svgf_ref.npz"), width=SW, height=SH, gbuf=gb, res0=res0, res1=res1,
                        out_result0=r0, out_filtered0=f0, out_cur0=cur0, out_result1=r1, out_filtered1=f1,
                        out_cur1=cur1, record_size=sz)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
