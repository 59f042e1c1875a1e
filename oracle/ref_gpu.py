"""The reference's own CUDA renderer on the GPU: its render kernel
(render.cuh:21-49, with RayTrace and everything it calls), compiled for
sm_103a from the reference's headers, launched as main.cu:134-150 launches it,
timed with CUDA events.  TEST AND MEASUREMENT INFRASTRUCTURE: bench.py's
reference leg runs it as the GPU baseline of the Mrays/s metric; nothing in
the product imports it.

Files (git-ignored, made by build() where the reference checkout is; device
code and data only, so they load on the GPU machine's host architecture):
  _ref/kgkref_render.cubin        render() and ApplySVGF() (ref/ref_gpu.cu, oracle/Makefile)
  _ref/kgkref_render_count.cubin  the same, counting traversal calls
  _ref/c1_scene.bin               the Cornell box with the reference's BVH
                                  (construct_BVH) and light CDF (calculate_Lss)
  _ref/kgkref_render.txt          the two kernels' symbol names

Two guards keep the launch inside defined behaviour, both outside the
reference's code:
  * pixel positions start at 1 (LoopID 1, OneLoopSize 1): pixel 0's seed
    divides by zero (render.cuh:29).  The launch covers positions 1..W*H, the
    last one a row below the image, and the buffers hold W*H + 1 records.
  * a zeroed Triangle sits in front of the triangle array:
    NextEventEstimation_PathTracing.cuh:18-19 reads Objects[-1] when its ray
    misses (material 0 of the zeroed record ends that branch).
The two device free() calls of stack arrays (ConstructBVH.cuh:365-366) are
compiled out by ref/ref_gpu_shim.h.  Disney scenes are not run: sample_BXDF
reads an uninitialised array (sampling.cuh:15-19); the Cornell box is Lambert.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
CUBIN = os.path.join(REF, "kgkref_render.cubin")
CUBIN_COUNT = os.path.join(REF, "kgkref_render_count.cubin")
SCENE_C1 = os.path.join(REF, "c1_scene.bin")
NAME_FILE = os.path.join(REF, "kgkref_render.txt")

_u64 = ctypes.c_uint64
_vp = ctypes.c_void_p


def build():
    """Compiles the cubins and writes the Cornell-box scene file (needs the
    reference checkout and its host build, oracle/_ref/libkgkref.so)."""
    from oracle import orc
    subprocess.run(["make", "-s", "-C", HERE, "refgpu", "REF_DIR=" + orc.reference_dir()], check=True)
    from kagayaki_gb300 import scenes
    tris, mats, _ = scenes.cornell_box()
    rc = orc.ref().ref_export_scene(tris.ctypes.data, len(tris), mats.ctypes.data, len(mats), SCENE_C1.encode())
    if rc != 0:
        raise RuntimeError("ref_export_scene failed")
    out = subprocess.run(["nm", "-D", orc.REF_SO], capture_output=True, text=True, check=True).stdout
    syms = [ln.split()[-1] for ln in out.splitlines() if ln.split()]
    names = [n for n in syms if n.startswith("_Z6renderP6Camera")]
    svgf = [n for n in syms if n.startswith("_Z9ApplySVGF")]
    if len(names) != 1 or len(svgf) != 1:
        raise RuntimeError("render() / ApplySVGF() symbol not found in the reference's host build")
    with open(NAME_FILE, "w") as f:
        f.write(names[0] + "\n" + svgf[0] + "\n")


def available():
    """None when the files are here, else the reason they are not."""
    missing = [os.path.basename(p) for p in (CUBIN, CUBIN_COUNT, SCENE_C1, NAME_FILE) if not os.path.exists(p)]
    if missing:
        return "not built (needs the reference checkout): " + ", ".join(missing)
    return None


class _Cuda:
    """The few CUDA driver calls the launch needs."""

    def __init__(self):
        self.L = ctypes.CDLL("libcuda.so.1")
        self.ck(self.L.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self.ck(self.L.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        self.dev = dev
        self.ctx = _vp()
        self.ck(self.L.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self.ck(self.L.cuCtxPushCurrent_v2(self.ctx), "cuCtxPushCurrent")
        self.allocs = []

    def ck(self, r, what):
        if r != 0:
            s = ctypes.c_char_p()
            self.L.cuGetErrorName(r, ctypes.byref(s))
            raise RuntimeError(f"{what}: {s.value.decode() if s.value else r}")

    def alloc(self, nbytes, data=None):
        p = _u64()
        self.ck(self.L.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(int(nbytes), 16))), "cuMemAlloc")
        self.allocs.append(p)
        if data is not None:
            b = np.ascontiguousarray(data)
            self.ck(self.L.cuMemcpyHtoD_v2(p, b.ctypes.data_as(_vp), ctypes.c_size_t(b.nbytes)), "cuMemcpyHtoD")
        else:
            self.ck(self.L.cuMemsetD8_v2(p, 0, ctypes.c_size_t(max(int(nbytes), 16))), "cuMemsetD8")
        return p.value

    def get(self, dptr, nbytes, dtype):
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype)
        self.ck(self.L.cuMemcpyDtoH_v2(out.ctypes.data_as(_vp), _u64(dptr), ctypes.c_size_t(out.nbytes)),
                "cuMemcpyDtoH")
        return out

    def close(self):
        for p in self.allocs:
            self.L.cuMemFree_v2(p)
        self.allocs = []
        self.L.cuCtxPopCurrent_v2(ctypes.byref(_vp()))
        self.L.cuDevicePrimaryCtxRelease_v2(self.dev)


def _read_scene(path):
    raw = open(path, "rb").read()
    if raw[:8] != b"KGKREFS1":
        raise RuntimeError(f"{path}: not a scene file of ref_export_scene")
    n, nm, nn, nf, nl, nolight = np.frombuffer(raw, np.int32, 6, 8)
    o = 32
    tris = np.frombuffer(raw, np.uint8, n * 156, o); o += n * 156
    mats = np.frombuffer(raw, np.uint8, nm * 96, o); o += nm * 96
    nodes = np.frombuffer(raw, np.uint8, nn * 72, o).copy(); o += nn * 72
    faces = np.frombuffer(raw, np.int32, nf, o); o += nf * 4
    lss = np.frombuffer(raw, np.float32, nl, o)
    return dict(tris=tris, mats=mats, nodes=nodes, faces=faces, lss=lss, n=int(n), nolight=int(nolight))


class _Module:
    def __init__(self, cu, path, name):
        self.cu = cu
        self.mod = _vp()
        cu.ck(cu.L.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad " + os.path.basename(path))
        self.fn = _vp()
        cu.ck(cu.L.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, name.encode()), "cuModuleGetFunction")

    def glob(self, name):
        p, sz = _u64(), ctypes.c_size_t()
        self.cu.ck(self.cu.L.cuModuleGetGlobal_v2(ctypes.byref(p), ctypes.byref(sz), self.mod, name.encode()),
                   "cuModuleGetGlobal " + name)
        return p.value, sz.value

    def set(self, name, value, ctype):
        p, sz = self.glob(name)
        v = ctype(value)
        assert ctypes.sizeof(v) <= sz
        self.cu.ck(self.cu.L.cuMemcpyHtoD_v2(_u64(p), ctypes.byref(v), ctypes.c_size_t(ctypes.sizeof(v))),
                   "set " + name)

    def unload(self):
        self.cu.L.cuModuleUnload(self.mod)


def _setup(cu, mod, sc, cam, W, H):
    """Device buffers and module globals for one W x H render; returns the
    kernel's arguments (positions 1..W*H, see the module docstring)."""
    npx1 = W * H + 1
    d_tris = cu.alloc(156 * (sc["n"] + 1), np.concatenate([np.zeros(156, np.uint8), sc["tris"]]))
    d_objects = d_tris + 156                       # Objects[-1] is the zeroed guard record
    d_mats = cu.alloc(len(sc["mats"]), sc["mats"])
    d_faces = cu.alloc(4 * len(sc["faces"]), sc["faces"])
    nodes = sc["nodes"].reshape(-1, 72).copy()   # the file's offsets stay untouched for the next setup
    off = nodes[:, 56:64].copy().view(np.int64)[:, 0]
    if (off >= len(sc["faces"])).any():
        raise RuntimeError("scene file: face-list offset out of range")
    ptr = np.where(off >= 0, d_faces + 4 * np.maximum(off, 0), 0).astype(np.uint64)
    nodes[:, 56:64] = ptr.view(np.uint8).reshape(-1, 8)
    d_bvh = cu.alloc(nodes.nbytes, nodes)
    d_lss = cu.alloc(4 * len(sc["lss"]), sc["lss"])
    d_lssh = cu.alloc(16)                          # no environment: never read
    d_tex = cu.alloc(48)                           # a zeroed Texture (no textures, no environment)
    c = np.ascontiguousarray(cam, np.float32)
    d_cam = cu.alloc(72, c)
    d_prev = cu.alloc(72, c)
    d_result = cu.alloc(16 * npx1)
    d_svgf = cu.alloc(112 * npx1)
    mod.set("image_sizeX_device", W, ctypes.c_int)
    mod.set("image_sizeY_device", H, ctypes.c_int)
    mod.set("ObjectsNum", sc["n"], ctypes.c_int)
    mod.set("Light_strength_sum_size", len(sc["lss"]), ctypes.c_int)
    mod.set("Light_strength_sum_HDR_size", 0, ctypes.c_int)
    mod.set("Exists_NoLight", bool(sc["nolight"]), ctypes.c_bool)
    mod.set("Exists_NoHDR", True, ctypes.c_bool)
    seeds, sz = mod.glob("randSeeds")
    assert sz >= 8 * npx1
    cu.ck(cu.L.cuMemsetD8_v2(_u64(seeds), 0, ctypes.c_size_t(8 * npx1)), "zero randSeeds")
    args = [_u64(d_prev), _u64(d_cam), _u64(d_result), _u64(d_objects), _u64(d_mats), _u64(d_tex), _u64(d_bvh),
            _u64(d_lss), _u64(d_lssh), _u64(d_tex), _u64(d_svgf), ctypes.c_int(1), ctypes.c_int(1)]
    return args, d_result, seeds


def _launch(cu, mod, args, W, H, stream=None):
    params = (_vp * len(args))(*[ctypes.addressof(a) for a in args])
    grid = (W * H + 255) // 256
    cu.ck(cu.L.cuLaunchKernel(mod.fn, grid, 1, 1, 256, 1, 1, 0, stream, params, None), "cuLaunchKernel")


def render_c1(cam, W=256, H=256, spp=16, repeats=2, check_samples=None, cubin=None):
    """Times the reference's render over `spp` chained one-sample launches of
    the Cornell box (one C1 frame), `repeats` times after a warm-up frame.
    check_samples: (pixel ids, first-frame samples (n, 3)) of the reference's
    host build, compared with the first launch's output.  Returns a dict:
    ms per frame (CUDA events around each launch, summed), rays per frame
    (traversal calls counted by the counting build), the agreement of the
    first frame with the host build, the warm-up frame's per-pixel mean
    (W*H + 1, 3; position 0 unused), the kernel's registers and stack."""
    why = available()
    if why:
        raise RuntimeError(why)
    name = open(NAME_FILE).read().split()[0]
    cubin = cubin or CUBIN
    sc = _read_scene(SCENE_C1)
    cu = _Cuda()
    try:
        mod = _Module(cu, cubin, name)
        regs, lmem = ctypes.c_int(), ctypes.c_int()
        cu.ck(cu.L.cuFuncGetAttribute(ctypes.byref(regs), 4, mod.fn), "registers")   # NUM_REGS
        cu.ck(cu.L.cuFuncGetAttribute(ctypes.byref(lmem), 3, mod.fn), "local size")  # LOCAL_SIZE_BYTES
        # the per-thread stack the kernel's frame needs (main.cu:141 sets 32 KB,
        # below the 68 KB frame; the driver would grow it at launch)
        cu.ck(cu.L.cuCtxSetLimit(0, ctypes.c_size_t(((lmem.value + 1023) // 1024 + 1) * 1024)), "stack limit")
        args, d_result, seeds = _setup(cu, mod, sc, cam, W, H)
        ev = [_vp(), _vp()]
        for e in ev:
            cu.ck(cu.L.cuEventCreate(ctypes.byref(e), 0), "cuEventCreate")
        agree = None
        # warm-up frame: its per-pixel mean, and the check of its first launch
        mean = np.zeros((W * H + 1, 3), np.float64)
        for f in range(spp):
            _launch(cu, mod, args, W, H)
            cu.ck(cu.L.cuCtxSynchronize(), "render (warm-up)")
            res = cu.get(d_result, 16 * (W * H + 1), np.float32).reshape(-1, 4)[:, :3]
            mean += res
            if f == 0 and check_samples is not None:
                px, ref = check_samples
                rel = np.abs(res[px] - ref) / np.maximum(np.abs(ref), 1e-4)
                agree = float((rel.max(-1) <= 1e-3).mean())
        mean /= spp
        ms = []
        for r in range(repeats):
            cu.ck(cu.L.cuMemsetD8_v2(_u64(seeds), 0, ctypes.c_size_t(8 * (W * H + 1))), "zero randSeeds")
            tot = 0.0
            for f in range(spp):
                cu.ck(cu.L.cuEventRecord(ev[0], None), "cuEventRecord")
                _launch(cu, mod, args, W, H)
                cu.ck(cu.L.cuEventRecord(ev[1], None), "cuEventRecord")
                cu.ck(cu.L.cuEventSynchronize(ev[1]), "render")
                t = ctypes.c_float()
                cu.ck(cu.L.cuEventElapsedTime_v2(ctypes.byref(t), ev[0], ev[1]), "cuEventElapsedTime")
                tot += t.value
            ms.append(tot)
        mod.unload()
        # ray count: the same frame with the counting build
        cm = _Module(cu, CUBIN_COUNT, name)
        args_c, _, _ = _setup(cu, cm, sc, cam, W, H)
        cnt, _ = cm.glob("kgk_ref_traversals")
        cu.ck(cu.L.cuMemsetD8_v2(_u64(cnt), 0, ctypes.c_size_t(8)), "zero counter")
        for f in range(spp):
            _launch(cu, cm, args_c, W, H)
        cu.ck(cu.L.cuCtxSynchronize(), "render (counting build)")
        rays = int(cu.get(cnt, 8, np.uint64)[0])
        cm.unload()
        for e in ev:
            cu.L.cuEventDestroy_v2(e)
    finally:
        cu.close()
    best = min(ms)
    return dict(ms_per_frame=best, ms_all=ms, rays_per_frame=rays, mrays=rays / (best / 1e3) / 1e6,
                first_launch_agreement=agree, mean=mean, registers=regs.value, stack_bytes=lmem.value,
                launches_per_frame=spp, pixels=W * H)


# struct_SVGFBuffers.cuh:7-23 `SVGFBuffer` (112 B)
_SVGF_REC = np.dtype({
    "names": ["Albedo", "Emission", "Normal", "ColorHistory", "ObjectID", "MaterialID", "PosLastFrameI",
              "PosLastFrameF", "sampleNum", "MomentOne", "MomentTwo", "Variance", "Depth",
              "willApplyATrousFilter", "willApplyTemporalAccumulation"],
    "formats": [("<f4", (4,)), ("<f4", (4,)), ("<f4", (4,)), ("<f4", (4,)), "<i4", "<i4", ("<i4", (2,)),
                ("<f4", (2,)), "<i4", "<f4", "<f4", "<f4", "<f4", "u1", "u1"],
    "offsets": [0, 16, 32, 48, 64, 68, 72, 80, 88, 92, 96, 100, 104, 108, 109],
    "itemsize": 112})


def cornell_svgf_inputs(W, H):
    """One frame of ApplySVGF input for the Cornell box at W x H, made on the
    CPU by the oracle: the compat estimator's one-sample frame
    (orc.render_compat) and the SVGFBuffer records render() fills at the
    primary hits (RayTrace.cuh:66-82): albedo (sINF when below 1e-5),
    emission, the normal turned against the ray, face and material ids, hit
    distance, and the reprojection left at (-1, -1) as the reference leaves
    it (struct_Camera.cuh:109-110); pixels that miss keep SVGFBuffer::init's
    values.  Returns (result (W*H, 4) float32, records (W*H * 112,) uint8)."""
    from kagayaki_gb300 import scenes
    from oracle import orc
    tris, mats, c = scenes.cornell_box()
    cam = orc.camera_setup(c["origin"], c["dist"], c["rot"], H)
    org, cdir, dist, sx, sy, psz = cam[0:3], cam[4:7], cam[8], cam[9:12], cam[13:16], cam[17]
    Y, X = np.divmod(np.arange(W * H, dtype=np.int64), W)
    d = (cdir[None, :] * dist + sx[None, :] * ((X - W / 2.0) * psz)[:, None].astype(np.float32) +
         sy[None, :] * ((H / 2.0 - Y) * psz)[:, None].astype(np.float32)).astype(np.float32)
    d /= np.sqrt((d * d).sum(1, keepdims=True))
    rays = np.zeros(W * H, np.dtype([("dir", "<f4", (4,)), ("org", "<f4", (4,)), ("_dummy", "<f8")], align=True))
    rays["dir"][:, :3] = d
    rays["org"][:, :3] = org
    ids, t = orc.closest_brute(tris, rays)
    rec = np.zeros(W * H, _SVGF_REC)
    rec["ObjectID"] = -1
    rec["MaterialID"] = -1
    rec["PosLastFrameI"] = -1
    rec["PosLastFrameF"] = -1.0
    rec["MomentOne"] = -1.0
    rec["MomentTwo"] = -1.0
    rec["willApplyATrousFilter"] = 1
    hit = ids >= 0
    h = ids[hit]
    v = tris["verts"][h][:, :, :3].astype(np.float64)      # (k, 3 vertices, xyz)
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(((n * d[hit]).sum(1) > 0)[:, None], -n, n)
    mid = tris["material_id"][h]
    dif = mats["diffuse"][mid][:, :3].astype(np.float32)
    dif = np.where((np.linalg.norm(dif, axis=1) < 1e-5)[:, None], np.float32(1e-4), dif)
    rec["Albedo"][hit, :3] = dif
    rec["Emission"][hit, :3] = mats["emission"][mid][:, :3]
    rec["Normal"][hit, :3] = n
    rec["ObjectID"][hit] = h
    rec["MaterialID"][hit] = mid
    rec["Depth"][hit] = t[hit]
    frames, _ = orc.render_compat(tris, mats, cam, W, H, 1)
    res = np.zeros((W * H, 4), np.float32)
    res[:, :3] = np.nan_to_num(frames[0], nan=0.0)
    return res, rec.view(np.uint8)


def apply_svgf(frames, W, H, repeats=3):
    """The reference's ApplySVGF (SVGF.cuh:495-522) on the GPU, launched as
    main.cu:160-166 launches it (W*H/256 blocks of 256 threads, LoopID 0)
    over a chain of frames: `frames` is a list of (result, records) pairs -
    the (W*H, 4) float32 radiance and the W*H 112-byte SVGFBuffer records of
    one frame - and, as main.cu:182 does, each frame's filtered records
    become the next frame's previous ones.  The kernel uses __syncthreads as
    if it were a grid barrier, so blocks race on their neighbours' records:
    the run ends (every barrier sits at function scope, every neighbour read
    is bounds-checked), its output is not the filter's.  Returns the CUDA-event
    time of each launch of the last repeat of the chain (ms) and the last
    frame's filtered output (W*H, 4)."""
    why = available()
    if why:
        raise RuntimeError(why)
    npx = W * H
    if npx % 256 or npx > 1920 * 1920:
        raise ValueError("ApplySVGF needs W*H a multiple of 256 and at most 1920*1920 (its moment maps)")
    name = open(NAME_FILE).read().split()[1]
    cu = _Cuda()
    try:
        mod = _Module(cu, CUBIN, name)
        mod.set("image_sizeX_device", W, ctypes.c_int)
        mod.set("image_sizeY_device", H, ctypes.c_int)
        d_res = cu.alloc(16 * npx)
        d_filt = cu.alloc(16 * npx)
        d_prev = cu.alloc(112 * npx)
        d_cur = cu.alloc(112 * npx)
        ev = [_vp(), _vp()]
        for e in ev:
            cu.ck(cu.L.cuEventCreate(ctypes.byref(e), 0), "cuEventCreate")
        ms = []
        for r in range(repeats):
            ms = []
            for f, (res, recs) in enumerate(frames):
                for d, a in ((d_res, res), (d_cur, recs)):
                    b = np.ascontiguousarray(a)
                    cu.ck(cu.L.cuMemcpyHtoD_v2(_u64(d), b.ctypes.data_as(_vp), ctypes.c_size_t(b.nbytes)), "upload")
                args = [_u64(d_res), _u64(d_filt), _u64(d_prev), _u64(d_cur), ctypes.c_int(0), ctypes.c_int(npx),
                        ctypes.c_int(f)]
                params = (_vp * len(args))(*[ctypes.addressof(a) for a in args])
                cu.ck(cu.L.cuEventRecord(ev[0], None), "cuEventRecord")
                cu.ck(cu.L.cuLaunchKernel(mod.fn, npx // 256, 1, 1, 256, 1, 1, 0, None, params, None), "ApplySVGF")
                cu.ck(cu.L.cuEventRecord(ev[1], None), "cuEventRecord")
                cu.ck(cu.L.cuEventSynchronize(ev[1]), "ApplySVGF")
                t = ctypes.c_float()
                cu.ck(cu.L.cuEventElapsedTime_v2(ctypes.byref(t), ev[0], ev[1]), "cuEventElapsedTime")
                ms.append(t.value)
                cu.ck(cu.L.cuMemcpyDtoD_v2(_u64(d_prev), _u64(d_cur), ctypes.c_size_t(112 * npx)), "prev = cur")
        filt = cu.get(d_filt, 16 * npx, np.float32).reshape(-1, 4)
        for e in ev:
            cu.L.cuEventDestroy_v2(e)
        mod.unload()
    finally:
        cu.close()
    return ms, filt


if __name__ == "__main__":
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    if "build" in sys.argv:
        build()
        print("built", CUBIN, SCENE_C1)
