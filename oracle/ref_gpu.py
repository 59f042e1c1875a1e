"""The reference's own CUDA renderer on the GPU: its render kernel
(render.cuh:21-49, with RayTrace and everything it calls), compiled for
sm_103a from the reference's headers, launched as main.cu:134-150 launches it,
timed with CUDA events.  TEST AND MEASUREMENT INFRASTRUCTURE: bench.py's
reference leg runs it as the GPU baseline of the Mrays/s metric; nothing in
the product imports it.

Files (git-ignored, made by build() where the reference checkout is; device
code and data only, so they load on the GPU machine's host architecture):
  _ref/kgkref_render.cubin        render() (ref/ref_gpu.cu, oracle/Makefile)
  _ref/kgkref_render_count.cubin  the same, counting traversal calls
  _ref/c1_scene.bin               the Cornell box with the reference's BVH
                                  (construct_BVH) and light CDF (calculate_Lss)
  _ref/kgkref_render.txt          the kernel's symbol name

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
    names = [ln.split()[-1] for ln in out.splitlines() if ln.split()[-1].startswith("_Z6renderP6Camera")]
    if len(names) != 1:
        raise RuntimeError("render() symbol not found in the reference's host build")
    with open(NAME_FILE, "w") as f:
        f.write(names[0] + "\n")


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
    name = open(NAME_FILE).read().strip()
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


if __name__ == "__main__":
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    if "build" in sys.argv:
        build()
        print("built", CUBIN, SCENE_C1)
