"""Host-side mirror of the reference's render interface over the C ABI.

    scene = Scene(triangles, materials, env=None)   # render_prepare + upload
    scene.build_bvh()                                # construct_BVH
    ids, t = scene.trace_closest(rays)               # willIntersectWithTriangle_nonRecursive
    cam = camera_setup(origin, dist, rot, height)    # Camera_SetUpCamera
    img = scene.render(cam, cfg)                     # render<<<>>>
    save_png(img, path)                              # save_png

Arrays are numpy structured arrays with the reference layouts
(kagayaki_gb300.structs).  Errors raise KgkError with the library's message.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import KgkError, check, lib
from .structs import (MATERIAL, MATERIALS_PBR, MATERIALS_REFERENCE, RAY, SVGF_BUFFER, TRIANGLE, KgkBvhInfo,  # noqa: F401
                      KgkCamera, KgkHostScene, KgkLoadOptions, KgkNrcConfig, KgkRenderConfig, KgkStats,
                      KgkSvgfConfig, KgkTexture, KgkTextureRGBA8, KgkVec)

ESTIMATOR_COMPAT = 0
ESTIMATOR_UNBIASED = 1


def _p(a):
    """A numpy array's data pointer; an int is taken as a (device) pointer."""
    if a is None:
        return None
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    return ctypes.c_void_p(a.ctypes.data)


def _as(a, dtype):
    a = np.ascontiguousarray(a)
    if a.dtype != dtype:
        a = a.astype(dtype)
    return a


def stats_dict(s):
    return {k: getattr(s, k) for k, _ in KgkStats._fields_}


class Scene:
    """A device-resident scene (owns a kgk_scene handle)."""

    def __init__(self, triangles, materials, textures=None, env=None):
        self._h = ctypes.c_void_p()
        tris = _as(triangles, TRIANGLE)
        mats = _as(materials, MATERIAL)
        self._keep = []
        tex_arr = None
        ntex = 0
        if textures:
            tex_arr = (KgkTexture * len(textures))()
            for i, t in enumerate(textures):
                t = np.ascontiguousarray(t, np.float32)
                self._keep.append(t)
                tex_arr[i].pixels = t.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
                tex_arr[i].height, tex_arr[i].width, tex_arr[i].bpp = t.shape
            ntex = len(textures)
        hdr = None
        if env is not None:
            e = np.ascontiguousarray(env, np.float32)
            self._keep.append(e)
            hdr = KgkTexture(e.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), e.shape[1], e.shape[0],
                             e.shape[2])
        check(lib().kgk_scene_create(_p(tris), len(tris), _p(mats), len(mats),
                                     ctypes.cast(tex_arr, ctypes.c_void_p) if tex_arr else None, ntex,
                                     ctypes.byref(hdr) if hdr is not None else None,
                                     ctypes.byref(self._h)))
        self.n_triangles = len(tris)
        self.bvh = None

    @classmethod
    def from_obj(cls, obj_path, hdr_path=None, materials=MATERIALS_REFERENCE, threads=0):
        """kgk_scene_load_obj_ex: an OBJ scene (and environment) straight to the device."""
        self = cls.__new__(cls)
        self._h = ctypes.c_void_p()
        self._keep = []
        opt = _load_options(materials, threads)
        check(lib().kgk_scene_load_obj_ex(str(obj_path).encode(), str(hdr_path).encode() if hdr_path else None,
                                          ctypes.byref(opt), ctypes.byref(self._h)))
        self.n_triangles = None
        self.bvh = None
        return self

    def close(self):
        if self._h:
            lib().kgk_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def build_bvh(self):
        info = KgkBvhInfo()
        check(lib().kgk_build_bvh(self._h, ctypes.byref(info)))
        self.bvh = {k: getattr(info, k) for k, _ in KgkBvhInfo._fields_}
        return self.bvh

    def validate_bvh(self):
        check(lib().kgk_bvh_validate(self._h))

    def trace_closest(self, rays, with_stats=False):
        rays = _as(rays, RAY)
        n = len(rays)
        ids = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        st = KgkStats()
        check(lib().kgk_trace_closest(self._h, _p(rays), n, _p(ids), _p(t), ctypes.byref(st)))
        return (ids, t, stats_dict(st)) if with_stats else (ids, t)

    def trace_any(self, rays, t_max=None):
        rays = _as(rays, RAY)
        n = len(rays)
        occ = np.empty(n, np.uint8)
        tm = _as(t_max, np.float32) if t_max is not None else None
        check(lib().kgk_trace_any(self._h, _p(rays), _p(tm), n, _p(occ), None))
        return occ

    def render(self, cam, width, height, spp=1, max_depth=0, rr_start_depth=3,
               estimator=ESTIMATOR_COMPAT, seed=1, frame_index=0, accumulate=False,
               count_work=False, write_gbuffer=False, use_cache=False, wave_paths=0, prev_cam=None,
               out=None, profile_stages=False, texture_filter=0, keep_on_device=False):
        """kgk_render.  out: a (height, width, 4) float32 host array (allocated
        when None) or a device pointer (int); keep_on_device: the frame stays
        in the scene for svgf_output(noisy=None) and None is returned for it."""
        cfg = KgkRenderConfig(width=width, height=height, spp=spp, max_depth=max_depth,
                              rr_start_depth=rr_start_depth, estimator=estimator, seed=seed,
                              frame_index=frame_index, accumulate=int(accumulate),
                              wave_paths=wave_paths, count_work=int(count_work),
                              write_gbuffer=int(write_gbuffer), use_cache=int(use_cache),
                              profile_stages=int(profile_stages), texture_filter=int(texture_filter))
        if keep_on_device:
            out = None
        elif out is None:
            out = np.empty((height, width, 4), np.float32)
        st = KgkStats()
        check(lib().kgk_render(self._h, ctypes.byref(cam),
                               ctypes.byref(prev_cam) if prev_cam is not None else None,
                               ctypes.byref(cfg), _p(out), ctypes.byref(st)))
        return out, stats_dict(st)

    def gbuffer_records(self, width, height):
        """kgk_gbuffer_records: the last write_gbuffer frame as the reference's
        SVGFBuffer records, a (height * width,) SVGF_BUFFER array."""
        out = np.zeros(width * height, SVGF_BUFFER)
        check(lib().kgk_gbuffer_records(self._h, _p(out)))
        return out

    def svgf_output(self, cfg, noisy=None, filtered=None, rgba8=None, async_=False):
        """kgk_svgf_output: noisy None = the frame kept by render(keep_on_device=True);
        filtered / rgba8: host arrays, device pointers (int) or None."""
        check(lib().kgk_svgf_output(self._h, ctypes.byref(cfg), _p(noisy), _p(filtered), _p(rgba8),
                                    int(async_)))

    def sync(self):
        """kgk_scene_sync: waits for queued work and output copies."""
        check(lib().kgk_scene_sync(self._h))

    def set_textures_rgba8(self, textures):
        """Replaces the scene's textures with RGBA8 ones: (height, width, 4) uint8 arrays."""
        arr = (KgkTextureRGBA8 * max(len(textures), 1))()
        keep = []
        for i, t in enumerate(textures):
            t = np.ascontiguousarray(t, np.uint8)
            assert t.ndim == 3 and t.shape[2] == 4
            keep.append(t)
            arr[i].pixels = t.ctypes.data
            arr[i].height, arr[i].width = t.shape[:2]
        check(lib().kgk_scene_set_textures_rgba8(self._h, ctypes.cast(arr, ctypes.c_void_p), len(textures)))

    def cache_init(self, **cfg):
        """(Re)initialises the learned radiance cache used by
        render(use_cache=True); keyword arguments are kgk_nrc_config fields
        (0 / absent = the library default)."""
        c = KgkNrcConfig(**cfg)
        check(lib().kgk_nrc_init(self._h, ctypes.byref(c)))

    def accum_reset(self, width, height):
        check(lib().kgk_accum_reset(self._h, width, height))

    def accum_read(self, width, height):
        mean = np.empty((height, width, 3), np.float64)
        var = np.empty((height, width, 3), np.float64)
        n = ctypes.c_uint64()
        check(lib().kgk_accum_read(self._h, _p(mean), _p(var), ctypes.byref(n)))
        return mean, var, n.value


class PinnedBuffer:
    """Page-locked host memory from kgk_host_alloc, viewed as a numpy array."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        self._ptr = ctypes.c_void_p()
        check(lib().kgk_host_alloc(n, ctypes.byref(self._ptr)))
        raw = (ctypes.c_uint8 * n).from_address(self._ptr.value)
        self.array = np.frombuffer(raw, np.uint8).view(dtype).reshape(shape)

    def free(self):
        if self._ptr:
            self.array = None
            lib().kgk_host_free(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _texture_array(t):
    n = t.width * t.height * t.bpp
    if not t.pixels or n == 0:
        return None
    return np.ctypeslib.as_array(ctypes.cast(t.pixels, ctypes.POINTER(ctypes.c_float)), (n,)).copy().reshape(
        t.height, t.width, t.bpp)


def load_image(path):
    """stbi_loadf semantics (FileIO/IO_load_images.cuh:10): float pixels
    (height, width, channels)."""
    t = KgkTexture()
    check(lib().kgk_load_image(str(path).encode(), ctypes.byref(t)))
    try:
        return _texture_array(t)
    finally:
        lib().kgk_image_free(ctypes.byref(t))


def _host_array(ptr, n, dtype):
    """A numpy copy of n records of dtype at the library-owned host pointer."""
    raw = (ctypes.c_uint8 * (n * dtype.itemsize)).from_address(ptr)
    return np.frombuffer(raw, np.uint8).view(dtype).copy()


def _load_options(materials, threads):
    opt = KgkLoadOptions()
    opt.material_model = int(materials)
    opt.threads = int(threads)
    return opt


def load_obj(obj_path, hdr_path=None, materials=MATERIALS_REFERENCE, threads=0):
    """load_object + load_Textures + load_HDR (FileIO/IO_load_WavefrontObj.cuh:10-127,
    FileIO/IO_load_images.cuh:9-29), through kgk_load_obj_ex.  materials:
    MATERIALS_REFERENCE (the reference's Lambert conversion) or MATERIALS_PBR
    (Disney from the MTL PBR keys); threads: 0 = all host threads.  Returns
    (triangles, materials, [texture arrays], environment array or None)."""
    hs = KgkHostScene()
    opt = _load_options(materials, threads)
    check(lib().kgk_load_obj_ex(str(obj_path).encode(), str(hdr_path).encode() if hdr_path else None,
                                ctypes.byref(opt), ctypes.byref(hs)))
    try:
        tris = _host_array(hs.triangles, hs.n_triangles, TRIANGLE)
        mats = _host_array(hs.materials, hs.n_materials, MATERIAL)
        texs = [_texture_array(hs.textures[i]) for i in range(hs.n_textures)]
        env = _texture_array(hs.hdr)
        return tris, mats, texs, env
    finally:
        lib().kgk_host_scene_free(ctypes.byref(hs))


def camera_setup(origin, dist, rot, image_height):
    """Camera_SetUpCamera (struct_Camera.cuh:27-35), PixelSize = 36/height."""
    cam = KgkCamera()
    o = KgkVec(float(origin[0]), float(origin[1]), float(origin[2]), 0.0)
    check(lib().kgk_camera_setup(o, float(dist), float(rot[0]), float(rot[1]), float(rot[2]),
                                 int(image_height), ctypes.byref(cam)))
    return cam


def camera_array(cam):
    return np.frombuffer(bytes(cam), dtype=np.float32).copy()


def tonemap(img):
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape[:2]
    out = np.empty((h, w, 4), np.uint8)
    check(lib().kgk_tonemap_rgba8(_p(img), w, h, _p(out)))
    return out


def save_exr(img, path, half=False):
    """kgk_save_exr: the linear RGB of a (height, width, 4) float32 host image
    as an uncompressed OpenEXR file, FP32 or (half=True) FP16 channels."""
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape[:2]
    check(lib().kgk_save_exr(_p(img), w, h, int(bool(half)), str(path).encode()))


def save_png(img, path):
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape[:2]
    check(lib().kgk_save_png(_p(img), w, h, path.encode()))
