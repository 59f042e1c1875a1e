"""Python bindings of the CPU oracle (orc.c) and of the reference's own code
built for the host (oracle/_ref).  TEST INFRASTRUCTURE ONLY: imported by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
product package.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_SO = os.path.join(HERE, "_build", "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libkgkref.so")


def reference_dir():
    """The reference checkout the `ref` build reads: $KGK_REFERENCE_DIR, else a
    directory named `reference` beside this repository."""
    d = os.environ.get("KGK_REFERENCE_DIR")
    if d:
        return d
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int
_f32 = ctypes.c_float


# The reference's vendored stb_image_write.h includes the C headers by
# Windows paths relative to itself (external_lib/stb/stb_image_write.h:154,
# 211-217, 244).  The `ref` build satisfies them with forwarding headers at
# the same relative paths below an include directory six levels deep inside
# oracle/_ref, so FileIO/IO_save_png.cuh compiles unchanged.
WIN_HEADERS = {
    "Program Files (x86)/Windows Kits/10/Include/10.0.22621.0/ucrt/stdlib.h": "stdlib.h",
    "Program Files (x86)/Windows Kits/10/Include/10.0.22621.0/ucrt/stdio.h": "stdio.h",
    "Program Files (x86)/Windows Kits/10/Include/10.0.22621.0/ucrt/string.h": "string.h",
    "Program Files (x86)/Windows Kits/10/Include/10.0.22621.0/ucrt/math.h": "math.h",
    "Program Files (x86)/Windows Kits/10/Include/10.0.22621.0/ucrt/assert.h": "assert.h",
    "Program Files (x86)/Microsoft Visual Studio/2019/Community/VC/Tools/MSVC/14.29.30133/include/stdarg.h":
        "stdarg.h",
}


def _win_include_shims():
    """Writes the forwarding headers; returns the include directory."""
    root = os.path.join(HERE, "_ref", "winshim")
    inc = os.path.join(root, "i1", "i2", "i3", "i4", "i5", "i6")
    os.makedirs(inc, exist_ok=True)
    for rel, std in WIN_HEADERS.items():
        path = os.path.join(root, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(f"#include <{std}>\n")
    return inc


def build(ref=False):
    """Builds liborc.so (and the reference library when ref=True; the caller
    checks that the reference checkout exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "orc"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF_DIR=" + reference_dir(),
                        "WINSHIM=" + _win_include_shims()], check=True)


def _ptr(a):
    return a.ctypes.data_as(_vp) if a is not None else None


_orc = None


def orc():
    global _orc
    if _orc is None:
        if not os.path.exists(ORC_SO):
            build()
        L = ctypes.CDLL(ORC_SO)
        L.orc_intersect_ref.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.orc_intersect_ref.restype = _i32
        L.orc_closest_brute.argtypes = [_vp, _i64, _vp, _i64, _vp, _vp, _i32]
        L.orc_classify.argtypes = [_vp, _i64, _vp, _i64, _vp, _vp, _vp, _i32]
        L.orc_bvh_build.argtypes = [_vp, _i64]
        L.orc_bvh_build.restype = _vp
        L.orc_bvh_closest.argtypes = [_vp, _vp, _i64, _vp, _vp, _i32]
        L.orc_bvh_free.argtypes = [_vp]
        L.orc_xorshift.argtypes = [ctypes.c_uint64]
        L.orc_xorshift.restype = ctypes.c_uint64
        L.orc_camera_setup.argtypes = [_vp, _f32, _f32, _f32, _f32, _i32, _vp]
        L.orc_tonemap_rgba8.argtypes = [_vp, _i64, _vp]
        L.orc_light_cdf.argtypes = [_vp, _i64, _vp, _vp]
        L.orc_env_cdf.argtypes = [_vp, _i32, _i32, _i32, _vp]
        L.orc_render_compat.argtypes = [_vp, _i64, _vp, _i64, _vp, _i32, _vp, _i32, _i32, _i32,
                                        _vp, _i32, _i32, _i32, _i32, _vp]
        L.orc_render_compat.restype = _i64
        L.orc_set_point_arg_order.argtypes = [_i32]
        L.orc_disney_eval.argtypes = [_vp, _i32, _vp, _vp, _vp, _vp, _vp]
        L.orc_render_compat_px.argtypes = [_vp, _i64, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32, _i32,
                                           _vp, _i64, _i32, _vp]
        L.orc_render_compat_px.restype = _i64
        L.orc_svgf_compat.argtypes = [_i32, _i32, _vp, _vp, _vp, _vp, _i32]
        _orc = L
    return _orc


def nthreads():
    return max(1, os.cpu_count() or 1)


def closest_brute(tris, rays):
    n = len(rays)
    ids = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    orc().orc_closest_brute(_ptr(tris), len(tris), _ptr(rays), n, _ptr(ids), _ptr(t), nthreads())
    return ids, t


def classify(tris, rays, ids, t):
    flags = np.empty(len(rays), np.uint8)
    orc().orc_classify(_ptr(tris), len(tris), _ptr(rays), len(rays), _ptr(ids), _ptr(t),
                       _ptr(flags), nthreads())
    return flags


def exact_hit(tri, ray):
    """The ray/triangle intersection of Triangle::intersectTest
    (struct_Triangle.cuh:41-57: Cramer's rule, hit when u, v >= 0, u + v <= 1
    and t >= 1e-5) in exact rational arithmetic on the float32 inputs:
    (hit, t, u, v) with t, u, v as Fractions (None when the ray is parallel).
    Settles which answer is geometrically right where the float expressions
    disagree near an edge."""
    from fractions import Fraction as Fr
    f = [Fr(float(c)) for c in np.asarray(tri["verts"][:3, :3], np.float64).ravel()]
    v0, v1, v2 = f[0:3], f[3:6], f[6:9]
    o = [Fr(float(c)) for c in ray["org"][:3]]
    d = [Fr(float(c)) for c in ray["dir"][:3]]

    def sub(a, b):
        return [a[0] - b[0], a[1] - b[1], a[2] - b[2]]

    def cross(a, b):
        return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]

    def dot(a, b):
        return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
    e1, e2, so = sub(v1, v0), sub(v2, v0), sub(o, v0)
    de2 = cross(d, e2)
    det = dot(de2, e1)
    if det == 0:
        return False, None, None, None
    se1 = cross(so, e1)
    t, u, v = dot(se1, e2) / det, dot(de2, so) / det, dot(se1, d) / det
    return bool(u >= 0 and v >= 0 and u + v <= 1 and t >= Fr(1, 100000)), t, u, v


def exact_winner(tris, ray, candidates):
    """The candidate triangle (-1: none) the ray hits first in exact
    arithmetic, and whether another candidate ties it exactly."""
    best, bt, tie = -1, None, False
    for k in candidates:
        if k < 0:
            continue
        hit, t, _, _ = exact_hit(tris[k], ray)
        if not hit:
            continue
        if bt is None or t < bt:
            best, bt, tie = int(k), t, False
        elif t == bt:
            tie = True
    return best, tie


def closest_bvh(tris, rays):
    L = orc()
    b = L.orc_bvh_build(_ptr(tris), len(tris))
    try:
        n = len(rays)
        ids = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        L.orc_bvh_closest(b, _ptr(rays), n, _ptr(ids), _ptr(t), nthreads())
    finally:
        L.orc_bvh_free(b)
    return ids, t


def disney_eval(mat, wo, wi, nrm):
    n = len(wo)
    brdf = np.empty((n, 3), np.float32)
    pdf = np.empty(n, np.float32)
    wo, wi, nrm = (np.ascontiguousarray(a, np.float32) for a in (wo, wi, nrm))
    orc().orc_disney_eval(_ptr(np.ascontiguousarray(mat)), n, _ptr(wo), _ptr(wi), _ptr(nrm),
                          _ptr(brdf), _ptr(pdf))
    return brdf, pdf


def camera_setup(org, dist, rot, image_height):
    out = np.zeros(18, np.float32)
    o = np.asarray(org, np.float32)
    orc().orc_camera_setup(_ptr(o), dist, rot[0], rot[1], rot[2], image_height, _ptr(out))
    return out


def tonemap(img_vec4):
    img = np.ascontiguousarray(img_vec4, np.float32).reshape(-1, 4)
    out = np.empty((len(img), 4), np.uint8)
    orc().orc_tonemap_rgba8(_ptr(img), len(img), _ptr(out))
    return out


def light_cdf(tris, mats):
    out = np.empty(len(tris), np.float32)
    orc().orc_light_cdf(_ptr(tris), len(tris), _ptr(mats), _ptr(out))
    return out


def env_cdf(env):
    env = np.ascontiguousarray(env, np.float32)
    h, w, bpp = env.shape
    out = np.empty(w * h, np.float32)
    orc().orc_env_cdf(_ptr(env), w, h, bpp, _ptr(out))
    return out


def _texture_table(textures):
    """Reference `Texture` records (pixels, width, height, bpp) over a list of
    (h, w, bpp) float32 arrays; returns (table or None, count, arrays kept)."""
    if not textures:
        return None, 0, []
    from kagayaki_gb300.structs import KgkTexture
    keep = [np.ascontiguousarray(t, np.float32) for t in textures]
    table = (KgkTexture * len(keep))()
    for i, t in enumerate(keep):
        table[i].pixels = t.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        table[i].height, table[i].width, table[i].bpp = t.shape
    return table, len(keep), keep


def render_compat(tris, mats, cam, width, height, frames, env=None, threads=None, textures=None):
    """Returns (frames, height*width, 3) float32 samples and the traversal
    count.  Pixel 0 is NaN (the reference's seed divides by zero there).
    textures: list of (h, w, bpp) float32 arrays, indexed by the materials'
    TEXTURE_BASECOLOR_ID."""
    out = np.empty((frames, width * height, 3), np.float32)
    env_p, hw, hh, hb = None, 0, 0, 0
    if env is not None:
        env = np.ascontiguousarray(env, np.float32)
        hh, hw, hb = env.shape
        env_p = _ptr(env)
    cam = np.ascontiguousarray(cam, np.float32)
    table, ntex, _keep = _texture_table(textures)
    n = orc().orc_render_compat(_ptr(tris), len(tris), _ptr(mats), len(mats),
                                ctypes.cast(table, _vp) if table is not None else None, ntex, env_p, hw,
                                hh, hb, _ptr(cam), width, height, frames,
                                threads or nthreads(), _ptr(out))
    return out, n


def svgf_compat(width, height, result, filtered, prev, cur, frame):
    """In-place ApplySVGF over numpy buffers (result/filtered (npx,4) f32,
    prev/cur uint8 arrays of 112-byte SVGFBuffer records)."""
    orc().orc_svgf_compat(width, height, _ptr(result), _ptr(filtered), _ptr(prev), _ptr(cur), frame)


class CpuBvh:
    """A CPU BVH of the oracle, built once and reused."""

    def __init__(self, tris):
        self.tris = np.ascontiguousarray(tris)
        self.h = orc().orc_bvh_build(_ptr(self.tris), len(self.tris))

    def close(self):
        if self.h:
            orc().orc_bvh_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def render_compat_px(bvh, mats, cam, width, height, px_list, env=None, threads=None):
    """Compat estimator, one sample for each pixel of px_list, closest hits
    from the CPU BVH.  Returns (n_px, 3) float32 and the traversal count."""
    px = np.ascontiguousarray(px_list, np.int32)
    out = np.zeros((len(px), 3), np.float32)
    env_p, hw, hh, hb = None, 0, 0, 0
    if env is not None:
        env = np.ascontiguousarray(env, np.float32)
        hh, hw, hb = env.shape
        env_p = _ptr(env)
    cam = np.ascontiguousarray(cam, np.float32)
    mats = np.ascontiguousarray(mats)
    n = orc().orc_render_compat_px(_ptr(bvh.tris), len(bvh.tris), _ptr(mats), bvh.h, env_p, hw, hh, hb,
                                   _ptr(cam), width, height, _ptr(px), len(px), threads or nthreads(),
                                   _ptr(out))
    return out, n


# ---------------------------------------------------------------------------
# The reference's own code (host build, this container only)
# ---------------------------------------------------------------------------
_ref = None


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        L.ref_trace_closest.argtypes = [_vp, _i32, _vp, ctypes.c_longlong, _vp, _vp, _vp, _i32, _vp]
        L.ref_trace_closest.restype = ctypes.c_longlong
        L.ref_bvh_stats.argtypes = [_vp]
        L.ref_render.argtypes = [_vp, _i32, _vp, _i32, _vp, _i32, _vp, _i32, _i32, _i32, _vp, _vp,
                                 _i32, _i32, _i32, _i32, _vp, _vp]
        L.ref_render.restype = ctypes.c_longlong
        L.ref_svgf.argtypes = [_i32, _i32, _vp, _vp, _vp, _vp, _i32]
        L.ref_svgf.restype = _i32
        L.ref_sizeof_svgfbuffer.restype = _i32
        L.ref_disney_eval.argtypes = [_vp, _i32, _vp, _vp, _vp, _vp, _vp]
        L.ref_camera_setup.argtypes = [_vp, _f32, _f32, _f32, _f32, _vp]
        L.ref_light_cdf.argtypes = [_vp, _i32, _vp, _i32, _vp]
        L.ref_env_cdf.argtypes = [_vp, _i32, _i32, _i32, _vp]
        L.ref_load_obj.argtypes = [ctypes.c_char_p, _vp, _vp, _vp]
        L.ref_load_obj.restype = _i32
        L.ref_obj_copy.argtypes = [_vp, _vp]
        L.ref_obj_texture.argtypes = [_i32, _vp, _vp, _vp, ctypes.POINTER(ctypes.POINTER(ctypes.c_float))]
        L.ref_load_image.argtypes = [ctypes.c_char_p, _vp, _vp, _vp]
        L.ref_load_image.restype = ctypes.POINTER(ctypes.c_float)
        L.ref_tinyobj_parse.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _vp]
        L.ref_tinyobj_parse.restype = _i32
        L.ref_tinyobj_copy.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.ref_source_dir.restype = ctypes.c_char_p
        L.ref_export_scene.argtypes = [_vp, _i32, _vp, _i32, ctypes.c_char_p]
        L.ref_export_scene.restype = _i32
        L.ref_save_png_bytes.argtypes = [_vp, ctypes.c_char_p, _vp]
        L.ref_save_png_bytes.restype = _i32
        L.ref_image_size.argtypes = [_vp, _vp]
        L.ref_image_size.restype = _i32
        _ref = L
    return _ref


def ref_load_obj(directory):
    """The reference's load_object run in `directory` (./OBJ.obj there).
    Returns (triangles, materials, [texture arrays (h, w, bpp)])."""
    from kagayaki_gb300.structs import MATERIAL, TRIANGLE
    nt, nm, nx = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = ref().ref_load_obj(directory.encode(), ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(nx))
    assert rc == 0
    tris = np.zeros(nt.value, TRIANGLE)
    mats = np.zeros(nm.value, MATERIAL)
    ref().ref_obj_copy(_ptr(tris), _ptr(mats))
    texs = []
    for i in range(nx.value):
        w, h, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        px = ctypes.POINTER(ctypes.c_float)()
        ref().ref_obj_texture(i, ctypes.byref(w), ctypes.byref(h), ctypes.byref(b), ctypes.byref(px))
        n = w.value * h.value * b.value
        texs.append(np.ctypeslib.as_array(px, (n,)).copy().reshape(h.value, w.value, b.value))
    return tris, mats, texs


def ref_models_dir():
    """tinyobjloader's vendored test models in the reference checkout the
    reference build came from, or None when that checkout is not here."""
    if not ref_available():
        return None
    d = os.path.join(ref().ref_source_dir().decode(), "external_lib", "tinyobjloader", "models")
    return d if os.path.isdir(d) else None


def ref_tinyobj(path):
    """tinyobjloader's own parse of `path` (MTL files beside it), as the
    reference's load_object configures it.  None when the reader rejects the
    file; else a dict: v (n,3), vn (n,3), vt (n,2), corners (t,3,3) of
    (vertex, texcoord, normal) indices, -1 = none, and per triangle
    material, smoothing group and shape index (t,3), and the material count."""
    counts = np.zeros(5, np.int64)
    d = os.path.dirname(os.path.abspath(path)) + "/"
    if not ref().ref_tinyobj_parse(path.encode(), d.encode(), _ptr(counts)):
        return None
    nv, nn, nt, ntri, nmat = (int(c) for c in counts)
    v = np.zeros((nv, 3), np.float32)
    vn = np.zeros((nn, 3), np.float32)
    vt = np.zeros((nt, 2), np.float32)
    corners = np.zeros((ntri, 3, 3), np.int32)
    face = np.zeros((ntri, 3), np.int32)
    ref().ref_tinyobj_copy(_ptr(v), _ptr(vn), _ptr(vt), _ptr(corners), _ptr(face))
    return dict(v=v, vn=vn, vt=vt, corners=corners, face=face, n_materials=nmat)


def ref_load_image(path):
    """stbi_loadf(path, ..., 0) as the reference calls it: (h, w, bpp) floats or None."""
    w, h, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    px = ref().ref_load_image(path.encode(), ctypes.byref(w), ctypes.byref(h), ctypes.byref(b))
    if not px:
        return None
    n = w.value * h.value * b.value
    return np.ctypeslib.as_array(px, (n,)).copy().reshape(h.value, w.value, b.value)


def ref_trace(tris, rays, threads=None):
    n = len(rays)
    ids = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    ok = np.empty(n, np.uint8)
    bs = ctypes.c_double()
    nodes = ref().ref_trace_closest(_ptr(tris), len(tris), _ptr(rays), n, _ptr(ids), _ptr(t),
                                    _ptr(ok), threads or nthreads(), ctypes.byref(bs))
    return ids, t, ok, nodes, bs.value


def ref_render(tris, mats, cam, width, height, frames, env=None, threads=None, gbuf=False, textures=None):
    """The reference's render() on the host: (frames, npx, 3) samples, the
    traversal count and (gbuf=True) the last frame's SVGFBuffer records."""
    out = np.empty((frames, width * height, 3), np.float32)
    table, ntex, _keep = _texture_table(textures)
    env_p, hw, hh, hb = None, 0, 0, 0
    if env is not None:
        env = np.ascontiguousarray(env, np.float32)
        hh, hw, hb = env.shape
        env_p = _ptr(env)
    cam = np.ascontiguousarray(cam, np.float32)
    gb = None
    if gbuf:
        gb = np.zeros(width * height * ref().ref_sizeof_svgfbuffer(), np.uint8)
    n = ref().ref_render(_ptr(tris), len(tris), _ptr(mats), len(mats),
                         ctypes.cast(table, _vp) if table is not None else None, ntex, env_p, hw, hh, hb,
                         _ptr(cam), _ptr(cam), width, height, frames, threads or nthreads(),
                         _ptr(out), _ptr(gb))
    return (out, n, gb) if gbuf else (out, n)
