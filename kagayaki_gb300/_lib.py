"""ctypes binding of libkagayaki_gb300.so (the C ABI of include/kagayaki.h).

There is no fallback: when the library is missing every call raises
RuntimeError telling the caller to build it.
"""
import ctypes
import os

from .structs import (KgkBvhInfo, KgkCamera, KgkRenderConfig, KgkStats, KgkSvgfConfig, KgkTexture,
                      KgkVec)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkagayaki_gb300.so")

# Every function declared in include/kagayaki.h: name -> (restype, argtypes).
_vp = ctypes.c_void_p
_st = ctypes.c_int
_sz = ctypes.c_size_t
_i32 = ctypes.c_int32
_f = ctypes.c_float
PROTOTYPES = {
    "kgk_version": (ctypes.c_char_p, []),
    "kgk_status_string": (ctypes.c_char_p, [_st]),
    "kgk_last_error": (_st, [ctypes.c_char_p, _sz]),
    "kgk_set_device": (_st, [ctypes.c_int]),
    "kgk_scene_create": (_st, [_vp, _sz, _vp, _sz, _vp, _sz, _vp, ctypes.POINTER(_vp)]),
    "kgk_scene_load_obj": (_st, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "kgk_scene_load_obj_ex": (_st, [ctypes.c_char_p, ctypes.c_char_p, _vp, ctypes.POINTER(_vp)]),
    "kgk_scene_destroy": (None, [_vp]),
    "kgk_build_bvh": (_st, [_vp, ctypes.POINTER(KgkBvhInfo)]),
    "kgk_bvh_validate": (_st, [_vp]),
    "kgk_trace_closest": (_st, [_vp, _vp, _sz, _vp, _vp, ctypes.POINTER(KgkStats)]),
    "kgk_trace_any": (_st, [_vp, _vp, _vp, _sz, _vp, ctypes.POINTER(KgkStats)]),
    "kgk_camera_setup": (_st, [KgkVec, _f, _f, _f, _f, _i32, ctypes.POINTER(KgkCamera)]),
    "kgk_render": (_st, [_vp, ctypes.POINTER(KgkCamera), ctypes.POINTER(KgkCamera),
                         ctypes.POINTER(KgkRenderConfig), _vp, ctypes.POINTER(KgkStats)]),
    "kgk_accum_reset": (_st, [_vp, _i32, _i32]),
    "kgk_accum_read": (_st, [_vp, _vp, _vp, ctypes.POINTER(ctypes.c_uint64)]),
    "kgk_svgf": (_st, [_vp, ctypes.POINTER(KgkSvgfConfig), _vp, _vp]),
    "kgk_svgf_output": (_st, [_vp, ctypes.POINTER(KgkSvgfConfig), _vp, _vp, _vp, _i32]),
    "kgk_scene_sync": (_st, [_vp]),
    "kgk_host_alloc": (_st, [_sz, ctypes.POINTER(_vp)]),
    "kgk_host_free": (None, [_vp]),
    "kgk_svgf_apply": (_st, [_vp, _vp, _vp, _vp, _i32, _i32, _i32]),
    "kgk_gbuffer_records": (_st, [_vp, _vp]),
    "kgk_disney_eval": (_st, [_vp, _i32, _vp, _vp, _vp, _vp, _vp]),
    "kgk_svgf_apply_noalloc": (_st, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "kgk_nrc_init": (_st, [_vp, _vp]),
    "kgk_nrc_set_weights": (_st, [_vp, _vp, _sz]),
    "kgk_nrc_get_weights": (_st, [_vp, _vp, _sz]),
    "kgk_nrc_infer": (_st, [_vp, _vp, _sz, _vp]),
    "kgk_nrc_gradients": (_st, [_vp, _vp, _vp, _sz, _vp, _vp]),
    "kgk_nrc_train": (_st, [_vp, _vp, _vp, _sz, _i32, _vp]),
    "kgk_nrc_loss_scale": (_st, [_vp, _vp]),
    "kgk_scene_set_textures_rgba8": (_st, [_vp, _vp, _sz]),
    "kgk_load_obj": (_st, [ctypes.c_char_p, ctypes.c_char_p, _vp]),
    "kgk_load_obj_ex": (_st, [ctypes.c_char_p, ctypes.c_char_p, _vp, _vp]),
    "kgk_host_scene_free": (None, [_vp]),
    "kgk_load_image": (_st, [ctypes.c_char_p, _vp]),
    "kgk_image_free": (None, [_vp]),
    "kgk_tonemap_rgba8": (_st, [_vp, _i32, _i32, _vp]),
    "kgk_save_png": (_st, [_vp, _i32, _i32, ctypes.c_char_p]),
    "kgk_save_exr": (_st, [_vp, _i32, _i32, _i32, ctypes.c_char_p]),
}

_lib = None


class KgkError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{status_name(status)}: {message}")
        self.status = status
        self.message = message


def lib():
    """The loaded library (built in-tree by kagayaki_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libkagayaki_gb300.so is not built: run `python -c \"import __graft_entry__ as g; g.build()\"` "
                "or `python kagayaki_gb300/build.py`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_name(st):
    try:
        return lib().kgk_status_string(st).decode()
    except Exception:
        return f"status {st}"


def last_error():
    buf = ctypes.create_string_buffer(2048)
    lib().kgk_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(st):
    if st != 0:
        raise KgkError(st, last_error())
