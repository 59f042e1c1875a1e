"""numpy / ctypes mirrors of the C-ABI structs in include/kagayaki.h.

The layouts are byte-compatible with the reference's structs
(struct_Triangle.cuh:8-20, struct_Material.cuh:6-11, struct_Camera.cuh:12-18,
struct_Ray.cuh:12-15, struct_Texture.cuh:6-8); the sizes are asserted here and
in the library.
"""
import ctypes

import numpy as np

# struct_Vec.cuh:4-8: x, y, z + pad.
VEC = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("align", "<f4")])

# struct_Triangle.cuh:8-20.  `verts` holds the nine Vec members in order:
# v0, v1, v2, v0_vn, v1_vn, v2_vn, v0_vt, v1_vt, v2_vt.
TRIANGLE = np.dtype({
    "names": ["verts", "material_id", "is_SmoothNormal", "shape_id"],
    "formats": [("<f4", (9, 4)), "<i4", "u1", "<i4"],
    "offsets": [0, 144, 148, 152],
    "itemsize": 156,
}, align=True)

# struct_Material.cuh:6-11 (field order of the struct, not of its constructor).
MATERIAL_PARAMS = ["subsurface", "metallic", "specular", "specularTint", "roughness",
                   "anisotropic", "sheen", "sheenTint", "clearcoat", "cloearcoatGloss",
                   "IOR", "mu_a", "mu_s", "scatter_g"]
MATERIAL = np.dtype([("MATERIAL_TYPE_ID", "<i4"), ("TEXTURE_BASECOLOR_ID", "<i4"),
                     ("diffuse", "<f4", (4,)), ("emission", "<f4", (4,))]
                    + [(p, "<f4") for p in MATERIAL_PARAMS], align=True)

# struct_Ray.cuh:12-15: dir, org, double pad.
RAY = np.dtype([("dir", "<f4", (4,)), ("org", "<f4", (4,)), ("_dummy", "<f8")], align=True)

# struct_SVGFBuffers.cuh:7-23 `SVGFBuffer` (112 B: two bytes of padding after
# the two flags).
SVGF_BUFFER = np.dtype({
    "names": ["Albedo", "Emission", "Normal", "ColorHistory", "ObjectID", "MaterialID",
              "PosLastFrameI", "PosLastFrameF", "sampleNum", "MomentOne", "MomentTwo", "Variance",
              "Depth", "willApplyATrousFilter", "willApplyTemporalAccumulation"],
    "formats": [("<f4", (4,)), ("<f4", (4,)), ("<f4", (4,)), ("<f4", (4,)), "<i4", "<i4",
                ("<i4", (2,)), ("<f4", (2,)), "<i4", "<f4", "<f4", "<f4", "<f4", "u1", "u1"],
    "offsets": [0, 16, 32, 48, 64, 68, 72, 80, 88, 92, 96, 100, 104, 108, 109],
    "itemsize": 112,
})

# align=True keeps numpy from repacking the records (dropping the C padding)
# when arrays are concatenated.
assert TRIANGLE.itemsize == 156 and TRIANGLE.isalignedstruct
assert MATERIAL.itemsize == 96
assert RAY.itemsize == 40
assert SVGF_BUFFER.itemsize == 112

LAMBERT = 0
DISNEY = 1


class KgkVec(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float),
                ("align", ctypes.c_float)]


class KgkCamera(ctypes.Structure):
    _fields_ = [("CamOrg", KgkVec), ("CamDir", KgkVec), ("CamToScreenDist", ctypes.c_float),
                ("ScreenXDir", KgkVec), ("ScreenYDir", KgkVec), ("PixelSize", ctypes.c_float)]


class KgkTexture(ctypes.Structure):
    _fields_ = [("pixels", ctypes.POINTER(ctypes.c_float)), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("bpp", ctypes.c_int32)]


class KgkRenderConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("spp", ctypes.c_int32), ("max_depth", ctypes.c_int32),
                ("rr_start_depth", ctypes.c_int32), ("estimator", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("frame_index", ctypes.c_int32),
                ("accumulate", ctypes.c_int32), ("wave_paths", ctypes.c_int32),
                ("count_work", ctypes.c_int32), ("write_gbuffer", ctypes.c_int32),
                ("use_cache", ctypes.c_int32), ("profile_stages", ctypes.c_int32),
                ("texture_filter", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4)]


class KgkTextureRGBA8(ctypes.Structure):
    _fields_ = [("pixels", ctypes.c_void_p), ("width", ctypes.c_int32), ("height", ctypes.c_int32)]


class KgkStats(ctypes.Structure):
    _fields_ = [("rays_closest", ctypes.c_uint64), ("rays_shadow", ctypes.c_uint64),
                ("traversal_overflows", ctypes.c_uint64), ("nodes_visited", ctypes.c_uint64),
                ("tris_tested", ctypes.c_uint64), ("paths", ctypes.c_uint64),
                ("ms_device", ctypes.c_double), ("kernel_launches", ctypes.c_uint64),
                ("ms_extend", ctypes.c_double), ("ms_shade", ctypes.c_double),
                ("ms_shadow", ctypes.c_double), ("extend_launches", ctypes.c_uint64),
                ("ms_tail", ctypes.c_double), ("rays_tail", ctypes.c_uint64)]


class KgkBvhInfo(ctypes.Structure):
    _fields_ = [("n_triangles", ctypes.c_uint64), ("n_wide_nodes", ctypes.c_uint64),
                ("n_binary_nodes", ctypes.c_uint64), ("max_depth", ctypes.c_uint32),
                ("max_leaf_size", ctypes.c_uint32), ("sah_cost", ctypes.c_double),
                ("ms_build", ctypes.c_double), ("device_bytes", ctypes.c_uint64)]


class KgkSvgfConfig(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("frame_index", ctypes.c_int32), ("atrous_iterations", ctypes.c_int32),
                ("atrous_repeats", ctypes.c_int32), ("alpha", ctypes.c_float),
                ("sigma_z", ctypes.c_float), ("sigma_n", ctypes.c_float),
                ("sigma_l", ctypes.c_float), ("reserved", ctypes.c_int32 * 6)]


class KgkHostScene(ctypes.Structure):
    _fields_ = [("triangles", ctypes.c_void_p), ("n_triangles", ctypes.c_size_t),
                ("materials", ctypes.c_void_p), ("n_materials", ctypes.c_size_t),
                ("textures", ctypes.POINTER(KgkTexture)), ("n_textures", ctypes.c_size_t),
                ("hdr", KgkTexture)]


MATERIALS_REFERENCE = 0
MATERIALS_PBR = 1


class KgkLoadOptions(ctypes.Structure):
    _fields_ = [("material_model", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 6)]


class KgkNrcConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("hidden_layers", ctypes.c_int32),
                ("learning_rate", ctypes.c_float), ("train_paths", ctypes.c_int32),
                ("train_suffix_max", ctypes.c_int32), ("train_steps", ctypes.c_int32),
                ("spread_c", ctypes.c_float), ("seed", ctypes.c_uint64),
                ("reserved", ctypes.c_int32 * 8)]


assert ctypes.sizeof(KgkCamera) == 72
assert ctypes.sizeof(KgkTexture) == 24


def camera_to_array(cam):
    """KgkCamera -> float32[18] view of its 72 bytes."""
    return np.frombuffer(bytes(cam), dtype="<f4").copy()


def make_material(mtype=LAMBERT, diffuse=(0.8, 0.8, 0.8), emission=(0.0, 0.0, 0.0), tex=-1,
                  **params):
    """One MATERIAL record with the reference constructor's defaults
    (struct_Material.cuh:22-30)."""
    m = np.zeros((), dtype=MATERIAL)
    m["MATERIAL_TYPE_ID"] = mtype
    m["TEXTURE_BASECOLOR_ID"] = tex
    m["diffuse"][:3] = diffuse
    m["emission"][:3] = emission
    defaults = dict(subsurface=0.0, metallic=0.0, specular=0.0, specularTint=0.0, roughness=0.0,
                    anisotropic=0.0, sheen=0.0, sheenTint=0.0, clearcoat=0.0,
                    cloearcoatGloss=0.0, IOR=1.45, mu_a=0.0, mu_s=0.0, scatter_g=0.5)
    defaults.update(params)
    for k, v in defaults.items():
        m[k] = v
    return m
