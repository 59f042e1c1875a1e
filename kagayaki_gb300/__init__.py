"""kagayaki_gb300 - GB300-native (sm_103a) drop-in for the kagayaki render path.

The compute path is the CUDA library libkagayaki_gb300.so (C ABI:
include/kagayaki.h); this package is its host-side mirror.
"""
from ._lib import KgkError, lib, last_error  # noqa: F401
from .api import (ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED, MATERIALS_PBR, MATERIALS_REFERENCE,  # noqa: F401
                  Scene, camera_array, camera_setup, load_image, load_obj, save_exr, save_png, tonemap)
