"""kagayaki_gb300 - GB300-native (sm_103a) drop-in for the kagayaki render path.

The compute path is the CUDA library libkagayaki_gb300.so (C ABI:
include/kagayaki.h); this package is its host-side mirror.
"""
from ._lib import KgkError, lib, last_error  # noqa: F401
from .api import (ESTIMATOR_COMPAT, ESTIMATOR_UNBIASED, Scene, camera_array,  # noqa: F401
                  camera_setup, load_image, load_obj, save_png, tonemap)
