"""GB300-native acoustic wave-propagation engine.

Drop-in for the time-stepping path of Nacnud04/wavefield_imaging's
sfAWEFD{cart,spher}{2D,3D}gpu programs (and the 2N-order scheme of its
cartesian CPU programs): hand-written sm_103a CUDA kernels behind the C-ABI
in include/awe.h, built into wavefield_imaging_gb300/_build/libawe.so.
"""
from .engine import (  # noqa: F401
    CART, CKPT_BF16, CKPT_BFP16, CKPT_FP16, CKPT_FP32, EXACT, FAST, IMAGE_BORN, IMAGE_XCORR, MOVE_DYN, MOVE_PER_STEP, SCHEME_CPU, SCHEME_GPU, SPHER, AweError,
    Batch, Desc, Plan, cloud_merge, cloud_window, lib, make_desc,
)

__all__ = ["Plan", "Batch", "cloud_window", "cloud_merge", "Desc", "make_desc", "AweError", "lib", "CART", "SPHER", "SCHEME_CPU", "SCHEME_GPU", "FAST",
           "EXACT", "CKPT_BF16", "CKPT_BFP16", "CKPT_FP16", "CKPT_FP32", "MOVE_PER_STEP", "MOVE_DYN", "IMAGE_XCORR", "IMAGE_BORN"]
