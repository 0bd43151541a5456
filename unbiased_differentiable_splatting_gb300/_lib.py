"""ctypes binding of libuds.so (the C ABI declared in include/uds.h).

The product path always runs these CUDA kernels: if the library cannot be
loaded, or a tensor is not a contiguous CUDA tensor of the right dtype, the
call raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import _build

_lock = threading.Lock()
_lib = None

c_int, c_float, c_size_t, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_size_t, ctypes.c_void_p
c_int64, c_uint64 = ctypes.c_int64, ctypes.c_uint64


class SampleParams(ctypes.Structure):
    """uds_sample_params (include/uds.h)."""

    _fields_ = [("B", ctypes.c_int32), ("N", ctypes.c_int32), ("W", ctypes.c_int32), ("H", ctypes.c_int32),
                ("K", ctypes.c_int32), ("focal", c_float), ("smoothing", c_float), ("precision", c_float),
                ("max_degree", ctypes.c_int32), ("std_batch", ctypes.c_int32), ("coef_pool", c_int64),
                ("seed", c_uint64), ("seed_dev", c_void_p), ("tile_x", ctypes.c_int32),
                ("fixed_degree", ctypes.c_int32), ("leaf_size", ctypes.c_int32),
                ("spread", ctypes.c_int32)]


class ViewDesc(ctypes.Structure):
    """uds_view_desc (include/uds.h)."""

    _fields_ = [("W", ctypes.c_int32), ("H", ctypes.c_int32), ("focal", c_float), ("reserved", ctypes.c_int32)]


VIEW_STATS_FIELDS = ("h", "radius", "n_visible", "n_coefs", "demoted", "overflow")

_SIGS = {
    "uds_status_string": (ctypes.c_char_p, [c_int]),
    "uds_last_error": (ctypes.c_char_p, []),
    "uds_version": (c_int, []),
    "uds_launch_count": (ctypes.c_ulonglong, []),
    "uds_transform_forward": (c_int, [c_int, c_int, c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "uds_transform_backward": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p,
                                       c_void_p, c_void_p]),
    "uds_view_matrix_forward": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_view_matrix_backward": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_backface_forward": (c_int, [c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_backface_backward": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                      c_void_p]),
    "uds_render_fused_forward": (c_int, [c_int, c_int, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p, c_int,
                                         c_int, c_void_p, c_float, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_render_fused_backward": (c_int, [c_int, c_int, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p,
                                          c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_float,
                                          c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_size_t, c_void_p]),
    "uds_sample_workspace_size": (c_size_t, [ctypes.POINTER(SampleParams)]),
    "uds_sample": (c_int, [ctypes.POINTER(SampleParams), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_sample_views": (c_int, [ctypes.POINTER(SampleParams), ctypes.POINTER(ViewDesc), c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_sample_stochastic": (c_int, [ctypes.POINTER(SampleParams), c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_tree_build": (c_int, [ctypes.POINTER(SampleParams), c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_sample_descent": (c_int, [ctypes.POINTER(SampleParams), c_int, c_void_p, c_void_p, c_void_p, c_size_t,
                                   c_void_p]),
    "uds_fgt_eval": (c_int, [ctypes.POINTER(SampleParams), c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_size_t, c_void_p]),
    "uds_mma_probe": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "uds_mlp_param_count": (c_int, []),
    "uds_mlp_forward": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_mlp_grad_workspace_size": (c_size_t, [c_int]),
    "uds_mlp_grad": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                             c_void_p]),
    "uds_mlp_adam": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float, c_float, c_float, c_float,
                             c_void_p]),
    "uds_mlp_forward_dev": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_mlp_forward_tiles": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_proposal_workspace_size": (c_size_t, [ctypes.POINTER(SampleParams)]),
    "uds_sample_proposal": (c_int, [ctypes.POINTER(SampleParams), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_float, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                                    c_void_p]),
    "uds_proposal_dataset": (c_int, [ctypes.POINTER(SampleParams), c_int, c_int, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "uds_pixel_scatter": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "uds_pixel_gather_workspace_size": (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    "uds_pixel_gather": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_int, c_int, c_void_p, c_void_p, c_int,
                                 c_void_p, c_size_t, c_void_p]),
    "uds_nearest_workspace_size": (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    "uds_nearest_samples": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int,
                                    c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_nearest_regularizer_workspace_size": (c_size_t, [c_int]),
    "uds_nearest_regularizer": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_float, c_int, c_void_p, c_void_p,
                                        c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_image_loss": (c_int, [c_int, c_size_t, c_void_p, c_void_p, c_float, c_void_p, c_void_p, c_void_p]),
    "uds_adam_splats": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                c_void_p, c_void_p, c_void_p, c_int, c_float, c_float, c_float, c_float, c_float,
                                c_float, c_int, c_void_p]),
    "uds_splat_workspace_size": (c_size_t, [c_int, c_int]),
    "uds_splat_forward": (c_int, [c_int, c_int, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p, c_int,
                                  c_int, c_void_p, c_float, c_void_p, c_void_p, c_size_t, c_void_p]),
    "uds_splat_backward": (c_int, [c_int, c_int, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_int, c_int, c_void_p, c_float, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_size_t, c_void_p]),
    "uds_splat_forward_static": (c_int, [c_int, c_int, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p,
                                         c_int, c_int, c_void_p, c_float, c_void_p, c_void_p]),
    "uds_filter_forward": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_float, c_int, c_int,
                                   c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_filter_backward": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_float, c_int,
                                    c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_interp_forward": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_int, c_int,
                                   c_void_p, c_void_p, c_void_p]),
    "uds_interp_backward": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int,
                                    c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_shade_forward": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                  c_void_p]),
    "uds_shade_backward": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_shade_sh_forward": (c_int, [c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "uds_shade_sh_backward": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p]),
    "uds_lambert_forward": (c_int, [c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p,
                                    c_void_p, c_int, c_void_p, c_void_p]),
    "uds_lambert_backward": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int,
                                     c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p]),
}


def exported_symbols():
    """Names of every entry point include/uds.h declares."""
    return tuple(_SIGS)


def load(build_if_missing: bool = True):
    """Load libuds.so, building it in-tree first when it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing and not os.path.exists(_build.LIB):
                _build.build()
            if not os.path.exists(_build.LIB):
                raise RuntimeError(f"libuds.so not found at {_build.LIB}; run __graft_entry__.build()")
            L = ctypes.CDLL(_build.LIB)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class UdsError(RuntimeError):
    pass


def check(status: int, what: str) -> None:
    if status != 0:
        L = load()
        msg = L.uds_status_string(status).decode()
        detail = L.uds_last_error().decode() if status in (3, 4) else ""
        raise UdsError(f"{what}: {msg}" + (f" ({detail})" if detail else ""))


def stream_ptr(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t):
    return None if t is None else t.data_ptr()


def need(t: torch.Tensor, name: str, dtype=torch.float32, device=None) -> torch.Tensor:
    """Validate an input like the reference's asserts (contiguous CUDA tensor),
    raising instead of aborting."""
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if device is not None and t.device != device:
        raise ValueError(f"{name} is on {t.device}, expected {device}")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t


class Workspace:
    """Per-device scratch buffer for the C ABI, taken from torch's caching
    allocator and grown on demand (never shrunk)."""

    _bufs: dict = {}

    @classmethod
    def get(cls, device: torch.device, nbytes: int, slot: str = "default") -> torch.Tensor:
        key = (device.index if device.index is not None else torch.cuda.current_device(), slot)
        buf = cls._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
            cls._bufs[key] = buf
        return buf

    @classmethod
    def reserve(cls, device: torch.device, nbytes: int, slot: str = "default") -> None:
        cls.get(device, nbytes, slot)
