"""Drop-in counterparts of the reference's compiled modules
``cudaExtensions.{transform,sampling,splatting,filtering,interpolation,shading}``
(setup.py:11-69): same function names, argument order and return values, each a
thin host wrapper over the C ABI of libuds.so running on the current CUDA
stream.  Inputs are validated (contiguous float32 / int32 CUDA tensors on one
device) and a bad input raises instead of asserting.
"""
from . import filtering, interpolation, nearestsamples, pixelgather, sampling, shading, splatting, transform  # noqa: F401,E501

__all__ = ["transform", "sampling", "splatting", "filtering", "interpolation", "shading", "pixelgather", "nearestsamples"]
