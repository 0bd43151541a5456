"""GB300 implementation of the differentiable Poisson-sampled EWA
surface-splatting path (FMM tree sampler, EWA weights, depth compositing,
shading, interpolation and their backward passes).

Layers:
* ``libuds.so`` - hand-written sm_103a CUDA kernels behind the C ABI declared
  in ``include/uds.h`` (built in-tree by ``_build.build()``);
* ``cudaExtensions`` - the reference's extension modules (same names and
  signatures) over that C ABI;
* ``extensions`` / ``render`` - the autograd functions and the ``Splatting``
  renderer module;
* ``scenes`` - seeded synthetic workloads.
"""
from . import _build, _lib  # noqa: F401

__version__ = "1.0.0"


def build(force: bool = False) -> str:
    """Compile libuds.so for sm_103a (no-op when up to date)."""
    return _build.build(force=force)


def load():
    """Load libuds.so (raises if it is missing or cannot be loaded)."""
    return _lib.load()
