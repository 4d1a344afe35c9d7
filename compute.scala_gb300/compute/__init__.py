"""GB300 (sm_103a) back-end for Compute.scala's fused-tensor path.

``from compute import cuda`` gives the device object; ``cuda.Tensor`` is the
reference's Tensor companion (``Tensor(...)``, ``Tensor.fill``, ``Tensor.random``,
``Tensor.join`` ...).  The native runtime is ``libcomputecuda.so`` next to this
file, reached through the C ABI declared in include/compute_cuda.h.
"""

from .tensors import (CachedTensor, FillTensor, InlineTensor, NonInlineTensor, Tensor, Tensors, TensorSeq,
                      TransformedTensor)
from ._native import IllegalArgumentException
from . import trees, affine


class _LazyDevice:
    """The ``cuda`` object, created on first attribute access."""

    def __init__(self, ordinal: int = 0):
        self._ordinal = ordinal
        self._device = None

    def _get(self) -> Tensors:
        if self._device is None:
            self._device = Tensors(device=self._ordinal)
        return self._device

    def __getattr__(self, name):
        return getattr(self._get(), name)


cuda = _LazyDevice(0)

__all__ = ["cuda", "Tensors", "Tensor", "InlineTensor", "TransformedTensor", "NonInlineTensor", "CachedTensor",
           "FillTensor", "TensorSeq", "IllegalArgumentException", "trees", "affine"]
