"""Evaluating many independent tensors together.

The reference evaluates each tensor with its own kernel launch
(Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:1331-1381).
``Batch`` takes many tensors whose expressions read their inputs without views
(the shape of programs that dominate real pipelines: long chains of
elementwise math over equally shaped buffers) and evaluates all of them in one
persistent kernel launch, or in one launch each, or in a replayed CUDA graph of
those launches; each mode computes identical bits.
"""

from __future__ import annotations

from typing import List, Sequence

from .tensors import CachedTensor, Tensor, Tensors, _Evaluation, _product


class Batch:
    PERSISTENT, PER_PROGRAM, GRAPH = 0, 1, 2

    def __init__(self, device: Tensors, tensors: Sequence[Tensor]):
        self.device = device
        self.tensors = list(tensors)
        self.serialized = [device.serialize(t.closure, t.shape) for t in self.tensors]
        self.handle = device.runtime.batch_create([s.text for s in self.serialized])
        self.outputs: List = []
        self._ev = None

    def bind(self, outputs=None):
        """Evaluates every input once, allocates (or takes) the outputs, and binds the buffers."""
        rt = self.device.runtime
        if self._ev is not None:
            self._ev.close()
        self._ev = _Evaluation(self.device)
        ptrs = []
        self.outputs = []
        for k, (t, ser) in enumerate(zip(self.tensors, self.serialized)):
            for p in ser.params:
                buf = p._buffer(self._ev)
                self._ev.wait(buf)  # the batch runs on the context stream
                ptrs.append(buf.device_ptr())
            out = outputs[k] if outputs is not None else rt.alloc(max(1, _product(t.shape)) * 4)
            if outputs is None:
                self._ev.owned.append(out)
            self.outputs.append(out)
            ptrs.append(out.device_ptr())
        rt.batch_bind(self.handle, ptrs)
        return self

    def run(self, mode: int = 0):
        self.device.runtime.batch_run(self.handle, mode)
        return self

    # host transfers in the event model: each returns an event for the next wait list
    def upload_ev(self, host_ptrs, wait=()):
        """Every input from pinned host memory: per program, its inputs in parameter order."""
        return self.device.runtime.batch_upload_ev(self.handle, host_ptrs, wait)

    def run_ev(self, mode: int = 0, wait=()):
        return self.device.runtime.batch_run_ev(self.handle, mode, wait)

    def download_ev(self, host_ptrs, wait=()):
        """Every output into pinned host memory (one pointer per program)."""
        return self.device.runtime.batch_download_ev(self.handle, host_ptrs, wait)

    def results(self):
        """The outputs, as cached tensors that stay valid until closed."""
        res = []
        for t, out in zip(self.tensors, self.outputs):
            out.retain()
            res.append(CachedTensor(self.device, t.shape, t.padding, out))
        return res

    def close(self):
        if self._ev is not None:
            self._ev.close()
            self._ev = None
        if self.handle:
            self.device.runtime.batch_release(self.handle)
            self.handle = 0
