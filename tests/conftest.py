import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "compute.scala_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


_cuda = {}


def cuda_tensors(**kw):
    """One native device object per flag set for the whole session (compiled programs are cached).
    The parity tests pin the standard kernels, so the tuner is off unless asked for; the
    tuner's own tests check that every configuration computes the standard kernel's bits."""
    from compute import Tensors
    kw.setdefault("tuner", "off")
    key = tuple(sorted(kw.items()))
    if key not in _cuda:
        _cuda[key] = Tensors(device=0, **kw)
    return _cuda[key]


@pytest.fixture
def oracle_device():
    from oracle_runtime import OracleRuntime
    from compute import Tensors
    return Tensors(runtime=OracleRuntime())


@pytest.fixture
def cuda_device():
    return cuda_tensors()


@pytest.fixture(params=["oracle", "cref", pytest.param("cuda", marks=pytest.mark.gpu)])
def device(request):
    """The reference's test cases run on three back-ends: the numpy oracle and the
    reference's generated OpenCL C compiled for the host (both CPU; they pin the
    oracles against the reference's goldens), and the CUDA runtime (GPU parity)."""
    from compute import Tensors, trees
    if request.param == "oracle":
        from oracle_runtime import OracleRuntime
        return Tensors(runtime=OracleRuntime())
    if request.param == "cref":
        from oracle.cref import CRuntime
        return Tensors(runtime=CRuntime(), planner=trees.Planner(enabled=False))
    return cuda_tensors()
