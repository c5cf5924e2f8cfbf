"""Shared fixtures: the libraries implementing the C ABI.

`port_lib`  the CPU oracle restatement (oracle/_build/liboracle_port.so)
`ref_lib`   the reference runtime built from its sources (only where present)
`gpu_lib`   the GB300 backend; tests using it are marked `gpu`
"""

import ctypes
import os
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

PORT_PATH = ROOT / "oracle" / "_build" / "liboracle_port.so"
REF_PATH = ROOT / "oracle" / "_ref" / "libsnnref.so"
GPU_PATH = ROOT / "snncuda_gb300" / "_lib" / "libsnncuda_gb300.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU")


def _ensure_built():
    if not PORT_PATH.exists() or not GPU_PATH.exists():
        import __graft_entry__
        __graft_entry__.build()


@pytest.fixture(scope="session")
def port_lib():
    _ensure_built()
    from snncuda_gb300 import _abi
    return _abi.bind(str(PORT_PATH))


@pytest.fixture(scope="session")
def ref_lib():
    if not REF_PATH.exists():
        pytest.skip("reference runtime not built here")
    from snncuda_gb300 import _abi
    lib = _abi.bind(str(REF_PATH))
    ctypes.CDLL(str(REF_PATH)).snnref_set_mode(1)
    return lib


@pytest.fixture(scope="session")
def gpu_lib():
    _ensure_built()
    from snncuda_gb300 import simulation
    lib = simulation.backend()
    if not lib.snncuda_cuda_available():
        pytest.fail("GPU test without a visible CUDA device")
    return lib
