"""The C-ABI libraries load and export every symbol include/snncuda_gb300.h
declares (no device calls: runs without a GPU)."""

import ctypes
import re

import pytest

from conftest import GPU_PATH, PORT_PATH, REF_PATH, ROOT, _ensure_built


def header_symbols():
    text = (ROOT / "include" / "snncuda_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\*?\s+\**(snncuda_[a-z_0-9]+)\(", text, re.M)))


def test_header_declares_the_abi():
    from snncuda_gb300._abi import ABI_SYMBOLS
    assert set(header_symbols()) == set(ABI_SYMBOLS)


@pytest.mark.parametrize("path", [GPU_PATH, PORT_PATH], ids=["gpu_backend", "oracle_port"])
def test_library_exports_every_symbol(path):
    _ensure_built()
    lib = ctypes.CDLL(str(path))
    for name in header_symbols():
        assert hasattr(lib, name), f"{path.name} lacks {name}"


def test_reference_harness_exports_every_symbol():
    if not REF_PATH.exists():
        pytest.skip("reference runtime not built here")
    lib = ctypes.CDLL(str(REF_PATH))
    for name in header_symbols():
        assert hasattr(lib, name)


def test_backend_version_and_config_defaults():
    _ensure_built()
    from snncuda_gb300 import _abi, default_config
    lib = _abi.bind(str(GPU_PATH))
    assert lib.snncuda_version().decode().startswith("0.1.0")
    cfg = default_config(lib)
    # learning::StdpConfig defaults (STDP.h:8-16)
    assert (cfg.stdp_enabled, cfg.ltp_amplitude, cfg.ltd_amplitude) == (1, pytest.approx(0.01), pytest.approx(0.012))
    assert (cfg.ltp_tau_ticks, cfg.ltd_tau_ticks, cfg.min_weight, cfg.max_weight) == (20.0, 20.0, 0.0, 2.0)
    assert cfg.temporal_learning_enabled == 1 and cfg.timing_wheel_slots == 4096


def test_missing_backend_fails_loudly(monkeypatch, tmp_path):
    from snncuda_gb300 import simulation
    monkeypatch.setattr(simulation, "_backend", None)
    monkeypatch.setenv("SNNCUDA_GB300_LIBRARY", str(tmp_path / "absent.so"))
    with pytest.raises(simulation.SNNCudaError):
        simulation.backend()
