"""The SNNCuda::snncuda CMake package: CMakeLists.txt builds the backend
library for sm_103a and installs SNNCudaConfig.cmake,
SNNCudaConfigVersion.cmake and SNNCudaTargets.cmake; a consumer written like
the reference's examples/cmake_consumer (find_package(SNNCuda CONFIG
REQUIRED), target_link_libraries(... SNNCuda::snncuda)) compiles, links and
runs against it.  On a machine with a GPU the consumer also runs the
reference's three-neuron propagation chain through the C ABI."""

import os
import pathlib
import re
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CONSUMER = ROOT / "tests" / "cmake_consumer"
CMAKE = shutil.which("cmake")

pytestmark = pytest.mark.skipif(CMAKE is None, reason="cmake not installed")


def _run(cmd, **kw):
    proc = subprocess.run([str(c) for c in cmd], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, **kw)
    assert proc.returncode == 0, proc.stdout[-4000:]
    return proc.stdout


@pytest.fixture(scope="module")
def consumer(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("cmake")
    gen = ["-G", "Ninja"] if shutil.which("ninja") else []
    _run([CMAKE, "-S", ROOT, "-B", tmp / "build", *gen, "-DCMAKE_BUILD_TYPE=Release"])
    _run([CMAKE, "--build", tmp / "build", "-j", str(os.cpu_count() or 4)])
    _run([CMAKE, "--install", tmp / "build", "--prefix", tmp / "prefix"])
    _run([CMAKE, "-S", CONSUMER, "-B", tmp / "consumer", *gen, f"-DCMAKE_PREFIX_PATH={tmp / 'prefix'}"])
    _run([CMAKE, "--build", tmp / "consumer"])
    return tmp / "prefix", tmp / "consumer" / "snncuda_consumer"


def _output(exe):
    out = _run([exe])
    fields = dict(re.findall(r"(\w+)=(\S+)", out))
    return out, fields


def test_package_installs_config_files_and_consumer_links(consumer):
    prefix, exe = consumer
    cfg_dirs = list(prefix.glob("lib*/cmake/SNNCuda"))
    assert cfg_dirs, "no lib/cmake/SNNCuda"
    names = {p.name for p in cfg_dirs[0].iterdir()}
    assert {"SNNCudaConfig.cmake", "SNNCudaConfigVersion.cmake", "SNNCudaTargets.cmake"} <= names
    targets = (cfg_dirs[0] / "SNNCudaTargets.cmake").read_text()
    assert "SNNCuda::snncuda" in targets and "SNNCUDA_HAS_CUDA=1" in targets
    assert (prefix / "include" / "snncuda_gb300.h").exists()
    assert (prefix / "include" / "snncuda" / "core" / "Version.h").exists()
    out, f = _output(exe)
    assert f["version"].startswith("0.1.0") and f["has_cuda_define"] == "1", out
    if f["cuda_available"] == "0":
        # no device here: creation fails with a CUDA error status, no crash
        assert f["create"] == "4", out


@pytest.mark.gpu
def test_consumer_runs_the_propagation_chain_on_the_gpu(consumer):
    _, exe = consumer
    out, f = _output(exe)
    assert f["cuda_available"] == "1" and f["create"] == "0" and f["status"] == "0", out
    assert f["delivered"] == "3" and f["fired"] == "3", out
    assert f["fires"] == "0:0,2:1,5:2", out
