"""Declarative loading of native `.snncuda.json` networks
(snncuda_gb300.declarative): the Connectome built from every document in
tests/golden/declarative/ must equal the one the reference's own
DeclarativeLoader + ConnectomeBuilder build (golden digests recorded by
tests/golden/make_declarative_golden.py), including the reference's error
for an invalid document; a loaded network then runs through the C ABI."""

import json
import os
import pathlib
import subprocess
import sys
import time

import numpy as np
import pytest

from snncuda_gb300 import declarative, synthetic
from snncuda_gb300.simulation import Simulation, default_config

HERE = pathlib.Path(__file__).resolve().parent
DOCS = HERE / "golden" / "declarative"
GOLDEN = json.loads((HERE / "golden" / "declarative.json").read_text())
sys.path.insert(0, str(HERE / "golden"))
from make_declarative_golden import DUMP, canonical_arrays, digests, record  # noqa: E402


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_loader_equals_reference_loader(name):
    want = GOLDEN[name]
    if "error" in want:
        with pytest.raises(ValueError, match=want["error"]):
            declarative.load(DOCS / name)
        return
    start = time.perf_counter()
    c, sim = declarative.load(DOCS / name)
    elapsed = time.perf_counter() - start
    assert c.neuron_count == want["neurons"] and c.synapse_count == want["synapses"]
    assert sim.stdp_enabled == want["stdp_enabled"]
    assert digests(canonical_arrays(c)) == want["digests"]
    if "populations" in want:
        assert {k: list(v) for k, v in c.populations.items()} == want["populations"]
    else:
        assert {k: len(v) for k, v in c.populations.items()} == want["populations_sizes"]
        assert elapsed < 60, f"{c.synapse_count} synapses took {elapsed:.1f} s"
    c.validate()


@pytest.mark.skipif(not DUMP.exists(), reason="reference loader not built here")
def test_loader_equals_reference_on_its_own_config():
    ref = pathlib.Path(os.environ.get("SNNCUDA_REFERENCE_DIR", "/root/reference")) / "configs" / "minimal.snncuda.json"
    if not ref.exists():
        pytest.skip("reference configs not present")
    want = record(ref)
    c, sim = declarative.load(ref)
    assert (c.neuron_count, c.synapse_count) == (want["neurons"], want["synapses"])
    assert digests(canonical_arrays(c)) == want["digests"]
    assert {k: list(v) for k, v in c.populations.items()} == want["populations"]


def _drive(c, ticks, seed):
    rng = np.random.default_rng(seed)
    n = rng.integers(0, c.neuron_count, 4 * ticks).astype(np.uint32)
    t = np.sort(rng.integers(0, ticks, n.size)).astype(np.uint64)
    return n, t, np.full(n.size, 0.9, np.float32)


def _run(lib, c, sim_spec, drive, ticks):
    cfg = default_config(lib, raster_capacity=1 << 16)
    cfg.stdp_enabled = 1 if sim_spec.stdp_enabled else 0
    s = Simulation(c, cfg, lib)
    s.inject(*drive)
    s.run_until(ticks - 1)
    out = (s.counters(), s.digest())
    s.close()
    return out


def test_loaded_network_runs_on_the_oracle(port_lib):
    c, spec = declarative.load(DOCS / "hierarchy.snncuda.json")
    counters, _ = _run(port_lib, c, spec, _drive(c, 60, 3), 60)
    assert counters["synaptic_events"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["flat_mixed.snncuda.json", "hierarchy.snncuda.json"])
def test_loaded_network_on_the_gpu_matches_the_oracle(gpu_lib, port_lib, name):
    c, spec = declarative.load(DOCS / name)
    drive = _drive(c, 80, 5)
    got = _run(gpu_lib, c, spec, drive, 80)
    want = _run(port_lib, c, spec, drive, 80)
    assert got[1] == want[1]
    assert got[0]["fired_spikes"] == want[0]["fired_spikes"]
