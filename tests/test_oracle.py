"""The CPU oracle restatement is pinned to the reference runtime: every
scenario (the reference test networks and seeded synthetic workloads) must
reproduce the committed golden fixtures, which were recorded from the
reference's own sources (tests/golden/make_golden.py)."""

import json
import pathlib

import pytest

from scenarios import SCENARIOS, run_scenario
from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import Simulation, default_config

GOLDEN = json.loads((pathlib.Path(__file__).parent / "golden" / "scenarios.json").read_text())


def test_golden_covers_every_scenario():
    assert set(GOLDEN) == set(SCENARIOS)


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_port_matches_reference_golden(port_lib, name):
    got = run_scenario(name, port_lib)
    assert got == GOLDEN[name]


@pytest.mark.parametrize("name", ["spike_code_02", "edge_cases", "toggles"])
def test_reference_harness_reproduces_golden(ref_lib, name):
    assert run_scenario(name, ref_lib) == GOLDEN[name]


def test_reference_printed_goldens():
    """Values the reference experiments print
    (network_learning_accuracy_experiment, spike_throughput_benchmark)."""
    assert GOLDEN["learning_accuracy"]["probes"][-1]["delivered_spikes"] == 560
    assert GOLDEN["learning_accuracy"]["probes"][-1]["fired_spikes"] == 300
    last = GOLDEN["throughput_27k"]["probes"][-1]
    assert last["delivered_spikes"] == last["fired_spikes"] == 27648


def test_planted_mistake_is_caught(port_lib):
    """A deliberately wrong oracle run (one extra input) must not match."""
    from scenarios import SCENARIOS as S
    sc = S["three_stage"]()
    from snncuda_gb300.simulation import Simulation, default_config
    sim = Simulation(sc.net, default_config(port_lib, timing_wheel_slots=8), port_lib)
    sim.inject(0, 0, 1.0)
    sim.inject(1, 1, 0.25)  # planted
    sim.run_until(5)
    nd, sd = sim.digest()
    assert f"{nd:016x}" != GOLDEN["three_stage"]["probes"][-1]["neuron_digest"]


def test_port_matches_reference_on_stdp_network(port_lib, ref_lib):
    """At the size the GPU parity tests use against the port: 5,000 neurons,
    fan-out 1,000 (5e6 synapses), the stdp_100k distributions, 200 ticks
    (~1.2e7 synaptic events) -- the port equals the reference runtime."""
    w = synthetic.STDP_100K.scaled(neurons=5_000, fanout=1000, weight_scale=0.01, max_weight=1.0, seed=21)
    net = synthetic.build_network(w)
    drive = synthetic.build_drive(w, 200)
    out = []
    for lib in (port_lib, ref_lib):
        sim = Simulation(net, default_config(lib, max_weight=1.0), lib)
        sim.inject(*drive)
        sim.run_until(199)
        out.append((sim.counters(), sim.digest()))
        sim.close()
    assert out[0][0]["synaptic_events"] > 1_000_000
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]
