"""GPU backend parity: bit-identical to the reference on every scenario
(golden fixtures recorded from the reference sources) and to the CPU oracle
on larger seeded networks; device-side capacity errors surface as status
codes."""

import json
import pathlib

import numpy as np
import pytest

from scenarios import SCENARIOS, STDP_CFG, run_scenario
from snncuda_gb300 import SNNCudaError, synthetic
from snncuda_gb300.simulation import Simulation, default_config

GOLDEN = json.loads((pathlib.Path(__file__).parent / "golden" / "scenarios.json").read_text())

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_gpu_matches_reference_golden(gpu_lib, name):
    assert run_scenario(name, gpu_lib) == GOLDEN[name]


def _compare(gpu_lib, port_lib, net, drive, ticks, cfg, *, toggles=()):
    results = []
    for lib in (gpu_lib, port_lib):
        c = default_config(lib, raster_capacity=1 << 24, **cfg)
        sim = Simulation(net, c, lib)
        sim.inject(*drive)
        last = 0
        for tick, what, value in list(toggles) + [(ticks - 1, None, None)]:
            sim.run_until(tick)
            if what == "stdp":
                sim.set_plasticity(value)
            elif what == "temporal":
                sim.set_temporal_learning(value)
        results.append((sim.counters(), sim.digest(), sim.raster(), sim.neurons(), sim.synapses()))
        sim.close()
    (cg, dg, rg, ng, sg), (co, do, ro, no, so) = results
    for k in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "pending_events"):
        assert cg[k] == co[k], k
    assert np.array_equal(rg[0], ro[0]) and np.array_equal(rg[1], ro[1])
    for k in ng:
        assert np.array_equal(ng[k], no[k]), k
    for k in sg:
        assert np.array_equal(sg[k], so[k]), k
    assert dg == do
    return cg


@pytest.mark.parametrize("neurons,fanout,ticks,g", [(20_000, 200, 300, 0.05), (5_000, 1000, 200, 0.01)])
def test_stdp_network_matches_oracle(gpu_lib, port_lib, neurons, fanout, ticks, g):
    w = synthetic.STDP_100K.scaled(neurons=neurons, fanout=fanout, weight_scale=g, max_weight=1.0, seed=21)
    net = synthetic.build_network(w)
    c = _compare(gpu_lib, port_lib, net, synthetic.build_drive(w, ticks), ticks, STDP_CFG)
    assert c["synaptic_events"] > 100_000


def test_recognition_network_with_toggles_matches_oracle(gpu_lib, port_lib):
    w = synthetic.RECOG_1M.scaled(neurons=10_000, fanout=200, weight_scale=0.03, max_weight=1.0, seed=23,
                                  stimulus_weight=0.25)
    net = synthetic.build_network(w)
    _compare(gpu_lib, port_lib, net, synthetic.build_drive(w, 300), 300, STDP_CFG,
             toggles=[(99, "stdp", False), (149, "temporal", False), (199, "stdp", True),
                      (249, "temporal", True)])


def test_slot_overflow_is_reported_and_poisons(gpu_lib):
    w = synthetic.PLAIN_1K
    net = synthetic.build_network(w)
    sim = Simulation(net, default_config(gpu_lib, slot_event_capacity=64), gpu_lib)
    sim.inject(*synthetic.build_drive(w, 200))
    with pytest.raises(SNNCudaError) as err:
        sim.run_until(199)
    assert err.value.status == 3
    with pytest.raises(SNNCudaError) as err:
        sim.run_until(300)
    assert err.value.status == 7
    assert sim.counters()["next_tick"] >= 0   # readers still work


@pytest.mark.gpu
def test_recognition_sums_match_oracle(gpu_lib, port_lib):
    """Device-reduced recognition sums (neuron temporal matches, synapse code
    matches) on the recognition workload's distributions."""
    w = synthetic.RECOG_1M.scaled(neurons=3000, fanout=80, weight_scale=0.05, max_weight=0.2, seed=31, ticks=300)
    net = synthetic.build_network(w)
    drive = synthetic.build_drive(w, 300)
    got = []
    for lib in (gpu_lib, port_lib):
        sim = Simulation(net, default_config(lib, max_weight=1.0), lib)
        sim.inject(*drive)
        sim.run_until(299)
        got.append(sim.recognition())
        n, s = sim.neurons(), sim.synapses()
        assert got[-1]["neuron_matches"] == int(n["match_count"].sum())
        assert got[-1]["synapse_code_matches"] == int(s["code_match_count"].sum())
        sim.close()
    assert got[0] == got[1]
    assert got[0]["neuron_matches"] > 0 and got[0]["synapse_code_matches"] > 0
