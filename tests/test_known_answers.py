"""The reference runtime's own tests, restated through the reference-shaped
NetworkPropagator interface and run on the CPU oracle and on the GPU backend.
Each test cites the reference test it restates."""

import numpy as np
import pytest

from scenarios import SCENARIOS, _i
from snncuda_gb300 import SNNCudaError
from snncuda_gb300.simulation import NetworkPropagator, Simulation, default_config

BACKENDS = [pytest.param("port", id="oracle"), pytest.param("gpu", id="gpu", marks=pytest.mark.gpu)]


@pytest.fixture(params=BACKENDS)
def lib(request):
    return request.getfixturevalue("port_lib" if request.param == "port" else "gpu_lib")


def propagator(name_or_net, lib, capacity=8, slots=8, **cfg):
    net = SCENARIOS[name_or_net]().net if isinstance(name_or_net, str) else name_or_net
    return net, NetworkPropagator(net, None, capacity, slots, config=default_config(lib, **cfg), lib=lib)


def test_three_stage_spike_propagation(lib):
    """propagation_tests.cpp:144-174"""
    net, p = propagator("three_stage", lib, 1, 8)
    inp, hid, out = (net.populations[k][0] for k in ("input", "hidden", "output"))
    p.inject(inp, 0, 1.0)
    p.run_until(0)
    assert (p.spike_count(inp), p.spike_count(hid), p.spike_count(out)) == (1, 0, 0)
    p.run_until(2)
    assert (p.spike_count(hid), p.spike_count(out)) == (1, 0)
    p.run_until(5)
    assert p.spike_count(out) == 1 and p.idle()
    for nid in (inp, hid, out):
        assert p.state(nid).membrane_potential == 0.0


def test_synapse_spike_code_pattern_propagates_and_matches(lib):
    """propagation_tests.cpp:92-142"""
    net, p = propagator("spike_code_02", lib, 2, 32)
    src = net.populations["source"][0]
    p.inject(src, 0, 1.0)
    p.inject(src, 20, 1.0)
    p.run_until(25)
    s = p.synapse_state(1)
    assert s is not None and s.spike_code_offsets == [0, 2]
    assert s.pre_spike_count == 4
    assert len(s.learned_code_patterns) >= 1 and s.code_match_count >= 1
    assert p.delivered_spike_count() == 6


def test_subthreshold_spike_does_not_propagate(lib):
    """propagation_tests.cpp:176-193"""
    net, p = propagator("subthreshold", lib, 2, 8)
    inp = net.populations["input"][0]
    p.inject(inp, 0, 0.5)
    p.run_until(10)
    assert sum(p.spike_count(i) for i in (1, 2, 3)) == 0
    assert p.state(inp).membrane_potential == 0.5 and p.idle()


def test_spike_enters_dendritic_compartment_before_soma(lib):
    """synapse_dendrite_tests.cpp:137-160"""
    net, p = propagator("apical", lib, 8, 8)
    p.inject(net.populations["input"][0], 0, 1.0)
    p.run_until(1)
    t = p.state(net.populations["target"][0])
    assert p.spike_count(t.id) == 0
    assert abs(t.soma.current) < 1e-4 and abs(t.apical.current - 0.6) < 1e-4
    assert abs(t.membrane_potential - 0.6) < 1e-4
    assert p.synapse_state(1).pre_spike_count == 1


def test_inhibitory_receptor_and_decay(lib):
    """synapse_dendrite_tests.cpp:162-187"""
    net, p = propagator("gaba_decay", lib, 8, 16)
    tgt = net.populations["target"][0]
    p.inject(net.populations["input"][0], 0, 1.0)
    p.run_until(1)
    inhibited = p.state(tgt)
    assert inhibited.inhibitory.current < -0.79 and inhibited.membrane_potential < 0.0
    assert p.spike_count(tgt) == 0
    p.inject(tgt, 11, 0.0)
    p.run_until(11)
    decayed = p.state(tgt)
    assert inhibited.inhibitory.current < decayed.inhibitory.current < 0.0


def test_post_after_pre_potentiates_synapse(lib):
    """synapse_dendrite_tests.cpp:189-210"""
    net, p = propagator("ltp", lib, 8, 8)
    p.inject(net.populations["input"][0], 0, 1.0)
    p.run_until(1)
    assert p.spike_count(net.populations["target"][0]) == 1
    s = p.synapse_state(1)
    assert s.weight > 0.5 and s.plasticity_update_count == 1


def test_pre_after_post_depresses_synapse(lib):
    """synapse_dendrite_tests.cpp:212-236"""
    net, p = propagator("ltd", lib, 8, 16)
    tgt = net.populations["target"][0]
    p.inject(tgt, 0, 1.0)
    p.run_until(0)
    assert p.spike_count(tgt) == 1
    p.inject(net.populations["input"][0], 5, 1.0)
    p.run_until(6)
    assert p.synapse_state(1).weight < 0.5 and p.spike_count(tgt) == 1


def test_temporal_pattern_state_learns_and_matches(lib):
    """synapse_dendrite_tests.cpp:238-259"""
    net, p = propagator("temporal_pattern", lib, 4, 64)
    t = net.populations["target"][0]
    p.inject(t, 10, 0.1)
    p.inject(t, 12, 0.1)
    p.run_until(12)
    st = p.state(t)
    assert len(st.temporal_pattern.learned_patterns) == 1 and st.temporal_pattern.match_count == 0
    p.inject(t, 30, 0.1)
    p.inject(t, 32, 0.1)
    p.run_until(32)
    st = p.state(t)
    assert st.temporal_pattern.last_match and st.temporal_pattern.match_count == 1


def test_state_paging_under_tiny_resident_capacity(lib):
    """synapse_dendrite_tests.cpp:261-276: a resident capacity of one neuron
    changes nothing about the results."""
    net, p = propagator("lru_paging", lib, 1, 8)
    p.inject(net.populations["input"][0], 0, 1.0)
    p.run_until(1)
    assert p.spike_count(1) == 1 and p.spike_count(2) == 1
    # no paging here: every neuron stays resident in device memory
    assert p.cache_eviction_count() == 0 and p.resident_neuron_count() == 2


def test_late_injection_is_clamped_to_next_tick(lib):
    """smoke_tests.cpp:344-368 through the runtime: wrapped and late events."""
    net, p = propagator("late_clamp", lib, 4, 4)
    p.inject(1, 3, 1.0)
    p.inject(2, 1, 1.0)
    p.inject(3, 7, 1.0)
    p.run_until(1)
    assert p.delivered_spike_count() == 1 and p.state(2).last_active_tick == 1
    p.run_until(6)
    assert p.delivered_spike_count() == 2 and p.state(1).last_active_tick == 3
    p.run_until(7)
    assert p.delivered_spike_count() == 3 and p.idle()
    p.inject(4, 2, 1.0)   # late: delivered at the next poll
    p.run_until(8)
    assert p.delivered_spike_count() == 4 and p.state(4).last_active_tick == 8


def test_learning_temporal_experiment(lib):
    """learning_temporal_experiment.cpp:125-194 (prints trained_plastic_weight=0.630242)."""
    net, p = propagator("learning_temporal", lib, 2, 256)
    cue, det, ro, probe = (net.populations[k][0] for k in ("cue", "detector", "readout", "temporal_probe"))
    initial = p.synapse_state(1).weight
    p.inject(cue, 0, 1.0)
    p.run_until(3)
    assert p.spike_count(det) == 0 and p.spike_count(ro) == 0
    for epoch in range(35):
        base = 20 + 100 * epoch
        p.inject(cue, base, 1.0)
        p.inject(det, base + 2, 1.0)
        p.run_until(base + 4)
    trained = p.synapse_state(1).weight
    assert trained > initial and trained >= 0.5
    assert abs(trained - 0.630242) < 5e-7
    d0, r0 = p.spike_count(det), p.spike_count(ro)
    test_tick = 20 + 100 * 35 + 20
    p.inject(cue, test_tick, 1.0)
    p.run_until(test_tick + 3)
    assert p.spike_count(det) - d0 == 1 and p.spike_count(ro) - r0 == 1
    p.inject(probe, test_tick + 20, 0.1)
    p.inject(probe, test_tick + 22, 0.1)
    p.run_until(test_tick + 22)
    assert len(p.state(probe).temporal_pattern.learned_patterns) == 1
    p.inject(probe, test_tick + 40, 0.1)
    p.inject(probe, test_tick + 42, 0.1)
    p.run_until(test_tick + 42)
    st = p.state(probe).temporal_pattern
    assert st.match_count == 1 and len(st.learned_patterns) == 1


def test_consistency_network(lib):
    """cuda_learning_consistency_experiment.cpp:255-297 (CPU side)."""
    sc = SCENARIOS["consistency_43"]()
    net, p = propagator(sc.net, lib, 4, 8192)
    for op in sc.ops:
        if op[0] == "inject":
            p.inject(op[1] + 1, op[2], op[3])
    p.run_until(3543)
    cue, det = net.populations["cue"][0], net.populations["detector"][0]
    plastic = next(i for i in range(net.synapse_count)
                   if net.source[i] == cue - 1 and net.target[i] == det - 1)
    assert p.synapse_state(plastic + 1).weight > 0.5
    assert p.state(net.populations["temporal_probe"][0]).temporal_pattern.match_count >= 1


def test_network_learning_accuracy_training_run(lib):
    """network_learning_accuracy_experiment.cpp:196-220; the reference prints
    delivered_spikes=560, fired_spikes=300 and class-0 weights
    0.699728 / 0.64159 / 0.0809823 / 0.0820542."""
    sc = SCENARIOS["learning_accuracy"]()
    net, p = propagator(sc.net, lib, 8, 4096)
    for op in sc.ops:
        if op[0] == "inject":
            p.inject(op[1] + 1, op[2], op[3])
        elif op[0] == "run":
            p.run_until(op[1])
    assert p.delivered_spike_count() == 560 and p.fired_spike_count() == 300
    class0 = net.populations["class0"][0]
    w = [p.synapse_state(i + 1).weight for i in range(net.synapse_count) if net.target[i] == class0 - 1]
    assert np.allclose(w, [0.699728, 0.64159, 0.0809823, 0.0820542], rtol=0, atol=6e-7)


def test_spike_throughput_network(lib):
    """spike_throughput_benchmark.cpp:137-210: delivered == fired == 27,648."""
    sc = SCENARIOS["throughput_27k"]()
    sim = Simulation(sc.net, default_config(lib, timing_wheel_slots=1024), lib)
    op = sc.ops[0]
    sim.inject(op[1], op[2], op[3])
    sim.run_until(6)
    c = sim.counters()
    assert c["delivered_spikes"] == c["fired_spikes"] == 27648


def test_disabled_stdp_freezes_but_still_clamps(lib):
    """STDP.cpp:20-40 / smoke_tests.cpp:136-154: a disabled rule adds no delta,
    but apply() still clamps the weight into [min, min(max, synapse max)]."""
    from snncuda_gb300.connectome import NetworkBuilder, NeuronParams, Projection
    b = NetworkBuilder()
    b.neuron_params["t"] = NeuronParams(threshold=0.3)
    b.add_population("pre", 1).add_population("post", 1, "t")
    b.projections.append(Projection("pre", "post", "one_to_one", 2.5, 1.2, 1))   # above its max
    net = b.build()
    sim = Simulation(net, default_config(lib, stdp_enabled=0), lib)
    sim.inject([0, 0], [0, 3], [1.0, 1.0])
    sim.run_until(5)
    syn = sim.synapses()
    assert syn["weight"][0] == np.float32(1.2)          # clamped, no delta
    assert syn["plasticity_update_count"][0] == 1        # only the clamp changed it
    sim.set_plasticity(True)
    sim.inject([0], [6], [1.0])
    sim.run_until(8)
    # pre at 6 arrives at 7: LTD against the post spike at 4, then the post
    # spike at 7 gives LTP (dt = 1)
    expected = np.float32(np.float32(1.2) + np.float32(-0.012 * np.exp(-2 / 20)))
    expected = np.float32(expected + np.float32(0.01 * np.exp(-1 / 20)))
    syn = sim.synapses()
    assert abs(syn["weight"][0] - expected) < 1e-6
    assert syn["plasticity_update_count"][0] == 3


def test_invalid_arguments_are_rejected(lib):
    """SpikeScheduler.cpp:10-12 (zero wheel slots) and bad inputs."""
    net = SCENARIOS["three_stage"]().net
    with pytest.raises(SNNCudaError) as err:
        Simulation(net, default_config(lib, timing_wheel_slots=0), lib)
    assert err.value.status == 1
    bad = net.copy_arrays()
    bad.max_reference_patterns[:] = 0
    with pytest.raises(SNNCudaError):
        Simulation(bad, default_config(lib), lib)
    sim = Simulation(net, default_config(lib), lib)
    with pytest.raises(SNNCudaError):
        sim.inject([7], [0], [1.0])
