"""Targets that fire inside a tick and keep receiving events: every event
after a fire redoes its STDP with the tick's fire count so far (on the GPU the
warp redoes up to 32 of them at once and the target's own lane runs the
physics over them; a synapse repeated after the fire takes the serial path).
A feed-forward fan-in network makes every such case common: 256 sources that
fire once per tick, all-to-all onto 64 plastic low-threshold targets that fire
several times per tick with hundreds of events after their first fire."""

import numpy as np
import pytest

from snncuda_gb300.connectome import AMPA, APICAL, BASAL, NMDA, NetworkBuilder, NeuronParams, Projection
from snncuda_gb300.simulation import Simulation, default_config

SOURCES, TARGETS, TICKS = 256, 64, 30


def fan_in_network(codes, threshold):
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(1.0, 12, 0.9, 3)
    b.neuron_params["target"] = NeuronParams(threshold, 12, 0.9, 3)
    b.add_population("a", SOURCES).add_population("b", TARGETS, "target")
    b.projections.append(Projection("a", "b", "all_to_all", 0.3, 0.5, 1, codes, BASAL, AMPA, True))
    b.projections.append(Projection("a", "b", "all_to_all", 0.2, 0.5, 2, (0,), APICAL, NMDA, True))
    return b.build()


def drive(net):
    src = np.array(net.populations["a"], np.uint32) - 1
    n = np.tile(src, TICKS)
    t = np.repeat(np.arange(TICKS, dtype=np.uint64), SOURCES)
    return n, t, np.ones(n.size, np.float32)


def run(lib, codes, stdp=True, threshold=3.0):
    net = fan_in_network(codes, threshold)
    cfg = default_config(lib, raster_capacity=1 << 20, max_weight=1.0)
    cfg.stdp_enabled = 1 if stdp else 0
    sim = Simulation(net, cfg, lib)
    sim.inject(*drive(net))
    sim.run_until(TICKS + 3)
    out = (sim.counters(), sim.digest(), sim.raster(), sim.neurons(), sim.synapses())
    sim.close()
    return out


@pytest.mark.parametrize("codes,threshold", [((0,), 3.0), ((0, 1), 40.0)])
def test_oracle_fan_in_has_many_events_after_fires(port_lib, codes, threshold):
    """The network does what the GPU test needs: several fires per target and
    tick (threshold 3: one every ~8 events, so the redone chunks restart
    often; threshold 40: one every ~100, so full chunks of 32 run between
    fires), hundreds of events per target and tick."""
    c = run(port_lib, codes, True, threshold)[0]
    fires_per_target_tick = (c["fired_spikes"] - SOURCES * TICKS) / (TARGETS * TICKS)
    events_per_target_tick = c["synaptic_events"] / (TARGETS * TICKS)
    assert fires_per_target_tick >= 3
    assert events_per_target_tick >= 2 * SOURCES - 8


@pytest.mark.parametrize("codes,threshold", [((0,), 3.0), ((0, 1), 40.0)])
def test_oracle_fan_in_matches_reference(port_lib, ref_lib, codes, threshold):
    """The CPU restatement against the reference runtime built from its own
    sources on the same fan-in network (pins the many-fires-per-tick case)."""
    got, want = run(port_lib, codes, True, threshold), run(ref_lib, codes, True, threshold)
    for k in want[0]:
        assert got[0][k] == want[0][k], k
    assert np.array_equal(got[2][0], want[2][0]) and np.array_equal(got[2][1], want[2][1])
    assert got[1] == want[1]


@pytest.mark.gpu
@pytest.mark.parametrize("codes,stdp,threshold", [((0,), True, 3.0), ((0,), True, 40.0), ((0, 1), True, 40.0),
                                                  ((0, 1), True, 3.0), ((0,), False, 40.0)])
def test_gpu_fan_in_matches_oracle(gpu_lib, port_lib, codes, stdp, threshold):
    got, want = run(gpu_lib, codes, stdp, threshold), run(port_lib, codes, stdp, threshold)
    for k in want[0]:
        assert got[0][k] == want[0][k], k
    assert np.array_equal(got[2][0], want[2][0]) and np.array_equal(got[2][1], want[2][1])
    for k in want[3]:
        assert np.array_equal(got[3][k], want[3][k]), k
    for k in want[4]:
        assert np.array_equal(got[4][k], want[4][k]), k
    assert got[1] == want[1]
