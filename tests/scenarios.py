"""Parity scenarios: networks plus scripts of runtime calls.

Each scenario restates a network and driving sequence from the reference
project's own tests (paths relative to the reference project), or a seeded
synthetic workload.  `run_scenario` drives any library implementing the C ABI
(the GPU backend, the CPU oracle port, the reference harness) through the
same calls and records counters, state digests, the fire raster and
intermediate probes, so results can be compared bit for bit and against the
committed golden fixtures in tests/golden/.
"""

from __future__ import annotations

import hashlib
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Tuple

import numpy as np

from snncuda_gb300 import synthetic
from snncuda_gb300.connectome import (AMPA, APICAL, BASAL, GABA_A, INHIBITORY, SOMA, Connectome,
                                      NetworkBuilder, NeuronParams, Projection)
from snncuda_gb300.simulation import Simulation, default_config

RASTER_CAPACITY = 1 << 22


@dataclass
class Scenario:
    net: Connectome
    ops: List[tuple]
    config: Dict = field(default_factory=dict)
    default_processor: bool = True   # the reference NetworkPropagator can run it as-is
    note: str = ""


def _two_neuron(threshold, weight, compartment=BASAL, receptor=AMPA, plastic=False):
    """synapse_dendrite_tests.cpp:24-91"""
    b = NetworkBuilder()
    b.neuron_params["input"] = NeuronParams(threshold=1.0)
    b.neuron_params["target"] = NeuronParams(threshold, 10, 0.99, 4)
    b.add_population("input", 1, "input").add_population("target", 1, "target")
    b.projections.append(Projection("input", "target", "one_to_one", weight, 2.0, 1, (0,), compartment,
                                    receptor, plastic))
    return b.build()


def _three_stage():
    """propagation_tests.cpp:16-90"""
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(1.0, 10, 0.9, 4)
    b.add_population("input", 1).add_population("hidden", 1).add_population("output", 1)
    b.projections.append(Projection("input", "hidden", "one_to_one", 1.0, 2.0, 2))
    b.projections.append(Projection("hidden", "output", "one_to_one", 1.0, 2.0, 3))
    return b.build()


def _i(net, pop, k=0):
    """0-based index of population member k."""
    return net.populations[pop][k] - 1


PROBE = ("probe",)


def sc_three_stage():
    """propagation_tests.cpp:144-174"""
    net = _three_stage()
    inp = _i(net, "input")
    return Scenario(net, [("inject", inp, 0, 1.0), ("run", 0), PROBE, ("run", 2), PROBE, ("run", 5), PROBE],
                    {"timing_wheel_slots": 8})


def sc_spike_code_02():
    """propagation_tests.cpp:92-142"""
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(1.0, 10, 0.9, 4)
    b.neuron_params["sink"] = NeuronParams(100.0, 8, 0.99, 4)
    b.add_population("source", 1).add_population("sink", 1, "sink")
    b.projections.append(Projection("source", "sink", "one_to_one", 0.1, 2.0, 1, (0, 2)))
    net = b.build()
    src = _i(net, "source")
    return Scenario(net, [("inject", src, 0, 1.0), ("inject", src, 20, 1.0), ("run", 25), PROBE],
                    {"timing_wheel_slots": 32})


def sc_subthreshold():
    """propagation_tests.cpp:176-193"""
    net = _three_stage()
    return Scenario(net, [("inject", _i(net, "input"), 0, 0.5), ("run", 10), PROBE], {"timing_wheel_slots": 8})


def sc_apical():
    """synapse_dendrite_tests.cpp:137-160"""
    net = _two_neuron(1.0, 0.6, APICAL)
    return Scenario(net, [("inject", _i(net, "input"), 0, 1.0), ("run", 1), PROBE], {"timing_wheel_slots": 8})


def sc_gaba_decay():
    """synapse_dendrite_tests.cpp:162-187"""
    net = _two_neuron(0.2, 0.8, INHIBITORY, GABA_A)
    return Scenario(net, [("inject", _i(net, "input"), 0, 1.0), ("run", 1), PROBE,
                          ("inject", _i(net, "target"), 11, 0.0), ("run", 11), PROBE],
                    {"timing_wheel_slots": 16})


def sc_ltp():
    """synapse_dendrite_tests.cpp:189-210"""
    net = _two_neuron(0.4, 0.5, BASAL, AMPA, True)
    return Scenario(net, [("inject", _i(net, "input"), 0, 1.0), ("run", 1), PROBE], {"timing_wheel_slots": 8})


def sc_ltd():
    """synapse_dendrite_tests.cpp:212-236"""
    net = _two_neuron(1.0, 0.5, BASAL, AMPA, True)
    return Scenario(net, [("inject", _i(net, "target"), 0, 1.0), ("run", 0), PROBE,
                          ("inject", _i(net, "input"), 5, 1.0), ("run", 6), PROBE],
                    {"timing_wheel_slots": 16})


def sc_temporal_pattern():
    """synapse_dendrite_tests.cpp:238-259"""
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(10.0, 10, 0.99, 2)
    b.add_population("target", 1)
    net = b.build()
    t = _i(net, "target")
    return Scenario(net, [("inject", t, 10, 0.1), ("inject", t, 12, 0.1), ("run", 12), PROBE,
                          ("inject", t, 30, 0.1), ("inject", t, 32, 0.1), ("run", 32), PROBE],
                    {"timing_wheel_slots": 64})


def sc_lru_paging():
    """synapse_dendrite_tests.cpp:261-276 (paging never changes results)"""
    net = _two_neuron(0.4, 0.5)
    return Scenario(net, [("inject", _i(net, "input"), 0, 1.0), ("run", 1), PROBE], {"timing_wheel_slots": 8})


def sc_late_clamp():
    """smoke_tests.cpp:344-368 through the runtime API: wrapped and late events"""
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(100.0, 16, 0.9, 4)
    b.add_population("n", 4)
    net = b.build()
    return Scenario(net, [("inject", 0, 3, 1.0), ("inject", 1, 1, 1.0), ("inject", 2, 7, 1.0), ("run", 1), PROBE,
                          ("run", 6), PROBE, ("run", 7), PROBE, ("inject", 3, 2, 1.0), ("run", 8), PROBE],
                    {"timing_wheel_slots": 4})


def _learning_temporal_net():
    """learning_temporal_experiment.cpp:17-112"""
    b = NetworkBuilder()
    b.neuron_params["input"] = NeuronParams(threshold=1.0)
    b.neuron_params["detector"] = NeuronParams(0.5, 12, 0.99, 8)
    b.neuron_params["readout"] = NeuronParams(threshold=0.5)
    b.neuron_params["temporal"] = NeuronParams(10.0, 8, 0.99, 4)
    for name, params in (("cue", "input"), ("detector", "detector"), ("readout", "readout"),
                         ("temporal_probe", "temporal")):
        b.add_population(name, 1, params)
    b.projections.append(Projection("cue", "detector", "one_to_one", 0.25, 1.5, 1, (0,), BASAL, AMPA, True))
    b.projections.append(Projection("detector", "readout", "one_to_one", 0.75, 1.0, 1, (0,), BASAL, AMPA, False))
    return b.build()


def sc_learning_temporal():
    """learning_temporal_experiment.cpp:125-194"""
    net = _learning_temporal_net()
    cue, det, probe = _i(net, "cue"), _i(net, "detector"), _i(net, "temporal_probe")
    ops = [("inject", cue, 0, 1.0), ("run", 3), PROBE]
    for epoch in range(35):
        base = 20 + 100 * epoch
        ops += [("inject", cue, base, 1.0), ("inject", det, base + 2, 1.0), ("run", base + 4)]
    ops.append(PROBE)
    test_tick = 20 + 100 * 35 + 20
    ops += [("inject", cue, test_tick, 1.0), ("run", test_tick + 3), PROBE,
            ("inject", probe, test_tick + 20, 0.1), ("inject", probe, test_tick + 22, 0.1),
            ("run", test_tick + 22), PROBE,
            ("inject", probe, test_tick + 40, 0.1), ("inject", probe, test_tick + 42, 0.1),
            ("run", test_tick + 42), PROBE]
    return Scenario(net, ops, {"timing_wheel_slots": 256})


def sc_consistency_43():
    """cuda_learning_consistency_experiment.cpp:28-248"""
    epochs, spacing = 35, 100
    b = NetworkBuilder()
    b.neuron_params["input"] = NeuronParams(threshold=1.0)
    b.neuron_params["detector"] = NeuronParams(threshold=0.5)
    b.neuron_params["readout"] = NeuronParams(threshold=0.5)
    b.neuron_params["temporal"] = NeuronParams(10.0, 8, 0.99, 1)
    for name, params in (("cue", "input"), ("detector", "detector"), ("readout", "readout"),
                         ("temporal_probe", "temporal")):
        b.add_population(name, 1, params)
    for s in range(4):
        b.add_population(f"temporal_source_{s}", 1, "input")
    for ep in range(epochs):
        b.add_population(f"teacher_{ep}", 1, "input")
    b.projections.append(Projection("cue", "cue", "one_to_one", 1.0, 1.0, spacing, (0,), BASAL, AMPA, False))
    b.projections.append(Projection("cue", "detector", "one_to_one", 0.25, 1.5, 1, (0,), BASAL, AMPA, True))
    b.projections.append(Projection("detector", "readout", "one_to_one", 0.75, 1.0, 1, (0,), BASAL, AMPA, False))
    delays = [3520, 3522, 3540, 3542]
    for s in range(4):
        b.projections.append(Projection(f"temporal_source_{s}", "temporal_probe", "one_to_one", 0.1, 0.1,
                                        delays[s], (0,), SOMA, AMPA, False))
    for ep in range(epochs):
        b.projections.append(Projection(f"teacher_{ep}", "detector", "one_to_one", 1.0, 1.0,
                                        2 + ep * spacing, (0,), SOMA, AMPA, False))
    net = b.build()
    active = [_i(net, "cue")] + [_i(net, f"teacher_{ep}") for ep in range(epochs)] + \
             [_i(net, f"temporal_source_{s}") for s in range(4)]
    ops = [("inject", a, 0, 1.0) for a in active] + [("run", 3543), PROBE]
    return Scenario(net, ops, {"timing_wheel_slots": 8192})


def sc_learning_accuracy():
    """network_learning_accuracy_experiment.cpp:46-146, :157-220 (training run)"""
    b = NetworkBuilder()
    b.neuron_params["input"] = NeuronParams(threshold=1.0)
    b.neuron_params["class"] = NeuronParams(0.45, 16, 0.98, 4)
    b.add_population("input", 4, "input").add_population("class0", 1, "class").add_population("class1", 1, "class")
    for c in ("class0", "class1"):
        b.projections.append(Projection("input", c, "all_to_all", 0.08, 1.2, 1, (0,), BASAL, AMPA, True))
    net = b.build()
    inputs = [_i(net, "input", k) for k in range(4)]
    classes = [_i(net, "class0"), _i(net, "class1")]
    train = [([0, 1], 0), ([2, 3], 1)]
    ops, tick = [], 0
    for _ in range(40):
        for active, label in train:
            for order, k in enumerate(active):
                ops.append(("inject", inputs[k], tick + order % 2, 1.0))
            ops.append(("inject", classes[label], tick + 3, 1.0))
            ops.append(("run", tick + 16))
            tick += 80
        ops.append(PROBE)
    return Scenario(net, ops, {"timing_wheel_slots": 4096})


def sc_throughput_27k():
    """spike_throughput_benchmark.cpp:17-154: 1,728 columns-layers of 16 neurons,
    one-to-one chains L0 -> ... -> L5, every L0 neuron injected at tick 0."""
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(1.0, 16, 0.9, 8)
    names = []
    for h in range(2):
        for lo in range(2):
            for r in range(3):
                for nu in range(3):
                    for c in range(8):
                        col = [f"H{h}_Lo{lo}_R{r}_N{nu}_C{c}_L{layer}" for layer in range(6)]
                        for name in col:
                            b.add_population(name, 16)
                        names.append(col)
    for col in names:
        for layer in range(5):
            b.projections.append(Projection(col[layer], col[layer + 1], "one_to_one", 1.0, 2.0, 1))
    net = b.build()
    l0 = sorted(i - 1 for col in names for i in net.populations[col[0]])
    ops = [("inject", np.array(l0), np.zeros(len(l0), np.uint64), np.ones(len(l0), np.float32)),
           ("run", 6), PROBE]
    return Scenario(net, ops, {"timing_wheel_slots": 1024})


def sc_edge_cases():
    """Duplicate synapses and offsets, zero delay (clamped to the next tick),
    self loops, multiple fires of one neuron inside a tick, far-future and
    late injections across several run_until calls."""
    b = NetworkBuilder()
    b.neuron_params["default"] = NeuronParams(0.3, 6, 0.9, 3)
    b.neuron_params["hub"] = NeuronParams(0.25, 6, 0.8, 2)
    b.add_population("a", 3).add_population("hub", 1, "hub").add_population("z", 2)
    b.projections.append(Projection("a", "hub", "all_to_all", 0.3, 2.0, 0, (0, 0, 1), BASAL, AMPA, True))
    b.projections.append(Projection("a", "hub", "all_to_all", 0.2, 0.5, 2, (1, 3), APICAL, AMPA, True))
    b.projections.append(Projection("hub", "hub", "one_to_one", 0.05, 2.0, 1, (0, 4), SOMA, AMPA, False))
    b.projections.append(Projection("hub", "z", "all_to_all", 0.35, 2.0, 3, (0, 1, 2), INHIBITORY, GABA_A, True))
    b.projections.append(Projection("z", "a", "all_to_all", 0.6, 2.0, 1, (2,), BASAL, AMPA, False))
    net = b.build()
    ops = [("inject", np.array([0, 1, 2, 0]), np.array([0, 0, 0, 1], np.uint64),
            np.array([1.0, 1.0, 1.0, 0.5], np.float32)),
           ("inject", 3, 500, 1.0), ("inject", 4, 9000, 2.0), ("run", 40), PROBE,
           ("inject", 0, 3, 1.0), ("inject", 1, 41, 1.0), ("inject", 2, 300, 1.0), ("run", 700), PROBE,
           ("inject", 5, 8990, 1.0), ("run", 9100), PROBE]
    return Scenario(net, ops, {"timing_wheel_slots": 16})


def _synthetic(w: synthetic.Workload, ticks: int, config: Dict, extra_ops=None):
    net = synthetic.build_network(w)
    n, t, wt = synthetic.build_drive(w, ticks)
    ops = [("inject", n, t, wt)]
    ops += extra_ops if extra_ops else [("run", ticks - 1), PROBE]
    return Scenario(net, ops, config)


def sc_plain_1k():
    """The 1k-neuron plain network (weight scale 0.3), 1,000 ticks."""
    return _synthetic(synthetic.PLAIN_1K, 1000, {})


def _stdp_small():
    return synthetic.STDP_100K.scaled(neurons=2000, fanout=100, weight_scale=0.12, max_weight=1.0, seed=5)


STDP_CFG = {"max_weight": 1.0}


def sc_stdp_2k():
    """stdp_100k distributions at 2,000 neurons x 100, 300 ticks."""
    w = _stdp_small()
    s = _synthetic(w, 300, STDP_CFG)
    s.default_processor = False
    return s


def sc_toggles():
    """STDP and temporal learning switched off and on mid-run."""
    w = _stdp_small()
    ops = [("run", 79), PROBE, ("stdp", False), ("run", 139), PROBE, ("temporal", False), ("run", 179), PROBE,
           ("stdp", True), ("run", 219), ("temporal", True), ("run", 299), PROBE]
    s = _synthetic(w, 300, STDP_CFG, ops)
    s.default_processor = False
    return s


def sc_recog_small():
    """recog_1m distributions (temporal-code stimulus) at 2,000 neurons."""
    w = synthetic.RECOG_1M.scaled(neurons=2000, fanout=100, weight_scale=0.06, max_weight=1.0, seed=9,
                                  stimulus_weight=0.25)
    s = _synthetic(w, 256, STDP_CFG)
    s.default_processor = False
    return s


SCENARIOS: Dict[str, Callable[[], Scenario]] = {
    "three_stage": sc_three_stage,
    "spike_code_02": sc_spike_code_02,
    "subthreshold": sc_subthreshold,
    "apical": sc_apical,
    "gaba_decay": sc_gaba_decay,
    "ltp": sc_ltp,
    "ltd": sc_ltd,
    "temporal_pattern": sc_temporal_pattern,
    "lru_paging": sc_lru_paging,
    "late_clamp": sc_late_clamp,
    "learning_temporal": sc_learning_temporal,
    "consistency_43": sc_consistency_43,
    "learning_accuracy": sc_learning_accuracy,
    "throughput_27k": sc_throughput_27k,
    "edge_cases": sc_edge_cases,
    "plain_1k": sc_plain_1k,
    "stdp_2k": sc_stdp_2k,
    "toggles": sc_toggles,
    "recog_small": sc_recog_small,
}

COUNTER_KEYS = ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "next_tick",
                "pending_events")


def raster_hash(ticks: np.ndarray, neurons: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(ticks, dtype=np.uint64).tobytes())
    h.update(np.ascontiguousarray(neurons, dtype=np.uint32).tobytes())
    return h.hexdigest()


def _snapshot(sim: Simulation, with_raster: bool, with_pending: bool) -> dict:
    c = sim.counters()
    out = {k: c[k] for k in COUNTER_KEYS if with_pending or k != "pending_events"}
    nd, sd = sim.digest()
    out["neuron_digest"] = f"{nd:016x}"
    out["synapse_digest"] = f"{sd:016x}"
    if with_raster:
        t, n = sim.raster()
        out["raster_len"] = int(len(t))
        out["raster_sha256"] = raster_hash(t, n)
    return out


def run_scenario(name: str, lib, *, with_raster: bool = True, with_pending: bool = True,
                 extra_config: Dict = None) -> dict:
    sc = SCENARIOS[name]()
    cfg = default_config(lib, **sc.config)
    if with_raster:
        cfg.raster_capacity = RASTER_CAPACITY
    for k, v in (extra_config or {}).items():
        setattr(cfg, k, v)
    sim = Simulation(sc.net, cfg, lib)
    probes = []
    try:
        for op in sc.ops:
            kind = op[0]
            if kind == "inject":
                sim.inject(op[1], op[2], op[3])
            elif kind == "run":
                sim.run_until(op[1])
            elif kind == "stdp":
                sim.set_plasticity(op[1])
            elif kind == "temporal":
                sim.set_temporal_learning(op[1])
            elif kind == "probe":
                probes.append(_snapshot(sim, with_raster, with_pending))
    finally:
        sim.close()
    return {"probes": probes}
