"""Eviction (engine extension, the device-residency counterpart of the
reference's NeuronStateCache write-back and reload, NeuronStateCache.cpp:
22-43): a simulation's state moves to host memory and back between runs
without changing any result."""

import numpy as np
import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import Simulation, default_config

pytestmark = pytest.mark.gpu


def _sim(lib, net, drive):
    cfg = default_config(lib, raster_capacity=1 << 20)
    cfg.stdp_enabled = 1
    cfg.max_weight = 1.0
    sim = Simulation(net, cfg, lib)
    sim.inject(*drive)
    return sim


def _residency(lib, sim):
    import ctypes
    r, n = ctypes.c_int32(), ctypes.c_uint64()
    assert lib.snncuda_sim_residency(sim.handle, ctypes.byref(r), ctypes.byref(n)) == 0
    return r.value, n.value


def test_evict_and_restore_keep_results_exact(gpu_lib, port_lib):
    w = synthetic.RECOG_1M.scaled(neurons=4000, fanout=150, weight_scale=0.04, max_weight=0.2, seed=41, ticks=260)
    net = synthetic.build_network(w)
    drive = synthetic.build_drive(w)
    ref = _sim(port_lib, net, drive)
    ref.run_until(w.ticks - 1)
    sim = _sim(gpu_lib, net, drive)
    sim.run_until(99)
    assert gpu_lib.snncuda_sim_evict(sim.handle) == 0
    assert _residency(gpu_lib, sim) == (0, 1)
    assert gpu_lib.snncuda_sim_restore(sim.handle) == 0
    assert _residency(gpu_lib, sim) == (1, 1)
    sim.run_until(179)
    assert gpu_lib.snncuda_sim_evict(sim.handle) == 0
    # a run on an evicted simulation brings its state back first
    sim.run_until(w.ticks - 1)
    assert _residency(gpu_lib, sim) == (1, 2)
    cg, co = sim.counters(), ref.counters()
    for k in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "pending_events"):
        assert cg[k] == co[k], k
    rg, ro = sim.raster(), ref.raster()
    assert np.array_equal(rg[0], ro[0]) and np.array_equal(rg[1], ro[1])
    assert sim.digest() == ref.digest()
    assert sim.recognition() == ref.recognition()
    # readers of an evicted simulation restore it too
    assert gpu_lib.snncuda_sim_evict(sim.handle) == 0
    assert sim.counters()["fired_spikes"] == co["fired_spikes"]
    assert _residency(gpu_lib, sim) == (1, 3)
    sim.close()
    ref.close()


def test_evicted_simulation_frees_device_memory(gpu_lib):
    import torch
    w = synthetic.STDP_100K.scaled(neurons=20_000, fanout=500, seed=42)
    net = synthetic.build_network(w)
    sim = _sim(gpu_lib, net, synthetic.build_drive(w, 60))
    sim.run_until(59)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    assert gpu_lib.snncuda_sim_evict(sim.handle) == 0
    torch.cuda.synchronize()
    after = torch.cuda.mem_get_info()[0]
    # 1e7 synapse records of 64 B alone are 640 MB
    assert after - before > 500e6, (before, after)
    sim.close()
