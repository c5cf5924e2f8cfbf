"""The tick's grouping on a network with hundreds of target buckets, with the
counting and placing grid of its default size and of one block per SM, and
with the due list placed in one pass or in passes of 4,096 events: every run
equals the oracle (digest, counters, raster)."""

import numpy as np
import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import Simulation, default_config

pytestmark = pytest.mark.gpu

TICKS = 60


def _config(lib):
    cfg = default_config(lib, raster_capacity=1 << 22)
    cfg.max_weight = 1.0
    return cfg


@pytest.fixture(scope="module")
def network():
    w = synthetic.STDP_100K.scaled(neurons=60_000, fanout=120, ticks=TICKS, seed=23, weight_scale=0.08,
                                   max_weight=0.08, drive_rate_hz=20.0)
    return w, synthetic.build_network(w), synthetic.build_drive(w, TICKS)


def _run(lib, net, drive, tuning=None):
    sim = Simulation(net, _config(lib), lib)
    if tuning is not None:
        sim.apply_tuning(tuning)
    sim.inject(*drive)
    sim.run_until(TICKS - 1)
    out = (sim.digest(), sim.counters(), sim.raster())
    sim.close()
    return out


def test_grouping_grids_and_passes_match_oracle(gpu_lib, port_lib, network):
    w, net, drive = network
    probe = Simulation(net, _config(gpu_lib), gpu_lib)
    base = probe.autotune(probe_ticks=1)
    probe.close()
    base["slot_event_capacity"] = 0
    runs = {}
    for passes in (0, 4096):
        for grid in (base["grid_bucket"], 152):
            runs[(passes, grid)] = _run(gpu_lib, net, drive, dict(base, scatter_pass_events=passes, grid_bucket=grid))
    ref = _run(port_lib, net, drive)
    assert ref[1]["synaptic_events"] > 100_000
    for key, (digest, counters, raster) in runs.items():
        assert digest == ref[0], key
        for k in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events"):
            assert counters[k] == ref[1][k], (key, k)
        assert np.array_equal(raster[0], ref[2][0]) and np.array_equal(raster[1], ref[2][1]), key
