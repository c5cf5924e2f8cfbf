"""Two-level placement of the tick's due list (coarse buckets, then buckets,
each tile sorted in shared memory before its coalesced writes): the same
grouping as the one-level placement, so results stay equal to the oracle.
The default turns it on only for networks of 2^27+ synapses; here it is
forced on a network with hundreds of buckets (and so 64 coarse buckets of
several buckets each), and compared with the one-level run and the oracle."""

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


def test_two_level_placement_matches_one_level_and_oracle(gpu_lib, port_lib, network):
    w, net, drive = network
    probe = Simulation(net, _config(gpu_lib), gpu_lib)
    base = probe.autotune(probe_ticks=1)
    probe.close()
    base["slot_event_capacity"] = 0
    runs = {}
    for two in (0, 1):
        for grid in (base["grid_bucket"], 152):
            runs[(two, grid)] = _run(gpu_lib, net, drive, dict(base, two_level=two, grid_bucket=grid))
    ref = _run(port_lib, net, drive)
    assert ref[1]["synaptic_events"] > 100_000
    for key, (digest, counters, raster) in runs.items():
        assert digest == ref[0], key
        for k in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events"):
            assert counters[k] == ref[1][k], (key, k)
        assert np.array_equal(raster[0], ref[2][0]) and np.array_equal(raster[1], ref[2][1]), key
