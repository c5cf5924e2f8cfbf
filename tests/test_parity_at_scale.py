"""Parity at the benchmarked sizes: the GPU backend and the CPU oracle run
the full stdp_100k network (1e5 neurons x 1,000 synapses, 1e8 synapses) and a
1e5-neuron network with the recog_1m distributions (16-code stimulus every
64 ticks over the Poisson background) from the same seed over a tick prefix;
counters, fire rasters, both full state digests and the recognition sums
must be identical.  The oracle runs in a second thread while the GPU runs."""

import threading

import numpy as np
import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import Simulation, default_config

pytestmark = pytest.mark.gpu


def _run(lib, w, net, drive, ticks, out):
    cfg = default_config(lib, raster_capacity=1 << 26)
    cfg.stdp_enabled = 1
    cfg.max_weight = 1.0  # StdpConfig clip [0, 1]; synapses carry their own max_weight
    sim = Simulation(net, cfg, lib)
    n, t, wt = drive
    keep = t < ticks
    sim.inject(n[keep], t[keep], wt[keep])
    sim.run_until(ticks - 1)
    out.update(counters=sim.counters(), raster=sim.raster(), digest=sim.digest(), recognition=sim.recognition())
    sim.close()


def _check(gpu_lib, port_lib, w, ticks):
    net = synthetic.build_network(w)
    drive = synthetic.build_drive(w, ticks)
    cpu, gpu = {}, {}
    th = threading.Thread(target=_run, args=(port_lib, w, net, drive, ticks, cpu))
    th.start()
    _run(gpu_lib, w, net, drive, ticks, gpu)
    th.join()
    assert cpu, "oracle run failed"
    for k in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "pending_events"):
        assert gpu["counters"][k] == cpu["counters"][k], k
    assert np.array_equal(gpu["raster"][0], cpu["raster"][0])
    assert np.array_equal(gpu["raster"][1], cpu["raster"][1])
    assert gpu["digest"] == cpu["digest"]
    assert gpu["recognition"] == cpu["recognition"]
    return gpu


@pytest.mark.timeout(900)
def test_full_stdp_100k_prefix(gpu_lib, port_lib):
    g = _check(gpu_lib, port_lib, synthetic.STDP_100K, 60)
    assert g["counters"]["synaptic_events"] > 40_000_000 and g["counters"]["fired_spikes"] > 10_000


@pytest.mark.timeout(900)
def test_recognition_network_at_1e5_neurons_prefix(gpu_lib, port_lib):
    w = synthetic.RECOG_1M.scaled(name="recog_100k", neurons=100_000)
    g = _check(gpu_lib, port_lib, w, 100)
    assert g["recognition"]["neuron_matches"] > 0 and g["recognition"]["synapse_code_matches"] > 0
