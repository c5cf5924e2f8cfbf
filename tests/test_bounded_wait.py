"""The tick's bounded device waits: k_process waits for the bulk copy of its
block's event inputs into shared memory, and the grouping's counting and
placing blocks for the bulk copies of their due-list tiles, each for at most
snncuda_config.stage_wait_ns.  With a limit of 0 every wait gives up at once:
the blocks read their inputs from global memory instead, so the results stay
bit-exact with the oracle, and the run reports SNNCUDA_ERR_TIMEOUT and
poisons the handle.  Nothing faults or hangs: the copies still complete and
are drained (with a bounded wait) before their buffers are reused."""

import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import SNNCudaError, Simulation, default_config

pytestmark = pytest.mark.gpu

SNNCUDA_ERR_TIMEOUT = 5
SNNCUDA_ERR_POISONED = 7


def _run(lib, net, drive, ticks, **cfg_fields):
    cfg = default_config(lib, raster_capacity=1 << 20, **cfg_fields)
    cfg.stdp_enabled = 1
    cfg.max_weight = 1.0
    sim = Simulation(net, cfg, lib)
    sim.inject(*drive)
    return sim


def test_wait_that_gives_up_keeps_results_exact(gpu_lib, port_lib):
    w = synthetic.STDP_100K.scaled(neurons=3000, fanout=200, ticks=80, weight_scale=0.05, max_weight=0.05,
                                   seed=5)
    net = synthetic.build_network(w)
    drive = synthetic.build_drive(w)
    ref = _run(port_lib, net, drive, w.ticks)
    ref.run_until(w.ticks - 1)
    gpu = _run(gpu_lib, net, drive, w.ticks, stage_wait_ns=0)
    with pytest.raises(SNNCudaError) as err:
        gpu.run_until(w.ticks - 1)
    assert err.value.status == SNNCUDA_ERR_TIMEOUT
    with pytest.raises(SNNCudaError) as err:
        gpu.run_until(w.ticks)
    assert err.value.status == SNNCUDA_ERR_POISONED
    # the readers keep working and every tick ran with exact results
    cg, co = gpu.counters(), ref.counters()
    assert cg["synaptic_events"] > 0 and cg["fired_spikes"] > 0
    for key in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "next_tick"):
        assert cg[key] == co[key], key
    rg, ro = gpu.raster(), ref.raster()
    assert (rg[0] == ro[0]).all() and (rg[1] == ro[1]).all()
    assert gpu.digest() == ref.digest()
    gpu.close()
    ref.close()
