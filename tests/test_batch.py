"""Batched form: several networks in one handle must each evolve exactly as
they do alone.  The CPU oracle's batch is a list of independent solo
simulations, so comparing the device batch network by network against it
(state digests, counters, fire rasters) checks the batch's isolation and
the per-network STDP rule switch bit for bit."""

import dataclasses

import numpy as np
import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import Batch, SNNCudaError, Simulation, default_config


def _members():
    base = synthetic.STDP_100K
    specs = [
        dict(neurons=400, fanout=30, seed=101),
        dict(neurons=900, fanout=60, seed=102, weight_scale=0.06),
        dict(neurons=250, fanout=12, seed=103, codes=(1, 1)),
        dict(neurons=1500, fanout=40, seed=104, codes=(2, 6), weight_scale=0.05, max_weight=0.1),
        dict(neurons=600, fanout=25, seed=105, max_reference_patterns=3),
        dict(neurons=120, fanout=8, seed=106),
    ]
    out = []
    for k in specs:
        k = {"weight_scale": 0.15, "max_weight": 0.3, **k}
        w = base.scaled(ticks=300, drive_rate_hz=10.0, **k)
        out.append((w, synthetic.build_network(w), synthetic.build_drive(w, 300)))
    # a network without synapses and one without spike-code lists
    w0 = base.scaled(neurons=50, fanout=0, ticks=300, seed=107, weight_scale=0.25, max_weight=1.0)
    out.append((w0, synthetic.build_network(w0), synthetic.build_drive(w0, 300)))
    w1, c1, d1 = out[2]
    out[2] = (w1, dataclasses.replace(c1, code_offset_ptr=None, code_offsets=None), d1)
    return out


@pytest.fixture(scope="module")
def members():
    return _members()


def _config(lib):
    cfg = default_config(lib, raster_capacity=1 << 20)
    cfg.max_weight = 1.0
    return cfg


def _drive_prefix(drive, upto):
    n, t, w = drive
    keep = t < upto
    return n[keep], t[keep], w[keep]


def _drive_rest(drive, frm):
    n, t, w = drive
    keep = t >= frm
    return n[keep], t[keep], w[keep]


def _run_batch(lib, members, rule):
    b = Batch([c for _, c, _ in members], _config(lib), lib, stdp_enabled=rule)
    for i, (_, _, d) in enumerate(members):
        b.inject(i, *_drive_prefix(d, 150))
    b.run_until(99)
    b.set_plasticity(False)          # toggled for every network mid-run
    b.run_until(129)
    b.set_plasticity(True)
    b.set_temporal_learning(False)
    b.run_until(149)
    b.set_temporal_learning(True)
    for i, (_, _, d) in enumerate(members):
        b.inject(i, *_drive_rest(d, 150))
        b.inject(i, [0], [10], [0.7])  # late: clamped to the next tick
    b.run_until(299)
    out = [(b.digests()[i], b.counters(i), b.raster(i)) for i in range(b.count)]
    b.close()
    return out


def _check_equal(got, want):
    for i, ((dg, cg, rg), (dw, cw, rw)) in enumerate(zip(got, want)):
        for key in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events",
                    "pending_events", "next_tick", "raster_count"):
            assert cg[key] == cw[key], (i, key, cg[key], cw[key])
        assert np.array_equal(rg[0], rw[0]) and np.array_equal(rg[1], rw[1]), f"network {i}: raster differs"
        assert dg == dw, f"network {i}: state digest differs"


RULE = [True, False, True, True, False, True, False]


def test_oracle_batch_matches_solo_runs(port_lib, members):
    """The oracle's batch API agrees with driving each network alone."""
    got = _run_batch(port_lib, members, RULE)
    for i, (w, c, d) in enumerate(members):
        cfg = _config(port_lib)
        cfg.stdp_enabled = 1 if RULE[i] else 0
        sim = Simulation(c, cfg, port_lib)
        sim.inject(*_drive_prefix(d, 150))
        sim.run_until(99)
        sim.set_plasticity(False)
        sim.run_until(129)
        sim.set_plasticity(bool(RULE[i]))
        sim.set_temporal_learning(False)
        sim.run_until(149)
        sim.set_temporal_learning(True)
        sim.inject(*_drive_rest(d, 150))
        sim.inject([0], [10], [0.7])
        sim.run_until(299)
        assert sim.digest() == got[i][0]
        assert sim.counters()["fired_spikes"] == got[i][1]["fired_spikes"]
        sim.close()


@pytest.mark.gpu
def test_device_batch_matches_oracle_per_network(gpu_lib, port_lib, members):
    got = _run_batch(gpu_lib, members, RULE)
    want = _run_batch(port_lib, members, RULE)
    assert sum(c["synaptic_events"] for _, c, _ in got) > 10_000
    assert sum(c["fired_spikes"] for _, c, _ in got) > 100
    _check_equal(got, want)


@pytest.mark.gpu
def test_device_batch_matches_device_solo_runs(gpu_lib, members):
    """Solo-vs-mix: a network's results do not depend on its batch mates."""
    got = _run_batch(gpu_lib, members, RULE)
    for i in (0, 3, 6):
        solo = _run_batch(gpu_lib, [members[i]], [RULE[i]])[0]
        _check_equal([got[i]], [solo])


@pytest.mark.gpu
def test_device_batch_readers(gpu_lib, members):
    b = Batch([c for _, c, _ in members[:3]], _config(gpu_lib), gpu_lib, stdp_enabled=RULE[:3])
    for i in range(3):
        b.inject(i, *members[i][2])
    b.run_until(120)
    for i in range(3):
        _, c, d = members[i]
        cfg = _config(gpu_lib)
        cfg.stdp_enabled = 1 if RULE[i] else 0
        sim = Simulation(c, cfg, gpu_lib)
        sim.inject(*d)
        sim.run_until(120)
        bn, sn = b.neurons(i), sim.neurons()
        for k in bn:
            assert np.array_equal(bn[k], sn[k]), (i, k)
        bs, ss = b.synapses(i), sim.synapses()
        for k in bs:
            assert np.array_equal(bs[k], ss[k]), (i, k)
        sim.close()
    b.close()


@pytest.mark.gpu
def test_autotuned_batch_keeps_results_and_checksums_match_solo(gpu_lib, port_lib, members):
    """The autotuner probes launch shapes on the batch's own ticks and
    shrinks the wheel slots: every network still equals its oracle run, and
    the device checksums of each member equal those of its solo run."""
    b = Batch([c for _, c, _ in members], _config(gpu_lib), gpu_lib, stdp_enabled=RULE)
    for i, (_, _, d) in enumerate(members):
        b.inject(i, *d)
    b.run_until(59)
    tuning = b.autotune(probe_ticks=8)
    assert tuning["probes"] >= 5 and tuning["max_slot_events"] > 0
    assert tuning["slot_event_capacity"] >= 2 * tuning["max_slot_events"]
    # the probes run the batch's own ticks: compare at a tick past them
    last = max(299, b.counters(0)["next_tick"] + 40)
    b.run_until(last)
    got = [(b.digests()[i], b.counters(i), b.raster(i)) for i in range(b.count)]
    sums = b.checksums()
    b.close()
    for i, (w, c, d) in enumerate(members):
        cfg = _config(port_lib)
        cfg.stdp_enabled = 1 if RULE[i] else 0
        ref = Simulation(c, cfg, port_lib)
        ref.inject(*d)
        ref.run_until(last)
        assert got[i][0] == ref.digest(), i
        assert got[i][1]["fired_spikes"] == ref.counters()["fired_spikes"], i
        ref.close()
        cfg = _config(gpu_lib)
        cfg.stdp_enabled = 1 if RULE[i] else 0
        solo = Simulation(c, cfg, gpu_lib)
        solo.inject(*d)
        solo.run_until(last)
        assert solo.checksum() == sums[i], i
        solo.close()


@pytest.mark.gpu
def test_slot_capacity_change_keeps_queued_events(gpu_lib, port_lib, members):
    w, c, d = members[3]
    sims = []
    for lib in (gpu_lib, port_lib):
        cfg = _config(lib)
        sim = Simulation(c, cfg, lib)
        sim.inject(*d)
        sim.run_until(100)
        if lib is gpu_lib:
            peak = sim.counters()["max_slot_events"]
            assert lib.snncuda_sim_set_slot_capacity(sim.handle, 2 * peak + 1000) == 0
        sim.run_until(299)
        sims.append(sim)
    assert sims[0].digest() == sims[1].digest()
    assert sims[0].counters()["fired_spikes"] == sims[1].counters()["fired_spikes"]
    for s in sims:
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("side", [0, 1])
def test_applied_tuning_keeps_results(gpu_lib, members, side):
    """A tuning applied by hand (multi-pass grouping with a tiny pass, each
    placement of the temporal update and post-spike STDP, other grid sizes)
    leaves every network's state and raster unchanged; a field outside the
    autotuner's ranges is refused before anything changes."""
    def run(tune):
        b = Batch([c for _, c, _ in members], _config(gpu_lib), gpu_lib, stdp_enabled=RULE)
        for i, (_, _, d) in enumerate(members):
            b.inject(i, *d)
        b.run_until(39)
        if tune:
            t = b.autotune(probe_ticks=2)  # about 70 ticks of probes: done well before tick 299
            assert b.counters(0)["next_tick"] < 250
            t.update(scatter_pass_events=64, side_serial=side, grid_bucket=7, ticks_per_graph=5)
            b.apply_tuning(t)
            bad = dict(t, grid_bucket=10 ** 6)
            with pytest.raises(SNNCudaError):
                b.apply_tuning(bad)
        b.run_until(299)
        out = ([b.digests()[i] for i in range(b.count)], [b.raster(i) for i in range(b.count)], b.checksums())
        b.close()
        return out

    plain, tuned = run(False), run(True)
    assert plain[0] == tuned[0]
    assert plain[2] == tuned[2]
    for x, y in zip(plain[1], tuned[1]):
        assert all(np.array_equal(p, q) for p, q in zip(x, y))
