"""Serving: jobs admitted under a device-memory budget and run side by side
must each give exactly the results of a solo run (solo-vs-mix equality),
whatever the admission order, slice length and number of jobs in flight."""

import numpy as np
import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.simulation import Server, Simulation, default_config


def _jobs():
    base = synthetic.RECOG_1M
    specs = [
        dict(neurons=800, fanout=40, seed=301, ticks=150),
        dict(neurons=2000, fanout=60, seed=302, ticks=90, stimulus_codes=0),
        dict(neurons=300, fanout=20, seed=303, ticks=200),
        dict(neurons=1200, fanout=30, seed=304, ticks=120, max_reference_patterns=2),
        dict(neurons=500, fanout=25, seed=305, ticks=64),
        dict(neurons=1500, fanout=50, seed=306, ticks=175),
    ]
    out = []
    for k in specs:
        w = base.scaled(weight_scale=0.06, max_weight=0.12, **k)
        out.append((w, synthetic.build_network(w), synthetic.build_drive(w, w.ticks)))
    return out


@pytest.fixture(scope="module")
def jobs():
    return _jobs()


def _config(lib, i):
    cfg = default_config(lib)
    cfg.max_weight = 1.0
    cfg.stdp_enabled = 1 if i % 3 != 1 else 0
    return cfg


def _solo(lib, job, i):
    w, c, d = job
    sim = Simulation(c, _config(lib, i), lib)
    sim.inject(*d)
    sim.run_until(w.ticks - 1)
    out = (sim.counters(), sim.digest())
    sim.close()
    return out


def _serve(lib, jobs, configs=None, **server_args):
    sv = Server(digests=True, lib=lib, **server_args)
    configs = configs or list(range(len(jobs)))
    ids = [sv.submit(c, _config(lib, k), d, w.ticks) for k, (w, c, d) in zip(configs, jobs)]
    for _ in range(100_000):
        if sv.step() == 0:
            break
    out = [sv.job(j) for j in ids]
    sv.close()
    return out


def _check(results, jobs, lib):
    for i, (r, job) in enumerate(zip(results, jobs)):
        assert r["state"] == 2, (i, r)
        counters, digest = _solo(lib, job, i)
        for key in ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "pending_events",
                    "next_tick"):
            assert r["counters"][key] == counters[key], (i, key)
        assert r["digest"] == digest, f"job {i}: state digest differs from its solo run"
        assert r["submitted_s"] <= r["admitted_s"] <= r["finished_s"]


def test_oracle_server_matches_solo_runs(port_lib, jobs):
    _check(_serve(port_lib, jobs[:3]), jobs[:3], port_lib)


@pytest.mark.gpu
def test_server_jobs_match_solo_runs(gpu_lib, jobs):
    results = _serve(gpu_lib, jobs, max_running=3, slice_ticks=16)
    assert sum(r["counters"]["synaptic_events"] for r in results) > 10_000
    _check(results, jobs, gpu_lib)


@pytest.mark.gpu
def test_server_budget_queues_jobs(gpu_lib, jobs):
    """A budget that holds about one job at a time still finishes every job
    with the same results; admission follows submission order."""
    one = max(_serve(gpu_lib, jobs[:1])[0]["device_bytes"], 1)
    results = _serve(gpu_lib, jobs, memory_budget_bytes=one + 1, slice_ticks=40)
    admitted = [r["admitted_s"] for r in results]
    assert admitted == sorted(admitted)
    _check(results, jobs, gpu_lib)


@pytest.mark.gpu
def test_server_matches_oracle(gpu_lib, port_lib, jobs):
    got = _serve(gpu_lib, jobs[:3], slice_ticks=7)
    want = _serve(port_lib, jobs[:3])
    for g, w in zip(got, want):
        assert g["digest"] == w["digest"]
        assert g["counters"]["fired_spikes"] == w["counters"]["fired_spikes"]


@pytest.mark.gpu
def test_server_eviction_preempts_long_job(gpu_lib, jobs):
    """With eviction on and a budget of about one job, a long job admitted
    first is evicted to host memory when shorter jobs arrive and resumes
    afterwards; every job still equals its solo run."""
    long_job = jobs[5]                  # 1500 neurons x 50, 175 ticks
    w, c, d = long_job
    long_job = (w.scaled(ticks=400), c, synthetic.build_drive(w.scaled(ticks=400), 400))
    order = [long_job, jobs[2], jobs[4]]
    one = max(_serve(gpu_lib, [long_job], [5])[0]["device_bytes"], 1)
    results = _serve(gpu_lib, order, [5, 2, 4], memory_budget_bytes=one + 1, slice_ticks=20, evict=True)
    assert results[0]["evictions"] >= 1
    assert results[1]["finished_s"] < results[0]["finished_s"]
    for i, (r, job) in enumerate(zip(results, order)):
        assert r["state"] == 2, (i, r)
        counters, digest = _solo(gpu_lib, job, [5, 2, 4][i])
        assert r["counters"]["fired_spikes"] == counters["fired_spikes"]
        assert r["digest"] == digest
