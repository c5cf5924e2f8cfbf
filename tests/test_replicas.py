"""Multi-GPU is replicas only: each rank runs its own copy of the network with
no collective on the data path, and bench.py combines the ranks' timings
(max) and work (sum).  Exercised here with two gloo ranks on the CPU, each
driving the CPU oracle, so the rank logic runs without a GPU."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import time

    import torch.distributed as dist

    import bench
    from snncuda_gb300 import _abi, synthetic
    from snncuda_gb300.simulation import Simulation

    dist.init_process_group("gloo", rank=rank, world_size=world)
    lib = _abi.bind(str(bench.ORACLE))
    w = synthetic.STDP_100K.scaled(neurons=300, fanout=20, ticks=120, weight_scale=0.25, max_weight=0.5, seed=5)
    sim = Simulation(synthetic.build_network(w), bench.sim_config(lib, w), lib)
    sim.inject(*synthetic.build_drive(w, 120))
    dist.barrier()
    t0 = time.perf_counter()
    sim.run_until(119)
    ms = (time.perf_counter() - t0) * 1e3 * (1 + rank)  # ranks report different times
    events = sim.counters()["synaptic_events"]
    ms_max, events_all = bench.combine_ranks(ms, events, world, dist)
    digest = sim.digest()
    sim.close()
    out.put((rank, ms, events, ms_max, events_all, digest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_combine_max_time_and_sum_of_work(port_lib):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, ev0, mx0, all0, d0), (r1, ms1, ev1, mx1, all1, d1) = res
    assert d0 == d1 and ev0 == ev1 > 0          # identical replicas
    assert mx0 == mx1 == pytest.approx(max(ms0, ms1))
    assert all0 == all1 == ev0 + ev1
