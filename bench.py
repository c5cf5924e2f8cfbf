"""Throughput benchmark: synaptic events/s of the per-tick SNN hot path.

Workload (default `stdp_100k`, the 100,000-neuron / 1e8-synapse STDP
network with 1-4 spike-code offsets per synapse, temporal-pattern matching,
5 Hz Poisson drive, 10,000 ticks): one *step* is `--ticks-per-step` ticks
(default 400) of the network; W warm-up steps then K timed steps cover the
workload's 10,000 ticks.

GPU arm (default)
  value   synaptic events/s with the whole drive injected before the timed
          region (inputs resident in HBM); CUDA events on the simulation's
          stream bracket the K timed steps.
  e2e     the same metric through the public API with host buffers: each step
          injects that step's drive from pinned host memory, runs, and reads
          back the step's fire raster and counters.
  roofline  the dominant kernel from a per-kernel profile of 200 extra ticks
          (graph event nodes around every kernel), algorithmic bytes per launch
          / average launch time, against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle port on a bounded prefix of the same workload.
Reference arm (--impl reference): the CPU oracle port (the reference's own
runtime cannot be built on the GPU host) on a bounded prefix of the workload.

Multi-GPU: replicas only (independent copies of the network, one per rank,
no collective on the data path); value = all ranks' events / max time.
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
if "--serve" in sys.argv:
    # one hardware work queue per concurrently running job's stream (read at
    # CUDA context creation; the default of 8 would serialize the streams)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "synaptic_events_per_s"
UNIT = "events/s"
ORACLE = ROOT / "oracle" / "_build" / "liboracle_port.so"
KERNELS_PER_TICK = 11   # launch_tick in snncuda_gb300/csrc/kernels.cu
# DRAM bytes (read + write) per launch of a kernel on the default stdp_100k
# workload, from one ncu capture of this code (profiles/); reported as
# roofline.traffic for the dominant kernel.
MEASURED_TRAFFIC = {("stdp_100k", "k_events"): 159.0e6 + 96.6e6}

# Algorithmic bytes of the two per-event kernels (device layout in
# snncuda_gb300/csrc/engine.h), per synaptic event, per external event and
# per touched target:
#   k_events   reads the grouped entry (8) and the synapse record (64), writes
#              the record (64), the event's input (16) and the STDP snapshot
#              (32); external events: entry + input; per target its
#              parameters (64) and segment bounds (12)
#   k_process  reads each event's input (16); per target its threshold (4)
#              and the physics fields of its record, read + write (2 x 52)
#   k_temporal per target: parameters (64), temporal record read + write
#              (2 x 32), the temporal fields of the neuron record (2 x 12) and
#              one run of the window (2 x 8)
BYTES_MODEL = {
    "k_events": (8 + 64 + 64 + 16 + 32, 8 + 16, 64 + 12),
    "k_process": (16, 16, 4 + 2 * 52),
    "k_temporal": (0, 0, 64 + 2 * 32 + 2 * 12 + 2 * 8),
}


def load_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def combine_ranks(ms, events, world, dist=None, device="cpu"):
    """Replicas only: every rank runs its own copy of the workload; the job's
    time is the slowest rank's, its work the sum over ranks."""
    if world <= 1 or dist is None:
        return ms, float(events)
    import torch
    t = torch.tensor([ms, float(events)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(t[1])


def tick_roofline(w, events, fires, ext, prof, ticks, ms):
    """Whole-tick roofline: minimal algorithmic bytes of the tick loop (a
    compact structure-of-arrays design, per-term below) over the timed ticks,
    against the measured HBM bandwidth.  Touched targets per tick come from the
    profiled ticks that follow the timed region."""
    if prof is None or prof["ticks"] == 0 or ms <= 0:
        return None
    fanout = fanin = w.fanout  # synapses per source and per target
    touched = prof["touched_targets"] / prof["ticks"] * ticks
    b = (fires * (8 + 7 * fanout)        # out-row pointers + per out-synapse index, delay, packed offsets
         + events * (8 + 8)             # event written into its wheel slot, read at delivery
         + events * (1 + 4 + 4 + 4 + 16)  # flags, weight, last_post, last_pre, code state read
         + events * 4 + events * 16     # weight and code-state writes
         + touched * 48 + ext * 8       # touched neurons' state read-modify-write, external inputs
         + fires * fanin * 16)          # post-spike STDP over the fired neurons' incoming synapses
    peak, kind = load_peaks()
    achieved = b / (ms / 1e3) / 1e9
    return {"bytes_per_event": b / max(events, 1), "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": kind}


def workload_from_args(args):
    from snncuda_gb300 import synthetic
    w = synthetic.WORKLOADS[args.workload]
    if args.weight_scale is not None:
        w = w.scaled(weight_scale=args.weight_scale)
    if args.neurons is not None:
        w = w.scaled(neurons=args.neurons)
    if args.fanout is not None:
        w = w.scaled(fanout=args.fanout)
    return w


SLOT_CAPACITY = 0  # --slot-capacity


def sim_config(lib, w, **extra):
    from snncuda_gb300.simulation import default_config
    if SLOT_CAPACITY:
        extra.setdefault("slot_event_capacity", SLOT_CAPACITY)
    cfg = default_config(lib, **extra)
    cfg.stdp_enabled = 1 if w.stdp_enabled else 0
    cfg.max_weight = 1.0  # StdpConfig clip [0, 1]; synapses carry their own max_weight
    return cfg


def cpu_sample(w, net, drive, budget_s: float, tick_chunk: int = 5, max_ticks: int = 400):
    """Run the CPU oracle on a prefix of the workload for about budget_s."""
    from snncuda_gb300 import _abi
    from snncuda_gb300.simulation import Simulation
    lib = _abi.bind(str(ORACLE))
    sim = Simulation(net, sim_config(lib, w), lib)
    n, t, wt = drive
    keep = t < max_ticks
    sim.inject(n[keep], t[keep], wt[keep])
    start = time.perf_counter()
    tick = 0
    while tick < max_ticks:
        tick += tick_chunk
        sim.run_until(tick - 1)
        if time.perf_counter() - start >= budget_s:
            break
    elapsed = time.perf_counter() - start
    c = sim.counters()
    sim.close()
    return {"value": c["synaptic_events"] / elapsed, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"ticks 0..{tick - 1} of {w.name} ({c['synaptic_events']} synaptic events, "
                      f"{elapsed:.1f} s, single-threaded oracle port)"}


def run_reference(args, w):
    from snncuda_gb300 import synthetic
    net = synthetic.build_network(w)
    drive = synthetic.build_drive(w, w.ticks)
    sample = cpu_sample(w, net, drive, budget_s=args.cpu_seconds)
    return {
        "metric": METRIC, "value": sample["value"], "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config_block(args, w),
        "cpu_baseline": sample,
        "e2e": {"value": sample["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def config_block(args, w):
    return {"workload": w.name, "neurons": w.neurons, "synapses": w.synapses, "fanout": w.fanout,
            "weight_scale": w.weight_scale, "ticks": w.ticks, "ticks_per_step": args.ticks_per_step,
            "stdp": w.stdp_enabled, "drive_hz": w.drive_rate_hz, "seed": w.seed,
            "l2": f"inputs larger than L2 (synapse state 64 B x {w.synapses:.0e} = {64 * w.synapses / 1e9:.1f} GB)",
            "parallelism": f"replicas x{args.gpus}"}


def batch_members(count, nmin, nmax, ticks):
    """Networks of the batched comparison: N log-uniform in [nmin, nmax],
    fan-out uniform in {100..1000} (at most N), stdp_100k distributions
    otherwise, seeds 1000 + i, the STDP rule on for even i."""
    from snncuda_gb300 import synthetic
    rng = np.random.default_rng(7)
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        fan = int(min(n, rng.integers(100, 1001)))
        w = synthetic.STDP_100K.scaled(name=f"member{i}", neurons=n, fanout=fan, ticks=ticks, seed=1000 + i,
                                       weight_scale=0.01 * 1000 / fan, max_weight=0.01 * 1000 / fan)
        out.append((w, i % 2 == 0))
    return out


def run_batched(args):
    """Synaptic events/s of `--batched` networks advanced together in one
    batch handle, against the same networks run one after another, one
    handle each (the reference's one-propagator-per-network usage).  Both
    legs time the tick loop only (networks built and drives injected before
    the timed region) with CUDA events; the batch's per-network digests must
    equal the solo runs'."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from snncuda_gb300 import synthetic
    from snncuda_gb300.simulation import Batch, Simulation, backend
    lib = backend()
    nmin, nmax = (int(x) for x in args.batch_neurons.split(","))
    T = args.batch_ticks
    members = batch_members(args.batched, nmin, nmax, T)
    nets = [synthetic.build_network(w) for w, _ in members]
    drives = [synthetic.build_drive(w, T) for w, _ in members]
    stream = torch.cuda.Stream()
    warm = min(50, T // 4)

    def cfg_for(rule):
        c = sim_config(lib, members[0][0], cuda_stream=stream.cuda_stream)
        c.stdp_enabled = 1 if rule else 0
        return c

    def timed(run):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # batched leg
    b = Batch(nets, cfg_for(True), lib, stdp_enabled=[r for _, r in members])
    for i, d in enumerate(drives):
        b.inject(i, *d)
    b.run_until(warm - 1)
    before = [b.counters(i)["synaptic_events"] for i in range(len(nets))]
    ms_batch = timed(lambda: b.run_until(T - 1))
    ev_batch = sum(b.counters(i)["synaptic_events"] - before[i] for i in range(len(nets)))
    dig_batch = b.digests()
    b.close()
    # sequential leg
    ms_seq, ev_seq, dig_seq = 0.0, 0, []
    for (w, rule), net, d in zip(members, nets, drives):
        sim = Simulation(net, cfg_for(rule), lib)
        sim.inject(*d)
        sim.run_until(warm - 1)
        c0 = sim.counters()["synaptic_events"]
        ms_seq += timed(lambda: sim.run_until(T - 1))
        ev_seq += sim.counters()["synaptic_events"] - c0
        dig_seq.append(sim.digest())
        sim.close()
    return {
        "metric": METRIC, "value": ev_batch / (ms_batch / 1e3), "unit": UNIT, "n_gpus": 1,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched x{len(nets)}", "neurons": [w.neurons for w, _ in members],
                   "fanout": [w.fanout for w, _ in members], "ticks": T, "timed_ticks": T - warm,
                   "stdp_rule_on_even": True, "synapses_total": int(sum(w.synapses for w, _ in members))},
        "ms_batched": ms_batch, "sequential": {"value": ev_seq / (ms_seq / 1e3), "ms": ms_seq},
        "speedup_vs_sequential": (ev_batch / ms_batch) / (ev_seq / ms_seq) if ev_seq else None,
        "events": ev_batch, "parity_per_network": dig_batch == dig_seq,
    }


def serving_jobs(args):
    """Arrival times (Poisson, seed 7) and workloads of the serving run: N
    log-uniform, fan-out uniform in {200..1000} (at most N), ticks uniform,
    recog_1m distributions (the 16-code stimulus over a 5 Hz background)
    with the initial and per-synapse max weights scaled by 1000 / fan-out."""
    from snncuda_gb300 import synthetic
    rng = np.random.default_rng(7)
    nmin, nmax = (int(x) for x in args.serve_neurons.split(","))
    tmin, tmax = (int(x) for x in args.serve_ticks.split(","))
    t, jobs = 0.0, []
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t > args.serve_seconds:
            break
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        fan = int(min(n, rng.integers(200, 1001)))
        ticks = int(rng.integers(tmin, tmax + 1))
        w = synthetic.RECOG_1M.scaled(name=f"job{len(jobs)}", neurons=n, fanout=fan, ticks=ticks,
                                      seed=7000 + len(jobs), weight_scale=0.01 * 1000 / fan,
                                      max_weight=0.01 * 1000 / fan)
        jobs.append((t, w))
    return jobs


def run_serving(args):
    """Serving run: jobs arrive as a Poisson process and are submitted to one
    Server (device-memory budget, jobs advanced side by side on their own
    streams) at their arrival times; latency = completion - submission on the
    server's clock.  Networks and drives are generated before the clock
    starts.  A few of the smallest jobs are then served again with state
    digests and compared with solo runs (solo-vs-mix equality)."""
    import __graft_entry__
    __graft_entry__.build()
    from snncuda_gb300 import synthetic
    from snncuda_gb300.simulation import Server, Simulation, backend
    lib = backend()
    plan = serving_jobs(args)
    built = [(t, w, synthetic.build_network(w), synthetic.build_drive(w, w.ticks)) for t, w in plan]

    def cfg():
        return sim_config(lib, plan[0][1])

    sv = Server(memory_budget_bytes=int(args.serve_budget_gb * (1 << 30)), max_running=args.serve_running,
                slice_ticks=args.serve_slice, lib=lib)
    ids = [None] * len(built)
    start = time.perf_counter()
    nxt = 0
    while True:
        now = time.perf_counter() - start
        while nxt < len(built) and built[nxt][0] <= now:
            _, w, net, drive = built[nxt]
            ids[nxt] = sv.submit(net, cfg(), drive, w.ticks)
            nxt += 1
        active = sv.step()
        if nxt == len(built) and active == 0:
            break
        if active == 0:
            time.sleep(0.0005)
    wall = time.perf_counter() - start
    res = [sv.job(j) for j in ids]
    sv.close()
    failed = [i for i, r in enumerate(res) if r["state"] != 2]
    lat = np.array([r["finished_s"] - r["submitted_s"] for r in res if r["state"] == 2])
    events = sum(r["counters"]["synaptic_events"] for r in res if r["state"] == 2)
    first = min(r["submitted_s"] for r in res)
    last = max(r["finished_s"] for r in res)
    # solo-vs-mix on the three smallest jobs
    small = sorted(range(len(built)), key=lambda i: built[i][1].synapses)[:3]
    sv2 = Server(digests=True, lib=lib)
    mix = [sv2.submit(built[i][2], cfg(), built[i][3], built[i][1].ticks) for i in small]
    while sv2.step():
        pass
    mixed = [sv2.job(j)["digest"] for j in mix]
    sv2.close()
    solo = []
    for i in small:
        sim = Simulation(built[i][2], cfg(), lib)
        sim.inject(*built[i][3])
        sim.run_until(built[i][1].ticks - 1)
        solo.append(sim.digest())
        sim.close()
    return {
        "metric": METRIC, "value": events / (last - first), "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serving", "jobs": len(built), "arrival_rate_per_s": args.serve_rate,
                   "arrival_seconds": args.serve_seconds, "neurons": args.serve_neurons,
                   "ticks": args.serve_ticks, "budget_gb": args.serve_budget_gb,
                   "synapses_total": int(sum(w.synapses for _, w, _, _ in built))},
        "latency_s": {"p50": float(np.percentile(lat, 50)) if lat.size else None,
                      "p99": float(np.percentile(lat, 99)) if lat.size else None,
                      "max": float(lat.max()) if lat.size else None},
        "events": int(events), "wall_s": wall, "failed_jobs": failed,
        "solo_vs_mix_equal": mixed == solo,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", default="stdp_100k")
    ap.add_argument("--ticks-per-step", type=int, default=400)
    ap.add_argument("--weight-scale", type=float, default=None)
    ap.add_argument("--neurons", type=int, default=None, help="smaller case of the workload (profiling)")
    ap.add_argument("--fanout", type=int, default=None)
    ap.add_argument("--profile-ticks", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--slot-capacity", type=int, default=0, help="events one wheel slot holds (0 = default)")
    ap.add_argument("--batched", type=int, default=0,
                    help="batched form: this many networks in one handle vs one handle per network")
    ap.add_argument("--batch-ticks", type=int, default=500)
    ap.add_argument("--batch-neurons", type=str, default="1000,20000", help="log-uniform range of N")
    ap.add_argument("--rmw-floor", action="store_true",
                    help="time random 64-byte record read-modify-writes (the per-event access floor)")
    ap.add_argument("--serve", action="store_true", help="serving: Poisson arrivals under a memory budget")
    ap.add_argument("--serve-rate", type=float, default=4.0, help="job arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=15.0, help="arrival window")
    ap.add_argument("--serve-neurons", type=str, default="10000,100000", help="log-uniform range of N")
    ap.add_argument("--serve-ticks", type=str, default="500,2000", help="uniform range of ticks per job")
    ap.add_argument("--serve-budget-gb", type=float, default=120.0)
    ap.add_argument("--serve-slice", type=int, default=32, help="ticks per job and scheduling round")
    ap.add_argument("--serve-running", type=int, default=32, help="jobs advanced side by side")
    args = ap.parse_args()
    if args.serve:
        print(json.dumps(run_serving(args)), flush=True)
        return
    if args.rmw_floor:
        import __graft_entry__
        exe = __graft_entry__.build_rmw_floor()
        out = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout
        print(out.strip(), flush=True)
        return
    if args.batched:
        print(json.dumps(run_batched(args)), flush=True)
        return
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    global SLOT_CAPACITY
    SLOT_CAPACITY = args.slot_capacity

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    w = workload_from_args(args)
    total_ticks = (args.warmup + args.steps) * args.ticks_per_step
    if total_ticks > w.ticks:
        w = w.scaled(ticks=total_ticks)

    if args.impl == "reference":
        if rank != 0:
            return
        if not ORACLE.exists():
            import __graft_entry__
            __graft_entry__.build()
        print(json.dumps(run_reference(args, w)), flush=True)
        return

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if world > 1:
        dist.barrier()
    from snncuda_gb300 import synthetic
    from snncuda_gb300.simulation import Simulation, backend

    lib = backend()
    net = synthetic.build_network(w)
    profile_end = total_ticks + args.profile_ticks
    drive_all = synthetic.build_drive(w, profile_end)
    dn, dt, dw = drive_all
    main_mask = dt < total_ticks
    drive = (dn[main_mask], dt[main_mask], dw[main_mask])
    stream = torch.cuda.Stream(device=dev)

    # ---- device-resident timing --------------------------------------------
    sim = Simulation(net, sim_config(lib, w, cuda_stream=stream.cuda_stream), lib)
    sim.inject(*drive)
    tps = args.ticks_per_step
    tick = 0
    for _ in range(args.warmup):
        tick += tps
        sim.run_until(tick - 1)
    c0 = sim.counters()
    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        tick += tps
        sim.run_until(tick - 1)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if world > 1:
        dist.barrier()
    c1 = sim.counters()
    # recognition workloads: the sums the reference's recognition metric adds up
    recognition = sim.recognition() if w.stimulus_codes else None
    ms = ev0.elapsed_time(ev1)
    events = c1["synaptic_events"] - c0["synaptic_events"]
    ext_events = c1["external_events"] - c0["external_events"]
    fires = c1["fired_spikes"] - c0["fired_spikes"]
    ms_max, events_all = combine_ranks(ms, events, world, dist if world > 1 else None, dev)
    value = events_all / (ms_max / 1e3)

    # ---- per-kernel profile for the roofline -------------------------------
    roofline = None
    prof = None
    if args.profile_ticks > 0:
        extra = ~main_mask
        sim.inject(dn[extra], dt[extra], dw[extra])
        prof = sim.profile(profile_end - 1)
        km = prof["kernel_ms"]
        top = max(km, key=km.get)
        launches = prof["ticks"]
        peak, peak_kind = load_peaks()
        if top in BYTES_MODEL:
            per_syn, per_ext, per_tgt = BYTES_MODEL[top]
            algo = (per_syn * prof["synaptic_events"] + per_ext * prof["external_events"] +
                    per_tgt * prof["touched_targets"]) / launches
        else:
            algo = None
        avg_ms = km[top] / launches
        achieved = algo / (avg_ms / 1e3) / 1e9 if algo else None
        roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": (achieved / peak) if achieved else None,
                    "traffic": MEASURED_TRAFFIC.get((w.name, top)) if args.neurons is None and args.fanout is None
                    else None,
                    "peak_source": peak_kind, "avg_launch_us": avg_ms * 1e3,
                    "algorithmic_bytes_per_launch": algo,
                    "kernel_share": {k: v / sum(km.values()) for k, v in km.items()}}
    sim.close()
    del sim

    # ---- end to end through the public API ---------------------------------
    e2e = None
    if not args.no_e2e:
        pin = lambda a, dt_: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        pn, pt, pw = pin(drive[0], np.uint32), pin(drive[1], np.uint64), pin(drive[2], np.float32)
        bounds = np.searchsorted(pt, np.arange(0, total_ticks + tps, tps))
        sim2 = Simulation(net, sim_config(lib, w, cuda_stream=stream.cuda_stream,
                                          raster_capacity=1 << 26), lib)
        h2d = d2h = 0
        raster_pos = 0
        tick = 0
        start = None
        for step in range(args.warmup + args.steps):
            if step == args.warmup:
                torch.cuda.synchronize()
                h2d = d2h = 0
                start = time.perf_counter()
                cs = sim2.counters()
            a, b = bounds[step], bounds[step + 1]
            sim2.inject(pn[a:b], pt[a:b], pw[a:b])
            h2d += (b - a) * 16
            tick += tps
            sim2.run_until(tick - 1)
            c = sim2.counters()
            new = c["raster_count"] - raster_pos
            sim2.raster(raster_pos, new)
            d2h += new * 8 + 64
            raster_pos = c["raster_count"]
        elapsed = time.perf_counter() - start
        ce = sim2.counters()
        sim2.close()
        e2e_events = ce["synaptic_events"] - cs["synaptic_events"]
        e2e = {"value": e2e_events / elapsed, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
               "d2h_bytes_per_step": int(d2h / args.steps)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_sample(w, net, drive_all, budget_s=args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_block(args, w),
            "ticks_per_s": args.steps * tps / (ms_max / 1e3),
            "fires_per_tick": fires / (args.steps * tps),
            "events_per_tick": events / (args.steps * tps),
            "gpu_launches": args.steps * tps * KERNELS_PER_TICK,
            "tick_roofline": tick_roofline(w, events, fires, ext_events, prof, args.steps * tps, ms_max),
            "clocks": clocks, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            **({"recognition": recognition} if recognition is not None else {}),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
