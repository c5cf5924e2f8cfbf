"""Throughput benchmark: synaptic events/s of the per-tick SNN hot path.

Headline workload (default `recog_1m`): 1,000,000 neurons, fan-out 1,000
(1e9 synapses, 64 GB of synapse state), lognormal weights, 1-4 spike-code
offsets per synapse, pair STDP, temporal-pattern matching, a 16-code
stimulus presented every 64 ticks to half the neurons over a 5 Hz Poisson
background, 2,000 ticks.  One *step* is `--ticks-per-step` ticks (80 by
default, so 5 warm-up and 20 timed steps cover the workload's 2,000 ticks).
`stdp_100k` (1e5 neurons, 1e8 synapses, 10,000 ticks) is measured beside it
and reported under the key "stdp_100k".

GPU arm (default)
  value     synaptic events/s with the whole drive injected before the timed
            region (inputs resident in HBM); CUDA events on the simulation's
            stream bracket the K timed steps.
  e2e       the same metric through the public API with host buffers: each
            step injects that step's drive from pinned host memory, runs, and
            reads back the step's fire raster and counters.
  roofline  the dominant kernel, from a per-kernel profile of extra ticks
            (graph event nodes around every kernel): the minimal algorithmic
            bytes of its work (MINIMAL_BYTES) per launch over its average
            launch time, against the measured HBM copy bandwidth; the bytes
            of this engine's own layout give `layout_frac`.
  tick_roofline  the whole tick loop's minimal bytes over the timed ticks.
  parity    the GPU and the CPU oracle run from the same seed over a tick
            prefix of the full stdp_100k network and of a 100,000-neuron
            network with the recog_1m distributions: counters, fire
            rasters, full state digests and recognition sums compared.
  batched   64 networks of the batched comparison (N log-uniform in
            1k-200k, fan-out 100-1,000, seeds 1000+i, STDP rule on for even
            i, 2,000 ticks) advanced together in one autotuned batch handle,
            against one handle per network over the same tick window, with
            every network's device state checksums equal to its solo run's;
            `--batched 256` runs all 256 networks (in waves that fit).
  cpu_baseline  the oracle's events/s over a steady-state window of that
            100,000-neuron recognition run (single-threaded, as the
            reference runtime is): the oracle cannot hold the 1e9-synapse
            network in host memory in a bounded time, so the CPU sample is
            the same per-event work on a 1e8-synapse network.
Reference arm (--impl reference): the CPU oracle on the same steady-state
window, with the same `same_config: false` note.

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
# kernels per tick (launch_tick in snncuda_gb300/csrc/kernels.cu): the
# profile API's kernel count; plus one injection kernel per timed step
def kernels_per_tick():
    from snncuda_gb300 import _abi
    return _abi.KERNEL_COUNT

# Minimal algorithmic bytes of a compact structure-of-arrays design of the
# tick, per fire F, synaptic event E, external event X, touched target U:
#   F * (8 + 7 * fanout)   out-row pointers, per out-synapse target index,
#                          delay and packed offsets
#   E * (8 + 8)            event written into its wheel slot, read at delivery
#   E * (1 + 4 + 4 + 4 + 16)  synapse flags, weight, last_post read,
#                          last_pre write, code-state read
#   E * (4 + 16)           weight write (counted for every event: an upper
#                          bound) and code-state write
#   U * 48 + X * 8         touched neurons' state read-modify-write, externals
#   F * fanin * 16         post-spike STDP over the fired neurons' in-rows
# Per kernel: the synapse-side kernel k_events carries the delivery read and
# the synapse terms (8 + 29 + 20 = 57 B per synaptic event, 8 B per
# external); k_process the touched-neuron term.  (per synaptic event, per
# external event, per touched target)
MINIMAL_BYTES = {
    "k_events": (57, 8, 0),
    "k_process": (0, 0, 48),
}
# Bytes of this engine's own layout (snncuda_gb300/csrc/engine.h) per
# synaptic event, external event and touched target:
#   k_events   grouped entry (8), synapse record read + write (2 x 64), event
#              input (16), the record's changing fields before the event (16);
#              externals: entry + input; per target its parameters (64) and
#              segment bounds (8)
#   k_process  event input (16); per target its threshold (4) and the
#              physics fields of its record, read + write (2 x 52)
LAYOUT_BYTES = {
    "k_events": (8 + 64 + 64 + 16 + 16, 8 + 16, 64 + 8),
    "k_process": (16, 16, 4 + 2 * 52),
}
# DRAM bytes (read + write) per synaptic event of a kernel, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of all 240 k_events
# launches of the timed steps of a 20,000-neuron case of recog_1m (7.863 GB
# over 59.87 M synaptic events: 127.2 B read, 4.2 B written; the records'
# write-back happens after the kernel); roofline.traffic scales it to the
# events of one full-size launch.
MEASURED_TRAFFIC_PER_EVENT = {"k_events": 131.3}


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


def minimal_tick_bytes(w, events, fires, ext, touched):
    """Minimal algorithmic bytes of the tick loop (the terms above MINIMAL_BYTES)."""
    fanout = fanin = w.fanout  # synapses per source and per target
    return (fires * (8 + 7 * fanout) + events * (8 + 8) + events * (1 + 4 + 4 + 4 + 16) + events * (4 + 16)
            + touched * 48 + ext * 8 + fires * fanin * 16)


def tick_roofline(w, events, fires, ext, prof, ticks, ms):
    """Whole-tick roofline over the timed ticks (touched targets per tick from
    the profiled ticks that follow the timed region)."""
    if prof is None or prof["ticks"] == 0 or ms <= 0:
        return None
    touched = prof["touched_targets"] / prof["ticks"] * ticks
    b = minimal_tick_bytes(w, events, fires, ext, touched)
    peak, kind = load_peaks()
    achieved = b / (ms / 1e3) / 1e9
    return {"bytes_per_event": b / max(events, 1), "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": kind}


def kernel_roofline(w, prof, full_size):
    """Roofline of the dominant kernel of a per-kernel profile."""
    km = prof["kernel_ms"]
    top = max(km, key=km.get)
    launches = prof["ticks"]
    peak, peak_kind = load_peaks()
    avg_s = km[top] / launches / 1e3

    def per_launch(model):
        if top not in model:
            return None
        per_syn, per_ext, per_tgt = model[top]
        return (per_syn * prof["synaptic_events"] + per_ext * prof["external_events"] +
                per_tgt * prof["touched_targets"]) / launches

    algo, layout = per_launch(MINIMAL_BYTES), per_launch(LAYOUT_BYTES)
    achieved = algo / avg_s / 1e9 if algo else None
    traffic = None
    if full_size and top in MEASURED_TRAFFIC_PER_EVENT:
        traffic = MEASURED_TRAFFIC_PER_EVENT[top] * prof["synaptic_events"] / launches
    return {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "traffic": traffic, "peak_source": peak_kind,
            "avg_launch_us": avg_s * 1e6, "algorithmic_bytes_per_launch": algo,
            "layout_bytes_per_launch": layout,
            "layout_frac": layout / avg_s / 1e9 / peak if layout else None,
            "kernel_share": {k: v / sum(km.values()) for k, v in km.items()}}


def workload_from_args(args, name=None):
    from snncuda_gb300 import synthetic
    w = synthetic.WORKLOADS[name or args.workload]
    if name is None:
        if args.weight_scale is not None:
            w = w.scaled(weight_scale=args.weight_scale)
        if args.neurons is not None:
            w = w.scaled(neurons=args.neurons)
        if args.fanout is not None:
            w = w.scaled(fanout=args.fanout)
    return w


def ticks_per_step(args, w):
    if args.ticks_per_step:
        return args.ticks_per_step
    return 80 if w.name == "recog_1m" else 400


SLOT_CAPACITY = 0  # --slot-capacity


def sim_config(lib, w, **extra):
    from snncuda_gb300.simulation import default_config
    if SLOT_CAPACITY:
        extra.setdefault("slot_event_capacity", SLOT_CAPACITY)
    cfg = default_config(lib, **extra)
    cfg.stdp_enabled = 1 if w.stdp_enabled else 0
    cfg.max_weight = 1.0  # StdpConfig clip [0, 1]; synapses carry their own max_weight
    return cfg


def config_block(args, w, tps):
    return {"workload": w.name, "neurons": w.neurons, "synapses": w.synapses, "fanout": w.fanout,
            "weight_scale": w.weight_scale, "synapse_max_weight": w.max_weight, "stdp_clip": [0.0, 1.0],
            "stdp": w.stdp_enabled, "drive_hz": w.drive_rate_hz, "drive_weight": w.drive_weight,
            **({"stimulus_codes": w.stimulus_codes, "stimulus_period": w.stimulus_period,
                "stimulus_weight": w.stimulus_weight, "stimulus_fraction": w.stimulus_fraction}
               if w.stimulus_codes else {}),
            "ticks": w.ticks, "ticks_per_step": tps, "seed": w.seed,
            "l2": f"inputs larger than L2 (synapse state 64 B x {w.synapses:.0e} = {64 * w.synapses / 1e9:.1f} GB)",
            "parallelism": f"replicas x{args.gpus}"}


# ---------------------------------------------------------------------------
# CPU oracle legs (parity and the CPU baseline)
# ---------------------------------------------------------------------------

def cpu_sample_workload():
    """The CPU sample's network: the recog_1m distributions at 1e5 neurons
    (fan-out 1,000: the same ~12.5 events per target and tick)."""
    from snncuda_gb300 import synthetic
    return synthetic.RECOG_1M.scaled(name="recog_100k", neurons=100_000)


def run_oracle(w, net, drive, ticks, timed_from=None, chunk=5):
    """The CPU oracle over ticks 0 .. ticks-1; returns its final counters,
    raster, digests and recognition sums, and the events/s of ticks
    timed_from .. ticks-1 (single-threaded)."""
    from snncuda_gb300 import _abi
    from snncuda_gb300.simulation import Simulation
    lib = _abi.bind(str(ORACLE))
    sim = Simulation(net, sim_config(lib, w, raster_capacity=1 << 26), lib)
    n, t, wt = drive
    keep = t < ticks
    sim.inject(n[keep], t[keep], wt[keep])
    tick, secs, events = 0, 0.0, 0
    while tick < ticks:
        nxt = min(ticks, tick + chunk)
        before = sim.counters()["synaptic_events"] if timed_from is not None and tick >= timed_from else None
        start = time.perf_counter()
        sim.run_until(nxt - 1)
        if before is not None:
            secs += time.perf_counter() - start
            events += sim.counters()["synaptic_events"] - before
        tick = nxt
    out = {"counters": sim.counters(), "raster": sim.raster(), "digest": sim.digest(),
           "recognition": sim.recognition(), "timed_events": events, "timed_seconds": secs}
    sim.close()
    return out


def run_gpu_prefix(lib, w, net, drive, ticks, stream_ptr=None):
    from snncuda_gb300.simulation import Simulation
    extra = {"raster_capacity": 1 << 26}
    if stream_ptr is not None:
        extra["cuda_stream"] = stream_ptr
    sim = Simulation(net, sim_config(lib, w, **extra), lib)
    n, t, wt = drive
    keep = t < ticks
    sim.inject(n[keep], t[keep], wt[keep])
    sim.run_until(ticks - 1)
    out = {"counters": sim.counters(), "raster": sim.raster(), "digest": sim.digest(),
           "recognition": sim.recognition()}
    sim.close()
    return out


def compare(gpu, cpu, w, ticks):
    keys = ("delivered_spikes", "fired_spikes", "synaptic_events", "external_events", "pending_events")
    counters_equal = all(gpu["counters"][k] == cpu["counters"][k] for k in keys)
    raster_equal = (np.array_equal(gpu["raster"][0], cpu["raster"][0]) and
                    np.array_equal(gpu["raster"][1], cpu["raster"][1]))
    return {"workload": w.name, "neurons": w.neurons, "synapses": w.synapses, "ticks": ticks,
            "synaptic_events": gpu["counters"]["synaptic_events"], "fires": gpu["counters"]["fired_spikes"],
            "counters_equal": counters_equal, "raster_equal": raster_equal,
            "digests_equal": gpu["digest"] == cpu["digest"],
            "recognition_equal": gpu["recognition"] == cpu["recognition"],
            "recognition": gpu["recognition"]}


class OracleThread(threading.Thread):
    """run_oracle in a thread (the ctypes calls release the GIL, so several
    oracle runs proceed on separate cores)."""

    def __init__(self, *args, **kwargs):
        super().__init__(daemon=True)
        self.args, self.kwargs, self.result, self.error = args, kwargs, None, None

    def run(self):
        try:
            self.result = run_oracle(*self.args, **self.kwargs)
        except Exception as ex:  # reported in the JSON line
            self.error = repr(ex)


PARITY_TICKS = {"stdp_100k": 60, "recog_100k": 100}
CPU_TIMED_FROM = 40  # the CPU sample's steady-state window starts here


def parity_legs(lib):
    """GPU vs oracle on the full stdp_100k network (ticks 0..59) and on the
    1e5-neuron recognition network (ticks 0..99, which include a stimulus
    presentation); the second run's ticks 40..99 are the CPU baseline."""
    from snncuda_gb300 import synthetic
    cases = []
    for w in (synthetic.STDP_100K, cpu_sample_workload()):
        T = PARITY_TICKS[w.name]
        net = synthetic.build_network(w)
        drive = synthetic.build_drive(w, T)
        th = OracleThread(w, net, drive, T, timed_from=CPU_TIMED_FROM if w.name == "recog_100k" else None)
        th.start()
        cases.append((w, net, drive, T, th))
    parity, cpu = {}, None
    for w, net, drive, T, th in cases:
        gpu = run_gpu_prefix(lib, w, net, drive, T)
        th.join()
        if th.error:
            parity[w.name] = {"error": th.error}
            continue
        parity[w.name] = compare(gpu, th.result, w, T)
        if w.name == "recog_100k":
            r = th.result
            cpu = {"value": r["timed_events"] / r["timed_seconds"], "unit": UNIT, "cores": 1, "kind": "port",
                   "same_config": False,
                   "sample": f"ticks {CPU_TIMED_FROM}..{T - 1} of recog_100k (recog_1m distributions at 1e5 "
                             f"neurons x 1,000: {r['timed_events']} synaptic events, {r['timed_seconds']:.1f} s, "
                             "single-threaded oracle port; the oracle cannot hold the 1e9-synapse network)"}
    return parity, cpu


def run_reference(args, w):
    """The CPU oracle (the reference runtime's semantics, single-threaded as
    the reference is) on the steady-state window of the CPU sample network."""
    from snncuda_gb300 import synthetic
    ws = cpu_sample_workload()
    T = PARITY_TICKS[ws.name]
    r = run_oracle(ws, synthetic.build_network(ws), synthetic.build_drive(ws, T), T, timed_from=CPU_TIMED_FROM)
    value = r["timed_events"] / r["timed_seconds"]
    sample = {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "same_config": False,
              "sample": f"ticks {CPU_TIMED_FROM}..{T - 1} of recog_100k (recog_1m distributions at 1e5 neurons x "
                        f"1,000: {r['timed_events']} synaptic events, {r['timed_seconds']:.1f} s, single-threaded "
                        "oracle port; the oracle cannot hold the 1e9-synapse network; ms_per_step: "
                        f"{ticks_per_step(args, w)} ticks of that network)"}
    tps = ticks_per_step(args, w)
    # one step = tps ticks of the sample network, at the sample's measured pace
    ms_step = r["timed_seconds"] / (T - CPU_TIMED_FROM) * tps * 1e3
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config_block(args, w, tps),
        "cpu_baseline": sample,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# GPU legs
# ---------------------------------------------------------------------------

def timed_leg(lib, w, net, drive_all, total_ticks, tps, warmup, steps, stream, dist=None, local=0,
              profile_ticks=0, clocks=True):
    """Device-resident timing: `warmup` untimed steps, then `steps` timed
    steps (CUDA events on the simulation's stream), then an optional
    per-kernel profile of `profile_ticks` more ticks."""
    import torch
    from snncuda_gb300.simulation import Simulation
    dn, dt, dw = drive_all
    main_mask = dt < total_ticks
    sim = Simulation(net, sim_config(lib, w, cuda_stream=stream.cuda_stream), lib)
    sim.inject(dn[main_mask], dt[main_mask], dw[main_mask])
    tick = 0
    for _ in range(warmup):
        tick += tps
        sim.run_until(tick - 1)
    c0 = sim.counters()
    sampler = ClockSampler(local) if clocks else None
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        tick += tps
        sim.run_until(tick - 1)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = sampler.stop() if sampler else None
    if dist is not None:
        dist.barrier()
    c1 = sim.counters()
    recognition = sim.recognition() if w.stimulus_codes else None
    ms = ev0.elapsed_time(ev1)
    prof = None
    if profile_ticks > 0:
        extra = ~main_mask
        sim.inject(dn[extra], dt[extra], dw[extra])
        prof = sim.profile(total_ticks + profile_ticks - 1)
    sim.close()
    events = c1["synaptic_events"] - c0["synaptic_events"]
    return {"ms": ms, "events": events, "ext": c1["external_events"] - c0["external_events"],
            "fires": c1["fired_spikes"] - c0["fired_spikes"], "clocks": clk, "recognition": recognition,
            "prof": prof}


def e2e_leg(lib, w, net, drive, total_ticks, tps, warmup, steps, stream):
    """The metric through the public API with host buffers: every step copies
    that step's injections from pinned host memory, runs, and reads back the
    step's fire raster and counters."""
    import torch
    from snncuda_gb300.simulation import Simulation
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    pn, pt, pw = pin(drive[0]), pin(drive[1]), pin(drive[2])
    bounds = np.searchsorted(pt, np.arange(0, total_ticks + tps, tps))
    sim = Simulation(net, sim_config(lib, w, cuda_stream=stream.cuda_stream, raster_capacity=1 << 26), lib)
    h2d = d2h = 0
    raster_pos = 0
    tick = 0
    start = None
    cs = None
    for step in range(warmup + steps):
        if step == warmup:
            torch.cuda.synchronize()
            h2d = d2h = 0
            start = time.perf_counter()
            cs = sim.counters()
        a, b = bounds[step], bounds[step + 1]
        sim.inject(pn[a:b], pt[a:b], pw[a:b])
        h2d += (b - a) * 16
        tick += tps
        sim.run_until(tick - 1)
        c = sim.counters()
        new = c["raster_count"] - raster_pos
        sim.raster(raster_pos, new)
        d2h += new * 12 + 64
        raster_pos = c["raster_count"]
    elapsed = time.perf_counter() - start
    ce = sim.counters()
    sim.close()
    return {"value": (ce["synaptic_events"] - cs["synaptic_events"]) / elapsed, "unit": UNIT,
            "h2d_bytes_per_step": int(h2d / steps), "d2h_bytes_per_step": int(d2h / steps)}


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


def member_waves(members, wave_synapses):
    """Consecutive members grouped into waves of at most `wave_synapses`
    synapses (a wave larger than one GPU's memory would not fit)."""
    waves, cur, acc = [], [], 0
    for m in members:
        if cur and acc + m[0].synapses > wave_synapses:
            waves.append(cur)
            cur, acc = [], 0
        cur.append(m)
        acc += m[0].synapses
    if cur:
        waves.append(cur)
    return waves


def batched_leg(lib, count, nmin, nmax, T, stream, wave_synapses=1.2e9, probe_ticks=20):
    """The batched form against one handle per network (the reference's one
    propagator per network), over the same tick window.  Members are built
    and run in waves of at most `wave_synapses` synapses.  Per wave: the
    batch runs `warm` untimed ticks, autotunes its launch shapes and slot
    capacity on its next ticks, then runs to tick T-1 timed (CUDA events);
    every member then runs alone to the batch's tuned tick untimed and on to
    T-1 timed.  Each member's device state checksums after tick T-1 must
    equal the batch's for it (per-network parity)."""
    import torch
    from snncuda_gb300 import synthetic
    from snncuda_gb300.simulation import Batch, Simulation
    members = batch_members(count, nmin, nmax, T)
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

    ms_b = ms_s = 0.0
    ev_b = ev_s = 0
    parity, tunings, timed_ticks, solo = [], [], [], []
    for wave in member_waves(members, wave_synapses):
        nets = [synthetic.build_network(w) for w, _ in wave]
        drives = [synthetic.build_drive(w, T) for w, _ in wave]
        b = Batch(nets, cfg_for(True), lib, stdp_enabled=[r for _, r in wave])
        for i, d in enumerate(drives):
            b.inject(i, *d)
        b.run_until(warm - 1)
        tuning = b.autotune(probe_ticks)
        t0 = b.counters(0)["next_tick"]
        before = [b.counters(i)["synaptic_events"] for i in range(len(nets))]
        ms_b += timed(lambda: b.run_until(T - 1))
        ev_b += sum(b.counters(i)["synaptic_events"] - before[i] for i in range(len(nets)))
        sums = b.checksums()
        b.close()
        tunings.append(tuning)
        timed_ticks.append(T - t0)
        for k, ((w, rule), net, d) in enumerate(zip(wave, nets, drives)):
            sim = Simulation(net, cfg_for(rule), lib)
            sim.inject(*d)
            sim.run_until(t0 - 1)
            c0 = sim.counters()["synaptic_events"]
            ms_one = timed(lambda: sim.run_until(T - 1))
            ev_one = sim.counters()["synaptic_events"] - c0
            ms_s += ms_one
            ev_s += ev_one
            solo.append((w.neurons, ev_one, ms_one))
            parity.append(sim.checksum() == sums[k])
            sim.close()
        del nets, drives
    return {
        "value": ev_b / (ms_b / 1e3), "unit": UNIT,
        "sequential": {"value": ev_s / (ms_s / 1e3), "ms": ms_s},
        "speedup_vs_sequential": (ev_b / ms_b) / (ev_s / ms_s) if ev_s else None,
        "ms_batched": ms_b, "events": ev_b, "parity_per_network": all(parity),
        "networks_equal": int(sum(parity)),
        "sequential_by_size": sequential_by_size(solo),
        "config": {"networks": count, "neurons_log_uniform": [nmin, nmax], "fanout_uniform": [100, 1000],
                   "ticks": T, "timed_ticks_per_wave": timed_ticks, "waves": len(tunings),
                   "wave_synapses_max": wave_synapses, "stdp_rule_on_even": True, "seeds": "1000 + i",
                   "synapses_total": int(sum(w.synapses for w, _ in members)),
                   "weights": "stdp_100k distributions, initial and per-synapse max weight x 1000 / fan-out"},
        "autotune": tunings,
    }


def sequential_by_size(solo):
    """Where the one-handle-per-network time goes: per band of network size,
    the networks, their synaptic events, their summed time and the rate one
    handle reaches on them; plus the speed-up the batch would show if it ran
    every event at the best single-handle rate (the bound that the large
    members, already near that rate alone, put on batched / sequential)."""
    bands = [(0, 10_000), (10_000, 50_000), (50_000, 1 << 40)]
    out = []
    for lo, hi in bands:
        sel = [(e, ms) for n, e, ms in solo if lo <= n < hi]
        ev = sum(e for e, _ in sel)
        ms = sum(ms for _, ms in sel)
        out.append({"neurons": [lo, hi if hi < (1 << 40) else None], "networks": len(sel), "events": ev,
                    "ms": ms, "events_per_s": ev / (ms / 1e3) if ms else None})
    best = max((e / (ms / 1e3) for _, e, ms in solo if ms > 0), default=0.0)
    ev = sum(e for _, e, _ in solo)
    ms = sum(ms for _, _, ms in solo)
    return {"bands": out, "best_single_rate": best,
            "speedup_if_batched_at_best_single_rate": (best * ms / 1e3) / ev if ev else None}


def run_group_bench(args):
    """`bench.py --group-bench EVENTS,TARGETS`: the tick's grouping kernels
    alone, through snncuda_group_events, on a seeded random due list (targets
    uniform, 1 % external inputs): `warmup` untimed calls, then `steps`
    calls timed with CUDA events.  A device case of the grouping at the
    recog_1m size (13e6 events, 1e6 targets) in about 0.5 GB, small enough
    for a multi-pass ncu capture of one kernel."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from snncuda_gb300.simulation import _check, backend
    lib = backend()
    count, targets = (int(float(x)) for x in args.group_bench.split(","))
    rng = np.random.default_rng(3)
    tgt = rng.integers(0, targets, count, dtype=np.uint64)
    ext = (rng.random(count) < 0.01).astype(np.uint64)
    payload = rng.integers(0, 1 << 32, count, dtype=np.uint64)
    ev = (payload << np.uint64(32)) | tgt | (ext << np.uint64(31))
    d_ev = torch.from_numpy(ev.view(np.int64)).cuda()
    d_out = torch.empty_like(d_ev)
    d_seg = torch.empty(targets + 1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()

    def call():
        _check(lib, lib.snncuda_group_events(d_ev.data_ptr(), count, targets, d_out.data_ptr(), d_seg.data_ptr(),
                                             stream.cuda_stream))

    for _ in range(max(args.warmup, 3)):
        call()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    seg = d_seg.cpu().numpy().view(np.uint32)
    ok = bool(seg[-1] == count and np.all(np.diff(seg.astype(np.int64)) == np.bincount(tgt.astype(np.int64),
                                                                                    minlength=targets)))
    return {"metric": "grouping_events_per_s", "value": count / (ms / 1e3), "unit": "events/s",
            "ms_per_call": ms, "events": count, "targets": targets, "steps": args.steps,
            "segments_match_counts": ok, "data": "synthetic (seed 3)"}


def run_batched(args):
    """`bench.py --batched N`: the batched form on its own (batched_leg)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from snncuda_gb300.simulation import backend
    lib = backend()
    nmin, nmax = (int(x) for x in args.batch_neurons.split(","))
    out = batched_leg(lib, args.batched, nmin, nmax, args.batch_ticks, torch.cuda.Stream(),
                      wave_synapses=args.batch_wave_synapses)
    return {"metric": METRIC, "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic", **out}


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
                slice_ticks=args.serve_slice, evict=args.serve_evict, lib=lib)
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
        "evictions": int(sum(r["evictions"] for r in res)), "evict": bool(args.serve_evict),
        "solo_vs_mix_equal": mixed == solo,
    }


def serving_leg(args):
    """A short serving run beside the headline: Poisson arrivals at 2 jobs/s
    for 8 s (recog_1m distributions, N log-uniform 1e4-1e5), a 16 GB budget
    with preemption by eviction, so some jobs wait in host memory; p50/p99
    latency, aggregate events/s, evictions and the solo-vs-mix check."""
    import copy
    a = copy.copy(args)
    a.serve_rate, a.serve_seconds, a.serve_budget_gb, a.serve_evict = 2.0, 8.0, 16.0, True
    out = run_serving(a)
    return {"value": out["value"], "unit": out["unit"], "latency_s": out["latency_s"], "events": out["events"],
            "wall_s": out["wall_s"], "evictions": out["evictions"], "failed_jobs": out["failed_jobs"],
            "solo_vs_mix_equal": out["solo_vs_mix_equal"], "config": out["config"]}


def side_leg(lib, args, stream):
    """stdp_100k beside the headline: 10 timed steps of 400 ticks after the
    headline's warm-up count, plus its per-kernel profile."""
    from snncuda_gb300 import synthetic
    w1, tps1, steps1 = synthetic.STDP_100K, 400, 10
    total1 = (args.warmup + steps1) * tps1
    net1 = synthetic.build_network(w1)
    d1 = synthetic.build_drive(w1, total1 + args.profile_ticks)
    r1 = timed_leg(lib, w1, net1, d1, total1, tps1, args.warmup, steps1, stream, clocks=False,
                   profile_ticks=args.profile_ticks)
    ticks1 = steps1 * tps1
    return {"value": r1["events"] / (r1["ms"] / 1e3), "unit": UNIT, "ticks_per_s": ticks1 / (r1["ms"] / 1e3),
            "ms_per_step": r1["ms"] / steps1, "steps": steps1, "ticks_per_step": tps1,
            "events_per_tick": r1["events"] / ticks1, "fires_per_tick": r1["fires"] / ticks1,
            "config": config_block(args, w1, tps1),
            "tick_roofline": tick_roofline(w1, r1["events"], r1["fires"], r1["ext"], r1["prof"], ticks1, r1["ms"]),
            "roofline": kernel_roofline(w1, r1["prof"], True) if r1["prof"] else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", default="recog_1m")
    ap.add_argument("--ticks-per-step", type=int, default=0, help="0: 80 for recog_1m, 400 otherwise")
    ap.add_argument("--weight-scale", type=float, default=None)
    ap.add_argument("--neurons", type=int, default=None, help="smaller case of the workload (profiling)")
    ap.add_argument("--fanout", type=int, default=None)
    ap.add_argument("--profile-ticks", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the parity legs and the CPU baseline")
    ap.add_argument("--no-side", action="store_true", help="skip the stdp_100k leg beside the headline")
    ap.add_argument("--slot-capacity", type=int, default=0, help="events one wheel slot holds (0 = default)")
    ap.add_argument("--batched", type=int, default=0,
                    help="batched form: this many networks in one handle vs one handle per network")
    ap.add_argument("--batch-ticks", type=int, default=2000)
    ap.add_argument("--batch-neurons", type=str, default="1000,200000", help="log-uniform range of N")
    ap.add_argument("--batch-wave-synapses", type=float, default=1.2e9, help="synapses per wave of the batch")
    ap.add_argument("--batch-networks", type=int, default=64,
                    help="networks of the batched leg of the default run (0 skips it)")
    ap.add_argument("--rmw-floor", action="store_true",
                    help="time random 64-byte record read-modify-writes (the per-event access floor)")
    ap.add_argument("--rmw-args", default="",
                    help="records events [bands band_len picks rows row_len] for --rmw-floor")
    ap.add_argument("--group-bench", default="",
                    help="EVENTS,TARGETS: time snncuda_group_events alone on a random due list of that size")
    ap.add_argument("--serve", action="store_true", help="serving: Poisson arrivals under a memory budget")
    ap.add_argument("--serve-rate", type=float, default=4.0, help="job arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=15.0, help="arrival window")
    ap.add_argument("--serve-neurons", type=str, default="10000,100000", help="log-uniform range of N")
    ap.add_argument("--serve-ticks", type=str, default="500,2000", help="uniform range of ticks per job")
    ap.add_argument("--serve-budget-gb", type=float, default=120.0)
    ap.add_argument("--serve-slice", type=int, default=32, help="ticks per job and scheduling round")
    ap.add_argument("--serve-running", type=int, default=32, help="jobs advanced side by side")
    ap.add_argument("--no-serve-leg", dest="serve_leg", action="store_false",
                    help="skip the short serving run beside the headline")
    ap.add_argument("--serve-evict", action="store_true",
                    help="queued jobs preempt running jobs with more remaining work (eviction to host memory)")
    args = ap.parse_args()
    if args.serve:
        print(json.dumps(run_serving(args)), flush=True)
        return
    if args.rmw_floor:
        import __graft_entry__
        exe = __graft_entry__.build_rmw_floor()
        out = subprocess.run([str(exe), *args.rmw_args.split()], check=True, stdout=subprocess.PIPE,
                             text=True).stdout
        print(out.strip(), flush=True)
        return
    if args.batched:
        print(json.dumps(run_batched(args)), flush=True)
        return
    if args.group_bench:
        print(json.dumps(run_group_bench(args)), flush=True)
        return
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    global SLOT_CAPACITY
    SLOT_CAPACITY = args.slot_capacity

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    w = workload_from_args(args)
    tps = ticks_per_step(args, w)
    total_ticks = (args.warmup + args.steps) * tps
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
    from snncuda_gb300.simulation import backend

    lib = backend()
    stream = torch.cuda.Stream(device=dev)
    full_size = args.neurons is None and args.fanout is None
    dist_or_none = dist if world > 1 else None

    # ---- headline workload: device-resident timing and per-kernel profile --
    net = synthetic.build_network(w)
    drive_all = synthetic.build_drive(w, total_ticks + args.profile_ticks)
    main_mask = drive_all[1] < total_ticks
    drive = tuple(a[main_mask] for a in drive_all)
    r = timed_leg(lib, w, net, drive_all, total_ticks, tps, args.warmup, args.steps, stream, dist_or_none, local,
                  profile_ticks=args.profile_ticks)
    ms_max, events_all = combine_ranks(r["ms"], r["events"], world, dist_or_none, dev)
    value = events_all / (ms_max / 1e3)
    prof = r["prof"]
    roofline = kernel_roofline(w, prof, full_size) if prof else None

    # ---- end to end through the public API ---------------------------------
    e2e = None
    if not args.no_e2e:
        e2e = e2e_leg(lib, w, net, drive, total_ticks, tps, args.warmup, args.steps, stream)
    del net, drive, drive_all

    # ---- stdp_100k beside the headline, the batched form, parity and the
    # CPU baseline ------------------------------------------------------------
    side = batched = parity = cpu = None
    if rank == 0 and not args.no_side and w.name != "stdp_100k":
        side = side_leg(lib, args, stream)
    if rank == 0 and args.batch_networks > 0 and full_size:
        nmin, nmax = (int(x) for x in args.batch_neurons.split(","))
        batched = batched_leg(lib, args.batch_networks, nmin, nmax, args.batch_ticks, stream,
                              wave_synapses=args.batch_wave_synapses)
    serving = None
    if rank == 0 and args.serve_leg and full_size:
        serving = serving_leg(args)
    if rank == 0 and not args.no_cpu:
        parity, cpu = parity_legs(lib)

    if rank == 0:
        steps_ticks = args.steps * tps
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_block(args, w, tps),
            "ticks_per_s": steps_ticks / (ms_max / 1e3),
            "fires_per_tick": r["fires"] / steps_ticks,
            "events_per_tick": r["events"] / steps_ticks,
            "gpu_launches": steps_ticks * kernels_per_tick() + args.steps,
            "tick_roofline": tick_roofline(w, r["events"], r["fires"], r["ext"], prof, steps_ticks, ms_max),
            "clocks": r["clocks"], "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            **({"recognition": r["recognition"]} if r["recognition"] is not None else {}),
            "parity": parity,
            **({"stdp_100k": side} if side is not None else {}),
            **({"batched": batched} if batched is not None else {}),
            **({"serving": serving} if serving is not None else {}),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
