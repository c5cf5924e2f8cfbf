"""Host-side API of the GB300 backend.

`Simulation` is a thin owner of one `snncuda_sim` handle (C ABI in
include/snncuda_gb300.h).  `NetworkPropagator` mirrors the reference
runtime::NetworkPropagator interface (runtime/NetworkPropagator.h:14-47):
`inject`, `run_until`, `state`, `spike_count`, `delivered_spike_count`,
`fired_spike_count`, `synapse_state`, `idle`, with 1-based neuron and synapse
ids, so code written against the reference reads the same.  Errors raise
`SNNCudaError` (the reference throws std::invalid_argument /
std::runtime_error).
"""

from __future__ import annotations

import ctypes
import os
import pathlib
from ctypes import c_float, c_int32, c_int64, c_uint8, c_uint32, c_uint64, c_void_p
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _abi
from .connectome import Connectome

_LIB_DIR = pathlib.Path(__file__).resolve().parent / "_lib"
BACKEND_LIBRARY = _LIB_DIR / "libsnncuda_gb300.so"

_backend: Optional[ctypes.CDLL] = None


class SNNCudaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def backend() -> ctypes.CDLL:
    """The GPU backend library.  Raises if it has not been built: there is no
    CPU fallback."""
    global _backend
    if _backend is None:
        path = os.environ.get("SNNCUDA_GB300_LIBRARY", str(BACKEND_LIBRARY))
        if not pathlib.Path(path).exists():
            raise SNNCudaError(_abi.SNNCUDA_ERR_DEVICE,
                               f"GPU backend library missing at {path}; run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        _backend = _abi.bind(path)
    return _backend


def default_config(lib: Optional[ctypes.CDLL] = None, **overrides) -> _abi.Config:
    lib = lib or backend()
    cfg = _abi.Config()
    lib.snncuda_config_default(ctypes.byref(cfg))
    for key, value in overrides.items():
        if not hasattr(cfg, key):
            raise AttributeError(f"unknown config field {key}")
        setattr(cfg, key, value)
    return cfg


def _check(lib, status: int) -> None:
    if status != _abi.SNNCUDA_OK:
        raise SNNCudaError(status, lib.snncuda_last_error().decode("utf-8", "replace"))


def _tuning_struct(tuning: Dict[str, object]) -> _abi.Tuning:
    """A Tuning from the dict autotune returns (missing fields stay 0)."""
    t = _abi.Tuning()
    for name, _ in _abi.Tuning._fields_:
        if name in tuning:
            setattr(t, name, tuning[name])
    return t


def _network_struct(c: Connectome):
    """snncuda_network view of a Connectome plus the arrays it points into
    (keep them alive until the create call returns)."""
    keep = [np.ascontiguousarray(a) for a in (
        c.threshold.astype(np.float32, copy=False), c.pattern_window_ticks.astype(np.uint64, copy=False),
        c.similarity_threshold.astype(np.float32, copy=False), c.max_reference_patterns.astype(np.uint64, copy=False),
        c.source.astype(np.uint32, copy=False), c.target.astype(np.uint32, copy=False), c.weight.astype(np.float32, copy=False),
        c.max_weight.astype(np.float32, copy=False), c.delay_ticks.astype(np.uint32, copy=False),
        c.compartment.astype(np.uint8, copy=False), c.receptor.astype(np.uint8, copy=False),
        c.plasticity_enabled.astype(np.uint8, copy=False))]
    (thr, win, sim, refs, src, tgt, w, mw, dly, comp, rec, pl) = keep
    code_ptr = code = None
    if c.code_offset_ptr is not None:
        code_ptr = np.ascontiguousarray(c.code_offset_ptr.astype(np.uint64, copy=False))
        code = np.ascontiguousarray(c.code_offsets.astype(np.uint32, copy=False))
        if code.size == 0:
            code = np.zeros(1, dtype=np.uint32)
        keep += [code_ptr, code]
    net = _abi.Network(
        c.neuron_count, _abi.ptr(thr, c_float), _abi.ptr(win, c_uint64), _abi.ptr(sim, c_float),
        _abi.ptr(refs, c_uint64), c.synapse_count, _abi.ptr(src, c_uint32),
        _abi.ptr(tgt, c_uint32), _abi.ptr(w, c_float), _abi.ptr(mw, c_float),
        _abi.ptr(dly, c_uint32), _abi.ptr(comp, c_uint8), _abi.ptr(rec, c_uint8),
        _abi.ptr(pl, c_uint8), _abi.ptr(code_ptr, c_uint64), _abi.ptr(code, c_uint32))
    return net, keep


def _neuron_arrays(n: int):
    arrays = {
        "membrane_potential": np.zeros(n, np.float32), "spike_count": np.zeros(n, np.uint64),
        "last_fired_tick": np.zeros(n, np.int64), "last_active_tick": np.zeros(n, np.uint64),
        "compartment_current": np.zeros(n * 4, np.float32),
        "compartment_last_update": np.zeros(n * 4, np.uint64),
        "compartment_tau": np.zeros(n * 4, np.float32),
        "window_start_tick": np.zeros(n, np.uint64), "offset_count": np.zeros(n, np.uint64),
        "learned_count": np.zeros(n, np.uint64), "match_count": np.zeros(n, np.uint64),
        "last_match": np.zeros(n, np.uint8),
    }
    types = dict(_abi.NeuronState._fields_)
    view = _abi.NeuronState(**{k: _abi.ptr(v, types[k]._type_) for k, v in arrays.items()})
    return arrays, view


def _finish_neurons(arrays, n: int):
    for k in ("compartment_current", "compartment_last_update", "compartment_tau"):
        arrays[k] = arrays[k].reshape(n, 4)
    return arrays


def _synapse_arrays(s: int):
    arrays = {
        "weight": np.zeros(s, np.float32), "last_pre_spike_tick": np.zeros(s, np.int64),
        "last_post_spike_tick": np.zeros(s, np.int64), "pre_spike_count": np.zeros(s, np.uint64),
        "plasticity_update_count": np.zeros(s, np.uint64),
        "last_weight_delta": np.zeros(s, np.float32),
        "code_window_start_tick": np.zeros(s, np.uint64),
        "code_offset_count": np.zeros(s, np.uint64), "learned_code_count": np.zeros(s, np.uint64),
        "code_match_count": np.zeros(s, np.uint64), "last_code_match": np.zeros(s, np.uint8),
    }
    types = dict(_abi.SynapseState._fields_)
    view = _abi.SynapseState(**{k: _abi.ptr(v, types[k]._type_) for k, v in arrays.items()})
    return arrays, view


def _inject_arrays(neurons, ticks, weights):
    n = np.ascontiguousarray(np.asarray(neurons, dtype=np.uint32).ravel())
    t = np.ascontiguousarray(np.asarray(ticks, dtype=np.uint64).ravel())
    w = np.ascontiguousarray(np.asarray(weights, dtype=np.float32).ravel())
    if not (n.size == t.size == w.size):
        raise ValueError("inject arrays must have equal length")
    return n, t, w


class Simulation:
    """One simulation handle over a Connectome (0-based neuron indices)."""

    def __init__(self, connectome: Connectome, config: Optional[_abi.Config] = None,
                 lib: Optional[ctypes.CDLL] = None):
        connectome.validate()
        self.lib = lib or backend()
        self.connectome = connectome
        self.config = config if config is not None else default_config(self.lib)
        net, self._keep = _network_struct(connectome)
        c = connectome
        handle = c_void_p()
        _check(self.lib, self.lib.snncuda_sim_create(ctypes.byref(net), ctypes.byref(self.config),
                                                     ctypes.byref(handle)))
        self._keep = None  # arrays were copied by create
        self.handle = handle
        self.neuron_count = c.neuron_count
        self.synapse_count = c.synapse_count

    # -- lifecycle -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.snncuda_sim_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- stepping --------------------------------------------------------------
    def inject(self, neurons, ticks, weights) -> None:
        n, t, w = _inject_arrays(neurons, ticks, weights)
        if n.size == 0:
            return
        _check(self.lib, self.lib.snncuda_sim_inject(self.handle, n.size, _abi.ptr(n, c_uint32),
                                                     _abi.ptr(t, c_uint64), _abi.ptr(w, c_float)))

    def run_until(self, inclusive_tick: int) -> None:
        _check(self.lib, self.lib.snncuda_sim_run_until(self.handle, int(inclusive_tick)))

    def set_plasticity(self, enabled: bool) -> None:
        _check(self.lib, self.lib.snncuda_sim_set_plasticity(self.handle, 1 if enabled else 0))

    def set_temporal_learning(self, enabled: bool) -> None:
        _check(self.lib, self.lib.snncuda_sim_set_temporal_learning(self.handle, 1 if enabled else 0))

    # -- readers -----------------------------------------------------------------
    def counters(self) -> Dict[str, int]:
        out = _abi.Counters()
        _check(self.lib, self.lib.snncuda_sim_counters(self.handle, ctypes.byref(out)))
        return {name: int(getattr(out, name)) for name, _ in _abi.Counters._fields_}

    def idle(self) -> bool:
        out = c_int32()
        _check(self.lib, self.lib.snncuda_sim_idle(self.handle, ctypes.byref(out)))
        return bool(out.value)

    def neurons(self) -> Dict[str, np.ndarray]:
        arrays, view = _neuron_arrays(self.neuron_count)
        _check(self.lib, self.lib.snncuda_sim_read_neurons(self.handle, ctypes.byref(view)))
        return _finish_neurons(arrays, self.neuron_count)

    def synapses(self) -> Dict[str, np.ndarray]:
        arrays, view = _synapse_arrays(self.synapse_count)
        _check(self.lib, self.lib.snncuda_sim_read_synapses(self.handle, ctypes.byref(view)))
        return arrays

    def pattern(self, kind: int, index: int, which: int = 0) -> List[int]:
        length = c_uint64()
        buf = np.zeros(64, dtype=np.uint32)
        _check(self.lib, self.lib.snncuda_sim_read_pattern(
            self.handle, kind, index, which, _abi.ptr(buf, c_uint32), buf.size, ctypes.byref(length)))
        if length.value > buf.size:
            buf = np.zeros(length.value, dtype=np.uint32)
            _check(self.lib, self.lib.snncuda_sim_read_pattern(
                self.handle, kind, index, which, _abi.ptr(buf, c_uint32), buf.size,
                ctypes.byref(length)))
        return [int(v) for v in buf[:length.value]]

    def profile(self, inclusive_tick: int) -> Dict[str, object]:
        """Run to `inclusive_tick` one tick at a time with per-kernel device
        timing (engine extension; CPU implementations fill only counters)."""
        out = _abi.Profile()
        _check(self.lib, self.lib.snncuda_sim_profile(self.handle, int(inclusive_tick), ctypes.byref(out)))
        names = [self.lib.snncuda_kernel_name(k).decode() for k in range(_abi.KERNEL_COUNT)]
        return {"ticks": int(out.ticks), "kernel_ms": dict(zip(names, list(out.kernel_ms))),
                "synaptic_events": int(out.synaptic_events), "external_events": int(out.external_events),
                "fires": int(out.fires), "touched_targets": int(out.touched_targets)}

    def recognition(self) -> Dict[str, int]:
        """Sum of the neurons' temporal match counts and of the synapses' code
        match counts."""
        a, b = c_uint64(), c_uint64()
        _check(self.lib, self.lib.snncuda_sim_recognition(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return {"neuron_matches": int(a.value), "synapse_code_matches": int(b.value)}

    def digest(self) -> tuple:
        a, b = c_uint64(), c_uint64()
        _check(self.lib, self.lib.snncuda_sim_state_digest(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def checksum(self) -> tuple:
        """Device-computed (neuron, synapse) state checksums (GPU engine only)."""
        a, b = c_uint64(), c_uint64()
        _check(self.lib, self.lib.snncuda_sim_state_checksum(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def autotune(self, probe_ticks: int = 20) -> Dict[str, object]:
        """Pick launch shapes and the wheel-slot capacity from timed probes of
        the next ticks (engine extension; results are unchanged)."""
        out = _abi.Tuning()
        _check(self.lib, self.lib.snncuda_sim_autotune(self.handle, int(probe_ticks), ctypes.byref(out)))
        return {name: (float(v) if isinstance(v, float) else int(v))
                for name, v in ((n, getattr(out, n)) for n, _ in _abi.Tuning._fields_)}

    def apply_tuning(self, tuning: Dict[str, object]) -> None:
        """Apply launch shapes found earlier by autotune (its returned dict);
        results do not depend on them (engine extension)."""
        _check(self.lib, self.lib.snncuda_sim_apply_tuning(self.handle, ctypes.byref(_tuning_struct(tuning))))

    def evict(self) -> None:
        """Move the state to host memory and free the device memory; the next
        call that needs the device brings it back (engine extension)."""
        _check(self.lib, self.lib.snncuda_sim_evict(self.handle))

    def restore(self) -> None:
        _check(self.lib, self.lib.snncuda_sim_restore(self.handle))

    def residency(self) -> tuple:
        """(state on the device, times evicted)."""
        r, n = c_int32(), c_uint64()
        _check(self.lib, self.lib.snncuda_sim_residency(self.handle, ctypes.byref(r), ctypes.byref(n)))
        return bool(r.value), int(n.value)

    def raster(self, first: int = 0, count: Optional[int] = None) -> tuple:
        """Fire records [first, first+count) as (ticks, neurons); all by default."""
        if count is None:
            count = self.counters()["raster_count"] - first
        ticks = np.zeros(count, np.uint64)
        neurons = np.zeros(count, np.uint32)
        if count:
            _check(self.lib, self.lib.snncuda_sim_read_raster(
                self.handle, first, count, _abi.ptr(ticks, c_uint64), _abi.ptr(neurons, c_uint32)))
        return ticks, neurons


class Batch:
    """Several independent networks advanced together in one handle (batched
    form).  Network i keeps its own 0-based neuron and synapse indices and
    evolves exactly as a Simulation of it alone would; stdp_enabled[i] is its
    StdpConfig::enabled, the rest of `config` is shared."""

    def __init__(self, connectomes: Sequence[Connectome], config: Optional[_abi.Config] = None,
                 lib: Optional[ctypes.CDLL] = None, stdp_enabled: Optional[Sequence[bool]] = None):
        self.lib = lib or backend()
        self.config = config if config is not None else default_config(self.lib)
        nets, keep = [], []
        for c in connectomes:
            c.validate()
            net, k = _network_struct(c)
            nets.append(net)
            keep.append(k)
        self.count = len(nets)
        arr = (_abi.Network * max(self.count, 1))(*nets)
        rule = None
        if stdp_enabled is not None:
            rule = np.ascontiguousarray(np.asarray([1 if x else 0 for x in stdp_enabled], dtype=np.int32))
            if rule.size != self.count:
                raise ValueError("stdp_enabled needs one entry per network")
        handle = c_void_p()
        _check(self.lib, self.lib.snncuda_batch_create(self.count, arr, _abi.ptr(rule, c_int32),
                                                       ctypes.byref(self.config), ctypes.byref(handle)))
        self.handle = handle
        self.neuron_counts = [c.neuron_count for c in connectomes]
        self.synapse_counts = [c.synapse_count for c in connectomes]

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.snncuda_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def inject(self, network: int, neurons, ticks, weights) -> None:
        n, t, w = _inject_arrays(neurons, ticks, weights)
        if n.size == 0:
            return
        _check(self.lib, self.lib.snncuda_batch_inject(self.handle, network, n.size, _abi.ptr(n, c_uint32),
                                                       _abi.ptr(t, c_uint64), _abi.ptr(w, c_float)))

    def run_until(self, inclusive_tick: int) -> None:
        _check(self.lib, self.lib.snncuda_batch_run_until(self.handle, int(inclusive_tick)))

    def set_plasticity(self, enabled: bool) -> None:
        _check(self.lib, self.lib.snncuda_batch_set_plasticity(self.handle, 1 if enabled else 0))

    def set_temporal_learning(self, enabled: bool) -> None:
        _check(self.lib, self.lib.snncuda_batch_set_temporal_learning(self.handle, 1 if enabled else 0))

    def counters(self, network: int) -> Dict[str, int]:
        out = _abi.Counters()
        _check(self.lib, self.lib.snncuda_batch_counters(self.handle, network, ctypes.byref(out)))
        return {name: int(getattr(out, name)) for name, _ in _abi.Counters._fields_}

    def neurons(self, network: int) -> Dict[str, np.ndarray]:
        n = self.neuron_counts[network]
        arrays, view = _neuron_arrays(n)
        _check(self.lib, self.lib.snncuda_batch_read_neurons(self.handle, network, ctypes.byref(view)))
        return _finish_neurons(arrays, n)

    def synapses(self, network: int) -> Dict[str, np.ndarray]:
        arrays, view = _synapse_arrays(self.synapse_counts[network])
        _check(self.lib, self.lib.snncuda_batch_read_synapses(self.handle, network, ctypes.byref(view)))
        return arrays

    def digests(self) -> List[tuple]:
        a = np.zeros(max(self.count, 1), np.uint64)
        b = np.zeros(max(self.count, 1), np.uint64)
        _check(self.lib, self.lib.snncuda_batch_state_digests(self.handle, _abi.ptr(a, c_uint64),
                                                              _abi.ptr(b, c_uint64)))
        return [(int(a[i]), int(b[i])) for i in range(self.count)]

    def autotune(self, probe_ticks: int = 20) -> Dict[str, object]:
        """Simulation.autotune on the batch's tick loop."""
        out = _abi.Tuning()
        _check(self.lib, self.lib.snncuda_batch_autotune(self.handle, int(probe_ticks), ctypes.byref(out)))
        return {name: (float(v) if isinstance(v, float) else int(v))
                for name, v in ((n, getattr(out, n)) for n, _ in _abi.Tuning._fields_)}

    def apply_tuning(self, tuning: Dict[str, object]) -> None:
        """Simulation.apply_tuning on the batch's tick loop."""
        _check(self.lib, self.lib.snncuda_batch_apply_tuning(self.handle, ctypes.byref(_tuning_struct(tuning))))

    def checksums(self) -> List[tuple]:
        """Device-computed (neuron, synapse) checksums of every network, equal
        to Simulation.checksum() of its solo run (GPU engine only)."""
        a = np.zeros(max(self.count, 1), np.uint64)
        b = np.zeros(max(self.count, 1), np.uint64)
        _check(self.lib, self.lib.snncuda_batch_state_checksums(self.handle, _abi.ptr(a, c_uint64),
                                                                _abi.ptr(b, c_uint64)))
        return [(int(a[i]), int(b[i])) for i in range(self.count)]

    def raster(self, network: int) -> tuple:
        count = self.counters(network)["raster_count"]
        ticks = np.zeros(count, np.uint64)
        neurons = np.zeros(count, np.uint32)
        if count:
            _check(self.lib, self.lib.snncuda_batch_read_raster(
                self.handle, network, 0, count, _abi.ptr(ticks, c_uint64), _abi.ptr(neurons, c_uint32)))
        return ticks, neurons


class Server:
    """Serving: jobs admitted in submission order under a device-memory
    budget and advanced `slice_ticks` at a time, each on its own stream.
    With `evict`, a queued job that does not fit preempts running jobs with
    more remaining work; they wait in host memory and resume later.  The
    caller drives it with step(); submit copies the job's arrays."""

    def __init__(self, memory_budget_bytes: int = 0, max_running: int = 0, slice_ticks: int = 0,
                 digests: bool = False, evict: bool = False, lib: Optional[ctypes.CDLL] = None):
        self.lib = lib or backend()
        cfg = _abi.ServerConfig(memory_budget_bytes, max_running, slice_ticks, 1 if digests else 0,
                                1 if evict else 0)
        handle = c_void_p()
        _check(self.lib, self.lib.snncuda_server_create(ctypes.byref(cfg), ctypes.byref(handle)))
        self.handle = handle
        self._keep = {}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.snncuda_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, connectome: Connectome, config: Optional[_abi.Config], drive, ticks: int) -> int:
        connectome.validate()
        net, keep = _network_struct(connectome)
        cfg = config if config is not None else default_config(self.lib)
        n, t, w = _inject_arrays(*drive)
        job = c_uint64()
        _check(self.lib, self.lib.snncuda_server_submit(
            self.handle, ctypes.byref(net), ctypes.byref(cfg), n.size, _abi.ptr(n, c_uint32), _abi.ptr(t, c_uint64),
            _abi.ptr(w, c_float), int(ticks), ctypes.byref(job)))
        return int(job.value)

    def step(self) -> int:
        active = c_uint32()
        _check(self.lib, self.lib.snncuda_server_step(self.handle, ctypes.byref(active)))
        return int(active.value)

    def job(self, job_id: int) -> Dict[str, object]:
        r = _abi.JobResult()
        _check(self.lib, self.lib.snncuda_server_job(self.handle, int(job_id), ctypes.byref(r)))
        return {"state": r.state, "error": r.error,
                "counters": {name: int(getattr(r.counters, name)) for name, _ in _abi.Counters._fields_},
                "digest": (int(r.neuron_digest), int(r.synapse_digest)), "device_bytes": int(r.device_bytes),
                "submitted_s": r.submitted_s, "admitted_s": r.admitted_s, "finished_s": r.finished_s,
                "evictions": int(r.evictions)}


class Readout:
    """The inference session's readout paths over a network's initial weights
    (CudaInferenceSession::run_feedforward_batch / run_recurrent_feedforward_batch).
    Samples are lists of (neuron, weight) pairs (0-based neurons)."""

    def __init__(self, connectome: Connectome, lib: Optional[ctypes.CDLL] = None):
        connectome.validate()
        self.lib = lib or backend()
        net, keep = _network_struct(connectome)
        handle = c_void_p()
        _check(self.lib, self.lib.snncuda_readout_create(ctypes.byref(net), ctypes.byref(handle)))
        self.handle = handle

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.snncuda_readout_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _samples(samples):
        ptr = np.zeros(len(samples) + 1, np.uint64)
        ptr[1:] = np.cumsum([len(s) for s in samples])
        n = np.ascontiguousarray([int(a) for s in samples for a, _ in s] or [0], np.uint32)
        w = np.ascontiguousarray([float(b) for s in samples for _, b in s] or [0.0], np.float32)
        return ptr, n, w

    def feedforward(self, samples, readouts):
        """(scores [samples, readouts] float32, spikes uint64, delivered per sample)."""
        ptr, n, w = self._samples(samples)
        ro = np.ascontiguousarray(readouts, np.uint32)
        S, R = len(samples), ro.size
        scores = np.zeros((S, R), np.float32)
        spikes = np.zeros((S, R), np.uint64)
        delivered = np.zeros(max(S, 1), np.uint64)
        _check(self.lib, self.lib.snncuda_readout_feedforward(
            self.handle, S, _abi.ptr(ptr, c_uint64), _abi.ptr(n, c_uint32), _abi.ptr(w, c_float), R,
            _abi.ptr(ro if R else np.zeros(1, np.uint32), c_uint32), _abi.ptr(scores, c_float),
            _abi.ptr(spikes, c_uint64), _abi.ptr(delivered, c_uint64)))
        return scores, spikes, delivered[:S]

    def recurrent(self, samples, readouts, hidden=None, **options):
        """(scores, spikes, delivered, time steps); options are the fields of
        snncuda_recurrent_options (iterations, feedback_decay,
        top_k_feedback_readouts, top_k_hidden, use_scores_not_spikes)."""
        opt = _abi.RecurrentOptions()
        self.lib.snncuda_recurrent_options_default(ctypes.byref(opt))
        for k, v in options.items():
            setattr(opt, k, v)
        ptr, n, w = self._samples(samples)
        ro = np.ascontiguousarray(readouts, np.uint32)
        hid = np.ascontiguousarray(hidden if hidden is not None else [], np.uint32)
        S, R = len(samples), ro.size
        scores = np.zeros((S, R), np.float32)
        spikes = np.zeros((S, R), np.uint64)
        delivered = np.zeros(max(S, 1), np.uint64)
        steps = c_uint64()
        _check(self.lib, self.lib.snncuda_readout_recurrent(
            self.handle, S, _abi.ptr(ptr, c_uint64), _abi.ptr(n, c_uint32), _abi.ptr(w, c_float), R,
            _abi.ptr(ro if R else np.zeros(1, np.uint32), c_uint32), hid.size,
            _abi.ptr(hid if hid.size else np.zeros(1, np.uint32), c_uint32), ctypes.byref(opt),
            _abi.ptr(scores, c_float), _abi.ptr(spikes, c_uint64), _abi.ptr(delivered, c_uint64),
            ctypes.byref(steps)))
        return scores, spikes, delivered[:S], int(steps.value)


# ---------------------------------------------------------------------------
# Reference-shaped interface
# ---------------------------------------------------------------------------

@dataclass
class CompartmentState:
    current: float
    last_update_tick: int
    decay_tau_ticks: float


@dataclass
class TemporalPatternState:
    window_start_tick: int
    spike_offsets: List[int]
    learned_patterns: List[List[int]]
    last_match: bool
    match_count: int


@dataclass
class NeuronStateView:
    """runtime::NeuronState (NeuronStateCache.h:15-45)."""
    id: int
    membrane_potential: float
    threshold: float
    last_active_tick: int
    last_fired_tick: Optional[int]
    spike_count: int
    soma: CompartmentState
    basal: CompartmentState
    apical: CompartmentState
    inhibitory: CompartmentState
    temporal_pattern: TemporalPatternState


@dataclass
class SynapseStateView:
    """runtime::SynapseRuntimeState (SynapseDendriteProcessor.h:14-35)."""
    id: int
    source: int
    target: int
    weight: float
    max_weight: float
    delay_ticks: int
    spike_code_offsets: List[int]
    plasticity_enabled: bool
    last_pre_spike_tick: Optional[int]
    last_post_spike_tick: Optional[int]
    pre_spike_count: int
    plasticity_update_count: int
    last_weight_delta: float
    code_window_start_tick: int
    code_offsets: List[int]
    learned_code_patterns: List[List[int]]
    code_match_count: int
    last_code_match: bool


class NetworkPropagator:
    """Drop-in for runtime::NetworkPropagator over the GPU backend.

    `store` and `resident_neuron_capacity` are accepted for signature parity:
    neuron state stays resident in device memory, so there is no LRU paging
    (NeuronStateCache only moved state, never changed it).
    """

    def __init__(self, connectome: Connectome, store=None, resident_neuron_capacity: int = 65536,
                 timing_wheel_slots: int = 4096, config: Optional[_abi.Config] = None,
                 lib: Optional[ctypes.CDLL] = None):
        if resident_neuron_capacity == 0:
            raise SNNCudaError(_abi.SNNCUDA_ERR_INVALID_ARGUMENT, "LRU cache capacity must be nonzero")
        lib = lib or backend()
        cfg = config if config is not None else default_config(lib)
        cfg.timing_wheel_slots = timing_wheel_slots
        self.connectome = connectome
        self.sim = Simulation(connectome, cfg, lib)
        self._pending: List[tuple] = []

    def _flush(self) -> None:
        if self._pending:
            n, t, w = zip(*self._pending)
            self._pending = []
            self.sim.inject(n, t, w)

    def inject(self, target: int, delivery_tick: int, weight: float) -> None:
        if not 1 <= target <= self.sim.neuron_count:
            raise SNNCudaError(_abi.SNNCUDA_ERR_INVALID_ARGUMENT, f"unknown neuron id {target}")
        self._pending.append((target - 1, delivery_tick, weight))

    def run_until(self, inclusive_tick: int) -> None:
        self._flush()
        self.sim.run_until(inclusive_tick)

    def set_plasticity(self, enabled: bool) -> None:
        self.sim.set_plasticity(enabled)

    def set_temporal_learning(self, enabled: bool) -> None:
        self.sim.set_temporal_learning(enabled)

    def state(self, neuron_id: int) -> NeuronStateView:
        self._flush()
        i = neuron_id - 1
        a = self.sim.neurons()
        comps = [CompartmentState(float(a["compartment_current"][i, k]),
                                  int(a["compartment_last_update"][i, k]),
                                  float(a["compartment_tau"][i, k])) for k in range(4)]
        learned = [self.sim.pattern(1, i, j) for j in range(int(a["learned_count"][i]))]
        tp = TemporalPatternState(int(a["window_start_tick"][i]), self.sim.pattern(0, i), learned,
                                  bool(a["last_match"][i]), int(a["match_count"][i]))
        lf = int(a["last_fired_tick"][i])
        return NeuronStateView(neuron_id, float(a["membrane_potential"][i]),
                               float(self.connectome.threshold[i]), int(a["last_active_tick"][i]),
                               None if lf < 0 else lf, int(a["spike_count"][i]), *comps, tp)

    def spike_count(self, neuron_id: int) -> int:
        return int(self.sim.neurons()["spike_count"][neuron_id - 1])

    def delivered_spike_count(self) -> int:
        return self.sim.counters()["delivered_spikes"]

    def fired_spike_count(self) -> int:
        return self.sim.counters()["fired_spikes"]

    def synapse_state(self, synapse_id: int) -> Optional[SynapseStateView]:
        i = synapse_id - 1
        if not 0 <= i < self.sim.synapse_count:
            return None
        a = self.sim.synapses()
        c = self.connectome

        def opt(v):
            return None if int(v) < 0 else int(v)

        learned = [self.sim.pattern(3, i, j) for j in range(int(a["learned_code_count"][i]))]
        return SynapseStateView(
            synapse_id, int(c.source[i]) + 1, int(c.target[i]) + 1, float(a["weight"][i]),
            float(c.max_weight[i]), int(c.delay_ticks[i]), c.spike_codes(i),
            bool(c.plasticity_enabled[i]), opt(a["last_pre_spike_tick"][i]),
            opt(a["last_post_spike_tick"][i]), int(a["pre_spike_count"][i]),
            int(a["plasticity_update_count"][i]), float(a["last_weight_delta"][i]),
            int(a["code_window_start_tick"][i]), self.sim.pattern(2, i), learned,
            int(a["code_match_count"][i]), bool(a["last_code_match"][i]))

    def cache_eviction_count(self) -> int:
        """NetworkPropagator::cache_eviction_count (NetworkPropagator.h:27):
        neuron state never leaves device memory here, so nothing is evicted
        (the reference counts its LRU page-outs)."""
        return 0

    def resident_neuron_count(self) -> int:
        """NetworkPropagator::resident_neuron_count (NetworkPropagator.h:28):
        every neuron is resident in device memory (the reference counts the
        neurons its LRU cache currently holds)."""
        return self.sim.neuron_count

    def idle(self) -> bool:
        self._flush()
        return self.sim.idle()
