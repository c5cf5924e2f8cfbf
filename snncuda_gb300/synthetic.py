"""Seeded synthetic SNN workloads (the named benchmark networks).

Wraps the host generator in csrc/gen.cpp (`_lib/libsnncuda_gen.so`).  Each
workload is a `Connectome` plus an injection schedule (external Poisson
drive, and for the recognition workload a repeating temporal-code
stimulus), injected before the run in (tick, neuron) order.

Workloads (the weight scale g is an explicit, recorded knob: at g = 1 the
described weight distributions drive these recurrent networks into runaway
firing under the reference semantics, where a neuron may refire within a
tick):

  plain_1k     1,000 neurons (800 E / 200 I), fan-out 100 (1e5 synapses),
               E weights U[0,0.5]g, I weights U[-1,0]g, delays U{1..20},
               2 compartments (E basal/apical alternating, I inhibitory),
               codes {0}, STDP off per synapse, default neuron params
               (threshold 1, window 500, similarity 0.93, 500 patterns),
               10 Hz drive of weight 1, 1,000 ticks, seed 0.
  stdp_100k    100,000 neurons (80/20), fan-out 1,000 (1e8 synapses),
               lognormal(-1.5, 0.5) weights times g = 0.01 (inhibitory as
               GABA_A magnitude), delays U{1..20}, 4 compartments, 1-4 code
               offsets in U{0..7}, pair STDP (A+ 0.01, A- 0.012, tau 20,
               StdpConfig weights in [0,1]; per-synapse max_weight = g, i.e.
               the [0,1] clip in units of g), window 32, similarity 0.9, 1
               pattern, 5 Hz drive, 10,000 ticks, seed 1.  The reference's
               pair rule potentiates every recently active input at each post
               spike, so with a clip of 1 the weights climb to it and the
               network runs away within a few hundred ticks.
  recog_1m     1,000,000 neurons, fan-out 1,000 (1e9 synapses), stdp_100k
               distributions, plus 16 fixed 8-offset codes (offsets in
               U{0..31}) presented every 64 ticks to the first half of the
               neurons over the 5 Hz background, 2,000 ticks.  Each code
               input has weight 0.1: at 0.25, coinciding offsets make the
               stimulated half fire in the same tick and the network runs
               away (measured on a 10,000-neuron version).
Any of them can be scaled down (neurons, fan-out, ticks) for parity tests.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
from ctypes import POINTER, Structure, c_double, c_float, c_int, c_uint8, c_uint32, c_uint64
from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

from .connectome import Connectome

GEN_LIBRARY = pathlib.Path(__file__).resolve().parent / "_lib" / "libsnncuda_gen.so"


class _Spec(Structure):
    _fields_ = [
        ("neuron_count", c_uint32), ("excitatory_count", c_uint32), ("fanout", c_uint32),
        ("weight_kind", c_uint32), ("weight_scale", c_float), ("lognormal_mu", c_float),
        ("lognormal_sigma", c_float), ("max_weight", c_float), ("delay_min", c_uint32),
        ("delay_max", c_uint32), ("codes_min", c_uint32), ("codes_max", c_uint32),
        ("code_offset_max", c_uint32), ("compartments", c_uint32), ("plastic", c_uint8),
        ("threshold", c_float), ("pattern_window_ticks", c_uint64),
        ("similarity_threshold", c_float), ("max_reference_patterns", c_uint64), ("seed", c_uint64),
    ]


class _Net(Structure):
    _fields_ = [
        ("threshold", POINTER(c_float)), ("pattern_window_ticks", POINTER(c_uint64)),
        ("similarity_threshold", POINTER(c_float)), ("max_reference_patterns", POINTER(c_uint64)),
        ("source", POINTER(c_uint32)), ("target", POINTER(c_uint32)), ("weight", POINTER(c_float)),
        ("max_weight", POINTER(c_float)), ("delay_ticks", POINTER(c_uint32)),
        ("compartment", POINTER(c_uint8)), ("receptor", POINTER(c_uint8)),
        ("plasticity_enabled", POINTER(c_uint8)), ("code_offset_ptr", POINTER(c_uint64)),
        ("code_offsets", POINTER(c_uint32)),
    ]


class _Drive(Structure):
    _fields_ = [("count", c_uint64), ("neuron", POINTER(c_uint32)), ("tick", POINTER(c_uint64)),
                ("weight", POINTER(c_float))]


_gen = None


def _lib():
    global _gen
    if _gen is None:
        path = os.environ.get("SNNCUDA_GEN_LIBRARY", str(GEN_LIBRARY))
        if not pathlib.Path(path).exists():
            raise RuntimeError(f"generator library missing at {path}; run __graft_entry__.build()")
        _gen = ctypes.CDLL(path)
        _gen.snngen_fill_network.argtypes = [POINTER(_Spec), POINTER(_Net), POINTER(c_uint64)]
        _gen.snngen_fill_network.restype = c_int
        _gen.snngen_build_drive.argtypes = [
            c_uint32, c_uint32, c_uint64, c_double, c_float, c_uint32, c_uint32, c_uint32, c_uint32,
            c_uint32, c_uint32, c_float, c_uint64, POINTER(_Drive)]
        _gen.snngen_build_drive.restype = c_int
        _gen.snngen_free_drive.argtypes = [POINTER(_Drive)]
    return _gen


@dataclass
class Workload:
    name: str
    neurons: int
    excitatory_fraction: float
    fanout: int
    weight_kind: int               # 0 uniform E/I, 1 lognormal
    weight_scale: float
    delay: tuple = (1, 20)
    codes: tuple = (1, 1)          # spike-code offsets per synapse
    code_offset_max: int = 0
    compartments: int = 2
    plastic: bool = False
    max_weight: float = 2.0
    threshold: float = 1.0
    pattern_window_ticks: int = 500
    similarity_threshold: float = 0.93
    max_reference_patterns: int = 500
    drive_rate_hz: float = 10.0    # per neuron, 1 ms ticks
    drive_weight: float = 1.0
    ticks: int = 1000
    seed: int = 0
    stdp_enabled: bool = False     # processor toggle
    stimulus_codes: int = 0
    stimulus_code_length: int = 8
    stimulus_offset_max: int = 31
    stimulus_period: int = 64
    stimulus_fraction: float = 0.5
    stimulus_weight: float = 0.25
    lognormal: tuple = (-1.5, 0.5)

    def scaled(self, **changes) -> "Workload":
        return replace(self, **changes)

    @property
    def synapses(self) -> int:
        return self.neurons * self.fanout

    def describe(self) -> dict:
        return {k: (list(v) if isinstance(v, tuple) else v) for k, v in self.__dict__.items()}


PLAIN_1K = Workload("plain_1k", 1000, 0.8, 100, 0, weight_scale=0.3, delay=(1, 20), codes=(1, 1),
                    compartments=2, plastic=False, drive_rate_hz=10.0, ticks=1000, seed=0)
STDP_100K = Workload("stdp_100k", 100_000, 0.8, 1000, 1, weight_scale=0.01, codes=(1, 4),
                     code_offset_max=7, compartments=4, plastic=True, max_weight=0.01,
                     pattern_window_ticks=32, similarity_threshold=0.9, max_reference_patterns=1,
                     drive_rate_hz=5.0, ticks=10_000, seed=1, stdp_enabled=True)
RECOG_1M = STDP_100K.scaled(name="recog_1m", neurons=1_000_000, ticks=2000, seed=2,
                            stimulus_codes=16, stimulus_weight=0.1)
WORKLOADS = {w.name: w for w in (PLAIN_1K, STDP_100K, RECOG_1M)}


def _view(ptr, n, dtype):
    """Copy n elements of a generator-owned C array into a numpy array."""
    dtype = np.dtype(dtype)
    if n == 0:
        return np.zeros(0, dtype=dtype)
    addr = ctypes.cast(ptr, ctypes.c_void_p).value
    raw = (ctypes.c_char * (int(n) * dtype.itemsize)).from_address(addr)
    return np.frombuffer(raw, dtype=dtype).copy()


def build_network(w: Workload) -> Connectome:
    spec = _Spec(
        w.neurons, int(round(w.neurons * w.excitatory_fraction)), w.fanout, w.weight_kind,
        w.weight_scale, w.lognormal[0], w.lognormal[1], w.max_weight, w.delay[0], w.delay[1],
        w.codes[0], w.codes[1], w.code_offset_max, w.compartments, 1 if w.plastic else 0,
        w.threshold, w.pattern_window_ticks, w.similarity_threshold, w.max_reference_patterns, w.seed)
    n, s = w.neurons, w.neurons * w.fanout
    a = dict(threshold=np.empty(n, np.float32), pattern_window_ticks=np.empty(n, np.uint64),
             similarity_threshold=np.empty(n, np.float32), max_reference_patterns=np.empty(n, np.uint64),
             source=np.empty(s, np.uint32), target=np.empty(s, np.uint32), weight=np.empty(s, np.float32),
             max_weight=np.empty(s, np.float32), delay_ticks=np.empty(s, np.uint32),
             compartment=np.empty(s, np.uint8), receptor=np.empty(s, np.uint8),
             plasticity_enabled=np.empty(s, np.uint8), code_offset_ptr=np.empty(s + 1, np.uint64),
             code_offsets=np.empty(max(1, s * w.codes[1]), np.uint32))
    types = dict(_Net._fields_)
    net = _Net(**{k: v.ctypes.data_as(types[k]) for k, v in a.items()})
    count = c_uint64()
    rc = _lib().snngen_fill_network(ctypes.byref(spec), ctypes.byref(net), ctypes.byref(count))
    if rc != 0:
        raise RuntimeError(f"network generation failed ({rc})")
    single = w.codes == (1, 1) and w.code_offset_max == 0
    if single:
        a["code_offset_ptr"] = a["code_offsets"] = None
    else:
        a["code_offsets"] = a["code_offsets"][:count.value]
    return Connectome(**a)


def build_drive(w: Workload, ticks: Optional[int] = None):
    """(neurons, ticks, weights) of the injection schedule, (tick, neuron) order."""
    ticks = w.ticks if ticks is None else ticks
    p = w.drive_rate_hz / 1000.0
    stim = int(w.neurons * w.stimulus_fraction) if w.stimulus_codes else 0
    d = _Drive()
    lib = _lib()
    rc = lib.snngen_build_drive(0, w.neurons, ticks, p, w.drive_weight, w.stimulus_codes,
                                w.stimulus_code_length, w.stimulus_offset_max, w.stimulus_period,
                                0, stim, w.stimulus_weight, w.seed, ctypes.byref(d))
    if rc != 0:
        raise RuntimeError(f"drive generation failed ({rc})")
    try:
        return (_view(d.neuron, d.count, np.uint32), _view(d.tick, d.count, np.uint64),
                _view(d.weight, d.count, np.float32))
    finally:
        lib.snngen_free_drive(ctypes.byref(d))
