"""ctypes description of the C ABI in include/snncuda_gb300.h.

`bind(path)` loads any shared library that implements that ABI and returns
it with argument/result types set.  The GPU backend (libsnncuda_gb300.so) is
the product; tests also bind the CPU oracle libraries through the same
description so that every implementation is driven identically.
"""

from __future__ import annotations

import ctypes
from ctypes import (POINTER, Structure, c_char_p, c_float, c_int, c_int32, c_int64,
                    c_uint8, c_uint32, c_uint64, c_void_p)

SNNCUDA_OK = 0
SNNCUDA_ERR_INVALID_ARGUMENT = 1
SNNCUDA_ERR_OUT_OF_MEMORY = 2
SNNCUDA_ERR_CAPACITY = 3
SNNCUDA_ERR_DEVICE = 4
SNNCUDA_ERR_TIMEOUT = 5
SNNCUDA_ERR_UNSUPPORTED = 6
SNNCUDA_ERR_POISONED = 7

STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "out of memory", 3: "capacity exceeded",
    4: "device error", 5: "device wait timeout", 6: "unsupported", 7: "poisoned",
}


class Network(Structure):
    _fields_ = [
        ("neuron_count", c_uint32),
        ("threshold", POINTER(c_float)),
        ("pattern_window_ticks", POINTER(c_uint64)),
        ("similarity_threshold", POINTER(c_float)),
        ("max_reference_patterns", POINTER(c_uint64)),
        ("synapse_count", c_uint64),
        ("source", POINTER(c_uint32)),
        ("target", POINTER(c_uint32)),
        ("weight", POINTER(c_float)),
        ("max_weight", POINTER(c_float)),
        ("delay_ticks", POINTER(c_uint32)),
        ("compartment", POINTER(c_uint8)),
        ("receptor", POINTER(c_uint8)),
        ("plasticity_enabled", POINTER(c_uint8)),
        ("code_offset_ptr", POINTER(c_uint64)),
        ("code_offsets", POINTER(c_uint32)),
    ]


class Config(Structure):
    _fields_ = [
        ("stdp_enabled", c_int32),
        ("ltp_amplitude", c_float),
        ("ltd_amplitude", c_float),
        ("ltp_tau_ticks", c_float),
        ("ltd_tau_ticks", c_float),
        ("min_weight", c_float),
        ("max_weight", c_float),
        ("temporal_learning_enabled", c_int32),
        ("timing_wheel_slots", c_uint64),
        ("slot_event_capacity", c_uint64),
        ("pattern_run_capacity", c_uint64),
        ("raster_capacity", c_uint64),
        ("cuda_stream", c_void_p),
        ("stage_wait_ns", c_uint64),
    ]


class Counters(Structure):
    _fields_ = [
        ("delivered_spikes", c_uint64),
        ("fired_spikes", c_uint64),
        ("synaptic_events", c_uint64),
        ("external_events", c_uint64),
        ("next_tick", c_uint64),
        ("pending_events", c_uint64),
        ("raster_count", c_uint64),
        ("max_slot_events", c_uint64),
    ]


class Tuning(Structure):
    _fields_ = [
        ("grid_events", c_uint32), ("grid_walk", c_uint32), ("grid_bucket", c_uint32),
        ("grid_temporal", c_uint32), ("ticks_per_graph", c_uint32), ("block_threads", c_uint32),
        ("slot_event_capacity", c_uint64), ("max_slot_events", c_uint64),
        ("ms_per_tick_before", ctypes.c_double), ("ms_per_tick_after", ctypes.c_double),
        ("probes", c_uint32), ("probe_ticks", c_uint64), ("scatter_pass_events", c_uint32),
        ("side_serial", c_uint32),
    ]


class RecurrentOptions(Structure):
    _fields_ = [
        ("iterations", c_uint32), ("feedback_decay", c_float), ("top_k_feedback_readouts", c_uint32),
        ("top_k_hidden", c_uint32), ("use_scores_not_spikes", c_int32),
    ]


class ServerConfig(Structure):
    _fields_ = [
        ("memory_budget_bytes", c_uint64),
        ("max_running", c_uint32),
        ("slice_ticks", c_uint32),
        ("digests", c_int32),
        ("evict", c_int32),
    ]


class JobResult(Structure):
    _fields_ = [
        ("state", c_int32),
        ("error", c_int32),
        ("counters", Counters),
        ("neuron_digest", c_uint64),
        ("synapse_digest", c_uint64),
        ("device_bytes", c_uint64),
        ("submitted_s", ctypes.c_double),
        ("admitted_s", ctypes.c_double),
        ("finished_s", ctypes.c_double),
        ("evictions", c_uint64),
    ]


class NeuronState(Structure):
    _fields_ = [
        ("membrane_potential", POINTER(c_float)),
        ("spike_count", POINTER(c_uint64)),
        ("last_fired_tick", POINTER(c_int64)),
        ("last_active_tick", POINTER(c_uint64)),
        ("compartment_current", POINTER(c_float)),
        ("compartment_last_update", POINTER(c_uint64)),
        ("compartment_tau", POINTER(c_float)),
        ("window_start_tick", POINTER(c_uint64)),
        ("offset_count", POINTER(c_uint64)),
        ("learned_count", POINTER(c_uint64)),
        ("match_count", POINTER(c_uint64)),
        ("last_match", POINTER(c_uint8)),
    ]


class SynapseState(Structure):
    _fields_ = [
        ("weight", POINTER(c_float)),
        ("last_pre_spike_tick", POINTER(c_int64)),
        ("last_post_spike_tick", POINTER(c_int64)),
        ("pre_spike_count", POINTER(c_uint64)),
        ("plasticity_update_count", POINTER(c_uint64)),
        ("last_weight_delta", POINTER(c_float)),
        ("code_window_start_tick", POINTER(c_uint64)),
        ("code_offset_count", POINTER(c_uint64)),
        ("learned_code_count", POINTER(c_uint64)),
        ("code_match_count", POINTER(c_uint64)),
        ("last_code_match", POINTER(c_uint8)),
    ]


KERNEL_COUNT = 10


class Profile(Structure):
    _fields_ = [
        ("ticks", c_uint64),
        ("kernel_ms", ctypes.c_double * KERNEL_COUNT),
        ("synaptic_events", c_uint64),
        ("external_events", c_uint64),
        ("fires", c_uint64),
        ("touched_targets", c_uint64),
    ]


_SIGNATURES = {
    "snncuda_version": (c_char_p, []),
    "snncuda_cuda_available": (c_int, []),
    "snncuda_last_error": (c_char_p, []),
    "snncuda_config_default": (None, [POINTER(Config)]),
    "snncuda_sim_create": (c_int, [POINTER(Network), POINTER(Config), POINTER(c_void_p)]),
    "snncuda_sim_destroy": (c_int, [c_void_p]),
    "snncuda_sim_inject": (c_int, [c_void_p, c_uint64, POINTER(c_uint32), POINTER(c_uint64),
                                   POINTER(c_float)]),
    "snncuda_sim_run_until": (c_int, [c_void_p, c_uint64]),
    "snncuda_sim_set_plasticity": (c_int, [c_void_p, c_int32]),
    "snncuda_sim_set_temporal_learning": (c_int, [c_void_p, c_int32]),
    "snncuda_sim_counters": (c_int, [c_void_p, POINTER(Counters)]),
    "snncuda_sim_idle": (c_int, [c_void_p, POINTER(c_int32)]),
    "snncuda_sim_read_neurons": (c_int, [c_void_p, POINTER(NeuronState)]),
    "snncuda_sim_read_synapses": (c_int, [c_void_p, POINTER(SynapseState)]),
    "snncuda_sim_read_pattern": (c_int, [c_void_p, c_int32, c_uint64, c_uint64, POINTER(c_uint32),
                                         c_uint64, POINTER(c_uint64)]),
    "snncuda_sim_state_digest": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_sim_read_raster": (c_int, [c_void_p, c_uint64, c_uint64, POINTER(c_uint64),
                                        POINTER(c_uint32)]),
    "snncuda_sim_profile": (c_int, [c_void_p, c_uint64, POINTER(Profile)]),
    "snncuda_kernel_name": (c_char_p, [c_int32]),
    "snncuda_sim_recognition": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_batch_create": (c_int, [c_uint32, POINTER(Network), POINTER(c_int32), POINTER(Config),
                                     POINTER(c_void_p)]),
    "snncuda_batch_destroy": (c_int, [c_void_p]),
    "snncuda_batch_inject": (c_int, [c_void_p, c_uint32, c_uint64, POINTER(c_uint32), POINTER(c_uint64),
                                     POINTER(c_float)]),
    "snncuda_batch_run_until": (c_int, [c_void_p, c_uint64]),
    "snncuda_batch_set_plasticity": (c_int, [c_void_p, c_int32]),
    "snncuda_batch_set_temporal_learning": (c_int, [c_void_p, c_int32]),
    "snncuda_batch_counters": (c_int, [c_void_p, c_uint32, POINTER(Counters)]),
    "snncuda_batch_read_neurons": (c_int, [c_void_p, c_uint32, POINTER(NeuronState)]),
    "snncuda_batch_read_synapses": (c_int, [c_void_p, c_uint32, POINTER(SynapseState)]),
    "snncuda_batch_state_digests": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_batch_read_raster": (c_int, [c_void_p, c_uint32, c_uint64, c_uint64, POINTER(c_uint64),
                                          POINTER(c_uint32)]),
    "snncuda_server_create": (c_int, [POINTER(ServerConfig), POINTER(c_void_p)]),
    "snncuda_server_destroy": (c_int, [c_void_p]),
    "snncuda_server_submit": (c_int, [c_void_p, POINTER(Network), POINTER(Config), c_uint64, POINTER(c_uint32),
                                      POINTER(c_uint64), POINTER(c_float), c_uint64, POINTER(c_uint64)]),
    "snncuda_server_step": (c_int, [c_void_p, POINTER(c_uint32)]),
    "snncuda_server_job": (c_int, [c_void_p, c_uint64, POINTER(JobResult)]),
    "snncuda_sim_estimate_bytes": (c_int, [POINTER(Network), POINTER(Config), POINTER(c_uint64)]),
    "snncuda_sim_state_checksum": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_batch_state_checksums": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_sim_autotune": (c_int, [c_void_p, c_uint64, POINTER(Tuning)]),
    "snncuda_batch_autotune": (c_int, [c_void_p, c_uint64, POINTER(Tuning)]),
    "snncuda_sim_apply_tuning": (c_int, [c_void_p, POINTER(Tuning)]),
    "snncuda_batch_apply_tuning": (c_int, [c_void_p, POINTER(Tuning)]),
    "snncuda_sim_set_slot_capacity": (c_int, [c_void_p, c_uint64]),
    "snncuda_readout_create": (c_int, [POINTER(Network), POINTER(c_void_p)]),
    "snncuda_readout_destroy": (c_int, [c_void_p]),
    "snncuda_readout_feedforward": (c_int, [c_void_p, c_uint32, POINTER(c_uint64), POINTER(c_uint32),
                                            POINTER(c_float), c_uint32, POINTER(c_uint32), POINTER(c_float),
                                            POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_recurrent_options_default": (None, [POINTER(RecurrentOptions)]),
    "snncuda_readout_recurrent": (c_int, [c_void_p, c_uint32, POINTER(c_uint64), POINTER(c_uint32),
                                          POINTER(c_float), c_uint32, POINTER(c_uint32), c_uint32,
                                          POINTER(c_uint32), POINTER(RecurrentOptions), POINTER(c_float),
                                          POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64)]),
    "snncuda_sim_evict": (c_int, [c_void_p]),
    "snncuda_sim_restore": (c_int, [c_void_p]),
    "snncuda_sim_residency": (c_int, [c_void_p, POINTER(c_int32), POINTER(c_uint64)]),
    "snncuda_group_events": (c_int, [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]),
    "snncuda_group_events_static": (c_int, [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]),
}

# Symbols every implementation of the ABI must export.
ABI_SYMBOLS = tuple(_SIGNATURES)


def bind(path: str) -> ctypes.CDLL:
    """Load a library implementing the ABI and set its ctypes signatures."""
    lib = ctypes.CDLL(path)
    for name, (restype, argtypes) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    return lib


def ptr(array, ctype):
    """ctypes pointer to a contiguous numpy array (None passes NULL)."""
    if array is None:
        return None
    return array.ctypes.data_as(POINTER(ctype))
