"""snncuda_group_events_static: the grouping entry point for callers that
cannot allocate device memory (its scratch is a static array inside the
library).  Through the C ABI, two calls in a row must give exactly the
results of snncuda_group_events (integer output: bit-exact) on the same
inputs, the largest case it accepts must equal the numpy restatement of the
grouping, and sizes beyond the static limits must be refused.  This file is
collected last so a failure here never hides the other tests."""

import numpy as np
import pytest

from test_group_events import expected_grouping

pytestmark = pytest.mark.gpu

MAX_EVENTS = 1 << 20    # SNNCUDA_GROUP_STATIC_MAX_EVENTS
MAX_NEURONS = 1 << 18   # SNNCUDA_GROUP_STATIC_MAX_NEURONS
SNNCUDA_ERR_CAPACITY = 3


def _call(lib, fn, events, neurons):
    import torch
    d_ev = torch.from_numpy(events.view(np.int64)).cuda()
    d_g = torch.full((max(events.size, 1),), -1, dtype=torch.int64, device="cuda")
    d_s = torch.full((neurons + 1,), -1, dtype=torch.int32, device="cuda")
    rc = getattr(lib, fn)(d_ev.data_ptr(), events.size, neurons, d_g.data_ptr(), d_s.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, d_g.cpu().numpy().view(np.uint64)[:events.size], d_s.cpu().numpy().view(np.uint32)


def _events(seed, count, neurons):
    rng = np.random.default_rng(seed)
    tgt = rng.integers(0, neurons, count, dtype=np.uint64)
    ext = np.where(rng.random(count) < 0.1, np.uint64(0x80000000), np.uint64(0))
    payload = rng.integers(0, 1 << 32, count, dtype=np.uint64)
    return (payload << np.uint64(32)) | tgt | ext


def test_static_scratch_matches_allocating_entry_point(gpu_lib):
    cases = [(1, 300_000, 100_000), (2, MAX_EVENTS, MAX_NEURONS), (3, 5_000, 70_000)]
    inputs = [(_events(seed, count, neurons), neurons) for seed, count, neurons in cases]
    expected = [_call(gpu_lib, "snncuda_group_events", ev, n) for ev, n in inputs]
    # the static calls follow one another: each finds the previous call's
    # counters and groups in the shared scratch, so each checks the clearing
    got = [_call(gpu_lib, "snncuda_group_events_static", ev, n) for ev, n in inputs]
    for (rc_a, g_a, s_a), (rc_b, g_b, s_b) in zip(expected, got):
        assert rc_a == 0 and rc_b == 0
        assert np.array_equal(s_a, s_b)
        assert np.array_equal(g_a, g_b)


def test_static_scratch_at_its_limits_equals_the_restatement(gpu_lib):
    ev = _events(4, MAX_EVENTS, MAX_NEURONS)
    rc, grouped, start = _call(gpu_lib, "snncuda_group_events_static", ev, MAX_NEURONS)
    want_g, want_s = expected_grouping(ev, MAX_NEURONS)
    assert rc == 0
    assert np.array_equal(start, want_s)
    assert np.array_equal(grouped, want_g)
    # no events over the largest neuron count: every segment empty
    rc, _, start = _call(gpu_lib, "snncuda_group_events_static", np.zeros(0, np.uint64), MAX_NEURONS)
    assert rc == 0 and not start.any()


def test_static_scratch_refuses_sizes_beyond_its_limits(gpu_lib):
    ev = _events(3, 16, 8)
    assert _call(gpu_lib, "snncuda_group_events_static", ev, MAX_NEURONS + 1)[0] == SNNCUDA_ERR_CAPACITY
    ev = _events(5, MAX_EVENTS + 1, 1000)
    assert _call(gpu_lib, "snncuda_group_events_static", ev, 1000)[0] == SNNCUDA_ERR_CAPACITY
