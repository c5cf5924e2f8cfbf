"""The grouping building block (snncuda_group_events): a tick's due events
regrouped by target neuron with due order kept inside each target, checked
against a numpy restatement on random event buffers (CPU oracle here, GPU
backend under the gpu mark)."""

import numpy as np
import pytest

EXT = np.uint64(0x80000000)


def make_events(rng, count, neurons, external_fraction=0.1):
    tgt = rng.integers(0, neurons, count, dtype=np.uint64)
    ext = rng.random(count) < external_fraction
    payload = rng.integers(0, 1 << 32, count, dtype=np.uint64)
    return (payload << np.uint64(32)) | tgt | np.where(ext, EXT, np.uint64(0))


def expected_grouping(events, neurons):
    lo = events & np.uint64(0xFFFFFFFF)
    tgt = (lo & np.uint64(0x7FFFFFFF)).astype(np.int64)
    order = np.argsort(tgt, kind="stable")
    idx = np.arange(events.size, dtype=np.uint64)
    word = (events & np.uint64(0xFFFFFFFF00000000)) | idx | (lo & EXT)
    start = np.zeros(neurons + 1, np.uint32)
    np.cumsum(np.bincount(tgt, minlength=neurons), out=start[1:])
    return word[order], start


def run_host(lib, events, neurons):
    grouped = np.zeros(max(events.size, 1), np.uint64)
    start = np.zeros(neurons + 1, np.uint32)
    rc = lib.snncuda_group_events(events.ctypes.data, events.size, neurons, grouped.ctypes.data,
                                  start.ctypes.data, None)
    return rc, grouped[:events.size], start


@pytest.mark.parametrize("count,neurons", [(0, 5), (1, 1), (1000, 37), (50_000, 4096)])
def test_oracle_grouping(port_lib, count, neurons):
    rng = np.random.default_rng(count + neurons)
    ev = make_events(rng, count, neurons)
    rc, g, s = run_host(port_lib, ev, neurons)
    assert rc == 0
    want_g, want_s = expected_grouping(ev, neurons)
    assert np.array_equal(g, want_g) and np.array_equal(s, want_s)


def test_oracle_rejects_bad_target(port_lib):
    ev = np.array([5], np.uint64)
    assert run_host(port_lib, ev, 5)[0] == 1


def test_oracle_rejects_overlapping_output(port_lib):
    """No in-place grouping: events and grouped must not overlap (the same
    contract on the GPU)."""
    ev = np.arange(8, dtype=np.uint64) % np.uint64(3)
    start = np.zeros(4, np.uint32)
    for shift in (0, 8, 56):
        rc = port_lib.snncuda_group_events(ev.ctypes.data, ev.size, 3, ev.ctypes.data + shift, start.ctypes.data,
                                           None)
        assert rc == 1, shift


def run_device(lib, events, neurons, fn="snncuda_group_events"):
    import torch
    d_ev = torch.from_numpy(events.view(np.int64)).cuda()
    d_g = torch.zeros(max(events.size, 1), dtype=torch.int64, device="cuda")
    d_s = torch.zeros(neurons + 1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = getattr(lib, fn)(d_ev.data_ptr(), events.size, neurons, d_g.data_ptr(), d_s.data_ptr(),
                          stream.cuda_stream)
    torch.cuda.synchronize()
    return rc, d_g.cpu().numpy().view(np.uint64)[:events.size], d_s.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("count,neurons", [(1, 1), (1000, 37), (300_000, 100_000), (200_000, 50)])
def test_gpu_grouping(gpu_lib, count, neurons):
    rng = np.random.default_rng(count * 7 + neurons)
    ev = make_events(rng, count, neurons)
    rc, g, s = run_device(gpu_lib, ev, neurons)
    assert rc == 0
    want_g, want_s = expected_grouping(ev, neurons)
    assert np.array_equal(s, want_s)
    assert np.array_equal(g, want_g)


@pytest.mark.gpu
def test_gpu_grouping_rejects_bad_target(gpu_lib):
    ev = np.array([3, 9], np.uint64)
    assert run_device(gpu_lib, ev, 5)[0] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("fn", ["snncuda_group_events", "snncuda_group_events_static"])
def test_gpu_grouping_rejects_overlapping_output(gpu_lib, fn):
    import torch
    d_ev = torch.zeros(16, dtype=torch.int64, device="cuda")
    d_s = torch.zeros(4, dtype=torch.int32, device="cuda")
    for shift in (0, 8, 120):
        rc = getattr(gpu_lib, fn)(d_ev.data_ptr(), 16, 3, d_ev.data_ptr() + shift, d_s.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream)
        assert rc == 1, shift


@pytest.mark.gpu
@pytest.mark.timeout(300)
@pytest.mark.parametrize("fn", ["snncuda_group_events", "snncuda_group_events_static"])
def test_gpu_grouping_one_hot_target(gpu_lib, fn):
    """2^20 events, most of them on one neuron: the long segment is merge-
    sorted by one warp (O(n log^2 n)), not ranked by counting (O(n^2))."""
    rng = np.random.default_rng(17)
    count, neurons = 1 << 20, 4096
    ev = make_events(rng, count, neurons)
    hot = rng.random(count) < 0.9
    ev[hot] = (ev[hot] & ~np.uint64(0x7FFFFFFF)) | np.uint64(123)
    rc, g, s = run_device(gpu_lib, ev, neurons, fn)
    assert rc == 0
    want_g, want_s = expected_grouping(ev, neurons)
    assert np.array_equal(s, want_s)
    assert np.array_equal(g, want_g)


@pytest.mark.gpu
@pytest.mark.timeout(300)
def test_gpu_grouping_unaligned_input_two_passes(gpu_lib):
    """An input array that starts 8 bytes past a 16-byte boundary and has an
    odd length (the counting and placing blocks stream their chunks with
    bulk copies, which need 16-byte alignment: the first and last entries of
    a chunk come in directly), and more than 2^22 events (placed in two
    passes over the bucket ranges)."""
    import torch
    rng = np.random.default_rng(29)
    count, neurons = (1 << 22) + 400_001, 300_000
    ev = make_events(rng, count, neurons)
    d_all = torch.zeros(count + 1, dtype=torch.int64, device="cuda")
    d_all[1:] = torch.from_numpy(ev.view(np.int64)).cuda()
    d_g = torch.zeros(count, dtype=torch.int64, device="cuda")
    d_s = torch.zeros(neurons + 1, dtype=torch.int32, device="cuda")
    rc = gpu_lib.snncuda_group_events(d_all.data_ptr() + 8, count, neurons, d_g.data_ptr(), d_s.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0
    want_g, want_s = expected_grouping(ev, neurons)
    assert np.array_equal(d_s.cpu().numpy().view(np.uint32), want_s)
    assert np.array_equal(d_g.cpu().numpy().view(np.uint64), want_g)
