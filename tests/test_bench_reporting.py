"""The bench line's derived figures, computed from known inputs on the CPU:
the dominant kernel's roofline (minimal bytes per launch over its launch
time, the layout's bytes, the measured traffic scaled to a launch), the
whole-tick roofline, and the batched leg's per-size breakdown and bound."""

import importlib.util
import pathlib

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _prof():
    # 100 profiled ticks: k_events 2.0 ms per tick in total, 1e6 synaptic and
    # 1e4 external events per tick, 5e4 touched targets per tick
    return {"ticks": 100, "kernel_ms": {"k_events": 200.0, "k_process": 50.0, "k_bcount": 10.0},
            "synaptic_events": 100_000_000, "external_events": 1_000_000, "touched_targets": 5_000_000,
            "fires": 50_000}


def test_kernel_roofline_from_counters(bench):
    from snncuda_gb300 import synthetic
    w = synthetic.RECOG_1M
    peak, _ = bench.load_peaks()
    r = bench.kernel_roofline(w, _prof(), full_size=True)
    assert r["kernel"] == "k_events" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    per_syn, per_ext, per_tgt = bench.MINIMAL_BYTES["k_events"]
    algo = (per_syn * 1e6 + per_ext * 1e4 + per_tgt * 5e4)  # bytes per launch
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(algo)
    assert r["avg_launch_us"] == pytest.approx(2000.0)
    assert r["achieved"] == pytest.approx(algo / 2e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    ls, le, lt = bench.LAYOUT_BYTES["k_events"]
    assert r["layout_bytes_per_launch"] == pytest.approx(ls * 1e6 + le * 1e4 + lt * 5e4)
    # measured DRAM bytes per synaptic event, scaled to the launch's events
    assert r["traffic"] == pytest.approx(bench.MEASURED_TRAFFIC_PER_EVENT["k_events"] * 1e6)
    assert sum(r["kernel_share"].values()) == pytest.approx(1.0)
    # a reduced case reports no full-size traffic
    assert bench.kernel_roofline(w, _prof(), full_size=False)["traffic"] is None


def test_tick_roofline_counts_every_term(bench):
    from snncuda_gb300 import synthetic
    w = synthetic.RECOG_1M
    events, fires, ext, ticks, ms = 80_000_000, 40_000, 800_000, 80, 160.0
    r = bench.tick_roofline(w, events, fires, ext, _prof(), ticks, ms)
    touched = 5_000_000 / 100 * ticks
    b = bench.minimal_tick_bytes(w, events, fires, ext, touched)
    assert r["bytes_per_event"] == pytest.approx(b / events)
    assert r["achieved"] == pytest.approx(b / 0.160 / 1e9)
    assert bench.tick_roofline(w, events, fires, ext, None, ticks, ms) is None


def test_sequential_by_size_bands_and_bound(bench):
    # (neurons, events, ms) of networks run one handle each
    solo = [(2_000, 1e8, 400.0), (5_000, 2e8, 500.0), (30_000, 2e9, 1_000.0), (150_000, 1e10, 2_000.0)]
    out = bench.sequential_by_size(solo)
    bands = out["bands"]
    assert [b["networks"] for b in bands] == [2, 1, 1]
    assert bands[0]["events"] == pytest.approx(3e8) and bands[0]["ms"] == pytest.approx(900.0)
    assert bands[2]["events_per_s"] == pytest.approx(1e10 / 2.0)
    best = max(e / (ms / 1e3) for _, e, ms in solo)
    assert out["best_single_rate"] == pytest.approx(best)
    total_e = sum(e for _, e, _ in solo)
    total_s = sum(ms for _, _, ms in solo) / 1e3
    assert out["speedup_if_batched_at_best_single_rate"] == pytest.approx(best * total_s / total_e)
