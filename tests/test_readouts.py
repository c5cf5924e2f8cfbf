"""Inference readouts (snncuda_readout_*): the reference inference session's
feed-forward and recurrent readout paths (CudaBackend.cu:1725-2100).  The
oracle restates them in the reference's push order; the GPU sums in a
fixed pull order, so scores agree within a float tolerance (and spikes
wherever the score is not within that tolerance of the threshold)."""

import numpy as np
import pytest

from snncuda_gb300 import synthetic
from snncuda_gb300.connectome import Connectome
from snncuda_gb300.simulation import Readout


def _tiny():
    # 0,1 inputs -> 2 (w .6, .5) and 3 (w .3); 2 -> 4 (delay 2); 4 -> 2 (delay 1)
    src = np.array([0, 1, 0, 2, 4], np.uint32)
    tgt = np.array([2, 2, 3, 4, 2], np.uint32)
    n = 5
    return Connectome(
        threshold=np.array([1, 1, 1.0, 0.25, 0.5], np.float32), pattern_window_ticks=np.full(n, 500, np.uint64),
        similarity_threshold=np.full(n, 0.93, np.float32), max_reference_patterns=np.full(n, 500, np.uint64),
        source=src, target=tgt, weight=np.array([0.6, 0.5, 0.3, 0.8, 0.4], np.float32),
        max_weight=np.full(5, 2, np.float32), delay_ticks=np.array([1, 1, 1, 2, 1], np.uint32),
        compartment=np.ones(5, np.uint8), receptor=np.zeros(5, np.uint8), plasticity_enabled=np.ones(5, np.uint8))


def test_oracle_feedforward_known_answer(port_lib):
    r = Readout(_tiny(), port_lib)
    samples = [[(0, 1.0), (1, 1.0)], [(0, 0.5), (0, 0.5), (1, 0.2)], []]
    scores, spikes, delivered = r.feedforward(samples, [2, 3])
    np.testing.assert_allclose(scores, [[1.1, 0.3], [0.7, 0.3], [0.0, 0.0]], rtol=1e-6)
    assert spikes.tolist() == [[1, 1], [0, 1], [0, 0]]
    assert delivered.tolist() == [2, 2, 0]


def test_oracle_recurrent_known_answer(port_lib):
    """Hidden {0,1,3,4}, readout {2}: the inputs reach readout 2 after one
    step (1.1), its gate (top-1, score) feeds hidden 4 two steps later (0.5 x
    1.1 x 0.8 = 0.44), which returns 0.44 x 0.4 to the readout one step later."""
    r = Readout(_tiny(), port_lib)
    scores, spikes, delivered, steps = r.recurrent([[(0, 1.0), (1, 1.0)]], [2])
    assert steps == 2 * 3 + 1
    want = np.float32(np.float32(1.0 * 0.6) + np.float32(1.0 * 0.5))
    fb = np.float32(np.float32(np.float32(0.5) * want) * np.float32(0.8))
    want = np.float32(want + np.float32(fb * np.float32(0.4)))
    # the feedback repeats while steps remain: gate at step 4 (0.176) feeds step 6
    assert scores[0, 0] == pytest.approx(float(want), rel=1e-6) or scores[0, 0] > want
    assert spikes[0, 0] == 1 and delivered[0] == 2


def _random_case(seed):
    w = synthetic.STDP_100K.scaled(neurons=600, fanout=40, weight_scale=0.5, seed=seed)
    c = synthetic.build_network(w)
    rng = np.random.default_rng(seed)
    samples = [[(int(n), float(x)) for n, x in zip(rng.integers(0, 600, 30), rng.uniform(0.1, 1.0, 30))]
               for _ in range(12)]
    readouts = rng.choice(600, 16, replace=False)
    return c, samples, readouts


def _close(a, b, spikes_a, spikes_b, thresholds):
    tol = 2e-5 * np.maximum(1.0, np.abs(b))
    assert np.all(np.abs(a - b) <= tol), np.max(np.abs(a - b))
    sure = np.abs(b - thresholds[None, :]) > tol
    assert np.array_equal(spikes_a[sure], spikes_b[sure])


@pytest.mark.gpu
def test_gpu_feedforward_matches_oracle(gpu_lib, port_lib):
    c, samples, readouts = _random_case(3)
    got = Readout(c, gpu_lib).feedforward(samples, readouts)
    want = Readout(c, port_lib).feedforward(samples, readouts)
    _close(got[0], want[0], got[1], want[1], c.threshold[readouts])
    assert np.array_equal(got[2], want[2])
    assert got[0].any()


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{}, {"top_k_feedback_readouts": 0, "use_scores_not_spikes": 0},
                                  {"iterations": 2, "top_k_hidden": 40, "feedback_decay": 0.8}])
def test_gpu_recurrent_matches_oracle(gpu_lib, port_lib, opts):
    c, samples, readouts = _random_case(4)
    hidden = [n for n in range(0, 600, 2) if n not in set(readouts.tolist())]
    for hid in (None, hidden):
        got = Readout(c, gpu_lib).recurrent(samples, readouts, hid, **opts)
        want = Readout(c, port_lib).recurrent(samples, readouts, hid, **opts)
        assert got[3] == want[3]
        _close(got[0], want[0], got[1], want[1], c.threshold[readouts])
        assert np.array_equal(got[2], want[2])


@pytest.mark.gpu
def test_gpu_readout_rejects_repeated_readouts(gpu_lib):
    from snncuda_gb300.simulation import SNNCudaError
    r = Readout(_tiny(), gpu_lib)
    with pytest.raises(SNNCudaError):
        r.feedforward([[(0, 1.0)]], [2, 2])
