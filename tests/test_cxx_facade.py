"""The header-only C++ facade (include/snncuda_gb300.hpp) with the reference's
CudaBackend / CudaInferenceSession names: a small program is compiled
against it, linked to a library implementing the C ABI, and its results are
compared with the Python API on the same network.  It is also compiled
against the reference's own declarative::Connectome where those headers are
present."""

import json
import os
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GPU_PATH, PORT_PATH, ROOT, _ensure_built
from snncuda_gb300.connectome import Connectome
from snncuda_gb300.simulation import Simulation, default_config

REF_INCLUDE = pathlib.Path(os.environ.get("SNNCUDA_REFERENCE_DIR", "/root/reference")) / "include"

MOCK = r"""
#include <cstdint>
#include <vector>
struct Params { float threshold{1.0F}; std::uint64_t pattern_window_ticks{500}; float similarity_threshold{0.93F};
                std::size_t max_reference_patterns{500}; };
struct Neuron { std::uint64_t id; Params params; };
enum class Comp { Soma, Basal, Apical, Inhibitory };
enum class Rec { Ampa, Nmda, GabaA, GabaB };
struct Syn { std::uint64_t id; std::uint64_t source, target; float weight{1.0F}; float max_weight{2.0F};
             std::uint32_t delay_ticks{1}; std::vector<std::uint32_t> spike_code_offsets{0};
             Comp compartment{Comp::Basal}; Rec receptor{Rec::Ampa}; bool plasticity_enabled{true}; };
struct Connectome { std::vector<Neuron> neurons; std::vector<Syn> synapses; };
using NeuronT = Neuron; using SynT = Syn; using Comp_ = Comp; using Rec_ = Rec;
"""

REAL = r"""
#include "snncuda/declarative/Connectome.h"
using Connectome = snncuda::declarative::Connectome;
using NeuronT = snncuda::declarative::ConnectomeNeuron;
using SynT = snncuda::declarative::ConnectomeSynapse;
using Comp_ = snncuda::snn::DendriticCompartment;
using Rec_ = snncuda::snn::ReceptorType;
"""

PROGRAM = r"""
#include <cstdio>
#include "snncuda_gb300.hpp"

// ring of 6 neurons (ids 1..6) with spike codes, and a side input
static Connectome make() {
    Connectome c;
    for (std::uint64_t i = 1; i <= 6; ++i) {
        NeuronT n;
        n.id = i;
        n.params.threshold = 1.0F;
        n.params.pattern_window_ticks = 20;
        n.params.similarity_threshold = 0.9F;
        n.params.max_reference_patterns = 2;
        c.neurons.push_back(n);
    }
    for (std::uint64_t i = 1; i <= 6; ++i) {
        SynT s;
        s.id = i;
        s.source = i;
        s.target = i % 6 + 1;
        s.weight = 2.0F;
        s.max_weight = 1.0F;
        s.delay_ticks = 1 + static_cast<std::uint32_t>(i % 3);
        s.spike_code_offsets = i % 2 ? std::vector<std::uint32_t>{0, 1} : std::vector<std::uint32_t>{0};
        s.compartment = static_cast<Comp_>(i % 4 == 3 ? 1 : i % 4);
        s.receptor = static_cast<Rec_>(i % 2);
        s.plasticity_enabled = i != 4;
        c.synapses.push_back(s);
    }
    return c;
}

int main() {
    const Connectome c = make();
    snncuda_gb300::CudaBackend backend;
    const auto r = backend.run_resident_propagation(c, {1, 3}, 40);
    std::printf("{\"executed\": %d, \"delivered\": %llu, \"fired\": %llu, \"weights\": [", r.executed ? 1 : 0,
                (unsigned long long)r.delivered_spikes, (unsigned long long)r.fired_spikes);
    for (std::size_t i = 0; i < r.final_synapse_weights.size(); ++i)
        std::printf("%s%.9g", i ? ", " : "", r.final_synapse_weights[i]);
    std::printf("], \"spikes\": [");
    for (std::size_t i = 0; i < r.final_neuron_spike_counts.size(); ++i)
        std::printf("%s%llu", i ? ", " : "", (unsigned long long)r.final_neuron_spike_counts[i]);
    std::printf("], \"matches\": [");
    for (std::size_t i = 0; i < r.final_temporal_match_counts.size(); ++i)
        std::printf("%s%llu", i ? ", " : "", (unsigned long long)r.final_temporal_match_counts[i]);
    std::printf("], \"code_matches\": [");
    for (std::size_t i = 0; i < r.final_synapse_code_match_counts.size(); ++i)
        std::printf("%s%llu", i ? ", " : "", (unsigned long long)r.final_synapse_code_match_counts[i]);
    std::printf("]");

    snncuda_gb300::CudaInferenceSession<Connectome> session(c);
    std::vector<snncuda_gb300::CudaInferenceSample> samples(3);
    samples[0].inputs = {{1, 1.5F, 0}};
    samples[1].inputs = {{2, 1.0F, 0}, {4, 0.7F, 2}};
    samples[2].inputs = {{6, 2.0F, 1}, {6, 2.0F, 5}};
    snncuda_gb300::CudaInferenceOptions opt;
    opt.max_steps = 12;
    opt.readout_neurons = {2, 3, 5};
    for (int reset = 1; reset >= 0; --reset) {
        opt.reset_state_between_samples = reset != 0;
        const auto b = session.run_batch(samples, opt);
        std::printf(", \"%s\": [", reset ? "stateless" : "stateful");
        for (std::size_t i = 0; i < b.samples.size(); ++i) {
            const auto& s = b.samples[i];
            std::printf("%s{\"readout\": [%llu, %llu, %llu], \"delivered\": %llu, \"fired\": %llu}", i ? ", " : "",
                        (unsigned long long)s.readout_spike_counts[0], (unsigned long long)s.readout_spike_counts[1],
                        (unsigned long long)s.readout_spike_counts[2], (unsigned long long)s.delivered_spikes,
                        (unsigned long long)s.fired_spikes);
        }
        std::printf("]");
    }
    // the readout paths: one hop, and the recurrent hidden/readout iteration
    opt.reset_state_between_samples = true;
    const auto ff = session.run_feedforward_batch(samples, opt);
    snncuda_gb300::CudaRecurrentFeedforwardOptions ro;
    ro.readout_neurons = {2, 5};
    ro.iterations = 2;
    ro.top_k_feedback_readouts = 1;
    const auto rec = session.run_recurrent_feedforward_batch(samples, ro);
    for (int which = 0; which < 2; ++which) {
        const auto& b = which == 0 ? ff : rec;
        std::printf(", \"%s\": [", which == 0 ? "feedforward" : "recurrent");
        for (std::size_t i = 0; i < b.samples.size(); ++i) {
            const auto& s = b.samples[i];
            std::printf("%s{\"scores\": [", i ? ", " : "");
            for (std::size_t k = 0; k < s.readout_scores.size(); ++k)
                std::printf("%s%.9g", k ? ", " : "", s.readout_scores[k]);
            std::printf("], \"spikes\": [");
            for (std::size_t k = 0; k < s.readout_spike_counts.size(); ++k)
                std::printf("%s%llu", k ? ", " : "", (unsigned long long)s.readout_spike_counts[k]);
            std::printf("], \"delivered\": %llu}", (unsigned long long)s.delivered_spikes);
        }
        std::printf("]");
    }
    std::printf("}\n");
    return 0;
}
"""


def _python_network():
    ids = np.arange(6)
    src = ids.astype(np.uint32)
    tgt = ((ids + 1) % 6).astype(np.uint32)
    i1 = ids + 1
    codes = []
    ptr = [0]
    for i in i1:
        codes += [0, 1] if i % 2 else [0]
        ptr.append(len(codes))
    comp = np.array([1 if i % 4 == 3 else i % 4 for i in i1], np.uint8)
    return Connectome(
        threshold=np.ones(6, np.float32), pattern_window_ticks=np.full(6, 20, np.uint64),
        similarity_threshold=np.full(6, 0.9, np.float32), max_reference_patterns=np.full(6, 2, np.uint64),
        source=src, target=tgt, weight=np.full(6, 2.0, np.float32), max_weight=np.ones(6, np.float32),
        delay_ticks=(1 + i1 % 3).astype(np.uint32), compartment=comp, receptor=(i1 % 2).astype(np.uint8),
        plasticity_enabled=(i1 != 4).astype(np.uint8), code_offset_ptr=np.array(ptr, np.uint64),
        code_offsets=np.array(codes, np.uint32))


def _build_and_run(tmp_path, lib_path, prelude, extra_include=()):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "facade.cpp"
    src.write_text(prelude + PROGRAM)
    exe = tmp_path / "facade"
    cmd = ["g++", "-std=c++20", "-O1", "-I", str(ROOT / "include"), *sum((["-I", str(p)] for p in extra_include), []),
           str(src), "-o", str(exe), str(lib_path), f"-Wl,-rpath,{lib_path.parent}"]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout
    return json.loads(out)


def _expected(lib):
    c = _python_network()
    cfg = default_config(lib)
    sim = Simulation(c, cfg, lib)
    sim.inject([0, 2], [0, 0], [1.0, 1.0])
    sim.run_until(40)
    cnt, n, s = sim.counters(), sim.neurons(), sim.synapses()
    sim.close()
    want = {"delivered": cnt["delivered_spikes"], "fired": cnt["fired_spikes"],
            "weights": [float(x) for x in s["weight"]], "spikes": [int(x) for x in n["spike_count"]],
            "matches": [int(x) for x in n["match_count"]], "code_matches": [int(x) for x in s["code_match_count"]]}
    samples = [[(0, 1.5, 0)], [(1, 1.0, 0), (3, 0.7, 2)], [(5, 2.0, 1), (5, 2.0, 5)]]
    readout = [1, 2, 4]
    stateless = []
    for smp in samples:
        sim = Simulation(c, default_config(lib), lib)
        sim.inject([a for a, _, _ in smp], [t for _, _, t in smp], [w for _, w, _ in smp])
        sim.run_until(12)
        sp = sim.neurons()["spike_count"]
        cc = sim.counters()
        stateless.append({"readout": [int(sp[i]) for i in readout], "delivered": cc["delivered_spikes"],
                          "fired": cc["fired_spikes"]})
        sim.close()
    stateful = []
    sim = Simulation(c, default_config(lib), lib)
    base = 0
    for smp in samples:
        before, c0 = sim.neurons()["spike_count"].copy(), sim.counters()
        sim.inject([a for a, _, _ in smp], [base + t for _, _, t in smp], [w for _, w, _ in smp])
        sim.run_until(base + 12)
        base += 13
        after, c1 = sim.neurons()["spike_count"], sim.counters()
        stateful.append({"readout": [int(after[i] - before[i]) for i in readout],
                         "delivered": c1["delivered_spikes"] - c0["delivered_spikes"],
                         "fired": c1["fired_spikes"] - c0["fired_spikes"]})
    sim.close()
    want["stateless"] = stateless
    want["stateful"] = stateful
    from snncuda_gb300.simulation import Readout
    r = Readout(c, lib)
    rs = [[(a, w) for a, w, _ in smp] for smp in samples]
    for key, (sc, sp, dl) in (("feedforward", r.feedforward(rs, [1, 2, 4])),
                              ("recurrent", r.recurrent(rs, [1, 4], iterations=2)[:3])):
        want[key] = [{"scores": [float(x) for x in sc[i]], "spikes": [int(x) for x in sp[i]], "delivered": int(dl[i])}
                     for i in range(len(rs))]
    r.close()
    return want


def _compare(got, want):
    assert got["executed"] == 1
    for key in want:
        if key == "weights":
            assert np.array_equal(np.float32(got[key]), np.float32(want[key]))
        elif key in ("feedforward", "recurrent"):
            # readout sums: the oracle adds in the reference's push order
            for g, w in zip(got[key], want[key]):
                np.testing.assert_allclose(np.float32(g["scores"]), np.float32(w["scores"]), rtol=2e-6, atol=1e-6)
                assert g["spikes"] == w["spikes"] and g["delivered"] == w["delivered"], key
        else:
            assert got[key] == want[key], key


def test_facade_on_the_oracle(tmp_path, port_lib):
    _ensure_built()
    got = _build_and_run(tmp_path, PORT_PATH, MOCK)
    want = _expected(port_lib)
    assert want["fired"] > 2
    _compare(got, want)


def test_facade_compiles_against_the_reference_connectome(tmp_path, port_lib):
    if not (REF_INCLUDE / "snncuda" / "declarative" / "Connectome.h").exists():
        pytest.skip("reference headers not present")
    _ensure_built()
    got = _build_and_run(tmp_path, PORT_PATH, REAL, [REF_INCLUDE])
    _compare(got, _expected(port_lib))


@pytest.mark.gpu
def test_facade_on_the_gpu(tmp_path, gpu_lib, port_lib):
    """The facade linked to the GPU library against the oracle's results."""
    got = _build_and_run(tmp_path, GPU_PATH, MOCK)
    _compare(got, _expected(port_lib))
