/*
 * snncuda_gb300.hpp -- header-only C++ facade over the C ABI with the
 * reference's backend names (snncuda/backends/CudaBackend.h): CudaBackend::
 * run_resident_propagation -> CudaPropagationResult / CudaDebugMetrics, and
 * CudaInferenceSession::run_batch.  It takes any Connectome-shaped object
 * with the reference's public fields (declarative/Connectome.h:13-37:
 * neurons[i].id / .params.{threshold, pattern_window_ticks,
 * similarity_threshold, max_reference_patterns}, synapses[k].{source, target,
 * weight, max_weight, delay_ticks, spike_code_offsets, compartment, receptor,
 * plasticity_enabled}), so declarative::Connectome works without this header
 * including the reference's.
 *
 * Semantics are the reference CPU runtime's (NetworkPropagator), which the
 * engine reproduces exactly; the reference CUDA backend's own results diverge
 * from them and are not reproduced.  In particular an initially active
 * neuron is an external input at tick 0 of weight equal to its threshold
 * (soma, AMPA), so it fires at tick 0 as a driven neuron would.
 *
 * Link against the library implementing include/snncuda_gb300.h.
 */
#pragma once

#include <chrono>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

#include "snncuda_gb300.h"

namespace snncuda_gb300 {

struct CudaDebugMetrics {
    std::uint64_t ticks_processed{0};
    std::uint64_t scheduled_event_requests{0};
    std::uint64_t scheduled_events{0};
    std::uint64_t processed_events{0};
    std::uint64_t dropped_events{0};
    std::uint64_t fired_appends{0};
    std::uint64_t fired_overflow{0};
    std::uint64_t lock_spin_iterations{0};
    std::uint64_t lock_timeouts{0};
    std::uint64_t stdp_updates{0};
    std::uint64_t stdp_ltp{0};
    std::uint64_t stdp_ltd{0};
    std::uint64_t receptor_ampa_events{0};
    std::uint64_t receptor_nmda_events{0};
    std::uint64_t receptor_gaba_a_events{0};
    std::uint64_t receptor_gaba_b_events{0};
    std::uint64_t dendritic_integrations{0};
    std::uint64_t post_plasticity_scans{0};
    std::uint64_t temporal_observations{0};
    std::uint64_t temporal_patterns_learned{0};
    std::uint64_t temporal_matches{0};
    std::uint64_t max_scheduled_events_per_tick{0};
    std::uint64_t max_fired_neurons_per_tick{0};
};

struct CudaPropagationResult {
    bool executed{false};
    std::uint64_t delivered_spikes{0};
    std::uint64_t fired_spikes{0};
    double elapsed_seconds{0.0};
    CudaDebugMetrics debug;
    std::vector<float> final_synapse_weights;
    std::vector<float> final_membrane_potentials;
    std::vector<std::uint64_t> final_neuron_spike_counts;
    std::vector<std::uint64_t> final_temporal_match_counts;
    std::vector<std::uint32_t> final_temporal_learned_pattern_counts;
    std::vector<std::uint64_t> final_synapse_code_match_counts;
    std::vector<std::uint32_t> final_synapse_code_learned_pattern_counts;
};

struct CudaWeightedInput {
    std::uint64_t neuron;
    float weight{1.0F};
    std::uint32_t tick{0};
};

struct CudaInferenceSample {
    std::vector<CudaWeightedInput> inputs;
};

struct CudaInferenceOptions {
    std::uint32_t max_steps{8};
    bool reset_state_between_samples{true};
    std::vector<std::uint64_t> readout_neurons;
};

struct CudaInferenceSampleResult {
    std::vector<std::uint64_t> readout_spike_counts;
    std::vector<float> readout_scores;  // = readout_spike_counts (spike-count readout)
    std::uint64_t delivered_spikes{0};
    std::uint64_t fired_spikes{0};
    CudaDebugMetrics debug;
};

struct CudaInferenceBatchResult {
    bool executed{false};
    double elapsed_seconds{0.0};
    std::vector<CudaInferenceSampleResult> samples;
};

namespace detail {

inline void check(int rc) {
    if (rc != SNNCUDA_OK) throw std::runtime_error(snncuda_last_error());
}

// The flattened arrays of one Connectome (ids mapped to dense indices in
// Connectome::neurons order) and the snncuda_network view of them.
struct Flat {
    std::unordered_map<std::uint64_t, std::uint32_t> index;
    std::vector<float> thr, sim, w, mw;
    std::vector<std::uint64_t> win, refs, cptr;
    std::vector<std::uint32_t> src, tgt, dly, codes;
    std::vector<std::uint8_t> comp, rec, plast;
    snncuda_network net{};

    template <class Connectome>
    explicit Flat(const Connectome& c) {
        const std::size_t n = c.neurons.size();
        thr.resize(n);
        sim.resize(n);
        win.resize(n);
        refs.resize(n);
        for (std::size_t i = 0; i < n; ++i) {
            const auto& nr = c.neurons[i];
            index.emplace(static_cast<std::uint64_t>(nr.id), static_cast<std::uint32_t>(i));
            thr[i] = nr.params.threshold;
            win[i] = nr.params.pattern_window_ticks;
            sim[i] = nr.params.similarity_threshold;
            refs[i] = nr.params.max_reference_patterns;
        }
        cptr.push_back(0);
        for (const auto& s : c.synapses) {  // synapses whose endpoints are unknown are skipped, as the reference does
            const auto a = index.find(static_cast<std::uint64_t>(s.source));
            const auto b = index.find(static_cast<std::uint64_t>(s.target));
            if (a == index.end() || b == index.end()) continue;
            src.push_back(a->second);
            tgt.push_back(b->second);
            w.push_back(s.weight);
            mw.push_back(s.max_weight);
            dly.push_back(s.delay_ticks);
            comp.push_back(static_cast<std::uint8_t>(s.compartment));
            rec.push_back(static_cast<std::uint8_t>(s.receptor));
            plast.push_back(s.plasticity_enabled ? 1 : 0);
            codes.insert(codes.end(), s.spike_code_offsets.begin(), s.spike_code_offsets.end());
            cptr.push_back(codes.size());
        }
        if (codes.empty()) codes.push_back(0);
        net = snncuda_network{static_cast<std::uint32_t>(n), thr.data(), win.data(), sim.data(), refs.data(),
                              src.size(), src.data(), tgt.data(), w.data(), mw.data(), dly.data(), comp.data(),
                              rec.data(), plast.data(), cptr.data(), codes.data()};
    }

    std::uint32_t dense(std::uint64_t id) const {
        const auto it = index.find(id);
        if (it == index.end()) throw std::invalid_argument("unknown neuron id");
        return it->second;
    }
};

inline snncuda_config default_config() {
    snncuda_config cfg;
    snncuda_config_default(&cfg);
    return cfg;
}

}  // namespace detail

class CudaBackend {
public:
    std::string_view name() const noexcept { return "cuda-gb300"; }
    bool available() const noexcept { return snncuda_cuda_available() != 0; }
    std::string availability_status() const { return available() ? "available" : "no CUDA device"; }

    // Runs ticks 0 .. max_steps with the initially active neurons driven at
    // tick 0 and returns the final state in Connectome order.
    template <class Connectome>
    CudaPropagationResult run_resident_propagation(const Connectome& connectome,
                                                   const std::vector<std::uint64_t>& initially_active,
                                                   std::uint32_t max_steps) const {
        CudaPropagationResult out;
        if (connectome.neurons.empty() || initially_active.empty()) {
            out.executed = true;
            return out;
        }
        const auto t0 = std::chrono::steady_clock::now();
        detail::Flat f(connectome);
        const snncuda_config cfg = detail::default_config();
        snncuda_sim* sim = nullptr;
        detail::check(snncuda_sim_create(&f.net, &cfg, &sim));
        try {
            std::vector<std::uint32_t> nn;
            std::vector<std::uint64_t> tt;
            std::vector<float> ww;
            std::unordered_map<std::uint32_t, bool> seen;
            for (std::uint64_t id : initially_active) {
                const auto it = f.index.find(id);
                if (it == f.index.end() || !seen.emplace(it->second, true).second) continue;
                nn.push_back(it->second);
                tt.push_back(0);
                ww.push_back(f.thr[it->second]);
            }
            detail::check(snncuda_sim_inject(sim, nn.size(), nn.data(), tt.data(), ww.data()));
            detail::check(snncuda_sim_run_until(sim, max_steps));
            snncuda_counters c;
            detail::check(snncuda_sim_counters(sim, &c));
            const std::size_t n = f.thr.size(), s = f.src.size();
            out.final_membrane_potentials.resize(n);
            out.final_neuron_spike_counts.resize(n);
            out.final_temporal_match_counts.resize(n);
            std::vector<std::uint64_t> learned(n), code_learned(s);
            out.final_synapse_weights.resize(s);
            out.final_synapse_code_match_counts.resize(s);
            snncuda_neuron_state ns{};
            ns.membrane_potential = out.final_membrane_potentials.data();
            ns.spike_count = out.final_neuron_spike_counts.data();
            ns.match_count = out.final_temporal_match_counts.data();
            ns.learned_count = learned.data();
            detail::check(snncuda_sim_read_neurons(sim, &ns));
            snncuda_synapse_state ss{};
            ss.weight = out.final_synapse_weights.data();
            ss.code_match_count = out.final_synapse_code_match_counts.data();
            ss.learned_code_count = code_learned.data();
            detail::check(snncuda_sim_read_synapses(sim, &ss));
            out.final_temporal_learned_pattern_counts.assign(learned.begin(), learned.end());
            out.final_synapse_code_learned_pattern_counts.assign(code_learned.begin(), code_learned.end());
            out.executed = true;
            out.delivered_spikes = c.delivered_spikes;
            out.fired_spikes = c.fired_spikes;
            out.debug.ticks_processed = static_cast<std::uint64_t>(max_steps) + 1;
            out.debug.processed_events = c.delivered_spikes;
            out.debug.fired_appends = c.fired_spikes;
            out.debug.max_scheduled_events_per_tick = c.max_slot_events;
            for (std::uint64_t m : out.final_temporal_match_counts) out.debug.temporal_matches += m;
        } catch (...) {
            snncuda_sim_destroy(sim);
            throw;
        }
        snncuda_sim_destroy(sim);
        out.elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return out;
    }
};

// CudaInferenceSession (CudaBackend.h:97-126): samples of weighted inputs,
// each run for ticks 0 .. max_steps; readouts are spike counts.  With
// reset_state_between_samples every sample starts from the initial state and
// all samples run side by side as one batch (snncuda_batch_*); otherwise they
// run one after another on one persistent simulation, each sample's ticks
// counted from where the previous one ended.
template <class Connectome>
class CudaInferenceSession {
public:
    explicit CudaInferenceSession(const Connectome& connectome) : flat_(connectome) {}
    ~CudaInferenceSession() { reset_state(); }
    CudaInferenceSession(const CudaInferenceSession&) = delete;
    CudaInferenceSession& operator=(const CudaInferenceSession&) = delete;

    bool available() const noexcept { return snncuda_cuda_available() != 0; }

    CudaInferenceBatchResult run_batch(const std::vector<CudaInferenceSample>& samples,
                                       const CudaInferenceOptions& options) {
        CudaInferenceBatchResult out;
        out.executed = true;
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::uint32_t> readout;
        for (std::uint64_t id : options.readout_neurons) readout.push_back(flat_.dense(id));
        if (options.reset_state_between_samples) {
            run_stateless(samples, options, readout, out);
        } else {
            run_stateful(samples, options, readout, out);
        }
        out.elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return out;
    }

    void reset_state() {
        if (sim_) snncuda_sim_destroy(sim_);
        sim_ = nullptr;
        base_tick_ = 0;
    }

private:
    static void inputs_of(const detail::Flat& f, const CudaInferenceSample& s, std::uint64_t base,
                          std::vector<std::uint32_t>& n, std::vector<std::uint64_t>& t, std::vector<float>& w) {
        n.clear();
        t.clear();
        w.clear();
        for (const auto& in : s.inputs) {
            n.push_back(f.dense(in.neuron));
            t.push_back(base + in.tick);
            w.push_back(in.weight);
        }
    }

    void run_stateless(const std::vector<CudaInferenceSample>& samples, const CudaInferenceOptions& options,
                       const std::vector<std::uint32_t>& readout, CudaInferenceBatchResult& out) {
        if (samples.empty()) return;
        std::vector<snncuda_network> nets(samples.size(), flat_.net);
        const snncuda_config cfg = detail::default_config();
        snncuda_batch* b = nullptr;
        detail::check(snncuda_batch_create(static_cast<std::uint32_t>(nets.size()), nets.data(), nullptr, &cfg, &b));
        try {
            std::vector<std::uint32_t> n;
            std::vector<std::uint64_t> t;
            std::vector<float> w;
            for (std::size_t i = 0; i < samples.size(); ++i) {
                inputs_of(flat_, samples[i], 0, n, t, w);
                detail::check(snncuda_batch_inject(b, static_cast<std::uint32_t>(i), n.size(), n.data(), t.data(), w.data()));
            }
            detail::check(snncuda_batch_run_until(b, options.max_steps));
            std::vector<std::uint64_t> spikes(flat_.thr.size());
            for (std::size_t i = 0; i < samples.size(); ++i) {
                snncuda_neuron_state ns{};
                ns.spike_count = spikes.data();
                detail::check(snncuda_batch_read_neurons(b, static_cast<std::uint32_t>(i), &ns));
                snncuda_counters c;
                detail::check(snncuda_batch_counters(b, static_cast<std::uint32_t>(i), &c));
                out.samples.push_back(sample_result(spikes, nullptr, readout, c, nullptr, options.max_steps));
            }
        } catch (...) {
            snncuda_batch_destroy(b);
            throw;
        }
        snncuda_batch_destroy(b);
    }

    void run_stateful(const std::vector<CudaInferenceSample>& samples, const CudaInferenceOptions& options,
                      const std::vector<std::uint32_t>& readout, CudaInferenceBatchResult& out) {
        if (!sim_) {
            const snncuda_config cfg = detail::default_config();
            detail::check(snncuda_sim_create(&flat_.net, &cfg, &sim_));
        }
        std::vector<std::uint32_t> n;
        std::vector<std::uint64_t> t;
        std::vector<float> w;
        std::vector<std::uint64_t> before(flat_.thr.size()), after(flat_.thr.size());
        for (const auto& s : samples) {
            snncuda_neuron_state ns{};
            ns.spike_count = before.data();
            detail::check(snncuda_sim_read_neurons(sim_, &ns));
            snncuda_counters c0;
            detail::check(snncuda_sim_counters(sim_, &c0));
            inputs_of(flat_, s, base_tick_, n, t, w);
            detail::check(snncuda_sim_inject(sim_, n.size(), n.data(), t.data(), w.data()));
            detail::check(snncuda_sim_run_until(sim_, base_tick_ + options.max_steps));
            base_tick_ += static_cast<std::uint64_t>(options.max_steps) + 1;
            ns.spike_count = after.data();
            detail::check(snncuda_sim_read_neurons(sim_, &ns));
            snncuda_counters c1;
            detail::check(snncuda_sim_counters(sim_, &c1));
            out.samples.push_back(sample_result(after, &before, readout, c1, &c0, options.max_steps));
        }
    }

    static CudaInferenceSampleResult sample_result(const std::vector<std::uint64_t>& spikes,
                                                   const std::vector<std::uint64_t>* before,
                                                   const std::vector<std::uint32_t>& readout, const snncuda_counters& c,
                                                   const snncuda_counters* c0, std::uint32_t max_steps) {
        CudaInferenceSampleResult r;
        for (std::uint32_t i : readout) {
            const std::uint64_t v = spikes[i] - (before ? (*before)[i] : 0);
            r.readout_spike_counts.push_back(v);
            r.readout_scores.push_back(static_cast<float>(v));
        }
        r.delivered_spikes = c.delivered_spikes - (c0 ? c0->delivered_spikes : 0);
        r.fired_spikes = c.fired_spikes - (c0 ? c0->fired_spikes : 0);
        r.debug.ticks_processed = static_cast<std::uint64_t>(max_steps) + 1;
        r.debug.processed_events = r.delivered_spikes;
        r.debug.fired_appends = r.fired_spikes;
        return r;
    }

    detail::Flat flat_;
    snncuda_sim* sim_{nullptr};
    std::uint64_t base_tick_{0};
};

}  // namespace snncuda_gb300
