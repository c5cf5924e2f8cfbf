/*
 * snncuda_gb300.hpp -- header-only C++ facade over the C ABI with the
 * reference's backend names (snncuda/backends/CudaBackend.h): CudaBackend::
 * run_resident_propagation -> CudaPropagationResult / CudaDebugMetrics, and
 * CudaInferenceSession::run_batch / run_feedforward_batch /
 * run_recurrent_feedforward_batch / reset_state.  It takes any Connectome-shaped object
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

#include <algorithm>
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

// CudaRecurrentFeedforwardOptions (CudaBackend.h:69-79).
struct CudaRecurrentFeedforwardOptions {
    std::uint32_t iterations{1};
    std::vector<std::uint64_t> readout_neurons;
    std::vector<std::uint64_t> hidden_neurons;
    float feedback_decay{0.5F};
    std::uint32_t top_k_feedback_readouts{1};
    std::uint32_t top_k_hidden{0};
    bool use_scores_not_spikes{true};
    bool use_full_spike_timing{false};
    std::uint32_t max_timing_steps{0};
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
    ~CudaInferenceSession() {
        reset_state();
        if (readout_) snncuda_readout_destroy(readout_);
    }
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

    // run_feedforward_batch (CudaBackend.cu:1725-1849): one hop from the
    // samples' inputs to the readouts over the initial weights; scores are
    // the weighted sums, spike counts 1 where a score reaches its readout's
    // threshold.
    CudaInferenceBatchResult run_feedforward_batch(const std::vector<CudaInferenceSample>& samples,
                                                   const CudaInferenceOptions& options) {
        CudaInferenceBatchResult out;
        out.executed = true;
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::uint32_t> readout = dense_list(options.readout_neurons);
        Inputs in(flat_, samples);
        const std::size_t S = samples.size(), R = readout.size();
        std::vector<float> scores(S * R);
        std::vector<std::uint64_t> spikes(S * R), delivered(S);
        detail::check(snncuda_readout_feedforward(readout_handle(), static_cast<std::uint32_t>(S), in.ptr.data(),
                                                  in.n.data(), in.w.data(), static_cast<std::uint32_t>(R),
                                                  readout.data(), scores.data(), spikes.data(), delivered.data()));
        readout_results(scores, spikes, delivered, R, 0, out);
        out.elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return out;
    }

    // run_recurrent_feedforward_batch (CudaBackend.cu:1851-2100): hidden and
    // readout events exchanged over max_delay x (1 + 2 x iterations) + 1 time
    // steps; with use_full_spike_timing the samples run through the tick
    // simulation instead (run_batch with that many ticks, or max_timing_steps).
    CudaInferenceBatchResult run_recurrent_feedforward_batch(const std::vector<CudaInferenceSample>& samples,
                                                             const CudaRecurrentFeedforwardOptions& options) {
        if (options.use_full_spike_timing) {
            CudaInferenceOptions timing;
            std::uint32_t max_delay = 1;
            for (std::uint32_t d : flat_.dly) max_delay = std::max(max_delay, std::max(1u, d));
            timing.max_steps = options.max_timing_steps != 0
                                   ? options.max_timing_steps
                                   : max_delay * (1u + 2u * options.iterations) + 1u;
            timing.reset_state_between_samples = true;
            timing.readout_neurons = options.readout_neurons;
            return run_batch(samples, timing);
        }
        CudaInferenceBatchResult out;
        out.executed = true;
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::uint32_t> readout = dense_list(options.readout_neurons);
        std::vector<std::uint32_t> hidden = dense_list(options.hidden_neurons);
        Inputs in(flat_, samples);
        const std::size_t S = samples.size(), R = readout.size();
        std::vector<float> scores(S * R);
        std::vector<std::uint64_t> spikes(S * R), delivered(S);
        snncuda_recurrent_options o;
        snncuda_recurrent_options_default(&o);
        o.iterations = options.iterations;
        o.feedback_decay = options.feedback_decay;
        o.top_k_feedback_readouts = options.top_k_feedback_readouts;
        o.top_k_hidden = options.top_k_hidden;
        o.use_scores_not_spikes = options.use_scores_not_spikes ? 1 : 0;
        std::uint64_t steps = 0;
        detail::check(snncuda_readout_recurrent(readout_handle(), static_cast<std::uint32_t>(S), in.ptr.data(),
                                                in.n.data(), in.w.data(), static_cast<std::uint32_t>(R),
                                                readout.data(), static_cast<std::uint32_t>(hidden.size()),
                                                hidden.data(), &o, scores.data(), spikes.data(), delivered.data(),
                                                &steps));
        readout_results(scores, spikes, delivered, R, steps, out);
        out.elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return out;
    }

    void reset_state() {
        if (sim_) snncuda_sim_destroy(sim_);
        sim_ = nullptr;
        base_tick_ = 0;
    }

private:
    // A batch's inputs as the readout entry points take them (unknown neuron
    // ids are skipped, as the reference does).
    struct Inputs {
        std::vector<std::uint64_t> ptr{0};
        std::vector<std::uint32_t> n;
        std::vector<float> w;
        Inputs(const detail::Flat& f, const std::vector<CudaInferenceSample>& samples) {
            for (const auto& s : samples) {
                for (const auto& in : s.inputs) {
                    const auto it = f.index.find(in.neuron);
                    if (it == f.index.end()) continue;
                    n.push_back(it->second);
                    w.push_back(in.weight);
                }
                ptr.push_back(n.size());
            }
            if (n.empty()) {
                n.push_back(0);
                w.push_back(0.0F);
            }
        }
    };

    std::vector<std::uint32_t> dense_list(const std::vector<std::uint64_t>& ids) const {
        std::vector<std::uint32_t> out;
        for (std::uint64_t id : ids) {
            const auto it = flat_.index.find(id);
            if (it != flat_.index.end()) out.push_back(it->second);
        }
        return out;
    }

    snncuda_readout* readout_handle() {
        if (!readout_) detail::check(snncuda_readout_create(&flat_.net, &readout_));
        return readout_;
    }

    static void readout_results(const std::vector<float>& scores, const std::vector<std::uint64_t>& spikes,
                                const std::vector<std::uint64_t>& delivered, std::size_t R, std::uint64_t steps,
                                CudaInferenceBatchResult& out) {
        for (std::size_t s = 0; s < delivered.size(); ++s) {
            CudaInferenceSampleResult r;
            for (std::size_t k = 0; k < R; ++k) {
                r.readout_scores.push_back(scores[s * R + k]);
                r.readout_spike_counts.push_back(spikes[s * R + k]);
                r.fired_spikes += spikes[s * R + k];
            }
            r.delivered_spikes = delivered[s];
            r.debug.ticks_processed = steps;
            r.debug.processed_events = delivered[s];
            r.debug.dendritic_integrations = delivered[s];
            out.samples.push_back(std::move(r));
        }
    }

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
    snncuda_readout* readout_{nullptr};
    std::uint64_t base_tick_{0};
};

}  // namespace snncuda_gb300
