// ORACLE -- test infrastructure only (see oracle/port/snn_port.cpp).
//
// Drives the SNNCuda reference CPU runtime, compiled unmodified from its own
// sources (oracle/Makefile), through the C ABI of include/snncuda_gb300.h so
// the oracle port and the GPU backend can be checked against it.
//
// Two modes (snnref_set_mode):
//   0  "propagator": the reference runtime::NetworkPropagator itself
//      (src/runtime/NetworkPropagator.cpp).  Its processor always uses the
//      default SynapseDendriteConfig, so toggles and non-default STDP
//      parameters are rejected, and fire rasters are not observable.
//   1  "mirror": this file's own tick loop restating
//      NetworkPropagator::process_tick (NetworkPropagator.cpp:78-132) over
//      the reference SpikeScheduler, SynapseDendriteProcessor (constructed
//      with the requested config) and NeuronStateCache, adding fire-raster
//      capture and the runtime toggles.  Tests pin mode 1 to mode 0 first.

#include "snncuda_gb300.h"

#include "snncuda/declarative/Connectome.h"
#include "snncuda/runtime/NetworkPropagator.h"
#include "snncuda/runtime/NeuronStateCache.h"
#include "snncuda/runtime/SpikeScheduler.h"
#include "snncuda/runtime/SynapseDendriteProcessor.h"

#include <cstring>
#include <exception>
#include <memory>
#include <optional>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_last_error;
int g_mode = 0;

int fail(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

using snncuda::core::NeuronId;
using snncuda::core::SynapseId;
namespace rt = snncuda::runtime;
namespace decl = snncuda::declarative;

struct Digest {
    uint64_t h{0xcbf29ce484222325ULL};
    void word(uint64_t w) { h = (h ^ w) * 0x100000001b3ULL; }
    void f32(float f) {
        uint32_t b;
        std::memcpy(&b, &f, 4);
        word(b);
    }
};

bool is_default(const snncuda_config& c) {
    snncuda_config d;
    snncuda_config_default(&d);
    return c.stdp_enabled == d.stdp_enabled && c.ltp_amplitude == d.ltp_amplitude &&
           c.ltd_amplitude == d.ltd_amplitude && c.ltp_tau_ticks == d.ltp_tau_ticks &&
           c.ltd_tau_ticks == d.ltd_tau_ticks && c.min_weight == d.min_weight &&
           c.max_weight == d.max_weight && c.temporal_learning_enabled == d.temporal_learning_enabled;
}

rt::SynapseDendriteConfig make_processor_config(const snncuda_config& c, bool stdp, bool temporal) {
    rt::SynapseDendriteConfig pc;
    pc.stdp.enabled = stdp;
    pc.stdp.ltp_amplitude = c.ltp_amplitude;
    pc.stdp.ltd_amplitude = c.ltd_amplitude;
    pc.stdp.ltp_tau_ticks = c.ltp_tau_ticks;
    pc.stdp.ltd_tau_ticks = c.ltd_tau_ticks;
    pc.stdp.min_weight = c.min_weight;
    pc.stdp.max_weight = c.max_weight;
    pc.temporal_learning_enabled = temporal;
    return pc;
}

}  // namespace

struct snncuda_sim {
    int mode{0};
    decl::Connectome connectome;
    snncuda_config config{};
    bool stdp_enabled{true};
    bool temporal_enabled{true};
    uint64_t injected_total{0};
    std::vector<uint64_t> inject_ticks;  // clamped delivery ticks, to split counters
    uint64_t processed_through{0};      // next tick to process
    // mode 0
    std::unique_ptr<rt::MemoryNeuronStateStore> store;
    std::unique_ptr<rt::NetworkPropagator> propagator;
    // mode 1
    std::unique_ptr<rt::NeuronStateCache> cache;
    std::unique_ptr<rt::SpikeScheduler> scheduler;
    rt::SynapseDendriteProcessor processor;
    std::unordered_map<SynapseId, rt::SynapseRuntimeState> synapses;
    std::unordered_map<NeuronId, std::vector<SynapseId>> outgoing;
    std::unordered_map<NeuronId, std::vector<SynapseId>> incoming;
    uint64_t delivered{0}, fired{0}, synaptic{0}, external{0}, max_due{0};
    std::vector<uint64_t> raster_tick;
    std::vector<uint32_t> raster_neuron;
    bool poisoned{false};

    rt::NeuronState neuron(uint32_t i) {
        const NeuronId id = i + 1;
        return mode == 0 ? propagator->state(id) : cache->load_for_spike(id);
    }
    const rt::SynapseRuntimeState* synapse(uint64_t s) {
        const SynapseId id = s + 1;
        if (mode == 0) return propagator->synapse_state(id);
        auto it = synapses.find(id);
        return it == synapses.end() ? nullptr : &it->second;
    }

    // Restatement of NetworkPropagator::process_tick (NetworkPropagator.cpp:78-132).
    int mirror_tick(uint64_t tick) {
        const auto due = scheduler->pop_due(tick);
        if (due.size() > max_due) max_due = due.size();
        for (const auto& event : due) {
            ++delivered;
            auto target = cache->load_for_spike(event.target_neuron);
            const auto found = synapses.find(event.synapse);
            const auto result = found == synapses.end()
                ? processor.process_external_input(target, event, tick)
                : processor.process_synaptic_input(target, found->second, event, tick);
            cache->store_after_compute(target);
            if (found == synapses.end()) ++external; else ++synaptic;
            if (!result.fired) continue;
            ++fired;
            if (config.raster_capacity > 0) {
                if (raster_tick.size() >= config.raster_capacity) {
                    poisoned = true;
                    return fail(SNNCUDA_ERR_CAPACITY, "raster capacity exceeded");
                }
                raster_tick.push_back(tick);
                raster_neuron.push_back(static_cast<uint32_t>(event.target_neuron - 1));
            }
            if (auto in = incoming.find(event.target_neuron); in != incoming.end()) {
                auto post_state = cache->load_for_spike(event.target_neuron);
                for (const auto sid : in->second)
                    processor.apply_post_spike_plasticity(post_state, synapses.at(sid), tick);
                cache->store_after_compute(post_state);
            }
            auto out = outgoing.find(event.target_neuron);
            if (out == outgoing.end()) continue;
            for (const auto sid : out->second) {
                const auto& s = synapses.at(sid);
                for (const auto offset : s.spike_code_offsets) {
                    scheduler->schedule({.source_neuron = s.source,
                                         .target_neuron = s.target,
                                         .synapse = s.id,
                                         .delivery_tick = tick + s.delay_ticks + offset,
                                         .weight = s.weight});
                }
            }
        }
        return SNNCUDA_OK;
    }
};

extern "C" {

void snnref_set_mode(int mode) { g_mode = mode; }

const char* snncuda_version(void) { return "0.1.0-reference-harness"; }
int snncuda_cuda_available(void) { return 0; }
const char* snncuda_last_error(void) { return g_last_error.c_str(); }

void snncuda_config_default(snncuda_config* c) {
    if (c == nullptr) return;
    std::memset(c, 0, sizeof(*c));
    c->stdp_enabled = 1;
    c->ltp_amplitude = 0.01F;
    c->ltd_amplitude = 0.012F;
    c->ltp_tau_ticks = 20.0F;
    c->ltd_tau_ticks = 20.0F;
    c->min_weight = 0.0F;
    c->max_weight = 2.0F;
    c->temporal_learning_enabled = 1;
    c->timing_wheel_slots = 4096;
    c->stage_wait_ns = 100000000ULL;  // engine option; no device waits here
}

int snncuda_sim_create(const snncuda_network* net, const snncuda_config* cfg, snncuda_sim** out) {
    if (net == nullptr || out == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_config def;
    snncuda_config_default(&def);
    if (cfg == nullptr) cfg = &def;
    try {
        auto sim = std::make_unique<snncuda_sim>();
        sim->mode = g_mode;
        sim->config = *cfg;
        sim->stdp_enabled = cfg->stdp_enabled != 0;
        sim->temporal_enabled = cfg->temporal_learning_enabled != 0;
        if (sim->mode == 0 && (!is_default(*cfg) || cfg->raster_capacity != 0))
            return fail(SNNCUDA_ERR_UNSUPPORTED,
                        "propagator mode runs the default processor config without rasters");
        auto& c = sim->connectome;
        c.neurons.resize(net->neuron_count);
        for (uint32_t i = 0; i < net->neuron_count; ++i) {
            auto& n = c.neurons[i];
            n.id = i + 1;
            n.params.threshold = net->threshold[i];
            n.params.pattern_window_ticks = net->pattern_window_ticks[i];
            n.params.similarity_threshold = net->similarity_threshold[i];
            n.params.max_reference_patterns = static_cast<size_t>(net->max_reference_patterns[i]);
        }
        c.synapses.resize(net->synapse_count);
        for (uint64_t s = 0; s < net->synapse_count; ++s) {
            auto& y = c.synapses[s];
            y.id = s + 1;
            y.source = net->source[s] + 1;
            y.target = net->target[s] + 1;
            y.weight = net->weight[s];
            y.max_weight = net->max_weight[s];
            y.delay_ticks = net->delay_ticks[s];
            y.compartment = static_cast<snncuda::snn::DendriticCompartment>(net->compartment[s]);
            y.receptor = static_cast<snncuda::snn::ReceptorType>(net->receptor[s]);
            y.plasticity_enabled = net->plasticity_enabled[s] != 0;
            y.spike_code_offsets = {0};
            if (net->code_offset_ptr != nullptr && net->code_offsets != nullptr) {
                const uint64_t b = net->code_offset_ptr[s], e = net->code_offset_ptr[s + 1];
                if (e > b) y.spike_code_offsets.assign(net->code_offsets + b, net->code_offsets + e);
            }
        }
        const size_t capacity = net->neuron_count > 0 ? net->neuron_count : 1;
        if (sim->mode == 0) {
            sim->store = std::make_unique<rt::MemoryNeuronStateStore>();
            sim->propagator = std::make_unique<rt::NetworkPropagator>(
                sim->connectome, *sim->store, capacity, static_cast<size_t>(cfg->timing_wheel_slots));
        } else {
            // NetworkPropagator.cpp:5-29, with a configurable processor.
            sim->store = std::make_unique<rt::MemoryNeuronStateStore>();
            sim->cache = std::make_unique<rt::NeuronStateCache>(capacity, *sim->store);
            sim->scheduler = std::make_unique<rt::SpikeScheduler>(static_cast<size_t>(cfg->timing_wheel_slots));
            sim->processor = rt::SynapseDendriteProcessor(
                make_processor_config(*cfg, sim->stdp_enabled, sim->temporal_enabled));
            for (const auto& n : c.neurons) {
                rt::NeuronState st;
                st.id = n.id;
                st.threshold = n.params.threshold;
                st.pattern_window_ticks = n.params.pattern_window_ticks;
                st.similarity_threshold = n.params.similarity_threshold;
                st.max_reference_patterns = n.params.max_reference_patterns;
                sim->store->save(st);
            }
            for (const auto& y : c.synapses) {
                sim->synapses[y.id] = sim->processor.initialize_synapse(y);
                sim->outgoing[y.source].push_back(y.id);
                sim->incoming[y.target].push_back(y.id);
            }
        }
        *out = sim.release();
        return SNNCUDA_OK;
    } catch (const std::invalid_argument& ex) {
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, ex.what());
    } catch (const std::exception& ex) {
        return fail(SNNCUDA_ERR_DEVICE, ex.what());
    }
}

int snncuda_sim_destroy(snncuda_sim* sim) {
    delete sim;
    return SNNCUDA_OK;
}

int snncuda_sim_inject(snncuda_sim* sim, uint64_t count, const uint32_t* neurons,
                       const uint64_t* ticks, const float* weights) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    for (uint64_t i = 0; i < count; ++i) {
        const uint64_t t = ticks[i] < sim->processed_through ? sim->processed_through : ticks[i];
        sim->inject_ticks.push_back(t);
        if (sim->mode == 0) {
            sim->propagator->inject(neurons[i] + 1, ticks[i], weights[i]);
        } else {
            sim->scheduler->schedule({.target_neuron = neurons[i] + 1,
                                      .delivery_tick = ticks[i],
                                      .weight = weights[i]});
        }
    }
    return SNNCUDA_OK;
}

int snncuda_sim_run_until(snncuda_sim* sim, uint64_t inclusive_tick) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->poisoned) return fail(SNNCUDA_ERR_POISONED, "simulation poisoned by an earlier error");
    try {
        if (sim->mode == 0) {
            sim->propagator->run_until(inclusive_tick);
        } else {
            for (uint64_t t = 0; t <= inclusive_tick; ++t) {
                const int rc = sim->mirror_tick(t);
                if (rc != SNNCUDA_OK) return rc;
            }
        }
    } catch (const std::exception& ex) {
        return fail(SNNCUDA_ERR_DEVICE, ex.what());
    }
    if (inclusive_tick + 1 > sim->processed_through) sim->processed_through = inclusive_tick + 1;
    return SNNCUDA_OK;
}

int snncuda_sim_set_plasticity(snncuda_sim* sim, int32_t enabled) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->mode == 0) return fail(SNNCUDA_ERR_UNSUPPORTED, "propagator mode has no toggle");
    sim->stdp_enabled = enabled != 0;
    sim->processor = rt::SynapseDendriteProcessor(
        make_processor_config(sim->config, sim->stdp_enabled, sim->temporal_enabled));
    return SNNCUDA_OK;
}

int snncuda_sim_set_temporal_learning(snncuda_sim* sim, int32_t enabled) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->mode == 0) return fail(SNNCUDA_ERR_UNSUPPORTED, "propagator mode has no toggle");
    sim->temporal_enabled = enabled != 0;
    sim->processor = rt::SynapseDendriteProcessor(
        make_processor_config(sim->config, sim->stdp_enabled, sim->temporal_enabled));
    return SNNCUDA_OK;
}

int snncuda_sim_counters(snncuda_sim* sim, snncuda_counters* out) {
    if (sim == nullptr || out == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    out->next_tick = sim->processed_through;
    if (sim->mode == 0) {
        out->delivered_spikes = sim->propagator->delivered_spike_count();
        out->fired_spikes = sim->propagator->fired_spike_count();
        uint64_t ext = 0;
        for (uint64_t t : sim->inject_ticks) ext += (t < sim->processed_through) ? 1 : 0;
        out->external_events = ext;
        out->synaptic_events = out->delivered_spikes - ext;
        out->pending_events = sim->propagator->idle() ? 0 : ~0ULL;  // count not observable
    } else {
        out->delivered_spikes = sim->delivered;
        out->fired_spikes = sim->fired;
        out->synaptic_events = sim->synaptic;
        out->external_events = sim->external;
        out->pending_events = sim->scheduler->pending_count();
        out->raster_count = sim->raster_tick.size();
        out->max_slot_events = sim->max_due;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_idle(snncuda_sim* sim, int32_t* out) {
    if (sim == nullptr || out == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->mode == 0 ? (sim->propagator->idle() ? 1 : 0) : (sim->scheduler->empty() ? 1 : 0);
    return SNNCUDA_OK;
}

int snncuda_sim_read_neurons(snncuda_sim* sim, const snncuda_neuron_state* o) {
    if (sim == nullptr || o == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    const uint32_t N = static_cast<uint32_t>(sim->connectome.neurons.size());
    for (uint32_t i = 0; i < N; ++i) {
        const rt::NeuronState n = sim->neuron(i);
        if (o->membrane_potential) o->membrane_potential[i] = n.membrane_potential;
        if (o->spike_count) o->spike_count[i] = n.spike_count;
        if (o->last_fired_tick) o->last_fired_tick[i] = n.last_fired_tick ? static_cast<int64_t>(*n.last_fired_tick) : -1;
        if (o->last_active_tick) o->last_active_tick[i] = n.last_active_tick;
        const rt::NeuronState::CompartmentState* comps[4] = {&n.soma, &n.basal, &n.apical, &n.inhibitory};
        for (int k = 0; k < 4; ++k) {
            if (o->compartment_current) o->compartment_current[i * 4 + k] = comps[k]->current;
            if (o->compartment_last_update) o->compartment_last_update[i * 4 + k] = comps[k]->last_update_tick;
            if (o->compartment_tau) o->compartment_tau[i * 4 + k] = comps[k]->decay_tau_ticks;
        }
        if (o->window_start_tick) o->window_start_tick[i] = n.temporal_pattern.window_start_tick;
        if (o->offset_count) o->offset_count[i] = n.temporal_pattern.spike_offsets.size();
        if (o->learned_count) o->learned_count[i] = n.temporal_pattern.learned_patterns.size();
        if (o->match_count) o->match_count[i] = n.temporal_pattern.match_count;
        if (o->last_match) o->last_match[i] = n.temporal_pattern.last_match ? 1 : 0;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_read_synapses(snncuda_sim* sim, const snncuda_synapse_state* o) {
    if (sim == nullptr || o == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    const uint64_t S = sim->connectome.synapses.size();
    for (uint64_t i = 0; i < S; ++i) {
        const rt::SynapseRuntimeState* s = sim->synapse(i);
        if (s == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "missing synapse state");
        if (o->weight) o->weight[i] = s->weight;
        if (o->last_pre_spike_tick) o->last_pre_spike_tick[i] = s->last_pre_spike_tick ? static_cast<int64_t>(*s->last_pre_spike_tick) : -1;
        if (o->last_post_spike_tick) o->last_post_spike_tick[i] = s->last_post_spike_tick ? static_cast<int64_t>(*s->last_post_spike_tick) : -1;
        if (o->pre_spike_count) o->pre_spike_count[i] = s->pre_spike_count;
        if (o->plasticity_update_count) o->plasticity_update_count[i] = s->plasticity_update_count;
        if (o->last_weight_delta) o->last_weight_delta[i] = s->last_weight_delta;
        if (o->code_window_start_tick) o->code_window_start_tick[i] = s->code_window_start_tick;
        if (o->code_offset_count) o->code_offset_count[i] = s->code_offsets.size();
        if (o->learned_code_count) o->learned_code_count[i] = s->learned_code_patterns.size();
        if (o->code_match_count) o->code_match_count[i] = s->code_match_count;
        if (o->last_code_match) o->last_code_match[i] = s->last_code_match ? 1 : 0;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_read_pattern(snncuda_sim* sim, int32_t kind, uint64_t index, uint64_t which,
                             uint32_t* values, uint64_t capacity, uint64_t* len) {
    if (sim == nullptr || len == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<uint32_t> v;
    if (kind == 0 || kind == 1) {
        if (index >= sim->connectome.neurons.size()) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "neuron out of range");
        const rt::NeuronState n = sim->neuron(static_cast<uint32_t>(index));
        if (kind == 0) v = n.temporal_pattern.spike_offsets;
        else if (which < n.temporal_pattern.learned_patterns.size()) v = n.temporal_pattern.learned_patterns[which].spike_offsets;
        else return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "pattern index out of range");
    } else if (kind == 2 || kind == 3) {
        const rt::SynapseRuntimeState* s = index < sim->connectome.synapses.size() ? sim->synapse(index) : nullptr;
        if (s == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse out of range");
        if (kind == 2) v = s->code_offsets;
        else if (which < s->learned_code_patterns.size()) v = s->learned_code_patterns[which].spike_offsets;
        else return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "pattern index out of range");
    } else {
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "unknown pattern kind");
    }
    *len = v.size();
    for (uint64_t i = 0; i < v.size() && i < capacity; ++i) values[i] = v[i];
    return SNNCUDA_OK;
}

int snncuda_sim_state_digest(snncuda_sim* sim, uint64_t* neuron_digest, uint64_t* synapse_digest) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (neuron_digest) {
        Digest d;
        const uint32_t N = static_cast<uint32_t>(sim->connectome.neurons.size());
        for (uint32_t i = 0; i < N; ++i) {
            const rt::NeuronState n = sim->neuron(i);
            d.f32(n.membrane_potential);
            d.word(n.spike_count);
            d.word(n.last_fired_tick ? *n.last_fired_tick : ~0ULL);
            d.word(n.last_active_tick);
            for (const auto* c : {&n.soma, &n.basal, &n.apical, &n.inhibitory}) {
                d.f32(c->current);
                d.word(c->last_update_tick);
                d.f32(c->decay_tau_ticks);
            }
            const auto& tp = n.temporal_pattern;
            d.word(tp.window_start_tick);
            d.word(tp.spike_offsets.size());
            for (uint32_t v : tp.spike_offsets) d.word(v);
            d.word(tp.learned_patterns.size());
            for (const auto& p : tp.learned_patterns) {
                d.word(p.spike_offsets.size());
                for (uint32_t v : p.spike_offsets) d.word(v);
            }
            d.word(tp.last_match ? 1 : 0);
            d.word(tp.match_count);
        }
        *neuron_digest = d.h;
    }
    if (synapse_digest) {
        Digest d;
        for (uint64_t i = 0; i < sim->connectome.synapses.size(); ++i) {
            const rt::SynapseRuntimeState* s = sim->synapse(i);
            if (s == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "missing synapse state");
            d.f32(s->weight);
            d.word(s->last_pre_spike_tick ? *s->last_pre_spike_tick : ~0ULL);
            d.word(s->last_post_spike_tick ? *s->last_post_spike_tick : ~0ULL);
            d.word(s->pre_spike_count);
            d.word(s->plasticity_update_count);
            d.f32(s->last_weight_delta);
            d.word(s->code_window_start_tick);
            d.word(s->code_offsets.size());
            for (uint32_t v : s->code_offsets) d.word(v);
            d.word(s->learned_code_patterns.size());
            for (const auto& p : s->learned_code_patterns) {
                d.word(p.spike_offsets.size());
                for (uint32_t v : p.spike_offsets) d.word(v);
            }
            d.word(s->code_match_count);
            d.word(s->last_code_match ? 1 : 0);
        }
        *synapse_digest = d.h;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_read_raster(snncuda_sim* sim, uint64_t first, uint64_t count, uint64_t* ticks,
                            uint32_t* neurons) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->mode == 0) return fail(SNNCUDA_ERR_UNSUPPORTED, "propagator mode keeps no raster");
    if (first + count > sim->raster_tick.size())
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "raster range out of bounds");
    for (uint64_t i = 0; i < count; ++i) {
        if (ticks) ticks[i] = sim->raster_tick[first + i];
        if (neurons) neurons[i] = sim->raster_neuron[first + i];
    }
    return SNNCUDA_OK;
}

// Per-kernel device time does not exist on the CPU: only the work counters
// of the processed ticks are filled.
int snncuda_sim_profile(snncuda_sim* sim, uint64_t inclusive_tick, snncuda_profile* out) {
    if (sim == nullptr || out == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_counters before, after;
    snncuda_sim_counters(sim, &before);
    const int rc = snncuda_sim_run_until(sim, inclusive_tick);
    snncuda_sim_counters(sim, &after);
    out->ticks += after.next_tick - before.next_tick;
    out->synaptic_events += after.synaptic_events - before.synaptic_events;
    out->external_events += after.external_events - before.external_events;
    out->fires += after.fired_spikes - before.fired_spikes;
    return rc;
}

const char* snncuda_kernel_name(int32_t) { return ""; }

int snncuda_sim_recognition(snncuda_sim* sim, uint64_t* neuron_matches, uint64_t* synapse_code_matches) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    uint64_t a = 0, b = 0;
    std::vector<uint64_t> m(sim->connectome.neurons.size()), c(sim->connectome.synapses.size());
    snncuda_neuron_state ns{};
    ns.match_count = m.data();
    snncuda_synapse_state ss{};
    ss.code_match_count = c.data();
    snncuda_sim_read_neurons(sim, &ns);
    snncuda_sim_read_synapses(sim, &ss);
    for (uint64_t v : m) a += v;
    for (uint64_t v : c) b += v;
    if (neuron_matches) *neuron_matches = a;
    if (synapse_code_matches) *synapse_code_matches = b;
    return SNNCUDA_OK;
}

// Stable grouping of an event buffer by target (host memory here).
int snncuda_group_events(const uint64_t* events, uint32_t count, uint32_t neuron_count, uint64_t* grouped,
                         uint32_t* segment_start, void*) {
    if ((count > 0 && (events == nullptr || grouped == nullptr)) || segment_start == nullptr)
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null array");
    if (count > 0 && events < grouped + count && grouped < events + count)
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "events and grouped overlap");
    std::vector<uint32_t> start(static_cast<size_t>(neuron_count) + 1, 0);
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t tgt = static_cast<uint32_t>(events[i]) & 0x7FFFFFFFu;
        if (tgt >= neuron_count) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "event target >= neuron_count");
        start[tgt + 1] += 1;
    }
    for (uint32_t n = 0; n < neuron_count; ++n) start[n + 1] += start[n];
    for (uint32_t n = 0; n <= neuron_count; ++n) segment_start[n] = start[n];
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t lo = static_cast<uint32_t>(events[i]);
        const uint32_t tgt = lo & 0x7FFFFFFFu;
        grouped[start[tgt]++] = (events[i] & 0xFFFFFFFF00000000ULL) | (i | (lo & 0x80000000u));
    }
    return SNNCUDA_OK;
}

// Same as snncuda_group_events here (the oracle has no device scratch).
int snncuda_group_events_static(const uint64_t* events, uint32_t count, uint32_t neuron_count,
                                uint64_t* grouped, uint32_t* segment_start, void* stream) {
    if (count > SNNCUDA_GROUP_STATIC_MAX_EVENTS || neuron_count > SNNCUDA_GROUP_STATIC_MAX_NEURONS)
        return fail(SNNCUDA_ERR_CAPACITY, "beyond the static grouping limits");
    return snncuda_group_events(events, count, neuron_count, grouped, segment_start, stream);
}

}  // extern "C"




#include "../batch_of_sims.inc"
#include "../readout_port.inc"
