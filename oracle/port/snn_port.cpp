// ORACLE -- test infrastructure only.  Nothing in the product (the
// snncuda_gb300 package) links, imports or calls this file; only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, as the
// checker.
//
// A plain single-threaded CPU restatement of the SNNCuda reference runtime's
// per-tick path, behind the same C ABI as the GPU backend
// (include/snncuda_gb300.h) so that parity tests drive both the same way.
// It follows, function by function (paths relative to the reference project):
//   runtime::SpikeScheduler          src/runtime/SpikeScheduler.cpp:15-47
//   runtime::NetworkPropagator       src/runtime/NetworkPropagator.cpp:5-132
//   runtime::SynapseDendriteProcessor src/runtime/SynapseDendriteProcessor.cpp:14-365
//   learning::StdpRule               src/learning/STDP.cpp:20-40
//   snn::TemporalPatternMatcher      src/snn/TemporalPattern.cpp:12-60
// The neuron-state LRU cache (NeuronStateCache / LruCache) only changes
// where state lives, never its values, so state is kept in plain vectors.
// Its results are pinned against the reference sources compiled as-is
// (oracle/refharness) and against the committed golden fixtures.
//
// Build with -ffp-contract=off: the reference arithmetic is evaluated as
// separately rounded float operations.

#include "snncuda_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

struct Compartment {
    float current{0.0F};
    uint64_t last_update_tick{0};
    float decay_tau_ticks{5.0F};
};

struct Neuron {
    float membrane{0.0F};
    float threshold{1.0F};
    uint64_t window{500};
    float similarity{0.93F};
    uint64_t max_refs{500};
    uint64_t last_active{0};
    bool has_fired{false};
    uint64_t last_fired{0};
    uint64_t spike_count{0};
    Compartment comp[4];  // soma, basal, apical, inhibitory
    uint64_t window_start{0};
    std::vector<uint32_t> offsets;
    std::vector<std::vector<uint32_t>> learned;
    bool last_match{false};
    uint64_t match_count{0};
};

struct Synapse {
    uint32_t source{0};
    uint32_t target{0};
    float weight{1.0F};
    float max_weight{2.0F};
    uint32_t delay{1};
    std::vector<uint32_t> codes{0};
    uint8_t compartment{1};
    uint8_t receptor{0};
    bool plastic{true};
    bool has_pre{false};
    bool has_post{false};
    uint64_t last_pre{0};
    uint64_t last_post{0};
    uint64_t pre_count{0};
    uint64_t update_count{0};
    float last_delta{0.0F};
    uint64_t code_window_start{0};
    std::vector<uint32_t> code_offsets;
    std::vector<std::vector<uint32_t>> learned;
    uint64_t code_match_count{0};
    bool last_code_match{false};
};

struct Event {
    uint32_t target;
    int64_t synapse;  // -1: external input
    uint64_t delivery;
    float weight;
};

// SpikeScheduler.cpp:15-47: circular wheel of FIFO buckets.
struct Scheduler {
    std::vector<std::vector<Event>> wheel;
    uint64_t next_pop{0};
    uint64_t pending{0};

    explicit Scheduler(size_t slots) : wheel(slots) {}
    size_t slot_for(uint64_t tick) const { return static_cast<size_t>(tick % wheel.size()); }

    void schedule(Event e) {
        if (e.delivery < next_pop) e.delivery = next_pop;  // late clamp :17-19
        wheel[slot_for(e.delivery)].push_back(e);
        ++pending;
    }

    void pop_due(uint64_t tick, std::vector<Event>& due) {
        due.clear();
        while (next_pop <= tick) {
            auto& bucket = wheel[slot_for(next_pop)];
            size_t keep = 0;
            for (size_t i = 0; i < bucket.size(); ++i) {
                if (bucket[i].delivery <= tick) {
                    due.push_back(bucket[i]);
                    --pending;
                } else {
                    bucket[keep++] = bucket[i];  // retained in order :30-42
                }
            }
            bucket.resize(keep);
            ++next_pop;
        }
    }
};

constexpr float kGain[4] = {1.0F, 0.55F, 1.0F, 0.65F};   // :231-243
constexpr float kTau[4] = {5.0F, 100.0F, 10.0F, 150.0F};  // :245-257
constexpr float kSign[4] = {1.0F, 1.0F, -1.0F, -1.0F};    // :259-269

// TemporalPattern.cpp:35-60 (left = learned reference, right = candidate).
float cosine_similarity(const std::vector<uint32_t>& left, const std::vector<uint32_t>& right) {
    if (left.empty() || right.empty()) return 0.0F;
    const size_t count = std::min(left.size(), right.size());
    double dot = 0.0;
    double left_norm = 0.0;
    double right_norm = 0.0;
    for (size_t i = 0; i < count; ++i) {
        const double l = static_cast<double>(left[i]);
        const double r = static_cast<double>(right[i]);
        dot += l * r;
        left_norm += l * l;
        right_norm += r * r;
    }
    if (left_norm == 0.0 || right_norm == 0.0) return 0.0F;
    return static_cast<float>(dot / (std::sqrt(left_norm) * std::sqrt(right_norm)));
}

// TemporalPattern.cpp:12-22: best = max(0, cos...) >= threshold.
bool matches(const std::vector<std::vector<uint32_t>>& refs, const std::vector<uint32_t>& cand,
             float threshold) {
    float best = 0.0F;
    for (const auto& ref : refs) best = std::max(best, cosine_similarity(ref, cand));
    return best >= threshold;
}

// FIFO learn with a capacity (TemporalPattern.cpp:24-29 and the explicit
// learn_pattern / code learn in SynapseDendriteProcessor.cpp:31-41, :361-364).
void fifo_push(std::vector<std::vector<uint32_t>>& refs, const std::vector<uint32_t>& pattern,
               uint64_t capacity) {
    if (refs.size() >= capacity) refs.erase(refs.begin());
    refs.push_back(pattern);
}

struct Digest {
    uint64_t h{0xcbf29ce484222325ULL};
    void word(uint64_t w) { h = (h ^ w) * 0x100000001b3ULL; }
    void f32(float f) {
        uint32_t b;
        std::memcpy(&b, &f, 4);
        word(b);
    }
};

}  // namespace

struct snncuda_sim {
    std::vector<Neuron> neurons;
    std::vector<Synapse> synapses;
    std::vector<std::vector<uint32_t>> outgoing;
    std::vector<std::vector<uint32_t>> incoming;
    Scheduler scheduler{1};
    // StdpConfig
    bool stdp_enabled{true};
    float ltp_amp{0.01F}, ltd_amp{0.012F}, ltp_tau{20.0F}, ltd_tau{20.0F}, min_w{0.0F}, max_w{2.0F};
    bool temporal_enabled{true};
    uint64_t delivered{0}, fired{0}, synaptic{0}, external{0}, max_due{0};
    uint64_t raster_capacity{0};
    std::vector<uint64_t> raster_tick;
    std::vector<uint32_t> raster_neuron;
    bool poisoned{false};
    std::vector<Event> due;

    // STDP.cpp:20-35
    float weight_delta(uint64_t pre, uint64_t post) const {
        if (!stdp_enabled) return 0.0F;
        const float dt = static_cast<float>(static_cast<long long>(post) - static_cast<long long>(pre));
        if (dt > 0.0F) return ltp_amp * std::exp(-dt / ltp_tau);
        if (dt < 0.0F) return -ltd_amp * std::exp(dt / ltd_tau);
        return 0.0F;
    }
    // STDP.cpp:37-40 + the update bookkeeping of SynapseDendriteProcessor.cpp:108-122
    void stdp_apply(Synapse& s, uint64_t pre, uint64_t post) const {
        const float before = s.weight;
        const float maximum = std::min(max_w, s.max_weight);
        s.weight = std::clamp(s.weight + weight_delta(pre, post), min_w, maximum);
        s.last_delta = s.weight - before;
        if (s.last_delta != 0.0F) ++s.update_count;
    }

    // SynapseDendriteProcessor.cpp:214-229
    static void decay(Neuron& n, uint64_t tick) {
        for (auto& c : n.comp) {
            if (tick <= c.last_update_tick || c.current == 0.0F) {
                c.last_update_tick = tick;
                continue;
            }
            const float elapsed = static_cast<float>(tick - c.last_update_tick);
            c.current = static_cast<float>(c.current * std::exp(-elapsed / c.decay_tau_ticks));
            c.last_update_tick = tick;
        }
    }

    // SynapseDendriteProcessor.cpp:294-316 with :14-41
    void update_temporal(Neuron& n, uint64_t tick) const {
        if (!temporal_enabled) {
            n.last_match = false;
            return;
        }
        if (n.offsets.empty() || tick - n.window_start > n.window) {
            n.window_start = tick;
            n.offsets.clear();
        }
        n.offsets.push_back(static_cast<uint32_t>(tick - n.window_start));
        n.last_match = !n.learned.empty() && n.offsets.size() >= 2 &&
                       matches(n.learned, n.offsets, n.similarity);
        if (n.last_match) {
            ++n.match_count;
            return;
        }
        if (n.offsets.size() < 2) return;
        fifo_push(n.learned, n.offsets, n.max_refs);
    }

    // SynapseDendriteProcessor.cpp:318-365
    void update_code(Synapse& s, const Neuron& target, uint64_t tick) const {
        if (!temporal_enabled) {
            s.last_code_match = false;
            return;
        }
        if (s.code_offsets.empty() || tick - s.code_window_start > target.window) {
            s.code_window_start = tick;
            s.code_offsets.clear();
        }
        s.code_offsets.push_back(static_cast<uint32_t>(tick - s.code_window_start));
        s.last_code_match = false;
        const size_t expected = std::max<size_t>(2, s.codes.size());
        if (s.code_offsets.size() < expected) return;
        if (s.code_offsets.size() > expected) {
            s.code_offsets.erase(s.code_offsets.begin(),
                                 s.code_offsets.end() - static_cast<std::ptrdiff_t>(expected));
        }
        s.last_code_match = matches(s.learned, s.code_offsets, target.similarity);
        if (s.last_code_match) {
            ++s.code_match_count;
            return;
        }
        fifo_push(s.learned, s.code_offsets, target.max_refs);
    }

    // SynapseDendriteProcessor.cpp:175-212; returns whether the neuron fired.
    bool process_input(Neuron& n, uint8_t compartment, uint8_t receptor, float weight,
                       uint64_t tick) const {
        decay(n, tick);
        const float applied = weight * kGain[receptor] * kSign[receptor];
        Compartment& c = n.comp[compartment];
        c.current += applied;
        c.last_update_tick = tick;
        c.decay_tau_ticks = kTau[receptor];
        n.last_active = tick;
        update_temporal(n, tick);
        n.membrane = n.comp[0].current + n.comp[1].current + n.comp[2].current + n.comp[3].current;
        if (n.membrane >= n.threshold) {
            n.membrane = 0.0F;
            const float reset_tau[4] = {kTau[0], kTau[0], kTau[1], kTau[2]};
            for (int k = 0; k < 4; ++k) {
                n.comp[k].current = 0.0F;
                n.comp[k].last_update_tick = tick;
                n.comp[k].decay_tau_ticks = reset_tau[k];
            }
            n.has_fired = true;
            n.last_fired = tick;
            ++n.spike_count;
            return true;
        }
        return false;
    }

    // SynapseDendriteProcessor.cpp:89-136
    bool process_synaptic(Neuron& n, Synapse& s, uint64_t tick) {
        const uint64_t pre_tick = tick >= s.delay ? tick - s.delay : tick;
        if (s.plastic && s.has_post) stdp_apply(s, pre_tick, s.last_post);
        s.has_pre = true;
        s.last_pre = pre_tick;
        ++s.pre_count;
        const bool fired_now = process_input(n, s.compartment, s.receptor, s.weight, tick);
        update_code(s, n, tick);
        return fired_now;
    }

    // SynapseDendriteProcessor.cpp:138-173
    void post_spike(Synapse& s, uint64_t tick) const {
        s.has_post = true;
        s.last_post = tick;
        if (!s.plastic || !s.has_pre) return;
        stdp_apply(s, s.last_pre, tick);
    }

    // NetworkPropagator.cpp:78-132
    int process_tick(uint64_t tick) {
        scheduler.pop_due(tick, due);
        max_due = std::max<uint64_t>(max_due, due.size());
        for (size_t i = 0; i < due.size(); ++i) {
            const Event e = due[i];
            ++delivered;
            Neuron& n = neurons[e.target];
            bool fired_now;
            if (e.synapse < 0) {
                ++external;
                fired_now = process_input(n, SNNCUDA_COMPARTMENT_SOMA, SNNCUDA_RECEPTOR_AMPA,
                                          e.weight, tick);
            } else {
                ++synaptic;
                fired_now = process_synaptic(n, synapses[static_cast<size_t>(e.synapse)], tick);
            }
            if (!fired_now) continue;
            ++fired;
            if (raster_capacity > 0) {
                if (raster_tick.size() >= raster_capacity) {
                    poisoned = true;
                    return fail(SNNCUDA_ERR_CAPACITY, "raster capacity exceeded");
                }
                raster_tick.push_back(tick);
                raster_neuron.push_back(e.target);
            }
            for (uint32_t sid : incoming[e.target]) post_spike(synapses[sid], tick);
            for (uint32_t sid : outgoing[e.target]) {
                const Synapse& s = synapses[sid];
                for (uint32_t off : s.codes) {
                    scheduler.schedule(Event{s.target, static_cast<int64_t>(sid),
                                             tick + s.delay + off, s.weight});
                }
            }
        }
        return SNNCUDA_OK;
    }
};

extern "C" {

const char* snncuda_version(void) { return "0.1.0-oracle-port"; }
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
    if (cfg->timing_wheel_slots == 0)
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT,
                    "Spike scheduler timing wheel must have at least one slot");
    try {
        auto* sim = new snncuda_sim();
        sim->scheduler = Scheduler(static_cast<size_t>(cfg->timing_wheel_slots));
        sim->stdp_enabled = cfg->stdp_enabled != 0;
        sim->ltp_amp = cfg->ltp_amplitude;
        sim->ltd_amp = cfg->ltd_amplitude;
        sim->ltp_tau = cfg->ltp_tau_ticks;
        sim->ltd_tau = cfg->ltd_tau_ticks;
        sim->min_w = cfg->min_weight;
        sim->max_w = cfg->max_weight;
        sim->temporal_enabled = cfg->temporal_learning_enabled != 0;
        sim->raster_capacity = cfg->raster_capacity;
        const uint32_t N = net->neuron_count;
        sim->neurons.resize(N);
        for (uint32_t i = 0; i < N; ++i) {
            Neuron& n = sim->neurons[i];
            if (net->threshold) n.threshold = net->threshold[i];
            if (net->pattern_window_ticks) n.window = net->pattern_window_ticks[i];
            if (net->similarity_threshold) n.similarity = net->similarity_threshold[i];
            if (net->max_reference_patterns) n.max_refs = net->max_reference_patterns[i];
            if (n.max_refs == 0) {
                delete sim;
                return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "max_reference_patterns must be >= 1");
            }
        }
        const uint64_t S = net->synapse_count;
        sim->synapses.resize(S);
        sim->outgoing.resize(N);
        sim->incoming.resize(N);
        for (uint64_t s = 0; s < S; ++s) {
            Synapse& y = sim->synapses[s];
            y.source = net->source[s];
            y.target = net->target[s];
            if (y.source >= N || y.target >= N) {
                delete sim;
                return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse endpoint out of range");
            }
            y.weight = net->weight ? net->weight[s] : 1.0F;
            y.max_weight = net->max_weight ? net->max_weight[s] : 2.0F;
            y.delay = net->delay_ticks ? net->delay_ticks[s] : 1U;
            y.compartment = net->compartment ? net->compartment[s] : SNNCUDA_COMPARTMENT_BASAL;
            y.receptor = net->receptor ? net->receptor[s] : SNNCUDA_RECEPTOR_AMPA;
            y.plastic = net->plasticity_enabled ? net->plasticity_enabled[s] != 0 : true;
            if (y.compartment > 3 || y.receptor > 3) {
                delete sim;
                return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "compartment/receptor out of range");
            }
            if (net->code_offset_ptr != nullptr && net->code_offsets != nullptr) {
                const uint64_t b = net->code_offset_ptr[s], e = net->code_offset_ptr[s + 1];
                if (e > b) y.codes.assign(net->code_offsets + b, net->code_offsets + e);
            }
            sim->outgoing[y.source].push_back(static_cast<uint32_t>(s));
            sim->incoming[y.target].push_back(static_cast<uint32_t>(s));
        }
        *out = sim;
        return SNNCUDA_OK;
    } catch (const std::bad_alloc&) {
        return fail(SNNCUDA_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& ex) {
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, ex.what());
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
        if (neurons[i] >= sim->neurons.size())
            return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "inject neuron out of range");
    }
    for (uint64_t i = 0; i < count; ++i)
        sim->scheduler.schedule(Event{neurons[i], -1, ticks[i], weights[i]});
    return SNNCUDA_OK;
}

int snncuda_sim_run_until(snncuda_sim* sim, uint64_t inclusive_tick) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->poisoned) return fail(SNNCUDA_ERR_POISONED, "simulation poisoned by an earlier error");
    // Ticks before next_pop are no-ops in the reference loop (pop_due returns nothing).
    for (uint64_t t = sim->scheduler.next_pop; t <= inclusive_tick; ++t) {
        const int rc = sim->process_tick(t);
        if (rc != SNNCUDA_OK) return rc;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_set_plasticity(snncuda_sim* sim, int32_t enabled) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    sim->stdp_enabled = enabled != 0;
    return SNNCUDA_OK;
}

int snncuda_sim_set_temporal_learning(snncuda_sim* sim, int32_t enabled) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    sim->temporal_enabled = enabled != 0;
    return SNNCUDA_OK;
}

int snncuda_sim_counters(snncuda_sim* sim, snncuda_counters* out) {
    if (sim == nullptr || out == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    out->delivered_spikes = sim->delivered;
    out->fired_spikes = sim->fired;
    out->synaptic_events = sim->synaptic;
    out->external_events = sim->external;
    out->next_tick = sim->scheduler.next_pop;
    out->pending_events = sim->scheduler.pending;
    out->raster_count = sim->raster_tick.size();
    out->max_slot_events = sim->max_due;
    return SNNCUDA_OK;
}

int snncuda_sim_idle(snncuda_sim* sim, int32_t* out) {
    if (sim == nullptr || out == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->scheduler.pending == 0 ? 1 : 0;
    return SNNCUDA_OK;
}

int snncuda_sim_read_neurons(snncuda_sim* sim, const snncuda_neuron_state* o) {
    if (sim == nullptr || o == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    for (size_t i = 0; i < sim->neurons.size(); ++i) {
        const Neuron& n = sim->neurons[i];
        if (o->membrane_potential) o->membrane_potential[i] = n.membrane;
        if (o->spike_count) o->spike_count[i] = n.spike_count;
        if (o->last_fired_tick) o->last_fired_tick[i] = n.has_fired ? static_cast<int64_t>(n.last_fired) : -1;
        if (o->last_active_tick) o->last_active_tick[i] = n.last_active;
        for (int k = 0; k < 4; ++k) {
            if (o->compartment_current) o->compartment_current[i * 4 + k] = n.comp[k].current;
            if (o->compartment_last_update) o->compartment_last_update[i * 4 + k] = n.comp[k].last_update_tick;
            if (o->compartment_tau) o->compartment_tau[i * 4 + k] = n.comp[k].decay_tau_ticks;
        }
        if (o->window_start_tick) o->window_start_tick[i] = n.window_start;
        if (o->offset_count) o->offset_count[i] = n.offsets.size();
        if (o->learned_count) o->learned_count[i] = n.learned.size();
        if (o->match_count) o->match_count[i] = n.match_count;
        if (o->last_match) o->last_match[i] = n.last_match ? 1 : 0;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_read_synapses(snncuda_sim* sim, const snncuda_synapse_state* o) {
    if (sim == nullptr || o == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    for (size_t i = 0; i < sim->synapses.size(); ++i) {
        const Synapse& s = sim->synapses[i];
        if (o->weight) o->weight[i] = s.weight;
        if (o->last_pre_spike_tick) o->last_pre_spike_tick[i] = s.has_pre ? static_cast<int64_t>(s.last_pre) : -1;
        if (o->last_post_spike_tick) o->last_post_spike_tick[i] = s.has_post ? static_cast<int64_t>(s.last_post) : -1;
        if (o->pre_spike_count) o->pre_spike_count[i] = s.pre_count;
        if (o->plasticity_update_count) o->plasticity_update_count[i] = s.update_count;
        if (o->last_weight_delta) o->last_weight_delta[i] = s.last_delta;
        if (o->code_window_start_tick) o->code_window_start_tick[i] = s.code_window_start;
        if (o->code_offset_count) o->code_offset_count[i] = s.code_offsets.size();
        if (o->learned_code_count) o->learned_code_count[i] = s.learned.size();
        if (o->code_match_count) o->code_match_count[i] = s.code_match_count;
        if (o->last_code_match) o->last_code_match[i] = s.last_code_match ? 1 : 0;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_read_pattern(snncuda_sim* sim, int32_t kind, uint64_t index, uint64_t which,
                             uint32_t* values, uint64_t capacity, uint64_t* len) {
    if (sim == nullptr || len == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    const std::vector<uint32_t>* v = nullptr;
    if (kind == 0 || kind == 1) {
        if (index >= sim->neurons.size()) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "neuron out of range");
        const Neuron& n = sim->neurons[index];
        if (kind == 0) v = &n.offsets;
        else if (which < n.learned.size()) v = &n.learned[which];
    } else if (kind == 2 || kind == 3) {
        if (index >= sim->synapses.size()) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse out of range");
        const Synapse& s = sim->synapses[index];
        if (kind == 2) v = &s.code_offsets;
        else if (which < s.learned.size()) v = &s.learned[which];
    } else {
        return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "unknown pattern kind");
    }
    if (v == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "pattern index out of range");
    *len = v->size();
    for (uint64_t i = 0; i < v->size() && i < capacity; ++i) values[i] = (*v)[i];
    return SNNCUDA_OK;
}

// Digest definition shared by every implementation of this ABI: a 64-bit
// FNV-style fold (h = (h ^ w) * 0x100000001b3) over 64-bit words, in the
// field order below.  Floats fold their IEEE bit pattern, optional ticks
// fold as int64 with -1 for "none", lists fold their length then values.
int snncuda_sim_state_digest(snncuda_sim* sim, uint64_t* neuron_digest, uint64_t* synapse_digest) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (neuron_digest) {
        Digest d;
        for (const Neuron& n : sim->neurons) {
            d.f32(n.membrane);
            d.word(n.spike_count);
            d.word(n.has_fired ? n.last_fired : ~0ULL);
            d.word(n.last_active);
            for (const auto& c : n.comp) {
                d.f32(c.current);
                d.word(c.last_update_tick);
                d.f32(c.decay_tau_ticks);
            }
            d.word(n.window_start);
            d.word(n.offsets.size());
            for (uint32_t v : n.offsets) d.word(v);
            d.word(n.learned.size());
            for (const auto& p : n.learned) {
                d.word(p.size());
                for (uint32_t v : p) d.word(v);
            }
            d.word(n.last_match ? 1 : 0);
            d.word(n.match_count);
        }
        *neuron_digest = d.h;
    }
    if (synapse_digest) {
        Digest d;
        for (const Synapse& s : sim->synapses) {
            d.f32(s.weight);
            d.word(s.has_pre ? s.last_pre : ~0ULL);
            d.word(s.has_post ? s.last_post : ~0ULL);
            d.word(s.pre_count);
            d.word(s.update_count);
            d.f32(s.last_delta);
            d.word(s.code_window_start);
            d.word(s.code_offsets.size());
            for (uint32_t v : s.code_offsets) d.word(v);
            d.word(s.learned.size());
            for (const auto& p : s.learned) {
                d.word(p.size());
                for (uint32_t v : p) d.word(v);
            }
            d.word(s.code_match_count);
            d.word(s.last_code_match ? 1 : 0);
        }
        *synapse_digest = d.h;
    }
    return SNNCUDA_OK;
}

int snncuda_sim_read_raster(snncuda_sim* sim, uint64_t first, uint64_t count, uint64_t* ticks,
                            uint32_t* neurons) {
    if (sim == nullptr) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
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
    std::vector<uint64_t> m(sim->neurons.size()), c(sim->synapses.size());
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
