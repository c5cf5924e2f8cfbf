// Synthetic SNN workloads for tests and benchmarks (host code).
//
// Networks are produced source-major: the synapses of neuron 0 first, in
// generation order, so Connectome order == generation order and every
// source's outgoing list is contiguous.  All randomness comes from a
// counter-based generator (splitmix64 of seed, stream, counter), and the
// transcendental functions below are written out from their series using
// only IEEE +,-,*,/ and exact exponent scaling, so a given spec yields
// bit-identical arrays on any host and any thread count.  Compile with
// -ffp-contract=off.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

namespace {

uint64_t splitmix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

struct Stream {
    uint64_t key;
    uint64_t counter{0};
    Stream(uint64_t seed, uint64_t stream) : key(splitmix(seed ^ splitmix(stream + 0x51ED))) {}
    uint64_t next() { return splitmix(key + 0xD1B54A32D192ED03ULL * (++counter)); }
    double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    uint32_t below(uint32_t n) { return static_cast<uint32_t>(((next() >> 32) * n) >> 32); }  // [0,n)
    uint32_t range(uint32_t lo, uint32_t hi) { return lo + below(hi - lo + 1); }             // [lo,hi]
};

// ln(x) for x > 0: x = m * 2^e, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)).
double det_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    const double t = (m - 1.0) / (m + 1.0);
    const double t2 = t * t;
    double term = t, sum = 0.0;
    for (int k = 1; k < 40; k += 2) {
        sum += term / k;
        term *= t2;
    }
    return 2.0 * sum + e * 0.69314718055994530942;
}

// exp(x): x = k ln2 + r, |r| <= ln2/2, Taylor series of exp(r), scaled by 2^k.
double det_exp(double x) {
    const double k = std::floor(x / 0.69314718055994530942 + 0.5);
    const double r = x - k * 0.69314718055994530942;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 30; ++n) {
        term = term * r / n;
        sum += term;
    }
    return std::ldexp(sum, static_cast<int>(k));
}

// Standard normal by the Marsaglia polar method.
double det_normal(Stream& s) {
    for (;;) {
        const double u = 2.0 * s.uniform() - 1.0;
        const double v = 2.0 * s.uniform() - 1.0;
        const double q = u * u + v * v;
        if (q > 0.0 && q < 1.0) return u * std::sqrt(-2.0 * det_log(q) / q);
    }
}

template <typename F>
void parallel_for(uint64_t n, F&& body) {
    unsigned threads = std::max(1U, std::min(64U, std::thread::hardware_concurrency()));
    if (n < 4096) threads = 1;
    std::vector<std::thread> pool;
    const uint64_t chunk = (n + threads - 1) / threads;
    for (unsigned t = 0; t < threads; ++t) {
        const uint64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        pool.emplace_back([b, e, &body] {
            for (uint64_t i = b; i < e; ++i) body(i);
        });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// Workload description.  Weight kinds: 0 = uniform (excitatory U[0,0.5],
// inhibitory U[-1,0], both times weight_scale, AMPA receptor, inhibitory
// synapses on the inhibitory compartment); 1 = lognormal(mu, sigma) times
// weight_scale, excitatory AMPA (NMDA on the apical compartment),
// inhibitory as a positive magnitude on a GABA_A receptor.
typedef struct snngen_spec {
    uint32_t neuron_count;
    uint32_t excitatory_count;       // neurons [0, excitatory_count) are excitatory
    uint32_t fanout;                 // outgoing synapses per neuron (targets with replacement)
    uint32_t weight_kind;
    float weight_scale;
    float lognormal_mu;
    float lognormal_sigma;
    float max_weight;
    uint32_t delay_min, delay_max;   // uniform integer
    uint32_t codes_min, codes_max;   // spike-code offsets per synapse, uniform integer
    uint32_t code_offset_max;        // each offset uniform in [0, code_offset_max]
    uint32_t compartments;           // 2: basal/apical alternating; 4: soma/basal/apical uniform
    uint8_t plastic;
    float threshold;
    uint64_t pattern_window_ticks;
    float similarity_threshold;
    uint64_t max_reference_patterns;
    uint64_t seed;
} snngen_spec;

// Caller-allocated output arrays (the generator fills them in parallel).
// code_offsets must hold neuron_count * fanout * codes_max entries; the
// number written is returned in *code_count.
typedef struct snngen_network {
    float* threshold;                  // [N]
    uint64_t* pattern_window_ticks;    // [N]
    float* similarity_threshold;       // [N]
    uint64_t* max_reference_patterns;  // [N]
    uint32_t* source;                  // [S]
    uint32_t* target;                  // [S]
    float* weight;                     // [S]
    float* max_weight;                 // [S]
    uint32_t* delay_ticks;             // [S]
    uint8_t* compartment;              // [S]
    uint8_t* receptor;                 // [S]
    uint8_t* plasticity_enabled;       // [S]
    uint64_t* code_offset_ptr;         // [S+1]
    uint32_t* code_offsets;            // [S * codes_max]
} snngen_network;

int snngen_fill_network(const snngen_spec* spec, const snngen_network* out, uint64_t* code_count) {
    if (spec == nullptr || out == nullptr || code_count == nullptr || spec->neuron_count == 0 ||
        spec->delay_min > spec->delay_max || spec->codes_min == 0 || spec->codes_min > spec->codes_max ||
        (spec->compartments != 2 && spec->compartments != 4))
        return 1;
    const uint32_t N = spec->neuron_count;
    const uint64_t S = static_cast<uint64_t>(N) * spec->fanout;
    const uint32_t F = spec->fanout;
    parallel_for(N, [&](uint64_t i) {
        out->threshold[i] = spec->threshold;
        out->pattern_window_ticks[i] = spec->pattern_window_ticks;
        out->similarity_threshold[i] = spec->similarity_threshold;
        out->max_reference_patterns[i] = spec->max_reference_patterns;
    });
    // Code counts per synapse (stream 2*src+1) into code_offset_ptr[s+1], then
    // an in-place prefix sum.
    out->code_offset_ptr[0] = 0;
    parallel_for(N, [&](uint64_t src) {
        Stream r(spec->seed, 2 * src + 1);
        for (uint32_t j = 0; j < F; ++j) out->code_offset_ptr[src * F + j + 1] = r.range(spec->codes_min, spec->codes_max);
    });
    for (uint64_t s = 0; s < S; ++s) out->code_offset_ptr[s + 1] += out->code_offset_ptr[s];
    *code_count = out->code_offset_ptr[S];
    parallel_for(N, [&](uint64_t src) {
        Stream r(spec->seed, 2 * src);
        Stream rc(spec->seed, 2 * src + 1);
        for (uint32_t j = 0; j < F; ++j) rc.next();  // skip the counts drawn above
        const bool exc = src < spec->excitatory_count;
        for (uint32_t j = 0; j < F; ++j) {
            const uint64_t s = src * F + j;
            out->source[s] = static_cast<uint32_t>(src);
            out->target[s] = r.below(N);
            float w;
            if (spec->weight_kind == 0) {
                w = exc ? static_cast<float>(0.5 * r.uniform()) : static_cast<float>(-r.uniform());
                out->receptor[s] = 0;  // AMPA
                out->compartment[s] = exc ? static_cast<uint8_t>(1 + (j & 1)) : 3;
            } else {
                const double z = det_normal(r);
                w = static_cast<float>(det_exp(spec->lognormal_mu + spec->lognormal_sigma * z));
                if (exc) {
                    const uint8_t comp = spec->compartments == 4 ? static_cast<uint8_t>(r.below(3))
                                                                 : static_cast<uint8_t>(1 + (j & 1));
                    out->compartment[s] = comp;
                    out->receptor[s] = comp == 2 ? 1 : 0;  // apical NMDA, else AMPA
                } else {
                    out->compartment[s] = 3;
                    out->receptor[s] = 2;  // GABA_A, positive magnitude
                }
            }
            out->weight[s] = w * spec->weight_scale;
            out->max_weight[s] = spec->max_weight;
            out->delay_ticks[s] = r.range(spec->delay_min, spec->delay_max);
            out->plasticity_enabled[s] = spec->plastic;
            for (uint64_t k = out->code_offset_ptr[s]; k < out->code_offset_ptr[s + 1]; ++k)
                out->code_offsets[k] = rc.range(0, spec->code_offset_max);
        }
    });
    return 0;
}

typedef struct snngen_drive {
    uint64_t count;
    uint32_t* neuron;
    uint64_t* tick;
    float* weight;
} snngen_drive;

void snngen_free_drive(snngen_drive* d) {
    if (d == nullptr) return;
    delete[] d->neuron;
    delete[] d->tick;
    delete[] d->weight;
    std::memset(d, 0, sizeof(*d));
}

// Independent Bernoulli(p) drive per neuron and tick in [0, ticks) (a
// Poisson process at p per tick), weight `weight`, over neurons
// [first, first+count); plus, when stimulus_codes > 0, a repeating temporal
// stimulus: every `period` ticks presentation k delivers code (k mod
// stimulus_codes) -- `code_length` offsets drawn once in [0, code_offset_max]
// -- to every neuron in [stim_first, stim_first+stim_count) at base + offset
// with weight stim_weight.  Output sorted by (tick, neuron, kind).
int snngen_build_drive(uint32_t first, uint32_t count, uint64_t ticks, double p, float weight,
                       uint32_t stimulus_codes, uint32_t code_length, uint32_t code_offset_max,
                       uint32_t period, uint32_t stim_first, uint32_t stim_count, float stim_weight,
                       uint64_t seed, snngen_drive* out) {
    if (out == nullptr || p < 0.0 || p >= 1.0) return 1;
    std::memset(out, 0, sizeof(*out));
    struct Item {
        uint64_t tick;
        uint32_t neuron;
        uint32_t kind;
        float weight;
    };
    std::vector<std::vector<Item>> per(count);
    if (p > 0.0) {
        const double lq = det_log(1.0 - p);
        parallel_for(count, [&](uint64_t i) {
            Stream r(seed ^ 0xD21FEULL, i + first);
            uint64_t t = 0;
            for (;;) {
                double u = r.uniform();
                if (u <= 0.0) u = 1e-300;
                const double gap = std::floor(det_log(u) / lq);  // failures before a success
                if (gap >= static_cast<double>(ticks)) break;
                t += static_cast<uint64_t>(gap);
                if (t >= ticks) break;
                per[i].push_back({t, static_cast<uint32_t>(i + first), 0, weight});
                ++t;
            }
        });
    }
    std::vector<Item> all;
    size_t total = 0;
    for (auto& v : per) total += v.size();
    all.reserve(total);
    for (auto& v : per) all.insert(all.end(), v.begin(), v.end());
    if (stimulus_codes > 0 && period > 0) {
        Stream r(seed ^ 0xC0DEULL, 0);
        std::vector<uint32_t> codes(static_cast<size_t>(stimulus_codes) * code_length);
        for (auto& c : codes) c = r.range(0, code_offset_max);
        for (uint64_t base = 0, k = 0; base < ticks; base += period, ++k) {
            const uint32_t* code = &codes[(k % stimulus_codes) * code_length];
            for (uint32_t j = 0; j < code_length; ++j) {
                const uint64_t t = base + code[j];
                if (t >= ticks) continue;
                for (uint32_t n = 0; n < stim_count; ++n) all.push_back({t, stim_first + n, 1, stim_weight});
            }
        }
    }
    std::stable_sort(all.begin(), all.end(), [](const Item& a, const Item& b) {
        if (a.tick != b.tick) return a.tick < b.tick;
        if (a.neuron != b.neuron) return a.neuron < b.neuron;
        return a.kind < b.kind;
    });
    try {
        out->count = all.size();
        out->neuron = new uint32_t[all.size() + 1];
        out->tick = new uint64_t[all.size() + 1];
        out->weight = new float[all.size() + 1];
    } catch (const std::bad_alloc&) {
        snngen_free_drive(out);
        return 2;
    }
    for (size_t i = 0; i < all.size(); ++i) {
        out->neuron[i] = all[i].neuron;
        out->tick[i] = all[i].tick;
        out->weight[i] = all[i].weight;
    }
    return 0;
}

}  // extern "C"
