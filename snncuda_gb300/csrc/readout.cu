// Inference readouts of the GB300 backend: the reference inference
// session's one-hop feed-forward readout and its recurrent hidden/readout
// iteration (CudaInferenceSession::run_feedforward_batch and
// run_recurrent_feedforward_batch, CudaBackend.cu:1725-2100), over the
// Connectome's initial weights.
//
// The reference pushes every contribution with a float atomicAdd, so its
// sums come out in an unspecified order.  Here every sum is pulled by one
// thread in a fixed order -- a readout's (or hidden neuron's) incoming
// synapses in Connectome order, and the time steps in order -- so results
// are deterministic and equal to the same sums computed sequentially.
//
//   k_feedforward   one block per sample, a thread per readout: the sum over
//                   the readout's incoming synapses whose source is one of the
//                   sample's (merged) inputs of input weight x synapse weight
//   k_recurrent     one block per sample running every time step: top-k of
//                   the hidden events, hidden -> readout propagation (delay
//                   d lands d steps later), readout gates (threshold or
//                   top-k), gated feedback readout -> hidden scaled by the
//                   feedback decay; the readout events summed over the steps

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "pack.h"
#include "snncuda_gb300.h"

namespace {

constexpr int kThreads = 256;
constexpr float kLowest = -3.402823466e+38F;

struct InEdges {
    const unsigned long long* ptr;  // [N+1]
    const uint32_t* src;
    const uint32_t* delay;           // max(1, delay_ticks)
    const float* w;                  // initial weight
};

// Weight of neuron n among a sample's merged inputs (sorted by neuron), or 0.
__device__ __forceinline__ float input_weight(const uint32_t* nb, const float* wb, uint32_t m, uint32_t n) {
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (nb[mid] < n) {
            lo = mid + 1;
        } else {
            hi = mid;
        }
    }
    return lo < m && nb[lo] == n ? wb[lo] : 0.0F;
}

__global__ void __launch_bounds__(kThreads) k_feedforward(InEdges g, const unsigned long long* in_ptr,
                                                          const uint32_t* in_n, const float* in_w, uint32_t R,
                                                          const uint32_t* readouts, const float* thresholds,
                                                          float* scores, unsigned long long* spikes) {
    const uint32_t s = blockIdx.x;
    const unsigned long long b = in_ptr[s];
    const uint32_t m = static_cast<uint32_t>(in_ptr[s + 1] - b);
    for (uint32_t r = threadIdx.x; r < R; r += blockDim.x) {
        const uint32_t n = readouts[r];
        float score = 0.0F;
        for (unsigned long long e = g.ptr[n]; e < g.ptr[n + 1]; ++e) {
            const float x = input_weight(in_n + b, in_w + b, m, g.src[e]);
            if (x != 0.0F) score = __fadd_rn(score, __fmul_rn(x, g.w[e]));
        }
        scores[static_cast<size_t>(s) * R + r] = score;
        spikes[static_cast<size_t>(s) * R + r] = score >= thresholds[r] ? 1ull : 0ull;
    }
}

struct RecurrentArgs {
    InEdges g;
    uint32_t H, R, T;
    const uint32_t* hidden;         // [H] dense neuron of each hidden index
    const uint32_t* readouts;       // [R]
    const int* to_hidden;           // [N] hidden index of a neuron, -1
    const int* to_readout;          // [N] readout index of a neuron, -1
    const float* thresholds;        // [R]
    float* hid;                     // [samples][T][H] hidden events
    float* out;                     // [samples][T][R] readout events
    float* gate;                    // [samples][R]
    int* hsel;                      // [samples][H] top-k scratch
    int* rsel;                      // [samples][R]
    float decay;
    uint32_t topk_readouts, topk_hidden;
    int use_scores;
    float* scores;                  // [samples][R]
    unsigned long long* spikes;     // [samples][R]
};

// Marks the k largest of v[0 .. n) (strictly larger wins: the first of equal
// values), one thread.
__device__ void top_k(const float* v, uint32_t n, uint32_t k, int* sel) {
    for (uint32_t i = 0; i < n; ++i) sel[i] = 0;
    const uint32_t limit = k < n ? k : n;
    for (uint32_t pass = 0; pass < limit; ++pass) {
        int best = -1;
        float best_score = kLowest;
        for (uint32_t i = 0; i < n; ++i) {
            if (sel[i] == 0 && v[i] > best_score) {
                best_score = v[i];
                best = static_cast<int>(i);
            }
        }
        if (best >= 0) sel[best] = 1;
    }
}

__global__ void __launch_bounds__(kThreads) k_recurrent(RecurrentArgs a) {
    const uint32_t s = blockIdx.x;
    float* hid = a.hid + static_cast<size_t>(s) * a.T * a.H;
    float* out = a.out + static_cast<size_t>(s) * a.T * a.R;
    float* gate = a.gate + static_cast<size_t>(s) * a.R;
    int* hsel = a.hsel + static_cast<size_t>(s) * a.H;
    int* rsel = a.rsel + static_cast<size_t>(s) * a.R;
    for (uint32_t t = 0; t < a.T; ++t) {
        float* ht = hid + static_cast<size_t>(t) * a.H;
        if (a.topk_hidden > 0 && a.topk_hidden < a.H) {
            if (threadIdx.x == 0) top_k(ht, a.H, a.topk_hidden, hsel);
            __syncthreads();
            for (uint32_t h = threadIdx.x; h < a.H; h += blockDim.x)
                if (hsel[h] == 0) ht[h] = 0.0F;
            __syncthreads();
        }
        // hidden events of step t reach the readouts d steps later
        for (uint32_t r = threadIdx.x; r < a.R; r += blockDim.x) {
            const uint32_t n = a.readouts[r];
            for (unsigned long long e = a.g.ptr[n]; e < a.g.ptr[n + 1]; ++e) {
                const int h = a.to_hidden[a.g.src[e]];
                const uint32_t at = t + a.g.delay[e];
                if (h < 0 || at >= a.T) continue;
                const float x = ht[h];
                if (x == 0.0F) continue;
                float* o = out + static_cast<size_t>(at) * a.R + r;
                *o = __fadd_rn(*o, __fmul_rn(x, a.g.w[e]));
            }
        }
        __syncthreads();
        // readout gates of step t
        const float* ot = out + static_cast<size_t>(t) * a.R;
        if (a.topk_readouts == 0) {
            for (uint32_t r = threadIdx.x; r < a.R; r += blockDim.x)
                gate[r] = ot[r] >= a.thresholds[r] ? (a.use_scores ? ot[r] : 1.0F) : 0.0F;
        } else if (threadIdx.x == 0) {
            top_k(ot, a.R, a.topk_readouts, rsel);
            for (uint32_t r = 0; r < a.R; ++r) gate[r] = rsel[r] ? (a.use_scores ? ot[r] : 1.0F) : 0.0F;
        }
        __syncthreads();
        // gated readouts feed back to the hidden neurons d steps later
        for (uint32_t h = threadIdx.x; h < a.H; h += blockDim.x) {
            const uint32_t n = a.hidden[h];
            for (unsigned long long e = a.g.ptr[n]; e < a.g.ptr[n + 1]; ++e) {
                const int r = a.to_readout[a.g.src[e]];
                const uint32_t at = t + a.g.delay[e];
                if (r < 0 || at >= a.T) continue;
                const float gr = gate[r];
                if (gr == 0.0F) continue;
                float* y = hid + static_cast<size_t>(at) * a.H + h;
                *y = __fadd_rn(*y, __fmul_rn(__fmul_rn(a.decay, gr), a.g.w[e]));
            }
        }
        __syncthreads();
    }
    for (uint32_t r = threadIdx.x; r < a.R; r += blockDim.x) {
        float sum = 0.0F;
        for (uint32_t t = 0; t < a.T; ++t) sum = __fadd_rn(sum, out[static_cast<size_t>(t) * a.R + r]);
        a.scores[static_cast<size_t>(s) * a.R + r] = sum;
        a.spikes[static_cast<size_t>(s) * a.R + r] = sum >= a.thresholds[r] ? 1ull : 0ull;
    }
}

struct Fail {
    int code;
    std::string msg;
};

void check(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return;
    const int code = err == cudaErrorMemoryAllocation ? SNNCUDA_ERR_OUT_OF_MEMORY : SNNCUDA_ERR_DEVICE;
    cudaGetLastError();
    throw Fail{code, std::string(what) + ": " + cudaGetErrorString(err)};
}

// Device buffers of one call, freed on scope exit.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    T* up(const std::vector<T>& v) {
        T* d = get<T>(v.size());
        if (!v.empty()) check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "copy");
        return d;
    }
    template <typename T>
    T* get(size_t n) {
        void* p = nullptr;
        check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "device allocation");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

// A sample's inputs merged per neuron (weights of one neuron summed in input
// order), sorted by neuron.
void merge_inputs(uint32_t samples, const uint64_t* ptr, const uint32_t* neurons, const float* weights, uint32_t N,
                  std::vector<unsigned long long>& mptr, std::vector<uint32_t>& mn, std::vector<float>& mw,
                  uint64_t* delivered) {
    mptr.assign(samples + 1, 0);
    for (uint32_t s = 0; s < samples; ++s) {
        std::map<uint32_t, float> merged;
        for (uint64_t i = ptr[s]; i < ptr[s + 1]; ++i) {
            if (neurons[i] >= N) throw Fail{SNNCUDA_ERR_INVALID_ARGUMENT, "input neuron out of range"};
            auto it = merged.find(neurons[i]);
            if (it == merged.end()) {
                merged.emplace(neurons[i], 0.0F + weights[i]);
            } else {
                it->second = it->second + weights[i];
            }
        }
        for (const auto& [n, w] : merged) {
            mn.push_back(n);
            mw.push_back(w);
        }
        mptr[s + 1] = mn.size();
        if (delivered) delivered[s] = merged.size();
    }
}

}  // namespace

struct snncuda_readout {
    uint32_t N{0};
    std::vector<float> threshold;
    uint32_t max_delay{1};
    unsigned long long* ptr{nullptr};
    uint32_t* src{nullptr};
    uint32_t* delay{nullptr};
    float* w{nullptr};
    ~snncuda_readout() {
        cudaFree(ptr);
        cudaFree(src);
        cudaFree(delay);
        cudaFree(w);
    }
    InEdges edges() const { return InEdges{ptr, src, delay, w}; }
};

namespace {

int fail_code(const Fail& f) {
    snngb::set_last_error_message(f.msg);
    return f.code;
}

// Readout neurons and their thresholds; rejects repeats.
void readout_list(const snncuda_readout* r, uint32_t count, const uint32_t* neurons, std::vector<uint32_t>& list,
                  std::vector<float>& thr) {
    std::vector<char> seen(r->N, 0);
    for (uint32_t i = 0; i < count; ++i) {
        if (neurons[i] >= r->N) throw Fail{SNNCUDA_ERR_INVALID_ARGUMENT, "neuron out of range"};
        if (seen[neurons[i]]) throw Fail{SNNCUDA_ERR_INVALID_ARGUMENT, "a neuron is listed twice"};
        seen[neurons[i]] = 1;
        list.push_back(neurons[i]);
        thr.push_back(r->threshold[neurons[i]]);
    }
}

}  // namespace

extern "C" {

int snncuda_readout_create(const snncuda_network* net, snncuda_readout** out) {
    if (net == nullptr || out == nullptr) return SNNCUDA_ERR_INVALID_ARGUMENT;
    snncuda_readout* r = new (std::nothrow) snncuda_readout();
    if (r == nullptr) return SNNCUDA_ERR_OUT_OF_MEMORY;
    int code = SNNCUDA_OK;
    try {
        const uint32_t N = net->neuron_count;
        const uint64_t S = net->synapse_count;
        if (N > 0 && net->threshold == nullptr) throw Fail{SNNCUDA_ERR_INVALID_ARGUMENT, "thresholds are required"};
        if (S > 0 && (!net->source || !net->target || !net->weight || !net->delay_ticks))
            throw Fail{SNNCUDA_ERR_INVALID_ARGUMENT, "synapse arrays are required"};
        r->N = N;
        r->threshold.assign(net->threshold, net->threshold + N);
        // incoming synapses of each neuron in Connectome order (stable
        // counting sort by target)
        std::vector<unsigned long long> ptr(static_cast<size_t>(N) + 1, 0);
        for (uint64_t k = 0; k < S; ++k) {
            if (net->source[k] >= N || net->target[k] >= N)
                throw Fail{SNNCUDA_ERR_INVALID_ARGUMENT, "synapse endpoint out of range"};
            ++ptr[net->target[k] + 1];
        }
        for (uint32_t n = 0; n < N; ++n) ptr[n + 1] += ptr[n];
        std::vector<unsigned long long> fill(ptr.begin(), ptr.end() - 1);
        std::vector<uint32_t> src(S), dly(S);
        std::vector<float> w(S);
        for (uint64_t k = 0; k < S; ++k) {
            const unsigned long long at = fill[net->target[k]]++;
            src[at] = net->source[k];
            dly[at] = std::max(1u, net->delay_ticks[k]);
            w[at] = net->weight[k];
            r->max_delay = std::max(r->max_delay, dly[at]);
        }
        auto upload = [](auto*& d, const auto& v) {
            using T = std::remove_reference_t<decltype(v[0])>;
            check(cudaMalloc(reinterpret_cast<void**>(&d), std::max<size_t>(v.size(), 1) * sizeof(T)), "device allocation");
            if (!v.empty()) check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "copy");
        };
        upload(r->ptr, ptr);
        upload(r->src, src);
        upload(r->delay, dly);
        upload(r->w, w);
    } catch (const Fail& f) {
        code = fail_code(f);
    } catch (const std::bad_alloc&) {
        snngb::set_last_error_message("host allocation failed");
        code = SNNCUDA_ERR_OUT_OF_MEMORY;
    }
    if (code != SNNCUDA_OK) {
        delete r;
        return code;
    }
    *out = r;
    return SNNCUDA_OK;
}

int snncuda_readout_destroy(snncuda_readout* r) {
    delete r;
    return SNNCUDA_OK;
}

int snncuda_readout_feedforward(snncuda_readout* r, uint32_t samples, const uint64_t* input_ptr,
                                const uint32_t* input_neurons, const float* input_weights, uint32_t readout_count,
                                const uint32_t* readout_neurons, float* scores, uint64_t* spikes,
                                uint64_t* delivered) {
    if (r == nullptr || (samples > 0 && input_ptr == nullptr)) return SNNCUDA_ERR_INVALID_ARGUMENT;
    int code = SNNCUDA_OK;
    try {
        if (delivered) std::fill(delivered, delivered + samples, 0);
        if (samples == 0 || readout_count == 0) return SNNCUDA_OK;
        std::vector<uint32_t> list;
        std::vector<float> thr;
        readout_list(r, readout_count, readout_neurons, list, thr);
        std::vector<unsigned long long> mptr;
        std::vector<uint32_t> mn;
        std::vector<float> mw;
        merge_inputs(samples, input_ptr, input_neurons, input_weights, r->N, mptr, mn, mw, delivered);
        Scratch sc;
        float* d_scores = sc.get<float>(static_cast<size_t>(samples) * readout_count);
        unsigned long long* d_spikes = sc.get<unsigned long long>(static_cast<size_t>(samples) * readout_count);
        k_feedforward<<<samples, kThreads>>>(r->edges(), sc.up(mptr), sc.up(mn), sc.up(mw), readout_count,
                                             sc.up(list), sc.up(thr), d_scores, d_spikes);
        check(cudaGetLastError(), "feedforward launch");
        check(cudaMemcpy(scores, d_scores, sizeof(float) * samples * readout_count, cudaMemcpyDeviceToHost), "copy");
        check(cudaMemcpy(spikes, d_spikes, sizeof(uint64_t) * samples * readout_count, cudaMemcpyDeviceToHost),
              "copy");
    } catch (const Fail& f) {
        code = fail_code(f);
    } catch (const std::bad_alloc&) {
        snngb::set_last_error_message("host allocation failed");
        code = SNNCUDA_ERR_OUT_OF_MEMORY;
    }
    return code;
}

void snncuda_recurrent_options_default(snncuda_recurrent_options* o) {
    if (o == nullptr) return;
    std::memset(o, 0, sizeof(*o));
    o->iterations = 1;
    o->feedback_decay = 0.5F;
    o->top_k_feedback_readouts = 1;
    o->top_k_hidden = 0;
    o->use_scores_not_spikes = 1;
}

int snncuda_readout_recurrent(snncuda_readout* r, uint32_t samples, const uint64_t* input_ptr,
                              const uint32_t* input_neurons, const float* input_weights, uint32_t readout_count,
                              const uint32_t* readout_neurons, uint32_t hidden_count, const uint32_t* hidden_neurons,
                              const snncuda_recurrent_options* options, float* scores, uint64_t* spikes,
                              uint64_t* delivered, uint64_t* time_steps) {
    if (r == nullptr || options == nullptr || (samples > 0 && input_ptr == nullptr))
        return SNNCUDA_ERR_INVALID_ARGUMENT;
    int code = SNNCUDA_OK;
    try {
        if (delivered) std::fill(delivered, delivered + samples, 0);
        const uint64_t T = static_cast<uint64_t>(r->max_delay) * (1 + 2ull * options->iterations) + 1;
        if (time_steps) *time_steps = T;
        if (samples == 0 || readout_count == 0) return SNNCUDA_OK;
        std::vector<uint32_t> rl, hl;
        std::vector<float> thr, hthr;
        readout_list(r, readout_count, readout_neurons, rl, thr);
        if (hidden_count > 0) {
            readout_list(r, hidden_count, hidden_neurons, hl, hthr);
        } else {  // every neuron that is not a readout, in index order
            std::vector<char> is_readout(r->N, 0);
            for (uint32_t n : rl) is_readout[n] = 1;
            for (uint32_t n = 0; n < r->N; ++n)
                if (!is_readout[n]) hl.push_back(n);
        }
        const uint32_t H = static_cast<uint32_t>(hl.size());
        if (H == 0) return SNNCUDA_OK;
        if (T > (1u << 20)) throw Fail{SNNCUDA_ERR_UNSUPPORTED, "more than 2^20 time steps"};
        std::vector<unsigned long long> mptr;
        std::vector<uint32_t> mn;
        std::vector<float> mw;
        merge_inputs(samples, input_ptr, input_neurons, input_weights, r->N, mptr, mn, mw, delivered);
        std::vector<int> to_hidden(r->N, -1), to_readout(r->N, -1);
        for (uint32_t h = 0; h < H; ++h) to_hidden[hl[h]] = static_cast<int>(h);
        for (uint32_t k = 0; k < readout_count; ++k) to_readout[rl[k]] = static_cast<int>(k);
        // hidden events of step 0: the merged inputs that are hidden neurons
        std::vector<float> hid0(static_cast<size_t>(samples) * H, 0.0F);
        for (uint32_t s = 0; s < samples; ++s)
            for (unsigned long long i = mptr[s]; i < mptr[s + 1]; ++i)
                if (to_hidden[mn[i]] >= 0) hid0[static_cast<size_t>(s) * H + to_hidden[mn[i]]] = mw[i];
        Scratch sc;
        RecurrentArgs a{};
        a.g = r->edges();
        a.H = H;
        a.R = readout_count;
        a.T = static_cast<uint32_t>(T);
        a.hidden = sc.up(hl);
        a.readouts = sc.up(rl);
        a.to_hidden = sc.up(to_hidden);
        a.to_readout = sc.up(to_readout);
        a.thresholds = sc.up(thr);
        a.hid = sc.get<float>(static_cast<size_t>(samples) * T * H);
        a.out = sc.get<float>(static_cast<size_t>(samples) * T * readout_count);
        a.gate = sc.get<float>(static_cast<size_t>(samples) * readout_count);
        a.hsel = sc.get<int>(static_cast<size_t>(samples) * H);
        a.rsel = sc.get<int>(static_cast<size_t>(samples) * readout_count);
        a.decay = options->feedback_decay;
        a.topk_readouts = options->top_k_feedback_readouts;
        a.topk_hidden = options->top_k_hidden;
        a.use_scores = options->use_scores_not_spikes ? 1 : 0;
        a.scores = sc.get<float>(static_cast<size_t>(samples) * readout_count);
        a.spikes = sc.get<unsigned long long>(static_cast<size_t>(samples) * readout_count);
        check(cudaMemset(a.hid, 0, sizeof(float) * samples * T * H), "memset");
        check(cudaMemset(a.out, 0, sizeof(float) * samples * T * readout_count), "memset");
        for (uint32_t s = 0; s < samples; ++s)
            check(cudaMemcpy(a.hid + static_cast<size_t>(s) * T * H, hid0.data() + static_cast<size_t>(s) * H,
                             sizeof(float) * H, cudaMemcpyHostToDevice), "copy");
        k_recurrent<<<samples, kThreads>>>(a);
        check(cudaGetLastError(), "recurrent launch");
        check(cudaMemcpy(scores, a.scores, sizeof(float) * samples * readout_count, cudaMemcpyDeviceToHost), "copy");
        check(cudaMemcpy(spikes, a.spikes, sizeof(uint64_t) * samples * readout_count, cudaMemcpyDeviceToHost),
              "copy");
    } catch (const Fail& f) {
        code = fail_code(f);
    } catch (const std::bad_alloc&) {
        snngb::set_last_error_message("host allocation failed");
        code = SNNCUDA_ERR_OUT_OF_MEMORY;
    }
    return code;
}

}  // extern "C"
