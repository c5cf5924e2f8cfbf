// Device-side packing of a flattened Connectome into the engine's layout.
//
// The reference builds its runtime maps on the host, one synapse at a time
// (NetworkPropagator.cpp:5-29, SynapseDendriteProcessor.cpp:59-75); at 1e9
// synapses that is minutes of single-threaded work.  Here the raw synapse
// arrays are copied to the device once and everything derived from them is
// built there:
//   * validation (endpoints, compartment/receptor, delay, code counts) and
//     the set of delivery delays delay + offset (>= 1);
//   * the target-major order: a stable radix sort of synapse indices by
//     target (Connectome order kept inside each target), its inverse, and the
//     row pointers of every target's incoming list;
//   * the 64-byte synapse records (SynapseDendriteProcessor.cpp:59-75);
//   * the pre-expanded outgoing events of every source, grouped by delivery
//     delay class in Connectome x offset order (NetworkPropagator.cpp:104-130)
//     from a stable sort by source and one thread per source.
// Temporary buffers are stream-ordered (cudaMallocAsync / cudaFreeAsync).

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "pack.h"
#include "snncuda_gb300.h"

namespace snngb {
namespace {

constexpr int kPackThreads = 256;
constexpr uint32_t kMaxDelta = 1u << 20;  // delivery delays must stay below the largest wheel

// status bits of the validation pass
constexpr uint32_t kBadEndpoint = 1u << 0;
constexpr uint32_t kBadCompartment = 1u << 1;
constexpr uint32_t kBadDelay = 1u << 2;
constexpr uint32_t kTooManyCodes = 1u << 3;
constexpr uint32_t kDelayTooLong = 1u << 4;
constexpr uint32_t kTooManyEvents = 1u << 5;

struct Raw {
    uint32_t N;
    unsigned long long S;
    const uint32_t* source;
    const uint32_t* target;
    const float* weight;
    const float* max_weight;
    const uint32_t* delay;
    const uint8_t* comp;
    const uint8_t* rec;
    const uint8_t* plastic;
    const unsigned long long* cptr;  // null: every synapse carries {0}
    const uint32_t* codes;
};

struct Scratch {
    uint32_t status;
    uint32_t max_expected;
    unsigned long long pre_total;
};

__device__ __forceinline__ void code_list(const Raw& r, unsigned long long s, unsigned long long& b, uint32_t& k) {
    if (r.cptr) {
        b = r.cptr[s];
        const unsigned long long e = r.cptr[s + 1];
        k = e > b ? static_cast<uint32_t>(e - b < 0xFFFFFFFFull ? e - b : 0xFFFFFFFFull) : 0u;
    } else {
        b = 0;
        k = 0;
    }
}

// Validation, per-target / per-source counts, delay classes present, the
// largest `expected` and the number of (synapse, offset) events.
__global__ void k_pack_scan(Raw r, Scratch* sc, unsigned long long* in_cnt, unsigned long long* out_cnt,
                            uint8_t* present) {
    uint32_t status = 0, max_exp = 2;
    unsigned long long events = 0;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long s = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; s < r.S;
         s += stride) {
        const uint32_t src = r.source[s], tgt = r.target[s];
        if (src >= r.N || tgt >= r.N) {
            status |= kBadEndpoint;
            continue;
        }
        if (r.comp[s] > 3 || r.rec[s] > 3) status |= kBadCompartment;
        const uint32_t d = r.delay[s];
        if (d > kMetaDelayMask) status |= kBadDelay;
        unsigned long long b;
        uint32_t k;
        code_list(r, s, b, k);
        if (k > static_cast<uint32_t>(kMaxExpected)) {
            status |= kTooManyCodes;
            continue;
        }
        max_exp = max(max_exp, max(2u, k));
        const uint32_t kk = k == 0 ? 1u : k;
        for (uint32_t j = 0; j < kk; ++j) {
            const unsigned long long c = k ? r.codes[b + j] : 0ull;
            unsigned long long delta = static_cast<unsigned long long>(d) + c;
            if (delta < 1) delta = 1;
            if (delta >= kMaxDelta) {
                status |= kDelayTooLong;
            } else {
                present[delta] = 1;
            }
        }
        events += kk;
        atomicAdd(in_cnt + tgt, 1ull);
        atomicAdd(out_cnt + src, 1ull);
    }
    if (status) atomicOr(&sc->status, status);
    atomicMax(&sc->max_expected, max_exp);
    if (events) atomicAdd(&sc->pre_total, events);
}

__global__ void k_iota(uint32_t* v, unsigned long long n) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
        v[i] = static_cast<uint32_t>(i);
}

__global__ void k_invert(const uint32_t* perm, uint32_t* inv, unsigned long long n) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
        inv[perm[i]] = static_cast<uint32_t>(i);
}

// SynapseDendriteProcessor::initialize_synapse (:59-75) into the 64-byte
// record at the synapse's target-major slot.
__global__ void k_pack_records(Raw r, const uint32_t* tm_of_c, SynAB* syn, float cfg_max_weight) {
    for (unsigned long long s = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; s < r.S;
         s += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        unsigned long long b;
        uint32_t k;
        code_list(r, s, b, k);
        const uint32_t expected = max(2u, k == 0 ? 1u : k);
        SynAB x;
        x.a.weight = r.weight[s];
        x.a.last_pre1 = 0;
        x.a.last_post1 = 0;
        x.a.meta = r.delay[s] | (static_cast<uint32_t>(r.comp[s]) << kMetaCompShift) |
                   (static_cast<uint32_t>(r.rec[s]) << kMetaRecShift) |
                   (static_cast<uint32_t>(r.plastic[s] ? 1 : 0) << kMetaPlasticBit) | (expected << kMetaExpectedShift);
        // std::min(config.max_weight, synapse.max_weight) (STDP.cpp:38)
        const float mw = r.max_weight[s];
        x.a.clamp_hi = mw < cfg_max_weight ? mw : cfg_max_weight;
        x.a.updates = 0;
        x.a.last_delta = 0.0f;
        x.a.post_cnt = 0;
        x.b = SynB{};
        x.b.flags = static_cast<uint8_t>(expected << 4);
        syn[tm_of_c[s]] = x;
    }
}

// Per source: events per delay class (row of D + 1 exclusive offsets).
__global__ void k_pack_class_rows(Raw r, const unsigned long long* out_ptr, const uint32_t* out_list,
                                  const uint8_t* class_of, uint32_t D, uint32_t* pre_off, unsigned long long* tot,
                                  Scratch* sc) {
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < r.N; n += gridDim.x * blockDim.x) {
        uint32_t* row = pre_off + static_cast<size_t>(n) * (D + 1);
        for (uint32_t d = 0; d <= D; ++d) row[d] = 0;
        for (unsigned long long i = out_ptr[n]; i < out_ptr[n + 1]; ++i) {
            const uint32_t s = out_list[i];
            unsigned long long b;
            uint32_t k;
            code_list(r, s, b, k);
            const uint32_t kk = k == 0 ? 1u : k;
            for (uint32_t j = 0; j < kk; ++j) {
                const unsigned long long c = k ? r.codes[b + j] : 0ull;
                unsigned long long delta = static_cast<unsigned long long>(r.delay[s]) + c;
                if (delta < 1) delta = 1;
                row[class_of[delta] + 1] += 1;
            }
        }
        unsigned long long acc = 0;
        for (uint32_t d = 1; d <= D; ++d) {
            acc += row[d];
            row[d] = static_cast<uint32_t>(acc < 0xFFFFFFFFull ? acc : 0xFFFFFFFFull);
        }
        if (acc >= (1ull << 30)) atomicOr(&sc->status, kTooManyEvents);
        tot[n] = acc;
    }
}

// Per source: its events in Connectome x offset order within each class.
__global__ void k_pack_events(Raw r, const unsigned long long* out_ptr, const uint32_t* out_list,
                              const uint8_t* class_of, uint32_t D, const uint32_t* pre_off,
                              const unsigned long long* pre_base, uint32_t* cursor, const uint32_t* tm_of_c,
                              unsigned long long* pre_ev) {
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < r.N; n += gridDim.x * blockDim.x) {
        const uint32_t* row = pre_off + static_cast<size_t>(n) * (D + 1);
        uint32_t* cur = cursor + static_cast<size_t>(n) * D;
        for (uint32_t d = 0; d < D; ++d) cur[d] = row[d];
        unsigned long long* dst = pre_ev + pre_base[n];
        for (unsigned long long i = out_ptr[n]; i < out_ptr[n + 1]; ++i) {
            const uint32_t s = out_list[i];
            unsigned long long b;
            uint32_t k;
            code_list(r, s, b, k);
            const uint32_t kk = k == 0 ? 1u : k;
            const unsigned long long word = (static_cast<unsigned long long>(tm_of_c[s]) << 32) | r.target[s];
            for (uint32_t j = 0; j < kk; ++j) {
                const unsigned long long c = k ? r.codes[b + j] : 0ull;
                unsigned long long delta = static_cast<unsigned long long>(r.delay[s]) + c;
                if (delta < 1) delta = 1;
                dst[cur[class_of[delta]]++] = word;
            }
        }
    }
}

int bits_for(unsigned long long n) {
    int b = 1;
    while (b < 32 && (1ull << b) < n) ++b;
    return b;
}

// Stream-ordered temporary buffers, released at scope end.
struct Temp {
    cudaStream_t st;
    std::vector<void*> v;
    explicit Temp(cudaStream_t s) : st(s) {}
    ~Temp() {
        for (void* p : v) cudaFreeAsync(p, st);
    }
    template <typename T>
    T* get(size_t count, const char*& err) {
        void* p = nullptr;
        if (count == 0) count = 1;
        if (cudaMallocAsync(&p, count * sizeof(T), st) != cudaSuccess) {
            err = "device memory exhausted while packing the network";
            return nullptr;
        }
        v.push_back(p);
        return static_cast<T*>(p);
    }
};

uint32_t grid_for(unsigned long long n) {
    const unsigned long long b = (n + kPackThreads - 1) / kPackThreads;
    return static_cast<uint32_t>(std::max<unsigned long long>(1, std::min<unsigned long long>(b, 65535ull * 8)));
}

}  // namespace

int pack_network_device(const snncuda_network* net, float cfg_max_weight, cudaStream_t st,
                        DeviceBuffers& owned, PackOut& out, std::string& msg) {
    const uint32_t N = net->neuron_count;
    const unsigned long long S = net->synapse_count;
    if (S >= (1ull << 31)) {
        msg = "at most 2^31-1 synapses per simulation";
        return SNNCUDA_ERR_UNSUPPORTED;
    }
    const bool has_codes = net->code_offset_ptr != nullptr && net->code_offsets != nullptr;
    const char* err = nullptr;
    auto fail = [&](int code, const std::string& m) {
        msg = m;
        return code;
    };
    auto ok = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess) {
            msg = std::string(what) + ": " + cudaGetErrorString(e);
            return false;
        }
        return true;
    };
    auto persist = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMallocAsync(&p, bytes ? bytes : 1, st) != cudaSuccess) return nullptr;
        owned.push_back({p, bytes ? bytes : 1, BufKind::kState});
        return p;
    };

    Temp tmp(st);
    // ---- raw arrays to the device ----
    Raw r{};
    r.N = N;
    r.S = S;
    auto up = [&](const void* src, size_t bytes) -> void* {
        void* d = tmp.get<unsigned char>(bytes, err);
        if (d && bytes) {
            if (cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) return nullptr;
        }
        return d;
    };
    unsigned long long codes_total = 0;
    if (has_codes) codes_total = net->code_offset_ptr[S];
    r.source = static_cast<const uint32_t*>(up(net->source, S * 4));
    r.target = static_cast<const uint32_t*>(up(net->target, S * 4));
    r.weight = static_cast<const float*>(up(net->weight, S * 4));
    r.max_weight = static_cast<const float*>(up(net->max_weight, S * 4));
    r.delay = static_cast<const uint32_t*>(up(net->delay_ticks, S * 4));
    r.comp = static_cast<const uint8_t*>(up(net->compartment, S));
    r.rec = static_cast<const uint8_t*>(up(net->receptor, S));
    r.plastic = static_cast<const uint8_t*>(up(net->plasticity_enabled, S));
    if (has_codes) {
        r.cptr = static_cast<const unsigned long long*>(up(net->code_offset_ptr, (S + 1) * 8));
        r.codes = static_cast<const uint32_t*>(up(net->code_offsets, codes_total * 4));
    }
    if (!r.source || !r.target || !r.weight || !r.max_weight || !r.delay || !r.comp || !r.rec || !r.plastic ||
        (has_codes && (!r.cptr || !r.codes)))
        return fail(SNNCUDA_ERR_OUT_OF_MEMORY, err ? err : "copy of the synapse arrays failed");

    // ---- validation and counts ----
    Scratch* sc = tmp.get<Scratch>(1, err);
    unsigned long long* in_cnt = tmp.get<unsigned long long>(static_cast<size_t>(N) + 1, err);
    unsigned long long* out_cnt = tmp.get<unsigned long long>(static_cast<size_t>(N) + 1, err);
    uint8_t* present = tmp.get<uint8_t>(kMaxDelta, err);
    if (!sc || !in_cnt || !out_cnt || !present) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, err);
    Scratch init{0u, 2u, 0ull};
    if (!ok(cudaMemcpyAsync(sc, &init, sizeof(init), cudaMemcpyHostToDevice, st), "copy") ||
        !ok(cudaMemsetAsync(in_cnt, 0, (static_cast<size_t>(N) + 1) * 8, st), "memset") ||
        !ok(cudaMemsetAsync(out_cnt, 0, (static_cast<size_t>(N) + 1) * 8, st), "memset") ||
        !ok(cudaMemsetAsync(present, 0, kMaxDelta, st), "memset"))
        return SNNCUDA_ERR_DEVICE;
    if (S > 0) k_pack_scan<<<grid_for(S), kPackThreads, 0, st>>>(r, sc, in_cnt, out_cnt, present);
    Scratch h{};
    std::vector<uint8_t> pres(kMaxDelta);
    if (!ok(cudaGetLastError(), "pack launch") ||
        !ok(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaMemcpyAsync(pres.data(), present, kMaxDelta, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaStreamSynchronize(st), "pack synchronize"))
        return SNNCUDA_ERR_DEVICE;
    if (h.status & kBadEndpoint) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse endpoint out of range");
    if (h.status & kBadCompartment) return fail(SNNCUDA_ERR_INVALID_ARGUMENT, "compartment/receptor out of range");
    if (h.status & kBadDelay) return fail(SNNCUDA_ERR_UNSUPPORTED, "delays above 65535 ticks are not supported");
    if (h.status & kTooManyCodes) return fail(SNNCUDA_ERR_UNSUPPORTED, "more than 8 spike-code offsets per synapse");
    if (h.status & kDelayTooLong) return fail(SNNCUDA_ERR_UNSUPPORTED, "delivery delays above 2^20 ticks");
    out.max_expected = h.max_expected;
    out.pre_total = h.pre_total;

    // ---- delay classes ----
    out.cls_delta.clear();
    std::vector<uint8_t> class_of_h(kMaxDelta, 0);
    for (uint32_t d = 1; d < kMaxDelta; ++d)
        if (pres[d]) {
            if (out.cls_delta.size() >= kMaxClasses) return fail(SNNCUDA_ERR_UNSUPPORTED, "more than 256 distinct delivery delays");
            class_of_h[d] = static_cast<uint8_t>(out.cls_delta.size());
            out.cls_delta.push_back(d);
        }
    const uint32_t D = static_cast<uint32_t>(out.cls_delta.size());
    uint8_t* class_of = static_cast<uint8_t*>(up(class_of_h.data(), kMaxDelta));
    if (!class_of) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, err);

    // ---- row pointers ----
    out.in_ptr_d = static_cast<unsigned long long*>(persist((static_cast<size_t>(N) + 1) * 8));
    unsigned long long* out_ptr = tmp.get<unsigned long long>(static_cast<size_t>(N) + 1, err);
    if (!out.in_ptr_d || !out_ptr) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, "device memory exhausted");
    {
        size_t bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, bytes, in_cnt, out.in_ptr_d, static_cast<int>(N) + 1, st);
        void* t = tmp.get<unsigned char>(bytes, err);
        if (!t) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, err);
        cub::DeviceScan::ExclusiveSum(t, bytes, in_cnt, out.in_ptr_d, static_cast<int>(N) + 1, st);
        cub::DeviceScan::ExclusiveSum(t, bytes, out_cnt, out_ptr, static_cast<int>(N) + 1, st);
    }

    // ---- target-major order and source order (stable radix sorts) ----
    out.c_of_tm_d = static_cast<uint32_t*>(persist(S * 4));
    out.tm_of_c_d = static_cast<uint32_t*>(persist(S * 4));
    uint32_t* iota = tmp.get<uint32_t>(S, err);
    uint32_t* keys_sorted = tmp.get<uint32_t>(S, err);
    uint32_t* out_list = tmp.get<uint32_t>(S, err);
    if (!out.c_of_tm_d || !out.tm_of_c_d || !iota || !keys_sorted || !out_list)
        return fail(SNNCUDA_ERR_OUT_OF_MEMORY, "device memory exhausted");
    if (S > 0) {
        k_iota<<<grid_for(S), kPackThreads, 0, st>>>(iota, S);
        const int bits = bits_for(N);
        size_t bytes = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, bytes, r.target, keys_sorted, iota, out.c_of_tm_d,
                                        static_cast<int>(S), 0, bits, st);
        void* t = tmp.get<unsigned char>(bytes, err);
        if (!t) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, err);
        cub::DeviceRadixSort::SortPairs(t, bytes, r.target, keys_sorted, iota, out.c_of_tm_d, static_cast<int>(S), 0,
                                        bits, st);
        cub::DeviceRadixSort::SortPairs(t, bytes, r.source, keys_sorted, iota, out_list, static_cast<int>(S), 0,
                                        bits, st);
        k_invert<<<grid_for(S), kPackThreads, 0, st>>>(out.c_of_tm_d, out.tm_of_c_d, S);
    }

    // ---- synapse records ----
    out.syn = static_cast<SynAB*>(persist(S * sizeof(SynAB)));
    if (!out.syn) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, "device memory exhausted");
    if (S > 0) k_pack_records<<<grid_for(S), kPackThreads, 0, st>>>(r, out.tm_of_c_d, out.syn, cfg_max_weight);

    // ---- pre-expanded outgoing events ----
    out.pre_off = static_cast<uint32_t*>(persist(static_cast<size_t>(N) * (D + 1) * 4));
    out.pre_base = static_cast<unsigned long long*>(persist(static_cast<size_t>(N) * 8));
    out.pre_ev = static_cast<unsigned long long*>(persist(std::max<unsigned long long>(out.pre_total, 1) * 8));
    unsigned long long* tot = tmp.get<unsigned long long>(N, err);
    uint32_t* cursor = tmp.get<uint32_t>(static_cast<size_t>(N) * std::max<uint32_t>(D, 1), err);
    if (!out.pre_off || !out.pre_base || !out.pre_ev || !tot || !cursor)
        return fail(SNNCUDA_ERR_OUT_OF_MEMORY, "device memory exhausted");
    if (N > 0) {
        k_pack_class_rows<<<grid_for(N), kPackThreads, 0, st>>>(r, out_ptr, out_list, class_of, D, out.pre_off, tot,
                                                                  sc);
        size_t bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, bytes, tot, out.pre_base, static_cast<int>(N), st);
        void* t = tmp.get<unsigned char>(bytes, err);
        if (!t) return fail(SNNCUDA_ERR_OUT_OF_MEMORY, err);
        cub::DeviceScan::ExclusiveSum(t, bytes, tot, out.pre_base, static_cast<int>(N), st);
        k_pack_events<<<grid_for(N), kPackThreads, 0, st>>>(r, out_ptr, out_list, class_of, D, out.pre_off,
                                                              out.pre_base, cursor, out.tm_of_c_d, out.pre_ev);
    }
    out.in_ptr.assign(static_cast<size_t>(N) + 1, 0);
    if (!ok(cudaGetLastError(), "pack launch") ||
        !ok(cudaMemcpyAsync(out.in_ptr.data(), out.in_ptr_d, (static_cast<size_t>(N) + 1) * 8,
                            cudaMemcpyDeviceToHost, st),
            "copy") ||
        !ok(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaStreamSynchronize(st), "pack synchronize"))
        return SNNCUDA_ERR_DEVICE;
    if (h.status & kTooManyEvents) return fail(SNNCUDA_ERR_UNSUPPORTED, "too many outgoing events per neuron");
    return SNNCUDA_OK;
}

}  // namespace snngb
