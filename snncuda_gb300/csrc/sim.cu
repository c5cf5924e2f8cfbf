// Host side of the GB300 engine: the C ABI of include/snncuda_gb300.h.
//
// create    packs a flattened Connectome into the device layout of engine.h
//           (replaces NetworkPropagator's constructor, NetworkPropagator.cpp:5-29
//           and SynapseDendriteProcessor::initialize_synapse, :59-75)
// inject    queues external inputs in call order (NetworkPropagator.cpp:31-37)
// run_until places due injections into the wheel and replays a CUDA graph of
//           the tick kernels once per tick (NetworkPropagator.cpp:39-43)
// readers   copy state back and present it with the reference field meaning.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <chrono>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <type_traits>
#include <condition_variable>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"
#include "pack.h"
#include "snncuda_gb300.h"

using namespace snngb;

namespace {

thread_local std::string g_last_error;

struct Failure {
    int code;
    std::string message;
};

[[noreturn]] void throw_fail(int code, const std::string& msg) { throw Failure{code, msg}; }

void check(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return;
    if (err == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        throw_fail(SNNCUDA_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(err));
    }
    throw_fail(SNNCUDA_ERR_DEVICE, std::string(what) + ": " + cudaGetErrorString(err));
}

int set_error(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

}  // namespace

void snngb::set_last_error_message(const std::string& msg) { g_last_error = msg; }

namespace {

constexpr float kTauValue[4] = {5.0F, 100.0F, 10.0F, 150.0F};  // receptor_decay_tau (:245-257)

// exp table entries e = 0.. until std::exp(-e / tau) is 0 for every tau,
// built with the host libm exactly as the reference evaluates
// static_cast<float>(current * std::exp(-elapsed / tau)) (:220-221).
std::vector<float> build_decay_table(uint32_t& len) {
    uint32_t n = 1;
    for (float tau : kTauValue) {
        uint32_t e = 1;
        while (std::exp(-static_cast<float>(e) / tau) != 0.0F) ++e;
        n = std::max(n, e + 1);
    }
    len = n;
    std::vector<float> t(4u * n);
    for (int k = 0; k < 4; ++k)
        for (uint32_t e = 0; e < n; ++e) t[k * n + e] = std::exp(-static_cast<float>(e) / kTauValue[k]);
    return t;
}

// StdpRule::weight_delta (STDP.cpp:25-34) per |post - pre|, until the
// exponential is 0; the last entry is the value for every larger distance.
void build_stdp_tables(const snncuda_config& c, std::vector<float>& ltp, std::vector<float>& ltd) {
    constexpr uint32_t kMax = 1u << 22;
    uint32_t n = 2;
    auto zero_at = [](float tau) {
        uint32_t m = 1;
        while (m < kMax && std::exp(-static_cast<float>(m) / tau) != 0.0F) ++m;
        return m;
    };
    n = std::max({n, zero_at(c.ltp_tau_ticks) + 1, zero_at(c.ltd_tau_ticks) + 1});
    if (n > kMax)
        throw_fail(SNNCUDA_ERR_UNSUPPORTED, "STDP time constant too large for the delta tables");
    ltp.assign(n, 0.0F);
    ltd.assign(n, 0.0F);
    for (uint32_t m = 1; m < n; ++m) {
        const float dt = static_cast<float>(m);
        ltp[m] = c.ltp_amplitude * std::exp(-dt / c.ltp_tau_ticks);
        ltd[m] = -c.ltd_amplitude * std::exp(-dt / c.ltd_tau_ticks);
    }
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

struct Pending {
    uint64_t tick;  // clamped delivery
    uint64_t event;
    // left uninitialised by resize(): the queue's new entries are written in
    // parallel right after
    Pending() {}
    Pending(uint64_t t, uint64_t ev) : tick(t), event(ev) {}
};

// f(begin, end) over [0, n) in contiguous chunks on up to 16 host threads
// (the calling thread takes the first chunk); serial below 2^20 items.  The
// injection queue's passes (a drive of millions of injections per call) are
// memory-bound loops that one host thread runs at a fraction of the host's
// bandwidth.
template <typename F>
void parallel_for(size_t n, F&& f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t threads = n < (size_t{1} << 20) ? 1 : std::min<size_t>({size_t{16}, hw, n >> 18});
    if (threads <= 1) {
        f(size_t{0}, n);
        return;
    }
    std::vector<std::thread> pool;
    const size_t chunk = (n + threads - 1) / threads;
    size_t t = 1;
    try {
        pool.reserve(threads - 1);
        for (; t < threads; ++t) {
            const size_t b = std::min(n, t * chunk), en = std::min(n, b + chunk);
            pool.emplace_back([&f, b, en] { f(b, en); });
        }
    } catch (...) {
        // a thread that could not start: its chunks run here
    }
    f(size_t{0}, std::min(n, chunk));
    for (; t < threads; ++t) f(std::min(n, t * chunk), std::min(n, std::min(n, t * chunk) + chunk));
    for (std::thread& th : pool) th.join();
}

template <typename T>
T* dalloc(std::vector<void*>& owned, size_t count) {
    void* p = nullptr;
    if (count == 0) count = 1;
    check(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
    owned.push_back(p);
    return static_cast<T*>(p);
}

}  // namespace

struct snncuda_sim {
    Engine e{};
    DeviceBuffers owned;
    cudaStream_t stream{nullptr};
    bool own_stream{false};
    snncuda_config config{};
    uint32_t N{0};
    uint64_t S{0};
    uint64_t next_tick{0};
    bool poisoned{false};
    int device{0};
    std::vector<uint32_t> c_of_tm;     // Connectome index of each target-major slot
    std::vector<uint32_t> tm_of_c;     // target-major slot of each Connectome index
    std::vector<uint64_t> in_ptr;      // host copy of the row pointers
    std::vector<NeuronParam> nparam;   // host copy
    std::vector<Pending> pending;      // queued injections; [pend_head, pend_sorted) sorted by tick
    size_t pend_head{0};
    size_t pend_sorted{0};
    // far-future buffers (stable addresses while a graph uses them)
    unsigned long long* far_ev{nullptr};
    uint32_t* far_idx{nullptr};
    size_t far_ev_cap{0}, far_idx_cap{0};
    // pinned host staging for injected events and their slot/tick indices
    unsigned long long* host_ev{nullptr};
    uint32_t* host_idx{nullptr};
    size_t host_ev_cap{0}, host_idx_cap{0};
    // injection staging
    unsigned long long* inj_ev{nullptr};
    uint32_t* inj_slot{nullptr};
    uint32_t* inj_off{nullptr};
    size_t inj_cap{0}, inj_groups_cap{0};
    // graphs
    cudaGraphExec_t graph_many{nullptr};
    cudaGraphExec_t graph_one{nullptr};
    cudaGraphExec_t graph_prof{nullptr};
    cudaEvent_t marks[2 * kKernelCount]{};
    uint32_t ticks_per_graph{16};  // ticks captured in graph_many
    uint32_t sms{1};

    // second stream of the tick graphs (k_temporal) and its fork/join events
    cudaStream_t side{nullptr};
    cudaEvent_t tick_ev[4]{};
    // eviction: the device state held in host memory (evict_impl / restore_impl)
    bool evicted{false};
    std::vector<std::vector<unsigned char>> evicted_data;  // per owned buffer
    uint64_t evictions{0};
    // asynchronous runs (run_enqueue / run_complete)
    TickState* ts_pinned{nullptr};  // tick state copied back at the end of a run
    cudaEvent_t run_done{nullptr};
    uint64_t run_target{0};         // inclusive tick of the run in flight
    bool run_in_flight{false};

    ~snncuda_sim() {
        if (run_done) cudaEventDestroy(run_done);
        for (cudaEvent_t ev : tick_ev)
            if (ev) cudaEventDestroy(ev);
        if (ts_pinned) cudaFreeHost(ts_pinned);
        if (graph_many) cudaGraphExecDestroy(graph_many);
        if (graph_one) cudaGraphExecDestroy(graph_one);
        if (graph_prof) cudaGraphExecDestroy(graph_prof);
        for (cudaEvent_t ev : marks)
            if (ev) cudaEventDestroy(ev);
        // device buffers are stream-ordered: freeing them does not stall
        // other streams (a server runs many simulations side by side)
        if (stream) cudaStreamSynchronize(stream);
        if (!evicted)  // an evicted simulation's buffers are already freed
            for (const DeviceBuffer& b : owned)
                if (b.p) cudaFreeAsync(b.p, stream);
        if (far_ev) cudaFreeAsync(far_ev, stream);
        if (far_idx) cudaFreeAsync(far_idx, stream);
        if (inj_ev) cudaFreeAsync(inj_ev, stream);
        if (inj_slot) cudaFreeAsync(inj_slot, stream);
        if (inj_off) cudaFreeAsync(inj_off, stream);
        if (host_ev) cudaFreeHost(host_ev);
        if (host_idx) cudaFreeHost(host_idx);
        if (side) cudaStreamDestroy(side);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    // Pinned host buffers for the host->device copies of injected events.
    void ensure_host(size_t events, size_t idx) {
        if (events > host_ev_cap) {
            if (host_ev) cudaFreeHost(host_ev);
            host_ev = nullptr;
            host_ev_cap = std::max<size_t>(events, 2 * host_ev_cap);
            check(cudaMallocHost(&host_ev, host_ev_cap * sizeof(unsigned long long)), "pinned staging");
        }
        if (idx > host_idx_cap) {
            if (host_idx) cudaFreeHost(host_idx);
            host_idx = nullptr;
            host_idx_cap = std::max<size_t>(idx, 2 * host_idx_cap);
            check(cudaMallocHost(&host_idx, host_idx_cap * sizeof(uint32_t)), "pinned staging");
        }
    }

    void drop_graphs() {
        if (graph_many) cudaGraphExecDestroy(graph_many);
        if (graph_one) cudaGraphExecDestroy(graph_one);
        if (graph_prof) cudaGraphExecDestroy(graph_prof);
        graph_many = graph_one = graph_prof = nullptr;
    }

    cudaGraphExec_t capture(int ticks, bool profiled = false) {
        cudaGraph_t g = nullptr;
        if (profiled && marks[0] == nullptr)
            for (cudaEvent_t& ev : marks) check(cudaEventCreate(&ev), "event");
        check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        const TickStreams ts{stream, side, {tick_ev[0], tick_ev[1], tick_ev[2], tick_ev[3]}};
        for (int i = 0; i < ticks; ++i) launch_tick(e, ts, profiled ? marks : nullptr);
        check(cudaStreamEndCapture(stream, &g), "end capture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t err = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        check(err, "graph instantiate");
        return exec;
    }

    void ensure_far(size_t events, size_t idx) {
        if (events > far_ev_cap) {
            if (far_ev) cudaFreeAsync(far_ev, stream);
            far_ev = nullptr;
            far_ev_cap = std::max<size_t>(events, 2 * far_ev_cap);
            check(cudaMallocAsync(&far_ev, far_ev_cap * sizeof(unsigned long long), stream), "far events");
            drop_graphs();
        }
        if (idx > far_idx_cap) {
            if (far_idx) cudaFreeAsync(far_idx, stream);
            far_idx = nullptr;
            far_idx_cap = std::max<size_t>(idx, 2 * far_idx_cap);
            check(cudaMallocAsync(&far_idx, far_idx_cap * sizeof(uint32_t), stream), "far index");
            drop_graphs();
        }
        e.far_ev = far_ev;
        e.far_idx = far_idx;
    }

    void ensure_inject(size_t events, size_t groups) {
        if (events > inj_cap) {
            if (inj_ev) cudaFreeAsync(inj_ev, stream);
            inj_ev = nullptr;
            inj_cap = std::max<size_t>(events, 2 * inj_cap);
            check(cudaMallocAsync(&inj_ev, inj_cap * sizeof(unsigned long long), stream), "inject events");
        }
        if (groups + 1 > inj_groups_cap) {
            if (inj_slot) cudaFreeAsync(inj_slot, stream);
            if (inj_off) cudaFreeAsync(inj_off, stream);
            inj_slot = nullptr;
            inj_off = nullptr;
            inj_groups_cap = std::max<size_t>(groups + 1, 2 * inj_groups_cap);
            check(cudaMallocAsync(&inj_slot, inj_groups_cap * sizeof(uint32_t), stream), "inject slots");
            check(cudaMallocAsync(&inj_off, inj_groups_cap * sizeof(uint32_t), stream), "inject offsets");
        }
    }

    TickState read_ts() {
        TickState ts;
        check(cudaMemcpyAsync(&ts, e.ts, sizeof(ts), cudaMemcpyDeviceToHost, stream), "read tick state");
        check(cudaStreamSynchronize(stream), "synchronize");
        return ts;
    }

    template <typename T>
    std::vector<T> d2h(const T* src, size_t count) {
        std::vector<T> v(count);
        if (count) {
            check(cudaMemcpyAsync(v.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost, stream), "copy back");
            check(cudaStreamSynchronize(stream), "synchronize");
        }
        return v;
    }
};

namespace {

// A persistent device buffer of the simulation, stream-ordered on its
// stream; `kind` says what an eviction keeps of it.
template <typename T>
T* salloc(snncuda_sim* sim, size_t count, BufKind kind = BufKind::kState) {
    void* p = nullptr;
    if (count == 0) count = 1;
    check(cudaMallocAsync(&p, count * sizeof(T), sim->stream), "device allocation");
    sim->owned.push_back({p, count * sizeof(T), kind});
    return static_cast<T*>(p);
}

void create_impl(const snncuda_network* net, const snncuda_config& cfg, snncuda_sim* sim) {
    const uint32_t N = net->neuron_count;
    const uint64_t S = net->synapse_count;
    if (cfg.timing_wheel_slots == 0)
        throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "Spike scheduler timing wheel must have at least one slot");
    if (N >= (1u << 31)) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "at most 2^31-1 neurons");
    if (S >= (1ull << 31)) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "at most 2^31-1 synapses per simulation");
    if (N > 0 && (!net->threshold || !net->pattern_window_ticks || !net->similarity_threshold ||
                  !net->max_reference_patterns))
        throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "neuron parameter arrays are required");
    if (S > 0 && (!net->source || !net->target || !net->weight || !net->max_weight || !net->delay_ticks ||
                  !net->compartment || !net->receptor || !net->plasticity_enabled))
        throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse arrays are required");

    check(cudaGetDevice(&sim->device), "cudaGetDevice");
    if (cfg.cuda_stream != nullptr) {
        sim->stream = static_cast<cudaStream_t>(cfg.cuda_stream);
    } else {
        check(cudaStreamCreateWithFlags(&sim->stream, cudaStreamNonBlocking), "stream");
        sim->own_stream = true;
    }
    check(cudaStreamCreateWithFlags(&sim->side, cudaStreamNonBlocking), "stream");
    for (cudaEvent_t& ev : sim->tick_ev) check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
    sim->N = N;
    sim->S = S;
    sim->config = cfg;
    Engine& e = sim->e;
    e.N = N;
    e.S = S;
    e.min_weight = cfg.min_weight;
    e.stage_wait_ns = cfg.stage_wait_ns;

    // ---- synapse side, packed on the device: validation, target-major
    // order, synapse records, pre-expanded outgoing events ----
    PackOut pk;
    {
        std::string msg;
        const int rc = pack_network_device(net, cfg.max_weight, sim->stream, sim->owned, pk, msg);
        if (rc != SNNCUDA_OK) throw_fail(rc, msg);
    }
    std::vector<uint64_t>& in_ptr = pk.in_ptr;
    const uint32_t max_expected = pk.max_expected;
    e.code_stride = max_expected;
    sim->c_of_tm.resize(S);
    sim->tm_of_c.resize(S);
    if (S > 0) {
        check(cudaMemcpyAsync(sim->c_of_tm.data(), pk.c_of_tm_d, S * 4, cudaMemcpyDeviceToHost, sim->stream), "copy");
        check(cudaMemcpyAsync(sim->tm_of_c.data(), pk.tm_of_c_d, S * 4, cudaMemcpyDeviceToHost, sim->stream), "copy");
    }
    // the synapse order maps live on the host from here on
    for (DeviceBuffer& b : sim->owned) {
        if (b.p == pk.c_of_tm_d || b.p == pk.tm_of_c_d) {
            check(cudaFreeAsync(b.p, sim->stream), "free");
            b.p = nullptr;
            b.bytes = 0;
        }
    }

    // ---- neuron parameters and temporal storage ----
    sim->nparam.resize(N);
    uint64_t cand_total = 0, meta_total = 0, ring_total = 0, lcode_total = 0;
    const uint64_t run_budget = cfg.pattern_run_capacity ? cfg.pattern_run_capacity : 4096;
    for (uint32_t n = 0; n < N; ++n) {
        NeuronParam& p = sim->nparam[n];
        std::memset(&p, 0, sizeof(p));
        const uint64_t window = net->pattern_window_ticks[n];
        const uint64_t refs = net->max_reference_patterns[n];
        if (refs == 0) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "max_reference_patterns must be >= 1");
        if (window > 0xFFFE) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "pattern windows above 65534 ticks");
        if (refs > 0xFFFF) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "more than 65535 reference patterns");
        p.threshold = net->threshold[n];
        p.window = static_cast<uint32_t>(window);
        p.similarity = net->similarity_threshold[n];
        p.max_refs = static_cast<uint32_t>(refs);
        const uint64_t full = refs * (window + 1);
        p.ring_cap = static_cast<uint32_t>(std::min<uint64_t>(full, std::max<uint64_t>(window + 1, run_budget)));
        p.in_begin = in_ptr[n];
        p.cand_base = cand_total;
        cand_total += window + 1;
        p.meta_base = meta_total;
        meta_total += refs;
        p.ring_base = ring_total;
        ring_total += p.ring_cap;
        p.lcode_base = lcode_total;
        if (!inline_code_pattern(p.max_refs, max_expected))
            lcode_total += (in_ptr[n + 1] - in_ptr[n]) * refs * max_expected;
    }

    // ---- delivery delay classes and the wheel ----
    const std::vector<uint32_t>& cls_delta = pk.cls_delta;
    const uint32_t D = static_cast<uint32_t>(cls_delta.size());
    const uint64_t pre_total = pk.pre_total;
    const uint64_t max_delta = cls_delta.empty() ? 1 : cls_delta.back();
    uint32_t W = 2;
    while (W <= max_delta) W <<= 1;
    if (W > (1u << 20)) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "delivery delays above 2^20 ticks");
    e.W = W;
    e.wmask = W - 1;
    e.D = D;

    // ---- capacities ----
    uint64_t slot_cap = cfg.slot_event_capacity;
    if (slot_cap == 0) slot_cap = std::min<uint64_t>(1ull << 27, std::max<uint64_t>(1ull << 16, pre_total / 8));
    if (slot_cap >= (1ull << 31)) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "slot capacity must be below 2^31");
    slot_cap = (slot_cap + 31) & ~31ull;
    e.slot_cap = slot_cap;
    const uint64_t fire_cap = std::min<uint64_t>(slot_cap, std::max<uint64_t>(65536, 4ull * N));
    e.fire_cap = static_cast<uint32_t>(fire_cap);
    e.raster_cap = cfg.raster_capacity;
    const uint64_t xblocks = (fire_cap + kExpandFires - 1) / kExpandFires;
    const uint64_t bit_words = slot_cap / 32;
    const uint64_t fire_tiles = (bit_words + 255) / 256;
    e.fire_tiles_cap = static_cast<uint32_t>(fire_tiles);

    // ---- grouping buckets and launch shapes ----
    int sms = 0;
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sim->device), "device attribute");
    e.bucket_shift = bucket_shift_for(N);
    if (e.bucket_shift == 0) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "at most 2^28 neurons");
    e.nbuckets = static_cast<uint32_t>(std::max<uint64_t>(1, (static_cast<uint64_t>(N) + (1u << e.bucket_shift) - 1) >> e.bucket_shift));
    // counting and placing blocks: two per SM, fewer for small networks (one
    // per 2^18 synapses), whose grids then leave room for other streams'
    // kernels (side-by-side jobs of a server)
    e.grid_bucket = static_cast<uint32_t>(
        std::max<uint64_t>(1, std::min<uint64_t>(sms * 2ull, (static_cast<uint64_t>(sim->S) + (1u << 18) - 1) >> 18)));
    e.scatter_pass_events = kScatterPassEvents;
    const uint32_t grid_bucket_max = static_cast<uint32_t>(std::max(1, sms * 4));  // the autotuner's largest

    // ---- tables ----
    uint32_t decay_len = 0;
    const std::vector<float> decay = build_decay_table(decay_len);
    std::vector<float> ltp, ltd;
    build_stdp_tables(cfg, ltp, ltd);

    // ---- device allocation ----
    auto* d_nparam = salloc<NeuronParam>(sim, N);
    e.nrec = salloc<NeuronRec>(sim, N);
    e.ntp = salloc<NeuronTp>(sim, N);
    e.cand = salloc<unsigned long long>(sim, cand_total);
    e.refmeta = salloc<RefMeta>(sim, meta_total);
    e.ring = salloc<unsigned long long>(sim, ring_total);
    e.lcode = salloc<uint16_t>(sim, lcode_total);
    auto* d_cls = salloc<uint32_t>(sim, D);
    e.wheel = salloc<unsigned long long>(sim, static_cast<size_t>(W) * slot_cap, BufKind::kWheel);
    e.slot_count = salloc<uint32_t>(sim, W);
    e.seg_start = salloc<uint32_t>(sim, static_cast<size_t>(N) + 1, BufKind::kScratch);
    e.bcnt = salloc<uint32_t>(sim, static_cast<size_t>(grid_bucket_max) * e.nbuckets, BufKind::kScratch);
    e.btot = salloc<uint32_t>(sim, e.nbuckets, BufKind::kZero);
    e.bstart = salloc<uint32_t>(sim, static_cast<size_t>(e.nbuckets) + 1, BufKind::kScratch);
    e.bcur = salloc<uint32_t>(sim, e.nbuckets, BufKind::kZero);
    e.grp = salloc<unsigned long long>(sim, slot_cap, BufKind::kScratch);
    e.grp_tmp = salloc<BucketEntry>(sim, slot_cap, BufKind::kScratch);
    e.evin = salloc<EvIn>(sim, slot_cap, BufKind::kScratch);
    e.ev_a0 = salloc<SynPre>(sim, slot_cap, BufKind::kScratch);
    e.fire_bits = salloc<uint32_t>(sim, bit_words, BufKind::kZero);
    e.fire_at = salloc<uint32_t>(sim, slot_cap, BufKind::kScratch);
    e.fire_tile = salloc<uint32_t>(sim, fire_tiles + 2, BufKind::kZero);
    e.fire_list = salloc<uint32_t>(sim, fire_cap, BufKind::kScratch);
    e.fired_tgt = salloc<uint32_t>(sim, N, BufKind::kScratch);
    e.fired_cnt = salloc<uint32_t>(sim, N, BufKind::kScratch);
    e.xsum = salloc<uint32_t>(sim, xblocks * std::max<uint32_t>(D, 1), BufKind::kZero);
    e.xdst = salloc<unsigned long long>(sim, xblocks * std::max<uint32_t>(D, 1), BufKind::kScratch);
    e.xdst_ok = salloc<uint32_t>(sim, std::max<uint32_t>(D, 1));
    e.raster = salloc<uint32_t>(sim, cfg.raster_capacity > 0 ? 2 * cfg.raster_capacity : 1);
    e.ts = salloc<TickState>(sim, 1);
    auto* d_decay = salloc<float>(sim, decay.size());
    auto* d_ltp = salloc<float>(sim, ltp.size());
    auto* d_ltd = salloc<float>(sim, ltd.size());

    cudaStream_t st = sim->stream;
    auto h2d = [&](void* dst, const void* src, size_t bytes) {
        if (bytes) check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "copy to device");
    };
    auto zero = [&](void* dst, size_t bytes) {
        if (bytes) check(cudaMemsetAsync(dst, 0, bytes, st), "memset");
    };
    h2d(d_nparam, sim->nparam.data(), sim->nparam.size() * sizeof(NeuronParam));
    // NeuronState defaults (NeuronStateCache.h:15-45): every compartment tau 5 (code 0).
    zero(e.nrec, sizeof(NeuronRec) * N);
    zero(e.ntp, sizeof(NeuronTp) * N);
    zero(e.lcode, sizeof(uint16_t) * lcode_total);
    h2d(d_cls, cls_delta.data(), cls_delta.size() * sizeof(uint32_t));
    zero(e.slot_count, sizeof(uint32_t) * W);
    zero(e.btot, sizeof(uint32_t) * e.nbuckets);
    zero(e.bcur, sizeof(uint32_t) * e.nbuckets);
    zero(e.fire_bits, sizeof(uint32_t) * bit_words);
    zero(e.xsum, sizeof(uint32_t) * xblocks * std::max<uint32_t>(D, 1));
    zero(e.fire_tile, sizeof(uint32_t) * (fire_tiles + 2));
    h2d(d_decay, decay.data(), decay.size() * sizeof(float));
    h2d(d_ltp, ltp.data(), ltp.size() * sizeof(float));
    h2d(d_ltd, ltd.data(), ltd.size() * sizeof(float));
    TickState ts{};
    ts.stdp_enabled = cfg.stdp_enabled ? 1 : 0;
    ts.temporal_enabled = cfg.temporal_learning_enabled ? 1 : 0;
    h2d(e.ts, &ts, sizeof(ts));
    e.in_ptr = pk.in_ptr_d;
    e.nparam = d_nparam;
    e.syn = pk.syn;
    e.pre_base = pk.pre_base;
    e.pre_off = pk.pre_off;
    e.pre_ev = pk.pre_ev;
    e.cls_delta = d_cls;
    e.tab.decay = d_decay;
    e.tab.decay_len = decay_len;
    e.tab.ltp = d_ltp;
    e.tab.ltd = d_ltd;
    e.tab.stdp_len = static_cast<uint32_t>(ltp.size());
    configure_kernels();
    check(cudaGetLastError(), "init launch");
    sim->in_ptr = std::move(in_ptr);

    e.grid_wide = static_cast<uint32_t>(std::max(1, sms * 2));
    e.grid_events = e.grid_wide * 4;
    sim->sms = static_cast<uint32_t>(std::max(1, sms));
    e.grid_process = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>((N + 255) / 256, sms * 8ull)));
    // k_process: at least three blocks per SM (of at least 64 targets) so its
    // one wave covers every SM; at most eight per SM
    e.grid_walk = static_cast<uint32_t>(std::max<uint64_t>(
        1, std::min<uint64_t>(std::max<uint64_t>((N + 255) / 256, std::min<uint64_t>(sms * 3ull, (N + 63) / 64)),
                              sms * 8ull)));
    e.grid_fire = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>(fire_tiles, sms * 8ull)));
    // large networks: the temporal update and post-spike STDP in tick order
    // (beside k_events they slowed it by more than their own time on a 1e9-
    // synapse network, and by about their own time at 1e8 synapses; on a
    // 2e7-synapse network the overlap still gains 15 %)
    e.side_serial = e.S >= (1ull << 26) ? 1u : 0u;
    sim->ensure_far(1, 2);
    check(cudaStreamSynchronize(st), "create synchronize");
}

// ---------------------------------------------------------------------------
// eviction: a simulation's device state moves to host memory and back
// (the reference's NeuronStateCache writes evicted NeuronStates to its
// backing store and loads them again on demand, NeuronStateCache.cpp:22-43;
// here the unit is a whole simulation, whose device memory a server needs
// for other jobs)
// ---------------------------------------------------------------------------

// Every device pointer of the engine that points into `from[i]` is moved to
// the same offset in `to[i]`.
void remap_engine(Engine& e, const DeviceBuffers& from, const DeviceBuffers& to) {
    auto fix = [&](auto& ptr) {
        if (ptr == nullptr) return;
        const auto* c = reinterpret_cast<const unsigned char*>(ptr);
        for (size_t i = 0; i < from.size(); ++i) {
            const auto* b = static_cast<const unsigned char*>(from[i].p);
            if (b != nullptr && c >= b && c < b + from[i].bytes) {
                ptr = reinterpret_cast<std::remove_reference_t<decltype(ptr)>>(static_cast<unsigned char*>(to[i].p) +
                                                                               (c - b));
                return;
            }
        }
        throw_fail(SNNCUDA_ERR_DEVICE, "eviction: a device pointer outside the simulation's buffers");
    };
    fix(e.in_ptr); fix(e.nparam); fix(e.nrec); fix(e.ntp); fix(e.cand); fix(e.refmeta); fix(e.ring); fix(e.syn);
    fix(e.lcode); fix(e.pre_base); fix(e.pre_off); fix(e.pre_ev); fix(e.cls_delta); fix(e.wheel);
    fix(e.slot_count); fix(e.bcnt); fix(e.btot); fix(e.bstart); fix(e.bcur); fix(e.seg_start); fix(e.grp);
    fix(e.grp_tmp); fix(e.evin); fix(e.ev_a0); fix(e.fire_bits); fix(e.fire_at);
    fix(e.fire_tile); fix(e.fire_list); fix(e.fired_tgt); fix(e.fired_cnt); fix(e.xsum); fix(e.xdst);
    fix(e.xdst_ok); fix(e.raster); fix(e.ts); fix(e.tab.decay); fix(e.tab.ltp); fix(e.tab.ltd);
}

bool run_complete(snncuda_sim* sim, bool wait);

// Copies the simulation's device state to host memory and frees its device
// buffers: state buffers whole, the wheel slot by slot up to each slot's
// event count, per-tick scratch not at all.
void evict_impl(snncuda_sim* sim) {
    if (sim->evicted) return;
    run_complete(sim, true);
    cudaStream_t st = sim->stream;
    Engine& e = sim->e;
    std::vector<uint32_t> counts(e.W);
    check(cudaMemcpyAsync(counts.data(), e.slot_count, e.W * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
          "eviction copy");
    check(cudaStreamSynchronize(st), "eviction synchronize");
    sim->evicted_data.assign(sim->owned.size(), {});
    for (size_t i = 0; i < sim->owned.size(); ++i) {
        const DeviceBuffer& b = sim->owned[i];
        std::vector<unsigned char>& h = sim->evicted_data[i];
        if (b.p == nullptr || b.kind == BufKind::kScratch || b.kind == BufKind::kZero) continue;
        if (b.kind == BufKind::kState) {
            h.resize(b.bytes);
            check(cudaMemcpyAsync(h.data(), b.p, b.bytes, cudaMemcpyDeviceToHost, st), "eviction copy");
            continue;
        }
        size_t total = 0;  // the wheel: the live prefix of every slot
        for (uint32_t c : counts) total += c;
        h.resize(total * 8);
        size_t at = 0;
        for (uint32_t slot = 0; slot < e.W; ++slot) {
            if (counts[slot] == 0) continue;
            check(cudaMemcpyAsync(h.data() + at * 8, static_cast<unsigned char*>(b.p) + slot * e.slot_cap * 8,
                                  counts[slot] * 8ull, cudaMemcpyDeviceToHost, st), "eviction copy");
            at += counts[slot];
        }
    }
    check(cudaStreamSynchronize(st), "eviction synchronize");
    sim->drop_graphs();
    for (DeviceBuffer& b : sim->owned)
        if (b.p) check(cudaFreeAsync(b.p, st), "eviction free");
    for (void** p : {reinterpret_cast<void**>(&sim->far_ev), reinterpret_cast<void**>(&sim->far_idx),
                     reinterpret_cast<void**>(&sim->inj_ev), reinterpret_cast<void**>(&sim->inj_slot),
                     reinterpret_cast<void**>(&sim->inj_off)}) {
        if (*p) check(cudaFreeAsync(*p, st), "eviction free");
        *p = nullptr;
    }
    sim->far_ev_cap = sim->far_idx_cap = sim->inj_cap = sim->inj_groups_cap = 0;
    e.far_ev = nullptr;
    e.far_idx = nullptr;
    check(cudaStreamSynchronize(st), "eviction synchronize");
    sim->evicted = true;
    sim->evictions += 1;
}

// Allocates the simulation's device buffers again, copies the evicted state
// back and points the engine at the new buffers.
void restore_impl(snncuda_sim* sim) {
    if (!sim->evicted) return;
    cudaStream_t st = sim->stream;
    Engine& e = sim->e;
    DeviceBuffers fresh = sim->owned;
    size_t made = 0;
    try {
        for (; made < fresh.size(); ++made) {
            DeviceBuffer& b = fresh[made];
            if (b.p == nullptr) continue;
            b.p = nullptr;
            check(cudaMallocAsync(&b.p, b.bytes, st), "restore allocation");
        }
    } catch (...) {
        for (size_t i = 0; i < made; ++i)
            if (fresh[i].p && sim->owned[i].p) cudaFreeAsync(fresh[i].p, st);
        cudaStreamSynchronize(st);
        throw;
    }
    std::vector<uint32_t> counts;
    for (size_t i = 0; i < fresh.size(); ++i) {
        const DeviceBuffer& b = fresh[i];
        const std::vector<unsigned char>& h = sim->evicted_data[i];
        if (b.p == nullptr || b.kind != BufKind::kState) continue;
        check(cudaMemcpyAsync(b.p, h.data(), b.bytes, cudaMemcpyHostToDevice, st), "restore copy");
        if (sim->owned[i].p == e.slot_count) {
            counts.resize(e.W);
            std::memcpy(counts.data(), h.data(), e.W * sizeof(uint32_t));
        }
    }
    for (size_t i = 0; i < fresh.size(); ++i) {
        if (fresh[i].p == nullptr || fresh[i].kind != BufKind::kWheel) continue;
        const std::vector<unsigned char>& h = sim->evicted_data[i];
        size_t at = 0;
        for (uint32_t slot = 0; slot < e.W && slot < counts.size(); ++slot) {
            if (counts[slot] == 0) continue;
            check(cudaMemcpyAsync(static_cast<unsigned char*>(fresh[i].p) + slot * e.slot_cap * 8,
                                  h.data() + at * 8, counts[slot] * 8ull, cudaMemcpyHostToDevice, st),
                  "restore copy");
            at += counts[slot];
        }
    }
    // scratch that reads zero between ticks comes back as zeros; the rest of
    // the scratch needs no contents
    for (const DeviceBuffer& b : fresh)
        if (b.p != nullptr && b.kind == BufKind::kZero) check(cudaMemsetAsync(b.p, 0, b.bytes, st), "restore zero");
    remap_engine(e, sim->owned, fresh);
    sim->owned = std::move(fresh);
    check(cudaStreamSynchronize(st), "restore synchronize");
    sim->evicted_data.clear();
    sim->evicted = false;
    sim->ensure_far(1, 2);
}

// ---------------------------------------------------------------------------
// wheel slot capacity and launch shapes
// ---------------------------------------------------------------------------

// Sizes that follow from the wheel slot capacity.
struct SlotSizes {
    uint64_t slot_cap, fire_cap, xblocks, bit_words, fire_tiles;
};
SlotSizes slot_sizes(uint64_t slot_cap, uint32_t N) {
    SlotSizes z;
    z.slot_cap = slot_cap;
    z.fire_cap = std::min<uint64_t>(slot_cap, std::max<uint64_t>(65536, 4ull * N));
    z.xblocks = (z.fire_cap + kExpandFires - 1) / kExpandFires;
    z.bit_words = slot_cap / 32;
    z.fire_tiles = (z.bit_words + 255) / 256;
    return z;
}

// Gives the wheel slots capacity `cap` (a multiple of 32 that holds every
// slot's queued events): the wheel moves slot by slot into a new buffer,
// the per-tick buffers sized by the capacity are allocated again (zeroed
// where they must read zero between ticks), and the graphs are recaptured
// on the next run.
void resize_slots(snncuda_sim* sim, uint64_t cap) {
    Engine& e = sim->e;
    cudaStream_t st = sim->stream;
    run_complete(sim, true);
    const std::vector<uint32_t> counts = sim->d2h(e.slot_count, e.W);
    for (uint32_t c : counts)
        if (c > cap) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "a wheel slot holds more events than the new capacity");
    const SlotSizes z = slot_sizes(cap, sim->N);
    const uint32_t D = std::max<uint32_t>(e.D, 1);
    auto entry = [&](const void* p) -> DeviceBuffer& {
        for (DeviceBuffer& b : sim->owned)
            if (b.p == p) return b;
        throw_fail(SNNCUDA_ERR_DEVICE, "resize: unknown buffer");
    };
    auto realloc_buf = [&](auto*& field, size_t bytes) {
        DeviceBuffer& b = entry(field);
        void* fresh = nullptr;
        check(cudaMallocAsync(&fresh, bytes, st), "resize allocation");
        if (b.kind == BufKind::kZero) check(cudaMemsetAsync(fresh, 0, bytes, st), "resize zero");
        if (b.kind == BufKind::kWheel) {
            for (uint32_t slot = 0; slot < e.W; ++slot)
                if (counts[slot])
                    check(cudaMemcpyAsync(static_cast<unsigned long long*>(fresh) + slot * cap,
                                          e.wheel + slot * e.slot_cap, counts[slot] * 8ull, cudaMemcpyDeviceToDevice,
                                          st), "resize copy");
        }
        check(cudaFreeAsync(b.p, st), "resize free");
        b.p = fresh;
        b.bytes = bytes;
        field = static_cast<std::remove_reference_t<decltype(field)>>(fresh);
    };
    sim->drop_graphs();
    realloc_buf(e.wheel, static_cast<size_t>(e.W) * cap * 8);
    realloc_buf(e.grp, cap * 8);
    realloc_buf(e.grp_tmp, cap * sizeof(BucketEntry));
    realloc_buf(e.evin, cap * sizeof(EvIn));
    realloc_buf(e.ev_a0, cap * sizeof(SynPre));
    realloc_buf(e.fire_at, cap * 4);
    realloc_buf(e.fire_bits, std::max<uint64_t>(z.bit_words, 1) * 4);
    realloc_buf(e.fire_tile, (z.fire_tiles + 2) * 4);
    realloc_buf(e.fire_list, z.fire_cap * 4);
    realloc_buf(e.xsum, z.xblocks * D * 4);
    realloc_buf(e.xdst, z.xblocks * D * 8);
    e.slot_cap = cap;
    e.fire_cap = static_cast<uint32_t>(z.fire_cap);
    e.fire_tiles_cap = static_cast<uint32_t>(z.fire_tiles);
    e.grid_fire = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>(z.fire_tiles, sim->sms * 8ull)));
    sim->config.slot_event_capacity = cap;
    check(cudaStreamSynchronize(st), "resize synchronize");
}

void run_enqueue(snncuda_sim* sim, uint64_t T, snncuda_profile* prof);
void resident(snncuda_sim* sim);

// Device time per tick of the next `ticks` ticks (they are the simulation's
// own ticks: launch shapes do not change results).
double probe_ms_per_tick(snncuda_sim* sim, uint64_t ticks) {
    cudaEvent_t a = nullptr, b = nullptr;
    check(cudaEventCreate(&a), "event");
    check(cudaEventCreate(&b), "event");
    float ms = 0.0F;
    cudaError_t err = cudaEventRecord(a, sim->stream);
    try {
        // the first launch of freshly captured graphs is not timed
        run_enqueue(sim, sim->next_tick + std::min<uint64_t>(ticks, sim->ticks_per_graph) - 1, nullptr);
        run_complete(sim, true);
        if (err == cudaSuccess) err = cudaEventRecord(a, sim->stream);
        run_enqueue(sim, sim->next_tick + ticks - 1, nullptr);
        if (err == cudaSuccess) err = cudaEventRecord(b, sim->stream);
        run_complete(sim, true);
    } catch (...) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        throw;
    }
    if (err == cudaSuccess) err = cudaEventSynchronize(b);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    check(err, "probe timing");
    return ms / static_cast<double>(ticks);
}

// Picks the launch shapes by timed probes of the next ticks (coordinate
// descent over k_events, k_process, grouping and k_temporal blocks per SM
// and the ticks per captured graph), then sizes the wheel slots to twice the
// largest due list seen plus 2^16 events when that is smaller than the
// current capacity.
void autotune_impl(snncuda_sim* sim, uint64_t probe_ticks, snncuda_tuning* out) {
    if (probe_ticks == 0) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "probe_ticks must be nonzero");
    resident(sim);
    run_complete(sim, true);
    Engine& e = sim->e;
    const uint32_t sms = sim->sms;
    const uint32_t walk_max = static_cast<uint32_t>(std::max<uint64_t>(1, (static_cast<uint64_t>(sim->N) + 63) / 64));
    uint32_t probes = 0;
    double best = probe_ms_per_tick(sim, probe_ticks);
    ++probes;
    const double first = best;
    struct Knob {
        uint32_t* field;
        std::vector<uint32_t> cands;
    };
    std::vector<Knob> knobs = {
        {&e.grid_events, {sms * 4, sms * 8, sms * 16}},
        {&e.grid_walk, {std::min(walk_max, sms * 2), std::min(walk_max, sms * 3), std::min(walk_max, sms * 4),
                        std::min(walk_max, sms * 6)}},
        {&e.grid_bucket, {sms, sms * 2, sms * 4}},
        {&e.scatter_pass_events, {kScatterPassEvents / 2, kScatterPassEvents * 2, 0u}},
        {&e.side_serial, {0u, 1u}},
        {&e.grid_process, {sms * 2, sms * 4, sms * 8}},
        {&sim->ticks_per_graph, {8, 16, 32}},
    };
    for (Knob& k : knobs) {
        const uint32_t keep = *k.field;
        uint32_t pick = keep;
        for (uint32_t c : k.cands) {
            if (c == keep || c == 0) continue;
            *k.field = c;
            sim->drop_graphs();
            const double ms = probe_ms_per_tick(sim, probe_ticks);
            ++probes;
            if (ms < best * 0.98) {
                best = ms;
                pick = c;
            }
        }
        *k.field = pick;
        sim->drop_graphs();
    }
    const TickState ts = sim->read_ts();
    const uint64_t want = (std::max<uint64_t>(65536, 2 * ts.max_slot_events + 65536) + 31) & ~31ull;
    if (want < e.slot_cap * 3 / 4) resize_slots(sim, want);
    const double last = probe_ms_per_tick(sim, probe_ticks);
    ++probes;
    if (out) {
        out->grid_events = e.grid_events;
        out->grid_walk = e.grid_walk;
        out->grid_bucket = e.grid_bucket;
        out->scatter_pass_events = e.scatter_pass_events;
        out->side_serial = e.side_serial;
        out->grid_temporal = e.grid_process;
        out->ticks_per_graph = sim->ticks_per_graph;
        out->block_threads = 256;
        out->slot_event_capacity = e.slot_cap;
        out->max_slot_events = ts.max_slot_events;
        out->ms_per_tick_before = first;
        out->ms_per_tick_after = last;
        out->probes = probes;
        out->probe_ticks = probe_ticks;
    }
}

// Applies launch shapes found earlier (by autotune_impl, here or on another
// simulation of the same network); every field must lie in the range the
// autotuner itself searches, and a slot capacity of 0 keeps the current one.
void apply_tuning_impl(snncuda_sim* sim, const snncuda_tuning& t) {
    resident(sim);
    run_complete(sim, true);
    Engine& e = sim->e;
    const uint32_t sms = sim->sms;
    const uint32_t walk_max = static_cast<uint32_t>(std::max<uint64_t>(1, (static_cast<uint64_t>(sim->N) + 63) / 64));
    auto in = [](uint32_t v, uint32_t lo, uint32_t hi) { return v >= lo && v <= hi; };
    if (!in(t.grid_events, 1, sms * 16) || !in(t.grid_walk, 1, std::max(walk_max, sms * 8)) ||
        !in(t.grid_bucket, 1, sms * 4) || !in(t.grid_temporal, 1, sms * 8) || !in(t.ticks_per_graph, 1, 64) ||
        t.side_serial > 1 || (t.block_threads != 0 && t.block_threads != 256))
        throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "tuning field outside the autotuner's ranges");
    e.grid_events = t.grid_events;
    e.grid_walk = t.grid_walk;
    e.grid_bucket = t.grid_bucket;
    e.grid_process = t.grid_temporal;
    e.scatter_pass_events = t.scatter_pass_events;
    e.side_serial = t.side_serial;
    sim->ticks_per_graph = t.ticks_per_graph;
    sim->drop_graphs();
    if (t.slot_event_capacity != 0 && t.slot_event_capacity != e.slot_cap) {
        if (t.slot_event_capacity >= (1ull << 31))
            throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "slot capacity must be below 2^31");
        resize_slots(sim, (t.slot_event_capacity + 31) & ~31ull);
    }
}

// The simulation's state on the device (restored on demand, as the
// reference's cache loads an evicted neuron state on its next use).
void resident(snncuda_sim* sim) {
    if (sim->evicted) restore_impl(sim);
}

int status_to_error(uint32_t status, std::string& msg) {
    msg.clear();
    if (status & kStatusSlotOverflow) msg += "wheel slot capacity exceeded (raise slot_event_capacity); ";
    if (status & kStatusRingOverflow) msg += "learned-pattern run storage exceeded (raise pattern_run_capacity); ";
    if (status & kStatusRasterOverflow) msg += "raster capacity exceeded; ";
    if (status & kStatusPostCountOverflow) msg += "a neuron fired 65536+ times in one tick; ";
    if (status & kStatusRunOverflow) msg += "temporal run list overflow; ";
    if (status & kStatusFireOverflow) msg += "fires per tick exceeded the fire capacity; ";
    if (status & kStatusStageTimeout) {
        msg += "a bulk copy into shared memory did not complete within its wait limit; ";
        return SNNCUDA_ERR_TIMEOUT;
    }
    return SNNCUDA_ERR_CAPACITY;
}

// Queued injections in (delivery, call order): new ones are sorted on their
// own (stable: call order kept), then merged behind the earlier ones they tie
// with.
void sort_pending(snncuda_sim* sim) {
    auto& pend = sim->pending;
    if (sim->pend_sorted < pend.size()) {
        auto by_tick = [](const Pending& a, const Pending& b) { return a.tick < b.tick; };
        const auto mid = pend.begin() + static_cast<std::ptrdiff_t>(sim->pend_sorted);
        // a drive injected in tick order (the common case) needs no sort, and
        // one that starts at or after every queued event needs no merge
        const Pending* q = &*mid;
        const size_t m = static_cast<size_t>(pend.end() - mid);
        std::atomic<bool> sorted{true};
        parallel_for(m, [&](size_t b, size_t en) {
            for (size_t i = b == 0 ? 1 : b; i < en; ++i)
                if (q[i].tick < q[i - 1].tick) {
                    sorted.store(false, std::memory_order_relaxed);
                    return;
                }
        });
        if (!sorted.load()) std::stable_sort(mid, pend.end(), by_tick);
        if (sim->pend_sorted > sim->pend_head && by_tick(*mid, *(mid - 1)))
            std::inplace_merge(pend.begin() + static_cast<std::ptrdiff_t>(sim->pend_head), mid, pend.end(), by_tick);
        sim->pend_sorted = pend.size();
    }
}

// Enqueues ticks next_tick .. T on the simulation's stream and returns
// without waiting; run_complete() waits and checks the device status.
void run_enqueue(snncuda_sim* sim, uint64_t T, snncuda_profile* prof) {
    const uint64_t p = sim->next_tick;
    if (sim->run_in_flight) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "a run is already in flight");
    if (T < p) return;
    if (T >= 0xFFFF0000ull) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "ticks beyond 2^32 - 2^16");
    Engine& e = sim->e;
    const uint64_t W = e.W;
    // Injections in (delivery, call order).  Those due within W ticks go into
    // their slots now, behind everything scheduled before this call; later
    // ones are copied in by k_bcount the tick their slot frees up; the rest wait.
    auto& pend = sim->pending;
    sort_pending(sim);
    const Pending* base = pend.data() + sim->pend_head;
    const size_t live = pend.size() - sim->pend_head;
    auto first_at_or_after = [&](uint64_t tick) {
        return static_cast<size_t>(std::partition_point(base, base + live,
                                                        [tick](const Pending& q) { return q.tick < tick; }) -
                                   base);
    };
    const size_t a_end = first_at_or_after(p + W);
    const size_t b_end = first_at_or_after(T + W);
    cudaStream_t st = sim->stream;
    if (a_end > 0) {
        // one group per delivery tick with injections (the queue is in tick
        // order: each tick's injections are one run, found by binary search)
        std::vector<uint32_t> slots, offs;
        for (size_t b = 0; b < a_end;) {
            const uint64_t tick = base[b].tick;
            slots.push_back(static_cast<uint32_t>(tick & (W - 1)));
            offs.push_back(static_cast<uint32_t>(b));
            b = std::min(a_end, first_at_or_after(tick + 1));
        }
        offs.push_back(static_cast<uint32_t>(a_end));
        sim->ensure_inject(a_end, slots.size());
        sim->ensure_host(a_end, 2 * slots.size() + 1);
        unsigned long long* hev = sim->host_ev;
        parallel_for(a_end, [&](size_t b, size_t en) {
            for (size_t i = b; i < en; ++i) hev[i] = base[i].event;
        });
        std::copy(slots.begin(), slots.end(), sim->host_idx);
        std::copy(offs.begin(), offs.end(), sim->host_idx + slots.size());
        check(cudaMemcpyAsync(sim->inj_ev, sim->host_ev, a_end * 8, cudaMemcpyHostToDevice, st), "inject copy");
        check(cudaMemcpyAsync(sim->inj_slot, sim->host_idx, slots.size() * 4, cudaMemcpyHostToDevice, st),
              "inject copy");
        check(cudaMemcpyAsync(sim->inj_off, sim->host_idx + slots.size(), offs.size() * 4, cudaMemcpyHostToDevice,
                              st), "inject copy");
        launch_inject(e, sim->inj_ev, sim->inj_slot, sim->inj_off, static_cast<uint32_t>(slots.size()), st);
        check(cudaGetLastError(), "inject launch");
        check(cudaStreamSynchronize(st), "inject synchronize");
    }
    uint32_t far_first = static_cast<uint32_t>(p + W);
    uint32_t far_ticks = 0;
    if (b_end > a_end) {
        far_ticks = static_cast<uint32_t>(T + W - 1 - (p + W) + 1);  // deliveries p+W .. T+W-1
        const size_t n = b_end - a_end;
        sim->ensure_far(n, static_cast<size_t>(far_ticks) + 1);
        sim->ensure_host(n, static_cast<size_t>(far_ticks) + 1);
        uint32_t* idx = sim->host_idx;  // idx[j]: far injections due before far_first + j
        for (uint32_t j = 0; j < far_ticks; ++j) idx[j] = static_cast<uint32_t>(first_at_or_after(far_first + j) - a_end);
        idx[far_ticks] = static_cast<uint32_t>(n);
        unsigned long long* hev = sim->host_ev;
        parallel_for(n, [&](size_t b, size_t en) {
            for (size_t i = b; i < en; ++i) hev[i] = base[a_end + i].event;
        });
        check(cudaMemcpyAsync(sim->far_ev, sim->host_ev, n * 8, cudaMemcpyHostToDevice, st), "far copy");
        check(cudaMemcpyAsync(sim->far_idx, idx, (static_cast<size_t>(far_ticks) + 1) * 4, cudaMemcpyHostToDevice,
                              st), "far copy");
        check(cudaStreamSynchronize(st), "far copy");
    }
    sim->pend_head += b_end;
    if (sim->pend_head == pend.size()) {
        pend.clear();
        sim->pend_head = sim->pend_sorted = 0;
    } else if (sim->pend_head > (1u << 16) && sim->pend_head > 3 * (pend.size() - sim->pend_head)) {
        // compaction once three quarters are consumed: the live quarter moves
        // to the front (no overlap), split across host threads
        const size_t head = sim->pend_head, live_n = pend.size() - head;
        Pending* q = pend.data();
        parallel_for(live_n, [&](size_t b, size_t en) { std::copy(q + head + b, q + head + en, q + b); });
        pend.resize(live_n);
        sim->pend_sorted -= head;
        sim->pend_head = 0;
    }
    // run parameters live in device memory so the captured graphs stay valid
    check(cudaMemcpyAsync(reinterpret_cast<char*>(e.ts) + offsetof(TickState, far_first_tick), &far_first, 4,
                          cudaMemcpyHostToDevice, st), "run params");
    check(cudaMemcpyAsync(reinterpret_cast<char*>(e.ts) + offsetof(TickState, far_ticks), &far_ticks, 4,
                          cudaMemcpyHostToDevice, st), "run params");
    uint64_t ticks = T - p + 1;
    if (prof != nullptr) {
        const TickState before = sim->read_ts();
        if (sim->graph_prof == nullptr) sim->graph_prof = sim->capture(1, true);
        for (uint64_t i = 0; i < ticks; ++i) {
            check(cudaGraphLaunch(sim->graph_prof, st), "graph launch");
            check(cudaStreamSynchronize(st), "profile synchronize");
            for (int k = 0; k < kKernelCount; ++k) {
                float ms = 0.0F;
                check(cudaEventElapsedTime(&ms, sim->marks[2 * k], sim->marks[2 * k + 1]), "event time");
                prof->kernel_ms[k] += ms;
            }
        }
        const TickState after = sim->read_ts();
        prof->ticks += ticks;
        prof->synaptic_events += (after.delivered - after.external) - (before.delivered - before.external);
        prof->external_events += after.external - before.external;
        prof->fires += after.fired - before.fired;
        prof->touched_targets += after.touched_total - before.touched_total;
        ticks = 0;
    }
    if (ticks >= sim->ticks_per_graph && sim->graph_many == nullptr)
        sim->graph_many = sim->capture(static_cast<int>(sim->ticks_per_graph));
    if (ticks > 0 && sim->graph_one == nullptr) sim->graph_one = sim->capture(1);
    while (ticks >= sim->ticks_per_graph) {
        check(cudaGraphLaunch(sim->graph_many, st), "graph launch");
        ticks -= sim->ticks_per_graph;
    }
    while (ticks > 0) {
        check(cudaGraphLaunch(sim->graph_one, st), "graph launch");
        ticks -= 1;
    }
    const uint32_t zero = 0;
    check(cudaMemcpyAsync(reinterpret_cast<char*>(e.ts) + offsetof(TickState, far_ticks), &zero, 4,
                          cudaMemcpyHostToDevice, st), "run params");
    if (sim->ts_pinned == nullptr) check(cudaMallocHost(&sim->ts_pinned, sizeof(TickState)), "pinned tick state");
    if (sim->run_done == nullptr) check(cudaEventCreateWithFlags(&sim->run_done, cudaEventDisableTiming), "event");
    check(cudaMemcpyAsync(sim->ts_pinned, e.ts, sizeof(TickState), cudaMemcpyDeviceToHost, st), "read tick state");
    check(cudaEventRecord(sim->run_done, st), "event record");
    sim->run_target = T;
    sim->run_in_flight = true;
}

// True once the run in flight (if any) has finished; then checks it.
// `wait` blocks until it has.
bool run_complete(snncuda_sim* sim, bool wait) {
    if (!sim->run_in_flight) return true;
    if (wait) {
        check(cudaEventSynchronize(sim->run_done), "run synchronize");
    } else {
        const cudaError_t q = cudaEventQuery(sim->run_done);
        if (q == cudaErrorNotReady) return false;
        check(q, "run query");
    }
    sim->run_in_flight = false;
    const TickState ts = *sim->ts_pinned;
    const uint64_t T = sim->run_target;
    sim->next_tick = T + 1;
    if (ts.tick != static_cast<uint32_t>(T + 1)) throw_fail(SNNCUDA_ERR_DEVICE, "device tick counter out of step");
    if (ts.status != 0) {
        sim->poisoned = true;
        std::string msg;
        const int code = status_to_error(ts.status, msg);
        throw_fail(code, msg);
    }
    return true;
}

void run_impl(snncuda_sim* sim, uint64_t T, snncuda_profile* prof = nullptr) {
    run_enqueue(sim, T, prof);
    run_complete(sim, true);
}

// Rebuild the offsets of a run list.
void expand_runs(const unsigned long long* runs, uint32_t nruns, uint32_t cap, uint32_t start, uint64_t limit,
                 std::vector<uint32_t>& out) {
    out.clear();
    for (uint32_t j = 0; j < nruns && out.size() < limit; ++j) {
        const unsigned long long r = runs[(start + j) % cap];
        for (unsigned long long c = 0; c < run_count(r) && out.size() < limit; ++c) out.push_back(run_value(r));
    }
}

struct HostState {
    std::vector<NeuronRec> nrec;
    std::vector<NeuronTp> ntp;
    std::vector<unsigned long long> cand, ring;
    std::vector<RefMeta> meta;
    std::vector<SynAB> syn;
    std::vector<uint16_t> lcode;
};

void neuron_offsets(const snncuda_sim* sim, const HostState& h, uint32_t n, std::vector<uint32_t>& out) {
    const NeuronParam& p = sim->nparam[n];
    expand_runs(h.cand.data() + p.cand_base, h.ntp[n].nruns, p.window + 1, 0, h.nrec[n].len, out);
}

void neuron_learned(const snncuda_sim* sim, const HostState& h, uint32_t n, uint32_t which, std::vector<uint32_t>& out) {
    const NeuronParam& p = sim->nparam[n];
    const RefMeta& m = h.meta[p.meta_base + (h.ntp[n].ref_head + which) % p.max_refs];
    expand_runs(h.ring.data() + p.ring_base, m.nruns, p.ring_cap, m.start, m.len, out);
}

uint32_t expected_of(const SynA& a) { return (a.meta >> kMetaExpectedShift) & 15u; }

void synapse_learned(const snncuda_sim* sim, const HostState& h, uint64_t tm, uint32_t which, std::vector<uint32_t>& out) {
    const uint32_t n = static_cast<uint32_t>(std::upper_bound(sim->in_ptr.begin(), sim->in_ptr.end(), tm) -
                                             sim->in_ptr.begin() - 1);
    const NeuronParam& p = sim->nparam[n];
    if (inline_code_pattern(p.max_refs, sim->e.code_stride)) {
        out.clear();
        for (uint32_t j = 0; j < expected_of(h.syn[tm].a); ++j) out.push_back(ring_get(h.syn[tm].b.ring_hi, 0, j));
        return;
    }
    const uint16_t* lc = h.lcode.data() + p.lcode_base + (tm - p.in_begin) * p.max_refs * sim->e.code_stride +
                         static_cast<size_t>(which) * sim->e.code_stride;
    out.assign(lc, lc + expected_of(h.syn[tm].a));
}

HostState fetch_all(snncuda_sim* sim, bool temporal) {
    HostState h;
    Engine& e = sim->e;
    h.nrec = sim->d2h(e.nrec, sim->N);
    h.ntp = sim->d2h(e.ntp, sim->N);
    h.syn = sim->d2h(e.syn, sim->S);
    if (temporal) {
        uint64_t cand = 0, ring = 0, meta = 0, lcode = 0;
        for (uint32_t n = 0; n < sim->N; ++n) {
            const NeuronParam& p = sim->nparam[n];
            cand += p.window + 1;
            ring += p.ring_cap;
            meta += p.max_refs;
            if (!inline_code_pattern(p.max_refs, e.code_stride))
                lcode += (sim->in_ptr[n + 1] - sim->in_ptr[n]) * p.max_refs * e.code_stride;
        }
        h.cand = sim->d2h(e.cand, cand);
        h.ring = sim->d2h(e.ring, ring);
        h.meta = sim->d2h(e.refmeta, meta);
        h.lcode = sim->d2h(e.lcode, lcode);
    }
    return h;
}

template <typename F>
int guarded(F&& body) {
    try {
        body();
        return SNNCUDA_OK;
    } catch (const Failure& f) {
        return set_error(f.code, f.message);
    } catch (const std::bad_alloc&) {
        return set_error(SNNCUDA_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& ex) {
        return set_error(SNNCUDA_ERR_DEVICE, ex.what());
    }
}

}  // namespace

extern "C" {

const char* snncuda_version(void) { return "0.1.0-gb300"; }

int snncuda_cuda_available(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return count > 0 ? 1 : 0;
}

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
    c->stage_wait_ns = 100000000ULL;
}

int snncuda_sim_create(const snncuda_network* net, const snncuda_config* config, snncuda_sim** out) {
    if (net == nullptr || out == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_config def;
    snncuda_config_default(&def);
    const snncuda_config& cfg = config ? *config : def;
    snncuda_sim* sim = nullptr;
    try {
        sim = new snncuda_sim();
    } catch (const std::bad_alloc&) {
        return set_error(SNNCUDA_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    const int rc = guarded([&] { create_impl(net, cfg, sim); });
    if (rc != SNNCUDA_OK) {
        delete sim;
        return rc;
    }
    *out = sim;
    return SNNCUDA_OK;
}

int snncuda_sim_destroy(snncuda_sim* sim) {
    delete sim;
    return SNNCUDA_OK;
}

int snncuda_sim_inject(snncuda_sim* sim, uint64_t count, const uint32_t* neurons, const uint64_t* ticks,
                       const float* weights) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (count > 0 && (!neurons || !ticks || !weights)) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null array");
    return guarded([&] {
        std::atomic<bool> in_range{true};
        parallel_for(count, [&](size_t b, size_t en) {
            for (size_t i = b; i < en; ++i)
                if (neurons[i] >= sim->N) {
                    in_range.store(false, std::memory_order_relaxed);
                    return;
                }
        });
        if (!in_range.load()) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "inject neuron out of range");
        const size_t at = sim->pending.size();
        sim->pending.resize(at + count);
        Pending* dst = sim->pending.data() + at;
        const uint64_t now = sim->next_tick;
        parallel_for(count, [&](size_t b, size_t en) {
            for (size_t i = b; i < en; ++i) {
                uint32_t wbits;
                std::memcpy(&wbits, &weights[i], 4);
                dst[i] = Pending(ticks[i] < now ? now : ticks[i],
                                 (static_cast<unsigned long long>(wbits) << 32) | neurons[i] | kExternalBit);
            }
        });
    });
}

int snncuda_sim_run_until(snncuda_sim* sim, uint64_t inclusive_tick) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->poisoned) return set_error(SNNCUDA_ERR_POISONED, "simulation poisoned by an earlier device error");
    const int rc = guarded([&] {
        resident(sim);
        run_impl(sim, inclusive_tick);
    });
    if (rc == SNNCUDA_ERR_DEVICE) sim->poisoned = true;
    return rc;
}

static int set_flag(snncuda_sim* sim, size_t offset, int32_t v) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] {
        resident(sim);
        check(cudaMemcpyAsync(reinterpret_cast<char*>(sim->e.ts) + offset, &v, 4, cudaMemcpyHostToDevice,
                              sim->stream), "toggle");
        check(cudaStreamSynchronize(sim->stream), "toggle");
    });
}

int snncuda_sim_set_plasticity(snncuda_sim* sim, int32_t enabled) {
    return set_flag(sim, offsetof(TickState, stdp_enabled), enabled ? 1 : 0);
}

int snncuda_sim_set_temporal_learning(snncuda_sim* sim, int32_t enabled) {
    return set_flag(sim, offsetof(TickState, temporal_enabled), enabled ? 1 : 0);
}

int snncuda_sim_counters(snncuda_sim* sim, snncuda_counters* out) {
    if (sim == nullptr || out == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        resident(sim);
        const TickState ts = sim->read_ts();
        const std::vector<uint32_t> counts = sim->d2h(sim->e.slot_count, sim->e.W);
        uint64_t pending = sim->pending.size() - sim->pend_head;
        for (uint32_t c : counts) pending += c;
        out->delivered_spikes = ts.delivered;
        out->fired_spikes = ts.fired;
        out->external_events = ts.external;
        out->synaptic_events = ts.delivered - ts.external;
        out->next_tick = sim->next_tick;
        out->pending_events = pending;
        out->raster_count = ts.raster_count;
        out->max_slot_events = ts.max_slot_events;
    });
}

int snncuda_sim_idle(snncuda_sim* sim, int32_t* out) {
    if (out == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_counters c;
    const int rc = snncuda_sim_counters(sim, &c);
    if (rc == SNNCUDA_OK) *out = c.pending_events == 0 ? 1 : 0;
    return rc;
}

// Neurons [n0, n1) into o[0 .. n1-n0).
static void read_neurons_range(snncuda_sim* sim, uint32_t n0, uint32_t n1, const snncuda_neuron_state* o) {
    const std::vector<NeuronRec> r = sim->d2h(sim->e.nrec + n0, n1 - n0);
    const std::vector<NeuronTp> q = sim->d2h(sim->e.ntp + n0, n1 - n0);
    for (uint32_t i = 0; i < n1 - n0; ++i) {
        if (o->membrane_potential) o->membrane_potential[i] = r[i].membrane;
        if (o->spike_count) o->spike_count[i] = r[i].spike_count;
        if (o->last_fired_tick) o->last_fired_tick[i] = r[i].last_fired1 ? static_cast<int64_t>(r[i].last_fired1) - 1 : -1;
        if (o->last_active_tick) o->last_active_tick[i] = r[i].last_active;
        for (int k = 0; k < 4; ++k) {
            if (o->compartment_current) o->compartment_current[i * 4 + k] = r[i].cur[k];
            if (o->compartment_last_update) o->compartment_last_update[i * 4 + k] = r[i].upd[k];
            if (o->compartment_tau) o->compartment_tau[i * 4 + k] = kTauValue[(r[i].flags >> (2 * k)) & 3u];
        }
        if (o->window_start_tick) o->window_start_tick[i] = r[i].ws;
        if (o->offset_count) o->offset_count[i] = r[i].len;
        if (o->learned_count) o->learned_count[i] = q[i].ref_count;
        if (o->match_count) o->match_count[i] = r[i].match_count;
        if (o->last_match) o->last_match[i] = q[i].last_match;
    }
}

int snncuda_sim_read_neurons(snncuda_sim* sim, const snncuda_neuron_state* o) {
    if (sim == nullptr || o == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        resident(sim);
        read_neurons_range(sim, 0, sim->N, o);
    });
}

// Synapses of Connectome indices [c0, c1), whose target-major slots are
// [t0, t1), into o[0 .. c1-c0).
static void read_synapses_range(snncuda_sim* sim, uint64_t c0, uint64_t c1, uint64_t t0, uint64_t t1,
                         const snncuda_synapse_state* o) {
    const std::vector<SynAB> rec = sim->d2h(sim->e.syn + t0, t1 - t0);
    for (uint64_t tm = t0; tm < t1; ++tm) {
        const uint64_t i = sim->c_of_tm[tm] - c0;
        const SynA& a = rec[tm - t0].a;
        const SynB& b = rec[tm - t0].b;
        if (o->weight) o->weight[i] = a.weight;
        if (o->last_pre_spike_tick) o->last_pre_spike_tick[i] = a.last_pre1 ? static_cast<int64_t>(a.last_pre1) - 1 : -1;
        if (o->last_post_spike_tick) o->last_post_spike_tick[i] = a.last_post1 ? static_cast<int64_t>(a.last_post1) - 1 : -1;
        if (o->pre_spike_count) o->pre_spike_count[i] = b.pre_count;
        if (o->plasticity_update_count) o->plasticity_update_count[i] = a.updates;
        if (o->last_weight_delta) o->last_weight_delta[i] = a.last_delta;
        if (o->code_window_start_tick) o->code_window_start_tick[i] = b.code_ws;
        if (o->code_offset_count) o->code_offset_count[i] = b.code_len;
        if (o->learned_code_count) o->learned_code_count[i] = b.learned_count;
        if (o->code_match_count) o->code_match_count[i] = b.code_matches;
        if (o->last_code_match) o->last_code_match[i] = b.flags & 1u;
    }
    (void)c1;
}

int snncuda_sim_read_synapses(snncuda_sim* sim, const snncuda_synapse_state* o) {
    if (sim == nullptr || o == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        resident(sim);
        read_synapses_range(sim, 0, sim->S, 0, sim->S, o);
    });
}

int snncuda_sim_read_pattern(snncuda_sim* sim, int32_t kind, uint64_t index, uint64_t which, uint32_t* values,
                             uint64_t capacity, uint64_t* len) {
    if (sim == nullptr || len == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        resident(sim);
        std::vector<uint32_t> v;
        if (kind == 0 || kind == 1) {
            if (index >= sim->N) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "neuron out of range");
            const uint32_t n = static_cast<uint32_t>(index);
            const NeuronParam& p = sim->nparam[n];
            const NeuronRec r = sim->d2h(sim->e.nrec + n, 1)[0];
            const NeuronTp q = sim->d2h(sim->e.ntp + n, 1)[0];
            if (kind == 0) {
                const auto cand = sim->d2h(sim->e.cand + p.cand_base, p.window + 1);
                expand_runs(cand.data(), q.nruns, p.window + 1, 0, r.len, v);
            } else {
                if (which >= q.ref_count) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "pattern index out of range");
                const RefMeta m = sim->d2h(sim->e.refmeta + p.meta_base + (q.ref_head + which) % p.max_refs, 1)[0];
                const auto ring = sim->d2h(sim->e.ring + p.ring_base, p.ring_cap);
                expand_runs(ring.data(), m.nruns, p.ring_cap, m.start, m.len, v);
            }
        } else if (kind == 2 || kind == 3) {
            if (index >= sim->S) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse out of range");
            const uint64_t tm = sim->tm_of_c[index];
            const SynAB rec = sim->d2h(sim->e.syn + tm, 1)[0];
            const SynA& a = rec.a;
            const SynB& b = rec.b;
            if (kind == 2) {
                for (uint32_t j = 0; j < b.code_len; ++j) v.push_back(ring_get(b.ring_lo, b.ring_hi, j));  // code_len <= 4 when inline
            } else {
                if (which >= b.learned_count) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "pattern index out of range");
                const uint32_t n = static_cast<uint32_t>(
                    std::upper_bound(sim->in_ptr.begin(), sim->in_ptr.end(), tm) - sim->in_ptr.begin() - 1);
                const NeuronParam& p = sim->nparam[n];
                if (inline_code_pattern(p.max_refs, sim->e.code_stride)) {
                    for (uint32_t j = 0; j < expected_of(a); ++j) v.push_back(ring_get(b.ring_hi, 0, j));
                } else {
                    const uint64_t off = p.lcode_base + (tm - p.in_begin) * p.max_refs * sim->e.code_stride +
                                         which * sim->e.code_stride;
                    const std::vector<uint16_t> lc = sim->d2h(sim->e.lcode + off, expected_of(a));
                    v.assign(lc.begin(), lc.end());
                }
            }
        } else {
            throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "unknown pattern kind");
        }
        *len = v.size();
        for (uint64_t i = 0; i < v.size() && i < capacity; ++i) values[i] = v[i];
    });
}

// Same digest definition as every other implementation of this ABI.
// State digests of neurons [n0, n1) and Connectome synapses [c0, c1): the
// same words, in the same order, a network alone would hash.
static void digest_range(snncuda_sim* sim, const HostState& h, uint32_t n0, uint32_t n1, uint64_t c0, uint64_t c1,
                  uint64_t* neuron_digest, uint64_t* synapse_digest) {
    std::vector<uint32_t> v;
    if (neuron_digest) {
        Digest d;
        for (uint32_t n = n0; n < n1; ++n) {
            const NeuronRec& r = h.nrec[n];
            d.f32(r.membrane);
            d.word(r.spike_count);
            d.word(r.last_fired1 ? static_cast<uint64_t>(r.last_fired1 - 1) : ~0ULL);
            d.word(r.last_active);
            for (int k = 0; k < 4; ++k) {
                d.f32(r.cur[k]);
                d.word(r.upd[k]);
                d.f32(kTauValue[(r.flags >> (2 * k)) & 3u]);
            }
            d.word(r.ws);
            neuron_offsets(sim, h, n, v);
            d.word(v.size());
            for (uint32_t x : v) d.word(x);
            d.word(h.ntp[n].ref_count);
            for (uint32_t j = 0; j < h.ntp[n].ref_count; ++j) {
                neuron_learned(sim, h, n, j, v);
                d.word(v.size());
                for (uint32_t x : v) d.word(x);
            }
            d.word(h.ntp[n].last_match);
            d.word(r.match_count);
        }
        *neuron_digest = d.h;
    }
    if (synapse_digest) {
        const std::vector<uint32_t>& tm_of_c = sim->tm_of_c;
        Digest d;
        for (uint64_t c = c0; c < c1; ++c) {
            const uint64_t tm = tm_of_c[c];
            const SynA& a = h.syn[tm].a;
            const SynB& b = h.syn[tm].b;
            d.f32(a.weight);
            d.word(a.last_pre1 ? static_cast<uint64_t>(a.last_pre1 - 1) : ~0ULL);
            d.word(a.last_post1 ? static_cast<uint64_t>(a.last_post1 - 1) : ~0ULL);
            d.word(b.pre_count);
            d.word(a.updates);
            d.f32(a.last_delta);
            d.word(b.code_ws);
            d.word(b.code_len);
            for (uint32_t j = 0; j < b.code_len; ++j) d.word(ring_get(b.ring_lo, b.ring_hi, j));
            d.word(b.learned_count);
            for (uint32_t j = 0; j < b.learned_count; ++j) {
                synapse_learned(sim, h, tm, j, v);
                d.word(v.size());
                for (uint32_t x : v) d.word(x);
            }
            d.word(b.code_matches);
            d.word(b.flags & 1u);
        }
        *synapse_digest = d.h;
    }
}

int snncuda_sim_state_digest(snncuda_sim* sim, uint64_t* neuron_digest, uint64_t* synapse_digest) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] {
        resident(sim);
        const HostState h = fetch_all(sim, true);
        digest_range(sim, h, 0, sim->N, 0, sim->S, neuron_digest, synapse_digest);
    });
}

int snncuda_sim_profile(snncuda_sim* sim, uint64_t inclusive_tick, snncuda_profile* out) {
    if (sim == nullptr || out == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    if (sim->poisoned) return set_error(SNNCUDA_ERR_POISONED, "simulation poisoned by an earlier device error");
    const int rc = guarded([&] {
        resident(sim);
        run_impl(sim, inclusive_tick, out);
    });
    if (rc == SNNCUDA_ERR_DEVICE) sim->poisoned = true;
    return rc;
}

const char* snncuda_kernel_name(int32_t index) { return kernel_name(index); }

namespace {

// Device checksums of a range of neurons and target-major synapses.
void checksum_range(snncuda_sim* sim, uint32_t n0, uint32_t n1, uint64_t t0, uint64_t t1, uint64_t* neuron_sum,
                    uint64_t* synapse_sum) {
    cudaStream_t st = sim->stream;
    unsigned long long* d = nullptr;
    check(cudaMallocAsync(&d, 2 * sizeof(unsigned long long), st), "device allocation");
    unsigned long long c[2] = {};
    cudaError_t err = cudaMemsetAsync(d, 0, sizeof(c), st);
    if (err == cudaSuccess) {
        launch_checksum(sim->e, n0, n1, t0, d, st);
        (void)t1;
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(c, d, sizeof(c), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    check(err, "state checksum");
    if (neuron_sum) *neuron_sum = c[0];
    if (synapse_sum) *synapse_sum = c[1];
}

}  // namespace

int snncuda_sim_state_checksum(snncuda_sim* sim, uint64_t* neuron_sum, uint64_t* synapse_sum) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] {
        resident(sim);
        checksum_range(sim, 0, sim->N, 0, sim->S, neuron_sum, synapse_sum);
    });
}

int snncuda_sim_autotune(snncuda_sim* sim, uint64_t probe_ticks, snncuda_tuning* out) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (sim->poisoned) return set_error(SNNCUDA_ERR_POISONED, "simulation poisoned by an earlier device error");
    const int rc = guarded([&] { autotune_impl(sim, probe_ticks, out); });
    if (rc == SNNCUDA_ERR_DEVICE) sim->poisoned = true;
    return rc;
}

int snncuda_sim_apply_tuning(snncuda_sim* sim, const snncuda_tuning* tuning) {
    if (sim == nullptr || tuning == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    if (sim->poisoned) return set_error(SNNCUDA_ERR_POISONED, "simulation poisoned by an earlier device error");
    return guarded([&] { apply_tuning_impl(sim, *tuning); });
}

int snncuda_sim_set_slot_capacity(snncuda_sim* sim, uint64_t capacity) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (capacity == 0 || capacity >= (1ull << 31))
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "slot capacity must be in [1, 2^31)");
    return guarded([&] {
        resident(sim);
        resize_slots(sim, (capacity + 31) & ~31ull);
    });
}

int snncuda_sim_evict(snncuda_sim* sim) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] { evict_impl(sim); });
}

int snncuda_sim_restore(snncuda_sim* sim) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] { restore_impl(sim); });
}

int snncuda_sim_residency(snncuda_sim* sim, int32_t* resident_out, uint64_t* evictions) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    if (resident_out) *resident_out = sim->evicted ? 0 : 1;
    if (evictions) *evictions = sim->evictions;
    return SNNCUDA_OK;
}

namespace {

// Scratch of one grouping call (device pointers).
struct GroupScratch {
    uint32_t* bcnt;       // kGroupGrid x buckets
    uint32_t* btot;       // buckets
    uint32_t* bstart;     // buckets + 1
    uint32_t* bcur;       // buckets
    BucketEntry* grp_tmp;  // count
    uint32_t* slot_count;
    TickState* ts;
};

// Blocks of the grouping entry points' counting and placing kernels (fixed,
// so the static scratch has a fixed size).
constexpr uint32_t kGroupGrid = 256;

uint32_t group_buckets(uint32_t neuron_count) {
    const uint32_t shift = bucket_shift_for(neuron_count);
    return static_cast<uint32_t>(std::max<uint64_t>(1, (static_cast<uint64_t>(neuron_count) + (1u << shift) - 1) >> shift));
}

// The tick's grouping kernels (k_bcount .. k_bsort) on a caller's event
// buffer seen as a one-slot wheel.  Scratch sizes: kGroupGrid x
// group_buckets() counts, group_buckets() (+1) bucket totals, starts and
// cursors, `count` bucket-ordered events (BucketEntry).
void group_run(const uint64_t* events, uint32_t count, uint32_t neuron_count, uint64_t* grouped,
               uint32_t* segment_start, cudaStream_t st, const GroupScratch& sc) {
    int dev = 0, sms = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    Engine e{};
    e.N = neuron_count;
    e.W = 1;
    e.wmask = 0;
    e.slot_cap = count;
    e.wheel = const_cast<unsigned long long*>(reinterpret_cast<const unsigned long long*>(events));
    e.slot_count = sc.slot_count;
    e.bucket_shift = bucket_shift_for(neuron_count);
    e.nbuckets = group_buckets(neuron_count);
    e.grid_bucket = kGroupGrid;
    e.scatter_pass_events = kScatterPassEvents;
    e.stage_wait_ns = 100000000ull;  // the bulk copies' wait limit (as snncuda_config's default)
    e.bcnt = sc.bcnt;
    e.btot = sc.btot;
    e.bstart = sc.bstart;
    e.bcur = sc.bcur;
    e.seg_start = segment_start;
    e.grp = reinterpret_cast<unsigned long long*>(grouped);
    e.grp_tmp = sc.grp_tmp;
    e.ts = sc.ts;
    e.grid_wide = static_cast<uint32_t>(std::max(1, sms * 2));
    configure_kernels();
    check(cudaMemsetAsync(sc.btot, 0, sizeof(uint32_t) * e.nbuckets, st), "memset");
    check(cudaMemsetAsync(sc.bcur, 0, sizeof(uint32_t) * e.nbuckets, st), "memset");
    check(cudaMemsetAsync(sc.ts, 0, sizeof(TickState), st), "memset");
    check(cudaMemcpyAsync(sc.slot_count, &count, sizeof(uint32_t), cudaMemcpyHostToDevice, st), "count");
    launch_group(e, st);
    check(cudaGetLastError(), "group launch");
    TickState ts;
    check(cudaMemcpyAsync(&ts, sc.ts, sizeof(ts), cudaMemcpyDeviceToHost, st), "status");
    check(cudaStreamSynchronize(st), "group synchronize");
    if (ts.status & kStatusBadEvent) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "event target >= neuron_count");
}

}  // namespace

int snncuda_group_events(const uint64_t* events, uint32_t count, uint32_t neuron_count, uint64_t* grouped,
                         uint32_t* segment_start, void* cuda_stream) {
    if ((count > 0 && (events == nullptr || grouped == nullptr)) || segment_start == nullptr)
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null array");
    if (count > 0 && events < grouped + count && grouped < events + count)
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "events and grouped overlap");
    if (count >= (1u << 31)) return set_error(SNNCUDA_ERR_UNSUPPORTED, "at most 2^31-1 events");
    if (bucket_shift_for(neuron_count) == 0) return set_error(SNNCUDA_ERR_UNSUPPORTED, "at most 2^28 neurons");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    std::vector<void*> owned;
    const int rc = guarded([&] {
        const uint32_t buckets = group_buckets(neuron_count);
        GroupScratch sc;
        sc.bcnt = dalloc<uint32_t>(owned, static_cast<size_t>(kGroupGrid) * buckets);
        sc.btot = dalloc<uint32_t>(owned, buckets);
        sc.bstart = dalloc<uint32_t>(owned, static_cast<size_t>(buckets) + 1);
        sc.bcur = dalloc<uint32_t>(owned, buckets);
        sc.grp_tmp = dalloc<BucketEntry>(owned, count);
        sc.slot_count = dalloc<uint32_t>(owned, 1);
        sc.ts = dalloc<TickState>(owned, 1);
        group_run(events, count, neuron_count, grouped, segment_start, st, sc);
    });
    if (rc != SNNCUDA_OK) cudaStreamSynchronize(st);
    for (void* p : owned) cudaFree(p);
    return rc;
}

namespace {

// Static scratch of snncuda_group_events_static: bucket counters and the
// bucket-ordered events for at most kStaticEvents events over kStaticNeurons
// neurons (about 17 MB).
constexpr size_t kStaticEvents = SNNCUDA_GROUP_STATIC_MAX_EVENTS;
constexpr size_t kStaticNeurons = SNNCUDA_GROUP_STATIC_MAX_NEURONS;
constexpr size_t kStaticBuckets = (kStaticNeurons + 255) / 256;  // bucket_shift_for(2^18) == 8
static_assert(kStaticBuckets <= kMaxBuckets, "static grouping buckets");
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffBcnt = 0;
constexpr size_t kOffBtot = kOffBcnt + align256(kGroupGrid * kStaticBuckets * 4);
constexpr size_t kOffBstart = kOffBtot + align256(kStaticBuckets * 4);
constexpr size_t kOffBcur = kOffBstart + align256((kStaticBuckets + 1) * 4);
constexpr size_t kOffGrpTmp = kOffBcur + align256(kStaticBuckets * 4);
constexpr size_t kOffSlot = kOffGrpTmp + align256(kStaticEvents * sizeof(BucketEntry));
constexpr size_t kOffTs = kOffSlot + 256;
constexpr size_t kStaticBytes = kOffTs + align256(sizeof(TickState));

static __device__ __align__(256) unsigned char g_group_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of the static scratch on the current device.  Set up on the
// first call on a device, with that device current (cudaGetSymbolAddress may
// load the module then, which a stream capture does not allow).  Later calls
// made outside a stream capture look it up again (a cheap table lookup), so
// the address follows the module if a cudaDeviceReset reloaded it; a call
// inside a capture uses the address of the last call.
unsigned char* static_scratch(cudaStream_t st) {
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) throw_fail(SNNCUDA_ERR_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (g_scratch_addr[dev] != nullptr) check(cudaStreamIsCapturing(st, &cap), "cudaStreamIsCapturing");
    if (g_scratch_addr[dev] == nullptr || cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        check(cudaGetSymbolAddress(&p, g_group_scratch), "cudaGetSymbolAddress");
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_addr[dev];
}

}  // namespace

int snncuda_group_events_static(const uint64_t* events, uint32_t count, uint32_t neuron_count,
                                uint64_t* grouped, uint32_t* segment_start, void* cuda_stream) {
    if ((count > 0 && (events == nullptr || grouped == nullptr)) || segment_start == nullptr)
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null array");
    if (count > 0 && events < grouped + count && grouped < events + count)
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "events and grouped overlap");
    if (count > kStaticEvents || neuron_count > kStaticNeurons)
        return set_error(SNNCUDA_ERR_CAPACITY,
                         "snncuda_group_events_static handles at most 2^20 events and 2^18 neurons; "
                         "use snncuda_group_events");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const int rc = guarded([&] {
        unsigned char* base = static_scratch(st);
        GroupScratch sc;
        sc.bcnt = reinterpret_cast<uint32_t*>(base + kOffBcnt);
        sc.btot = reinterpret_cast<uint32_t*>(base + kOffBtot);
        sc.bstart = reinterpret_cast<uint32_t*>(base + kOffBstart);
        sc.bcur = reinterpret_cast<uint32_t*>(base + kOffBcur);
        sc.grp_tmp = reinterpret_cast<BucketEntry*>(base + kOffGrpTmp);
        sc.slot_count = reinterpret_cast<uint32_t*>(base + kOffSlot);
        sc.ts = reinterpret_cast<TickState*>(base + kOffTs);
        group_run(events, count, neuron_count, grouped, segment_start, st, sc);
    });
    // a failed call may have left kernels writing the shared scratch and the
    // caller's buffers: they finish before the caller's next call can start
    if (rc != SNNCUDA_OK) cudaStreamSynchronize(st);
    return rc;
}

int snncuda_sim_read_raster(snncuda_sim* sim, uint64_t first, uint64_t count, uint64_t* ticks, uint32_t* neurons) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] {
        resident(sim);
        const TickState ts = sim->read_ts();
        const uint64_t have = std::min<uint64_t>(ts.raster_count, sim->e.raster_cap);
        if (first + count > have) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "raster range out of bounds");
        const std::vector<uint32_t> r = sim->d2h(sim->e.raster + 2 * first, 2 * count);
        for (uint64_t i = 0; i < count; ++i) {
            if (ticks) ticks[i] = r[2 * i];
            if (neurons) neurons[i] = r[2 * i + 1];
        }
    });
}


int snncuda_sim_recognition(snncuda_sim* sim, uint64_t* neuron_matches, uint64_t* synapse_code_matches) {
    if (sim == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null sim");
    return guarded([&] {
        resident(sim);
        cudaStream_t st = sim->stream;
        unsigned long long* d = nullptr;
        check(cudaMallocAsync(&d, 5 * sizeof(unsigned long long), st), "device allocation");
        unsigned long long c[5] = {};
        cudaError_t err = cudaMemsetAsync(d, 0, sizeof(c), st);
        if (err == cudaSuccess) {
            launch_range_counts(sim->e, 0, sim->N, 0, sim->S, d, st);
            err = cudaGetLastError();
        }
        if (err == cudaSuccess) err = cudaMemcpyAsync(c, d, sizeof(c), cudaMemcpyDeviceToHost, st);
        cudaFreeAsync(d, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
        check(err, "recognition sums");
        if (neuron_matches) *neuron_matches = c[3];
        if (synapse_code_matches) *synapse_code_matches = c[4];
    });
}

// ---------------------------------------------------------------------------
// batched form: the networks of a batch are one disjoint union inside a
// single simulation.  Network i owns neurons [nbase[i], nbase[i+1]) and
// Connectome synapses [sbase[i], sbase[i+1]); since its synapses only target
// its own neurons, its target-major synapses are one range too.  Nothing in a
// tick couples two networks: each target's events keep their network's own
// order (fires in due order, expansion in Connectome x offset order, the
// network's injections in call order), so every network follows its solo
// trajectory exactly.
// ---------------------------------------------------------------------------

struct snncuda_batch {
    snncuda_sim* sim{nullptr};
    uint32_t count{0};
    std::vector<uint32_t> nbase;                   // [count + 1]
    std::vector<uint64_t> sbase;                   // [count + 1]
    std::vector<std::vector<uint64_t>> inj_ticks;  // per network: clamped delivery tick of each injection
    unsigned long long* d_counts{nullptr};         // [5] scratch of launch_range_counts
    ~snncuda_batch() {
        if (d_counts) cudaFree(d_counts);
        delete sim;
    }
    uint64_t tm_begin(uint32_t i) const { return sim->in_ptr[nbase[i]]; }
    uint64_t tm_end(uint32_t i) const { return sim->in_ptr[nbase[i + 1]]; }
};

static snncuda_batch* batch_create_impl(uint32_t count, const snncuda_network* nets, const int32_t* stdp_enabled,
                                        const snncuda_config& cfg) {
    std::unique_ptr<snncuda_batch> b(new snncuda_batch());
    b->count = count;
    b->nbase.assign(count + 1, 0);
    b->sbase.assign(count + 1, 0);
    b->inj_ticks.resize(count);
    uint64_t codes_total = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const snncuda_network& n = nets[i];
        if (static_cast<uint64_t>(b->nbase[i]) + n.neuron_count >= (1u << 31))
            throw_fail(SNNCUDA_ERR_UNSUPPORTED, "at most 2^31-1 neurons per batch");
        b->nbase[i + 1] = b->nbase[i] + n.neuron_count;
        b->sbase[i + 1] = b->sbase[i] + n.synapse_count;
        if (n.code_offset_ptr && n.code_offsets) codes_total += n.code_offset_ptr[n.synapse_count];
    }
    const uint32_t N = b->nbase[count];
    const uint64_t S = b->sbase[count];
    std::vector<float> thr(N), sim_thr(N), w(S), mw(S);
    std::vector<uint64_t> win(N), refs(N), cptr(S + 1, 0);
    std::vector<uint32_t> src(S), tgt(S), dly(S), codes;
    std::vector<uint8_t> comp(S), rec(S), plast(S);
    codes.reserve(codes_total);
    for (uint32_t i = 0; i < count; ++i) {
        const snncuda_network& n = nets[i];
        const uint32_t nb = b->nbase[i];
        const uint64_t sb = b->sbase[i];
        if (n.neuron_count > 0 && (!n.threshold || !n.pattern_window_ticks || !n.similarity_threshold ||
                                   !n.max_reference_patterns))
            throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "neuron parameter arrays are required");
        if (n.synapse_count > 0 && (!n.source || !n.target || !n.weight || !n.max_weight || !n.delay_ticks ||
                                    !n.compartment || !n.receptor || !n.plasticity_enabled))
            throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse arrays are required");
        std::copy(n.threshold, n.threshold + n.neuron_count, thr.begin() + nb);
        std::copy(n.pattern_window_ticks, n.pattern_window_ticks + n.neuron_count, win.begin() + nb);
        std::copy(n.similarity_threshold, n.similarity_threshold + n.neuron_count, sim_thr.begin() + nb);
        std::copy(n.max_reference_patterns, n.max_reference_patterns + n.neuron_count, refs.begin() + nb);
        const bool has_codes = n.code_offset_ptr && n.code_offsets;
        for (uint64_t k = 0; k < n.synapse_count; ++k) {
            if (n.source[k] >= n.neuron_count || n.target[k] >= n.neuron_count)
                throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "synapse endpoint out of range");
            src[sb + k] = nb + n.source[k];
            tgt[sb + k] = nb + n.target[k];
            if (has_codes)
                codes.insert(codes.end(), n.code_offsets + n.code_offset_ptr[k], n.code_offsets + n.code_offset_ptr[k + 1]);
            cptr[sb + k + 1] = codes.size();
        }
        std::copy(n.weight, n.weight + n.synapse_count, w.begin() + sb);
        std::copy(n.max_weight, n.max_weight + n.synapse_count, mw.begin() + sb);
        std::copy(n.delay_ticks, n.delay_ticks + n.synapse_count, dly.begin() + sb);
        std::copy(n.compartment, n.compartment + n.synapse_count, comp.begin() + sb);
        std::copy(n.receptor, n.receptor + n.synapse_count, rec.begin() + sb);
        std::copy(n.plasticity_enabled, n.plasticity_enabled + n.synapse_count, plast.begin() + sb);
    }
    snncuda_network u{N,        thr.data(), win.data(),  sim_thr.data(), refs.data(),  S,
                      src.data(), tgt.data(), w.data(),   mw.data(),      dly.data(),   comp.data(),
                      rec.data(), plast.data(), cptr.data(), codes.data()};
    b->sim = new snncuda_sim();
    create_impl(&u, cfg, b->sim);
    for (uint32_t i = 0; i < count; ++i)
        if (stdp_enabled && !stdp_enabled[i]) launch_rule_off(b->sim->e, b->tm_begin(i), b->tm_end(i), b->sim->stream);
    check(cudaGetLastError(), "batch rule launch");
    check(cudaMalloc(&b->d_counts, 5 * sizeof(unsigned long long)), "cudaMalloc");
    check(cudaStreamSynchronize(b->sim->stream), "batch create synchronize");
    return b.release();
}

// The network's fire records, in order, from the batch's raster.
static void batch_raster(snncuda_batch* b, uint32_t i, std::vector<uint64_t>& ticks, std::vector<uint32_t>& neurons) {
    snncuda_sim* sim = b->sim;
    const TickState ts = sim->read_ts();
    const uint64_t have = std::min<uint64_t>(ts.raster_count, sim->e.raster_cap);
    const std::vector<uint32_t> r = sim->d2h(sim->e.raster, 2 * have);
    ticks.clear();
    neurons.clear();
    for (uint64_t j = 0; j < have; ++j) {
        const uint32_t n = r[2 * j + 1];
        if (n >= b->nbase[i] && n < b->nbase[i + 1]) {
            ticks.push_back(r[2 * j]);
            neurons.push_back(n - b->nbase[i]);
        }
    }
}

int snncuda_batch_create(uint32_t count, const snncuda_network* networks, const int32_t* stdp_enabled,
                         const snncuda_config* config, snncuda_batch** out) {
    if ((count > 0 && networks == nullptr) || out == nullptr)
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_config def;
    snncuda_config_default(&def);
    const snncuda_config& cfg = config ? *config : def;
    snncuda_batch* b = nullptr;
    const int rc = guarded([&] { b = batch_create_impl(count, networks, stdp_enabled, cfg); });
    if (rc == SNNCUDA_OK) *out = b;
    return rc;
}

int snncuda_batch_destroy(snncuda_batch* batch) {
    delete batch;
    return SNNCUDA_OK;
}

int snncuda_batch_inject(snncuda_batch* b, uint32_t network, uint64_t count, const uint32_t* neurons,
                         const uint64_t* ticks, const float* weights) {
    if (b == nullptr || network >= b->count) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "bad batch or network");
    if (count > 0 && (!neurons || !ticks || !weights)) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null array");
    const uint32_t nb = b->nbase[network], nn = b->nbase[network + 1] - nb;
    std::vector<uint32_t> g(count);
    for (uint64_t k = 0; k < count; ++k) {
        if (neurons[k] >= nn) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "inject neuron out of range");
        g[k] = nb + neurons[k];
    }
    const int rc = snncuda_sim_inject(b->sim, count, g.data(), ticks, weights);
    if (rc == SNNCUDA_OK) {
        auto& v = b->inj_ticks[network];
        for (uint64_t k = 0; k < count; ++k) v.push_back(std::max<uint64_t>(ticks[k], b->sim->next_tick));
    }
    return rc;
}

int snncuda_batch_run_until(snncuda_batch* b, uint64_t inclusive_tick) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return snncuda_sim_run_until(b->sim, inclusive_tick);
}

int snncuda_batch_set_plasticity(snncuda_batch* b, int32_t enabled) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return snncuda_sim_set_plasticity(b->sim, enabled);
}

int snncuda_batch_set_temporal_learning(snncuda_batch* b, int32_t enabled) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return snncuda_sim_set_temporal_learning(b->sim, enabled);
}

int snncuda_batch_counters(snncuda_batch* b, uint32_t i, snncuda_counters* out) {
    if (b == nullptr || out == nullptr || i >= b->count) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "bad argument");
    return guarded([&] {
        snncuda_sim* sim = b->sim;
        cudaStream_t st = sim->stream;
        check(cudaMemsetAsync(b->d_counts, 0, 5 * sizeof(unsigned long long), st), "memset");
        launch_range_counts(sim->e, b->nbase[i], b->nbase[i + 1], b->tm_begin(i), b->tm_end(i), b->d_counts, st);
        check(cudaGetLastError(), "count launch");
        unsigned long long c[5];
        check(cudaMemcpyAsync(c, b->d_counts, sizeof(c), cudaMemcpyDeviceToHost, st), "counts");
        const TickState ts = sim->read_ts();  // synchronizes the stream
        uint64_t external = 0;
        for (uint64_t t : b->inj_ticks[i]) external += t < sim->next_tick;
        uint64_t pending = c[2];
        for (size_t k = sim->pend_head; k < sim->pending.size(); ++k) {
            const uint32_t n = static_cast<uint32_t>(sim->pending[k].event) & ~kExternalBit;
            pending += n >= b->nbase[i] && n < b->nbase[i + 1];
        }
        std::vector<uint64_t> rt;
        std::vector<uint32_t> rn;
        batch_raster(b, i, rt, rn);
        out->fired_spikes = c[0];
        out->synaptic_events = c[1];
        out->external_events = external;
        out->delivered_spikes = c[1] + external;
        out->next_tick = sim->next_tick;
        out->pending_events = pending;
        out->raster_count = rt.size();
        out->max_slot_events = ts.max_slot_events;
    });
}

int snncuda_batch_read_neurons(snncuda_batch* b, uint32_t i, const snncuda_neuron_state* out) {
    if (b == nullptr || out == nullptr || i >= b->count) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "bad argument");
    return guarded([&] { read_neurons_range(b->sim, b->nbase[i], b->nbase[i + 1], out); });
}

int snncuda_batch_read_synapses(snncuda_batch* b, uint32_t i, const snncuda_synapse_state* out) {
    if (b == nullptr || out == nullptr || i >= b->count) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "bad argument");
    return guarded([&] { read_synapses_range(b->sim, b->sbase[i], b->sbase[i + 1], b->tm_begin(i), b->tm_end(i), out); });
}

int snncuda_batch_state_digests(snncuda_batch* b, uint64_t* neuron_digests, uint64_t* synapse_digests) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return guarded([&] {
        const HostState h = fetch_all(b->sim, true);
        for (uint32_t i = 0; i < b->count; ++i)
            digest_range(b->sim, h, b->nbase[i], b->nbase[i + 1], b->sbase[i], b->sbase[i + 1],
                         neuron_digests ? neuron_digests + i : nullptr, synapse_digests ? synapse_digests + i : nullptr);
    });
}

int snncuda_batch_state_checksums(snncuda_batch* b, uint64_t* neuron_sums, uint64_t* synapse_sums) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return guarded([&] {
        for (uint32_t i = 0; i < b->count; ++i)
            checksum_range(b->sim, b->nbase[i], b->nbase[i + 1], b->tm_begin(i), b->tm_end(i),
                           neuron_sums ? neuron_sums + i : nullptr, synapse_sums ? synapse_sums + i : nullptr);
    });
}

int snncuda_batch_autotune(snncuda_batch* b, uint64_t probe_ticks, snncuda_tuning* out) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return snncuda_sim_autotune(b->sim, probe_ticks, out);
}

int snncuda_batch_apply_tuning(snncuda_batch* b, const snncuda_tuning* tuning) {
    if (b == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null batch");
    return snncuda_sim_apply_tuning(b->sim, tuning);
}

int snncuda_batch_read_raster(snncuda_batch* b, uint32_t i, uint64_t first, uint64_t count, uint64_t* ticks,
                              uint32_t* neurons) {
    if (b == nullptr || i >= b->count) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "bad argument");
    return guarded([&] {
        std::vector<uint64_t> rt;
        std::vector<uint32_t> rn;
        batch_raster(b, i, rt, rn);
        if (first + count > rt.size()) throw_fail(SNNCUDA_ERR_INVALID_ARGUMENT, "raster range out of bounds");
        for (uint64_t k = 0; k < count; ++k) {
            if (ticks) ticks[k] = rt[first + k];
            if (neurons) neurons[k] = rn[first + k];
        }
    });
}


// ---------------------------------------------------------------------------
// serving: jobs admitted under a device-memory budget, each simulation on its
// own stream, advanced slice by slice so that many run side by side
// ---------------------------------------------------------------------------

// Device bytes of a simulation of `net` (persistent buffers plus the
// transient buffers of creation), from one host pass over its synapses.
static uint64_t estimate_bytes_impl(const snncuda_network* net, const snncuda_config& cfg) {
    const uint64_t N = net->neuron_count, S = net->synapse_count;
    const bool has_codes = net->code_offset_ptr != nullptr && net->code_offsets != nullptr;
    uint64_t pre_total = 0, max_delta = 1, max_code = 0;
    std::vector<uint8_t> present(1u << 20, 0);
    uint64_t D = 0;
    for (uint64_t s = 0; s < S; ++s) {
        const uint64_t k = has_codes ? net->code_offset_ptr[s + 1] - net->code_offset_ptr[s] : 0;
        pre_total += k == 0 ? 1 : k;
        for (uint64_t j = 0; j < (k == 0 ? 1 : k); ++j) {
            const uint64_t c = k ? net->code_offsets[net->code_offset_ptr[s] + j] : 0;
            const uint64_t d = std::max<uint64_t>(1, static_cast<uint64_t>(net->delay_ticks[s]) + c);
            max_code = std::max(max_code, c);
            if (d < present.size() && !present[d]) {
                present[d] = 1;
                ++D;
            }
            max_delta = std::max(max_delta, d);
        }
    }
    uint64_t W = 2;
    while (W <= max_delta) W <<= 1;
    const uint64_t run_budget = cfg.pattern_run_capacity ? cfg.pattern_run_capacity : 4096;
    uint64_t neuron_bytes = 0, refs_max = 1;
    for (uint64_t n = 0; n < N; ++n) {
        const uint64_t window = net->pattern_window_ticks[n], refs = std::max<uint64_t>(1, net->max_reference_patterns[n]);
        refs_max = std::max(refs_max, refs);
        const uint64_t ring = std::min<uint64_t>(refs * (window + 1), std::max<uint64_t>(window + 1, run_budget));
        neuron_bytes += 64 + 64 + 32 + 8 * (window + 1) + sizeof(RefMeta) * refs + 8 * ring + 8 + 4 * (D + 1) + 24;
    }
    uint64_t slot_cap = cfg.slot_event_capacity;
    if (slot_cap == 0) slot_cap = std::min<uint64_t>(1ull << 27, std::max<uint64_t>(1ull << 16, pre_total / 8));
    const uint64_t fire_cap = std::min<uint64_t>(slot_cap, std::max<uint64_t>(65536, 4ull * N));
    const uint64_t lcode = refs_max > 1 ? 2ull * S * refs_max * kMaxExpected : 0;
    // grouping: bucket counters of up to 512 chunks
    const uint64_t buckets = (N + 255) / 256 < kMaxBuckets ? (N + 255) / 256 + 1 : kMaxBuckets;
    const uint64_t persistent = 64 * S + 8 * S + 8 * pre_total + neuron_bytes + lcode +
                                W * slot_cap * 8 + slot_cap * (8 + 16 + 16 + 16 + 4 + 1) + 512 * 4 * buckets +
                                fire_cap * 4 + (fire_cap / 8 + 1) * 12 * std::max<uint64_t>(D, 1) +
                                16 * cfg.raster_capacity + (16u << 20);
    const uint64_t transient = S * (23 + 8 + 12 + 8) + 4 * (has_codes ? net->code_offset_ptr[S] : 0) +
                               N * (16 + 8 + 4 * D) + (4u << 20);
    (void)max_code;
    return persistent + transient;
}

// A job's own copy of its network's arrays (submit copies them, so the
// caller's buffers may go away before the worker thread creates the job).
extern "C++" {
struct NetworkCopy {
    std::vector<float> threshold, similarity, weight, max_weight;
    std::vector<uint64_t> window, refs, code_ptr;
    std::vector<uint32_t> source, target, delay, codes;
    std::vector<uint8_t> compartment, receptor, plastic;

    template <typename T>
    static void take(std::vector<T>& v, const T* p, uint64_t n) {
        if (p) v.assign(p, p + n);
    }
    // The copy, seen as an snncuda_network (null where the caller's was).
    snncuda_network copy_of(const snncuda_network& n) {
        const uint32_t N = n.neuron_count;
        const uint64_t S = n.synapse_count;
        take(threshold, n.threshold, N);
        take(window, n.pattern_window_ticks, N);
        take(similarity, n.similarity_threshold, N);
        take(refs, n.max_reference_patterns, N);
        take(source, n.source, S);
        take(target, n.target, S);
        take(weight, n.weight, S);
        take(max_weight, n.max_weight, S);
        take(delay, n.delay_ticks, S);
        take(compartment, n.compartment, S);
        take(receptor, n.receptor, S);
        take(plastic, n.plasticity_enabled, S);
        const bool codes_given = n.code_offset_ptr != nullptr && n.code_offsets != nullptr;
        if (codes_given) {
            take(code_ptr, n.code_offset_ptr, S + 1);
            take(codes, n.code_offsets, n.code_offset_ptr[S]);
            if (codes.empty()) codes.push_back(0);  // a non-null array of no offsets
        }
        auto at = [](auto& v, const void* orig) { return orig ? v.data() : nullptr; };
        snncuda_network c = n;
        c.threshold = at(threshold, n.threshold);
        c.pattern_window_ticks = at(window, n.pattern_window_ticks);
        c.similarity_threshold = at(similarity, n.similarity_threshold);
        c.max_reference_patterns = at(refs, n.max_reference_patterns);
        c.source = at(source, n.source);
        c.target = at(target, n.target);
        c.weight = at(weight, n.weight);
        c.max_weight = at(max_weight, n.max_weight);
        c.delay_ticks = at(delay, n.delay_ticks);
        c.compartment = at(compartment, n.compartment);
        c.receptor = at(receptor, n.receptor);
        c.plasticity_enabled = at(plastic, n.plasticity_enabled);
        c.code_offset_ptr = codes_given ? code_ptr.data() : nullptr;
        c.code_offsets = codes_given ? codes.data() : nullptr;
        return c;
    }
    void release() { *this = NetworkCopy{}; }
};
}  // extern "C++"

struct ServerJob {
    NetworkCopy arrays;     // owned copy of the network's arrays (freed once created)
    snncuda_network net{};
    snncuda_config cfg{};
    std::vector<uint32_t> inj_n;
    std::vector<uint64_t> inj_t;
    std::vector<float> inj_w;
    uint64_t ticks{0};
    uint64_t bytes{0};
    snncuda_sim* sim{nullptr};
    snncuda_job_result res{};
};

// Jobs are created (host packing, uploads) by a worker thread, so that the
// caller's thread keeps the running jobs' streams fed meanwhile.
struct snncuda_server {
    snncuda_server_config cfg{};
    std::vector<std::unique_ptr<ServerJob>> jobs;
    std::deque<uint64_t> queue;     // submitted, not admitted
    std::vector<uint64_t> running;  // created, advanced by step()
    std::deque<uint64_t> evicted;   // preempted to host memory, waiting to run again
    uint64_t used{0};               // admission estimate of admitted jobs
    uint32_t creating{0};           // admitted, not yet created
    int device{0};
    std::chrono::steady_clock::time_point t0{std::chrono::steady_clock::now()};
    // worker
    std::mutex mu;
    std::condition_variable cv;
    std::deque<uint64_t> to_create;
    std::vector<uint64_t> created;  // with the worker's status in the job
    bool stop{false};
    std::thread worker;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void work() {
        cudaSetDevice(device);
        for (;;) {
            uint64_t id;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv.wait(lock, [&] { return stop || !to_create.empty(); });
                if (stop) return;
                id = to_create.front();
                to_create.pop_front();
            }
            ServerJob& j = *jobs_at(id);
            j.sim = new (std::nothrow) snncuda_sim();
            int rc = j.sim ? SNNCUDA_OK : SNNCUDA_ERR_OUT_OF_MEMORY;
            if (rc == SNNCUDA_OK) rc = guarded([&] { create_impl(&j.net, j.cfg, j.sim); });
            if (rc == SNNCUDA_OK)
                rc = snncuda_sim_inject(j.sim, j.inj_n.size(), j.inj_n.data(), j.inj_t.data(), j.inj_w.data());
            if (rc == SNNCUDA_OK) sort_pending(j.sim);  // host work off the stepping thread
            j.arrays.release();                          // the device holds the network now
            std::lock_guard<std::mutex> lock(mu);
            j.res.error = rc;
            created.push_back(id);
        }
    }
    ServerJob* jobs_at(uint64_t id) {
        std::lock_guard<std::mutex> lock(mu);
        return jobs[id].get();
    }
    ~snncuda_server() {
        {
            std::lock_guard<std::mutex> lock(mu);
            stop = true;
        }
        cv.notify_all();
        if (worker.joinable()) worker.join();
        for (auto& j : jobs)
            if (j->sim) delete j->sim;
    }
};

static void server_finish(snncuda_server* sv, ServerJob& j, int state, int error) {
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        j.res.state = state;
        j.res.error = error;
        j.res.finished_s = sv->now();
    }
    delete j.sim;
    j.sim = nullptr;
    sv->used -= j.bytes;
}

int snncuda_server_create(const snncuda_server_config* config, snncuda_server** out) {
    if (out == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_server* sv = new (std::nothrow) snncuda_server();
    if (sv == nullptr) return set_error(SNNCUDA_ERR_OUT_OF_MEMORY, "host allocation failed");
    if (config) sv->cfg = *config;
    if (sv->cfg.memory_budget_bytes == 0) sv->cfg.memory_budget_bytes = 120ull << 30;
    if (sv->cfg.max_running == 0) sv->cfg.max_running = 64;
    if (sv->cfg.slice_ticks == 0) sv->cfg.slice_ticks = 64;
    const int rc = guarded([&] {
        check(cudaGetDevice(&sv->device), "cudaGetDevice");
        sv->worker = std::thread([sv] { sv->work(); });
    });
    if (rc != SNNCUDA_OK) {
        delete sv;
        return rc;
    }
    *out = sv;
    return SNNCUDA_OK;
}

int snncuda_server_destroy(snncuda_server* server) {
    delete server;
    return SNNCUDA_OK;
}

int snncuda_server_submit(snncuda_server* sv, const snncuda_network* network, const snncuda_config* config,
                          uint64_t inject_count, const uint32_t* neurons, const uint64_t* ticks, const float* weights,
                          uint64_t run_ticks, uint64_t* job_id) {
    if (sv == nullptr || network == nullptr || job_id == nullptr)
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    if (inject_count > 0 && (!neurons || !ticks || !weights)) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null array");
    return guarded([&] {
        std::unique_ptr<ServerJob> j(new ServerJob());
        j->net = j->arrays.copy_of(*network);
        snncuda_config_default(&j->cfg);
        if (config) j->cfg = *config;
        j->cfg.cuda_stream = nullptr;  // every job on a stream of its own
        j->inj_n.assign(neurons, neurons + inject_count);
        j->inj_t.assign(ticks, ticks + inject_count);
        j->inj_w.assign(weights, weights + inject_count);
        j->ticks = run_ticks;
        j->bytes = estimate_bytes_impl(network, j->cfg);
        j->res.state = 0;
        j->res.device_bytes = j->bytes;
        j->res.submitted_s = sv->now();
        std::lock_guard<std::mutex> lock(sv->mu);
        *job_id = sv->jobs.size();
        sv->queue.push_back(sv->jobs.size());
        sv->jobs.push_back(std::move(j));
    });
}

int snncuda_server_step(snncuda_server* sv, uint32_t* active) {
    if (sv == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null server");
    const uint64_t slice = sv->cfg.slice_ticks;
    // advance or retire the running jobs
    for (size_t i = 0; i < sv->running.size();) {
        ServerJob& j = *sv->jobs_at(sv->running[i]);
        bool ready = false, finished = false;
        int rc = guarded([&] {
            ready = run_complete(j.sim, false);
            if (!ready) return;
            if (j.sim->next_tick >= j.ticks) {
                finished = true;
                return;
            }
            run_enqueue(j.sim, std::min<uint64_t>(j.sim->next_tick + slice, j.ticks) - 1, nullptr);
        });
        if (rc == SNNCUDA_OK && finished) {
            rc = snncuda_sim_counters(j.sim, &j.res.counters);
            if (rc == SNNCUDA_OK && sv->cfg.digests)
                rc = snncuda_sim_state_digest(j.sim, &j.res.neuron_digest, &j.res.synapse_digest);
        }
        if (rc != SNNCUDA_OK || finished) {
            server_finish(sv, j, rc == SNNCUDA_OK ? 2 : 3, rc);
            sv->running.erase(sv->running.begin() + static_cast<std::ptrdiff_t>(i));
            continue;
        }
        ++i;
    }
    // jobs the worker has created start running
    std::vector<uint64_t> ready;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        ready.swap(sv->created);
    }
    for (uint64_t id : ready) {
        ServerJob& j = *sv->jobs_at(id);
        sv->creating -= 1;
        int rc;
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            rc = j.res.error;
        }
        if (rc == SNNCUDA_OK && j.ticks > 0)
            rc = guarded([&] { run_enqueue(j.sim, std::min<uint64_t>(slice, j.ticks) - 1, nullptr); });
        if (rc != SNNCUDA_OK) {
            server_finish(sv, j, 3, rc);
            continue;
        }
        j.res.state = 1;
        sv->running.push_back(id);
    }
    // admit queued jobs in submission order while they fit; the worker
    // creates them.  With eviction on, a queued job that does not fit takes
    // the device memory of running jobs with more remaining work than its
    // own (synapses x ticks left), largest first, which wait in host memory
    // until the budget has room again.
    auto remaining = [](const ServerJob& j, uint64_t done) { return (j.ticks - done) * std::max<uint64_t>(1, j.net.synapse_count); };
    while (!sv->queue.empty() && sv->running.size() + sv->creating < sv->cfg.max_running) {
        const uint64_t id = sv->queue.front();
        ServerJob& j = *sv->jobs_at(id);
        if (sv->used + j.bytes > sv->cfg.memory_budget_bytes && (!sv->running.empty() || sv->creating > 0)) {
            if (!sv->cfg.evict) break;
            const uint64_t need = remaining(j, 0);
            std::vector<std::pair<uint64_t, size_t>> cand;  // (remaining work, index in running)
            uint64_t freeable = 0;
            for (size_t i = 0; i < sv->running.size(); ++i) {
                const ServerJob& r = *sv->jobs_at(sv->running[i]);
                const uint64_t left = remaining(r, std::min(r.sim->run_target + 1, r.ticks));
                if (left > need) {
                    cand.emplace_back(left, i);
                    freeable += r.bytes;
                }
            }
            // room after evicting every candidate (or nothing left running)?
            const bool room = sv->used - std::min(sv->used, freeable) + j.bytes <= sv->cfg.memory_budget_bytes ||
                              (cand.size() == sv->running.size() && sv->creating == 0);
            if (cand.empty() || !room) break;
            std::sort(cand.begin(), cand.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
            std::vector<size_t> gone;
            for (const auto& c : cand) {
                if (sv->used + j.bytes <= sv->cfg.memory_budget_bytes) break;
                const uint64_t rid = sv->running[c.second];
                ServerJob& r = *sv->jobs_at(rid);
                const int rc = guarded([&] { evict_impl(r.sim); });
                gone.push_back(c.second);
                if (rc != SNNCUDA_OK) {
                    server_finish(sv, r, 3, rc);
                    continue;
                }
                sv->used -= r.bytes;
                {
                    std::lock_guard<std::mutex> lock(sv->mu);
                    r.res.state = 4;
                    r.res.evictions += 1;
                }
                sv->evicted.push_back(rid);
            }
            std::sort(gone.rbegin(), gone.rend());
            for (size_t g : gone) sv->running.erase(sv->running.begin() + static_cast<std::ptrdiff_t>(g));
            if (sv->used + j.bytes > sv->cfg.memory_budget_bytes && (!sv->running.empty() || sv->creating > 0)) break;
        }
        sv->queue.pop_front();
        j.res.admitted_s = sv->now();
        sv->used += j.bytes;
        sv->creating += 1;
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            sv->to_create.push_back(id);
        }
        sv->cv.notify_one();
    }
    // evicted jobs come back while they fit, the least remaining work first
    // (the rule that preempted them)
    std::stable_sort(sv->evicted.begin(), sv->evicted.end(), [&](uint64_t x, uint64_t y) {
        const ServerJob& a = *sv->jobs[x];
        const ServerJob& b = *sv->jobs[y];
        return remaining(a, a.sim->next_tick) < remaining(b, b.sim->next_tick);
    });
    while (!sv->evicted.empty() && sv->running.size() + sv->creating < sv->cfg.max_running) {
        const uint64_t id = sv->evicted.front();
        ServerJob& j = *sv->jobs_at(id);
        if (sv->used + j.bytes > sv->cfg.memory_budget_bytes && (!sv->running.empty() || sv->creating > 0)) break;
        sv->evicted.pop_front();
        sv->used += j.bytes;
        const int rc = guarded([&] {
            restore_impl(j.sim);
            run_enqueue(j.sim, std::min<uint64_t>(j.sim->next_tick + slice, j.ticks) - 1, nullptr);
        });
        if (rc != SNNCUDA_OK) {
            server_finish(sv, j, 3, rc);
            continue;
        }
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            j.res.state = 1;
        }
        sv->running.push_back(id);
    }
    if (active)
        *active = static_cast<uint32_t>(sv->queue.size() + sv->running.size() + sv->creating + sv->evicted.size());
    return SNNCUDA_OK;
}

int snncuda_server_job(snncuda_server* sv, uint64_t job_id, snncuda_job_result* out) {
    if (sv == nullptr || out == nullptr || job_id >= sv->jobs.size())
        return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "bad server or job");
    std::lock_guard<std::mutex> lock(sv->mu);
    *out = sv->jobs[job_id]->res;
    return SNNCUDA_OK;
}

int snncuda_sim_estimate_bytes(const snncuda_network* network, const snncuda_config* config, uint64_t* bytes) {
    if (network == nullptr || bytes == nullptr) return set_error(SNNCUDA_ERR_INVALID_ARGUMENT, "null argument");
    snncuda_config def;
    snncuda_config_default(&def);
    return guarded([&] { *bytes = estimate_bytes_impl(network, config ? *config : def); });
}

}  // extern "C"
