// Device data layout and kernel interface of the GB300 tick engine.
//
// One simulation = one network resident in HBM:
//   * neurons: NeuronRec (64 B, dynamic state), NeuronTp (32 B, temporal
//     bookkeeping), NeuronParam (64 B, read-only) -- one per neuron;
//   * synapses in target-major order (incoming lists of each target
//     contiguous, Connectome order inside a list), one 64 B record each:
//     SynA (weight, STDP state, static fields) + SynB (code-pattern state,
//     counters), so the per-event work touches one DRAM line per event;
//   * pre-expanded outgoing events: for every source, its (synapse, code
//     offset) events grouped by delivery delay class, each class in
//     Connectome x offset order -- spike-code expansion is then a copy;
//   * a timing wheel of W slots, each a buffer of 64-bit events in exact
//     scheduling order (the reference bucket FIFO order).
#pragma once

#include <cstdint>

namespace snngb {

// Event word: low 32 bits = target neuron, bit 31 set for an external input;
// high 32 bits = target-major synapse index, or the float weight bits of an
// external input.
constexpr uint32_t kExternalBit = 0x80000000u;

// Status bits raised by kernels (host maps them to SNNCUDA_ERR_*).
constexpr uint32_t kStatusSlotOverflow = 1u << 0;
constexpr uint32_t kStatusRingOverflow = 1u << 1;
constexpr uint32_t kStatusRasterOverflow = 1u << 2;
constexpr uint32_t kStatusPostCountOverflow = 1u << 3;
constexpr uint32_t kStatusRunOverflow = 1u << 4;
constexpr uint32_t kStatusFireOverflow = 1u << 5;
constexpr uint32_t kStatusBadEvent = 1u << 6;       // event target out of range (grouping input)
constexpr uint32_t kStatusStageTimeout = 1u << 7;   // a bounded wait for a bulk copy ran out

// SynA.meta bit fields.
constexpr uint32_t kMetaDelayMask = 0xFFFFu;
constexpr int kMetaCompShift = 16;      // 2 bits
constexpr int kMetaRecShift = 18;       // 2 bits
constexpr int kMetaPlasticBit = 20;     // 1 bit
constexpr int kMetaExpectedShift = 21;  // 4 bits: max(2, #code offsets), <= 8
constexpr int kMetaRuleOffBit = 25;     // the synapse's network runs with the STDP rule disabled

constexpr int kMaxExpected = 8;

struct alignas(32) SynA {
    float weight;
    uint32_t last_pre1;   // last_pre_spike_tick + 1, 0 = none
    uint32_t last_post1;  // last_post_spike_tick + 1, 0 = none
    uint32_t meta;
    float clamp_hi;       // min(StdpConfig::max_weight, synapse max_weight)
    uint32_t updates;     // plasticity_update_count
    float last_delta;     // last_weight_delta
    uint32_t post_cnt;    // target fires already applied at tick last_post1-1
};

struct alignas(32) SynB {
    uint32_t pre_count;
    uint32_t code_ws;       // code_window_start_tick
    uint32_t code_matches;  // code_match_count
    uint8_t code_len;       // code_offsets.size() (<= expected)
    uint8_t flags;          // bit 0: last_code_match; bits 4-7: expected = max(2, #code offsets)
    uint16_t learned_count; // learned_code_patterns.size()
    // code_offsets in order, 16 bits each: offsets 0-3 in ring_lo, 4-7 in
    // ring_hi.  When the target keeps a single reference pattern and no code
    // has more than 4 offsets (inline_code_pattern), ring_hi instead holds the
    // synapse's one learned code pattern.
    unsigned long long ring_lo;
    unsigned long long ring_hi;
};

struct alignas(64) SynAB {
    SynA a;
    SynB b;
};

// Per-event input of the neuron walk, written by k_events in due order inside
// every target's group: the weight after the event's pre-spike STDP (computed
// as if the target had not fired earlier in the tick), compartment, receptor
// and flags, the synapse and the due position.
struct alignas(16) EvIn {
    float weight;
    uint32_t bits;  // comp | rec << 2 | external << 4 | repeat << 5
    uint32_t tm;    // target-major synapse index (synaptic events)
    uint32_t due;   // position in the tick's due list
};
// The fields of a synapse record that an event's pre-spike work changes, as
// they were before the event (k_events writes one per synaptic event; the
// per-target walk redoes an event that follows a fire of its target from
// them and the record's other fields, which that work does not change).
struct alignas(16) SynPre {
    float weight;
    uint32_t last_pre1;
    uint32_t updates;
    float last_delta;
};
constexpr uint32_t kEvExternal = 1u << 4;
constexpr uint32_t kEvRepeat = 1u << 5;  // not the first event of its synapse in this tick

__host__ __device__ inline bool inline_code_pattern(uint32_t max_refs, uint32_t code_stride) {
    return max_refs == 1 && code_stride <= 4;
}

__host__ __device__ inline uint32_t ring_get(unsigned long long lo, unsigned long long hi, uint32_t j) {
    return static_cast<uint32_t>((j < 4 ? lo >> (16 * j) : hi >> (16 * (j - 4))) & 0xFFFFu);
}

struct alignas(64) NeuronRec {
    float cur[4];          // soma, basal, apical, inhibitory current
    uint32_t upd[4];       // compartment last_update_tick
    float membrane;
    uint32_t spike_count;
    uint32_t last_fired1;  // last_fired_tick + 1, 0 = none
    uint32_t last_active;
    uint32_t flags;        // 4 x 2-bit tau code
    // temporal pattern fields (written by k_temporal only)
    uint32_t match_count;
    uint32_t ws;           // temporal window_start_tick
    uint32_t len;          // spike_offsets.size()
};

struct alignas(32) NeuronTp {
    unsigned long long cn;  // sum of squares of the current window's offsets
    uint32_t nruns;         // runs in the current window's run list
    uint32_t ref_head;      // FIFO index of the oldest learned pattern
    uint32_t ref_count;
    uint32_t ring_head;     // next free run slot of the learned-pattern run ring
    uint32_t ring_used;
    uint32_t last_match;    // temporal_pattern.last_match
};

struct alignas(64) NeuronParam {
    float threshold;
    uint32_t window;        // pattern_window_ticks
    float similarity;
    uint32_t max_refs;      // max_reference_patterns
    uint32_t ring_cap;      // runs in the learned-pattern ring
    uint32_t pad;
    unsigned long long in_begin;    // first target-major synapse index
    unsigned long long cand_base;   // run list of the current window (window+1 runs)
    unsigned long long meta_base;   // max_refs RefMeta entries
    unsigned long long ring_base;   // ring_cap runs
    unsigned long long lcode_base;  // learned code patterns of the incoming synapses
};

// A learned temporal pattern: runs in the neuron's ring plus the running
// prefix sums of its cosine against the current window.
struct alignas(16) RefMeta {
    unsigned long long dot, rn, cn;  // exact integer sums over min(len, window length)
    uint32_t start;                  // first run (ring position)
    uint32_t nruns;
    uint32_t len;                    // pattern length
    uint32_t cur_run;                // cursor into the pattern (run, position)
    uint32_t cur_pos;
    uint32_t match;                  // 0 no, 1 yes, 2 unknown (recompute from sums)
};

// A run of equal offsets: value in the low 16 bits, count in the high 48.
__host__ __device__ inline uint32_t run_value(unsigned long long r) { return static_cast<uint32_t>(r & 0xFFFFu); }
__host__ __device__ inline unsigned long long run_count(unsigned long long r) { return r >> 16; }

// Per-tick scratch and counters that live on the device.
struct TickState {
    unsigned long long delivered;
    unsigned long long external;
    unsigned long long fired;
    unsigned long long max_slot_events;
    unsigned long long raster_count;
    unsigned long long touched_total;  // sum of n_touched over ticks
    uint32_t status;
    uint32_t tick;            // tick being processed
    uint32_t n_due;           // events due this tick
    uint32_t n_touched;       // targets with at least one due event
    uint32_t n_fires;         // fires this tick
    uint32_t n_fired_targets; // distinct targets that fired this tick (reset by k_bcount)
    uint32_t post_tick;       // tick of the pending post-spike STDP (set by k_bcount; read by k_post)
    uint32_t expand_fires;    // fires whose events k_expand copies
    uint32_t far_first_tick;  // delivery tick of far_idx[0] for the current run
    uint32_t far_ticks;       // entries of far_idx minus one (0 = none)
    int32_t stdp_enabled;     // StdpRule::enabled (runtime toggle)
    int32_t temporal_enabled; // SynapseDendriteConfig::temporal_learning_enabled
    uint32_t done_scan;       // "last block" counters
    uint32_t done_fire_list;
};

struct Tables {
    const float* decay;     // [4][decay_len]: expf(-e / tau_k), e = 0..decay_len-1
    uint32_t decay_len;
    const float* ltp;       // [stdp_len]: A+ expf(-dt / tau+)
    const float* ltd;       // [stdp_len]: -A- expf(-dt / tau-)
    uint32_t stdp_len;
};

// Everything a tick needs, passed by value to the kernels.
// One due event placed in its bucket by k_bscatter: the due-list word with
// its due index in the low bits (payload << 32 | due index | external bit)
// and its target within the bucket.  16 bytes, so the scattered placement is
// one store per event.
struct alignas(16) BucketEntry {
    unsigned long long ev;
    uint32_t ltgt;
    uint32_t unused;
};

struct Engine {
    uint32_t N;
    uint32_t W;             // wheel slots (power of two)
    uint32_t wmask;
    uint32_t D;             // delay classes
    unsigned long long S;
    unsigned long long slot_cap;
    uint32_t code_stride;   // max expected over the network
    unsigned long long raster_cap;
    uint32_t fire_cap;
    uint32_t fire_tiles_cap;
    float min_weight;
    unsigned long long stage_wait_ns;  // limit of k_process's wait for its staged event inputs

    // network
    const unsigned long long* in_ptr;      // [N+1] target-major row pointers
    const NeuronParam* nparam;             // [N]
    NeuronRec* nrec;                       // [N]
    NeuronTp* ntp;                         // [N]
    unsigned long long* cand;              // run lists of current windows
    RefMeta* refmeta;
    unsigned long long* ring;              // learned-pattern runs
    SynAB* syn;                            // [S] target-major
    uint16_t* lcode;                       // learned code patterns
    const unsigned long long* pre_base;    // [N] first pre-expanded event of a source
    const uint32_t* pre_off;               // [N*(D+1)] class offsets within a source
    const unsigned long long* pre_ev;      // pre-expanded events
    const uint32_t* cls_delta;             // [D] delivery delay of each class (>= 1)

    // wheel
    unsigned long long* wheel;             // [W * slot_cap]
    uint32_t* slot_count;                  // [W]

    // per-tick scratch: grouping by target.  Targets are bucketed by
    // bucket_shift (2^bucket_shift consecutive targets per bucket, at most
    // kMaxBuckets buckets); grid_bucket blocks each count and place one
    // contiguous chunk of the due list.
    uint32_t bucket_shift;
    uint32_t nbuckets;
    uint32_t grid_bucket;
    // Due-list events per placing pass of k_bscatter (0: one pass): a due
    // list longer than this is placed in passes over disjoint bucket ranges,
    // so the lines of grp_tmp being filled stay in L2 until
    // complete instead of going to DRAM half-written.
    uint32_t scatter_pass_events;
    // 1: k_temporal and k_post run on the main stream in tick order instead
    // of on the side stream beside k_events / k_process and beside the fire
    // ordering (two random-access kernels side by side can take longer than
    // one after the other).
    uint32_t side_serial;
    uint32_t* bcnt;                        // [grid_bucket][nbuckets] events of each (chunk, bucket)
    uint32_t* btot;                        // [nbuckets] events per bucket (zero between ticks)
    uint32_t* bstart;                      // [nbuckets + 1] first grouped position of each bucket
    uint32_t* bcur;                        // [nbuckets] placement cursor of each bucket
    uint32_t* seg_start;                   // [N + 1] first grouped position of each target
    unsigned long long* grp;               // [slot_cap] due events grouped by target, due order inside
                                           // a target: (payload << 32) | (due index | ext << 31)
    BucketEntry* grp_tmp;                  // [slot_cap] the due events in bucket order (unsorted inside)
    EvIn* evin;                            // [slot_cap] per-event inputs of k_process, grouped, due order
    SynPre* ev_a0;                         // [slot_cap] each synaptic event's changing fields before it
    uint32_t* fire_bits;                   // [slot_cap/32] bitmap of due positions that fired
    uint32_t* fire_at;                     // [slot_cap] firing neuron at a due position
    uint32_t* fire_tile;                   // fires per bitmap tile of kThreads words (zero between ticks)
    uint32_t* fire_list;                   // [fire_cap] firing neurons in reference order
    uint32_t* fired_tgt;                   // [N] targets that fired this tick
    uint32_t* fired_cnt;                   // [N] their fire counts
    uint32_t* xsum;                        // [fire_cap/8][D] events per (expansion block, class)
    unsigned long long* xdst;              // [fire_cap/8][D] wheel position of each
    uint32_t* xdst_ok;                     // [D] class destination fits its slot
    uint32_t* raster;                      // [raster_cap * 2] (tick, neuron)

    // far-future injections for the current run (see TickState)
    const unsigned long long* far_ev;
    const uint32_t* far_idx;

    TickState* ts;
    Tables tab;

    // launch shapes (results do not depend on them; snncuda_sim_autotune
    // picks grid_events, grid_walk, grid_bucket and grid_process)
    uint32_t grid_wide;
    uint32_t grid_process;  // k_temporal blocks
    uint32_t grid_walk;     // k_process blocks
    uint32_t grid_fire;
    uint32_t grid_events;   // k_events blocks
};

constexpr uint32_t kMaxBuckets = 16384;   // target buckets of the grouping (shared-memory counters)
constexpr uint32_t kScatterPassEvents = 1u << 22;  // default Engine::scatter_pass_events (64 MB of grp_tmp)
constexpr uint32_t kMaxBucketShift = 14;  // at most 2^14 targets per bucket: N <= 2^28

// Targets per bucket (log2) for N targets: the smallest 2^s >= 256 with at
// most kMaxBuckets buckets.  Returns 0 when N needs more than 2^28 targets.
__host__ __device__ inline uint32_t bucket_shift_for(uint32_t N) {
    uint32_t s = 8;
    while (((static_cast<unsigned long long>(N) + (1ull << s) - 1) >> s) > kMaxBuckets) ++s;
    return s <= kMaxBucketShift ? s : 0;
}
constexpr int kExpandFires = 8;          // fires per expansion block (one warp each)
constexpr uint32_t kMaxClasses = 256;    // distinct delivery delays

// Host-side launchers (kernels.cu).
// `marks` (optional) holds 2 * kKernelCount events recorded around every
// kernel (before, after) for profiling graphs.
constexpr int kKernelCount = 10;
// The streams of a tick: k_temporal and k_post run on `side`, forked from
// `main` with ev[0] / ev[2] and joined back with ev[1] / ev[3].
struct TickStreams {
    cudaStream_t main;
    cudaStream_t side;
    cudaEvent_t ev[4];
};
void launch_tick(const Engine& e, const TickStreams& s, cudaEvent_t* marks = nullptr);
const char* kernel_name(int index);
void launch_inject(const Engine& e, const unsigned long long* ev, const uint32_t* slot_of_group,
                   const uint32_t* group_off, uint32_t groups, cudaStream_t stream);
// Groups the W == 1 "wheel" of e (a caller's event buffer) by target: the
// tick's four grouping kernels.
void launch_group(const Engine& e, cudaStream_t stream);
// Batched form: one handle simulates several networks side by side.
// Sets kMetaRuleOffBit on target-major synapses [tm_begin, tm_end).
void launch_rule_off(const Engine& e, unsigned long long tm_begin, unsigned long long tm_end, cudaStream_t stream);
// out[0] += spike counts of neurons [n_begin, n_end); out[1] += pre-spike
// counts of target-major synapses [tm_begin, tm_end); out[2] += wheel events
// (all slots) whose target is in [n_begin, n_end); out[3] += the neurons'
// temporal match counts; out[4] += the synapses' code match counts.  out (5
// entries) must start at zero.
void launch_range_counts(const Engine& e, uint32_t n_begin, uint32_t n_end, unsigned long long tm_begin,
                         unsigned long long tm_end, unsigned long long* out, cudaStream_t stream);
// out[0] += checksum of neurons [n_begin, n_end), out[1] += checksum of
// their incoming synapses, whose target-major range starts at tm_begin
// (k_checksum); out must start at zero.
void launch_checksum(const Engine& e, uint32_t n_begin, uint32_t n_end, unsigned long long tm_begin,
                     unsigned long long* out, cudaStream_t stream);
// One-time kernel attributes (dynamic shared memory of k_process); call with
// the device current before the first tick.
void configure_kernels();
// Builds the synapse records from SynA images (`a`, S entries): code-pattern
// state zeroed, each synapse's `expected` stored.
void launch_init_syn(const Engine& e, const SynA* a, cudaStream_t stream);

}  // namespace snngb
