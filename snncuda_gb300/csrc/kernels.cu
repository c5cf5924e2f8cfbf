// Tick kernels of the GB300 engine (sm_103a).
//
// One tick t processes wheel slot t mod W, whose buffer holds the events due
// at t in the exact order the reference scheduler would pop them
// (SpikeScheduler.cpp:25-47: bucket FIFO order).  Per tick, on the main
// stream:
//
//  1. k_bcount     count due events per bucket of consecutive targets, per
//                   chunk of the due list (and copy far-future injections
//                   that become reachable into the wheel)
//  2. k_bscatter   bucket starts; place every event in its bucket
//  3. k_bsort      per bucket: group by target, segment starts
//  4. k_events     one warp per target with events: restore due order inside
//                  its group, then per synapse (lanes in parallel) the event's
//                  pre-spike STDP, pre-spike count and spike-code pattern
//                  (SynapseDendriteProcessor.cpp:104-133, :318-365); writes
//                  each event's input for the neuron walk
//  5. k_process    one thread per touched target: the neuron's physics over
//                  its events in due order (:175-229), redoing the STDP of
//                  events that follow a fire of the target; fires into a
//                  due-position bitmap
//  6. k_fire_list  fires in due order (= reference fire order), raster
//  7. k_fire_count events per (fire block, delay class); the last block scans
//                  destinations and finishes the tick
//  8. k_expand     copy each fire's pre-expanded (synapse, offset) events into
//                  their delivery slots, order-preserving
//
// and two more, on a second stream (graph fork/join) beside the others, or
// for networks of 2^26+ synapses on the main stream in tick order
// (Engine::side_serial):
//
//  9. k_temporal   the neuron temporal pattern of every touched target, once
//                  per tick, beside 4-5 (or before 4)
// 10. k_post       post-spike STDP over the in-rows of targets that fired
//                  (:138-173), beside 6-8 (or after 5)
//
// Main-stream kernels that directly follow another are launched as
// programmatic dependents (tick_enter), so each is scheduled while the one
// before it drains.
//
// Every wait is a kernel boundary (a programmatic dependent's grid
// dependency wait included), a "last block" hand-off (an atomic counter, no
// spinning) or the time-bounded mbarrier wait of k_process's staging copy,
// so no kernel here can hang.
// Float arithmetic uses explicitly rounded intrinsics so nothing is
// contracted into an FMA: each operation rounds exactly as the reference's
// separately evaluated float expressions.

#include <cuda_runtime.h>

#include "engine.h"

namespace snngb {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kStageEvents = 3584;  // event inputs k_process stages per block (56 KB)
constexpr uint32_t kLtpShared = 2560;    // longest LTP table k_process copies to shared memory (10 KB)
constexpr size_t kProcessSmem = kStageEvents * sizeof(EvIn) + kLtpShared * sizeof(float);
constexpr int kFireCountThreads = 1024;  // k_fire_count's last block scans up to 32 delay classes at once

// Minimum resident blocks per SM requested for k_process and k_events
// (register budget).
#ifndef SNNGB_PROCESS_MIN_BLOCKS
#define SNNGB_PROCESS_MIN_BLOCKS 3
#endif
#ifndef SNNGB_EVENTS_MIN_BLOCKS
#define SNNGB_EVENTS_MIN_BLOCKS 4
#endif

__device__ __forceinline__ float rec_gain(uint32_t r) { return r == 1 ? 0.55f : (r == 3 ? 0.65f : 1.0f); }
__device__ __forceinline__ float rec_sign(uint32_t r) { return r >= 2 ? -1.0f : 1.0f; }

__device__ __forceinline__ void raise_status(const Engine& e, uint32_t bit) { atomicOr(&e.ts->status, bit); }

// First statement of every main-stream tick kernel.  A kernel launched as a
// programmatic dependent of the previous kernel on its stream is scheduled
// while that kernel still runs and waits here until it has completed and its
// writes are visible (for any other launch the wait returns at once); then it
// lets its own dependent be scheduled.  The wait is the hardware's grid
// dependency, not a spin on memory.
__device__ __forceinline__ void tick_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------------------
// bulk copies into shared memory (TMA, cp.async.bulk) with an mbarrier
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: expect `bytes` on the barrier and copy them from global memory
// (16-byte aligned, a multiple of 16 bytes) into shared memory.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long v;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(v));
    return v;
}

// Waits for phase `parity` of the barrier to complete, for at most
// `limit_ns` nanoseconds (and at most 2^24 polls); returns false if it did
// not.  A limit of 0 gives up without polling.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, unsigned long long limit_ns) {
    if (limit_ns == 0) return false;
    const uint32_t a = smem_addr(bar);
    const unsigned long long t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 24); ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && global_ns() - t0 > limit_ns) break;
    }
    return false;
}

// Limit of the wait that drains a bulk copy still in flight before its
// shared-memory buffer is reused or the block exits (1 s: a copy of at most
// 64 KB completes in microseconds).
constexpr unsigned long long kDrainWaitNs = 1000000000ull;

// ---------------------------------------------------------------------------
// block-level helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += n;
    }
    return v;
}

// Exclusive block scan of one value per thread (blockDim.x == kThreads).
// Returns the exclusive prefix; *total receives the block sum.
template <int kBlock>
__device__ uint32_t block_excl_scan_t(uint32_t v, uint32_t* total) {
    constexpr int kWarps = kBlock / 32;
    static_assert(kWarps >= 1 && kWarps <= 32, "block size");
    __shared__ uint32_t warp_sums[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t incl = warp_incl_scan(v);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kWarps ? warp_sums[lane] : 0;
        s = warp_incl_scan(s);
        if (lane < kWarps) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t base = warp > 0 ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[kWarps - 1];
    __syncthreads();
    return base + incl - v;
}

__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) { return block_excl_scan_t<kThreads>(v, total); }

// "Last block" hand-off: returns true in exactly one block, after every
// block's prior global writes are visible.
__device__ bool last_block(uint32_t* counter) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t v = atomicAdd(counter, 1u);
        is_last = (v == gridDim.x - 1);
        if (is_last) *counter = 0;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// ---------------------------------------------------------------------------
// per-event physics
// ---------------------------------------------------------------------------

// Approximate u64 -> f32 (relative error < 2^-22) from 32-bit bit operations.
// Conversions with 64-bit operands run on the FP64 pipe, which GB300 keeps
// small; this estimate only feeds the threshold screen below.
__device__ __forceinline__ float u64_to_f32_approx(unsigned long long x) {
    if (x < (1ull << 23)) return __int_as_float(0x4B000000u | static_cast<uint32_t>(x)) - 8388608.0f;
    const int sh = 41 - __clzll(static_cast<long long>(x));  // x >> sh < 2^23
    const uint32_t m = static_cast<uint32_t>(x >> sh);
    const float f = __int_as_float(0x4B000000u | m) - 8388608.0f;
    return f * __int_as_float((127 + sh) << 23);
}

// The reference's exact expression, in double.  Kept out of line: inlined,
// its 64-bit conversions get hoisted above the branch into every call and
// occupy GB300's small FP64 pipe.
__device__ __noinline__ bool cos_ge_exact(unsigned long long dot, unsigned long long rn, unsigned long long cn,
                                          float sim) {
    const double q = __ddiv_rn(__ull2double_rn(dot),
                               __dmul_rn(__dsqrt_rn(__ull2double_rn(rn)), __dsqrt_rn(__ull2double_rn(cn))));
    return __double2float_rn(q) >= sim;
}

// float(dot / (sqrt(rn) * sqrt(cn))) >= sim for sim > 0
// (TemporalPattern.cpp:35-60, :20-22).  dot, rn, cn are the exact integer
// sums the reference accumulates in double.  A single-precision estimate
// (relative error < 1e-6) decides every case farther than 2e-5 from the
// threshold; the rest take the reference's exact double expression.
__device__ __forceinline__ bool cos_ge(unsigned long long dot, unsigned long long rn, unsigned long long cn,
                                       float sim) {
    if (rn == 0 || cn == 0) return false;  // similarity 0.0f < sim
    const float est = __fmul_rn(__fmul_rn(u64_to_f32_approx(dot), rsqrtf(u64_to_f32_approx(rn))),
                                rsqrtf(u64_to_f32_approx(cn)));
    if (est >= sim * 1.00002f) return true;
    if (est <= sim * 0.99998f) return false;
    return cos_ge_exact(dot, rn, cn, sim);
}

// (a + b) mod m for a < m and b <= m, without an integer division.
__device__ __forceinline__ uint32_t wrap_add(uint32_t a, uint32_t b, uint32_t m) {
    const uint32_t x = a + b;
    return x >= m ? x - m : x;
}

struct NState {
    float cur[4];
    uint32_t upd[4];
    uint32_t flags;  // tau codes (2 bits each); in k_temporal: last_match << 8
    float membrane;
    uint32_t spikes, last_fired1, last_active, match_count, ws, len;
    unsigned long long cn;
    uint32_t nruns, ref_head, ref_count, ring_head, ring_used;
    unsigned long long last_run;  // cand[nruns-1], kept in a register while nruns > 0
    RefMeta one;                  // the learned pattern when max_reference_patterns == 1
    // kOne: the newest pattern's runs are copied into the ring once, at the
    // end of the target's tick (until then nothing reads them)
    bool snap_pending;
    uint32_t snap_nruns;
    unsigned long long snap_last;
};

__device__ __forceinline__ float decay_factor(const Tables& tb, uint32_t code, uint32_t elapsed) {
    const uint32_t i = elapsed < tb.decay_len ? elapsed : tb.decay_len - 1;
    return tb.decay[code * tb.decay_len + i];
}

// SynapseDendriteProcessor.cpp:294-316 (+ :14-41), on the exact run-length
// representation: offsets inside a window never decrease, so the window is
// kept as runs (value, count); learned patterns are run lists in a per-neuron
// ring, each with running integer sums of its cosine against the window.
//
// Applied once per target and tick for all k of its events: every event of
// tick t appends the same offset t - window_start (only the first can restart
// the window), and nothing in the neuron's temporal state feeds the membrane,
// so the reference's per-event sequence of appends is reproduced here in one
// pass.  Once no learned pattern is still being compared element by element
// and a cached result already matches, every remaining append matches too
// (the sums are frozen), which makes the common case O(1) per tick.
// kOne: max_reference_patterns == 1, the single pattern lives in s.one.
template <bool kOne>
__device__ void temporal_tick(NState& s, const NeuronParam& p, uint32_t t, const Engine& e, int enabled,
                              uint32_t k) {
    if (k == 0) return;
    if (!enabled) {
        s.flags &= ~(1u << 8);
        return;
    }
    unsigned long long* cand = e.cand + p.cand_base;
    RefMeta* meta = e.refmeta + p.meta_base;
    unsigned long long* ring = e.ring + p.ring_base;
    auto ref = [&](uint32_t r) -> RefMeta& {
        if constexpr (kOne) {
            return s.one;
        } else {
            return meta[wrap_add(s.ref_head, r, p.max_refs)];
        }
    };
    if (s.len == 0 || t - s.ws > p.window) {
        s.ws = t;
        s.len = 0;
        s.nruns = 0;
        s.cn = 0;
        for (uint32_t r = 0; r < s.ref_count; ++r) {
            RefMeta& m = ref(r);
            m.dot = 0;
            m.rn = 0;
            m.cn = 0;
            m.cur_run = 0;
            m.cur_pos = 0;
            m.match = 2;
        }
    }
    const uint32_t o = t - s.ws;
    const uint32_t oo = o * o;  // o < 2^16, so o * o fits 32 bits
    for (uint32_t j = 0; j < k; ++j) {
        if (s.len >= 1 && s.ref_count > 0 && s.nruns > 0 && run_value(s.last_run) == o) {
            bool frozen = true;
            bool hit = 0.0f >= p.similarity;
            for (uint32_t r = 0; r < s.ref_count; ++r) {
                RefMeta& m = ref(r);
                if (s.len + 1 <= m.len) {
                    frozen = false;
                    break;
                }
                if (!hit) {
                    if (m.match == 2) m.match = cos_ge(m.dot, m.rn, m.cn, p.similarity) ? 1 : 0;
                    hit = m.match == 1;
                }
            }
            if (frozen && hit) {
                const uint32_t n = k - j;
                s.last_run += static_cast<unsigned long long>(n) << 16;
                s.len += n;
                s.cn += static_cast<unsigned long long>(oo) * n;
                s.match_count += n;
                s.flags |= (1u << 8);
                return;
            }
        }
        // one append (spike_offsets.push_back, :309)
        if (s.nruns > 0 && run_value(s.last_run) == o) {
            s.last_run += (1ull << 16);
        } else {
            if (s.nruns > p.window) {  // cannot happen: at most window+1 distinct offsets
                raise_status(e, kStatusRunOverflow);
                return;
            }
            if (s.nruns > 0) cand[s.nruns - 1] = s.last_run;
            s.last_run = static_cast<unsigned long long>(o) | (1ull << 16);
            s.nruns += 1;
        }
        s.len += 1;
        s.cn += oo;
        for (uint32_t r = 0; r < s.ref_count; ++r) {
            RefMeta& m = ref(r);
            if (s.len <= m.len) {
                const unsigned long long run = ring[wrap_add(m.start, m.cur_run, p.ring_cap)];
                const unsigned long long v = run_value(run);
                if (++m.cur_pos == run_count(run)) {
                    m.cur_run += 1;
                    m.cur_pos = 0;
                }
                m.dot += static_cast<uint32_t>(v) * o;  // 16-bit values: 32-bit products
                m.rn += static_cast<uint32_t>(v) * static_cast<uint32_t>(v);
                m.cn += oo;
                m.match = 2;
            }
        }
        bool match = false;
        if (s.ref_count > 0 && s.len >= 2) {
            if (0.0f >= p.similarity) {
                match = true;
            } else {
                for (uint32_t r = 0; r < s.ref_count && !match; ++r) {
                    RefMeta& m = ref(r);
                    if (m.match == 2) m.match = cos_ge(m.dot, m.rn, m.cn, p.similarity) ? 1 : 0;
                    match = m.match == 1;
                }
            }
        }
        if (match) {
            s.flags |= (1u << 8);
            s.match_count += 1;
            continue;
        }
        s.flags &= ~(1u << 8);
        if (s.len < 2) continue;
        // learn_pattern (:31-41): FIFO with max_reference_patterns entries.
        if (s.ref_count >= p.max_refs) {
            s.ring_used -= ref(0).nruns;
            s.ref_head = wrap_add(s.ref_head, 1, p.max_refs);
            s.ref_count -= 1;
        }
        if (s.ring_used + s.nruns > p.ring_cap) {
            raise_status(e, kStatusRingOverflow);
            return;
        }
        const uint32_t start = s.ring_head;
        if constexpr (kOne) {
            s.snap_pending = true;
            s.snap_nruns = s.nruns;
            s.snap_last = s.last_run;
        } else {
            cand[s.nruns - 1] = s.last_run;
            for (uint32_t i = 0; i < s.nruns; ++i) ring[wrap_add(start, i, p.ring_cap)] = cand[i];
        }
        s.ring_head = wrap_add(start, s.nruns, p.ring_cap);
        s.ring_used += s.nruns;
        RefMeta& m = ref(s.ref_count);
        m.dot = s.cn;
        m.rn = s.cn;
        m.cn = s.cn;
        m.start = start;
        m.nruns = s.nruns;
        m.len = s.len;
        m.cur_run = 0;
        m.cur_pos = 0;
        m.match = 2;
        s.ref_count += 1;
    }
}

// The decay step of SynapseDendriteProcessor.cpp:175-229: every compartment
// is brought forward to tick t.  All events of a target in one tick share t,
// so after the first event every compartment is already at t and the step
// does nothing; it is therefore applied once per target and tick, before the
// first event (a fire's reset also leaves every compartment at t).
__device__ __forceinline__ void decay_to(NState& s, uint32_t t, const Engine& e) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (t <= s.upd[k] || s.cur[k] == 0.0f) {
            s.upd[k] = t;
        } else {
            const uint32_t code = (s.flags >> (2 * k)) & 3u;
            s.cur[k] = __fmul_rn(s.cur[k], decay_factor(e.tab, code, t - s.upd[k]));
            s.upd[k] = t;
        }
    }
}

// The rest of SynapseDendriteProcessor.cpp:175-229 for one event at tick t,
// every compartment already at t (decay_to).  Returns whether the neuron
// fired.
__device__ __forceinline__ bool process_input(NState& s, float threshold, uint32_t comp, uint32_t rec, float w,
                                              uint32_t t) {
    const float applied = __fmul_rn(__fmul_rn(w, rec_gain(rec)), rec_sign(rec));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (static_cast<uint32_t>(k) == comp) {
            s.cur[k] = __fadd_rn(s.cur[k], applied);  // its update tick is already t
            s.flags = (s.flags & ~(3u << (2 * k))) | (rec << (2 * k));
        }
    }
    s.last_active = t;  // the temporal-pattern update of this event is done by temporal_tick
    s.membrane = __fadd_rn(__fadd_rn(__fadd_rn(s.cur[0], s.cur[1]), s.cur[2]), s.cur[3]);
    if (s.membrane >= threshold) {
        s.membrane = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s.cur[k] = 0.0f;
            s.upd[k] = t;
        }
        // reset taus: soma AMPA, basal AMPA, apical NMDA, inhibitory GABA_A
        s.flags = (s.flags & ~0xFFu) | (0u << 0) | (0u << 2) | (1u << 4) | (2u << 6);
        s.last_fired1 = t + 1;
        s.spikes += 1;
        return true;
    }
    return false;
}

// StdpRule::weight_delta + apply (STDP.cpp:20-40) and the update bookkeeping
// of SynapseDendriteProcessor.cpp:108-122 / :158-172.  `ltp` is the LTP delta
// table (e.tab.ltp, or k_process's copy of it in shared memory).
__device__ void stdp_apply(SynA& a, uint32_t pre, uint32_t post, const Engine& e, int stdp, const float* ltp) {
    const float before = a.weight;
    float delta = 0.0f;
    if (stdp && !((a.meta >> kMetaRuleOffBit) & 1u)) {
        if (post > pre) {
            const uint32_t dt = post - pre;
            delta = ltp[dt < e.tab.stdp_len ? dt : e.tab.stdp_len - 1];
        } else if (post < pre) {
            const uint32_t dt = pre - post;
            delta = e.tab.ltd[dt < e.tab.stdp_len ? dt : e.tab.stdp_len - 1];
        }
    }
    float v = __fadd_rn(a.weight, delta);
    v = v < e.min_weight ? e.min_weight : (a.clamp_hi < v ? a.clamp_hi : v);
    a.weight = v;
    a.last_delta = __fsub_rn(v, before);
    if (a.last_delta != 0.0f) a.updates += 1;
}

// apply_post_spike_plasticity for every target fire at tick t not yet
// applied to this synapse (fires = target fires so far this tick).
__device__ __forceinline__ bool post_catch_up(SynA& a, uint32_t t, uint32_t fires, const Engine& e, int stdp,
                                              const float* ltp) {
    const uint32_t applied = a.last_post1 == t + 1 ? a.post_cnt : 0u;
    if (fires <= applied) return false;
    const bool plastic = (a.meta >> kMetaPlasticBit) & 1u;
    for (uint32_t k = applied; k < fires; ++k) {
        a.last_post1 = t + 1;
        if (plastic && a.last_pre1 != 0) stdp_apply(a, a.last_pre1 - 1, t, e, stdp, ltp);
    }
    a.post_cnt = fires;
    return true;
}

__device__ __forceinline__ void ring_set(unsigned long long& lo, unsigned long long& hi, uint32_t j,
                                         uint32_t v) {
    if (j < 4) {
        const int sh = 16 * j;
        lo = (lo & ~(0xFFFFull << sh)) | (static_cast<unsigned long long>(v) << sh);
    } else {
        const int sh = 16 * (j - 4);
        hi = (hi & ~(0xFFFFull << sh)) | (static_cast<unsigned long long>(v) << sh);
    }
}

// A learned code pattern of `stride` 16-bit offsets, loaded with the widest
// aligned access the stride allows.
__device__ __forceinline__ void load_pattern(const uint16_t* pat, uint32_t stride, unsigned long long& lo,
                                             unsigned long long& hi) {
    if (stride == 4) {
        lo = *reinterpret_cast<const unsigned long long*>(pat);
        hi = 0;
    } else if (stride == 8) {
        const uint4 v = *reinterpret_cast<const uint4*>(pat);
        lo = (static_cast<unsigned long long>(v.y) << 32) | v.x;
        hi = (static_cast<unsigned long long>(v.w) << 32) | v.z;
    } else if (stride == 2) {
        lo = *reinterpret_cast<const uint32_t*>(pat);
        hi = 0;
    } else {
        lo = hi = 0;
        for (uint32_t j = 0; j < stride; ++j) ring_set(lo, hi, j, pat[j]);
    }
}

__device__ __forceinline__ void store_pattern(uint16_t* pat, uint32_t stride, unsigned long long lo,
                                              unsigned long long hi) {
    if (stride == 4) {
        *reinterpret_cast<unsigned long long*>(pat) = lo;
    } else if (stride == 8) {
        *reinterpret_cast<uint4*>(pat) = make_uint4(static_cast<uint32_t>(lo), static_cast<uint32_t>(lo >> 32),
                                                    static_cast<uint32_t>(hi), static_cast<uint32_t>(hi >> 32));
    } else if (stride == 2) {
        *reinterpret_cast<uint32_t*>(pat) = static_cast<uint32_t>(lo);
    } else {
        for (uint32_t j = 0; j < stride; ++j) pat[j] = static_cast<uint16_t>(ring_get(lo, hi, j));
    }
}

// SynapseDendriteProcessor.cpp:318-365 on a fixed ring of `expected` offsets
// held in two 64-bit words.  `inline_pattern`: the target keeps one reference
// pattern and codes have at most 4 offsets, so the single learned code
// pattern is stored in ring_hi instead of the pattern pool.
// Sum of the squares / of the products of four 16-bit lanes (offsets below
// 2^16: every product fits 32 bits).
__device__ __forceinline__ unsigned long long lanes_dot(unsigned long long a, unsigned long long b) {
    const uint32_t a0 = static_cast<uint32_t>(a), a1 = static_cast<uint32_t>(a >> 32);
    const uint32_t b0 = static_cast<uint32_t>(b), b1 = static_cast<uint32_t>(b >> 32);
    return static_cast<unsigned long long>((a0 & 0xFFFFu) * (b0 & 0xFFFFu)) + ((a0 >> 16) * (b0 >> 16)) +
           static_cast<unsigned long long>((a1 & 0xFFFFu) * (b1 & 0xFFFFu)) + ((a1 >> 16) * (b1 >> 16));
}

// code_update for inline_code_pattern (one reference pattern, at most 4
// offsets): the window is the four 16-bit lanes of ring_lo, the learned
// pattern those of ring_hi; lanes at or above `expected` are always zero, so
// the sums run over all four lanes.
__device__ __forceinline__ void code_update_inline(SynB& b, uint32_t window, float sim, uint32_t t) {
    b.flags &= 0xF0u;  // last_code_match = false
    if (b.code_len == 0 || t - b.code_ws > window) {
        b.code_ws = t;
        b.code_len = 0;
    }
    const uint32_t o = t - b.code_ws;
    const uint32_t expected = b.flags >> 4;
    if (b.code_len < expected) {
        const int sh = 16 * b.code_len;
        b.ring_lo = (b.ring_lo & ~(0xFFFFull << sh)) | (static_cast<unsigned long long>(o) << sh);
        b.code_len += 1;
        if (b.code_len < expected) return;
    } else {
        const int sh = 16 * (expected - 1);
        b.ring_lo = ((b.ring_lo >> 16) & ~(0xFFFFull << sh)) | (static_cast<unsigned long long>(o) << sh);
    }
    bool match = 0.0f >= sim;
    if (!match && b.learned_count > 0)
        match = cos_ge(lanes_dot(b.ring_hi, b.ring_lo), lanes_dot(b.ring_hi, b.ring_hi),
                       lanes_dot(b.ring_lo, b.ring_lo), sim);
    if (match) {
        b.code_matches += 1;
        b.flags |= 1u;
        return;
    }
    b.ring_hi = b.ring_lo;
    b.learned_count = 1;
}

__device__ void code_update(SynB& b, const NeuronParam& p, uint32_t t, uint16_t* lc, uint32_t stride, int enabled,
                            bool inline_pattern) {
    if (inline_pattern) {
        if (enabled) {
            code_update_inline(b, p.window, p.similarity, t);
        } else {
            b.flags &= 0xF0u;
        }
        return;
    }
    b.flags &= 0xF0u;  // last_code_match = false
    if (!enabled) return;
    if (b.code_len == 0 || t - b.code_ws > p.window) {
        b.code_ws = t;
        b.code_len = 0;
    }
    const uint32_t o = t - b.code_ws;
    const uint32_t expected = b.flags >> 4;
    if (b.code_len < expected) {
        ring_set(b.ring_lo, b.ring_hi, b.code_len, o);
        b.code_len += 1;
    } else if (inline_pattern) {  // keep the last `expected` offsets (all in ring_lo)
        b.ring_lo >>= 16;
        ring_set(b.ring_lo, b.ring_hi, expected - 1, o);
    } else {
        b.ring_lo = (b.ring_lo >> 16) | (b.ring_hi << 48);
        b.ring_hi >>= 16;
        ring_set(b.ring_lo, b.ring_hi, expected - 1, o);
    }
    if (b.code_len < expected) return;
    bool match = 0.0f >= p.similarity;
    unsigned long long cn = 0;
    for (uint32_t j = 0; j < expected; ++j) {
        const uint32_t v = ring_get(b.ring_lo, inline_pattern ? 0ull : b.ring_hi, j);
        cn += v * v;  // 16-bit offsets: 32-bit products, 64-bit sums
    }
    for (uint32_t i = 0; i < b.learned_count && !match; ++i) {
        unsigned long long plo, phi = 0;
        if (inline_pattern) {
            plo = b.ring_hi;
        } else {
            load_pattern(lc + static_cast<size_t>(i) * stride, stride, plo, phi);
        }
        unsigned long long dot = 0, rn = 0;
        for (uint32_t j = 0; j < expected; ++j) {
            const uint32_t pv = ring_get(plo, phi, j);
            dot += pv * ring_get(b.ring_lo, inline_pattern ? 0ull : b.ring_hi, j);
            rn += pv * pv;
        }
        match = cos_ge(dot, rn, cn, p.similarity);
    }
    if (match) {
        b.code_matches += 1;
        b.flags |= 1u;
        return;
    }
    if (inline_pattern) {
        b.ring_hi = b.ring_lo;
        b.learned_count = 1;
        return;
    }
    if (b.learned_count >= p.max_refs) {
        for (uint32_t i = 1; i < b.learned_count; ++i)
            for (uint32_t j = 0; j < stride; ++j)
                lc[static_cast<size_t>(i - 1) * stride + j] = lc[static_cast<size_t>(i) * stride + j];
        b.learned_count -= 1;
    }
    store_pattern(lc + static_cast<size_t>(b.learned_count) * stride, stride, b.ring_lo, b.ring_hi);
    b.learned_count += 1;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// ---------------------------------------------------------------------------
// grouping: the tick's due list regrouped by target (ascending), each
// target's events in due order, in four kernels:
//   k_bcount    a block per contiguous chunk of the due list: events per
//               bucket of 2^bucket_shift consecutive targets, counted in
//               shared memory; the block's row of counts goes to bcnt and is
//               added into the bucket totals (one atomic per nonzero bucket)
//   k_bscatter  a block per chunk: the bucket starts (every block scans the
//               totals itself), one reservation per (chunk, bucket), then
//               every event goes to its bucket's range of grp_tmp (order
//               inside a bucket arbitrary)
//   k_bsort     a block per bucket: a counting sort of the bucket's events by
//               target (in shared memory when the bucket fits), segment
//               starts written; inside a target the order stays arbitrary
//               (k_events ranks a target's events by due index, the grouping
//               entry point sorts them with k_segsort)
// Per event that is two or more reads of the due list (k_bscatter places a
// long list in passes over disjoint bucket ranges, so the lines it fills stay
// in L2 until complete), one scattered write, and a coalesced read and write
// per bucket: no per-target global atomics.
// ---------------------------------------------------------------------------

// Block-wide exclusive scan of a[0 .. n) in shared memory (n <= 64 *
// kThreads), in place; returns the total.  Every thread takes a run of
// consecutive entries.
__device__ uint32_t block_scan_shared(uint32_t* a, uint32_t n) {
    const uint32_t per = (n + kThreads - 1) / kThreads;
    const uint32_t b = threadIdx.x * per;
    const uint32_t en = b + per < n ? b + per : n;
    uint32_t sum = 0;
    for (uint32_t i = b; i < en; ++i) sum += a[i];
    uint32_t total;
    uint32_t run = block_excl_scan(sum, &total);
    for (uint32_t i = b; i < en; ++i) {
        const uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
    return total;
}

// The far-future injections whose delivery tick t + W - 1 becomes
// addressable at tick t: far_ev[b, en), for wheel slot `slot`.
__device__ __forceinline__ bool far_range(const Engine& e, uint32_t t, uint32_t& b, uint32_t& en, uint32_t& slot) {
    const uint32_t ft = e.ts->far_ticks;
    if (ft == 0) return false;
    const long long rel = static_cast<long long>(t) + e.W - 1 - e.ts->far_first_tick;
    if (rel < 0 || rel >= ft) return false;
    b = e.far_idx[rel];
    en = e.far_idx[rel + 1];
    slot = (t + e.W - 1) & e.wmask;
    return en > b;
}

// Copies them behind the slot's current events, spread over the whole grid
// (k_bcount; the slot is not the one being grouped, and its count changes
// only in k_bscatter, after every block has copied its share).
__device__ void copy_far_injections(const Engine& e, uint32_t t) {
    uint32_t b, en, slot;
    if (!far_range(e, t, b, en, slot)) return;
    const uint32_t base = e.slot_count[slot];
    if (static_cast<unsigned long long>(base) + (en - b) > e.slot_cap) return;  // k_bscatter raises it
    unsigned long long* dst = e.wheel + static_cast<size_t>(slot) * e.slot_cap + base;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < en - b; i += gridDim.x * blockDim.x)
        dst[i] = e.far_ev[b + i];
}

// Their slot's new count (one thread of k_bscatter).
__device__ void count_far_injections(const Engine& e, uint32_t t) {
    uint32_t b, en, slot;
    if (!far_range(e, t, b, en, slot)) return;
    const uint32_t base = e.slot_count[slot];
    if (static_cast<unsigned long long>(base) + (en - b) > e.slot_cap) {
        raise_status(e, kStatusSlotOverflow);
        return;
    }
    e.slot_count[slot] = base + (en - b);
}

// This block's chunk [beg, end) of a due list of n events.
__device__ __forceinline__ void chunk_of(uint32_t n, uint32_t& beg, uint32_t& end) {
    const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const unsigned long long b = static_cast<unsigned long long>(blockIdx.x) * chunk;
    beg = b < n ? static_cast<uint32_t>(b) : n;
    end = n - beg < chunk ? n : beg + chunk;
}

// Threads of the counting and placing blocks, and the due-list entries each
// thread has in flight per round (independent loads: the kernels stream the
// due list and would otherwise wait a DRAM latency per entry).
constexpr int kBucketThreads = 1024;

// The counting and placing blocks stream their chunk of the due list through
// shared memory: tiles of kStreamTile entries (32 KB) by bulk copy (TMA),
// kStreamBufs copies in flight per block, each waited for at most
// Engine::stage_wait_ns.
constexpr uint32_t kStreamTile = 4096;
constexpr uint32_t kStreamBufs = 2;

struct DueStream {
    unsigned long long* buf;  // kStreamBufs x kStreamTile entries (shared memory)
    unsigned long long* bar;  // kStreamBufs mbarriers (shared memory)
    uint32_t parity;          // bit b: phase buffer b's barrier completes next
    bool staging;             // false after a copy outlived its wait: no more copies
};

// Shared memory of k_bcount / k_bscatter: the bucket counters, then the
// stream's two tiles (16-byte aligned).
__host__ __device__ inline size_t stream_buf_offset(uint32_t nbuckets) {
    return (static_cast<size_t>(nbuckets) * sizeof(uint32_t) + 15) & ~static_cast<size_t>(15);
}

// Calls f(i, src[i]) once for every i in [beg, end), spread over the block's
// threads (every thread of the block must call it: it has block barriers;
// the order of the calls is unspecified).  The 16-byte aligned even-length
// body comes in by bulk copies; an unaligned first entry and an odd last
// entry are read directly.  If a copy outlives
// its wait, the block raises kStatusStageTimeout, drains the copies in
// flight (bounded), and reads the rest from global memory, now and in later
// calls.  Returns false only if a drain also failed (the block must exit).
template <typename F>
__device__ bool stream_due(const Engine& e, const unsigned long long* src, uint32_t beg, uint32_t end, DueStream& s,
                           F&& f) {
    uint32_t a0 = beg;
    if (a0 < end && (reinterpret_cast<uintptr_t>(src + a0) & 15u) != 0) ++a0;
    const uint32_t a1 = a0 + ((end - a0) & ~1u);
    if (threadIdx.x == 0 && beg < a0) f(beg, src[beg]);
    if (threadIdx.x == blockDim.x - 1 && a1 < end) f(a1, src[a1]);
    // Read directly (four loads in flight per thread): a chunk shorter than
    // two tiles, where waiting for a whole tile costs more than it hides, an
    // array that is not even 8-byte aligned, and after a failed copy.
    if (!s.staging || a1 - a0 < 2 * kStreamTile || (reinterpret_cast<uintptr_t>(src + a0) & 15u) != 0) {
        for (uint32_t i0 = a0 + threadIdx.x; i0 < a1; i0 += 4 * blockDim.x) {
            unsigned long long v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t i = i0 + u * blockDim.x;
                v[u] = i < a1 ? __ldcs(src + i) : 0ull;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + u * blockDim.x < a1) f(i0 + u * blockDim.x, v[u]);
        }
        return true;
    }
    const uint32_t ntiles = (a1 - a0 + kStreamTile - 1) / kStreamTile;
    auto tile_len = [&](uint32_t k) {
        const uint32_t st = a0 + k * kStreamTile;
        return a1 - st < kStreamTile ? a1 - st : kStreamTile;
    };
    auto issue = [&](uint32_t k) {
        const uint32_t b = k % kStreamBufs;
        bulk_load(s.buf + b * kStreamTile, src + a0 + k * kStreamTile,
                  tile_len(k) * static_cast<uint32_t>(sizeof(unsigned long long)), &s.bar[b]);
    };
    if (threadIdx.x == 0)
        for (uint32_t k = 0; k < kStreamBufs && k < ntiles; ++k) issue(k);
    for (uint32_t k = 0; k < ntiles; ++k) {
        const uint32_t b = k % kStreamBufs;
        const uint32_t st = a0 + k * kStreamTile;
        const uint32_t cnt = tile_len(k);
        // one thread polls the barrier; the block barrier then orders its
        // observation of the completed copy before every thread's reads
        bool ready = true;
        if (threadIdx.x == 0) ready = mbar_wait(&s.bar[b], (s.parity >> b) & 1u, e.stage_wait_ns);
        if (!__syncthreads_and(ready)) {
            // tiles k .. k + kStreamBufs - 1 (those that exist) are still in
            // flight: drain them before the block goes on without shared memory
            bool drained = true;
            if (threadIdx.x == 0) raise_status(e, kStatusStageTimeout);
            for (uint32_t j = 0; j < kStreamBufs && k + j < ntiles; ++j) {
                const uint32_t bj = (k + j) % kStreamBufs;
                if (threadIdx.x == 0) drained = mbar_wait(&s.bar[bj], (s.parity >> bj) & 1u, kDrainWaitNs) && drained;
                s.parity ^= 1u << bj;
            }
            if (!__syncthreads_and(drained)) return false;
            s.staging = false;
            for (uint32_t i = st + threadIdx.x; i < a1; i += blockDim.x) f(i, __ldcs(src + i));
            return true;
        }
        const unsigned long long* tile = s.buf + b * kStreamTile;
        for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) f(st + i, tile[i]);
        s.parity ^= 1u << b;
        __syncthreads();  // the buffer is read: it may take tile k + kStreamBufs
        if (threadIdx.x == 0 && k + kStreamBufs < ntiles) issue(k + kStreamBufs);
    }
    return true;
}

__global__ void __launch_bounds__(kBucketThreads) k_bcount(Engine e) {
    tick_enter();
    extern __shared__ __align__(16) uint32_t s_hist[];  // [nbuckets], then the stream's tiles
    __shared__ unsigned long long s_bar[kStreamBufs];
    const uint32_t t = e.ts->tick;
    copy_far_injections(e, t);
    const uint32_t B = e.nbuckets;
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) s_hist[b] = 0;
    if (threadIdx.x == 0)
        for (uint32_t j = 0; j < kStreamBufs; ++j) mbar_init(&s_bar[j], 1);
    __syncthreads();
    const uint32_t slot = t & e.wmask;
    const uint32_t n = e.slot_count[slot];
    const unsigned long long* ev = e.wheel + static_cast<size_t>(slot) * e.slot_cap;
    uint32_t beg, end;
    chunk_of(n, beg, end);
    DueStream ds{reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(s_hist) + stream_buf_offset(B)),
                 s_bar, 0u, true};
    uint32_t ext = 0;
    const bool ok = stream_due(e, ev, beg, end, ds, [&](uint32_t, unsigned long long v) {
        const uint32_t lo = static_cast<uint32_t>(v);
        const uint32_t tgt = lo & ~kExternalBit;
        if (tgt >= e.N) {  // only reachable through snncuda_group_events with bad input
            raise_status(e, kStatusBadEvent);
            return;
        }
        atomicAdd(&s_hist[tgt >> e.bucket_shift], 1u);
        ext += lo >> 31;
    });
    // (if a drain failed the counts are partial and the tick is already
    // flagged; the row is still written, and k_bscatter / k_bsort keep every
    // access in bounds whatever the counts)
    (void)ok;
    ext = __reduce_add_sync(0xffffffffu, ext);
    if ((threadIdx.x & 31) == 0 && ext) atomicAdd(&e.ts->external, static_cast<unsigned long long>(ext));
    __syncthreads();
    uint32_t* row = e.bcnt + static_cast<size_t>(blockIdx.x) * B;
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) {
        const uint32_t c = s_hist[b];
        row[b] = c;
        if (c) atomicAdd(&e.btot[b], c);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        e.ts->n_due = n;
        e.ts->post_tick = t;        // the previous tick's k_post has finished
        e.ts->n_fired_targets = 0;
    }
}

__global__ void __launch_bounds__(kBucketThreads) k_bscatter(Engine e) {
    tick_enter();
    extern __shared__ __align__(16) uint32_t s_pos[];  // [nbuckets] next position of this chunk in each bucket
    __shared__ unsigned long long s_bar[kStreamBufs];
    const uint32_t B = e.nbuckets;
    {
        // bucket starts: every block scans the bucket totals itself (a run of
        // consecutive buckets per thread); block 0 publishes them
        const uint32_t per = (B + blockDim.x - 1) / blockDim.x;
        const uint32_t b0 = threadIdx.x * per < B ? threadIdx.x * per : B;
        const uint32_t b1 = b0 + per < B ? b0 + per : B;
        uint32_t sum = 0;
        for (uint32_t b = b0; b < b1; ++b) {
            const uint32_t c = __ldcg(e.btot + b);
            s_pos[b] = c;
            sum += c;
        }
        uint32_t total;
        uint32_t run = block_excl_scan_t<kBucketThreads>(sum, &total);
        for (uint32_t b = b0; b < b1; ++b) {
            const uint32_t c = s_pos[b];
            s_pos[b] = run;
            if (blockIdx.x == 0) e.bstart[b] = run;
            run += c;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            e.bstart[B] = total;
            e.seg_start[e.N] = total;
            count_far_injections(e, e.ts->tick);
        }
        __syncthreads();
    }
    // this chunk's place in each bucket: behind the chunks that reserved
    // before it (the cursors start at zero every tick; k_bsort clears them)
    const uint32_t* row = e.bcnt + static_cast<size_t>(blockIdx.x) * B;
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) {
        const uint32_t c = row[b];
        if (c) s_pos[b] += atomicAdd(&e.bcur[b], c);
    }
    if (threadIdx.x == 0)
        for (uint32_t j = 0; j < kStreamBufs; ++j) mbar_init(&s_bar[j], 1);
    __syncthreads();
    DueStream ds{reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(s_pos) + stream_buf_offset(B)),
                 s_bar, 0u, true};
    const uint32_t slot = e.ts->tick & e.wmask;
    const uint32_t n = e.ts->n_due;
    const unsigned long long* ev = e.wheel + static_cast<size_t>(slot) * e.slot_cap;
    const uint32_t lmask = (1u << e.bucket_shift) - 1u;
    uint32_t beg, end;
    chunk_of(n, beg, end);
    // passes over disjoint bucket ranges (Engine::scatter_pass_events): the
    // due list is streamed again per pass
    const uint32_t per = e.scatter_pass_events;
    const uint32_t passes = per != 0 && n > per ? (n + per - 1) / per : 1u;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        const uint32_t blo = static_cast<uint32_t>(static_cast<unsigned long long>(B) * pass / passes);
        const uint32_t bhi = static_cast<uint32_t>(static_cast<unsigned long long>(B) * (pass + 1) / passes);
        const bool ok = stream_due(e, ev, beg, end, ds, [&](uint32_t i, unsigned long long v) {
            const uint32_t lo = static_cast<uint32_t>(v);
            const uint32_t tgt = lo & ~kExternalBit;
            if (tgt >= e.N) return;
            const uint32_t b = tgt >> e.bucket_shift;
            if (b < blo || b >= bhi) return;
            const uint32_t pos = atomicAdd(&s_pos[b], 1u);
            if (pos >= e.slot_cap) return;  // only after a failed stream (counts partial)
            reinterpret_cast<uint4*>(e.grp_tmp)[pos] =
                make_uint4(i | (lo & kExternalBit), static_cast<uint32_t>(v >> 32), tgt & lmask, 0u);
        });
        if (!ok) return;
    }
}

// Sort key of a grouped entry: its due index (unique within one due list).
__device__ __forceinline__ uint32_t grp_key(unsigned long long v) { return static_cast<uint32_t>(v) & ~kExternalBit; }

// Ascending bitonic sort of one entry per lane by key (lanes without an
// entry carry key 0xFFFFFFFF and sort last).
__device__ __forceinline__ void warp_bitonic(unsigned long long& v, uint32_t& key) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const uint32_t ok = __shfl_xor_sync(0xffffffffu, key, stride);
            const unsigned long long ov = __shfl_xor_sync(0xffffffffu, v, stride);
            const bool up = ((lane & size) == 0);
            const bool lower = (lane & stride) == 0;
            const bool take_min = (lower == up);
            if (take_min ? (ok < key) : (ok > key)) {
                key = ok;
                v = ov;
            }
        }
    }
}

// One warp sorts entries [0, len) of `a` by key into `b` (a is scratch and
// is overwritten).  Runs of 32 are sorted in registers, then runs are merged
// pairwise, doubling their width: an entry's place in the merged run is its
// index in its own run plus the number of keys below it in the other run
// (a binary search; keys are unique).  O(len log^2 len) work per warp, so a
// segment of 2^20 entries takes milliseconds, not the len^2 of a rank count.
__device__ void warp_merge_sort(unsigned long long* a, unsigned long long* b, uint32_t len) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c = 0; c < len; c += 32) {
        const uint32_t n = len - c < 32 ? len - c : 32;
        unsigned long long v = lane < n ? a[c + lane] : ~0ull;
        uint32_t key = lane < n ? grp_key(v) : 0xFFFFFFFFu;
        warp_bitonic(v, key);
        if (lane < n) a[c + lane] = v;
    }
    __syncwarp();
    unsigned long long* src = a;
    unsigned long long* dst = b;
    for (uint32_t w = 32; w < len; w <<= 1) {
        for (uint32_t base = 0; base < len; base += 2 * w) {
            const uint32_t la = len - base < w ? len - base : w;
            const uint32_t lb = len - base - la < w ? len - base - la : w;
            const unsigned long long* L = src + base;
            const unsigned long long* R = L + la;
            for (uint32_t j = lane; j < la + lb; j += 32) {
                const bool left = j < la;
                const unsigned long long v = left ? L[j] : R[j - la];
                const uint32_t key = grp_key(v);
                const unsigned long long* other = left ? R : L;
                uint32_t lo = 0, hi = left ? lb : la;  // keys of `other` below key
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (grp_key(other[mid]) < key) {
                        lo = mid + 1;
                    } else {
                        hi = mid;
                    }
                }
                dst[base + (left ? j : j - la) + lo] = v;
            }
        }
        __syncwarp();
        unsigned long long* t = src;
        src = dst;
        dst = t;
    }
    if (src != b) {
        for (uint32_t j = lane; j < len; j += 32) b[j] = src[j];
        __syncwarp();
    }
}



// Events k_bsort places in shared memory before writing them out; each
// thread holds its share of such a bucket in registers.
constexpr uint32_t kSortSmemEvents = 4096;
constexpr uint32_t kSortPerThread = kSortSmemEvents / kThreads;
constexpr size_t kSortSmemBytes = kSortSmemEvents * sizeof(unsigned long long);

// One block per bucket: a counting sort of the bucket's events by target.
// The events of each target end up contiguous in grp (in arbitrary order;
// k_events ranks them by due index) and the targets' segment starts are
// written.  A bucket of at most kSortSmemEvents events is loaded once into
// registers (every load in flight at once), counted, placed in shared memory
// and written out coalesced; a larger one is counted and placed in grp
// directly from global memory.
__global__ void __launch_bounds__(kThreads) k_bsort(Engine e) {
    tick_enter();
    extern __shared__ __align__(16) unsigned long long s_sort[];  // kSortSmemEvents, then counters
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_sort + kSortSmemEvents);  // [2^bucket_shift]
    const uint32_t width = 1u << e.bucket_shift;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t b = blockIdx.x; b < e.nbuckets; b += gridDim.x) {
        const uint32_t lo = e.bstart[b], hi = e.bstart[b + 1], m = hi - lo;
        const uint32_t n0 = b << e.bucket_shift;
        const uint32_t nw = e.N - n0 < width ? e.N - n0 : width;
        const uint4* in = reinterpret_cast<const uint4*>(e.grp_tmp) + lo;
        const bool small = m <= kSortSmemEvents;
        unsigned long long v[kSortPerThread];
        uint32_t t16[kSortPerThread];
        if (small) {
#pragma unroll
            for (uint32_t k = 0; k < kSortPerThread; ++k) {
                const uint32_t i = threadIdx.x + k * kThreads;
                const uint4 q = i < m ? in[i] : make_uint4(0u, 0u, 0u, 0u);
                t16[k] = q.z;
                v[k] = (static_cast<unsigned long long>(q.y) << 32) | q.x;
            }
        }
        for (uint32_t j = threadIdx.x; j < nw; j += blockDim.x) s_cnt[j] = 0;
        __syncthreads();
        if (small) {
#pragma unroll
            for (uint32_t k = 0; k < kSortPerThread; ++k)
                if (threadIdx.x + k * kThreads < m && t16[k] < nw) atomicAdd(&s_cnt[t16[k]], 1u);
        } else {
            for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
                const uint32_t z = in[i].z;
                if (z < nw) atomicAdd(&s_cnt[z], 1u);
            }
        }
        __syncthreads();
        uint32_t nz = 0;  // targets with events (statistics)
        for (uint32_t j = threadIdx.x; j < nw; j += blockDim.x) nz += s_cnt[j] != 0;
        nz = __reduce_add_sync(0xffffffffu, nz);
        if (lane == 0 && nz) atomicAdd(&e.ts->n_touched, nz);
        block_scan_shared(s_cnt, nw);  // segment starts relative to lo
        for (uint32_t j = threadIdx.x; j < nw; j += blockDim.x) e.seg_start[n0 + j] = lo + s_cnt[j];
        __syncthreads();
        if (threadIdx.x == 0) {  // the bucket's total and cursor start at zero next tick
            e.btot[b] = 0;
            e.bcur[b] = 0;
        }
        if (small) {
#pragma unroll
            for (uint32_t k = 0; k < kSortPerThread; ++k)
                if (threadIdx.x + k * kThreads < m && t16[k] < nw) s_sort[atomicAdd(&s_cnt[t16[k]], 1u)] = v[k];
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) e.grp[lo + i] = s_sort[i];
        } else {
            for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
                const uint4 q = in[i];
                if (q.z < nw) e.grp[lo + atomicAdd(&s_cnt[q.z], 1u)] = (static_cast<unsigned long long>(q.y) << 32) | q.x;
            }
        }
        __syncthreads();
    }
}

// Grouping entry point only: due order inside every target's group of grp
// (one warp per target: up to 32 events bitonic-sorted in registers, longer
// groups merge-sorted with grp_tmp as scratch).
__global__ void __launch_bounds__(kThreads) k_segsort(Engine e) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t n = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); n < e.N; n += warps) {
        const uint32_t beg = e.seg_start[n];
        const uint32_t len = e.seg_start[n + 1] - beg;
        if (len <= 1) continue;
        unsigned long long* g = e.grp + beg;
        if (len <= 32) {
            unsigned long long v = lane < static_cast<int>(len) ? g[lane] : ~0ull;
            uint32_t key = lane < static_cast<int>(len) ? grp_key(v) : 0xFFFFFFFFu;
            warp_bitonic(v, key);
            if (lane < static_cast<int>(len)) g[lane] = v;
        } else {
            unsigned long long* tmp = reinterpret_cast<unsigned long long*>(e.grp_tmp) + beg;
            warp_merge_sort(g, tmp, len);  // sorted into tmp
            for (uint32_t k = lane; k < len; k += 32) g[k] = tmp[k];
            __syncwarp();
        }
    }
}

// Pre-spike part of one synaptic event on its synapse record, in the
// reference's order (SynapseDendriteProcessor.cpp:104-133): pre-spike STDP
// against the last post spike, last_pre, the pre-spike count, and the
// spike-code pattern (:318-365).  None of it depends on the target's neuron
// state; only the STDP part depends on whether the target fired earlier in the
// tick, which k_process handles by redoing it (walk_fired_targets).
__device__ __forceinline__ void pre_event(SynAB& r, const NeuronParam& p, uint32_t t, uint16_t* lc,
                                          const Engine& e, int stdp, int temporal, bool inl) {
    SynA& a = r.a;
    const uint32_t delay = a.meta & kMetaDelayMask;
    const uint32_t pre_tick = t >= delay ? t - delay : t;
    if (((a.meta >> kMetaPlasticBit) & 1u) && a.last_post1 != 0)
        stdp_apply(a, pre_tick, a.last_post1 - 1, e, stdp, e.tab.ltp);
    a.last_pre1 = pre_tick + 1;
    r.b.pre_count += 1;
    code_update(r.b, p, t, lc, e.code_stride, temporal, inl);
}

__device__ __forceinline__ SynPre pre_fields(const SynA& a) {
    SynPre f;
    f.weight = a.weight;
    f.last_pre1 = a.last_pre1;
    f.updates = a.updates;
    f.last_delta = a.last_delta;
    return f;
}

// The record as it was before an event: the fields pre_event changes from
// the event's SynPre, the others (static fields, last_post1, post_cnt) from
// the record, which nothing but the post-spike catch-up changes.
__device__ __forceinline__ SynA before_event(SynA a, const SynPre& f) {
    a.weight = f.weight;
    a.last_pre1 = f.last_pre1;
    a.updates = f.updates;
    a.last_delta = f.last_delta;
    return a;
}

__device__ __forceinline__ uint32_t ev_bits(const SynA& a) {
    return ((a.meta >> kMetaCompShift) & 3u) | (((a.meta >> kMetaRecShift) & 3u) << 2);
}

// All events of synapse tm in one target's group, in due order: `first` is
// the group position of the first, `more(q)` says whether position q > first
// is another one.  Snapshots each event's SynA, applies pre_event and writes
// the event's input record.
template <typename More, typename DueOf>
__device__ __forceinline__ void synapse_events(const Engine& e, const NeuronParam& p, uint32_t beg, uint32_t first,
                                               uint32_t last, uint32_t tm, uint32_t t, int stdp, int temporal,
                                               More more, DueOf due_of) {
    uint16_t* lc = e.lcode + p.lcode_base + static_cast<size_t>(tm - p.in_begin) * p.max_refs * e.code_stride;
    const bool inl = inline_code_pattern(p.max_refs, e.code_stride);
    SynAB r = e.syn[tm];
    for (uint32_t q = first; q <= last; ++q) {
        if (q != first && !more(q)) continue;
        e.ev_a0[beg + q] = pre_fields(r.a);
        pre_event(r, p, t, lc, e, stdp, temporal, inl);
        EvIn in;
        in.weight = r.a.weight;
        in.bits = ev_bits(r.a) | (q != first ? kEvRepeat : 0u);
        in.tm = tm;
        in.due = due_of[q];
        e.evin[beg + q] = in;
    }
    e.syn[tm] = r;
}

// Due position of entry q of a group sorted in memory.
struct SortedDue {
    const unsigned long long* s;
    __device__ uint32_t operator[](uint32_t q) const { return static_cast<uint32_t>(s[q]) & ~kExternalBit; }
};

// One target's group in k_events.  Groups of up to 32 events stay in lanes:
// each event's position in due order is its rank among the group's due
// indices, and the events of each synapse are found with one match; the
// synapse's earliest event's lane then processes all of them in due order.
// Longer groups are merge-sorted into grp_tmp and scanned.
// A synapse with a single event in its target's group this tick: the unit
// of work k_events queues so that all 32 lanes of a warp carry one.
struct EvItem {
    uint32_t tm, pos, due, n;
};

// Pre-spike work of a queued event (one lane).
__device__ __forceinline__ void synapse_item(const Engine& e, const EvItem& it, uint32_t t, int stdp, int temporal) {
    const NeuronParam p = e.nparam[it.n];
    const bool inl = inline_code_pattern(p.max_refs, e.code_stride);
    uint16_t* lc =
        inl ? nullptr : e.lcode + p.lcode_base + static_cast<size_t>(it.tm - p.in_begin) * p.max_refs * e.code_stride;
    SynAB r = e.syn[it.tm];
    e.ev_a0[it.pos] = pre_fields(r.a);
    pre_event(r, p, t, lc, e, stdp, temporal, inl);
    EvIn in;
    in.weight = r.a.weight;
    in.bits = ev_bits(r.a);
    in.tm = it.tm;
    in.due = it.due;
    e.evin[it.pos] = in;
    e.syn[it.tm] = r;
}

__device__ __forceinline__ void events_of_target(const Engine& e, uint32_t n, uint32_t beg, uint32_t len, uint32_t t,
                                                 int stdp, int temporal, uint32_t* wdue, uint32_t* wrank,
                                                 EvItem* queue, uint32_t& qn) {
    const uint32_t lane = threadIdx.x & 31;
    if (len <= 32) {
        const bool valid = lane < len;
        const unsigned long long v = valid ? e.grp[beg + lane] : 0ull;
        const uint32_t lo = static_cast<uint32_t>(v);
        const uint32_t key = lo & ~kExternalBit;
        uint32_t rank = 0;
        for (uint32_t i = 0; i < len; ++i) rank += __shfl_sync(0xffffffffu, key, i) < key;
        const bool syn = valid && !(lo & kExternalBit);
        const uint32_t tm = static_cast<uint32_t>(v >> 32);
        const uint32_t same = __match_any_sync(0xffffffffu, syn ? tm : 0xFFFFFFFFu);
        wdue[lane] = key;
        wrank[lane] = rank;
        __syncwarp();
        if (valid && !syn) {
            EvIn in;
            in.weight = __uint_as_float(tm);
            in.bits = kEvExternal;
            in.tm = 0;
            in.due = key;
            e.evin[beg + rank] = in;
        }
        const bool single = syn && same == (1u << lane);
        const uint32_t qmask = __ballot_sync(0xffffffffu, single);
        if (single) {  // the common case: queued, processed 32 at a time
            EvItem it;
            it.tm = tm;
            it.pos = beg + rank;
            it.due = key;
            it.n = n;
            queue[qn + __popc(qmask & ((1u << lane) - 1u))] = it;
        }
        qn += __popc(qmask);
        bool leader = syn && !single;
        if (leader) {
            for (uint32_t m = same; m; m &= m - 1) leader = leader && wrank[__ffs(m) - 1] >= rank;
        }
        if (leader) {
            const NeuronParam p = e.nparam[n];
            uint16_t* lc = e.lcode + p.lcode_base + static_cast<size_t>(tm - p.in_begin) * p.max_refs * e.code_stride;
            const bool inl = inline_code_pattern(p.max_refs, e.code_stride);
            SynAB r = e.syn[tm];
            uint32_t rest = same, repeat = 0;
            while (rest) {  // the synapse's events in due order (rank order)
                uint32_t j = __ffs(rest) - 1, best = wrank[j];
                for (uint32_t m = rest & (rest - 1); m; m &= m - 1) {
                    const uint32_t c = __ffs(m) - 1;
                    if (wrank[c] < best) {
                        best = wrank[c];
                        j = c;
                    }
                }
                rest &= ~(1u << j);
                e.ev_a0[beg + best] = pre_fields(r.a);
                pre_event(r, p, t, lc, e, stdp, temporal, inl);
                EvIn in;
                in.weight = r.a.weight;
                in.bits = ev_bits(r.a) | repeat;
                in.tm = tm;
                in.due = wdue[j];
                e.evin[beg + best] = in;
                repeat = kEvRepeat;
            }
            e.syn[tm] = r;
        }
        __syncwarp();
        return;
    }
    // grp_tmp is free once the groups are built (16 bytes per event: room for
    // two 8-byte words each)
    unsigned long long* srt = reinterpret_cast<unsigned long long*>(e.grp_tmp) + beg;
    warp_merge_sort(e.grp + beg, srt, len);
    const NeuronParam p = e.nparam[n];
    for (uint32_t j = lane; j < len; j += 32) {
        const unsigned long long x = srt[j];
        const uint32_t lo = static_cast<uint32_t>(x);
        const uint32_t tm = static_cast<uint32_t>(x >> 32);
        if (lo & kExternalBit) {
            EvIn in;
            in.weight = __uint_as_float(tm);
            in.bits = kEvExternal;
            in.tm = 0;
            in.due = lo & ~kExternalBit;
            e.evin[beg + j] = in;
            continue;
        }
        auto same_syn = [&](uint32_t q) {
            const unsigned long long y = srt[q];
            return !(static_cast<uint32_t>(y) & kExternalBit) && static_cast<uint32_t>(y >> 32) == tm;
        };
        bool first = true;
        for (uint32_t q = 0; q < j && first; ++q) first = !same_syn(q);
        if (!first) continue;
        synapse_events(e, p, beg, j, len - 1, tm, t, stdp, temporal, same_syn, SortedDue{srt});
    }
    __syncwarp();
}

// One warp per target with due events (events_of_target).  Synapses with a
// single event this tick go to a per-warp queue in shared memory and are
// processed 32 at a time, one per lane, whatever targets they belong to;
// repeats and long groups are processed in place.
__global__ void __launch_bounds__(kThreads, SNNGB_EVENTS_MIN_BLOCKS) k_events(Engine e) {
    tick_enter();
    __shared__ uint32_t s_due[kThreads], s_rank[kThreads];
    __shared__ EvItem s_queue[kThreads / 32][64];
    const uint32_t t = e.ts->tick;
    const int stdp = e.ts->stdp_enabled;
    const int temporal = e.ts->temporal_enabled;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wbase = threadIdx.x & ~31u;
    EvItem* queue = s_queue[threadIdx.x >> 5];
    uint32_t qn = 0;  // warp-uniform
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t n = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); n < e.N; n += warps) {
        const uint32_t beg = e.seg_start[n];
        const uint32_t end = e.seg_start[n + 1];
        if (end == beg) continue;
        events_of_target(e, n, beg, end - beg, t, stdp, temporal, s_due + wbase, s_rank + wbase, queue, qn);
        if (qn >= 32) {
            __syncwarp();
            synapse_item(e, queue[qn - 32 + lane], t, stdp, temporal);
            qn -= 32;
            __syncwarp();
        }
    }
    __syncwarp();
    if (lane < qn) synapse_item(e, queue[lane], t, stdp, temporal);
}

// The block's event inputs: entries [lo, lo + cnt) of evin staged in shared
// memory once `ready()` returns true; the rest read from global memory.
struct Staged {
    const EvIn* s;
    uint32_t lo, cnt;
    __device__ __forceinline__ EvIn at(const Engine& e, uint32_t g) const {
        const uint32_t o = g - lo;
        return o < cnt ? s[o] : e.evin[g];
    }
};

// Applies to a synapse record the post-spike STDP owed for the target's fires
// so far and the event's pre-spike STDP (the record is the synapse's state
// before the event) and returns the weight the event delivers.  Both STDP
// steps have post >= pre, so they read only the LTP table.
__device__ __forceinline__ float redo_pre_stdp(const Engine& e, SynA& a, uint32_t t, uint32_t fires, int stdp,
                                               const float* ltp) {
    post_catch_up(a, t, fires, e, stdp, ltp);
    const uint32_t delay = a.meta & kMetaDelayMask;
    const uint32_t pre_tick = t >= delay ? t - delay : t;
    if (((a.meta >> kMetaPlasticBit) & 1u) && a.last_post1 != 0)
        stdp_apply(a, pre_tick, a.last_post1 - 1, e, stdp, ltp);
    a.last_pre1 = pre_tick + 1;
    return a.weight;
}

__device__ __forceinline__ SynA shfl_syn(const SynA& a, uint32_t src) {
    SynA r;
    r.weight = __shfl_sync(0xffffffffu, a.weight, src);
    r.last_pre1 = __shfl_sync(0xffffffffu, a.last_pre1, src);
    r.last_post1 = __shfl_sync(0xffffffffu, a.last_post1, src);
    r.meta = __shfl_sync(0xffffffffu, a.meta, src);
    r.clamp_hi = __shfl_sync(0xffffffffu, a.clamp_hi, src);
    r.updates = __shfl_sync(0xffffffffu, a.updates, src);
    r.last_delta = __shfl_sync(0xffffffffu, a.last_delta, src);
    r.post_cnt = __shfl_sync(0xffffffffu, a.post_cnt, src);
    return r;
}

// One target's walk (the reference's sequential per-event loop,
// NetworkPropagator.cpp:80-131, restricted to that target): its neuron state
// and how far the walk has got.
struct Walk {
    NState s;
    float threshold;
    uint32_t n, beg, len;
    uint32_t i;           // next event
    uint32_t fires;       // target fires so far this tick
    uint32_t first_fire;  // event of the first fire
};

// A fire at due position `due`: its bit in the fire bitmap, the neuron, and
// one more fire in the bitmap tile (kThreads words) for k_fire_list.
__device__ __forceinline__ void record_fire(const Engine& e, const Walk& w, uint32_t due) {
    atomicOr(&e.fire_bits[due >> 5], 1u << (due & 31));
    e.fire_at[due] = w.n;
    atomicAdd(&e.fire_tile[(due >> 5) / kThreads], 1u);
}

// Phase 1 of a target's walk: load the neuron (the physics fields only: the
// temporal ones belong to k_temporal, which may be running at the same time)
// and process its events in due order up to and including its first fire.
// Every event before the first fire uses the weight k_events computed.
// Returns whether the target fired.
template <typename Ready>
__device__ __forceinline__ bool walk_to_first_fire(const Engine& e, Walk& w, uint32_t t, Staged& st, Ready ready) {
    NState& s = w.s;
    const NeuronRec* rec = e.nrec + w.n;
    w.threshold = e.nparam[w.n].threshold;
    {
        const float4 c = reinterpret_cast<const float4*>(rec->cur)[0];
        const uint4 u = reinterpret_cast<const uint4*>(rec->upd)[0];
        const uint4 m = *reinterpret_cast<const uint4*>(&rec->membrane);
        s.cur[0] = c.x;
        s.cur[1] = c.y;
        s.cur[2] = c.z;
        s.cur[3] = c.w;
        s.upd[0] = u.x;
        s.upd[1] = u.y;
        s.upd[2] = u.z;
        s.upd[3] = u.w;
        s.membrane = __uint_as_float(m.x);
        s.spikes = m.y;
        s.last_fired1 = m.z;
        s.last_active = m.w;
        s.flags = rec->flags;
    }
    w.fires = 0;
    w.first_fire = 0;
    if (w.len > 0) decay_to(s, t, e);
    if (!ready()) st.cnt = 0;
    for (uint32_t i = 0; i < w.len; ++i) {
        const EvIn x = st.at(e, w.beg + i);
        if (process_input(s, w.threshold, x.bits & 3u, (x.bits >> 2) & 3u, x.weight, t)) {
            record_fire(e, w, x.due);
            w.fires = 1;
            w.first_fire = i;
            w.i = i + 1;
            return true;
        }
    }
    w.i = w.len;
    return false;
}

// Phase 2, one warp: the rest of the walks of its lanes' fired targets, one
// target at a time.  Every synaptic event after a fire redoes its STDP with
// the target's fire count so far, starting from the synapse's state before
// the event: k_events' snapshot, or, when the same synapse already had an
// event after the first fire, the record that event left.  The warp redoes up
// to 32 events at once (an event whose predecessor is in the same chunk waits
// a round and takes its record by shuffle); the target's own lane then runs
// the neuron physics over them in order.  If the target fires again inside the
// chunk, the events after that fire are redone with the new count; only the
// records of events before it are stored (the last event of each synapse
// stores).  The result is the sequential order's.
__device__ __forceinline__ void walk_fired_targets(const Engine& e, Walk& w, bool fired, uint32_t t, int stdp,
                                                   Staged st, const float* ltp, float* s_wt) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned pend = __ballot_sync(0xffffffffu, fired);
    while (pend) {
        const uint32_t L = __ffs(pend) - 1;
        pend &= pend - 1;
        const uint32_t beg = __shfl_sync(0xffffffffu, w.beg, L);
        const uint32_t len = __shfl_sync(0xffffffffu, w.len, L);
        const uint32_t after = __shfl_sync(0xffffffffu, w.first_fire, L) + 1;  // first event after the first fire
        uint32_t pos = __shfl_sync(0xffffffffu, w.i, L);
        uint32_t fires = __shfl_sync(0xffffffffu, w.fires, L);
        while (pos < len) {
            const uint32_t m = len - pos < 32 ? len - pos : 32;
            const uint32_t j = pos + lane;
            EvIn x{};
            if (lane < m) x = st.at(e, beg + j);
            const bool syn = lane < m && !(x.bits & kEvExternal);
            // the synapse's latest earlier event after the first fire
            uint32_t pred = 0xFFFFFFFFu;
            if (syn && (x.bits & kEvRepeat)) {
                for (uint32_t q = j; q-- > after;) {
                    const EvIn y = st.at(e, beg + q);
                    if (!(y.bits & kEvExternal) && y.tm == x.tm) {
                        pred = q;
                        break;
                    }
                }
            }
            const bool wait = pred != 0xFFFFFFFFu && pred >= pos;  // predecessor in this chunk
            SynA a{};
            float wt = x.weight;
            bool done = !syn;
            if (syn && !wait) {
                a = pred != 0xFFFFFFFFu ? e.syn[x.tm].a : before_event(e.syn[x.tm].a, e.ev_a0[beg + j]);
                wt = redo_pre_stdp(e, a, t, fires, stdp, ltp);
                done = true;
            }
            while (!__all_sync(0xffffffffu, done)) {
                const uint32_t src = wait ? pred - pos : lane;
                const SynA pa = shfl_syn(a, src);
                const bool pdone = __shfl_sync(0xffffffffu, done, src);
                if (!done && pdone) {
                    a = pa;
                    wt = redo_pre_stdp(e, a, t, fires, stdp, ltp);
                    done = true;
                }
            }
            if (lane < m) s_wt[lane] = wt;
            __syncwarp();
            uint32_t next = pos + m;
            if (lane == L) {
                for (uint32_t c = 0; c < m; ++c) {
                    const EvIn y = st.at(e, beg + pos + c);
                    if (process_input(w.s, w.threshold, y.bits & 3u, (y.bits >> 2) & 3u, s_wt[c], t)) {
                        record_fire(e, w, y.due);
                        w.fires += 1;
                        if (c + 1 < m) {
                            next = pos + c + 1;
                            break;
                        }
                    }
                }
                w.i = next;
            }
            next = __shfl_sync(0xffffffffu, next, L);
            // store the records of the events before `next`, the last one of
            // each synapse
            const bool store = syn && j < next;
            const unsigned long long key = store ? x.tm : (1ull << 32) | lane;
            const unsigned same = __match_any_sync(0xffffffffu, key);
            if (store && lane == 31u - __clz(same)) e.syn[x.tm].a = a;
            pos = next;
            fires = __shfl_sync(0xffffffffu, w.fires, L);
            __syncwarp();
        }
    }
}

// Stores a finished walk's neuron state and lists the target if it fired.
__device__ __forceinline__ void finish_walk(const Engine& e, const Walk& w) {
    const NState& s = w.s;
    NeuronRec* rec = e.nrec + w.n;
    reinterpret_cast<float4*>(rec->cur)[0] = make_float4(s.cur[0], s.cur[1], s.cur[2], s.cur[3]);
    reinterpret_cast<uint4*>(rec->upd)[0] = make_uint4(s.upd[0], s.upd[1], s.upd[2], s.upd[3]);
    *reinterpret_cast<uint4*>(&rec->membrane) =
        make_uint4(__float_as_uint(s.membrane), s.spikes, s.last_fired1, s.last_active);
    rec->flags = s.flags;
    if (w.fires > 0) {
        const uint32_t j = atomicAdd(&e.ts->n_fired_targets, 1u);
        e.fired_tgt[j] = w.n;
        e.fired_cnt[j] = w.fires;
    }
}

// One thread per touched target: the neuron's physics over its events in
// due order.  Exact because every state an event reads or writes belongs to
// its target (the target's neuron state and the target's incoming synapses);
// post-spike STDP of a fire is applied lazily to synapses touched later in the
// tick and in bulk by k_post for the rest.
// A block's targets are consecutive touched targets, so their event inputs
// are one contiguous range: one thread copies it into shared memory with a
// bulk copy while every thread loads its neuron's records.
__global__ void __launch_bounds__(kThreads, SNNGB_PROCESS_MIN_BLOCKS) k_process(Engine e) {
    tick_enter();
    extern __shared__ __align__(128) EvIn s_ev[];  // kStageEvents entries
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ uint32_t s_lo, s_cnt;
    __shared__ float s_wt[kThreads / 32][32];  // per warp: weights of the events redone after a fire
    const uint32_t t = e.ts->tick;
    const uint32_t N = e.N;
    const int stdp = e.ts->stdp_enabled;
    if (threadIdx.x == 0) mbar_init(&s_bar, 1);
    __syncthreads();
    // the LTP table goes to shared memory (when it fits) during the first
    // round's copy: the STDP redone after a fire then makes no dependent
    // global load besides the snapshot
    const bool ltp_shared = stdp && e.tab.stdp_len <= kLtpShared;
    const float* ltp = ltp_shared ? reinterpret_cast<const float*>(s_ev + kStageEvents) : e.tab.ltp;
    uint32_t parity = 0;
    bool staging = true;  // false after a copy outlived its wait: shared memory is no longer used
    // `per` consecutive targets per block and round (their events are one
    // contiguous range of the grouped list): the grid has at least three
    // blocks per SM, so one wave of equal blocks spreads over every SM (the
    // block scheduler fills each SM to its occupancy limit)
    const uint32_t per_even = (N + gridDim.x - 1) / gridDim.x;
    const uint32_t per = per_even < blockDim.x ? per_even : blockDim.x;
    for (uint32_t k0 = blockIdx.x * per; k0 < N; k0 += gridDim.x * per) {
        if (threadIdx.x == 0) {
            const uint32_t k1 = k0 + per < N ? k0 + per : N;
            const uint32_t lo = e.seg_start[k0];
            const uint32_t hi = e.seg_start[k1];
            const uint32_t cnt = staging ? (hi - lo < kStageEvents ? hi - lo : kStageEvents) : 0u;
            s_lo = lo;
            s_cnt = cnt;
            if (cnt > 0) bulk_load(s_ev, e.evin + lo, cnt * static_cast<uint32_t>(sizeof(EvIn)), &s_bar);
        }
        if (ltp_shared && k0 == blockIdx.x * per) {
            float* s_ltp = reinterpret_cast<float*>(s_ev + kStageEvents);
            for (uint32_t i = threadIdx.x; i < e.tab.stdp_len; i += blockDim.x) s_ltp[i] = e.tab.ltp[i];
        }
        __syncthreads();
        const Staged st{s_ev, s_lo, s_cnt};
        bool waited = st.cnt == 0;
        bool ok = true;
        auto ready = [&]() {
            if (!waited) {
                ok = mbar_wait(&s_bar, parity, e.stage_wait_ns);
                waited = true;
            }
            return ok;
        };
        const uint32_t k = k0 + threadIdx.x;
        Walk w;
        w.n = w.beg = w.len = w.i = w.fires = w.first_fire = 0;
        if (threadIdx.x < per && k < N) {
            w.n = k;
            w.beg = e.seg_start[k];
            w.len = e.seg_start[k + 1] - w.beg;
        }
        const bool mine_target = w.len > 0;  // a target with due events
        bool fired = false;
        Staged mine = st;
        if (mine_target) fired = walk_to_first_fire(e, w, t, mine, ready);
        if (!ready()) mine.cnt = 0;
        walk_fired_targets(e, w, fired, t, stdp, mine, ltp, s_wt[threadIdx.x >> 5]);
        if (mine_target) finish_walk(e, w);
        const bool failed = __syncthreads_or(!ok);
        if (st.cnt > 0) {
            if (failed) {
                // the block read its inputs from global memory; wait once more
                // for the copy before the buffer is reused or the block exits
                if (threadIdx.x == 0) raise_status(e, kStatusStageTimeout);
                if (!__syncthreads_and(mbar_wait(&s_bar, parity, kDrainWaitNs))) return;
            }
            parity ^= 1u;
        }
        if (failed) staging = false;
    }
}

// The temporal pattern update of every touched target (SynapseDendriteProcessor
// .cpp:294-316), once per tick for all its k events (temporal_tick).  It reads
// and writes only the neuron's temporal fields, which nothing else in the tick
// touches, so it can run beside k_events / k_process.
template <bool kOne>
__device__ __forceinline__ void temporal_target(const Engine& e, uint32_t n, uint32_t k, uint32_t t, int temporal) {
    const NeuronParam p = e.nparam[n];
    NeuronRec* rec = e.nrec + n;
    const NeuronTp q = e.ntp[n];
    NState s;
    s.match_count = rec->match_count;
    s.ws = rec->ws;
    s.len = rec->len;
    s.flags = q.last_match << 8;
    s.cn = q.cn;
    s.nruns = q.nruns;
    s.ref_head = q.ref_head;
    s.ref_count = q.ref_count;
    s.ring_head = q.ring_head;
    s.ring_used = q.ring_used;
    s.last_run = s.nruns > 0 ? e.cand[p.cand_base + s.nruns - 1] : 0ull;
    if (kOne && s.ref_count > 0) s.one = e.refmeta[p.meta_base];
    s.snap_pending = false;
    temporal_tick<kOne>(s, p, t, e, temporal, k);
    if (s.nruns > 0) e.cand[p.cand_base + s.nruns - 1] = s.last_run;
    if (kOne && s.ref_count > 0) e.refmeta[p.meta_base] = s.one;
    if (kOne && s.snap_pending) {
        // runs 0 .. snap_nruns-2 are final in cand; the last one was saved
        unsigned long long* ring = e.ring + p.ring_base;
        const unsigned long long* cand = e.cand + p.cand_base;
        for (uint32_t j = 0; j + 1 < s.snap_nruns; ++j) ring[wrap_add(s.one.start, j, p.ring_cap)] = cand[j];
        ring[wrap_add(s.one.start, s.snap_nruns - 1, p.ring_cap)] = s.snap_last;
    }
    rec->match_count = s.match_count;
    rec->ws = s.ws;
    rec->len = s.len;
    NeuronTp wq;
    wq.cn = s.cn;
    wq.nruns = s.nruns;
    wq.ref_head = s.ref_head;
    wq.ref_count = s.ref_count;
    wq.ring_head = s.ring_head;
    wq.ring_used = s.ring_used;
    wq.last_match = (s.flags >> 8) & 1u;
    e.ntp[n] = wq;
}

__global__ void __launch_bounds__(kThreads) k_temporal(Engine e) {
    const uint32_t t = e.ts->tick;
    const int temporal = e.ts->temporal_enabled;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < e.N; n += gridDim.x * blockDim.x) {
        const uint32_t len = e.seg_start[n + 1] - e.seg_start[n];
        if (len == 0) continue;
        if (e.nparam[n].max_refs == 1) {
            temporal_target<true>(e, n, len, t, temporal);
        } else {
            temporal_target<false>(e, n, len, t, temporal);
        }
    }
}

__global__ void k_init_syn(SynAB* syn, const SynA* a, unsigned long long S) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < S;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        SynAB r;
        r.a = a[i];
        r.b = SynB{};
        r.b.flags = static_cast<uint8_t>(((r.a.meta >> kMetaExpectedShift) & 15u) << 4);
        syn[i] = r;
    }
}

// Post-spike STDP over the incoming rows of every target that fired
// (NetworkPropagator.cpp:95-102), one block per fired target, coalesced over
// the target-major row.  Runs on the side stream beside k_fire_list ..
// k_expand (none of which touches synapse records), so it reads the tick
// from post_tick, not from the tick counter k_fire_count advances.
__global__ void k_post(Engine e) {
    const uint32_t t = e.ts->post_tick;
    const uint32_t nf = e.ts->n_fired_targets;
    const int stdp = e.ts->stdp_enabled;
    for (uint32_t j = blockIdx.x; j < nf; j += gridDim.x) {
        const uint32_t n = e.fired_tgt[j];
        const uint32_t fires = e.fired_cnt[j];
        if (fires >= 0x10000u) {
            if (threadIdx.x == 0) raise_status(e, kStatusPostCountOverflow);
            continue;
        }
        const unsigned long long b = e.in_ptr[n], en = e.in_ptr[n + 1];
        for (unsigned long long tm = b + threadIdx.x; tm < en; tm += blockDim.x) {
            SynA a = e.syn[tm].a;
            if (post_catch_up(a, t, fires, e, stdp, e.tab.ltp)) e.syn[tm].a = a;
        }
    }
}

// Fires in due order, one thread per bitmap word (a tile is kThreads words).
// k_process counted every tile's fires, so a block finds the first rank of
// its tile by adding the counts of the tiles before it.  A fire's rank r is
// its position in the reference's fire order (due order,
// NetworkPropagator.cpp:80-93); the fire list and the raster are written here
// and the bitmap is cleared.
__global__ void k_fire_list(Engine e) {
    tick_enter();
    const uint32_t t = e.ts->tick;
    const uint32_t words = (e.ts->n_due + 31) / 32;
    const uint32_t tiles = (words + kThreads - 1) / kThreads;
    const unsigned long long raster0 = e.ts->raster_count;
    uint32_t part = 0, base = 0;
    for (uint32_t i = threadIdx.x; i < blockIdx.x && i < tiles; i += blockDim.x) part += __ldcg(e.fire_tile + i);
    block_excl_scan(part, &base);
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t w = tile * kThreads + threadIdx.x;
        uint32_t bits = w < words ? e.fire_bits[w] : 0u;
        uint32_t r = base + block_excl_scan(__popc(bits), nullptr);
        if (bits) e.fire_bits[w] = 0;
        while (bits) {
            const uint32_t bit = __ffs(bits) - 1;
            bits &= bits - 1;
            const uint32_t n = e.fire_at[w * 32 + bit];
            if (r < e.fire_cap) e.fire_list[r] = n;
            if (e.raster_cap > 0) {
                const unsigned long long pos = raster0 + r;
                if (pos < e.raster_cap) {
                    e.raster[2 * pos] = t;
                    e.raster[2 * pos + 1] = n;
                }
            }
            r += 1;
        }
        // the base of this block's next tile
        part = 0;
        for (uint32_t i = tile + threadIdx.x; i < tile + gridDim.x && i < tiles; i += blockDim.x)
            part += __ldcg(e.fire_tile + i);
        uint32_t step;
        block_excl_scan(part, &step);
        base += step;
    }
}

// Events per (expansion block of kExpandFires fires, delay class), one warp
// per fire and one lane per class.  The last block turns the counts into wheel positions
// (exclusive scan over blocks per class, appended behind each delivery slot's
// current contents) and finishes the tick.
__global__ void __launch_bounds__(kFireCountThreads, 1) k_fire_count(Engine e) {
    tick_enter();
    const uint32_t t = e.ts->tick;
    // the tick's fire count: the sum of k_process's per-tile counts
    const uint32_t tiles = ((e.ts->n_due + 31) / 32 + kThreads - 1) / kThreads;
    __shared__ uint32_t s_nf;
    if (threadIdx.x == 0) s_nf = 0;
    __syncthreads();
    uint32_t part = 0;
    for (uint32_t i = threadIdx.x; i < tiles; i += blockDim.x) part += __ldcg(e.fire_tile + i);
    part = __reduce_add_sync(0xffffffffu, part);
    if ((threadIdx.x & 31) == 0 && part) atomicAdd(&s_nf, part);
    __syncthreads();
    const uint32_t nfires = s_nf;
    const uint32_t nf = nfires < e.fire_cap ? nfires : e.fire_cap;
    const uint32_t D = e.D;
    // one warp per fire, one lane per delay class
    const uint32_t lane0 = threadIdx.x & 31;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nf; r += nwarps) {
        const uint32_t* row = e.pre_off + static_cast<size_t>(e.fire_list[r]) * (D + 1);
        uint32_t* xs = e.xsum + static_cast<size_t>(r / kExpandFires) * D;
        for (uint32_t d = lane0; d < D; d += 32) {
            const uint32_t c = row[d + 1] - row[d];
            if (c) atomicAdd(xs + d, c);
        }
    }
    if (!last_block(&e.ts->done_fire_list)) return;
    for (uint32_t i = threadIdx.x; i < tiles; i += blockDim.x) e.fire_tile[i] = 0;  // zero for the next tick
    if (nfires > e.fire_cap && threadIdx.x == 0) raise_status(e, kStatusFireOverflow);
    const uint32_t blocks = (nf + kExpandFires - 1) / kExpandFires;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // one warp per class; lane i scans a contiguous run of expansion blocks
    // (its loads are independent, so they are all in flight at once), then
    // the lanes' totals are scanned across the warp
    const uint32_t per = (blocks + 31) / 32;
    const uint32_t b0 = lane * per < blocks ? lane * per : blocks;
    const uint32_t b1 = b0 + per < blocks ? b0 + per : blocks;
    for (uint32_t d = warp; d < D; d += blockDim.x / 32) {
        const uint32_t slot = (t + e.cls_delta[d]) & e.wmask;
        const uint32_t start = e.slot_count[slot];
        uint32_t sum = 0;
        for (uint32_t b = b0; b < b1; ++b) sum += __ldcg(e.xsum + static_cast<size_t>(b) * D + d);
        const uint32_t incl = warp_incl_scan(sum);
        const uint32_t carry = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long pos = static_cast<unsigned long long>(slot) * e.slot_cap + start + (incl - sum);
        for (uint32_t b = b0; b < b1; ++b) {
            e.xdst[static_cast<size_t>(b) * D + d] = pos;
            pos += __ldcg(e.xsum + static_cast<size_t>(b) * D + d);
        }
        if (lane == 0) {
            if (static_cast<unsigned long long>(start) + carry > e.slot_cap) {
                raise_status(e, kStatusSlotOverflow);
                e.xdst_ok[d] = 0;
            } else {
                e.xdst_ok[d] = 1;
                e.slot_count[slot] = start + carry;
            }
        }
    }
    // the class counts back to zero for the next tick, once every warp has
    // read its classes
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < blocks * D; i += blockDim.x) e.xsum[i] = 0;
    if (threadIdx.x == 0) {
        TickState* ts = e.ts;
        ts->n_fires = nfires;
        const uint32_t due = ts->n_due;
        const unsigned long long raster0 = ts->raster_count;
        ts->delivered += due;
        ts->fired += nfires;
        ts->touched_total += ts->n_touched;
        if (due > ts->max_slot_events) ts->max_slot_events = due;
        if (e.raster_cap > 0) {
            if (raster0 + nfires > e.raster_cap) raise_status(e, kStatusRasterOverflow);
            ts->raster_count = raster0 + nfires;
        }
        ts->expand_fires = nf;
        e.slot_count[t & e.wmask] = 0;
        ts->n_touched = 0;
        ts->tick = t + 1;
    }
}

// Spike-code offset expansion (NetworkPropagator.cpp:104-130): one block per
// fire, one warp per delay class.  A fire's events of one class are
// contiguous in its pre-expanded list and go to one contiguous range of their
// delivery slot: the range k_fire_count reserved for the fire's expansion
// block, behind the block's earlier fires.  So the wheel ends up in exactly
// the reference's scheduling order.
__global__ void __launch_bounds__(kThreads) k_expand(Engine e) {
    tick_enter();
    __shared__ uint32_t s_rows[kExpandFires][kMaxClasses + 1];
    __shared__ unsigned long long s_dst[kMaxClasses];
    __shared__ uint8_t s_ok[kMaxClasses];  // the class's slot had room
    __shared__ unsigned long long s_base;
    const uint32_t nf = e.ts->expand_fires;
    const uint32_t D = e.D;
    for (uint32_t r = blockIdx.x; r < nf; r += gridDim.x) {
        const uint32_t first = r - r % kExpandFires;
        const uint32_t m = r - first + 1;  // fires first .. r of the expansion block
        // everything the copies depend on, fetched together: the class rows of
        // the block's fires, the block's destinations, the fire's event list
        for (uint32_t i = threadIdx.x; i < m * (D + 1); i += blockDim.x) {
            const uint32_t q = i / (D + 1), d = i - q * (D + 1);
            s_rows[q][d] = e.pre_off[static_cast<size_t>(e.fire_list[first + q]) * (D + 1) + d];
        }
        for (uint32_t d = threadIdx.x; d < D; d += blockDim.x) {
            s_ok[d] = e.xdst_ok[d] ? 1 : 0;
            s_dst[d] = s_ok[d] ? __ldcg(e.xdst + static_cast<size_t>(r / kExpandFires) * D + d) : 0ull;
        }
        if (threadIdx.x == 0) s_base = e.pre_base[e.fire_list[r]];
        __syncthreads();
        const uint32_t* row = s_rows[m - 1];
        // this fire's place in each class: the block's destination behind
        // the class's events of the block's earlier fires
        for (uint32_t d = threadIdx.x; d < D; d += blockDim.x) {
            uint32_t before = 0;
            for (uint32_t q = 0; q + 1 < m; ++q) before += s_rows[q][d + 1] - s_rows[q][d];
            // then event k of class d goes to s_dst[d] + k (64-bit wrap-around
            // arithmetic: exact once k >= row[d] is added back)
            s_dst[d] = s_dst[d] + static_cast<unsigned long long>(before) - static_cast<unsigned long long>(row[d]);
        }
        __syncthreads();
        // every event by its own thread (consecutive threads, consecutive
        // events: coalesced within a class); its class by binary search of
        // the fire's class offsets
        const unsigned long long* src = e.pre_ev + s_base;
        const uint32_t k0 = row[0], k1 = row[D];
        auto class_of = [&](uint32_t k) {
            uint32_t lo = 0, hi = D;  // row[lo] <= k < row[hi]
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (row[mid] <= k) {
                    lo = mid;
                } else {
                    hi = mid;
                }
            }
            return lo;
        };
        for (uint32_t k = k0 + threadIdx.x; k < k1; k += 4 * blockDim.x) {
            unsigned long long v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t kk = k + u * blockDim.x;
                v[u] = kk < k1 ? src[kk] : 0ull;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t kk = k + u * blockDim.x;
                if (kk >= k1) continue;
                const uint32_t d = class_of(kk);
                if (s_ok[d]) e.wheel[s_dst[d] + kk] = v[u];
            }
        }
        __syncthreads();
    }
}

__global__ void k_inject(Engine e, const unsigned long long* ev, const uint32_t* slot_of_group,
                         const uint32_t* group_off, uint32_t groups) {
    for (uint32_t gi = blockIdx.x; gi < groups; gi += gridDim.x) {
        const uint32_t slot = slot_of_group[gi];
        const uint32_t b = group_off[gi], en = group_off[gi + 1];
        const uint32_t base = e.slot_count[slot];
        if (static_cast<unsigned long long>(base) + (en - b) > e.slot_cap) {
            if (threadIdx.x == 0) raise_status(e, kStatusSlotOverflow);
            continue;
        }
        unsigned long long* dst = e.wheel + static_cast<size_t>(slot) * e.slot_cap + base;
        for (uint32_t i = threadIdx.x; i < en - b; i += blockDim.x) dst[i] = ev[b + i];
        __syncthreads();
        if (threadIdx.x == 0) e.slot_count[slot] = base + (en - b);
        __syncthreads();
    }
}

__global__ void k_rule_off(SynAB* syn, unsigned long long b, unsigned long long en) {
    for (unsigned long long i = b + blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < en;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
        syn[i].a.meta |= 1u << kMetaRuleOffBit;
}

__global__ void k_range_counts(Engine e, uint32_t nb, uint32_t ne, unsigned long long tb, unsigned long long te,
                               unsigned long long* out) {
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    const unsigned long long first = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    unsigned long long spikes = 0, pre = 0, wheel = 0, matches = 0, code_matches = 0;
    for (unsigned long long n = nb + first; n < ne; n += stride) {
        spikes += e.nrec[n].spike_count;
        matches += e.nrec[n].match_count;
    }
    for (unsigned long long i = tb + first; i < te; i += stride) {
        pre += e.syn[i].b.pre_count;
        code_matches += e.syn[i].b.code_matches;
    }
    for (uint32_t slot = 0; slot < e.W; ++slot) {
        const uint32_t cnt = e.slot_count[slot];
        const unsigned long long* ev = e.wheel + static_cast<size_t>(slot) * e.slot_cap;
        for (unsigned long long i = first; i < cnt; i += stride) {
            const uint32_t tgt = static_cast<uint32_t>(ev[i]) & ~kExternalBit;
            wheel += tgt >= nb && tgt < ne;
        }
    }
    if (spikes) atomicAdd(out, spikes);
    if (pre) atomicAdd(out + 1, pre);
    if (wheel) atomicAdd(out + 2, wheel);
    if (matches) atomicAdd(out + 3, matches);
    if (code_matches) atomicAdd(out + 4, code_matches);
}

// 64-bit mix of one word into a running hash (multiply / xor-shift rounds).
__device__ __forceinline__ unsigned long long mix64(unsigned long long h, unsigned long long w) {
    h ^= w + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    h *= 0xbf58476d1ce4e5b9ull;
    h ^= h >> 31;
    return h;
}

template <int kWords>
__device__ __forceinline__ unsigned long long record_hash(unsigned long long index, const uint32_t* w) {
    unsigned long long h = mix64(0x6a09e667f3bcc908ull, index);
#pragma unroll
    for (int i = 0; i < kWords; ++i) h = mix64(h, w[i]);
    return h;
}

// Order-independent checksums of neurons [nb, ne) (NeuronRec + NeuronTp)
// and of their incoming synapses: the sum over records of a hash of (index
// within the range, the record's meaning).  A synapse contributes its SynA
// words (the rule-off bit masked), its code-pattern counters, its code
// offsets and its learned code patterns, wherever the layout keeps them
// (inline in the record or in the pattern pool, which depends on the widest
// code of the whole simulation), so a batch member and its solo run give
// equal sums exactly when their states are equal (up to hash collisions).
__global__ void k_checksum(Engine e, uint32_t nb, uint32_t ne, unsigned long long tb, unsigned long long* out) {
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    const unsigned long long first = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    unsigned long long hn = 0, hs = 0;
    for (unsigned long long n = nb + first; n < ne; n += stride) {
        uint32_t w[24];
        const uint4* r = reinterpret_cast<const uint4*>(e.nrec + n);
        const uint4* q = reinterpret_cast<const uint4*>(e.ntp + n);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint4 v = r[i];
            w[4 * i] = v.x; w[4 * i + 1] = v.y; w[4 * i + 2] = v.z; w[4 * i + 3] = v.w;
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const uint4 v = q[i];
            w[16 + 4 * i] = v.x; w[17 + 4 * i] = v.y; w[18 + 4 * i] = v.z; w[19 + 4 * i] = v.w;
        }
        hn += record_hash<24>(n - nb, w);
    }
    // synapses: a warp per target
    const uint32_t lane = threadIdx.x & 31;
    const unsigned long long warps = stride / 32;
    for (unsigned long long n = nb + first / 32; n < ne; n += warps) {
        const NeuronParam p = e.nparam[n];
        const bool inl = inline_code_pattern(p.max_refs, e.code_stride);
        for (unsigned long long i = e.in_ptr[n] + lane; i < e.in_ptr[n + 1]; i += 32) {
            const SynAB rec = e.syn[i];
            const SynA& a = rec.a;
            const SynB& sb = rec.b;
            unsigned long long h = mix64(0x6a09e667f3bcc908ull, i - tb);
            h = mix64(h, __float_as_uint(a.weight));
            h = mix64(h, a.last_pre1);
            h = mix64(h, a.last_post1);
            h = mix64(h, a.meta & ~(1u << kMetaRuleOffBit));
            h = mix64(h, __float_as_uint(a.clamp_hi));
            h = mix64(h, a.updates);
            h = mix64(h, __float_as_uint(a.last_delta));
            h = mix64(h, a.post_cnt);
            h = mix64(h, sb.pre_count);
            h = mix64(h, sb.code_ws);
            h = mix64(h, sb.code_matches);
            h = mix64(h, sb.code_len | (static_cast<uint32_t>(sb.flags) << 8) |
                             (static_cast<uint32_t>(sb.learned_count) << 16));
            for (uint32_t j = 0; j < sb.code_len; ++j) h = mix64(h, ring_get(sb.ring_lo, sb.ring_hi, j));
            const uint32_t expected = (a.meta >> kMetaExpectedShift) & 15u;
            const uint16_t* lc =
                e.lcode + p.lcode_base + static_cast<size_t>(i - p.in_begin) * p.max_refs * e.code_stride;
            for (uint32_t k = 0; k < sb.learned_count; ++k)
                for (uint32_t j = 0; j < expected; ++j)
                    h = mix64(h, inl ? ring_get(sb.ring_hi, 0ull, j) : lc[static_cast<size_t>(k) * e.code_stride + j]);
            hs += h;
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        hn += __shfl_down_sync(0xffffffffu, hn, d);
        hs += __shfl_down_sync(0xffffffffu, hs, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, hn);
        atomicAdd(out + 1, hs);
    }
}

}  // namespace

void launch_checksum(const Engine& e, uint32_t n_begin, uint32_t n_end, unsigned long long tm_begin,
                     unsigned long long* out, cudaStream_t stream) {
    k_checksum<<<e.grid_wide * 2, kThreads, 0, stream>>>(e, n_begin, n_end, tm_begin, out);
}

void launch_rule_off(const Engine& e, unsigned long long tm_begin, unsigned long long tm_end, cudaStream_t stream) {
    if (tm_end > tm_begin) k_rule_off<<<1024, kThreads, 0, stream>>>(e.syn, tm_begin, tm_end);
}

void launch_range_counts(const Engine& e, uint32_t n_begin, uint32_t n_end, unsigned long long tm_begin,
                         unsigned long long tm_end, unsigned long long* out, cudaStream_t stream) {
    k_range_counts<<<e.grid_wide, kThreads, 0, stream>>>(e, n_begin, n_end, tm_begin, tm_end, out);
}

// Launch of a main-stream tick kernel.  `dependent` makes it a programmatic
// dependent of the kernel before it on the stream (see tick_enter): its
// blocks are scheduled while that kernel drains instead of after it.
static void launch_main(void (*kernel)(Engine), uint32_t grid, uint32_t block, size_t smem, cudaStream_t stream,
                        bool dependent, const Engine& e) {
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = &attr;
    cfg.numAttrs = dependent ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, e);
}

// Dynamic shared memory of the grouping kernels.
static size_t bucket_smem(const Engine& e) {
    return stream_buf_offset(e.nbuckets) + kStreamBufs * kStreamTile * sizeof(unsigned long long);
}
static size_t bsort_smem(const Engine& e) {
    return kSortSmemBytes + (static_cast<size_t>(1) << e.bucket_shift) * sizeof(uint32_t);
}
static uint32_t bsort_grid(const Engine& e) { return e.nbuckets; }

void launch_tick(const Engine& e, const TickStreams& s, cudaEvent_t* marks) {
    const uint32_t wide = e.grid_wide;
    cudaStream_t stream = s.main;
    // Kernels that follow another kernel directly on the main stream are
    // programmatic dependents; the per-kernel profile (event marks between
    // the kernels) launches them plainly so each kernel is timed alone.
    const bool dep = marks == nullptr;
    int k = 0;
    auto mark = [&](bool after) {
        if (marks) cudaEventRecordWithFlags(marks[2 * k + (after ? 1 : 0)], stream, cudaEventRecordExternal);
        if (after) ++k;
    };
    auto side_mark = [&](int index, bool after) {
        if (marks)
            cudaEventRecordWithFlags(marks[2 * index + (after ? 1 : 0)],
                                     e.side_serial ? stream : s.side,
                                     cudaEventRecordExternal);
    };
    // k_bcount follows a wait on the side stream: a full dependency
    mark(false); launch_main(k_bcount, e.grid_bucket, kBucketThreads, bucket_smem(e), stream, false, e); mark(true);
    mark(false); launch_main(k_bscatter, e.grid_bucket, kBucketThreads, bucket_smem(e), stream, dep, e); mark(true);
    mark(false); launch_main(k_bsort, bsort_grid(e), kThreads, bsort_smem(e), stream, dep, e); mark(true);
    if (e.side_serial) {
        // everything in tick order on the main stream; k_temporal, k_events,
        // k_post and the fire ordering take full dependencies (as
        // programmatic dependents they made the tick 7 % slower on recog_1m:
        // their blocks, launched early, held SM resources the kernel before
        // them needed)
        side_mark(8, false);
        launch_main(k_temporal, e.grid_process, kThreads, 0, stream, false, e);
        side_mark(8, true);
        mark(false); launch_main(k_events, e.grid_events, kThreads, 0, stream, false, e); mark(true);
        mark(false); launch_main(k_process, e.grid_walk, kThreads, kProcessSmem, stream, dep, e); mark(true);
        side_mark(9, false);
        launch_main(k_post, wide * 4, kThreads, 0, stream, false, e);
        side_mark(9, true);
        mark(false); launch_main(k_fire_list, e.grid_fire, kThreads, 0, stream, false, e); mark(true);
        mark(false); launch_main(k_fire_count, e.grid_wide / 4 + 1, kFireCountThreads, 0, stream, false, e); mark(true);
        mark(false); launch_main(k_expand, e.grid_wide * 4, kThreads, 0, stream, dep, e); mark(true);
        return;
    }
    // the temporal update forks off here and runs beside k_events / k_process
    // (it needs only the segment starts)
    cudaEventRecord(s.ev[0], stream);
    cudaStreamWaitEvent(s.side, s.ev[0], 0);
    side_mark(8, false);
    k_temporal<<<e.grid_process, kThreads, 0, s.side>>>(e);
    side_mark(8, true);
    cudaEventRecord(s.ev[1], s.side);
    mark(false); launch_main(k_events, e.grid_events, kThreads, 0, stream, dep, e); mark(true);
    mark(false); launch_main(k_process, e.grid_walk, kThreads, kProcessSmem, stream, dep, e); mark(true);
    // post-spike STDP of the fired targets runs beside the fire ordering and
    // the expansion (synapse records are not touched by those)
    cudaEventRecord(s.ev[2], stream);
    cudaStreamWaitEvent(s.side, s.ev[2], 0);
    side_mark(9, false);
    k_post<<<wide * 4, kThreads, 0, s.side>>>(e);
    side_mark(9, true);
    cudaEventRecord(s.ev[3], s.side);
    mark(false); launch_main(k_fire_list, e.grid_fire, kThreads, 0, stream, dep, e); mark(true);
    cudaStreamWaitEvent(stream, s.ev[1], 0);  // k_temporal reads the tick counter k_fire_count advances
    mark(false); launch_main(k_fire_count, e.grid_wide / 4 + 1, kFireCountThreads, 0, stream, false, e); mark(true);
    mark(false); launch_main(k_expand, e.grid_wide * 4, kThreads, 0, stream, dep, e); mark(true);
    cudaStreamWaitEvent(stream, s.ev[3], 0);  // the next tick's k_events reads the synapse records
}

const char* kernel_name(int index) {
    static const char* names[kKernelCount] = {"k_bcount",    "k_bscatter",  "k_bsort",    "k_events",
                                              "k_process",   "k_fire_list", "k_fire_count", "k_expand",
                                              "k_temporal",  "k_post"};
    return index >= 0 && index < kKernelCount ? names[index] : "";
}

void launch_group(const Engine& e, cudaStream_t stream) {
    k_bcount<<<e.grid_bucket, kBucketThreads, bucket_smem(e), stream>>>(e);
    k_bscatter<<<e.grid_bucket, kBucketThreads, bucket_smem(e), stream>>>(e);
    k_bsort<<<bsort_grid(e), kThreads, bsort_smem(e), stream>>>(e);
    k_segsort<<<e.grid_wide * 4, kThreads, 0, stream>>>(e);
}

void configure_kernels() {
    cudaFuncSetAttribute(k_process, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kProcessSmem));
    const int bucket_bytes =
        static_cast<int>(stream_buf_offset(kMaxBuckets) + kStreamBufs * kStreamTile * sizeof(unsigned long long));
    cudaFuncSetAttribute(k_bcount, cudaFuncAttributeMaxDynamicSharedMemorySize, bucket_bytes);
    cudaFuncSetAttribute(k_bscatter, cudaFuncAttributeMaxDynamicSharedMemorySize, bucket_bytes);
    cudaFuncSetAttribute(k_bsort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kSortSmemBytes + (1u << kMaxBucketShift) * sizeof(uint32_t)));
}

void launch_init_syn(const Engine& e, const SynA* a, cudaStream_t stream) {
    if (e.S == 0) return;
    k_init_syn<<<1024, kThreads, 0, stream>>>(e.syn, a, e.S);
}

void launch_inject(const Engine& e, const unsigned long long* ev, const uint32_t* slot_of_group,
                   const uint32_t* group_off, uint32_t groups, cudaStream_t stream) {
    if (groups == 0) return;
    k_inject<<<groups < 1024 ? groups : 1024, kThreads, 0, stream>>>(e, ev, slot_of_group, group_off, groups);
}

}  // namespace snngb
