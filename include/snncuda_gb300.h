/*
 * snncuda_gb300.h -- C ABI of the GB300 spiking-simulation backend.
 *
 * The backend advances a flattened SNNCuda Connectome tick by tick with the
 * semantics of the reference CPU runtime (runtime::NetworkPropagator):
 * timing-wheel spike delivery with spike-code offset expansion,
 * synapse -> dendrite -> receptor integration, threshold and reset, pair STDP
 * with a runtime toggle, and neuron / synapse temporal-pattern recording with
 * cosine matching.
 *
 * Conventions
 *  - Every call returns an int status (SNNCUDA_OK on success).  No C++
 *    exception crosses this boundary.  snncuda_last_error() returns a
 *    thread-local message describing the last failure.
 *  - Neurons are dense 0-based indices in Connectome::neurons order.
 *    Synapses are dense 0-based indices in Connectome::synapses order; that
 *    order defines the outgoing/incoming list order of the reference
 *    (NetworkPropagator.cpp:24-28) and therefore the event order.
 *  - All input arrays are caller-owned and copied at create.
 *  - A handle is used by one host thread at a time.
 *  - After a device-side error (capacity overflow, wait timeout) the handle
 *    is poisoned: later stepping calls return SNNCUDA_ERR_POISONED; readers
 *    keep working.
 */
#ifndef SNNCUDA_GB300_H
#define SNNCUDA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SNNCUDA_OK 0
#define SNNCUDA_ERR_INVALID_ARGUMENT 1 /* std::invalid_argument in the reference */
#define SNNCUDA_ERR_OUT_OF_MEMORY 2
#define SNNCUDA_ERR_CAPACITY 3         /* a fixed device capacity would overflow */
#define SNNCUDA_ERR_DEVICE 4           /* CUDA runtime error (check_cuda in the reference) */
#define SNNCUDA_ERR_TIMEOUT 5          /* a bounded device-side wait gave up */
#define SNNCUDA_ERR_UNSUPPORTED 6      /* input outside the engine's stated limits */
#define SNNCUDA_ERR_POISONED 7         /* an earlier device error left the handle unusable */

/* ---- enumerations (snn/Synapse.h:9-21 in the reference) ----------------- */
#define SNNCUDA_COMPARTMENT_SOMA 0
#define SNNCUDA_COMPARTMENT_BASAL 1
#define SNNCUDA_COMPARTMENT_APICAL 2
#define SNNCUDA_COMPARTMENT_INHIBITORY 3

#define SNNCUDA_RECEPTOR_AMPA 0
#define SNNCUDA_RECEPTOR_NMDA 1
#define SNNCUDA_RECEPTOR_GABA_A 2
#define SNNCUDA_RECEPTOR_GABA_B 3

/* ---- reference C ABI, kept unchanged ------------------------------------
 * Replaces include/snncuda/c/SNNCudaC.h:7-8 (src/c/SNNCudaC.cpp:5-11).
 * snncuda_cuda_available reports a usable device at run time (the reference
 * reports the compile-time flag, core/Version.cpp:9-11). */
const char* snncuda_version(void);
int snncuda_cuda_available(void);

/* Thread-local description of the last failing call ("" if none). */
const char* snncuda_last_error(void);

/* ---- network input -------------------------------------------------------
 * Flattened declarative::Connectome (declarative/Connectome.h:13-37) with the
 * per-neuron NeuronParamsIR (declarative/NetworkIR.h:14-19). */
typedef struct snncuda_network {
    uint32_t neuron_count;
    const float* threshold;                  /* [neuron_count] */
    const uint64_t* pattern_window_ticks;    /* [neuron_count] */
    const float* similarity_threshold;       /* [neuron_count] */
    const uint64_t* max_reference_patterns;  /* [neuron_count], >= 1 */

    uint64_t synapse_count;
    const uint32_t* source;                  /* [synapse_count] neuron index */
    const uint32_t* target;                  /* [synapse_count] neuron index */
    const float* weight;                     /* [synapse_count] */
    const float* max_weight;                 /* [synapse_count] */
    const uint32_t* delay_ticks;             /* [synapse_count] */
    const uint8_t* compartment;              /* [synapse_count] SNNCUDA_COMPARTMENT_* */
    const uint8_t* receptor;                 /* [synapse_count] SNNCUDA_RECEPTOR_* */
    const uint8_t* plasticity_enabled;       /* [synapse_count] 0/1 */
    /* Spike-code offsets as CSR: offsets of synapse s are
     * code_offsets[code_offset_ptr[s] .. code_offset_ptr[s+1]).  An empty
     * list means {0} (SynapseDendriteProcessor.cpp:68-70).  NULL pointers
     * mean every synapse carries {0}. */
    const uint64_t* code_offset_ptr;         /* [synapse_count + 1] or NULL */
    const uint32_t* code_offsets;
} snncuda_network;

/* ---- processor configuration ---------------------------------------------
 * SynapseDendriteConfig (runtime/SynapseDendriteProcessor.h:37-40) holding a
 * learning::StdpConfig (learning/STDP.h:8-16), plus engine options. */
typedef struct snncuda_config {
    int32_t stdp_enabled;              /* StdpConfig::enabled, default 1 */
    float ltp_amplitude;               /* 0.01 */
    float ltd_amplitude;               /* 0.012 */
    float ltp_tau_ticks;               /* 20 */
    float ltd_tau_ticks;               /* 20 */
    float min_weight;                  /* 0 */
    float max_weight;                  /* 2 */
    int32_t temporal_learning_enabled; /* 1 */

    /* Engine options (0 = default, except stage_wait_ns). */
    uint64_t timing_wheel_slots;       /* accepted for parity with the reference
                                          constructor; must be nonzero
                                          (SpikeScheduler.cpp:10-12) */
    uint64_t slot_event_capacity;      /* events one wheel slot can hold */
    uint64_t pattern_run_capacity;     /* per-neuron run storage for learned
                                          temporal patterns */
    uint64_t raster_capacity;          /* fire records kept for read-back;
                                          0 disables capture */
    void* cuda_stream;                 /* cudaStream_t to launch on; NULL =
                                          the handle creates its own */
    uint64_t stage_wait_ns;            /* limit of the tick's bounded wait for
                                          a bulk copy into shared memory
                                          (default 100 ms).  When it runs out
                                          the tick reads its inputs from
                                          global memory (results unchanged)
                                          and the run returns
                                          SNNCUDA_ERR_TIMEOUT, poisoning the
                                          handle; 0 gives up without waiting */
} snncuda_config;

/* Fills the reference defaults. */
void snncuda_config_default(snncuda_config* config);

typedef struct snncuda_sim snncuda_sim;

/* Replaces NetworkPropagator(const Connectome&, NeuronStateStore&, size_t,
 * size_t) (runtime/NetworkPropagator.h:16-20, NetworkPropagator.cpp:5-29):
 * initial neuron state from the params, synapse runtime state from the
 * Connectome (SynapseDendriteProcessor.cpp:59-75). */
int snncuda_sim_create(const snncuda_network* network, const snncuda_config* config,
                       snncuda_sim** out);
int snncuda_sim_destroy(snncuda_sim* sim);

/* Replaces NetworkPropagator::inject (NetworkPropagator.cpp:31-37), applied
 * in array order.  A tick earlier than the next tick to process is clamped
 * to it (SpikeScheduler.cpp:17-19). */
int snncuda_sim_inject(snncuda_sim* sim, uint64_t count, const uint32_t* neurons,
                       const uint64_t* ticks, const float* weights);

/* Replaces NetworkPropagator::run_until (NetworkPropagator.cpp:39-43):
 * processes every tick up to and including inclusive_tick that has not been
 * processed yet.  Blocks until the device has finished. */
int snncuda_sim_run_until(snncuda_sim* sim, uint64_t inclusive_tick);

/* Runtime toggles: StdpRule::set_enabled (STDP.cpp:12-14) -- a disabled rule
 * still clamps the weight (STDP.cpp:37-40) -- and
 * SynapseDendriteConfig::temporal_learning_enabled. */
int snncuda_sim_set_plasticity(snncuda_sim* sim, int32_t enabled);
int snncuda_sim_set_temporal_learning(snncuda_sim* sim, int32_t enabled);

typedef struct snncuda_counters {
    uint64_t delivered_spikes;  /* NetworkPropagator::delivered_spike_count
                                   (synaptic + external events) */
    uint64_t fired_spikes;      /* NetworkPropagator::fired_spike_count */
    uint64_t synaptic_events;   /* delivered (synapse, offset) events */
    uint64_t external_events;   /* delivered injected events */
    uint64_t next_tick;         /* first tick not yet processed */
    uint64_t pending_events;    /* SpikeScheduler::pending_count */
    uint64_t raster_count;      /* fire records captured so far */
    uint64_t max_slot_events;   /* largest per-tick due list seen (engine stat) */
} snncuda_counters;
int snncuda_sim_counters(snncuda_sim* sim, snncuda_counters* out);

/* NetworkPropagator::idle (NetworkPropagator.cpp:74-76). */
int snncuda_sim_idle(snncuda_sim* sim, int32_t* out);

/* NeuronState (runtime/NeuronStateCache.h:15-45) of every neuron.  Any
 * pointer may be NULL.  Ticks that are std::nullopt in the reference read -1. */
typedef struct snncuda_neuron_state {
    float* membrane_potential;          /* [N] */
    uint64_t* spike_count;              /* [N] */
    int64_t* last_fired_tick;           /* [N] */
    uint64_t* last_active_tick;         /* [N] */
    float* compartment_current;         /* [N*4] soma, basal, apical, inhibitory */
    uint64_t* compartment_last_update;  /* [N*4] */
    float* compartment_tau;             /* [N*4] */
    uint64_t* window_start_tick;        /* [N] temporal_pattern.window_start_tick */
    uint64_t* offset_count;             /* [N] temporal_pattern.spike_offsets.size() */
    uint64_t* learned_count;            /* [N] temporal_pattern.learned_patterns.size() */
    uint64_t* match_count;              /* [N] */
    uint8_t* last_match;                /* [N] */
} snncuda_neuron_state;
int snncuda_sim_read_neurons(snncuda_sim* sim, const snncuda_neuron_state* out);

/* SynapseRuntimeState (runtime/SynapseDendriteProcessor.h:14-35) of every
 * synapse, in Connectome order.  Any pointer may be NULL. */
typedef struct snncuda_synapse_state {
    float* weight;
    int64_t* last_pre_spike_tick;
    int64_t* last_post_spike_tick;
    uint64_t* pre_spike_count;
    uint64_t* plasticity_update_count;
    float* last_weight_delta;
    uint64_t* code_window_start_tick;
    uint64_t* code_offset_count;
    uint64_t* learned_code_count;
    uint64_t* code_match_count;
    uint8_t* last_code_match;
} snncuda_synapse_state;
int snncuda_sim_read_synapses(snncuda_sim* sim, const snncuda_synapse_state* out);

/* One variable-length temporal list:
 *   kind 0: neuron `index` temporal_pattern.spike_offsets
 *   kind 1: neuron `index` learned_patterns[which]
 *   kind 2: synapse `index` code_offsets
 *   kind 3: synapse `index` learned_code_patterns[which]
 * Writes min(len, capacity) values and the full length to *len. */
int snncuda_sim_read_pattern(snncuda_sim* sim, int32_t kind, uint64_t index, uint64_t which,
                             uint32_t* values, uint64_t capacity, uint64_t* len);

/* 64-bit digests of the complete neuron and synapse state, defined over the
 * reference field values (see the implementation of digest_neurons /
 * digest_synapses); equal digests mean bit-identical state. */
int snncuda_sim_state_digest(snncuda_sim* sim, uint64_t* neuron_digest, uint64_t* synapse_digest);

/* Engine extension: order-independent 64-bit checksums of the neuron records
 * and of the synapse records (target-major, Connectome order inside each
 * target), computed on the device without copying the state back.  Equal
 * checksums of two runs of the same network mean equal state up to hash
 * collisions; they are comparable between a batch member
 * (snncuda_batch_state_checksums) and its solo run, not between
 * implementations (use snncuda_sim_state_digest for that).  CPU
 * implementations return SNNCUDA_ERR_UNSUPPORTED. */
int snncuda_sim_state_checksum(snncuda_sim* sim, uint64_t* neuron_sum, uint64_t* synapse_sum);

/* Fire records in processing order: (tick, neuron).  Requires
 * config.raster_capacity > 0. */
int snncuda_sim_read_raster(snncuda_sim* sim, uint64_t first, uint64_t count, uint64_t* ticks,
                            uint32_t* neurons);

/* ---- autotuning (engine extension) ----------------------------------------
 * No counterpart in the reference, whose CUDA backend launches fixed shapes
 * (CudaBackend.cu).  snncuda_sim_autotune runs the simulation's next ticks
 * in timed probes of probe_ticks ticks (each probe first runs up to one
 * captured graph of ticks untimed) and keeps, per knob, the fastest of a few
 * candidates: blocks of the synapse-event kernel (events per warp), of the
 * per-target walk, of the grouping and of the temporal update, and the ticks
 * per captured graph; then it shrinks the wheel-slot capacity to twice the
 * largest per-tick due list seen plus 2^16 events when that saves a quarter
 * or more of it.  The probed ticks are ordinary ticks of the simulation and
 * launch shapes never change results.  Threads per block stay 256: the
 * kernels' shared-memory layouts are built for it, and blocks per SM (the
 * knobs above) are the occupancy lever. */
typedef struct snncuda_tuning {
    uint32_t grid_events, grid_walk, grid_bucket, grid_temporal;  /* blocks */
    uint32_t ticks_per_graph;
    uint32_t block_threads;
    uint64_t slot_event_capacity;   /* after tuning */
    uint64_t max_slot_events;       /* largest due list seen so far */
    double ms_per_tick_before;      /* first probe */
    double ms_per_tick_after;       /* last probe, with the chosen shapes */
    uint32_t probes;
    uint64_t probe_ticks;
    uint32_t scatter_pass_events;   /* due-list events per grouping pass (0: one pass) */
    uint32_t side_serial;           /* 1: the neuron temporal update and post-spike STDP run in
                                       tick order instead of beside the synapse kernels and the
                                       fire ordering */
} snncuda_tuning;
int snncuda_sim_autotune(snncuda_sim* sim, uint64_t probe_ticks, snncuda_tuning* out);
/* Applies a tuning found earlier (by snncuda_sim_autotune on this or another
 * simulation; results do not depend on it).  Every field must lie in the
 * range the autotuner searches (SNNCUDA_ERR_INVALID_ARGUMENT otherwise);
 * slot_event_capacity 0 keeps the current capacity; the statistics fields
 * are ignored.  No reference counterpart (engine extension). */
int snncuda_sim_apply_tuning(snncuda_sim* sim, const snncuda_tuning* tuning);
/* Sets the wheel-slot capacity (rounded up to a multiple of 32); fails with
 * SNNCUDA_ERR_INVALID_ARGUMENT if a slot already holds more events. */
int snncuda_sim_set_slot_capacity(snncuda_sim* sim, uint64_t capacity);

/* ---- eviction: a simulation's device state to host memory and back ------
 * Replaces, for a whole simulation, the reference's write-back of evicted
 * neuron states to its NeuronStateStore and their reload on the next access
 * (NeuronStateCache.cpp:22-43, LruCache.h:44-63): the reference pages single
 * neuron states through an LRU cache; here the state stays resident on the
 * device and a simulation whose device memory is needed elsewhere (a
 * server's budget) is evicted as a whole.
 * snncuda_sim_evict waits for the simulation's work, copies its state (neuron
 * and synapse records, temporal patterns, the wheel's queued events, counters,
 * the raster) to host memory and frees its device memory.
 * snncuda_sim_restore allocates it again and copies the state back; every
 * call that needs the device state (run_until, readers, toggles) restores an
 * evicted simulation first.  Results are identical to never evicting.
 * snncuda_sim_residency reports whether the state is on the device and how
 * many times it was evicted. */
int snncuda_sim_evict(snncuda_sim* sim);
int snncuda_sim_restore(snncuda_sim* sim);
int snncuda_sim_residency(snncuda_sim* sim, int32_t* resident, uint64_t* evictions);

/* ---- batched form: many independent networks in one handle --------------
 * The reference runs one NetworkPropagator per network, one after the other
 * (or one CudaInferenceSession per network, CudaBackend.h:97-126).  A batch
 * holds `count` networks and advances all of them in one tick loop; every
 * network evolves exactly as it would alone under snncuda_sim_* (bit for
 * bit), with its own neuron and synapse numbering (0-based, in its own
 * Connectome order).  stdp_enabled[i] (NULL = all 1) is network i's
 * StdpConfig::enabled; the other config fields are shared.  The runtime
 * toggles apply to all networks (a network created with its rule disabled
 * stays disabled).  max_slot_events in the counters is batch-wide. */
typedef struct snncuda_batch snncuda_batch;
int snncuda_batch_create(uint32_t count, const snncuda_network* networks, const int32_t* stdp_enabled,
                         const snncuda_config* config, snncuda_batch** out);
int snncuda_batch_destroy(snncuda_batch* batch);
int snncuda_batch_inject(snncuda_batch* batch, uint32_t network, uint64_t count, const uint32_t* neurons,
                         const uint64_t* ticks, const float* weights);
int snncuda_batch_run_until(snncuda_batch* batch, uint64_t inclusive_tick);
int snncuda_batch_set_plasticity(snncuda_batch* batch, int32_t enabled);
int snncuda_batch_set_temporal_learning(snncuda_batch* batch, int32_t enabled);
int snncuda_batch_counters(snncuda_batch* batch, uint32_t network, snncuda_counters* out);
int snncuda_batch_read_neurons(snncuda_batch* batch, uint32_t network, const snncuda_neuron_state* out);
int snncuda_batch_read_synapses(snncuda_batch* batch, uint32_t network, const snncuda_synapse_state* out);
/* Digests of every network (arrays of `count`), as snncuda_sim_state_digest. */
int snncuda_batch_state_digests(snncuda_batch* batch, uint64_t* neuron_digests, uint64_t* synapse_digests);
/* snncuda_sim_autotune on the batch's one tick loop. */
int snncuda_batch_autotune(snncuda_batch* batch, uint64_t probe_ticks, snncuda_tuning* out);
/* snncuda_sim_apply_tuning on the batch's tick loop. */
int snncuda_batch_apply_tuning(snncuda_batch* batch, const snncuda_tuning* tuning);
/* Checksums of every network (arrays of `count`), as snncuda_sim_state_checksum. */
int snncuda_batch_state_checksums(snncuda_batch* batch, uint64_t* neuron_sums, uint64_t* synapse_sums);
/* Network's fire records [first, first + count) in its own processing order. */
int snncuda_batch_read_raster(snncuda_batch* batch, uint32_t network, uint64_t first, uint64_t count,
                              uint64_t* ticks, uint32_t* neurons);

/* ---- serving: jobs admitted under a device-memory budget -----------------
 * No counterpart in the reference, whose per-request path is one
 * NetworkPropagator (or CudaInferenceSession) built and run per request
 * (CudaBackend.h:97-126) with an LRU of neuron states for what does not fit
 * (NeuronStateCache.cpp:22-43).  A server takes jobs (a network, its
 * config, its injections, a tick count), admits them in submission order
 * while their estimated device bytes fit the budget, and advances every
 * admitted job by `slice_ticks` per scheduling round, each on its own CUDA
 * stream, so the GPU runs many jobs at once; a finished job's memory goes
 * back to the budget.  Every job's results equal a solo run of it.
 * Single host thread; the caller drives it with snncuda_server_step. */
typedef struct snncuda_server snncuda_server;
typedef struct snncuda_server_config {
    uint64_t memory_budget_bytes;  /* device bytes running jobs may hold (0 = 120 GB) */
    uint32_t max_running;          /* jobs advanced side by side (0 = 64) */
    uint32_t slice_ticks;          /* ticks per job and scheduling round (0 = 64) */
    int32_t digests;               /* compute state digests of finished jobs */
    int32_t evict;                 /* 1: a queued job that does not fit the budget
                                      preempts running jobs with more remaining
                                      work (synapses x ticks left), which are
                                      evicted to host memory (snncuda_sim_evict)
                                      and resume when the budget has room */
} snncuda_server_config;
int snncuda_server_create(const snncuda_server_config* config, snncuda_server** out);
int snncuda_server_destroy(snncuda_server* server);
/* Queues a job that runs ticks 0 .. ticks-1.  The network's arrays and the
 * injections are copied here: the caller may free them when the call
 * returns.  *job_id numbers jobs from 0 in submission order. */
int snncuda_server_submit(snncuda_server* server, const snncuda_network* network, const snncuda_config* config,
                          uint64_t inject_count, const uint32_t* neurons, const uint64_t* ticks,
                          const float* weights, uint64_t run_ticks, uint64_t* job_id);
/* One scheduling round: finished slices are checked, finished jobs retired,
 * the next slice of every running job enqueued, then queued jobs admitted
 * while they fit.  *active = jobs queued or running afterwards. */
int snncuda_server_step(snncuda_server* server, uint32_t* active);
typedef struct snncuda_job_result {
    int32_t state;                 /* 0 queued, 1 running, 2 done, 3 failed,
                                      4 evicted (waiting in host memory) */
    int32_t error;                 /* SNNCUDA_ERR_* of a failed job */
    snncuda_counters counters;     /* of a finished job */
    uint64_t neuron_digest, synapse_digest;  /* when config.digests */
    uint64_t device_bytes;         /* the admission estimate */
    double submitted_s, admitted_s, finished_s;  /* seconds since server creation */
    uint64_t evictions;            /* times the job was evicted to host memory */
} snncuda_job_result;
int snncuda_server_job(snncuda_server* server, uint64_t job_id, snncuda_job_result* out);
/* Device bytes a simulation of `network` under `config` holds at most
 * (creation included); the admission estimate of the server. */
int snncuda_sim_estimate_bytes(const snncuda_network* network, const snncuda_config* config, uint64_t* bytes);

/* ---- engine extension: per-kernel device time ----------------------------
 * No counterpart in the reference (which times the whole tick loop on the
 * host clock, spike_throughput_benchmark.cpp:137-140).  Processes ticks like
 * snncuda_sim_run_until, but launches one tick at a time from a graph whose
 * event nodes bracket every kernel, and accumulates device time per kernel
 * plus the work counters of the profiled ticks into *out (zero it first). */
#define SNNCUDA_KERNEL_COUNT 10
typedef struct snncuda_profile {
    uint64_t ticks;
    double kernel_ms[SNNCUDA_KERNEL_COUNT];
    uint64_t synaptic_events;
    uint64_t external_events;
    uint64_t fires;
    uint64_t touched_targets;   /* sum over ticks of targets with due events */
} snncuda_profile;
int snncuda_sim_profile(snncuda_sim* sim, uint64_t inclusive_tick, snncuda_profile* out);

/* Recognition sums (engine extension): the sum over neurons of
 * temporal_pattern.match_count and over synapses of code_match_count,
 * reduced on the device (reading every record back would move the whole
 * synapse state). */
int snncuda_sim_recognition(snncuda_sim* sim, uint64_t* neuron_matches, uint64_t* synapse_code_matches);
const char* snncuda_kernel_name(int32_t index);

/* ---- inference readouts -------------------------------------------------
 * Replace the reference inference session's readout paths
 * (CudaInferenceSession::run_feedforward_batch and
 * run_recurrent_feedforward_batch, CudaBackend.h:115-121,
 * CudaBackend.cu:1725-2100) over a network's initial weights.  Samples are
 * CSR: sample s's inputs are input_neurons / input_weights
 * [input_ptr[s], input_ptr[s+1]); a sample's inputs to one neuron are summed
 * first (in input order) and delivered[s] receives the number of distinct
 * input neurons.  scores and spikes are [samples][readout_count]: spikes
 * are 1 where the score reaches the readout neuron's threshold.  Every sum
 * is formed in a fixed order (a neuron's incoming synapses in Connectome
 * order, time steps in order) where the reference adds with float atomics in
 * an unspecified order.  A neuron listed twice among the readouts or among
 * the hidden neurons is rejected (SNNCUDA_ERR_INVALID_ARGUMENT). */
typedef struct snncuda_readout snncuda_readout;
int snncuda_readout_create(const snncuda_network* network, snncuda_readout** out);
int snncuda_readout_destroy(snncuda_readout* readout);
/* One hop: score = sum over the readout's incoming synapses whose source is
 * an input of input weight x synapse weight. */
int snncuda_readout_feedforward(snncuda_readout* readout, uint32_t samples, const uint64_t* input_ptr,
                                const uint32_t* input_neurons, const float* input_weights, uint32_t readout_count,
                                const uint32_t* readout_neurons, float* scores, uint64_t* spikes,
                                uint64_t* delivered);
/* CudaRecurrentFeedforwardOptions (CudaBackend.h:69-79) without the
 * full-spike-timing switch (that mode is the tick simulation itself). */
typedef struct snncuda_recurrent_options {
    uint32_t iterations;              /* 1 */
    float feedback_decay;             /* 0.5 */
    uint32_t top_k_feedback_readouts; /* 1; 0 = every readout at or above its threshold */
    uint32_t top_k_hidden;            /* 0 = no hidden selection */
    int32_t use_scores_not_spikes;    /* 1: gates carry the readout score, 0: 1 */
} snncuda_recurrent_options;
void snncuda_recurrent_options_default(snncuda_recurrent_options* options);
/* max_delay x (1 + 2 x iterations) + 1 time steps (*time_steps): the inputs
 * that are hidden neurons start as hidden events at step 0; each step keeps
 * the top_k_hidden largest hidden events (when 0 < top_k_hidden <
 * hidden_count), sends hidden events to the readouts (a synapse of delay d,
 * at least 1, lands d steps later), gates the readouts of the step and feeds
 * the gated readouts back to the hidden neurons scaled by feedback_decay;
 * scores are the readout events summed over the steps.  hidden_count 0 =
 * every neuron that is not a readout, in index order. */
int snncuda_readout_recurrent(snncuda_readout* readout, uint32_t samples, const uint64_t* input_ptr,
                              const uint32_t* input_neurons, const float* input_weights, uint32_t readout_count,
                              const uint32_t* readout_neurons, uint32_t hidden_count, const uint32_t* hidden_neurons,
                              const snncuda_recurrent_options* options, float* scores, uint64_t* spikes,
                              uint64_t* delivered, uint64_t* time_steps);

/* ---- building block: group a tick's due events by target ----------------
 * Replaces, for one tick, the due list SpikeScheduler::pop_due returns
 * (SpikeScheduler.cpp:25-47) as NetworkPropagator::process_tick consumes it
 * per target (NetworkPropagator.cpp:80-131): the events regrouped by target
 * neuron with their due order kept inside each target -- the engine's own
 * grouping step.
 *   events         device array of `count` event words: low 32 bits target
 *                  neuron (bit 31 set for an external input), high 32 bits
 *                  payload (synapse slot or input weight bits)
 *   grouped        device array of `count` words: targets in ascending order,
 *                  each target's events as (payload << 32) | (input index |
 *                  external bit), in input order
 *   segment_start  device array of neuron_count + 1 entries: first grouped
 *                  word of each target; [neuron_count] = count
 * Runs on cuda_stream (NULL: the legacy default stream) and returns when the
 * device has finished.  Allocates and frees its scratch on every call.
 * A target >= neuron_count, or events overlapping grouped (no in-place
 * grouping), fails with SNNCUDA_ERR_INVALID_ARGUMENT. */
int snncuda_group_events(const uint64_t* events, uint32_t count, uint32_t neuron_count, uint64_t* grouped,
                         uint32_t* segment_start, void* cuda_stream);

/* ---- no-allocation variant of snncuda_group_events -----------------------
 * Has no counterpart in the reference.  For callers that cannot allocate
 * device memory at the point of the call: code whose device memory is owned
 * by another allocator's pool or budget (a host framework's caching
 * allocator), and latency-critical loops that must not pay cudaMalloc /
 * cudaFree, which can synchronize the whole device and stall other streams.
 * Same arguments and results as snncuda_group_events; the caller still
 * provides the inputs and outputs, but the scratch (bucket counters, the
 * events in bucket order) lives in one static device array compiled
 * into the library (about 17 MB, held on every GPU that loads the library
 * until the process exits).  Limits: count <= SNNCUDA_GROUP_STATIC_MAX_EVENTS
 * and neuron_count <= SNNCUDA_GROUP_STATIC_MAX_NEURONS, otherwise
 * SNNCUDA_ERR_CAPACITY.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture (later calls made outside a capture
 * look the address up again, so it stays valid across a cudaDeviceReset).
 * Every call shares the one array:
 * calls that overlap on the GPU (other streams or host threads) race and must
 * be serialized by the caller. */
#define SNNCUDA_GROUP_STATIC_MAX_EVENTS (1u << 20)
#define SNNCUDA_GROUP_STATIC_MAX_NEURONS (1u << 18)
int snncuda_group_events_static(const uint64_t* events, uint32_t count, uint32_t neuron_count,
                                uint64_t* grouped, uint32_t* segment_start, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* SNNCUDA_GB300_H */
