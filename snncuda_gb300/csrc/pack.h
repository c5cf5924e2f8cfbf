// Device-side packing of a flattened Connectome (pack.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "engine.h"
#include "snncuda_gb300.h"

namespace snngb {

// One device allocation of a simulation and what an eviction to host memory
// keeps of it: the whole buffer (state), nothing (per-tick scratch whose
// contents do not outlive a tick), or the live prefix of every wheel slot.
// kZero buffers are scratch that must read zero between ticks (restored as
// zeros).
enum class BufKind : uint8_t { kState, kScratch, kWheel, kZero };
struct DeviceBuffer {
    void* p;
    size_t bytes;
    BufKind kind;
};
using DeviceBuffers = std::vector<DeviceBuffer>;

struct PackOut {
    // device buffers, owned by the caller's `owned` list
    SynAB* syn{nullptr};                      // [S] target-major records
    unsigned long long* in_ptr_d{nullptr};    // [N+1] incoming row pointers
    unsigned long long* pre_base{nullptr};    // [N] first pre-expanded event of each source
    uint32_t* pre_off{nullptr};               // [N*(D+1)] class offsets within a source
    unsigned long long* pre_ev{nullptr};      // [pre_total] pre-expanded events
    uint32_t* c_of_tm_d{nullptr};             // [S] Connectome index of each target-major slot
    uint32_t* tm_of_c_d{nullptr};             // [S] inverse
    // host results
    std::vector<uint64_t> in_ptr;             // [N+1]
    std::vector<uint32_t> cls_delta;          // delivery delay of each class, ascending
    uint32_t max_expected{2};
    unsigned long long pre_total{0};
};

// Validates the synapse arrays of `net` and builds the engine's synapse-side
// layout on the device (stream `st`).  Persistent buffers are allocated
// stream-ordered on `st` (cudaMallocAsync) and appended to `owned`.  Returns SNNCUDA_OK or an SNNCUDA_ERR_* code with
// `msg` set.
int pack_network_device(const snncuda_network* net, float cfg_max_weight, cudaStream_t st,
                        DeviceBuffers& owned, PackOut& out, std::string& msg);

// Sets the thread-local message snncuda_last_error() returns (sim.cu).
void set_last_error_message(const std::string& msg);

}  // namespace snngb
