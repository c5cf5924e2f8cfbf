// Measurement helper (not part of the engine): throughput of random 64-byte
// record read-modify-writes on this GPU, the access pattern of the per-event
// synapse update.  Prints one JSON object: microseconds per batch of
// `events` random records out of `records` (64 B each), for a read-modify-
// write and for a read-only pass, at three grid sizes.
//
// With the optional band and row arguments it also times the two patterns
// of the other synapse order (records of one source contiguous, sorted by
// delay) beside the target-major one, for one tick's work:
//   band_rmw  `bands` runs of `band_len` consecutive records, `picks`
//             random records read-modified-written in each (the events of
//             one source and one due tick: its synapses whose delay plus a
//             code offset equals that tick, a band of the sorted row);
//   row_rmw   `rows` runs of `row_len` consecutive records, every record
//             read-modified-written (post-spike STDP over a fired target's
//             incoming synapses, contiguous when records are target-major);
//   post_rmw  rows x row_len random records (the same STDP when records
//             are source-major).
//   rmw_floor [records] [events] [bands band_len picks rows row_len]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

namespace {

struct alignas(64) Rec {
    unsigned int w[16];
};

__device__ __forceinline__ unsigned long long mix(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__global__ void rmw(Rec* r, unsigned long long n, unsigned long long records, unsigned long long seed) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long j = __umul64hi(mix(i + seed), records);  // uniform in [0, records)
        Rec x = r[j];
        x.w[0] += 1;
        x.w[9] += 2;
        r[j] = x;
    }
}

__global__ void rd(const Rec* r, unsigned long long n, unsigned long long records, unsigned long long seed,
                   unsigned int* out) {
    unsigned int acc = 0;
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long j = __umul64hi(mix(i + seed), records);
        acc += r[j].w[0] + r[j].w[9];
    }
    if (acc == 0xFFFFFFFFu) *out = acc;
}

// A warp per band: picks random records of a random run of band_len.
__global__ void band_rmw(Rec* r, unsigned long long bands, unsigned long long band_len, unsigned int picks,
                         unsigned long long records, unsigned long long seed) {
    const unsigned int lane = threadIdx.x & 31;
    const unsigned long long warps = static_cast<unsigned long long>(gridDim.x) * blockDim.x / 32;
    for (unsigned long long b = (blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x) / 32;
         b < bands; b += warps) {
        const unsigned long long start = __umul64hi(mix(b + seed), records - band_len);
        for (unsigned int k = lane; k < picks; k += 32) {
            const unsigned long long j = start + __umul64hi(mix(b * picks + k + seed * 3), band_len);
            Rec x = r[j];
            x.w[0] += 1;
            x.w[9] += 2;
            r[j] = x;
        }
    }
}

// A warp per row: every record of a random run of row_len.
__global__ void row_rmw(Rec* r, unsigned long long rows, unsigned long long row_len, unsigned long long records,
                        unsigned long long seed) {
    const unsigned int lane = threadIdx.x & 31;
    const unsigned long long warps = static_cast<unsigned long long>(gridDim.x) * blockDim.x / 32;
    for (unsigned long long b = (blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x) / 32;
         b < rows; b += warps) {
        const unsigned long long start = __umul64hi(mix(b + seed), records - row_len);
        for (unsigned long long k = lane; k < row_len; k += 32) {
            Rec x = r[start + k];
            x.w[0] += 1;
            x.w[9] += 2;
            r[start + k] = x;
        }
    }
}

}  // namespace

int main(int argc, char** argv) {
    const unsigned long long records = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 100000000ull;
    const unsigned long long events = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1260000ull;
    const bool patterns = argc > 7;
    const unsigned long long bands = patterns ? std::strtoull(argv[3], nullptr, 10) : 0;
    const unsigned long long band_len = patterns ? std::strtoull(argv[4], nullptr, 10) : 1;
    const unsigned int picks = patterns ? static_cast<unsigned int>(std::strtoul(argv[5], nullptr, 10)) : 0;
    const unsigned long long rows = patterns ? std::strtoull(argv[6], nullptr, 10) : 0;
    const unsigned long long row_len = patterns ? std::strtoull(argv[7], nullptr, 10) : 1;
    if (records == 0 || band_len == 0 || row_len == 0 || band_len >= records || row_len >= records) {
        std::printf("{\"error\": \"records must exceed band_len and row_len, all nonzero\"}\n");
        return 1;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    Rec* r = nullptr;
    unsigned int* o = nullptr;
    if (cudaMalloc(&r, records * sizeof(Rec)) != cudaSuccess || cudaMalloc(&o, 4) != cudaSuccess) {
        std::printf("{\"error\": \"allocation failed\"}\n");
        return 1;
    }
    cudaMemset(r, 0, records * sizeof(Rec));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    std::printf("{\"records\": %llu, \"events\": %llu, \"runs\": [", records, events);
    const int mult[3] = {8, 16, 32};
    for (int g = 0; g < 3; ++g) {
        const int grid = sms * mult[g];
        for (int it = 0; it < 3; ++it) rmw<<<grid, 256>>>(r, events, records, 1000 + it);
        cudaEventRecord(a);
        for (int it = 0; it < 20; ++it) rmw<<<grid, 256>>>(r, events, records, 77 + it * 1000003ull);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms_rmw = 0.0f, ms_rd = 0.0f;
        cudaEventElapsedTime(&ms_rmw, a, b);
        cudaEventRecord(a);
        for (int it = 0; it < 20; ++it) rd<<<grid, 256>>>(r, events, records, 99 + it * 1000003ull, o);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms_rd, a, b);
        std::printf("%s{\"grid\": %d, \"rmw_us\": %.1f, \"read_us\": %.1f}", g ? ", " : "", grid, ms_rmw * 50.0f,
                    ms_rd * 50.0f);
    }
    std::printf("]");
    if (patterns) {
        const int grid = sms * 32;
        float ms[3] = {0.0f, 0.0f, 0.0f};
        for (int kind = 0; kind < 3; ++kind) {
            for (int it = 0; it < 23; ++it) {
                if (it == 3) cudaEventRecord(a);
                const unsigned long long seed = 55 + it * 1000003ull;
                if (kind == 0) band_rmw<<<grid, 256>>>(r, bands, band_len, picks, records, seed);
                if (kind == 1) row_rmw<<<grid, 256>>>(r, rows, row_len, records, seed);
                if (kind == 2) rmw<<<grid, 256>>>(r, rows * row_len, records, seed);
            }
            cudaEventRecord(b);
            cudaEventSynchronize(b);
            cudaEventElapsedTime(&ms[kind], a, b);
        }
        std::printf(", \"bands\": %llu, \"band_len\": %llu, \"picks\": %u, \"rows\": %llu, \"row_len\": %llu, "
                    "\"band_rmw_us\": %.1f, \"row_rmw_us\": %.1f, \"post_random_rmw_us\": %.1f",
                    bands, band_len, picks, rows, row_len, ms[0] * 50.0f, ms[1] * 50.0f, ms[2] * 50.0f);
    }
    const cudaError_t err = cudaGetLastError();
    std::printf(", \"status\": \"%s\"}\n", cudaGetErrorString(err));
    return err == cudaSuccess ? 0 : 1;
}
