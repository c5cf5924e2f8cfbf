// Measurement helper (not part of the engine): throughput of random 64-byte
// record read-modify-writes on this GPU, the access pattern of the per-event
// synapse update.  Prints one JSON object: microseconds per batch of
// `events` random records out of `records` (64 B each), for a read-modify-
// write and for a read-only pass, at three grid sizes.
//   rmw_floor [records] [events]
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

}  // namespace

int main(int argc, char** argv) {
    const unsigned long long records = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 100000000ull;
    const unsigned long long events = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1260000ull;
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
    const cudaError_t err = cudaGetLastError();
    std::printf("], \"status\": \"%s\"}\n", cudaGetErrorString(err));
    return err == cudaSuccess ? 0 : 1;
}
