// Random-access ceiling of the device memory: chains of dependent 8-byte loads at random
// addresses, for several footprints, with one warp per SM (latency) and with 512 threads per
// SM (throughput), each warp either over the whole footprint or confined to its own 32 MB
// region (the per-source state of a Brandes unit).  The Brandes kernels touch most vertex
// state once per pass at scattered addresses, so this ceiling -- sectors per second, not the
// streaming bandwidth -- is what bounds them on million-vertex graphs.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o random_access_probe \
//        fast-bc_gb300/random_access_probe.cu && ./random_access_probe
//
// Every index is reduced modulo its region, so every load stays inside the buffer; each chain
// has a fixed length, so every launch ends.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

__global__ void fill(uint64_t* b, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = mix64(i * 0x9E3779B97F4A7C15ULL + 1);
}

// region: words of each warp's region (0 = the whole buffer)
__global__ void chase(const uint64_t* b, uint64_t n, uint64_t region, int steps, uint64_t* sink) {
    const uint64_t gt = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t base = 0, span = n;
    if (region) {
        const uint64_t nreg = n / region;
        base = ((gt >> 5) % nreg) * region;
        span = region;
    }
    uint64_t idx = mix64(gt + 12345) % span, acc = 0;
    for (int s = 0; s < steps; ++s) {
        const uint64_t v = __ldcg(b + base + idx);
        acc += v;
        idx = (v ^ (uint64_t)s) % span;
    }
    if (acc == 42) sink[0] = acc;
}

int main() {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const uint64_t maxw = (64ull << 30) / 8;
    uint64_t *b = nullptr, *sink = nullptr;
    if (cudaMalloc(&b, maxw * 8) != cudaSuccess || cudaMalloc(&sink, 8) != cudaSuccess) {
        std::printf("allocation failed\n");
        return 1;
    }
    fill<<<sms * 8, 256>>>(b, maxw);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const uint64_t foots[] = {16ull << 20, 128ull << 20, 1ull << 30, 8ull << 30, 32ull << 30, 64ull << 30};
    const int thr[] = {32, 512};
    for (uint64_t f : foots)
        for (int t : thr)
            for (int loc = 0; loc < 2; ++loc) {
                const uint64_t n = f / 8, region = loc ? (32ull << 20) / 8 : 0;
                if (loc && n <= region) continue;
                const int steps = 2000;
                chase<<<sms, t>>>(b, n, region, 50, sink);
                cudaEventRecord(e0);
                chase<<<sms, t>>>(b, n, region, steps, sink);
                cudaEventRecord(e1);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                std::printf("footprint %6.2f GB  threads/SM %4d  %-11s  latency %7.1f ns/load  %6.2f G loads/s\n",
                            f / 1073741824.0, t, loc ? "32MB-region" : "whole", ms * 1e6 / steps,
                            (double)sms * t * steps / (ms * 1e-3) / 1e9);
            }
    const cudaError_t err = cudaGetLastError();
    std::printf("status %s\n", cudaGetErrorString(err));
    cudaFree(b);
    cudaFree(sink);
    return err == cudaSuccess ? 0 : 1;
}
