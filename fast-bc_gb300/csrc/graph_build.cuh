// Edge list -> CSR on the device, with the rules of DirectedWeightedGraph (DirectedWeightedGraph.h:
// 67-96, 136-170): n = 1 + the largest source id, a destination id >= n is an error, a weight
// must be > 0, and a repeated (source, destination) pair has its weights summed (in input
// order, as the host path does).  The engine then needs integer weights below 2^31.
//
// Rows are built by a counting scatter on the source id, each row is sorted by
// (destination, input index) -- one thread per row, rows of up to kRowMax edges (longer rows:
// the host path) -- and equal destinations are merged.
#pragma once
#include <cstdint>

namespace fbc {

constexpr int kRowMax = 1024;

// error bits
constexpr int kGbNegId = 1;      // negative vertex id
constexpr int kGbWeight = 2;     // weight <= 0 (or NaN)
constexpr int kGbDst = 4;        // destination >= n
constexpr int kGbLongRow = 8;    // a row longer than kRowMax (host path)
constexpr int kGbNonInt = 16;    // merged weight not an integer below 2^31

__global__ void gb_check_kernel(int64_t m, const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                const double* __restrict__ w, int* maxsrc, int* err) {
    int mx = -1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (src[i] < 0 || dst[i] < 0) atomicOr(err, kGbNegId);
        if (!(w[i] > 0)) atomicOr(err, kGbWeight);
        mx = max(mx, src[i]);
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0) atomicMax(maxsrc, mx);
}

__global__ void gb_count_kernel(int64_t m, const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                int32_t n, int32_t* deg, int* err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (dst[i] >= n) atomicOr(err, kGbDst);
        atomicAdd(deg + src[i], 1);
    }
}

// keys[rs[src] + k] = (dst << 32 | i) in any order within the row (sorted afterwards)
__global__ void gb_scatter_kernel(int64_t m, const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                  const int32_t* __restrict__ rs, int32_t* cursor, unsigned long long* keys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t s = src[i];
        const int32_t k = atomicAdd(cursor + s, 1);
        keys[rs[s] + k] = ((unsigned long long)(uint32_t)dst[i] << 32) | (unsigned long long)(uint32_t)i;
    }
}

// sort each row's keys (insertion sort, rows <= kRowMax) and count its distinct destinations
__global__ void gb_sort_rows_kernel(int32_t n, const int32_t* __restrict__ rs, unsigned long long* keys,
                                    int32_t* ndeg, int* err) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = rs[v], b = rs[v + 1];
        if (b - a > kRowMax) {
            atomicOr(err, kGbLongRow);
            ndeg[v] = 0;
            continue;
        }
        for (int32_t i = a + 1; i < b; ++i) {
            const unsigned long long k = keys[i];
            int32_t j = i - 1;
            while (j >= a && keys[j] > k) {
                keys[j + 1] = keys[j];
                --j;
            }
            keys[j + 1] = k;
        }
        int32_t d = 0;
        for (int32_t i = a; i < b; ++i) d += (i == a || (keys[i] >> 32) != (keys[i - 1] >> 32));
        ndeg[v] = d;
    }
}

// merged rows: (dst, sum of its weights in input order) at rp[v] ..; per-graph statistics
__global__ void gb_merge_kernel(int32_t n, const int32_t* __restrict__ rs, const unsigned long long* __restrict__ keys,
                                const double* __restrict__ w, const int32_t* __restrict__ rp, int2* adj,
                                int32_t* indeg, int* maxw, unsigned long long* sumw, int* err) {
    int mw = 0;
    unsigned long long sw = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = rs[v], b = rs[v + 1];
        int32_t o = rp[v];
        for (int32_t i = a; i < b;) {
            const uint32_t d = (uint32_t)(keys[i] >> 32);
            double x = 0.0;
            int32_t j = i;
            for (; j < b && (uint32_t)(keys[j] >> 32) == d; ++j) x += w[(uint32_t)keys[j]];
            int32_t wi = 0;
            if (x != floor(x) || x > 2147483647.0) atomicOr(err, kGbNonInt);
            else wi = (int32_t)x;
            adj[o++] = make_int2((int32_t)d, wi);
            atomicAdd(indeg + d, 1);
            mw = max(mw, wi);
            sw += (unsigned long long)wi;
            i = j;
        }
    }
    mw = __reduce_max_sync(0xffffffffu, mw);
    for (int d = 16; d > 0; d >>= 1) sw += __shfl_down_sync(0xffffffffu, sw, d);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxw, mw);
        atomicAdd(sumw, sw);  // one per warp: a per-thread add to one word serialises
    }
}

__global__ void gb_max_kernel(int32_t n, const int32_t* __restrict__ x, int* out) {
    int mx = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        mx = max(mx, x[v]);
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

}  // namespace fbc
