// The k-means step of the clustered pivot selection on the device:
// PlusPlusKMeans::computeCentroids (libfastbc/include/kmeans/PlusPlusKMeans.h:76-147) with its
// k-means++ initialisation (PlusPlusKMeans.h:150-183) and stopping rule (PlusPlusKMeans.h:186-207),
// for many independent point sets (one per Louvain community) at once, one thread block per set.
//
// A point is a vertex's border vector, normalized (VertexInfo::normalize): integer lengths and
// integer path counts.  Between two points VertexInfo::squaredDistance is a sum of integer squares,
// computed here in int64 -- the same value the reference's double sum holds exactly (the host
// refuses sets whose sums could pass 2^53).  The rounded steps keep the reference's operation
// order, each product and sum rounded separately (no fused multiply-add):
//   * the running mean distance of the initialisation, cdist = cdist * (1 - 1/i) + d * (1/i);
//   * a centroid's mean vector, the exact member sums divided by the member count;
//   * the distance of the mean to a member, summed over the borders in order.
// Ties keep the reference's sequential choices: the first point of largest running distance, the
// first centroid of least distance, the first member (in point order) nearest to the mean.
// Every loop is bounded by k, the set size and max_iter + 1 Lloyd steps.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fbc {

struct KMSet {
    int64_t x_off;     // first entry of the set's points in X: entry i * np + j = border i of point j
    int64_t ws_off;    // byte offset of the set's work area in KMParams::ws
    int64_t out_off;   // first output entry (k of them)
    int64_t p_off;     // first point of the set in the weight array
    int32_t np, nb, k, pad;
};

struct KMParams {
    const KMSet* sets;
    const int2* X;            // (length, count) per border and point, sets back to back
    const int32_t* wt;        // point weights
    char* ws;
    double min_variance;
    int32_t max_iter;
    int32_t* out_idx;         // centroid c of set s: point index within the set
    int32_t* out_w;           // summed weights of its members in the last assignment
};

// Work area of one set (all offsets 256-byte aligned).
struct KMWork {
    double* cdist;            // np
    double* mdist;            // np: distance of each point to its centroid's mean
    int32_t* assign;          // np
    int32_t* cent;            // k: the centroids of the current Lloyd step
    int32_t* ncent;           // k: the next step's
    int32_t* cnt;             // k
    int32_t* wsum;            // k
    unsigned long long* best; // k: least mean distance (bits of a non-negative double)
    int32_t* bestj;           // k
    long long* suml;          // k * nb
    long long* sumc;          // k * nb
};

__host__ __device__ inline int64_t km_al(int64_t x) { return (x + 255) & ~int64_t(255); }
__host__ __device__ inline int64_t km_work_bytes(int64_t np, int64_t nb, int64_t k) {
    return 2 * km_al(np * 8) + km_al(np * 4) + 4 * km_al(k * 4) + km_al(k * 8) + km_al(k * 4) +
           2 * km_al(k * (nb > 0 ? nb : 1) * 8);
}
__device__ inline KMWork km_carve(char* p, int64_t np, int64_t nb, int64_t k) {
    KMWork w;
    w.cdist = (double*)p; p += km_al(np * 8);
    w.mdist = (double*)p; p += km_al(np * 8);
    w.assign = (int32_t*)p; p += km_al(np * 4);
    w.cent = (int32_t*)p; p += km_al(k * 4);
    w.ncent = (int32_t*)p; p += km_al(k * 4);
    w.cnt = (int32_t*)p; p += km_al(k * 4);
    w.wsum = (int32_t*)p; p += km_al(k * 4);
    w.best = (unsigned long long*)p; p += km_al(k * 8);
    w.bestj = (int32_t*)p; p += km_al(k * 4);
    w.suml = (long long*)p; p += km_al(k * (nb > 0 ? nb : 1) * 8);
    w.sumc = (long long*)p;
    return w;
}

// squared distance of points a and b (exact)
__device__ __forceinline__ long long km_sqd(const int2* X, int np, int nb, int a, int b) {
    long long s = 0;
    for (int i = 0; i < nb; ++i) {
        const int2 xa = __ldg(X + (int64_t)i * np + a), xb = __ldg(X + (int64_t)i * np + b);
        const long long d = (long long)xa.x - xb.x, e = (long long)xa.y - xb.y;
        s += d * d + e * e;
    }
    return s;
}

// Block-wide reduction of (value, index): the largest value (kMax) or the smallest, the smallest
// index among equal values.  Every thread gets the result.
template <bool kMax>
__device__ inline void km_block_pick(double& v, int& j, double* sv, int* sj) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const double v2 = __shfl_down_sync(0xffffffffu, v, o);
        const int j2 = __shfl_down_sync(0xffffffffu, j, o);
        if ((kMax ? v2 > v : v2 < v) || (v2 == v && j2 < j)) { v = v2; j = j2; }
    }
    __syncthreads();  // sv/sj free from any earlier use
    if (lane == 0) { sv[w] = v; sj[w] = j; }
    __syncthreads();
    if (w == 0) {
        v = lane < nw ? sv[lane] : (kMax ? -1.0 : 1.8e308);
        j = lane < nw ? sj[lane] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            const double v2 = __shfl_down_sync(0xffffffffu, v, o);
            const int j2 = __shfl_down_sync(0xffffffffu, j, o);
            if ((kMax ? v2 > v : v2 < v) || (v2 == v && j2 < j)) { v = v2; j = j2; }
        }
        if (lane == 0) { sv[0] = v; sj[0] = j; }
    }
    __syncthreads();
    v = sv[0];
    j = sj[0];
}

__global__ void __launch_bounds__(1024) kmeans_kernel(KMParams P) {
    __shared__ double sv[32];
    __shared__ int sj[32];
    const KMSet S = P.sets[blockIdx.x];
    const int np = S.np, nb = S.nb, k = S.k, tid = threadIdx.x, nth = blockDim.x;
    const int2* X = P.X + S.x_off;
    const KMWork W = km_carve(P.ws + S.ws_off, np, nb, k);

    // ---------------------------------------------- k-means++ initialisation (_initPlusPlus)
    for (int j = tid; j < np; j += nth) W.cdist[j] = 0.0;
    if (tid == 0) W.ncent[0] = 0;
    __syncthreads();
    for (int i = 1; i < k; ++i) {
        const int lc = W.ncent[i - 1];
        const double p = 1.0 / (double)i;
        const double q = 1.0 - p;
        double bv = -1.0;
        int bj = 0x7fffffff;
        for (int j = tid; j < np; j += nth) {
            const double d = (double)km_sqd(X, np, nb, lc, j);
            const double c = __dadd_rn(__dmul_rn(W.cdist[j], q), __dmul_rn(d, p));
            W.cdist[j] = c;
            if (c > bv || (c == bv && j < bj)) { bv = c; bj = j; }
        }
        km_block_pick<true>(bv, bj, sv, sj);
        if (tid == 0) W.ncent[i] = bj;
        __syncthreads();
    }

    // ------------------------------------------------------------------ Lloyd steps
    int iter = 0;
    for (;;) {
        ++iter;
        for (int c = tid; c < k; c += nth) {
            W.cent[c] = W.ncent[c];
            W.cnt[c] = 0;
            W.best[c] = ~0ull;
            W.bestj[c] = 0x7fffffff;
        }
        for (int64_t e = tid; e < (int64_t)k * nb; e += nth) {
            W.suml[e] = 0;
            W.sumc[e] = 0;
        }
        __syncthreads();
        // each point to its nearest centroid, first on ties; exact integer sums per centroid
        for (int j = tid; j < np; j += nth) {
            int best = 0;
            long long bd = km_sqd(X, np, nb, W.cent[0], j);
            for (int c = 1; c < k; ++c) {
                const long long d = km_sqd(X, np, nb, W.cent[c], j);
                if (d < bd) { bd = d; best = c; }
            }
            W.assign[j] = best;
            atomicAdd(W.cnt + best, 1);
            for (int i = 0; i < nb; ++i) {
                const int2 x = __ldg(X + (int64_t)i * np + j);
                atomicAdd((unsigned long long*)(W.suml + (int64_t)best * nb + i), (unsigned long long)(long long)x.x);
                atomicAdd((unsigned long long*)(W.sumc + (int64_t)best * nb + i), (unsigned long long)(long long)x.y);
            }
        }
        __syncthreads();
        // distance of each point to its centroid's mean (the mean's entries: exact sum / count)
        for (int j = tid; j < np; j += nth) {
            const int c = W.assign[j];
            const double n = (double)W.cnt[c];
            double s = 0.0;
            for (int i = 0; i < nb; ++i) {
                const int2 x = __ldg(X + (int64_t)i * np + j);
                const double ml = __ddiv_rn((double)W.suml[(int64_t)c * nb + i], n);
                const double mc = __ddiv_rn((double)W.sumc[(int64_t)c * nb + i], n);
                const double d = __dsub_rn(ml, (double)x.x);
                s = __dadd_rn(s, __dmul_rn(d, d));
                const double e = __dsub_rn(mc, (double)x.y);
                s = __dadd_rn(s, __dmul_rn(e, e));
            }
            W.mdist[j] = s;
            atomicMin(W.best + c, (unsigned long long)__double_as_longlong(s));  // s >= 0: bits order as values
        }
        __syncthreads();
        for (int j = tid; j < np; j += nth) {
            const int c = W.assign[j];
            if ((unsigned long long)__double_as_longlong(W.mdist[j]) == W.best[c]) atomicMin(W.bestj + c, j);
        }
        __syncthreads();
        for (int c = tid; c < k; c += nth) W.ncent[c] = W.cnt[c] ? W.bestj[c] : W.cent[c];
        __syncthreads();
        // the largest move of a centroid (_centroidVariance)
        double var = 0.0;
        int dummy = 0;
        for (int c = tid; c < k; c += nth) {
            const double d = (double)km_sqd(X, np, nb, W.cent[c], W.ncent[c]);
            if (d > var) var = d;
        }
        km_block_pick<true>(var, dummy, sv, sj);
        if (!(var > P.min_variance && iter <= P.max_iter)) break;
    }
    // weights of the last assignment; the centroids of that assignment are the result
    for (int c = tid; c < k; c += nth) W.wsum[c] = 0;
    __syncthreads();
    for (int j = tid; j < np; j += nth) atomicAdd(W.wsum + W.assign[j], __ldg(P.wt + S.p_off + j));
    __syncthreads();
    for (int c = tid; c < k; c += nth) {
        P.out_idx[S.out_off + c] = W.cent[c];
        P.out_w[S.out_off + c] = W.wsum[c];
    }
}

}  // namespace fbc
