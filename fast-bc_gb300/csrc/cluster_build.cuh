// Cluster subgraphs on the device: what SubGraph does on the host for every cluster
// (SubGraph.h:59-148, 165-189) -- the cluster id and local id of every vertex, the border set
// (a vertex with an edge to or from another cluster, listed in ascending id), and the
// induced-subgraph CSR with local ids (forwardStar keeps the intra-cluster edges, in the
// full graph's row order) -- as a few grid-stride kernels and one exclusive scan over the
// cluster vertices.  The host validates only the cluster offsets.
#pragma once
#include <cstdint>

namespace fbc {

// error bits of the cluster kernels
constexpr int kCluRange = 1;   // cluster vertex id outside [0, n)
constexpr int kCluDup = 2;     // vertex listed twice
constexpr int kCluBorder = 4;  // given border not in its cluster
constexpr int kCluOrder = 8;   // computed border list not ascending (host sorts it)

// index of the segment of `off` (ncl + 1 ascending offsets) holding position i
__device__ __forceinline__ int seg_of(const int64_t* __restrict__ off, int ncl, int64_t i) {
    int lo = 0, hi = ncl;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// cid[v] = cluster of v, lid[v] = position of v in its cluster; cid must start at -1.
__global__ void clu_ids_kernel(int64_t nv, const int64_t* __restrict__ coff, int ncl,
                               const int32_t* __restrict__ cverts, int32_t n, int32_t* cid, int32_t* lid,
                               int* err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = cverts[i];
        if (v < 0 || v >= n) {
            atomicOr(err, kCluRange);
            continue;
        }
        const int c = seg_of(coff, ncl, i);
        if (atomicCAS(cid + v, -1, c) != -1) {
            atomicOr(err, kCluDup);
            continue;
        }
        lid[v] = (int32_t)(i - coff[c]);
    }
}

// deg[i] = intra-cluster out-degree of the i-th cluster vertex
__global__ void clu_degree_kernel(int64_t nv, const int32_t* __restrict__ cverts, const int32_t* __restrict__ rp,
                                  const int2* __restrict__ adj, const int32_t* __restrict__ cid, int32_t* deg) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = cverts[i];
        const int32_t c = cid[v];
        int32_t d = 0;
        for (int32_t e = rp[v]; e < rp[v + 1]; ++e) d += cid[adj[e].x] == c;
        deg[i] = d;
    }
}

// isb[v] = 1 for both ends of every edge between different clusters (or from / to a vertex
// in no cluster), over all vertices of the graph
__global__ void clu_border_flag_kernel(int32_t n, const int32_t* __restrict__ rp, const int2* __restrict__ adj,
                                       const int32_t* __restrict__ cid, uint8_t* isb) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = cid[v];
        for (int32_t e = rp[v]; e < rp[v + 1]; ++e) {
            const int32_t x = adj[e].x;
            if (cid[x] != c) {
                isb[v] = 1;
                isb[x] = 1;
            }
        }
    }
}

// flag[i] = isb[cverts[i]]
__global__ void clu_gather_flag_kernel(int64_t nv, const int32_t* __restrict__ cverts, const uint8_t* __restrict__ isb,
                                       int32_t* flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = isb[cverts[i]];
}

// stable compaction of the flagged cluster vertices (pos = exclusive scan of the flags);
// clusters are contiguous, so cluster c's borders land in [pos[coff[c]], pos[coff[c+1]]).
// A list that is not ascending is flagged for the host to sort.
__global__ void clu_border_scatter_kernel(int64_t nv, const int64_t* __restrict__ coff, int ncl,
                                          const int32_t* __restrict__ cverts, const int32_t* __restrict__ flag,
                                          const int32_t* __restrict__ pos, int32_t* borders, int* err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        borders[pos[i]] = cverts[i];
        // the previous border of the same cluster must have a smaller id
        const int c = seg_of(coff, ncl, i);
        for (int64_t j = i - 1; j >= coff[c]; --j)
            if (flag[j]) {
                if (cverts[j] > cverts[i]) atomicOr(err, kCluOrder);
                break;
            }
    }
}

// local CSR: row i of cluster c at crp[coff[c] + c + (i - coff[c])], edges (lid[x], w) at
// cadj[S[i] ..) where S is the exclusive scan of deg (nv + 1 entries); each cluster's rows are
// relative to its first edge S[coff[c]]
__global__ void clu_fill_kernel(int64_t nv, const int64_t* __restrict__ coff, int ncl,
                                const int32_t* __restrict__ cverts, const int32_t* __restrict__ rp,
                                const int2* __restrict__ adj, const int32_t* __restrict__ cid,
                                const int32_t* __restrict__ lid, const int32_t* __restrict__ S, int32_t* crp,
                                int2* cadj) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = cverts[i];
        const int32_t c = cid[v];
        const int64_t c0 = coff[c];
        crp[c0 + c + (i - c0)] = S[i] - S[c0];
        int32_t o = S[i];
        for (int32_t e = rp[v]; e < rp[v + 1]; ++e) {
            const int2 a = adj[e];
            if (cid[a.x] == c) cadj[o++] = make_int2(lid[a.x], a.y);
        }
    }
}

// the closing row offset of every cluster (its edge count, also returned in m_out) and its
// first edge in the concatenated adjacency (e0_out); rows of empty clusters are the closing one
__global__ void clu_close_kernel(int ncl, const int64_t* __restrict__ coff, const int32_t* __restrict__ S,
                                 int32_t* crp, int64_t* m_out, int64_t* e0_out) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncl; c += gridDim.x * blockDim.x) {
        const int32_t m = S[coff[c + 1]] - S[coff[c]];
        crp[coff[c + 1] + c] = m;
        m_out[c] = m;
        e0_out[c] = S[coff[c]];
    }
}

// local ids of given borders, checked against their cluster
__global__ void clu_border_map_kernel(int64_t nb, const int64_t* __restrict__ boff, int ncl,
                                      const int32_t* __restrict__ borders, int32_t n, const int32_t* __restrict__ cid,
                                      const int32_t* __restrict__ lid, int32_t* cbord, int* err) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nb; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = borders[j];
        const int c = seg_of(boff, ncl, j);
        if (b < 0 || b >= n || cid[b] != c) {
            atomicOr(err, kCluBorder);
            cbord[j] = 0;
            continue;
        }
        cbord[j] = lid[b];
    }
}

// ---------------------------------------------------------------- exclusive scan (int32)
// out[i] = sum of in[0 .. i) for i in [0, len], three passes: per-block sums, a scan of the
// block sums by one block, and the per-block scans with their offsets.
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int32_t block_incl_scan(int32_t x, int32_t* sh) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    if (w > 0) x += sh[w - 1];
    __syncthreads();
    return x;
}

__global__ void __launch_bounds__(kScanBlock) scan_sums_kernel(const int32_t* __restrict__ in, int64_t len,
                                                               int32_t* sums) {
    __shared__ int32_t sh[32];
    const int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
    const int32_t x = i < len ? in[i] : 0;
    const int32_t s = block_incl_scan(x, sh);
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = s;
}

// exclusive scan of nb block sums in place, one block, any nb
__global__ void __launch_bounds__(kScanBlock) scan_top_kernel(int32_t* sums, int64_t nb) {
    __shared__ int32_t sh[32];
    __shared__ int32_t tot;
    int32_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += kScanBlock) {
        const int64_t i = b0 + threadIdx.x;
        const int32_t x = i < nb ? sums[i] : 0;
        const int32_t s = block_incl_scan(x, sh);
        if (i < nb) sums[i] = carry + s - x;
        if (threadIdx.x == kScanBlock - 1) tot = s;
        __syncthreads();
        carry += tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanBlock) scan_apply_kernel(const int32_t* __restrict__ in, int64_t len,
                                                                const int32_t* __restrict__ sums, int32_t* out) {
    __shared__ int32_t sh[32];
    const int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
    const int32_t x = i < len ? in[i] : 0;
    const int32_t s = block_incl_scan(x, sh);
    if (i < len) out[i] = sums[blockIdx.x] + s - x;
    if (i == len - 1) out[len] = sums[blockIdx.x] + s;
}

}  // namespace fbc
