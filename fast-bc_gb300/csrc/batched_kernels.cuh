// Batched schedule, small segments: a persistent kernel whose blocks pull (segment, chunk of
// sources) work items from a queue; a block stages the segment's CSR in shared memory once
// per chunk and each of its warps runs one source at a time with all per-source state in
// shared memory as well, so the three Brandes passes read no global memory at all; only the
// border output and the BC reduction (FP64 red.add) leave the SM.
//
// Same three passes and the same predecessor rule as brandes_kernels.cuh (near-far
// distances, Kahn sigma, reverse-level dependency pull); what makes it fit and run fast:
//   * segments of at most 65,535 vertices and weights below 65,536 (the host checks):
//     16-bit local ids and queue entries, edges packed as (dst:16 | weight:16);
//   * only native 32-bit shared-memory atomics: atomicMin relaxes, atomicExch of the
//     vertex's queue stamp de-duplicates pushes (no intra-warp matching needed), path
//     counts are two 32-bit words with an explicit carry;
//   * a warp owns a source: queue counters are registers, pushes are ballots, and each lane
//     walks the adjacency of one queued vertex (road-like graphs have degree <= ~6), four
//     edges at a time so that their shared-memory loads and atomics overlap;
//   * per-vertex state is 24 bytes: dist (4) + sigma (8) + three 4-byte planes reused per
//     pass (queues + stamps -> counters/order/levels -> delta/order/levels);
//   * the warps of a block adapt to the chunk's segment size: as many as its state fits;
//   * when sigma_v == sigma_w the ratio is exactly 1 and the division is skipped (the
//     result is bit-identical to dividing).
#pragma once
#include "brandes_kernels.cuh"

namespace fbc {

// A work item of the small-segment kernel: units [first, first + count) of one segment.
struct Chunk {
    int32_t seg;
    int32_t first;
    int32_t count;
    int32_t pad;
};

struct SmallParams {
    KParams k;
    const Chunk* chunks;
    int32_t nchunks;
    int32_t nmax;      // largest segment (vertices) of the launch
    int32_t mmax;      // largest segment (edges)
    int32_t smem;      // dynamic shared memory of a block (bytes)
    unsigned long long* next_chunk;
};

__host__ __device__ inline int64_t al16(int64_t x) { return (x + 15) & ~int64_t(15); }

// Shared memory of one block: CSR for the largest segment, then a pool of per-warp states.
struct SmallLayout {
    int64_t rp, adj, pool;
    __host__ __device__ SmallLayout(int nmax, int mmax) {
        rp = 0;
        adj = al16(4 * (int64_t)(nmax + 1));
        pool = al16(adj + 4 * (int64_t)mmax);
    }
    // state of one warp for a segment of n vertices: dist, sigma (lo, hi), planes 0, 2, 1
    __host__ __device__ static int64_t per_warp(int n) {
        return 3 * al16(4 * (int64_t)n) + 2 * al16(4 * (int64_t)n) + al16(4 * (int64_t)n + 8);
    }
};

// Warp-aggregated append to a shared queue whose counter is a warp-uniform register.
__device__ __forceinline__ void wpush16(bool want, int x, uint16_t* q, int& cnt) {
    const unsigned m = __ballot_sync(kFull, want);
    if (want) q[cnt + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = (uint16_t)x;
    cnt += __popc(m);
}

// 64-bit path counts kept as two 32-bit words so that every update is a native 32-bit
// shared-memory atomic: the low word takes the addition, a carry goes to the high word.
__device__ __forceinline__ unsigned long long sig_get(const unsigned* lo, const unsigned* hi, int v) {
    return ((unsigned long long)hi[v] << 32) | lo[v];
}
__device__ __forceinline__ bool sig_add(unsigned* lo, unsigned* hi, int x, unsigned long long a) {
    const unsigned al = (unsigned)a;
    const unsigned ah = (unsigned)(a >> 32);
    const unsigned old = atomicAdd(lo + x, al);
    const unsigned carry = (unsigned)(old + al < old);
    if (ah | carry) {
        const unsigned oh = atomicAdd(hi + x, ah + carry);
        return oh + ah + carry < oh || (ah == 0xffffffffu && carry);  // overflow of 2^64
    }
    return false;
}

template <class Prec>
__device__ void small_unit(const KParams& K, const Seg& sg, const Unit& u, const uint32_t* rp,
                           const uint32_t* adj, char* wbase) {
    const int lane = threadIdx.x & 31;
    const int n = sg.n;
    const int64_t q4 = al16(4 * (int64_t)n);
    int* dist = (int*)wbase;
    unsigned* slo = (unsigned*)(wbase + q4);
    unsigned* shi = (unsigned*)(wbase + 2 * q4);
    char* P0 = wbase + 3 * q4;   // planes 0 and 2 are adjacent: delta spans both
    char* P2 = P0 + q4;
    char* P1 = P2 + q4;          // n + 2 entries of 2 x u16
    uint16_t* const qn0 = (uint16_t*)P0;           // distance pass: near queues
    uint16_t* const qn1 = qn0 + n;
    uint16_t* const qf0 = (uint16_t*)P2;           // far piles
    uint16_t* const qf1 = qf0 + n;
    unsigned* const stamp_of = (unsigned*)P1;      // distance pass: queue stamp per vertex
    unsigned* const cnt = (unsigned*)P0;           // sigma pass: tight in-edge counters
    uint16_t* const order = (uint16_t*)P1;         // sigma + dependency passes
    uint16_t* const lvl = order + n;               // n + 1 entries (n + 4 fit)
    typename Prec::D* const dlt = (typename Prec::D*)P0;  // dependency pass
    const int src = u.src;
    const int delta = sg.delta > 0 ? sg.delta : 1;
    int bad = 0;

    for (int v = lane; v < n; v += 32) {
        dist[v] = kInf;
        slo[v] = 0u;
        shi[v] = 0u;
        stamp_of[v] = 0u;
    }
    __syncwarp();
    if (lane == 0) {
        dist[src] = 0;
        slo[src] = 1u;
        qn0[0] = (uint16_t)src;
    }
    __syncwarp();

    // ---------------------------------------------------------------- distances
    // Queue stamps: every round and every far generation gets a fresh value (0 = none).  A
    // relaxation that lowers x swaps in the stamp of the queue x now belongs to; x is pushed
    // only if it did not already carry that stamp.
    int T = delta;
    int ncur = 1, nfar = 0, qs = 0, fs = 0;
    unsigned stamp = 1u, fst = 1u;
    const int64_t capl = (int64_t)K.iter_mult * ((int64_t)n + 2);
    const unsigned cap = (unsigned)(capl < 0x7ffffff0LL ? capl : 0x7ffffff0LL);
    for (;;) {
        if (ncur > 0) {
            if (++stamp > cap) { bad = kErrIter; break; }
            const unsigned nst = stamp;
            const uint16_t* qc = qs ? qn1 : qn0;
            uint16_t* qnx = qs ? qn0 : qn1;
            uint16_t* qfx = fs ? qf1 : qf0;
            int nnext = 0;
            for (int base = 0; base < ncur; base += 32) {
                const int i = base + lane;
                int e = 0, e1 = 0, dv = 0;
                if (i < ncur) {
                    const int v = qc[i];
                    dv = dist[v];
                    e = (int)rp[v];
                    e1 = (int)rp[v + 1];
                }
                while (__any_sync(kFull, e < e1)) {
                    // up to four edges of the lane's vertex at once: their atomics overlap
                    int x[4], nd[4], od[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        x[k] = -1;
                        if (e + k < e1) {
                            const uint32_t a = adj[e + k];
                            x[k] = (int)(a & 0xffffu);
                            nd[k] = dv + (int)(a >> 16);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x[k] >= 0) od[k] = atomicMin(dist + x[k], nd[k]);
                    unsigned os[4], sk[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x[k] >= 0 && nd[k] < od[k]) {
                            sk[k] = nd[k] < T ? nst : fst;
                            os[k] = atomicExch(stamp_of + x[k], sk[k]);
                        }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        bool pn = false, pf = false;
                        if (x[k] >= 0 && nd[k] < od[k] && os[k] != sk[k]) {
                            pn = nd[k] < T;
                            pf = !pn;
                        }
                        wpush16(pn, x[k], qnx, nnext);
                        wpush16(pf, x[k], qfx, nfar);
                    }
                    e += 4;
                }
            }
            __syncwarp();
            ncur = nnext;
            qs ^= 1;
            continue;
        }
        if (nfar == 0) break;
        if (++stamp > cap) { bad = kErrIter; break; }
        // advance T to the bucket of the closest live far vertex
        const uint16_t* qfc = fs ? qf1 : qf0;
        int dmin = kInf;
        for (int i = lane; i < nfar; i += 32) {
            const int d = dist[qfc[i]];
            if (d >= T) dmin = min(dmin, d);
        }
        dmin = __reduce_min_sync(kFull, dmin);
        if (dmin == kInf) break;
        const int Told = T;
        const int64_t tn = ((int64_t)dmin / delta + 1) * (int64_t)delta;
        T = tn > (int64_t)kInf ? kInf : (int)tn;
        const unsigned nsplit = stamp;
        fst = ++stamp;                       // new far generation
        uint16_t* qnx = qs ? qn1 : qn0;
        uint16_t* qf2 = fs ? qf0 : qf1;
        int nn = 0, nf = 0;
        for (int base = 0; base < nfar; base += 32) {
            const int i = base + lane;
            bool pn = false, pf = false;
            int x = 0;
            if (i < nfar) {
                x = qfc[i];
                const int d = dist[x];
                if (d >= Told) {  // the far pile holds x once per generation
                    pn = d < T;
                    pf = !pn;
                    stamp_of[x] = pn ? nsplit : fst;
                }
            }
            wpush16(pn, x, qnx, nn);
            wpush16(pf, x, qf2, nf);
        }
        __syncwarp();
        ncur = nn;
        nfar = nf;
        fs ^= 1;
    }
    __syncwarp();

    int nlev = 0;
    if (!bad) {
        // ------------------------------------------------------------- sigma (Kahn)
        for (int v = lane; v < n; v += 32) cnt[v] = 0u;
        __syncwarp();
        for (int base = 0; base < n; base += 32) {
            const int v = base + lane;
            if (v < n) {
                const int dv = dist[v];
                if (dv != kInf) {
                    const int e1 = (int)rp[v + 1];
                    for (int e = (int)rp[v]; e < e1; e += 4) {
                        int x[4], dx[4], nd[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            x[k] = -1;
                            if (e + k < e1) {
                                const uint32_t a = adj[e + k];
                                x[k] = (int)(a & 0xffffu);
                                nd[k] = dv + (int)(a >> 16);
                            }
                        }
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (x[k] >= 0) dx[k] = dist[x[k]];
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (x[k] >= 0 && nd[k] == dx[k]) atomicAdd(cnt + x[k], 1u);
                    }
                }
            }
        }
        __syncwarp();  // order/lvl reuse the stamp plane from here on
        if (lane == 0) {
            order[0] = (uint16_t)src;
            lvl[0] = 0;
        }
        __syncwarp();
        int lo = 0, hi = 1;
        while (lo < hi) {
            if (nlev >= n) { bad = kErrIter; break; }
            int nxt = hi;
            for (int base = lo; base < hi; base += 32) {
                const int i = base + lane;
                int e = 0, e1 = 0, dv = 0;
                unsigned long long sv = 0;
                if (i < hi) {
                    const int v = order[i];
                    dv = dist[v];
                    sv = sig_get(slo, shi, v);
                    e = (int)rp[v];
                    e1 = (int)rp[v + 1];
                }
                while (__any_sync(kFull, e < e1)) {
                    int x[4], nd[4], dx[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        x[k] = -1;
                        if (e + k < e1) {
                            const uint32_t a = adj[e + k];
                            x[k] = (int)(a & 0xffffu);
                            nd[k] = dv + (int)(a >> 16);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x[k] >= 0) dx[k] = dist[x[k]];
                    bool push[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        push[k] = false;
                        if (x[k] >= 0 && nd[k] == dx[k]) {
                            if (sig_add(slo, shi, x[k], sv)) bad |= kErrSigma;
                            push[k] = atomicSub(cnt + x[k], 1u) == 1u;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) wpush16(push[k], x[k], order, nxt);
                    e += 4;
                }
            }
            __syncwarp();
            ++nlev;
            if (lane == 0) lvl[nlev] = (uint16_t)hi;
            lo = hi;
            hi = nxt;
            __syncwarp();
        }
        bad = __reduce_or_sync(kFull, bad);
        if (!bad && u.bout >= 0) {
            for (int j = lane; j < sg.nb; j += 32) {
                const int b = sg.border[j];
                const int d = dist[b];
                K.bdist[u.bout + j] = d != kInf ? nonneg_int_to_double(d) : 0.0;
                K.bsig[u.bout + j] = sig_get(slo, shi, b);
            }
        }
    }
    if (!bad) {
        // --------------------------------------------------------- dependency
        const double card = u.card;
        const bool card1 = __double_as_longlong(card) == 0x3ff0000000000000ll;  // card == 1.0, bitwise
        for (int L = nlev - 1; L >= 0; --L) {
            const int a1 = lvl[L + 1];
            for (int i = lvl[L] + lane; i < a1; i += 32) {
                const int v = order[i];
                const int dv = dist[v];
                const unsigned long long sv = sig_get(slo, shi, v);
                typename Prec::Acc acc = Prec::zero();
                const int e1 = (int)rp[v + 1];
                for (int e = (int)rp[v]; e < e1; e += 4) {
                    int x[4];
                    bool tight[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        x[k] = -1;
                        tight[k] = false;
                        if (e + k < e1) {
                            const uint32_t a = adj[e + k];
                            x[k] = (int)(a & 0xffffu);
                            tight[k] = dv + (int)(a >> 16) == dist[x[k]];
                        }
                    }
                    // accumulate in adjacency order (deterministic)
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (tight[k]) {
                            const unsigned long long sx = sig_get(slo, shi, x[k]);
                            if (sx == sv) Prec::add_same(acc, dlt[x[k]]);
                            else Prec::add(acc, sv, sx, dlt[x[k]]);
                        }
                }
                dlt[v] = Prec::store(acc);
                if (v != src) {
                    double* o = K.bc + sg.out_base + (sg.gid ? sg.gid[v] : v);
                    if (card1) Prec::red_add(o, acc);
                    else atomicAdd(o, card * Prec::value(acc));
                }
            }
            __syncwarp();
        }
    }
    if (bad && lane == 0) {
        if (bad == kErrSigma) request_retry(K, u, kErrSigma);  // recomputed with FP64 counts
        else atomicOr(K.err, bad);
    }
    __syncwarp();
}

template <class Prec>
__global__ void __launch_bounds__(512, 1) small_seg_kernel(SmallParams SP) {
    extern __shared__ __align__(16) char smem[];
    __shared__ int s_chunk, s_next;
    const SmallLayout L(SP.nmax, SP.mmax);
    uint32_t* rp = (uint32_t*)(smem + L.rp);
    uint32_t* adj = (uint32_t*)(smem + L.adj);
    const int w = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) {
            s_chunk = (int)atomicAdd(SP.next_chunk, 1ull);
            s_next = 0;
        }
        __syncthreads();
        const int ci = s_chunk;
        if (ci >= SP.nchunks) break;
        const Chunk ch = SP.chunks[ci];
        const Seg sg = SP.k.segs[ch.seg];
        const int n = sg.n;
        const int m = (int)sg.rp[n];
        for (int i = threadIdx.x; i <= n; i += blockDim.x) rp[i] = (uint32_t)sg.rp[i];
        for (int i = threadIdx.x; i < m; i += blockDim.x) {  // (dst:16 | weight:16)
            const int2 a = __ldg(sg.adj + i);
            adj[i] = (uint32_t)a.x | ((uint32_t)a.y << 16);
        }
        __syncthreads();
        const int64_t per = SmallLayout::per_warp(n);
        const int64_t fit = ((int64_t)SP.smem - L.pool) / per;
        const int active = (int)(fit < (int64_t)(blockDim.x >> 5) ? fit : (int64_t)(blockDim.x >> 5));
        if (active < 1 && threadIdx.x == 0) atomicOr(SP.k.err, kErrQueue);  // host sizing bug
        if (w < active) {
            char* wbase = smem + L.pool + (int64_t)w * per;
            for (;;) {
                int k = 0;
                if ((threadIdx.x & 31) == 0) k = atomicAdd(&s_next, 1);
                k = __shfl_sync(kFull, k, 0);
                if (k >= ch.count) break;
                const Unit u = SP.k.units[ch.first + k];
                small_unit<Prec>(SP.k, sg, u, rp, adj, wbase);
            }
        }
        __syncthreads();
    }
}

}  // namespace fbc
