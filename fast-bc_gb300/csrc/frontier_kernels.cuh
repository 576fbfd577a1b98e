// Batched schedule, large segments (whole graphs: pivots, exact mode, big graphs of a
// batch): one source per thread block, per-source state in a global-memory slot, blocks
// pulling units from a shared counter.  Same passes and predecessor rule as
// brandes_kernels.cuh; what shortens each step's chain of dependent memory accesses:
//   * one 64-bit word per vertex, (dist << 32 | stamp): a single global atomicMin both relaxes
//     the edge and reports whether the vertex already sits in the queue the relaxation
//     pushes it to (the queue's stamp), so there is no second atomic on a flag array;
//   * queue entries carry the vertex's row (loaded alongside the atomic that pushed it) and
//     Kahn-level entries carry distance, row and final path count, so a step starts with
//     its adjacency loads; path count and the Kahn counter share one 64-bit word
//     (sigma << 16 | counter), so one atomic both adds sigma_v and retires the edge, and the
//     thread that retires the last tight in-edge learns the final count;
//   * each thread takes one queued vertex and issues up to four of its edges at once, so
//     their loads and atomics are in flight together (road-like graphs: degree <= ~6);
//   * sigma_v == sigma_w takes the exact ratio-1 path in the dependency pass.
#pragma once
#include "batched_kernels.cuh"

namespace fbc {

// A queued vertex with what the next step needs, so the step starts with its adjacency
// loads instead of re-reading the row offsets.
struct QEnt {
    int v, e0, deg, pad;
};
// A vertex of a Kahn level: distance, row start, final path count, and `dm`: the mask of its
// tight out-edges found by the counting sweep (bit k: edge e0 + k), so that the Kahn and
// dependency passes touch only those; all ones for rows longer than 32 edges (then every edge
// of the row is re-tested).
struct LEnt {
    int v, d, e0;
    unsigned dm;
    unsigned long long sig;
};

// Near queues and far piles hold a vertex at most once each, but the frontiers of road-like
// graphs are far smaller than n: they get qcap entries, and a unit that would overflow them is
// handed to the plain kernel (whose queues hold n).
__host__ __device__ inline int64_t fqcap(int64_t cap) {
    const int64_t q = cap / 4 + 1 > 65536 ? cap / 4 + 1 : 65536;
    return q < cap + 1 ? q : cap + 1;
}

template <class Prec>
struct FState {
    unsigned long long* word;     // (dist << 32 | queue stamp)
    unsigned long long* sc;       // (sigma << 16 | tight in-edges still unprocessed)
    typename Prec::D* dlt;
    QEnt* q[4];                   // near0, near1, far0, far1 (fqcap(cap) entries)
    LEnt* order;                  // cap + 1 entries
    int* lvl;                     // cap + 1 entries
    unsigned* tmask;              // tight out-edge mask per vertex (cap entries)
};

template <class Prec>
__host__ __device__ inline int64_t fstate_bytes(int64_t cap) {
    auto al = [](int64_t x) { return (x + 255) & ~int64_t(255); };
    return al(cap * 8) + al(cap * 8) + al(cap * (int64_t)sizeof(typename Prec::D)) +
           4 * al(fqcap(cap) * (int64_t)sizeof(QEnt)) + al((cap + 1) * (int64_t)sizeof(LEnt)) +
           al((cap + 1) * 4) + al(cap * 4);
}

template <class Prec>
__device__ inline FState<Prec> fstate_carve(char* p, int64_t cap) {
    auto al = [](int64_t x) { return (x + 255) & ~int64_t(255); };
    FState<Prec> s;
    s.word = (unsigned long long*)p; p += al(cap * 8);
    s.sc = (unsigned long long*)p; p += al(cap * 8);
    s.dlt = (typename Prec::D*)p; p += al(cap * (int64_t)sizeof(typename Prec::D));
    for (int i = 0; i < 4; ++i) { s.q[i] = (QEnt*)p; p += al(fqcap(cap) * (int64_t)sizeof(QEnt)); }
    s.order = (LEnt*)p; p += al((cap + 1) * (int64_t)sizeof(LEnt));
    s.lvl = (int*)p; p += al((cap + 1) * 4);
    s.tmask = (unsigned*)p;
    return s;
}

struct FCtl {
    int ncnt[2];
    int fcnt[2];
    int ocnt;
    int dmin;
    int unit;
    int bad;
    int ovf;   // a queue push did not fit
};

// Path counts share a word with the counter, so they are limited to 2^48 - 1 here; a unit
// that exceeds it stops before its dependency pass and is recomputed by the plain kernel.
constexpr unsigned long long kSigMax = (1ull << 48) - 1ull;

__device__ __forceinline__ unsigned long long ldcg64(const unsigned long long* p) { return __ldcg(p); }
__device__ __forceinline__ int dist_of(unsigned long long w) { return (int)(w >> 32); }

// Block-wide push (warp-aggregated slot reservation on a shared-memory counter); a push past
// the capacity is dropped and raises *ovf (the unit is then recomputed elsewhere).
template <class E>
__device__ __forceinline__ void bpush(bool want, const E& x, E* q, int* c, int cap, int* ovf) {
    const unsigned m = __ballot_sync(kFull, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(c, __popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (want) {
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) q[pos] = x;
        else *ovf = 1;
    }
}

template <class Prec>
__device__ void frontier_unit(const KParams& P, int64_t ui, const Unit& u, const FState<Prec>& S,
                              FCtl& C, int cap) {
    const Seg sg = P.segs[u.seg];
    const int n = sg.n;
    const int* __restrict__ rp = sg.rp;
    const int2* __restrict__ adj = sg.adj;
    const int src = u.src;
    const int delta = sg.delta > 0 ? sg.delta : 1;
    const int tid = threadIdx.x, nth = blockDim.x;
    const int qc_cap = (int)fqcap(cap);
    int bad = 0;

    // ---------------------------------------------------------------- distances
    int T = delta;
    int qs = 0, fs = 0;
    unsigned stamp = 1u, fst = 1u;
    if (tid == 0) {
        S.word[src] = 0ull;  // dist 0, stamp 0
        const int e0 = __ldg(rp + src);
        S.q[0][0] = QEnt{src, e0, __ldg(rp + src + 1) - e0, 0};
        C.ncnt[0] = 1;
        C.ncnt[1] = 0;
        C.fcnt[0] = 0;
        C.fcnt[1] = 0;
        C.ovf = 0;
    }
    __syncthreads();
    const int64_t capr = (int64_t)P.iter_mult * ((int64_t)n + 2);
    int64_t rounds = 0;
    for (;;) {
        const int ncur = C.ncnt[qs];
        if (ncur > 0) {
            if (++rounds > capr) { bad = kErrIter; break; }
            const unsigned nst = ++stamp;
            const QEnt* qc = qs ? S.q[1] : S.q[0];
            QEnt* qnx = qs ? S.q[0] : S.q[1];
            QEnt* qfx = fs ? S.q[3] : S.q[2];
            // warp-uniform trip count so that every lane reaches the ballots
            for (int base = tid & ~31; base < ncur; base += nth) {
                const int i = base + (tid & 31);
                int e = 0, e1 = 0, dv = 0;
                if (i < ncur) {
                    const QEnt q = qc[i];
                    e = q.e0;
                    e1 = q.e0 + q.deg;
                    dv = dist_of(ldcg64(S.word + q.v));  // may have dropped since the push
                }
                while (__any_sync(kFull, e < e1)) {
                    int x[4], nd[4], r0[4], r1[4];
                    unsigned long long old[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        x[k] = -1;
                        if (e + k < e1) {
                            const int2 a = __ldg(adj + e + k);
                            x[k] = a.x;
                            nd[k] = dv + a.y;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x[k] >= 0) {
                            old[k] = atomicMin(S.word + x[k],
                                               ((unsigned long long)(unsigned)nd[k] << 32) | (nd[k] < T ? nst : fst));
                            r0[k] = __ldg(rp + x[k]);      // in flight with the atomic
                            r1[k] = __ldg(rp + x[k] + 1);
                        }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        bool pn = false, pf = false;
                        if (x[k] >= 0) {
                            const bool near = nd[k] < T;
                            if (nd[k] < dist_of(old[k]) && (unsigned)old[k] != (near ? nst : fst)) {
                                pn = near;
                                pf = !near;
                            }
                        }
                        const QEnt qe{x[k], r0[k], r1[k] - r0[k], 0};
                        bpush(pn, qe, qnx, &C.ncnt[qs ^ 1], qc_cap, &C.ovf);
                        bpush(pf, qe, qfx, &C.fcnt[fs], qc_cap, &C.ovf);
                    }
                    e += 4;
                }
            }
            __syncthreads();
            if (C.ovf) { bad = kErrRetry; break; }
            if (tid == 0) C.ncnt[qs] = 0;
            qs ^= 1;
            __syncthreads();
            continue;
        }
        const int nfar = C.fcnt[fs];
        if (nfar == 0) break;
        if (++rounds > capr) { bad = kErrIter; break; }
        if (tid == 0) C.dmin = kInf;
        __syncthreads();
        const QEnt* qfc = fs ? S.q[3] : S.q[2];
        for (int i = tid; i < nfar; i += nth) {
            const int d = dist_of(ldcg64(S.word + qfc[i].v));
            if (d >= T) atomicMin(&C.dmin, d);
        }
        __syncthreads();
        const int dmin = C.dmin;
        if (dmin == kInf) break;
        const int Told = T;
        const int64_t tn = ((int64_t)dmin / delta + 1) * (int64_t)delta;
        T = tn > (int64_t)kInf ? kInf : (int)tn;
        const unsigned nsplit = ++stamp;
        fst = ++stamp;
        QEnt* qnx = qs ? S.q[1] : S.q[0];
        QEnt* qf2 = fs ? S.q[2] : S.q[3];
        for (int base = tid & ~31; base < nfar; base += nth) {
            const int i = base + (tid & 31);
            bool pn = false, pf = false;
            QEnt qe{0, 0, 0, 0};
            if (i < nfar) {
                qe = qfc[i];
                const int d = dist_of(ldcg64(S.word + qe.v));
                if (d >= Told) {  // the far pile holds a vertex once per generation
                    pn = d < T;
                    pf = !pn;
                    S.word[qe.v] = ((unsigned long long)(unsigned)d << 32) | (pn ? nsplit : fst);
                }
            }
            bpush(pn, qe, qnx, &C.ncnt[qs], qc_cap, &C.ovf);
            bpush(pf, qe, qf2, &C.fcnt[fs ^ 1], qc_cap, &C.ovf);
        }
        __syncthreads();
        if (C.ovf) { bad = kErrRetry; break; }
        if (tid == 0) C.fcnt[fs] = 0;
        fs ^= 1;
        __syncthreads();
    }
    __syncthreads();

    int nlev = 0;
    if (!bad) {
        // ------------------------------------------------------------- sigma (Kahn)
        // tight in-edge counts and each vertex's tight out-edge mask: a sweep over all
        // vertices, four per thread in flight
        for (int v0 = tid; v0 < n; v0 += 4 * nth) {
            int dv[4], e[4], e1[4], eb[4];
            unsigned mk[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int v = v0 + k * nth;
                dv[k] = kInf;
                e[k] = e1[k] = eb[k] = 0;
                mk[k] = 0u;
                if (v < n) {
                    dv[k] = dist_of(ldcg64(S.word + v));
                    if (dv[k] != kInf) {
                        e[k] = eb[k] = __ldg(rp + v);
                        e1[k] = __ldg(rp + v + 1);
                    }
                }
            }
            for (;;) {
                int x[4], nd[4];
                bool any = false;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    x[k] = -1;
                    if (e[k] < e1[k]) {
                        const int2 a = __ldg(adj + e[k]++);
                        x[k] = a.x;
                        nd[k] = dv[k] + a.y;
                        any = true;
                    }
                }
                if (!any) break;
                int dx[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) dx[k] = x[k] >= 0 ? dist_of(ldcg64(S.word + x[k])) : -1;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (x[k] >= 0 && nd[k] == dx[k]) {
                        atomicAdd(S.sc + x[k], 1ull);
                        const int bit = e[k] - 1 - eb[k];
                        if (bit < 32) mk[k] |= 1u << bit;
                    }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int v = v0 + k * nth;
                if (v < n && dv[k] != kInf) S.tmask[v] = e1[k] - eb[k] > 32 ? 0xffffffffu : mk[k];
            }
        }
        __syncthreads();
        if (tid == 0) {
            const int e0 = __ldg(rp + src);
            S.order[0] = LEnt{src, 0, e0, __ldcg(S.tmask + src), 1ull};
            S.lvl[0] = 0;
            C.ocnt = 1;
        }
        __syncthreads();
        int lo = 0, hi = 1;
        while (lo < hi) {
            if (nlev >= n) { bad = kErrIter; break; }
            for (int base = lo + (tid & ~31); base < hi; base += nth) {
                const int i = base + (tid & 31);
                int dv = 0, e0 = 0, e = 0, e1 = 0;
                unsigned mk = 0u;
                unsigned long long sv = 0;
                if (i < hi) {
                    const LEnt o = S.order[i];
                    dv = o.d;
                    sv = o.sig;
                    e0 = o.e0;
                    mk = o.dm;
                    if (mk == 0xffffffffu) {  // long row: walk it and re-test every edge
                        e = e0;
                        e1 = __ldg(rp + o.v + 1);
                        mk = 0u;
                    }
                }
                while (__any_sync(kFull, mk != 0u || e < e1)) {
                    int x[4], nd[4];
                    bool tight[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        x[k] = -1;
                        tight[k] = false;
                        int ei = -1;
                        if (mk) {  // tight by the counting sweep
                            ei = e0 + __ffs(mk) - 1;
                            mk &= mk - 1u;
                            tight[k] = true;
                        } else if (e < e1) {
                            ei = e++;
                        }
                        if (ei >= 0) {
                            const int2 a = __ldg(adj + ei);
                            x[k] = a.x;
                            nd[k] = dv + a.y;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x[k] >= 0 && !tight[k]) tight[k] = nd[k] == dist_of(ldcg64(S.word + x[k]));
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        bool push = false;
                        LEnt le{x[k], nd[k], 0, 0u, 0ull};
                        if (tight[k]) {
                            // one atomic adds sigma_v and retires the edge; the thread that
                            // retires the last tight in-edge knows x's final count
                            const unsigned long long old = atomicAdd(S.sc + x[k], (sv << 16) - 1ull);
                            const unsigned long long sx = (old >> 16) + sv;
                            if (sx > kSigMax || sv > kSigMax) bad |= kErrRetry;
                            push = (old & 0xffffull) == 1ull;
                            le.sig = sx;
                            le.e0 = __ldg(rp + x[k]);        // in flight with the atomic
                            le.dm = __ldcg(S.tmask + x[k]);
                        }
                        bpush(push, le, S.order, &C.ocnt, cap + 1, &C.ovf);
                    }
                }
            }
            __syncthreads();
            ++nlev;
            if (tid == 0) S.lvl[nlev] = hi;
            lo = hi;
            hi = C.ocnt;
            __syncthreads();
        }
        // block-wide OR of the status bits (__syncthreads_or would only say "some bit")
        if (tid == 0) C.bad = 0;
        __syncthreads();
        if (bad) atomicOr(&C.bad, bad);
        __syncthreads();
        bad = C.bad;
        if (!bad && u.bout >= 0) {
            for (int j = tid; j < sg.nb; j += nth) {
                const int b = sg.border[j];
                const int d = dist_of(ldcg64(S.word + b));
                P.bdist[u.bout + j] = d != kInf ? (double)d : 0.0;
                P.bsig[u.bout + j] = d != kInf ? (d == 0 ? 1ull : __ldcg(S.sc + b) >> 16) : 0ull;
            }
        }
    }
    if (!bad) {
        // --------------------------------------------------------- dependency
        const double card = u.card;
        for (int L = nlev - 1; L >= 0; --L) {
            const int a0 = __ldcg(S.lvl + L), a1 = __ldcg(S.lvl + L + 1);
            for (int i = a0 + tid; i < a1; i += nth) {
                const LEnt o = S.order[i];
                const int v = o.v, dv = o.d;
                const unsigned long long sv = o.sig;
                typename Prec::Acc acc = Prec::zero();
                if (o.dm != 0xffffffffu) {
                    // tight out-edges only, four at a time (the mask was set by the Kahn pass)
                    unsigned mk = o.dm;
                    while (mk) {
                        int x[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            x[k] = -1;
                            if (mk) {
                                const int b = __ffs(mk) - 1;
                                mk &= mk - 1u;
                                x[k] = __ldg(adj + o.e0 + b).x;
                            }
                        }
                        unsigned long long sx[4];
                        typename Prec::D dx[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (x[k] >= 0) {
                                sx[k] = __ldcg(S.sc + x[k]) >> 16;
                                dx[k] = S.dlt[x[k]];
                            }
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (x[k] >= 0) {
                                if (sx[k] == sv) Prec::add_same(acc, dx[k]);
                                else Prec::add(acc, sv, sx[k], dx[k]);
                            }
                    }
                } else {
                    const int e1 = __ldg(rp + v + 1);
                    for (int e = o.e0; e < e1; ++e) {
                        const int2 a = __ldg(adj + e);
                        if (dv + a.y == dist_of(ldcg64(S.word + a.x))) {
                            const unsigned long long sx = __ldcg(S.sc + a.x) >> 16;
                            if (sx == sv) Prec::add_same(acc, S.dlt[a.x]);
                            else Prec::add(acc, sv, sx, S.dlt[a.x]);
                        }
                    }
                }
                S.dlt[v] = Prec::store(acc);
                if (v != src) {
                    const int64_t ov = sg.gid ? (int64_t)sg.gid[v] : sg.out_base + v;
                    atomicAdd(P.bc + ov, card == 1.0 ? Prec::value(acc) : card * Prec::value(acc));
                }
            }
            __syncthreads();
        }
    }
    if (tid == 0 && bad) {
        if (bad == kErrRetry) request_retry(P, u, kErrRetry);  // recomputed with 64-bit counts
        else atomicOr(P.err, bad);
    }
    if (P.dbg_dist) {
        for (int v = tid; v < n; v += nth) {
            const int d = dist_of(ldcg64(S.word + v));
            P.dbg_dist[v] = d != kInf ? d : -1;
            P.dbg_sig[v] = d != kInf ? (v == src ? 1ull : __ldcg(S.sc + v) >> 16) : 0ull;
            P.dbg_dlt[v] = d != kInf ? Prec::value(Prec::load(S.dlt[v])) : 0.0;
        }
    }
    __syncthreads();
    // restore: word = (inf, 0), sigma/counter = 0
    for (int v = tid; v < n; v += nth) {
        S.word[v] = (unsigned long long)(unsigned)kInf << 32;
        S.sc[v] = 0ull;
    }
    __syncthreads();
}

// kWide: 512-thread blocks for segments whose frontiers span many hundreds of vertices
// (millions of vertices); otherwise 128-thread blocks, five per SM.
template <class Prec, bool kWide>
__global__ void __launch_bounds__(kWide ? 512 : 128, kWide ? 1 : 5) frontier_kernel(KParams P) {
    __shared__ FCtl C;
    char* slot = P.ws + (int64_t)blockIdx.x * P.ws_stride;
    unsigned* hdr = (unsigned*)slot;
    FState<Prec> S = fstate_carve<Prec>(slot + 256, P.ws_n);
    if (hdr[0] == 0u) {  // fresh slot: establish the between-units invariant
        for (int i = threadIdx.x; i < P.ws_n; i += blockDim.x) {
            S.word[i] = (unsigned long long)(unsigned)kInf << 32;
            S.sc[i] = 0ull;
        }
        __syncthreads();
        if (threadIdx.x == 0) hdr[0] = 1u;
    }
    for (;;) {
        if (threadIdx.x == 0) C.unit = (int)atomicAdd(P.next_unit, 1ull);
        __syncthreads();
        const int64_t ui = C.unit;
        __syncthreads();
        if (ui >= P.nunits) break;
        frontier_unit<Prec>(P, ui, P.units[ui], S, C, P.ws_n);
    }
}

}  // namespace fbc
