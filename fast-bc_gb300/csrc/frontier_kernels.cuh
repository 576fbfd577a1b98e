// Batched schedule, large segments (whole graphs: pivots, exact mode, big graphs of a
// batch): one source (or a group of K sources) per thread block, per-source state in a
// global-memory slot, blocks pulling units from a shared counter.  Same passes and predecessor
// rule as brandes_kernels.cuh.  On million-vertex graphs the kernel is bound by random DRAM
// sector accesses (every vertex's state and row is touched cold once per pass), so the
// design counts sectors and dependent steps:
//   * one 64-bit word per vertex, (dist << 32 | stamp): a single global atomicMin both relaxes
//     the edge and reports whether the vertex already sits in the queue the relaxation
//     pushes it to (the queue's stamp), so there is no second atomic on a flag array;
//   * queue entries carry the vertex's row (loaded from the small, L2-resident row offsets
//     alongside the atomic that pushed it) and Kahn-level entries carry distance, row, final
//     path count and tight-edge mask, so a step starts with its adjacency loads;
//   * path count and Kahn counter share one 64-bit word (sigma << B | counter; B = 8 bits when
//     no vertex has 255 or more in-edges, else 16), so one atomic
//     both adds sigma_v and retires the edge, and the thread that retires the last tight
//     in-edge learns the final count; the word sits in a 16-byte record with the dependency
//     (which holds the tight-edge mask until the dependency pass), so a Kahn push and a
//     dependency pull each touch one sector of the pushed/pulled vertex;
//   * each thread takes one queued vertex and issues up to four of its edges at once (and
//     one or two level entries at once in the Kahn and dependency passes), so their loads
//     and atomics are in flight together;
//   * sigma_v == sigma_w takes the exact ratio-1 path in the dependency pass.
#pragma once
#include "batched_kernels.cuh"

namespace fbc {

// A queued entry with its row start, so the step issues its adjacency loads at once (the
// row end comes from the small, L2-resident row offsets, loaded alongside).
struct QEnt {
    int v, e0;
};
// A Kahn-level entry: row start and (final path count << B | tight-edge mask), B the launch's
// field width (8 or 16 bits).  The mask is the vertex's tight out-edges found by the counting
// sweep (bit k: edge e0 + k), so that the Kahn and dependency passes touch only those; all B
// bits set (the long-row mark) for rows of B or more edges (then every edge of the row is
// re-tested against the distances).  Path counts are below 2^(64 - B) here.  (Entries of 8 bytes,
// the count and mask read from the vertex's record instead, measured 0.5% faster on the 4M-vertex
// grid and 7% slower on graphs whose state stays in L2: one more dependent load per entry.)
struct LEnt {
    int v, e0;
    unsigned long long sigdm;
};
// the packed fields of one launch: B = cb bits of counter / mask next to the path count
struct Packing {
    int cb;
    unsigned long long low;      // (1 << cb) - 1: counter mask, long-row mark
    unsigned long long sigmax;   // 2^(64 - cb) - 1
    __device__ explicit Packing(int bits)
        : cb(bits), low((1ull << bits) - 1ull), sigmax((1ull << (64 - bits)) - 1ull) {}
    __device__ unsigned long long sig_dm(unsigned long long sig, unsigned mask) const {
        return (sig << cb) | (mask == 0xffffffffu ? low : ((unsigned long long)mask & low));
    }
};

// Near queues and far piles hold a vertex at most once each, but the frontiers of road-like
// graphs are far smaller than n: they get qcap entries, and a unit that would overflow them is
// handed to the plain kernel (whose queues hold n).
__host__ __device__ inline int64_t fqcap(int64_t cap) {
    const int64_t q = cap / 8 + 1 > 65536 ? cap / 8 + 1 : 65536;
    return q < cap + 1 ? q : cap + 1;
}

// Path count and dependency of a vertex side by side, so the dependency pass reads both with
// one 16-byte load.  Until the dependency pass writes it, the dependency slot holds the
// vertex's tight out-edge mask (bit k: edge e0 + k; all ones for rows of B or more edges),
// so the Kahn pass finds a released vertex's mask in the sector its count atomic just touched.
template <class Prec>
struct __align__(16) FRec {
    unsigned long long sc;        // (sigma << B | tight in-edges still unprocessed)
    union {
        typename Prec::D dlt;
        unsigned mask;
    };
};

template <class Prec>
struct FState {
    unsigned long long* word;     // (dist << 32 | queue stamp)
    FRec<Prec>* rec;
    QEnt* q[4];                   // near0, near1, far0, far1 (fqcap(cap) entries)
    LEnt* order;                  // cap + 1 entries
    int* lvl;                     // cap + 1 entries
};

template <class Prec>
__host__ __device__ inline int64_t fstate_bytes(int64_t cap) {
    auto al = [](int64_t x) { return (x + 255) & ~int64_t(255); };
    return al(cap * 8) + al(cap * (int64_t)sizeof(FRec<Prec>)) + 4 * al(fqcap(cap) * (int64_t)sizeof(QEnt)) + al((cap + 1) * (int64_t)sizeof(LEnt)) +
           al((cap + 1) * 4);
}

template <class Prec>
__device__ inline FState<Prec> fstate_carve(char* p, int64_t cap) {
    auto al = [](int64_t x) { return (x + 255) & ~int64_t(255); };
    FState<Prec> s;
    s.word = (unsigned long long*)p; p += al(cap * 8);
    s.rec = (FRec<Prec>*)p; p += al(cap * (int64_t)sizeof(FRec<Prec>));
    for (int i = 0; i < 4; ++i) { s.q[i] = (QEnt*)p; p += al(fqcap(cap) * (int64_t)sizeof(QEnt)); }
    s.order = (LEnt*)p; p += al((cap + 1) * (int64_t)sizeof(LEnt));
    s.lvl = (int*)p;
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

// Path counts share a word with the counter, so they are limited to 2^(64 - B) - 1 here; a
// unit that exceeds it stops before its dependency pass and is recomputed by the plain kernel.

__device__ __forceinline__ unsigned long long ldcg64(const unsigned long long* p) { return __ldcg(p); }

// The 8 bytes of a dependency value read as part of a 16-byte record load.
template <class D>
__device__ __forceinline__ D bits_to(unsigned long long b);
template <>
__device__ __forceinline__ double bits_to<double>(unsigned long long b) {
    return __longlong_as_double((long long)b);
}
template <>
__device__ __forceinline__ float2 bits_to<float2>(unsigned long long b) {
    return make_float2(__int_as_float((int)(unsigned)b), __int_as_float((int)(unsigned)(b >> 32)));
}

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

// One group of K sources of the same segment per block: the sources share the distance
// rounds, the Kahn levels and the dependency levels (one barrier per round or level for all
// of them), and their per-vertex state is interleaved, entry v*K + k for source k, so the
// words of nearby sources' wavefronts share sectors and the adjacency rows they read are the
// same.  Queue and level entries name an entry vk = v*K + k.  K = 1 is one source per block.
// kV: level entries per lane in the Kahn and dependency passes (2: their loads and atomics are
// in flight together; 4 measured slower, spilling at the register caps); kE:
// queued entries per lane in the distance pass (1: two measured slower on the wide blocks,
// which then spill at their 128-register cap).
// One adjacency entry (destination, weight): from the int2 array, or with kA4 from the packed
// 4-byte form (destination in the low 24 bits, weight in the high 8), which halves the bytes
// of every row access.
template <bool kA4>
__device__ __forceinline__ int2 adj_at(const Seg& sg, int e) {
    if constexpr (kA4) {
        const uint32_t u = __ldg(sg.adj4 + e);
        return make_int2((int)(u & 0xffffffu), (int)(u >> 24));
    } else {
        return __ldg(sg.adj + e);
    }
}

template <class Prec, int kV, int K, int kE, bool kA4>
__device__ void frontier_group(const KParams& P, const Unit* us, const FState<Prec>& S, FCtl& C,
                               int64_t cap) {
    static_assert(K == 1 || K == 2 || K == 4 || K == 8, "K is a power of two up to 8");
    constexpr int kSh = K == 1 ? 0 : K == 2 ? 1 : K == 4 ? 2 : 3;
    const Seg sg = P.segs[us[0].seg];
    const int n = sg.n;
    const int nK = n * K;
    const int* __restrict__ rp = sg.rp;
    const int delta = sg.delta > 0 ? sg.delta : 1;
    const int tid = threadIdx.x, nth = blockDim.x;
    const int qc_cap = (int)fqcap(cap);
    const Packing pk(P.cnt_bits);
    const int mask_edges = pk.cb - 1;  // rows of more edges carry the long-row mark
    int bad = 0;

    // ---------------------------------------------------------------- distances
    int T = delta;
    int qs = 0, fs = 0;
    unsigned stamp = 1u, fst = 1u;
    if (tid == 0) {
        int c = 0;
        for (int k = 0; k < K; ++k) {
            const int src = us[k].src;
            if (src < 0) continue;
            S.word[src * K + k] = 0ull;  // dist 0, stamp 0
            S.q[0][c++] = QEnt{src * K + k, __ldg(rp + src)};
        }
        C.ncnt[0] = c;
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
            // warp-uniform trip count so that every lane reaches the ballots; each lane takes
            // kE queued entries (entries j*32 + lane of the warp's span) and issues up to four
            // edges of each at once
            for (int base = (tid & ~31) * kE; base < ncur; base += nth * kE) {
                int e[kE], e1[kE], dv[kE], kk[kE];
#pragma unroll
                for (int j = 0; j < kE; ++j) {
                    const int i = base + j * 32 + (tid & 31);
                    e[j] = e1[j] = dv[j] = kk[j] = 0;
                    if (i < ncur) {
                        const QEnt q = qc[i];
                        e[j] = q.e0;
                        e1[j] = __ldg(rp + (q.v >> kSh) + 1);
                        kk[j] = q.v & (K - 1);
                        dv[j] = dist_of(ldcg64(S.word + q.v));  // may have dropped since the push
                    }
                }
                for (;;) {
                    bool more = false;
#pragma unroll
                    for (int j = 0; j < kE; ++j) more |= e[j] < e1[j];
                    if (!__any_sync(kFull, more)) break;
                    int x[kE * 4], nd[kE * 4], r0[kE * 4];
                    unsigned long long old[kE * 4];
#pragma unroll
                    for (int t = 0; t < kE * 4; ++t) {
                        const int j = t / 4, q = t % 4;
                        x[t] = -1;
                        if (e[j] + q < e1[j]) {
                            const int2 a = adj_at<kA4>(sg, e[j] + q);
                            x[t] = (a.x << kSh) + kk[j];
                            nd[t] = dv[j] + a.y;
                            r0[t] = __ldg(rp + a.x);  // x's row, in flight with the atomic
                        }
                    }
                    // on the large relabelled graphs (packed adjacency) a relaxation that cannot
                    // lower the current distance is dropped after a plain load (distances only
                    // fall, so a stale word can only overstate it): most edges of a settled
                    // wavefront fail, and a scattered load costs the memory system about half of
                    // what a scattered atomic does (1% there; on graphs whose state stays in L2 the
                    // extra dependent load costs more than it saves)
#pragma unroll
                    for (int t = 0; t < kE * 4; ++t)
                        old[t] = kA4 && x[t] >= 0 ? ldcg64(S.word + x[t]) : (unsigned long long)(unsigned)kInf << 32;
#pragma unroll
                    for (int t = 0; t < kE * 4; ++t)
                        if (x[t] >= 0 && nd[t] < dist_of(old[t]))
                            old[t] = atomicMin(S.word + x[t],
                                               ((unsigned long long)(unsigned)nd[t] << 32) | (nd[t] < T ? nst : fst));
#pragma unroll
                    for (int t = 0; t < kE * 4; ++t) {
                        bool pn = false, pf = false;
                        if (x[t] >= 0) {
                            const bool near = nd[t] < T;
                            if (nd[t] < dist_of(old[t]) && (unsigned)old[t] != (near ? nst : fst)) {
                                pn = near;
                                pf = !near;
                            }
                        }
                        const QEnt qe{x[t], r0[t]};
                        bpush(pn, qe, qnx, &C.ncnt[qs ^ 1], qc_cap, &C.ovf);
                        bpush(pf, qe, qfx, &C.fcnt[fs], qc_cap, &C.ovf);
                    }
#pragma unroll
                    for (int j = 0; j < kE; ++j) e[j] += 4;
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
            QEnt qe{0, 0};
            if (i < nfar) {
                qe = qfc[i];
                const int d = dist_of(ldcg64(S.word + qe.v));
                if (d >= Told) {  // the far pile holds an entry once per generation
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
        // tight in-edge counts and each entry's tight out-edge mask: a sweep over all
        // entries, four per thread in flight; the K entries of a vertex sit on adjacent lanes,
        // so their row and neighbour-word loads coalesce.  With reverse weights (pull) a vertex
        // counts its own tight in-edges from the same neighbour words and stores its whole
        // record at once; else each tight edge adds to its head's counter atomically.
        const bool pull = sg.revw != nullptr;
        for (int v0 = tid; v0 < nK; v0 += 4 * nth) {
            int dv[4], e[4], e1[4], eb[4];
            unsigned mk[4], cn[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int vk = v0 + j * nth;
                dv[j] = kInf;
                e[j] = e1[j] = eb[j] = 0;
                mk[j] = cn[j] = 0u;
                if (vk < nK) {
                    dv[j] = dist_of(ldcg64(S.word + vk));
                    if (dv[j] != kInf) {
                        e[j] = eb[j] = __ldg(rp + (vk >> kSh));
                        e1[j] = __ldg(rp + (vk >> kSh) + 1);
                    }
                }
            }
            for (;;) {
                int x[4], nd[4], rw[4];
                bool any = false;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    x[j] = -1;
                    if (e[j] < e1[j]) {
                        const int ee = e[j]++;
                        const int2 a = adj_at<kA4>(sg, ee);
                        x[j] = (a.x << kSh) + ((v0 + j * nth) & (K - 1));
                        nd[j] = dv[j] + a.y;
                        rw[j] = pull ? (int)__ldg(sg.revw + ee) : 0;
                        any = true;
                    }
                }
                if (!any) break;
                int dx[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) dx[j] = x[j] >= 0 ? dist_of(ldcg64(S.word + x[j])) : -1;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (x[j] >= 0) {
                        if (nd[j] == dx[j]) {
                            if (!pull) atomicAdd(&S.rec[x[j]].sc, 1ull);
                            const int bit = e[j] - 1 - eb[j];
                            if (bit < 32) mk[j] |= 1u << bit;
                        }
                        if (pull && dx[j] != kInf && dx[j] + rw[j] == dv[j]) ++cn[j];  // x -> v is tight
                    }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int vk = v0 + j * nth;
                if (vk < nK && dv[j] != kInf) {
                    const unsigned mv = e1[j] - eb[j] > mask_edges ? 0xffffffffu : mk[j];
                    if (pull)  // count (sigma 0) and mask: the whole record, one 16-byte store
                        *reinterpret_cast<ulonglong2*>(S.rec + vk) = make_ulonglong2(cn[j], mv);
                    else
                        S.rec[vk].mask = mv;
                }
            }
        }
        __syncthreads();
        if (tid == 0) {
            int c = 0;
            for (int k = 0; k < K; ++k) {
                const int src = us[k].src;
                if (src < 0) continue;
                S.order[c++] = LEnt{src * K + k, __ldg(rp + src), pk.sig_dm(1ull, __ldcg(&S.rec[src * K + k].mask))};
            }
            S.lvl[0] = 0;
            C.ocnt = c;
        }
        __syncthreads();
        int lo = 0, hi = C.ocnt;
        while (lo < hi) {
            if (nlev >= n) { bad = kErrIter; break; }
            // each lane takes kV entries of the level (coalesced: entries j*32 + lane of the
            // warp's span) and issues one tight edge of each per step, so kV atomics are in
            // flight together (the DAG of a road-like graph has about one tight out-edge per
            // vertex)
            for (int base = lo + (tid & ~31) * kV; base < hi; base += nth * kV) {
                int dv[kV], e0[kV], e[kV], e1[kV], kk[kV];
                unsigned mk[kV];
                unsigned long long sv[kV];
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    const int i = base + j * 32 + (tid & 31);
                    dv[j] = e0[j] = e[j] = e1[j] = kk[j] = 0;
                    mk[j] = 0u;
                    sv[j] = 0ull;
                    if (i < hi) {
                        const LEnt o = S.order[i];
                        sv[j] = o.sigdm >> pk.cb;
                        e0[j] = o.e0;
                        mk[j] = (unsigned)(o.sigdm & pk.low);
                        kk[j] = o.v & (K - 1);
                        if (mk[j] == (unsigned)pk.low) {  // long row: walk it and re-test every edge
                            dv[j] = dist_of(ldcg64(S.word + o.v));
                            e[j] = o.e0;
                            e1[j] = __ldg(rp + (o.v >> kSh) + 1);
                            mk[j] = 0u;
                        }
                    }
                }
                for (;;) {
                    bool more = false;
#pragma unroll
                    for (int j = 0; j < kV; ++j) more |= mk[j] != 0u || e[j] < e1[j];
                    if (!__any_sync(kFull, more)) break;
                    int x[kV], nd[kV], r0[kV];
                    bool tight[kV];
#pragma unroll
                    for (int j = 0; j < kV; ++j) {
                        x[j] = -1;
                        tight[j] = false;
                        int ei = -1;
                        if (mk[j]) {  // tight by the counting sweep
                            ei = e0[j] + __ffs(mk[j]) - 1;
                            mk[j] &= mk[j] - 1u;
                            tight[j] = true;
                        } else if (e[j] < e1[j]) {
                            ei = e[j]++;
                        }
                        if (ei >= 0) {
                            const int2 a = adj_at<kA4>(sg, ei);
                            x[j] = (a.x << kSh) + kk[j];
                            nd[j] = dv[j] + a.y;
                            r0[j] = __ldg(rp + a.x);  // row offsets: small and shared, L2-resident
                        }
                    }
#pragma unroll
                    for (int j = 0; j < kV; ++j)
                        if (x[j] >= 0 && !tight[j]) tight[j] = nd[j] == dist_of(ldcg64(S.word + x[j]));
                    unsigned long long old[kV];
                    unsigned tm[kV];
#pragma unroll
                    for (int j = 0; j < kV; ++j)
                        if (tight[j]) {
                            // one atomic adds sigma_v and retires the edge; the thread that
                            // retires the last tight in-edge knows x's final count
                            old[j] = atomicAdd(&S.rec[x[j]].sc, (sv[j] << pk.cb) - 1ull);
                            tm[j] = __ldcg(&S.rec[x[j]].mask);  // same sector as the atomic
                        }
#pragma unroll
                    for (int j = 0; j < kV; ++j) {
                        bool push = false;
                        LEnt le{x[j], 0, 0ull};
                        if (tight[j]) {
                            const unsigned long long sx = (old[j] >> pk.cb) + sv[j];
                            if (sx > pk.sigmax || sv[j] > pk.sigmax) bad |= kErrRetry;
                            push = (old[j] & pk.low) == 1ull;
                            le.e0 = r0[j];
                            le.sigdm = pk.sig_dm(sx, tm[j]);
                        }
                        bpush(push, le, S.order, &C.ocnt, (int)cap + 1, &C.ovf);
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
        if (!bad) {
            for (int k = 0; k < K; ++k) {
                const Unit& u = us[k];
                if (u.src < 0 || u.bout < 0) continue;
                for (int j = tid; j < sg.nb; j += nth) {
                    const int b = sg.border[j] * K + k;
                    const int d = dist_of(ldcg64(S.word + b));
                    P.bdist[u.bout + j] = d != kInf ? (double)d : 0.0;
                    P.bsig[u.bout + j] = d != kInf ? (d == 0 ? 1ull : __ldcg(&S.rec[b].sc) >> pk.cb) : 0ull;
                }
            }
        }
    }
    if (!bad) {
        // --------------------------------------------------------- dependency
        for (int L = nlev - 1; L >= 0; --L) {
            const int a0 = __ldcg(S.lvl + L), a1 = __ldcg(S.lvl + L + 1);
            // kV entries per lane, one tight edge of each per step (as in the Kahn pass)
            for (int base = a0 + (tid & ~31) * kV; base < a1; base += nth * kV) {
                LEnt o[kV];
                unsigned mk[kV];
                typename Prec::Acc acc[kV];
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    const int i = base + j * 32 + (tid & 31);
                    acc[j] = Prec::zero();
                    o[j].v = -1;
                    mk[j] = 0u;
                    if (i < a1) {
                        o[j] = S.order[i];
                        mk[j] = (unsigned)(o[j].sigdm & pk.low);
                        if (mk[j] == (unsigned)pk.low) mk[j] = 0u;
                    }
                }
                for (;;) {
                    bool more = false;
#pragma unroll
                    for (int j = 0; j < kV; ++j) more |= mk[j] != 0u;
                    if (!more) break;
                    int x[kV];
#pragma unroll
                    for (int j = 0; j < kV; ++j) {
                        x[j] = -1;
                        if (mk[j]) {
                            const int b = __ffs(mk[j]) - 1;
                            mk[j] &= mk[j] - 1u;
                            x[j] = (adj_at<kA4>(sg, o[j].e0 + b).x << kSh) + (o[j].v & (K - 1));
                        }
                    }
                    unsigned long long sx[kV];
                    typename Prec::D dx[kV];
#pragma unroll
                    for (int j = 0; j < kV; ++j)
                        if (x[j] >= 0) {
                            const ulonglong2 r = __ldcg(reinterpret_cast<const ulonglong2*>(S.rec + x[j]));
                            sx[j] = r.x >> pk.cb;
                            dx[j] = bits_to<typename Prec::D>(r.y);
                        }
#pragma unroll
                    for (int j = 0; j < kV; ++j)
                        if (x[j] >= 0) {
                            const unsigned long long sv = o[j].sigdm >> pk.cb;
                            if (sx[j] == sv) Prec::add_same(acc[j], dx[j]);
                            else Prec::add(acc[j], sv, sx[j], dx[j]);
                        }
                }
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    if (o[j].v < 0) continue;
                    const int v = o[j].v >> kSh, k = o[j].v & (K - 1);
                    if ((o[j].sigdm & pk.low) == pk.low) {  // long row: re-test every edge
                        const int e1 = __ldg(rp + v + 1);
                        const int dv = dist_of(ldcg64(S.word + o[j].v));
                        const unsigned long long sv = o[j].sigdm >> pk.cb;
                        for (int e = o[j].e0; e < e1; ++e) {
                            const int2 a = adj_at<kA4>(sg, e);
                            const int xk = (a.x << kSh) + k;
                            if (dv + a.y == dist_of(ldcg64(S.word + xk))) {
                                const ulonglong2 r = __ldcg(reinterpret_cast<const ulonglong2*>(S.rec + xk));
                                const unsigned long long s2 = r.x >> pk.cb;
                                const typename Prec::D d2 = bits_to<typename Prec::D>(r.y);
                                if (s2 == sv) Prec::add_same(acc[j], d2);
                                else Prec::add(acc[j], sv, s2, d2);
                            }
                        }
                    }
                    S.rec[o[j].v].dlt = Prec::store(acc[j]);
                    if (v != us[k].src && !P.bc_seg) {
                        const double card = us[k].card;
                        const int64_t ov = sg.out_base + (sg.gid ? sg.gid[v] : v);
                        atomicAdd(P.bc + ov, card == 1.0 ? Prec::value(acc[j]) : card * Prec::value(acc[j]));
                    }
                }
            }
            __syncthreads();
        }
    }
    if (tid == 0 && bad) {
        for (int k = 0; k < K; ++k) {
            if (us[k].src < 0) continue;
            if (bad == kErrRetry) request_retry(P, us[k], kErrRetry);  // recomputed with 64-bit counts
            else atomicOr(P.err, bad);
        }
    }
    if (P.dbg_dist) {  // single-source debug runs: source 0 of the group
        const int src = us[0].src;
        for (int v = tid; v < n; v += nth) {
            const int d = dist_of(ldcg64(S.word + v * K));
            P.dbg_dist[v] = d != kInf ? d : -1;
            P.dbg_sig[v] = d != kInf ? (v == src ? 1ull : __ldcg(&S.rec[v * K].sc) >> pk.cb) : 0ull;
            P.dbg_dlt[v] = d != kInf ? Prec::value(Prec::load(S.rec[v * K].dlt)) : 0.0;
        }
    }
    __syncthreads();
    // restore: word = (inf, 0), sigma/counter = 0 (not with reverse weights: the counting sweep
    // then stores every reached record whole, and the slot header records the extent left
    // unclean for a later atomic-count unit).  With a segment-order accumulator this sweep
    // also adds card * delta of every reached vertex but the source, coalesced, instead of the
    // dependency pass's scattered reductions through gid (the host adds it into bc at the end).
    if (P.bc_seg && !bad) {
        for (int i = tid; i < nK; i += nth) {
            const int k = i & (K - 1);
            const int v = i >> kSh;
            if (dist_of(ldcg64(S.word + i)) != kInf && v != us[k].src && us[k].src >= 0) {
                const double d = Prec::value(Prec::load(S.rec[i].dlt));
                const double card = us[k].card;
                atomicAdd(P.bc_seg + v, card == 1.0 ? d : card * d);
            }
            S.word[i] = (unsigned long long)(unsigned)kInf << 32;
            if (!sg.revw) S.rec[i].sc = 0ull;
        }
    } else {
        for (int i = tid; i < nK; i += nth) {
            S.word[i] = (unsigned long long)(unsigned)kInf << 32;
            if (!sg.revw) S.rec[i].sc = 0ull;
        }
    }
    __syncthreads();
}

// kForm: 0 = 128-thread blocks, five per SM; 1 = 512-thread blocks for segments whose frontiers
// span many hundreds of vertices (millions of vertices); 2 = 1024-thread blocks (64 registers),
// two level entries per lane; 3 = the same with one level entry per lane (fewer spills).
// K: sources per block; units come in groups of K of one segment (padded with src = -1),
// P.nunits counts groups.  kA4: the segments' packed 4-byte adjacency.
template <class Prec, int kForm, int K, bool kA4 = false>
__global__ void __launch_bounds__(kForm >= 2 ? 1024 : kForm == 1 ? 512 : 128, kForm == 0 ? 5 : 1)
    frontier_kernel(KParams P) {
    __shared__ FCtl C;
    __shared__ Unit us[K];
    char* slot = P.ws + (int64_t)blockIdx.x * P.ws_stride;
    unsigned* hdr = (unsigned*)slot;
    const int64_t cap = P.ws_n;  // entries of the slot (its layout depends on nothing else)
    FState<Prec> S = fstate_carve<Prec>(slot + 256, cap);
    if (hdr[0] == 0u) {  // fresh slot: establish the between-units invariant
        for (int64_t i = threadIdx.x; i < cap; i += blockDim.x) {
            S.word[i] = (unsigned long long)(unsigned)kInf << 32;
            S.rec[i].sc = 0ull;
        }
        __syncthreads();
        if (threadIdx.x == 0) hdr[0] = 1u;
    }
    for (;;) {
        if (threadIdx.x == 0) C.unit = (int)atomicAdd(P.next_unit, 1ull);
        __syncthreads();
        const int64_t gi = C.unit;
        if (gi < P.nunits && threadIdx.x < K) us[threadIdx.x] = P.units[gi * K + threadIdx.x];
        __syncthreads();
        if (gi >= P.nunits) break;
        // header word 1: entries whose counters a pull-count unit (reverse weights) left
        // non-zero; an atomic-count unit clears them first
        const Seg& sgu = P.segs[us[0].seg];
        const bool pull = sgu.revw != nullptr;
        if (!pull) {
            const unsigned dirty = __ldcg(hdr + 1);
            if (dirty) {
                for (int64_t i = threadIdx.x; i < (int64_t)dirty; i += blockDim.x) S.rec[i].sc = 0ull;
                __syncthreads();
                if (threadIdx.x == 0) hdr[1] = 0u;
            }
        }
        frontier_group<Prec, kForm == 3 ? 1 : 2, K, 1, kA4>(P, us, S, C, cap);
        if (pull && threadIdx.x == 0) {
            const unsigned nk = (unsigned)sgu.n * (unsigned)K;
            if (__ldcg(hdr + 1) < nk) hdr[1] = nk;
        }
    }
}

// bc[out_base + gid[v]] += acc[v]: a one-segment launch's accumulator (segment order) added into
// the output (gid injective, so plain read-modify-writes suffice on the launch's stream).
__global__ void add_seg_kernel(const double* __restrict__ acc, const int32_t* __restrict__ gid, int64_t out_base,
                               int n, double* bc) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        bc[out_base + gid[v]] += acc[v];
}

}  // namespace fbc
