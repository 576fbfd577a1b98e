// Device side of the GB300 Brandes engine.
//
// One "unit" is one source vertex in one CSR segment (a whole graph, the induced
// subgraph of one Louvain cluster, or one graph of a multi-graph batch).  A unit runs
// the three passes of the reference's single-source Brandes
// (ExactBrandesBC.h:97-161 forward, ExactBrandesBC.h:73-90 backward):
//
//   1. distances   near-far delta-stepping over int32 weights: near queue = vertices with
//                  tentative distance below the bucket threshold T, far pile = the rest;
//                  relaxation by atomicMin on int32 distances, warp-cooperative over the
//                  concatenated adjacency of 32 queued vertices.
//   2. sigma       exact uint64 path counts in topological order of the shortest-path DAG
//                  (Kahn): a tight in-edge counter per vertex; a vertex joins the next
//                  level when its last predecessor has pushed its count.  The predecessor
//                  sets are implicit: v precedes w iff dist[v] + w(v,w) == dist[w], which
//                  is exactly the reference's list after its clear-on-improve rule
//                  (ExactBrandesBC.h:142-156).
//   3. dependency  Kahn levels walked in reverse; each vertex pulls
//                  sigma_v / sigma_w * (1 + delta_w) from its tight out-edges
//                  (ExactBrandesBC.h:81) in adjacency order, so no atomics and a
//                  deterministic sum; then BC[v] += card * delta_v (ExactBrandesBC.h:86-89,
//                  ClusteredBrandesBC.h:151-155).
//
// The block-per-source kernel below (per-source state in a global-memory slot) is the plain
// schedule; batched_kernels.cuh holds the batched one.  Two precision forms share the code
// through the Prec template:
//   PrecF64     FP64 dependency arithmetic (the plain form)
//   PrecDF32    FP32 double-float (two-sum compensated) dependency arithmetic; FP64 only
//               for sigma ratios whose operands exceed 2^24 and for the BC reduction.
//
// Every loop is bounded: the distance pass stops after iter_cap rounds, the Kahn and
// backward passes after n levels; a unit that hits a bound sets an error bit that the
// host turns into a status code, and the state is still restored for the next unit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fbc {

constexpr int32_t kInf = 0x7fffffff;
constexpr unsigned kFull = 0xffffffffu;

enum : int { kErrIter = 1, kErrSigma = 2, kErrQueue = 4, kErrRetry = 8 };

// One CSR segment (device pointers).
struct Seg {
    const int32_t* rp;      // n+1 row offsets into adj
    const int2* adj;        // packed (destination, weight) pairs, rows ascending
    const int32_t* gid;     // n local -> output ids; BC index = out_base + (gid ? gid[v] : v)
    const int32_t* border;  // nb local ids of the border vertices (ascending global id)
    const uint32_t* adj4;   // the same adjacency packed as (destination | weight << 24), or null
    const uint8_t* revw;    // weight of each edge's reverse (every edge has one, weights < 256),
                            // or null: the frontier kernel then counts tight in-edges without atomics
    int64_t out_base;
    int32_t n;              // vertices
    int32_t nb;             // border vertices (cluster segments), else 0
    int32_t delta;          // bucket width of the near-far pass
    int32_t pad;
};

// One source.
struct Unit {
    int32_t seg;
    int32_t src;     // local id in the segment
    double card;     // multiplicity of this source's dependency (pivot class cardinality)
    int64_t bout;    // first border-output entry of this source, or -1
};

// A unit whose path counts outgrew the kernel's representation.  It stopped before its
// dependency pass (nothing accumulated) and the host recomputes it one level up:
// code kErrRetry -> plain kernel with 64-bit counts, kErrSigma -> plain kernel with FP64
// counts (the reference's own representation, exact below 2^53).
struct RetryRec {
    Unit u;
    int32_t code;
    int32_t pad;
};

struct KParams {
    const Seg* segs;
    const Unit* units;
    int64_t nunits;
    double* bc;                  // BC accumulator (FP64)
    double* bc_seg;              // frontier kernel, one-segment launches: the accumulator in the
                                 // segment's own vertex order, filled by the restore sweep (null:
                                 // the dependency pass adds into bc through gid)
    double* bdist;               // border distances (0 when unreached)
    unsigned long long* bsig;    // border path counts
    unsigned long long* next_unit;
    int* err;
    char* ws;                    // global-memory slots (BlockGroup)
    int64_t ws_stride;
    int32_t ws_n;                // capacity (vertices) of one slot / one shared-memory state
    int32_t iter_mult;           // distance-pass round cap = iter_mult * (n + 2)
    int* retry_count;            // units to recompute one level up (null: report an error)
    RetryRec* retry;
    int32_t retry_cap;
    int32_t cnt_bits;            // frontier kernel: counter / mask bits next to the path count
    int32_t* dbg_dist;           // debug dump of one unit (may be null)
    unsigned long long* dbg_sig;
    double* dbg_dlt;
};

// Hand a unit back to the host (see RetryRec); without a retry list, report the error.
__device__ __forceinline__ void request_retry(const KParams& P, const Unit& u, int code) {
    if (!P.retry) {
        atomicOr(P.err, code == kErrRetry ? kErrSigma : code);
        return;
    }
    const int r = atomicAdd(P.retry_count, 1);
    if (r < P.retry_cap) P.retry[r] = RetryRec{u, code, 0};
    else atomicOr(P.err, kErrQueue);
}

// ----------------------------------------------------------------------------- groups
struct BlockGroup {
    static constexpr bool kShared = false;
    __device__ static int rank() { return threadIdx.x; }
    __device__ static int size() { return blockDim.x; }
    __device__ static void sync() { __syncthreads(); }
    __device__ static int warp() { return threadIdx.x >> 5; }
    __device__ static int nwarps() { return blockDim.x >> 5; }
};

// Loads of state that other threads modify with atomics: from L2 for global slots,
// volatile for shared memory.
template <bool kShared>
__device__ __forceinline__ int ld_i32(const int* p) {
    if constexpr (kShared) return *(const volatile int*)p;
    else return __ldcg(p);
}
template <bool kShared>
__device__ __forceinline__ unsigned long long ld_u64(const unsigned long long* p) {
    if constexpr (kShared) return *(const volatile unsigned long long*)p;
    else return __ldcg(p);
}

// ------------------------------------------------------------ FP64 values from integer ops
// Exact conversions to double assembled with integer instructions, for kernels whose other work
// has no FP64 instruction (GB300's FP64 pipe is a small fraction of its FP32 rate).
// d >= 0: the double of an int32 distance
__device__ __forceinline__ double nonneg_int_to_double(int d) {
    if (d <= 0) return 0.0;
    const int e = 31 - __clz(d);
    const unsigned long long mant = ((unsigned long long)(unsigned)d << (52 - e)) & ((1ull << 52) - 1ull);
    return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | mant));
}
// the double of a float (every float exactly: zero, subnormal, normal, inf and nan)
__device__ __forceinline__ double float_to_double(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned ex = (u >> 23) & 0xffu, mant = u & 0x7fffffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    unsigned long long e, m;
    if (ex == 0u) {
        if (mant == 0u) return __longlong_as_double((long long)sign);
        const int t = 31 - __clz(mant);  // subnormal: mant * 2^-149, leading bit t
        e = (unsigned long long)(t + 874);
        m = ((unsigned long long)mant << (52 - t)) & ((1ull << 52) - 1ull);
    } else {
        e = ex == 0xffu ? 0x7ffull : (unsigned long long)(ex + 896u);  // rebias 127 -> 1023
        m = (unsigned long long)mant << 29;
    }
    return __longlong_as_double((long long)(sign | (e << 52) | m));
}

// ------------------------------------------------------------------------- precision
struct PrecF64 {
    using D = double;
    struct Acc { double s; };
    __device__ static Acc zero() { return {0.0}; }
    // ExactBrandesBC.h:81: sigma[v] / sigma[w] * (1.0 + delta[w]), division first
    // path counts arrive as doubles: exact below 2^53, where the reference's double counts
    // are exact too
    __device__ static void add_d(Acc& a, double sv, double sw, D dw) {
        a.s += sv / sw * (1.0 + dw);
    }
    // uint64 counts (exact below 2^53 as doubles, rounded as the reference's double sums)
    __device__ static void add(Acc& a, unsigned long long sv, unsigned long long sw, D dw) {
        add_d(a, (double)sv, (double)sw, dw);
    }
    // sigma_v == sigma_w: the ratio is exactly 1.0 and 1.0 * y == y
    __device__ static void add_same(Acc& a, D dw) { a.s += 1.0 + dw; }
    __device__ static D store(const Acc& a) { return a.s; }
    __device__ static Acc load(D d) { return {d}; }
    __device__ static double value(const Acc& a) { return a.s; }
    __device__ static void red_add(double* p, const Acc& a) { atomicAdd(p, a.s); }
};

struct PrecDF32 {
    using D = float2;  // (hi, lo) double-float
    struct Acc { float hi, lo; };
    __device__ static Acc zero() { return {0.f, 0.f}; }
    // Knuth TwoSum and Dekker FastTwoSum / TwoProduct (via FMA), round-to-nearest intrinsics
    // so that no contraction or reassociation changes them.
    __device__ static void two_sum(float a, float b, float& s, float& e) {
        s = __fadd_rn(a, b);
        float bb = __fsub_rn(s, a);
        e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    }
    __device__ static void fast_two_sum(float a, float b, float& s, float& e) {
        s = __fadd_rn(a, b);
        e = __fsub_rn(b, __fsub_rn(s, a));
    }
    // ratio r = x / y of two counts up to 2^24 (exact in FP32) as a double-float
    __device__ static void ratio32(float x, float y, float& rh, float& rl) {
        rh = __fdiv_rn(x, y);
        rl = __fdiv_rn(__fmaf_rn(-rh, y, x), y);  // the remainder x - rh*y is exact
    }
    // counts above 2^24: the ratio in FP64, split into a double-float
    __device__ static void ratio64(double sv, double sw, float& rh, float& rl) {
        const double rd = sv / sw;
        rh = __double2float_rn(rd);
        rl = __double2float_rn(rd - (double)rh);
    }
    // uint64 counts: compared with 2^24 and converted to FP32 as integers, so a ratio of small
    // counts (every ratio on road-like graphs) touches no FP64 instruction
    __device__ static void add(Acc& a, unsigned long long sv, unsigned long long sw, D dw) {
        float rh, rl;
        if (sv <= 16777216ull && sw <= 16777216ull)
            ratio32(__uint2float_rn((unsigned)sv), __uint2float_rn((unsigned)sw), rh, rl);
        else
            ratio64((double)sv, (double)sw, rh, rl);
        mul_add(a, rh, rl, dw);
    }
    // FP64 counts (the plain kernel's rerun of units whose uint64 counts overflowed)
    __device__ static void add_d(Acc& a, double sv, double sw, D dw) {
        float rh, rl;
        if (sv <= 16777216.0 && sw <= 16777216.0) ratio32((float)sv, (float)sw, rh, rl);
        else ratio64(sv, sw, rh, rl);
        mul_add(a, rh, rl, dw);
    }
    // acc += (rh, rl) * (1 + dw)
    __device__ static void mul_add(Acc& a, float rh, float rl, D dw) {
        // t = 1 + delta_w
        float s, e, th, tl;
        two_sum(1.0f, dw.x, s, e);
        e = __fadd_rn(e, dw.y);
        fast_two_sum(s, e, th, tl);
        // c = r * t
        float p = __fmul_rn(rh, th);
        float pe = __fmaf_rn(rh, th, -p);
        pe = __fadd_rn(pe, __fadd_rn(__fmul_rn(rh, tl), __fmul_rn(rl, th)));
        float ch, cl;
        fast_two_sum(p, pe, ch, cl);
        // acc += c
        two_sum(a.hi, ch, s, e);
        e = __fadd_rn(e, __fadd_rn(a.lo, cl));
        fast_two_sum(s, e, a.hi, a.lo);
    }
    // sigma_v == sigma_w: r = (1, 0), so c = t exactly (the general path gives the same bits)
    __device__ static void add_same(Acc& a, D dw) {
        float s, e, th, tl;
        two_sum(1.0f, dw.x, s, e);
        e = __fadd_rn(e, dw.y);
        fast_two_sum(s, e, th, tl);
        two_sum(a.hi, th, s, e);
        e = __fadd_rn(e, __fadd_rn(a.lo, tl));
        fast_two_sum(s, e, a.hi, a.lo);
    }
    __device__ static D store(const Acc& a) { return make_float2(a.hi, a.lo); }
    __device__ static Acc load(D d) { return {d.x, d.y}; }
    __device__ static double value(const Acc& a) { return (double)a.hi + (double)a.lo; }
    // BC[o] += value: the halves widened by integer ops (the same doubles as a conversion) and
    // reduced one after the other, so the cross-source sum is the only FP64 arithmetic, done by
    // the reductions in L2 (the FP64 pipe stays idle)
    __device__ static void red_add(double* p, const Acc& a) {
        atomicAdd(p, float_to_double(a.hi));
        if (a.lo != 0.f) atomicAdd(p, float_to_double(a.lo));
    }
};

// ------------------------------------------------------------------------ warp helpers
// Visit every edge of up to 32 vertices (one per lane: row start e0, degree deg) with the
// whole warp, edges of consecutive lanes back to back, so the adjacency reads of a round are
// contiguous runs.  f(active, owner_lane, edge_index) is called by all 32 lanes each round.
template <class F>
__device__ __forceinline__ void warp_edges(int e0, int deg, F&& f) {
    const int lane = threadIdx.x & 31;
    int incl = deg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    const int excl = incl - deg;
    for (int kb = 0; kb < total; kb += 32) {
        const int k = kb + lane;
        int j = 0;  // owner: the largest lane whose exclusive prefix is <= k
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
            int ex = __shfl_sync(kFull, excl, j + s);
            if (ex <= k) j += s;
        }
        const int ev = __shfl_sync(kFull, e0, j) + (k - __shfl_sync(kFull, excl, j));
        f(k < total, j, ev);
    }
}

// Warp-aggregated append of x (where want) to q[0..cap), counter *cnt.
__device__ __forceinline__ void warp_push(bool want, int x, int* q, int* cnt, int cap, int* err) {
    const unsigned m = __ballot_sync(kFull, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(cnt, __popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (want) {
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) q[pos] = x;
        else atomicOr(err, kErrQueue);
    }
}

// ----------------------------------------------------------------------- unit state
// Per-source arrays (capacity cap vertices).  Invariant between units:
// dist == kInf, sig == 0, cnt == 0 everywhere; nflag/fflag hold stamps < epoch.
template <class Prec>
struct State {
    int* dist;
    unsigned long long* sig;
    typename Prec::D* dlt;
    int* q[4];        // near0, near1, far0, far1 (cap+1 entries each)
    unsigned* nflag;
    unsigned* fflag;
    int* cnt;
};

template <class Prec>
__host__ __device__ inline int64_t state_bytes(int64_t cap) {
    int64_t b = 0;
    auto al = [](int64_t x) { return (x + 255) & ~int64_t(255); };
    b += al(cap * 4);                               // dist
    b += al(cap * 8);                               // sig
    b += al(cap * (int64_t)sizeof(typename Prec::D));  // dlt
    b += 4 * al((cap + 1) * 4);                     // queues
    b += 2 * al(cap * 4);                           // flags
    b += al(cap * 4);                               // cnt
    return b;
}

template <class Prec>
__device__ inline State<Prec> state_carve(char* base, int64_t cap) {
    auto al = [](int64_t x) { return (x + 255) & ~int64_t(255); };
    State<Prec> s;
    char* p = base;
    s.dist = (int*)p; p += al(cap * 4);
    s.sig = (unsigned long long*)p; p += al(cap * 8);
    s.dlt = (typename Prec::D*)p; p += al(cap * (int64_t)sizeof(typename Prec::D));
    for (int i = 0; i < 4; ++i) { s.q[i] = (int*)p; p += al((cap + 1) * 4); }
    s.nflag = (unsigned*)p; p += al(cap * 4);
    s.fflag = (unsigned*)p; p += al(cap * 4);
    s.cnt = (int*)p;
    return s;
}

// Control words of one group (in shared memory).
struct Ctl {
    int ncnt[2];
    int fcnt[2];
    int dmin;
    int ocnt;
    int unit;
    unsigned epoch;
    int sbad;        // path-count overflow seen by any thread of the unit
};

// Fill a state with the invariant values (all cap entries).
template <class G, class Prec>
__device__ void state_init(const State<Prec>& s, int cap) {
    for (int i = G::rank(); i < cap; i += G::size()) {
        s.dist[i] = kInf;
        s.sig[i] = 0ull;
        s.nflag[i] = 0u;
        s.fflag[i] = 0u;
        s.cnt[i] = 0;
    }
    G::sync();
}

// Path counts: uint64 (exact; overflow hands the unit back for FP64 counts) or FP64 (the
// reference's own representation), in the same 8-byte array.
template <bool kF64>
__device__ __forceinline__ double sig_val(unsigned long long bits) {
    if constexpr (kF64) return __longlong_as_double((long long)bits);
    else return (double)bits;
}
template <bool kF64>
__device__ __forceinline__ unsigned long long sig_one() {
    if constexpr (kF64) return (unsigned long long)__double_as_longlong(1.0);
    else return 1ull;
}
// adds the count of a predecessor (raw bits); true when a uint64 count overflowed
template <bool kF64>
__device__ __forceinline__ bool sig_add_g(unsigned long long* p, unsigned long long a) {
    if constexpr (kF64) {
        atomicAdd((double*)p, __longlong_as_double((long long)a));
        return false;
    } else {
        const unsigned long long old = atomicAdd(p, a);
        return old + a < old;
    }
}
// uint64 border/debug output of a count (FP64 counts saturate at 2^64 - 1)
template <bool kF64>
__device__ __forceinline__ unsigned long long sig_out(unsigned long long bits) {
    if constexpr (kF64) {
        const double d = __longlong_as_double((long long)bits);
        return d >= 18446744073709551615.0 ? ~0ull : (unsigned long long)d;
    } else {
        return bits;
    }
}

// ---------------------------------------------------------------------- one unit
template <class G, class Prec, bool kSigF64 = false>
__device__ void run_unit(const KParams& P, const Unit& u, const State<Prec>& S, Ctl& C,
                         unsigned& epoch, int cap) {
    constexpr bool kSh = G::kShared;
    const Seg sg = P.segs[u.seg];
    const int n = sg.n;
    const int* __restrict__ rp = sg.rp;
    const int2* __restrict__ adj = sg.adj;
    const int lane = threadIdx.x & 31;
    const int src = u.src;
    const int delta = sg.delta > 0 ? sg.delta : 1;
    int bad = 0;

    // Stamps must never repeat within the flag arrays' lifetime: renew them well before
    // the 32-bit counter could wrap (the round cap bounds the stamps one unit uses).
    const int64_t cap_rounds = (int64_t)P.iter_mult * ((int64_t)n + 2);
    if ((int64_t)epoch + 2 * cap_rounds + 16 > 0x7fffffffLL) {
        for (int i = G::rank(); i < cap; i += G::size()) { S.nflag[i] = 0u; S.fflag[i] = 0u; }
        epoch = 1;
        G::sync();
    }

    // ---------------------------------------------------------------- 1. distances
    int T = delta;          // bucket threshold: near = tentative distance < T
    int qs = 0, fs = 0;     // current near / far buffers
    unsigned fgen = ++epoch;
    if (G::rank() == 0) {
        S.dist[src] = 0;
        S.sig[src] = sig_one<kSigF64>();
        S.q[0][0] = src;
        S.nflag[src] = epoch + 1;
        C.sbad = 0;
        C.ncnt[0] = 1;
        C.ncnt[1] = 0;
        C.fcnt[0] = 0;
        C.fcnt[1] = 0;
    }
    G::sync();
    int64_t rounds = 0;
    for (;;) {
        int ncur = C.ncnt[qs];
        if (ncur > 0) {
            if (++rounds > cap_rounds) { bad = kErrIter; break; }
            const unsigned stamp = ++epoch;
            const int* qc = S.q[qs];
            int* qn = S.q[qs ^ 1];
            int* qf = S.q[2 + fs];
            for (int base = G::warp() * 32; base < ncur; base += G::nwarps() * 32) {
                const int i = base + lane;
                int e0 = 0, deg = 0, dv = 0;
                if (i < ncur) {
                    const int v = qc[i];
                    dv = ld_i32<kSh>(S.dist + v);
                    e0 = rp[v];
                    deg = rp[v + 1] - e0;
                }
                warp_edges(e0, deg, [&](bool act, int j, int ev) {
                    const int dvv = __shfl_sync(kFull, dv, j);
                    bool pn = false, pf = false;
                    int x = 0;
                    if (act) {
                        const int2 a = __ldg(adj + ev);
                        x = a.x;
                        const int nd = dvv + a.y;
                        const int old = atomicMin(S.dist + x, nd);
                        if (nd < old) {
                            if (nd < T) pn = atomicExch(S.nflag + x, stamp) != stamp;
                            else pf = atomicExch(S.fflag + x, fgen) != fgen;
                        }
                    }
                    warp_push(pn, x, qn, &C.ncnt[qs ^ 1], cap + 1, P.err);
                    warp_push(pf, x, qf, &C.fcnt[fs], cap + 1, P.err);
                });
            }
            G::sync();
            if (G::rank() == 0) C.ncnt[qs] = 0;
            qs ^= 1;
            G::sync();
            continue;
        }
        // near queue empty: advance the threshold to the bucket of the closest far vertex
        const int nfar = C.fcnt[fs];
        if (nfar == 0) break;
        if (++rounds > cap_rounds) { bad = kErrIter; break; }
        if (G::rank() == 0) C.dmin = kInf;
        G::sync();
        const int* qf = S.q[2 + fs];
        for (int i = G::rank(); i < nfar; i += G::size()) {
            const int d = ld_i32<kSh>(S.dist + qf[i]);
            if (d >= T) atomicMin(&C.dmin, d);
        }
        G::sync();
        const int dmin = C.dmin;
        if (dmin == kInf) break;  // every far entry was already settled
        const int Told = T;
        const int64_t tn = ((int64_t)dmin / delta + 1) * (int64_t)delta;
        T = tn > (int64_t)kInf ? kInf : (int)tn;
        const unsigned stamp = ++epoch;
        fgen = ++epoch;
        int* qn = S.q[qs];
        int* qf2 = S.q[2 + (fs ^ 1)];
        for (int base = G::warp() * 32; base < nfar; base += G::nwarps() * 32) {
            const int i = base + lane;
            bool pn = false, pf = false;
            int x = 0;
            if (i < nfar) {
                x = qf[i];
                const int d = ld_i32<kSh>(S.dist + x);
                if (d >= Told) {
                    if (d < T) pn = atomicExch(S.nflag + x, stamp) != stamp;
                    else pf = atomicExch(S.fflag + x, fgen) != fgen;
                }
            }
            warp_push(pn, x, qn, &C.ncnt[qs], cap + 1, P.err);
            warp_push(pf, x, qf2, &C.fcnt[fs ^ 1], cap + 1, P.err);
        }
        G::sync();
        if (G::rank() == 0) C.fcnt[fs] = 0;
        fs ^= 1;
        G::sync();
    }
    G::sync();

    int* order = S.q[0];
    int* lvl = S.q[1];
    int nlev = 0;
    int reached = 0;
    if (!bad) {
        // ---------------------------------------------------------- 2. sigma (Kahn)
        // tight in-edge counts
        for (int base = G::warp() * 32; base < n; base += G::nwarps() * 32) {
            const int v = base + lane;
            int e0 = 0, deg = 0, dv = kInf;
            if (v < n) {
                dv = ld_i32<kSh>(S.dist + v);
                if (dv != kInf) {
                    e0 = rp[v];
                    deg = rp[v + 1] - e0;
                }
            }
            warp_edges(e0, deg, [&](bool act, int j, int ev) {
                const int dvv = __shfl_sync(kFull, dv, j);
                if (act) {
                    const int2 a = __ldg(adj + ev);
                    if (dvv + a.y == ld_i32<kSh>(S.dist + a.x)) atomicAdd(S.cnt + a.x, 1);
                }
            });
        }
        if (G::rank() == 0) {
            order[0] = src;
            lvl[0] = 0;
            C.ocnt = 1;
        }
        G::sync();
        int lo = 0, hi = 1;
        while (lo < hi) {
            if (nlev >= n) { bad = kErrIter; break; }
            for (int base = lo + G::warp() * 32; base < hi; base += G::nwarps() * 32) {
                const int i = base + lane;
                int e0 = 0, deg = 0, dv = 0;
                unsigned long long sv = 0;
                if (i < hi) {
                    const int v = order[i];
                    dv = ld_i32<kSh>(S.dist + v);
                    sv = ld_u64<kSh>(S.sig + v);
                    e0 = rp[v];
                    deg = rp[v + 1] - e0;
                }
                warp_edges(e0, deg, [&](bool act, int j, int ev) {
                    const int dvv = __shfl_sync(kFull, dv, j);
                    const unsigned long long svv = __shfl_sync(kFull, sv, j);
                    bool push = false;
                    int x = 0;
                    if (act) {
                        const int2 a = __ldg(adj + ev);
                        x = a.x;
                        if (dvv + a.y == ld_i32<kSh>(S.dist + x)) {
                            if (sig_add_g<kSigF64>(S.sig + x, svv)) C.sbad = 1;
                            push = atomicSub(S.cnt + x, 1) == 1;
                        }
                    }
                    warp_push(push, x, order, &C.ocnt, cap + 1, P.err);
                });
            }
            G::sync();
            ++nlev;                                // level nlev-1 = order[lo, hi) is done
            if (G::rank() == 0) lvl[nlev] = hi;    // lvl[L] = first entry of level L
            lo = hi;
            hi = C.ocnt;
            G::sync();
        }
        reached = hi;
        G::sync();
        const bool overflow = C.sbad != 0;  // uint64 counts overflowed: retry with FP64 counts
        if (overflow) bad = kErrSigma;

        // border (dist or 0 when unreached, sigma) of this source: DijkstraClusterEvaluator.h:166-177
        if (!overflow && u.bout >= 0) {
            const int* bl = sg.border;
            for (int j = G::rank(); j < sg.nb; j += G::size()) {
                const int b = bl[j];
                const int d = ld_i32<kSh>(S.dist + b);
                P.bdist[u.bout + j] = d != kInf ? (double)d : 0.0;
                P.bsig[u.bout + j] = sig_out<kSigF64>(ld_u64<kSh>(S.sig + b));
            }
        }
    }
    if (!bad) {
        // ------------------------------------------------------- 3. dependency
        const int* gid = sg.gid;
        const double card = u.card;
        for (int L = nlev - 1; L >= 0; --L) {
            const int a0 = lvl[L], a1 = lvl[L + 1];
            for (int i = a0 + G::rank(); i < a1; i += G::size()) {
                const int v = order[i];
                const int dv = ld_i32<kSh>(S.dist + v);
                const unsigned long long bv = ld_u64<kSh>(S.sig + v);  // raw count bits
                typename Prec::Acc acc = Prec::zero();
                const int e1 = rp[v + 1];
                for (int e = rp[v]; e < e1; ++e) {
                    const int2 a = __ldg(adj + e);
                    if (dv + a.y == ld_i32<kSh>(S.dist + a.x)) {
                        const unsigned long long bx = ld_u64<kSh>(S.sig + a.x);
                        if (bx == bv) Prec::add_same(acc, S.dlt[a.x]);
                        else if constexpr (kSigF64) Prec::add_d(acc, sig_val<true>(bv), sig_val<true>(bx), S.dlt[a.x]);
                        else Prec::add(acc, bv, bx, S.dlt[a.x]);
                    }
                }
                S.dlt[v] = Prec::store(acc);
                if (v != src) {
                    const int64_t o = sg.out_base + (gid ? gid[v] : v);
                    atomicAdd(P.bc + o, card * Prec::value(acc));
                }
            }
            G::sync();
        }
    }
    (void)reached;
    if (bad && G::rank() == 0) {
        if (bad == kErrSigma) request_retry(P, u, kErrSigma);
        else atomicOr(P.err, bad);
    }
    if (P.dbg_dist) {
        for (int v = G::rank(); v < n; v += G::size()) {
            const int d = ld_i32<kSh>(S.dist + v);
            P.dbg_dist[v] = d != kInf ? d : -1;
            P.dbg_sig[v] = sig_out<kSigF64>(ld_u64<kSh>(S.sig + v));
            P.dbg_dlt[v] = d != kInf ? Prec::value(Prec::load(S.dlt[v])) : 0.0;
        }
        G::sync();
    }

    // ------------------------------------------------------------ restore invariant
    for (int v = G::rank(); v < n; v += G::size()) {
        S.dist[v] = kInf;
        S.sig[v] = 0ull;
        S.cnt[v] = 0;
    }
    G::sync();
}

// ------------------------------------------------------------------------- kernels
// Block per source, state in a global-memory slot per block; blocks pull units from a
// shared counter until none are left (persistent grid, sized by the host).
template <class Prec, bool kSigF64 = false>
__global__ void __launch_bounds__(1024) brandes_block_kernel(KParams P) {
    __shared__ Ctl C;
    char* slot = P.ws + (int64_t)blockIdx.x * P.ws_stride;
    unsigned* hdr = (unsigned*)slot;  // persistent stamp counter of this slot
    State<Prec> S = state_carve<Prec>(slot + 256, P.ws_n);
    unsigned epoch = hdr[0];
    if (epoch == 0u) {  // fresh slot
        state_init<BlockGroup, Prec>(S, P.ws_n);
        epoch = 1u;
    }
    for (;;) {
        if (threadIdx.x == 0) C.unit = (int)atomicAdd(P.next_unit, 1ull);
        __syncthreads();
        const int64_t ui = C.unit;
        __syncthreads();
        if (ui >= P.nunits) break;
        const Unit u = P.units[ui];
        run_unit<BlockGroup, Prec, kSigF64>(P, u, S, C, epoch, P.ws_n);
    }
    if (threadIdx.x == 0) hdr[0] = epoch;
}

}  // namespace fbc
