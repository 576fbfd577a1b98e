// Edge-list text -> (source, destination, weight) arrays on the device, with the reading rules of
// DirectedWeightedGraph(std::istream&) (DirectedWeightedGraph.h:67-96): whitespace-separated
// triples "src dst weight", src and dst read as int (operator>>(int&)), the weight as double
// (operator>>(double&), which libstdc++ hands to strtod in the "C" locale), a weight <= 0 rejected
// ("Edge weight must be greater than zero"), and reading ends at the end of the text.
//
// Two passes over the bytes, each thread loading 64 of them as four 16-byte loads:
//   tx_count  -- token starts per 16 KiB tile (a non-space byte after a space byte or the start);
//   (a scan of the tile counts gives every token its index k in the text)
//   tx_tokens -- the block of a tile lists the triples whose first token (index k = 3e) starts
//                in it, then one thread per triple parses its three tokens (so the threads of a
//                warp run the same int, int, double steps together).
// A weight is converted on the device when its decimal significand has at most 19 digits, is
// at most 2^53 and its power of ten is within 10^+-22: one correctly rounded IEEE multiply or
// divide of two exact doubles then gives the correctly rounded value (Clinger's fast path,
// "How to read floating point numbers accurately", PLDI 1990).  Other valid weights (long
// significands, large exponents) are listed for the host, which converts them with strtod.
#pragma once
#include <cstdint>

namespace fbc {

constexpr int kTxThreads = 256;
constexpr int kTxBytes = 64;                      // per thread: four 16-byte loads in flight
constexpr int kTxTile = kTxThreads * kTxBytes;    // bytes per block tile

// per-triple findings, kept as the least triple index showing each
struct TxFind {
    int32_t bad_id;   // a vertex-id token that is not a decimal int32
    int32_t bad_w;    // a weight token that is not a number, or a weight <= 0
    int32_t nslow;    // weights left to the host conversion
};

__device__ __forceinline__ bool tx_space(unsigned c) { return c == 32u || (c >= 9u && c <= 13u); }

// bit i set where byte i of the 16 is a space, four bytes per step: per-byte compares give 0xff
// or 0 per byte, and the multiply gathers the low bit of each byte into bits 28-31 (the partial
// products of 0x10204080 put every other bit below 28 or above 31, with no carries between them)
__device__ __forceinline__ unsigned tx_space4(unsigned x) {
    const unsigned sp = __vcmpeq4(x, 0x20202020u) | __vcmpltu4(__vsub4(x, 0x09090909u), 0x05050505u);
    return ((sp & 0x01010101u) * 0x10204080u) >> 28;
}

__device__ __forceinline__ unsigned tx_space_bits(uint4 q) {
    return tx_space4(q.x) | (tx_space4(q.y) << 4) | (tx_space4(q.z) << 8) | (tx_space4(q.w) << 12);
}

// token starts among the kTxBytes bytes q (at off): not a space, and the byte before is one (or
// the text starts there)
__device__ __forceinline__ unsigned long long tx_start_bits(const uint4 (&q)[kTxBytes / 16],
                                                            const unsigned char* __restrict__ text, int64_t off) {
    const unsigned prev = off > 0 ? (unsigned)text[off - 1] : 32u;
    unsigned long long sp = 0;
#pragma unroll
    for (int i = 0; i < kTxBytes / 16; ++i) sp |= (unsigned long long)tx_space_bits(q[i]) << (16 * i);
    const unsigned long long before = (sp << 1) | (tx_space(prev) ? 1ull : 0ull);  // predecessor is a space
    return ~sp & before;
}

__device__ __forceinline__ void tx_load(const unsigned char* __restrict__ text, int64_t off, uint4 (&q)[kTxBytes / 16]) {
    const uint4* p = reinterpret_cast<const uint4*>(text + off);
#pragma unroll
    for (int i = 0; i < kTxBytes / 16; ++i) q[i] = p[i];
}

__global__ void __launch_bounds__(kTxThreads) tx_count_kernel(int64_t ntiles, const unsigned char* __restrict__ text,
                                                              int32_t* __restrict__ cnt) {
    __shared__ int ws[kTxThreads / 32];
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t off = t * kTxTile + kTxBytes * (int64_t)threadIdx.x;
        uint4 q[kTxBytes / 16];
        tx_load(text, off, q);
        int c = __popcll(tx_start_bits(q, text, off));
        c = __reduce_add_sync(0xffffffffu, c);
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0;
            for (int k = 0; k < kTxThreads / 32; ++k) s += ws[k];
            cnt[t] = s;
        }
        __syncthreads();
    }
}

// The bytes of a block's tile (and a halo after it) in shared memory, the rest of the text in
// global memory: a triple that starts in the tile is read from shared memory unless it runs past
// the halo.
struct TxBytes {
    const unsigned char* sm;
    const unsigned char* __restrict__ g;
    int32_t base, lim;
    __device__ __forceinline__ unsigned operator()(int32_t pos) const {
        const int32_t r = pos - base;
        return r < lim ? (unsigned)sm[r] : (unsigned)g[pos];
    }
};

// operator>>(int&) on a whole token: [+-]?[0-9]+ within int32.  Returns the token's length (it
// ends at a space; the text ends in one, so the scan stops inside the buffer); ok tells whether
// the token is such an int.
__device__ __forceinline__ int tx_int(const TxBytes& s, int32_t p, int32_t& out, bool& ok) {
    int k = 0;
    bool neg = false;
    const unsigned c0 = s(p);
    if (c0 == '+' || c0 == '-') {
        neg = c0 == '-';
        k = 1;
    }
    long long v = 0;
    int nd = 0;
    ok = true;
    for (;; ++k) {
        const unsigned c = s(p + k);
        if (tx_space(c)) break;
        if (c < '0' || c > '9') {
            ok = false;
            continue;
        }
        if (v <= 2147483648ll) v = v * 10 + (long long)(c - '0');
        ++nd;
    }
    if (neg) v = -v;
    ok = ok && nd > 0 && v >= -2147483648ll && v <= 2147483647ll;
    out = ok ? (int32_t)v : 0;
    return k;
}

__device__ __forceinline__ int tx_spaces(const TxBytes& s, int32_t p) {
    int k = 0;
    while (tx_space(s(p + k))) ++k;
    return k;
}

// weight token: 0 = converted (value in out), 1 = valid but left to the host, 2 = not a number
// or a value <= 0.  Grammar (what libstdc++ collects for a double and strtod accepts whole):
// [+-]? (digits [. digits?] | . digits) ([eE] [+-]? digits)?
__device__ __forceinline__ int tx_weight(const TxBytes& s, int32_t p, double& out) {
    int k = 0;
    bool neg = false;
    const unsigned c0 = s(p);
    if (c0 == '+' || c0 == '-') {
        neg = c0 == '-';
        k = 1;
    }
    unsigned long long m = 0;
    int nsig = 0, nd = 0, dexp = 0;
    bool slow = false, point = false;
    unsigned c;
    for (;; ++k) {
        c = s(p + k);
        if (c == '.' && !point) {
            point = true;
            continue;
        }
        if (c < '0' || c > '9') break;
        ++nd;
        const unsigned d = c - '0';
        if (m == 0 && d == 0) {  // a leading zero
            if (point) --dexp;
            continue;
        }
        if (nsig < 19) {
            m = m * 10 + d;
            ++nsig;
            if (point) --dexp;
        } else {
            slow = true;  // more than 19 significant digits
        }
    }
    if (nd == 0) return 2;
    int e = 0;
    if (c == 'e' || c == 'E') {
        ++k;
        bool eneg = false;
        c = s(p + k);
        if (c == '+' || c == '-') {
            eneg = c == '-';
            ++k;
        }
        int ne = 0;
        for (;; ++k) {
            c = s(p + k);
            if (c < '0' || c > '9') break;
            if (e < 100000) e = e * 10 + (int)(c - '0');
            ++ne;
        }
        if (ne == 0) return 2;
        if (eneg) e = -e;
    }
    if (!tx_space(c)) return 2;
    if (m == 0 || neg) return 2;  // zero (of any exponent) or negative: not > 0
    const int e10 = dexp + e;
    if (slow || m > (1ull << 53) || e10 < -22 || e10 > 22) return 1;
    if (e10 == 0) {  // integers: the conversion of m is exact
        out = (double)m;
        return 0;
    }
    // 10^a for a <= 22 is an exact double (5^22 < 2^53), so each partial product below is exact
    double pw = 1.0;
    const int a = e10 < 0 ? -e10 : e10;
    for (int i = 0; i < a / 8; ++i) pw *= 1e8;
    for (int i = 0; i < a % 8; ++i) pw *= 10.0;
    out = e10 >= 0 ? __dmul_rn((double)m, pw) : __ddiv_rn((double)m, pw);
    return 0;
}

// ---- fast path: whole tokens read eight bytes at a time from the staged tile ----

// The 8 bytes at staged offset r, byte 0 first (r + 16 <= the staged length).
__device__ __forceinline__ unsigned long long tx_load8(const unsigned char* sm, int r) {
    const unsigned long long* wv = reinterpret_cast<const unsigned long long*>(sm + (r & ~7));
    const unsigned sh = 8u * (unsigned)(r & 7);
    const unsigned long long lo = wv[0], hi = wv[1];
    return sh ? (lo >> sh) | (hi << (64u - sh)) : lo;
}

// bit i set where byte i of the 8 is a space
__device__ __forceinline__ unsigned tx_space8(unsigned long long x) {
    return tx_space4((unsigned)x) | (tx_space4((unsigned)(x >> 32)) << 4);
}

// The value of a token of len (1..8) bytes at the start of x when all of them are decimal digits,
// else -1.  The digits are moved to the top of the word behind '0' bytes; a byte is a digit iff
// adding 0x46 and subtracting 0x30 both leave its top bit clear; then pairs, quads and the two
// halves are combined (10, 100, 10^4), each step staying inside its lane (99, 9999 and
// 99,999,999 fit their 8, 16 and 32 bits).
__device__ __forceinline__ long long tx_digits8(unsigned long long x, int len) {
    const unsigned sh = 8u * (unsigned)(8 - len);
    const unsigned long long z = 0x3030303030303030ull;
    const unsigned long long t = sh ? (x << sh) | (z >> (64u - sh)) : x;
    if (((t + 0x4646464646464646ull) | (t - z)) & 0x8080808080808080ull) return -1;
    unsigned long long v = t - z;
    v = ((v * 10u) + (v >> 8)) & 0x00FF00FF00FF00FFull;
    v = ((v * 100u) + (v >> 16)) & 0x0000FFFF0000FFFFull;
    v = ((v * 10000u) + (v >> 32)) & 0xFFFFFFFFull;
    return (long long)v;
}

// A triple of plain decimal tokens of at most 8 digits each, separated by runs of fewer than 8
// spaces, starting at staged offset r: its values (the weight > 0).  False when any of that does
// not hold; the general path then reads the triple and reports what is wrong with it.
__device__ __forceinline__ bool tx_triple_fast(const unsigned char* sm, int r, int lim, int32_t& a, int32_t& b,
                                               double& x) {
    long long val[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        if (r + 16 > lim) return false;
        unsigned long long w8 = tx_load8(sm, r);
        unsigned sp = tx_space8(w8);
        if (f > 0) {  // r is at the spaces after the previous token
            const unsigned tok = ~sp & 0xffu;
            if (!tok) return false;  // eight or more spaces
            r += __ffs(tok) - 1;
            if (r + 16 > lim) return false;
            w8 = tx_load8(sm, r);
            sp = tx_space8(w8);
        }
        if (!sp) return false;          // a token of more than 8 bytes
        const int len = __ffs(sp) - 1;  // >= 1: r is at a token start
        val[f] = tx_digits8(w8, len);
        if (val[f] < 0) return false;   // a sign, point, exponent or other byte
        r += len;
    }
    if (val[2] == 0) return false;  // a zero weight: the general path rejects it
    a = (int32_t)val[0];
    b = (int32_t)val[1];
    x = (double)val[2];
    return true;
}

// One tile per block iteration: token ranks from the scan (tile_off), the first-token offsets of
// the triples starting in the tile gathered in shared memory, then one thread per triple.
// Tokens past the last complete triple (text ending inside a triple) are left alone.
constexpr int kTxTileTriples = kTxTile / 6 + 2;  // a token and its space take >= 2 bytes
constexpr int kTxHalo = 512;                        // bytes after the tile also staged (the text
                                                    // buffer has this much padding past its tiles)

__global__ void __launch_bounds__(kTxThreads) tx_tokens_kernel(int64_t ntiles, const unsigned char* __restrict__ text,
                                                               const int32_t* __restrict__ tile_off,
                                                               int32_t* __restrict__ src, int32_t* __restrict__ dst,
                                                               double* __restrict__ w, TxFind* find, int2* slow) {
    __shared__ int ws[kTxThreads / 32];
    __shared__ int32_t first[kTxTileTriples];
    __shared__ __align__(16) unsigned char bytes[kTxTile + kTxHalo];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int32_t nfull = tile_off[ntiles] / 3 * 3;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int32_t t0 = tile_off[t], t1 = min(tile_off[t + 1], nfull);
        const int32_t e0 = (t0 + 2) / 3, e1 = (t1 + 2) / 3;  // triples whose token 3e is in [t0, t1)
        const int64_t off = t * kTxTile + kTxBytes * (int64_t)threadIdx.x;
        uint4 q[kTxBytes / 16];
        tx_load(text, off, q);
#pragma unroll
        for (int i = 0; i < kTxBytes / 16; ++i)
            reinterpret_cast<uint4*>(bytes)[threadIdx.x * (kTxBytes / 16) + i] = q[i];
        if (threadIdx.x < kTxHalo / 16)
            reinterpret_cast<uint4*>(bytes + kTxTile)[threadIdx.x] =
                reinterpret_cast<const uint4*>(text + (t + 1) * kTxTile)[threadIdx.x];
        unsigned long long bits = tx_start_bits(q, text, off);
        const int c = __popcll(bits);
        int incl = c;  // inclusive warp scan
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) ws[wid] = incl;
        __syncthreads();
        int32_t k = t0 + incl - c;
        for (int j = 0; j < wid; ++j) k += ws[j];
        for (; bits; bits &= bits - 1, ++k)
            if (k < t1 && k % 3 == 0) first[k / 3 - e0] = (int32_t)(off + __ffsll((long long)bits) - 1);
        __syncthreads();
        const TxBytes by{bytes, text, (int32_t)(t * kTxTile), kTxTile + kTxHalo};
        for (int32_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            int32_t p = first[e - e0], a = 0, b = 0;
            double xf = 0.0;
            if (tx_triple_fast(bytes, p - by.base, by.lim, a, b, xf)) {
                src[e] = a;
                dst[e] = b;
                w[e] = xf;
                continue;
            }
            bool oka, okb;
            p += tx_int(by, p, a, oka);
            p += tx_spaces(by, p);
            p += tx_int(by, p, b, okb);
            p += tx_spaces(by, p);
            if (!(oka && okb)) atomicMin(&find->bad_id, e);
            double x = 0.0;
            const int r = tx_weight(by, p, x);
            if (r == 2) atomicMin(&find->bad_w, e);
            if (r == 1) slow[atomicAdd(&find->nslow, 1)] = make_int2(e, p);  // one per triple
            src[e] = a;
            dst[e] = b;
            w[e] = x;
        }
        __syncthreads();
    }
}

// host-converted weights back into place
__global__ void tx_fix_kernel(int32_t count, const int32_t* __restrict__ idx, const double* __restrict__ val,
                              double* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        w[idx[i]] = val[i];
}

}  // namespace fbc
