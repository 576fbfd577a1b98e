// Edge-list text -> (source, destination, weight) arrays on the device, with the reading rules of
// DirectedWeightedGraph(std::istream&) (DirectedWeightedGraph.h:67-96): whitespace-separated
// triples "src dst weight", src and dst read as int (operator>>(int&)), the weight as double
// (operator>>(double&), which libstdc++ hands to strtod in the "C" locale), a weight <= 0 rejected
// ("Edge weight must be greater than zero"), and reading ends at the end of the text.
//
// Three passes over the bytes, each a coalesced 16-byte load per thread:
//   tx_count  -- token starts per 4 KiB tile (a non-space byte after a space byte or the start);
//   (a scan of the tile counts)
//   tx_starts -- the byte offset of every token, in text order;
//   tx_edges  -- one thread per triple parses its three tokens.
// A weight is converted on the device when its decimal significand has at most 19 digits, is
// at most 2^53 and its power of ten is within 10^+-22: one correctly rounded IEEE multiply or
// divide of two exact doubles then gives the correctly rounded value (Clinger's fast path,
// "How to read floating point numbers accurately", PLDI 1990).  Other valid weights (long
// significands, large exponents) are listed for the host, which converts them with strtod.
#pragma once
#include <cstdint>

namespace fbc {

constexpr int kTxTile = 4096;  // bytes per block tile: 256 threads x 16 bytes
constexpr int kTxThreads = 256;

// per-triple findings, kept as the least triple index showing each
struct TxFind {
    int32_t bad_id;   // a vertex-id token that is not a decimal int32
    int32_t bad_w;    // a weight token that is not a number, or a weight <= 0
    int32_t nslow;    // weights left to the host conversion
};

__device__ __forceinline__ bool tx_space(unsigned c) { return c == 32u || (c >= 9u && c <= 13u); }

// bit i set where byte i of the 16 (bit 16: the byte before them) is a space
__device__ __forceinline__ unsigned tx_space_bits(uint4 q, unsigned prev) {
    unsigned bits = 0;
    const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 16; ++k) bits |= (tx_space((w[k >> 2] >> (8 * (k & 3))) & 0xffu) ? 1u : 0u) << k;
    return bits | (tx_space(prev) ? 1u << 16 : 0u);
}

// token starts among the 16 bytes: not a space, and the byte before is one
__device__ __forceinline__ unsigned tx_start_bits(const unsigned char* __restrict__ text, int64_t off) {
    const uint4 q = *reinterpret_cast<const uint4*>(text + off);
    const unsigned prev = off > 0 ? (unsigned)text[off - 1] : 32u;
    const unsigned sp = tx_space_bits(q, prev);
    const unsigned before = ((sp << 1) & 0xfffeu) | (sp >> 16);  // space bit of each byte's predecessor
    return ~sp & before & 0xffffu;
}

__global__ void __launch_bounds__(kTxThreads) tx_count_kernel(int64_t ntiles, const unsigned char* __restrict__ text,
                                                              int32_t* __restrict__ cnt) {
    __shared__ int ws[kTxThreads / 32];
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t off = t * kTxTile + 16 * (int64_t)threadIdx.x;
        int c = __popc(tx_start_bits(text, off));
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

// tok[tile_off[t] + rank] = byte offset of each token start of tile t
__global__ void __launch_bounds__(kTxThreads) tx_starts_kernel(int64_t ntiles, const unsigned char* __restrict__ text,
                                                               const int32_t* __restrict__ tile_off,
                                                               int32_t* __restrict__ tok) {
    __shared__ int ws[kTxThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t off = t * kTxTile + 16 * (int64_t)threadIdx.x;
        unsigned bits = tx_start_bits(text, off);
        const int c = __popc(bits);
        int incl = c;  // inclusive warp scan
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) ws[wid] = incl;
        __syncthreads();
        int base = tile_off[t];
        for (int k = 0; k < wid; ++k) base += ws[k];
        int r = base + incl - c;
        while (bits) {
            const int k = __ffs(bits) - 1;
            bits &= bits - 1;
            tok[r++] = (int32_t)(off + k);
        }
        __syncthreads();
    }
}

// operator>>(int&) on a whole token: [+-]?[0-9]+ within int32; the text ends in a space, so the
// scan stops inside the buffer
__device__ __forceinline__ bool tx_int(const unsigned char* __restrict__ s, int32_t& out) {
    int k = 0;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
        neg = s[0] == '-';
        k = 1;
    }
    long long v = 0;
    int nd = 0;
    for (;; ++k) {
        const unsigned c = s[k];
        if (tx_space(c)) break;
        if (c < '0' || c > '9') return false;
        v = v * 10 + (long long)(c - '0');
        if (v > 2147483648ll) return false;
        ++nd;
    }
    if (nd == 0) return false;
    if (neg) v = -v;
    if (v > 2147483647ll) return false;
    out = (int32_t)v;
    return true;
}

// weight token: 0 = converted (value in out), 1 = valid but left to the host, 2 = not a number
// or a value <= 0.  Grammar (what libstdc++ collects for a double and strtod accepts whole):
// [+-]? (digits [. digits?] | . digits) ([eE] [+-]? digits)?
__device__ __forceinline__ int tx_weight(const unsigned char* __restrict__ s, double& out) {
    int k = 0;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
        neg = s[0] == '-';
        k = 1;
    }
    unsigned long long m = 0;
    int nsig = 0, nd = 0, dexp = 0;
    bool slow = false, point = false;
    for (;; ++k) {
        const unsigned c = s[k];
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
    if (s[k] == 'e' || s[k] == 'E') {
        ++k;
        bool eneg = false;
        if (s[k] == '+' || s[k] == '-') {
            eneg = s[k] == '-';
            ++k;
        }
        int ne = 0;
        for (;; ++k) {
            const unsigned c = s[k];
            if (c < '0' || c > '9') break;
            if (e < 100000) e = e * 10 + (int)(c - '0');
            ++ne;
        }
        if (ne == 0) return 2;
        if (eneg) e = -e;
    }
    if (!tx_space(s[k])) return 2;
    if (m == 0 || neg) return 2;  // zero (of any exponent) or negative: not > 0
    const int e10 = dexp + e;
    if (slow || m > (1ull << 53) || e10 < -22 || e10 > 22) return 1;
    // 10^a for a <= 22 is an exact double (5^22 < 2^53), so each partial product below is exact
    double p = 1.0;
    const int a = e10 < 0 ? -e10 : e10;
    for (int i = 0; i < a / 8; ++i) p *= 1e8;
    for (int i = 0; i < a % 8; ++i) p *= 10.0;
    out = e10 >= 0 ? __dmul_rn((double)m, p) : __ddiv_rn((double)m, p);
    return 0;
}

// one thread per triple; the token count comes from the scan (*ntok), so no host round trip
// sits between the passes
__global__ void tx_edges_kernel(const int32_t* __restrict__ ntok, const unsigned char* __restrict__ text,
                                const int32_t* __restrict__ tok, int32_t* __restrict__ src, int32_t* __restrict__ dst,
                                double* __restrict__ w, TxFind* find, int2* slow) {
    const int64_t nedges = *ntok / 3;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nedges; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ps = tok[3 * e], pd = tok[3 * e + 1], pw = tok[3 * e + 2];
        int32_t a = 0, b = 0;
        const bool ok = tx_int(text + ps, a) && tx_int(text + pd, b);
        if (!ok) atomicMin(&find->bad_id, (int32_t)e);
        src[e] = a;
        dst[e] = b;
        double x = 0.0;
        const int r = tx_weight(text + pw, x);
        if (r == 2) atomicMin(&find->bad_w, (int32_t)e);
        if (r == 1) {
            const int32_t k = atomicAdd(&find->nslow, 1);
            slow[k] = make_int2((int32_t)e, pw);  // at most one per triple: k < nedges
        }
        w[e] = x;
    }
}

// host-converted weights back into place
__global__ void tx_fix_kernel(int32_t count, const int32_t* __restrict__ idx, const double* __restrict__ val,
                              double* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        w[idx[i]] = val[i];
}

}  // namespace fbc
