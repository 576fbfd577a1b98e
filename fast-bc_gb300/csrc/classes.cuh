// Topological classes of the cluster vertices on the device -- VertexInfoPivotSelector::
// selectPivots (VertexInfoPivotSelector.h:30-123) for every cluster at once: two vertices of a
// cluster are in one class when their border vectors, lengths shifted by their minimum
// (VertexInfo::normalize, VertexInfo.h:269-278), are equal entry by entry (VertexInfo::compare,
// VertexInfo.h:553-569); classes are numbered in the order of their first member in the cluster
// list; a class's pivot is its non-border member of least BC (the first such in list order on
// ties), or its first member when every member is a border; its cardinality is its size.
//
// The reference compares every vertex with every class representative (O(n * classes * b));
// here each vertex's normalized vector is hashed, grouped through a per-cluster open-addressing
// table, and checked entry by entry against its class's first member (a hash collision between
// different vectors is reported, never merged).
#pragma once
#include <cstdint>

namespace fbc {

constexpr int kClsCollision = 1;  // two different vectors with one hash (reported)
constexpr int kClsFull = 2;       // a table probe ran past its table (sizing bug)
constexpr unsigned long long kClsEmpty = 0ull;
constexpr int kClsNone = 0x7f7f7f7f;  // "no position yet" (what a 0x7f byte fill leaves)

__device__ __forceinline__ unsigned long long cls_mix(unsigned long long h, unsigned long long x) {
    h ^= x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    h ^= h >> 31;
    h *= 0xbf58476d1ce4e5b9ull;
    h ^= h >> 29;
    return h;
}

// Per cluster vertex p (position in the concatenated cluster lists): the hash of its normalized
// border vector.  Entries of vertex i of cluster c: ent[c] + i * nb[c] + j.
struct ClsArgs {
    const int64_t* coff;   // ncl + 1
    const int64_t* boff;   // ncl + 1 (border counts per cluster)
    const int64_t* eoff;   // ncl + 1 (first border-vector entry of each cluster)
    const int64_t* toff;   // ncl + 1 (first table slot of each cluster; sizes powers of two)
    int ncl;
    int64_t nv;
    const double* bdist;
    const unsigned long long* bsig;
    unsigned long long* thash;  // table keys (kClsEmpty = free)
    int* tfirst;                // table: first member position
    unsigned long long* vhash;  // per position
    int* vrep;                  // per position: first member of its class
    int* err;
};

__device__ __forceinline__ void cls_vec(const ClsArgs& A, int64_t p, int& c, int64_t& e, int& b, double& mn) {
    c = seg_of(A.coff, A.ncl, p);
    b = (int)(A.boff[c + 1] - A.boff[c]);
    e = A.eoff[c] + (p - A.coff[c]) * (int64_t)b;
    mn = 0.0;
    for (int j = 0; j < b; ++j) {
        const double x = A.bdist[e + j];
        if (j == 0 || x < mn) mn = x;
    }
}

__global__ void cls_hash_kernel(ClsArgs A) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.nv; p += (int64_t)gridDim.x * blockDim.x) {
        int c, b;
        int64_t e;
        double mn;
        cls_vec(A, p, c, e, b, mn);
        unsigned long long h = 0x243f6a8885a308d3ull ^ (unsigned long long)b;
        for (int j = 0; j < b; ++j) {
            h = cls_mix(h, A.bsig[e + j]);
            h = cls_mix(h, (unsigned long long)__double_as_longlong(A.bdist[e + j] - mn));
        }
        h |= 1ull;  // never the empty key
        A.vhash[p] = h;
        // insert into the cluster's table; the slot keeps the least member position
        const int64_t t0 = A.toff[c], tn = A.toff[c + 1] - t0;
        int64_t s = (int64_t)(h & (unsigned long long)(tn - 1));
        bool placed = false;
        for (int64_t k = 0; k < tn; ++k) {
            const unsigned long long old = atomicCAS(A.thash + t0 + s, kClsEmpty, h);
            if (old == kClsEmpty || old == h) {
                atomicMin(A.tfirst + t0 + s, (int)p);
                placed = true;
                break;
            }
            s = (s + 1) & (tn - 1);
        }
        if (!placed) atomicOr(A.err, kClsFull);
    }
}

// each position's class representative (the table slot's first member), checked entry by entry
__global__ void cls_rep_kernel(ClsArgs A) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.nv; p += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long h = A.vhash[p];
        int c, b;
        int64_t e;
        double mn;
        cls_vec(A, p, c, e, b, mn);
        const int64_t t0 = A.toff[c], tn = A.toff[c + 1] - t0;
        int64_t s = (int64_t)(h & (unsigned long long)(tn - 1));
        int rep = -1;
        for (int64_t k = 0; k < tn; ++k) {
            if (A.thash[t0 + s] == h) {
                rep = A.tfirst[t0 + s];
                break;
            }
            s = (s + 1) & (tn - 1);
        }
        if (rep < 0) {
            atomicOr(A.err, kClsFull);
            A.vrep[p] = (int)p;
            continue;
        }
        A.vrep[p] = rep;
        if (rep != p) {
            int rc, rb;
            int64_t re;
            double rmn;
            cls_vec(A, rep, rc, re, rb, rmn);
            bool same = rc == c && rb == b;
            for (int j = 0; same && j < b; ++j)
                same = A.bsig[e + j] == A.bsig[re + j] && A.bdist[e + j] - mn == A.bdist[re + j] - rmn;
            if (!same) atomicOr(A.err, kClsCollision);
        }
    }
}

// flag[p] = 1 where p starts a class (clusters with borders only)
__global__ void cls_flag_kernel(ClsArgs A, int32_t* flag) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.nv; p += (int64_t)gridDim.x * blockDim.x) {
        const int c = seg_of(A.coff, A.ncl, p);
        flag[p] = (A.boff[c + 1] > A.boff[c] && A.vrep[p] == p) ? 1 : 0;
    }
}

// class sizes and the least BC among each class's non-border members
__global__ void cls_card_kernel(ClsArgs A, const int32_t* __restrict__ cls_of_first, const int32_t* __restrict__ cverts,
                                const uint8_t* __restrict__ isborder, const double* __restrict__ bc, int* card,
                                unsigned long long* minbc) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.nv; p += (int64_t)gridDim.x * blockDim.x) {
        const int c = seg_of(A.coff, A.ncl, p);
        if (A.boff[c + 1] == A.boff[c]) continue;
        const int k = cls_of_first[A.vrep[p]];
        atomicAdd(card + k, 1);
        // BC values are >= 0, so their bit patterns order as the values do
        if (!isborder[p]) atomicMin(minbc + k, (unsigned long long)__double_as_longlong(bc[cverts[p]]));
    }
}

// the first non-border member holding that least BC
__global__ void cls_pick_kernel(ClsArgs A, const int32_t* __restrict__ cls_of_first, const int32_t* __restrict__ cverts,
                                const uint8_t* __restrict__ isborder, const double* __restrict__ bc,
                                const unsigned long long* __restrict__ minbc, int* pick) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.nv; p += (int64_t)gridDim.x * blockDim.x) {
        const int c = seg_of(A.coff, A.ncl, p);
        if (A.boff[c + 1] == A.boff[c] || isborder[p]) continue;
        const int k = cls_of_first[A.vrep[p]];
        if ((unsigned long long)__double_as_longlong(bc[cverts[p]]) == minbc[k]) atomicMin(pick + k, (int)p);
    }
}

// per class: pivot vertex (the pick, else the first member) and cardinality
__global__ void cls_out_kernel(ClsArgs A, const int32_t* __restrict__ flag, const int32_t* __restrict__ cls_of_first,
                               const int32_t* __restrict__ cverts, const int* __restrict__ card,
                               const int* __restrict__ pick, int32_t* pivots, int32_t* cards) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.nv; p += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[p]) continue;
        const int k = cls_of_first[p];
        const int q = pick[k];
        pivots[k] = cverts[q != kClsNone ? q : p];
        cards[k] = card[k];
    }
}

// isborder[coff[c] + local id] = 1 for the (local) border ids of every cluster
__global__ void cls_mark_border_kernel(int64_t nb, const int64_t* __restrict__ boff, int ncl,
                                       const int64_t* __restrict__ coff, const int32_t* __restrict__ cbord,
                                       uint8_t* isborder) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nb; j += (int64_t)gridDim.x * blockDim.x) {
        const int c = seg_of(boff, ncl, j);
        isborder[coff[c] + cbord[j]] = 1;
    }
}

}  // namespace fbc
