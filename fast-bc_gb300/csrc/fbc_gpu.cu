// libfbcgpu: C ABI over the GB300 Brandes engine (declarations and contracts in
// include/fbc_gpu.h).  Host side: graph upload/validation, segment and unit planning,
// workspace sizing, launches on the library stream, result download, status mapping.
#include "fbc_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <numeric>
#include <string>
#include <system_error>
#include <thread>
#include <climits>
#include <clocale>
#include <cstdlib>
#include <locale.h>
#include <vector>

#include "cluster_build.cuh"
#include "classes.cuh"
#include "graph_build.cuh"
#include "text_parse.cuh"
#include "frontier_kernels.cuh"
#include "kmeans.cuh"
#include "host_order.hpp"

namespace {

using fbc::KParams;
using fbc::Seg;
using fbc::Unit;

thread_local std::string g_err;
std::recursive_mutex g_mu;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define FBC_CK(call)                                                                     \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            int code_ = (e_ == cudaErrorMemoryAllocation) ? FBC_ERR_OOM : FBC_ERR_CUDA;  \
            return fail(code_, std::string(#call) + ": " + cudaGetErrorString(e_));      \
        }                                                                                \
    } while (0)

#define FBC_TRY(expr)          \
    do {                       \
        int rc_ = (expr);      \
        if (rc_) return rc_;   \
    } while (0)

// Growable device buffer.
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    // zero: clear a new allocation on `zst`, the stream its first user runs on (a plain
    // cudaMemset would run on the legacy stream, unordered with a non-blocking stream)
    cudaError_t ensure(size_t bytes, bool zero = false, cudaStream_t zst = nullptr) {
        if (p && bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        if (zero) return cudaMemsetAsync(p, 0, want, zst);
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const {
        return (T*)p;
    }
};

struct Options {
    int64_t delta = 0;          // bucket width; 0 = 4 x mean edge weight of the graph
    int64_t block_threads = 256;    // plain schedule
    int64_t frontier_threads = 128; // batched schedule, large segments
    int64_t chunk_max = 512;        // batched small segments: sources per work item
    int64_t wide_n = 1 << 20;       // batched large segments: 512-thread blocks from this size
    int64_t warp_max_n = 4096;  // batched: segments up to this size run one source per warp
    int64_t iter_mult = 16;
    int64_t ws_budget_mb = 0;   // 0 = 60% of the free device memory
    int64_t group = 0;          // frontier kernel sources per block (1, 2, 4); 0 = automatic
    int64_t order_min_n = 65536;   // batched runs relabel graphs of at least this many vertices
    int64_t csr_device_min_m = 65536;  // edge lists of at least this many edges are built on the device
    int64_t wide_threads = 1024;       // block size of the wide frontier kernel (<= 1024)
    int64_t wide_kv = 1;               // level entries per lane of the 1024-thread form (1 or 2)
    int64_t adj4 = 1;                  // use the packed 4-byte adjacency where it exists
    int64_t bc_sweep = 1;              // one-segment, one-source-per-block launches add BC in the restore sweep
    int64_t pull_count = 1;            // count tight in-edges by pulling over reverse weights where they exist
    int64_t source_order = 1;          // batched sources of a relabelled graph run in its locality order
    int64_t debug_sched = FBC_SCHED_PLAIN;  // schedule used by fbc_sssp_debug
    int64_t scratch_keep_mb = 8192;  // per-call scratch the memory pool keeps for later calls
};

// A persistent workspace of equally sized slots.  Slot headers keep stamp counters, so a
// workspace is reused across calls as long as its geometry still fits.
struct Workspace {
    DBuf buf;
    int64_t stride = 0;
    int64_t slots = 0;
    int ws_n = -1;
    int dsize = 0;
};

struct Ctx {
    bool init = false;
    int dev = 0;
    int nsm = 0;
    int smem_optin = 0;
    cudaStream_t st = nullptr;
    cudaMemPool_t pool = nullptr;  // per-call scratch (TmpBuf), stream-ordered on st
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm = nullptr;
    Options opt;
    DBuf retry, segs, units_b, units_w, chunks, crp, cadj, cgid, cbord, bc, bdist, bsig, ctr, dbg, bcseg;
    // cluster extraction scratch: offsets, ids, flags, scans, given borders, error word
    DBuf c_off, c_id, c_lid, c_isb, c_flag, c_scan, c_sums, c_boff, c_bsrc, c_m, c_err;
    Workspace wsb, wsw;
};
Ctx g;

// Makes the library's device current for one entry point and gives the caller's back on return
// (OpenMP workers calling in start on device 0, and allocations and launches must land on the
// device of the library stream; a caller working on another device keeps it).
struct DevGuard {
    int prev = -1;
    void enter() {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != g.dev && cudaSetDevice(g.dev) == cudaSuccess) prev = cur;
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};


double now_ms() {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

}  // namespace

struct fbc_graph_s {
    int32_t n = 0;
    int64_t m = 0;
    int32_t maxw = 0;
    int32_t maxindeg = 0;
    double meanw = 1.0;
    int32_t* d_rp = nullptr;
    int2* d_adj = nullptr;
    // host copy of the CSR (bisection order, downloads, debug predecessor counts); a graph
    // built on the device fetches it on first use
    bool host_ok = true;
    std::vector<int64_t> h_rp;
    std::vector<int32_t> h_col;
    std::vector<int32_t> h_w;
    // locality order for the batched schedule, built on first use: the CSR relabelled by
    // recursive BFS bisection (ord_new: input id -> new id; d_ord_inv: new id -> input id)
    bool ord_built = false;
    int32_t* d_ord_rp = nullptr;
    int2* d_ord_adj = nullptr;
    uint32_t* d_ord_adj4 = nullptr;  // packed (destination | weight << 24) when n < 2^24, weights < 256
    uint8_t* d_ord_revw = nullptr;   // weight of each relabelled edge's reverse, when every edge has one
                                     // and weights are below 256
    int32_t* d_ord_inv = nullptr;
    std::vector<int32_t> ord_new;
};

struct fbc_plan_s {
    fbc_graph_s* G = nullptr;
    int prec = FBC_PREC_FP32C;
    int64_t n = 0, ent = 0;
    DBuf crp, cadj, cgid, cbord, segs, units, chunks, bc, bdist, bsig, ctr, retry, bunits, ws;
    double* h_bc = nullptr;
    double* h_bdist = nullptr;
    uint64_t* h_bsig = nullptr;
    int* h_ctl = nullptr;
    cudaGraph_t graph[2] = {nullptr, nullptr};  // resets + shared-memory kernel; frontier kernel + downloads
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    bool captured = false;
    double relax = 0, wbytes = 0, bbytes = 0;
    int64_t nunits = 0, wunits = 0, bunits_n = 0;
    int launches = 0;
    std::vector<int64_t> coff, boff;
    std::vector<int32_t> cverts, borders;
    // frees everything the plan holds, also when its creation stopped half way
    ~fbc_plan_s() {
        DevGuard dg_;
        if (g.init) {  // no launch in flight still uses a buffer
            dg_.enter();
            cudaStreamSynchronize(g.st);
        }
        for (int i = 0; i < 2; ++i) {
            if (exec[i]) cudaGraphExecDestroy(exec[i]);
            if (graph[i]) cudaGraphDestroy(graph[i]);
        }
        for (DBuf* b : {&crp, &cadj, &cgid, &cbord, &segs, &units, &chunks, &bc, &bdist, &bsig, &ctr, &retry,
                        &bunits, &ws})
            b->release();
        if (h_bc) cudaFreeHost(h_bc);
        if (h_bdist) cudaFreeHost(h_bdist);
        if (h_bsig) cudaFreeHost(h_bsig);
        if (h_ctl) cudaFreeHost(h_ctl);
    }
};

namespace {

// Every entry point: the library is initialised and its device is current.
int check_init(DevGuard& dg) {
    if (!g.init) return fail(FBC_ERR_NOT_INIT, "fbc_gpu_init has not been called");
    dg.enter();
    return FBC_OK;
}

// Validate a host CSR with double weights and build the device graph.
int make_graph(int32_t n, std::vector<int64_t>&& rp, std::vector<int32_t>&& col, const double* w,
               fbc_graph* out) {
    if (n < 0) return fail(FBC_ERR_INVALID_ARG, "vertex count must be >= 0");
    if (rp.size() != (size_t)n + 1 || rp[0] != 0) return fail(FBC_ERR_INVALID_ARG, "row_ptr[0] must be 0");
    const int64_t m = rp[n];
    if (m < 0 || m >= (int64_t)0x7fffffff) return fail(FBC_ERR_RANGE, "edge count outside [0, 2^31-1)");
    std::vector<int32_t> wi((size_t)m);
    int32_t maxw = 0;
    double sumw = 0;
    for (int32_t v = 0; v < n; ++v) {
        if (rp[v + 1] < rp[v]) return fail(FBC_ERR_INVALID_ARG, "row_ptr is not monotone");
        for (int64_t e = rp[v]; e < rp[v + 1]; ++e) {
            if (col[e] < 0 || col[e] >= n)
                return fail(FBC_ERR_INVALID_ARG,
                            "edge destination out of range at vertex " + std::to_string(v));
            if (e > rp[v] && col[e] <= col[e - 1])
                return fail(FBC_ERR_INVALID_ARG,
                            "CSR row not strictly ascending at vertex " + std::to_string(v));
            const double x = w[e];
            if (!(x > 0)) return fail(FBC_ERR_INVALID_ARG, "Edge weight must be greater than zero");
            if (x != std::floor(x) || x > 2147483647.0)
                return fail(FBC_ERR_RANGE, "edge weights must be integers below 2^31");
            wi[e] = (int32_t)x;
            maxw = std::max(maxw, wi[e]);
            sumw += x;
        }
    }
    if ((double)n * (double)maxw > 2147483646.0)
        return fail(FBC_ERR_RANGE, "n * max_weight exceeds the int32 distance range");
    std::vector<int32_t> indeg((size_t)std::max(n, 1), 0);
    for (int64_t e = 0; e < m; ++e) indeg[col[e]]++;
    auto* G = new fbc_graph_s();
    G->maxindeg = n ? *std::max_element(indeg.begin(), indeg.begin() + n) : 0;
    G->n = n;
    G->m = m;
    G->maxw = maxw;
    G->meanw = m ? sumw / (double)m : 1.0;
    std::vector<int32_t> rp32((size_t)n + 1);
    for (int32_t v = 0; v <= n; ++v) rp32[v] = (int32_t)rp[v];
    std::vector<int2> adj((size_t)std::max<int64_t>(m, 1));
    for (int64_t e = 0; e < m; ++e) adj[e] = make_int2(col[e], wi[e]);
    cudaError_t e1 = cudaMalloc(&G->d_rp, sizeof(int32_t) * ((size_t)n + 1));
    cudaError_t e2 = cudaMalloc(&G->d_adj, sizeof(int2) * adj.size());
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        if (e1 == cudaSuccess) cudaFree(G->d_rp);
        if (e2 == cudaSuccess) cudaFree(G->d_adj);
        delete G;
        return fail(FBC_ERR_OOM, "device allocation of the graph failed");
    }
    cudaError_t e3 = cudaMemcpyAsync(G->d_rp, rp32.data(), sizeof(int32_t) * rp32.size(),
                                     cudaMemcpyHostToDevice, g.st);
    cudaError_t e4 = cudaMemcpyAsync(G->d_adj, adj.data(), sizeof(int2) * adj.size(),
                                     cudaMemcpyHostToDevice, g.st);
    cudaError_t e5 = cudaStreamSynchronize(g.st);
    if (e3 != cudaSuccess || e4 != cudaSuccess || e5 != cudaSuccess) {
        cudaFree(G->d_rp);
        cudaFree(G->d_adj);
        delete G;
        return fail(FBC_ERR_CUDA, "graph upload failed");
    }
    G->h_rp = std::move(rp);
    G->h_col = std::move(col);
    G->h_w = std::move(wi);
    *out = G;
    return FBC_OK;
}

int delta_for(double meanw) {
    if (g.opt.delta > 0) return (int)std::min<int64_t>(g.opt.delta, 0x3fffffff);
    return std::max(1, (int)std::lround(4.0 * meanw));
}

// A batch of work: segments + units, output sizes and debug pointers.
struct Plan {
    std::vector<Seg> segs;
    std::vector<int64_t> seg_m;
    std::vector<int32_t> seg_maxw;
    std::vector<int32_t> seg_maxindeg;
    std::vector<Unit> units;
    int64_t bc_len = 0;
    int64_t border_entries = 0;
    int prec = FBC_PREC_FP64;
    int sched = FBC_SCHED_PLAIN;
    int32_t* dbg_dist = nullptr;
    unsigned long long* dbg_sig = nullptr;
    double* dbg_dlt = nullptr;
};

// The host copy of a device-built graph's CSR, downloaded once.
int ensure_host_csr(fbc_graph_s* G) {
    if (G->host_ok) return FBC_OK;
    const int32_t n = G->n;
    std::vector<int32_t> rp32((size_t)n + 1);
    std::vector<int2> adj((size_t)std::max<int64_t>(G->m, 1));
    FBC_CK(cudaMemcpyAsync(rp32.data(), G->d_rp, sizeof(int32_t) * rp32.size(), cudaMemcpyDeviceToHost, g.st));
    if (G->m > 0)
        FBC_CK(cudaMemcpyAsync(adj.data(), G->d_adj, sizeof(int2) * (size_t)G->m, cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    G->h_rp.assign(rp32.begin(), rp32.end());
    G->h_col.resize((size_t)G->m);
    G->h_w.resize((size_t)G->m);
    for (int64_t k = 0; k < G->m; ++k) {
        G->h_col[k] = adj[k].x;
        G->h_w[k] = adj[k].y;
    }
    G->host_ok = true;
    return FBC_OK;
}

// Build (once) the relabelled device CSR of a graph: rows ascending in the new ids.
int ensure_order(fbc_graph_s* G) {
    if (G->ord_built) return FBC_OK;
    FBC_TRY(ensure_host_csr(G));
    const int32_t n = G->n;
    std::vector<int32_t> nw = fbc_host::bisection_order(n, G->h_rp, G->h_col, 16);
    std::vector<int32_t> inv((size_t)std::max(n, 1));
    fbc_host::host_parallel(n, [&](int64_t lo, int64_t hi) {
        for (int64_t v = lo; v < hi; ++v) inv[nw[v]] = (int32_t)v;
    });
    // the relabelled rows: offsets by a scan of the degrees in the new order, then each row filled
    // and sorted by destination on its own
    std::vector<int32_t> rp32((size_t)n + 1, 0);
    for (int32_t u = 0; u < n; ++u) rp32[u + 1] = rp32[u] + (int32_t)(G->h_rp[inv[u] + 1] - G->h_rp[inv[u]]);
    std::vector<int2> adj((size_t)std::max<int64_t>(G->m, 1));
    fbc_host::host_parallel(n, [&](int64_t lo, int64_t hi) {
        for (int64_t u = lo; u < hi; ++u) {
            const int32_t v = inv[u];
            int64_t e = rp32[u];
            for (int64_t k = G->h_rp[v]; k < G->h_rp[v + 1]; ++k) adj[e++] = make_int2(nw[G->h_col[k]], G->h_w[k]);
            std::sort(adj.begin() + rp32[u], adj.begin() + e, [](const int2& a, const int2& c) { return a.x < c.x; });
        }
    });
    FBC_CK(cudaMalloc(&G->d_ord_rp, sizeof(int32_t) * rp32.size()));
    FBC_CK(cudaMalloc(&G->d_ord_adj, sizeof(int2) * adj.size()));
    FBC_CK(cudaMalloc(&G->d_ord_inv, sizeof(int32_t) * inv.size()));
    FBC_CK(cudaMemcpyAsync(G->d_ord_rp, rp32.data(), sizeof(int32_t) * rp32.size(), cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(G->d_ord_adj, adj.data(), sizeof(int2) * adj.size(), cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(G->d_ord_inv, inv.data(), sizeof(int32_t) * inv.size(), cudaMemcpyHostToDevice, g.st));
    std::vector<uint32_t> adj4;
    if (n < (1 << 24) && G->maxw < 256) {
        adj4.resize(adj.size());
        fbc_host::host_parallel((int64_t)adj.size(), [&](int64_t lo, int64_t hi) {
            for (int64_t k = lo; k < hi; ++k) adj4[k] = (uint32_t)adj[k].x | ((uint32_t)adj[k].y << 24);
        });
        FBC_CK(cudaMalloc(&G->d_ord_adj4, sizeof(uint32_t) * adj4.size()));
        FBC_CK(cudaMemcpyAsync(G->d_ord_adj4, adj4.data(), sizeof(uint32_t) * adj4.size(), cudaMemcpyHostToDevice,
                               g.st));
    }
    // reverse weights: edge u -> x gets the weight of x -> u (rows are sorted by destination);
    // a graph with an edge that has no reverse gets none
    std::vector<uint8_t> revw;
    if (n > 0 && G->maxw < 256) {
        revw.resize(adj.size());
        std::atomic<bool> sym{true};
        fbc_host::host_parallel(n, [&](int64_t lo, int64_t hi) {
            for (int64_t u = lo; u < hi && sym.load(std::memory_order_relaxed); ++u)
                for (int32_t k = rp32[u]; k < rp32[u + 1]; ++k) {
                    const int32_t x = adj[k].x;
                    const auto b = adj.begin() + rp32[x], en = adj.begin() + rp32[x + 1];
                    const auto it = std::lower_bound(b, en, (int32_t)u, [](const int2& a, int32_t v) { return a.x < v; });
                    if (it == en || it->x != (int32_t)u) {
                        sym.store(false, std::memory_order_relaxed);
                        return;
                    }
                    revw[(size_t)k] = (uint8_t)it->y;
                }
        });
        if (sym.load()) {
            FBC_CK(cudaMalloc(&G->d_ord_revw, revw.size()));
            FBC_CK(cudaMemcpyAsync(G->d_ord_revw, revw.data(), revw.size(), cudaMemcpyHostToDevice, g.st));
        }
    }
    FBC_CK(cudaStreamSynchronize(g.st));
    G->ord_new = std::move(nw);
    G->ord_built = true;
    return FBC_OK;
}

Seg whole_graph_seg(const fbc_graph_s* G, int64_t out_base) {
    Seg s{};
    s.rp = G->d_rp;
    s.adj = G->d_adj;
    s.gid = nullptr;
    s.border = nullptr;
    s.out_base = out_base;
    s.n = G->n;
    s.nb = 0;
    s.delta = delta_for(G->meanw);
    return s;
}

KParams base_params(const Plan& P) {
    KParams K{};
    K.segs = g.segs.as<Seg>();
    K.bc = g.bc.as<double>();
    K.bdist = g.bdist.as<double>();
    K.bsig = g.bsig.as<unsigned long long>();
    K.err = (int*)(g.ctr.as<unsigned long long>() + 2);
    K.retry_count = K.err + 1;
    K.retry = g.retry.as<fbc::RetryRec>();
    K.retry_cap = (int32_t)(g.retry.cap / sizeof(fbc::RetryRec));
    K.iter_mult = (int32_t)g.opt.iter_mult;
    K.dbg_dist = P.dbg_dist;
    K.dbg_sig = P.dbg_sig;
    K.dbg_dlt = P.dbg_dlt;
    return K;
}

// (Re)size a workspace for `slots` slots of at least `ws_n` vertices; reuse it when it
// already fits (then the existing, possibly larger, capacity and stride are used).
int ensure_ws(Workspace& W, int64_t slots, int64_t stride, int ws_n, int dsize) {
    if (W.buf.p && W.ws_n >= ws_n && W.dsize == dsize && W.slots >= slots) return FBC_OK;
    W.buf.release();
    FBC_CK(W.buf.ensure((size_t)(slots * stride), true, g.st));
    W.stride = stride;
    W.slots = slots;
    W.ws_n = ws_n;
    W.dsize = dsize;
    return FBC_OK;
}

int64_t ws_budget() {
    size_t freeb = 0, totalb = 0;
    if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) return (int64_t)1 << 30;
    int64_t b = g.opt.ws_budget_mb > 0 ? g.opt.ws_budget_mb * (int64_t)1048576
                                        : (int64_t)((double)freeb * 0.6);
    return b + (int64_t)g.wsb.buf.cap + (int64_t)g.wsw.buf.cap;
}

using KernFn = void (*)(fbc::KParams);

template <class Prec>
KernFn frontier_variant(bool wide, int K, int threads, bool a4) {
    if (a4 && wide && K == 1) {  // one source per block on a packed adjacency
        if (threads > 512) return g.opt.wide_kv == 1 ? fbc::frontier_kernel<Prec, 3, 1, true>
                                                     : fbc::frontier_kernel<Prec, 2, 1, true>;
        return fbc::frontier_kernel<Prec, 1, 1, true>;
    }
    if (wide && threads > 512 && g.opt.wide_kv == 1) {
        if (K == 4) return fbc::frontier_kernel<Prec, 3, 4>;
        if (K == 2) return fbc::frontier_kernel<Prec, 3, 2>;
        return fbc::frontier_kernel<Prec, 3, 1>;
    }
    if (wide && threads > 512) {
        if (K == 4) return fbc::frontier_kernel<Prec, 2, 4>;
        if (K == 2) return fbc::frontier_kernel<Prec, 2, 2>;
        return fbc::frontier_kernel<Prec, 2, 1>;
    }
    if (wide) {
        if (K == 4) return fbc::frontier_kernel<Prec, 1, 4>;
        if (K == 2) return fbc::frontier_kernel<Prec, 1, 2>;
        return fbc::frontier_kernel<Prec, 1, 1>;
    }
    if (K == 4) return fbc::frontier_kernel<Prec, 0, 4>;
    if (K == 2) return fbc::frontier_kernel<Prec, 0, 2>;
    return fbc::frontier_kernel<Prec, 0, 1>;
}

// Units of each segment in groups of K (a segment's last group padded with src = -1).
std::vector<Unit> group_units(const std::vector<Unit>& units, int K) {
    std::vector<Unit> out;
    out.reserve(units.size() + (size_t)K * 8);
    for (size_t i = 0; i < units.size();) {
        size_t j = i;
        while (j < units.size() && units[j].seg == units[i].seg) out.push_back(units[j++]);
        while (out.size() % (size_t)K) out.push_back(Unit{units[i].seg, -1, 0.0, -1});
        i = j;
    }
    return out;
}

// Launch configuration of a block-per-source launch with global-memory slots.  Plain schedule:
// brandes_block_kernel; batched schedule: frontier_kernel, K sources of one segment per block.
struct BlockCfg {
    KernFn kern = nullptr;
    bool fr = false;           // frontier kernel (else the plain block kernel)
    int K = 1, threads = 0;
    int64_t stride = 0, slots = 0;
    int32_t cnt_bits = 8;
    std::vector<Unit> units;   // grouped by K (K > 1: each segment's last group padded)
};

template <class Prec>
int block_config(const Plan& P, const std::vector<Unit>& units_in, int ws_n, bool force_plain, bool sig_f64,
                 int64_t budget, BlockCfg& c) {
    const bool fr = P.sched == FBC_SCHED_BATCHED && !force_plain && !sig_f64;
    // wide blocks for segments of millions of vertices (their frontiers are hundreds wide)
    const bool wide = fr && (g.opt.frontier_threads > 128 || (int64_t)ws_n >= g.opt.wide_n);
    int threads = (int)std::min<int64_t>(std::max<int64_t>(fr ? g.opt.frontier_threads : g.opt.block_threads, 32),
                                         fr ? 128 : 1024);
    if (wide) threads = (int)g.opt.wide_threads;
    threads = (threads / 32) * 32;
    // units sorted so that each segment's units are adjacent (the caller sorts by size)
    std::vector<Unit> sorted(units_in);
    std::stable_sort(sorted.begin(), sorted.end(), [&](const Unit& a, const Unit& b) {
        const int na = P.segs[a.seg].n, nb = P.segs[b.seg].n;
        return na != nb ? na > nb : a.seg < b.seg;
    });
    c = BlockCfg{};
    c.fr = fr;
    c.threads = threads;
    if (fr) {
        // sources per block (option "group" forces one): sharing rounds and levels pays where
        // a source's frontier is much narrower than the block -- segments of up to 32K
        // vertices (Louvain clusters: 4 per block measured 1.26x one per block); whole
        // graphs of 64K+ vertices measured faster one per block.  K > 1 also needs a group
        // for every block slot.
        const int forced = (int)g.opt.group;
        const int cand[3] = {4, 2, 1};
        bool a4 = true;  // every segment of the launch has the packed adjacency
        for (const Unit& u : sorted) a4 = a4 && P.segs[u.seg].adj4 != nullptr;
        for (int K : cand) {
            if (forced > 0 ? K != forced : (K > 1 && ws_n > 32768)) continue;
            if ((int64_t)ws_n * K >= ((int64_t)1 << 31) - 1) continue;
            KernFn f = frontier_variant<Prec>(wide, K, threads, a4);
            int b = 0;
            FBC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, threads, 0));
            const int64_t full = (int64_t)g.nsm * std::max(b, 1);  // units resident at once
            const int64_t sb = fbc::fstate_bytes<Prec>((int64_t)ws_n * K);
            const int64_t strd = 256 + ((sb + 255) & ~int64_t(255));
            std::vector<Unit> gu = K > 1 ? group_units(sorted, K) : sorted;
            const int64_t groups = (int64_t)gu.size() / K;
            const int64_t sl = std::max<int64_t>(1, std::min<int64_t>(std::min(full, groups), budget / strd));
            const bool ok = K == 1 || forced > 0 || (groups >= full && sl >= full);
            if (!ok) continue;
            c.kern = f;
            c.K = K;
            c.stride = strd;
            c.slots = sl;
            c.units.swap(gu);
            break;
        }
        // 8-bit counters (path counts up to 2^56) when no vertex of the launch's segments has
        // 255 or more in-edges, else 16-bit (the host keeps segments of 65,535+ off this kernel)
        int32_t maxin = 0;
        for (const Unit& u : c.units) maxin = std::max(maxin, P.seg_maxindeg[u.seg]);
        c.cnt_bits = maxin < 255 ? 8 : 16;
    } else {
        const int64_t sb = fbc::state_bytes<Prec>(ws_n);
        c.stride = 256 + ((sb + 255) & ~int64_t(255));
        c.kern = sig_f64 ? fbc::brandes_block_kernel<Prec, true> : fbc::brandes_block_kernel<Prec>;
        int bps = 1;
        FBC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, c.kern, threads, 0));
        bps = std::max(bps, 1);
        c.slots = std::min<int64_t>((int64_t)g.nsm * bps, (int64_t)sorted.size());
        c.slots = std::max<int64_t>(1, std::min<int64_t>(c.slots, budget / c.stride));
        c.units.swap(sorted);
    }
    if (!c.kern) return fail(FBC_ERR_INVALID_ARG, "no frontier kernel variant fits this segment");
    return FBC_OK;
}

// The launch of a block configuration: one block per slot.
cudaError_t launch_units(const BlockCfg& c, const KParams& K, cudaStream_t st) {
    c.kern<<<(unsigned)c.slots, c.threads, 0, st>>>(K);
    return cudaGetLastError();
}

// Block-per-source launch on the library's workspace.
template <class Prec>
int launch_block(const Plan& P, const std::vector<Unit>& units_in, int ws_n, fbc_stats* st,
                 int& launches, bool force_plain = false, bool sig_f64 = false) {
    if (units_in.empty()) return FBC_OK;
    BlockCfg c;
    FBC_TRY(block_config<Prec>(P, units_in, ws_n, force_plain, sig_f64, ws_budget(), c));
    // the two kernels keep different between-unit invariants: never share a workspace
    Workspace& W = c.fr ? g.wsw : g.wsb;
    FBC_TRY(ensure_ws(W, c.slots, c.stride, ws_n * c.K, (int)sizeof(typename Prec::D)));
    FBC_CK(g.units_b.ensure(sizeof(Unit) * c.units.size()));
    FBC_CK(cudaMemcpyAsync(g.units_b.p, c.units.data(), sizeof(Unit) * c.units.size(),
                           cudaMemcpyHostToDevice, g.st));
    if (st) st->h2d_bytes += (int64_t)(sizeof(Unit) * c.units.size());
    KParams K = base_params(P);
    K.units = g.units_b.as<Unit>();
    K.nunits = (int64_t)c.units.size() / c.K;
    if (c.fr) K.cnt_bits = c.cnt_bits;
    K.next_unit = g.ctr.as<unsigned long long>() + 0;
    K.ws = W.buf.as<char>();
    K.ws_stride = W.stride;
    K.ws_n = (int32_t)W.ws_n;  // block kernel: vertices; frontier kernel: entries (v*K + k)
    // one source per block, one segment: the restore sweep accumulates BC in the segment's order,
    // coalesced (directly into bc without a map; through a segment-order buffer and one scatter
    // afterwards with one), instead of a scattered reduction per vertex in the dependency pass
    const Seg* one = nullptr;
    if (c.fr && c.K == 1 && g.opt.bc_sweep) {
        one = &P.segs[c.units[0].seg];
        for (const Unit& u : c.units)
            if (u.seg != c.units[0].seg) { one = nullptr; break; }
    }
    if (one) {
        if (one->gid) {
            FBC_CK(g.bcseg.ensure(sizeof(double) * (size_t)one->n));
            FBC_CK(cudaMemsetAsync(g.bcseg.p, 0, sizeof(double) * (size_t)one->n, g.st));
            K.bc_seg = g.bcseg.as<double>();
        } else {
            K.bc_seg = K.bc + one->out_base;
        }
    }
    FBC_CK(launch_units(c, K, g.st));
    if (one && one->gid) {
        const unsigned gb = (unsigned)std::max<int64_t>(1, std::min<int64_t>((one->n + 255) / 256, 8192));
        fbc::add_seg_kernel<<<gb, 256, 0, g.st>>>(K.bc_seg, one->gid, one->out_base, one->n, K.bc);
        FBC_CK(cudaGetLastError());
        ++launches;
    }
    ++launches;
    if (st) {
        st->slots = (int32_t)c.slots;
        st->group = c.K;
    }
    return FBC_OK;
}

// Batched schedule, small segments: (segment, chunk of sources) items, CSR and state in
// shared memory.  `units` are grouped by segment.
int64_t small_dyn_smem() { return (int64_t)g.smem_optin - 64; }

bool small_fits(int nmax, int mmax, int warps) {
    const fbc::SmallLayout L(nmax, mmax);
    return L.pool + warps * fbc::SmallLayout::per_warp(nmax) <= small_dyn_smem();
}

// Host side of a small-segment launch: warps per block, dynamic shared memory, the
// (segment, chunk) work items (units grouped by segment, biggest segments first) and the grid.
struct SmallCfg {
    int wpb = 0;
    int64_t dyn = 0;
    int64_t blocks = 0;
    std::vector<fbc::Chunk> chunks;
};

int small_config(const Plan& P, const std::vector<Unit>& units, int nmax, int mmax, int nmin, SmallCfg& c) {
    const fbc::SmallLayout L(nmax, mmax);
    c.dyn = small_dyn_smem();
    if (!small_fits(nmax, mmax, 1)) return fail(FBC_ERR_INVALID_ARG, "small-segment kernel does not fit");
    c.wpb = (int)std::max<int64_t>(
        1, std::min<int64_t>(16, (c.dyn - L.pool) / fbc::SmallLayout::per_warp(std::max(nmin, 1))));
    // large chunks keep the block's warps busy between the barriers that reload the CSR;
    // about two chunks per block still balance the blocks
    const int64_t per_chunk = std::max<int64_t>(
        4 * c.wpb, std::min<int64_t>(g.opt.chunk_max, (int64_t)units.size() / std::max<int64_t>(1, (int64_t)g.nsm * 2)));
    c.chunks.clear();
    for (size_t i = 0; i < units.size();) {
        size_t j = i;
        while (j < units.size() && units[j].seg == units[i].seg && (int64_t)(j - i) < per_chunk) ++j;
        c.chunks.push_back(fbc::Chunk{units[i].seg, (int32_t)i, (int32_t)(j - i), 0});
        i = j;
    }
    std::stable_sort(c.chunks.begin(), c.chunks.end(), [&](const fbc::Chunk& a, const fbc::Chunk& b) {
        return P.segs[a.seg].n > P.segs[b.seg].n;
    });
    c.blocks = std::min<int64_t>((int64_t)g.nsm, (int64_t)c.chunks.size());
    return FBC_OK;
}

template <class Prec>
int small_launch(const SmallCfg& c, const fbc::SmallParams& S) {
    auto kern = fbc::small_seg_kernel<Prec>;
    FBC_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.dyn));
    kern<<<(unsigned)c.blocks, 32 * c.wpb, (size_t)c.dyn, g.st>>>(S);
    FBC_CK(cudaGetLastError());
    return FBC_OK;
}

template <class Prec>
int launch_small(const Plan& P, const std::vector<Unit>& units, int nmax, int mmax, int nmin,
                 fbc_stats* st, int& launches) {
    if (units.empty()) return FBC_OK;
    SmallCfg c;
    FBC_TRY(small_config(P, units, nmax, mmax, nmin, c));
    FBC_CK(g.units_w.ensure(sizeof(Unit) * units.size()));
    FBC_CK(cudaMemcpyAsync(g.units_w.p, units.data(), sizeof(Unit) * units.size(),
                           cudaMemcpyHostToDevice, g.st));
    FBC_CK(g.chunks.ensure(sizeof(fbc::Chunk) * c.chunks.size()));
    FBC_CK(cudaMemcpyAsync(g.chunks.p, c.chunks.data(), sizeof(fbc::Chunk) * c.chunks.size(),
                           cudaMemcpyHostToDevice, g.st));
    if (st) st->h2d_bytes += (int64_t)(sizeof(Unit) * units.size() + sizeof(fbc::Chunk) * c.chunks.size());
    fbc::SmallParams S{};
    S.k = base_params(P);
    S.k.units = g.units_w.as<Unit>();
    S.k.nunits = (int64_t)units.size();
    S.chunks = g.chunks.as<fbc::Chunk>();
    S.nchunks = (int32_t)c.chunks.size();
    S.nmax = nmax;
    S.mmax = mmax;
    S.smem = (int32_t)c.dyn;
    S.next_chunk = g.ctr.as<unsigned long long>() + 1;
    FBC_TRY(small_launch<Prec>(c, S));
    ++launches;
    return FBC_OK;
}

int map_err(int e) {
    if (e & fbc::kErrQueue) return fail(FBC_ERR_QUEUE, "device work queue overflow");
    if (e & fbc::kErrIter) return fail(FBC_ERR_ITER_LIMIT, "a device loop reached its iteration bound");
    if (e & fbc::kErrSigma) return fail(FBC_ERR_SIGMA_OVERFLOW, "a shortest-path count exceeded 2^64-1");
    return FBC_OK;
}

// Upload the plan, launch, wait, and check the device status.  Results stay on the device
// (g.bc, g.bdist, g.bsig) for the caller to download.
template <class Prec>
int run_plan_t(Plan& P, fbc_stats* st) {
    FBC_CK(g.bc.ensure(sizeof(double) * std::max<int64_t>(P.bc_len, 1)));
    FBC_CK(cudaMemsetAsync(g.bc.p, 0, sizeof(double) * std::max<int64_t>(P.bc_len, 1), g.st));
    FBC_CK(g.bdist.ensure(sizeof(double) * std::max<int64_t>(P.border_entries, 1)));
    FBC_CK(g.bsig.ensure(sizeof(uint64_t) * std::max<int64_t>(P.border_entries, 1)));
    FBC_CK(g.ctr.ensure(64));
    FBC_CK(cudaMemsetAsync(g.ctr.p, 0, 64, g.st));
    if (st) st->h2d_bytes += (int64_t)(sizeof(Seg) * P.segs.size());

    // split units by schedule.  Batched: segments that fit the shared-memory kernel run
    // there (grouped by segment); the rest run block-per-source, biggest segments first.
    std::vector<Unit> ub, uw;
    int nb_max = 0, nw_max = 0, mw_max = 0;
    std::vector<char> small(P.segs.size(), 0);
    if (P.sched == FBC_SCHED_BATCHED && !P.dbg_dist) {  // debug dumps come from block kernels
        for (size_t s = 0; s < P.segs.size(); ++s) {
            const int n = P.segs[s].n;
            small[s] = n <= std::min<int64_t>(g.opt.warp_max_n, 65535) && P.seg_maxw[s] < 65536 &&
                       P.seg_m[s] < ((int64_t)1 << 30);
        }
    }
    // the shared-memory layout is sized by the largest small segment: demote the largest
    // ones until at least two warps fit
    for (;;) {
        int nm = 0, mm = 0, arg = -1;
        for (size_t s = 0; s < P.segs.size(); ++s)
            if (small[s]) {
                mm = std::max<int>(mm, (int)P.seg_m[s]);
                if (P.segs[s].n >= nm) { nm = P.segs[s].n; arg = (int)s; }
            }
        if (arg < 0 || small_fits(nm, mm, 2)) break;
        small[arg] = 0;
    }
    int nw_min = 1 << 30;
    std::vector<std::vector<Unit>> by_seg(P.segs.size());
    for (const Unit& u : P.units) {
        if (small[u.seg]) {
            by_seg[u.seg].push_back(u);
            nw_max = std::max(nw_max, P.segs[u.seg].n);
            nw_min = std::min(nw_min, P.segs[u.seg].n);
            mw_max = std::max<int>(mw_max, (int)P.seg_m[u.seg]);
        } else {
            ub.push_back(u);
            nb_max = std::max(nb_max, P.segs[u.seg].n);
        }
    }
    for (auto& v : by_seg) uw.insert(uw.end(), v.begin(), v.end());
    std::stable_sort(ub.begin(), ub.end(), [&](const Unit& a, const Unit& b) {
        return P.segs[a.seg].n > P.segs[b.seg].n;
    });
    // the batched block kernel keeps tight in-edge counts in at most 16 bits
    if (P.sched == FBC_SCHED_BATCHED)
        for (const Unit& u : ub)
            if (P.seg_maxindeg[u.seg] >= 65535) {
                P.sched = FBC_SCHED_PLAIN;
                break;
            }
    FBC_CK(g.segs.ensure(sizeof(Seg) * std::max<size_t>(P.segs.size(), 1)));
    FBC_CK(cudaMemcpyAsync(g.segs.p, P.segs.data(), sizeof(Seg) * P.segs.size(),
                           cudaMemcpyHostToDevice, g.st));
    int launches = 0;
    FBC_CK(cudaEventRecord(g.ev0, g.st));
    FBC_CK(g.retry.ensure(sizeof(fbc::RetryRec) * std::max<size_t>(P.units.size(), 1)));
    FBC_TRY(launch_small<Prec>(P, uw, nw_max, mw_max, nw_min, st, launches));
    FBC_CK(cudaEventRecord(g.evm, g.st));
    {
        // batched: segments of up to 32K vertices run in a launch of their own (where several
        // sources share a block, their rounds and levels), the larger ones one source per block
        std::vector<Unit> us_small, us_large;
        int ns_max = 0, nl_max = 0;
        if (P.sched == FBC_SCHED_BATCHED && !P.dbg_dist)
            for (const Unit& u : ub) {
                const int sn = P.segs[u.seg].n;
                if (sn <= 32768) { us_small.push_back(u); ns_max = std::max(ns_max, sn); }
                else { us_large.push_back(u); nl_max = std::max(nl_max, sn); }
            }
        if (!us_small.empty() && !us_large.empty()) {
            // the launch with the larger slot layout first, so that the second reuses it
            const bool small_first = (int64_t)ns_max * 4 >= (int64_t)nl_max;
            FBC_TRY(launch_block<Prec>(P, small_first ? us_small : us_large, small_first ? ns_max : nl_max, st, launches));
            FBC_CK(cudaMemsetAsync(g.ctr.p, 0, 8, g.st));  // the unit counter of the next launch
            FBC_TRY(launch_block<Prec>(P, small_first ? us_large : us_small, small_first ? nl_max : ns_max, st, launches));
        } else {
            FBC_TRY(launch_block<Prec>(P, ub, nb_max, st, launches));
        }
    }
    int err[2] = {0, 0};
    FBC_CK(cudaMemcpyAsync(err, (char*)g.ctr.p + 16, 2 * sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    // Units whose path counts outgrew their kernel's representation stopped before their
    // dependency pass (nothing of theirs was accumulated): recompute them one level up,
    // 48-bit packed -> 64-bit (plain kernel) -> FP64 counts (plain kernel).
    for (int round = 0; round < 3 && err[0] == 0 && err[1] > 0; ++round) {
        std::vector<fbc::RetryRec> rec((size_t)err[1]);
        if (st) st->retries += err[1];
        FBC_CK(cudaMemcpy(rec.data(), g.retry.p, sizeof(fbc::RetryRec) * rec.size(), cudaMemcpyDeviceToHost));
        std::vector<Unit> to64, tof64;
        int nmax = 0;
        for (const auto& r : rec) {
            (r.code == fbc::kErrRetry ? to64 : tof64).push_back(r.u);
            nmax = std::max(nmax, P.segs[r.u.seg].n);
        }
        FBC_CK(cudaMemsetAsync(g.ctr.p, 0, 8, g.st));
        FBC_CK(cudaMemsetAsync((char*)g.ctr.p + 20, 0, 4, g.st));
        FBC_TRY(launch_block<Prec>(P, to64, nmax, st, launches, true, false));
        if (!to64.empty() && !tof64.empty()) {
            FBC_CK(cudaMemsetAsync(g.ctr.p, 0, 8, g.st));
        }
        FBC_TRY(launch_block<Prec>(P, tof64, nmax, st, launches, true, true));
        FBC_CK(cudaMemcpyAsync(err, (char*)g.ctr.p + 16, 2 * sizeof(int), cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
    }
    if (err[0] == 0 && err[1] > 0) err[0] = fbc::kErrSigma;
    FBC_CK(cudaEventRecord(g.ev1, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    int errv = err[0];
    if (st) {
        float ms = 0.f, mw = 0.f, mb = 0.f;
        FBC_CK(cudaEventElapsedTime(&ms, g.ev0, g.ev1));
        FBC_CK(cudaEventElapsedTime(&mw, g.ev0, g.evm));
        FBC_CK(cudaEventElapsedTime(&mb, g.evm, g.ev1));
        st->kernel_ms += ms;
        st->warp_ms += uw.empty() ? 0.0 : mw;
        st->block_ms += ub.empty() ? 0.0 : mb;
        st->warp_units += (int64_t)uw.size();
        st->block_units += (int64_t)ub.size();
        for (const Unit& u : uw) st->warp_bytes += 40.0 * (double)P.seg_m[u.seg] + 52.0 * P.segs[u.seg].n;
        for (const Unit& u : ub) st->block_bytes += 40.0 * (double)P.seg_m[u.seg] + 52.0 * P.segs[u.seg].n;
        st->units += (int64_t)P.units.size();
        double rel = 0;
        for (const Unit& u : P.units) rel += (double)P.seg_m[u.seg];
        st->relaxations += rel;
        st->launches += launches;
    }
    return map_err(errv);
}

int run_plan(Plan& P, fbc_stats* st) {
    if (P.prec == FBC_PREC_FP32C) return run_plan_t<fbc::PrecDF32>(P, st);
    if (P.prec == FBC_PREC_FP64) return run_plan_t<fbc::PrecF64>(P, st);
    return fail(FBC_ERR_INVALID_ARG, "unknown precision");
}

int check_sched(int sched) {
    if (sched != FBC_SCHED_PLAIN && sched != FBC_SCHED_BATCHED)
        return fail(FBC_ERR_INVALID_ARG, "unknown schedule");
    return FBC_OK;
}

int download_bc(double* out, int64_t len, bool accumulate, fbc_stats* st) {
    if (!out || len <= 0) return FBC_OK;
    std::vector<double> tmp;
    double* dst = out;
    if (accumulate) {
        tmp.resize((size_t)len);
        dst = tmp.data();
    }
    FBC_CK(cudaMemcpyAsync(dst, g.bc.p, sizeof(double) * (size_t)len, cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    if (st) st->d2h_bytes += (int64_t)(sizeof(double) * (size_t)len);
    if (accumulate)
        for (int64_t i = 0; i < len; ++i) out[i] += tmp[(size_t)i];
    return FBC_OK;
}

// Border vertices of each cluster: a member with an in- or out-edge crossing the cluster
// (SubGraph.h:70-135), ascending global id (the std::set order of SubGraph::borders).
// kernels launched by the cluster-build helpers since the counter was last read
int g_aux_launches = 0;

unsigned grid_for(int64_t items, int threads = 256) {
    ++g_aux_launches;  // every caller launches one kernel with the returned grid
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((items + threads - 1) / threads, (int64_t)g.nsm * 16));
}

// Exclusive scan of `len` int32 values on the library stream: out[0 .. len] (len + 1 entries).
int device_scan(const int32_t* in, int64_t len, int32_t* out) {
    if (len <= 0) {
        FBC_CK(cudaMemsetAsync(out, 0, sizeof(int32_t), g.st));
        return FBC_OK;
    }
    const int64_t nb = (len + fbc::kScanBlock - 1) / fbc::kScanBlock;
    g_aux_launches += 3;
    FBC_CK(g.c_sums.ensure(sizeof(int32_t) * (size_t)nb));
    int32_t* sums = g.c_sums.as<int32_t>();
    fbc::scan_sums_kernel<<<(unsigned)nb, fbc::kScanBlock, 0, g.st>>>(in, len, sums);
    fbc::scan_top_kernel<<<1, fbc::kScanBlock, 0, g.st>>>(sums, nb);
    fbc::scan_apply_kernel<<<(unsigned)nb, fbc::kScanBlock, 0, g.st>>>(in, len, sums, out);
    FBC_CK(cudaGetLastError());
    return FBC_OK;
}

int check_cluster_offsets(const fbc_graph_s* G, int32_t nclusters, const int64_t* coff, const int32_t* cverts) {
    if (nclusters < 0 || !coff || (nclusters > 0 && !cverts))
        return fail(FBC_ERR_INVALID_ARG, "bad cluster arrays");
    if (coff[0] != 0) return fail(FBC_ERR_INVALID_ARG, "cluster_off[0] must be 0");
    for (int32_t c = 0; c < nclusters; ++c)
        if (coff[c + 1] < coff[c]) return fail(FBC_ERR_INVALID_ARG, "cluster_off is not monotone");
    if (coff[nclusters] > (int64_t)G->n) return fail(FBC_ERR_INVALID_ARG, "vertex listed in two clusters or twice");
    return FBC_OK;
}

int cluster_error(int e) {
    if (e & fbc::kCluRange) return fail(FBC_ERR_INVALID_ARG, "cluster vertex id out of range");
    if (e & fbc::kCluDup) return fail(FBC_ERR_INVALID_ARG, "vertex listed in two clusters or twice");
    if (e & fbc::kCluBorder) return fail(FBC_ERR_INVALID_ARG, "border vertex not in its cluster");
    return FBC_OK;
}

// Cluster ids on the device (g.c_id, g.c_lid; g.cgid holds the cluster vertex lists), the
// offsets in g.c_off; the error word is cleared.
int device_cluster_ids(const fbc_graph_s* G, int32_t nclusters, const int64_t* coff, const int32_t* cverts,
                       fbc_stats* st) {
    FBC_TRY(check_cluster_offsets(G, nclusters, coff, cverts));
    const int64_t nv = coff[nclusters];
    const int32_t n = G->n;
    FBC_CK(g.c_off.ensure(sizeof(int64_t) * ((size_t)nclusters + 1)));
    FBC_CK(g.cgid.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nv, 1)));
    FBC_CK(g.c_id.ensure(sizeof(int32_t) * (size_t)std::max(n, 1)));
    FBC_CK(g.c_lid.ensure(sizeof(int32_t) * (size_t)std::max(n, 1)));
    FBC_CK(g.c_err.ensure(64));
    FBC_CK(cudaMemcpyAsync(g.c_off.p, coff, sizeof(int64_t) * ((size_t)nclusters + 1), cudaMemcpyHostToDevice, g.st));
    if (nv > 0)
        FBC_CK(cudaMemcpyAsync(g.cgid.p, cverts, sizeof(int32_t) * (size_t)nv, cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemsetAsync(g.c_id.p, 0xff, sizeof(int32_t) * (size_t)std::max(n, 1), g.st));
    FBC_CK(cudaMemsetAsync(g.c_err.p, 0, 64, g.st));
    if (st) st->h2d_bytes += (int64_t)(sizeof(int64_t) * ((size_t)nclusters + 1) + sizeof(int32_t) * (size_t)nv);
    if (nv > 0) {
        fbc::clu_ids_kernel<<<grid_for(nv), 256, 0, g.st>>>(nv, g.c_off.as<int64_t>(), nclusters, g.cgid.as<int32_t>(),
                                                            n, g.c_id.as<int32_t>(), g.c_lid.as<int32_t>(),
                                                            g.c_err.as<int>());
        FBC_CK(cudaGetLastError());
        // every later kernel indexes rows by these ids: stop here on a bad list
        int err = 0;
        FBC_CK(cudaMemcpyAsync(&err, g.c_err.p, sizeof(int), cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
        FBC_TRY(cluster_error(err));
    }
    return FBC_OK;
}

// Border discovery on the device (after device_cluster_ids): boff (nclusters + 1) and the
// borders of every cluster in ascending id, on the host; the device copy (global ids) stays in
// g.c_bsrc with the offsets in g.c_boff.
int device_borders(const fbc_graph_s* G, int32_t nclusters, const int64_t* coff, std::vector<int64_t>& boff,
                   std::vector<int32_t>& bl, fbc_stats* st) {
    const int64_t nv = coff[nclusters];
    const int32_t n = G->n;
    FBC_CK(g.c_isb.ensure((size_t)std::max(n, 1)));
    FBC_CK(g.c_flag.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nv, 1)));
    FBC_CK(g.c_scan.ensure(sizeof(int32_t) * (size_t)(nv + 1)));
    FBC_CK(cudaMemsetAsync(g.c_isb.p, 0, (size_t)std::max(n, 1), g.st));
    if (n > 0)
        fbc::clu_border_flag_kernel<<<grid_for(n), 256, 0, g.st>>>(n, G->d_rp, G->d_adj, g.c_id.as<int32_t>(),
                                                                   g.c_isb.as<uint8_t>());
    if (nv > 0)
        fbc::clu_gather_flag_kernel<<<grid_for(nv), 256, 0, g.st>>>(nv, g.cgid.as<int32_t>(), g.c_isb.as<uint8_t>(),
                                                                    g.c_flag.as<int32_t>());
    FBC_CK(cudaGetLastError());
    FBC_TRY(device_scan(g.c_flag.as<int32_t>(), nv, g.c_scan.as<int32_t>()));
    // border offsets: the scan at every cluster start
    std::vector<int32_t> pos((size_t)nv + 1);
    FBC_CK(cudaMemcpyAsync(pos.data(), g.c_scan.p, sizeof(int32_t) * pos.size(), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    boff.assign((size_t)nclusters + 1, 0);
    for (int32_t c = 0; c <= nclusters; ++c) boff[c] = pos[coff[c]];
    const int64_t nb = boff[nclusters];
    FBC_CK(g.c_bsrc.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nb, 1)));
    FBC_CK(g.c_boff.ensure(sizeof(int64_t) * ((size_t)nclusters + 1)));
    if (nv > 0)
        fbc::clu_border_scatter_kernel<<<grid_for(nv), 256, 0, g.st>>>(
            nv, g.c_off.as<int64_t>(), nclusters, g.cgid.as<int32_t>(), g.c_flag.as<int32_t>(),
            g.c_scan.as<int32_t>(), g.c_bsrc.as<int32_t>(), g.c_err.as<int>());
    FBC_CK(cudaGetLastError());
    bl.resize((size_t)nb);
    int err = 0;
    if (nb > 0)
        FBC_CK(cudaMemcpyAsync(bl.data(), g.c_bsrc.p, sizeof(int32_t) * (size_t)nb, cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaMemcpyAsync(&err, g.c_err.p, sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    if (st) st->d2h_bytes += (int64_t)(sizeof(int32_t) * ((size_t)nv + 1 + (size_t)nb));
    FBC_TRY(cluster_error(err));
    if (err & fbc::kCluOrder) {  // cluster lists not ascending: sort every cluster's borders
        for (int32_t c = 0; c < nclusters; ++c) std::sort(bl.begin() + boff[c], bl.begin() + boff[c + 1]);
        if (nb > 0)
            FBC_CK(cudaMemcpyAsync(g.c_bsrc.p, bl.data(), sizeof(int32_t) * (size_t)nb, cudaMemcpyHostToDevice, g.st));
    }
    FBC_CK(cudaMemcpyAsync(g.c_boff.p, boff.data(), sizeof(int64_t) * boff.size(), cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    return FBC_OK;
}

// A batched cluster evaluation's device side: cluster ids, borders (discovered when not
// given), the induced-subgraph CSR of every cluster with local ids (SubGraph::forwardStar keeps
// the intra-cluster edges) built by device kernels into the given buffers, and the plan's
// segments and units (border-output row of the i-th vertex of cluster c: E_c + i * nb_c).
int prepare_clusters(const fbc_graph_s* G, int32_t nclusters, const int64_t* coff, const int32_t* cverts,
                     const int64_t* border_off, const int32_t* borders, int precision, int sched,
                     DBuf& crp, DBuf& cadj, DBuf& cgid, DBuf& cbord, Plan& P, int64_t& ent, fbc_stats* st) {
    g_aux_launches = 0;
    FBC_TRY(device_cluster_ids(G, nclusters, coff, cverts, st));
    const int64_t nv = coff[nclusters];
    std::vector<int64_t> boff_v;
    std::vector<int32_t> bl_v;
    if (!border_off) {
        FBC_TRY(device_borders(G, nclusters, coff, boff_v, bl_v, st));
        border_off = boff_v.data();
    } else {
        if (border_off[0] != 0) return fail(FBC_ERR_INVALID_ARG, "border_off[0] must be 0");
        for (int32_t c = 0; c < nclusters; ++c)
            if (border_off[c + 1] < border_off[c]) return fail(FBC_ERR_INVALID_ARG, "border_off is not monotone");
        const int64_t nb = border_off[nclusters];
        FBC_CK(g.c_bsrc.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nb, 1)));
        FBC_CK(g.c_boff.ensure(sizeof(int64_t) * ((size_t)nclusters + 1)));
        if (nb > 0)
            FBC_CK(cudaMemcpyAsync(g.c_bsrc.p, borders, sizeof(int32_t) * (size_t)nb, cudaMemcpyHostToDevice, g.st));
        FBC_CK(cudaMemcpyAsync(g.c_boff.p, border_off, sizeof(int64_t) * ((size_t)nclusters + 1),
                               cudaMemcpyHostToDevice, g.st));
        if (st) st->h2d_bytes += (int64_t)(sizeof(int32_t) * (size_t)nb + sizeof(int64_t) * ((size_t)nclusters + 1));
    }
    const int64_t nbt = border_off[nclusters];
    // intra-cluster degrees, their scan, the local CSRs and the local border ids
    FBC_CK(g.c_flag.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nv, 1)));
    FBC_CK(g.c_scan.ensure(sizeof(int32_t) * (size_t)(nv + 1)));
    FBC_CK(g.c_m.ensure(sizeof(int64_t) * 2 * (size_t)std::max(nclusters, 1)));
    FBC_CK(crp.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nv + nclusters, 1)));
    FBC_CK(cbord.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nbt, 1)));
    if (nv > 0)
        fbc::clu_degree_kernel<<<grid_for(nv), 256, 0, g.st>>>(nv, g.cgid.as<int32_t>(), G->d_rp, G->d_adj,
                                                               g.c_id.as<int32_t>(), g.c_flag.as<int32_t>());
    FBC_CK(cudaGetLastError());
    FBC_TRY(device_scan(g.c_flag.as<int32_t>(), nv, g.c_scan.as<int32_t>()));
    int32_t medges = 0;
    FBC_CK(cudaMemcpyAsync(&medges, g.c_scan.as<int32_t>() + nv, sizeof(int32_t), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    FBC_CK(cadj.ensure(sizeof(int2) * (size_t)std::max(medges, 1)));
    if (nv > 0)
        fbc::clu_fill_kernel<<<grid_for(nv), 256, 0, g.st>>>(nv, g.c_off.as<int64_t>(), nclusters, g.cgid.as<int32_t>(),
                                                             G->d_rp, G->d_adj, g.c_id.as<int32_t>(),
                                                             g.c_lid.as<int32_t>(), g.c_scan.as<int32_t>(),
                                                             crp.as<int32_t>(), cadj.as<int2>());
    if (nclusters > 0)
        fbc::clu_close_kernel<<<grid_for(nclusters), 256, 0, g.st>>>(nclusters, g.c_off.as<int64_t>(),
                                                                     g.c_scan.as<int32_t>(), crp.as<int32_t>(),
                                                                     g.c_m.as<int64_t>(),
                                                                     g.c_m.as<int64_t>() + nclusters);
    if (nbt > 0)
        fbc::clu_border_map_kernel<<<grid_for(nbt), 256, 0, g.st>>>(nbt, g.c_boff.as<int64_t>(), nclusters,
                                                                    g.c_bsrc.as<int32_t>(), G->n, g.c_id.as<int32_t>(),
                                                                    g.c_lid.as<int32_t>(), cbord.as<int32_t>(),
                                                                    g.c_err.as<int>());
    FBC_CK(cudaGetLastError());
    // per cluster: edge count and first edge (the scan at the cluster's first vertex)
    std::vector<int64_t> seg_m(2 * (size_t)std::max(nclusters, 1), 0);
    int err = 0;
    if (nclusters > 0)
        FBC_CK(cudaMemcpyAsync(seg_m.data(), g.c_m.p, sizeof(int64_t) * 2 * (size_t)nclusters, cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaMemcpyAsync(&err, g.c_err.p, sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    FBC_TRY(cluster_error(err));
    // the cluster vertex lists are the output index maps of the segments
    if (&cgid != &g.cgid && nv > 0) {
        FBC_CK(cgid.ensure(sizeof(int32_t) * (size_t)nv));
        FBC_CK(cudaMemcpyAsync(cgid.p, g.cgid.p, sizeof(int32_t) * (size_t)nv, cudaMemcpyDeviceToDevice, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
    }
    P.prec = precision;
    P.sched = sched;
    ent = 0;
    const int dl = delta_for(G->meanw);
    for (int32_t c = 0; c < nclusters; ++c) {
        Seg s{};
        s.rp = crp.as<int32_t>() + coff[c] + c;
        s.adj = cadj.as<int2>() + seg_m[(size_t)nclusters + c];  // rows are relative to the first edge
        s.gid = cgid.as<int32_t>() + coff[c];
        s.border = cbord.as<int32_t>() + border_off[c];
        s.out_base = 0;
        s.n = (int32_t)(coff[c + 1] - coff[c]);
        s.nb = (int32_t)(border_off[c + 1] - border_off[c]);
        s.delta = dl;
        P.segs.push_back(s);
        P.seg_m.push_back(seg_m[c]);
        P.seg_maxw.push_back(G->maxw);
        P.seg_maxindeg.push_back(G->maxindeg);
        for (int32_t i = 0; i < s.n; ++i) P.units.push_back(Unit{c, i, 1.0, ent + (int64_t)i * s.nb});
        ent += (int64_t)s.n * s.nb;
    }
    P.bc_len = G->n;
    P.border_entries = ent;
    if (st) st->launches += g_aux_launches;
    return FBC_OK;
}

// A device buffer released when it goes out of scope (temporaries of a graph build).
// Scratch of one call, allocated from the library's memory pool in the order of the library
// stream and freed the same way (no device-wide synchronisation of cudaFree; the pool keeps up
// to scratch_keep_mb of it for the next call).
struct TmpBuf {
    void* p = nullptr;
    size_t cap = 0;
    TmpBuf() = default;
    TmpBuf(const TmpBuf&) = delete;
    TmpBuf& operator=(const TmpBuf&) = delete;
    ~TmpBuf() {
        if (p) cudaFreeAsync(p, g.st);
    }
    cudaError_t ensure(size_t bytes, bool zero = false) {
        if (p && bytes <= cap) return cudaSuccess;
        if (p) cudaFreeAsync(p, g.st);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMallocFromPoolAsync(&p, want, g.pool, g.st);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        if (zero) return cudaMemsetAsync(p, 0, want, g.st);
        return cudaSuccess;
    }
    template <class T>
    T* as() const {
        return (T*)p;
    }
};

// Edge list already on the device -> device CSR (graph_build.cuh).  Returns FBC_OK with *out
// set, FBC_OK with *out null when a row is longer than the device sort handles (the caller then
// builds on the host), or an error.  The edge arrays are only read.
int device_csr_build(int64_t count, const int32_t* dsrc, const int32_t* ddst, const double* dw, fbc_graph* out) {
    *out = nullptr;
    TmpBuf ints, deg, rs, cursor, keys, ndeg, indeg;
    FBC_CK(ints.ensure(64));
    // ints: [0] max source, [1] error bits, [2] max weight, [3] max in-degree, [4..5] weight sum
    int hi[6] = {-1, 0, 0, 0, 0, 0};
    FBC_CK(cudaMemcpyAsync(ints.p, hi, sizeof(hi), cudaMemcpyHostToDevice, g.st));
    int* di = ints.as<int>();
    fbc::gb_check_kernel<<<grid_for(count), 256, 0, g.st>>>(count, dsrc, ddst,
                                                            dw, di, di + 1);
    FBC_CK(cudaGetLastError());
    FBC_CK(cudaMemcpyAsync(hi, ints.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    if (hi[1] & fbc::kGbWeight) return fail(FBC_ERR_INVALID_ARG, "Edge weight must be greater than zero");
    if (hi[1] & fbc::kGbNegId) return fail(FBC_ERR_INVALID_ARG, "negative vertex id");
    const int32_t n = hi[0] + 1;
    FBC_CK(deg.ensure(sizeof(int32_t) * (size_t)n));
    FBC_CK(rs.ensure(sizeof(int32_t) * ((size_t)n + 1)));
    FBC_CK(cursor.ensure(sizeof(int32_t) * (size_t)n));
    FBC_CK(keys.ensure(sizeof(unsigned long long) * (size_t)count));
    FBC_CK(ndeg.ensure(sizeof(int32_t) * (size_t)n));
    FBC_CK(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * (size_t)n, g.st));
    FBC_CK(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * (size_t)n, g.st));
    fbc::gb_count_kernel<<<grid_for(count), 256, 0, g.st>>>(count, dsrc, ddst, n,
                                                            deg.as<int32_t>(), di + 1);
    FBC_CK(cudaGetLastError());
    FBC_TRY(device_scan(deg.as<int32_t>(), n, rs.as<int32_t>()));
    fbc::gb_scatter_kernel<<<grid_for(count), 256, 0, g.st>>>(count, dsrc, ddst,
                                                              rs.as<int32_t>(), cursor.as<int32_t>(),
                                                              keys.as<unsigned long long>());
    fbc::gb_sort_rows_kernel<<<grid_for(n), 256, 0, g.st>>>(n, rs.as<int32_t>(), keys.as<unsigned long long>(),
                                                            ndeg.as<int32_t>(), di + 1);
    FBC_CK(cudaGetLastError());
    FBC_CK(cudaMemcpyAsync(hi + 1, di + 1, sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    if (hi[1] & fbc::kGbDst) return fail(FBC_ERR_INVALID_ARG, "destination id is not below 1 + max source id");
    if (hi[1] & fbc::kGbLongRow) return FBC_OK;  // host path
    auto* G = new fbc_graph_s();
    std::unique_ptr<fbc_graph_s> guard(G);
    G->n = n;
    const cudaError_t ea = cudaMalloc(&G->d_rp, sizeof(int32_t) * ((size_t)n + 1));
    if (ea != cudaSuccess) {
        G->d_rp = nullptr;
        return fail(FBC_ERR_OOM, "device allocation of the graph failed");
    }
    auto drop = [&]() {
        if (G->d_rp) cudaFree(G->d_rp);
        if (G->d_adj) cudaFree(G->d_adj);
        G->d_rp = nullptr;
        G->d_adj = nullptr;
    };
    if (device_scan(ndeg.as<int32_t>(), n, G->d_rp) != FBC_OK) { drop(); return FBC_ERR_CUDA; }
    int32_t medges = 0;
    if (cudaMemcpyAsync(&medges, G->d_rp + n, sizeof(int32_t), cudaMemcpyDeviceToHost, g.st) != cudaSuccess ||
        cudaStreamSynchronize(g.st) != cudaSuccess) { drop(); return fail(FBC_ERR_CUDA, "graph build failed"); }
    if (cudaMalloc(&G->d_adj, sizeof(int2) * (size_t)std::max(medges, 1)) != cudaSuccess) {
        G->d_adj = nullptr;
        drop();
        return fail(FBC_ERR_OOM, "device allocation of the graph failed");
    }
    if (indeg.ensure(sizeof(int32_t) * (size_t)n) != cudaSuccess ||
        cudaMemsetAsync(indeg.p, 0, sizeof(int32_t) * (size_t)n, g.st) != cudaSuccess) {
        drop();
        return fail(FBC_ERR_OOM, "device allocation failed");
    }
    fbc::gb_merge_kernel<<<grid_for(n), 256, 0, g.st>>>(n, rs.as<int32_t>(), keys.as<unsigned long long>(),
                                                        dw, G->d_rp, G->d_adj, indeg.as<int32_t>(),
                                                        di + 2, (unsigned long long*)(di + 4), di + 1);
    fbc::gb_max_kernel<<<grid_for(n), 256, 0, g.st>>>(n, indeg.as<int32_t>(), di + 3);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hi, ints.p, sizeof(hi), cudaMemcpyDeviceToHost, g.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.st);
    if (e != cudaSuccess) { drop(); return fail(FBC_ERR_CUDA, std::string("graph build: ") + cudaGetErrorString(e)); }
    if (hi[1] & fbc::kGbNonInt) { drop(); return fail(FBC_ERR_RANGE, "edge weights must be integers below 2^31"); }
    unsigned long long sumw = 0;
    std::memcpy(&sumw, hi + 4, sizeof(sumw));
    G->m = medges;
    G->maxw = hi[2];
    G->maxindeg = hi[3];
    G->meanw = medges ? (double)sumw / (double)medges : 1.0;
    if ((double)n * (double)G->maxw > 2147483646.0) {
        drop();
        return fail(FBC_ERR_RANGE, "n * max_weight exceeds the int32 distance range");
    }
    G->host_ok = false;  // the host copy is fetched when something needs it
    *out = guard.release();
    return FBC_OK;
}

// Edge list in host memory -> device CSR: upload, then device_csr_build.
int device_graph_from_edges(int64_t count, const int32_t* src, const int32_t* dst, const double* w,
                            fbc_graph* out) {
    TmpBuf dsrc, ddst, dw;
    FBC_CK(dsrc.ensure(sizeof(int32_t) * (size_t)count));
    FBC_CK(ddst.ensure(sizeof(int32_t) * (size_t)count));
    FBC_CK(dw.ensure(sizeof(double) * (size_t)count));
    FBC_CK(cudaMemcpyAsync(dsrc.p, src, sizeof(int32_t) * (size_t)count, cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(ddst.p, dst, sizeof(int32_t) * (size_t)count, cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(dw.p, w, sizeof(double) * (size_t)count, cudaMemcpyHostToDevice, g.st));
    return device_csr_build(count, dsrc.as<int32_t>(), ddst.as<int32_t>(), dw.as<double>(), out);
}

// Edge list -> CSR on the host (DirectedWeightedGraph.h:136-170): rows by source, each row
// ascending by destination (the std::map order), a repeated pair's weights summed in input order.
int host_graph_from_edges(int64_t count, const int32_t* src, const int32_t* dst, const double* w, fbc_graph* out) {
    int32_t maxs = -1;
    for (int64_t i = 0; i < count; ++i) {
        if (!(w[i] > 0)) return fail(FBC_ERR_INVALID_ARG, "Edge weight must be greater than zero");
        if (src[i] < 0 || dst[i] < 0) return fail(FBC_ERR_INVALID_ARG, "negative vertex id");
        maxs = std::max(maxs, src[i]);
    }
    const int32_t n = maxs + 1;
    std::vector<int64_t> idx((size_t)count);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) {
        return src[a] != src[b] ? src[a] < src[b] : dst[a] < dst[b];
    });
    std::vector<int64_t> rp((size_t)n + 1, 0);
    std::vector<int32_t> col;
    std::vector<double> ww;
    col.reserve((size_t)count);
    ww.reserve((size_t)count);
    int32_t ps = -1, pd = -1;
    for (int64_t k = 0; k < count; ++k) {
        const int64_t i = idx[(size_t)k];
        if (dst[i] >= n)
            return fail(FBC_ERR_INVALID_ARG, "destination id " + std::to_string(dst[i]) +
                                                 " is not below 1 + max source id");
        if (src[i] == ps && dst[i] == pd) {
            ww.back() += w[i];  // DirectedWeightedGraph.h:154-155: repeated pair, weights summed
        } else {
            col.push_back(dst[i]);
            ww.push_back(w[i]);
            rp[(size_t)src[i] + 1]++;
            ps = src[i];
            pd = dst[i];
        }
    }
    for (int32_t v = 0; v < n; ++v) rp[(size_t)v + 1] += rp[(size_t)v];
    return make_graph(n, std::move(rp), std::move(col), ww.data(), out);
}

// A weight token the device left to the host, converted as operator>>(double&) does it in the
// classic locale (libstdc++ hands the token to strtod there): overflow gives HUGE_VAL, which
// operator>> turns into the largest double with failbit set, so the reference loop ends
// (DirectedWeightedGraph.h:78-86); underflow gives 0 (rejected) or a subnormal.
enum class TxHost { kValue, kStop, kNotPositive };
TxHost tx_host_weight(const char* text, int64_t len, int64_t pos, double& v) {
    static const locale_t c_locale = newlocale(LC_ALL_MASK, "C", (locale_t)0);
    int64_t end = pos;
    while (end < len && !(text[end] == ' ' || (text[end] >= 9 && text[end] <= 13))) ++end;
    char small[64];
    std::string big;
    const size_t n = (size_t)(end - pos);
    char* buf = small;
    if (n >= sizeof(small)) {
        big.assign(text + pos, n);
        buf = &big[0];
    } else {
        std::memcpy(small, text + pos, n);
        small[n] = 0;
    }
    v = strtod_l(buf, nullptr, c_locale);
    if (v == HUGE_VAL) return TxHost::kStop;
    if (!(v > 0)) return TxHost::kNotPositive;
    return TxHost::kValue;
}

// The host conversions of a text, split over the host's cores when there are many.
void tx_host_weights(const char* text, int64_t len, const std::vector<int2>& sl, std::vector<int32_t>& fi,
                     std::vector<double>& fv, int64_t& stop, int64_t& bad_w) {
    const size_t nt = sl.size() < 65536 ? 1 : std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::vector<int32_t>> ti(nt);
    std::vector<std::vector<double>> tv(nt);
    std::vector<int64_t> ts(nt, stop), tb(nt, bad_w);
    auto work = [&](size_t k) {
        for (size_t i = sl.size() * k / nt; i < sl.size() * (k + 1) / nt; ++i) {
            double v = 0.0;
            switch (tx_host_weight(text, len, sl[i].y, v)) {
                case TxHost::kValue: ti[k].push_back(sl[i].x); tv[k].push_back(v); break;
                case TxHost::kStop: ts[k] = std::min<int64_t>(ts[k], sl[i].x); break;
                case TxHost::kNotPositive: tb[k] = std::min<int64_t>(tb[k], sl[i].x); break;
            }
        }
    };
    std::vector<std::thread> th;
    for (size_t k = 1; k < nt; ++k) th.emplace_back(work, k);
    work(0);
    for (auto& t : th) t.join();
    for (size_t k = 0; k < nt; ++k) {
        fi.insert(fi.end(), ti[k].begin(), ti[k].end());
        fv.insert(fv.end(), tv[k].begin(), tv[k].end());
        stop = std::min(stop, ts[k]);
        bad_w = std::min(bad_w, tb[k]);
    }
}

}  // namespace

// Error text of the calling thread, shared with the other translation units of the library.
void fbc_internal_set_error(const char* msg) { g_err = msg ? msg : ""; }

// ============================================================================ C ABI
extern "C" {

const char* fbc_last_error_string(void) { return g_err.c_str(); }

int fbc_gpu_init(int device) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (g.init) {
        if (device == g.dev) return FBC_OK;
        return fail(FBC_ERR_INVALID_ARG, "already initialised on another device");
    }
    int count = 0;
    FBC_CK(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return fail(FBC_ERR_INVALID_ARG, "no such CUDA device");
    FBC_CK(cudaSetDevice(device));
    FBC_CK(cudaDeviceGetAttribute(&g.nsm, cudaDevAttrMultiProcessorCount, device));
    FBC_CK(cudaDeviceGetAttribute(&g.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    FBC_CK(cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking));
    FBC_CK(cudaEventCreate(&g.ev0));
    FBC_CK(cudaEventCreate(&g.ev1));
    FBC_CK(cudaEventCreate(&g.evm));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    FBC_CK(cudaMemPoolCreate(&g.pool, &props));
    uint64_t keep = (uint64_t)g.opt.scratch_keep_mb << 20;
    FBC_CK(cudaMemPoolSetAttribute(g.pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g.dev = device;
    g.init = true;
    return FBC_OK;
}

int fbc_gpu_shutdown(void) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.init) return FBC_OK;
    cudaStreamSynchronize(g.st);
    for (DBuf* b : {&g.c_off, &g.c_id, &g.c_lid, &g.c_isb, &g.c_flag, &g.c_scan, &g.c_sums, &g.c_boff,
                    &g.c_bsrc, &g.c_m, &g.c_err, &g.retry, &g.segs, &g.units_b, &g.units_w, &g.chunks, &g.crp, &g.cadj, &g.cgid, &g.cbord, &g.bc,
                    &g.bdist, &g.bsig, &g.ctr, &g.dbg})
        b->release();
    g.wsb.buf.release();
    g.wsw.buf.release();
    g.wsb = Workspace();
    g.wsw = Workspace();
    cudaEventDestroy(g.ev0);
    cudaEventDestroy(g.ev1);
    cudaEventDestroy(g.evm);
    cudaStreamSynchronize(g.st);
    cudaMemPoolDestroy(g.pool);
    g.pool = nullptr;
    cudaStreamDestroy(g.st);
    g.init = false;
    return FBC_OK;
}

int fbc_set_option(const char* key, int64_t value) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!key) return fail(FBC_ERR_INVALID_ARG, "null option key");
    std::string k(key);
    if (k == "delta") g.opt.delta = std::max<int64_t>(0, value);
    else if (k == "block_threads") g.opt.block_threads = std::max<int64_t>(32, std::min<int64_t>(1024, value));
    else if (k == "chunk_max") g.opt.chunk_max = std::max<int64_t>(1, value);
    else if (k == "wide_n") g.opt.wide_n = std::max<int64_t>(1, value);
    else if (k == "frontier_threads") g.opt.frontier_threads = std::max<int64_t>(32, std::min<int64_t>(512, value));
    else if (k == "warp_max_n") g.opt.warp_max_n = std::max<int64_t>(0, value);
    else if (k == "iter_mult") g.opt.iter_mult = std::max<int64_t>(0, std::min<int64_t>(1 << 20, value));
    else if (k == "ws_budget_mb") g.opt.ws_budget_mb = std::max<int64_t>(0, value);
    else if (k == "order_min_n") g.opt.order_min_n = std::max<int64_t>(0, value);
    else if (k == "csr_device_min_m") g.opt.csr_device_min_m = std::max<int64_t>(0, value);
    else if (k == "wide_threads") g.opt.wide_threads = std::max<int64_t>(64, std::min<int64_t>(1024, value / 32 * 32));
    else if (k == "wide_kv") g.opt.wide_kv = value <= 1 ? 1 : 2;
    else if (k == "adj4") g.opt.adj4 = value != 0;
    else if (k == "pull_count") g.opt.pull_count = value != 0;
    else if (k == "source_order") g.opt.source_order = value != 0;
    else if (k == "bc_sweep") g.opt.bc_sweep = value != 0;
    else if (k == "group") {
        if (value != 0 && value != 1 && value != 2 && value != 4) return fail(FBC_ERR_INVALID_ARG, "group must be 0, 1, 2 or 4");
        g.opt.group = value;
    }
    else if (k == "debug_sched") g.opt.debug_sched = value ? FBC_SCHED_BATCHED : FBC_SCHED_PLAIN;
    else if (k == "scratch_keep_mb") {
        g.opt.scratch_keep_mb = std::max<int64_t>(0, value);
        if (g.pool) {
            uint64_t keep = (uint64_t)g.opt.scratch_keep_mb << 20;
            cudaMemPoolSetAttribute(g.pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    else return fail(FBC_ERR_INVALID_ARG, "unknown option " + k);
    return FBC_OK;
}

int fbc_get_option(const char* key, int64_t* value) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!key || !value) return fail(FBC_ERR_INVALID_ARG, "null argument");
    std::string k(key);
    if (k == "delta") *value = g.opt.delta;
    else if (k == "block_threads") *value = g.opt.block_threads;
    else if (k == "chunk_max") *value = g.opt.chunk_max;
    else if (k == "wide_n") *value = g.opt.wide_n;
    else if (k == "frontier_threads") *value = g.opt.frontier_threads;
    else if (k == "warp_max_n") *value = g.opt.warp_max_n;
    else if (k == "iter_mult") *value = g.opt.iter_mult;
    else if (k == "ws_budget_mb") *value = g.opt.ws_budget_mb;
    else if (k == "group") *value = g.opt.group;
    else if (k == "order_min_n") *value = g.opt.order_min_n;
    else if (k == "csr_device_min_m") *value = g.opt.csr_device_min_m;
    else if (k == "wide_threads") *value = g.opt.wide_threads;
    else if (k == "wide_kv") *value = g.opt.wide_kv;
    else if (k == "adj4") *value = g.opt.adj4;
    else if (k == "bc_sweep") *value = g.opt.bc_sweep;
    else if (k == "pull_count") *value = g.opt.pull_count;
    else if (k == "source_order") *value = g.opt.source_order;
    else if (k == "debug_sched") *value = g.opt.debug_sched;
    else if (k == "scratch_keep_mb") *value = g.opt.scratch_keep_mb;
    else return fail(FBC_ERR_INVALID_ARG, "unknown option " + k);
    return FBC_OK;
}

int fbc_graph_upload(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                     fbc_graph* out) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!out || !row_ptr || n < 0) return fail(FBC_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::vector<int64_t> rp(row_ptr, row_ptr + (size_t)n + 1);
    const int64_t m = rp[n];
    if (m < 0) return fail(FBC_ERR_INVALID_ARG, "negative edge count");
    if (m > 0 && (!col || !w)) return fail(FBC_ERR_INVALID_ARG, "null edge arrays");
    std::vector<int32_t> c(col, col + (size_t)m);
    return make_graph(n, std::move(rp), std::move(c), w, out);
}

int fbc_graph_from_edges(int64_t count, const int32_t* src, const int32_t* dst, const double* w,
                         fbc_graph* out) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!out || count < 0 || (count > 0 && (!src || !dst || !w)))
        return fail(FBC_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (count >= g.opt.csr_device_min_m && count < ((int64_t)1 << 31) - 1) {
        FBC_TRY(device_graph_from_edges(count, src, dst, w, out));
        if (*out) return FBC_OK;  // else a row too long for the device sort: the host path
    }
    return host_graph_from_edges(count, src, dst, w, out);
}

int fbc_graph_from_text(const char* text, int64_t len, fbc_graph* out, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!out || len < 0 || (len > 0 && !text)) return fail(FBC_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (st) std::memset(st, 0, sizeof(*st));
    const double t0 = now_ms();
    if (len > (int64_t)INT32_MAX - 2 * fbc::kTxTile) return fail(FBC_ERR_RANGE, "edge-list text longer than 2 GiB");
    // the device copy ends in at least one space, so every token scan stops inside it, and has
    // a halo of spaces past its last tile
    const int64_t ntiles = (len + 1 + fbc::kTxTile - 1) / fbc::kTxTile;
    const size_t padded = (size_t)ntiles * fbc::kTxTile + fbc::kTxHalo;
    // capacity from the length alone (a token and its separator take two bytes, a triple six),
    // so the passes run back to back with no host round trip
    const int64_t edge_cap = (len + 1) / 6 + 1;
    TmpBuf dtext, cnt, toff, dsrc, ddst, dw, find, slow, fix_i, fix_v;
    FBC_CK(dtext.ensure(padded));
    FBC_CK(cnt.ensure(sizeof(int32_t) * (size_t)ntiles));
    FBC_CK(toff.ensure(sizeof(int32_t) * ((size_t)ntiles + 1)));
    FBC_CK(dsrc.ensure(sizeof(int32_t) * (size_t)edge_cap));
    FBC_CK(ddst.ensure(sizeof(int32_t) * (size_t)edge_cap));
    FBC_CK(dw.ensure(sizeof(double) * (size_t)edge_cap));
    FBC_CK(slow.ensure(sizeof(int2) * (size_t)edge_cap));
    FBC_CK(find.ensure(sizeof(fbc::TxFind)));
    if (len > 0) FBC_CK(cudaMemcpyAsync(dtext.p, text, (size_t)len, cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemsetAsync((char*)dtext.p + len, ' ', padded - (size_t)len, g.st));
    fbc::TxFind hf{INT32_MAX, INT32_MAX, 0};
    FBC_CK(cudaMemcpyAsync(find.p, &hf, sizeof(hf), cudaMemcpyHostToDevice, g.st));
    cudaEvent_t ev[2];
    FBC_CK(cudaEventCreate(&ev[0]));
    FBC_CK(cudaEventCreate(&ev[1]));
    cudaEventRecord(ev[0], g.st);
    const unsigned char* dt = (const unsigned char*)dtext.p;
    const unsigned tgrid = (unsigned)ntiles;  // one tile per block: many blocks in flight hide latency
    const int aux0 = g_aux_launches;
    fbc::tx_count_kernel<<<tgrid, fbc::kTxThreads, 0, g.st>>>(ntiles, dt, cnt.as<int32_t>());
    int rc = device_scan(cnt.as<int32_t>(), ntiles, toff.as<int32_t>());
    if (rc == FBC_OK)
        fbc::tx_tokens_kernel<<<tgrid, fbc::kTxThreads, 0, g.st>>>(ntiles, dt, toff.as<int32_t>(), dsrc.as<int32_t>(),
                                                                  ddst.as<int32_t>(), dw.as<double>(),
                                                                  find.as<fbc::TxFind>(), slow.as<int2>());
    cudaEventRecord(ev[1], g.st);
    int32_t ntok = 0;
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&hf, find.p, sizeof(hf), cudaMemcpyDeviceToHost, g.st);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(&ntok, toff.as<int32_t>() + ntiles, sizeof(int32_t), cudaMemcpyDeviceToHost, g.st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(g.st);
    float parse_ms = 0.f;
    if (ce == cudaSuccess) cudaEventElapsedTime(&parse_ms, ev[0], ev[1]);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (rc != FBC_OK) return rc;
    if (ce != cudaSuccess) return fail(FBC_ERR_CUDA, std::string("text parse: ") + cudaGetErrorString(ce));
    if (st) {
        st->kernel_ms = parse_ms;
        st->launches = 2 + (g_aux_launches - aux0);  // count, tokens, and the scan's kernels
        st->h2d_bytes = len;
    }
    const int64_t nedges = ntok / 3;
    // weights left to the host, and where reading ends (a weight that overflows a double)
    int64_t stop = nedges, bad_w = hf.bad_w;
    std::vector<int32_t> fi;
    std::vector<double> fv;
    if (hf.nslow > 0) {
        std::vector<int2> sl((size_t)hf.nslow);
        FBC_CK(cudaMemcpyAsync(sl.data(), slow.p, sizeof(int2) * sl.size(), cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
        tx_host_weights(text, len, sl, fi, fv, stop, bad_w);
    }
    // the first finding in text order decides (an id before the weight of its triple); nothing
    // after the end of reading counts
    if (std::min<int64_t>(hf.bad_id, bad_w) <= stop) {
        if (hf.bad_id <= bad_w)
            return fail(FBC_ERR_INVALID_ARG, "edge " + std::to_string(hf.bad_id) + ": a vertex id is not a decimal int32");
        return fail(FBC_ERR_INVALID_ARG, "Edge weight must be greater than zero (edge " + std::to_string(bad_w) + ")");
    }
    if (stop == nedges && ntok % 3 != 0)
        return fail(FBC_ERR_INVALID_ARG, "the text ends inside an edge (" + std::to_string(ntok % 3) + " of 3 fields)");
    if (!fi.empty()) {
        FBC_CK(fix_i.ensure(sizeof(int32_t) * fi.size()));
        FBC_CK(fix_v.ensure(sizeof(double) * fv.size()));
        FBC_CK(cudaMemcpyAsync(fix_i.p, fi.data(), sizeof(int32_t) * fi.size(), cudaMemcpyHostToDevice, g.st));
        FBC_CK(cudaMemcpyAsync(fix_v.p, fv.data(), sizeof(double) * fv.size(), cudaMemcpyHostToDevice, g.st));
        fbc::tx_fix_kernel<<<grid_for((int64_t)fi.size()), 256, 0, g.st>>>((int32_t)fi.size(), fix_i.as<int32_t>(),
                                                                           fix_v.as<double>(), dw.as<double>());
        FBC_CK(cudaGetLastError());
    }
    const int64_t count = stop;
    if (count > 0) {
        FBC_TRY(device_csr_build(count, dsrc.as<int32_t>(), ddst.as<int32_t>(), dw.as<double>(), out));
        if (*out) {
            if (st) {
                st->wall_ms = now_ms() - t0;
                st->d2h_bytes = (int64_t)sizeof(fbc::TxFind) + 4 + 24;  // findings, token count, build summary
            }
            return FBC_OK;
        }
    }
    // no edges, or a row too long for the device sort: the host build from the parsed arrays
    std::vector<int32_t> hs((size_t)count), hd((size_t)count);
    std::vector<double> hw((size_t)count);
    if (count > 0) {
        FBC_CK(cudaMemcpyAsync(hs.data(), dsrc.p, sizeof(int32_t) * hs.size(), cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaMemcpyAsync(hd.data(), ddst.p, sizeof(int32_t) * hd.size(), cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaMemcpyAsync(hw.data(), dw.p, sizeof(double) * hw.size(), cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
    }
    FBC_TRY(host_graph_from_edges(count, hs.data(), hd.data(), hw.data(), out));
    if (st) st->wall_ms = now_ms() - t0;
    return FBC_OK;
}

int fbc_graph_info(fbc_graph G, int32_t* n, int64_t* m) {
    if (!G) return fail(FBC_ERR_INVALID_ARG, "null graph");
    if (n) *n = G->n;
    if (m) *m = G->m;
    return FBC_OK;
}

int fbc_graph_download(fbc_graph G, int64_t* row_ptr, int32_t* col, double* w) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!G) return fail(FBC_ERR_INVALID_ARG, "null graph");
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    FBC_TRY(ensure_host_csr(G));
    if (row_ptr) std::copy(G->h_rp.begin(), G->h_rp.end(), row_ptr);
    if (col) std::copy(G->h_col.begin(), G->h_col.end(), col);
    if (w)
        for (size_t e = 0; e < G->h_w.size(); ++e) w[e] = (double)G->h_w[e];
    return FBC_OK;
}

// The whole-graph segment a batched run uses: graphs of at least `order_min_n` vertices run on
// their relabelled CSR (outputs go back to input ids through gid); `map` then translates source
// ids.  Plain runs and debug dumps use the input order.
int batched_graph_seg(fbc_graph_s* G, int64_t out_base, int sched, Seg& s, const int32_t*& map) {
    s = whole_graph_seg(G, out_base);
    map = nullptr;
    if (sched != FBC_SCHED_BATCHED || (int64_t)G->n < g.opt.order_min_n) return FBC_OK;
    FBC_TRY(ensure_order(G));
    s.rp = G->d_ord_rp;
    s.adj = G->d_ord_adj;
    s.adj4 = g.opt.adj4 ? G->d_ord_adj4 : nullptr;
    s.revw = g.opt.pull_count ? G->d_ord_revw : nullptr;
    s.gid = G->d_ord_inv;
    map = G->ord_new.data();
    return FBC_OK;
}

int fbc_graph_free(fbc_graph G) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!G) return FBC_OK;
    DevGuard dg_;
    if (g.init) {
        dg_.enter();
        cudaStreamSynchronize(g.st);
    }
    cudaFree(G->d_rp);
    cudaFree(G->d_adj);
    if (G->d_ord_rp) cudaFree(G->d_ord_rp);
    if (G->d_ord_adj) cudaFree(G->d_ord_adj);
    if (G->d_ord_adj4) cudaFree(G->d_ord_adj4);
    if (G->d_ord_revw) cudaFree(G->d_ord_revw);
    if (G->d_ord_inv) cudaFree(G->d_ord_inv);
    delete G;
    return FBC_OK;
}

int fbc_exact_bc(fbc_graph G, int precision, int sched, double* out_bc, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G || (!out_bc && G->n > 0)) return fail(FBC_ERR_INVALID_ARG, "null argument");
    FBC_TRY(check_sched(sched));
    const double t0 = now_ms();
    if (st) std::memset(st, 0, sizeof(*st));
    Plan P;
    P.prec = precision;
    P.sched = sched;
    Seg sg;
    const int32_t* map = nullptr;
    FBC_TRY(batched_graph_seg(G, 0, sched, sg, map));
    P.segs.push_back(sg);
    P.seg_m.push_back(G->m);
    P.seg_maxw.push_back(G->maxw);
    P.seg_maxindeg.push_back(G->maxindeg);
    for (int32_t s = 0; s < G->n; ++s) P.units.push_back(Unit{0, s, 1.0, -1});
    P.bc_len = G->n;
    FBC_TRY(run_plan(P, st));
    FBC_TRY(download_bc(out_bc, G->n, false, st));
    if (st) st->wall_ms = now_ms() - t0;
    return FBC_OK;
}

int fbc_sssp_dependency_batch(fbc_graph G, int64_t count, const int32_t* sources,
                              const double* cards, int precision, int sched, double* out_bc_accum,
                              fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G || count < 0 || (count > 0 && !sources) || (!out_bc_accum && G->n > 0))
        return fail(FBC_ERR_INVALID_ARG, "null argument");
    FBC_TRY(check_sched(sched));
    const double t0 = now_ms();
    if (st) std::memset(st, 0, sizeof(*st));
    Plan P;
    P.prec = precision;
    P.sched = sched;
    for (int64_t i = 0; i < count; ++i)
        if (sources[i] < 0 || sources[i] >= G->n) return fail(FBC_ERR_INVALID_ARG, "source out of range");
    Seg sg;
    const int32_t* map = nullptr;
    FBC_TRY(batched_graph_seg(G, 0, sched, sg, map));
    P.segs.push_back(sg);
    P.seg_m.push_back(G->m);
    P.seg_maxw.push_back(G->maxw);
    P.seg_maxindeg.push_back(G->maxindeg);
    for (int64_t i = 0; i < count; ++i)
        P.units.push_back(Unit{0, map ? map[sources[i]] : sources[i], cards ? cards[i] : 1.0, -1});
    // on a relabelled graph, sources in the locality order: the sources running at once then
    // start near each other, and their wavefronts read the same rows at about the same time
    if (map && g.opt.source_order)
        std::stable_sort(P.units.begin(), P.units.end(), [](const Unit& a, const Unit& b) { return a.src < b.src; });
    P.bc_len = G->n;
    if (st) st->h2d_bytes += count * (int64_t)(sizeof(int32_t) + sizeof(double));
    FBC_TRY(run_plan(P, st));
    FBC_TRY(download_bc(out_bc_accum, G->n, true, st));
    if (st) st->wall_ms = now_ms() - t0;
    return FBC_OK;
}

int fbc_single_source(fbc_graph G, int32_t source, int precision, double* out_dep, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G || !out_dep) return fail(FBC_ERR_INVALID_ARG, "null argument");
    std::fill(out_dep, out_dep + G->n, 0.0);
    const double one = 1.0;
    return fbc_sssp_dependency_batch(G, 1, &source, &one, precision, FBC_SCHED_PLAIN, out_dep, st);
}

int fbc_cluster_border_count(fbc_graph G, int32_t nclusters, const int64_t* coff,
                             const int32_t* cverts, const int64_t* border_off, int64_t* out_nb,
                             int64_t* out_entries) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G) return fail(FBC_ERR_INVALID_ARG, "null graph");
    std::vector<int64_t> boff;
    std::vector<int32_t> bl;
    if (!border_off) {
        FBC_TRY(device_cluster_ids(G, nclusters, coff, cverts, nullptr));
        FBC_TRY(device_borders(G, nclusters, coff, boff, bl, nullptr));
        border_off = boff.data();
    } else {
        FBC_TRY(check_cluster_offsets(G, nclusters, coff, cverts));
    }
    int64_t nb = 0, ent = 0;
    for (int32_t c = 0; c < nclusters; ++c) {
        const int64_t b = border_off[c + 1] - border_off[c];
        nb += b;
        ent += b * (coff[c + 1] - coff[c]);
    }
    if (out_nb) *out_nb = nb;
    if (out_entries) *out_entries = ent;
    return FBC_OK;
}

int fbc_cluster_borders(fbc_graph G, int32_t nclusters, const int64_t* coff, const int32_t* cverts,
                        int64_t* out_boff, int32_t* out_borders) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G) return fail(FBC_ERR_INVALID_ARG, "null graph");
    std::vector<int64_t> boff;
    std::vector<int32_t> bl;
    FBC_TRY(device_cluster_ids(G, nclusters, coff, cverts, nullptr));
    FBC_TRY(device_borders(G, nclusters, coff, boff, bl, nullptr));
    if (out_boff) std::copy(boff.begin(), boff.end(), out_boff);
    if (out_borders) std::copy(bl.begin(), bl.end(), out_borders);
    return FBC_OK;
}

int fbc_kmeans(int32_t nsets, const int64_t* set_off, const int32_t* nb, const int64_t* vec_off, const double* len,
               const int32_t* cnt, const int32_t* wt, const int32_t* k, double min_variance, int32_t max_iter,
               int32_t* out_idx, int32_t* out_w, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (nsets < 0 || (nsets > 0 && (!set_off || !nb || !vec_off || !k || !wt || !out_idx || !out_w)))
        return fail(FBC_ERR_INVALID_ARG, "null argument");
    if (max_iter < 0) return fail(FBC_ERR_INVALID_ARG, "max_iter < 0");
    const double t0 = now_ms();
    if (st) std::memset(st, 0, sizeof(*st));
    if (nsets == 0) return FBC_OK;
    // sets, their points as (length, count) int pairs transposed per set (border-major), work areas
    std::vector<fbc::KMSet> sets((size_t)nsets);
    int64_t xs = 0, ws = 0, outs = 0;
    for (int32_t s = 0; s < nsets; ++s) {
        const int64_t np = set_off[s + 1] - set_off[s];
        if (np <= 0 || np > 0x7fffffff || nb[s] < 0 || k[s] < 1 || k[s] > np)
            return fail(FBC_ERR_INVALID_ARG, "set " + std::to_string(s) + ": needs 1 <= k <= points, nb >= 0");
        if (nb[s] > 0 && (!len || !cnt)) return fail(FBC_ERR_INVALID_ARG, "null vectors");
        fbc::KMSet& S = sets[(size_t)s];
        S.np = (int32_t)np;
        S.nb = nb[s];
        S.k = k[s];
        S.x_off = xs;
        S.ws_off = ws;
        S.out_off = outs;
        S.p_off = set_off[s];
        xs += np * nb[s];
        ws += fbc::km_work_bytes(np, nb[s], k[s]);
        outs += k[s];
    }
    std::vector<int2> X((size_t)std::max<int64_t>(xs, 1));
    for (int32_t s = 0; s < nsets; ++s) {
        const fbc::KMSet& S = sets[(size_t)s];
        double lmax = 0.0, cmax = 0.0;
        for (int64_t j = 0; j < S.np; ++j)
            for (int32_t i = 0; i < S.nb; ++i) {
                const double l = len[vec_off[s] + j * S.nb + i];
                const int32_t c = cnt[vec_off[s] + j * S.nb + i];
                if (!(l >= 0.0 && l <= 2147483647.0) || l != std::floor(l))
                    return fail(FBC_ERR_INVALID_ARG, "lengths must be integers in [0, 2^31)");
                lmax = std::max(lmax, l);
                cmax = std::max(cmax, std::fabs((double)c));
                X[(size_t)(S.x_off + (int64_t)i * S.np + j)] = make_int2((int32_t)l, c);
            }
        // every squared distance exact in a double, as the reference's sums are on these inputs
        if ((double)S.nb * (lmax * lmax + 4.0 * cmax * cmax) >= 9007199254740992.0)
            return fail(FBC_ERR_RANGE, "set " + std::to_string(s) + ": squared distances may exceed 2^53");
    }
    TmpBuf dsets, dx, dwt, dws, didx, dw;
    FBC_CK(dsets.ensure(sizeof(fbc::KMSet) * sets.size()));
    FBC_CK(dx.ensure(sizeof(int2) * X.size()));
    FBC_CK(dwt.ensure(sizeof(int32_t) * (size_t)set_off[nsets]));
    FBC_CK(dws.ensure((size_t)std::max<int64_t>(ws, 256)));
    FBC_CK(didx.ensure(sizeof(int32_t) * (size_t)outs));
    FBC_CK(dw.ensure(sizeof(int32_t) * (size_t)outs));
    FBC_CK(cudaMemcpyAsync(dsets.p, sets.data(), sizeof(fbc::KMSet) * sets.size(), cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(dx.p, X.data(), sizeof(int2) * X.size(), cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(dwt.p, wt, sizeof(int32_t) * (size_t)set_off[nsets], cudaMemcpyHostToDevice, g.st));
    fbc::KMParams K{};
    K.sets = dsets.as<fbc::KMSet>();
    K.X = dx.as<int2>();
    K.wt = dwt.as<int32_t>();
    K.ws = dws.as<char>();
    K.min_variance = min_variance;
    K.max_iter = max_iter;
    K.out_idx = didx.as<int32_t>();
    K.out_w = dw.as<int32_t>();
    FBC_CK(cudaEventRecord(g.ev0, g.st));
    fbc::kmeans_kernel<<<(unsigned)nsets, 1024, 0, g.st>>>(K);
    FBC_CK(cudaGetLastError());
    FBC_CK(cudaEventRecord(g.ev1, g.st));
    FBC_CK(cudaMemcpyAsync(out_idx, didx.p, sizeof(int32_t) * (size_t)outs, cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaMemcpyAsync(out_w, dw.p, sizeof(int32_t) * (size_t)outs, cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    if (st) {
        float ms = 0.f;
        FBC_CK(cudaEventElapsedTime(&ms, g.ev0, g.ev1));
        st->kernel_ms = ms;
        st->launches = 1;
        st->h2d_bytes = (int64_t)(sizeof(int2) * X.size() + sizeof(int32_t) * set_off[nsets]);
        st->d2h_bytes = (int64_t)(8 * outs);
        st->wall_ms = now_ms() - t0;
    }
    return FBC_OK;
}

int fbc_cluster_classes(fbc_graph G, int32_t nclusters, const int64_t* coff, const int32_t* cverts,
                        const int64_t* border_off, const int32_t* borders, const double* bc,
                        const double* bdist, const uint64_t* bsig, int64_t* out_class_off,
                        int32_t* out_pivots, int32_t* out_cards) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G || !bc || !out_class_off || (border_off && !borders)) return fail(FBC_ERR_INVALID_ARG, "null argument");
    FBC_TRY(device_cluster_ids(G, nclusters, coff, cverts, nullptr));
    const int64_t nv = coff[nclusters];
    std::vector<int64_t> boff_v;
    std::vector<int32_t> bl_v;
    if (!border_off) {
        FBC_TRY(device_borders(G, nclusters, coff, boff_v, bl_v, nullptr));
        border_off = boff_v.data();
    } else {
        if (border_off[0] != 0) return fail(FBC_ERR_INVALID_ARG, "border_off[0] must be 0");
        for (int32_t c = 0; c < nclusters; ++c)
            if (border_off[c + 1] < border_off[c]) return fail(FBC_ERR_INVALID_ARG, "border_off is not monotone");
        const int64_t nb = border_off[nclusters];
        FBC_CK(g.c_bsrc.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nb, 1)));
        FBC_CK(g.c_boff.ensure(sizeof(int64_t) * ((size_t)nclusters + 1)));
        if (nb > 0)
            FBC_CK(cudaMemcpyAsync(g.c_bsrc.p, borders, sizeof(int32_t) * (size_t)nb, cudaMemcpyHostToDevice, g.st));
        FBC_CK(cudaMemcpyAsync(g.c_boff.p, border_off, sizeof(int64_t) * ((size_t)nclusters + 1),
                               cudaMemcpyHostToDevice, g.st));
    }
    const int64_t nbt = border_off[nclusters];
    if (nv > 0 && (!out_pivots || !out_cards)) return fail(FBC_ERR_INVALID_ARG, "null argument");
    // border-vector entries and table slots of every cluster
    std::vector<int64_t> eoff((size_t)nclusters + 1, 0), toff((size_t)nclusters + 1, 0);
    for (int32_t c = 0; c < nclusters; ++c) {
        const int64_t nc = coff[c + 1] - coff[c];
        eoff[c + 1] = eoff[c] + nc * (border_off[c + 1] - border_off[c]);
        int64_t t = 2;
        while (t < 2 * nc) t <<= 1;
        toff[c + 1] = toff[c] + (nc > 0 ? t : 0);
    }
    if ((bdist == nullptr || bsig == nullptr) && eoff[nclusters] > 0) return fail(FBC_ERR_INVALID_ARG, "null argument");
    TmpBuf d_eoff, d_toff, d_bd, d_bs, d_bc, thash, tfirst, vhash, vrep, flag, scan, isb, cbord, card, minbc, pick, piv, crd;
    const size_t ne = (size_t)std::max<int64_t>(eoff[nclusters], 1), nts = (size_t)std::max<int64_t>(toff[nclusters], 1);
    const size_t nvv = (size_t)std::max<int64_t>(nv, 1);
    FBC_CK(d_eoff.ensure(sizeof(int64_t) * eoff.size()));
    FBC_CK(d_toff.ensure(sizeof(int64_t) * toff.size()));
    FBC_CK(d_bd.ensure(sizeof(double) * ne));
    FBC_CK(d_bs.ensure(sizeof(uint64_t) * ne));
    FBC_CK(d_bc.ensure(sizeof(double) * (size_t)std::max(G->n, 1)));
    FBC_CK(thash.ensure(sizeof(unsigned long long) * nts));
    FBC_CK(tfirst.ensure(sizeof(int) * nts));
    FBC_CK(vhash.ensure(sizeof(unsigned long long) * nvv));
    FBC_CK(vrep.ensure(sizeof(int) * nvv));
    FBC_CK(flag.ensure(sizeof(int32_t) * nvv));
    FBC_CK(scan.ensure(sizeof(int32_t) * (nvv + 1)));
    FBC_CK(isb.ensure(nvv));
    FBC_CK(cbord.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nbt, 1)));
    FBC_CK(cudaMemcpyAsync(d_eoff.p, eoff.data(), sizeof(int64_t) * eoff.size(), cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemcpyAsync(d_toff.p, toff.data(), sizeof(int64_t) * toff.size(), cudaMemcpyHostToDevice, g.st));
    if (eoff[nclusters] > 0) {
        FBC_CK(cudaMemcpyAsync(d_bd.p, bdist, sizeof(double) * (size_t)eoff[nclusters], cudaMemcpyHostToDevice, g.st));
        FBC_CK(cudaMemcpyAsync(d_bs.p, bsig, sizeof(uint64_t) * (size_t)eoff[nclusters], cudaMemcpyHostToDevice, g.st));
    }
    FBC_CK(cudaMemcpyAsync(d_bc.p, bc, sizeof(double) * (size_t)G->n, cudaMemcpyHostToDevice, g.st));
    FBC_CK(cudaMemsetAsync(thash.p, 0, sizeof(unsigned long long) * nts, g.st));
    FBC_CK(cudaMemsetAsync(tfirst.p, 0x7f, sizeof(int) * nts, g.st));
    FBC_CK(cudaMemsetAsync(isb.p, 0, nvv, g.st));
    g_aux_launches = 0;
    if (nbt > 0) {
        fbc::clu_border_map_kernel<<<grid_for(nbt), 256, 0, g.st>>>(nbt, g.c_boff.as<int64_t>(), nclusters,
                                                                    g.c_bsrc.as<int32_t>(), G->n, g.c_id.as<int32_t>(),
                                                                    g.c_lid.as<int32_t>(), cbord.as<int32_t>(),
                                                                    g.c_err.as<int>());
        fbc::cls_mark_border_kernel<<<grid_for(nbt), 256, 0, g.st>>>(nbt, g.c_boff.as<int64_t>(), nclusters,
                                                                     g.c_off.as<int64_t>(), cbord.as<int32_t>(),
                                                                     isb.as<uint8_t>());
    }
    FBC_CK(cudaGetLastError());
    int err = 0;
    FBC_CK(cudaMemcpyAsync(&err, g.c_err.p, sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    FBC_TRY(cluster_error(err));
    FBC_CK(cudaMemsetAsync(g.c_err.p, 0, sizeof(int), g.st));  // the class kernels' own bits
    fbc::ClsArgs A{};
    A.coff = g.c_off.as<int64_t>();
    A.boff = g.c_boff.as<int64_t>();
    A.eoff = d_eoff.as<int64_t>();
    A.toff = d_toff.as<int64_t>();
    A.ncl = nclusters;
    A.nv = nv;
    A.bdist = d_bd.as<double>();
    A.bsig = d_bs.as<unsigned long long>();
    A.thash = thash.as<unsigned long long>();
    A.tfirst = tfirst.as<int>();
    A.vhash = vhash.as<unsigned long long>();
    A.vrep = vrep.as<int>();
    A.err = g.c_err.as<int>();
    if (nv > 0) {
        fbc::cls_hash_kernel<<<grid_for(nv), 256, 0, g.st>>>(A);
        fbc::cls_rep_kernel<<<grid_for(nv), 256, 0, g.st>>>(A);
        fbc::cls_flag_kernel<<<grid_for(nv), 256, 0, g.st>>>(A, flag.as<int32_t>());
        FBC_CK(cudaGetLastError());
    }
    FBC_TRY(device_scan(flag.as<int32_t>(), nv, scan.as<int32_t>()));
    std::vector<int32_t> sc((size_t)nv + 1);
    FBC_CK(cudaMemcpyAsync(sc.data(), scan.p, sizeof(int32_t) * sc.size(), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaMemcpyAsync(&err, g.c_err.p, sizeof(int), cudaMemcpyDeviceToHost, g.st));
    FBC_CK(cudaStreamSynchronize(g.st));
    if (err & fbc::kClsCollision) return fail(FBC_ERR_HASH, "two different border vectors share a hash");
    if (err & fbc::kClsFull) return fail(FBC_ERR_QUEUE, "class table full (sizing)");
    const int32_t ncls = sc[(size_t)nv];
    for (int32_t c = 0; c <= nclusters; ++c) out_class_off[c] = sc[(size_t)coff[c]];
    if (ncls > 0) {
        FBC_CK(card.ensure(sizeof(int) * (size_t)ncls));
        FBC_CK(minbc.ensure(sizeof(unsigned long long) * (size_t)ncls));
        FBC_CK(pick.ensure(sizeof(int) * (size_t)ncls));
        FBC_CK(piv.ensure(sizeof(int32_t) * (size_t)ncls));
        FBC_CK(crd.ensure(sizeof(int32_t) * (size_t)ncls));
        FBC_CK(cudaMemsetAsync(card.p, 0, sizeof(int) * (size_t)ncls, g.st));
        FBC_CK(cudaMemsetAsync(minbc.p, 0xff, sizeof(unsigned long long) * (size_t)ncls, g.st));
        FBC_CK(cudaMemsetAsync(pick.p, 0x7f, sizeof(int) * (size_t)ncls, g.st));
        fbc::cls_card_kernel<<<grid_for(nv), 256, 0, g.st>>>(A, scan.as<int32_t>(), g.cgid.as<int32_t>(),
                                                             isb.as<uint8_t>(), d_bc.as<double>(), card.as<int>(),
                                                             minbc.as<unsigned long long>());
        fbc::cls_pick_kernel<<<grid_for(nv), 256, 0, g.st>>>(A, scan.as<int32_t>(), g.cgid.as<int32_t>(),
                                                             isb.as<uint8_t>(), d_bc.as<double>(),
                                                             minbc.as<unsigned long long>(), pick.as<int>());
        fbc::cls_out_kernel<<<grid_for(nv), 256, 0, g.st>>>(A, flag.as<int32_t>(), scan.as<int32_t>(),
                                                            g.cgid.as<int32_t>(), card.as<int>(), pick.as<int>(),
                                                            piv.as<int32_t>(), crd.as<int32_t>());
        FBC_CK(cudaGetLastError());
        FBC_CK(cudaMemcpyAsync(out_pivots, piv.p, sizeof(int32_t) * (size_t)ncls, cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaMemcpyAsync(out_cards, crd.p, sizeof(int32_t) * (size_t)ncls, cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
    }
    return FBC_OK;
}

int fbc_cluster_eval_batch(fbc_graph G, int32_t nclusters, const int64_t* coff,
                           const int32_t* cverts, const int64_t* border_off, const int32_t* borders,
                           int precision, int sched, double* out_intra_bc, double* out_bdist,
                           uint64_t* out_bsig, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G) return fail(FBC_ERR_INVALID_ARG, "null graph");
    FBC_TRY(check_sched(sched));
    if (border_off && !borders && nclusters > 0 && border_off[nclusters] > 0)
        return fail(FBC_ERR_INVALID_ARG, "border_off without borders");
    const double t0 = now_ms();
    if (st) std::memset(st, 0, sizeof(*st));
    Plan P;
    int64_t ent = 0;
    FBC_TRY(prepare_clusters(G, nclusters, coff, cverts, border_off, borders, precision, sched,
                             g.crp, g.cadj, g.cgid, g.cbord, P, ent, st));
    FBC_TRY(run_plan(P, st));
    FBC_TRY(download_bc(out_intra_bc, G->n, true, st));
    if (ent > 0 && (out_bdist || out_bsig)) {
        if (out_bdist)
            FBC_CK(cudaMemcpyAsync(out_bdist, g.bdist.p, sizeof(double) * (size_t)ent, cudaMemcpyDeviceToHost, g.st));
        if (out_bsig)
            FBC_CK(cudaMemcpyAsync(out_bsig, g.bsig.p, sizeof(uint64_t) * (size_t)ent, cudaMemcpyDeviceToHost, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
        if (st) st->d2h_bytes += ent * (int64_t)((out_bdist ? 8 : 0) + (out_bsig ? 8 : 0));
    }
    if (st) st->wall_ms = now_ms() - t0;
    return FBC_OK;
}

}  // extern "C"

namespace {
// Capture of a prepared cluster sweep: counter and accumulator resets, the shared-memory kernel
// for the communities that fit it, the frontier kernel (four sources per block) for the larger
// ones on a workspace of the plan's own, and the downloads into pinned memory, as two CUDA graphs
// replayed back to back (an event between them times the two kernels apart).  Communities that
// need the plain kernels (above 32K vertices, in-degrees of 65,535 or more) leave the plan
// uncaptured: fbc_plan_run then takes the general path.
template <class Prec>
int plan_capture(fbc_plan_s* p, Plan& P) {
    std::vector<char> small(P.segs.size(), 0);
    for (size_t s = 0; s < P.segs.size(); ++s)
        small[s] = P.segs[s].n <= std::min<int64_t>(g.opt.warp_max_n, 65535) && P.seg_maxw[s] < 65536 &&
                   P.seg_m[s] < ((int64_t)1 << 30);
    for (;;) {  // the shared-memory layout fits at least two warps of the largest small segment
        int nm = 0, mm = 0, arg = -1;
        for (size_t s = 0; s < P.segs.size(); ++s)
            if (small[s]) {
                mm = std::max<int>(mm, (int)P.seg_m[s]);
                if (P.segs[s].n >= nm) { nm = P.segs[s].n; arg = (int)s; }
            }
        if (arg < 0 || small_fits(nm, mm, 2)) break;
        small[arg] = 0;
    }
    std::vector<std::vector<Unit>> by_seg(P.segs.size());
    std::vector<Unit> uw, ub;
    int nw_max = 0, mw_max = 0, nw_min = 1 << 30, nb_max = 0;
    for (const Unit& u : P.units) {
        const Seg& sg = P.segs[u.seg];
        if (small[u.seg]) {
            by_seg[u.seg].push_back(u);
            nw_max = std::max(nw_max, sg.n);
            nw_min = std::min(nw_min, sg.n);
            mw_max = std::max<int>(mw_max, (int)P.seg_m[u.seg]);
        } else {
            if (sg.n > 32768 || P.seg_maxindeg[u.seg] >= 65535) return FBC_OK;  // general path
            ub.push_back(u);
            nb_max = std::max(nb_max, sg.n);
        }
    }
    for (auto& v : by_seg) uw.insert(uw.end(), v.begin(), v.end());
    std::stable_sort(ub.begin(), ub.end(), [&](const Unit& a, const Unit& b) { return P.segs[a.seg].n > P.segs[b.seg].n; });
    const size_t n8 = sizeof(double) * (size_t)std::max<int64_t>(p->n, 1);
    const size_t e8 = 8 * (size_t)std::max<int64_t>(p->ent, 1);
    FBC_CK(p->segs.ensure(sizeof(Seg) * P.segs.size()));
    FBC_CK(p->bc.ensure(n8));
    FBC_CK(p->bdist.ensure(e8));
    FBC_CK(p->bsig.ensure(e8));
    FBC_CK(p->ctr.ensure(64));
    FBC_CK(p->retry.ensure(sizeof(fbc::RetryRec) * P.units.size()));
    FBC_CK(cudaMemcpyAsync(p->segs.p, P.segs.data(), sizeof(Seg) * P.segs.size(), cudaMemcpyHostToDevice, g.st));
    KParams base{};
    base.segs = p->segs.as<Seg>();
    base.bc = p->bc.as<double>();
    base.bdist = p->bdist.as<double>();
    base.bsig = p->bsig.as<unsigned long long>();
    base.err = (int*)(p->ctr.as<unsigned long long>() + 2);
    base.retry_count = base.err + 1;
    base.retry = p->retry.as<fbc::RetryRec>();
    base.retry_cap = (int32_t)P.units.size();
    base.iter_mult = (int32_t)g.opt.iter_mult;
    SmallCfg cfg;
    fbc::SmallParams S{};
    if (!uw.empty()) {
        FBC_TRY(small_config(P, uw, nw_max, mw_max, nw_min, cfg));
        FBC_CK(p->units.ensure(sizeof(Unit) * uw.size()));
        FBC_CK(p->chunks.ensure(sizeof(fbc::Chunk) * cfg.chunks.size()));
        FBC_CK(cudaMemcpyAsync(p->units.p, uw.data(), sizeof(Unit) * uw.size(), cudaMemcpyHostToDevice, g.st));
        FBC_CK(cudaMemcpyAsync(p->chunks.p, cfg.chunks.data(), sizeof(fbc::Chunk) * cfg.chunks.size(),
                               cudaMemcpyHostToDevice, g.st));
        S.k = base;
        S.k.units = p->units.as<Unit>();
        S.k.nunits = (int64_t)uw.size();
        S.chunks = p->chunks.as<fbc::Chunk>();
        S.nchunks = (int32_t)cfg.chunks.size();
        S.nmax = nw_max;
        S.mmax = mw_max;
        S.smem = (int32_t)cfg.dyn;
        S.next_chunk = p->ctr.as<unsigned long long>() + 1;
        FBC_CK(cudaFuncSetAttribute(fbc::small_seg_kernel<Prec>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.dyn));
    }
    BlockCfg bc;
    KParams K = base;
    if (!ub.empty()) {
        FBC_TRY(block_config<Prec>(P, ub, nb_max, false, false, ws_budget(), bc));
        if (!bc.fr) return FBC_OK;
        FBC_CK(p->bunits.ensure(sizeof(Unit) * bc.units.size()));
        FBC_CK(cudaMemcpyAsync(p->bunits.p, bc.units.data(), sizeof(Unit) * bc.units.size(), cudaMemcpyHostToDevice,
                               g.st));
        FBC_CK(p->ws.ensure((size_t)(bc.slots * bc.stride), true, g.st));  // zeroed: fresh slots
        K.units = p->bunits.as<Unit>();
        K.nunits = (int64_t)bc.units.size() / bc.K;
        K.cnt_bits = bc.cnt_bits;
        K.next_unit = p->ctr.as<unsigned long long>() + 0;
        K.ws = p->ws.as<char>();
        K.ws_stride = bc.stride;
        K.ws_n = (int32_t)(nb_max * bc.K);
    }
    FBC_CK(cudaStreamSynchronize(g.st));
    for (const Unit& u : uw) p->wbytes += 40.0 * (double)P.seg_m[u.seg] + 52.0 * P.segs[u.seg].n;
    for (const Unit& u : ub) p->bbytes += 40.0 * (double)P.seg_m[u.seg] + 52.0 * P.segs[u.seg].n;
    p->wunits = (int64_t)uw.size();
    p->bunits_n = (int64_t)ub.size();
    p->launches = (uw.empty() ? 0 : 1) + (ub.empty() ? 0 : 1);
    FBC_CK(cudaStreamBeginCapture(g.st, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(p->ctr.p, 0, 64, g.st);
    cudaMemsetAsync(p->bc.p, 0, n8, g.st);
    if (!uw.empty()) fbc::small_seg_kernel<Prec><<<(unsigned)cfg.blocks, 32 * cfg.wpb, (size_t)cfg.dyn, g.st>>>(S);
    cudaError_t ce = cudaStreamEndCapture(g.st, &p->graph[0]);
    if (ce != cudaSuccess) return fail(FBC_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
    FBC_CK(cudaGraphInstantiate(&p->exec[0], p->graph[0], 0));
    FBC_CK(cudaStreamBeginCapture(g.st, cudaStreamCaptureModeThreadLocal));
    if (!ub.empty()) launch_units(bc, K, g.st);
    cudaMemcpyAsync(p->h_bc, p->bc.p, n8, cudaMemcpyDeviceToHost, g.st);
    if (p->ent > 0) {
        cudaMemcpyAsync(p->h_bdist, p->bdist.p, e8, cudaMemcpyDeviceToHost, g.st);
        cudaMemcpyAsync(p->h_bsig, p->bsig.p, e8, cudaMemcpyDeviceToHost, g.st);
    }
    cudaMemcpyAsync(p->h_ctl, (char*)p->ctr.p + 16, 8, cudaMemcpyDeviceToHost, g.st);
    ce = cudaStreamEndCapture(g.st, &p->graph[1]);
    if (ce != cudaSuccess) return fail(FBC_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
    FBC_CK(cudaGraphInstantiate(&p->exec[1], p->graph[1], 0));
    p->captured = true;
    return FBC_OK;
}

}  // namespace

extern "C" {

int fbc_cluster_plan_create(fbc_graph G, int32_t nclusters, const int64_t* coff, const int32_t* cverts,
                            const int64_t* border_off, const int32_t* borders, int precision,
                            fbc_plan* out) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G || !out || nclusters < 0 || !coff) return fail(FBC_ERR_INVALID_ARG, "null argument");
    if (precision != FBC_PREC_FP64 && precision != FBC_PREC_FP32C) return fail(FBC_ERR_INVALID_ARG, "unknown precision");
    *out = nullptr;
    auto* p = new fbc_plan_s();
    std::unique_ptr<fbc_plan_s> guard(p);
    p->G = G;
    p->prec = precision;
    p->n = G->n;
    p->coff.assign(coff, coff + nclusters + 1);
    p->cverts.assign(cverts, cverts + coff[nclusters]);
    if (border_off) {
        p->boff.assign(border_off, border_off + nclusters + 1);
        p->borders.assign(borders, borders + border_off[nclusters]);
    }
    Plan P;
    FBC_TRY(prepare_clusters(G, nclusters, coff, cverts, border_off, borders, precision, FBC_SCHED_BATCHED,
                             p->crp, p->cadj, p->cgid, p->cbord, P, p->ent, nullptr));
    for (const Unit& u : P.units) p->relax += (double)P.seg_m[u.seg];
    p->nunits = (int64_t)P.units.size();
    const size_t n8 = sizeof(double) * (size_t)std::max<int64_t>(p->n, 1);
    const size_t e8 = 8 * (size_t)std::max<int64_t>(p->ent, 1);
    FBC_CK(cudaMallocHost(&p->h_bc, n8));
    FBC_CK(cudaMallocHost(&p->h_bdist, e8));
    FBC_CK(cudaMallocHost(&p->h_bsig, e8));
    FBC_CK(cudaMallocHost(&p->h_ctl, 64));
    if (!P.units.empty()) {
        if (precision == FBC_PREC_FP64) FBC_TRY(plan_capture<fbc::PrecF64>(p, P));
        else FBC_TRY(plan_capture<fbc::PrecDF32>(p, P));
    }
    *out = guard.release();
    return FBC_OK;
}

int fbc_plan_run(fbc_plan p, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!p) return fail(FBC_ERR_INVALID_ARG, "null plan");
    const double t0 = now_ms();
    if (st) std::memset(st, 0, sizeof(*st));
    if (p->captured) {
        FBC_CK(cudaEventRecord(g.ev0, g.st));
        FBC_CK(cudaGraphLaunch(p->exec[0], g.st));
        FBC_CK(cudaEventRecord(g.evm, g.st));
        FBC_CK(cudaGraphLaunch(p->exec[1], g.st));
        FBC_CK(cudaEventRecord(g.ev1, g.st));
        FBC_CK(cudaStreamSynchronize(g.st));
        if (p->h_ctl[0] == 0 && p->h_ctl[1] == 0) {
            if (st) {
                float ms = 0.f, mw = 0.f;
                FBC_CK(cudaEventElapsedTime(&ms, g.ev0, g.ev1));
                FBC_CK(cudaEventElapsedTime(&mw, g.ev0, g.evm));
                st->kernel_ms = ms;
                st->warp_ms = p->wunits ? mw : 0.0;
                st->block_ms = p->bunits_n ? ms - mw : 0.0;
                st->units = p->nunits;
                st->warp_units = p->wunits;
                st->block_units = p->bunits_n;
                st->relaxations = p->relax;
                st->warp_bytes = p->wbytes;
                st->block_bytes = p->bbytes;
                st->launches = p->launches;
                st->d2h_bytes = 8 * (p->n + 2 * p->ent);
                st->wall_ms = now_ms() - t0;
            }
            return FBC_OK;
        }
        if (p->h_ctl[0] != 0 && p->h_ctl[1] == 0) return map_err(p->h_ctl[0]);
    }
    // not captured, or path counts needed a wider representation: the general path
    std::memset(p->h_bc, 0, sizeof(double) * (size_t)p->n);
    return fbc_cluster_eval_batch(p->G, (int32_t)p->coff.size() - 1, p->coff.data(), p->cverts.data(),
                                  p->boff.empty() ? nullptr : p->boff.data(),
                                  p->borders.empty() ? nullptr : p->borders.data(), p->prec,
                                  FBC_SCHED_BATCHED, p->h_bc, p->h_bdist, p->h_bsig, st);
}

int fbc_plan_results(fbc_plan p, const double** intra_bc, const double** border_dist,
                     const uint64_t** border_sigma, int64_t* entries, int32_t* captured) {
    if (!p) return fail(FBC_ERR_INVALID_ARG, "null plan");
    if (intra_bc) *intra_bc = p->h_bc;
    if (border_dist) *border_dist = p->h_bdist;
    if (border_sigma) *border_sigma = p->h_bsig;
    if (entries) *entries = p->ent;
    if (captured) *captured = p->captured ? 1 : 0;
    return FBC_OK;
}

int fbc_plan_free(fbc_plan p) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!p) return FBC_OK;
    delete p;
    return FBC_OK;
}

int fbc_multi_exact_bc(int32_t ngraphs, const fbc_graph* graphs, int precision, int sched,
                       double* const* out_bc, fbc_stats* st) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (ngraphs < 0 || (ngraphs > 0 && (!graphs || !out_bc))) return fail(FBC_ERR_INVALID_ARG, "null argument");
    FBC_TRY(check_sched(sched));
    const double t0 = now_ms();
    if (st) std::memset(st, 0, sizeof(*st));
    Plan P;
    P.prec = precision;
    P.sched = sched;
    std::vector<int64_t> base((size_t)ngraphs + 1, 0);
    for (int32_t i = 0; i < ngraphs; ++i) {
        if (!graphs[i]) return fail(FBC_ERR_INVALID_ARG, "null graph in batch");
        Seg sg;
        const int32_t* map = nullptr;
        FBC_TRY(batched_graph_seg(graphs[i], base[i], sched, sg, map));
        P.segs.push_back(sg);
        P.seg_m.push_back(graphs[i]->m);
        P.seg_maxw.push_back(graphs[i]->maxw);
        P.seg_maxindeg.push_back(graphs[i]->maxindeg);
        for (int32_t s = 0; s < graphs[i]->n; ++s) P.units.push_back(Unit{i, s, 1.0, -1});
        base[i + 1] = base[i] + graphs[i]->n;
    }
    P.bc_len = base[ngraphs];
    FBC_TRY(run_plan(P, st));
    std::vector<double> all((size_t)std::max<int64_t>(P.bc_len, 1));
    FBC_TRY(download_bc(all.data(), P.bc_len, false, st));
    for (int32_t i = 0; i < ngraphs; ++i)
        std::copy(all.begin() + base[i], all.begin() + base[i + 1], out_bc[i]);
    if (st) st->wall_ms = now_ms() - t0;
    return FBC_OK;
}

int fbc_sssp_debug(fbc_graph G, int32_t source, int32_t* out_dist, uint64_t* out_sigma,
                   double* out_delta, int32_t* out_npred) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevGuard dg_;
    FBC_TRY(check_init(dg_));
    if (!G || source < 0 || source >= G->n) return fail(FBC_ERR_INVALID_ARG, "bad graph or source");
    const size_t n = (size_t)G->n;
    FBC_CK(g.dbg.ensure(n * (4 + 8 + 8) + 512));
    char* base = g.dbg.as<char>();
    Plan P;
    P.prec = FBC_PREC_FP64;
    P.sched = (int)g.opt.debug_sched;
    P.segs.push_back(whole_graph_seg(G, 0));
    P.seg_m.push_back(G->m);
    P.seg_maxw.push_back(G->maxw);
    P.seg_maxindeg.push_back(G->maxindeg);
    P.units.push_back(Unit{0, source, 1.0, -1});
    P.bc_len = G->n;
    P.dbg_sig = (unsigned long long*)base;
    P.dbg_dlt = (double*)(base + n * 8);
    P.dbg_dist = (int32_t*)(base + n * 16);
    FBC_TRY(run_plan(P, nullptr));
    std::vector<int32_t> dist(n);
    FBC_CK(cudaMemcpy(dist.data(), P.dbg_dist, 4 * n, cudaMemcpyDeviceToHost));
    if (out_dist) std::copy(dist.begin(), dist.end(), out_dist);
    if (out_sigma) FBC_CK(cudaMemcpy(out_sigma, P.dbg_sig, 8 * n, cudaMemcpyDeviceToHost));
    if (out_delta) FBC_CK(cudaMemcpy(out_delta, P.dbg_dlt, 8 * n, cudaMemcpyDeviceToHost));
    if (out_npred) {
        FBC_TRY(ensure_host_csr(G));
        std::fill(out_npred, out_npred + n, 0);
        for (int32_t v = 0; v < G->n; ++v) {
            if (dist[v] < 0) continue;
            for (int64_t e = G->h_rp[v]; e < G->h_rp[v + 1]; ++e) {
                const int32_t x = G->h_col[e];
                if (dist[x] >= 0 && (int64_t)dist[v] + G->h_w[e] == dist[x]) out_npred[x]++;
            }
        }
    }
    return FBC_OK;
}

}  // extern "C"
