// fbc_single_source_noalloc: one source's Brandes dependency on a graph that the caller
// already holds in device memory, computed without allocating anything.
//
// Some callers cannot call cudaMalloc at the point where they need a dependency vector:
// code running inside a framework's memory pool or a custom allocator that owns every
// device byte, code that must not grow the device footprint after start-up, or a
// library that was handed device buffers and a stream by its host application and may not
// take more.  For them this entry point takes device pointers for the graph and the
// output, uses the caller's stream, and keeps its per-source work area in a file-scope
// device array of fixed size (fbc_noalloc_scratch below), which every GPU that loads the
// library holds until the process exits.
//
// The kernel is the plain schedule's block-per-source kernel (run_unit<BlockGroup>) with
// its global-memory slot placed in that array.
#include "fbc_gpu.h"

#include <cstring>
#include <mutex>
#include <string>

#include "brandes_kernels.cuh"

// Shared with the rest of the library (fbc_gpu.cu): the calling thread's last error message.
void fbc_internal_set_error(const char* msg);

namespace {

constexpr int64_t kAl = 256;
constexpr int64_t al256(int64_t x) { return (x + kAl - 1) & ~(kAl - 1); }
// Bytes of one per-source state (state_bytes in brandes_kernels.cuh, 8-byte delta).
constexpr int64_t state_bytes_8(int64_t cap) {
    return al256(cap * 4) + al256(cap * 8) + al256(cap * 8) + 4 * al256((cap + 1) * 4) + 2 * al256(cap * 4) +
           al256(cap * 4);
}
// Layout of the array: [segment record][control words][per-source state].
constexpr int64_t kSegOff = 0;
constexpr int64_t kCtlOff = 256;
constexpr int64_t kStateOff = 512;
constexpr int64_t kScratchBytes = kStateOff + state_bytes_8(FBC_NOALLOC_MAX_N);

// The scratch array.  In host code this name is only a host-side stand-in for the symbol,
// not a device address: the kernel is always given the address that cudaGetSymbolAddress
// returned for the current device.
static __device__ __align__(256) char fbc_noalloc_scratch[kScratchBytes];

int nfail(int code, const std::string& m) {
    fbc_internal_set_error(m.c_str());  // read back through fbc_last_error_string
    return code;
}

// Per-device address of the array, looked up once per device with that device current.
constexpr int kMaxDev = 64;
std::mutex g_addr_mu;
char* g_addr[kMaxDev] = {};

int scratch_address(int dev, char** out) {
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (dev < 0 || dev >= kMaxDev) return nfail(FBC_ERR_INVALID_ARG, "device id beyond the supported range");
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, fbc_noalloc_scratch);
        if (e != cudaSuccess)
            return nfail(FBC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_addr[dev] = (char*)p;
    }
    *out = g_addr[dev];
    return FBC_OK;
}

// One block: validates the device CSR, clears the output and the state (the array keeps the
// previous call's contents), runs the source, and leaves the status in the control words.
// The CSR checks read only the caller's buffers: row_ptr[0..n] and adj[0..m), m given by the
// caller; a row is walked only after its bounds were found inside [0, m].  kSigF64: path counts
// held as FP64 (the reference's own representation), for sources whose uint64 counts overflow.
template <class Prec, bool kSigF64>
__global__ void __launch_bounds__(1024) noalloc_kernel(fbc::Seg sg, int m, fbc::Unit u, fbc::KParams P,
                                                       char* base) {
    __shared__ fbc::Ctl C;
    int* ctl = (int*)(base + kCtlOff);  // [0] status bits, [1] bad-input flag, [2] max weight
    if (threadIdx.x == 0) {
        *(fbc::Seg*)(base + kSegOff) = sg;
        ctl[0] = 0;
        ctl[1] = (sg.rp[0] != 0 || sg.rp[sg.n] != m) ? 1 : 0;
        ctl[2] = 0;
    }
    __syncthreads();
    const int n = sg.n;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        P.bc[v] = 0.0;
        const int a = sg.rp[v], b = sg.rp[v + 1];
        if (a < 0 || b < a || b > m) {
            atomicOr(ctl + 1, 1);
            continue;
        }
        // destinations in range and strictly ascending (sorted, no repeats), weights > 0
        int prev = -1, wmax = 0;
        bool ok = true;
        for (int e = a; e < b; ++e) {
            const int2 x = sg.adj[e];
            ok = ok && x.x > prev && x.x < n && x.y > 0;
            prev = x.x;
            wmax = max(wmax, x.y);
        }
        if (!ok) atomicOr(ctl + 1, 1);
        else if (wmax > 0) atomicMax(ctl + 2, wmax);
    }
    __syncthreads();
    if (ctl[1] || (double)n * (double)ctl[2] > 2147483646.0) return;
    fbc::State<Prec> S = fbc::state_carve<Prec>(base + kStateOff, n);
    fbc::state_init<fbc::BlockGroup, Prec>(S, n);
    unsigned epoch = 1u;
    fbc::run_unit<fbc::BlockGroup, Prec, kSigF64>(P, u, S, C, epoch, n);
}

template <bool kSigF64>
void launch_noalloc(int precision, const fbc::Seg& sg, int m, const fbc::Unit& u, const fbc::KParams& P, char* base,
                    cudaStream_t st) {
    if (precision == FBC_PREC_FP64)
        noalloc_kernel<fbc::PrecF64, kSigF64><<<1, 512, 0, st>>>(sg, m, u, P, base);
    else
        noalloc_kernel<fbc::PrecDF32, kSigF64><<<1, 512, 0, st>>>(sg, m, u, P, base);
}

// Launch, then read the control words back (the call's one synchronisation, on the caller's stream).
int run_noalloc(bool sig_f64, int precision, const fbc::Seg& sg, int m, const fbc::Unit& u, const fbc::KParams& P,
                char* base, cudaStream_t st, int ctl[3]) {
    if (sig_f64) launch_noalloc<true>(precision, sg, m, u, P, base, st);
    else launch_noalloc<false>(precision, sg, m, u, P, base, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return nfail(FBC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(ctl, base + kCtlOff, 3 * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nfail(FBC_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
    return FBC_OK;
}

}  // namespace

extern "C" int fbc_single_source_noalloc(int32_t n, int64_t m, const int32_t* d_row_ptr, const int32_t* d_adj,
                                         int32_t source, int precision, double* d_dep, void* stream) {
    if (n <= 0 || n > FBC_NOALLOC_MAX_N)
        return nfail(FBC_ERR_RANGE, "n must be in [1, " + std::to_string(FBC_NOALLOC_MAX_N) +
                                        "] for fbc_single_source_noalloc (size of its fixed work area)");
    if (m < 0 || m > 2147483646) return nfail(FBC_ERR_INVALID_ARG, "edge count out of range");
    if (!d_row_ptr || !d_adj || !d_dep) return nfail(FBC_ERR_INVALID_ARG, "null device pointer");
    if (source < 0 || source >= n) return nfail(FBC_ERR_INVALID_ARG, "source out of range");
    if (precision != FBC_PREC_FP64 && precision != FBC_PREC_FP32C)
        return nfail(FBC_ERR_INVALID_ARG, "unknown precision");
    static_assert(kStateOff + state_bytes_8(FBC_NOALLOC_MAX_N) <= kScratchBytes, "scratch too small");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nfail(FBC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    char* base = nullptr;
    if (int rc = scratch_address(dev, &base)) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    fbc::Seg sg{};
    sg.rp = d_row_ptr;
    sg.adj = (const int2*)d_adj;
    sg.gid = nullptr;
    sg.border = nullptr;
    sg.out_base = 0;
    sg.n = n;
    sg.nb = 0;
    sg.delta = 64;  // bucket width: any width gives the same results, 64 suits road weights
    fbc::KParams P{};
    P.segs = (const fbc::Seg*)(base + kSegOff);
    P.bc = d_dep;
    P.err = (int*)(base + kCtlOff);
    P.iter_mult = 16;
    const fbc::Unit u{0, source, 1.0, -1};
    int ctl[3] = {0, 0, 0};
    if (int rc = run_noalloc(false, precision, sg, (int)m, u, P, base, st, ctl)) return rc;
    // path counts beyond 2^64 - 1: the source again with FP64 counts, as fbc_single_source does
    // (the kernel stopped before its dependency pass and the relaunch clears everything again)
    if (ctl[1] == 0 && (ctl[0] & fbc::kErrSigma))
        if (int rc = run_noalloc(true, precision, sg, (int)m, u, P, base, st, ctl)) return rc;
    if (ctl[1])
        return nfail(FBC_ERR_INVALID_ARG,
                     "device CSR is malformed: row_ptr[0] != 0, row_ptr[n] != m, a row outside [0, m], "
                     "a destination out of range or not ascending, or a weight <= 0");
    if ((double)n * (double)ctl[2] > 2147483646.0)
        return nfail(FBC_ERR_RANGE, "n * max_weight exceeds the int32 distance range");
    if (ctl[0] & fbc::kErrQueue) return nfail(FBC_ERR_QUEUE, "device work queue overflow");
    if (ctl[0] & fbc::kErrIter) return nfail(FBC_ERR_ITER_LIMIT, "a device loop reached its iteration bound");
    if (ctl[0] & fbc::kErrSigma) return nfail(FBC_ERR_SIGMA_OVERFLOW, "a shortest-path count overflowed");
    return FBC_OK;
}
