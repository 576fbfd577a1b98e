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
template <class Prec>
__global__ void __launch_bounds__(1024) noalloc_kernel(fbc::Seg sg, fbc::Unit u, fbc::KParams P,
                                                       char* base) {
    __shared__ fbc::Ctl C;
    int* ctl = (int*)(base + kCtlOff);  // [0] status bits, [1] bad-input flag, [2] max weight
    if (threadIdx.x == 0) {
        *(fbc::Seg*)(base + kSegOff) = sg;
        ctl[0] = 0;
        ctl[1] = 0;
        ctl[2] = 0;
    }
    __syncthreads();
    const int n = sg.n;
    const int m = sg.rp[n];
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        P.bc[v] = 0.0;
        const int a = sg.rp[v], b = sg.rp[v + 1];
        if (a < 0 || b < a || b > m) atomicOr(ctl + 1, 1);
    }
    for (int e = threadIdx.x; e < m; e += blockDim.x) {
        const int2 a = sg.adj[e];
        if (a.x < 0 || a.x >= n || a.y <= 0) atomicOr(ctl + 1, 1);
        else atomicMax(ctl + 2, a.y);
    }
    __syncthreads();
    if (ctl[1] || (double)n * (double)ctl[2] > 2147483646.0) return;
    fbc::State<Prec> S = fbc::state_carve<Prec>(base + kStateOff, n);
    fbc::state_init<fbc::BlockGroup, Prec>(S, n);
    unsigned epoch = 1u;
    fbc::run_unit<fbc::BlockGroup, Prec>(P, u, S, C, epoch, n);
}

}  // namespace

extern "C" int fbc_single_source_noalloc(int32_t n, const int32_t* d_row_ptr, const int32_t* d_adj,
                                         int32_t source, int precision, double* d_dep,
                                         void* stream) {
    if (n <= 0 || n > FBC_NOALLOC_MAX_N)
        return nfail(FBC_ERR_RANGE, "n must be in [1, " + std::to_string(FBC_NOALLOC_MAX_N) +
                                        "] for fbc_single_source_noalloc (size of its fixed work area)");
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
    if (precision == FBC_PREC_FP64)
        noalloc_kernel<fbc::PrecF64><<<1, 512, 0, st>>>(sg, u, P, base);
    else
        noalloc_kernel<fbc::PrecDF32><<<1, 512, 0, st>>>(sg, u, P, base);
    e = cudaGetLastError();
    if (e != cudaSuccess) return nfail(FBC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    int ctl[3] = {0, 0, 0};
    e = cudaMemcpyAsync(ctl, base + kCtlOff, sizeof ctl, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nfail(FBC_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
    if (ctl[1]) return nfail(FBC_ERR_INVALID_ARG, "device CSR has an out-of-range id or a weight <= 0");
    if ((double)n * (double)ctl[2] > 2147483646.0)
        return nfail(FBC_ERR_RANGE, "n * max_weight exceeds the int32 distance range");
    if (ctl[0] & fbc::kErrQueue) return nfail(FBC_ERR_QUEUE, "device work queue overflow");
    if (ctl[0] & fbc::kErrIter) return nfail(FBC_ERR_ITER_LIMIT, "a device loop reached its iteration bound");
    if (ctl[0] & fbc::kErrSigma) return nfail(FBC_ERR_SIGMA_OVERFLOW, "a shortest-path count exceeded 2^64-1");
    return FBC_OK;
}
