// Allocation-free block-Jacobi PCG: the stand-alone solve of bcsr_pcg.h with its workspace in
// a fixed, file-scope device array instead of device memory allocated for each call.  The
// reference has no counterpart of this entry point.
//
// Who needs it: callers that must not allocate device memory while they run.  One kind has
// all of its device memory reserved up front (a caching allocator, or a fixed per-process
// budget, already holds the rest of HBM, so a cudaMalloc would fail or force the cache to be
// given back).  The other cannot afford what cudaFree does besides freeing: it waits for the
// whole device, so the caller's other streams stall until it returns.
//
// Rules of use:
//  * Single precision, at most kNoAllocMaxBlocks = 65,536 block rows (196,608 unknowns).  A
//    larger system is refused with an error before anything is launched.
//  * The scratch array is one per device and process, and every call uses all of it.  Calls
//    that overlap on one device (two host threads, or two streams) race on it and give wrong
//    results: run them one after the other.  Each call returns with its stream synchronized.
//  * Set-up: the first call on a device, with that device current, looks up the array's
//    device address (cudaGetSymbolAddress) and caches it together with the device's current
//    context.  A call that finds another context current (after cudaDeviceReset, or a new
//    primary context) looks the address up again, so a cached address never outlives the
//    context it belongs to.  If that first call is the set-up step of a program that later
//    captures streams, it must come before any stream capture.
//  * Device assumption: the reduction partials have room for kNoAllocPartials = 2,048
//    per-block sums.  The widest PCG launch is one block of 256 threads per resident slot,
//    i.e. SMs x resident blocks per SM (GB300: 152 x 8 = 1,216).  A device with room for more
//    resident blocks than 2,048 is refused by run_bcsr_pcg before any launch.
//  * What must be zero when the kernels start: the eight completion tickets of the
//    reductions and the missing-diagonal counter.  Every call clears them on its stream
//    (cudaMemsetAsync / cudaMemcpyAsync into the array) before its first kernel.  Everything
//    else in the array is written before it is read.
#include "bcsr_pcg.h"

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

namespace {

constexpr int kNoAllocMaxBlocks = 65536;
// Room for the per-block partial sums of the widest PCG launch (152 SMs x 8 blocks of 256
// threads = 1,216 on GB300); run_bcsr_pcg checks the real grid against it.
constexpr unsigned kNoAllocPartials = 2048;
constexpr size_t kNoAllocBytes = symxg::bcsr_pcg_workspace_size(kNoAllocMaxBlocks, kNoAllocPartials, sizeof(float));

}  // namespace

// The whole workspace: about 9.5 MB.
static __device__ __align__(256) unsigned char g_pcg_noalloc_scratch[kNoAllocBytes];

namespace symxg {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct ScratchAddress {
    void* context = nullptr;  // the context the address was looked up in
    void* address = nullptr;
};
ScratchAddress g_scratch_address[kMaxDevices];

// The current context, or null before the runtime has made one current (driver entry point
// cuCtxGetCurrent, resolved at run time like the rest of this library's driver calls, so the
// library still loads without a driver).
void* current_context()
{
    using CtxGetCurrent = int (*)(void**);
    static CtxGetCurrent fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<CtxGetCurrent>(p);
    }();
    void* ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of the scratch array in the current device's current context (looked up
// once per device, and again whenever that device's context has changed).
void* scratch_on_current_device()
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("bcsr_pcg_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchAddress& a = g_scratch_address[dev];
    void* ctx = current_context();
    if (ctx && a.address && a.context == ctx) return a.address;
    // first call in this context: the lookup also makes the runtime's context current if no
    // context was yet
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch);
    if (e != cudaSuccess || !p)
        throw std::runtime_error(std::string("bcsr_pcg_noalloc: cudaGetSymbolAddress of the scratch array: ") +
                                 cudaGetErrorString(e));
    ctx = current_context();
    if (!ctx) throw std::runtime_error("bcsr_pcg_noalloc: no current CUDA context");
    a.context = ctx;
    a.address = p;
    return p;
}

}  // namespace

int bcsr_pcg_noalloc_max_blocks() { return kNoAllocMaxBlocks; }

BcsrPcgResult run_bcsr_pcg_noalloc_f32(int n_blocks, const int32_t* row_ptr, const int32_t* cols, const float* vals,
                                       int64_t vals_stride, const float* b, float* x, double abs_tol, double rel_tol,
                                       int max_iterations, cudaStream_t s)
{
    if (n_blocks > kNoAllocMaxBlocks)
        throw std::invalid_argument("bcsr_pcg_noalloc: " + std::to_string(n_blocks) +
                                    " block rows exceed the maximum of " + std::to_string(kNoAllocMaxBlocks) +
                                    " of the allocation-free solver");
    if (n_blocks == 0) {
        BcsrPcgResult r;
        r.converged = 1;
        return r;
    }
    void* ws = scratch_on_current_device();
    return run_bcsr_pcg<float>(n_blocks, row_ptr, cols, vals, vals_stride, b, x, abs_tol, rel_tol, max_iterations, ws,
                               kNoAllocBytes, kNoAllocPartials, s);
}

}  // namespace symxg
