// anl_static.cu -- the compliance dot product without any device allocation.
//
// Who needs this: callers that cannot call cudaMalloc at the point where they need the
// compliance. Examples are a memory-pool hook or allocator callback (which must not
// re-enter the allocator), embedders whose framework owns the whole device memory pool and
// hands out only the tensors it created, and real-time loops that must not risk an
// allocation (or its implicit device synchronisation) in the middle of a step. They cannot
// create an anl_ctx either, because anl_ctx_create allocates the solver workspaces. (Code
// inside a CUDA host function or stream callback may make no CUDA call at all, so it cannot
// use this entry point either.)
//
// anl_dot_static gives them the same FP64 dot product as anl_dot (the compliance f . u of a
// SIMP iteration) with caller-owned inputs and output. The reduction scratch (one partial
// sum per CTA and a ticket counter) is a fixed array in this library's device memory. Every
// GPU that loads the library holds it (33 KB) until the process exits.
#include <mutex>

#include "anl_common.cuh"

namespace anl {

namespace {

constexpr int kStaticThreads = 256;
constexpr int kStaticBlocks = 4096;                   // partial sums the scratch can hold
constexpr int64_t kStaticChunk = 65536;               // values reduced by one CTA
constexpr int64_t kStaticMaxN = (int64_t)kStaticBlocks * kStaticChunk;  // 268,435,456 values
constexpr int kScratchWords = kStaticBlocks + 32;     // partials, then the ticket counter

// File-scope scratch shared by every call on a device: partials[0..kStaticBlocks) and the
// ticket counter in word kStaticBlocks. Host code must not take its address directly (the
// host-side name is only a stand-in); every call asks the runtime for the device address in
// the current device's context (cheap once the module is loaded, and never stale after a
// device reset or under another context). The lookup holds the library's device lock, as
// every call that may load a module or synchronise does, so it cannot invalidate a graph
// capture running on another thread.
static __device__ __align__(256) double g_static_scratch[kScratchWords];

int scratch_on_current_device(double** out) {
    void* p = nullptr;
    cudaError_t e;
    {
        std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
        e = cudaGetSymbolAddress(&p, g_static_scratch);
    }
    if (e != cudaSuccess || p == nullptr) {
        int dev = -1;
        cudaGetDevice(&dev);
        set_error("anl_dot_static: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
        return ANL_ERR_CUDA;
    }
    *out = (double*)p;
    return ANL_OK;
}

// One CTA reduces one chunk of kStaticChunk values (FP64 products and sums); the last CTA
// to finish adds the partial sums in CTA order, so the result does not depend on timing.
__global__ void __launch_bounds__(kStaticThreads) k_dot_static(const double* a, const double* b, int64_t n,
                                                               double* scratch, double* out) {
    __shared__ double sm[kStaticThreads / 32];
    const int64_t lo = (int64_t)blockIdx.x * kStaticChunk;
    const int64_t hi = lo + kStaticChunk < n ? lo + kStaticChunk : n;
    double v[1] = {0.0};
    for (int64_t i = lo + threadIdx.x; i < hi; i += kStaticThreads) v[0] = fma(a[i], b[i], v[0]);
    block_sum<1, kStaticThreads>(v, sm, threadIdx.x);
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + kStaticBlocks);
    __shared__ double res[1];
    if (finish_reduction<1, kStaticThreads>(v, blockIdx.x, gridDim.x, scratch, counter, res, threadIdx.x, sm)) {
        if (threadIdx.x == 0) *out = res[0];
    }
}

}  // namespace

}  // namespace anl

extern "C" int anl_dot_static(const double* a, const double* b, int64_t n, double* out, anl_stream_t stream) {
    using namespace anl;
    if (!a || !b || !out || n < 0) {
        set_error("anl_dot_static: null pointer or negative length");
        return ANL_ERR_BADARG;
    }
    if (n > kStaticMaxN) {
        set_error("anl_dot_static: %lld values exceed the maximum of %lld (the fixed scratch holds %d partial "
                  "sums of %lld values each); use anl_dot with a context for longer vectors",
                  (long long)n, (long long)kStaticMaxN, kStaticBlocks, (long long)kStaticChunk);
        return ANL_ERR_BADARG;
    }
    const cudaStream_t s = (cudaStream_t)stream;
    if (n == 0) {
        ANL_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
        return ANL_OK;
    }
    double* scratch = nullptr;
    ANL_TRY(scratch_on_current_device(&scratch));
    // the ticket counter must start at zero; the partials are overwritten by every CTA
    ANL_CUDA(cudaMemsetAsync(scratch + kStaticBlocks, 0, sizeof(unsigned), s));
    const int blocks = (int)((n + kStaticChunk - 1) / kStaticChunk);
    k_dot_static<<<blocks, kStaticThreads, 0, s>>>(a, b, n, scratch, out);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}
