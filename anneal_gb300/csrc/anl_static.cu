// anl_static.cu -- the compliance dot product without any device allocation.
//
// Who needs this: callers that cannot call cudaMalloc at the point where they need the
// compliance. Examples are code running inside a CUDA host callback or a memory-pool hook
// (where allocating is not allowed), embedders whose framework owns the whole device memory
// pool and hands out only the tensors it created, and real-time loops that must not risk an
// allocation (or its implicit device synchronisation) in the middle of a step. They cannot create
// an anl_ctx either, because anl_ctx_create allocates the solver workspaces.
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
// host-side name is only a stand-in); it asks the runtime for the device address once per
// device (scratch_on_current_device).
static __device__ __align__(256) double g_static_scratch[kScratchWords];

std::mutex g_mu;
void* g_scratch_ptr[64] = {};

int scratch_on_current_device(double** out) {
    int dev = -1;
    ANL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("anl_dot_static: device ordinal %d is outside the supported range 0..63", dev);
        return ANL_ERR_BADARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("anl_dot_static: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
            return ANL_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = (double*)g_scratch_ptr[dev];
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
