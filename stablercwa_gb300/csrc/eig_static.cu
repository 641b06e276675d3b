// eig_static.cu -- the batched eigensolver with its workspace in a fixed device array, for callers
// that may not allocate device memory.
//
// rcwa_gpu_eig_batch_dev takes its per-matrix workspace from the stream-ordered allocator on every
// call. Some callers cannot allow that: a host that has handed (nearly) all of HBM to its own
// caching allocator, where a further allocation fails or forces that allocator to release blocks;
// and a latency-bound loop that must not pay for an allocator call, nor for the device-wide
// synchronisation a cudaFree can imply. rcwa_gpu_eig_batch_static serves them: the workspace lives
// in the file-scope array below, the caller passes device inputs and outputs, and the call
// allocates nothing.
//
// Set-up is once per device context: the first call made with a device current looks up the array's
// address with cudaGetSymbolAddress and loads the kernel variants. Make that first call before any
// stream capture begins on the device. The address is cached together with the id of the CUDA context
// it belongs to; a call under another context (after cudaDeviceReset, or with a context of the
// caller's own) repeats the set-up instead of using a stale address. Every call uses the same array,
// so calls that overlap in time on one device (issued on different streams, or from several host
// threads without ordering) race on it; calls on one stream are ordered and safe. The kernel form
// (lanes per matrix, a CTA or a thread-block cluster per matrix) is chosen as rcwa_gpu_eig_batch_dev
// chooses it: RCWA_GB300_EIG_GROUP when set, else a form the autotuner has recorded for the order and
// batch, else the built-in rule. This entry never starts the autotuner itself, because tuning allocates
// its trial buffers; with RCWA_GB300_AUTOTUNE=auto the allocating entry may tune a key that this one
// then leaves on the built-in rule until a table entry exists, so the two agree to rounding, not bit
// for bit, in that case only.
#include <cstdlib>
#include <mutex>

#include "eig.cuh"
#include "engine.h"

namespace {

using rcwa_gb300::zc;

constexpr unsigned long long kScratchBytes = RCWA_GPU_EIG_STATIC_SCRATCH_BYTES;
static_assert(kScratchBytes % 256 == 0, "scratch size must keep the 256-byte alignment");

// The workspace of every matrix of one call: batch * (3n^2 + 4n + 8) complex doubles. The solver
// writes each element before it reads it, so nothing here has to start at zero.
static __device__ __align__(256) unsigned char eig_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
struct DeviceSetup {
    unsigned long long ctx_id = 0;
    zc* scratch = nullptr;
};
DeviceSetup g_setup[kMaxDevices];

template <int G>
cudaError_t load_kernel() {
    cudaFuncAttributes attr;
    if constexpr (G > 32) return cudaFuncGetAttributes(&attr, rcwa_gb300::eig_block_kernel<G>);
    else return cudaFuncGetAttributes(&attr, rcwa_gb300::eig_batch_kernel<G>);
}

// Id of the calling thread's current CUDA context, through the driver's own entry points (resolved by
// the runtime, so the library needs no link-time driver dependency); 0 when none is current.
unsigned long long current_context_id() {
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Address of the array in the current device context; set up on the context's first call.
int scratch_for_current_context(zc** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return RCWA_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return RCWA_EUNSUPPORTED;
    std::lock_guard<std::mutex> guard(g_setup_lock);
    DeviceSetup& d = g_setup[dev];
    const unsigned long long id = current_context_id();
    if (!d.scratch || id == 0 || id != d.ctx_id) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, eig_static_scratch) != cudaSuccess || !p) return RCWA_ECUDA;
        if (load_kernel<4>() != cudaSuccess || load_kernel<8>() != cudaSuccess || load_kernel<16>() != cudaSuccess ||
            load_kernel<32>() != cudaSuccess || load_kernel<64>() != cudaSuccess || load_kernel<128>() != cudaSuccess ||
            load_kernel<256>() != cudaSuccess)
            return RCWA_ECUDA;
        rcwa_gb300::preload_eig_cluster_kernel();  // the cluster form too (a few matrices of order >= 384)
        d.scratch = static_cast<zc*>(p);
        d.ctx_id = current_context_id();  // the symbol lookup made the device's context current
    }
    *out = d.scratch;
    return RCWA_OK;
}

}  // namespace

extern "C" int rcwa_gpu_eig_batch_static(void* stream, int n, int batch, const rcwa_complex* d_a, double eps,
                                         int max_iter, rcwa_complex* d_values, rcwa_complex* d_vectors, int* d_info,
                                         int* d_sweeps) {
    using namespace rcwa_gb300;
    if (n < 0 || batch < 0 || max_iter < 1 || !(eps >= 0.0) || !std::isfinite(eps)) return RCWA_EINVAL;
    if (n == 0 || batch == 0) return RCWA_OK;
    if (!d_a || !d_values || !d_vectors || !d_info) return RCWA_EINVAL;
    const unsigned long long per_matrix = (unsigned long long)eig_workspace_elems(n) * sizeof(zc);
    if (per_matrix > kScratchBytes || (unsigned long long)batch > kScratchBytes / per_matrix) return RCWA_ESCRATCH;

    zc* ws = nullptr;
    const int rc = scratch_for_current_context(&ws);
    if (rc != RCWA_OK) return rc;

    int group = 0;
    if (const char* g = std::getenv("RCWA_GB300_EIG_GROUP")) group = std::atoi(g);
    if (group == 0) group = tuned_eig_form(0, n, batch);  // a recorded form; never a tuning run
    if (group == 0) group = eig_cluster_wanted(n, batch) ? -1 : eig_default_group(n, batch);
    try {
        launch_eig(static_cast<cudaStream_t>(stream), n, batch, reinterpret_cast<const zc*>(d_a), (long long)n * n,
                   reinterpret_cast<zc*>(d_values), reinterpret_cast<zc*>(d_vectors), d_info, d_sweeps, ws, eps,
                   max_iter, group);
    } catch (const EngineError& e) {
        return e.code;
    }
    return RCWA_OK;
}
