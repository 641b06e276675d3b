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
// Set-up is once per device: the first call made with a device current looks up the array's
// address with cudaGetSymbolAddress and loads the kernel variants. Make that first call before
// any stream capture begins on the device. Every call uses the same array, so calls that overlap in
// time on one device (issued on different streams, or from several host threads without ordering)
// race on it; calls on one stream are ordered and safe.
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
zc* g_scratch[kMaxDevices] = {};

template <int G>
cudaError_t load_kernel() {
    cudaFuncAttributes attr;
    if constexpr (G > 32) return cudaFuncGetAttributes(&attr, rcwa_gb300::eig_block_kernel<G>);
    else return cudaFuncGetAttributes(&attr, rcwa_gb300::eig_batch_kernel<G>);
}

// Address of this device's copy of the array; looked up on the device's first call.
int scratch_for_current_device(zc** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return RCWA_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return RCWA_EUNSUPPORTED;
    std::lock_guard<std::mutex> guard(g_setup_lock);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, eig_static_scratch) != cudaSuccess || !p) return RCWA_ECUDA;
        if (load_kernel<4>() != cudaSuccess || load_kernel<8>() != cudaSuccess || load_kernel<16>() != cudaSuccess ||
            load_kernel<32>() != cudaSuccess || load_kernel<128>() != cudaSuccess || load_kernel<256>() != cudaSuccess)
            return RCWA_ECUDA;
        g_scratch[dev] = static_cast<zc*>(p);
    }
    *out = g_scratch[dev];
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
    const int rc = scratch_for_current_device(&ws);
    if (rc != RCWA_OK) return rc;

    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int group = eig_default_group(n, batch);
    const int tpb = 128;
    const unsigned blocks = (unsigned)(((long long)batch * group + tpb - 1) / tpb);
    const zc* a = reinterpret_cast<const zc*>(d_a);
    zc* w = reinterpret_cast<zc*>(d_values);
    zc* v = reinterpret_cast<zc*>(d_vectors);
    const long long a_stride = (long long)n * n;
    switch (group) {
        case 4: eig_batch_kernel<4><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, d_info, d_sweeps, ws, eps, max_iter, nullptr, 1, nullptr); break;
        case 8: eig_batch_kernel<8><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, d_info, d_sweeps, ws, eps, max_iter, nullptr, 1, nullptr); break;
        case 16: eig_batch_kernel<16><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, d_info, d_sweeps, ws, eps, max_iter, nullptr, 1, nullptr); break;
        case 128: eig_block_kernel<128><<<(unsigned)batch, 128, 0, st>>>(n, batch, a, a_stride, w, v, d_info, d_sweeps, ws, eps, max_iter, nullptr, 1, nullptr); break;
        case 256: eig_block_kernel<256><<<(unsigned)batch, 256, 0, st>>>(n, batch, a, a_stride, w, v, d_info, d_sweeps, ws, eps, max_iter, nullptr, 1, nullptr); break;
        default: eig_batch_kernel<32><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, d_info, d_sweeps, ws, eps, max_iter, nullptr, 1, nullptr); break;
    }
    ++launch_count();
    return cudaGetLastError() == cudaSuccess ? RCWA_OK : RCWA_ECUDA;
}
