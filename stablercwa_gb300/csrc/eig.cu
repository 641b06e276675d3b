// eig.cu -- launchers of the batched eigensolver (kernel in eig.cuh).
#include <algorithm>

#include "eig.cuh"
#include "engine.h"

namespace rcwa_gb300 {

long long eig_workspace_bytes(int n, int batch) { return (long long)batch * eig_workspace_elems(n) * (long long)sizeof(zc); }

// Lanes per matrix. Small groups keep the per-lane share of each sweep's O(n) updates large
// compared with the work every lane of a group repeats (forming the rotation, the shift); a group
// of 32 (a warp per matrix) is used when the batch is too small to fill the GPU otherwise, and a
// whole CTA per matrix when even warps leave most of the GPU idle (few matrices of order >= 64).
int eig_default_group(int n, int batch) {
    const long long lanes_wanted = 152LL * 4 * 32 * 2;  // two warps per SM sub-partition
    for (int g : {4, 8, 16})
        if ((long long)batch * g >= lanes_wanted && n >= 4 * g) return g;
    if (batch * 16LL >= lanes_wanted) return 16;
    if (n < 64) return 32;
    if (n >= 384) {
        // large orders: a CTA per matrix until the batch fills the GPU twice over with warps
        // (measured at n = 882: 152 matrices 35 s at 256 threads vs 131 s at 32 lanes; 768 matrices
        // 61 s at 128 threads vs 75 s at 32 lanes)
        if (batch <= 152) return 256;
        return batch * 32LL < 2 * lanes_wanted ? 128 : 32;
    }
    return batch * 32LL * 4 >= lanes_wanted ? 32 : 128;
}

void launch_eig(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info, int* sweeps,
                zc* ws, double eps, int max_iter, int group, const int* skip, int skip_value, zc* t_out) {
    if (batch <= 0 || n <= 0) return;
    if (group == 0 && !skip && !t_out) {
        if (autotune_wanted(0, n, batch)) autotune_eig(st, 0, n, batch, a, a_stride, nullptr);
        group = tuned_eig_form(0, n, batch);
    }
    if (group == -1 || (group == 0 && eig_cluster_wanted(n, batch))) {
        TimedLaunch timed(TK_EIG, st);
        launch_eig_cluster(st, n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out);
        return;
    }
    if (group <= 0) group = eig_default_group(n, batch);
    TimedLaunch timed(TK_EIG, st);
    if (group > 32) {
        switch (group) {
            case 64: eig_block_kernel<64><<<(unsigned)batch, 64, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
            case 128: eig_block_kernel<128><<<(unsigned)batch, 128, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
            case 256: eig_block_kernel<256><<<(unsigned)batch, 256, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
            default: throw EngineError{RCWA_EINVAL, "eig: group must be 4, 8, 16, 32, 64, 128 or 256"};
        }
        ++launch_count();
        RCWA_CUDA(cudaGetLastError());
        return;
    }
    const int tpb = 128;
    const long long threads = (long long)batch * group;
    const unsigned blocks = (unsigned)((threads + tpb - 1) / tpb);
    switch (group) {
        case 4: eig_batch_kernel<4><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
        case 8: eig_batch_kernel<8><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
        case 16: eig_batch_kernel<16><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
        case 32: eig_batch_kernel<32><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter, skip, skip_value, t_out); break;
        default: throw EngineError{RCWA_EINVAL, "eig: group must be 4, 8, 16, 32, 64, 128 or 256"};
    }
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

// QL rotations applied by the Hermitian eigensolver since the last read (the work of its sweeps, 12 n flops
// each, for the benchmark's roofline)
unsigned long long* rotation_counter() {
    return static_cast<unsigned long long*>(device_word(0, sizeof(unsigned long long)));
}

void* device_word(int which, size_t bytes) {
    static std::mutex lock;
    static std::vector<std::vector<void*>> words;  // [which][device]
    int dev = 0;
    RCWA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(lock);
    if ((int)words.size() <= which) words.resize(which + 1);
    std::vector<void*>& per_device = words[which];
    if ((int)per_device.size() <= dev) per_device.resize(dev + 1, nullptr);
    if (!per_device[dev]) {
        void* d = nullptr;
        RCWA_CUDA(cudaMalloc(&d, bytes));
        const cudaError_t rc = cudaMemset(d, 0, bytes);
        if (rc != cudaSuccess) {
            cudaFree(d);
            RCWA_CUDA(rc);
        }
        per_device[dev] = d;
    }
    return per_device[dev];
}

void ensure_smem_optin(const void* func, int bytes) {
    static std::mutex lock;
    static std::vector<std::pair<std::pair<const void*, int>, int>> done;  // ((func, device), bytes)
    int dev = 0;
    RCWA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(lock);
    for (auto& e : done)
        if (e.first.first == func && e.first.second == dev) {
            if (bytes > e.second) {
                RCWA_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
                e.second = bytes;
            }
            return;
        }
    RCWA_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    done.push_back({{func, dev}, bytes});
}
long long take_rotation_count() {
    unsigned long long h = 0;
    unsigned long long* d = rotation_counter();
    RCWA_CUDA(cudaDeviceSynchronize());
    RCWA_CUDA(cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost));
    RCWA_CUDA(cudaMemset(d, 0, sizeof(unsigned long long)));
    return (long long)h;
}

// Hermitian matrices: the tridiagonalisation with G lanes per matrix, the QL iteration one lane per matrix,
// the rotations applied row-parallel, and the fused kernel for any matrix whose rotation log overflowed.
// While 32 rows of the real rotation product fit in shared memory (n <= 904) the rotations go to a real
// identity Y, in fixed point on the integer pipes, and the eigenvectors are Q Y; otherwise they are applied
// to the complex Q in place in FP64.
namespace {
template <int G>
void herm_reduce_launch(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* q, zc* ws) {
    if constexpr (G > 32) {
        herm_reduce_block_kernel<G><<<(unsigned)batch, G, 0, st>>>(n, batch, a, a_stride, q, ws);
    } else {
        const int tpb = 128;
        const unsigned blocks = (unsigned)(((long long)batch * G + tpb - 1) / tpb);
        herm_reduce_batch_kernel<G><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, q, ws);
    }
}
void herm_reduce_dispatch(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* q, zc* ws, int group) {
    switch (group) {
        case 4: herm_reduce_launch<4>(st, n, batch, a, a_stride, q, ws); break;
        case 8: herm_reduce_launch<8>(st, n, batch, a, a_stride, q, ws); break;
        case 16: herm_reduce_launch<16>(st, n, batch, a, a_stride, q, ws); break;
        case 32: herm_reduce_launch<32>(st, n, batch, a, a_stride, q, ws); break;
        case 64: herm_reduce_launch<64>(st, n, batch, a, a_stride, q, ws); break;
        case 128: herm_reduce_launch<128>(st, n, batch, a, a_stride, q, ws); break;
        case 256: herm_reduce_launch<256>(st, n, batch, a, a_stride, q, ws); break;
        default: throw EngineError{RCWA_EINVAL, "eig: group must be 4, 8, 16, 32, 64, 128 or 256"};
    }
    RCWA_CUDA(cudaGetLastError());
}
template <int G>
void herm_panel_launch(cudaStream_t st, int n, int batch, int k0, const zc* a, long long a_stride, zc* ws, zc* pan,
                       zc* vall, zc* mall, int pnb) {
    const int tpb = 128;
    const unsigned blocks = (unsigned)(((long long)batch * G + tpb - 1) / tpb);
    herm_panel_batch_kernel<G><<<blocks, tpb, 0, st>>>(n, batch, k0, a, a_stride, ws, pan, vall, mall, pnb);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

// The blocked tridiagonalisation (eig.cuh herm_panel_one): per panel one kernel over all matrices, then the
// trailing block's rank-2 nb update A -= V W^H + W V^H as two batched products (the tensor cores for
// orders >= 32). vall receives the reflectors, mall the panels' T V^H.
void herm_blocked_reduce(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* ws, zc* pan, zc* vall,
                         zc* mall, int group) {
    const int nb = kHermNb, P = herm_panel_count(n), pnb = P * nb;
    const long long ws_stride = eig_workspace_elems(n), pan_stride = herm_panel_elems(n);
    for (int b = 0; b < P; ++b) {
        const int k0 = b * nb;
        switch (group) {
            case 4: herm_panel_launch<4>(st, n, batch, k0, a, a_stride, ws, pan, vall, mall, pnb); break;
            case 8: herm_panel_launch<8>(st, n, batch, k0, a, a_stride, ws, pan, vall, mall, pnb); break;
            case 16: herm_panel_launch<16>(st, n, batch, k0, a, a_stride, ws, pan, vall, mall, pnb); break;
            case 32: herm_panel_launch<32>(st, n, batch, k0, a, a_stride, ws, pan, vall, mall, pnb); break;
            default: throw EngineError{RCWA_EINVAL, "eig: the blocked Hermitian reduction takes 4, 8, 16 or 32 lanes"};
        }
        if (k0 + nb < n - 1) {  // another panel follows: bring its trailing block up to date
            // as two products, V W^H and W V^H: the tensor-core product scales each row and column by its
            // largest entry, and a row of [V W] mixes V's entries (order 1) with W's (order |A|)
            const int t0 = k0 + nb, m2 = n - t0;
            zc* blk = ws + (long long)t0 * n + t0;
            const zc* bt = pan + 2LL * nb * n + (long long)t0 * 2 * nb;
            launch_zgemm_untimed(st, m2, m2, nb, batch, pan + t0, n, pan_stride, bt, 2 * nb, pan_stride, blk, ws_stride, blk,
                                 n, ws_stride, -1.0, 1.0);
            launch_zgemm_untimed(st, m2, m2, nb, batch, pan + (long long)nb * n + t0, n, pan_stride, bt + nb, 2 * nb,
                                 pan_stride, blk, ws_stride, blk, n, ws_stride, -1.0, 1.0);
        }
    }
}

// X (the eigenvectors, in place) = Q Y = Q_0 (Q_1 (.. (Q_last Y))) with Q_b = I - V_b T_b V_b^H, applied
// as X(k0+1:, :) -= V_b (M_b X(k0+1:, :)) with M_b = T_b V_b^H; u is nb x n scratch per matrix.
void herm_blocked_back(cudaStream_t st, int n, int batch, zc* x, const zc* vall, const zc* mall, zc* u, const int* skip) {
    const int nb = kHermNb, P = herm_panel_count(n), pnb = P * nb;
    const long long nn = (long long)n * n;
    for (int b = P - 1; b >= 0; --b) {
        const int k0 = b * nb, nbp = std::min(nb, n - 1 - k0), r0 = k0 + 1, mr = n - r0;
        launch_zgemm_untimed(st, nbp, n, mr, batch, mall + b * nb + (long long)r0 * pnb, pnb, (long long)pnb * n, x + r0, n,
                             nn, nullptr, 0, u, nb, (long long)nb * n, 1.0, 0.0, skip, 1);
        launch_zgemm_untimed(st, mr, n, nbp, batch, vall + (long long)k0 * n + r0, n, nn, u, nb, (long long)nb * n, x + r0,
                             nn, x + r0, n, nn, -1.0, 1.0, skip, 1);
    }
}

__global__ void real_to_complex_kernel(long long count, const double* __restrict__ y, zc* __restrict__ x) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) x[i] = zc{y[i], 0.0};
}

template <int G>
void herm_dc_launch(cudaStream_t st, int n, int batch, zc* ws, double* y, zc* w, int* info, double eps, int max_iter) {
    const int tpb = 128;
    const unsigned blocks = (unsigned)(((long long)batch * G + tpb - 1) / tpb);
    herm_dc_batch_kernel<G><<<blocks, tpb, 0, st>>>(n, batch, ws, y, w, info, eps, max_iter);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

// divide and conquer (eig.cuh herm_dc_one) in place of the QL iteration and its rotations, for batched groups
// of lanes, when RCWA_GB300_HERM_DC=1. Off by default: on this GPU it is FP64-bound with about half of
// each warp's lanes active (4096 matrices of order 121: 244 ms against 203 ms for QL and the rotations).
bool herm_dc_wanted(int group) {
    const char* env = std::getenv("RCWA_GB300_HERM_DC");
    return env && env[0] == '1' && group <= 32;
}

// the blocked reduction replaces the unblocked one for batched groups of lanes where the products run on the
// tensor cores; RCWA_GB300_HERM_BLOCKED=0 keeps the unblocked kernel
bool herm_blocked_wanted(int n, int group) {
    const char* env = std::getenv("RCWA_GB300_HERM_BLOCKED");
    if (env && env[0] == '0') return false;
    return group <= 32 && n >= 64 && tc_gemm_enabled() && !Fp64ProductsGuard::active();
}

void herm_fused_dispatch(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info,
                         zc* ws, double eps, int max_iter, int group, const int* only) {
    const int tpb = 128;
    const unsigned blocks = (unsigned)(((long long)batch * std::min(group, 32) + tpb - 1) / tpb);
    unsigned long long* rot = rotation_counter();
    switch (group) {
        case 4: herm_batch_kernel<4><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        case 8: herm_batch_kernel<8><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        case 16: herm_batch_kernel<16><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        case 32: herm_batch_kernel<32><<<blocks, tpb, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        case 64: herm_block_kernel<64><<<(unsigned)batch, 64, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        case 128: herm_block_kernel<128><<<(unsigned)batch, 128, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        case 256: herm_block_kernel<256><<<(unsigned)batch, 256, 0, st>>>(n, batch, a, a_stride, w, v, info, ws, eps, max_iter, rot, only); break;
        default: throw EngineError{RCWA_EINVAL, "eig: group must be 4, 8, 16, 32, 64, 128 or 256"};
    }
    RCWA_CUDA(cudaGetLastError());
}
}  // namespace

void launch_eig_herm(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info, zc* ws,
                     double eps, int max_iter, int group) {
    if (batch <= 0 || n <= 0) return;
    if (group == 0) {
        if (autotune_wanted(1, n, batch)) autotune_eig(st, 1, n, batch, a, a_stride, nullptr);
        group = tuned_eig_form(1, n, batch);
    }
    if (group <= 0) group = eig_default_group(n, batch);
    TimedLaunch timed(TK_EIG, st);
    const size_t ysm = (size_t)n * kHermRows * sizeof(double);
    const bool real_form = ysm + kHermApplyStaticSmem <= 227 * 1024;
    zc* q = v;
    double* y = nullptr;
    const bool blocked = real_form && herm_blocked_wanted(n, group);
    zc *pan = nullptr, *mall = nullptr, *u = nullptr;
    if (real_form) {
        RCWA_CUDA(cudaMallocAsync(&q, (size_t)batch * n * n * sizeof(zc), st));  // Q, or the reflectors when blocked
        RCWA_CUDA(cudaMallocAsync(&y, (size_t)batch * n * n * sizeof(double), st));
    }
    if (blocked) {
        const size_t pnb = (size_t)herm_panel_count(n) * kHermNb;
        RCWA_CUDA(cudaMallocAsync(&pan, (size_t)batch * herm_panel_elems(n) * sizeof(zc), st));
        RCWA_CUDA(cudaMallocAsync(&mall, (size_t)batch * pnb * n * sizeof(zc), st));
        RCWA_CUDA(cudaMallocAsync(&u, (size_t)batch * kHermNb * n * sizeof(zc), st));
        herm_blocked_reduce(st, n, batch, a, a_stride, ws, pan, q, mall, group);
    } else {
        herm_reduce_dispatch(st, n, batch, a, a_stride, q, ws, group);
    }
    const bool dc = real_form && herm_dc_wanted(group);
    const size_t qsm = (size_t)2 * n * kHermQlThreads * sizeof(double);
    if (dc) {
        switch (group) {
            case 4: herm_dc_launch<4>(st, n, batch, ws, y, w, info, eps, max_iter); break;
            case 8: herm_dc_launch<8>(st, n, batch, ws, y, w, info, eps, max_iter); break;
            case 16: herm_dc_launch<16>(st, n, batch, ws, y, w, info, eps, max_iter); break;
            default: herm_dc_launch<32>(st, n, batch, ws, y, w, info, eps, max_iter); break;
        }
    } else if (qsm <= 227 * 1024) {
        if (qsm > 48 * 1024) ensure_smem_optin(reinterpret_cast<const void*>(herm_ql_kernel<true, true>), (int)qsm);
        // the real form's log is fixed point (herm_apply_real_kernel); the shared-memory form implies it
        herm_ql_kernel<true, true><<<(unsigned)((batch + kHermQlThreads - 1) / kHermQlThreads), kHermQlThreads, qsm, st>>>(
            n, batch, w, info, ws, eps, max_iter, rotation_counter());
    } else if (real_form) {
        herm_ql_kernel<false, true><<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(n, batch, w, info, ws, eps,
                                                                                     max_iter, rotation_counter());
    } else {
        herm_ql_kernel<false, false><<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(n, batch, w, info, ws, eps,
                                                                                      max_iter, rotation_counter());
    }
    RCWA_CUDA(cudaGetLastError());
    int* only = nullptr;  // matrices whose log overflowed: the fused kernel, masked to them
    RCWA_CUDA(cudaMallocAsync(&only, (size_t)batch * sizeof(int), st));
    herm_overflow_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(n, batch, ws, only);
    RCWA_CUDA(cudaGetLastError());
    if (real_form) {
        if (ysm > 48 * 1024) ensure_smem_optin(reinterpret_cast<const void*>(herm_apply_real_kernel), (int)ysm);
        if (!dc) {  // divide and conquer has left Y in y already
            const dim3 grid((unsigned)batch, (unsigned)((n + kHermRows - 1) / kHermRows));
            herm_apply_real_kernel<<<grid, kHermRows, ysm, st>>>(n, batch, y, ws, info);
            RCWA_CUDA(cudaGetLastError());
        }
        if (blocked) {
            const long long cnt = (long long)batch * n * n;
            real_to_complex_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(cnt, y, v);
            RCWA_CUDA(cudaGetLastError());
            herm_blocked_back(st, n, batch, v, q, mall, u, only);
        } else {
            launch_zdgemm(st, n, n, n, batch, q, n, (long long)n * n, y, n, (long long)n * n, v, n, (long long)n * n, only, 1);
        }
        launch_count() += dc ? 3 : 5;  // the overflow flags, the fused redo, and the reduction or r2c; QL and rotations
    } else {
        herm_apply_kernel<<<(unsigned)(((long long)batch * n + 127) / 128), 128, 0, st>>>(n, batch, v, ws, info);
        RCWA_CUDA(cudaGetLastError());
        launch_count() += 4;
    }
    herm_fused_dispatch(st, n, batch, a, a_stride, w, v, info, ws, eps, max_iter, group, only);
    RCWA_CUDA(cudaFreeAsync(only, st));
    if (real_form) {
        RCWA_CUDA(cudaFreeAsync(q, st));
        RCWA_CUDA(cudaFreeAsync(y, st));
    }
    if (blocked) {
        RCWA_CUDA(cudaFreeAsync(pan, st));
        RCWA_CUDA(cudaFreeAsync(mall, st));
        RCWA_CUDA(cudaFreeAsync(u, st));
    }
}

}  // namespace rcwa_gb300
