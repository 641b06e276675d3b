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
    static unsigned long long* d = nullptr;
    if (!d) {
        RCWA_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
        RCWA_CUDA(cudaMemset(d, 0, sizeof(unsigned long long)));
    }
    return d;
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
// While a row of the real rotation product fits in shared memory (n <= 887) the rotations go to a real
// identity Y and the eigenvectors are Q Y; otherwise they are applied to the complex Q in place.
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
    const bool real_form = ysm <= 227 * 1024;
    zc* q = v;
    double* y = nullptr;
    if (real_form) {
        RCWA_CUDA(cudaMallocAsync(&q, (size_t)batch * n * n * sizeof(zc), st));
        RCWA_CUDA(cudaMallocAsync(&y, (size_t)batch * n * n * sizeof(double), st));
    }
    herm_reduce_dispatch(st, n, batch, a, a_stride, q, ws, group);
    const size_t qsm = (size_t)2 * n * kHermQlThreads * sizeof(double);
    if (qsm <= 227 * 1024) {
        if (qsm > 48 * 1024) {
            static int opted = 0;  // the largest opt-in requested so far
            if ((int)qsm > opted) {
                RCWA_CUDA(cudaFuncSetAttribute(herm_ql_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)qsm));
                opted = (int)qsm;
            }
        }
        herm_ql_kernel<true><<<(unsigned)((batch + kHermQlThreads - 1) / kHermQlThreads), kHermQlThreads, qsm, st>>>(
            n, batch, w, info, ws, eps, max_iter, rotation_counter());
    } else {
        herm_ql_kernel<false><<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(n, batch, w, info, ws, eps, max_iter,
                                                                               rotation_counter());
    }
    RCWA_CUDA(cudaGetLastError());
    int* only = nullptr;  // matrices whose log overflowed: the fused kernel, masked to them
    RCWA_CUDA(cudaMallocAsync(&only, (size_t)batch * sizeof(int), st));
    herm_overflow_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(n, batch, ws, only);
    RCWA_CUDA(cudaGetLastError());
    if (real_form) {
        if (ysm > 48 * 1024) {
            static int opted = 0;  // the largest opt-in requested so far (the attribute is per function)
            if ((int)ysm > opted) {
                RCWA_CUDA(cudaFuncSetAttribute(herm_apply_real_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)ysm));
                opted = (int)ysm;
            }
        }
        const dim3 grid((unsigned)batch, (unsigned)((n + kHermRows - 1) / kHermRows));
        herm_apply_real_kernel<<<grid, kHermRows, ysm, st>>>(n, batch, y, ws, info);
        RCWA_CUDA(cudaGetLastError());
        launch_zdgemm(st, n, n, n, batch, q, n, (long long)n * n, y, n, (long long)n * n, v, n, (long long)n * n, only, 1);
        launch_count() += 5;
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
}

}  // namespace rcwa_gb300
