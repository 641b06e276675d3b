// eig.cu -- launchers of the batched eigensolver (kernel in eig.cuh).
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

}  // namespace rcwa_gb300
