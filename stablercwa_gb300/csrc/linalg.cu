// linalg.cu -- launchers of the batched LU solve and GEMM (kernels in linalg.cuh).
#include "engine.h"
#include "linalg.cuh"

namespace rcwa_gb300 {

long long& launch_count() {
    static long long count = 0;
    return count;
}

KernelTimer*& current_timer() {
    thread_local KernelTimer* t = nullptr;
    return t;
}

void KernelTimer::collect() {
    for (Rec& r : pending) {
        float ms_ = 0.0f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms_, r.a, r.b) == cudaSuccess) {
            ms[r.kind] += ms_;
            count[r.kind] += 1;
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    pending.clear();
}

KernelTimer::~KernelTimer() { collect(); }

TimedLaunch::TimedLaunch(int kind, cudaStream_t st) : t_(current_timer()), st_(st) {
    if (!t_) return;
    KernelTimer::Rec r{kind, nullptr, nullptr};
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, st);
    idx_ = t_->pending.size();
    t_->pending.push_back(r);
}

TimedLaunch::~TimedLaunch() {
    if (t_) cudaEventRecord(t_->pending[idx_].b, st_);
}

void launch_lu_solve(cudaStream_t st, int n, int nrhs, int batch, const zc* a, long long a_stride, zc* lu,
                     long long lu_stride, int rhs_kind, const zc* rhs, long long rhs_stride, zc* x, long long x_stride,
                     int* singular, const int* skip, int skip_value) {
    if (batch <= 0 || n <= 0) return;
    const long long threads = (long long)batch * 32;
    const unsigned blocks = (unsigned)((threads + 127) / 128);
    TimedLaunch timed(TK_LU, st);
    lu_solve_kernel<<<blocks, 128, 0, st>>>(n, nrhs, batch, a, a_stride, lu, lu_stride, rhs_kind, rhs, rhs_stride, x,
                                            x_stride, singular, skip, skip_value);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

void launch_zgemm(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride, const zc* B,
                  int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc, long long c_stride,
                  double s_ab, double s_c, const int* skip, int skip_value) {
    if (batch <= 0 || m <= 0 || n <= 0) return;
    const long long warps = (long long)batch * ((m + 31) / 32) * ((n + 7) / 8);
    const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
    TimedLaunch timed(TK_GEMM, st);
    zgemm_kernel<<<blocks, 128, 0, st>>>(m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C0, c0_stride, C, ldc,
                                         c_stride, s_ab, s_c, skip, skip_value);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

}  // namespace rcwa_gb300
