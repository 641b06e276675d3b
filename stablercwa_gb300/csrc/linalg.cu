// linalg.cu -- launchers of the batched LU solve and GEMM (kernels in linalg.cuh).
#include <algorithm>
#include <cstdlib>

#include "engine.h"
#include "linalg.cuh"

namespace rcwa_gb300 {

std::atomic<long long>& launch_count() {
    static std::atomic<long long> count{0};
    return count;
}

KernelTimer*& current_timer() {
    thread_local KernelTimer* t = nullptr;
    return t;
}

void KernelTimer::collect() {
    std::lock_guard<std::mutex> hold(lock);
    for (Rec& r : pending) {
        float ms_ = 0.0f, t0 = 0.0f, t1 = 0.0f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms_, r.a, r.b) == cudaSuccess) {
            ms[r.kind] += ms_;
            count[r.kind] += 1;
            if (base && cudaEventElapsedTime(&t0, base, r.a) == cudaSuccess &&
                cudaEventElapsedTime(&t1, base, r.b) == cudaSuccess)
                spans[r.kind].push_back({t0, t1});
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    pending.clear();
}

double KernelTimer::busy_ms(int kind) {
    collect();
    std::lock_guard<std::mutex> hold(lock);
    std::vector<std::pair<double, double>>& v = spans[kind];
    std::sort(v.begin(), v.end());
    double total = 0.0, lo = 0.0, hi = -1.0;
    for (const auto& iv : v) {
        if (iv.first > hi) {
            if (hi > lo) total += hi - lo;
            lo = iv.first;
            hi = iv.second;
        } else {
            hi = std::max(hi, iv.second);
        }
    }
    if (hi > lo) total += hi - lo;
    v.clear();
    return total;
}

KernelTimer::~KernelTimer() {
    collect();
    if (base) cudaEventDestroy(base);
}

TimedLaunch::TimedLaunch(int kind, cudaStream_t st) : t_(current_timer()), st_(st) {
    if (!t_) return;
    KernelTimer::Rec r{kind, nullptr, nullptr};
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, st);
    std::lock_guard<std::mutex> hold(t_->lock);
    idx_ = t_->pending.size();
    t_->pending.push_back(r);
}

TimedLaunch::~TimedLaunch() {
    if (!t_) return;
    std::lock_guard<std::mutex> hold(t_->lock);
    cudaEventRecord(t_->pending[idx_].b, st_);
}

namespace {

// Orders from which the blocked LU replaces the warp-per-system kernel (RCWA_GB300_LU_BLOCKED_MIN_N
// overrides it for measurements).
int lu_blocked_min_n() {
    static const int v = [] {
        const char* e = std::getenv("RCWA_GB300_LU_BLOCKED_MIN_N");
        return e ? std::atoi(e) : 100;
    }();
    return v;
}

constexpr int kPanel = 32;

void zgemm_raw(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride, const zc* B,
               int ldb, long long b_stride, zc* C, int ldc, long long c_stride, double s_ab, const int* skip, int skip_value) {
    if (batch <= 0 || m <= 0 || n <= 0 || k <= 0) return;
    if (tc_gemm_wanted(m, n, k)) {
        launch_zgemm_tc(st, m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C, c_stride, C, ldc, c_stride, s_ab, 1.0,
                        skip, skip_value);
        return;
    }
    const long long warps = (long long)batch * ((m + 31) / 32) * ((n + 7) / 8);
    const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
    zgemm_kernel<<<blocks, 128, 0, st>>>(m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C, c_stride, C, ldc,
                                         c_stride, s_ab, 1.0, skip, skip_value, TRI_NONE);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

void lu_solve_blocked(cudaStream_t st, int n, int nrhs, int batch, const zc* a, long long a_stride, zc* lu,
                      long long lu_stride, int rhs_kind, const zc* rhs, long long rhs_stride, zc* x, long long x_stride,
                      int* singular, const int* skip, int skip_value) {
    int* sing_local = nullptr;
    RCWA_CUDA(cudaMallocAsync(&sing_local, (size_t)batch * sizeof(int), st));
    RCWA_CUDA(cudaMemsetAsync(sing_local, 0, (size_t)batch * sizeof(int), st));
    const long long init = (long long)batch * n * (n + nrhs);
    lu_init_kernel<<<(unsigned)((init + 255) / 256), 256, 0, st>>>(n, nrhs, batch, a, a_stride, lu, lu_stride, rhs_kind, rhs,
                                                                   rhs_stride, x, x_stride, skip, skip_value);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
    // a warp per system once the batch gives every SM sub-partition a system of moderate order
    const bool warp_panels = n <= 256 && batch >= 608;
    for (int k0 = 0; k0 < n; k0 += kPanel) {
        const int kend = std::min(k0 + kPanel, n);
        if (warp_panels)
            lu_panel_warp_kernel<<<(unsigned)(((long long)batch * 32 + 127) / 128), 128, 0, st>>>(
                n, nrhs, batch, lu, lu_stride, x, x_stride, k0, kPanel, sing_local, skip, skip_value);
        else
            lu_panel_kernel<<<(unsigned)batch, 256, 0, st>>>(n, nrhs, batch, lu, lu_stride, x, x_stride, k0, kPanel,
                                                             sing_local, skip, skip_value);
        ++launch_count();
        RCWA_CUDA(cudaGetLastError());
        const long long tcols = (long long)batch * (n + nrhs - kend);
        if (tcols > 0) {
            lu_trsm_lower_kernel<<<(unsigned)((tcols + 127) / 128), 128, 0, st>>>(n, nrhs, batch, lu, lu_stride, x, x_stride,
                                                                                  k0, kend, skip, skip_value);
            ++launch_count();
            RCWA_CUDA(cudaGetLastError());
        }
        const int rest = n - kend, w = kend - k0;
        // trailing matrix and right-hand sides: C -= L21 U12
        zgemm_raw(st, rest, rest, w, batch, lu + (long long)k0 * n + kend, n, lu_stride, lu + (long long)kend * n + k0, n,
                  lu_stride, lu + (long long)kend * n + kend, n, lu_stride, -1.0, skip, skip_value);
        zgemm_raw(st, rest, nrhs, w, batch, lu + (long long)k0 * n + kend, n, lu_stride, x + k0, n, x_stride, x + kend, n,
                  x_stride, -1.0, skip, skip_value);
    }
    const int nblk = (n + kPanel - 1) / kPanel;
    for (int kb = nblk - 1; kb >= 0; --kb) {
        const int r0 = kb * kPanel, r1 = std::min(r0 + kPanel, n);
        const long long t = (long long)batch * nrhs;
        lu_trsm_upper_kernel<<<(unsigned)((t + 127) / 128), 128, 0, st>>>(n, nrhs, batch, lu, lu_stride, x, x_stride, r0, r1,
                                                                          skip, skip_value);
        ++launch_count();
        RCWA_CUDA(cudaGetLastError());
        // rows above: X[0:r0] -= U[0:r0, r0:r1] X[r0:r1]
        zgemm_raw(st, r0, nrhs, r1 - r0, batch, lu + (long long)r0 * n, n, lu_stride, x + r0, n, x_stride, x, n, x_stride,
                  -1.0, skip, skip_value);
    }
    const long long xt = (long long)batch * n * nrhs;
    lu_nan_fill_kernel<<<(unsigned)((xt + 255) / 256), 256, 0, st>>>(n, nrhs, batch, x, x_stride, sing_local, singular);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
    RCWA_CUDA(cudaFreeAsync(sing_local, st));
}

}  // namespace

void launch_lu_solve(cudaStream_t st, int n, int nrhs, int batch, const zc* a, long long a_stride, zc* lu,
                     long long lu_stride, int rhs_kind, const zc* rhs, long long rhs_stride, zc* x, long long x_stride,
                     int* singular, const int* skip, int skip_value) {
    if (batch <= 0 || n <= 0) return;
    // blocked from n = 100, and for a handful of systems of moderate order (the per-layer inverses),
    // where one warp per system would leave the GPU idle
    if ((n >= lu_blocked_min_n() || (batch < 152 && n >= 32)) && nrhs > 0) {
        TimedLaunch timed(TK_LU, st);
        lu_solve_blocked(st, n, nrhs, batch, a, a_stride, lu, lu_stride, rhs_kind, rhs, rhs_stride, x, x_stride, singular,
                         skip, skip_value);
        return;
    }
    const long long threads = (long long)batch * 32;
    const unsigned blocks = (unsigned)((threads + 127) / 128);
    TimedLaunch timed(TK_LU, st);
    lu_solve_kernel<<<blocks, 128, 0, st>>>(n, nrhs, batch, a, a_stride, lu, lu_stride, rhs_kind, rhs, rhs_stride, x,
                                            x_stride, singular, skip, skip_value);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

// The tensor-core product costs about the same per tile of the real-ified product whatever m and n fill of
// it, and its digit planes are padded to 64 in K; the FP64 kernel costs 8 m n k flops at 1.1 TFLOP/s. A
// product goes to the tensor cores when every dimension is at least 16 and m n k >= 2^15 (a 57 x 57 x 32
// trailing update or a 24 x 121 x 120 back-transformation panel does; an order-25 trailing update of
// 25 x 25 x 32, or a one-column solve, does not).
bool tc_gemm_wanted(int m, int n, int k) {
    return k >= 16 && m >= 16 && n >= 16 && (long long)m * n * k >= (1LL << 15) && tc_gemm_enabled() &&
           !Fp64ProductsGuard::active();
}

cudaError_t stream_wait(cudaStream_t st) {
    struct Ev {
        cudaEvent_t e = nullptr;
        int device = -1;
        ~Ev() {
            if (e) cudaEventDestroy(e);
        }
    };
    thread_local Ev ev;
    int dev = 0;
    cudaError_t r = cudaGetDevice(&dev);
    if (r != cudaSuccess) return r;
    if (!ev.e || ev.device != dev) {
        if (ev.e) cudaEventDestroy(ev.e);
        ev.e = nullptr;
        r = cudaEventCreateWithFlags(&ev.e, cudaEventBlockingSync | cudaEventDisableTiming);
        if (r != cudaSuccess) return r;
        ev.device = dev;
    }
    r = cudaEventRecord(ev.e, st);
    if (r != cudaSuccess) return r;
    return cudaEventSynchronize(ev.e);
}

void launch_zgemm(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride, const zc* B,
                  int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc, long long c_stride,
                  double s_ab, double s_c, const int* skip, int skip_value, int tri) {
    if (batch <= 0 || m <= 0 || n <= 0) return;
    TimedLaunch timed(TK_GEMM, st);
    launch_zgemm_untimed(st, m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C0, c0_stride, C, ldc, c_stride, s_ab, s_c,
                         skip, skip_value, tri);
}

void launch_zgemm_untimed(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                          const zc* B, int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc,
                          long long c_stride, double s_ab, double s_c, const int* skip, int skip_value, int tri) {
    if (batch <= 0 || m <= 0 || n <= 0) return;
    if (tc_gemm_wanted(m, n, k)) {
        launch_zgemm_tc(st, m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C0, c0_stride, C, ldc, c_stride, s_ab, s_c,
                        skip, skip_value);
        return;
    }
    const long long warps = (long long)batch * ((m + 31) / 32) * ((n + 7) / 8);
    const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
    zgemm_kernel<<<blocks, 128, 0, st>>>(m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C0, c0_stride, C, ldc,
                                         c_stride, s_ab, s_c, skip, skip_value, tri);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

void launch_zdgemm(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                   const double* B, int ldb, long long b_stride, zc* C, int ldc, long long c_stride, const int* skip,
                   int skip_value) {
    if (batch <= 0 || m <= 0 || n <= 0) return;
    if (tc_gemm_wanted(m, n, k)) {
        launch_zdgemm_tc(st, m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C, ldc, c_stride, skip, skip_value);
        return;
    }
    const long long warps = (long long)batch * ((m + 31) / 32) * ((n + 7) / 8);
    const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
    zdgemm_kernel<<<blocks, 128, 0, st>>>(m, n, k, batch, A, lda, a_stride, B, ldb, b_stride, C, ldc, c_stride, skip,
                                          skip_value);
    ++launch_count();
    RCWA_CUDA(cudaGetLastError());
}

}  // namespace rcwa_gb300
