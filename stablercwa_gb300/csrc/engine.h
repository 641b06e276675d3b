// engine.h -- internal interfaces between the engine's translation units (not installed).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <complex>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/stablercwa_gb300.h"
#include "common.cuh"

namespace rcwa_gb300 {

// Thrown inside the engine, turned into a return code at the C ABI.
struct EngineError {
    int code;
    std::string message;
};

#define RCWA_CUDA(call)                                                                                   \
    do {                                                                                                  \
        cudaError_t err_ = (call);                                                                        \
        if (err_ != cudaSuccess)                                                                          \
            throw ::rcwa_gb300::EngineError{err_ == cudaErrorMemoryAllocation ? RCWA_ENOMEM : RCWA_ECUDA,   \
                                            std::string(#call) + ": " + cudaGetErrorString(err_)};        \
    } while (0)

// Stream-ordered device allocations released together when the scope ends.
class DeviceScratch {
public:
    explicit DeviceScratch(cudaStream_t s) : stream_(s) {}
    ~DeviceScratch() { release(); }
    DeviceScratch(const DeviceScratch&) = delete;
    DeviceScratch& operator=(const DeviceScratch&) = delete;
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (count == 0) count = 1;
        RCWA_CUDA(cudaMallocAsync(&p, count * sizeof(T), stream_));
        ptrs_.push_back(p);
        return static_cast<T*>(p);
    }
    template <class T>
    T* zeros(size_t count) {
        T* p = get<T>(count);
        RCWA_CUDA(cudaMemsetAsync(p, 0, (count ? count : 1) * sizeof(T), stream_));
        return p;
    }
    void free(void* p) {
        for (size_t k = 0; k < ptrs_.size(); ++k)
            if (ptrs_[k] == p) {
                cudaFreeAsync(p, stream_);
                ptrs_[k] = ptrs_.back();
                ptrs_.pop_back();
                return;
            }
    }
    void release() {
        for (void* p : ptrs_) cudaFreeAsync(p, stream_);
        ptrs_.clear();
    }

private:
    cudaStream_t stream_;
    std::vector<void*> ptrs_;
};

struct KernelCounter {
    long long launches = 0;
};

// Launchers (linalg.cu, eig.cu)
void launch_lu_solve(cudaStream_t st, int n, int nrhs, int batch, const zc* a, long long a_stride, zc* lu,
                     long long lu_stride, int rhs_kind, const zc* rhs, long long rhs_stride, zc* x, long long x_stride,
                     int* singular, const int* skip = nullptr, int skip_value = 1);
void launch_zgemm(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride, const zc* B,
                  int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc, long long c_stride,
                  double s_ab, double s_c, const int* skip = nullptr, int skip_value = 1, int tri = 0);
// Waits for the work queued on st like cudaStreamSynchronize, but sleeping (an event with blocking sync)
// instead of spinning: the serving loop's slot threads wait on their own streams while others launch.
cudaError_t stream_wait(cudaStream_t st);
// the same without the per-kind kernel timer (products inside another timed stage, e.g. the eigensolver's)
void launch_zgemm_untimed(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                          const zc* B, int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc,
                          long long c_stride, double s_ab, double s_c, const int* skip = nullptr, int skip_value = 1,
                          int tri = 0);
// The eigensolver's form per (kind 0 general / 1 Hermitian, order, batch) from timing (autotune.cu): the
// tuned form, 0 when none is recorded; autotune_eig times every applicable form on the given matrices and
// records the fastest (returns it; best_ms its time if non-null).
int tuned_eig_form(int kind, int n, int batch);
bool autotune_wanted(int kind, int n, int batch);
int autotune_eig(cudaStream_t st, int kind, int n, int batch, const zc* a, long long a_stride, double* best_ms);
void set_tuned_eig_form(int kind, int n, int batch, int form);
std::string autotune_table_text();
// One matrix per thread-block cluster (eig_cluster.cu) for a few large matrices: the same algorithm as
// launch_eig's kernels, spread over 8 or 16 SMs. launch_eig takes it by itself (eig_cluster_wanted).
bool eig_cluster_wanted(int n, int batch);
bool eig_cluster_possible(int n, int batch);
void preload_eig_cluster_kernel();
void launch_eig_cluster(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info,
                        int* sweeps, zc* ws, double eps, int max_iter, const int* skip, int skip_value, zc* t_out);
// The same product on the tensor cores (gemm_tc.cu: Ozaki-split bf16 tcgen05 products, FP64-accurate);
// launch_zgemm takes it for products of order >= 32 unless RCWA_GB300_GEMM=fp64. The triangular hint
// does not apply (the full product is formed; zero entries contribute exact zeros).
void launch_zgemm_tc(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                     const zc* B, int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc,
                     long long c_stride, double s_ab, double s_c, const int* skip = nullptr, int skip_value = 1);
void launch_zdgemm_tc(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                      const double* B, int ldb, long long b_stride, zc* C, int ldc, long long c_stride,
                      const int* skip = nullptr, int skip_value = 1);
bool tc_gemm_enabled();
bool tc_gemm_wanted(int m, int n, int k);  // this product goes to the tensor cores (linalg.cu)
// Products launched by this host thread while a guard lives stay on the FP64 pipe (the 2-D solve: its
// operands span many decades within a row or column, where an FP64 product's error, relative to the
// terms it sums, is smaller than the slice products', relative to the row and column maxima).
struct Fp64ProductsGuard {
    Fp64ProductsGuard();
    ~Fp64ProductsGuard();
    Fp64ProductsGuard(const Fp64ProductsGuard&) = delete;
    Fp64ProductsGuard& operator=(const Fp64ProductsGuard&) = delete;
    static bool active();
};
int tc_gemm_slices();
int tc_gemm_error();  // nonzero once a tensor-core product kernel gave up on a stuck wait (synchronous read)
// C = A B with A complex, B real (C does not alias A or B)
void launch_zdgemm(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                   const double* B, int ldb, long long b_stride, zc* C, int ldc, long long c_stride,
                   const int* skip = nullptr, int skip_value = 1);
// tri: a triangular factor whose zero part the product skips (TRI_*, common.cuh)
// group: lanes per matrix (0 = choose)
// skip: optional per-matrix flags, a matrix whose flag equals skip_value is left untouched.
// t_out: when non-null, the Schur form is returned instead of eigenvectors (v receives Z, t_out T).
void launch_eig(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info, int* sweeps,
                zc* ws, double eps, int max_iter, int group, const int* skip = nullptr, int skip_value = 1,
                zc* t_out = nullptr);
// Hermitian A (only the Hermitian part is used): real eigenvalues in w (imaginary parts 0), orthonormal
// eigenvectors in v; info as launch_eig.
void launch_eig_herm(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info, zc* ws,
                     double eps, int max_iter, int group);
// Per-device launcher state, safe for several host threads and several devices in one process: a zeroed
// device word per (use, device), allocated on its first use with that device current (which 0: the
// rotation counter, 1: the tensor-core products' stuck-wait flag); and a dynamic shared memory opt-in of
// func for the current device, made once per (func, device) and raised when a larger size is needed.
void* device_word(int which, size_t bytes);
void ensure_smem_optin(const void* func, int bytes);
unsigned long long* rotation_counter();  // device counter the Hermitian eigensolver adds its QL rotations to
long long take_rotation_count();         // read and reset it (synchronises the device)
long long eig_workspace_bytes(int n, int batch);
int eig_default_group(int n, int batch);

// Kernel launch accounting for the benchmark's gpu_launches claim.
std::atomic<long long>& launch_count();  // engine launches of this process (all threads)

// Optional CUDA-event timing of the heavy kernels (enabled per context; the context installs its
// timer as the calling thread's current timer for the duration of a call).
enum TimedKind : int { TK_EIG = 0, TK_LU = 1, TK_GEMM = 2, TK_COUNT = 3 };
struct KernelTimer {
    struct Rec {
        int kind;
        cudaEvent_t a, b;
    };
    std::mutex lock;  // calls may run two streams from two host threads (both polarizations at once)
    std::vector<Rec> pending;
    double ms[TK_COUNT] = {0, 0, 0};
    long long count[TK_COUNT] = {0, 0, 0};
    // launch intervals in ms after `base` (recorded when timing is switched on), for busy-time unions
    cudaEvent_t base = nullptr;
    std::vector<std::pair<double, double>> spans[TK_COUNT];
    void collect();
    double busy_ms(int kind);  // length of the union of the kind's launch intervals
    ~KernelTimer();
};
KernelTimer*& current_timer();
class TimedLaunch {
public:
    TimedLaunch(int kind, cudaStream_t st);
    ~TimedLaunch();

private:
    KernelTimer* t_;
    cudaStream_t st_;
    size_t idx_ = 0;
};

struct Options {
    int fast_path = 1;
    int diagnostics = 0;
    int max_iter = 30;
    double eps = 2.220446049250313e-16;
    int eig_group = 0;
};

// Batched 1-D solve (rcwa1d.cu). d_s[p] = nI sin(theta_p) and d_wl[p] = wavelength_p are device
// arrays; results go to the device arrays of d_out. Throws EngineError.
// Near fields of a 1-D solve (include/stablercwa/rcwa1d_fields.hpp:55-189): harmonics of the six field
// components (Ex, Ey, Ez, Hx, Hy, Hz; H is Z0 H) at depths zs (z = 0 at the top of the first layer,
// increasing downwards), from the modes and amplitudes of the same solve. out: device memory of
// n_points x 6 x (2M+1) x nz, out[((p * 6 + c) * (2M+1) + j) * nz + iz].
struct FieldSpec {
    std::vector<double> zs;
    zc* out = nullptr;
    std::vector<std::complex<double>> jones;  // conical: normalised (Es, Ep) per point; empty = (1, 0)
    int* layer_info = nullptr;  // optional, device, n_points x stack layers: planar the number of modes with q
                                // exactly 0 (finite-zero basis), conical 1 where the layer took the Schur basis
};
void solve1d_device(cudaStream_t st, const rcwa_stack1d& stack, const double* d_s, const double* d_wl, int n_points,
                    int M, int pol, const Options& opt, const rcwa_result1d& d_out, size_t chunk_bytes, const FieldSpec* fields = nullptr);
// Device-side check of the sweep points (finite positive wavelength, |theta| < 90) and
// s = nI sin(theta) with the device sin; returns false when some point is invalid.
bool prepare_points_device(cudaStream_t st, const rcwa_point1d* d_points, int n_points, double nI, double* d_s,
                           double* d_wl);

// Batched conical solve (conical.cu). Per-point host-evaluated trigonometry: s_cphi = nI sin(theta)
// cos(phi), ky = nI sin(theta) sin(phi), cphi = cos(phi), sphi = sin(phi), ctheta = cos(theta), wl;
// all device arrays of n_points. Results go to the device arrays of d_out.
struct ConicalPointsDev {
    const double *s_cphi, *ky, *cphi, *sphi, *ctheta, *wl;
};
void solve_conical_device(cudaStream_t st, const rcwa_stack1d& stack, const ConicalPointsDev& pts, int n_points, int M,
                          const Options& opt, const rcwa_result_conical& d_out, size_t chunk_bytes,
                          const FieldSpec* fields = nullptr);
void validate_conical(const rcwa_stack1d& stack, const rcwa_point_conical* h_points, int n_points, int M);

// 2-D crossed gratings (rcwa2d.cu): validation where the reference throws std::invalid_argument,
// the batched solve over host points into host result arrays, and one layer's Fourier operators.
void validate2d(const rcwa_stack2d& stack, const rcwa_point2d* points, int n_points, int M1, int M2, int factorization);
void solve2d_host(cudaStream_t st, const rcwa_stack2d& stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                  int factorization, const Options& opt, const rcwa_result2d& out, size_t chunk_bytes,
                  const FieldSpec* fields = nullptr);  // fields->out: HOST memory, n_points x 6 x N x nz
void layer_operators2d(cudaStream_t st, const rcwa_layer2d& layer, double Lx, double Ly, int M1, int M2,
                       int factorization, rcwa_complex* eps, rcwa_complex* cx, rcwa_complex* cy, int* singular);

// Field slices and phase maps (fields_post.cu).
void field_slice_api(cudaStream_t st, const rcwa_complex* harmonics, int n, int nz, const double* kx, const double* ky,
                     int plane, int nt, double period, double at, rcwa_complex* out);
void phase_data_api(cudaStream_t st, const rcwa_complex* field, int nt, int nz, int reference, const double* incident_k,
                    const double* x, const double* y, const double* z, const rcwa_complex* custom, double phase_floor,
                    int unwrap, double* phase, double* amplitude, unsigned char* mask, rcwa_complex* reference_out);

// Coefficients of one piecewise-constant profile, closed form (method 0) or FFT-sampled (method 1).
void fourier_coefficients_api(cudaStream_t st, const double* edges, const rcwa_complex* values, int K, double period,
                              int hmax, int method, int samples, rcwa_complex* out);

// Validation of a 1-D problem exactly where the reference throws std::invalid_argument.
void validate1d(const rcwa_stack1d& stack, const rcwa_point1d* h_points, int n_points, int M, int pol);

}  // namespace rcwa_gb300
