/* stablercwa_gb300.h -- C ABI of the GB300 RCWA solve engine (libstablercwa_gb300.so).
 *
 * The engine is a drop-in for StableRCWA's solve path. Every entry point below names the
 * StableRCWA interface it replaces (paths are relative to the StableRCWA project root).
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, doubles. Complex numbers are rcwa_complex, laid out as
 *     two doubles {re, im} (the layout of std::complex<double> and cuDoubleComplex).
 *   - Matrices are column-major (element (i, j) at [i + j*rows]), batches are contiguous.
 *   - Return value of every call: RCWA_OK (0) or a negative RCWA_E* code. A negative code means the
 *     call did no work (invalid argument, CUDA error); the message is read with rcwa_gpu_last_error.
 *     Invalid input is rejected exactly where the reference throws std::invalid_argument
 *     (include/stablercwa/rcwa1d.hpp:191-229).
 *   - Numerical failures are per sample, never a call failure: the sample's R/T/DEr/DEt are NaN and
 *     its status word says why, as the reference fills NaN on NumericalFailure
 *     (include/stablercwa/rcwa1d.hpp:1064-1067, :810-816).
 *   - Host-pointer calls copy inputs to the device and results back inside the call. *_dev calls take
 *     device pointers and leave everything resident in device memory (inputs already in HBM).
 *   - A context is internally synchronised: calls from several host threads serialise on it.
 */
#ifndef STABLERCWA_GB300_H
#define STABLERCWA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RCWA_GB300_ABI_VERSION 1

/* call status */
#define RCWA_OK 0
#define RCWA_EINVAL (-1)       /* invalid argument: the reference throws std::invalid_argument */
#define RCWA_ECUDA (-2)        /* CUDA runtime error (no device, launch failure, ...) */
#define RCWA_ENOMEM (-3)       /* device allocation failed */
#define RCWA_EUNSUPPORTED (-4) /* option value the engine does not implement */
#define RCWA_ESCRATCH (-5)     /* problem larger than rcwa_gpu_eig_batch_static's fixed workspace */
#define RCWA_ETIMEOUT (-6)     /* rcwa_gpu_server_wait: the request has not finished yet */
#define RCWA_ENUMERIC (-7)     /* non-finite result where the reference throws std::runtime_error */
#define RCWA_ECANCELLED (-8)   /* rcwa_gpu_server_wait: the server was destroyed before the request started */

/* per-sample status word */
#define RCWA_SAMPLE_OK 0
#define RCWA_SAMPLE_NUMERICAL 1      /* zero pivot / non-finite value: results are NaN */
#define RCWA_SAMPLE_EIG_NOCONV 2     /* an eigensolve hit max_iter: results NaN, eig_info set */
#define RCWA_SAMPLE_RAYLEIGH 3       /* 2-D: an order has kz exactly 0 in a homogeneous region
                                        (include/stablercwa/rcwa2d.hpp:1099-1113): results NaN */

#define RCWA_TE 0
#define RCWA_TM 1
#define RCWA_TE_TM 2  /* rcwa_gpu_solve1d_batch_dev only: both polarizations, TE results then TM */

/* 2-D factorization rule (include/stablercwa/rcwa2d_types.hpp:30) */
#define RCWA_FACTORIZATION_LI 0
#define RCWA_FACTORIZATION_LAURENT 1

typedef struct rcwa_complex {
    double re, im;
} rcwa_complex;

/* One layer (include/stablercwa/rcwa1d.hpp:80-106). homogeneous != 0: a uniform film of index n.
 * Otherwise a grating: n_segments indices n_values[K] and K+1 strictly increasing edges spanning one
 * period. fourier_method 0 = analytic coefficients (the reference default), 1 = FFT-sampled with
 * fft_samples samples (0: automatic; rcwa::FourierMethod, include/stablercwa/fourier.hpp:15-43). */
typedef struct rcwa_layer1d {
    double d;
    int homogeneous;
    rcwa_complex n;
    int n_segments;
    const double* edges;
    const rcwa_complex* n_values;
    int fourier_method;
    int fft_samples;
} rcwa_layer1d;

/* Top to bottom: incident medium nI, layers, exit medium nII (include/stablercwa/rcwa1d.hpp:109-114). */
typedef struct rcwa_stack1d {
    rcwa_complex nI;
    rcwa_complex nII;
    double period;
    int n_layers;
    const rcwa_layer1d* layers;
} rcwa_stack1d;

/* One sweep point (include/stablercwa/rcwa1d.hpp:139). */
typedef struct rcwa_point1d {
    double wavelength;
    double theta_deg;
} rcwa_point1d;

/* Solve options (include/stablercwa/rcwa1d.hpp:116-137, include/stablercwa/eig_types.hpp:25-31).
 * The engine implements eig = QR, linear = LU with partial pivoting and the homogeneous fast path;
 * other values return RCWA_EUNSUPPORTED. rcwa_options_default fills the reference defaults. */
typedef struct rcwa_options {
    int eig_method;            /* 0 = QR (EigMethod::QR) */
    int linear_solver;         /* 0 = LU with partial pivoting (LinearSolver::LUPartial) */
    int homogeneous_fast_path; /* 1 (default) */
    int diagnostics;           /* 1: fill max_eig_residual per sample */
    int eig_max_iter;          /* 30 */
    double eig_eps;            /* DBL_EPSILON */
} rcwa_options;

/* Batched 1-D results; every array is caller-allocated with n_points rows of n = 2M+1 orders
 * (point p, order m at [p*n + m + M]) or n_points entries (include/stablercwa/rcwa1d.hpp:145-164).
 * Optional arrays may be NULL. */
typedef struct rcwa_result1d {
    rcwa_complex* R;
    rcwa_complex* T;
    double* DEr;
    double* DEt;
    int* status;               /* RCWA_SAMPLE_* */
    int* eig_info;             /* optional */
    int* n_eig;                /* optional */
    int* n_dense_solve;        /* optional: the reference's count of dense solves for the point */
    double* max_eig_residual;  /* optional, filled when options.diagnostics */
    int* n_lu;                 /* optional: dense LU factorisations the engine itself ran for the point
                                  (reduced seams need fewer than n_dense_solve; per-layer factorisations
                                  shared by every point of the call are not counted) */
} rcwa_result1d;

/* One conical sweep point (include/stablercwa/rcwa1d_conical.hpp:186). */
typedef struct rcwa_point_conical {
    double wavelength;
    double theta_deg;
    double phi_deg;
} rcwa_point_conical;

/* Batched conical results (include/stablercwa/rcwa1d_conical.hpp:105-183), caller-allocated.
 * n = 2M+1 orders; point p, order m (index m+M): Jones entries at [(p*n + m+M)*4 + k] with
 * k = 0 ss, 1 sp, 2 ps, 3 pp (output <- input); channel efficiencies in the same layout.
 * Optional arrays may be NULL. */
typedef struct rcwa_result_conical {
    rcwa_complex* Jr;
    rcwa_complex* Jt;
    double* DEr;
    double* DEt;
    int* status;                   /* RCWA_SAMPLE_* */
    int* eig_info;                 /* optional */
    int* n_eig;                    /* optional */
    int* n_dense_solve;            /* optional: the reference's count */
    int* n_schur;                  /* optional: layers switched to Schur propagation */
    double* min_abs_lambda;        /* optional */
    int* degenerate_mode_warning;  /* optional */
    double* kx;                    /* optional, n_points * n */
    double* ky;                    /* optional, n_points */
    double* flux_r;                /* optional, n_points * n */
    double* flux_t;                /* optional, n_points * n */
    int* n_lu;                     /* optional: dense LU factorisations the engine ran for the point (as in
                                      rcwa_result1d) */
} rcwa_result_conical;

/* ---- 2-D crossed gratings ------------------------------------------------------------------ */

/* Piecewise-constant x profile of one y strip (include/stablercwa/rcwa2d_types.hpp:40-43):
 * n_segments + 1 increasing edges spanning one x period, n_segments complex indices. */
typedef struct rcwa_xprofile2d {
    int n_segments;
    const double* edges;
    const rcwa_complex* n_values;
} rcwa_xprofile2d;

/* Layer2D (include/stablercwa/rcwa2d_types.hpp:45-71): a uniform layer of index n, or n_strips
 * y strips (n_strips + 1 increasing y_edges spanning one y period), strip k having x_profiles[k]. */
typedef struct rcwa_layer2d {
    double d;
    int homogeneous;
    rcwa_complex n;
    int n_strips;
    const double* y_edges;
    const rcwa_xprofile2d* x_profiles;
} rcwa_layer2d;

/* Stack2D (include/stablercwa/rcwa2d_types.hpp:73-78): incident medium nI (real), layers top
 * down, exit medium nII, periods Lx, Ly. */
typedef struct rcwa_stack2d {
    double nI;
    rcwa_complex nII;
    double Lx;
    double Ly;
    int n_layers;
    const rcwa_layer2d* layers;
} rcwa_stack2d;

/* One 2-D point: the wavelength, angles and Jones vector [Es, Ep] of one rcwa::solve2d call
 * (include/stablercwa/rcwa2d.hpp:1359). */
typedef struct rcwa_point2d {
    double wavelength;
    double theta_deg;
    double phi_deg;
    rcwa_complex Es;
    rcwa_complex Ep;
} rcwa_point2d;

/* Result2D arrays (include/stablercwa/rcwa2d_types.hpp:112-130), caller-allocated, point p and
 * harmonic i = (m+M1)(2M2+1) + (n+M2) at [p*N + i], N = (2M1+1)(2M2+1). Kinematic arrays (Kx, Ky,
 * kzI, kzII, prop_r, prop_t) are filled for every point; the amplitudes and efficiencies are NaN
 * where status is not RCWA_SAMPLE_OK. rayleigh_regions[p*(n_layers+2) + r] is 1 where region r
 * (0 incident medium, 1..n_layers the layers, n_layers+1 exit medium) has an order with kz exactly
 * 0. Arrays marked optional may be NULL. */
typedef struct rcwa_result2d {
    double* Kx;
    double* Ky;
    rcwa_complex* kzI;
    rcwa_complex* kzII;
    rcwa_complex* Ex_r;
    rcwa_complex* Ey_r;
    rcwa_complex* Ez_r;
    rcwa_complex* Ex_t;
    rcwa_complex* Ey_t;
    rcwa_complex* Ez_t;
    rcwa_complex* Rs;
    rcwa_complex* Rp;
    rcwa_complex* Ts;
    rcwa_complex* Tp;
    double* DEr;
    double* DEt;
    unsigned char* prop_r;
    unsigned char* prop_t;
    int* status;                    /* RCWA_SAMPLE_* */
    int* eig_info;                  /* optional */
    int* n_eig;                     /* optional */
    int* n_dense_solve;             /* optional */
    double* max_eig_residual;       /* optional, filled when options.diagnostics */
    unsigned char* rayleigh_regions; /* optional, n_points * (n_layers + 2) */
} rcwa_result2d;

typedef struct rcwa_gpu_config {
    int device;                /* CUDA device ordinal */
    size_t workspace_limit;    /* bytes of device workspace the context may hold; 0 = 8 GiB */
} rcwa_gpu_config;

typedef struct rcwa_gpu_ctx rcwa_gpu_ctx;

int rcwa_gpu_abi_version(void);
void rcwa_options_default(rcwa_options* options);
/* Number of engine kernels launched by this process so far (all contexts). No reference
 * counterpart; it lets a caller count the device launches of a call. */
long long rcwa_gpu_launch_count(void);
/* QL rotations applied by the Hermitian eigensolver (the solve path for layers of real permittivity) on the
 * current device since the previous call; reading resets the count and synchronises the device. For work
 * accounting: each rotation is 6 n real operations on the real eigenvector factor Y (orders up to 904,
 * carried out in 64-bit fixed point on the integer pipes), or 12 n real flops on the complex eigenvector
 * matrix above that order. -1 on a device error. */
long long rcwa_gpu_eig_rotations(void);

/* Context lifetime. No reference counterpart: the reference keeps no state between calls
 * (include/stablercwa/rcwa1d.hpp:851); the context owns the device workspace and stream. */
int rcwa_gpu_create(const rcwa_gpu_config* config, rcwa_gpu_ctx** ctx);
void rcwa_gpu_destroy(rcwa_gpu_ctx* ctx);
/* Copies the last error message of this context (or of a failed create when ctx is NULL). */
int rcwa_gpu_last_error(const rcwa_gpu_ctx* ctx, char* buffer, size_t size);

/* Batched 1-D TE/TM solve over sweep points on one stack: replaces rcwa::sweep
 * (include/stablercwa/rcwa1d.hpp:1084-1091) and, with n_points = 1, rcwa::solve
 * (include/stablercwa/rcwa1d.hpp:1077-1080). Host buffers in and out. */
int rcwa_gpu_solve1d_batch(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point1d* points,
                           int n_points, int M, int polarization, const rcwa_options* options,
                           rcwa_result1d* out);

/* 1-D solve with near fields: rcwa::solve_with_fields + field_at (include/stablercwa/rcwa1d_fields.hpp:55-198)
 * at every point. Besides the results of rcwa_gpu_solve1d_batch, fields receives the harmonics of the six
 * field components at the nz depths zs (z = 0 at the top of the first layer, increasing downwards; z < 0
 * the incident medium, z past the last layer the exit medium; a depth on an interface belongs to the
 * layer above): fields[((p * 6 + c) * (2M+1) + j) * nz + iz], c = Ex, Ey, Ez, Hx, Hy, Hz (H is Z0 H),
 * j the order m + M. Taken from the modes and amplitudes of the same solve; NaN where the point failed.
 * layer_info (optional, n_points x n_layers): the number of the layer's modes with q exactly 0, which the
 * reference propagates in its finite-zero basis (FieldLayerInfo::finite_zero_mode_count). */
int rcwa_gpu_solve1d_fields(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point1d* points, int n_points,
                            int M, int polarization, const rcwa_options* options, const double* zs, int nz,
                            rcwa_result1d* out, rcwa_complex* fields, int* layer_info);

/* Same solve with device-resident sweep points and device-resident result arrays (every pointer in
 * out is a device pointer). The stack description is host memory. Asynchronous with respect to the
 * host on the context's stream; rcwa_gpu_synchronize waits for it. polarization = RCWA_TE_TM solves
 * both polarizations of the points in one call (two sweeps of the reference): every result array
 * then holds 2 n_points entries per point slot, the TE sweep first and the TM sweep after it, and the
 * two sweeps run concurrently on the device (the context's stream and a second one it owns). */
int rcwa_gpu_solve1d_batch_dev(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point1d* d_points,
                               int n_points, int M, int polarization, const rcwa_options* options,
                               rcwa_result1d* d_out);
int rcwa_gpu_synchronize(rcwa_gpu_ctx* ctx);

/* Batched conical-incidence solve over (lambda, theta, phi) points on one stack: replaces
 * rcwa::sweep_conical (include/stablercwa/rcwa1d_conical.hpp:992-999) and, with n_points = 1,
 * rcwa::solve_conical (:985-988). Host buffers in and out. */
int rcwa_gpu_solve_conical_batch(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point_conical* points,
                                 int n_points, int M, const rcwa_options* options, rcwa_result_conical* out);

/* Conical solve with near fields: rcwa::solve_conical_with_fields + field_at(context, zs, jones)
 * (include/stablercwa/rcwa1d_conical_fields.hpp:52-97, :243-248) at every point. jones: 2 complex per
 * point (Es, Ep of the incident field), normalised like rcwa::normalized_jones (rcwa_fields.hpp:218-230);
 * nullptr means (1, 0) everywhere; a non-finite or zero Jones vector is RCWA_EINVAL. Depths and the
 * layout of fields are those of rcwa_gpu_solve1d_fields; NaN where the point failed. layer_info (optional,
 * n_points x n_layers): 1 where the layer took the Schur basis at that point (FieldPropagation::Schur). */
int rcwa_gpu_solve_conical_fields(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point_conical* points,
                                  int n_points, int M, const rcwa_options* options, const rcwa_complex* jones,
                                  const double* zs, int nz, rcwa_result_conical* out, rcwa_complex* fields,
                                  int* layer_info);

/* Fourier coefficients c[h + hmax], h = -hmax..hmax, of a piecewise-constant profile (K values, K + 1
 * increasing edges spanning one period). method 0: the closed form (rcwa::detail::fourier_coefficients,
 * include/stablercwa/rcwa1d.hpp:366-388), on the host; method 1: the FFT of `samples` cell-midpoint
 * samples with the origin and half-cell phase correction (rcwa::fourier_coefficients_fft,
 * include/stablercwa/fourier.hpp:49-83), evaluated on the device. Layers select the same two forms
 * through rcwa_layer1d.fourier_method / fft_samples (0 samples: automatic, as resolve_fft_samples). */
int rcwa_gpu_fourier_coefficients(rcwa_gpu_ctx* ctx, const double* edges, const rcwa_complex* values, int K,
                                  double period, int hmax, int method, int samples, rcwa_complex* out);

/* Batched 2-D solve over points on one stack: replaces rcwa::solve2d
 * (include/stablercwa/rcwa2d.hpp:1359-1413) called once per point, with Options2D::factorization
 * = factorization and the eigensolver / fast-path / diagnostics fields of options (QR and the
 * homogeneous fast path only). Host buffers in and out. */
int rcwa_gpu_solve2d_batch(rcwa_gpu_ctx* ctx, const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points,
                           int M1, int M2, int factorization, const rcwa_options* options, rcwa_result2d* out);

/* 2-D solve with near fields: rcwa::solve2d_with_fields + field_at (include/stablercwa/rcwa2d_fields.hpp:356-390)
 * at every point. Besides the results of rcwa_gpu_solve2d_batch, fields receives the harmonics of the six
 * components at the nz depths zs: fields[((p * 6 + c) * N + j) * nz + iz], N = (2 M1 + 1)(2 M2 + 1), j the
 * harmonic index (m + M1)(2 M2 + 1) + (n + M2), c = Ex, Ey, Ez, Hx, Hy, Hz (H is Z0 H). Region rule of
 * rcwa2d_fields.hpp:117-124: z < 0 region I, z > the stack's bottom region II, else the first layer (zero
 * thickness included) with z <= its bottom + 1e-12. The Jones vector of each point is not normalised (the
 * incident |E| is its 2-norm). NaN where the point failed or hit a Rayleigh anomaly. */
int rcwa_gpu_solve2d_fields(rcwa_gpu_ctx* ctx, const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points,
                            int M1, int M2, int factorization, const rcwa_options* options, const double* zs, int nz,
                            rcwa_result2d* out, rcwa_complex* fields);

/* Real-space slice of one point's field harmonics: rcwa::field_slice / field_map
 * (detail::reconstruct_field_slice and reconstruct_field_grid, include/stablercwa/rcwa_fields.hpp:326-385).
 * harmonics: host, 6 x n x nz in the layout of the field entries above ([(c * n + j) * nz + iz]); kx, ky: the
 * physical wavevector components of each harmonic (the reference's kxm and, per harmonic, its ky: the constant
 * k0 ky of a 1-D solve, kyn of a 2-D one). The horizontal axis is x (RCWA_SLICE_XZ, y = at) or y
 * (RCWA_SLICE_YZ, x = at) at t_it = (it / nt) period. out: host, 6 x nz x nt, out[(c * nz + iz) * nt + it],
 * the value at (t_it, z_iz) = sum_j exp(-i (kx_j x + ky_j y)) harmonics[c][j][iz]. nt <= 0, a non-finite
 * at or a non-positive period is RCWA_EINVAL; a non-finite carrier or result is RCWA_ENUMERIC. */
#define RCWA_SLICE_XZ 0
#define RCWA_SLICE_YZ 1
int rcwa_gpu_field_slice(rcwa_gpu_ctx* ctx, const rcwa_complex* harmonics, int n, int nz, const double* kx,
                         const double* ky, int plane, int nt, double period, double at, rcwa_complex* out);

/* Phase map of one complex scalar grid: rcwa::phase_data (include/stablercwa/rcwa_phase.hpp:229-271).
 * field: host, nz x nt, field[iz * nt + it]. reference: RCWA_PHASE_ABSOLUTE, RCWA_PHASE_INCIDENT (the carrier
 * exp(i (-kx0 x_it - ky0 y_it + kz0 z_iz)) with incident_k = {kx0, ky0, kz0}, the real parts of the incident
 * order's physical wavevector, and the grid coordinates x, y (nt each) and z (nz)) or RCWA_PHASE_CUSTOM
 * (custom: nz x nt values, already broadcast). A value is masked when it is non-finite, its amplitude is at
 * most phase_floor times the largest finite amplitude, or its reference is non-finite or zero. unwrap: none,
 * along the horizontal axis, along z, or both (horizontal first). Outputs (host, nz x nt): phase (NaN where
 * masked), amplitude, mask (1 = masked) and, when reference_out != NULL and a reference is used, the
 * reference. */
#define RCWA_PHASE_ABSOLUTE 0
#define RCWA_PHASE_INCIDENT 1
#define RCWA_PHASE_CUSTOM 2
#define RCWA_UNWRAP_NONE 0
#define RCWA_UNWRAP_X 1
#define RCWA_UNWRAP_Z 2
#define RCWA_UNWRAP_BOTH 3
int rcwa_gpu_phase_data(rcwa_gpu_ctx* ctx, const rcwa_complex* field, int nt, int nz, int reference,
                        const double* incident_k, const double* x, const double* y, const double* z,
                        const rcwa_complex* custom, double phase_floor, int unwrap, double* phase, double* amplitude,
                        unsigned char* mask, rcwa_complex* reference_out);

/* The Fourier operators Eps, Cx, Cy of one patterned layer, each N x N column-major with row and
 * column index (m+M1)(2M2+1) + (n+M2): replaces rcwa::detail2d::layer_operators
 * (include/stablercwa/rcwa2d_operators.hpp:325-429). Invalid geometry or indices return
 * RCWA_EINVAL (the reference's std::invalid_argument); a singular inverse-rule Toeplitz matrix or
 * a non-finite operator (the reference's std::runtime_error) sets *singular to 1. */
int rcwa_gpu_layer_operators2d(rcwa_gpu_ctx* ctx, const rcwa_layer2d* layer, double Lx, double Ly, int M1, int M2,
                               int factorization, rcwa_complex* eps, rcwa_complex* cx, rcwa_complex* cy, int* singular);

/* The context's CUDA stream (a cudaStream_t), for callers that order their own work or events
 * against the engine's. No reference counterpart. */
void* rcwa_gpu_stream(rcwa_gpu_ctx* ctx);

/* Per-kernel device timing on the context's stream. No reference counterpart: the reference's
 * Timing{eig, linear, product} (include/stablercwa/rcwa1d.hpp:141-143) is host wall time per solve.
 * With timing enabled, CUDA events bracket every launch of the eigensolver ("eig"), the LU solve
 * ("lu") and the GEMM ("gemm"); rcwa_gpu_kernel_time reads the accumulated milliseconds and launch
 * count of one kind (after the work has finished) and resets it. */
int rcwa_gpu_set_kernel_timing(rcwa_gpu_ctx* ctx, int enable);
int rcwa_gpu_kernel_time(rcwa_gpu_ctx* ctx, const char* kind, double* milliseconds, long long* launches);
/* Busy time of one kind since the last query: the length of the union of its launch intervals, which
 * is less than the summed durations when launches of both polarizations overlap. */
int rcwa_gpu_kernel_busy(rcwa_gpu_ctx* ctx, const char* kind, double* milliseconds);

/* Batched general complex eigensolver, CORTH + COMQR2 (include/stablercwa/eig_qr.hpp:1008-1124):
 * the engine behind Options::custom_eig (include/stablercwa/rcwa1d.hpp:122-124). a holds batch
 * n x n matrices; values[batch*n], vectors[batch*n*n] (2-norm normalised columns), info[batch]
 * (0 or the 1-based index of the eigenvalue that hit max_iter), sweeps[batch] (may be NULL). */
int rcwa_gpu_eig_batch(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* a, double eps, int max_iter,
                       rcwa_complex* values, rcwa_complex* vectors, int* info, int* sweeps);
int rcwa_gpu_eig_batch_dev(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* d_a, double eps,
                           int max_iter, rcwa_complex* d_values, rcwa_complex* d_vectors, int* d_info,
                           int* d_sweeps);

/* Batched Hermitian eigensolver. No counterpart in the reference: the solver the engine uses for layers
 * with real permittivities (Householder tridiagonalisation, implicit QL with Wilkinson shifts, eigenvectors
 * accumulated). It solves the Hermitian part (a + a^H) / 2 of each of the batch n x n matrices in a (a itself
 * when a is Hermitian). values[batch*n] are real (imaginary parts 0) in the order the QL iteration leaves
 * them, not sorted; vectors[batch*n*n] have orthonormal columns; info[batch] is 0 or the 1-based index of
 * the eigenvalue that hit max_iter. eps and max_iter as in rcwa_gpu_eig_batch. */
int rcwa_gpu_eig_hermitian_batch(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* a, double eps, int max_iter,
                                 rcwa_complex* values, rcwa_complex* vectors, int* info);
int rcwa_gpu_eig_hermitian_batch_dev(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* d_a, double eps,
                                     int max_iter, rcwa_complex* d_values, rcwa_complex* d_vectors, int* d_info);

/* Batched eigensolver that allocates nothing. No counterpart in the reference: it is the
 * rcwa_gpu_eig_batch_dev computation (same kernel and default lanes per matrix, so the same results) for callers
 * that may not allocate device memory -- a host whose own caching allocator holds the HBM, or a
 * latency-bound loop that cannot pay for an allocator call or the synchronisation a free implies.
 * The per-matrix workspace, 16 * (3n^2 + 4n + 8) bytes, comes from one fixed device array of
 * RCWA_GPU_EIG_STATIC_SCRATCH_BYTES per device (about 94 matrices of n = 121); a larger
 * batch * workspace returns RCWA_ESCRATCH without launching. Arguments as rcwa_gpu_eig_batch_dev,
 * all device pointers, with stream a cudaStream_t (NULL: the legacy default stream) in place of a
 * context; the work is queued on that stream and the call returns without waiting for it.
 * The first call with a device current looks up that device's array and loads the kernels; make it
 * before any stream capture begins on the device. Calls that overlap in time on one device (on
 * different streams, or unordered host threads) share the array and race; calls on one stream are
 * ordered. It never starts the autotuner (tuning allocates trial buffers): a form recorded for the key
 * is used, else the built-in rule. Errors are reported by the return code only. */
#define RCWA_GPU_EIG_STATIC_SCRATCH_BYTES (64ULL << 20)
int rcwa_gpu_eig_batch_static(void* stream, int n, int batch, const rcwa_complex* d_a, double eps,
                              int max_iter, rcwa_complex* d_values, rcwa_complex* d_vectors, int* d_info,
                              int* d_sweeps);

/* Batched A X = B with partial-pivot LU (include/stablercwa/lu.hpp:427-436): the engine behind
 * Options::custom_solve (include/stablercwa/rcwa1d.hpp:130-136). a: batch n x n, b: batch n x nrhs,
 * x: batch n x nrhs. singular[batch] is 1 where a zero pivot appeared (the reference throws
 * std::runtime_error there); x is then NaN. */
int rcwa_gpu_solve_batch(rcwa_gpu_ctx* ctx, int n, int nrhs, int batch, const rcwa_complex* a,
                         const rcwa_complex* b, rcwa_complex* x, int* singular);

/* Batched C = A B (include/stablercwa/matrix.hpp:170-192): the engine behind
 * Options::custom_multiply (include/stablercwa/rcwa1d.hpp:125-129). a: batch m x k, b: batch k x n. */
int rcwa_gpu_multiply_batch(rcwa_gpu_ctx* ctx, int m, int k, int n, int batch, const rcwa_complex* a,
                            const rcwa_complex* b, rcwa_complex* c);

/* Host-only argument checks of the three solves, the checks rcwa::solve, rcwa::solve_conical and
 * rcwa::solve2d make before any work (include/stablercwa/rcwa1d.hpp:191-229, rcwa1d_conical.hpp:688-689,
 * rcwa2d.hpp:1042-1070): RCWA_OK, or RCWA_EINVAL with the reference's std::invalid_argument message
 * copied into message (size bytes, NUL-terminated). No device is needed; the batched solves make the
 * same checks themselves. */
int rcwa_validate_solve1d(const rcwa_stack1d* stack, const rcwa_point1d* points, int n_points, int M, int polarization,
                          char* message, size_t size);
int rcwa_validate_solve_conical(const rcwa_stack1d* stack, const rcwa_point_conical* points, int n_points, int M,
                                char* message, size_t size);
int rcwa_validate_solve2d(const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                          int factorization, char* message, size_t size);

/* No reference counterpart: the autotuner of the eigensolvers' kernel form. The batched eigensolvers run
 * a matrix on G = 4..32 lanes of a warp, on a CTA of 64, 128 or 256 threads, or (general solver, order
 * >= 384) on a thread-block cluster; a fixed rule picks one unless a tuned form is recorded for the key
 * (solver, order, batch size rounded down to a power of two). rcwa_gpu_autotune_eig times every
 * applicable form on batch device matrices d_a (column-major, n x n each) on the context's stream, keeps
 * only forms that converge where the rule's form does, records the fastest for the key and returns it in
 * *form (-1 = cluster, else threads per matrix) with its time in *milliseconds. hermitian selects the
 * Hermitian solver (lossless layers) instead of the general one. rcwa_gpu_autotune_set records a form
 * directly (a table saved earlier); rcwa_gpu_autotune_table writes the table as text lines
 * "<general|hermitian> <order> <batch bucket> <form>" and returns its length. The table is process-wide.
 * RCWA_GB300_AUTOTUNE=0 makes the solves ignore it; =auto also tunes each new key (at least 64 matrices)
 * on the first call that meets it, on that call's own matrices. */
int rcwa_gpu_autotune_eig(rcwa_gpu_ctx* ctx, int hermitian, int n, int batch, const rcwa_complex* d_a, int* form,
                          double* milliseconds);
int rcwa_gpu_autotune_set(int hermitian, int n, int batch, int form);
int rcwa_gpu_autotune_table(char* buffer, size_t size);

/* No reference counterpart: how the engine forms its complex products. Products whose three orders are
 * all >= 16 with m n k >= 2^15 run on the tensor cores (tcgen05, bf16 digit slices of each FP64 operand, exact FP32
 * accumulation of the slice products, FP64 sums: accurate to about k 2^-53 of the largest entries of
 * the row and column, like an FP64 GEMM) unless RCWA_GB300_GEMM=fp64 is set, in which case every product
 * runs on the FP64 pipe. *tensor_cores: 1 when the tensor-core path is on; *slices: digits per operand
 * (RCWA_GB300_TC_SLICES, default 7); *stuck: nonzero once a tensor-core product kernel gave up on a
 * wait that never completed (its output was then not written). Any pointer may be NULL. */
int rcwa_gpu_gemm_info(int* tensor_cores, int* slices, int* stuck);

/* ---- Serving: a request loop over worker slots -------------------------------------------- */

/* No reference counterpart: the reference serves one solve per call (rcwa_json.hpp:1287-1312,
 * the CLI). The server keeps `slots` engine contexts, each with its own CUDA stream and host
 * worker. Submitted requests (deep-copied, so the caller's buffers may be released at once) wait
 * in queues bucketed by matrix order; a free slot takes the oldest request whose estimated device
 * footprint fits what remains of hbm_budget, else the oldest smaller one (backfilling, bounded so
 * the oldest is never passed over for longer than max_bypass_ms). Requests on different slots run
 * concurrently on the device. Each request is one solve: 1-D (rcwa::solve), conical
 * (rcwa::solve_conical) or 2-D (rcwa::solve2d). A slot that takes a request also takes up to
 * max_batch - 1 queued requests that differ from it only in the point (wavelength, angles, Jones
 * vector) and solves them in one batched call; their results equal the lone ones within the parity
 * tolerances (1e-10 on efficiencies), and rcwa_response.batch reports the call's size. Creating a
 * server runs a few small solves on one context first, so that CUDA has loaded the engine's kernels
 * before the slots start. */
#define RCWA_REQ_1D 0
#define RCWA_REQ_CONICAL 1
#define RCWA_REQ_2D 2

typedef struct rcwa_server_config {
    int device;
    int slots;              /* concurrent requests on the device (worker slots); 0 = 32 */
    size_t hbm_budget;      /* bytes the admitted requests may hold together; 0 = 80 % of free memory */
    int max_bypass_ms;      /* how long backfilling may pass over the oldest request; 0 = 2000 */
    int max_batch;          /* queued requests of one structure solved together in one call; 0 = 256, 1 = never */
} rcwa_server_config;

typedef struct rcwa_request {
    int kind;                       /* RCWA_REQ_* */
    const rcwa_stack1d* stack1d;    /* 1-D and conical */
    const rcwa_stack2d* stack2d;    /* 2-D */
    double wavelength;
    double theta_deg;
    double phi_deg;                 /* conical and 2-D */
    int M;                          /* 1-D and conical truncation */
    int polarization;               /* 1-D: RCWA_TE / RCWA_TM */
    int M1, M2, factorization;      /* 2-D */
    rcwa_complex Es, Ep;            /* 2-D Jones vector */
    rcwa_options options;
} rcwa_request;

/* Timing of one request on the server's clock (seconds since the server was created). */
typedef struct rcwa_response {
    int code;           /* return code of the solve (RCWA_OK or an RCWA_E* code) */
    int slot;           /* worker slot that ran it */
    double submit_s;
    double start_s;
    double finish_s;
    double footprint_bytes;  /* device footprint the admission charged */
    int batch;               /* requests solved in the same call as this one (1: alone) */
} rcwa_response;

typedef struct rcwa_gpu_server rcwa_gpu_server;
int rcwa_gpu_server_create(const rcwa_server_config* config, rcwa_gpu_server** server);
/* Stops the server: requests still queued are cancelled (their waiters return RCWA_ECANCELLED),
 * requests already running finish, and the call returns once every thread blocked in
 * rcwa_gpu_server_wait has left it. No call may use the server after destroy has begun. */
void rcwa_gpu_server_destroy(rcwa_gpu_server* server);
/* Validates the request's shape (the solve itself validates the physics) and queues it. */
int rcwa_gpu_server_submit(rcwa_gpu_server* server, const rcwa_request* request, unsigned long long* ticket);
/* Waits up to timeout_ms (< 0: forever) for the request, then copies its result into result (an
 * rcwa_result1d*, rcwa_result_conical* or rcwa_result2d* of host arrays sized for one point, by
 * kind; may be NULL) and releases it. Returns RCWA_OK, RCWA_ETIMEOUT if it has not finished, or
 * RCWA_ECANCELLED if the server was destroyed before the request started. A ticket is released by the
 * first wait that returns its result; any other wait on it, concurrent or later, returns RCWA_EINVAL. */
int rcwa_gpu_server_wait(rcwa_gpu_server* server, unsigned long long ticket, int timeout_ms, rcwa_response* response,
                         void* result);
/* ---- JSON front end ------------------------------------------------------------------------- */

/* rcwa::solve_json_reply (include/stablercwa/rcwa_json.hpp:1287-1309): one JSON request (mode "planar",
 * "conical" or "periodic2d"; one point or a "points" array) in, one JSON reply out, in the reference's wire
 * format: {"ok": true, "version": 1, "mode", "M", ["My",] "orders", "threads", "results": [...]} with the
 * reference's per-point fields and order, or {"ok": false, "error": message, "where": field path} for a
 * request error (unknown keys, invalid values, and the options this engine does not implement: eig "lr",
 * linear "lu_nopivot" / "qr", homogeneous_fast_path false, backend "mkl"). Numbers are the engine's results
 * written with the shortest round-trip decimal (NaN and infinities as null). indent < 0: one line; >= 0:
 * objects one item per line. *reply is allocated here (free it with rcwa_json_free); *ok (may be NULL) is the
 * reply's "ok". rcwa_gpu_solve_json runs all points as one batched call on ctx; rcwa_gpu_server_solve_json
 * submits one serving-loop request per point and waits for them; rcwa_json_validate only checks the request
 * (*reply is "" when it is valid) and needs no device. Return RCWA_OK whenever a reply was produced. */
int rcwa_gpu_solve_json(rcwa_gpu_ctx* ctx, const char* request, int indent, char** reply, int* ok);
int rcwa_gpu_server_solve_json(rcwa_gpu_server* server, const char* request, int indent, char** reply, int* ok);
int rcwa_json_validate(const char* request, int indent, char** reply, int* ok);
void rcwa_json_free(char* reply);

/* The near-field protocol, rcwa::solve_fields_json_reply (include/stablercwa/rcwa_fields_json.hpp):
 * {"solve": <a one-point request of rcwa_gpu_solve_json; conical needs an "input">, "sampling": {"z": [...],
 * "nx": n, "y": y} (planar / conical) or {"z": [...], "plane": "xz" | "yz", "nt": n, "at": a} (periodic2d),
 * "output_dir": a directory that must not exist yet, "request_id": a 1..128 byte token}. The point is solved
 * with its fields on ctx; the map / slice at the depths and its absolute and incident-referenced phase maps
 * (floor 1e-6, not unwrapped) are formed on the device and written as fields.npy <c16 [6, nz, n],
 * phase.npy <f8 [2, 6, nz, n], phase_mask.npy |u1 [2, 6, nz, n], x.npy (and t.npy, y.npy in 2-D) and z.npy
 * into a temporary sibling directory that is renamed onto output_dir at the end. The reply is the far-field
 * reply of that point followed by "protocol": "stablercwa-fields" and the "field_data" manifest; a failed
 * solve, a non-finite sample or an existing output_dir gives {"ok": false, ..., "where": "fields"} and
 * publishes nothing. Reply handling as rcwa_gpu_solve_json. */
int rcwa_gpu_solve_fields_json(rcwa_gpu_ctx* ctx, const char* request, int indent, char** reply, int* ok);
/* The request checks of rcwa_gpu_solve_fields_json alone (no solve, no files, no device): *reply is "" when
 * the request is valid, else the error reply. */
int rcwa_fields_json_validate(const char* request, int indent, char** reply, int* ok);

#ifdef __cplusplus
}
#endif

#endif /* STABLERCWA_GB300_H */
