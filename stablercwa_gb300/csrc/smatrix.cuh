// smatrix.cuh -- batched S-matrix operator algebra shared by the 1-D, conical and 2-D solves.
//
// The reference's operators come in three kinds, Zero / Diag / Dense (include/stablercwa/rcwa1d.hpp:
// 549-629); here each is a B x n vector or a B x n x n matrix holding one operator per sample of a
// chunk, and every operation (product, sum, stack_on, linear solve) is one batched launch. Kinds depend
// only on the structure, so one host-side sequence serves the whole chunk. Vectors that carry several
// right-hand sides (the conical s and p inputs) are B x n x cols, column-major per sample.
#pragma once

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <complex>
#include <vector>

#include "engine.h"
#include "fourier.cuh"
#include "launch.cuh"
#include "rcwa1d_kernels.cuh"

namespace rcwa_gb300 {
namespace {

// ---------------------------------------------------------------- small per-sample vector kernels

__global__ void k0_kernel(int B, const double* __restrict__ wl, double* __restrict__ k0) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B) k0[b] = __ddiv_rn(2.0 * 3.141592653589793238462643383279502884, wl[b]);
}

__global__ void finite_check_kernel(int B, long long per, const zc* __restrict__ a, int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * per) return;
    if (!zfinite(a[idx])) fail[idx / per] = 1;
}

__global__ void eig_info_kernel(int B, const int* __restrict__ info, int* __restrict__ eig_info, int* __restrict__ fail) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    if (info[b] != 0) {
        if (eig_info[b] == 0) eig_info[b] = info[b];
        fail[b] = 1;
    }
}

// out column oc of a B x n x ocols vector = column col of each n x n matrix
__global__ void col_extract_kernel(int B, int n, const zc* __restrict__ m, int col, zc* __restrict__ out, int ocols,
                                   int oc) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const int b = (int)(idx / n), i = (int)(idx - (long long)b * n);
    out[((long long)b * ocols + oc) * n + i] = m[(long long)b * n * n + (long long)col * n + i];
}

// y = s_c * y0 + s_ab * (A x), warp per sample, lanes along rows; the sum over columns is ascending
// like the reference's matrix-vector product (include/stablercwa/matrix.hpp:186-194).
__global__ void matvec_kernel(int B, int n, int cols, const zc* __restrict__ A, const zc* __restrict__ x,
                              const zc* y0, zc* y, double s_ab, double s_c) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    const zc* As = A + b * n * n;
    for (int c = 0; c < cols; ++c) {
        const long long base = (b * cols + c) * n;
        const zc* xs = x + base;
        for (int i = lane; i < n; i += 32) {
            zc acc = zc{0.0, 0.0};
            for (int k = 0; k < n; ++k) acc = zfma(As[(long long)k * n + i], xs[k], acc);
            zc v = zc{s_ab * acc.re, s_ab * acc.im};
            if (y0 && s_c != 0.0) v = zc{s_c * y0[base + i].re + v.re, s_c * y0[base + i].im + v.im};
            y[base + i] = v;
        }
    }
}

// g applied to a vector: diagonal g, or the per-sample dense alternative where alt_flag is set.
__global__ void apply_g_kernel(int B, int n, int cols, int kind, const zc* __restrict__ g, const zc* __restrict__ alt,
                               const int* __restrict__ alt_flag, const zc* __restrict__ x, zc* __restrict__ y) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    const bool dense = kind == 2 || (alt_flag && alt_flag[b]);
    const zc* Ms = kind == 2 ? g + b * n * n : (alt ? alt + b * n * n : nullptr);
    for (int c = 0; c < cols; ++c) {
        const long long base = (b * cols + c) * n;
        const zc* xs = x + base;
        for (int i = lane; i < n; i += 32) {
            zc v;
            if (kind == 0) {
                v = zc{0.0, 0.0};
            } else if (!dense) {
                v = g[b * n + i] * xs[i];
            } else {
                zc acc = zc{0.0, 0.0};
                for (int k = 0; k < n; ++k) acc = zfma(Ms[(long long)k * n + i], xs[k], acc);
                v = acc;
            }
            y[base + i] = v;
        }
    }
}

__global__ void any_flag_kernel(int B, const int* __restrict__ f, int* __restrict__ any) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B && f[b]) atomicOr(any, 1);
}
__global__ void inc_flagged_kernel(int B, const int* __restrict__ f, int* __restrict__ cnt) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B && f[b]) cnt[b] += 1;
}

__global__ void vec_mul_kernel(long long total, const zc* __restrict__ d, const zc* __restrict__ x, zc* __restrict__ y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) y[idx] = d ? d[idx] * x[idx] : zc{0.0, 0.0};
}
__global__ void vec_add_kernel(long long total, const zc* __restrict__ a, zc* __restrict__ y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) y[idx] = a[idx] + y[idx];
}
// down[j] = down[j] / (1 - k[j]) for every column (include/stablercwa/rcwa1d.hpp:997-998)
__global__ void vec_div_one_minus_kernel(int B, int n, int cols, zc* __restrict__ down, const zc* __restrict__ k) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n * cols) return;
    const long long b = idx / ((long long)n * cols);
    const int i = (int)(idx % n);
    down[idx] = zdiv(down[idx], zc{1.0, 0.0} - k[b * n + i]);
}
// Relative eigen-pair residual max_j ||A v_j - l_j v_j|| / (||A||_F ||v_j||), warp per sample
// (include/stablercwa/eig.hpp:38-69); av = A V precomputed.
__global__ void eig_residual_kernel(int B, int n, const zc* __restrict__ A, const zc* __restrict__ AV,
                                    const zc* __restrict__ V, const zc* __restrict__ lam, const int* __restrict__ info,
                                    double* __restrict__ out) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    double fro = 0.0;
    for (long long k = lane; k < nn; k += 32) fro += norm2(A[b * nn + k]);
    for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
    fro = sqrt(fro);
    double worst = 0.0;
    bool nan = info[b] != 0;
    for (int j = 0; j < n; ++j) {
        double dn = 0.0, vn = 0.0;
        const zc l = lam[b * n + j];
        for (int i = lane; i < n; i += 32) {
            const zc v = V[b * nn + (long long)j * n + i];
            dn += norm2(AV[b * nn + (long long)j * n + i] - l * v);
            vn += norm2(v);
        }
        for (int o = 16; o > 0; o >>= 1) {
            dn += __shfl_xor_sync(0xffffffffu, dn, o);
            vn += __shfl_xor_sync(0xffffffffu, vn, o);
        }
        const double val = (sqrt(dn) / fro) / sqrt(vn);
        if (isnan(val)) nan = true;
        worst = fmax(worst, val);
    }
    if (lane == 0) out[b] = (nan || isnan(out[b])) ? __longlong_as_double(0x7ff8000000000000LL) : fmax(out[b], worst);
}

// ---------------------------------------------------------------- batched operator algebra

// KSeam: g = p + alt rp (tp + tm r' of a reduced seam), kept as its three factors and applied to vectors only
enum Kind { KZero = 0, KDiag = 1, KDense = 2, KSeam = 3 };
struct DOp {
    Kind kind = KZero;
    zc* p = nullptr;
    zc* alt = nullptr;           // per-sample dense alternative of a Diag g (exact q == 0 under dense r)
    const int* alt_flag = nullptr;
    zc* rp = nullptr;            // KSeam: r'
};
struct DSBlock {
    DOp Tdd, Rdu, Rud, Tuu;
};
struct Batch {
    cudaStream_t st;
    DeviceScratch* mem;
    int B, n, M;
    int* fail;
    int* extra_solves;
    int n_solve = 0;  // the reference's dense solves per sample (rcwa1d.hpp's count)
    int n_lu = 0;     // the LU factorisations per sample this engine runs
    long long nn() const { return (long long)n * n; }
    zc* dense() { return mem->get<zc>((size_t)B * nn()); }
    zc* vec() { return mem->get<zc>((size_t)B * n); }
};

// linear_solve (include/stablercwa/rcwa1d.hpp:248-281): a zero pivot fails the sample.
zc* solve(Batch& c, zc* a, bool consume_a, int rhs_kind, const zc* rhs, int nrhs = -1) {
    ++c.n_solve;
    ++c.n_lu;
    if (nrhs < 0) nrhs = c.n;
    zc* x = c.mem->get<zc>((size_t)c.B * c.n * nrhs);
    zc* lu = consume_a ? a : c.dense();
    launch_lu_solve(c.st, c.n, nrhs, c.B, a, c.nn(), lu, c.nn(), rhs_kind, rhs,
                    rhs_kind == RHS_DIAG ? c.n : (long long)c.n * nrhs, x, (long long)c.n * nrhs, c.fail);
    if (!consume_a) c.mem->free(lu);
    return x;
}

zc* gemm(Batch& c, const zc* A, long long a_stride, const zc* Bm, const zc* C0, double s_ab, double s_c,
         zc* out = nullptr, const int* skip = nullptr, int skip_value = 1) {
    if (!out) out = c.dense();
    launch_zgemm(c.st, c.n, c.n, c.n, c.B, A, c.n, a_stride, Bm, c.n, c.nn(), C0, c.nn(), out, c.n, c.nn(), s_ab, s_c, skip,
                 skip_value);
    return out;
}

// a * b (include/stablercwa/rcwa1d.hpp:569-580)
DOp op_mul(Batch& c, const DOp& a, const DOp& b) {
    DOp o;
    if (a.kind == KZero || b.kind == KZero) return o;
    const long long nv = (long long)c.B * c.n, nd = (long long)c.B * c.nn();
    if (a.kind == KDiag && b.kind == KDiag) {
        o.kind = KDiag;
        o.p = c.vec();
        LAUNCH(vec_mul_kernel, nblocks(nv), kTpb, c.st, nv, a.p, b.p, o.p);
        return o;
    }
    o.kind = KDense;
    o.p = c.dense();
    if (a.kind == KDiag) {
        LAUNCH(scale_rows_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, b.p, a.p, o.p, nullptr, 1);
    } else if (b.kind == KDiag) {
        LAUNCH(scale_cols_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, a.p, b.p, o.p, nullptr, 1);
    } else {
        gemm(c, a.p, c.nn(), b.p, nullptr, 1.0, 0.0, o.p);
    }
    return o;
}

// a + b (include/stablercwa/rcwa1d.hpp:583-603); reuses a's or b's storage
DOp op_add(Batch& c, DOp a, const DOp& b) {
    if (b.kind == KZero) return a;
    if (a.kind == KZero) return b;
    const long long nv = (long long)c.B * c.n, nd = (long long)c.B * c.nn();
    if (a.kind == KDiag && b.kind == KDiag) {
        LAUNCH(vec_add_kernel, nblocks(nv), kTpb, c.st, nv, b.p, a.p);  // a += b
        return a;
    }
    if (a.kind == KDense && b.kind == KDense) {
        LAUNCH(add_dense_kernel, nblocks(nd), kTpb, c.st, nd, a.p, b.p);
        return a;
    }
    if (a.kind == KDense) {
        LAUNCH(add_diag_kernel, nblocks(nv), kTpb, c.st, c.B, c.n, a.p, b.p, nullptr, 1);
        return a;
    }
    DOp out = b;  // diag a + dense b: dense b with a added to its diagonal
    LAUNCH(add_diag_kernel, nblocks(nv), kTpb, c.st, c.B, c.n, out.p, a.p, nullptr, 1);
    return out;
}

zc* to_dense(Batch& c, const DOp& a) {
    if (a.kind == KDense) return a.p;
    zc* m = c.mem->zeros<zc>((size_t)c.B * c.nn());
    if (a.kind == KDiag) LAUNCH(diag_to_dense_kernel, nblocks((long long)c.B * c.nn()), kTpb, c.st, c.B, c.n, a.p, m, nullptr, 1);
    return m;
}

struct Seam {
    DOp g, r;
};

// include/stablercwa/rcwa1d.hpp:794-808 for blocks whose kinds are uniform over the batch
Seam stack_on(Batch& c, DSBlock&& s, const DOp& r) {
    Seam out;
    DOp k = op_mul(c, s.Rdu, r);
    const long long nv = (long long)c.B * c.n;
    if (k.kind == KZero) {
        out.g = s.Tdd;
    } else if (k.kind == KDiag) {
        // g = (1/(1-k)) Tdd
        if (s.Tdd.kind == KDiag) {
            out.g = {KDiag, c.vec()};
            zc* one = c.vec();
            // reuse the diagonal stack_on kernel for the scalar recurrence on each order
            LAUNCH(stack_on_diag_kernel, nblocks(nv), kTpb, c.st, nv, s.Tdd.p, s.Rdu.p, nullptr, s.Tdd.p, r.p,
                   out.g.p, one);
            c.mem->free(one);
        } else {
            throw EngineError{RCWA_EUNSUPPORTED, "diagonal Rdu r with a dense Tdd"};
        }
    } else {
        zc* ik = k.p;
        LAUNCH(identity_minus_kernel, nblocks((long long)c.B * c.nn()), kTpb, c.st, c.B, c.n, ik, nullptr, 1);
        zc* td = to_dense(c, s.Tdd);
        out.g = {KDense, solve(c, ik, true, RHS_DENSE, td)};
        c.mem->free(ik);
        if (td != s.Tdd.p) c.mem->free(td);
    }
    out.r = op_add(c, s.Rud, op_mul(c, s.Tuu, op_mul(c, r, out.g)));
    return out;
}


// The reduced form of an interface block with a dense side stacked on the reflection r below it. With the
// interface relations d_b = tp d_a + tm u_a, u_b = tm d_a + tp u_a (b below, a above; tp, tm from
// interface_matching) and u_b = r d_b:
//     r' = (tp - r tm)^-1 (r tp - tm),    g = tp + tm r',
// one LU with n right-hand sides (and two products when r is dense) in place of the reference's tp^-1,
// three products, the stacking solve and two more products (rcwa1d.hpp:694-712, :794-808). g is only ever
// applied to vectors, so it stays as its factors (KSeam). tp - r tm = (I - r Rdu) tp is singular exactly
// when tp or I - Rdu r is (Sylvester's determinant identity), so the failing samples are the same;
// n_solve keeps the reference's count.
Seam reduced_seam(Batch& c, zc* tp, zc* tm, const DOp& r) {
    const long long nd = (long long)c.B * c.nn();
    zc* lhs = c.dense();
    zc* rhs = c.dense();
    if (r.kind == KDense) {
        gemm(c, r.p, c.nn(), tm, tp, -1.0, 1.0, lhs);  // tp - r tm
        gemm(c, r.p, c.nn(), tp, tm, 1.0, -1.0, rhs);  // r tp - tm
    } else {
        LAUNCH(seam_system_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, tp, tm, r.kind == KDiag ? r.p : nullptr, lhs, rhs);
    }
    zc* rp = solve(c, lhs, true, RHS_DENSE, rhs);
    if (r.kind != KZero) ++c.n_solve;  // the reference's stacking solve (I - Rdu r)^-1 Tdd
    c.mem->free(lhs);
    c.mem->free(rhs);
    Seam out;
    out.g = {KSeam, tp, tm, nullptr, rp};
    out.r = {KDense, rp};
    return out;
}

// An analytic medium above (diagonal field factors w, v; w = null for the planar form, where w = 1) and a
// dense region below (W, V) with the dense reflection r under the interface. With
// w (d_a + u_a) = W (I + r) d_b and v (d_a - u_a) = V (I - r) d_b:
//     (v W + w V + (v W - w V) r) d_b = 2 w v d_a,  so g = (P + Q r)^-1 diag(2 w v),
// and u_a from the E relation (rows with |w| >= |v|; every row of the planar form) or the H relation:
//     r' = diag(1/w) Z g - I  or  I - diag(1/v) Z g,  Z = W (I + r) or V (I - r) row by row,
// so nothing is divided by a vanishing factor. Three GEMMs and one LU with n right-hand sides for the
// reference's interface matching (two LUs), interface block (one LU, three GEMMs) and stacking (one LU,
// three GEMMs): 35 n^3 instead of 69 n^3 flops. n_solve keeps the reference's count.
Seam analytic_over_dense_seam(Batch& c, const zc* W, const zc* V, const zc* w, const zc* v, const DOp& r) {
    const long long nd = (long long)c.B * c.nn(), nv = (long long)c.B * c.n;
    zc* P = c.dense();
    zc* Q = c.dense();
    LAUNCH(analytic_pq_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, W, V, w, v, P, Q);
    gemm(c, Q, c.nn(), r.p, P, 1.0, 1.0, P);
    zc* dv = c.vec();
    LAUNCH(two_wv_kernel, nblocks(nv), kTpb, c.st, nv, w, v, dv);
    zc* g = solve(c, P, true, RHS_DIAG, dv);
    c.n_solve += 3;  // the reference: W^-1 and V^-1 of the matching, tp^-1, the stacking solve
    c.mem->free(dv);
    LAUNCH(z_rows_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, W, V, w, v, P, Q);  // P, Q reused as Z0, Z1
    gemm(c, Q, c.nn(), r.p, P, 1.0, 1.0, P);                                     // Z = Z0 + Z1 r
    zc* rp = gemm(c, P, c.nn(), g, nullptr, 1.0, 0.0);
    LAUNCH(seam_reflection_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, rp, w, v);
    c.mem->free(P);
    c.mem->free(Q);
    Seam out;
    out.g = {KDense, g};
    out.r = {KDense, rp};
    return out;
}

// y = g x for a KSeam g = tp + tm r' (cols right-hand sides); t is scratch of the size of x
inline void apply_seam(Batch& c, const DOp& g, int cols, const zc* x, zc* t, zc* y) {
    LAUNCH(matvec_kernel, warp_blocks(c.B), 128, c.st, c.B, c.n, cols, g.rp, x, nullptr, t, 1.0, 0.0);
    LAUNCH(matvec_kernel, warp_blocks(c.B), 128, c.st, c.B, c.n, cols, g.alt, t, nullptr, y, 1.0, 0.0);
    LAUNCH(matvec_kernel, warp_blocks(c.B), 128, c.st, c.B, c.n, cols, g.p, x, y, y, 1.0, 1.0);
}

// ---------------------------------------------------------------- Fourier coefficients (host)

using cd = std::complex<double>;
constexpr double kPiD = 3.141592653589793238462643383279502884;

// ---------------------------------------------------------------- FFT-sampled coefficients

// The reference's FFT alternative (include/stablercwa/fourier.hpp:26-83): the profile is sampled at
// S cell midpoints u_j = (j + 1/2) P / S, forward-transformed with 1/S scaling, and bin h is phase-
// corrected by exp(-2 pi i h (origin/P + 1/(2S))). The samples of one segment form a run of equal
// values, and the transform of a run of m samples starting at sample a is the Dirichlet kernel
//     sum_j exp(-2 pi i h j / S) = exp(-i pi h (2a + m - 1) / S) sin(pi h m / S) / sin(pi h / S),
// so the device evaluates exactly the sampled DFT the reference's FFT computes, in O(K H) instead
// of touching all S samples. Angles are reduced in integer arithmetic before sinpi/cospi.
constexpr int kMaxFFTSamples = 4194304;

// Sample count for truncation M (resolve_fft_samples, fourier.hpp:26-43); throws like the reference.
inline int resolve_fft_samples(int M, int samples) {
    if (samples < 0 || samples > kMaxFFTSamples)
        throw EngineError{RCWA_EINVAL, "rcwa: fft_samples must be 0..4194304 (0 for automatic)"};
    if (M < 0) throw EngineError{RCWA_EINVAL, "rcwa: FFT truncation order M must be nonnegative"};
    if (M > (kMaxFFTSamples - 1) / 4) throw EngineError{RCWA_EINVAL, "rcwa: FFT truncation requires more than 4194304 samples"};
    if (samples == 0) {
        const long long target = std::max(8192LL, 64LL * (2LL * M + 1));
        if (target > kMaxFFTSamples) throw EngineError{RCWA_EINVAL, "rcwa: automatic FFT exceeds 4194304 samples"};
        samples = 1;
        while (samples < target) samples *= 2;
    }
    if (samples <= 4 * M) throw EngineError{RCWA_EINVAL, "rcwa: fft_samples must be at least 4*M+1"};
    return samples;
}

// first sample of each segment (K + 1 entries, the last = S): sample j belongs to the last segment
// s with u_j >= edges[s] - edges[0], with u_j evaluated as the reference evaluates it
inline std::vector<long long> fft_runs(const std::vector<double>& edges, int S, double period) {
    const int K = (int)edges.size() - 1;
    std::vector<long long> start(K + 1, 0);
    const auto u = [&](long long j) { return (static_cast<double>(j) + 0.5) / S * period; };
    for (int s = 1; s < K; ++s) {
        const double t = edges[s] - edges.front();
        long long j = (long long)std::ceil(t / period * S - 0.5);
        j = std::min<long long>(std::max<long long>(j, 0), S);
        while (j > 0 && u(j - 1) >= t) --j;
        while (j < S && u(j) < t) ++j;
        start[s] = std::max(j, start[s - 1]);
    }
    start[K] = S;
    return start;
}

__global__ void fft_coeff_kernel(int hmax, int K, long long S, const long long* __restrict__ start,
                                 const zc* __restrict__ vals, const zc* __restrict__ phase, zc* __restrict__ c) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > 2 * hmax) return;
    const long long h = t - hmax;
    const long long two_s = 2 * S;
    zc acc{0.0, 0.0};
    for (int s = 0; s < K; ++s) {
        const long long a = start[s], m = start[s + 1] - a;
        if (m <= 0) continue;
        zc d;
        if (h == 0) {
            d = zc{(double)m, 0.0};
        } else {
            long long r1 = (h * (2 * a + m - 1)) % two_s;
            if (r1 < 0) r1 += two_s;
            long long r2 = (h * m) % two_s;
            if (r2 < 0) r2 += two_s;
            double sp, cp;
            sincospi((double)r1 / (double)S, &sp, &cp);
            const double ratio = sinpi((double)r2 / (double)S) / sinpi((double)h / (double)S);
            d = zc{cp * ratio, -sp * ratio};
        }
        acc = acc + vals[s] * d;
    }
    const double inv = 1.0 / (double)S;
    c[t] = zc{acc.re * inv, acc.im * inv} * phase[t];
}

// FFT-sampled coefficients c[h + hmax] (h = -hmax..hmax) with S samples into device memory
inline zc* fft_coefficients_dev(cudaStream_t st, DeviceScratch& mem, const std::vector<double>& edges,
                                const std::vector<cd>& values, double period, int hmax, int S) {
    const int H = 2 * hmax + 1;
    zc* d = mem.get<zc>(H);
    const std::vector<long long> start = fft_runs(edges, S, period);
    double origin = std::fmod(edges.front(), period);
    if (origin < 0) origin += period;
    const double offset = origin / period + 0.5 / S;
    std::vector<cd> phase(H);
    for (int h = -hmax; h <= hmax; ++h) {
        const double arg = -2.0 * kPiD * h * offset;
        phase[h + hmax] = cd{std::cos(arg), std::sin(arg)};
    }
    long long* d_start = mem.get<long long>(start.size());
    zc* d_vals = mem.get<zc>(values.size());
    zc* d_phase = mem.get<zc>(H);
    RCWA_CUDA(cudaMemcpyAsync(d_start, start.data(), start.size() * sizeof(long long), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_vals, values.data(), values.size() * sizeof(zc), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_phase, phase.data(), H * sizeof(zc), cudaMemcpyHostToDevice, st));
    LAUNCH(fft_coeff_kernel, nblocks(H), kTpb, st, hmax, (int)values.size(), (long long)S, d_start, d_vals, d_phase, d);
    RCWA_CUDA(stream_wait(st));  // the host staging vectors end with this function
    mem.free(d_start);
    mem.free(d_vals);
    mem.free(d_phase);
    return d;
}

// Coefficients c[h + 2M] (h = -2M..2M) of a grating layer's segment values on the device: the closed
// form (fourier_method 0, rcwa1d.hpp:366-388) or the FFT-sampled form (fourier_method 1). A non-finite
// value with the FFT method is the reference's numerical failure (rcwa1d.hpp:392-397): *fail is set.
inline zc* layer_coefficients(cudaStream_t st, DeviceScratch& mem, const std::vector<double>& edges,
                              const std::vector<cd>& values, double period, int M, int method, int samples, int* fail) {
    if (method != 1) return closed_form_coefficients(st, mem, edges, values, period, 2 * M);
    for (const cd& v : values)
        if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) {
            zc* d = mem.zeros<zc>(4 * M + 1);
            static const int one = 1;
            RCWA_CUDA(cudaMemcpyAsync(fail, &one, sizeof(int), cudaMemcpyHostToDevice, st));
            return d;
        }
    return fft_coefficients_dev(st, mem, edges, values, period, 2 * M, resolve_fft_samples(M, samples));
}


// ---------------------------------------------------------------- Hermitian layer operators
//
// A layer of real permittivities has Hermitian Toeplitz operators ([[eps]], [[1/eps]]: c_{-h} = conj(c_h)),
// so its TE matrix Kx^2 - [[eps]] is Hermitian and its TM (and conical B C) eigenproblem is the Hermitian-
// definite pencil (Kx [[eps]]^{-1} Kx - I, [[1/eps]]). Those are solved with the Hermitian eigensolver
// (launch_eig_herm): the same eigenpairs as the general QR to rounding (eigenvectors up to a phase per
// eigenvalue, and any orthonormal basis of a repeated eigenvalue), with orthonormal W. Only with the
// default iteration settings, so that non-default eps / max_iter keep the general solver's semantics.

// The reduced seam algebra (one LU per seam); RCWA_GB300_SEAMS=reference keeps the reference's sequence of
// interface blocks and stacking for timing and comparison.
inline bool reduced_seams_enabled() {
    const char* env = std::getenv("RCWA_GB300_SEAMS");
    return !(env && std::strcmp(env, "reference") == 0);
}

inline bool hermitian_path_enabled(const Options& opt) {
    const char* env = std::getenv("RCWA_GB300_HERMITIAN");
    if (env && env[0] == '0') return false;
    return opt.eps == 2.220446049250313e-16 && opt.max_iter == 30;
}

// True when a grating layer's operators are Hermitian: every segment value (eps, or 1/eps) real, finite and
// nonzero, with a spread of magnitudes below 1e10 so that the Toeplitz matrix of 1/eps stays numerically
// positive definite (its eigenvalues lie between the smallest and largest value; the Cholesky factorisation
// keeps its pivots positive while that ratio is far above n eps). A decision on the inputs alone, taken
// on the host without reading anything back from the device.
inline bool real_profile(const std::vector<std::complex<double>>& values) {
    double lo = INFINITY, hi = 0.0;
    for (const std::complex<double>& v : values) {
        if (v.imag() != 0.0 || !std::isfinite(v.real()) || v.real() == 0.0) return false;
        lo = std::min(lo, std::fabs(v.real()));
        hi = std::max(hi, std::fabs(v.real()));
    }
    return !values.empty() && hi <= 1e10 * lo;
}

// Coefficients of a real profile made exactly conjugate-symmetric on the device (the closed form already is;
// the FFT-sampled form is to rounding).
inline void make_hermitian_coefficients(cudaStream_t st, zc* c, int M) {
    LAUNCH(hermitian_coeff_kernel, nblocks(2 * M + 1), kTpb, st, 2 * M, c);
}

// Cholesky factor T = L L^H of the Hermitian Toeplitz matrix T(i, j) = c[i - j + 2M] (n = 2M + 1), one CTA,
// right-looking: at step j the pivot is the updated T(j, j), column j below it is divided by its square
// root and the trailing lower triangle takes the rank-one update. L is column-major, zero above the
// diagonal, held in global memory (the CTA's barriers order it). A pivot that is not positive and finite
// sets *fail and leaves L incomplete.
__global__ void __launch_bounds__(1024) toeplitz_cholesky_kernel(int M, const zc* __restrict__ c, zc* __restrict__ L,
                                                                 int* __restrict__ fail) {
    const int n = 2 * M + 1, tid = threadIdx.x, nt = blockDim.x;
    __shared__ double s_piv;
    __shared__ int s_bad;
    for (long long idx = tid; idx < (long long)n * n; idx += nt) {
        const int j = (int)(idx / n), i = (int)(idx - (long long)j * n);
        L[idx] = i >= j ? c[i - j + 2 * M] : zc{0.0, 0.0};
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        zc* colj = L + (long long)j * n;
        if (tid == 0) {
            const double d = colj[j].re;
            const int bad = !(d > 0.0) || !isfinite(d);
            s_bad = bad;
            s_piv = bad ? 1.0 : sqrt(d);
            if (bad) atomicOr(fail, 1);
        }
        __syncthreads();
        if (s_bad) return;  // uniform: every thread read the same flag after the barrier
        const double piv = s_piv, rpiv = 1.0 / piv;
        for (int i = j + tid; i < n; i += nt) colj[i] = i == j ? zc{piv, 0.0} : colj[i] * rpiv;
        __syncthreads();
        const int m = n - j - 1;
        for (long long idx = tid; idx < (long long)m * m; idx += nt) {
            const int kk = (int)(idx / m), ii = (int)(idx - (long long)kk * m);
            if (ii < kk) continue;
            const int k = j + 1 + kk, i = j + 1 + ii;
            L[(long long)k * n + i] = zfms(colj[i], conj(colj[k]), L[(long long)k * n + i]);
        }
        __syncthreads();
    }
}

// X = L^{-1} of a lower-triangular L with a real positive diagonal (column-major), one warp per column of X:
// forward substitution down the column, each row's dot product split over the lanes. XH = X^H as well.
__global__ void lower_inverse_kernel(int n, const zc* __restrict__ L, zc* __restrict__ X, zc* __restrict__ XH) {
    const long long j = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= n) return;
    const int lane = threadIdx.x & 31;
    zc* x = X + j * n;
    for (int i = lane; i < n; i += 32) x[i] = zc{0.0, 0.0};
    __syncwarp();
    if (lane == 0) x[j] = zc{1.0 / L[j * n + j].re, 0.0};
    __syncwarp();
    for (int i = (int)j + 1; i < n; ++i) {
        zc s{0.0, 0.0};
        for (int k = (int)j + lane; k < i; k += 32) s = zfma(L[(long long)k * n + i], x[k], s);
        for (int o = 16; o > 0; o >>= 1) {
            s.re += __shfl_xor_sync(0xffffffffu, s.re, o);
            s.im += __shfl_xor_sync(0xffffffffu, s.im, o);
        }
        if (lane == 0) x[i] = s * (-1.0 / L[(long long)i * n + i].re);
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) XH[(long long)i * n + j] = conj(x[i]);
}

// L, L^{-1} and L^{-H} of [[1/eps]] = L L^H for a layer's device coefficients c, all on the device and
// stream-ordered (nothing read back). A failed factorisation sets *fail (the layer's samples then fail);
// real_profile keeps it from happening for the profiles this is called with.
inline void toeplitz_cholesky_inverse(cudaStream_t st, const zc* c, int M, DeviceScratch& mem, int* fail, zc*& Lfac,
                                      zc*& Linv, zc*& LinvH) {
    const int n = 2 * M + 1;
    Lfac = mem.get<zc>((size_t)n * n);
    Linv = mem.get<zc>((size_t)n * n);
    LinvH = mem.get<zc>((size_t)n * n);
    LAUNCH(toeplitz_cholesky_kernel, 1, 1024, st, M, c, Lfac, fail);
    LAUNCH(lower_inverse_kernel, warp_blocks(n), 128, st, n, Lfac, Linv, LinvH);
}

// The four constant parts of a Hermitian-definite pencil layer (E Hermitian, [[1/eps]] = L L^H):
// part[0..2] = L^-1 X L^-H for X = E, (m_i + m_j) E, m_i m_j E and part[3] = L^-1 L^-H, so that for a sample
// with kx_j = a + b m_j, L^-1 (Kx E Kx - I) L^-H = a^2 part[0] + a b part[1] + b^2 part[2] - part[3]: the
// per-sample matrix costs O(n^2) instead of two triangular products. The combination's rounding is a few
// eps of the matrix's norm, the eigensolver's own backward error.
inline void pencil_parts(cudaStream_t st, DeviceScratch& mem, int M, const zc* E, const zc* Linv, const zc* LinvH,
                         zc* part[4]) {
    const int n = 2 * M + 1;
    const size_t nn = (size_t)n * n;
    zc* X1 = mem.get<zc>(nn);
    zc* X2 = mem.get<zc>(nn);
    zc* t = mem.get<zc>(nn);
    LAUNCH(pencil_parts_kernel, nblocks((long long)nn), kTpb, st, n, M, E, X1, X2);
    const zc* X[3] = {E, X1, X2};
    for (int q = 0; q < 4; ++q) {
        part[q] = mem.get<zc>(nn);
        if (q < 3) {
            launch_zgemm(st, n, n, n, 1, X[q], n, 0, LinvH, n, 0, nullptr, 0, t, n, 0, 1.0, 0.0, nullptr, 1, TRI_B_UPPER);
            launch_zgemm(st, n, n, n, 1, Linv, n, 0, t, n, 0, nullptr, 0, part[q], n, 0, 1.0, 0.0, nullptr, 1, TRI_A_LOWER);
        } else {
            launch_zgemm(st, n, n, n, 1, Linv, n, 0, LinvH, n, 0, nullptr, 0, part[q], n, 0, 1.0, 0.0, nullptr, 1,
                         TRI_A_LOWER);
        }
    }
    mem.free(X1);
    mem.free(X2);
    mem.free(t);
}

// out = (E + E^H) / 2 of one n x n matrix
__global__ void hermitian_part_kernel(int n, const zc* __restrict__ E, zc* __restrict__ out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * n) return;
    const int j = idx / n, i = idx - j * n;
    const zc a = E[idx], b = E[(long long)i * n + j];
    out[idx] = zc{0.5 * (a.re + b.re), 0.5 * (a.im - b.im)};
}

// every column of every matrix scaled to unit 2-norm (warp per column); the same column of U (if given) is
// scaled by the same factor
__global__ void normalize_cols_kernel(int B, int n, zc* __restrict__ W, zc* __restrict__ U) {
    const long long col = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (col >= (long long)B * n) return;
    const int lane = threadIdx.x & 31;
    zc* w = W + col * n;
    double big = 0.0;
    for (int i = lane; i < n; i += 32) big = fmax(big, fmax(fabs(w[i].re), fabs(w[i].im)));
    for (int o = 16; o > 0; o >>= 1) big = fmax(big, __shfl_xor_sync(0xffffffffu, big, o));
    if (!(big > 0.0) || !isfinite(big)) return;
    double ssq = 0.0;
    for (int i = lane; i < n; i += 32) ssq += norm2(zdivr(w[i], big));
    for (int o = 16; o > 0; o >>= 1) ssq += __shfl_xor_sync(0xffffffffu, ssq, o);
    const double inv = 1.0 / (big * sqrt(ssq));
    for (int i = lane; i < n; i += 32) w[i] = w[i] * inv;
    if (U)
        for (int i = lane; i < n; i += 32) U[col * n + i] = U[col * n + i] * inv;
}

__global__ void toeplitz_kernel(int M, const zc* __restrict__ c, zc* __restrict__ m) {
    const int n = 2 * M + 1;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * n) return;
    const int j = idx / n, i = idx - j * n;
    m[idx] = c[i - j + 2 * M];
}
}  // namespace
}  // namespace rcwa_gb300
