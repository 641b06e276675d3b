// linalg.cuh -- batched complex FP64 LU solve and GEMM for sm_103a.
//
// Both are bound by the FP64 pipe (about 2 lane-FMAs per clock per SM on GB300), not by memory: a
// complex multiply-add is 4 FP64 FMAs per 16-32 bytes touched, and GB300's HBM/L2 deliver far more
// bytes per FP64 operation than that. So the kernels spend nothing on elaborate tiling; they keep
// every lane busy with independent FP64 work and read operands coalesced (column-major, lanes along
// rows) or as warp broadcasts.
#pragma once

#include "common.cuh"

namespace rcwa_gb300 {

// Batched A X = B with partial pivoting, one warp per system (include/stablercwa/lu.hpp:268-396 and
// :233-266). Pivot: first entry of largest |z| (hypot) at or below the diagonal; multipliers
// a*(1/pivot) unless 1/pivot overflows; a zero pivot marks the system singular and the step is
// skipped, exactly as the reference continues past it before refusing to solve. The right-hand
// sides are eliminated together with the matrix (an augmented sweep performs the same per-element
// operations, in the same order, as factor-then-forward-substitute), then back-substituted.
//
// a      : batch n x n (column-major), read; factored into lu (may alias a when in_place)
// rhs    : RHS_DENSE: batch n x nrhs; RHS_DIAG: batch n-vectors (nrhs = n); RHS_IDENTITY: none
// x      : batch n x nrhs output
// skip   : optional per-system flag; a nonzero entry leaves that system untouched
// singular: per-system output flag (set to 1 on a zero pivot, never cleared)
__global__ void __launch_bounds__(128) lu_solve_kernel(int n, int nrhs, int batch, const zc* a, long long a_stride,
                                                       zc* lu, long long lu_stride, int rhs_kind, const zc* rhs,
                                                       long long rhs_stride, zc* x, long long x_stride,
                                                       int* __restrict__ singular,
                                                       const int* __restrict__ skip, int skip_value) {
    const long long sys = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (sys >= batch) return;
    if (skip && skip[sys] == skip_value) return;
    const int lane = threadIdx.x & 31;
    const zc* A = a + sys * a_stride;
    zc* L = lu + sys * lu_stride;
    zc* Xs = x + sys * x_stride;
    const long long nn = (long long)n * n;
    if (L != A)
        for (long long i = lane; i < nn; i += 32) L[i] = A[i];
    const long long xn = (long long)n * nrhs;
    if (rhs_kind == RHS_DENSE) {
        const zc* Bs = rhs + sys * rhs_stride;
        if (Bs != Xs)
            for (long long i = lane; i < xn; i += 32) Xs[i] = Bs[i];
    } else {
        const zc* d = rhs_kind == RHS_DIAG ? rhs + sys * rhs_stride : nullptr;
        for (long long i = lane; i < xn; i += 32) {
            const int c = (int)(i / n), r = (int)(i - (long long)c * n);
            Xs[i] = r == c ? (d ? d[r] : zc{1.0, 0.0}) : zc{0.0, 0.0};
        }
    }
    __syncwarp();
    int sing = 0;
    for (int k = 0; k < n; ++k) {
        zc* ck = L + (long long)k * n;
        // pivot search: first index of the largest |z| in rows k..n-1
        double best = -1.0;
        int bi = n;
        for (int i = k + lane; i < n; i += 32) {
            const double v = zabs(ck[i]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        const int p = (best < 0.0 || bi >= n) ? k : bi;  // all-NaN column: keep the diagonal
        if (p != k) {
            for (int c = lane; c < n; c += 32) {
                zc* col = L + (long long)c * n;
                const zc t = col[k];
                col[k] = col[p];
                col[p] = t;
            }
            for (int c = lane; c < nrhs; c += 32) {
                zc* col = Xs + (long long)c * n;
                const zc t = col[k];
                col[k] = col[p];
                col[p] = t;
            }
        }
        __syncwarp();
        const zc piv = ck[k];
        if (is_zero(piv)) {
            sing = 1;
            for (int i = k + 1 + lane; i < n; i += 32) ck[i] = zc{0.0, 0.0};
            __syncwarp();
            continue;
        }
        const zc inv = zinv(piv);
        const bool inv_ok = zfinite(inv);
        // multipliers for the rows this lane owns (at most 8 register slots; rows beyond stay in memory)
        for (int i = k + 1 + lane; i < n; i += 32) ck[i] = inv_ok ? ck[i] * inv : zdiv(ck[i], piv);
        // trailing update of matrix columns and right-hand sides: col[i] -= l_i * col[k]
        for (int c = k + 1; c < n + nrhs; ++c) {
            zc* col = c < n ? L + (long long)c * n : Xs + (long long)(c - n) * n;
            const zc t = col[k];
            if (is_zero(t)) continue;
            for (int i = k + 1 + lane; i < n; i += 32) col[i] = zfms(ck[i], t, col[i]);
        }
        __syncwarp();
    }
    if (sing) {
        // the reference refuses to solve (std::runtime_error); the solution is reported as NaN
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        for (long long i = lane; i < xn; i += 32) Xs[i] = zc{nan, nan};
        if (lane == 0) singular[sys] = 1;
        return;
    }
    // back substitution U X = Y
    if (nrhs >= 16) {
        // lanes own right-hand-side columns
        for (int c = lane; c < nrhs; c += 32) {
            zc* xc = Xs + (long long)c * n;
            for (int k = n - 1; k >= 0; --k) {
                const zc* uk = L + (long long)k * n;
                const zc xk = zdiv(xc[k], uk[k]);
                xc[k] = xk;
                if (is_zero(xk)) continue;
                for (int i = 0; i < k; ++i) xc[i] = zfms(uk[i], xk, xc[i]);
            }
        }
    } else {
        // lanes own rows
        for (int c = 0; c < nrhs; ++c) {
            zc* xc = Xs + (long long)c * n;
            for (int k = n - 1; k >= 0; --k) {
                const zc* uk = L + (long long)k * n;
                const zc xk = zdiv(xc[k], uk[k]);
                __syncwarp();
                if (lane == (k & 31)) xc[k] = xk;
                if (!is_zero(xk))
                    for (int i = lane; i < k; i += 32) xc[i] = zfms(uk[i], xk, xc[i]);
                __syncwarp();
            }
        }
    }
}

// ---------------------------------------------------------------- blocked LU for large n
//
// The same partial-pivot elimination of [A | B] as lu_solve_kernel, reorganised for orders where a
// warp per system cannot keep the trailing matrix anywhere near the FP64 pipe: panels of nb columns
// are factored by one CTA per system (pivot search, full-row swaps over A and the right-hand sides,
// multipliers, rank-1 updates inside the panel), the panel rows of the remaining columns are solved
// with the unit lower triangle (same subtraction order as the unblocked sweep), and the trailing
// matrix and right-hand sides are updated with zgemm_kernel. Back substitution runs block by block
// from the bottom: a triangular solve of the block rows, then a GEMM update of the rows above.

__device__ __forceinline__ zc* aug_col(zc* L, zc* X, int n, int c) {
    return c < n ? L + (long long)c * n : X + (long long)(c - n) * n;
}

// lu = a (if distinct), x = rhs (dense, identity or diagonal)
__global__ void lu_init_kernel(int n, int nrhs, int batch, const zc* a, long long a_stride, zc* lu, long long lu_stride,
                               int rhs_kind, const zc* rhs, long long rhs_stride, zc* x, long long x_stride,
                               const int* __restrict__ skip, int skip_value) {
    const long long per = (long long)n * (n + nrhs);
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)batch * per) return;
    const long long sys = idx / per;
    if (skip && skip[sys] == skip_value) return;
    const long long e = idx - sys * per;
    const long long nn = (long long)n * n;
    if (e < nn) {
        const zc* A = a + sys * a_stride;
        zc* L = lu + sys * lu_stride;
        if (L != A) L[e] = A[e];
        return;
    }
    const long long xe = e - nn;
    zc* Xs = x + sys * x_stride;
    if (rhs_kind == RHS_DENSE) {
        const zc* Bs = rhs + sys * rhs_stride;
        if (Bs != Xs) Xs[xe] = Bs[xe];
    } else {
        const int c = (int)(xe / n), r = (int)(xe - (long long)c * n);
        const zc* d = rhs_kind == RHS_DIAG ? rhs + sys * rhs_stride : nullptr;
        Xs[xe] = r == c ? (d ? d[r] : zc{1.0, 0.0}) : zc{0.0, 0.0};
    }
}

// The same panel factorisation with one warp per system (rows strided over the lanes, warp shuffles for
// the pivot search, no block barriers): the form for many systems of moderate order, where a CTA per
// system spends most of its time in barriers. Same pivot rule and the same arithmetic per element as
// lu_panel_kernel, so the factors are identical.
__global__ void __launch_bounds__(128) lu_panel_warp_kernel(int n, int nrhs, int batch, zc* lu, long long lu_stride, zc* x,
                                                            long long x_stride, int k0, int nb, int* __restrict__ sing_local,
                                                            const int* __restrict__ skip, int skip_value) {
    const long long sys = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (sys >= batch) return;
    if (skip && skip[sys] == skip_value) return;
    const int lane = threadIdx.x & 31;
    zc* L = lu + sys * lu_stride;
    zc* X = x + sys * x_stride;
    const int kend = min(k0 + nb, n);
    for (int j = k0; j < kend; ++j) {
        zc* col = L + (long long)j * n;
        double best = -1.0;
        int bi = n;
        for (int i = j + lane; i < n; i += 32) {
            const double v = zabs(col[i]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        const int p = (best < 0.0 || bi >= n) ? j : bi;  // all-NaN column: keep the diagonal
        if (p != j) {
            for (int c = lane; c < n + nrhs; c += 32) {
                zc* cc = aug_col(L, X, n, c);
                const zc t = cc[j];
                cc[j] = cc[p];
                cc[p] = t;
            }
            __syncwarp();
        }
        const zc piv = col[j];
        if (is_zero(piv)) {
            if (lane == 0) sing_local[sys] = 1;
            for (int i = j + 1 + lane; i < n; i += 32) col[i] = zc{0.0, 0.0};
            __syncwarp();
            continue;
        }
        const zc inv = zinv(piv);
        const bool inv_ok = zfinite(inv);
        for (int i = j + 1 + lane; i < n; i += 32) col[i] = inv_ok ? col[i] * inv : zdiv(col[i], piv);
        // each lane updates the rows whose multipliers it just wrote; row j of the panel's columns was
        // settled by the swap above
        for (int c = j + 1; c < kend; ++c) {
            zc* cc = L + (long long)c * n;
            const zc u = cc[j];
            for (int i = j + 1 + lane; i < n; i += 32) cc[i] = zfms(col[i], u, cc[i]);
        }
        __syncwarp();
    }
}

// Factor columns k0 .. k0+nb-1 (all rows below the diagonal), one 256-thread CTA per system.
__global__ void __launch_bounds__(256) lu_panel_kernel(int n, int nrhs, int batch, zc* lu, long long lu_stride, zc* x,
                                                       long long x_stride, int k0, int nb, int* __restrict__ sing_local,
                                                       const int* __restrict__ skip, int skip_value) {
    const long long sys = blockIdx.x;
    if (sys >= batch) return;
    if (skip && skip[sys] == skip_value) return;
    __shared__ double s_best[8];
    __shared__ int s_idx[8];
    __shared__ int s_piv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    zc* L = lu + sys * lu_stride;
    zc* X = x + sys * x_stride;
    const int kend = min(k0 + nb, n);
    for (int j = k0; j < kend; ++j) {
        zc* col = L + (long long)j * n;
        double best = -1.0;
        int bi = n;
        for (int i = j + tid; i < n; i += 256) {
            const double v = zabs(col[i]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_best[warp] = best;
            s_idx[warp] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            double b = s_best[0];
            int ix = s_idx[0];
            for (int w = 1; w < 8; ++w)
                if (s_best[w] > b || (s_best[w] == b && s_idx[w] < ix)) {
                    b = s_best[w];
                    ix = s_idx[w];
                }
            s_piv = (b < 0.0 || ix >= n) ? j : ix;  // all-NaN column: keep the diagonal
        }
        __syncthreads();
        const int p = s_piv;
        if (p != j) {
            for (int c = tid; c < n + nrhs; c += 256) {
                zc* cc = aug_col(L, X, n, c);
                const zc t = cc[j];
                cc[j] = cc[p];
                cc[p] = t;
            }
            __syncthreads();
        }
        const zc piv = col[j];
        if (is_zero(piv)) {
            if (tid == 0) sing_local[sys] = 1;
            for (int i = j + 1 + tid; i < n; i += 256) col[i] = zc{0.0, 0.0};
            __syncthreads();
            continue;
        }
        const zc inv = zinv(piv);
        const bool inv_ok = zfinite(inv);
        for (int i = j + 1 + tid; i < n; i += 256) col[i] = inv_ok ? col[i] * inv : zdiv(col[i], piv);
        __syncthreads();
        const int rows = n - j - 1, cols = kend - j - 1;
        const long long total = (long long)rows * cols;
        for (long long t = tid; t < total; t += 256) {
            const int c = j + 1 + (int)(t / rows), i = j + 1 + (int)(t % rows);
            zc* cc = L + (long long)c * n;
            cc[i] = zfms(col[i], cc[j], cc[i]);
        }
        __syncthreads();
    }
}

// Rows k0+1 .. kend-1 of columns kend .. n+nrhs-1: forward substitution with the panel's unit lower
// triangle, one thread per (system, column).
__global__ void lu_trsm_lower_kernel(int n, int nrhs, int batch, zc* lu, long long lu_stride, zc* x, long long x_stride,
                                     int k0, int kend, const int* __restrict__ skip, int skip_value) {
    const int cols = n + nrhs - kend;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)batch * cols) return;
    const long long sys = idx / cols;
    if (skip && skip[sys] == skip_value) return;
    const int c = kend + (int)(idx - sys * cols);
    zc* L = lu + sys * lu_stride;
    zc* cc = aug_col(L, x + sys * x_stride, n, c);
    for (int r = k0 + 1; r < kend; ++r) {
        zc acc = cc[r];
        for (int q = k0; q < r; ++q) acc = zfms(L[(long long)q * n + r], cc[q], acc);
        cc[r] = acc;
    }
}

// Rows r0 .. r1-1 of the right-hand sides: backward substitution with the diagonal block of U.
__global__ void lu_trsm_upper_kernel(int n, int nrhs, int batch, const zc* lu, long long lu_stride, zc* x,
                                     long long x_stride, int r0, int r1, const int* __restrict__ skip, int skip_value) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)batch * nrhs) return;
    const long long sys = idx / nrhs;
    if (skip && skip[sys] == skip_value) return;
    const int c = (int)(idx - sys * nrhs);
    const zc* U = lu + sys * lu_stride;
    zc* xc = x + sys * x_stride + (long long)c * n;
    for (int r = r1 - 1; r >= r0; --r) {
        zc acc = xc[r];
        for (int q = r + 1; q < r1; ++q) acc = zfms(U[(long long)q * n + r], xc[q], acc);
        xc[r] = zdiv(acc, U[(long long)r * n + r]);
    }
}

// a zero pivot in this call: the reference refuses to solve; the solution is reported as NaN
__global__ void lu_nan_fill_kernel(int n, int nrhs, int batch, zc* x, long long x_stride, const int* __restrict__ sing_local,
                                   int* __restrict__ singular) {
    const long long per = (long long)n * nrhs;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)batch * per) return;
    const long long sys = idx / per;
    if (!sing_local[sys]) return;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    x[sys * x_stride + (idx - sys * per)] = zc{nan, nan};
    if (idx - sys * per == 0) singular[sys] = 1;
}

// Batched complex GEMM: C = s_ab * (A B) + s_c * C0, one warp per 32 x 8 tile of C, lanes along rows.
// A: m x k (lda), B: k x n (ldb), C/C0: m x n (ldc); any stride may be 0 to broadcast one operand
// to the whole batch. s_ab, s_c in {-1, 0, 1}. C may alias C0 (each element is read then written by
// the same lane). The sum over k runs in ascending order, as the reference's column GEMM adds
// (include/stablercwa/matrix.hpp:170-192).
__global__ void __launch_bounds__(128) zgemm_kernel(int m, int n, int k, int batch, const zc* __restrict__ A, int lda,
                                                    long long a_stride, const zc* __restrict__ B, int ldb,
                                                    long long b_stride, const zc* C0, long long c0_stride, zc* C,
                                                    int ldc, long long c_stride, double s_ab, double s_c,
                                                    const int* __restrict__ skip, int skip_value, int tri) {
    const int tiles_m = (m + 31) / 32, tiles_n = (n + 7) / 8;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long per = (long long)tiles_m * tiles_n;
    const long long sys = warp / per;
    if (sys >= batch) return;
    if (skip && skip[sys] == skip_value) return;
    const int t = (int)(warp - sys * per);
    const int tm = t % tiles_m, tn = t / tiles_m;
    const int lane = threadIdx.x & 31;
    const int row = tm * 32 + lane;
    const int c0 = tn * 8;
    const int cols = min(8, n - c0);
    const zc* As = A + sys * a_stride;
    const zc* Bs = B + sys * b_stride;
    double ar[8], ai[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) ar[j] = ai[j] = 0.0;
    // a triangular factor: the k range that can hold nonzeros for this warp's rows / columns
    int p_begin = 0, p_end = k;
    if (tri == TRI_A_LOWER) p_end = min(k, tm * 32 + 32);
    else if (tri == TRI_A_UPPER) p_begin = tm * 32;
    else if (tri == TRI_B_UPPER) p_end = min(k, c0 + 8);
    if (row < m) {
        for (int p = p_begin; p < p_end; ++p) {
            const zc av = As[(long long)p * lda + row];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (j < cols) {
                    const zc bv = Bs[(long long)(c0 + j) * ldb + p];
                    ar[j] = ar[j] + av.re * bv.re - av.im * bv.im;
                    ai[j] = ai[j] + av.re * bv.im + av.im * bv.re;
                }
            }
        }
        const zc* C0s = C0 ? C0 + sys * c0_stride : nullptr;
        zc* Cs = C + sys * c_stride;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j < cols) {
                zc v = zc{s_ab * ar[j], s_ab * ai[j]};
                if (C0s && s_c != 0.0) {
                    const zc cv = C0s[(long long)(c0 + j) * ldc + row];
                    v = zc{s_c * cv.re + v.re, s_c * cv.im + v.im};
                }
                Cs[(long long)(c0 + j) * ldc + row] = v;
            }
        }
    }
}

// C = A B with A complex and B real (the eigenvectors Q Y of the Hermitian solver), zgemm_kernel's tiling:
// one warp per 32 x 8 tile of C, two fused multiply-adds per term.
__global__ void __launch_bounds__(128) zdgemm_kernel(int m, int n, int k, int batch, const zc* __restrict__ A, int lda,
                                                     long long a_stride, const double* __restrict__ B, int ldb,
                                                     long long b_stride, zc* __restrict__ C, int ldc, long long c_stride,
                                                     const int* __restrict__ skip, int skip_value) {
    const int tiles_m = (m + 31) / 32, tiles_n = (n + 7) / 8;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long per = (long long)tiles_m * tiles_n;
    const long long sys = warp / per;
    if (sys >= batch) return;
    if (skip && skip[sys] == skip_value) return;
    const int t = (int)(warp - sys * per);
    const int tm = t % tiles_m, tn = t / tiles_m;
    const int row = tm * 32 + (threadIdx.x & 31);
    const int c0 = tn * 8;
    const int cols = min(8, n - c0);
    if (row >= m) return;
    const zc* As = A + sys * a_stride;
    const double* Bs = B + sys * b_stride;
    double ar[8], ai[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) ar[j] = ai[j] = 0.0;
    for (int p = 0; p < k; ++p) {
        const zc av = As[(long long)p * lda + row];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j < cols) {
                const double bv = Bs[(long long)(c0 + j) * ldb + p];
                ar[j] = fma(av.re, bv, ar[j]);
                ai[j] = fma(av.im, bv, ai[j]);
            }
        }
    }
    zc* Cs = C + sys * c_stride;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (j < cols) Cs[(long long)(c0 + j) * ldc + row] = zc{ar[j], ai[j]};
}

}  // namespace rcwa_gb300
