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

// Batched complex GEMM: C = s_ab * (A B) + s_c * C0, one warp per 32 x 8 tile of C, lanes along rows.
// A: m x k (lda), B: k x n (ldb), C/C0: m x n (ldc); any stride may be 0 to broadcast one operand
// to the whole batch. s_ab, s_c in {-1, 0, 1}. C may alias C0 (each element is read then written by
// the same lane). The sum over k runs in ascending order, as the reference's column GEMM adds
// (include/stablercwa/matrix.hpp:170-192).
__global__ void __launch_bounds__(128) zgemm_kernel(int m, int n, int k, int batch, const zc* __restrict__ A, int lda,
                                                    long long a_stride, const zc* __restrict__ B, int ldb,
                                                    long long b_stride, const zc* C0, long long c0_stride, zc* C,
                                                    int ldc, long long c_stride, double s_ab, double s_c,
                                                    const int* __restrict__ skip, int skip_value) {
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
    if (row < m) {
        for (int p = 0; p < k; ++p) {
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

}  // namespace rcwa_gb300
