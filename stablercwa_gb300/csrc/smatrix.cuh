// smatrix.cuh -- batched S-matrix operator algebra shared by the 1-D, conical and 2-D solves.
//
// The reference's operators come in three kinds, Zero / Diag / Dense (include/stablercwa/rcwa1d.hpp:
// 549-629); here each is a B x n vector or a B x n x n matrix holding one operator per sample of a
// chunk, and every operation (product, sum, stack_on, linear solve) is one batched launch. Kinds depend
// only on the structure, so one host-side sequence serves the whole chunk. Vectors that carry several
// right-hand sides (the conical s and p inputs) are B x n x cols, column-major per sample.
#pragma once

#include <complex>
#include <vector>

#include "engine.h"
#include "rcwa1d_kernels.cuh"

namespace rcwa_gb300 {
namespace {

constexpr int kTpb = 256;
inline unsigned nblocks(long long total, int tpb = kTpb) {
    return static_cast<unsigned>((total + tpb - 1) / tpb > 0 ? (total + tpb - 1) / tpb : 1);
}
inline unsigned warp_blocks(long long warps) { return static_cast<unsigned>((warps * 32 + 127) / 128); }

#define LAUNCH(kernel, grid, block, st, ...)                      \
    do {                                                         \
        kernel<<<(grid), (block), 0, (st)>>>(__VA_ARGS__);       \
        ++launch_count();                                        \
        RCWA_CUDA(cudaGetLastError());                           \
    } while (0)

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

enum Kind { KZero = 0, KDiag = 1, KDense = 2 };
struct DOp {
    Kind kind = KZero;
    zc* p = nullptr;
    zc* alt = nullptr;           // per-sample dense alternative of a Diag g (exact q == 0 under dense r)
    const int* alt_flag = nullptr;
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
    int n_solve = 0;
    long long nn() const { return (long long)n * n; }
    zc* dense() { return mem->get<zc>((size_t)B * nn()); }
    zc* vec() { return mem->get<zc>((size_t)B * n); }
};

// linear_solve (include/stablercwa/rcwa1d.hpp:248-281): a zero pivot fails the sample.
zc* solve(Batch& c, zc* a, bool consume_a, int rhs_kind, const zc* rhs, int nrhs = -1) {
    ++c.n_solve;
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


// ---------------------------------------------------------------- Fourier coefficients (host)

using cd = std::complex<double>;
constexpr double kPiD = 3.141592653589793238462643383279502884;

// c_h, h = -hmax..hmax, of a piecewise-constant profile (include/stablercwa/rcwa1d.hpp:366-388)
std::vector<cd> fourier_coefficients(const std::vector<double>& edges, const std::vector<cd>& values, double period,
                                     int hmax) {
    std::vector<cd> c(2 * hmax + 1);
    const size_t segments = values.size();
    std::vector<cd> phase(edges.size());
    for (int h = -hmax; h <= hmax; ++h) {
        cd sum{};
        if (h == 0) {
            for (size_t j = 0; j < segments; ++j) sum += values[j] * (edges[j + 1] - edges[j]) / period;
        } else {
            for (size_t k = 0; k < edges.size(); ++k) {
                const double arg = -2.0 * kPiD * h * edges[k] / period;
                phase[k] = cd{std::cos(arg), std::sin(arg)};
            }
            const double w = -2.0 * kPiD * h;
            for (size_t j = 0; j < segments; ++j) {
                const cd t = values[j] * (phase[j + 1] - phase[j]);
                sum += cd{t.imag() / w, -t.real() / w};
            }
        }
        c[h + hmax] = sum;
    }
    return c;
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
