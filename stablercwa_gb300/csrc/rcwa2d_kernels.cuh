// rcwa2d_kernels.cuh -- device kernels of the batched 2-D (crossed-grating) solve.
//
// Layouts (every array holds the B samples of a chunk back to back):
//   - harmonics i = (m+M1)(2M2+1) + (n+M2), N of them; mode vectors have 2N entries (Ex block, Ey block);
//   - dense operators are 2N x 2N column-major;
//   - a 2x2 block-diagonal operator ("BD", four N-vectors a11, a12, a21, a22: the reference's
//     BlockDiag2, include/stablercwa/rcwa2d.hpp:128-285) is stored as 4N entries [a11 | a12 | a21 | a22].
#pragma once

#include "rcwa1d_kernels.cuh"

namespace rcwa_gb300 {
namespace {

struct Bd {
    zc a11, a12, a21, a22;
};

__device__ __forceinline__ Bd bd_load(const zc* p, int N, int i) { return {p[i], p[N + i], p[2 * N + i], p[3 * N + i]}; }
__device__ __forceinline__ void bd_store(zc* p, int N, int i, const Bd& a) {
    p[i] = a.a11;
    p[N + i] = a.a12;
    p[2 * N + i] = a.a21;
    p[3 * N + i] = a.a22;
}
__device__ __forceinline__ Bd bd_zero() { return {zc{0, 0}, zc{0, 0}, zc{0, 0}, zc{0, 0}}; }
__device__ __forceinline__ Bd bd_eye() { return {zc{1, 0}, zc{0, 0}, zc{0, 0}, zc{1, 0}}; }
// b2_mul, b2_inv, b2_add, b2_sub, b2_scale, b2_neg, b2_eye_minus (rcwa2d.hpp:140-214)
__device__ __forceinline__ Bd bd_mul(const Bd& A, const Bd& B) {
    return {A.a11 * B.a11 + A.a12 * B.a21, A.a11 * B.a12 + A.a12 * B.a22, A.a21 * B.a11 + A.a22 * B.a21,
            A.a21 * B.a12 + A.a22 * B.a22};
}
__device__ __forceinline__ Bd bd_inv(const Bd& A) {
    const zc det = A.a11 * A.a22 - A.a12 * A.a21;
    return {zdiv(A.a22, det), zdiv(-A.a12, det), zdiv(-A.a21, det), zdiv(A.a11, det)};
}
__device__ __forceinline__ Bd bd_add(const Bd& A, const Bd& B) { return {A.a11 + B.a11, A.a12 + B.a12, A.a21 + B.a21, A.a22 + B.a22}; }
__device__ __forceinline__ Bd bd_sub(const Bd& A, const Bd& B) { return {A.a11 - B.a11, A.a12 - B.a12, A.a21 - B.a21, A.a22 - B.a22}; }
__device__ __forceinline__ Bd bd_scale(const Bd& A, double s) { return {s * A.a11, s * A.a12, s * A.a21, s * A.a22}; }
__device__ __forceinline__ Bd bd_neg(const Bd& A) { return {-A.a11, -A.a12, -A.a21, -A.a22}; }
__device__ __forceinline__ Bd bd_eye_minus(const Bd& A) {
    Bd C = bd_neg(A);
    C.a11 = C.a11 + zc{1.0, 0.0};
    C.a22 = C.a22 + zc{1.0, 0.0};
    return C;
}
__device__ __forceinline__ Bd bd_eye_plus(const Bd& A) { return bd_add(bd_eye(), A); }

// The four blocks of the interface S block between two homogeneous regions (interface_bd,
// rcwa2d.hpp:578-592): Mm = I, Nn = Vb_low^-1 Vb_up.
struct BdIface {
    Bd tdd, rdu, rud, tuu;
};
__device__ __forceinline__ BdIface bd_interface(const Bd& up, const Bd& low) {
    const Bd nn = bd_mul(bd_inv(low), up);
    const Bd mm = bd_eye();
    const Bd tp = bd_scale(bd_add(mm, nn), 0.5), tm = bd_scale(bd_sub(mm, nn), 0.5);
    const Bd tpi = bd_inv(tp);
    BdIface s;
    s.tdd = bd_sub(tp, bd_mul(bd_mul(tm, tpi), tm));
    s.rdu = bd_mul(tm, tpi);
    s.rud = bd_neg(bd_mul(tpi, tm));
    s.tuu = tpi;
    return s;
}

// ---------------------------------------------------------------- Fourier operators

// Eps(r, c) = sum_k wy[k][dn] ce[k][dm] (layer_operators' Eps, rcwa2d_operators.hpp:355-366 with
// assemble_xfirst :183-200): the Toeplitz block of strip k is ce[k][i - j + 2M1].
__global__ void op_eps_kernel(int M1, int M2, int K, const zc* __restrict__ wy, const zc* __restrict__ ce,
                              zc* __restrict__ out) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)N * N) return;
    const int col = (int)(idx / N), row = (int)(idx - (long long)col * N);
    const int dm = row / n2 - col / n2 + 2 * M1, dn = row % n2 - col % n2 + 2 * M2;
    zc acc{0.0, 0.0};
    for (int k = 0; k < K; ++k) acc = acc + wy[(long long)k * (4 * M2 + 1) + dn] * ce[(long long)k * (4 * M1 + 1) + dm];
    out[idx] = acc;
}

// Cx(r, c) = sum_k wy[k][dn] invx_k(m, m') (rcwa2d_operators.hpp:374-384): x-first blocks.
__global__ void op_cx_kernel(int M1, int M2, int K, const zc* __restrict__ wy, const zc* __restrict__ invx,
                             zc* __restrict__ out) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)N * N) return;
    const int col = (int)(idx / N), row = (int)(idx - (long long)col * N);
    const int a = row / n2, ap = col / n2, dn = row % n2 - col % n2 + 2 * M2;
    zc acc{0.0, 0.0};
    for (int k = 0; k < K; ++k)
        acc = acc + wy[(long long)k * (4 * M2 + 1) + dn] * invx[(long long)k * n1 * n1 + (long long)ap * n1 + a];
    out[idx] = acc;
}

// Cy(r, c) = sum_j wx[j][dm] invy_j(n, n') (rcwa2d_operators.hpp:387-404 with assemble_yfirst
// :205-222): y-first blocks over the merged x cuts.
__global__ void op_cy_kernel(int M1, int M2, int Kx, const zc* __restrict__ wx, const zc* __restrict__ invy,
                             zc* __restrict__ out) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)N * N) return;
    const int col = (int)(idx / N), row = (int)(idx - (long long)col * N);
    const int b = row % n2, bp = col % n2, dm = row / n2 - col / n2 + 2 * M1;
    zc acc{0.0, 0.0};
    for (int j = 0; j < Kx; ++j)
        acc = acc + wx[(long long)j * (4 * M1 + 1) + dm] * invy[(long long)j * n2 * n2 + (long long)bp * n2 + b];
    out[idx] = acc;
}

// count Toeplitz matrices of order 2M+1 from their 4M+1 coefficients (toeplitz_1d, :110-118)
__global__ void toeplitz_batch_kernel(int count, int M, const zc* __restrict__ c, zc* __restrict__ out) {
    const int n = 2 * M + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)count * n * n) return;
    const long long k = idx / ((long long)n * n);
    const int r = (int)(idx - k * n * n);
    const int j = r / n, i = r - j * n;
    out[idx] = c[k * (4 * M + 1) + i - j + 2 * M];
}

__global__ void any_nonfinite_kernel(long long total, const zc* __restrict__ a, int* __restrict__ flag) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total && !zfinite(a[idx])) atomicOr(flag, 1);
}
__global__ void any_set_kernel(int count, const int* __restrict__ f, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count && f[i]) atomicOr(flag, 1);
}

// ---------------------------------------------------------------- structured modes (rcwa2d.hpp:412-540)

// pc1 = [Kx Ei Ky; Ky Ei Ky - I], pc2 = [I - Kx Ei Kx; -Ky Ei Kx] (2N x N each), Ei shared by the batch
__global__ void pc_kernel(int B, int N, const zc* __restrict__ Ei, const double* __restrict__ Kx,
                          const double* __restrict__ Ky, zc* __restrict__ pc1, zc* __restrict__ pc2) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long NN = (long long)N * N;
    if (idx >= (long long)B * NN) return;
    const long long b = idx / NN;
    const int r = (int)(idx - b * NN);
    const int j = r / N, i = r - j * N;
    const double* kx = Kx + b * N;
    const double* ky = Ky + b * N;
    const zc e = Ei[(long long)j * N + i];
    const zc kxe = e * kx[i], kye = e * ky[i];
    const double delta = i == j ? 1.0 : 0.0;
    zc* c1 = pc1 + b * 2 * NN + (long long)j * 2 * N;
    zc* c2 = pc2 + b * 2 * NN + (long long)j * 2 * N;
    c1[i] = kxe * ky[j];
    c2[i] = zc{delta, 0.0} - kxe * kx[j];
    c1[N + i] = kye * ky[j] - zc{delta, 0.0};
    c2[N + i] = -(kye * kx[j]);
}

// q12 = Cy - Kx^2, q21 = Ky^2 - Cx (N x N per sample)
__global__ void q_blocks_kernel(int B, int N, const zc* __restrict__ cx, const zc* __restrict__ cy,
                                const double* __restrict__ Kx, const double* __restrict__ Ky, zc* __restrict__ q12,
                                zc* __restrict__ q21) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long NN = (long long)N * N;
    if (idx >= (long long)B * NN) return;
    const long long b = idx / NN;
    const int r = (int)(idx - b * NN);
    const int j = r / N, i = r - j * N;
    zc a = cy[r], c = -cx[r];
    if (i == j) {
        const double kx = Kx[b * N + i], ky = Ky[b * N + i];
        a.re = a.re - kx * kx;
        c.re = c.re + ky * ky;
    }
    q12[idx] = a;
    q21[idx] = c;
}

// H = [t1 + pc1 Kx Ky | t2 - pc2 Ky Kx] with t1 = pc2 q21, t2 = pc1 q12 (rcwa2d.hpp:449-467)
__global__ void h_assemble_kernel(int B, int N, const zc* __restrict__ t1, const zc* __restrict__ t2,
                                  const zc* __restrict__ pc1, const zc* __restrict__ pc2, const double* __restrict__ Kx,
                                  const double* __restrict__ Ky, zc* __restrict__ H) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long half = (long long)n * N;
    if (idx >= (long long)B * half) return;
    const long long b = idx / half;
    const long long r = idx - b * half;  // element (i, j) of the 2N x N blocks
    const int j = (int)(r / n);
    const double kx = Kx[b * N + j], ky = Ky[b * N + j];
    const double d1 = kx * ky, d2 = -(ky * kx);
    zc* Hs = H + b * (long long)n * n;
    Hs[r] = t1[idx] + pc1[idx] * d1;
    Hs[half + r] = t2[idx] + pc2[idx] * d2;
}

__global__ void q_from_values_kernel(long long total, const zc* __restrict__ w, zc* __restrict__ q) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) q[idx] = branch(zsqrt(w[idx]));
}

// V = (Q W)/q: [top + Wt Kx Ky; bot - Wb Ky Kx] / q_j, top = q12 Wb, bot = q21 Wt (rcwa2d.hpp:517-533)
__global__ void v_assemble_kernel(int B, int N, const zc* __restrict__ top, const zc* __restrict__ bot,
                                  const zc* __restrict__ W, const zc* __restrict__ q, const double* __restrict__ Kx,
                                  const double* __restrict__ Ky, zc* __restrict__ V) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * n;  // N x 2N
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int j = (int)(r / N), i = (int)(r - (long long)j * N);
    const double kx = Kx[b * N + i], ky = Ky[b * N + i];
    const zc* Ws = W + b * (long long)n * n + (long long)j * n;
    const zc qj = q[b * n + j];
    const zc up = top[idx] + Ws[i] * (kx * ky);
    const zc dn = bot[idx] + Ws[N + i] * (-(ky * kx));
    zc* Vs = V + b * (long long)n * n + (long long)j * n;
    Vs[i] = zdiv(up, qj);
    Vs[N + i] = zdiv(dn, qj);
}

// Homogeneous region: q1 = branch(-i kz), Vb = [[Kx Ky, n^2 - Kx^2], [Ky^2 - n^2, -Ky Kx]] / q1
// (homogeneous_modes, rcwa2d.hpp:386-404)
__global__ void homog_modes_kernel(int B, int N, const zc* __restrict__ kz, zc n2, const double* __restrict__ Kx,
                                   const double* __restrict__ Ky, zc* __restrict__ q, zc* __restrict__ vb) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const zc k = kz[idx];
    const zc q1 = branch(zc{k.im, -k.re});
    q[b * 2 * N + i] = q1;
    q[b * 2 * N + N + i] = q1;
    const double kx = Kx[idx], ky = Ky[idx];
    Bd v;
    v.a11 = zdiv(zc{kx * ky, 0.0}, q1);
    v.a12 = zdiv(zc{n2.re - kx * kx, n2.im}, q1);
    v.a21 = zdiv(zc{ky * ky - n2.re, -n2.im}, q1);
    v.a22 = zdiv(zc{-(ky * kx), 0.0}, q1);
    bd_store(vb + b * 4 * N, N, i, v);
}

// ---------------------------------------------------------------- block-diagonal S-matrix steps

// Interface between two homogeneous regions over a block-diagonal (or zero) r: first branch of
// stack_on (rcwa2d.hpp:689-703). rr == nullptr is the zero r.
__global__ void iface_bd_kernel(int B, int N, const zc* __restrict__ up, const zc* __restrict__ low,
                                const zc* __restrict__ rr, zc* __restrict__ r_out, zc* __restrict__ gt) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const BdIface s = bd_interface(bd_load(up + b * 4 * N, N, i), bd_load(low + b * 4 * N, N, i));
    const Bd r = rr ? bd_load(rr + b * 4 * N, N, i) : bd_zero();
    const Bd g = bd_mul(bd_inv(bd_eye_minus(bd_mul(s.rdu, r))), s.tdd);
    const Bd out = rr ? bd_add(s.rud, bd_mul(bd_mul(s.tuu, r), g)) : s.rud;
    bd_store(r_out + b * 4 * N, N, i, out);
    bd_store(gt + b * 4 * N, N, i, g);
}

// Propagation X = exp(-k0 q d) (propagation_block, rcwa2d.hpp:612-627): gt = diag(X) as a BD and,
// over a block-diagonal (or zero) r, r' = X r X (first branch of stack_on with Rdu = 0).
__global__ void prop_bd_kernel(int B, int N, const zc* __restrict__ q, double d, const double* __restrict__ k0,
                               const zc* __restrict__ rr, zc* __restrict__ r_out, zc* __restrict__ gt,
                               zc* __restrict__ xvec) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const double k = k0[b];
    const zc q1 = q[b * 2 * N + i], q2 = q[b * 2 * N + N + i];
    const zc x1 = zexp(zc{-k * q1.re * d, -k * q1.im * d});
    const zc x2 = zexp(zc{-k * q2.re * d, -k * q2.im * d});
    const Bd t = {x1, zc{0, 0}, zc{0, 0}, x2};
    bd_store(gt + b * 4 * N, N, i, t);
    if (xvec) {
        xvec[b * 2 * N + i] = x1;
        xvec[b * 2 * N + N + i] = x2;
    }
    if (r_out) {
        const Bd out = rr ? bd_add(bd_zero(), bd_mul(bd_mul(t, bd_load(rr + b * 4 * N, N, i)), t)) : bd_zero();
        bd_store(r_out + b * 4 * N, N, i, out);
    }
}

// r' = diag(X) r diag(X) over a dense r (second branch of stack_on with Rdu = 0, rcwa2d.hpp:707-713)
__global__ void prop_dense_kernel(int B, int n, const zc* __restrict__ x, const zc* __restrict__ r, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nn = (long long)n * n;
    if (idx >= (long long)B * nn) return;
    const long long b = idx / nn;
    const int rr = (int)(idx - b * nn);
    const int j = rr / n, i = rr - j * n;
    out[idx] = (x[b * n + i] * r[idx]) * x[b * n + j];
}

// Blocks of direct_bd_over_dense (rcwa2d.hpp:791-809): nn = Vb_low^-1 Vb_up, nn + I, nn - I and
// Tm = -(nn - I)/2.
__global__ void bd_over_dense_prep_kernel(int B, int N, const zc* __restrict__ up, const zc* __restrict__ low,
                                          zc* __restrict__ nn, zc* __restrict__ np1, zc* __restrict__ nm1,
                                          zc* __restrict__ tm) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const Bd v = bd_mul(bd_inv(bd_load(low + b * 4 * N, N, i)), bd_load(up + b * 4 * N, N, i));
    const Bd p = bd_add(v, bd_eye()), m = bd_sub(v, bd_eye());
    bd_store(nn + b * 4 * N, N, i, v);
    bd_store(np1 + b * 4 * N, N, i, p);
    bd_store(nm1 + b * 4 * N, N, i, m);
    bd_store(tm + b * 4 * N, N, i, bd_scale(m, -0.5));
}

// out = M bdense(R) + bdense(add) (b2_rmul then b2_add_to, rcwa2d.hpp:237-270); mode selects R:
// 0 R as given, 1 I + R, 2 I - R. add may be null.
__global__ void rmul_bd_kernel(int B, int N, const zc* __restrict__ M, const zc* __restrict__ R, int mode,
                               const zc* __restrict__ add, zc* __restrict__ out) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * N;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int j = (int)(r / n), i = (int)(r - (long long)j * n);
    Bd bj = bd_load(R + b * 4 * N, N, j);
    if (mode == 1) bj = bd_eye_plus(bj);
    else if (mode == 2) bj = bd_eye_minus(bj);
    const zc* Ms = M + b * (long long)n * n;
    const zc x1 = Ms[(long long)j * n + i], x2 = Ms[(long long)(N + j) * n + i];
    zc y1 = x1 * bj.a11 + x2 * bj.a21;
    zc y2 = x1 * bj.a12 + x2 * bj.a22;
    if (add) {
        const Bd a = bd_load(add + b * 4 * N, N, j);
        if (i == j) {
            y1 = y1 + a.a11;
            y2 = y2 + a.a12;
        } else if (i == N + j) {
            y1 = y1 + a.a21;
            y2 = y2 + a.a22;
        }
    }
    zc* Os = out + b * (long long)n * n;
    Os[(long long)j * n + i] = y1;
    Os[(long long)(N + j) * n + i] = y2;
}

// out = bdense(L) M (b2_apply_rows, rcwa2d.hpp:223-235), mode 0 L, 1 I + L, 2 I - L, 3 L^-1;
// M has cols columns of 2N rows. add (optional, same shape as out) is added afterwards.
__global__ void apply_rows_bd_kernel(int B, int N, int cols, const zc* __restrict__ L, int mode,
                                     const zc* __restrict__ M, const zc* __restrict__ add, zc* __restrict__ out) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cols;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int j = (int)(r / N), i = (int)(r - (long long)j * N);
    Bd l = bd_load(L + b * 4 * N, N, i);
    if (mode == 1) l = bd_eye_plus(l);
    else if (mode == 2) l = bd_eye_minus(l);
    else if (mode == 3) l = bd_inv(l);
    const long long base = b * (long long)n * cols + (long long)j * n;
    const zc x1 = M[base + i], x2 = M[base + N + i];
    zc y1 = l.a11 * x1 + l.a12 * x2;
    zc y2 = l.a21 * x1 + l.a22 * x2;
    if (add) {
        y1 = y1 + add[base + i];
        y2 = y2 + add[base + N + i];
    }
    out[base + i] = y1;
    out[base + N + i] = y2;
}

// dense 2N x 2N form of a BD into a zeroed matrix (b2_dense, rcwa2d.hpp:206-217)
__global__ void bd_to_dense_kernel(int B, int N, const zc* __restrict__ bd, zc* __restrict__ out) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const Bd a = bd_load(bd + b * 4 * N, N, i);
    zc* o = out + b * (long long)n * n;
    o[(long long)i * n + i] = a.a11;
    o[(long long)(N + i) * n + i] = a.a12;
    o[(long long)i * n + N + i] = a.a21;
    o[(long long)(N + i) * n + N + i] = a.a22;
}

// p, q -> p + q, p - q in place (A+ and A- of direct_dense, rcwa2d.hpp:774-777)
__global__ void sum_diff_kernel(long long total, zc* __restrict__ p, zc* __restrict__ q) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const zc a = p[idx], c = q[idx];
    p[idx] = a + c;
    q[idx] = a - c;
}

// mm = (mm - nn) * 0.5 (Tm of direct_dense, rcwa2d.hpp:782-783)
__global__ void half_diff_kernel(long long total, zc* __restrict__ mm, const zc* __restrict__ nn) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) mm[idx] = (mm[idx] - nn[idx]) * 0.5;
}

// The interface blocks of two homogeneous regions, stored as BDs (top block, rcwa2d.hpp:829-842)
__global__ void iface_blocks_kernel(int B, int N, const zc* __restrict__ up, const zc* __restrict__ low,
                                    zc* __restrict__ tdd, zc* __restrict__ rdu, zc* __restrict__ rud,
                                    zc* __restrict__ tuu) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const BdIface s = bd_interface(bd_load(up + b * 4 * N, N, i), bd_load(low + b * 4 * N, N, i));
    bd_store(tdd + b * 4 * N, N, i, s.tdd);
    bd_store(rdu + b * 4 * N, N, i, s.rdu);
    bd_store(rud + b * 4 * N, N, i, s.rud);
    bd_store(tuu + b * 4 * N, N, i, s.tuu);
}

// y = bd x (b2_apply), or with mode 4: y = (I - rdu rr)^-1 tdd x (the top block over a
// block-diagonal r, rcwa2d.hpp:833-836), for x of 2N entries per sample
__global__ void bd_apply_vec_kernel(int B, int N, const zc* __restrict__ a, const zc* __restrict__ x, zc* __restrict__ y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const Bd l = bd_load(a + b * 4 * N, N, i);
    const zc x1 = x[b * 2 * N + i], x2 = x[b * 2 * N + N + i];
    y[b * 2 * N + i] = l.a11 * x1 + l.a12 * x2;
    y[b * 2 * N + N + i] = l.a21 * x1 + l.a22 * x2;
}

// Top block with both regions homogeneous over a zero or block-diagonal r (rcwa2d.hpp:829-842):
// down1 = ((I - Rdu r)^-1 Tdd) inc, R = Rud inc + Tuu (r down1).
__global__ void top_bd_kernel(int B, int N, const zc* __restrict__ up, const zc* __restrict__ low,
                              const zc* __restrict__ rr, const zc* __restrict__ inc, zc* __restrict__ down,
                              zc* __restrict__ R) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const BdIface s = bd_interface(bd_load(up + b * 4 * N, N, i), bd_load(low + b * 4 * N, N, i));
    const Bd r = rr ? bd_load(rr + b * 4 * N, N, i) : bd_zero();
    const Bd g = bd_inv(bd_eye_minus(bd_mul(s.rdu, r)));
    const Bd gt = bd_mul(g, s.tdd);
    const zc e1 = inc[b * 2 * N + i], e2 = inc[b * 2 * N + N + i];
    const zc d1 = gt.a11 * e1 + gt.a12 * e2, d2 = gt.a21 * e1 + gt.a22 * e2;
    down[b * 2 * N + i] = d1;
    down[b * 2 * N + N + i] = d2;
    zc r1 = s.rud.a11 * e1 + s.rud.a12 * e2, r2 = s.rud.a21 * e1 + s.rud.a22 * e2;
    const zc v1 = rr ? r.a11 * d1 + r.a12 * d2 : zc{0.0, 0.0};
    const zc v2 = rr ? r.a21 * d1 + r.a22 * d2 : zc{0.0, 0.0};
    r1 = r1 + (s.tuu.a11 * v1 + s.tuu.a12 * v2);
    r2 = r2 + (s.tuu.a21 * v1 + s.tuu.a22 * v2);
    R[b * 2 * N + i] = r1;
    R[b * 2 * N + N + i] = r2;
}

// R = Rud inc + Tuu back (top block over a dense r, rcwa2d.hpp:839-841)
__global__ void top_bd_finish_kernel(int B, int N, const zc* __restrict__ rud, const zc* __restrict__ tuu,
                                     const zc* __restrict__ inc, const zc* __restrict__ back, zc* __restrict__ R) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const Bd a = bd_load(rud + b * 4 * N, N, i), t = bd_load(tuu + b * 4 * N, N, i);
    const zc e1 = inc[b * 2 * N + i], e2 = inc[b * 2 * N + N + i];
    const zc v1 = back[b * 2 * N + i], v2 = back[b * 2 * N + N + i];
    R[b * 2 * N + i] = (a.a11 * e1 + a.a12 * e2) + (t.a11 * v1 + t.a12 * v2);
    R[b * 2 * N + N + i] = (a.a21 * e1 + a.a22 * e2) + (t.a21 * v1 + t.a22 * v2);
}

// y = tm u + nn x for block-diagonal tm, nn (step_apply of a block-diagonal interface, rcwa2d.hpp:663-668)
__global__ void iface_bd_step_kernel(int B, int N, const zc* __restrict__ tm, const zc* __restrict__ nn,
                                     const zc* __restrict__ u, const zc* __restrict__ x, zc* __restrict__ y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const Bd t = bd_load(tm + b * 4 * N, N, i), m = bd_load(nn + b * 4 * N, N, i);
    const zc u1 = u[b * 2 * N + i], u2 = u[b * 2 * N + N + i];
    const zc x1 = x[b * 2 * N + i], x2 = x[b * 2 * N + N + i];
    y[b * 2 * N + i] = (t.a11 * u1 + t.a12 * u2) + (m.a11 * x1 + m.a12 * x2);
    y[b * 2 * N + N + i] = (t.a21 * u1 + t.a22 * u2) + (m.a21 * x1 + m.a22 * x2);
}

// incident vector: Ex at i0, Ey at N + i0 (rcwa2d.hpp:1163-1167)
__global__ void incident_kernel(int B, int N, int i0, const zc* __restrict__ e, zc* __restrict__ inc) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * 2 * N) return;
    const long long b = idx / (2 * N);
    const int i = (int)(idx - b * 2 * N);
    inc[idx] = i == i0 ? e[2 * b] : (i == N + i0 ? e[2 * b + 1] : zc{0.0, 0.0});
}
__global__ void scale_vec_kernel(long long total, const zc* __restrict__ x, double s, zc* __restrict__ y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) y[idx] = x[idx] * s;
}

// Efficiencies and s/p amplitudes of one side (the efficiency and spol lambdas of solve_impl,
// rcwa2d.hpp:1236-1266). sign = -1 reflection, +1 transmission.
__device__ __forceinline__ void side_outputs(zc ex, zc ey, double kx, double ky, zc kz, zc n_med, double sign,
                                            double nI_cos, double sin_ph, double cos_ph, zc& ez, double& de, zc& s_,
                                            zc& p_) {
    ez = zc{0.0, 0.0};
    de = 0.0;
    if (kz.re > 1e-12) {
        const zc t = kx * ex + ky * ey;
        ez = zdiv(zc{-sign * t.re, -sign * t.im}, kz);
        const double e2 = norm2(ex) + norm2(ey) + norm2(ez);
        de = kz.re * e2 / nI_cos;
    }
    const double kt = hypot(kx, ky);
    const zc cth = zabs(kz) > 1e-12 ? zdiv(kz, n_med) : zc{1.0, 0.0};
    if (kt > 1e-12) {
        const zc a = -ky * ex + kx * ey;
        s_ = zdivr(a, kt);
        const zc c = kx * ex + ky * ey;
        p_ = zdiv(zc{sign * c.re, sign * c.im}, cth * kt);
    } else {
        s_ = -sin_ph * ex + cos_ph * ey;
        const zc c = cos_ph * ex + sin_ph * ey;
        p_ = zdiv(zc{sign * c.re, sign * c.im}, cth);
    }
}

struct Outputs2D {
    zc *Ex_r, *Ey_r, *Ez_r, *Ex_t, *Ey_t, *Ez_t, *Rs, *Rp, *Ts, *Tp;
    double *DEr, *DEt;
};

__global__ void finalize2d_kernel(int B, int N, const zc* __restrict__ R, const zc* __restrict__ T,
                                  const double* __restrict__ Kx, const double* __restrict__ Ky,
                                  const zc* __restrict__ kzI, const zc* __restrict__ kzII, double nI, zc nII,
                                  const double* __restrict__ nI_cos, const double* __restrict__ sin_ph,
                                  const double* __restrict__ cos_ph, Outputs2D o, int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const long long b = idx / N;
    const int i = (int)(idx - b * N);
    const zc exr = R[b * 2 * N + i], eyr = R[b * 2 * N + N + i];
    const zc ext = T[b * 2 * N + i], eyt = T[b * 2 * N + N + i];
    bool bad = !zfinite(exr) || !zfinite(eyr) || !zfinite(ext) || !zfinite(eyt);
    zc ezr, ezt, rs, rp, ts, tp;
    double der, det;
    side_outputs(exr, eyr, Kx[idx], Ky[idx], kzI[idx], zc{nI, 0.0}, -1.0, nI_cos[b], sin_ph[b], cos_ph[b], ezr, der, rs, rp);
    side_outputs(ext, eyt, Kx[idx], Ky[idx], kzII[idx], nII, 1.0, nI_cos[b], sin_ph[b], cos_ph[b], ezt, det, ts, tp);
    bad = bad || !isfinite(der) || !isfinite(det) || !zfinite(rs) || !zfinite(rp) || !zfinite(ts) || !zfinite(tp);
    o.Ex_r[idx] = exr;
    o.Ey_r[idx] = eyr;
    o.Ez_r[idx] = ezr;
    o.Ex_t[idx] = ext;
    o.Ey_t[idx] = eyt;
    o.Ez_t[idx] = ezt;
    o.Rs[idx] = rs;
    o.Rp[idx] = rp;
    o.Ts[idx] = ts;
    o.Tp[idx] = tp;
    o.DEr[idx] = der;
    o.DEt[idx] = det;
    if (bad) fail[b] = 1;
}

__global__ void nan_fill2d_kernel(int B, int N, Outputs2D o, const int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    if (!fail[idx / N]) return;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const zc cn{nan, nan};
    o.Ex_r[idx] = cn; o.Ey_r[idx] = cn; o.Ez_r[idx] = cn;
    o.Ex_t[idx] = cn; o.Ey_t[idx] = cn; o.Ez_t[idx] = cn;
    o.Rs[idx] = cn; o.Rp[idx] = cn; o.Ts[idx] = cn; o.Tp[idx] = cn;
    o.DEr[idx] = nan;
    o.DEt[idx] = nan;
}

// first nonzero eig info over the layers, in layer order (rcwa2d.hpp:1154-1158)
__global__ void eig_info_layers_kernel(int B, int P, const int* __restrict__ info, int* __restrict__ eig_info,
                                       int* __restrict__ fail) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int first = 0;
    for (int p = 0; p < P; ++p)
        if (info[(long long)p * B + b] != 0 && first == 0) first = info[(long long)p * B + b];
    eig_info[b] = first;
    if (first != 0) fail[b] = 1;
}

// ---------------------------------------------------------------- near fields (rcwa2d_fields.hpp:169-290)

// S = p + m and D = m - p at the group's depths in layer j: p = a+ exp(-k0 q t), m = a- exp(-k0 q (d - t)),
// t the depth below the layer's top clamped to [0, d] (layer_chunk_fields, rcwa2d_fields.hpp:209-223).
// Per sample 2N x cnt column-major.
__global__ void fields2d_layer_kernel(int B, int n, int cnt, const double* __restrict__ zl, double d,
                                      const double* __restrict__ k0, const zc* __restrict__ ap, const zc* __restrict__ am,
                                      const zc* __restrict__ q, zc* __restrict__ S, zc* __restrict__ D) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / n), j = (int)(r - (long long)col * n);
    const double from_top = fmax(0.0, fmin(d, zl[col])), from_bottom = d - from_top;
    const double k = k0[b];
    const zc a = ap[b * n + j], bm = am[b * n + j], qj = q[b * n + j];
    const zc p = is_zero(a) ? zc{0.0, 0.0} : a * zexp((-k * from_top) * qj);
    const zc m = is_zero(bm) ? zc{0.0, 0.0} : bm * zexp((-k * from_bottom) * qj);
    S[idx] = p + m;
    D[idx] = m - p;
}

// Y = BD X for every column of X (2N x cnt per sample; b2_apply_rows, rcwa2d.hpp:253-265)
__global__ void bd_rows_kernel(int B, int N, int cnt, const zc* __restrict__ bd, const zc* __restrict__ X,
                               zc* __restrict__ Y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / N), i = (int)(r - (long long)col * N);
    const Bd l = bd_load(bd + b * 4 * N, N, i);
    const long long base = (b * cnt + col) * 2 * N;
    const zc x1 = X[base + i], x2 = X[base + N + i];
    Y[base + i] = l.a11 * x1 + l.a12 * x2;
    Y[base + N + i] = l.a21 * x1 + l.a22 * x2;
}

// F = [Ex; Ey] and G = [hx; hy] in region I (z < 0: reflected orders exp(+k0 q z), the incident (0,0)
// order exp(-k0 q z)) or region II (transmitted exp(-k0 q (z - z_bot))), G = V v with V the region's
// block-diagonal modes (region_I/II_chunk_fields, rcwa2d_fields.hpp:226-279). Thread per (sample, depth, i < N).
__global__ void fields2d_region_kernel(int B, int N, int i0, int cnt, const double* __restrict__ zs, int region,
                                       double z_bot, const double* __restrict__ k0, const zc* __restrict__ q,
                                       const zc* __restrict__ vb, const zc* __restrict__ inc, const zc* __restrict__ amp,
                                       zc* __restrict__ F, zc* __restrict__ G) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / N), i = (int)(r - (long long)col * N);
    const int n = 2 * N;
    const double z = zs[col], k = k0[b];
    zc f[2], v[2];
    for (int h = 0; h < 2; ++h) {
        const int j = h * N + i;
        const zc a = amp[b * n + j], qj = q[b * n + j];
        if (region == -1) {
            f[h] = is_zero(a) ? zc{0.0, 0.0} : a * zexp((k * z) * qj);
            v[h] = f[h];
            if (i == i0) {
                const zc in = inc[b * n + j];
                const zc ix = is_zero(in) ? zc{0.0, 0.0} : in * zexp((-k * z) * qj);
                f[h] = f[h] + ix;
                v[h] = v[h] - ix;
            }
        } else {
            f[h] = is_zero(a) ? zc{0.0, 0.0} : a * zexp((-k * (z - z_bot)) * qj);
            v[h] = -f[h];
        }
    }
    const Bd l = bd_load(vb + b * 4 * N, N, i);
    const long long base = (b * cnt + col) * n;
    F[base + i] = f[0];
    F[base + N + i] = f[1];
    G[base + i] = l.a11 * v[0] + l.a12 * v[1];
    G[base + N + i] = l.a21 * v[0] + l.a22 * v[1];
}

// Ex, Ey, Hx = -i hx, Hy = -i hy, Hz = -i hz with hz = i (Ky Ex - Kx Ey) into out[b][c][j][iz]; the
// right-hand side Ky hx - Kx hy of Ez into t (per sample N x cnt) (emit_field_chunk, rcwa2d_fields.hpp:169-205)
__global__ void fields2d_out_kernel(int B, int N, int cnt, int nz, const int* __restrict__ cols, const double* __restrict__ Kx,
                                    const double* __restrict__ Ky, const zc* __restrict__ F, const zc* __restrict__ G,
                                    zc* __restrict__ t, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / N), j = (int)(r - (long long)col * N);
    const long long base = (b * cnt + col) * 2 * N;
    const zc ex = F[base + j], ey = F[base + N + j], hx = G[base + j], hy = G[base + N + j];
    const double kx = Kx[b * N + j], ky = Ky[b * N + j];
    const zc w = ky * ex - kx * ey;
    const zc hz{-w.im, w.re};  // i (Ky Ex - Kx Ey)
    const long long cstride = (long long)N * nz;
    zc* o = out + b * 6LL * N * nz + (long long)j * nz + cols[col];
    o[0 * cstride] = ex;
    o[1 * cstride] = ey;
    o[3 * cstride] = zc{hx.im, -hx.re};
    o[4 * cstride] = zc{hy.im, -hy.re};
    o[5 * cstride] = zc{hz.im, -hz.re};
    t[idx] = ky * hx - kx * hy;
}

// Ez = i (Ei t) (e = Ei t given) or i (inv_eps t) into out[b][2][j][iz]
__global__ void fields2d_ez_kernel(int B, int N, int cnt, int nz, const int* __restrict__ cols, const zc* __restrict__ e,
                                   const zc* inv_eps, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / N), j = (int)(r - (long long)col * N);
    const zc v = inv_eps ? *inv_eps * e[idx] : e[idx];
    out[b * 6LL * N * nz + 2LL * N * nz + (long long)j * nz + cols[col]] = zc{-v.im, v.re};
}

__global__ void nan_fields2d_kernel(int B, long long per, const int* __restrict__ fail, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * per) return;
    if (!fail[idx / per]) return;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    out[idx] = zc{nan, nan};
}

}  // namespace
}  // namespace rcwa_gb300
