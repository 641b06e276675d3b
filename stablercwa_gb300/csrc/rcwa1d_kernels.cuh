// rcwa1d_kernels.cuh -- per-sample elementwise kernels of the batched 1-D TE/TM solve.
//
// Every kernel works on a chunk of B sweep points. Diagonal operators are B x n vectors, dense
// operators B x n x n column-major matrices. Where the reference's result depends on an exact
// floating-point equality (q == 0 selects the linear-field branch, include/stablercwa/rcwa1d.hpp:
// 534, :756, :956), the operands are formed with explicitly rounded intrinsics so that no fused
// multiply-add changes which branch a sample takes.
#pragma once

#include "common.cuh"

namespace rcwa_gb300 {
namespace {  // internal linkage: included by several translation units

// kx_m = s - (m - M) lambda / period (include/stablercwa/rcwa1d.hpp:410-415). s = nI sin(theta) is
// computed on the host with the host's libm, exactly as the reference does, and passed per sample.
__global__ void kx_kernel(int B, int M, const double* __restrict__ s, const double* __restrict__ wl, double period,
                          double* __restrict__ kx) {
    const int n = 2 * M + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const int b = (int)(idx / n), j = (int)(idx - (long long)b * n);
    kx[idx] = __dsub_rn(s[b], __ddiv_rn(__dmul_rn((double)(j - M), wl[b]), period));
}

// Analytic modes of a homogeneous region of index nidx (include/stablercwa/rcwa1d.hpp:522-544):
// kz = sqrt(n^2 - kx^2) with Im kz >= 0 (Re >= 0 when Im ~ 0), q = -i kz, p = q (TE) or q/n^2 (TM);
// with finite_zero_basis an exact q == 0 uses the auxiliary basis q = 1 in p.
__device__ __forceinline__ bool analytic_mode(double k, zc nidx, int pol, int fzb, zc& q, zc& p) {
    const zc n2 = zc{__dsub_rn(__dmul_rn(nidx.re, nidx.re), __dmul_rn(nidx.im, nidx.im)),
                     __dadd_rn(__dmul_rn(nidx.re, nidx.im), __dmul_rn(nidx.im, nidx.re))};
    zc kz = zsqrt(zc{__dsub_rn(n2.re, __dmul_rn(k, k)), n2.im});
    if (kz.im < 0.0) kz = -kz;
    if (fabs(kz.im) < 1e-12 && kz.re < 0.0) kz = -kz;
    const zc qq = zc{kz.im, -kz.re};
    q = qq;
    const bool zero = is_zero(qq);
    const zc bq = (fzb && zero) ? zc{1.0, 0.0} : qq;
    p = pol == 0 ? bq : zdiv(bq, n2);
    return zero;
}

__global__ void analytic_modes_kernel(int B, int n, const double* __restrict__ kx, zc nidx, int pol, int fzb,
                                      zc* __restrict__ q, zc* __restrict__ p, int* __restrict__ zero_flag) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    zc qq, pp;
    const bool zero = analytic_mode(kx[idx], nidx, pol, fzb, qq, pp);
    q[idx] = qq;
    p[idx] = pp;
    if (zero_flag && fzb && zero) zero_flag[idx / n] = 1;
}

// The analytic modes of several homogeneous regions in one launch: region r (index n_r, exact-zero basis
// flag fzb_r) writes q and p at offset r * B * n; inactive regions (gratings) are skipped.
struct AnalyticRegion {
    zc n;
    int fzb;
    int active;
};
__global__ void analytic_modes_all_kernel(int R, int B, int n, const double* __restrict__ kx,
                                          const AnalyticRegion* __restrict__ regions, int pol, zc* __restrict__ q,
                                          zc* __restrict__ p) {
    const long long nv = (long long)B * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)R * nv) return;
    const int r = (int)(idx / nv);
    const AnalyticRegion reg = regions[r];
    if (!reg.active) return;
    const long long e = idx - (long long)r * nv;
    zc qq, pp;
    analytic_mode(kx[e], reg.n, pol, reg.fzb, qq, pp);
    q[idx] = qq;
    p[idx] = pp;
}

// The run of homogeneous regions at the bottom of a stack, every block diagonal: one thread per (sample,
// order) carries the reflection r up through the run, block by block from the exit medium, with the
// Fresnel interface (diagonal_interface_kernel's formulas), the propagation factor of each film
// (propagation_kernel's, exact q == 0 included) and the diagonal stack_on step (stack_on_diag_kernel's),
// and stores each block's g for the downward pass; the final r is the run's reflection. The same
// arithmetic in the same order as the per-block launches (include/stablercwa/rcwa1d.hpp:644-661,
// :751-808), in one launch.
struct FilmBlock {
    int propagate;  // 1: through the film of region `up`, thickness d; 0: interface between `up` and `low`
    int up, low;
    int fzb;
    double d;
};
__global__ void film_run_kernel(int B, int n, int nblk, const FilmBlock* __restrict__ blk, const zc* __restrict__ aq,
                                const zc* __restrict__ ap, const double* __restrict__ k0, zc* __restrict__ g_out,
                                zc* __restrict__ r_out, int* __restrict__ fail) {
    const long long nv = (long long)B * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nv) return;
    const int b = (int)(idx / n);
    bool rzero = true;
    zc r{0.0, 0.0};
    for (int t = 0; t < nblk; ++t) {
        const FilmBlock fb = blk[t];
        zc tdd, rdu, rud, tuu;
        if (!fb.propagate) {
            const zc a = ap[(long long)fb.up * nv + idx], c = ap[(long long)fb.low * nv + idx];
            const zc inv = zinv(a + c);
            tdd = (2.0 * a) * inv;
            rdu = (c - a) * inv;
            rud = (a - c) * inv;
            tuu = (2.0 * c) * inv;
        } else {
            const zc qq = aq[(long long)fb.up * nv + idx];
            const double kd = k0[b];
            if (fb.fzb && is_zero(qq)) {
                const double h = kd * fb.d;
                if (!isfinite(h)) fail[b] = 1;
                const double den = 1.0 + 0.5 * h;
                tdd = zc{1.0 / den, 0.0};
                rdu = zc{(0.5 * h) / den, 0.0};
            } else {
                const double f = -kd * fb.d;
                tdd = zexp(zc{f * qq.re, f * qq.im});
                rdu = zc{0.0, 0.0};
            }
            rud = rdu;
            tuu = tdd;
        }
        zc gv;
        if (!rzero) {
            const zc k = rdu * r;
            const zc f = zinv(zc{1.0, 0.0} - k);
            gv = f * tdd;
            r = rud + tuu * (r * gv);
        } else {
            gv = tdd;
            r = rud;
            rzero = false;
        }
        g_out[(long long)t * nv + idx] = gv;
    }
    r_out[idx] = r;
}

// y = g_0 (g_1 (... (g_{nblk-1} x))) elementwise: the downward pass through the run, top block first
__global__ void film_push_kernel(long long nv, int nblk, const zc* __restrict__ g, const zc* __restrict__ x,
                                 zc* __restrict__ y) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nv) return;
    zc v = x[idx];
    for (int t = nblk - 1; t >= 0; --t) v = g[(long long)t * nv + idx] * v;
    y[idx] = v;
}

// TE layer matrix A = Kx^2 - [[eps]] from the Toeplitz coefficients c_h, h = -2M..2M
// (include/stablercwa/rcwa1d.hpp:450-457): A(i,j) = -c_{i-j}, plus kx_i^2 on the diagonal.
__global__ void assemble_te_kernel(int B, int M, const zc* __restrict__ c, const double* __restrict__ kx,
                                   zc* __restrict__ A) {
    const int n = 2 * M + 1;
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    const zc v = c[i - j + 2 * M];
    zc a = zc{-v.re, -v.im};
    if (i == j) {
        const double k = kx[(long long)b * n + i];
        a.re = __dadd_rn(a.re, __dmul_rn(k, k));
    }
    A[idx] = a;
}

// TM: the per-sample middle factor Kx [[eps]]^{-1} Kx - I of
// A = [[1/eps]]^{-1} (Kx [[eps]]^{-1} Kx - I) (include/stablercwa/rcwa1d.hpp:459-466).
// einv is the sample-independent inverse of [[eps]].
__global__ void tm_middle_kernel(int B, int n, const zc* __restrict__ einv, const double* __restrict__ kx,
                                 zc* __restrict__ out) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    const double kj = kx[(long long)b * n + j], ki = kx[(long long)b * n + i];
    const zc e = einv[rem];
    zc v = zc{(e.re * kj) * ki, (e.im * kj) * ki};
    if (i == j) v.re -= 1.0;
    out[idx] = v;
}

// The parts of Kx E Kx for kx_j = a + b m_j, m_j = j - M (every sample's kx has this form):
// Kx E Kx = a^2 E + a b X1 + b^2 X2 with X1_ij = (m_i + m_j) E_ij, X2_ij = m_i m_j E_ij (one n x n matrix)
__global__ void pencil_parts_kernel(int n, int M, const zc* __restrict__ E, zc* __restrict__ X1, zc* __restrict__ X2) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * n) return;
    const int j = idx / n, i = idx - j * n;
    const double mi = (double)(i - M), mj = (double)(j - M);
    const zc e = E[idx];
    X1[idx] = (mi + mj) * e;
    X2[idx] = (mi * mj) * e;
}
// A = a^2 S0 + a b S1 + b^2 S2 - C per sample, a = a_s[b] (the order-0 kx), b = -wl[b] / period: the pencil's
// Hermitian matrix L^-1 (Kx E Kx - I) L^-H from the layer's four constant parts
__global__ void pencil_combine_kernel(int B, int n, const zc* __restrict__ S0, const zc* __restrict__ S1,
                                      const zc* __restrict__ S2, const zc* __restrict__ C, const double* __restrict__ a_s,
                                      const double* __restrict__ wl, double period, zc* __restrict__ A) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const long long b = idx / nn, e = idx - b * nn;
    const double a = a_s[b], bb = -wl[b] / period;
    const double c0 = a * a, c1 = a * bb, c2 = bb * bb;
    const zc s0 = S0[e], s1 = S1[e], s2 = S2[e], cc = C[e];
    A[idx] = zc{c0 * s0.re + c1 * s1.re + c2 * s2.re - cc.re, c0 * s0.im + c1 * s1.im + c2 * s2.im - cc.im};
}

// Modes of an eigen-decomposed layer (include/stablercwa/rcwa1d.hpp:949-958):
// q = branch(sqrt(lambda)) with Re q >= 0 and Im q <= 0 when Re q < 1e-10; basis q = 1 where q == 0.
__device__ __forceinline__ zc branch(zc q) {
    if (q.re < 0.0) q = -q;
    if (q.re < 1e-10 && q.im > 0.0) q = -q;
    return q;
}
__global__ void eig_modes_q_kernel(int B, int n, const zc* __restrict__ lambda, zc* __restrict__ q,
                                   zc* __restrict__ bq, int* __restrict__ zero_flag) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const zc qq = branch(zsqrt(lambda[idx]));
    q[idx] = qq;
    const bool zero = is_zero(qq);
    bq[idx] = zero ? zc{1.0, 0.0} : qq;
    if (zero) zero_flag[idx / n] = 1;
}

// dst(i,j) = src(i,j) * d_j  (scale_columns, include/stablercwa/matrix.hpp:194-201)
__global__ void scale_cols_kernel(int B, int n, const zc* __restrict__ src, const zc* __restrict__ d,
                                  zc* __restrict__ dst, const int* __restrict__ skip, int skip_value) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    if (skip && skip[b] == skip_value) return;
    const int j = (int)((idx - (long long)b * nn) / n);
    dst[idx] = src[idx] * d[(long long)b * n + j];
}
// dst(i,j) = d_i * src(i,j)  (scale_rows, include/stablercwa/matrix.hpp:202-210)
__global__ void scale_rows_kernel(int B, int n, const zc* __restrict__ src, const zc* __restrict__ d,
                                  zc* __restrict__ dst, const int* __restrict__ skip, int skip_value) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    if (skip && skip[b] == skip_value) return;
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    (void)j;
    dst[idx] = src[idx] * d[(long long)b * n + i];
}
// dst(i,j) = d_i * src(i,j) * e_j  (Diag * Dense * Diag)
__global__ void scale_both_kernel(int B, int n, const zc* __restrict__ src, const zc* __restrict__ dl,
                                  const zc* __restrict__ dr, zc* __restrict__ dst, const int* __restrict__ skip,
                                  int skip_value) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    if (skip && skip[b] == skip_value) return;
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    dst[idx] = dl[(long long)b * n + i] * (src[idx] * dr[(long long)b * n + j]);
}

// tp = (mm + nn)/2, tm = (mm - nn)/2 with nn = rows of V scaled by 1/p_low (the lower side analytic; the
// reciprocals precomputed) or nn given (include/stablercwa/rcwa1d.hpp:664-692).
__global__ void tp_tm_kernel(int B, int n, const zc* __restrict__ mm, const zc* __restrict__ nn_or_v,
                             const zc* __restrict__ inv_p_low, zc* __restrict__ tp, zc* __restrict__ tm) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    zc v = nn_or_v[idx];
    if (inv_p_low) {
        const int b = (int)(idx / nn);
        const int i = (int)((idx - (long long)b * nn) % n);
        v = v * inv_p_low[(long long)b * n + i];
    }
    const zc m = mm[idx];
    tp[idx] = 0.5 * (m + v);
    tm[idx] = 0.5 * (m - v);
}
// out = 1 / p elementwise (Smith's reciprocal, the value the per-element form would compute)
__global__ void reciprocal_kernel(long long total, const zc* __restrict__ p, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) out[idx] = zinv(p[idx]);
}

// lhs = tp - r tm, rhs = r tp - tm with r diagonal (r = null: zero), for the seam of a dense region
// over an analytic one
__global__ void seam_system_kernel(int B, int n, const zc* __restrict__ tp, const zc* __restrict__ tm,
                                   const zc* __restrict__ r, zc* __restrict__ lhs, zc* __restrict__ rhs) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const zc a = tp[idx], m = tm[idx];
    if (!r) {
        lhs[idx] = a;
        rhs[idx] = zc{-m.re, -m.im};
        return;
    }
    const long long b = idx / nn;
    const zc ri = r[b * n + (idx - b * nn) % n];
    lhs[idx] = a - ri * m;
    rhs[idx] = ri * a - m;
}
// rhs = 2 p0_M e_M per sample
__global__ void top_rhs_kernel(int B, int n, int M, const zc* __restrict__ p0, zc* __restrict__ rhs) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const long long b = idx / n;
    const int i = (int)(idx - b * n);
    rhs[idx] = i == M ? 2.0 * p0[b * n + M] : zc{0.0, 0.0};
}
// R_M -= 1 (the incident order's own amplitude)
__global__ void sub_incident_kernel(int B, int n, int M, zc* __restrict__ R) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    R[b * n + M].re -= 1.0;
}

// An analytic medium (diagonal field factors w, v; w = null: 1, the planar form) over a dense region (W, V):
// the row-scaled combinations of the tangential relations w (d_a + u_a) = W (I + r) d_b and
// v (d_a - u_a) = V (I - r) d_b. Row i uses the E relation when |w_i| >= |v_i| (always when w is null).
__device__ __forceinline__ bool e_row(const zc* w, const zc* v, long long bi) {
    return !w || zabs(w[bi]) >= zabs(v[bi]);
}
// P = v W + w V, Q = v W - w V
__global__ void analytic_pq_kernel(int B, int n, const zc* __restrict__ W, const zc* __restrict__ V,
                                   const zc* __restrict__ w, const zc* __restrict__ v, zc* __restrict__ P,
                                   zc* __restrict__ Q) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const long long b = idx / nn;
    const long long bi = b * n + (idx - b * nn) % n;
    const zc a = v[bi] * W[idx], c = w ? w[bi] * V[idx] : V[idx];
    P[idx] = a + c;
    Q[idx] = a - c;
}
// out = 2 w v per (sample, order)
__global__ void two_wv_kernel(long long total, const zc* __restrict__ w, const zc* __restrict__ v, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) out[idx] = 2.0 * (w ? w[idx] * v[idx] : v[idx]);
}
// Z0 + Z1 r is W (I + r) in E rows and V (I - r) in H rows: Z0 = W or V, Z1 = W or -V by row
__global__ void z_rows_kernel(int B, int n, const zc* __restrict__ W, const zc* __restrict__ V, const zc* __restrict__ w,
                              const zc* __restrict__ v, zc* __restrict__ Z0, zc* __restrict__ Z1) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const long long b = idx / nn;
    const long long bi = b * n + (idx - b * nn) % n;
    if (e_row(w, v, bi)) {
        Z0[idx] = W[idx];
        Z1[idx] = W[idx];
    } else {
        Z0[idx] = V[idx];
        Z1[idx] = zc{-V[idx].re, -V[idx].im};
    }
}
// r' from Zg = Z g in place: E rows Zg / w - I, H rows I - Zg / v
__global__ void seam_reflection_kernel(int B, int n, zc* __restrict__ Zg, const zc* __restrict__ w,
                                       const zc* __restrict__ v) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const long long b = idx / nn;
    const long long rem = idx - b * nn;
    const int j = (int)(rem / n), i = (int)(rem - (long long)j * n);
    const long long bi = b * n + i;
    const double d = i == j ? 1.0 : 0.0;
    if (e_row(w, v, bi)) {
        const zc x = w ? zdiv(Zg[idx], w[bi]) : Zg[idx];
        Zg[idx] = zc{x.re - d, x.im};
    } else {
        const zc y = zdiv(Zg[idx], v[bi]);
        Zg[idx] = zc{d - y.re, -y.im};
    }
}

// I - m in place (include/stablercwa/rcwa1d.hpp:623-629)
__global__ void identity_minus_kernel(int B, int n, zc* __restrict__ m, const int* __restrict__ skip, int skip_value) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    if (skip && skip[b] == skip_value) return;
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    zc v = -m[idx];
    if (i == j) v.re += 1.0;
    m[idx] = v;
}

// dense += diag (or dense = diag + dense when the diagonal comes first; same sums)
__global__ void add_diag_kernel(int B, int n, zc* __restrict__ m, const zc* __restrict__ d, const int* __restrict__ skip,
                                int skip_value) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const int b = (int)(idx / n);
    if (skip && skip[b] == skip_value) return;
    const int i = (int)(idx - (long long)b * n);
    zc* p = m + (long long)b * n * n + (long long)i * n + i;
    *p = *p + d[idx];
}

// dense a += dense b
__global__ void add_dense_kernel(long long total, zc* __restrict__ a, const zc* __restrict__ b) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) a[idx] = a[idx] + b[idx];
}

// densify a diagonal operator
__global__ void diag_to_dense_kernel(int B, int n, const zc* __restrict__ d, zc* __restrict__ m,
                                     const int* __restrict__ skip, int skip_value) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    if (skip && skip[b] == skip_value) return;
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    m[idx] = i == j ? d[(long long)b * n + i] : zc{0.0, 0.0};
}

// Fresnel blocks between two analytic regions (include/stablercwa/rcwa1d.hpp:644-661)
__global__ void diagonal_interface_kernel(long long total, const zc* __restrict__ p1, const zc* __restrict__ p2,
                                          zc* __restrict__ tdd, zc* __restrict__ rdu, zc* __restrict__ rud,
                                          zc* __restrict__ tuu) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const zc a = p1[idx], b = p2[idx];
    const zc inv = zinv(a + b);
    tdd[idx] = (2.0 * a) * inv;
    rdu[idx] = (b - a) * inv;
    rud[idx] = (a - b) * inv;
    tuu[idx] = (2.0 * b) * inv;
}

// Propagation factors exp(-k0 d q) and the exact q == 0 linear-field block
// (include/stablercwa/rcwa1d.hpp:751-784): Tdd = Tuu = 1/(1 + h/2), Rdu = Rud = (h/2)/(1 + h/2), h = k0 d.
__global__ void propagation_kernel(int B, int n, const zc* __restrict__ q, const double* __restrict__ k0, double d,
                                   int fzb, zc* __restrict__ x, zc* __restrict__ refl, int* __restrict__ has_zero,
                                   int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const int b = (int)(idx / n);
    const zc qq = q[idx];
    const double kd = k0[b];
    if (fzb && is_zero(qq)) {
        const double h = kd * d;
        if (!isfinite(h)) fail[b] = 1;
        const double den = 1.0 + 0.5 * h;
        x[idx] = zc{1.0 / den, 0.0};
        refl[idx] = zc{(0.5 * h) / den, 0.0};
        has_zero[b] = 1;
    } else {
        const double f = -kd * d;
        x[idx] = zexp(zc{f * qq.re, f * qq.im});
        refl[idx] = zc{0.0, 0.0};
    }
}

// Diagonal stack_on step: k = Rdu r, g = Tdd / (1 - k), r' = Rud + Tuu r g
// (include/stablercwa/rcwa1d.hpp:794-808 with every operator diagonal; a missing Rdu/Rud is zero).
__global__ void stack_on_diag_kernel(long long total, const zc* __restrict__ tdd, const zc* __restrict__ rdu,
                                     const zc* __restrict__ rud, const zc* __restrict__ tuu, const zc* __restrict__ r,
                                     zc* __restrict__ g, zc* __restrict__ rout) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const zc t = tdd[idx];
    const zc rv = r ? r[idx] : zc{0.0, 0.0};
    zc gv;
    if (rdu && r) {
        const zc k = rdu[idx] * rv;
        const zc f = zinv(zc{1.0, 0.0} - k);
        gv = f * t;
    } else {
        gv = t;
    }
    g[idx] = gv;
    zc out = r ? tuu[idx] * (rv * gv) : zc{0.0, 0.0};
    if (rud) out = rud[idx] + out;
    rout[idx] = out;
}

// ---------------------------------------------------------------- near fields (rcwa1d_fields.hpp:107-189)

// Orders other than M carry nothing in a stack of films (clear_unexcited, rcwa1d.hpp:1011-1019)
__global__ void clear_unexcited_kernel(int B, int n, int M, zc* __restrict__ v) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    if ((int)(idx % n) != M) v[idx] = zc{0.0, 0.0};
}

// S and U harmonics of layer j at the given depths from the amplitudes anchored at the layer's top
// (a+) and bottom (a-); U is scaled by the analytic V diagonal p when p != null. Layout per sample:
// n x nz column-major.
__global__ void layer_su_kernel(int B, int n, int nz, const double* __restrict__ zl, double d, const double* __restrict__ k0,
                                const zc* __restrict__ ap, const zc* __restrict__ am, const zc* __restrict__ q, int fzb,
                                const zc* __restrict__ p, zc* __restrict__ S, zc* __restrict__ U) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * nz;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / n), j = (int)(r - (long long)col * n);
    const double z = fmax(0.0, fmin(d, zl[col]));
    const double k = k0[b];
    const zc a = ap[b * n + j], bm = am[b * n + j], qj = q[b * n + j];
    zc s, u;
    if (fzb && is_zero(qj)) {
        const double den = 1.0 + 0.5 * k * d;
        const double from_bottom = (1.0 + k * (d - z)) / den, from_top = (1.0 + k * z) / den;
        s = from_bottom * a + from_top * bm;
        u = zdivr(-a, den) + zdivr(bm, den);
    } else {
        const zc pp = is_zero(a) ? zc{0.0, 0.0} : a * zexp((-k * z) * qj);
        const zc mm = is_zero(bm) ? zc{0.0, 0.0} : bm * zexp((-k * (d - z)) * qj);
        s = pp + mm;
        u = mm - pp;
    }
    if (p) u = p[b * n + j] * u;
    S[idx] = s;
    U[idx] = u;
}

// S and U of the incident (region -1) or exit (region -2) medium (rcwa1d_fields.hpp:147-161)
__global__ void region_su_kernel(int B, int n, int M, int nz, const double* __restrict__ zs, int region, double z_bottom,
                                 const double* __restrict__ k0, const zc* __restrict__ q, const zc* __restrict__ p,
                                 const zc* __restrict__ R, const zc* __restrict__ T, zc* __restrict__ S, zc* __restrict__ U) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * nz;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / n), j = (int)(r - (long long)col * n);
    const double z = zs[col], k = k0[b];
    const zc qj = q[b * n + j];
    const zc kz{-k * qj.im, k * qj.re};  // kz = i k0 q
    zc pp{0.0, 0.0}, rr{0.0, 0.0}, tt{0.0, 0.0};
    if (region == -1) {
        if (j == M) {
            const zc q0 = q[b * n + M];
            const zc kz0{-k * q0.im, k * q0.re};
            pp = zexp(zc{-kz0.im * z, kz0.re * z});  // exp(i kz0 z)
        }
        const zc Rj = R[b * n + j];
        if (!is_zero(Rj)) rr = Rj * zexp(zc{kz.im * z, -kz.re * z});  // exp(-i kz z)
    } else {
        const zc Tj = T[b * n + j];
        const double dz = z - z_bottom;
        if (!is_zero(Tj)) tt = Tj * zexp(zc{-kz.im * dz, kz.re * dz});  // exp(i kz (z - z_bottom))
    }
    S[idx] = pp + rr + tt;
    U[idx] = p[b * n + j] * ((rr - pp) - tt);
}

// Scatter S, U (and Ez for TM) of one depth group into the field harmonics out[b][c][j][iz]
// (components Ex, Ey, Ez, Hx, Hy, Hz): TE Ey = S, Hx = i U, Hz = -kx S; TM Ex = -i U, Ez, Hy = S.
__global__ void field_out_kernel(int B, int n, int nzg, int nz, const int* __restrict__ cols, int pol,
                                 const double* __restrict__ kx, const zc* __restrict__ S, const zc* __restrict__ U,
                                 const zc* __restrict__ Ez, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * nzg;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / n), j = (int)(r - (long long)col * n);
    const int iz = cols[col];
    const zc s = S[idx], u = U[idx];
    zc* o = out + b * 6LL * n * nz + (long long)j * nz + iz;
    const long long cstride = (long long)n * nz;
    if (pol == 0) {
        o[1 * cstride] = s;
        o[3 * cstride] = zc{-u.im, u.re};
        o[5 * cstride] = -kx[b * n + j] * s;
    } else {
        o[0 * cstride] = zc{u.im, -u.re};
        o[2 * cstride] = Ez[idx];
        o[4 * cstride] = s;
    }
}

// Ez = kx S / eps for a scalar eps (analytic layers and the two media)
__global__ void ez_scalar_kernel(long long total, int n, const double* __restrict__ kx, int nzg, const zc* __restrict__ S,
                                 zc inv_eps, zc* __restrict__ Ez) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long per = (long long)n * nzg;
    const long long b = idx / per;
    const int j = (int)((idx - b * per) % n);
    Ez[idx] = (kx[b * n + j] * S[idx]) * inv_eps;
}

// rows of S scaled by kx (the right-hand side of the Eps solve for Ez in a grating layer)
__global__ void kx_rows_kernel(long long total, int n, const double* __restrict__ kx, int nzg, const zc* __restrict__ S,
                               zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long per = (long long)n * nzg;
    const long long b = idx / per;
    const int j = (int)((idx - b * per) % n);
    out[idx] = kx[b * n + j] * S[idx];
}

// number of modes with q exactly 0 in one layer, per sample (the finite-zero-basis modes of the field metadata,
// include/stablercwa/rcwa1d_fields.hpp:99)
__global__ void zero_q_count_kernel(int B, int n, const zc* __restrict__ q, int* __restrict__ out, int stride) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int count = 0;
    for (int j = 0; j < n; ++j) count += is_zero(q[(long long)b * n + j]) ? 1 : 0;
    out[(long long)b * stride] = count;
}

__global__ void nan_fields_kernel(int B, long long per, const int* __restrict__ fail, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * per) return;
    if (!fail[idx / per]) return;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    out[idx] = zc{nan, nan};
}

}  // namespace
}  // namespace rcwa_gb300
