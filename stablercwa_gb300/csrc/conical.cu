// conical.cu -- batched conical-incidence RCWA solve on the GPU (the engine behind rcwa::solve_conical
// and rcwa::sweep_conical, include/stablercwa/rcwa1d_conical.hpp:678-999).
//
// Per grating layer and sample: A = Kx^2 - [[eps]] and B C with B = Kx [[eps]]^{-1} Kx - I,
// C = [[1/eps]]^{-1} (the two inverses are sample-independent and formed once per call), two N x N
// eigensolves in one batched launch (2B matrices), then the 2N modes in the per-order (s, t) basis.
// A layer whose reduced eigenvalues come within 1e-2 |ky|^1.5 of zero switches, for that sample
// only, to the Schur basis of the full 2N operator (eig with the accumulated transform, an upper
// triangular square root, a triangular solve for V and triangular_exp for the propagation), through
// masked launches that leave the other samples untouched. The S-matrix recursion is the shared
// batched algebra of smatrix.cuh at order 2N with two right-hand sides (s and p input).
#include <cmath>
#include <complex>
#include <vector>

#include "smatrix.cuh"

namespace rcwa_gb300 {
namespace {

constexpr double kDegenerateWarn = 1e-2;  // rcwa1d_conical.hpp:191

// kz = sqrt(n^2 - kx^2 - ky^2), Im >= 0 (Re >= 0 when Im ~ 0); real radicand splits by sign so
// propagating orders have an exactly zero imaginary part (rcwa1d_conical.hpp:195-203).
__device__ zc longitudinal(zc n, double kx, double ky) {
    const zc n2 = zc{__dsub_rn(__dmul_rn(n.re, n.re), __dmul_rn(n.im, n.im)),
                     __dadd_rn(__dmul_rn(n.re, n.im), __dmul_rn(n.im, n.re))};
    const zc z = zc{__dsub_rn(__dsub_rn(n2.re, __dmul_rn(kx, kx)), __dmul_rn(ky, ky)), n2.im};
    if (z.im == 0.0) return z.re >= 0.0 ? zc{sqrt(z.re), 0.0} : zc{0.0, sqrt(-z.re)};
    zc kz = zsqrt(z);
    if (kz.im < 0.0) kz = -kz;
    if (fabs(kz.im) < 1e-12 && kz.re < 0.0) kz = -kz;
    return kz;
}
// the zeroth order from the incidence cosine (rcwa1d_conical.hpp:251-258)
__device__ zc longitudinal0(zc n, double nI, double cosine) {
    const zc a = zc{__dsub_rn(n.re, nI), n.im}, b = zc{__dadd_rn(n.re, nI), n.im};
    const zc ab = zc{__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
                     __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re))};
    const double c = __dmul_rn(nI, cosine);
    const zc z = zc{__dadd_rn(ab.re, __dmul_rn(c, c)), ab.im};
    if (z.im == 0.0) return z.re >= 0.0 ? zc{sqrt(z.re), 0.0} : zc{0.0, sqrt(-z.re)};
    zc kz = zsqrt(z);
    if (kz.im < 0.0) kz = -kz;
    if (fabs(kz.im) < 1e-12 && kz.re < 0.0) kz = -kz;
    return kz;
}

// Per-order kinematics (rcwa1d_conical.hpp:723-747): kx_m, cos/sin of the diffraction-plane
// azimuth, kz and flux factors in the two outer media, k0.
__global__ void conical_setup_kernel(int B, int M, ConicalPointsDev pts, double period, zc nI, zc nII, double* kx,
                                     double* cs, double* sn, zc* kzI, zc* kzII, double* flux_r, double* flux_t,
                                     double* k0, double* ky_out) {
    const int N = 2 * M + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const int b = (int)(idx / N), j = (int)(idx - (long long)b * N);
    const double ky = pts.ky[b];
    const double kxj = __dsub_rn(pts.s_cphi[b], __ddiv_rn(__dmul_rn((double)(j - M), pts.wl[b]), period));
    const double kt = hypot(kxj, ky);
    kx[idx] = kxj;
    if (kt <= 1e-14) {
        cs[idx] = pts.cphi[b];
        sn[idx] = pts.sphi[b];
    } else {
        cs[idx] = kxj / kt;
        sn[idx] = ky / kt;
    }
    const zc a = j == M ? longitudinal0(nI, nI.re, pts.ctheta[b]) : longitudinal(nI, kxj, ky);
    const zc c = j == M ? longitudinal0(nII, nI.re, pts.ctheta[b]) : longitudinal(nII, kxj, ky);
    kzI[idx] = a;
    kzII[idx] = c;
    const double unit = __dmul_rn(nI.re, pts.ctheta[b]);
    flux_r[idx] = a.re / unit;
    flux_t[idx] = c.re / unit;
    if (j == 0) {
        k0[b] = __ddiv_rn(2.0 * 3.141592653589793238462643383279502884, pts.wl[b]);
        if (ky_out) ky_out[b] = ky;
    }
}

// Analytic region of index nidx: s branch (w, v) = (1, q), t branch (kz/n, -i n), q = -i kz
// (rcwa1d_conical.hpp:259-283). With check_zero, an exact q == 0 fails the sample unless the
// stack is pure films and the order is not the zeroth (rcwa1d_conical.hpp:787-790).
__global__ void conical_analytic_kernel(int B, int M, const double* kx, const double* ky, const double* ctheta, zc nidx,
                                        double nI, zc* q, zc* w, zc* v, int check_zero, int pure_films, int* fail) {
    const int N = 2 * M + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * N) return;
    const int b = (int)(idx / N), j = (int)(idx - (long long)b * N);
    const zc kz = j == M ? longitudinal0(nidx, nI, ctheta[b]) : longitudinal(nidx, kx[idx], ky[b]);
    const zc qq = zc{kz.im, -kz.re};
    const long long base = (long long)b * 2 * N;
    q[base + j] = qq;
    q[base + N + j] = qq;
    w[base + j] = zc{1.0, 0.0};
    v[base + j] = qq;
    w[base + N + j] = zdiv(kz, nidx);
    v[base + N + j] = zc{nidx.im, -nidx.re};
    if (check_zero && is_zero(qq) && (!pure_films || j == M)) fail[b] = 1;
}

// B = Kx [[eps]]^{-1} Kx - I with the reference's order (kx_i e_ij) kx_j (rcwa1d_conical.hpp:320-325)
__global__ void conical_b_kernel(int B, int n, const zc* __restrict__ einv, const double* __restrict__ kx,
                                 zc* __restrict__ out) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    const int rem = (int)(idx - (long long)b * nn);
    const int j = rem / n, i = rem - j * n;
    const double ki = kx[(long long)b * n + i], kj = kx[(long long)b * n + j];
    const zc e = einv[rem];
    zc v = zc{(ki * e.re) * kj, (ki * e.im) * kj};
    if (i == j) v.re -= 1.0;
    out[idx] = v;
}

// min |lambda| over the two eigensolves of one layer; updates the sample's global minimum and flags
// the layer for the Schur basis when ky != 0 and the minimum is below 1e-2 |ky|^1.5
// (rcwa1d_conical.hpp:814-835, :838-849).
__global__ void conical_lambda_kernel(int B, int N, const zc* __restrict__ lam, const int* __restrict__ info,
                                      const double* __restrict__ ky, double* __restrict__ min_abs, int* __restrict__ schur,
                                      int* __restrict__ any_schur) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    double local = INFINITY;
    for (int t = 0; t < 2; ++t) {
        const long long m = b + (long long)t * B;
        if (info[m] != 0) continue;
        for (int j = lane; j < N; j += 32) local = fmin(local, zabs(lam[m * N + j]));
    }
    for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_xor_sync(0xffffffffu, local, o));
    if (lane == 0) {
        // the global minimum skips unconverged solves; the local one the reference takes over both anyway
        min_abs[b] = fmin(min_abs[b], local);
        double loc_all = local;
        const double k = ky[b];
        const double scale = fabs(k) * sqrt(fabs(k));
        const int s = (k != 0.0 && loc_all < kDegenerateWarn * scale) ? 1 : 0;
        schur[b] = s;
        if (s) atomicAdd(any_schur, 1);  // the number of Schur samples
    }
}

// The 2N modes of a general region from the two eigensolves (rcwa1d_conical.hpp:341-411): warp per
// (sample, eigenvector j); columns j (first group) and N + j (second group) of W and V, each
// normalised by the 2-norm of [W; V] (a zero column fails the sample).
__global__ void conical_general_region_kernel(int B, int N, const zc* __restrict__ lam, const zc* __restrict__ vec,
                                              const zc* __restrict__ cw, const zc* __restrict__ coupling,
                                              const double* __restrict__ kx, const double* __restrict__ ky,
                                              const double* __restrict__ cs, const double* __restrict__ sn,
                                              zc* __restrict__ q, zc* __restrict__ W, zc* __restrict__ V,
                                              const int* __restrict__ schur, int* __restrict__ fail) {
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= (long long)B * N) return;
    const int b = (int)(warp / N), j = (int)(warp - (long long)b * N);
    if (schur && schur[b]) return;
    const int lane = threadIdx.x & 31;
    const int n = 2 * N;
    const long long NN = (long long)N * N, nn = (long long)n * n;
    const double k = ky[b];
    const double* kxs = kx + (long long)b * N;
    const double* css = cs + (long long)b * N;
    const double* sns = sn + (long long)b * N;
    zc* Wb = W + b * nn;
    zc* Vb = V + b * nn;
    // first group: Ex = 0, Ey = W1 q1^2, hx = -W1 lambda1 q1, hy = -ky Kx W1 q1
    {
        const zc l1 = lam[(long long)b * N + j];
        const zc q1 = branch(zsqrt(zc{l1.re + k * k, l1.im}));
        if (lane == 0) q[(long long)b * n + j] = q1;
        const zc fy = q1 * q1, gx = -(l1 * q1), gy = (-k) * q1;
        const zc* w1 = vec + b * NN + (long long)j * N;
        zc* wc = Wb + (long long)j * n;
        zc* vc = Vb + (long long)j * n;
        double sum = 0.0;
        for (int m = lane; m < N; m += 32) {
            const zc ey = w1[m] * fy, hx = w1[m] * gx, hy = (kxs[m] * w1[m]) * gy;
            const zc a = css[m] * ey, c = sns[m] * ey;
            const zc d = -(css[m] * hx) - sns[m] * hy, e = css[m] * hy - sns[m] * hx;
            wc[m] = a;
            wc[N + m] = c;
            vc[m] = d;
            vc[N + m] = e;
            sum += norm2(a) + norm2(c) + norm2(d) + norm2(e);
        }
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const double scale = sqrt(sum);
        if (!(scale > 0.0) || !isfinite(scale)) {
            if (lane == 0) fail[b] = 1;
        } else {
            for (int m = lane; m < n; m += 32) {
                wc[m] = zdivr(wc[m], scale);
                vc[m] = zdivr(vc[m], scale);
            }
        }
    }
    // second group: Ex = W2 lambda2, Ey = ky [[eps]]^{-1} Kx C W2, hx = 0, hy = -C W2 q2
    {
        const zc l2 = lam[((long long)B + b) * N + j];
        const zc q2 = branch(zsqrt(zc{l2.re + k * k, l2.im}));
        if (lane == 0) q[(long long)b * n + N + j] = q2;
        const zc* w2 = vec + ((long long)B + b) * NN + (long long)j * N;
        const zc* cwj = cw + b * NN + (long long)j * N;
        const zc* yj = coupling + b * NN + (long long)j * N;
        zc* wc = Wb + (long long)(N + j) * n;
        zc* vc = Vb + (long long)(N + j) * n;
        double sum = 0.0;
        for (int m = lane; m < N; m += 32) {
            const zc ex = w2[m] * l2, ey = yj[m], hy = -(cwj[m] * q2);
            const zc a = css[m] * ey - sns[m] * ex, c = css[m] * ex + sns[m] * ey;
            const zc d = -(sns[m] * hy), e = css[m] * hy;
            wc[m] = a;
            wc[N + m] = c;
            vc[m] = d;
            vc[N + m] = e;
            sum += norm2(a) + norm2(c) + norm2(d) + norm2(e);
        }
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const double scale = sqrt(sum);
        if (!(scale > 0.0) || !isfinite(scale)) {
            if (lane == 0) fail[b] = 1;
        } else {
            for (int m = lane; m < n; m += 32) {
                wc[m] = zdivr(wc[m], scale);
                vc[m] = zdivr(vc[m], scale);
            }
        }
    }
}

// rows of C W2 scaled by ky kx_m (rcwa1d_conical.hpp:351-356)
__global__ void conical_scale_kykx_kernel(int B, int N, const zc* __restrict__ cw, const double* __restrict__ kx,
                                          const double* __restrict__ ky, zc* __restrict__ out) {
    const long long NN = (long long)N * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * NN) return;
    const int b = (int)(idx / NN);
    const int m = (int)((idx - (long long)b * NN) % N);
    out[idx] = (ky[b] * kx[(long long)b * N + m]) * cw[idx];
}

// Full 2N operators P, Q and the (s, t) rotations of the Schur branch (rcwa1d_conical.hpp:468-485)
__global__ void conical_schur_pq_kernel(int B, int N, const zc* __restrict__ inv_eps, const zc* __restrict__ A,
                                        const zc* __restrict__ c, const double* __restrict__ kx,
                                        const double* __restrict__ ky, const double* __restrict__ cs,
                                        const double* __restrict__ sn, zc* __restrict__ P, zc* __restrict__ Q,
                                        zc* __restrict__ RE, zc* __restrict__ RV, const int* __restrict__ schur) {
    const int n = 2 * N;
    const long long nn = (long long)n * n, NN = (long long)N * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * NN) return;
    const int b = (int)(idx / NN);
    if (!schur[b]) return;
    const int rem = (int)(idx - (long long)b * NN);
    const int j = rem / N, i = rem - j * N;
    const double k = ky[b];
    const double kxi = kx[(long long)b * N + i], kxj = kx[(long long)b * N + j];
    const zc id = zc{i == j ? 1.0 : 0.0, 0.0};
    const zc e = inv_eps[rem];
    zc* p = P + b * nn;
    zc* q = Q + b * nn;
    const zc a = A[b * NN + rem];
    const zc cc = c[rem];
    p[(long long)j * n + i] = (k * kxi) * e;
    p[(long long)(N + j) * n + i] = id - (kxi * e) * kxj;
    p[(long long)j * n + N + i] = (k * k) * e - id;
    p[(long long)(N + j) * n + N + i] = ((-k) * e) * kxj;
    q[(long long)j * n + i] = (k * kxi) * id;
    q[(long long)(N + j) * n + i] = -a;
    q[(long long)j * n + N + i] = (k * k) * id - cc;
    q[(long long)(N + j) * n + N + i] = -((k * kxi) * id);
    // rotations: written densely once per sample (only the diagonal band is nonzero)
    zc* re = RE + b * nn;
    zc* rv = RV + b * nn;
    const zc z0 = zc{0.0, 0.0};
    re[(long long)j * n + i] = z0;
    re[(long long)(N + j) * n + i] = z0;
    re[(long long)j * n + N + i] = z0;
    re[(long long)(N + j) * n + N + i] = z0;
    rv[(long long)j * n + i] = z0;
    rv[(long long)(N + j) * n + i] = z0;
    rv[(long long)j * n + N + i] = z0;
    rv[(long long)(N + j) * n + N + i] = z0;
    if (i == j) {
        const double c_ = cs[(long long)b * N + i], s_ = sn[(long long)b * N + i];
        re[(long long)i * n + i] = zc{-s_, 0.0};
        re[(long long)(N + i) * n + i] = zc{c_, 0.0};
        re[(long long)i * n + N + i] = zc{c_, 0.0};
        re[(long long)(N + i) * n + N + i] = zc{s_, 0.0};
        rv[(long long)i * n + i] = zc{-c_, 0.0};
        rv[(long long)(N + i) * n + i] = zc{-s_, 0.0};
        rv[(long long)i * n + N + i] = zc{-s_, 0.0};
        rv[(long long)(N + i) * n + N + i] = zc{c_, 0.0};
    }
}

__device__ double warp_norm1_upper(const zc* a, int n, int lane) {
    double best = 0.0;
    for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int i = lane; i < n; i += 32) s += zabs(a[(long long)j * n + i]);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        best = fmax(best, s);
    }
    return best;
}

// Principal square root of the Schur form T, diagonal by diagonal, and the residual check
// ||G G - T||_1 <= 1e-10 ||T||_1 (rcwa1d_conical.hpp:415-437). Warp per sample; gg holds G G.
__global__ void triangular_root_kernel(int B, int n, const zc* __restrict__ T, zc* __restrict__ G, zc* __restrict__ gg,
                                       const int* __restrict__ schur, int* __restrict__ fail) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B || !schur[b]) return;
    const int lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    const zc* t = T + b * nn;
    zc* g = G + b * nn;
    bool bad = false;
    for (long long k = lane; k < nn; k += 32) {
        if (!zfinite(t[k])) bad = true;
        g[k] = zc{0.0, 0.0};
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
        const zc r = branch(zsqrt(t[(long long)i * n + i]));
        if (is_zero(r) || !zfinite(r)) bad = true;
        g[(long long)i * n + i] = r;
    }
    __syncwarp();
    for (int gap = 1; gap < n; ++gap) {
        for (int i = lane; i + gap < n; i += 32) {
            const int j = i + gap;
            zc v = t[(long long)j * n + i];
            for (int k = i + 1; k < j; ++k) v = v - g[(long long)k * n + i] * g[(long long)j * n + k];
            const zc den = g[(long long)i * n + i] + g[(long long)j * n + j];
            if (is_zero(den)) bad = true;
            g[(long long)j * n + i] = zdiv(v, den);
        }
        __syncwarp();
    }
    // residual G G - T
    zc* rr = gg + b * nn;
    for (long long k = lane; k < nn; k += 32) {
        const int j = (int)(k / n), i = (int)(k - (long long)j * n);
        zc acc = zc{0.0, 0.0};
        for (int q = 0; q < n; ++q) acc = zfma(g[(long long)q * n + i], g[(long long)j * n + q], acc);
        if (!zfinite(g[k])) bad = true;
        rr[k] = acc - t[k];
    }
    __syncwarp();
    const double scale = warp_norm1_upper(t, n, lane), error = warp_norm1_upper(rr, n, lane);
    if (!isfinite(scale) || !isfinite(error) || error > 1e-10 * fmax(scale, 2.2250738585072014e-308)) bad = true;
    bad = __any_sync(0xffffffffu, bad);
    if (bad && lane == 0) fail[b] = 1;
}

// V G = Q Z solved for V by rows (rcwa1d_conical.hpp:494-500); q = diag(G).
__global__ void right_triangular_solve_kernel(int B, int n, zc* __restrict__ Vm, const zc* __restrict__ G,
                                              zc* __restrict__ q, const int* __restrict__ schur, int* __restrict__ fail) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B || !schur[b]) return;
    const int lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    zc* v = Vm + b * nn;
    const zc* g = G + b * nn;
    bool bad = false;
    for (int i = lane; i < n; i += 32) {
        for (int j = 0; j < n; ++j) {
            zc x = v[(long long)j * n + i];
            for (int k = 0; k < j; ++k) x = x - v[(long long)k * n + i] * g[(long long)j * n + k];
            x = zdiv(x, g[(long long)j * n + j]);
            if (!zfinite(x)) bad = true;
            v[(long long)j * n + i] = x;
        }
        q[b * n + i] = g[(long long)i * n + i];
    }
    bad = __any_sync(0xffffffffu, bad);
    if (bad && lane == 0) fail[b] = 1;
}

// exp(-k0 d G) for the Schur samples by scaling and squaring (rcwa1d_conical.hpp:439-464), with the
// n x n products done by batched GEMMs over the Schur samples (a product of two upper triangular
// matrices by a full GEMM adds only exact zeros outside the triangle, so every entry equals the
// triangular product). Host-driven: prep, Taylor
// terms until every sample has converged (at most 40), then the squarings. Per sample, work holds
// a = -k0 d G, bm = a 2^-s, term and tmp; iter[b] is 1 while sample b sums Taylor terms, done[b]
// is 1 once its sum has converged.
__global__ void texp_prep_kernel(int B, int n, const zc* __restrict__ G, const double* __restrict__ k0, double d,
                                 zc* __restrict__ E, zc* __restrict__ work, const int* __restrict__ schur,
                                 int* __restrict__ iter, int* __restrict__ done, int* __restrict__ scal,
                                 int* __restrict__ max_scal, int* __restrict__ fail) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        iter[b] = 0;
        done[b] = 0;
        scal[b] = 0;
    }
    if (!schur[b]) return;
    const long long nn = (long long)n * n;
    const double f = -k0[b] * d;
    zc* a = work + b * 4 * nn;
    zc* bm = a + nn;
    zc* term = bm + nn;
    zc* e = E + b * nn;
    const zc* g = G + b * nn;
    for (long long k = lane; k < nn; k += 32) a[k] = zc{f * g[k].re, f * g[k].im};
    __syncwarp();
    const double size = warp_norm1_upper(a, n, lane);
    bool bad = !isfinite(size);
    const int scaling = size > .25 ? max(0, (int)ceil(log2(size) + 2.)) : 0;
    if (scaling > 1020) bad = true;
    if (bad) {
        if (lane == 0) fail[b] = 1;
        return;
    }
    const double sf = ldexp(1., -scaling);
    for (long long k = lane; k < nn; k += 32) {
        const int j = (int)(k / n), i = (int)(k - (long long)j * n);
        bm[k] = zc{a[k].re * sf, a[k].im * sf};
        e[k] = zc{i == j ? 1.0 : 0.0, 0.0};
        term[k] = e[k];
    }
    if (lane == 0) {
        if (n == 0) done[b] = 1;
        else iter[b] = 1;
        scal[b] = scaling;
        atomicMax(max_scal, scaling);
    }
}

// term = tmp / kk, e += term, then the convergence test ||term||_1 <= eps max(1, ||e||_1)
__global__ void texp_term_kernel(int B, int n, int kk, zc* __restrict__ E, zc* __restrict__ work, int* __restrict__ iter,
                                 int* __restrict__ done, int* __restrict__ any_iter, int* __restrict__ fail) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B || !iter[b]) return;
    const int lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    zc* term = work + b * 4 * nn + 2 * nn;
    const zc* tmp = term + nn;
    zc* e = E + b * nn;
    const double inv = 1. / kk;
    bool bad = false;
    for (long long k = lane; k < nn; k += 32) {
        term[k] = tmp[k] * zc{inv, 0.0};
        e[k] = e[k] + term[k];
        if (!zfinite(e[k]) || !zfinite(term[k])) bad = true;
    }
    __syncwarp();
    bad = __any_sync(0xffffffffu, bad);
    bool converged = false;
    if (!bad) converged = warp_norm1_upper(term, n, lane) <= 2.220446049250313e-16 * fmax(1., warp_norm1_upper(e, n, lane));
    if (lane == 0) {
        if (bad || (!converged && kk == 40)) {
            fail[b] = 1;
            iter[b] = 0;
        } else if (converged) {
            iter[b] = 0;
            done[b] = 1;
        } else {
            atomicOr(any_iter, 1);
        }
    }
}

// e_ii = exp(a_ii 2^(k+1-s)): after the Taylor sum (mode 0, k = -1), or after squaring k (mode 1,
// which first copies the product in), for converged samples with k < s
__global__ void texp_fix_kernel(int B, int n, int k, int mode, zc* __restrict__ E, const zc* __restrict__ work,
                                const int* __restrict__ done, const int* __restrict__ scal, int* __restrict__ fail) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B || !done[b]) return;
    const int s_ = scal[b];
    if (mode == 1 && k >= s_) return;
    const int lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    const zc* a = work + b * 4 * nn;
    const zc* tmp = a + 3 * nn;
    zc* e = E + b * nn;
    bool bad = false;
    if (mode == 1) {
        for (long long q = lane; q < nn; q += 32) {
            e[q] = tmp[q];
            if (!zfinite(e[q])) bad = true;
        }
        __syncwarp();
    }
    const double s2 = ldexp(1., k + 1 - s_);
    for (int i = lane; i < n; i += 32) {
        const zc ai = a[(long long)i * n + i];
        e[(long long)i * n + i] = zexp(zc{ai.re * s2, ai.im * s2});
    }
    bad = __any_sync(0xffffffffu, bad);
    if (bad && lane == 0) fail[b] = 1;
}

// 1 where sample b squares at step k
__global__ void texp_square_mask_kernel(int B, int k, const int* __restrict__ done, const int* __restrict__ scal,
                                        int* __restrict__ mask) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B) mask[b] = done[b] && k < scal[b];
}

// Fresnel blocks between two analytic regions in the (w, v) form (rcwa1d_conical.hpp:513-533)
__global__ void conical_diag_interface_kernel(long long total, const zc* __restrict__ w1, const zc* __restrict__ v1,
                                              const zc* __restrict__ w2, const zc* __restrict__ v2, zc* tdd, zc* rdu,
                                              zc* rud, zc* tuu) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const zc a = w1[idx] * v2[idx], b = v1[idx] * w2[idx];
    const zc inv = zinv(a + b);
    tdd[idx] = (2.0 * (w1[idx] * v1[idx])) * inv;
    rdu[idx] = (a - b) * inv;
    rud[idx] = (b - a) * inv;
    tuu[idx] = (2.0 * (w2[idx] * v2[idx])) * inv;
}

// lower side analytic: mm = rows of W scaled by 1/w, nn = rows of V by 1/v; tp, tm = (mm +- nn)/2;
// a zero w or v fails the sample (rcwa1d_conical.hpp:539-547)
__global__ void conical_tp_tm_low_kernel(int B, int n, const zc* __restrict__ W, const zc* __restrict__ V,
                                         const zc* __restrict__ w, const zc* __restrict__ v, zc* __restrict__ tp,
                                         zc* __restrict__ tm, int* __restrict__ fail) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    const int i = (int)((idx - (long long)b * nn) % n);
    const zc wi = w[(long long)b * n + i], vi = v[(long long)b * n + i];
    if (is_zero(wi) || is_zero(vi)) fail[b] = 1;
    const zc mm = W[idx] * zinv(wi), nv = V[idx] * zinv(vi);
    tp[idx] = 0.5 * (mm + nv);
    tm[idx] = 0.5 * (mm - nv);
}

// top block of two analytic regions: columns M and N + M of Tdd and Rud (rcwa1d_conical.hpp:600-609)
__global__ void conical_top_diag_kernel(int B, int n, int M, const zc* __restrict__ tdd_d, const zc* __restrict__ rud_d,
                                        zc* __restrict__ tdd, zc* __restrict__ rud) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n * 2) return;
    const long long b = idx / (2LL * n);
    const int c = (int)((idx / n) % 2), i = (int)(idx % n);
    const int col = c == 0 ? M : n / 2 + M;
    tdd[idx] = i == col ? tdd_d[b * n + i] : zc{0.0, 0.0};
    rud[idx] = i == col ? rud_d[b * n + i] : zc{0.0, 0.0};
}

// Jones matrices, channel efficiencies and the failure contract (rcwa1d_conical.hpp:920-956)
__global__ void conical_finalize_kernel(int B, int N, int M, int pure_films, const zc* __restrict__ up,
                                        const zc* __restrict__ down, const double* __restrict__ flux_r,
                                        const double* __restrict__ flux_t, int* __restrict__ fail, zc* __restrict__ Jr,
                                        zc* __restrict__ Jt, double* __restrict__ DEr, double* __restrict__ DEt) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    const int n = 2 * N;
    bool bad = fail[b] != 0;
    const zc* u = up + b * 2 * n;
    const zc* dn = down + b * 2 * n;
    for (int j = lane; j < N; j += 32) {
        zc jr[4] = {u[j], u[n + j], -u[N + j], -u[n + N + j]};
        zc jt[4] = {dn[j], dn[n + j], dn[N + j], dn[n + N + j]};
        if (pure_films && j != M)
            for (int k = 0; k < 4; ++k) {
                if (!zfinite(jr[k])) jr[k] = zc{0.0, 0.0};
                if (!zfinite(jt[k])) jt[k] = zc{0.0, 0.0};
            }
        const double fr = flux_r[b * N + j], ft = flux_t[b * N + j];
        for (int k = 0; k < 4; ++k) {
            if (!zfinite(jr[k]) || !zfinite(jt[k])) bad = true;
            const double er = fr * norm2(jr[k]), et = ft * norm2(jt[k]);
            if (!isfinite(er) || !isfinite(et)) bad = true;
            Jr[(b * N + j) * 4 + k] = jr[k];
            Jt[(b * N + j) * 4 + k] = jt[k];
            DEr[(b * N + j) * 4 + k] = er;
            DEt[(b * N + j) * 4 + k] = et;
        }
    }
    bad = __any_sync(0xffffffffu, bad);
    if (bad) {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        for (int j = lane; j < N; j += 32)
            for (int k = 0; k < 4; ++k) {
                Jr[(b * N + j) * 4 + k] = zc{nan, nan};
                Jt[(b * N + j) * 4 + k] = zc{nan, nan};
                DEr[(b * N + j) * 4 + k] = nan;
                DEt[(b * N + j) * 4 + k] = nan;
            }
        if (lane == 0) fail[b] = 1;
    }
}

__global__ void conical_status_kernel(int B, const int* __restrict__ fail, const int* __restrict__ eig_info,
                                      int base_eig, const int* __restrict__ schur_count, int base_solves,
                                      const double* __restrict__ min_abs, const double* __restrict__ ky, int* status,
                                      int* info_out, int* n_eig, int* n_solve, int* n_schur, double* min_abs_out,
                                      int* warning) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    if (status) status[b] = fail[b] ? (eig_info[b] ? RCWA_SAMPLE_EIG_NOCONV : RCWA_SAMPLE_NUMERICAL) : RCWA_SAMPLE_OK;
    if (info_out) info_out[b] = eig_info[b];
    if (n_eig) n_eig[b] = base_eig + schur_count[b];
    if (n_solve) n_solve[b] = base_solves;
    if (n_schur) n_schur[b] = schur_count[b];
    if (min_abs_out) min_abs_out[b] = min_abs[b];
    if (warning) {
        const double k = ky[b];
        warning[b] = (k != 0.0 && min_abs[b] < kDegenerateWarn * (fabs(k) * sqrt(fabs(k)))) ? 1 : 0;
    }
}

// dst = src for the flagged samples only
__global__ void copy_masked_kernel(int B, long long per, const zc* __restrict__ src, zc* __restrict__ dst,
                                   const int* __restrict__ flag) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * per) return;
    if (flag[idx / per]) dst[idx] = src[idx];
}
// a non-finite entry fails the sample (flagged samples only)
__global__ void finite_check_masked_kernel(int B, long long per, const zc* __restrict__ a, const int* __restrict__ flag,
                                           int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * per) return;
    if (flag[idx / per] && !zfinite(a[idx])) fail[idx / per] = 1;
}

__global__ void add_flag_kernel(int B, const int* __restrict__ f, int* __restrict__ cnt) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B && f[b]) cnt[b] += 1;
}
__global__ void eig_info_pair_kernel(int B, const int* __restrict__ info, int* __restrict__ eig_info,
                                     int* __restrict__ fail) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    for (int t = 0; t < 2; ++t) {
        const int v = info[b + (long long)t * B];
        if (v != 0) {
            if (eig_info[b] == 0) eig_info[b] = v;
            fail[b] = 1;
        }
    }
}
__global__ void schur_info_kernel(int B, const int* __restrict__ info, const int* __restrict__ schur,
                                  int* __restrict__ eig_info, int* __restrict__ fail) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B || !schur[b]) return;
    if (info[b] != 0) {
        if (eig_info[b] == 0) eig_info[b] = info[b];
        fail[b] = 1;
    }
}

// exp(-k0 d G) of the Schur samples into E (B x n x n); work holds 4 n x n per sample
void batched_triangular_exp(Batch& c, int n, const zc* G, const double* k0, double d, zc* E, zc* work, const int* schur) {
    const cudaStream_t st = c.st;
    const int B = c.B;
    const long long nn = (long long)n * n;
    int* iter = c.mem->zeros<int>(B);
    int* done = c.mem->zeros<int>(B);
    int* scal = c.mem->zeros<int>(B);
    int* mask = c.mem->zeros<int>(B);
    int* flags = c.mem->zeros<int>(2);  // [0] largest scaling, [1] any sample still summing terms
    LAUNCH(texp_prep_kernel, warp_blocks(B), 128, st, B, n, G, k0, d, E, work, schur, iter, done, scal, flags, c.fail);
    for (int kk = 1; kk <= 40; ++kk) {
        // tmp = term bm for the samples still summing
        launch_zgemm(st, n, n, n, B, work + 2 * nn, n, 4 * nn, work + nn, n, 4 * nn, nullptr, 0, work + 3 * nn, n, 4 * nn,
                     1.0, 0.0, iter, 0);
        RCWA_CUDA(cudaMemsetAsync(flags + 1, 0, sizeof(int), st));
        LAUNCH(texp_term_kernel, warp_blocks(B), 128, st, B, n, kk, E, work, iter, done, flags + 1, c.fail);
        int any = 0;
        RCWA_CUDA(cudaMemcpyAsync(&any, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaStreamSynchronize(st));
        if (!any) break;
    }
    LAUNCH(texp_fix_kernel, warp_blocks(B), 128, st, B, n, -1, 0, E, work, done, scal, c.fail);
    int max_scal = 0;
    RCWA_CUDA(cudaMemcpyAsync(&max_scal, flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < max_scal; ++k) {
        LAUNCH(texp_square_mask_kernel, nblocks(B), kTpb, st, B, k, done, scal, mask);
        launch_zgemm(st, n, n, n, B, E, n, nn, E, n, nn, nullptr, 0, work + 3 * nn, n, 4 * nn, 1.0, 0.0, mask, 0);
        LAUNCH(texp_fix_kernel, warp_blocks(B), 128, st, B, n, k, 1, E, work, done, scal, c.fail);
    }
    for (int* p : {iter, done, scal, mask, flags}) c.mem->free(p);
}

struct Region {
    bool analytic = true;
    zc *q = nullptr, *w = nullptr, *v = nullptr;  // analytic: B x 2N diagonals
    zc *W = nullptr, *V = nullptr;                // general: B x 2N x 2N
    zc* G = nullptr;                              // Schur samples: upper triangular square root
    int* schur = nullptr;                         // per-sample Schur flag (nullptr: none)
};

void interface_matching(Batch& c, const Region& up, const Region& low, zc*& tp, zc*& tm) {
    const long long nd = (long long)c.B * c.nn();
    tp = c.dense();
    tm = c.dense();
    if (low.analytic) {
        LAUNCH(conical_tp_tm_low_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, up.W, up.V, low.w, low.v, tp, tm, c.fail);
        return;
    }
    zc *mm, *nn;
    if (up.analytic) {
        mm = solve(c, low.W, true, RHS_DIAG, up.w);
        nn = solve(c, low.V, true, RHS_DIAG, up.v);
    } else {
        mm = solve(c, low.W, true, RHS_DENSE, up.W);
        nn = solve(c, low.V, true, RHS_DENSE, up.V);
    }
    LAUNCH(tp_tm_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, mm, nn, nullptr, tp, tm);
    c.mem->free(mm);
    c.mem->free(nn);
}

DSBlock interface_block(Batch& c, const Region& up, const Region& low) {
    DSBlock s;
    if (up.analytic && low.analytic) {
        const long long nv = (long long)c.B * c.n;
        s.Tdd = {KDiag, c.vec()};
        s.Rdu = {KDiag, c.vec()};
        s.Rud = {KDiag, c.vec()};
        s.Tuu = {KDiag, c.vec()};
        LAUNCH(conical_diag_interface_kernel, nblocks(nv), kTpb, c.st, nv, up.w, up.v, low.w, low.v, s.Tdd.p, s.Rdu.p,
               s.Rud.p, s.Tuu.p);
        return s;
    }
    zc *tp, *tm;
    interface_matching(c, up, low, tp, tm);
    zc* tpi = solve(c, tp, false, RHS_IDENTITY, nullptr);
    zc* rdu = gemm(c, tm, c.nn(), tpi, nullptr, 1.0, 0.0);
    gemm(c, rdu, c.nn(), tm, tp, -1.0, 1.0, tp);
    zc* rud = gemm(c, tpi, c.nn(), tm, nullptr, -1.0, 0.0);
    c.mem->free(tm);
    s.Tdd = {KDense, tp};
    s.Rdu = {KDense, rdu};
    s.Rud = {KDense, rud};
    s.Tuu = {KDense, tpi};
    return s;
}

}  // namespace

// include/stablercwa/rcwa1d_conical.hpp:684-695 (the checks the reference adds to rcwa1d's)
void validate_conical(const rcwa_stack1d& stack, const rcwa_point_conical* h_points, int n_points, int M) {
    std::vector<rcwa_point1d> p1(h_points ? n_points : 0);
    for (int p = 0; h_points && p < n_points; ++p) {
        p1[p] = {h_points[p].wavelength, h_points[p].theta_deg};
        if (!std::isfinite(h_points[p].phi_deg)) throw EngineError{RCWA_EINVAL, "rcwa: azimuth angle must be finite"};
    }
    validate1d(stack, h_points ? p1.data() : nullptr, n_points, M, RCWA_TE);
    if (stack.nII.im != 0.0)
        throw EngineError{RCWA_EINVAL, "rcwa: conical incidence needs a real index in the exit medium"};
}

void solve_conical_device(cudaStream_t st, const rcwa_stack1d& stack, const ConicalPointsDev& pts, int n_points, int M,
                          const Options& opt, const rcwa_result_conical& d_out, size_t chunk_bytes) {
    const int N = 2 * M + 1, n = 2 * N;
    const long long NN = (long long)N * N, nn = (long long)n * n;
    if (n_points <= 0) return;
    // zero-thickness layers do not take part (rcwa1d_conical.hpp:699-703)
    std::vector<const rcwa_layer1d*> layers;
    for (int k = 0; k < stack.n_layers; ++k)
        if (stack.layers[k].d > 0.0) layers.push_back(&stack.layers[k]);
    const int L = static_cast<int>(layers.size());
    const auto uniform = [](const rcwa_layer1d& Ly) {
        if (Ly.homogeneous) return true;
        for (int j = 1; j < Ly.n_segments; ++j)
            if (Ly.n_values[j].re != Ly.n_values[0].re || Ly.n_values[j].im != Ly.n_values[0].im) return false;
        return true;
    };
    std::vector<int> grating;
    for (int k = 0; k < L; ++k)
        if (!uniform(*layers[k])) grating.push_back(k);
    const bool pure_films = grating.empty();
    const zc nI{stack.nI.re, stack.nI.im}, nII{stack.nII.re, stack.nII.im};

    // per grating layer, sample-independent: Toeplitz of eps, [[eps]]^{-1}, C = [[1/eps]]^{-1}
    DeviceScratch persist(st);
    int* layer_fail = persist.zeros<int>(1);
    struct LayerData {
        zc *c_eps = nullptr, *einv = nullptr, *cmat = nullptr;
    };
    std::vector<LayerData> ld(L);
    for (int k : grating) {
        const rcwa_layer1d& Ly = *layers[k];
        std::vector<double> edges(Ly.edges, Ly.edges + Ly.n_segments + 1);
        std::vector<std::complex<double>> eps, inv;
        for (int j = 0; j < Ly.n_segments; ++j) {
            const std::complex<double> nv{Ly.n_values[j].re, Ly.n_values[j].im};
            eps.push_back(nv * nv);
            inv.push_back(1.0 / (nv * nv));
        }
        ld[k].c_eps = layer_coefficients(st, persist, edges, eps, stack.period, M, Ly.fourier_method, Ly.fft_samples,
                                         layer_fail);
        zc* c_inv = layer_coefficients(st, persist, edges, inv, stack.period, M, Ly.fourier_method, Ly.fft_samples,
                                       layer_fail);
        zc* E = persist.get<zc>(NN);
        zc* Ci = persist.get<zc>(NN);
        LAUNCH(toeplitz_kernel, nblocks(NN), kTpb, st, M, ld[k].c_eps, E);
        LAUNCH(toeplitz_kernel, nblocks(NN), kTpb, st, M, c_inv, Ci);
        ld[k].einv = persist.get<zc>(NN);
        ld[k].cmat = persist.get<zc>(NN);
        launch_lu_solve(st, N, N, 1, E, NN, E, NN, RHS_IDENTITY, nullptr, NN, ld[k].einv, NN, layer_fail);
        launch_lu_solve(st, N, N, 1, Ci, NN, Ci, NN, RHS_IDENTITY, nullptr, NN, ld[k].cmat, NN, layer_fail);
    }
    const int base_solves = 2 * static_cast<int>(grating.size());

    const long long per_sample = 16LL * (nn * 16 + NN * 12 * (long long)grating.size() + (long long)n * 8 * (L + 2)) +
                                 2 * eig_workspace_bytes(N, 1) * (long long)std::max<size_t>(1, grating.size());
    long long chunk = chunk_bytes > 0 ? (long long)chunk_bytes / std::max(1LL, per_sample) : n_points;
    chunk = std::max(1LL, std::min<long long>(chunk, n_points));

    for (int p0 = 0; p0 < n_points; p0 += (int)chunk) {
        const int B = (int)std::min<long long>(chunk, n_points - p0);
        DeviceScratch mem(st);
        Batch c{st, &mem, B, n, M, nullptr, nullptr};
        c.fail = mem.zeros<int>(B);
        c.extra_solves = mem.zeros<int>(B);
        c.n_solve = base_solves;
        int* eig_info = mem.zeros<int>(B);
        int* schur_count = mem.zeros<int>(B);
        int* any_flag = mem.zeros<int>(1);
        double* min_abs = mem.get<double>(B);
        {
            std::vector<double> inf(B, INFINITY);
            RCWA_CUDA(cudaMemcpyAsync(min_abs, inf.data(), B * sizeof(double), cudaMemcpyHostToDevice, st));
            RCWA_CUDA(cudaStreamSynchronize(st));
        }
        const long long nvN = (long long)B * N, nv = (long long)B * n, nd = (long long)B * nn, ndN = (long long)B * NN;
        ConicalPointsDev P{pts.s_cphi + p0, pts.ky + p0, pts.cphi + p0, pts.sphi + p0, pts.ctheta + p0, pts.wl + p0};
        double* kx = mem.get<double>(nvN);
        double* cs = mem.get<double>(nvN);
        double* sn = mem.get<double>(nvN);
        zc* kzI = mem.get<zc>(nvN);
        zc* kzII = mem.get<zc>(nvN);
        double* flux_r = d_out.flux_r ? d_out.flux_r + (long long)p0 * N : mem.get<double>(nvN);
        double* flux_t = d_out.flux_t ? d_out.flux_t + (long long)p0 * N : mem.get<double>(nvN);
        double* k0 = mem.get<double>(B);
        LAUNCH(conical_setup_kernel, nblocks(nvN), kTpb, st, B, M, P, stack.period, nI, nII, kx, cs, sn, kzI, kzII, flux_r,
               flux_t, k0, d_out.ky ? d_out.ky + p0 : nullptr);
        if (d_out.kx) RCWA_CUDA(cudaMemcpyAsync(d_out.kx + (long long)p0 * N, kx, nvN * sizeof(double), cudaMemcpyDeviceToDevice, st));

        // ---- 1. modes
        std::vector<Region> modes(L + 2);
        const auto analytic = [&](Region& r, rcwa_complex idx, int check) {
            r.analytic = true;
            r.q = c.vec();
            r.w = c.vec();
            r.v = c.vec();
            LAUNCH(conical_analytic_kernel, nblocks(nvN), kTpb, st, B, M, kx, P.ky, P.ctheta, zc{idx.re, idx.im}, nI.re,
                   r.q, r.w, r.v, check, pure_films ? 1 : 0, c.fail);
        };
        analytic(modes[0], stack.nI, 0);
        analytic(modes[L + 1], stack.nII, 0);
        for (int k = 0; k < L; ++k)
            if (uniform(*layers[k])) {
                const rcwa_layer1d& Ly = *layers[k];
                analytic(modes[k + 1], Ly.homogeneous ? Ly.n : Ly.n_values[0], 1);
            }
        if (!grating.empty()) {
            // A and B C of every grating layer, then one eigensolve launch over all of them
            const int n_gr = (int)grating.size();
            zc* ABall = mem.get<zc>(2 * ndN * n_gr);
            zc* lamall = mem.get<zc>(2 * nvN * n_gr);
            zc* vecall = mem.get<zc>(2 * ndN * n_gr);
            int* infoall = mem.get<int>(2 * (size_t)B * n_gr);
            for (int gi = 0; gi < n_gr; ++gi) {
                const int k = grating[gi];
                zc* AB = ABall + 2 * ndN * gi;
                LAUNCH(assemble_te_kernel, nblocks(ndN), kTpb, st, B, M, ld[k].c_eps, kx, AB);
                zc* Bm = mem.get<zc>(ndN);
                LAUNCH(conical_b_kernel, nblocks(ndN), kTpb, st, B, N, ld[k].einv, kx, Bm);
                launch_zgemm(st, N, N, N, B, Bm, N, NN, ld[k].cmat, N, 0, nullptr, 0, AB + ndN, N, NN, 1.0, 0.0);
                mem.free(Bm);
                LAUNCH(finite_check_kernel, nblocks(ndN), kTpb, st, B, NN, AB, c.fail);
                LAUNCH(finite_check_kernel, nblocks(ndN), kTpb, st, B, NN, AB + ndN, c.fail);
            }
            {
                zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(N, 2 * B * n_gr) / sizeof(zc)) + 1);
                launch_eig(st, N, 2 * B * n_gr, ABall, NN, lamall, vecall, infoall, nullptr, ws, opt.eps, opt.max_iter,
                           opt.eig_group);
                mem.free(ws);
            }
            for (int gi = 0; gi < n_gr; ++gi) {
                const int k = grating[gi];
                zc* AB = ABall + 2 * ndN * gi;
                zc* lam = lamall + 2 * nvN * gi;
                zc* vec = vecall + 2 * ndN * gi;
                int* info = infoall + 2 * (size_t)B * gi;
                LAUNCH(eig_info_pair_kernel, nblocks(B), kTpb, st, B, info, eig_info, c.fail);
                Region& R = modes[k + 1];
                R.analytic = false;
                R.schur = mem.zeros<int>(B);
                RCWA_CUDA(cudaMemsetAsync(any_flag, 0, sizeof(int), st));
                LAUNCH(conical_lambda_kernel, warp_blocks(B), 128, st, B, N, lam, info, P.ky, min_abs, R.schur, any_flag);
                // general region (every sample not switched to the Schur basis)
                zc* cw = mem.get<zc>(ndN);
                launch_zgemm(st, N, N, N, B, ld[k].cmat, N, 0, vec + ndN, N, NN, nullptr, 0, cw, N, NN, 1.0, 0.0);
                zc* sc = mem.get<zc>(ndN);
                LAUNCH(conical_scale_kykx_kernel, nblocks(ndN), kTpb, st, B, N, cw, kx, P.ky, sc);
                zc* coupling = mem.get<zc>(ndN);
                launch_zgemm(st, N, N, N, B, ld[k].einv, N, 0, sc, N, NN, nullptr, 0, coupling, N, NN, 1.0, 0.0);
                mem.free(sc);
                R.q = c.vec();
                R.W = c.dense();
                R.V = c.dense();
                LAUNCH(conical_general_region_kernel, warp_blocks(nvN), 128, st, B, N, lam, vec, cw, coupling, kx, P.ky, cs,
                       sn, R.q, R.W, R.V, R.schur, c.fail);
                mem.free(cw);
                mem.free(coupling);
                int any = 0;
                RCWA_CUDA(cudaMemcpyAsync(&any, any_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
                RCWA_CUDA(cudaStreamSynchronize(st));
                if (any) {
                    // Schur basis of the full 2N operator for the flagged samples (rcwa1d_conical.hpp:466-502)
                    zc* Pm = c.dense();
                    zc* Qm = c.dense();
                    zc* RE = c.dense();
                    zc* RV = c.dense();
                    LAUNCH(conical_schur_pq_kernel, nblocks(ndN), kTpb, st, B, N, ld[k].einv, AB, ld[k].cmat, kx, P.ky, cs, sn,
                           Pm, Qm, RE, RV, R.schur);
                    zc* t1 = gemm(c, RE, nn, Pm, nullptr, 1.0, 0.0, nullptr, R.schur, 0);
                    gemm(c, t1, nn, RV, nullptr, 1.0, 0.0, Pm, R.schur, 0);
                    gemm(c, RV, nn, Qm, nullptr, 1.0, 0.0, t1, R.schur, 0);
                    gemm(c, t1, nn, RE, nullptr, 1.0, 0.0, Qm, R.schur, 0);
                    zc* H = gemm(c, Pm, nn, Qm, nullptr, 1.0, 0.0, t1, R.schur, 0);
                    LAUNCH(finite_check_masked_kernel, nblocks(nd), kTpb, st, B, nn, H, R.schur, c.fail);
                    zc* ws2 = mem.get<zc>((size_t)(eig_workspace_bytes(n, B) / sizeof(zc)) + 1);
                    zc* w2 = c.vec();
                    zc* Z = c.dense();
                    zc* Tm = c.dense();
                    int* info2 = mem.zeros<int>(B);
                    // few flagged samples: size the lanes per matrix by their number, not by the chunk
                    const int schur_group = opt.eig_group ? opt.eig_group : eig_default_group(n, any);
                    launch_eig(st, n, B, H, nn, w2, Z, info2, nullptr, ws2, 2.220446049250313e-16, 100, schur_group,
                               R.schur, 0, Tm);
                    mem.free(ws2);
                    LAUNCH(schur_info_kernel, nblocks(B), kTpb, st, B, info2, R.schur, eig_info, c.fail);
                    R.G = c.dense();
                    zc* gg = c.dense();
                    LAUNCH(triangular_root_kernel, warp_blocks(B), 128, st, B, n, Tm, R.G, gg, R.schur, c.fail);
                    // W = Z; V = Q Z, then V G = Q Z solved for V; q = diag(G)
                    LAUNCH(copy_masked_kernel, nblocks(nd), kTpb, st, B, nn, Z, R.W, R.schur);
                    gemm(c, Qm, nn, Z, nullptr, 1.0, 0.0, R.V, R.schur, 0);
                    LAUNCH(right_triangular_solve_kernel, warp_blocks(B), 128, st, B, n, R.V, R.G, R.q, R.schur, c.fail);
                    LAUNCH(add_flag_kernel, nblocks(B), kTpb, st, B, R.schur, schur_count);
                    for (zc* ptr : {gg, Tm, Z, w2, Pm, Qm, RE, RV, t1}) mem.free(ptr);
                    mem.free(info2);
                }
            }
            for (void* p : {(void*)ABall, (void*)lamall, (void*)vecall, (void*)infoall}) mem.free(p);
        }

        // ---- 2. bottom-up recursion at order 2N
        const int block_count = 2 * L + 1;
        std::vector<DOp> g(block_count);
        DOp r;
        for (int b = block_count - 1; b >= 1; --b) {
            const int j = b / 2;
            if (b % 2 == 0) {
                DSBlock blk = interface_block(c, modes[j], modes[j + 1]);
                if (blk.Tdd.kind == KDiag && r.kind != KDense) {
                    zc* gv = c.vec();
                    zc* rv = c.vec();
                    LAUNCH(stack_on_diag_kernel, nblocks(nv), kTpb, st, nv, blk.Tdd.p, blk.Rdu.p, blk.Rud.p, blk.Tuu.p,
                           r.kind == KZero ? nullptr : r.p, gv, rv);
                    g[b] = {KDiag, gv};
                    r = {KDiag, rv};
                    continue;
                }
                Seam seam = stack_on(c, std::move(blk), r);
                g[b] = seam.g;
                r = seam.r;
                continue;
            }
            const Region& m = modes[j + 1];
            const double d = layers[j]->d;
            zc* x = c.vec();
            zc* refl = c.vec();
            int* hz = mem.zeros<int>(B);
            LAUNCH(propagation_kernel, nblocks(nv), kTpb, st, B, n, m.q, k0, d, 0, x, refl, hz, c.fail);
            if (r.kind != KDense) {
                zc* gv = c.vec();
                zc* rv = c.vec();
                LAUNCH(stack_on_diag_kernel, nblocks(nv), kTpb, st, nv, x, nullptr, nullptr, x,
                       r.kind == KZero ? nullptr : r.p, gv, rv);
                g[b] = {KDiag, gv};
                r = {KDiag, rv};
                continue;
            }
            zc* rn = c.dense();
            const int* skip = m.G ? m.schur : nullptr;
            LAUNCH(scale_both_kernel, nblocks(nd), kTpb, st, B, n, r.p, x, x, rn, skip, 1);
            if (m.G) {
                // Schur samples: Tdd = Tuu = exp(-k0 d G), r' = E (r E) (rcwa1d_conical.hpp:871-874)
                zc* E = c.dense();
                zc* work = mem.get<zc>(4 * (size_t)nd);
                batched_triangular_exp(c, n, m.G, k0, d, E, work, m.schur);
                mem.free(work);
                zc* y = gemm(c, r.p, nn, E, nullptr, 1.0, 0.0, nullptr, m.schur, 0);
                gemm(c, E, nn, y, nullptr, 1.0, 0.0, rn, m.schur, 0);
                mem.free(y);
                g[b] = {KDiag, x, E, m.schur};
            } else {
                g[b] = {KDiag, x};
            }
            r = {KDense, rn};
        }

        // ---- 3. top interface, columns M and N + M (rcwa1d_conical.hpp:891-919)
        zc* tdd = mem.get<zc>(2 * nv);
        zc* rud = mem.get<zc>(2 * nv);
        DOp topRdu, topTuu;
        if (modes[0].analytic && modes[1].analytic) {
            zc* Tdd = c.vec();
            zc* Rdu = c.vec();
            zc* Rud = c.vec();
            zc* Tuu = c.vec();
            LAUNCH(conical_diag_interface_kernel, nblocks(nv), kTpb, st, nv, modes[0].w, modes[0].v, modes[1].w,
                   modes[1].v, Tdd, Rdu, Rud, Tuu);
            LAUNCH(conical_top_diag_kernel, nblocks(2 * nv), kTpb, st, B, n, M, Tdd, Rud, tdd, rud);
            topRdu = {KDiag, Rdu};
            topTuu = {KDiag, Tuu};
        } else {
            zc *tp, *tm;
            interface_matching(c, modes[0], modes[1], tp, tm);
            zc* tpi = solve(c, tp, false, RHS_IDENTITY, nullptr);
            zc* rdu = gemm(c, tm, nn, tpi, nullptr, 1.0, 0.0);
            zc* tm_e = mem.get<zc>(2 * nv);
            LAUNCH(col_extract_kernel, nblocks(nv), kTpb, st, B, n, tm, M, tm_e, 2, 0);
            LAUNCH(col_extract_kernel, nblocks(nv), kTpb, st, B, n, tm, N + M, tm_e, 2, 1);
            LAUNCH(col_extract_kernel, nblocks(nv), kTpb, st, B, n, tp, M, tdd, 2, 0);
            LAUNCH(col_extract_kernel, nblocks(nv), kTpb, st, B, n, tp, N + M, tdd, 2, 1);
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 2, rdu, tm_e, tdd, tdd, -1.0, 1.0);
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 2, tpi, tm_e, nullptr, rud, -1.0, 0.0);
            mem.free(tp);
            mem.free(tm);
            topRdu = {KDense, rdu};
            topTuu = {KDense, tpi};
        }
        DOp k = op_mul(c, topRdu, r);
        zc* down = tdd;
        if (k.kind == KDiag) {
            LAUNCH(vec_div_one_minus_kernel, nblocks(2 * nv), kTpb, st, B, n, 2, down, k.p);
        } else if (k.kind == KDense) {
            LAUNCH(identity_minus_kernel, nblocks(nd), kTpb, st, B, n, k.p, nullptr, 1);
            down = solve(c, k.p, true, RHS_DENSE, tdd, 2);
        }
        zc* rdn = mem.get<zc>(2 * nv);
        LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 2, (int)r.kind, r.p, nullptr, nullptr, down, rdn);
        zc* back = mem.get<zc>(2 * nv);
        LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 2, (int)topTuu.kind, topTuu.p, nullptr, nullptr, rdn, back);
        LAUNCH(vec_add_kernel, nblocks(2 * nv), kTpb, st, 2 * nv, back, rud);
        zc* cur = down;
        zc* nxt = mem.get<zc>(2 * nv);
        for (int b = 1; b < block_count; ++b) {
            LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 2, (int)g[b].kind, g[b].p, g[b].alt, g[b].alt_flag, cur,
                   nxt);
            std::swap(cur, nxt);
        }

        // ---- 4. Jones matrices, efficiencies, status
        LAUNCH(conical_finalize_kernel, warp_blocks(B), 128, st, B, N, M, pure_films ? 1 : 0, rud, cur, flux_r, flux_t,
               c.fail, reinterpret_cast<zc*>(d_out.Jr) + (long long)p0 * N * 4,
               reinterpret_cast<zc*>(d_out.Jt) + (long long)p0 * N * 4, d_out.DEr + (long long)p0 * N * 4,
               d_out.DEt + (long long)p0 * N * 4);
        LAUNCH(conical_status_kernel, nblocks(B), kTpb, st, B, c.fail, eig_info, 2 * (int)grating.size(), schur_count,
               c.n_solve, min_abs, P.ky, d_out.status ? d_out.status + p0 : nullptr,
               d_out.eig_info ? d_out.eig_info + p0 : nullptr, d_out.n_eig ? d_out.n_eig + p0 : nullptr,
               d_out.n_dense_solve ? d_out.n_dense_solve + p0 : nullptr, d_out.n_schur ? d_out.n_schur + p0 : nullptr,
               d_out.min_abs_lambda ? d_out.min_abs_lambda + p0 : nullptr,
               d_out.degenerate_mode_warning ? d_out.degenerate_mode_warning + p0 : nullptr);
        mem.release();
    }
    int lf = 0;
    RCWA_CUDA(cudaMemcpyAsync(&lf, layer_fail, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(cudaStreamSynchronize(st));
    if (lf) {
        const double nan = std::nan("");
        const size_t cnt = (size_t)n_points * N * 4;
        std::vector<double> nans(cnt * 2, nan);
        RCWA_CUDA(cudaMemcpyAsync(d_out.Jr, nans.data(), cnt * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_out.Jt, nans.data(), cnt * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_out.DEr, nans.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_out.DEt, nans.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, st));
        if (d_out.status) {
            std::vector<int> s(n_points, RCWA_SAMPLE_NUMERICAL);
            RCWA_CUDA(cudaMemcpyAsync(d_out.status, s.data(), n_points * sizeof(int), cudaMemcpyHostToDevice, st));
        }
        RCWA_CUDA(cudaStreamSynchronize(st));
    }
}

}  // namespace rcwa_gb300
