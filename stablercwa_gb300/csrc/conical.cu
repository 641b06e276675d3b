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

// right-hand sides 2 w_j v_j e_j for the incident orders j = M (s input) and N + M (p input)
__global__ void conical_top_rhs_kernel(int B, int n, int N, int M, const zc* __restrict__ w, const zc* __restrict__ v,
                                       zc* __restrict__ rhs) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2LL * B * n) return;
    const long long b = idx / (2LL * n);
    const int rem = (int)(idx - b * 2 * n), col = rem / n, i = rem - col * n;
    const int j = col == 0 ? M : N + M;
    rhs[idx] = i == j ? 2.0 * (w[b * n + j] * v[b * n + j]) : zc{0.0, 0.0};
}
// R from X = W (d_b + r d_b) and Y = V (d_b - r d_b), with d_a the unit incident column: row i from the
// tangential E relation w_i (d_a + R)_i = X_i when |w_i| >= |v_i|, else from the H relation
// v_i (d_a - R)_i = Y_i (w_i and v_i never vanish together)
__global__ void conical_top_reflection_kernel(int B, int n, int N, int M, const zc* __restrict__ w,
                                              const zc* __restrict__ v, const zc* __restrict__ X,
                                              const zc* __restrict__ Y, zc* __restrict__ R) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2LL * B * n) return;
    const long long b = idx / (2LL * n);
    const int rem = (int)(idx - b * 2 * n), col = rem / n, i = rem - col * n;
    const double d = i == (col == 0 ? M : N + M) ? 1.0 : 0.0;
    const zc wi = w[b * n + i], vi = v[b * n + i];
    if (zabs(wi) >= zabs(vi)) {
        const zc x = zdiv(X[idx], wi);
        R[idx] = zc{x.re - d, x.im};
    } else {
        const zc y = zdiv(Y[idx], vi);
        R[idx] = zc{d - y.re, -y.im};
    }
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

// The Schur-branch kernels below run one CTA of kSchurThreads per flagged sample (the launches span the
// chunk and unflagged samples return at once): a chunk has few flagged samples, so the work of each must
// spread over many threads.
constexpr int kSchurThreads = 256;

// max_j sum_{i <= j} |a_ij| of one sample's upper triangle (the 1-norm of an upper triangular matrix),
// one column per thread then a block maximum (fmax: a NaN column sum is passed over; the callers test the
// entries' finiteness themselves); every thread gets the result
__device__ double block_norm1_upper(const zc* a, int n, double* red) {
    double best = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i <= j; ++i) s += zabs(a[(long long)j * n + i]);
        best = fmax(best, s);
    }
    for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
    __syncthreads();
    double out = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) out = fmax(out, red[w]);
    __syncthreads();
    return out;
}

// Principal square root G of the Schur form T, diagonal by diagonal (rcwa1d_conical.hpp:415-437); the
// residual G G - T is checked by schur_root_check_kernel after a batched product
__global__ void __launch_bounds__(kSchurThreads) triangular_root_kernel(int B, int n, const zc* __restrict__ T,
                                                                       zc* __restrict__ G, const int* __restrict__ schur,
                                                                       int* __restrict__ fail) {
    const long long b = blockIdx.x;
    if (b >= B || !schur[b]) return;
    const long long nn = (long long)n * n;
    const zc* t = T + b * nn;
    zc* g = G + b * nn;
    int bad = 0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) {
        if (!zfinite(t[k])) bad = 1;
        g[k] = zc{0.0, 0.0};
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const zc r = branch(zsqrt(t[(long long)i * n + i]));
        if (is_zero(r) || !zfinite(r)) bad = 1;
        g[(long long)i * n + i] = r;
    }
    __syncthreads();
    for (int gap = 1; gap < n; ++gap) {
        for (int i = threadIdx.x; i + gap < n; i += blockDim.x) {
            const int j = i + gap;
            zc v = t[(long long)j * n + i];
            for (int k = i + 1; k < j; ++k) v = v - g[(long long)k * n + i] * g[(long long)j * n + k];
            const zc den = g[(long long)i * n + i] + g[(long long)j * n + j];
            if (is_zero(den)) bad = 1;
            g[(long long)j * n + i] = zdiv(v, den);
        }
        __syncthreads();
    }
    for (long long k = threadIdx.x; k < nn; k += blockDim.x)
        if (!zfinite(g[k])) bad = 1;
    if (__syncthreads_or(bad) && threadIdx.x == 0) fail[b] = 1;
}

// ||G G - T||_1 <= 1e-10 ||T||_1 (rcwa1d_conical.hpp:430-436), with gg = G G from a batched product
__global__ void __launch_bounds__(kSchurThreads) schur_root_check_kernel(int B, int n, const zc* __restrict__ T,
                                                                        zc* __restrict__ gg, const int* __restrict__ schur,
                                                                        int* __restrict__ fail) {
    __shared__ double red[kSchurThreads / 32];
    const long long b = blockIdx.x;
    if (b >= B || !schur[b]) return;
    const long long nn = (long long)n * n;
    const zc* t = T + b * nn;
    zc* rr = gg + b * nn;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) rr[k] = rr[k] - t[k];
    __syncthreads();
    const double scale = block_norm1_upper(t, n, red), error = block_norm1_upper(rr, n, red);
    if (threadIdx.x == 0 &&
        (!isfinite(scale) || !isfinite(error) || error > 1e-10 * fmax(scale, 2.2250738585072014e-308)))
        fail[b] = 1;
}

// V G = Q Z solved for V by rows (rcwa1d_conical.hpp:494-500), one thread per (sample, row); q = diag(G)
__global__ void right_triangular_solve_kernel(int B, int n, zc* __restrict__ Vm, const zc* __restrict__ G,
                                              zc* __restrict__ q, const int* __restrict__ schur, int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const long long b = idx / n;
    if (!schur[b]) return;
    const int i = (int)(idx - b * n);
    const long long nn = (long long)n * n;
    zc* v = Vm + b * nn;
    const zc* g = G + b * nn;
    bool bad = false;
    for (int j = 0; j < n; ++j) {
        zc x = v[(long long)j * n + i];
        for (int k = 0; k < j; ++k) x = x - v[(long long)k * n + i] * g[(long long)j * n + k];
        x = zdiv(x, g[(long long)j * n + j]);
        if (!zfinite(x)) bad = true;
        v[(long long)j * n + i] = x;
    }
    q[b * n + i] = g[(long long)i * n + i];
    if (bad) fail[b] = 1;
}

// exp(-k0 d G) for the Schur samples by scaling and squaring (rcwa1d_conical.hpp:439-464), with the
// n x n products done by batched GEMMs over the Schur samples (a product of two upper triangular
// matrices by a full GEMM adds only exact zeros outside the triangle, so every entry equals the
// triangular product). Host-driven: prep, Taylor
// terms until every sample has converged (at most 40), then the squarings. Per sample, work holds
// a = -k0 d G, bm = a 2^-s, term and tmp; iter[b] is 1 while sample b sums Taylor terms, done[b]
// is 1 once its sum has converged.
__global__ void __launch_bounds__(kSchurThreads) texp_prep_kernel(int B, int n, const zc* __restrict__ G,
                                                                  const double* __restrict__ k0, double d,
                                                                  zc* __restrict__ E, zc* __restrict__ work,
                                                                  const int* __restrict__ schur, int* __restrict__ iter,
                                                                  int* __restrict__ done, int* __restrict__ scal,
                                                                  int* __restrict__ max_scal, int* __restrict__ fail) {
    __shared__ double red[kSchurThreads / 32];
    const long long b = blockIdx.x;
    if (b >= B) return;
    if (threadIdx.x == 0) {
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
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) a[k] = zc{f * g[k].re, f * g[k].im};
    __syncthreads();
    const double size = block_norm1_upper(a, n, red);
    const int scaling = isfinite(size) && size > .25 ? max(0, (int)ceil(log2(size) + 2.)) : 0;
    if (!isfinite(size) || scaling > 1020) {
        if (threadIdx.x == 0) fail[b] = 1;
        return;
    }
    const double sf = ldexp(1., -scaling);
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) {
        const int j = (int)(k / n), i = (int)(k - (long long)j * n);
        bm[k] = zc{a[k].re * sf, a[k].im * sf};
        e[k] = zc{i == j ? 1.0 : 0.0, 0.0};
        term[k] = e[k];
    }
    if (threadIdx.x == 0) {
        if (n == 0) done[b] = 1;
        else iter[b] = 1;
        scal[b] = scaling;
        atomicMax(max_scal, scaling);
    }
}

// term = tmp / kk, e += term, then the convergence test ||term||_1 <= eps max(1, ||e||_1)
__global__ void __launch_bounds__(kSchurThreads) texp_term_kernel(int B, int n, int kk, zc* __restrict__ E,
                                                                  zc* __restrict__ work, int* __restrict__ iter,
                                                                  int* __restrict__ done, int* __restrict__ any_iter,
                                                                  int* __restrict__ fail) {
    __shared__ double red[kSchurThreads / 32];
    const long long b = blockIdx.x;
    if (b >= B || !iter[b]) return;
    const long long nn = (long long)n * n;
    zc* term = work + b * 4 * nn + 2 * nn;
    const zc* tmp = term + nn;
    zc* e = E + b * nn;
    const double inv = 1. / kk;
    int bad = 0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) {
        term[k] = tmp[k] * zc{inv, 0.0};
        e[k] = e[k] + term[k];
        if (!zfinite(e[k]) || !zfinite(term[k])) bad = 1;
    }
    bad = __syncthreads_or(bad);
    bool converged = false;
    if (!bad) {
        const double nt = block_norm1_upper(term, n, red), ne = block_norm1_upper(e, n, red);
        converged = nt <= 2.220446049250313e-16 * fmax(1., ne);
    }
    if (threadIdx.x == 0) {
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
__global__ void __launch_bounds__(kSchurThreads) texp_fix_kernel(int B, int n, int k, int mode, zc* __restrict__ E,
                                                                 const zc* __restrict__ work, const int* __restrict__ done,
                                                                 const int* __restrict__ scal, int* __restrict__ fail) {
    const long long b = blockIdx.x;
    if (b >= B || !done[b]) return;
    const int s_ = scal[b];
    if (mode == 1 && k >= s_) return;
    const long long nn = (long long)n * n;
    const zc* a = work + b * 4 * nn;
    const zc* tmp = a + 3 * nn;
    zc* e = E + b * nn;
    int bad = 0;
    if (mode == 1) {
        for (long long q = threadIdx.x; q < nn; q += blockDim.x) {
            e[q] = tmp[q];
            if (!zfinite(e[q])) bad = 1;
        }
        __syncthreads();
    }
    const double s2 = ldexp(1., k + 1 - s_);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const zc ai = a[(long long)i * n + i];
        e[(long long)i * n + i] = zexp(zc{ai.re * s2, ai.im * s2});
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) fail[b] = 1;
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
                                         const zc* __restrict__ inv_w, const zc* __restrict__ inv_v, zc* __restrict__ tp,
                                         zc* __restrict__ tm) {
    const long long nn = (long long)n * n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * nn) return;
    const int b = (int)(idx / nn);
    const long long bi = (long long)b * n + (idx - (long long)b * nn) % n;
    const zc mm = W[idx] * inv_w[bi], nv = V[idx] * inv_v[bi];
    tp[idx] = 0.5 * (mm + nv);
    tm[idx] = 0.5 * (mm - nv);
}
// 1/w and 1/v of an analytic region's diagonal field factors; a zero factor fails the sample
__global__ void conical_inv_wv_kernel(int B, int n, const zc* __restrict__ w, const zc* __restrict__ v,
                                      zc* __restrict__ inv_w, zc* __restrict__ inv_v, int* __restrict__ fail) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const zc wi = w[idx], vi = v[idx];
    if (is_zero(wi) || is_zero(vi)) fail[idx / n] = 1;
    inv_w[idx] = zinv(wi);
    inv_v[idx] = zinv(vi);
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
                                      int base_lu, const double* __restrict__ min_abs, const double* __restrict__ ky,
                                      int* status, int* info_out, int* n_eig, int* n_solve, int* n_lu, int* n_schur,
                                      double* min_abs_out, int* warning) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    if (status) status[b] = fail[b] ? (eig_info[b] ? RCWA_SAMPLE_EIG_NOCONV : RCWA_SAMPLE_NUMERICAL) : RCWA_SAMPLE_OK;
    if (info_out) info_out[b] = eig_info[b];
    if (n_eig) n_eig[b] = base_eig + schur_count[b];
    if (n_solve) n_solve[b] = base_solves;
    if (n_lu) n_lu[b] = base_lu;
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
    LAUNCH(texp_prep_kernel, (unsigned)B, kSchurThreads, st, B, n, G, k0, d, E, work, schur, iter, done, scal, flags,
           c.fail);
    for (int kk = 1; kk <= 40; ++kk) {
        // tmp = term bm for the samples still summing
        launch_zgemm(st, n, n, n, B, work + 2 * nn, n, 4 * nn, work + nn, n, 4 * nn, nullptr, 0, work + 3 * nn, n, 4 * nn,
                     1.0, 0.0, iter, 0);
        RCWA_CUDA(cudaMemsetAsync(flags + 1, 0, sizeof(int), st));
        LAUNCH(texp_term_kernel, (unsigned)B, kSchurThreads, st, B, n, kk, E, work, iter, done, flags + 1, c.fail);
        int any = 0;
        RCWA_CUDA(cudaMemcpyAsync(&any, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(stream_wait(st));
        if (!any) break;
    }
    LAUNCH(texp_fix_kernel, (unsigned)B, kSchurThreads, st, B, n, -1, 0, E, work, done, scal, c.fail);
    int max_scal = 0;
    RCWA_CUDA(cudaMemcpyAsync(&max_scal, flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    for (int k = 0; k < max_scal; ++k) {
        LAUNCH(texp_square_mask_kernel, nblocks(B), kTpb, st, B, k, done, scal, mask);
        launch_zgemm(st, n, n, n, B, E, n, nn, E, n, nn, nullptr, 0, work + 3 * nn, n, 4 * nn, 1.0, 0.0, mask, 0);
        LAUNCH(texp_fix_kernel, (unsigned)B, kSchurThreads, st, B, n, k, 1, E, work, done, scal, c.fail);
    }
    for (int* p : {iter, done, scal, mask, flags}) c.mem->free(p);
}

// ---------------------------------------------------------------- near fields (rcwa1d_conical_fields.hpp)

// rows whose order is not M cleared in B x cols x 2N vectors (clear_unexcited, rcwa1d_conical.hpp:239-243)
__global__ void conical_clear_unexcited_kernel(long long total, int n, int N, int M, zc* __restrict__ v) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    if ((int)(idx % n) % N != M) v[idx] = zc{0.0, 0.0};
}

// a = A(:, 0) Es + A(:, 1) Ep per sample, A of B x 2 x n (field_jones_response, rcwa1d_conical_fields.hpp:100-104)
__global__ void jones_response_kernel(int B, int n, const zc* __restrict__ A, const zc* __restrict__ jones,
                                      zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const long long b = idx / n;
    const int i = (int)(idx - b * n);
    out[idx] = A[(b * 2) * n + i] * jones[2 * b] + A[(b * 2 + 1) * n + i] * jones[2 * b + 1];
}

// Down and up parts at the group's depths, P = a exp(-k0 q t), Mm = b exp(-k0 q (d - t)) with t the depth
// below the layer's top clamped to [0, d], for the samples that propagate mode by mode (Schur samples are
// filled by conical_schur_apply_kernel). Per sample n x cnt, column-major (rcwa1d_conical_fields.hpp:179-190).
__global__ void conical_layer_pm_kernel(int B, int n, int cnt, const double* __restrict__ zl, double d,
                                        const double* __restrict__ k0, const zc* __restrict__ a, const zc* __restrict__ bm,
                                        const zc* __restrict__ q, const int* __restrict__ schur, zc* __restrict__ P,
                                        zc* __restrict__ Mm) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    if (schur && schur[b]) return;
    const long long r = idx - b * per;
    const int col = (int)(r / n), j = (int)(r - (long long)col * n);
    const double from_top = fmax(0.0, fmin(d, zl[col])), from_bottom = d - from_top;
    const double k = k0[b];
    const zc av = a[b * n + j], bv = bm[b * n + j], qj = q[b * n + j];
    P[idx] = is_zero(av) ? zc{0.0, 0.0} : av * zexp((-k * from_top) * qj);
    Mm[idx] = is_zero(bv) ? zc{0.0, 0.0} : bv * zexp((-k * from_bottom) * qj);
}

// out column col of the Schur samples = E x (E = nullptr: x itself, a zero distance); warp per sample
__global__ void conical_schur_apply_kernel(int B, int n, const zc* __restrict__ E, const zc* __restrict__ x,
                                           const int* __restrict__ schur, zc* __restrict__ out, int cnt, int col) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B || !schur[b]) return;
    const int lane = threadIdx.x & 31;
    const zc* xs = x + b * n;
    zc* o = out + (b * cnt + col) * n;
    if (!E) {
        for (int i = lane; i < n; i += 32) o[i] = xs[i];
        return;
    }
    const zc* Es = E + b * (long long)n * n;
    for (int i = lane; i < n; i += 32) {
        zc acc{0.0, 0.0};
        for (int k = 0; k < n; ++k) acc = zfma(Es[(long long)k * n + i], xs[k], acc);
        o[i] = acc;
    }
}

// F = P + Mm and G = Mm - P, scaled by the diagonal modes w, v of an analytic region
__global__ void conical_fg_kernel(long long total, int n, int cnt, const zc* __restrict__ P, const zc* __restrict__ Mm,
                                  const zc* __restrict__ w, const zc* __restrict__ v, zc* __restrict__ F,
                                  zc* __restrict__ G) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    zc f = P[idx] + Mm[idx], g = -P[idx] + Mm[idx];
    if (w) {
        const long long per = (long long)n * cnt;
        const long long b = idx / per;
        const int j = (int)((idx - b * per) % n);
        f = f * w[b * n + j];
        g = g * v[b * n + j];
    }
    F[idx] = f;
    G[idx] = g;
}

// F and G of the incident (region -1) or exit (region -2) medium from the Jones-combined response
// (rcwa1d_conical_fields.hpp:195-210); kz is the normalised kzI or kzII of the region
__global__ void conical_region_fg_kernel(int B, int N, int M, int cnt, const double* __restrict__ zs, int region,
                                         double z_bottom, const double* __restrict__ k0, const zc* __restrict__ kz,
                                         const zc* __restrict__ resp, const zc* __restrict__ jones,
                                         const zc* __restrict__ w, const zc* __restrict__ v, zc* __restrict__ F,
                                         zc* __restrict__ G) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / n), j = (int)(r - (long long)col * n);
    const int order = j % N;
    const double z = zs[col], k = k0[b];
    const zc kzo = k * kz[b * N + order];  // physical kz of this order
    const zc rj = resp[b * n + j];
    zc a{0.0, 0.0}, bb{0.0, 0.0}, t{0.0, 0.0};
    if (region == -1) {
        if (order == M) {
            const zc kz0 = k * kz[b * N + M];
            const zc inc = zexp(zc{-kz0.im * z, kz0.re * z});  // exp(i kz z)
            a = (j < N ? jones[2 * b] : jones[2 * b + 1]) * inc;
        }
        if (!is_zero(rj)) bb = rj * zexp(zc{kzo.im * z, -kzo.re * z});  // exp(-i kz z)
    } else if (!is_zero(rj)) {
        const double dz = z - z_bottom;
        t = rj * zexp(zc{-kzo.im * dz, kzo.re * dz});  // exp(i kz (z - z_bottom))
    }
    F[idx] = w[b * n + j] * ((a + bb) + t);
    G[idx] = v[b * n + j] * ((-a + bb) - t);
}

// The six components from the (s, t) parts of F and G (rcwa1d_conical_fields.hpp:212-222): Ex, Ey, Hx, Hy, Hz
// into out[b][c][j][iz]; Ez before the 1/eps factor into ez (per sample N x cnt).
__global__ void conical_field_out_kernel(int B, int N, int cnt, int nz, const int* __restrict__ cols,
                                         const double* __restrict__ kx, const double* __restrict__ ky,
                                         const double* __restrict__ cs, const double* __restrict__ sn,
                                         const zc* __restrict__ F, const zc* __restrict__ G, zc* __restrict__ ez,
                                         zc* __restrict__ out) {
    const int n = 2 * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / N), j = (int)(r - (long long)col * N);
    const long long base = (b * cnt + col) * n;
    const zc f1 = F[base + j], f2 = F[base + N + j], g1 = G[base + j], g2 = G[base + N + j];
    const double c = cs[b * N + j], s = sn[b * N + j], kxj = kx[b * N + j], kyb = ky[b];
    const zc ex = (-s) * f1 + c * f2;
    const zc ey = c * f1 + s * f2;
    const zc hx = (-c) * g1 - s * g2;
    const zc hy = (-s) * g1 + c * g2;
    const zc hz = kyb * ex - kxj * ey;
    const zc e = kyb * hx - kxj * hy;
    const long long cstride = (long long)N * nz;
    zc* o = out + b * 6LL * N * nz + (long long)j * nz + cols[col];
    o[0 * cstride] = ex;
    o[1 * cstride] = ey;
    o[3 * cstride] = zc{hx.im, -hx.re};  // -i hx
    o[4 * cstride] = zc{hy.im, -hy.re};  // -i hy
    o[5 * cstride] = hz;
    ez[idx] = zc{-e.im, e.re};  // i (ky hx - kx hy)
}

// Ez (per sample N x cnt) into out[b][2][j][iz], times the scalar 1/eps when scale != null
__global__ void ez_out_kernel(int B, int N, int cnt, int nz, const int* __restrict__ cols, const zc* __restrict__ ez,
                              const zc* scale, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)N * cnt;
    if (idx >= (long long)B * per) return;
    const long long b = idx / per;
    const long long r = idx - b * per;
    const int col = (int)(r / N), j = (int)(r - (long long)col * N);
    const zc e = scale ? ez[idx] * *scale : ez[idx];
    out[b * 6LL * N * nz + 2LL * N * nz + (long long)j * nz + cols[col]] = e;
}

struct Region {
    bool analytic = true;
    zc *q = nullptr, *w = nullptr, *v = nullptr;  // analytic: B x 2N diagonals
    zc *W = nullptr, *V = nullptr;                // general: B x 2N x 2N
    zc* G = nullptr;                              // Schur samples: upper triangular square root
    int* schur = nullptr;                         // per-sample Schur flag (nullptr: none)
};

// One grating's flagged samples awaiting the Schur basis: H = P Q of the full 2N operator and Q, both in the
// chunk's layout and meaningful where the region's schur flag is set
struct SchurJob {
    int layer;
    zc* H;
    zc* Q;
};

// the flagged samples' matrices gathered from the per-grating buffers into one compact batch, and back:
// compact matrix t is sample map[t].y of grating job map[t].x
__global__ void gather_flagged_kernel(int total, long long per, const zc* const* __restrict__ src,
                                      const int2* __restrict__ map, zc* __restrict__ dst) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)total * per) return;
    const long long t = idx / per, e = idx - t * per;
    const int2 m = map[t];
    dst[idx] = src[m.x][(long long)m.y * per + e];
}
__global__ void scatter_flagged_kernel(int total, long long per, zc* const* __restrict__ dst,
                                       const int2* __restrict__ map, const zc* __restrict__ src) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)total * per) return;
    const long long t = idx / per, e = idx - t * per;
    const int2 m = map[t];
    dst[m.x][(long long)m.y * per + e] = src[idx];
}
__global__ void scatter_flagged_info_kernel(int total, int* const* __restrict__ dst, const int2* __restrict__ map,
                                            const int* __restrict__ src) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    dst[map[t].x][map[t].y] = src[t];
}

// The Schur basis of every flagged sample of every grating (rcwa1d_conical.hpp:466-502). A grating has a
// few such samples and each eigensolve of order 2N runs on one SM, so the gratings' H matrices are gathered
// into one batch and solved in one launch, side by side rather than one grating after another. Then per
// grating: the principal square root G of the Schur form T, W = Z, V from V G = Q Z, q = diag(G).
void conical_schur_modes(Batch& c, const std::vector<SchurJob>& jobs, std::vector<Region>& modes, int* eig_info,
                         int* schur_count, int eig_group) {
    const cudaStream_t st = c.st;
    DeviceScratch& mem = *c.mem;
    const int B = c.B, n = c.n, J = (int)jobs.size();
    const long long nn = c.nn(), nd = (long long)B * nn;
    std::vector<int> flags((size_t)J * B);
    for (int q = 0; q < J; ++q)
        RCWA_CUDA(cudaMemcpyAsync(flags.data() + (size_t)q * B, modes[jobs[q].layer + 1].schur, B * sizeof(int),
                                  cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    std::vector<int2> map;
    for (int q = 0; q < J; ++q)
        for (int b = 0; b < B; ++b)
            if (flags[(size_t)q * B + b]) map.push_back(make_int2(q, b));
    const int total = (int)map.size();
    std::vector<zc*> ptrs(3 * (size_t)J);  // H sources, Z and T destinations
    std::vector<int*> infos(J);
    for (int q = 0; q < J; ++q) {
        ptrs[q] = jobs[q].H;
        ptrs[J + q] = c.dense();
        ptrs[2 * J + q] = c.dense();
        infos[q] = mem.zeros<int>(B);
    }
    if (total > 0) {
        int2* dmap = mem.get<int2>(total);
        zc** dptrs = mem.get<zc*>(3 * (size_t)J);
        int** dinfos = mem.get<int*>(J);
        RCWA_CUDA(cudaMemcpyAsync(dmap, map.data(), total * sizeof(int2), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dptrs, ptrs.data(), ptrs.size() * sizeof(zc*), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dinfos, infos.data(), infos.size() * sizeof(int*), cudaMemcpyHostToDevice, st));
        const long long per = (long long)total * nn;
        zc* Hc = mem.get<zc>((size_t)per);
        LAUNCH(gather_flagged_kernel, nblocks(per), kTpb, st, total, nn, dptrs, dmap, Hc);
        zc* wc = mem.get<zc>((size_t)total * n);
        zc* Zc = mem.get<zc>((size_t)per);
        zc* Tc = mem.get<zc>((size_t)per);
        int* infoc = mem.zeros<int>(total);
        zc* wsc = mem.get<zc>((size_t)(eig_workspace_bytes(n, total) / sizeof(zc)) + 1);
        const int group = eig_group ? eig_group : eig_default_group(n, total);
        launch_eig(st, n, total, Hc, nn, wc, Zc, infoc, nullptr, wsc, 2.220446049250313e-16, 100, group, nullptr, 0, Tc);
        LAUNCH(scatter_flagged_kernel, nblocks(per), kTpb, st, total, nn, dptrs + J, dmap, Zc);
        LAUNCH(scatter_flagged_kernel, nblocks(per), kTpb, st, total, nn, dptrs + 2 * J, dmap, Tc);
        LAUNCH(scatter_flagged_info_kernel, nblocks(total), kTpb, st, total, dinfos, dmap, infoc);
        for (zc* ptr : {Hc, wc, Zc, Tc, wsc}) mem.free(ptr);
        mem.free(infoc);
        mem.free(dmap);
        mem.free(dptrs);
        mem.free(dinfos);
    }
    for (int q = 0; q < J; ++q) {
        Region& R = modes[jobs[q].layer + 1];
        zc* Z = ptrs[J + q];
        zc* Tm = ptrs[2 * J + q];
        LAUNCH(schur_info_kernel, nblocks(B), kTpb, st, B, infos[q], R.schur, eig_info, c.fail);
        R.G = c.dense();
        zc* gg = c.dense();
        LAUNCH(triangular_root_kernel, (unsigned)B, kSchurThreads, st, B, n, Tm, R.G, R.schur, c.fail);
        gemm(c, R.G, nn, R.G, nullptr, 1.0, 0.0, gg, R.schur, 0);
        LAUNCH(schur_root_check_kernel, (unsigned)B, kSchurThreads, st, B, n, Tm, gg, R.schur, c.fail);
        LAUNCH(copy_masked_kernel, nblocks(nd), kTpb, st, B, nn, Z, R.W, R.schur);
        gemm(c, jobs[q].Q, nn, Z, nullptr, 1.0, 0.0, R.V, R.schur, 0);
        LAUNCH(right_triangular_solve_kernel, nblocks((long long)B * n), kTpb, st, B, n, R.V, R.G, R.q, R.schur, c.fail);
        LAUNCH(add_flag_kernel, nblocks(B), kTpb, st, B, R.schur, schur_count);
        for (zc* ptr : {gg, Tm, Z, jobs[q].H, jobs[q].Q}) mem.free(ptr);
        mem.free(infos[q]);
    }
}

void interface_matching(Batch& c, const Region& up, const Region& low, zc*& tp, zc*& tm) {
    const long long nd = (long long)c.B * c.nn();
    tp = c.dense();
    tm = c.dense();
    if (low.analytic) {
        zc* inv_w = c.vec();
        zc* inv_v = c.vec();
        LAUNCH(conical_inv_wv_kernel, nblocks((long long)c.B * c.n), kTpb, c.st, c.B, c.n, low.w, low.v, inv_w, inv_v, c.fail);
        LAUNCH(conical_tp_tm_low_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, up.W, up.V, inv_w, inv_v, tp, tm);
        c.mem->free(inv_w);
        c.mem->free(inv_v);
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

// The field harmonics of one chunk (ConicalFieldSampler::sample, include/stablercwa/rcwa1d_conical_fields.hpp:163-236):
// depths grouped by region like field_depth_groups (rcwa_fields.hpp:253-279) over the layers of nonzero
// thickness, the Jones-combined amplitudes propagated mode by mode (or by exp(-k0 t G) for Schur samples),
// W F and V G for eigen-decomposed layers, the six components, Ez through [[eps]]^{-1} or 1/eps. Failed
// samples get NaN fields (the reference leaves their context unavailable).
struct ConicalCapture {
    std::vector<zc*> W, V;           // retained mode matrices of the grating layers (B x n x n)
    std::vector<DOp> r_below;        // reflection below each layer
    std::vector<zc*> a_plus, a_minus;  // B x 2 x n per layer, columns s and p input
    std::vector<const zc*> einv;     // [[eps]]^{-1} of grating layers (N x N, shared by the samples)
    std::vector<std::complex<double>> inv_eps;  // 1/eps of uniform layers
};

void sample_conical_fields(Batch& c, const FieldSpec& f, const std::vector<const rcwa_layer1d*>& layers,
                           const rcwa_stack1d& stack, int M, int p0, const std::vector<Region>& modes,
                           const ConicalCapture& cap, const zc* refl, const zc* trans, const double* kx, const double* ky,
                           const double* cs, const double* sn, const zc* kzI, const zc* kzII, const double* k0) {
    const cudaStream_t st = c.st;
    DeviceScratch& mem = *c.mem;
    const int B = c.B, n = c.n, N = n / 2, L = (int)layers.size(), nz = (int)f.zs.size();
    if (nz == 0) return;
    const long long nn = (long long)n * n, NN = (long long)N * N, nv = (long long)B * n;
    zc* out = f.out + (size_t)p0 * 6 * N * nz;
    RCWA_CUDA(cudaMemsetAsync(out, 0, (size_t)B * 6 * N * nz * sizeof(zc), st));
    // the normalised Jones vectors of this chunk
    std::vector<zc> hj(2 * (size_t)B);
    for (int b = 0; b < B; ++b) {
        if (f.jones.empty()) {
            hj[2 * b] = zc{1.0, 0.0};
            hj[2 * b + 1] = zc{0.0, 0.0};
        } else {
            const std::complex<double> e = f.jones[2 * (size_t)(p0 + b)], p = f.jones[2 * (size_t)(p0 + b) + 1];
            hj[2 * b] = zc{e.real(), e.imag()};
            hj[2 * b + 1] = zc{p.real(), p.imag()};
        }
    }
    zc* jones = mem.get<zc>(2 * (size_t)B);
    RCWA_CUDA(cudaMemcpyAsync(jones, hj.data(), 2 * (size_t)B * sizeof(zc), cudaMemcpyHostToDevice, st));
    std::vector<double> ztop(L), zbot(L);
    double z = 0.0;
    for (int j = 0; j < L; ++j) {
        ztop[j] = z;
        z += layers[j]->d;
        zbot[j] = z;
    }
    const double zb = z;
    std::vector<std::vector<int>> groups(L + 2);  // 0 incident side, 1 exit side, 2 + j layer j
    for (int iz = 0; iz < nz; ++iz) {
        const double zz = f.zs[iz];
        int g = zz < 0.0 ? 0 : 1;
        if (zz >= 0.0 && zz <= zb && L > 0)
            for (int j = 0; j < L; ++j)
                if (zz <= zbot[j] + 1e-12) {
                    g = 2 + j;
                    break;
                }
        groups[g].push_back(iz);
    }
    const std::complex<double> nI{stack.nI.re, stack.nI.im}, nII{stack.nII.re, stack.nII.im};
    zc* a = mem.get<zc>(nv);
    zc* bmv = mem.get<zc>(nv);
    zc* scale = mem.get<zc>(1);
    for (int g = 0; g < L + 2; ++g) {
        const std::vector<int>& cols = groups[g];
        if (cols.empty()) continue;
        const int cnt = (int)cols.size();
        const long long tot = (long long)B * n * cnt, totN = (long long)B * N * cnt;
        std::vector<double> local(cnt);
        for (int k = 0; k < cnt; ++k) local[k] = g >= 2 ? f.zs[cols[k]] - ztop[g - 2] : f.zs[cols[k]];
        double* d_z = mem.get<double>(cnt);
        int* d_cols = mem.get<int>(cnt);
        RCWA_CUDA(cudaMemcpyAsync(d_z, local.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_cols, cols.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, st));
        zc* F = mem.get<zc>(tot);
        zc* G = mem.get<zc>(tot);
        zc* ez = mem.get<zc>(totN);
        std::complex<double> ie{0.0, 0.0};
        const zc* einv = nullptr;
        if (g < 2) {
            const Region& m = g == 0 ? modes[0] : modes[L + 1];
            LAUNCH(jones_response_kernel, nblocks(nv), kTpb, st, B, n, g == 0 ? refl : trans, jones, a);
            LAUNCH(conical_region_fg_kernel, nblocks(tot), kTpb, st, B, N, M, cnt, d_z, g == 0 ? -1 : -2, zb, k0,
                   g == 0 ? kzI : kzII, a, jones, m.w, m.v, F, G);
            ie = 1.0 / (g == 0 ? nI * nI : nII * nII);
        } else {
            const int j = g - 2;
            const Region& m = modes[j + 1];
            const double d = layers[j]->d;
            LAUNCH(jones_response_kernel, nblocks(nv), kTpb, st, B, n, cap.a_plus[j], jones, a);
            LAUNCH(jones_response_kernel, nblocks(nv), kTpb, st, B, n, cap.a_minus[j], jones, bmv);
            zc* P = mem.get<zc>(tot);
            zc* Mm = mem.get<zc>(tot);
            LAUNCH(conical_layer_pm_kernel, nblocks(tot), kTpb, st, B, n, cnt, d_z, d, k0, a, bmv, m.q, m.G ? m.schur : nullptr,
                   P, Mm);
            if (m.G) {  // Schur samples: exp(-k0 t G) applied to the anchors (rcwa1d_conical_fields.hpp:109-160)
                zc* E = mem.get<zc>((size_t)B * nn);
                zc* work = mem.get<zc>(4 * (size_t)B * nn);
                for (int col = 0; col < cnt; ++col) {
                    const double from_top = std::max(0.0, std::min(d, local[col])), from_bottom = d - from_top;
                    for (int side = 0; side < 2; ++side) {
                        const double dist = side == 0 ? from_top : from_bottom;
                        if (dist != 0.0) batched_triangular_exp(c, n, m.G, k0, dist, E, work, m.schur);
                        LAUNCH(conical_schur_apply_kernel, warp_blocks(B), 128, st, B, n, dist != 0.0 ? E : nullptr,
                               side == 0 ? a : bmv, m.schur, side == 0 ? P : Mm, cnt, col);
                    }
                }
                mem.free(work);
                mem.free(E);
            }
            LAUNCH(conical_fg_kernel, nblocks(tot), kTpb, st, tot, n, cnt, P, Mm, m.analytic ? m.w : nullptr,
                   m.analytic ? m.v : nullptr, F, G);
            mem.free(P);
            mem.free(Mm);
            if (!m.analytic) {
                zc* F2 = mem.get<zc>(tot);
                zc* G2 = mem.get<zc>(tot);
                launch_zgemm(st, n, cnt, n, B, cap.W[j], n, nn, F, n, (long long)n * cnt, nullptr, 0, F2, n, (long long)n * cnt,
                             1.0, 0.0);
                launch_zgemm(st, n, cnt, n, B, cap.V[j], n, nn, G, n, (long long)n * cnt, nullptr, 0, G2, n, (long long)n * cnt,
                             1.0, 0.0);
                mem.free(F);
                mem.free(G);
                F = F2;
                G = G2;
                einv = cap.einv[j];
            } else {
                ie = cap.inv_eps[j];
            }
        }
        LAUNCH(conical_field_out_kernel, nblocks(totN), kTpb, st, B, N, cnt, nz, d_cols, kx, ky, cs, sn, F, G, ez, out);
        if (einv) {
            zc* ez2 = mem.get<zc>(totN);
            launch_zgemm(st, N, cnt, N, B, einv, N, 0, ez, N, (long long)N * cnt, nullptr, 0, ez2, N, (long long)N * cnt, 1.0,
                         0.0);
            LAUNCH(ez_out_kernel, nblocks(totN), kTpb, st, B, N, cnt, nz, d_cols, ez2, nullptr, out);
            RCWA_CUDA(stream_wait(st));
            mem.free(ez2);
        } else {
            const zc hs{ie.real(), ie.imag()};
            RCWA_CUDA(cudaMemcpyAsync(scale, &hs, sizeof(zc), cudaMemcpyHostToDevice, st));
            LAUNCH(ez_out_kernel, nblocks(totN), kTpb, st, B, N, cnt, nz, d_cols, ez, scale, out);
            RCWA_CUDA(stream_wait(st));  // the host values of this group end here
        }
        for (void* p : {(void*)F, (void*)G, (void*)ez, (void*)d_z, (void*)d_cols}) mem.free(p);
    }
    for (void* p : {(void*)a, (void*)bmv, (void*)scale, (void*)jones}) mem.free(p);
    LAUNCH(nan_fields_kernel, nblocks((long long)B * 6 * N * nz), kTpb, st, B, 6LL * N * nz, c.fail, out);
    (void)NN;
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
                          const Options& opt, const rcwa_result_conical& d_out, size_t chunk_bytes,
                          const FieldSpec* fields) {
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
        bool herm = false;       // real permittivities: the Hermitian eigensolver
        zc* einv_h = nullptr;    // Hermitian part of [[eps]]^{-1}
        zc *Lchol = nullptr, *Linv = nullptr, *LinvH = nullptr;  // [[1/eps]] = L L^H
        zc* pencil[4] = {nullptr, nullptr, nullptr, nullptr};    // constant parts of L^-1 B L^-H
    };
    std::vector<LayerData> ld(L);
    const bool try_herm = hermitian_path_enabled(opt);
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
        ld[k].herm = try_herm && real_profile(eps) && real_profile(inv);
        if (ld[k].herm) {
            make_hermitian_coefficients(st, ld[k].c_eps, M);
            make_hermitian_coefficients(st, c_inv, M);
            toeplitz_cholesky_inverse(st, c_inv, M, persist, layer_fail, ld[k].Lchol, ld[k].Linv, ld[k].LinvH);
        }
        zc* E = persist.get<zc>(NN);
        zc* Ci = persist.get<zc>(NN);
        LAUNCH(toeplitz_kernel, nblocks(NN), kTpb, st, M, ld[k].c_eps, E);
        LAUNCH(toeplitz_kernel, nblocks(NN), kTpb, st, M, c_inv, Ci);
        ld[k].einv = persist.get<zc>(NN);
        ld[k].cmat = persist.get<zc>(NN);
        launch_lu_solve(st, N, N, 1, E, NN, E, NN, RHS_IDENTITY, nullptr, NN, ld[k].einv, NN, layer_fail);
        launch_lu_solve(st, N, N, 1, Ci, NN, Ci, NN, RHS_IDENTITY, nullptr, NN, ld[k].cmat, NN, layer_fail);
        if (ld[k].herm) {
            ld[k].einv_h = persist.get<zc>(NN);
            LAUNCH(hermitian_part_kernel, nblocks(NN), kTpb, st, N, ld[k].einv, ld[k].einv_h);
            pencil_parts(st, persist, M, ld[k].einv_h, ld[k].Linv, ld[k].LinvH, ld[k].pencil);
        }
    }
    bool all_herm = !grating.empty();
    for (int k : grating) all_herm = all_herm && ld[k].herm;
    const bool reduced = reduced_seams_enabled();
    const int base_solves = 2 * static_cast<int>(grating.size());

    long long per_sample = 16LL * (nn * 16 + NN * 12 * (long long)grating.size() + (long long)n * 8 * (L + 2)) +
                           2 * eig_workspace_bytes(N, 1) * (long long)std::max<size_t>(1, grating.size());
    if (fields)  // retained W, V and reflections, amplitudes, one depth group's buffers
        per_sample += 16LL * (nn * 3 * (long long)grating.size() + (long long)n * 8 * L +
                              (long long)n * 6 * (long long)fields->zs.size());
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
            RCWA_CUDA(stream_wait(st));
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
                if (all_herm) {
                    // B C x = lambda x with C = [[1/eps]]^{-1} = (L L^H)^{-1} is the Hermitian-definite pencil
                    // (B, L L^H): L^{-1} B L^{-H} z = lambda z, x = L z; L^{-1} B L^{-H} from the layer's constant
                    // parts (kx_j = s cos(phi) - (j - M) lambda / period)
                    LAUNCH(pencil_combine_kernel, nblocks(ndN), kTpb, st, B, N, ld[k].pencil[0], ld[k].pencil[1],
                           ld[k].pencil[2], ld[k].pencil[3], P.s_cphi, P.wl, stack.period, AB + ndN);
                } else {
                    zc* Bm = mem.get<zc>(ndN);
                    LAUNCH(conical_b_kernel, nblocks(ndN), kTpb, st, B, N, ld[k].einv, kx, Bm);
                    launch_zgemm(st, N, N, N, B, Bm, N, NN, ld[k].cmat, N, 0, nullptr, 0, AB + ndN, N, NN, 1.0, 0.0);
                    mem.free(Bm);
                }
                LAUNCH(finite_check_kernel, nblocks(ndN), kTpb, st, B, NN, AB, c.fail);
                LAUNCH(finite_check_kernel, nblocks(ndN), kTpb, st, B, NN, AB + ndN, c.fail);
            }
            {
                zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(N, 2 * B * n_gr) / sizeof(zc)) + 1);
                if (all_herm)
                    launch_eig_herm(st, N, 2 * B * n_gr, ABall, NN, lamall, vecall, infoall, ws, opt.eps, opt.max_iter,
                                    opt.eig_group);
                else
                    launch_eig(st, N, 2 * B * n_gr, ABall, NN, lamall, vecall, infoall, nullptr, ws, opt.eps, opt.max_iter,
                               opt.eig_group);
                mem.free(ws);
            }
            std::vector<SchurJob> schur_jobs;
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
                if (all_herm) {
                    // x = L z and C x = L^{-H} z (the pencil's vectors; the region normalises each mode itself)
                    zc* x = mem.get<zc>(ndN);
                    launch_zgemm(st, N, N, N, B, ld[k].Lchol, N, 0, vec + ndN, N, NN, nullptr, 0, x, N, NN, 1.0, 0.0,
                                 nullptr, 1, TRI_A_LOWER);
                    launch_zgemm(st, N, N, N, B, ld[k].LinvH, N, 0, vec + ndN, N, NN, nullptr, 0, cw, N, NN, 1.0, 0.0,
                                 nullptr, 1, TRI_A_UPPER);
                    RCWA_CUDA(cudaMemcpyAsync(vec + ndN, x, ndN * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                    mem.free(x);
                } else {
                    launch_zgemm(st, N, N, N, B, ld[k].cmat, N, 0, vec + ndN, N, NN, nullptr, 0, cw, N, NN, 1.0, 0.0);
                }
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
                RCWA_CUDA(stream_wait(st));
                if (any) {
                    // Schur basis of the full 2N operator for the flagged samples (rcwa1d_conical.hpp:466-502): H here,
                    // its eigensolve below together with the other gratings' flagged samples
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
                    for (zc* ptr : {Pm, RE, RV}) mem.free(ptr);
                    schur_jobs.push_back(SchurJob{k, H, Qm});
                }
            }
            if (!schur_jobs.empty())
                conical_schur_modes(c, schur_jobs, modes, eig_info, schur_count, opt.eig_group);
            for (void* p : {(void*)ABall, (void*)lamall, (void*)vecall, (void*)infoall}) mem.free(p);
        }
        ConicalCapture cap;
        if (fields) {  // the interface above a layer consumes its W and V; the field sampler needs them after
            cap.W.assign(L, nullptr);
            cap.V.assign(L, nullptr);
            cap.r_below.assign(L, DOp{});
            cap.a_plus.assign(L, nullptr);
            cap.a_minus.assign(L, nullptr);
            cap.einv.assign(L, nullptr);
            cap.inv_eps.assign(L, {0.0, 0.0});
            for (int k = 0; k < L; ++k) {
                if (modes[k + 1].analytic) {
                    const rcwa_complex idx = layers[k]->homogeneous ? layers[k]->n : layers[k]->n_values[0];
                    const std::complex<double> nl{idx.re, idx.im};
                    cap.inv_eps[k] = 1.0 / (nl * nl);
                    continue;
                }
                cap.W[k] = c.dense();
                cap.V[k] = c.dense();
                RCWA_CUDA(cudaMemcpyAsync(cap.W[k], modes[k + 1].W, nd * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                RCWA_CUDA(cudaMemcpyAsync(cap.V[k], modes[k + 1].V, nd * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                cap.einv[k] = ld[k].einv;
            }
        }

        // ---- 2. bottom-up recursion at order 2N
        const int block_count = 2 * L + 1;
        std::vector<DOp> g(block_count);
        DOp r;
        for (int b = block_count - 1; b >= 1; --b) {
            const int j = b / 2;
            if (b % 2 == 0 && reduced && modes[j].analytic && !modes[j + 1].analytic && r.kind == KDense) {
                // a film over a grating
                Seam seam = analytic_over_dense_seam(c, modes[j + 1].W, modes[j + 1].V, modes[j].w, modes[j].v, r);
                mem.free(r.p);
                g[b] = seam.g;
                r = seam.r;
                continue;
            }
            if (b % 2 == 0 && reduced && !(modes[j].analytic && modes[j + 1].analytic)) {
                zc *tp, *tm;
                interface_matching(c, modes[j], modes[j + 1], tp, tm);
                Seam seam = reduced_seam(c, tp, tm, r);
                if (r.kind != KZero) mem.free(r.p);
                g[b] = seam.g;
                r = seam.r;
                continue;
            }
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
            if (fields) {  // the reflection seen below layer j's bottom (rcwa1d_conical.hpp:866)
                cap.r_below[j].kind = r.kind;
                if (r.kind != KZero) {
                    const size_t cnt = r.kind == KDense ? (size_t)nd : (size_t)nv;
                    cap.r_below[j].p = mem.get<zc>(cnt);
                    RCWA_CUDA(cudaMemcpyAsync(cap.r_below[j].p, r.p, cnt * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                }
            }
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
        zc* down = nullptr;
        if (reduced && modes[0].analytic && !modes[1].analytic && r.kind == KDense) {
            // With the incident medium's diagonal field factors w, v: w (d_a + u_a) = W (I + r) d_b and
            // v (d_a - u_a) = V (I - r) d_b, so (v W + w V + (v W - w V) r) d_b = 2 w v d_a -- one GEMM and one LU
            // with the two incident columns for the reference's three LUs with 2N right-hand sides and one with
            // two; R from whichever relation has the larger coefficient in each row, so no division by a
            // vanishing w or v (an order grazing in the incident medium).
            zc* Pm = c.dense();
            zc* Qm = c.dense();
            LAUNCH(analytic_pq_kernel, nblocks(nd), kTpb, st, B, n, modes[1].W, modes[1].V, modes[0].w, modes[0].v, Pm, Qm);
            gemm(c, Qm, nn, r.p, Pm, 1.0, 1.0, Pm);
            mem.free(Qm);
            zc* rhs = mem.get<zc>(2 * nv);
            LAUNCH(conical_top_rhs_kernel, nblocks(2 * nv), kTpb, st, B, n, N, M, modes[0].w, modes[0].v, rhs);
            down = solve(c, Pm, true, RHS_DENSE, rhs, 2);
            c.n_solve += 3;
            mem.free(Pm);
            mem.free(rhs);
            zc* t1 = mem.get<zc>(2 * nv);
            zc* t2 = mem.get<zc>(2 * nv);
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 2, r.p, down, down, t1, 1.0, 1.0);
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 2, r.p, down, down, t2, -1.0, 1.0);
            zc* X = mem.get<zc>(2 * nv);
            zc* Y = mem.get<zc>(2 * nv);
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 2, modes[1].W, t1, nullptr, X, 1.0, 0.0);
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 2, modes[1].V, t2, nullptr, Y, 1.0, 0.0);
            LAUNCH(conical_top_reflection_kernel, nblocks(2 * nv), kTpb, st, B, n, N, M, modes[0].w, modes[0].v, X, Y, rud);
            for (zc* ptr : {t1, t2, X, Y}) mem.free(ptr);
        } else {
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
            down = tdd;
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
        }
        zc* cur = down;
        zc* nxt = mem.get<zc>(2 * nv);
        zc* seam_t = mem.get<zc>(2 * nv);
        for (int b = 1; b < block_count; ++b) {
            const int j = b / 2;
            if (fields && b % 2 != 0) {  // amplitudes at the layer's top (rcwa1d_conical.hpp:921-925)
                cap.a_plus[j] = mem.get<zc>(2 * nv);
                RCWA_CUDA(cudaMemcpyAsync(cap.a_plus[j], cur, 2 * nv * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                if (pure_films)
                    LAUNCH(conical_clear_unexcited_kernel, nblocks(2 * nv), kTpb, st, 2 * nv, n, N, M, cap.a_plus[j]);
            }
            if (g[b].kind == KSeam)
                apply_seam(c, g[b], 2, cur, seam_t, nxt);
            else
                LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 2, (int)g[b].kind, g[b].p, g[b].alt, g[b].alt_flag,
                       cur, nxt);
            std::swap(cur, nxt);
            if (fields && b % 2 != 0) {  // the reflection below applied at the layer's bottom (:926-931)
                zc* bottom = cur;
                zc* cleared = nullptr;
                if (pure_films) {
                    cleared = mem.get<zc>(2 * nv);
                    RCWA_CUDA(cudaMemcpyAsync(cleared, cur, 2 * nv * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                    LAUNCH(conical_clear_unexcited_kernel, nblocks(2 * nv), kTpb, st, 2 * nv, n, N, M, cleared);
                    bottom = cleared;
                }
                cap.a_minus[j] = mem.get<zc>(2 * nv);
                LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 2, (int)cap.r_below[j].kind, cap.r_below[j].p, nullptr,
                       nullptr, bottom, cap.a_minus[j]);
                if (pure_films)
                    LAUNCH(conical_clear_unexcited_kernel, nblocks(2 * nv), kTpb, st, 2 * nv, n, N, M, cap.a_minus[j]);
                if (cleared) mem.free(cleared);
            }
        }

        // ---- 4. Jones matrices, efficiencies, status
        LAUNCH(conical_finalize_kernel, warp_blocks(B), 128, st, B, N, M, pure_films ? 1 : 0, rud, cur, flux_r, flux_t,
               c.fail, reinterpret_cast<zc*>(d_out.Jr) + (long long)p0 * N * 4,
               reinterpret_cast<zc*>(d_out.Jt) + (long long)p0 * N * 4, d_out.DEr + (long long)p0 * N * 4,
               d_out.DEt + (long long)p0 * N * 4);
        LAUNCH(conical_status_kernel, nblocks(B), kTpb, st, B, c.fail, eig_info, 2 * (int)grating.size(), schur_count,
               c.n_solve, c.n_lu, min_abs, P.ky, d_out.status ? d_out.status + p0 : nullptr,
               d_out.eig_info ? d_out.eig_info + p0 : nullptr, d_out.n_eig ? d_out.n_eig + p0 : nullptr,
               d_out.n_dense_solve ? d_out.n_dense_solve + p0 : nullptr, d_out.n_lu ? d_out.n_lu + p0 : nullptr,
               d_out.n_schur ? d_out.n_schur + p0 : nullptr,
               d_out.min_abs_lambda ? d_out.min_abs_lambda + p0 : nullptr,
               d_out.degenerate_mode_warning ? d_out.degenerate_mode_warning + p0 : nullptr);
        if (fields) {
            if (pure_films) {  // rcwa1d_conical.hpp:963-966
                LAUNCH(conical_clear_unexcited_kernel, nblocks(2 * nv), kTpb, st, 2 * nv, n, N, M, rud);
                LAUNCH(conical_clear_unexcited_kernel, nblocks(2 * nv), kTpb, st, 2 * nv, n, N, M, cur);
            }
            sample_conical_fields(c, *fields, layers, stack, M, p0, modes, cap, rud, cur, kx, P.ky, cs, sn, kzI, kzII, k0);
            if (fields->layer_info) {  // per original layer: 1 where it took the Schur basis
                const int LO = stack.n_layers;
                RCWA_CUDA(cudaMemset2DAsync(fields->layer_info + (size_t)p0 * LO, LO * sizeof(int), 0, LO * sizeof(int), B, st));
                for (int k = 0, e = 0; k < LO; ++k) {
                    if (!(stack.layers[k].d > 0.0)) continue;
                    const Region& m = modes[e + 1];
                    if (m.schur)
                        RCWA_CUDA(cudaMemcpy2DAsync(fields->layer_info + (size_t)p0 * LO + k, LO * sizeof(int), m.schur, sizeof(int),
                                                    sizeof(int), B, cudaMemcpyDeviceToDevice, st));
                    ++e;
                }
            }
        }
        mem.release();
    }
    int lf = 0;
    RCWA_CUDA(cudaMemcpyAsync(&lf, layer_fail, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
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
        if (fields && !fields->zs.empty()) {
            const size_t cf = (size_t)n_points * 6 * N * fields->zs.size();
            std::vector<double> fn(cf * 2, nan);
            RCWA_CUDA(cudaMemcpyAsync(fields->out, fn.data(), cf * sizeof(zc), cudaMemcpyHostToDevice, st));
            RCWA_CUDA(stream_wait(st));
        }
        RCWA_CUDA(stream_wait(st));
    }
}

}  // namespace rcwa_gb300
