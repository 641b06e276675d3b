// eig.cuh -- batched general complex eigensolver for sm_103a: unitary Hessenberg reduction plus
// shifted complex QR with deflation and eigenvector back-transformation (EISPACK CORTH + COMQR2,
// as restated by include/stablercwa/eig_qr.hpp).
//
// Mapping to GB300. The FP64 pipe (about 2 lane-operations per clock per SM) issues a warp
// instruction in the same time whether 1 or 32 lanes are active, so every FP64 instruction must carry
// 32 lanes of useful work. A group of G adjacent lanes owns one matrix and a warp holds 32/G
// matrices; the inherently serial steps of QR (forming a rotation, the shift, the deflation test)
// are computed by all lanes of a group from the same data, so each warp instruction forms the
// rotations of 32/G matrices at once, and the O(n^2)-per-sweep updates are split across the G lanes
// by row or by column. Groups synchronise with __syncwarp only; there is no block-wide barrier and
// no spin-wait. H, Z and the back-substitution vectors live in a per-matrix global workspace (the FP64
// pipe, not memory, bounds every phase: about one 16-byte load per 12 FP64 operations).
//
// Per-element arithmetic follows the reference: the same Householder vector scaling, rotation
// formulas (eig_qr.hpp:450-528), Wilkinson and exceptional shifts (:535-544, :1082-1086), the
// deflation test (:1063-1065), max_iter/info semantics (:1074-1077) and the back substitution with
// its coincident-eigenvalue floor and overflow control (:886-951). Reductions are lane trees instead
// of the reference's four-way partial sums, so results agree to rounding, not bit for bit.
#pragma once

#include <float.h>

#include "common.cuh"

namespace rcwa_gb300 {

struct Rot {
    double cr, ci, s;
};

// Per-matrix workspace layout in units of zc.
__host__ __device__ inline long long eig_workspace_elems(int n) { return 3LL * n * n + 4LL * n + 8; }

// Synchronisation and reductions of the threads that own one matrix: a group of G <= 32 lanes inside
// a warp (32/G matrices per warp, __syncwarp only), or a whole CTA of G = 64..256 threads for one
// matrix when the batch is too small to fill the GPU with warp groups (CTA barriers and a shared-
// memory reduction over the warps). Either way every member ends with the same reduced value.
template <int G, bool Block = (G > 32)>
struct Grp;

template <int G>
struct Grp<G, false> {
    unsigned mask;
    __device__ __forceinline__ Grp(double*, int*) : mask(group_mask<G>()) {}
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ double sum(double v) const { return group_sum<G>(v, mask); }
    __device__ __forceinline__ double max(double v) const { return group_max<G>(v, mask); }
    // smallest member index whose ok is set, or -1
    __device__ __forceinline__ int first(bool ok) const {
        const unsigned bits = __ballot_sync(mask, ok);
        const unsigned mine = G == 32 ? bits : (bits >> ((threadIdx.x & 31) & ~(G - 1))) & ((1u << G) - 1u);
        return mine ? __ffs(mine) - 1 : -1;
    }
};

template <int G>
struct Grp<G, true> {
    double* red;  // G / 32 doubles of shared memory
    int* ired;    // G / 32 ints of shared memory
    __device__ __forceinline__ Grp(double* r, int* ir) : red(r), ired(ir) {}
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ double sum(double v) const {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();  // earlier readers of red are done
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        double s = red[0];
#pragma unroll
        for (int w = 1; w < G / 32; ++w) s += red[w];
        return s;
    }
    __device__ __forceinline__ double max(double v) const {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        double s = red[0];
#pragma unroll
        for (int w = 1; w < G / 32; ++w) s = fmax(s, red[w]);
        return s;
    }
    __device__ __forceinline__ int first(bool ok) const {
        const unsigned bits = __ballot_sync(0xffffffffu, ok);
        const int f = bits ? (int)(threadIdx.x & ~31u) + __ffs(bits) - 1 : G;
        __syncthreads();
        if ((threadIdx.x & 31) == 0) ired[threadIdx.x >> 5] = f;
        __syncthreads();
        int m = ired[0];
#pragma unroll
        for (int w = 1; w < G / 32; ++w) m = min(m, ired[w]);
        return m < G ? m : -1;
    }
};

template <int G>
__device__ __forceinline__ int first_owned(int start, int g) {
    // smallest r >= start with r % G == g
    const int r0 = start + ((g - start) % G + G) % G;
    return r0;
}

// unit-modulus z/|z| and |z| with power-of-two pre-scaling (eig_qr.hpp:216-222)
__device__ __forceinline__ zc unit_phase(zc z, double& modulus) {
    const int e = bexp(fmax(fabs(z.re), fabs(z.im)));
    z = scale2(z, -e);
    const double r = hypot(z.re, z.im);
    modulus = ldexp(r, e);
    return zc{z.re / r, z.im / r};
}

// Rotation that zeroes the real subdiagonal below x (eig_qr.hpp:450-464).
__device__ __forceinline__ Rot make_rotation(zc x, double sub, zc& top) {
    double xr = x.re, xi = x.im;
    const double m = fmax(fmax(fabs(xr), fabs(xi)), fabs(sub));
    int e = 0;
    if (!(m > 1e-140 && m < 1e140)) {
        e = bexp(m);
        xr = ldexp(xr, -e);
        xi = ldexp(xi, -e);
        sub = ldexp(sub, -e);
    }
    const double nrm = sqrt(xr * xr + xi * xi + sub * sub);
    top = zc{e ? ldexp(nrm, e) : nrm, 0.0};
    return Rot{xr / nrm, xi / nrm, sub / nrm};
}

// Wilkinson shift from the trailing 2x2 block [a b; c d] (eig_qr.hpp:535-544)
__device__ __forceinline__ zc wilkinson_shift(zc a, zc b, double c, zc d) {
    const zc y = zc{(a.re - d.re) / 2.0, (a.im - d.im) / 2.0};
    const int e = bexp(fmax(fmax(abs1(b), fabs(c)), abs1(y)));
    const zc x = scale2(b, -e) * ldexp(c, -e);
    if (is_zero(x)) return d;
    const zc ys = scale2(y, -e);
    zc zz = zsqrt(ys * ys + x);
    if (ys.re * zz.re + ys.im * zz.im < 0.0) zz = -zz;
    return d - scale2(zdiv(x, ys + zz), e);
}

// Householder reduction of A to upper Hessenberg form H with the reflectors accumulated into Z, the
// entries below the subdiagonal cleared and the subdiagonal made real by a unitary diagonal similarity
// (CORTH and the preparation of COMQR2, eig_qr.hpp:231-439). For a Hermitian A the result is Hermitian
// tridiagonal up to rounding: real diagonal and real subdiagonal.
template <int G>
__device__ void reduce_to_hessenberg(int n, const zc* __restrict__ A, zc* __restrict__ H, zc* __restrict__ Z,
                                     zc* __restrict__ ort, zc* __restrict__ wk, const Grp<G>& grp, int g) {
    for (long long idx = g; idx < (long long)n * n; idx += G) H[idx] = A[idx];
    grp.sync();

    // ---------------- CORTH: Householder reduction to upper Hessenberg (eig_qr.hpp:231-272)
    // lane g owns rows r with r % G == g in every column.
    for (int m = 1; m < n - 1; ++m) {
        zc* x = H + (long long)(m - 1) * n;
        const int r0 = first_owned<G>(m, g);
        double sc = 0.0;
        for (int i = r0; i < n; i += G) sc += abs1(x[i]);
        sc = grp.sum(sc);
        if (sc == 0.0) {
            if (g == 0) ort[m] = zc{0.0, 0.0};
            grp.sync();
            continue;
        }
        double h = 0.0;
        for (int i = r0; i < n; i += G) {
            const zc u = zdivr(x[i], sc);
            ort[i] = u;
            h += norm2(u);
        }
        h = grp.sum(h);
        grp.sync();
        double gg = sqrt(h);
        zc om = ort[m];
        const double f = zabs(om);
        if (f == 0.0) {
            om = zc{gg, 0.0};
        } else {
            h += f * gg;
            gg /= f;
            om = om * (1.0 + gg);
        }
        grp.sync();
        if ((m % G) == g) {
            ort[m] = om;
            if (f == 0.0) x[m] = zc{sc, 0.0};
        }
        grp.sync();
        // left multiply P_m on columns n-1 .. m (rows >= m), accumulating wk = (P_m A)(:, m:) u
        for (int i = g; i < n; i += G) wk[i] = zc{0.0, 0.0};
        for (int j = n - 1; j >= m; --j) {
            zc* aj = H + (long long)j * n;
            double dr = 0.0, di = 0.0;
            for (int i = r0; i < n; i += G) {
                const zc u = ort[i], a = aj[i];
                dr += u.re * a.re + u.im * a.im;
                di += u.re * a.im - u.im * a.re;
            }
            dr = grp.sum(dr);
            di = grp.sum(di);
            const zc t = zc{-dr / h, -di / h};
            for (int i = r0; i < n; i += G) aj[i] = zfma(t, ort[i], aj[i]);
            const zc uj = ort[j];
            for (int i = g; i < n; i += G) wk[i] = zfma(uj, aj[i], wk[i]);
        }
        // right multiply: A(:, m:) -= (wk / h) u^H
        for (int i = g; i < n; i += G) wk[i] = zdivr(wk[i], h);
        for (int j = m; j < n; ++j) {
            zc* aj = H + (long long)j * n;
            const zc cu = -conj(ort[j]);
            for (int i = g; i < n; i += G) aj[i] = zfma(cu, wk[i], aj[i]);
        }
        grp.sync();
        if ((m % G) == g) {
            ort[m] = om * sc;
            x[m] = x[m] * (-gg);
        }
        grp.sync();
    }

    // ---------------- accumulate the reflectors into Z (eig_qr.hpp:354-373)
    for (long long idx = g; idx < (long long)n * n; idx += G) {
        const int c = (int)(idx / n), r = (int)(idx - (long long)c * n);
        Z[idx] = zc{r == c ? 1.0 : 0.0, 0.0};
    }
    grp.sync();
    for (int i = n - 2; i >= 1; --i) {
        const zc oi = ort[i];
        const zc hs = H[(long long)(i - 1) * n + i];
        grp.sync();  // every member has read ort[i] before the owner of row i overwrites it below
        if (is_zero(oi) || is_zero(hs)) continue;
        const int e = bexp(abs1(oi));
        const zc sub = scale2(hs, -e);
        const zc v0 = scale2(oi, -e);
        const double minus_h = sub.re * v0.re + sub.im * v0.im;
        const int r0 = first_owned<G>(i, g);
        for (int k = r0; k < n; k += G) ort[k] = k == i ? v0 : scale2(H[(long long)(i - 1) * n + k], -e);
        for (int j = i; j < n; ++j) {
            zc* zj = Z + (long long)j * n;
            double dr = 0.0, di = 0.0;
            for (int k = r0; k < n; k += G) {
                const zc u = ort[k], a = zj[k];
                dr += u.re * a.re + u.im * a.im;
                di += u.re * a.im - u.im * a.re;
            }
            dr = grp.sum(dr);
            di = grp.sum(di);
            const zc t = zc{dr / minus_h, di / minus_h};
            for (int k = r0; k < n; k += G) zj[k] = zfma(t, ort[k], zj[k]);
        }
    }
    grp.sync();

    // ---------------- clean Hessenberg form, real subdiagonal (eig_qr.hpp:420-439)
    for (int j = 0; j + 2 < n; ++j)
        for (int r = first_owned<G>(j + 2, g); r < n; r += G) H[(long long)j * n + r] = zc{0.0, 0.0};
    grp.sync();
    for (int i = 1; i < n; ++i) {
        const zc sub = H[(long long)(i - 1) * n + i];
        if (sub.im == 0.0) continue;
        double nrm = 0.0;
        const zc y = unit_phase(sub, nrm);
        const zc cy = conj(y);
        for (int j = first_owned<G>(i, g); j < n; j += G) {  // row i, by column owner
            zc* p = H + (long long)j * n + i;
            *p = cy * *p;
        }
        grp.sync();
        if ((i % G) == g) H[(long long)(i - 1) * n + i] = zc{nrm, 0.0};
        const int last = min(i + 1, n - 1);
        for (int r = g; r <= last; r += G) {
            zc* p = H + (long long)i * n + r;
            *p = y * *p;
        }
        for (int r = g; r < n; r += G) {
            zc* p = Z + (long long)i * n + r;
            *p = y * *p;
        }
        grp.sync();
    }

}

// With T != nullptr the call returns the Schur form instead of eigenvectors (keep_transform with
// vectors = false, eig_qr.hpp:1106-1122): V receives Z and T receives the upper triangular T with
// Z^H A Z = T.
template <int G>
__device__ void eig_one(int n, const zc* __restrict__ A, zc* __restrict__ W, zc* __restrict__ V,
                        int* __restrict__ info_out, int* __restrict__ sweeps_out, zc* __restrict__ ws, double eps,
                        int max_iter, zc* __restrict__ T = nullptr, double* red = nullptr, int* ired = nullptr) {
    const int g = threadIdx.x & (G - 1);
    const Grp<G> grp(red, ired);
    zc* __restrict__ H = ws;
    zc* __restrict__ Z = H + (long long)n * n;
    zc* __restrict__ X = Z + (long long)n * n;
    zc* __restrict__ ort = X + (long long)n * n;
    zc* __restrict__ wk = ort + n;
    double* __restrict__ rotd = reinterpret_cast<double*>(wk + n);  // 3n doubles (<= 2n zc)

    reduce_to_hessenberg<G>(n, A, H, Z, ort, wk, grp, g);

    // ---------------- shifted QR (eig_qr.hpp:1039-1096), full updates of H and Z
    zc t = zc{0.0, 0.0};
    int en = n - 1, its = 0, sweeps = 0, info = 0;
    while (en >= 0) {
        // deflation: largest l <= en with negligible h(l, l-1); lanes test G candidates at a time
        int l = 0;
        for (int base = en; base >= 1; base -= G) {
            const int cand = base - g;
            bool ok = false;
            if (cand >= 1) {
                const zc hsub = H[(long long)(cand - 1) * n + cand];
                const zc hd0 = H[(long long)(cand - 1) * n + cand - 1];
                const zc hd1 = H[(long long)cand * n + cand];
                ok = abs1(hsub) <= eps * (abs1(hd0) + abs1(hd1));
            }
            const int f = grp.first(ok);
            if (f >= 0) {
                l = base - f;
                break;
            }
        }
        if (l == en) {
            const zc hd = H[(long long)en * n + en];
            const zc wv = hd + t;
            grp.sync();
            if ((en % G) == g) H[(long long)en * n + en] = wv;
            if (g == 0) W[en] = wv;
            grp.sync();
            --en;
            its = 0;
            continue;
        }
        if (its == max_iter) {
            info = en + 1;
            break;
        }
        zc s;
        if (its == 10 || its == 20) {
            s = zc{fabs(H[(long long)(en - 1) * n + en].re) + (en >= 2 ? fabs(H[(long long)(en - 2) * n + en - 1].re) : 0.0), 0.0};
        } else {
            s = wilkinson_shift(H[(long long)(en - 1) * n + en - 1], H[(long long)en * n + en - 1],
                                H[(long long)(en - 1) * n + en].re, H[(long long)en * n + en]);
        }
        grp.sync();
        for (int r = g; r <= en; r += G) {
            zc* p = H + (long long)r * n + r;
            *p = *p - s;
        }
        t = t + s;
        ++its;
        ++sweeps;
        grp.sync();

        // (1) left multiply Q^H: rotation G_i from column i-1, applied to columns i..n-1 (rows i-1, i)
        for (int i = l + 1; i <= en; ++i) {
            zc* cprev = H + (long long)(i - 1) * n;
            zc top;
            const Rot q = make_rotation(cprev[i - 1], cprev[i].re, top);
            grp.sync();
            if (((i - 1) % G) == g) {
                cprev[i - 1] = top;
                cprev[i] = zc{0.0, 0.0};
            }
            if (g == 0) {
                rotd[3 * i] = q.cr;
                rotd[3 * i + 1] = q.ci;
                rotd[3 * i + 2] = q.s;
            }
            for (int c = first_owned<G>(i, g); c < n; c += G) {
                zc* col = H + (long long)c * n;
                const zc y = col[i - 1], z = col[i];
                col[i - 1] = zc{q.cr * y.re + q.ci * y.im + q.s * z.re, q.cr * y.im - q.ci * y.re + q.s * z.im};
                col[i] = zc{q.cr * z.re - q.ci * z.im - q.s * y.re, q.cr * z.im + q.ci * z.re - q.s * y.im};
            }
            grp.sync();
        }
        // (2) phase that makes r(en, en) real (eig_qr.hpp:588-596)
        const zc hee = H[(long long)en * n + en];
        const bool has_phase = hee.im != 0.0;
        zc phase = zc{1.0, 0.0};
        if (has_phase) {
            double nrm = 0.0;
            phase = unit_phase(hee, nrm);
            grp.sync();
            if ((en % G) == g) H[(long long)en * n + en] = zc{nrm, 0.0};
            const zc cp = conj(phase);
            for (int j = first_owned<G>(en + 1, g); j < n; j += G) {
                zc* p = H + (long long)j * n + en;
                *p = cp * *p;
            }
        }
        grp.sync();
        // (3) right multiply by Q on H rows 0..en and on all rows of Z (eig_qr.hpp:598-606)
        for (int r = g; r <= en; r += G) {
            int j = max(l + 1, r);
            if (j > en) continue;
            zc a = H[(long long)(j - 1) * n + r];
            for (; j <= en; ++j) {
                const double cr = rotd[3 * j], ci = rotd[3 * j + 1], sn = rotd[3 * j + 2];
                const zc b = H[(long long)j * n + r];
                H[(long long)(j - 1) * n + r] = zc{cr * a.re - ci * a.im + sn * b.re, cr * a.im + ci * a.re + sn * b.im};
                a = zc{cr * b.re + ci * b.im - sn * a.re, cr * b.im - ci * b.re - sn * a.im};
            }
            H[(long long)en * n + r] = has_phase ? phase * a : a;
        }
        for (int r = g; r < n; r += G) {
            zc a = Z[(long long)l * n + r];
            for (int j = l + 1; j <= en; ++j) {
                const double cr = rotd[3 * j], ci = rotd[3 * j + 1], sn = rotd[3 * j + 2];
                const zc b = Z[(long long)j * n + r];
                Z[(long long)(j - 1) * n + r] = zc{cr * a.re - ci * a.im + sn * b.re, cr * a.im + ci * a.re + sn * b.im};
                a = zc{cr * b.re + ci * b.im - sn * a.re, cr * b.im - ci * b.re - sn * a.im};
            }
            Z[(long long)en * n + r] = has_phase ? phase * a : a;
        }
        grp.sync();
    }
    if (g == 0) {
        *info_out = info;
        if (sweeps_out) *sweeps_out = sweeps;
    }
    if (info != 0) {
        // not converged: unconverged diagonal plus accumulated shift (eig_qr.hpp:1098-1103); no vectors
        for (int i = g; i <= en; i += G) W[i] = H[(long long)i * n + i] + t;
        return;
    }
    if (T) {
        // Schur form: T = H with the negligible subdiagonal cleared, Z as accumulated
        for (long long idx = g; idx < (long long)n * n; idx += G) {
            const int c = (int)(idx / n), r = (int)(idx - (long long)c * n);
            T[idx] = r > c ? zc{0.0, 0.0} : H[idx];
            V[idx] = Z[idx];
        }
        return;
    }

    // ---------------- eigenvectors of T by back substitution, times Z, normalised (eig_qr.hpp:886-961)
    double tn = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = g; i <= j; i += G) tn = fmax(tn, abs1(H[(long long)j * n + i]));
    tn = grp.max(tn);
    const double rel = fmax(eps, DBL_EPSILON);
    double tiny = rel * tn;
    if (tiny == 0.0) tiny = DBL_MIN;
    grp.sync();
    // the diagonal of H now holds the eigenvalues; read them from W (written above) for clarity
    const double kQuotientMax = 1e300;
    const double kShrink = 0x1p-512;
    for (int j = g; j < n; j += G) {
        zc* x = X + (long long)j * n;
        for (int k = 0; k < j; ++k) x[k] = H[(long long)j * n + k];
        x[j] = zc{1.0, 0.0};
        const zc wj = W[j];
        for (int i = j - 1; i >= 0; --i) {
            const zc wi = W[i];
            zc y = wj - wi;
            if (is_zero(y)) {
                y = zc{tiny, 0.0};
            } else {
                const double floor_value = rel * fmax(abs1(wj), abs1(wi));
                if (abs1(y) < floor_value) y = zc{floor_value, 0.0};
            }
            for (int pass = 0; pass < 3 && abs1(x[i]) > abs1(y) * kQuotientMax; ++pass)
                for (int k = 0; k <= j; ++k) x[k] = x[k] * kShrink;
            const zc xi = zdiv(x[i], y);
            x[i] = xi;
            const double tr = abs1(xi);
            zc xs = xi;
            if (tr != 0.0 && tr + 1.0 / tr <= tr) {
                for (int k = 0; k <= j; ++k) x[k] = zdivr(x[k], tr);
                xs = x[i];
            }
            const zc* ti = H + (long long)i * n;
            for (int k = 0; k < i; ++k) x[k] = zfma(xs, ti[k], x[k]);
        }
    }
    grp.sync();
    // V = Z X (X upper triangular), then each column scaled to unit 2-norm
    for (int j = 0; j < n; ++j) {
        const zc* xj = X + (long long)j * n;
        zc* vj = V + (long long)j * n;
        double big = 0.0;
        for (int r = g; r < n; r += G) {
            zc acc = zc{0.0, 0.0};
            for (int k = 0; k <= j; ++k) acc = zfma(xj[k], Z[(long long)k * n + r], acc);
            vj[r] = acc;
            big = fmax(big, fmax(fabs(acc.re), fabs(acc.im)));
        }
        big = grp.max(big);
        if (big == 0.0 || !isfinite(big)) continue;
        double ssq = 0.0;
        for (int r = g; r < n; r += G) {
            const zc u = zdivr(vj[r], big);
            ssq += norm2(u);
        }
        ssq = grp.sum(ssq);
        const double inv = 1.0 / sqrt(ssq);
        for (int r = g; r < n; r += G) vj[r] = zdivr(vj[r], big) * inv;
    }
}

// Eigen-decomposition of a Hermitian matrix: the reduction above gives a Hermitian tridiagonal matrix with
// real diagonal d and real subdiagonal e (entries of order eps |A| elsewhere are rounding and are dropped),
// whose eigenvalues and eigenvectors follow from the implicit symmetric QL iteration with Wilkinson's
// shift (Bowdler, Martin, Reinsch and Wilkinson, "The QR and QL algorithms for symmetric matrices",
// Numer. Math. 11, 1968). The plane rotations of a QL sweep act on the columns of Z, whose columns are
// then orthonormal eigenvectors; the eigenvalues are real. One lane per group runs the scalar sweep and
// records its rotations; then every lane applies them to its rows of Z, each row's entries read and written
// once per sweep. info = l + 1 when eigenvalue l does not converge within max_iter sweeps.
template <int G>
__device__ void herm_one(int n, const zc* __restrict__ A, zc* __restrict__ W, zc* __restrict__ V, int* __restrict__ info_out,
                         zc* __restrict__ ws, double eps, int max_iter, unsigned long long* rotations,
                         double* red = nullptr, int* ired = nullptr) {
    const int g = threadIdx.x & (G - 1);
    const Grp<G> grp(red, ired);
    zc* __restrict__ H = ws;
    zc* __restrict__ Z = H + (long long)n * n;
    zc* __restrict__ X = Z + (long long)n * n;
    zc* __restrict__ ort = X + (long long)n * n;
    zc* __restrict__ wk = ort + n;
    double* __restrict__ d = reinterpret_cast<double*>(X);  // n doubles
    double* __restrict__ e = d + n;                          // n doubles, e[i] couples i and i+1
    double* __restrict__ rc = e + n;                         // cosines of a sweep
    double* __restrict__ rs = rc + n;                        // sines of a sweep
    int* __restrict__ meta = reinterpret_cast<int*>(rs + n);  // [0] first rotation, [1] last, [2] state

    reduce_to_hessenberg<G>(n, A, H, Z, ort, wk, grp, g);
    for (int i = g; i < n; i += G) {
        d[i] = H[(long long)i * n + i].re;
        e[i] = i + 1 < n ? H[(long long)i * n + i + 1].re : 0.0;
    }
    grp.sync();

    int info = 0;
    unsigned long long applied = 0;
    for (int l = 0; l < n && info == 0; ++l) {
        for (int its = 0;; ++its) {
            if (g == 0) {
                // m: first index >= l whose coupling to m+1 is negligible (n-1 when there is none)
                int m = l;
                for (; m < n - 1; ++m) {
                    const double dd = fabs(d[m]) + fabs(d[m + 1]);
                    if (fabs(e[m]) <= eps * dd || fabs(e[m]) <= DBL_MIN) break;
                }
                int state = 0, first = m, last = m;  // state 0: sweep recorded, 1: converged, 2: no convergence
                if (m == l) {
                    state = 1;
                } else if (its >= max_iter) {
                    state = 2;
                } else {
                    // Wilkinson shift from the leading 2x2 block of [l, m]
                    double gg = (d[l + 1] - d[l]) / (2.0 * e[l]);
                    double r = hypot(gg, 1.0);
                    gg = d[m] - d[l] + e[l] / (gg + copysign(r, gg));
                    double s = 1.0, c = 1.0, p = 0.0;
                    bool split = false;
                    int i = m - 1;
                    for (; i >= l; --i) {
                        const double f = s * e[i], b = c * e[i];
                        r = hypot(f, gg);
                        e[i + 1] = r;
                        if (r == 0.0) {  // the sweep splits the block: recover and restart
                            d[i + 1] -= p;
                            e[m] = 0.0;
                            split = true;
                            break;
                        }
                        s = f / r;
                        c = gg / r;
                        gg = d[i + 1] - p;
                        r = (d[i] - gg) * s + 2.0 * c * b;
                        p = s * r;
                        d[i + 1] = gg + p;
                        gg = c * r - b;
                        rc[i] = c;
                        rs[i] = s;
                    }
                    if (!split) {
                        d[l] -= p;
                        e[l] = gg;
                        e[m] = 0.0;
                        first = l;
                    } else {
                        first = i + 1;
                    }
                    last = m - 1;
                }
                meta[0] = first;
                meta[1] = last;
                meta[2] = state;
            }
            grp.sync();
            const int first = meta[0], last = meta[1], state = meta[2];
            grp.sync();  // every member has read meta before the next sweep may rewrite it
            if (state == 1) break;
            if (state == 2) {
                info = l + 1;
                break;
            }
            // the recorded rotations i = last .. first mix columns i and i+1 of Z
            applied += (unsigned long long)(last - first + 1);
            for (int r = g; r < n; r += G) {
                zc cur = Z[(long long)(last + 1) * n + r];
                for (int i = last; i >= first; --i) {
                    const double c = rc[i], s = rs[i];
                    const zc zi = Z[(long long)i * n + r];
                    Z[(long long)(i + 1) * n + r] = zc{s * zi.re + c * cur.re, s * zi.im + c * cur.im};
                    cur = zc{c * zi.re - s * cur.re, c * zi.im - s * cur.im};
                }
                Z[(long long)first * n + r] = cur;
            }
            grp.sync();
        }
    }
    if (g == 0) {
        *info_out = info;
        if (rotations) atomicAdd(rotations, applied);
    }
    if (info != 0) {
        for (int i = g; i < n; i += G) W[i] = zc{d[i], 0.0};
        return;
    }
    for (int i = g; i < n; i += G) W[i] = zc{d[i], 0.0};
    for (long long idx = g; idx < (long long)n * n; idx += G) V[idx] = Z[idx];
}

template <int G>
__global__ void __launch_bounds__(128) herm_batch_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride,
                                                         zc* __restrict__ w, zc* __restrict__ v, int* __restrict__ info,
                                                         zc* __restrict__ ws, double eps, int max_iter,
                                                         unsigned long long* rotations, const int* __restrict__ only) {
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (gid >= batch) return;
    if (only && !only[gid]) return;
    herm_one<G>(n, a + gid * a_stride, w + gid * n, v + gid * (long long)n * n, info + gid, ws + gid * eig_workspace_elems(n),
                eps, max_iter, rotations);
}

template <int G>
__global__ void __launch_bounds__(G) herm_block_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride,
                                                       zc* __restrict__ w, zc* __restrict__ v, int* __restrict__ info,
                                                       zc* __restrict__ ws, double eps, int max_iter,
                                                       unsigned long long* rotations, const int* __restrict__ only) {
    __shared__ double red[G / 32];
    __shared__ int ired[G / 32];
    const long long gid = blockIdx.x;
    if (gid >= batch) return;
    if (only && !only[gid]) return;
    herm_one<G>(n, a + gid * a_stride, w + gid * n, v + gid * (long long)n * n, info + gid, ws + gid * eig_workspace_elems(n),
                eps, max_iter, rotations, red, ired);
}


// ---------------------------------------------------------------- the Hermitian solver in three launches
//
// The fused herm_one runs the scalar QL sweep on one lane of its group; on this GPU a warp FP64
// instruction costs the same pipe time whatever the number of active lanes, so that chain is paid at
// 1/G utilisation. The batched form splits the work: (1) the Householder tridiagonalisation with G lanes
// per matrix, Q written to the output and (d, e) kept; (2) the QL iteration with one lane per matrix, 32 matrices per warp
// instruction, which logs each sweep's rotations; (3) the rotations applied to Z with one thread per
// (matrix, row): within a sweep a row's entries are read and written once, with the running column kept
// in registers. A matrix whose log would overflow its capacity is flagged and redone by the fused kernel.
//
// Per-matrix workspace (eig_workspace_elems(n) zc): during the reduction [0, n^2) the matrix and its
// reflectors, [n^2, 2n^2) Q, d and e from 2n^2, w and tau from 3n^2. Then [0, n^2) holds d, e (2n doubles)
// and the sweep table (first, last) pairs, [n^2, 3n^2) the rotation log (c, s) with room for 2 n^2
// rotations, and the tail the counts and the overflow flag.

__host__ __device__ inline long long herm_log_capacity(int n) { return 2LL * n * n; }
__host__ __device__ inline long long herm_table_capacity(int n) { return 2LL * ((long long)n * n - n); }

// Householder tridiagonalisation of the Hermitian part of A: T = Q^H A Q with T real
// symmetric tridiagonal, Q = H_0 H_1 ... H_{n-2}, H_k = I - tau_k v_k v_k^H acting on indices k+1..n-1 and
// chosen so that H_k^H x = beta_k e_1 with beta_k real (Golub and Van Loan, Matrix Computations, 4th ed.,
// sections 5.1 and 8.3.1). The trailing block is updated as A - v w^H - w v^H with y = A v,
// w = tau y - (|tau|^2 (v^H y) / 2) v. Every lane owns whole rows (i % G) of the trailing block, so the
// product A v and the rank-2 update read and write consecutive rows across the group (coalesced); a column
// step needs three group barriers and one group reduction. Q = H_0 (H_1 (... (H_{n-2} I))) is then formed
// in V with every lane owning whole columns: H_k touches only rows and columns k+1.. of the partial product
// and each lane applies the reflectors in order to its own columns, so no barrier is needed there.
// Output: Q in V, d (n) and e (n-1, e_i = T(i+1, i)) in the third block of ws.
template <int G>
__device__ void herm_tridiag_one(int n, const zc* __restrict__ A0, zc* __restrict__ V, zc* __restrict__ ws, double* red,
                                 int* ired) {
    const int g = threadIdx.x & (G - 1);
    const Grp<G> grp(red, ired);
    zc* __restrict__ A = ws;
    double* __restrict__ d = reinterpret_cast<double*>(ws + 2LL * n * n);
    double* __restrict__ e = d + n;
    zc* __restrict__ ww = ws + 3LL * n * n;  // y, then w, of the current step (n)
    zc* __restrict__ taus = ww + n;          // tau_k (n)
    // the Hermitian part (A0 + A0^H) / 2, which is A0 itself (to the bit) for an exactly Hermitian input
    for (long long idx = g; idx < (long long)n * n; idx += G) {
        const int j = (int)(idx / n), i = (int)(idx - (long long)j * n);
        const zc a = A0[idx], b = A0[(long long)i * n + j];
        A[idx] = zc{0.5 * (a.re + b.re), 0.5 * (a.im - b.im)};
    }
    grp.sync();
    for (int k = 0; k + 1 < n; ++k) {
        zc* __restrict__ col = A + (long long)k * n;  // rows k+2.. become v_k (v_{k+1} = 1 implied)
        if (g == 0) d[k] = col[k].re;
        const zc alpha = col[k + 1];
        const int r2 = first_owned<G>(k + 2, g), r1 = first_owned<G>(k + 1, g);
        double xs = 0.0;
        for (int i = r2; i < n; i += G) xs += norm2(col[i]);
        xs = grp.sum(xs);
        zc tau{0.0, 0.0};
        double beta = alpha.re;
        if (xs != 0.0 || alpha.im != 0.0) {
            const double nrm = hypot(hypot(alpha.re, alpha.im), sqrt(xs));
            beta = alpha.re >= 0.0 ? -nrm : nrm;
            tau = zc{(beta - alpha.re) / beta, -alpha.im / beta};
            const zc scal = zinv(alpha - zc{beta, 0.0});
            for (int i = r2; i < n; i += G) col[i] = col[i] * scal;
        }
        if (g == 0) {
            e[k] = beta;
            taus[k] = tau;
        }
        if (is_zero(tau)) {
            grp.sync();
            continue;
        }
        grp.sync();  // v is complete
        // y_i = sum_j A(i, j) v_j over the trailing block, for owned rows i, four rows per pass with their
        // sums in registers (independent chains sharing each v_j)
        for (int i0 = r1; i0 < n; i0 += 4 * G) {
            zc acc[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * G;
                acc[u] = i < n ? A[(long long)(k + 1) * n + i] : zc{0.0, 0.0};
            }
            for (int j = k + 2; j < n; ++j) {
                const zc vj = col[j];
                const zc* aj = A + (long long)j * n;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * G;
                    if (i < n) acc[u] = zmac(aj[i], vj, acc[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * G;
                if (i < n) ww[i] = acc[u];
            }
        }
        double mr = 0.0;
        for (int i = r1; i < n; i += G) {
            const zc vi = i == k + 1 ? zc{1.0, 0.0} : col[i];
            mr += vi.re * ww[i].re + vi.im * ww[i].im;  // Re(conj(v_i) y_i); v^H y is real for Hermitian A
        }
        const double half = 0.5 * norm2(tau) * grp.sum(mr);
        for (int i = r1; i < n; i += G) {
            const zc vi = i == k + 1 ? zc{1.0, 0.0} : col[i];
            ww[i] = tau * ww[i] - zc{half * vi.re, half * vi.im};
        }
        grp.sync();  // w is complete
        // A(i, j) -= v_i conj(w_j) + w_i conj(v_j) over the trailing block, owned rows i, four rows per pass
        // with their v_i and w_i in registers
        for (int i0 = r1; i0 < n; i0 += 4 * G) {
            zc vi[4], wi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * G;
                vi[u] = i < n ? (i == k + 1 ? zc{1.0, 0.0} : col[i]) : zc{0.0, 0.0};
                wi[u] = i < n ? ww[i] : zc{0.0, 0.0};
            }
            for (int j = k + 1; j < n; ++j) {
                zc* aj = A + (long long)j * n;
                const zc cvj = j == k + 1 ? zc{1.0, 0.0} : conj(col[j]);
                const zc cwj = conj(ww[j]);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * G;
                    if (i < n) aj[i] = zfms(vi[u], cwj, zfms(wi[u], cvj, aj[i]));
                }
            }
        }
        grp.sync();  // the next column reads the updated block
    }
    if (g == 0) {
        d[n - 1] = A[(long long)(n - 1) * n + n - 1].re;
        e[n - 1] = 0.0;
    }
    for (int j = g; j < n; j += G) {
        zc* vj = V + (long long)j * n;
        for (int i = 0; i < n; ++i) vj[i] = zc{i == j ? 1.0 : 0.0, 0.0};
    }
    for (int k = n - 2; k >= 0; --k) {
        const zc tau = taus[k];
        if (is_zero(tau)) continue;
        const zc* vk = A + (long long)k * n;
        // two owned columns per pass: independent dot products sharing the loads of v_k
        for (int j = first_owned<G>(k + 1, g); j < n; j += 2 * G) {
            zc* v0 = V + (long long)j * n;
            zc* v1 = V + (long long)(j + G) * n;
            const bool two = j + G < n;
            zc t0 = v0[k + 1], t1 = two ? v1[k + 1] : zc{0.0, 0.0};
            for (int i = k + 2; i < n; ++i) {
                const zc x = vk[i];
                t0 = zmacc(x, v0[i], t0);
                if (two) t1 = zmacc(x, v1[i], t1);
            }
            const zc f0 = tau * t0, f1 = tau * t1;
            v0[k + 1] = v0[k + 1] - f0;
            if (two) v1[k + 1] = v1[k + 1] - f1;
            for (int i = k + 2; i < n; ++i) {
                const zc x = vk[i];
                v0[i] = zfms(x, f0, v0[i]);
                if (two) v1[i] = zfms(x, f1, v1[i]);
            }
        }
    }
}

template <int G>
__global__ void __launch_bounds__(128) herm_reduce_batch_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride,
                                                                zc* __restrict__ v, zc* __restrict__ ws) {
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (gid >= batch) return;
    herm_tridiag_one<G>(n, a + gid * a_stride, v + gid * (long long)n * n, ws + gid * eig_workspace_elems(n), nullptr, nullptr);
}
template <int G>
__global__ void __launch_bounds__(G) herm_reduce_block_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride,
                                                              zc* __restrict__ v, zc* __restrict__ ws) {
    __shared__ double red[G / 32];
    __shared__ int ired[G / 32];
    const long long gid = blockIdx.x;
    if (gid >= batch) return;
    herm_tridiag_one<G>(n, a + gid * a_stride, v + gid * (long long)n * n, ws + gid * eig_workspace_elems(n), red, ired);
}

// ---------------------------------------------------------------- (1') the blocked tridiagonalisation
//
// The same reduction T = Q^H A Q (same reflectors H_k = I - tau_k v_k v_k^H, same d and e) in panels of
// kHermNb columns, after LAPACK's zhetrd / zlatrd (Dongarra, Hammarling and Sorensen, "Block reduction of
// matrices to condensed forms for eigenvalue computations", J. Comput. Appl. Math. 27, 1989). Within a
// panel the trailing matrix is left as it was at the panel's start, A0; after i reflectors of the panel
// the reduced matrix is A0 - V W^H - W V^H with V = [v_0 .. v_{i-1}] and W = [w_0 .. w_{i-1}], so
//   * column j = k0 + i is first brought up to date: A(:, j) -= V W(j, :)^H + W V(j, :)^H (rows >= j);
//   * its reflector is formed as in herm_tridiag_one;
//   * y = A0 v - V (W^H v) - W (V^H v) (the product with A0 reads the trailing block once and writes
//     nothing), w = tau y - (|tau|^2 (v^H y) / 2) v.
// After the panel the whole trailing block takes A -= V W^H + W V^H as two complex products of inner
// dimension kHermNb (the tensor cores), launched by the host between panel launches.
// The reflectors are also kept for the back-transformation instead of forming Q: the panel's
// H_{k0} .. H_{k0+nb-1} = I - V T V^H with T upper triangular (LAPACK's zlarft, forward and columnwise:
// T(i, i) = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) (V^H v_i), and V^H v_i is the t2 the panel computes
// anyway), and the panel stores M = T V^H, so Q Y = Q_0 (Q_1 (.. (Q_last Y))) is applied as
// X -= V (M X), two products per panel.
//
// Per-matrix panel scratch (herm_panel_elems(n) zc): [V | W] (n x 2 nb, column-major), Bt = [W | V]^H
// (2 nb x n, column-major: the second operand of the trailing update), T (nb x nb), t2 (nb). The reflectors
// go to vall (n x n: column k is v_k, zero above row k + 1, one at k + 1) and M to mall (rows
// b nb .. b nb + nb - 1 of a pnb x n column-major matrix for panel b). d, e, tau and the work matrix keep
// herm_tridiag_one's places in ws.
constexpr int kHermNb = 32;
__host__ __device__ inline long long herm_panel_elems(int n) { return 4LL * kHermNb * n + kHermNb * kHermNb + kHermNb; }
__host__ __device__ inline int herm_panel_count(int n) { return n > 1 ? (n - 2) / kHermNb + 1 : 0; }

template <int G>
__device__ void herm_panel_one(int n, int k0, const zc* __restrict__ A0, zc* __restrict__ ws, zc* __restrict__ pan,
                               zc* __restrict__ vall, zc* __restrict__ mall, int pnb) {
    constexpr int nb = kHermNb;
    const int g = threadIdx.x & (G - 1);
    const Grp<G> grp(nullptr, nullptr);
    zc* __restrict__ A = ws;
    double* __restrict__ d = reinterpret_cast<double*>(ws + 2LL * n * n);
    double* __restrict__ e = d + n;
    zc* __restrict__ ww = ws + 3LL * n * n;  // y, then w, of the current column (n)
    zc* __restrict__ taus = ww + n;
    zc* __restrict__ VW = pan;                 // V(r, p) = VW[p n + r], W(r, p) = VW[(nb + p) n + r]
    zc* __restrict__ Bt = pan + 2LL * nb * n;  // Bt(q, r) = Bt[r 2 nb + q]
    zc* __restrict__ T = Bt + 2LL * nb * n;    // T(p, q) = T[q nb + p]
    zc* __restrict__ t2 = T + nb * nb;         // V^H v of the current column
    const int nbp = min(nb, n - 1 - k0);       // reflectors in this panel
    const zc one{1.0, 0.0}, zero{0.0, 0.0};
    if (k0 == 0) {  // the Hermitian part (A0 + A0^H) / 2, as herm_tridiag_one starts
        for (long long idx = g; idx < (long long)n * n; idx += G) {
            const int j = (int)(idx / n), i = (int)(idx - (long long)j * n);
            const zc a = A0[idx], b = A0[(long long)i * n + j];
            A[idx] = zc{0.5 * (a.re + b.re), 0.5 * (a.im - b.im)};
        }
    }
    for (int c = 0; c < 2 * nb; ++c)
        for (int r = g; r < n; r += G) VW[(long long)c * n + r] = zero;
    for (int idx = g; idx < nb * nb; idx += G) T[idx] = zero;
    grp.sync();
    for (int i = 0; i < nbp; ++i) {
        const int j = k0 + i;
        zc* __restrict__ col = A + (long long)j * n;
        if (i > 0) {  // column j as the panel's earlier reflectors leave it (rows >= j)
            for (int r = first_owned<G>(j, g); r < n; r += G) {
                zc acc = col[r];
                for (int p = 0; p < i; ++p) {
                    acc = zfms(VW[(long long)p * n + r], conj(VW[(long long)(nb + p) * n + j]), acc);
                    acc = zfms(VW[(long long)(nb + p) * n + r], conj(VW[(long long)p * n + j]), acc);
                }
                col[r] = acc;
            }
            grp.sync();
        }
        if (g == 0) d[j] = col[j].re;
        const zc alpha = col[j + 1];
        const int r2 = first_owned<G>(j + 2, g), r1 = first_owned<G>(j + 1, g);
        double xs = 0.0;
        for (int r = r2; r < n; r += G) xs += norm2(col[r]);
        xs = grp.sum(xs);
        zc tau{0.0, 0.0};
        double beta = alpha.re;
        if (xs != 0.0 || alpha.im != 0.0) {
            const double nrm = hypot(hypot(alpha.re, alpha.im), sqrt(xs));
            beta = alpha.re >= 0.0 ? -nrm : nrm;
            tau = zc{(beta - alpha.re) / beta, -alpha.im / beta};
            const zc scal = zinv(alpha - zc{beta, 0.0});
            for (int r = r2; r < n; r += G) col[r] = col[r] * scal;
        }
        if (g == 0) {
            e[j] = beta;
            taus[j] = tau;
        }
        zc* __restrict__ vcol = vall + (long long)j * n;
        for (int r = g; r < n; r += G) {
            const zc vr = r <= j ? zero : (r == j + 1 ? one : col[r]);
            vcol[r] = vr;
            VW[(long long)i * n + r] = vr;
        }
        if (is_zero(tau)) {  // H_j = I: w = 0 and T's column is zero (both already)
            grp.sync();
            continue;
        }
        grp.sync();  // v is complete
        // y = A0 v over the trailing block, owned rows, four rows per pass
        for (int i0 = r1; i0 < n; i0 += 4 * G) {
            zc acc[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = i0 + u * G;
                acc[u] = r < n ? A[(long long)(j + 1) * n + r] : zero;
            }
            for (int c = j + 2; c < n; ++c) {
                const zc vc = col[c];
                const zc* ac = A + (long long)c * n;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int r = i0 + u * G;
                    if (r < n) acc[u] = zmac(ac[r], vc, acc[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = i0 + u * G;
                if (r < n) ww[r] = acc[u];
            }
        }
        // y -= V (W^H v) + W (V^H v), one earlier reflector at a time
        for (int p = 0; p < i; ++p) {
            const zc* vp = VW + (long long)p * n;
            const zc* wp = VW + (long long)(nb + p) * n;
            zc a1 = zero, a2 = zero;
            for (int r = r1; r < n; r += G) {
                const zc vr = r == j + 1 ? one : col[r];
                a1 = zmacc(wp[r], vr, a1);
                a2 = zmacc(vp[r], vr, a2);
            }
            const zc s1{grp.sum(a1.re), grp.sum(a1.im)}, s2{grp.sum(a2.re), grp.sum(a2.im)};
            for (int r = r1; r < n; r += G) ww[r] = zfms(wp[r], s2, zfms(vp[r], s1, ww[r]));
            if (g == 0) t2[p] = s2;
        }
        double mr = 0.0;
        for (int r = r1; r < n; r += G) {
            const zc vr = r == j + 1 ? one : col[r];
            mr += vr.re * ww[r].re + vr.im * ww[r].im;  // Re(conj(v_r) y_r)
        }
        const double half = 0.5 * norm2(tau) * grp.sum(mr);
        zc* __restrict__ wi = VW + (long long)(nb + i) * n;
        for (int r = r1; r < n; r += G) {
            const zc vr = r == j + 1 ? one : col[r];
            wi[r] = tau * ww[r] - zc{half * vr.re, half * vr.im};
        }
        grp.sync();  // t2 is complete
        // T(0:i, i) = -tau T(0:i, 0:i) t2, T(i, i) = tau
        for (int p = g; p < i; p += G) {
            zc z = zero;
            for (int q = p; q < i; ++q) z = zmac(T[q * nb + p], t2[q], z);
            T[i * nb + p] = zc{0.0, 0.0} - tau * z;
        }
        if (g == 0) T[i * nb + i] = tau;
        grp.sync();  // w and T's column are complete
    }
    if (k0 + nbp == n - 1 && g == 0) {  // the last panel: the last diagonal entry takes its updates too
        zc a = A[(long long)(n - 1) * n + n - 1];
        for (int p = 0; p < nbp; ++p) {
            a = zfms(VW[(long long)p * n + n - 1], conj(VW[(long long)(nb + p) * n + n - 1]), a);
            a = zfms(VW[(long long)(nb + p) * n + n - 1], conj(VW[(long long)p * n + n - 1]), a);
        }
        d[n - 1] = a.re;
        e[n - 1] = 0.0;
    }
    // the trailing update's second operand, and M = T V^H (rows of V above k0 + 1 are zero)
    for (int r = g; r < n; r += G) {
        zc* bt = Bt + (long long)r * 2 * nb;
        for (int q = 0; q < nb; ++q) {
            bt[q] = conj(VW[(long long)(nb + q) * n + r]);
            bt[nb + q] = conj(VW[(long long)q * n + r]);
        }
    }
    const int b = k0 / nb;
    for (int r = first_owned<G>(k0 + 1, g); r < n; r += G) {
        zc* m = mall + (long long)r * pnb + b * nb;
        for (int p = 0; p < nbp; ++p) {
            zc acc = zero;
            for (int q = p; q < nbp; ++q) acc = zmac(T[q * nb + p], conj(VW[(long long)q * n + r]), acc);
            m[p] = acc;
        }
    }
}

template <int G>
__global__ void __launch_bounds__(128) herm_panel_batch_kernel(int n, int batch, int k0, const zc* __restrict__ a,
                                                               long long a_stride, zc* __restrict__ ws,
                                                               zc* __restrict__ pan, zc* __restrict__ vall,
                                                               zc* __restrict__ mall, int pnb) {
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (gid >= batch) return;
    herm_panel_one<G>(n, k0, a + gid * a_stride, ws + gid * eig_workspace_elems(n), pan + gid * herm_panel_elems(n),
                      vall + gid * (long long)n * n, mall + gid * (long long)pnb * n, pnb);
}

// round(x 2^62) for |x| <= 1, saturated to +-(2^62 - 1), with integer operations only: the QL kernel runs
// one thread per matrix and is bound by its warp's FP64 instructions, so converting each rotation's
// (c, s) to fixed point there must not add any.
__device__ inline long long herm_q62(double x) {
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);                          // x = +-m 2^(e - 1075)
    const long long m = (b & 0xfffffffffffffLL) | 0x10000000000000LL;  // 2^52 <= m < 2^53
    const int sh = 1013 - e;                                          // x 2^62 = m 2^-sh
    long long v;
    if (e >= 1023) v = 0x3fffffffffffffffLL;  // |x| >= 1 (c or s one ulp above 1 included)
    else if (sh <= 0) v = m << -sh;           // 2^-10 <= |x| < 1: exact
    else if (sh < 64) v = (m + (1LL << (sh - 1))) >> sh;
    else v = 0;
    return b < 0 ? -v : v;
}
// The fixed-point log entry of a rotation: S = herm_q62(s) and M = herm_q62(-c) as 31-bit limbs,
// (S >> 31, S & (2^31 - 1), M >> 31, M & (2^31 - 1)); the high limbs are signed, the low ones in [0, 2^31).
__device__ inline int4 herm_fixed_entry(double c, double s) {
    const long long sq = herm_q62(s), mq = herm_q62(-c);
    return make_int4((int)(sq >> 31), (int)(sq & 0x7fffffff), (int)(mq >> 31), (int)(mq & 0x7fffffff));
}

// (2) implicit symmetric QL with Wilkinson's shift on (d, e), one thread per matrix; rotations logged. The
// rotation chain is the whole cost, so with SMEM the thread's d and e live in shared memory (kHermQlThreads
// threads per CTA, 16 n bytes each) rather than in the workspace, whose loads would sit on the chain.
// FIXED logs each rotation as herm_fixed_entry(c, s), the fixed-point form herm_apply_real_kernel applies
// on the integer pipes; else as the doubles (c, s) herm_apply_kernel applies to the complex Q.
constexpr int kHermQlThreads = 32;
template <bool SMEM, bool FIXED>
__global__ void __launch_bounds__(128) herm_ql_kernel(int n, int batch, zc* __restrict__ w, int* __restrict__ info,
                                                      zc* __restrict__ ws, double eps, int max_iter,
                                                      unsigned long long* rotations) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= batch) return;
    zc* base = ws + gid * eig_workspace_elems(n);
    // d and e: this thread's column of the CTA's shared array (SMEM), else the H block of the workspace
    double* d;
    int sd;
    if constexpr (SMEM) {
        RCWA_DYN_SMEM(double, de_sm);
        d = de_sm + threadIdx.x;
        sd = kHermQlThreads;
    } else {
        d = reinterpret_cast<double*>(base);
        sd = 1;
    }
    double* e = d + (long long)n * sd;
    const double* src = reinterpret_cast<const double*>(base + 2LL * n * n);  // written by the reduction
    for (int k = 0; k < n; ++k) {
        d[(k) * sd] = src[k];
        e[(k) * sd] = src[n + k];
    }
    int2* table = reinterpret_cast<int2*>(reinterpret_cast<double*>(base) + 2 * n);
    double* log = reinterpret_cast<double*>(base + (long long)n * n);
    int* tail = reinterpret_cast<int*>(base + 3LL * n * n);  // [0] sweeps, [1] overflow
    const long long log_cap = herm_log_capacity(n), table_cap = herm_table_capacity(n);
    long long pos = 0, sweeps = 0;
    int status = 0, overflow = 0;
    for (int l = 0; l < n && status == 0 && !overflow; ++l) {
        for (int its = 0;; ++its) {
            // first m >= l with a negligible e[m]; four tests per pass, independent of one another
            int m = l;
            for (; m + 3 < n - 1; m += 4) {
                bool hit[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const double dd = fabs(d[(m + u) * sd]) + fabs(d[(m + u + 1) * sd]);
                    const double em = fabs(e[(m + u) * sd]);
                    hit[u] = em <= eps * dd || em <= DBL_MIN;
                }
                if (hit[0] || hit[1] || hit[2] || hit[3]) {
                    m += hit[0] ? 0 : hit[1] ? 1 : hit[2] ? 2 : 3;
                    goto found;
                }
            }
            for (; m < n - 1; ++m) {
                const double dd = fabs(d[(m) * sd]) + fabs(d[(m + 1) * sd]);
                if (fabs(e[(m) * sd]) <= eps * dd || fabs(e[(m) * sd]) <= DBL_MIN) break;
            }
        found:
            if (m == l) break;
            if (its >= max_iter) {
                status = l + 1;
                break;
            }
            if (pos + (m - l) > log_cap || sweeps + 1 > table_cap) {
                overflow = 1;
                break;
            }
            double gg = (d[(l + 1) * sd] - d[(l) * sd]) / (2.0 * e[(l) * sd]);
            double r = hypot(gg, 1.0);
            gg = d[(m) * sd] - d[(l) * sd] + e[(l) * sd] / (gg + copysign(r, gg));
            double s = 1.0, c = 1.0, p = 0.0;
            bool split = false;
            int i = m - 1;
            for (; i >= l; --i) {
                const double f = s * e[(i) * sd], b = c * e[(i) * sd];
                // r = |(f, g)| and 1/r from one reciprocal square root: the rotation chain is the whole cost
                // of this one-thread-per-matrix kernel; hypot and a division where f^2 + g^2 could under- or
                // overflow
                const double q = fma(f, f, gg * gg);
                double inv;
                if (q > 1e-290 && q < 1e290) {
                    inv = rsqrt(q);
                    r = q * inv;
                } else {
                    r = hypot(f, gg);
                    inv = r == 0.0 ? 0.0 : 1.0 / r;
                }
                e[(i + 1) * sd] = r;
                if (r == 0.0) {
                    d[(i + 1) * sd] -= p;
                    e[(m) * sd] = 0.0;
                    split = true;
                    break;
                }
                s = f * inv;
                c = gg * inv;
                gg = d[(i + 1) * sd] - p;
                r = (d[(i) * sd] - gg) * s + 2.0 * c * b;
                p = s * r;
                d[(i + 1) * sd] = gg + p;
                gg = c * r - b;
                if constexpr (FIXED) {
                    reinterpret_cast<int4*>(log)[pos] = herm_fixed_entry(c, s);
                } else {
                    log[2 * pos] = c;
                    log[2 * pos + 1] = s;
                }
                ++pos;
            }
            const int first = split ? i + 1 : l;
            if (!split) {
                d[(l) * sd] -= p;
                e[(l) * sd] = gg;
                e[(m) * sd] = 0.0;
            }
            if (m - 1 >= first) table[sweeps++] = make_int2(first, m - 1);
        }
    }
    tail[0] = (int)sweeps;
    tail[1] = overflow;
    info[gid] = overflow ? 0 : status;
    if (!overflow) {
        for (int k = 0; k < n; ++k) w[gid * n + k] = zc{d[(k) * sd], 0.0};
        if (rotations) atomicAdd(rotations, (unsigned long long)pos);
    }
}

// ---------------------------------------------------------------- (2') divide and conquer on (d, e)
//
// The eigenvectors Y of the real tridiagonal T = tridiag(e, d, e) by Cuppen's divide and conquer with the
// Gu-Eisenstat eigenvectors (Gu and Eisenstat, "A divide-and-conquer algorithm for the symmetric tridiagonal
// eigenproblem", SIAM J. Matrix Anal. Appl. 16, 1995; the merge and deflation steps of LAPACK's dstedc /
// dlaed0-dlaed4, restated), as the replacement of the QL iteration plus its rotations applied to a real
// identity: T is torn at the boundaries of 2^L leaves of at most kDcLeaf rows (T = diag(T_1, T_2) +
// |beta| u u^T with u = e_b + sign(beta) e_{b+1}, the two touching diagonal entries lowered by |beta|), each
// leaf is solved by the QL iteration with its rotations applied directly, and neighbouring blocks are merged
// level by level: with Q = diag(Q_1, Q_2), D their eigenvalues and z = Q^T u, the merged problem is
// D + rho z z^T. Entries with rho |z_i| below tol and pairs of nearly equal d_i (a rotation of theirs whose
// coupling is below tol) deflate; the k others give the secular equation 1 + rho sum z_i^2 / (d_i - lambda)
// = 0 with one root in each gap, found from the nearer pole (the differences d_i - lambda kept exact) by a
// two-pole rational model (Bunch, Nielsen and Sorensen 1978) safeguarded by bisection; z is then recomputed
// from the roots by Loewner's formula, so the eigenvectors (z_i / (d_i - lambda_j), normalised) are
// orthogonal to working accuracy, and Y's block takes Y U. Work per matrix: the products Y U (about m^3 for
// a merge of order m) and O(k^2) per merge for the roots, against 6 n flops for each of the ~n^2 QL
// rotations; the roots and the products are spread over the group's lanes instead of one thread's chain.
constexpr int kDcLeaf = 8;

// QL with Wilkinson shifts on a leaf: d[0..m), e[0..m-1), eigenvectors into the m x m block y (leading
// dimension ld), which it sets to the identity first. 0, or l + 1 when eigenvalue l did not converge.
__device__ inline int dc_leaf(int m, double* d, double* e, double* y, int ld, double eps, int max_iter) {
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) y[(long long)j * ld + i] = i == j ? 1.0 : 0.0;
    if (m <= 1) return 0;
    e[m - 1] = 0.0;
    for (int l = 0; l < m; ++l) {
        for (int its = 0;; ++its) {
            int mm = l;
            for (; mm < m - 1; ++mm) {
                const double dd = fabs(d[mm]) + fabs(d[mm + 1]);
                if (fabs(e[mm]) <= eps * dd || fabs(e[mm]) <= DBL_MIN) break;
            }
            if (mm == l) break;
            if (its >= max_iter) return l + 1;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = hypot(g, 1.0);
            g = d[mm] - d[l] + e[l] / (g + copysign(r, g));
            double s = 1.0, c = 1.0, p = 0.0;
            bool split = false;
            for (int i = mm - 1; i >= l; --i) {
                const double f = s * e[i], b = c * e[i];
                r = hypot(f, g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= p;
                    e[mm] = 0.0;
                    split = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
                double* yi = y + (long long)i * ld;
                double* yj = yi + ld;
                for (int q = 0; q < m; ++q) {
                    const double a0 = yi[q], a1 = yj[q];
                    yj[q] = s * a0 + c * a1;
                    yi[q] = c * a0 - s * a1;
                }
            }
            if (!split) {
                d[l] -= p;
                e[l] = g;
                e[mm] = 0.0;
            }
        }
    }
    return 0;
}

// Root j of 1 + sum_i w_i / (d_i - lambda) = 0 (d ascending, w_i = rho z_i^2 > 0): lambda in (d_j, d_{j+1}),
// or in (d_{k-1}, d_{k-1} + sum w) for j = k - 1. Returns the pole o it is measured from and tau = lambda -
// d_o; every d_i - lambda is then formed as (d_i - d_o) - tau.
__device__ inline void dc_root(int k, int j, const double* d, const double* w, double wsum, double eps, int& o,
                               double& tau) {
    double lo, hi;
    if (j < k - 1) {
        const double mid = 0.5 * (d[j + 1] - d[j]);
        double f = 1.0;
        for (int i = 0; i < k; ++i) f += w[i] / ((d[i] - d[j]) - mid);
        if (f > 0.0) {  // f rises through each gap: the root lies left of the middle
            o = j;
            lo = 0.0;
            hi = mid;
        } else {
            o = j + 1;
            lo = -mid;
            hi = 0.0;
        }
    } else {
        o = j;
        lo = 0.0;
        hi = wsum;
    }
    const double dl = d[j] - d[o], dr = j < k - 1 ? d[j + 1] - d[o] : 0.0;  // the two poles, shifted
    tau = 0.5 * (lo + hi);
    for (int it = 0; it < 200; ++it) {
        double psi = 0.0, dpsi = 0.0, phi = 0.0, dphi = 0.0;
        for (int i = 0; i < k; ++i) {
            const double r = 1.0 / ((d[i] - d[o]) - tau);
            const double v = w[i] * r;
            if (i <= j) {
                psi += v;
                dpsi += v * r;
            } else {
                phi += v;
                dphi += v * r;
            }
        }
        const double f = 1.0 + psi + phi;
        if (f == 0.0) return;
        if (f > 0.0) hi = tau;
        else lo = tau;
        if (hi - lo <= 2.0 * eps * fmax(fabs(lo), fabs(hi))) break;
        // two-pole model c + s1 / (DL - eta) + s2 / (DR - eta) = 0 (one pole for the last root)
        const double DL = dl - tau, s1 = DL * DL * dpsi;
        double next;
        if (j < k - 1) {
            const double DR = dr - tau, s2 = DR * DR * dphi;
            const double c = f - DL * dpsi - DR * dphi;
            const double B = c * (DL + DR) + s1 + s2, C = c * DL * DR + s1 * DR + s2 * DL;
            double eta;
            if (c == 0.0) {
                eta = C / B;
            } else {
                const double disc = sqrt(fmax(0.0, B * B - 4.0 * c * C));
                const double q = B >= 0.0 ? B + disc : B - disc;
                const double r1 = q / (2.0 * c), r2 = q != 0.0 ? 2.0 * C / q : r1;
                eta = (r1 > DL && r1 < DR) ? r1 : r2;
            }
            next = tau + eta;
        } else {
            const double c = f - DL * dpsi;
            next = c > 0.0 ? tau + DL + s1 / c : 0.5 * (lo + hi);
        }
        if (!(next > lo && next < hi)) next = 0.5 * (lo + hi);
        const bool done = fabs(next - tau) <= 4.0 * eps * fabs(next);
        tau = next;
        if (done) break;
    }
}

// an unsigned integer that orders finite doubles as their values (the sign-magnitude bits mapped to a
// monotone range), so comparisons run on the integer pipe
__device__ __forceinline__ unsigned long long dc_order_key(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Merge of the block [o, o + m) of y (its halves [o, o + n1) and [o + n1, o + m) already diagonalised, their
// eigenvalues in lam) across the tear beta. Scratch from sc: 8 m doubles, 3 m ints, 2 m^2 doubles.
template <int G>
__device__ void dc_merge(int n, int o, int n1, int m, double beta, double* y, double* lam, double* sc, double eps,
                         const Grp<G>& grp) {
    const int g = threadIdx.x & (G - 1);
    double* D = sc;            // unsorted eigenvalues of the halves
    double* Z = D + m;         // z
    double* ds = Z + m;        // sorted d, rotated by deflation
    double* zs = ds + m;       // sorted z
    double* dk = zs + m;       // the k secular poles
    double* wk = dk + m;       // rho z^2 of the poles
    double* tk = wk + m;       // roots: tau
    double* zh = tk + m;       // Loewner z
    int* perm = reinterpret_cast<int*>(zh + m);  // sorted position -> block column
    int* nd = perm + m;                          // secular pole -> sorted position
    int* ok = nd + m;                            // root -> its origin pole; [m] k, [m+1] rotations
    double* U = reinterpret_cast<double*>(ok + m + 2 + ((m + 2) & 1));  // k x k (column-major)
    double* tmp = U + (long long)m * m;          // m x k
    const double sg = beta >= 0.0 ? 1.0 : -1.0;
    double zz = 0.0;
    for (int i = g; i < m; i += G) {
        D[i] = lam[o + i];
        Z[i] = i < n1 ? y[(long long)(o + i) * n + o + n1 - 1] : sg * y[(long long)(o + i) * n + o + n1];
        zz += Z[i] * Z[i];
    }
    zz = grp.sum(zz);
    const double rho = fabs(beta) * zz, zscale = 1.0 / sqrt(zz);
    grp.sync();
    for (int i = g; i < m; i += G) {  // rank sort, ties by index; doubles compared as ordered integer keys
        const double di = D[i];
        const unsigned long long ki = dc_order_key(di);
        int r = 0;
        for (int q = 0; q < m; ++q) {
            const unsigned long long kq = dc_order_key(D[q]);
            r += (kq < ki || (kq == ki && q < i)) ? 1 : 0;
        }
        perm[r] = i;
        ds[r] = di;
        zs[r] = Z[i] * zscale;
    }
    grp.sync();
    double dmax = 0.0, zmax = 0.0;
    for (int i = g; i < m; i += G) {
        dmax = fmax(dmax, fabs(ds[i]));
        zmax = fmax(zmax, fabs(zs[i]));
    }
    dmax = grp.max(dmax);
    zmax = grp.max(zmax);
    const double tol = 8.0 * eps * fmax(dmax, rho * zmax);
    // deflation scan (one lane): small rho z_i, then nearly equal poles rotated together; the rotations are
    // kept (in tk, zh, nd as c, s, pair) and applied to y's columns afterwards in order
    if (g == 0) {
        int nrot = 0, pj = -1;
        for (int j = 0; j < m; ++j) {
            if (rho * fabs(zs[j]) <= tol) continue;  // deflated: eigenpair (ds[j], column perm[j])
            if (pj >= 0) {
                const double c0 = zs[j], s0 = zs[pj], t = hypot(c0, s0);
                const double c = c0 / t, s = -s0 / t;
                if (fabs((ds[j] - ds[pj]) * c * s) <= tol) {
                    zs[j] = t;
                    zs[pj] = 0.0;
                    const double dp = ds[pj] * c * c + ds[j] * s * s;
                    ds[j] = ds[pj] * s * s + ds[j] * c * c;
                    ds[pj] = dp;
                    tk[nrot] = c;
                    zh[nrot] = s;
                    ok[nrot] = pj;  // the pair (pj, j), stashed below
                    nd[nrot] = j;
                    ++nrot;
                }
            }
            pj = j;
        }
        ok[m] = nrot;
        // rotations are applied below before nd / ok are rebuilt: stash them in U's space
        for (int r = 0; r < nrot; ++r) {
            U[4 * r] = tk[r];
            U[4 * r + 1] = zh[r];
            U[4 * r + 2] = (double)ok[r];
            U[4 * r + 3] = (double)nd[r];
        }
        int q = 0;
        for (int j = 0; j < m; ++j)
            if (zs[j] != 0.0 && rho * fabs(zs[j]) > tol) nd[q++] = j;
        ok[m + 1] = q;
    }
    grp.sync();
    const int nrot = ok[m], k = ok[m + 1];
    // the deflation rotations on y's columns (rows of the block), in order: col_p' = c col_p + s col_j,
    // col_j' = c col_j - s col_p
    for (int r = 0; r < nrot; ++r) {
        const double c = U[4 * r], s = U[4 * r + 1];
        double* yp = y + (long long)(o + perm[(int)U[4 * r + 2]]) * n + o;
        double* yj = y + (long long)(o + perm[(int)U[4 * r + 3]]) * n + o;
        for (int i = g; i < m; i += G) {
            const double a = yp[i], b = yj[i];
            yp[i] = c * a + s * b;
            yj[i] = c * b - s * a;
        }
    }
    grp.sync();
    for (int i = g; i < k; i += G) {
        dk[i] = ds[nd[i]];
        wk[i] = rho * zs[nd[i]] * zs[nd[i]];
    }
    double wsum = 0.0;
    for (int i = g; i < k; i += G) wsum += rho * zs[nd[i]] * zs[nd[i]];
    wsum = grp.sum(wsum);
    grp.sync();
    for (int j = g; j < k; j += G) {
        int oj;
        double t;
        dc_root(k, j, dk, wk, wsum, eps, oj, t);
        ok[j] = oj;
        tk[j] = t;
    }
    grp.sync();
    // Loewner: zh_i^2 = prod_j (lambda_j - d_i) / (rho prod_{j != i} (d_j - d_i)), each root paired with a
    // neighbouring pole so the partial products stay near one
    for (int i = g; i < k; i += G) {
        double p = -((dk[i] - dk[ok[k - 1]]) - tk[k - 1]) / rho;  // lambda_{k-1} - d_i
        for (int j = 0; j < k - 1; ++j) {
            const double lj = -((dk[i] - dk[ok[j]]) - tk[j]);  // lambda_j - d_i
            p *= j < i ? lj / (dk[j] - dk[i]) : lj / (dk[j + 1] - dk[i]);
        }
        const double zi = zs[nd[i]];
        zh[i] = copysign(sqrt(fabs(p)), zi);
    }
    grp.sync();
    for (int j = g; j < k; j += G) {  // the merged eigenvectors, normalised
        double* u = U + (long long)j * k;
        double nrm = 0.0;
        for (int i = 0; i < k; ++i) {
            const double v = zh[i] / ((dk[i] - dk[ok[j]]) - tk[j]);
            u[i] = v;
            nrm += v * v;
        }
        const double inv = 1.0 / sqrt(nrm);
        for (int i = 0; i < k; ++i) u[i] *= inv;
    }
    grp.sync();
    // y's columns of the poles <- (those columns) U; lam <- roots and deflated values. tmp holds the k
    // columns (m rows, column-major), so the lanes' row accesses are consecutive
    for (int l = 0; l < k; ++l) {
        const double* yc = y + (long long)(o + perm[nd[l]]) * n + o;
        for (int i = g; i < m; i += G) tmp[(long long)l * m + i] = yc[i];
    }
    grp.sync();
    for (int j0 = 0; j0 < k; j0 += 4) {  // four output columns per pass over tmp
        const int nj = min(4, k - j0);
        const double* u0 = U + (long long)j0 * k;
        const double* u1 = nj > 1 ? u0 + k : u0;
        const double* u2 = nj > 2 ? u0 + 2 * k : u0;
        const double* u3 = nj > 3 ? u0 + 3 * k : u0;
        for (int i = g; i < m; i += G) {
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            for (int l = 0; l < k; ++l) {
                const double t = tmp[(long long)l * m + i];
                a0 = fma(t, u0[l], a0);
                a1 = fma(t, u1[l], a1);
                a2 = fma(t, u2[l], a2);
                a3 = fma(t, u3[l], a3);
            }
            y[(long long)(o + perm[nd[j0]]) * n + o + i] = a0;
            if (nj > 1) y[(long long)(o + perm[nd[j0 + 1]]) * n + o + i] = a1;
            if (nj > 2) y[(long long)(o + perm[nd[j0 + 2]]) * n + o + i] = a2;
            if (nj > 3) y[(long long)(o + perm[nd[j0 + 3]]) * n + o + i] = a3;
        }
    }
    for (int q = g; q < m; q += G) lam[o + perm[q]] = ds[q];  // deflated values (the poles' are replaced below)
    grp.sync();
    for (int j = g; j < k; j += G) lam[o + perm[nd[j]]] = dk[ok[j]] + tk[j];
    grp.sync();
}

// The whole solve for one matrix: d, e at ws + 2 n^2 (as the reductions leave them), eigenvalues to w,
// eigenvectors to y (n x n, column-major), info 0 or the failing leaf's QL index; scratch in ws [0, 2 n^2)
// doubles and ws + n^2 onwards.
template <int G>
__device__ void herm_dc_one(int n, zc* __restrict__ ws, double* __restrict__ y, zc* __restrict__ w, int* info, double eps,
                            int max_iter) {
    const int g = threadIdx.x & (G - 1);
    const Grp<G> grp(nullptr, nullptr);
    const double* src = reinterpret_cast<const double*>(ws + 2LL * n * n);
    double* d = reinterpret_cast<double*>(ws + 3LL * n * n + 2LL * n);  // own copies: d, e, lam, the tears
    double* e = d + n;
    double* lam = e + n;
    double* sc = reinterpret_cast<double*>(ws);  // merge scratch: 2 n^2 + 11 n doubles fit in [0, 2 n^2 + ...)
    int L = 0;
    while ((n >> L) > kDcLeaf) ++L;
    const int leaves = 1 << L;
    for (int i = g; i < n; i += G) {
        d[i] = src[i];
        e[i] = i < n - 1 ? src[n + i] : 0.0;
    }
    grp.sync();
    // tears at every leaf boundary b (between rows b - 1 and b); beta stays in e[b - 1]
    if (g == 0)
        for (int q = 1; q < leaves; ++q) {
            const int b = (int)(((long long)q * n) >> L);
            const double a = fabs(e[b - 1]);
            d[b - 1] -= a;
            d[b] -= a;
        }
    grp.sync();
    int bad = 0;
    for (int q = g; q < leaves; q += G) {
        const int b0 = (int)(((long long)q * n) >> L), b1 = (int)(((long long)(q + 1) * n) >> L);
        double* dl = lam + b0;
        double el[kDcLeaf + 1];
        for (int i = b0; i < b1; ++i) {
            dl[i - b0] = d[i];
            el[i - b0] = i < b1 - 1 ? e[i] : 0.0;
        }
        const int r = dc_leaf(b1 - b0, dl, el, y + (long long)b0 * n + b0, n, eps, max_iter);
        if (r && !bad) bad = b0 + r;
    }
    // zero the off-diagonal blocks of y
    for (long long idx = g; idx < (long long)n * n; idx += G) {
        const int col = (int)(idx / n), row = (int)(idx - (long long)col * n);
        const int qc = (int)((((long long)col + 1) << L) - 1) / n, qr = (int)((((long long)row + 1) << L) - 1) / n;
        if (qc != qr) y[idx] = 0.0;
    }
    bad = (int)grp.max((double)bad);
    grp.sync();
    for (int lev = L - 1; lev >= 0; --lev) {
        const int blocks = 1 << lev;
        for (int q = 0; q < blocks; ++q) {
            const int o = (int)(((long long)q * n) >> lev), mid = (int)(((long long)(2 * q + 1) * n) >> (lev + 1));
            const int end = (int)(((long long)(q + 1) * n) >> lev);
            const double beta = e[mid - 1];
            if (beta != 0.0) dc_merge<G>(n, o, mid - o, end - o, beta, y, lam, sc, eps, grp);
        }
    }
    for (int i = g; i < n; i += G) w[i] = zc{lam[i], 0.0};
    if (g == 0) {
        *info = bad;
        int* tail = reinterpret_cast<int*>(ws + 3LL * n * n);  // no rotation log: nothing overflowed
        tail[0] = 0;
        tail[1] = 0;
    }
}

template <int G>
__global__ void __launch_bounds__(128) herm_dc_batch_kernel(int n, int batch, zc* __restrict__ ws, double* __restrict__ y,
                                                            zc* __restrict__ w, int* __restrict__ info, double eps,
                                                            int max_iter) {
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (gid >= batch) return;
    herm_dc_one<G>(n, ws + gid * eig_workspace_elems(n), y + gid * (long long)n * n, w + gid * n, info + gid, eps,
                   max_iter);
}

// (3) the logged rotations applied to Z (in v), thread per (matrix, row)
static __global__ void __launch_bounds__(128) herm_apply_kernel(int n, int batch, zc* __restrict__ v, const zc* __restrict__ ws,
                                                         const int* __restrict__ info) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)batch * n) return;
    const long long gid = tid / n;
    const int r = (int)(tid - gid * n);
    const zc* base = ws + gid * eig_workspace_elems(n);
    const int* tail = reinterpret_cast<const int*>(base + 3LL * n * n);
    if (tail[1] || info[gid]) return;  // overflow (redone by the fused kernel) or not converged
    const int2* table = reinterpret_cast<const int2*>(reinterpret_cast<const double*>(base) + 2 * n);
    const double* log = reinterpret_cast<const double*>(base + (long long)n * n);
    zc* z = v + gid * (long long)n * n + r;
    const int sweeps = tail[0];
    long long pos = 0;
    for (int k = 0; k < sweeps; ++k) {
        const int2 fl = table[k];
        zc cur = z[(long long)(fl.y + 1) * n];
        for (int i = fl.y; i >= fl.x; --i, ++pos) {
            const double c = log[2 * pos], s = log[2 * pos + 1];
            const zc zi = z[(long long)i * n];
            z[(long long)(i + 1) * n] = zc{s * zi.re + c * cur.re, s * zi.im + c * cur.im};
            cur = zc{c * zi.re - s * cur.re, c * zi.im - s * cur.im};
        }
        z[(long long)fl.x * n] = cur;
    }
}

// (3, real form) the logged rotations applied to a real identity instead of to the complex Q: Y = R_1 R_2 ...
// is real orthogonal and the eigenvectors are Q Y, a complex-by-real product. One thread per (matrix, row),
// kHermRows rows per CTA, each row kept in shared memory (row t of the CTA at element i * kHermRows + t)
// until every sweep has passed, so Y meets HBM only once. A matrix that overflowed its log or did not
// converge gets Y = I.
//
// The arithmetic is 64-bit fixed point on the integer pipes, not FP64: this GPU issues FP64 at 2 lanes a
// cycle per SM and 32-bit integer multiply-adds at 64, and every quantity here lies in [-1, 1] (the rotation
// coefficients, and the entries of an orthogonal Y). Y is held as Y = round(y 2^60) and the coefficients as
// S = round(s 2^62), M = round(-c 2^62), all three split into 31-bit limbs (X = X1 2^31 + X0, X0 in
// [0, 2^31)). A product of coefficient and entry in Y's scale, C Y 2^-62, is then
//   R(C, Y) = C1 Y1 + (C1 Y0 + C0 Y1) 2^-31   (+ C0 Y0 2^-62, below one unit, dropped)
// -- three 32 x 32 -> 64 multiply-adds -- and the rotation y_{i+1} <- s y_i + c y_{i+1}, y_i <- c y_i -
// s y_{i+1} is
//   y_{i+1} = R(S, y_i) - R(M, y_{i+1}),   y_i = -R(M, y_i) - R(S, y_{i+1}),
// six limb products an output (signs carried by the entry limbs): the two high-by-high terms added whole, the
// four cross terms gathered in one 64-bit accumulator and rounded to nearest once. Each output is the difference of two products that drop
// the same kind of term, so those errors (under a unit each) cancel on average instead of drifting over the
// ~2 n rotations an entry takes. Resolution 2^-60 absolute against FP64's 2^-53 relative: as accurate for
// entries near 1/sqrt(n), more so near 1. No intermediate overflows: |Y| <= 2^60 and s^2 + c^2 = 1 keep the
// accumulator below 2^63. The entries leave as doubles.
//
// A rotation then costs tens of cycles, less than a load of its log entry from L2 or HBM, so the log is
// streamed through shared memory: the CTA's one warp holds 32 entries in stage[b], has the next 32 in flight
// in registers (one entry a lane, loaded 32 rotations before use) and swaps at each chunk boundary. The
// reads run to the log's capacity at most, inside the workspace; entries past the last rotation are never
// used.
constexpr int kHermRows = 32;
constexpr int kHermApplyStaticSmem = 2 * kHermRows * (int)sizeof(int4);  // stage
static __global__ void __launch_bounds__(kHermRows) herm_apply_real_kernel(int n, int batch, double* __restrict__ y_out,
                                                                           const zc* __restrict__ ws,
                                                                           const int* __restrict__ info) {
    RCWA_DYN_SMEM(long long, yfix_sm);
    const long long gid = blockIdx.x;
    const int t = threadIdx.x;
    const int r = blockIdx.y * kHermRows + t;  // lanes past the last row stage log entries and rotate zeros
    if (gid >= batch) return;
    long long* y = yfix_sm + t;
    const long long one = 1LL << 60;
    for (int i = 0; i < n; ++i) y[i * kHermRows] = i == r ? one : 0;
    const zc* base = ws + gid * eig_workspace_elems(n);
    const int* tail = reinterpret_cast<const int*>(base + 3LL * n * n);
    __shared__ int4 stage[2][kHermRows];
    const bool applied = !tail[1] && !info[gid];
    if (applied) {
        const int2* table = reinterpret_cast<const int2*>(reinterpret_cast<const double*>(base) + 2 * n);
        const int4* log = reinterpret_cast<const int4*>(base + (long long)n * n);  // (S1, S0, M1, M0)
        const long long cap = herm_log_capacity(n);
        const int sweeps = tail[0];
        const int4 zero4 = make_int4(0, 0, 0, 0);
        // entries [cb, cb + 32) in stage[b], [cb + 32, cb + 64) in next
        long long cb = 0;
        int b = 0;
        stage[0][t] = t < cap ? log[t] : zero4;
        int4 next = kHermRows + t < cap ? log[kHermRows + t] : zero4;
        __syncwarp();
        long long pos = 0;
        for (int k = 0; k < sweeps; ++k) {
            const int2 fl = table[k];
            long long cur = y[(fl.y + 1) * kHermRows];
            for (int i = fl.y; i >= fl.x; --i, ++pos) {
                if (pos == cb + kHermRows) {  // the next chunk: stage it, start loading the one after
                    stage[b ^ 1][t] = next;
                    b ^= 1;
                    cb += kHermRows;
                    const long long q = cb + kHermRows + t;
                    next = q < cap ? log[q] : zero4;
                    __syncwarp();
                }
                const int4 e = stage[b][pos - cb];
                const long long yi = y[i * kHermRows];
                const int a1 = (int)(yi >> 31), a0 = (int)(yi & 0x7fffffff);
                const int b1 = (int)(cur >> 31), b0 = (int)(cur & 0x7fffffff);
                // the y_i terms first: they do not wait for the previous rotation's output
                long long u1 = (long long)e.x * a0 + (long long)e.y * a1 + (1LL << 30);
                long long u2 = (long long)e.z * -a0 + (long long)e.w * -a1 + (1LL << 30);
                const long long v1 = (long long)e.x * a1, v2 = (long long)e.z * -a1;
                u1 += (long long)e.z * -b0 + (long long)e.w * -b1;
                u2 += (long long)e.x * -b0 + (long long)e.y * -b1;
                y[(i + 1) * kHermRows] = v1 + (long long)e.z * -b1 + (u1 >> 31);
                cur = v2 + (long long)e.x * -b1 + (u2 >> 31);
            }
            y[fl.x * kHermRows] = cur;
        }
    }
    if (r >= n) return;
    double* yo = y_out + gid * (long long)n * n + r;
    for (int i = 0; i < n; ++i) yo[(long long)i * n] = (double)y[i * kHermRows] * 0x1p-60;
}

// 1 where the matrix overflowed its log (the fused kernel redoes it)
static __global__ void herm_overflow_kernel(int n, int batch, const zc* __restrict__ ws, int* __restrict__ flag) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= batch) return;
    const int* tail = reinterpret_cast<const int*>(ws + gid * eig_workspace_elems(n) + 3LL * n * n);
    flag[gid] = tail[1];
}

// One group of G <= 32 lanes per matrix; matrices at a_stride / w_stride / v_stride elements apart.
template <int G>
__global__ void __launch_bounds__(128) eig_batch_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride,
                                                        zc* __restrict__ w, zc* __restrict__ v, int* __restrict__ info,
                                                        int* __restrict__ sweeps, zc* __restrict__ ws, double eps,
                                                        int max_iter, const int* __restrict__ skip, int skip_value,
                                                        zc* __restrict__ t_out) {
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (gid >= batch) return;
    if (skip && skip[gid] == skip_value) return;
    eig_one<G>(n, a + gid * a_stride, w + gid * n, v + gid * (long long)n * n, info + gid, sweeps ? sweeps + gid : nullptr,
               ws + gid * eig_workspace_elems(n), eps, max_iter, t_out ? t_out + gid * (long long)n * n : nullptr);
}

// One CTA of G = 64..256 threads per matrix (grid = batch), for batches too small to fill the GPU
// with warp groups.
template <int G>
__global__ void __launch_bounds__(G) eig_block_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride,
                                                      zc* __restrict__ w, zc* __restrict__ v, int* __restrict__ info,
                                                      int* __restrict__ sweeps, zc* __restrict__ ws, double eps,
                                                      int max_iter, const int* __restrict__ skip, int skip_value,
                                                      zc* __restrict__ t_out) {
    static_assert(G > 32 && G % 32 == 0, "block groups are whole warps");
    __shared__ double red[G / 32];
    __shared__ int ired[G / 32];
    const long long gid = blockIdx.x;
    if (gid >= batch) return;
    if (skip && skip[gid] == skip_value) return;
    eig_one<G>(n, a + gid * a_stride, w + gid * n, v + gid * (long long)n * n, info + gid, sweeps ? sweeps + gid : nullptr,
               ws + gid * eig_workspace_elems(n), eps, max_iter, t_out ? t_out + gid * (long long)n * n : nullptr, red, ired);
}

}  // namespace rcwa_gb300
