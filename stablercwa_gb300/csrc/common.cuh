// common.cuh -- FP64 complex arithmetic and small helpers shared by the engine's kernels.
//
// Complex numbers are plain {re, im} doubles, laid out like std::complex<double> and the public
// rcwa_complex. Products are written out component by component, as the reference writes its inner
// loops (include/stablercwa/lu.hpp:82-85, include/stablercwa/eig_qr.hpp:87-96).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

// A kernel's dynamically sized shared array (a host emulation of the kernels for tests predefines it)
#ifndef RCWA_DYN_SMEM
#define RCWA_DYN_SMEM(T, name) extern __shared__ T name[]
#endif

namespace rcwa_gb300 {

struct __align__(16) zc {
    double re, im;
};

__host__ __device__ __forceinline__ zc mk(double r, double i) { return zc{r, i}; }
__host__ __device__ __forceinline__ zc operator+(zc a, zc b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ zc operator-(zc a, zc b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ zc operator-(zc a) { return {-a.re, -a.im}; }
__host__ __device__ __forceinline__ zc operator*(zc a, zc b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ __forceinline__ zc operator*(double s, zc a) { return {s * a.re, s * a.im}; }
__host__ __device__ __forceinline__ zc operator*(zc a, double s) { return {a.re * s, a.im * s}; }
__host__ __device__ __forceinline__ bool operator==(zc a, zc b) { return a.re == b.re && a.im == b.im; }
__host__ __device__ __forceinline__ bool operator!=(zc a, zc b) { return !(a == b); }
__host__ __device__ __forceinline__ zc conj(zc a) { return {a.re, -a.im}; }
__host__ __device__ __forceinline__ bool is_zero(zc a) { return a.re == 0.0 && a.im == 0.0; }
__host__ __device__ __forceinline__ double abs1(zc a) { return fabs(a.re) + fabs(a.im); }
__host__ __device__ __forceinline__ double norm2(zc a) { return a.re * a.re + a.im * a.im; }
__host__ __device__ __forceinline__ double zabs(zc a) { return hypot(a.re, a.im); }
__host__ __device__ __forceinline__ bool zfinite(zc a) { return isfinite(a.re) && isfinite(a.im); }

// c + a*b (the accumulate form of the reference's add_column / axpy kernels)
__host__ __device__ __forceinline__ zc zfma(zc a, zc b, zc c) {
    return {c.re + (a.re * b.re - a.im * b.im), c.im + (a.re * b.im + a.im * b.re)};
}
// c + a*b and c + conj(a)*b as four fused multiply-adds each (a*b is not rounded on its own), for the
// eigensolver's inner loops
__host__ __device__ __forceinline__ zc zmac(zc a, zc b, zc c) {
    return {fma(-a.im, b.im, fma(a.re, b.re, c.re)), fma(a.im, b.re, fma(a.re, b.im, c.im))};
}
__host__ __device__ __forceinline__ zc zmacc(zc a, zc b, zc c) {
    return {fma(a.im, b.im, fma(a.re, b.re, c.re)), fma(-a.im, b.re, fma(a.re, b.im, c.im))};
}
// c - a*b
__host__ __device__ __forceinline__ zc zfms(zc a, zc b, zc c) {
    return {c.re - a.re * b.re + a.im * b.im, c.im - a.re * b.im - a.im * b.re};
}

// Smith's division: scale by the larger component of the divisor so |b|^2 never forms
// (include/stablercwa/lu.hpp:88-97).
__host__ __device__ __forceinline__ zc zdiv(zc a, zc b) {
    const double br = b.re, bi = b.im;
    if (fabs(br) >= fabs(bi)) {
        const double r = bi / br, d = br + bi * r;
        return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
    }
    const double r = br / bi, d = bi + br * r;
    return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}

// Division by a real scalar, component-wise.
__host__ __device__ __forceinline__ zc zdivr(zc a, double s) { return {a.re / s, a.im / s}; }

// Exponent e with m = f * 2^e, f in [0.5, 1) for finite m > 0, else 0 (frexp semantics,
// include/stablercwa/eig_qr.hpp:206-210).
__host__ __device__ __forceinline__ int bexp(double m) {
    if (!(m > 0.0) || !isfinite(m)) return 0;
    int e;
    frexp(m, &e);
    return e;
}
__host__ __device__ __forceinline__ zc scale2(zc z, int e) { return {ldexp(z.re, e), ldexp(z.im, e)}; }

// Principal complex square root by the half-angle formulas: with d = |z|, the component of larger
// magnitude is sqrt((d + |x|)/2) and the other is y/(2 * that), so nothing cancels. Arguments are
// pre-scaled by a power of two when they are extreme so |z| neither overflows nor underflows.
// The branch cut and signed zeros follow C99 csqrt (Annex G): Re >= 0, Im carries the sign of y.
__host__ __device__ inline zc zsqrt(zc z) {
    const double x = z.re, y = z.im;
    if (x == 0.0 && y == 0.0) return {0.0, y};
    if (isinf(y)) return {INFINITY, y};
    if (isnan(x) || isnan(y)) return {NAN, NAN};
    if (y == 0.0) {
        if (x < 0.0) return {0.0, copysign(sqrt(-x), y)};
        return {sqrt(x), y};
    }
    const double big = fmax(fabs(x), fabs(y));
    int e = 0;
    double xs = x, ys = y;
    if (big > 1e300 || big < 1e-300) {
        e = bexp(big) & ~1;  // even, so sqrt of 2^e is exact
        xs = ldexp(x, -e);
        ys = ldexp(y, -e);
    }
    const double d = hypot(xs, ys);
    double r, s;
    if (xs >= 0.0) {
        r = sqrt(0.5 * (d + xs));
        s = 0.5 * (ys / r);
    } else {
        s = sqrt(0.5 * (d - xs));
        r = fabs(0.5 * (ys / s));
        s = copysign(s, ys);
    }
    if (e) {
        r = ldexp(r, e / 2);
        s = ldexp(s, e / 2);
    }
    return {r, s};
}

// exp(z) = e^re (cos im + i sin im)
__host__ __device__ __forceinline__ zc zexp(zc z) {
    const double m = exp(z.re);
    double s, c;
    sincos(z.im, &s, &c);
    return {m * c, m * s};
}

// Reciprocal 1/z by Smith's method.
__host__ __device__ __forceinline__ zc zinv(zc z) { return zdiv(zc{1.0, 0.0}, z); }

__device__ __forceinline__ zc ldz(const zc* p) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    return {v.x, v.y};
}
__device__ __forceinline__ void stz(zc* p, zc v) { *reinterpret_cast<double2*>(p) = make_double2(v.re, v.im); }

// Right-hand side forms of the batched solve.
enum RhsKind : int { RHS_DENSE = 0, RHS_IDENTITY = 1, RHS_DIAG = 2 };

// Group-of-G-lanes helpers: the G lanes of a group are contiguous in the warp.
template <int G>
__device__ __forceinline__ unsigned group_mask() {
    if constexpr (G == 32) {
        return 0xffffffffu;
    } else {
        const unsigned lane = threadIdx.x & 31u;
        return ((1u << G) - 1u) << (lane & ~(unsigned)(G - 1));
    }
}
template <int G>
__device__ __forceinline__ double group_sum(double v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
    return v;
}
template <int G>
__device__ __forceinline__ double group_max(double v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(mask, v, o, G));
    return v;
}
template <int G>
__device__ __forceinline__ int group_or(int v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v |= __shfl_xor_sync(mask, v, o, G);
    return v;
}
template <int G>
__device__ __forceinline__ int group_min_int(int v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(mask, v, o, G));
    return v;
}
template <int G>
__device__ __forceinline__ int group_max_int(int v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(mask, v, o, G));
    return v;
}

// triangular factors of a product (launch_zgemm): the zero part's terms are exact zeros and are skipped
enum { TRI_NONE = 0, TRI_A_LOWER = 1, TRI_A_UPPER = 2, TRI_B_UPPER = 3 };

}  // namespace rcwa_gb300
