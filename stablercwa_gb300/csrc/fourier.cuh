// fourier.cuh -- closed-form Fourier coefficients of piecewise-constant profiles, on the device.
//
// A profile with edges x_0 < ... < x_K over one period P and value v_s on [x_s, x_{s+1}) has
//     c_h = sum_s v_s w_s(h),   w_s(0) = (x_{s+1} - x_s) / P,
//     w_s(h) = (e(x_{s+1}) - e(x_s)) / (-2 pi i h),   e(x) = exp(-2 pi i h x / P),
// the exact integral of each constant piece against the harmonic (the 1-D operators of
// include/stablercwa/rcwa1d.hpp:366-388 and the 2-D strip, column and segment weights of
// include/stablercwa/rcwa2d_operators.hpp:97-140). Here every segment weight is evaluated by one
// thread with sincospi on the reduced argument 2 h x / P (no rounded pi inside the argument), and a
// coefficient is the dot product of the segment values with one column of weights. Because
// sincospi(-t) is the exact mirror of sincospi(t), w_s(-h) is exactly conj(w_s(h)): a profile of real
// values gets exactly conjugate-symmetric coefficients.
//
// 2-D layers (Li's factorisation, include/stablercwa/rcwa2d_operators.hpp:325-429) need, per layer:
//   wy[k][h]   the weights of the y strips (period Ly, |h| <= 2 M2),
//   ce[k][h]   each strip's x profile of eps = n^2 (|h| <= 2 M1), ci[k][h] the same of 1/eps,
//   wx[j][h]   the weights of the merged x cuts (period Lx, |h| <= 2 M1),
//   cyc[j][h]  the y profile of 1/eps in the column between cuts j and j + 1 (|h| <= 2 M2),
// all formed here on the device from one packed upload of the layer's geometry.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "engine.h"
#include "launch.cuh"

namespace rcwa_gb300 {
namespace {

// w_s(h) for the segment [xa, xb] of period P (h != 0 by the closed form, h == 0 the length fraction)
__device__ __forceinline__ zc segment_weight(double xa, double xb, long long h, double period) {
    if (h == 0) return zc{(xb - xa) / period, 0.0};
    const double two_h = 2.0 * (double)h;
    double sa, ca, sb, cb;
    sincospi(two_h * xa / period, &sa, &ca);
    sincospi(two_h * xb / period, &sb, &cb);
    // e(x) = (cos, -sin); (e(xb) - e(xa)) / (i w) with w = -2 pi h is (d.im / w, -d.re / w)
    const double dre = cb - ca, dim = -(sb - sa);
    const double w = -2.0 * 3.141592653589793238462643383279502884 * (double)h;
    return zc{dim / w, -dre / w};
}

// value transforms applied to a profile's stored values before the sum
enum ProfileMap : int { MAP_AS_IS = 0, MAP_SQUARE = 1, MAP_INV_SQUARE = 2 };

__device__ __forceinline__ zc map_value(zc v, int map) {
    if (map == MAP_AS_IS) return v;
    const zc sq = v * v;
    return map == MAP_SQUARE ? sq : zinv(sq);
}

// c[p][h + hmax] of P profiles: profile p has edges edges[eoff[p] .. eoff[p + 1]) and the values
// vals[eoff[p] - p .. eoff[p + 1] - p - 1) (one fewer than its edges). One thread per (profile, h).
__global__ void profile_coeff_kernel(int P, int hmax, double period, const int* __restrict__ eoff,
                                     const double* __restrict__ edges, const zc* __restrict__ vals, int map,
                                     zc* __restrict__ out) {
    const int H = 2 * hmax + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)P * H) return;
    const int p = (int)(idx / H), t = (int)(idx - (long long)p * H);
    const long long h = t - hmax;
    const int e0 = eoff[p], e1 = eoff[p + 1];
    zc acc{0.0, 0.0};
    for (int e = e0; e + 1 < e1; ++e) acc = acc + map_value(vals[e - p], map) * segment_weight(edges[e], edges[e + 1], h, period);
    out[idx] = acc;
}

// w[s][h + hmax] of the S segments of one edge list (S + 1 edges)
__global__ void segment_weight_kernel(int S, int hmax, double period, const double* __restrict__ edges,
                                      zc* __restrict__ out) {
    const int H = 2 * hmax + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)S * H) return;
    const int s = (int)(idx / H), t = (int)(idx - (long long)s * H);
    out[idx] = segment_weight(edges[s], edges[s + 1], t - hmax, period);
}

// x mod Lx with the sign of Lx (Lx > 0), +0 for an exact multiple: Python's float %, which the
// reference's column rule follows (rcwa2d_operators.hpp:144-154)
__host__ __device__ __forceinline__ double wrap_period(double x, double Lx) {
    double r = fmod(x, Lx);
    if (r < 0.0) r += Lx;
    return r == 0.0 ? 0.0 : r;
}

// 1/eps of strip k at the midpoint of column j: the strip's profile repeats with period Lx from its
// first edge, and the segment is the last one starting at or before the wrapped point (clamped to the
// profile), as rcwa2d_operators.hpp:162-171 evaluates it. One thread per (column, strip).
__global__ void column_inv_eps_kernel(int Kx, int K, double Lx, const double* __restrict__ cuts,
                                      const int* __restrict__ eoff, const double* __restrict__ xedges,
                                      const zc* __restrict__ nvals, zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Kx * K) return;
    const int j = (int)(idx / K), k = (int)(idx - (long long)j * K);
    const double xm = 0.5 * (cuts[j] + cuts[j + 1]);
    const int e0 = eoff[k], ne = eoff[k + 1] - e0;
    const double* xe = xedges + e0;
    const double xx = xe[0] + wrap_period(xm - xe[0], Lx);
    int lo = 0, hi = ne;  // first edge index with xe[i] > xx
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (xe[mid] > xx) hi = mid;
        else lo = mid + 1;
    }
    const int seg = min(max(lo - 1, 0), ne - 2);
    out[idx] = map_value(nvals[e0 - k + seg], MAP_INV_SQUARE);
}

// out[j][h] = sum_k v[j][k] w[k][h] (Kx x K times K x H)
__global__ void coeff_contract_kernel(int J, int K, int H, const zc* __restrict__ v, const zc* __restrict__ w,
                                      zc* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)J * H) return;
    const int j = (int)(idx / H), t = (int)(idx - (long long)j * H);
    zc acc{0.0, 0.0};
    for (int k = 0; k < K; ++k) acc = acc + v[(long long)j * K + k] * w[(long long)k * H + t];
    out[idx] = acc;
}

// c[h + hmax] and c[hmax - h] made exactly conjugate (their average), c_0 real: a profile of real values
// has coefficients conjugate-symmetric to rounding (the FFT-sampled form); this makes the Toeplitz
// operators exactly Hermitian for the Hermitian eigensolver
__global__ void hermitian_coeff_kernel(int hmax, zc* __restrict__ c) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > hmax) return;
    if (k == 0) {
        c[hmax].im = 0.0;
        return;
    }
    const zc a = c[hmax + k], b = c[hmax - k];
    const zc avg{0.5 * (a.re + b.re), 0.5 * (a.im - b.im)};
    c[hmax + k] = avg;
    c[hmax - k] = zc{avg.re, -avg.im};
}

// ---------------------------------------------------------------- host launchers

// Closed-form coefficients c[h + hmax] (h = -hmax..hmax) of one profile into device memory.
inline zc* closed_form_coefficients(cudaStream_t st, DeviceScratch& mem, const std::vector<double>& edges,
                                    const std::vector<std::complex<double>>& values, double period, int hmax) {
    const int H = 2 * hmax + 1, ne = (int)edges.size();
    zc* c = mem.get<zc>(H);
    double* d_edges = mem.get<double>(ne);
    zc* d_vals = mem.get<zc>(values.size());
    int* d_off = mem.get<int>(2);
    const int off[2] = {0, ne};
    RCWA_CUDA(cudaMemcpyAsync(d_edges, edges.data(), ne * sizeof(double), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_vals, values.data(), values.size() * sizeof(zc), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_off, off, sizeof(off), cudaMemcpyHostToDevice, st));
    LAUNCH(profile_coeff_kernel, nblocks(H), kTpb, st, 1, hmax, period, d_off, d_edges, d_vals, MAP_AS_IS, c);
    mem.free(d_edges);
    mem.free(d_vals);
    mem.free(d_off);
    return c;
}

// The boundaries of the columns of constant permittivity of a 2-D layer: every strip's x edges wrapped
// into [0, Lx) plus 0 and Lx, each snapped to a 1e-12 grid (rounded half to even, like numpy.round to
// 12 decimals), kept inside [-1e-12, Lx + 1e-12] and deduplicated in ascending order; 0 is restored
// at the front and Lx at the back if snapping moved them away by more than 1e-12
// (the rule of include/stablercwa/rcwa2d_operators.hpp:178-192).
inline std::vector<double> column_cuts(const std::vector<std::vector<double>>& strip_edges, double Lx) {
    const auto snap = [](double x) { return std::nearbyint(x * 1e12) / 1e12; };
    std::vector<double> cuts{snap(0.0), snap(Lx)};
    for (const std::vector<double>& e : strip_edges)
        for (double x : e) cuts.push_back(snap(wrap_period(x, Lx)));
    cuts.erase(std::remove_if(cuts.begin(), cuts.end(), [&](double c) { return !(c >= -1e-12 && c <= Lx + 1e-12); }),
               cuts.end());
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    if (cuts.empty() || cuts.front() > 1e-12) cuts.insert(cuts.begin(), 0.0);
    if (cuts.back() < Lx - 1e-12) cuts.push_back(Lx);
    return cuts;
}

// Device Fourier data of one patterned 2-D layer (layout: row-major [profile][h + hmax]).
struct LayerFourier2D {
    int K = 0, Kx = 0;
    zc *wy = nullptr, *ce = nullptr, *ci = nullptr, *wx = nullptr, *cyc = nullptr;
};

// y_edges: K + 1 strip boundaries; strip k has x edges strip_edges[k] and indices strip_n[k].
inline LayerFourier2D layer_fourier2d(cudaStream_t st, DeviceScratch& mem, const std::vector<double>& y_edges,
                                      const std::vector<std::vector<double>>& strip_edges,
                                      const std::vector<std::vector<std::complex<double>>>& strip_n, double Lx,
                                      double Ly, int M1, int M2, bool li) {
    LayerFourier2D F;
    F.K = (int)strip_edges.size();
    const int Hx = 4 * M1 + 1, Hy = 4 * M2 + 1;
    std::vector<int> eoff{0};
    std::vector<double> xe;
    std::vector<std::complex<double>> nv;
    for (int k = 0; k < F.K; ++k) {
        xe.insert(xe.end(), strip_edges[k].begin(), strip_edges[k].end());
        nv.insert(nv.end(), strip_n[k].begin(), strip_n[k].end());
        eoff.push_back((int)xe.size());
    }
    const std::vector<double> cuts = li ? column_cuts(strip_edges, Lx) : std::vector<double>{};
    F.Kx = li ? (int)cuts.size() - 1 : 0;

    int* d_eoff = mem.get<int>(eoff.size());
    double* d_xe = mem.get<double>(xe.size());
    zc* d_nv = mem.get<zc>(nv.size());
    double* d_ye = mem.get<double>(y_edges.size());
    RCWA_CUDA(cudaMemcpyAsync(d_eoff, eoff.data(), eoff.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_xe, xe.data(), xe.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_nv, nv.data(), nv.size() * sizeof(zc), cudaMemcpyHostToDevice, st));
    RCWA_CUDA(cudaMemcpyAsync(d_ye, y_edges.data(), y_edges.size() * sizeof(double), cudaMemcpyHostToDevice, st));

    F.wy = mem.get<zc>((size_t)F.K * Hy);
    LAUNCH(segment_weight_kernel, nblocks((long long)F.K * Hy), kTpb, st, F.K, 2 * M2, Ly, d_ye, F.wy);
    F.ce = mem.get<zc>((size_t)F.K * Hx);
    LAUNCH(profile_coeff_kernel, nblocks((long long)F.K * Hx), kTpb, st, F.K, 2 * M1, Lx, d_eoff, d_xe, d_nv,
                                                                                MAP_SQUARE, F.ce);
    if (li) {
        F.ci = mem.get<zc>((size_t)F.K * Hx);
        LAUNCH(profile_coeff_kernel, nblocks((long long)F.K * Hx), kTpb, st, F.K, 2 * M1, Lx, d_eoff, d_xe, d_nv,
                                                                                    MAP_INV_SQUARE, F.ci);
        double* d_cuts = mem.get<double>(cuts.size());
        RCWA_CUDA(cudaMemcpyAsync(d_cuts, cuts.data(), cuts.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        F.wx = mem.get<zc>((size_t)F.Kx * Hx);
        LAUNCH(segment_weight_kernel, nblocks((long long)F.Kx * Hx), kTpb, st, F.Kx, 2 * M1, Lx, d_cuts, F.wx);
        zc* col = mem.get<zc>((size_t)F.Kx * F.K);
        LAUNCH(column_inv_eps_kernel, nblocks((long long)F.Kx * F.K), kTpb, st, F.Kx, F.K, Lx, d_cuts, d_eoff,
                                                                                      d_xe, d_nv, col);
        F.cyc = mem.get<zc>((size_t)F.Kx * Hy);
        LAUNCH(coeff_contract_kernel, nblocks((long long)F.Kx * Hy), kTpb, st, F.Kx, F.K, Hy, col, F.wy, F.cyc);
        mem.free(col);
        mem.free(d_cuts);
    }
    mem.free(d_eoff);
    mem.free(d_xe);
    mem.free(d_nv);
    mem.free(d_ye);
    return F;
}

inline void free_layer_fourier2d(DeviceScratch& mem, LayerFourier2D& F) {
    for (zc* p : {F.wy, F.ce, F.ci, F.wx, F.cyc})
        if (p) mem.free(p);
    F = LayerFourier2D{};
}

}  // namespace
}  // namespace rcwa_gb300
