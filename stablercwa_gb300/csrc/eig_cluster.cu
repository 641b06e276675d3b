// eig_cluster.cu -- one large general eigenproblem spread over a thread-block cluster.
//
// The batched solver (eig.cuh) gives each matrix a lane group or one CTA; a lone matrix of order
// several hundred then runs on one SM, whose FP64 rate (about 8 GFLOP/s) sets the solve time. Here the
// same algorithm (EISPACK CORTH + COMQR2 as include/stablercwa/eig_qr.hpp restates it: Householder
// reduction with the reflectors accumulated, the real subdiagonal, single-shift QR with Wilkinson and
// exceptional shifts and the same deflation test, back substitution with the coincident-eigenvalue floor
// and overflow control, V = Z X normalised) runs on a cluster of C CTAs (8 or 16, one per SM) that
// share the matrix through L2 and exchange partial sums and rotation logs through distributed shared
// memory:
//   * reduction to Hessenberg form: columns are dealt to the CTAs; every CTA forms the reflector from
//     the current column redundantly, updates its own columns from the left, and contributes its share
//     of the rank-one term w = (P A) u, which the CTAs sum by reading each other's shared memory; two
//     cluster barriers per column;
//   * the reflectors are accumulated into Z column by column by each column's owner (no barrier);
//   * each QR sweep: the leader CTA runs the rotation chain on the active window only (one CTA barrier
//     per rotation; a rotation needs just the column it zeroes; each thread carries its columns' current
//     row in registers and loads the next one a step ahead), logging the rotations in its shared
//     memory; then every CTA reads the log (DSMEM) and applies it to its share of the work that does not
//     feed the chain: H's rows 0..en from the right, the columns right of the window from the left, and
//     all rows of Z; two cluster barriers per sweep;
//   * eigenvectors: one warp per column for the back substitution, CTAs by columns for V = Z X.
// Per-element arithmetic is the batched solver's, so the QR phase matches it operation for operation;
// the reduction sums are partitioned differently, so results agree to rounding. No thread waits on
// anything but CTA and cluster barriers that every thread reaches.
#include <cuda_runtime.h>
#include <float.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "eig.cuh"
#include "engine.h"

namespace rcwa_gb300 {
namespace {

constexpr int kCT = 512;  // threads per CTA
constexpr int kWarps = kCT / 32;
constexpr int kMaxCarry = 4;  // window columns per thread in the leader's chain: orders up to 4 kCT

__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster; release/acquire at cluster scope orders global and shared memory
__device__ __forceinline__ void cl_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t sh_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
// a double in the shared memory of CTA `rank` of this cluster, at the same offset as p here
__device__ __forceinline__ double ld_remote(const double* p, unsigned rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(sh_u32(p)), "r"(rank));
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(r) : "memory");
    return v;
}
__device__ __forceinline__ int ld_remote_i(const int* p, unsigned rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(sh_u32(p)), "r"(rank));
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(r) : "memory");
    return v;
}
__device__ __forceinline__ zc ld_remote_z(const zc* p, unsigned rank) {
    const double* d = reinterpret_cast<const double*>(p);
    return zc{ld_remote(d, rank), ld_remote(d + 1, rank)};
}

// CTA-wide sum / max: every thread gets the result (red: kWarps doubles of shared memory)
__device__ __forceinline__ double cta_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = red[0];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) s += red[w];
    return s;
}
__device__ __forceinline__ double cta_max(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = red[0];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) s = fmax(s, red[w]);
    return s;
}
__device__ __forceinline__ int cta_max_int(int v, int* ired) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) ired[threadIdx.x >> 5] = v;
    __syncthreads();
    int s = ired[0];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) s = max(s, ired[w]);
    return s;
}

__device__ __forceinline__ zc warp_zsum(zc v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
        v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
    }
    return v;
}

// left and right rotation of a pair by the logged (cr, ci, s) (the batched solver's formulas)
__device__ __forceinline__ void rot_left(double cr, double ci, double s, zc& y, zc& z) {
    const zc y0 = y, z0 = z;
    y = zc{cr * y0.re + ci * y0.im + s * z0.re, cr * y0.im - ci * y0.re + s * z0.im};
    z = zc{cr * z0.re - ci * z0.im - s * y0.re, cr * z0.im + ci * z0.re - s * y0.im};
}
__device__ __forceinline__ zc rot_right(double cr, double ci, double s, zc& a, zc b) {
    const zc out = zc{cr * a.re - ci * a.im + s * b.re, cr * a.im + ci * a.re + s * b.im};
    a = zc{cr * b.re + ci * b.im - s * a.re, cr * b.im - ci * b.re - s * a.im};
    return out;
}

}  // namespace

size_t eig_cluster_smem_bytes(int n) { return (size_t)n * (5 * sizeof(zc) + 3 * sizeof(double)) + 256; }

// One cluster per matrix (grid = batch x C CTAs, cluster dimension C). ws: eig_workspace_elems(n) per matrix.
__global__ void __launch_bounds__(kCT, 1)
    eig_cluster_kernel(int n, int batch, const zc* __restrict__ a, long long a_stride, zc* __restrict__ w,
                       zc* __restrict__ v, int* __restrict__ info_out, int* __restrict__ sweeps_out,
                       zc* __restrict__ ws, double eps, int max_iter, const int* __restrict__ skip, int skip_value,
                       zc* __restrict__ t_out) {
    const unsigned C = cl_size(), rank = cl_rank();
    const long long gid = blockIdx.x / C;
    if (gid >= batch) return;                                // uniform over the cluster
    if (skip && skip[gid] == skip_value) return;             // uniform over the cluster
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ double red_s[kWarps];
    __shared__ int ired_s[kWarps];
    __shared__ zc s_phase;
    __shared__ int s_state[4];  // the leader's en, l, done (0 sweep, 1 converged, 2 not converged), has_phase
    zc* su = reinterpret_cast<zc*>(dsm);
    zc* sort = su + n;
    zc* swkp = sort + n;
    zc* swk = swkp + n;
    zc* syph = swk + n;
    double* rcr = reinterpret_cast<double*>(syph + n);
    double* rci = rcr + n;
    double* rs = rci + n;

    const int t = threadIdx.x, lane = t & 31, wp = t >> 5;
    const int gt = (int)rank * kCT + t, GT = (int)C * kCT;              // thread index within the cluster
    const int gw = (int)rank * kWarps + wp, GW = (int)C * kWarps;       // warp index within the cluster
    const zc* A = a + gid * a_stride;
    zc* W = w + gid * n;
    zc* V = v + gid * (long long)n * n;
    zc* H = ws + gid * eig_workspace_elems(n);
    zc* Z = H + (long long)n * n;
    zc* X = Z + (long long)n * n;
    zc* T = t_out ? t_out + gid * (long long)n * n : nullptr;

    for (long long idx = gt; idx < (long long)n * n; idx += GT) H[idx] = A[idx];
    for (int i = t; i < n; i += kCT) sort[i] = zc{0.0, 0.0};
    cl_sync();

    // ---------------- Householder reduction (CORTH, eig_qr.hpp:231-272); column j belongs to CTA j % C
    for (int m = 1; m < n - 1; ++m) {
        const zc* x = H + (long long)(m - 1) * n;
        double sc = 0.0;
        for (int i = m + t; i < n; i += kCT) sc += abs1(x[i]);
        sc = cta_sum(sc, red_s);
        if (sc == 0.0) continue;  // every CTA sees the same column: uniform
        double h = 0.0;
        for (int i = m + t; i < n; i += kCT) {
            const zc uu = zdivr(x[i], sc);
            su[i] = uu;
            h += norm2(uu);
        }
        h = cta_sum(h, red_s);  // its barriers also publish su
        double gg = sqrt(h);
        zc om = su[m];
        const double f = zabs(om);
        if (f == 0.0) {
            om = zc{gg, 0.0};
        } else {
            h += f * gg;
            gg /= f;
            om = om * (1.0 + gg);
        }
        __syncthreads();
        if (t == 0) su[m] = om;
        __syncthreads();
        // left: own columns j >= m, a warp per column, rows >= m
        for (int j = m + (int)((rank + C - (unsigned)(m % C)) % C) + wp * (int)C; j < n; j += kWarps * (int)C) {
            zc* aj = H + (long long)j * n;
            zc d{0.0, 0.0};
            for (int i = m + lane; i < n; i += 32) {
                const zc uu = su[i], av = aj[i];
                d.re += uu.re * av.re + uu.im * av.im;
                d.im += uu.re * av.im - uu.im * av.re;
            }
            d = warp_zsum(d);
            const zc tt = zc{-d.re / h, -d.im / h};
            for (int i = m + lane; i < n; i += 32) aj[i] = zfma(tt, su[i], aj[i]);
        }
        __syncthreads();
        // own share of w = sum_j u_j (P A)(:, j), all rows
        for (int i = t; i < n; i += kCT) {
            zc acc{0.0, 0.0};
            for (int j = m + (int)((rank + C - (unsigned)(m % C)) % C); j < n; j += (int)C) acc = zfma(su[j], H[(long long)j * n + i], acc);
            swkp[i] = acc;
        }
        cl_sync();
        for (int i = t; i < n; i += kCT) {
            zc acc{0.0, 0.0};
            for (unsigned r = 0; r < C; ++r) acc = acc + ld_remote_z(swkp + i, r);
            swk[i] = zdivr(acc, h);
        }
        __syncthreads();
        // right: own columns j >= m, all rows: A(:, j) -= w conj(u_j)
        for (int j = m + (int)((rank + C - (unsigned)(m % C)) % C); j < n; j += (int)C) {
            zc* aj = H + (long long)j * n;
            const zc cu = -conj(su[j]);
            for (int i = t; i < n; i += kCT) aj[i] = zfma(cu, swk[i], aj[i]);
        }
        if (t == 0) {
            sort[m] = om * sc;
            if ((unsigned)((m - 1) % C) == rank) {
                zc* xm = H + (long long)(m - 1) * n + m;
                *xm = (f == 0.0 ? zc{sc, 0.0} : *xm) * (-gg);
            }
        }
        cl_sync();  // the next column and everyone's partial buffer are free
    }

    // ---------------- reflectors accumulated into Z (eig_qr.hpp:354-373): each CTA its own columns
    for (int j = (int)rank; j < n; j += (int)C)
        for (int r = t; r < n; r += kCT) Z[(long long)j * n + r] = zc{r == j ? 1.0 : 0.0, 0.0};
    __syncthreads();
    for (int i = n - 2; i >= 1; --i) {
        const zc oi = sort[i];
        const zc hs = H[(long long)(i - 1) * n + i];
        if (is_zero(oi) || is_zero(hs)) continue;
        const int e = bexp(abs1(oi));
        const zc sub = scale2(hs, -e);
        const zc v0 = scale2(oi, -e);
        const double minus_h = sub.re * v0.re + sub.im * v0.im;
        for (int k = i + t; k < n; k += kCT) su[k] = k == i ? v0 : scale2(H[(long long)(i - 1) * n + k], -e);
        __syncthreads();
        for (int j = i + (int)((rank + C - (unsigned)(i % C)) % C) + wp * (int)C; j < n; j += kWarps * (int)C) {
            zc* zj = Z + (long long)j * n;
            zc d{0.0, 0.0};
            for (int k = i + lane; k < n; k += 32) {
                const zc uu = su[k], av = zj[k];
                d.re += uu.re * av.re + uu.im * av.im;
                d.im += uu.re * av.im - uu.im * av.re;
            }
            d = warp_zsum(d);
            const zc tt = zc{d.re / minus_h, d.im / minus_h};
            for (int k = i + lane; k < n; k += 32) zj[k] = zfma(tt, su[k], zj[k]);
        }
        __syncthreads();
    }
    cl_sync();

    // ---------------- clean Hessenberg form with a real subdiagonal (eig_qr.hpp:420-439). The phase
    // y_i of step i depends on the subdiagonal as step i - 1 left it; the chain is formed first (one
    // thread per CTA, each CTA the same), then every entry is scaled once.
    if (t == 0) {
        zc yprev{1.0, 0.0};
        bool prev_set = false;
        syph[0] = zc{1.0, 0.0};
        for (int i = 1; i < n; ++i) {
            zc sub = H[(long long)(i - 1) * n + i];
            if (prev_set) sub = yprev * sub;
            if (sub.im == 0.0) {
                syph[i] = zc{1.0, 0.0};
                swk[i] = sub;  // the final subdiagonal entry
                prev_set = false;
                continue;
            }
            double nrm = 0.0;
            const zc y = unit_phase(sub, nrm);
            syph[i] = y;
            swk[i] = zc{nrm, 0.0};
            yprev = y;
            prev_set = true;
        }
    }
    __syncthreads();
    cl_sync();  // every CTA has read the subdiagonal before it changes
    for (long long idx = gt; idx < (long long)n * n; idx += GT) {
        const int c = (int)(idx / n), r = (int)(idx - (long long)c * n);
        if (r >= c + 2) {
            H[idx] = zc{0.0, 0.0};
        } else if (r == c + 1) {
            H[idx] = swk[r];
        } else {
            zc hv = H[idx];
            if (syph[r].im != 0.0 || syph[r].re != 1.0) hv = conj(syph[r]) * hv;
            if (syph[c].im != 0.0 || syph[c].re != 1.0) hv = syph[c] * hv;
            H[idx] = hv;
        }
        if (syph[c].im != 0.0 || syph[c].re != 1.0) Z[idx] = syph[c] * Z[idx];
    }
    cl_sync();

    // ---------------- shifted QR (eig_qr.hpp:1039-1096). The leader CTA decides every deflation, shift and
    // the outcome and runs each sweep's chain; the state and the rotation log reach the other CTAs through
    // their shared memory after the first barrier of the sweep.
    zc tsh{0.0, 0.0};
    int en = n - 1, its = 0, sweeps = 0, info = 0, l = 0;
    for (;;) {
        int done = 0;
        if (rank == 0) {
            for (;;) {  // deflate as long as the bottom entry has converged
                if (en < 0) {
                    done = 1;
                    break;
                }
                int cand = 0;
                for (int c = 1 + t; c <= en; c += kCT) {
                    const zc hsub = H[(long long)(c - 1) * n + c];
                    const zc hd0 = H[(long long)(c - 1) * n + c - 1];
                    const zc hd1 = H[(long long)c * n + c];
                    if (abs1(hsub) <= eps * (abs1(hd0) + abs1(hd1))) cand = max(cand, c);
                }
                l = cta_max_int(cand, ired_s);
                if (l != en) break;
                if (t == 0) {
                    const zc wv = H[(long long)en * n + en] + tsh;
                    H[(long long)en * n + en] = wv;
                    W[en] = wv;
                }
                --en;
                its = 0;
            }
            if (!done && its == max_iter) {
                done = 2;
                info = en + 1;
            }
            if (!done) {
                zc s;
                if (its == 10 || its == 20) {
                    s = zc{fabs(H[(long long)(en - 1) * n + en].re) + (en >= 2 ? fabs(H[(long long)(en - 2) * n + en - 1].re) : 0.0),
                           0.0};
                } else {
                    s = wilkinson_shift(H[(long long)(en - 1) * n + en - 1], H[(long long)en * n + en - 1],
                                        H[(long long)(en - 1) * n + en].re, H[(long long)en * n + en]);
                }
                tsh = tsh + s;
                ++its;
                ++sweeps;
                __syncthreads();  // every thread has read the shift's inputs
                for (int r = t; r <= en; r += kCT) {
                    zc* p = H + (long long)r * n + r;
                    *p = *p - s;
                }
                __syncthreads();
                // the chain: rotation i from column i - 1, applied to window columns i..en. Thread t owns the
                // window columns c = l + 1 + t + k kCT; each keeps its column's current row i - 1 (cy) and the
                // next row i (cz, loaded one step ahead) in registers, so a step stores one entry per column
                // and reads none; the owner of column i forms rotation i + 1 from its carried row and the
                // subdiagonal entry it loaded a step ahead (csub).
                const int c_first = l + 1;
                zc cy[kMaxCarry], cz[kMaxCarry];
                double csub = 0.0;
#pragma unroll
                for (int k = 0; k < kMaxCarry; ++k) {
                    const int c = c_first + t + k * kCT;
                    if (c <= en) {
                        cy[k] = H[(long long)c * n + l];
                        cz[k] = H[(long long)c * n + l + 1];
                    }
                }
                if (t == 0) {
                    zc* cp = H + (long long)l * n;
                    zc top;
                    const Rot q = make_rotation(cp[l], cp[l + 1].re, top);
                    cp[l] = top;
                    cp[l + 1] = zc{0.0, 0.0};
                    rcr[l + 1] = q.cr;
                    rci[l + 1] = q.ci;
                    rs[l + 1] = q.s;
                    if (c_first < en) csub = H[(long long)c_first * n + c_first + 1].re;
                }
                __syncthreads();
                for (int i = l + 1; i <= en; ++i) {
                    const double cr = rcr[i], ci = rci[i], sn = rs[i];
#pragma unroll
                    for (int k = 0; k < kMaxCarry; ++k) {
                        const int c = c_first + t + k * kCT;
                        if (c < i || c > en) continue;
                        zc* col = H + (long long)c * n;
                        zc y = cy[k], z = cz[k];
                        rot_left(cr, ci, sn, y, z);
                        col[i - 1] = y;
                        if (c == i) {
                            if (i < en) {
                                zc top;
                                const Rot q = make_rotation(z, csub, top);
                                col[i] = top;
                                col[i + 1] = zc{0.0, 0.0};
                                rcr[i + 1] = q.cr;
                                rci[i + 1] = q.ci;
                                rs[i + 1] = q.s;
                            } else {
                                col[i] = z;
                            }
                        } else {
                            cy[k] = z;
                            cz[k] = col[i + 1];
                            if (c == i + 1 && i + 1 < en) csub = col[i + 2].re;
                        }
                    }
                    __syncthreads();
                }
            }
            if (t == 0) {
                int has_phase = 0;
                s_phase = zc{1.0, 0.0};
                if (!done) {
                    const zc hee = H[(long long)en * n + en];
                    if (hee.im != 0.0) {
                        double nrm = 0.0;
                        s_phase = unit_phase(hee, nrm);
                        H[(long long)en * n + en] = zc{nrm, 0.0};
                        has_phase = 1;
                    }
                }
                s_state[0] = en;
                s_state[1] = l;
                s_state[2] = done;
                s_state[3] = has_phase;
            }
        }
        cl_sync();  // the leader's state, log and window are complete
        if (rank != 0) {
            if (t == 0) {
                for (int k = 0; k < 4; ++k) s_state[k] = ld_remote_i(s_state + k, 0);
                s_phase = ld_remote_z(&s_phase, 0);
            }
            __syncthreads();
            en = s_state[0];
            l = s_state[1];
            done = s_state[2];
            if (!done)
                for (int i = l + 1 + t; i <= en; i += kCT) {
                    rcr[i] = ld_remote(rcr + i, 0);
                    rci[i] = ld_remote(rci + i, 0);
                    rs[i] = ld_remote(rs + i, 0);
                }
        }
        __syncthreads();
        if (done) break;
        const bool has_phase = s_state[3] != 0;
        const zc phase = s_phase;
        // items: H rows 0..en (right), H columns en+1..n-1 (left), Z rows 0..n-1 (right)
        const int items = (en + 1) + (n - 1 - en) + n;
        for (int it = gt; it < items; it += GT) {
            if (it <= en) {
                const int r = it;
                int j = max(l + 1, r);
                if (j > en) continue;
                zc av = H[(long long)(j - 1) * n + r];
                for (; j <= en; ++j) H[(long long)(j - 1) * n + r] = rot_right(rcr[j], rci[j], rs[j], av, H[(long long)j * n + r]);
                H[(long long)en * n + r] = has_phase ? phase * av : av;
            } else if (it < n) {
                const int c = it;
                zc* col = H + (long long)c * n;
                zc y = col[l];
                for (int i = l + 1; i <= en; ++i) {
                    zc z = col[i];
                    rot_left(rcr[i], rci[i], rs[i], y, z);
                    col[i - 1] = y;
                    y = z;
                }
                col[en] = has_phase ? conj(phase) * y : y;
            } else {
                const int r = it - n;
                zc av = Z[(long long)l * n + r];
                for (int j = l + 1; j <= en; ++j) Z[(long long)(j - 1) * n + r] = rot_right(rcr[j], rci[j], rs[j], av, Z[(long long)j * n + r]);
                Z[(long long)en * n + r] = has_phase ? phase * av : av;
            }
        }
        cl_sync();  // every CTA is done with the log and H before the leader's next sweep
    }
    const int outcome = s_state[2];

    if (rank == 0 && t == 0) {
        info_out[gid] = info;
        if (sweeps_out) sweeps_out[gid] = sweeps;
    }
    if (outcome == 2) {
        // not converged: unconverged diagonal plus the accumulated shift (eig_qr.hpp:1098-1103); no vectors
        if (rank == 0)
            for (int i = t; i <= en; i += kCT) W[i] = H[(long long)i * n + i] + tsh;
        cl_sync();
        return;
    }
    if (T) {
        for (long long idx = gt; idx < (long long)n * n; idx += GT) {
            const int c = (int)(idx / n), r = (int)(idx - (long long)c * n);
            T[idx] = r > c ? zc{0.0, 0.0} : H[idx];
            V[idx] = Z[idx];
        }
        cl_sync();
        return;
    }

    // ---------------- eigenvectors of T by back substitution (eig_qr.hpp:886-951), a warp per column
    double tn = 0.0;
    for (long long idx = t; idx < (long long)n * n; idx += kCT) {
        const int c = (int)(idx / n), r = (int)(idx - (long long)c * n);
        if (r <= c) tn = fmax(tn, abs1(H[idx]));
    }
    tn = cta_max(tn, red_s);
    const double rel = fmax(eps, DBL_EPSILON);
    double tiny = rel * tn;
    if (tiny == 0.0) tiny = DBL_MIN;
    const double kQuotientMax = 1e300;
    const double kShrink = 0x1p-512;
    for (int j = gw; j < n; j += GW) {
        zc* x = X + (long long)j * n;
        for (int k = lane; k < j; k += 32) x[k] = H[(long long)j * n + k];
        if (lane == 0) x[j] = zc{1.0, 0.0};
        __syncwarp();
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
            for (int pass = 0; pass < 3 && abs1(x[i]) > abs1(y) * kQuotientMax; ++pass) {
                __syncwarp();
                for (int k = lane; k <= j; k += 32) x[k] = x[k] * kShrink;
                __syncwarp();
            }
            const zc xi = zdiv(x[i], y);
            __syncwarp();
            if (lane == 0) x[i] = xi;
            __syncwarp();
            const double tr = abs1(xi);
            zc xs = xi;
            if (tr != 0.0 && tr + 1.0 / tr <= tr) {
                for (int k = lane; k <= j; k += 32) x[k] = zdivr(x[k], tr);
                __syncwarp();
                xs = x[i];
                __syncwarp();
            }
            const zc* ti = H + (long long)i * n;
            for (int k = lane; k < i; k += 32) x[k] = zfma(xs, ti[k], x[k]);
            __syncwarp();
        }
    }
    cl_sync();
    // V = Z X (X upper triangular), each column scaled to unit 2-norm; columns dealt to the CTAs
    for (int j = (int)rank; j < n; j += (int)C) {
        const zc* xj = X + (long long)j * n;
        zc* vj = V + (long long)j * n;
        double big = 0.0;
        for (int r = t; r < n; r += kCT) {
            zc acc = zc{0.0, 0.0};
            for (int k = 0; k <= j; ++k) acc = zfma(xj[k], Z[(long long)k * n + r], acc);
            vj[r] = acc;
            big = fmax(big, fmax(fabs(acc.re), fabs(acc.im)));
        }
        big = cta_max(big, red_s);
        if (big == 0.0 || !isfinite(big)) continue;
        double ssq = 0.0;
        for (int r = t; r < n; r += kCT) ssq += norm2(zdivr(vj[r], big));
        ssq = cta_sum(ssq, red_s);
        const double inv = 1.0 / sqrt(ssq);
        for (int r = t; r < n; r += kCT) vj[r] = zdivr(vj[r], big) * inv;
    }
    cl_sync();
}

}  // namespace rcwa_gb300

namespace rcwa_gb300 {
namespace {

// cluster size for the kernel at this shared-memory size: 16 CTAs when the device can co-schedule them,
// else 8, else 0 (no cluster form); decided once per (device, order). The kernel's dynamic shared memory
// opt-in only ever grows (ensure_smem_optin), so a launch of one order never finds it lowered by a
// concurrent call for a smaller order.
int cluster_size_for(int n) {
    static std::mutex lock;
    static std::vector<std::pair<std::pair<int, int>, int>> sizes;  // ((device, order), cluster size)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::lock_guard<std::mutex> g(lock);
    for (const auto& e : sizes)
        if (e.first.first == dev && e.first.second == n) return e.second;
    const size_t smem = eig_cluster_smem_bytes(n);
    int c = 0;
    bool opted = false;
    if (smem <= 200 * 1024 && n <= kMaxCarry * kCT) {
        try {
            ensure_smem_optin(reinterpret_cast<const void*>(eig_cluster_kernel), (int)smem);
            opted = true;
        } catch (const EngineError&) {
        }
    }
    if (opted && cudaFuncSetAttribute(eig_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
        for (int want : {16, 8}) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = want;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(want, 1, 1);
            cfg.blockDim = dim3(kCT, 1, 1);
            cfg.dynamicSmemBytes = smem;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, eig_cluster_kernel, &cfg) == cudaSuccess && clusters > 0) {
                c = want;
                break;
            }
        }
    }
    cudaGetLastError();  // a refused size leaves no error behind
    sizes.push_back({{dev, n}, c});
    return c;
}

}  // namespace

void preload_eig_cluster_kernel() {
    cudaFuncAttributes attr;
    cudaFuncGetAttributes(&attr, eig_cluster_kernel);  // loads the kernel under lazy module loading
    cudaGetLastError();
}

namespace {
int cluster_mode() {
    static const int mode = [] {
        const char* e = std::getenv("RCWA_GB300_EIG_CLUSTER");
        return e ? std::atoi(e) : 1;
    }();
    return mode;
}
}  // namespace

// The built-in rule: orders >= 384, up to 64 matrices. Measured on GB300 (one second call, RCWA-type
// matrices): a lone matrix of order 121 takes 63 ms on a 16-CTA cluster against 97 on one CTA, 2 of order
// 162 111 against 201, 4 of order 242 266 against 481, 8 of order 301 791 against 905, but 8 of order 162
// 221 against 203 and 8 of order 121 125 against 97 (eight 16-CTA clusters fill the GPU and share it).
// Below 384 the rule leaves the choice to the autotuner, which times the cluster form whenever it applies.
bool eig_cluster_wanted(int n, int batch) { return cluster_mode() != 0 && n >= 384 && batch <= 64 && cluster_size_for(n) > 0; }

// the cluster form can run this key (the autotuner's candidates)
bool eig_cluster_possible(int n, int batch) {
    return cluster_mode() != 0 && n >= 96 && batch <= 64 && cluster_size_for(n) > 0;
}

void launch_eig_cluster(cudaStream_t st, int n, int batch, const zc* a, long long a_stride, zc* w, zc* v, int* info,
                        int* sweeps, zc* ws, double eps, int max_iter, const int* skip, int skip_value, zc* t_out) {
    const int C = cluster_size_for(n);
    if (C == 0) throw EngineError{RCWA_EUNSUPPORTED, "eig: no cluster form for this order on this device"};
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(batch * C), 1, 1);
    cfg.blockDim = dim3(kCT, 1, 1);
    cfg.dynamicSmemBytes = eig_cluster_smem_bytes(n);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RCWA_CUDA(cudaLaunchKernelEx(&cfg, eig_cluster_kernel, n, batch, a, a_stride, w, v, info, sweeps, ws, eps, max_iter,
                                 skip, skip_value, t_out));
    ++launch_count();
}

}  // namespace rcwa_gb300
