// rcwa1d.cu -- batched 1-D TE/TM RCWA solve on the GPU (the engine behind rcwa::solve / rcwa::sweep).
//
// The host code here mirrors include/stablercwa/rcwa1d.hpp:853-1074 step by step, but every step
// is one batched kernel launch over a chunk of sweep points: per-layer assembly, the batched
// eigensolver (eig.cuh), and the S-matrix recursion in which each Zero/Diag/Dense operator of the
// reference (rcwa1d.hpp:549-629) becomes a B x n vector or a B x n x n matrix in device memory.
// Operator kinds depend only on the stack (which layers are gratings), so one launch sequence
// serves the whole chunk. The single sample-dependent kind change of the reference -- an exact
// q == 0 inside a layer whose propagation block meets a dense reflection (rcwa1d.hpp:751-784,
// :797-805) -- is taken by the affected samples only, through masked launches.
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "smatrix.cuh"

namespace rcwa_gb300 {
namespace {

// top block of two analytic regions: only column M of Tdd and Rud (include/stablercwa/rcwa1d.hpp:723-732)
__global__ void top_diag_vectors_kernel(int B, int n, int M, const zc* __restrict__ tdd_d, const zc* __restrict__ rud_d,
                                        zc* __restrict__ tdd, zc* __restrict__ rud) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * n) return;
    const int i = (int)(idx % n);
    tdd[idx] = i == M ? tdd_d[idx] : zc{0.0, 0.0};
    rud[idx] = i == M ? rud_d[idx] : zc{0.0, 0.0};
}

// Efficiencies and the failure contract (include/stablercwa/rcwa1d.hpp:1024-1055, :810-816).
__global__ void finalize_kernel(int B, int n, int M, int pol, int pure_films, const zc* __restrict__ R,
                                const zc* __restrict__ T, const zc* __restrict__ qI, const zc* __restrict__ qII,
                                const double* __restrict__ k0, zc nI, zc nII, int* __restrict__ fail,
                                zc* __restrict__ outR, zc* __restrict__ outT, double* __restrict__ DEr,
                                double* __restrict__ DEt) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= B) return;
    const int lane = threadIdx.x & 31;
    const double kk = k0[b];
    const zc qIM = qI[b * n + M];
    const zc den = zc{-kk * qIM.im, kk * qIM.re};
    const zc nI2 = nI * nI, nII2 = nII * nII;
    bool bad = fail[b] != 0;
    for (int j = lane; j < n; j += 32) {
        zc r = R[b * n + j], t = T[b * n + j];
        if (pure_films && j != M) {
            if (!zfinite(r)) r = zc{0.0, 0.0};
            if (!zfinite(t)) t = zc{0.0, 0.0};
        }
        if (!zfinite(r) || !zfinite(t)) bad = true;
        const zc q1 = qI[b * n + j], q2 = qII[b * n + j];
        const zc kIz = zc{-kk * q1.im, kk * q1.re};
        const zc kIIz = zc{-kk * q2.im, kk * q2.re};
        const double der = norm2(r) * zdiv(kIz, den).re;
        const zc factor = pol == 0 ? zdiv(kIIz, den) : zdiv(zdiv(kIIz, nII2), zdiv(den, nI2));
        const double det = norm2(t) * factor.re;
        if (!isfinite(der) || !isfinite(det)) bad = true;
        outR[b * n + j] = r;
        outT[b * n + j] = t;
        DEr[b * n + j] = der;
        DEt[b * n + j] = det;
    }
    bad = __any_sync(0xffffffffu, bad);
    if (bad) {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        for (int j = lane; j < n; j += 32) {
            outR[b * n + j] = zc{nan, nan};
            outT[b * n + j] = zc{nan, nan};
            DEr[b * n + j] = nan;
            DEt[b * n + j] = nan;
        }
        if (lane == 0) fail[b] = 1;
    }
}

__global__ void status_kernel(int B, const int* __restrict__ fail, const int* __restrict__ eig_info, int base_solves,
                              int base_lu, const int* __restrict__ extra_solves, int n_eig, int* __restrict__ status,
                              int* __restrict__ info_out, int* __restrict__ n_eig_out, int* __restrict__ n_solve_out,
                              int* __restrict__ n_lu_out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    if (status) status[b] = fail[b] ? (eig_info[b] ? RCWA_SAMPLE_EIG_NOCONV : RCWA_SAMPLE_NUMERICAL) : RCWA_SAMPLE_OK;
    if (info_out) info_out[b] = eig_info[b];
    if (n_eig_out) n_eig_out[b] = n_eig;
    if (n_solve_out) n_solve_out[b] = base_solves + extra_solves[b];
    if (n_lu_out) n_lu_out[b] = base_lu + extra_solves[b];  // the flagged samples' extra solve is an LU here too
}

struct DModes {
    bool analytic = true;
    bool fzb = false;
    zc* q = nullptr;
    zc* p = nullptr;
    zc* W = nullptr;
    zc* V = nullptr;
};

// tp, tm of an interface with at least one general side (include/stablercwa/rcwa1d.hpp:664-692).
// The lower side's W and V are consumed (factored in place): this interface is their last use.
void interface_matching(Batch& c, const DModes& up, const DModes& low, zc*& tp, zc*& tm) {
    const long long nd = (long long)c.B * c.nn();
    tp = c.dense();
    tm = c.dense();
    if (low.analytic) {
        zc* inv_p = c.vec();
        LAUNCH(reciprocal_kernel, nblocks((long long)c.B * c.n), kTpb, c.st, (long long)c.B * c.n, low.p, inv_p);
        LAUNCH(tp_tm_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, up.W, up.V, inv_p, tp, tm);
        c.mem->free(inv_p);
        return;
    }
    zc *mm, *nn;
    if (up.analytic) {
        mm = solve(c, low.W, true, RHS_IDENTITY, nullptr);
        nn = solve(c, low.V, true, RHS_DIAG, up.p);
    } else {
        mm = solve(c, low.W, true, RHS_DENSE, up.W);
        nn = solve(c, low.V, true, RHS_DENSE, up.V);
    }
    LAUNCH(tp_tm_kernel, nblocks(nd), kTpb, c.st, c.B, c.n, mm, nn, nullptr, tp, tm);
    c.mem->free(mm);
    c.mem->free(nn);
}

// include/stablercwa/rcwa1d.hpp:694-712
DSBlock interface_block(Batch& c, const DModes& up, const DModes& low) {
    DSBlock s;
    if (up.analytic && low.analytic) {
        const long long nv = (long long)c.B * c.n;
        s.Tdd = {KDiag, c.vec()};
        s.Rdu = {KDiag, c.vec()};
        s.Rud = {KDiag, c.vec()};
        s.Tuu = {KDiag, c.vec()};
        LAUNCH(diagonal_interface_kernel, nblocks(nv), kTpb, c.st, nv, up.p, low.p, s.Tdd.p, s.Rdu.p, s.Rud.p, s.Tuu.p);
        return s;
    }
    zc *tp, *tm;
    interface_matching(c, up, low, tp, tm);
    zc* tpi = solve(c, tp, false, RHS_IDENTITY, nullptr);
    zc* rdu = gemm(c, tm, c.nn(), tpi, nullptr, 1.0, 0.0);
    gemm(c, rdu, c.nn(), tm, tp, -1.0, 1.0, tp);  // tp -= rdu tm: tp is now Tdd
    zc* rud = gemm(c, tpi, c.nn(), tm, nullptr, -1.0, 0.0);
    c.mem->free(tm);
    s.Tdd = {KDense, tp};
    s.Rdu = {KDense, rdu};
    s.Rud = {KDense, rud};
    s.Tuu = {KDense, tpi};
    return s;
}

}  // namespace

// ---------------------------------------------------------------- validation

namespace {
void check_index(rcwa_complex n) {
    const bool fin = std::isfinite(n.re) && std::isfinite(n.im);
    if (!fin || std::abs(std::complex<double>(n.re, n.im)) == 0.0 || n.re < 0.0 || n.im < 0.0)
        throw EngineError{RCWA_EINVAL, "rcwa: refractive index must be finite, nonzero, with Re n >= 0 and Im n >= 0"};
}
}  // namespace

// include/stablercwa/rcwa1d.hpp:191-229 and :859-866
void validate1d(const rcwa_stack1d& stack, const rcwa_point1d* h_points, int n_points, int M, int pol) {
    if (M < 0 || M > (2147483647 - 1) / 4) throw EngineError{RCWA_EINVAL, "rcwa: invalid truncation order M"};
    if (pol != RCWA_TE && pol != RCWA_TM) throw EngineError{RCWA_EINVAL, "rcwa: polarization must be TE or TM"};
    if (!std::isfinite(stack.period) || stack.period <= 0.0)
        throw EngineError{RCWA_EINVAL, "rcwa: wavelength and period must be finite and positive"};
    if (h_points)
        for (int p = 0; p < n_points; ++p) {
            if (!std::isfinite(h_points[p].wavelength) || h_points[p].wavelength <= 0.0)
                throw EngineError{RCWA_EINVAL, "rcwa: wavelength and period must be finite and positive"};
            if (!std::isfinite(h_points[p].theta_deg) || std::fabs(h_points[p].theta_deg) >= 90.0)
                throw EngineError{RCWA_EINVAL, "rcwa: incidence angle must lie strictly between -90 and 90 degrees"};
        }
    check_index(stack.nI);
    if (stack.nI.im != 0.0 || stack.nI.re <= 0.0)
        throw EngineError{RCWA_EINVAL, "rcwa: the incident medium must have a real positive index"};
    check_index(stack.nII);
    if (stack.n_layers < 0 || (stack.n_layers > 0 && !stack.layers))
        throw EngineError{RCWA_EINVAL, "rcwa: layer array missing"};
    for (int k = 0; k < stack.n_layers; ++k) {
        const rcwa_layer1d& L = stack.layers[k];
        if (L.fourier_method != 0 && L.fourier_method != 1) throw EngineError{RCWA_EINVAL, "rcwa: invalid Fourier method"};
        if (L.fft_samples < 0 || L.fft_samples > kMaxFFTSamples)
            throw EngineError{RCWA_EINVAL, "rcwa: fft_samples must be 0..4194304 (0 for automatic)"};
        if (!L.homogeneous && L.fourier_method == 1 && M >= 0) (void)resolve_fft_samples(M, L.fft_samples);
        if (!std::isfinite(L.d) || L.d < 0.0) throw EngineError{RCWA_EINVAL, "rcwa: layer thickness must be finite and >= 0"};
        if (L.homogeneous) {
            check_index(L.n);
            continue;
        }
        if (L.n_segments < 1 || !L.edges || !L.n_values)
            throw EngineError{RCWA_EINVAL, "rcwa: a grating layer needs K indices and K+1 edges"};
        for (int j = 0; j <= L.n_segments; ++j)
            if (!std::isfinite(L.edges[j]) || (j > 0 && L.edges[j] <= L.edges[j - 1]))
                throw EngineError{RCWA_EINVAL, "rcwa: grating edges must be finite and strictly increasing"};
        if (std::fabs((L.edges[L.n_segments] - L.edges[0]) - stack.period) > 1e-10 * stack.period)
            throw EngineError{RCWA_EINVAL, "rcwa: grating edges must span exactly one period"};
        for (int j = 0; j < L.n_segments; ++j) check_index(L.n_values[j]);
    }
}


// ---------------------------------------------------------------- the solve

namespace {

// The field harmonics of one chunk (PlanarFieldSampler::sample, include/stablercwa/rcwa1d_fields.hpp:107-189):
// depths grouped by region like field_depth_groups (rcwa_fields.hpp:253-279), S and U per group, W S and
// V U for eigen-decomposed layers, Ez from [[eps]]^{-1} (TM), then scattered per component. Failed
// samples get NaN fields (the reference leaves their context unavailable).
void sample_fields(Batch& c, const FieldSpec& f, const rcwa_stack1d& stack, int pol, int M, int p0,
                   const std::vector<DModes>& modes, const std::vector<zc*>& capW, const std::vector<zc*>& capV,
                   const std::vector<const zc*>& einv, const std::vector<zc*>& ap, const std::vector<zc*>& am,
                   const double* kx, const double* k0, const zc* R, const zc* T) {
    const cudaStream_t st = c.st;
    DeviceScratch& mem = *c.mem;
    const int B = c.B, n = c.n, L = stack.n_layers, nz = (int)f.zs.size();
    if (nz == 0) return;
    const long long nn = (long long)n * n;
    zc* out = f.out + (size_t)p0 * 6 * n * nz;
    RCWA_CUDA(cudaMemsetAsync(out, 0, (size_t)B * 6 * n * nz * sizeof(zc), st));
    std::vector<double> ztop(L), zbot(L);
    double z = 0.0;
    bool finite_layer = false;
    for (int j = 0; j < L; ++j) {
        ztop[j] = z;
        z += stack.layers[j].d;
        zbot[j] = z;
        finite_layer = finite_layer || stack.layers[j].d > 0.0;
    }
    const double zb = z;
    std::vector<std::vector<int>> groups(L + 2);  // 0 incident side, 1 exit side, 2 + j layer j
    for (int iz = 0; iz < nz; ++iz) {
        const double zz = f.zs[iz];
        int g = zz < 0.0 ? 0 : 1;
        if (zz >= 0.0 && zz <= zb && finite_layer)
            for (int j = 0; j < L; ++j)
                if (zz <= zbot[j] + 1e-12) {
                    g = 2 + j;
                    break;
                }
        groups[g].push_back(iz);
    }
    const cd nI{stack.nI.re, stack.nI.im}, nII{stack.nII.re, stack.nII.im};
    for (int g = 0; g < L + 2; ++g) {
        const std::vector<int>& cols = groups[g];
        if (cols.empty()) continue;
        const int cnt = (int)cols.size();
        const long long tot = (long long)B * n * cnt;
        std::vector<double> local(cnt);
        for (int k = 0; k < cnt; ++k) local[k] = g >= 2 ? f.zs[cols[k]] - ztop[g - 2] : f.zs[cols[k]];
        double* d_z = mem.get<double>(cnt);
        int* d_cols = mem.get<int>(cnt);
        RCWA_CUDA(cudaMemcpyAsync(d_z, local.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_cols, cols.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, st));
        zc* S = mem.get<zc>(tot);
        zc* U = mem.get<zc>(tot);
        zc* Ez = pol == RCWA_TM ? mem.get<zc>(tot) : nullptr;
        if (g < 2) {
            const DModes& m = g == 0 ? modes[0] : modes[L + 1];
            LAUNCH(region_su_kernel, nblocks(tot), kTpb, st, B, n, M, cnt, d_z, g == 0 ? -1 : -2, zb, k0, m.q, m.p, R, T, S, U);
            if (Ez) {
                const cd ie = 1.0 / (g == 0 ? nI * nI : nII * nII);
                LAUNCH(ez_scalar_kernel, nblocks(tot), kTpb, st, tot, n, kx, cnt, S, zc{ie.real(), ie.imag()}, Ez);
            }
        } else {
            const int j = g - 2;
            const DModes& m = modes[j + 1];
            LAUNCH(layer_su_kernel, nblocks(tot), kTpb, st, B, n, cnt, d_z, stack.layers[j].d, k0, ap[j], am[j], m.q,
                   m.fzb ? 1 : 0, m.analytic ? m.p : nullptr, S, U);
            if (!m.analytic) {
                zc* S2 = mem.get<zc>(tot);
                zc* U2 = mem.get<zc>(tot);
                launch_zgemm(st, n, cnt, n, B, capW[j], n, nn, S, n, (long long)n * cnt, nullptr, 0, S2, n, (long long)n * cnt,
                             1.0, 0.0);
                launch_zgemm(st, n, cnt, n, B, capV[j], n, nn, U, n, (long long)n * cnt, nullptr, 0, U2, n, (long long)n * cnt,
                             1.0, 0.0);
                mem.free(S);
                mem.free(U);
                S = S2;
                U = U2;
            }
            if (Ez) {
                if (m.analytic) {
                    const cd nl{stack.layers[j].n.re, stack.layers[j].n.im};
                    const cd ie = 1.0 / (nl * nl);
                    LAUNCH(ez_scalar_kernel, nblocks(tot), kTpb, st, tot, n, kx, cnt, S, zc{ie.real(), ie.imag()}, Ez);
                } else {
                    zc* ks = mem.get<zc>(tot);
                    LAUNCH(kx_rows_kernel, nblocks(tot), kTpb, st, tot, n, kx, cnt, S, ks);
                    launch_zgemm(st, n, cnt, n, B, einv[j], n, 0, ks, n, (long long)n * cnt, nullptr, 0, Ez, n,
                                 (long long)n * cnt, 1.0, 0.0);
                    mem.free(ks);
                }
            }
        }
        LAUNCH(field_out_kernel, nblocks(tot), kTpb, st, B, n, cnt, nz, d_cols, pol, kx, S, U, Ez, out);
        RCWA_CUDA(stream_wait(st));  // the host vectors of this group end here
        for (void* p : {(void*)S, (void*)U, (void*)Ez, (void*)d_z, (void*)d_cols})
            if (p) mem.free(p);
    }
    LAUNCH(nan_fields_kernel, nblocks((long long)B * 6 * n * nz), kTpb, st, B, 6LL * n * nz, c.fail, out);
}

}  // namespace

void solve1d_device(cudaStream_t st, const rcwa_stack1d& stack, const double* d_s, const double* d_wl, int n_points,
                    int M, int pol, const Options& opt, const rcwa_result1d& d_out, size_t chunk_bytes, const FieldSpec* fields) {
    const int n = 2 * M + 1;
    const long long nn = (long long)n * n;
    const int L = stack.n_layers;
    if (n_points <= 0) return;
    std::vector<int> grating;
    for (int k = 0; k < L; ++k)
        if (!stack.layers[k].homogeneous) grating.push_back(k);
    const bool pure_films = grating.empty();
    const bool reduced = reduced_seams_enabled();
    const zc nI{stack.nI.re, stack.nI.im}, nII{stack.nII.re, stack.nII.im};

    // Per-layer, sample-independent operators: Toeplitz coefficients; for TM the inverse of [[eps]] and
    // of [[1/eps]] and [[1/eps]] itself (include/stablercwa/rcwa1d.hpp:432-468).
    DeviceScratch persist(st);
    int* layer_fail = persist.zeros<int>(1);
    struct LayerData {
        zc* c_eps = nullptr;
        zc* inv_eps = nullptr;   // [[1/eps]] (TM)
        zc* einv = nullptr;      // [[eps]]^{-1} (TM)
        zc* cinv = nullptr;      // [[1/eps]]^{-1} (TM)
        bool herm = false;       // Hermitian operators: the Hermitian eigensolver path
        zc* einv_h = nullptr;    // Hermitian part of [[eps]]^{-1} (TM, herm)
        zc *Lchol = nullptr, *Linv = nullptr, *LinvH = nullptr;  // L, L^{-1}, L^{-H} of [[1/eps]] = L L^H (TM, herm)
        zc* pencil[4] = {nullptr, nullptr, nullptr, nullptr};    // constant parts of L^-1 (Kx E Kx - I) L^-H
    };
    const bool try_herm = hermitian_path_enabled(opt);
    std::vector<LayerData> ld(L);
    for (int k : grating) {
        const rcwa_layer1d& Ly = stack.layers[k];
        std::vector<double> edges(Ly.edges, Ly.edges + Ly.n_segments + 1);
        std::vector<cd> eps, inv;
        for (int j = 0; j < Ly.n_segments; ++j) {
            const cd nv{Ly.n_values[j].re, Ly.n_values[j].im};
            eps.push_back(nv * nv);
            inv.push_back(1.0 / (nv * nv));
        }
        ld[k].c_eps = layer_coefficients(st, persist, edges, eps, stack.period, M, Ly.fourier_method, Ly.fft_samples,
                                         layer_fail);
        ld[k].herm = try_herm && real_profile(eps) && real_profile(inv);
        if (ld[k].herm) make_hermitian_coefficients(st, ld[k].c_eps, M);
        if (pol == RCWA_TM) {
            zc* c_inv = layer_coefficients(st, persist, edges, inv, stack.period, M, Ly.fourier_method, Ly.fft_samples,
                                           layer_fail);
            if (ld[k].herm) {
                make_hermitian_coefficients(st, c_inv, M);
                toeplitz_cholesky_inverse(st, c_inv, M, persist, layer_fail, ld[k].Lchol, ld[k].Linv, ld[k].LinvH);
            }
            zc* E = persist.get<zc>(nn);
            ld[k].inv_eps = persist.get<zc>(nn);
            LAUNCH(toeplitz_kernel, nblocks(nn), kTpb, st, M, ld[k].c_eps, E);
            LAUNCH(toeplitz_kernel, nblocks(nn), kTpb, st, M, c_inv, ld[k].inv_eps);
            zc* C = persist.get<zc>(nn);
            RCWA_CUDA(cudaMemcpyAsync(C, ld[k].inv_eps, nn * sizeof(zc), cudaMemcpyDeviceToDevice, st));
            ld[k].einv = persist.get<zc>(nn);
            ld[k].cinv = persist.get<zc>(nn);
            launch_lu_solve(st, n, n, 1, E, nn, E, nn, RHS_IDENTITY, nullptr, nn, ld[k].einv, nn, layer_fail);
            launch_lu_solve(st, n, n, 1, C, nn, C, nn, RHS_IDENTITY, nullptr, nn, ld[k].cinv, nn, layer_fail);
            if (ld[k].herm) {
                ld[k].einv_h = persist.get<zc>(nn);
                LAUNCH(hermitian_part_kernel, nblocks(nn), kTpb, st, n, ld[k].einv, ld[k].einv_h);
                pencil_parts(st, persist, M, ld[k].einv_h, ld[k].Linv, ld[k].LinvH, ld[k].pencil);
            }
        }
    }

    std::vector<const zc*> ld_einv(L, nullptr);  // [[eps]]^{-1} of TM grating layers, for Ez in the fields
    for (int k = 0; k < L; ++k) ld_einv[k] = ld[k].einv;
    // chunk size: rough upper bound of live device bytes per sample
    const long long per_sample = 16LL * (nn * (12 + 4 * (long long)grating.size()) + (long long)n * (8LL * (L + 2) + 64)) +
                                 eig_workspace_bytes(n, 1);
    long long chunk = chunk_bytes > 0 ? (long long)chunk_bytes / std::max(1LL, per_sample) : n_points;
    chunk = std::max(1LL, std::min<long long>(chunk, n_points));

    for (int p0 = 0; p0 < n_points; p0 += (int)chunk) {
        const int B = (int)std::min<long long>(chunk, n_points - p0);
        DeviceScratch mem(st);
        Batch c{st, &mem, B, n, M, nullptr, nullptr};
        c.fail = mem.zeros<int>(B);
        c.extra_solves = mem.zeros<int>(B);
        int* eig_info = mem.zeros<int>(B);
        int* zero_any = mem.zeros<int>(1);
        const long long nv = (long long)B * n, nd = (long long)B * nn;

        double* kx = mem.get<double>(nv);
        double* k0 = mem.get<double>(B);
        LAUNCH(kx_kernel, nblocks(nv), kTpb, st, B, M, d_s + p0, d_wl + p0, stack.period, kx);
        LAUNCH(k0_kernel, nblocks(B), kTpb, st, B, d_wl + p0, k0);

        // ---- 1. modes of every region (region 0: nI, region j+1: layer j, region L+1: nII)
        std::vector<DModes> modes(L + 2);
        std::vector<zc*> cap_W(L, nullptr), cap_V(L, nullptr);  // retained W, V of grating layers (fields)
        std::vector<DOp> r_below(L);                             // reflection below each layer (fields)
        // the analytic modes of every homogeneous region in one launch, region r at offset r * B * n
        zc* aq = mem.get<zc>((size_t)(L + 2) * nv);
        zc* ap = mem.get<zc>((size_t)(L + 2) * nv);
        {
            std::vector<AnalyticRegion> regs(L + 2);
            regs[0] = {zc{stack.nI.re, stack.nI.im}, 0, 1};
            regs[L + 1] = {nII, 0, 1};
            for (int k = 0; k < L; ++k) {
                const rcwa_layer1d& Ly = stack.layers[k];
                regs[k + 1] = Ly.homogeneous ? AnalyticRegion{zc{Ly.n.re, Ly.n.im}, 1, 1} : AnalyticRegion{zc{0.0, 0.0}, 0, 0};
            }
            AnalyticRegion* d_regs = mem.get<AnalyticRegion>(regs.size());
            RCWA_CUDA(cudaMemcpyAsync(d_regs, regs.data(), regs.size() * sizeof(AnalyticRegion), cudaMemcpyHostToDevice, st));
            LAUNCH(analytic_modes_all_kernel, nblocks((long long)(L + 2) * nv), kTpb, st, L + 2, B, n, kx, d_regs, pol, aq, ap);
            for (int r = 0; r < L + 2; ++r)
                if (regs[r].active) {
                    modes[r].analytic = true;
                    modes[r].fzb = regs[r].fzb != 0;
                    modes[r].q = aq + (long long)r * nv;
                    modes[r].p = ap + (long long)r * nv;
                }
        }

        if (!grating.empty()) {
            zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(n, B) / sizeof(zc)) + 1);
            int* info = mem.get<int>(B);
            double* resid = nullptr;
            if (opt.diagnostics) resid = mem.zeros<double>(B);
            for (int k : grating) {
                // 1a. layer matrix
                const bool herm = ld[k].herm;
                zc* A = c.dense();
                zc* mid = nullptr;
                if (pol == RCWA_TE) {
                    LAUNCH(assemble_te_kernel, nblocks(nd), kTpb, st, B, M, ld[k].c_eps, kx, A);
                } else {
                    if (herm) {
                        // the pencil (Kx E Kx - I, [[1/eps]]) as the Hermitian L^{-1} (Kx E Kx - I) L^{-H}, from the
                        // layer's constant parts
                        LAUNCH(pencil_combine_kernel, nblocks(nd), kTpb, st, B, n, ld[k].pencil[0], ld[k].pencil[1],
                               ld[k].pencil[2], ld[k].pencil[3], d_s + p0, d_wl + p0, stack.period, A);
                        if (opt.diagnostics) {  // the residual is taken on [[1/eps]]^{-1} mid, the reference's A
                            mid = c.dense();
                            LAUNCH(tm_middle_kernel, nblocks(nd), kTpb, st, B, n, ld[k].einv_h, kx, mid);
                        }
                    } else {
                        mid = c.dense();
                        LAUNCH(tm_middle_kernel, nblocks(nd), kTpb, st, B, n, ld[k].einv, kx, mid);
                        gemm(c, ld[k].cinv, 0, mid, nullptr, 1.0, 0.0, A);
                    }
                    c.n_solve += 2;  // the reference forms A with two dense solves per sample
                }
                LAUNCH(finite_check_kernel, nblocks(nd), kTpb, st, B, nn, A, c.fail);
                // 1b. eigen-decomposition
                DModes& m = modes[k + 1];
                m.analytic = false;
                m.fzb = true;
                zc* lam = c.vec();
                m.W = c.dense();
                zc* ly = nullptr;  // [[1/eps]] W (TM, herm)
                if (herm) {
                    launch_eig_herm(st, n, B, A, nn, lam, m.W, info, ws, opt.eps, opt.max_iter, opt.eig_group);
                    if (pol == RCWA_TM) {
                        // x = L^{-H} y, unit 2-norm like the general solver's vectors, and [[1/eps]] x = L y with the
                        // same column scale (V = [[1/eps]] W q without a full product)
                        zc* y = m.W;
                        m.W = c.dense();
                        ly = c.dense();
                        launch_zgemm(st, n, n, n, B, ld[k].LinvH, n, 0, y, n, nn, nullptr, 0, m.W, n, nn, 1.0, 0.0,
                                     nullptr, 1, TRI_A_UPPER);
                        launch_zgemm(st, n, n, n, B, ld[k].Lchol, n, 0, y, n, nn, nullptr, 0, ly, n, nn, 1.0, 0.0, nullptr, 1,
                                     TRI_A_LOWER);
                        mem.free(y);
                        LAUNCH(normalize_cols_kernel, warp_blocks(nv), 128, st, B, n, m.W, ly);
                        if (opt.diagnostics) gemm(c, ld[k].cinv, 0, mid, nullptr, 1.0, 0.0, A);  // the solve's A
                    }
                } else {
                    launch_eig(st, n, B, A, nn, lam, m.W, info, nullptr, ws, opt.eps, opt.max_iter, opt.eig_group);
                }
                if (mid) mem.free(mid);
                LAUNCH(eig_info_kernel, nblocks(B), kTpb, st, B, info, eig_info, c.fail);
                if (opt.diagnostics) {
                    zc* av = gemm(c, A, nn, m.W, nullptr, 1.0, 0.0);
                    LAUNCH(eig_residual_kernel, warp_blocks(B), 128, st, B, n, A, av, m.W, lam, info, resid);
                    mem.free(av);
                }
                mem.free(A);
                // 1c. q = branch(sqrt(lambda)), V = W q (TE) or [[1/eps]] W q (TM)
                m.q = c.vec();
                zc* bq = c.vec();
                int* zf = mem.zeros<int>(B);
                LAUNCH(eig_modes_q_kernel, nblocks(nv), kTpb, st, B, n, lam, m.q, bq, zf);
                m.V = c.dense();
                if (pol == RCWA_TE) {
                    LAUNCH(scale_cols_kernel, nblocks(nd), kTpb, st, B, n, m.W, bq, m.V, nullptr, 1);
                } else if (ly) {
                    LAUNCH(scale_cols_kernel, nblocks(nd), kTpb, st, B, n, ly, bq, m.V, nullptr, 1);
                    mem.free(ly);
                } else {
                    zc* cw = gemm(c, ld[k].inv_eps, 0, m.W, nullptr, 1.0, 0.0);
                    LAUNCH(scale_cols_kernel, nblocks(nd), kTpb, st, B, n, cw, bq, m.V, nullptr, 1);
                    mem.free(cw);
                }
                mem.free(lam);
                mem.free(bq);
                if (fields) {  // the interface above consumes W and V; the field sampler needs them after
                    cap_W[k] = c.dense();
                    cap_V[k] = c.dense();
                    RCWA_CUDA(cudaMemcpyAsync(cap_W[k], m.W, nd * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                    RCWA_CUDA(cudaMemcpyAsync(cap_V[k], m.V, nd * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                }
            }
            if (opt.diagnostics)
                RCWA_CUDA(cudaMemcpyAsync(d_out.max_eig_residual + p0, resid, B * sizeof(double), cudaMemcpyDeviceToDevice, st));
            mem.free(ws);
        } else if (opt.diagnostics && d_out.max_eig_residual) {
            RCWA_CUDA(cudaMemsetAsync(d_out.max_eig_residual + p0, 0, B * sizeof(double), st));
        }

        // ---- 2. bottom-up recursion (include/stablercwa/rcwa1d.hpp:965-987)
        const int block_count = 2 * L + 1;
        std::vector<DOp> g(block_count);
        DOp r;  // Zero: nothing comes up from the exit medium
        // The run of homogeneous regions at the bottom (every block diagonal) in one launch when no fields are
        // captured: blocks [b_stop, block_count) (film_run_kernel), their g kept for one downward launch.
        int b_stop = block_count;
        zc* g_run = nullptr;
        if (!fields) {
            int b = block_count - 1;
            while (b >= 1) {
                const int j = b / 2;
                if (!(b % 2 == 0 ? (modes[j].analytic && modes[j + 1].analytic) : modes[j + 1].analytic)) break;
                --b;
            }
            if (block_count - 1 - b >= 2) b_stop = b + 1;
        }
        if (b_stop < block_count) {
            const int nblk = block_count - b_stop;
            std::vector<FilmBlock> fb(nblk);
            for (int t = 0; t < nblk; ++t) {
                const int bb = block_count - 1 - t, j = bb / 2;
                fb[t] = bb % 2 == 0 ? FilmBlock{0, j, j + 1, 0, 0.0}
                                    : FilmBlock{1, j + 1, 0, modes[j + 1].fzb ? 1 : 0, stack.layers[j].d};
            }
            FilmBlock* d_fb = mem.get<FilmBlock>(nblk);
            RCWA_CUDA(cudaMemcpyAsync(d_fb, fb.data(), nblk * sizeof(FilmBlock), cudaMemcpyHostToDevice, st));
            g_run = mem.get<zc>((size_t)nblk * nv);
            zc* rv = c.vec();
            LAUNCH(film_run_kernel, nblocks(nv), kTpb, st, B, n, nblk, d_fb, aq, ap, k0, g_run, rv, c.fail);
            r = {KDiag, rv};
        }
        for (int b = b_stop - 1; b >= 1; --b) {
            const int j = b / 2;
            if (b % 2 == 0 && modes[j].analytic && modes[j + 1].analytic && r.kind != KDense) {
                // Fresnel block between two analytic regions stacked on a diagonal (or zero) reflection
                DSBlock blk = interface_block(c, modes[j], modes[j + 1]);
                zc* gv = c.vec();
                zc* rv = c.vec();
                LAUNCH(stack_on_diag_kernel, nblocks(nv), kTpb, st, nv, blk.Tdd.p, blk.Rdu.p, blk.Rud.p, blk.Tuu.p,
                       r.kind == KZero ? nullptr : r.p, gv, rv);
                mem.free(blk.Tdd.p);
                mem.free(blk.Rdu.p);
                mem.free(blk.Rud.p);
                mem.free(blk.Tuu.p);
                if (r.kind == KDiag) mem.free(r.p);
                g[b] = {KDiag, gv};
                r = {KDiag, rv};
                continue;
            }
            if (b % 2 == 0 && reduced && modes[j].analytic && !modes[j + 1].analytic && r.kind == KDense) {
                // a film (or the incident medium's counterpart) over a grating
                Seam seam = analytic_over_dense_seam(c, modes[j + 1].W, modes[j + 1].V, nullptr, modes[j].p, r);
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
                Seam seam = stack_on(c, std::move(blk), r);
                g[b] = seam.g;
                r = seam.r;
                continue;
            }
            // propagation through layer j (include/stablercwa/rcwa1d.hpp:751-784)
            if (fields) {  // the reflection seen below layer j's bottom (rcwa1d.hpp:981)
                r_below[j].kind = r.kind;
                if (r.kind != KZero) {
                    const size_t cnt = r.kind == KDiag ? (size_t)nv : (size_t)nd;
                    r_below[j].p = mem.get<zc>(cnt);
                    RCWA_CUDA(cudaMemcpyAsync(r_below[j].p, r.p, cnt * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                }
            }
            const DModes& m = modes[j + 1];
            zc* x = c.vec();
            zc* refl = c.vec();
            int* hz = mem.zeros<int>(B);
            LAUNCH(propagation_kernel, nblocks(nv), kTpb, st, B, n, m.q, k0, stack.layers[j].d, m.fzb ? 1 : 0, x, refl, hz,
                   c.fail);
            if (r.kind != KDense) {
                // every operator diagonal: k = Rdu r is zero unless q == 0 somewhere, which the diagonal
                // recurrence evaluates exactly as the reference's Zero path would
                zc* gv = c.vec();
                zc* rv = c.vec();
                LAUNCH(stack_on_diag_kernel, nblocks(nv), kTpb, st, nv, x, refl, refl, x, r.kind == KZero ? nullptr : r.p, gv, rv);
                g[b] = {KDiag, gv};
                r = {KDiag, rv};
                continue;
            }
            // dense r: g = Tdd (diagonal) and r' = x r x, except for samples with an exact q == 0 in this
            // layer, which take the dense branch g = (I - Rdu r)^{-1} Tdd, r' = Rud + Tuu r g.
            zc* rn = c.dense();
            LAUNCH(scale_both_kernel, nblocks(nd), kTpb, st, B, n, r.p, x, x, rn, hz, 1);
            {
                int any = 0;
                const unsigned rb = nblocks(B);
                // reduce the per-sample flags into one word and read it back
                RCWA_CUDA(cudaMemsetAsync(zero_any, 0, sizeof(int), st));
                LAUNCH(any_flag_kernel, rb, kTpb, st, B, hz, zero_any);
                RCWA_CUDA(cudaMemcpyAsync(&any, zero_any, sizeof(int), cudaMemcpyDeviceToHost, st));
                RCWA_CUDA(stream_wait(st));
                if (any) {
                    zc* k = c.dense();
                    LAUNCH(scale_rows_kernel, nblocks(nd), kTpb, st, B, n, r.p, refl, k, hz, 0);
                    LAUNCH(identity_minus_kernel, nblocks(nd), kTpb, st, B, n, k, hz, 0);
                    zc* td = c.mem->zeros<zc>((size_t)nd);
                    LAUNCH(diag_to_dense_kernel, nblocks(nd), kTpb, st, B, n, x, td, hz, 0);
                    zc* gd = c.dense();
                    launch_lu_solve(st, n, n, B, k, nn, k, nn, RHS_DENSE, td, nn, gd, nn, c.fail, hz, 0);
                    LAUNCH(inc_flagged_kernel, rb, kTpb, st, B, hz, c.extra_solves);
                    zc* y = gemm(c, r.p, nn, gd, nullptr, 1.0, 0.0, nullptr, hz, 0);
                    LAUNCH(scale_rows_kernel, nblocks(nd), kTpb, st, B, n, y, x, rn, hz, 0);
                    LAUNCH(add_diag_kernel, nblocks(nv), kTpb, st, B, n, rn, refl, hz, 0);
                    mem.free(k);
                    mem.free(td);
                    mem.free(y);
                    g[b] = {KDiag, x, gd, hz};
                } else {
                    g[b] = {KDiag, x};
                }
            }
            r = {KDense, rn};
        }

        // ---- 3. top interface, only column M (include/stablercwa/rcwa1d.hpp:714-746, :989-1023)
        zc* down = nullptr;
        zc* Rv = nullptr;
        if (reduced && modes[0].analytic && !modes[1].analytic && r.kind == KDense) {
            // Analytic incident medium over a dense region with the dense reflection r below the interface:
            // with W (I + r) d_b = d_a + u_a, V (I - r) d_b = p0 (d_a - u_a) and d_a = e_M,
            //     (p0 W + V + (p0 W - V) r) d_b = 2 p0_M e_M,    R = u_a = W (d_b + r d_b) - e_M:
            // one LU with one right-hand side for the reference's three with n (W^-1, V^-1 p0, tp^-1) and one
            // with a single column; no division by p0, so an order grazing in the incident medium is fine.
            zc* P = c.dense();
            zc* Q = c.dense();
            LAUNCH(analytic_pq_kernel, nblocks(nd), kTpb, st, B, n, modes[1].W, modes[1].V, nullptr, modes[0].p, P, Q);
            gemm(c, Q, nn, r.p, P, 1.0, 1.0, P);
            mem.free(Q);
            zc* rhs = c.vec();
            LAUNCH(top_rhs_kernel, nblocks(nv), kTpb, st, B, n, M, modes[0].p, rhs);
            down = solve(c, P, true, RHS_DENSE, rhs, 1);
            c.n_solve += 3;
            mem.free(P);
            mem.free(rhs);
            zc* t = c.vec();
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, r.p, down, down, t, 1.0, 1.0);
            Rv = c.vec();
            LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, modes[1].W, t, nullptr, Rv, 1.0, 0.0);
            LAUNCH(sub_incident_kernel, nblocks(B), kTpb, st, B, n, M, Rv);
            mem.free(t);
        } else {
            zc* tdd = c.vec();
            zc* rud = c.vec();
            DOp topRdu, topTuu;
            if (modes[0].analytic && modes[1].analytic) {
                zc* Tdd = c.vec();
                zc* Rdu = c.vec();
                zc* Rud = c.vec();
                zc* Tuu = c.vec();
                LAUNCH(diagonal_interface_kernel, nblocks(nv), kTpb, st, nv, modes[0].p, modes[1].p, Tdd, Rdu, Rud, Tuu);
                LAUNCH(top_diag_vectors_kernel, nblocks(nv), kTpb, st, B, n, M, Tdd, Rud, tdd, rud);
                topRdu = {KDiag, Rdu};
                topTuu = {KDiag, Tuu};
            } else {
                zc *tp, *tm;
                interface_matching(c, modes[0], modes[1], tp, tm);
                zc* tpi = solve(c, tp, false, RHS_IDENTITY, nullptr);
                zc* rdu = gemm(c, tm, nn, tpi, nullptr, 1.0, 0.0);
                zc* tm_e = c.vec();
                LAUNCH(col_extract_kernel, nblocks(nv), kTpb, st, B, n, tm, M, tm_e, 1, 0);
                LAUNCH(col_extract_kernel, nblocks(nv), kTpb, st, B, n, tp, M, tdd, 1, 0);
                LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, rdu, tm_e, tdd, tdd, -1.0, 1.0);
                LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, tpi, tm_e, nullptr, rud, -1.0, 0.0);
                mem.free(tp);
                mem.free(tm);
                topRdu = {KDense, rdu};
                topTuu = {KDense, tpi};
            }
            DOp k = op_mul(c, topRdu, r);
            down = tdd;
            if (k.kind == KDiag) {
                LAUNCH(vec_div_one_minus_kernel, nblocks(nv), kTpb, st, B, n, 1, down, k.p);
            } else if (k.kind == KDense) {
                LAUNCH(identity_minus_kernel, nblocks(nd), kTpb, st, B, n, k.p, nullptr, 1);
                down = solve(c, k.p, true, RHS_DENSE, tdd, 1);
            }
            // R = rud + Tuu (r down)
            zc* rdn = c.vec();
            LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 1, (int)r.kind, r.p, nullptr, nullptr, down, rdn);
            zc* back = c.vec();
            LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 1, (int)topTuu.kind, topTuu.p, nullptr, nullptr, rdn, back);
            LAUNCH(vec_add_kernel, nblocks(nv), kTpb, st, nv, back, rud);  // rud = back + rud
            Rv = rud;
        }
        // T = g[2L] ... g[1] down
        zc* cur = down;
        zc* nxt = c.vec();
        zc* seam_t = c.vec();
        std::vector<zc*> a_plus(L, nullptr), a_minus(L, nullptr);
        for (int b = 1; b < block_count; ++b) {
            const int j = b / 2;
            if (b == b_stop) {  // the fused bottom run: all of its blocks in one launch
                LAUNCH(film_push_kernel, nblocks(nv), kTpb, st, nv, block_count - b_stop, g_run, cur, nxt);
                std::swap(cur, nxt);
                break;
            }
            if (fields && b % 2 != 0) {  // amplitude at the layer's top (rcwa1d.hpp:1008-1012)
                a_plus[j] = c.vec();
                RCWA_CUDA(cudaMemcpyAsync(a_plus[j], cur, nv * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                if (pure_films) LAUNCH(clear_unexcited_kernel, nblocks(nv), kTpb, st, B, n, M, a_plus[j]);
            }
            if (g[b].kind == KSeam) {
                apply_seam(c, g[b], 1, cur, seam_t, nxt);
            } else {
                LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 1, (int)g[b].kind, g[b].p, g[b].alt, g[b].alt_flag,
                       cur, nxt);
            }
            std::swap(cur, nxt);
            if (fields && b % 2 != 0) {  // the reflection below applied at the layer's bottom (:1013-1020)
                zc* bottom = cur;
                if (pure_films) {
                    bottom = c.vec();
                    RCWA_CUDA(cudaMemcpyAsync(bottom, cur, nv * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                    LAUNCH(clear_unexcited_kernel, nblocks(nv), kTpb, st, B, n, M, bottom);
                }
                a_minus[j] = c.vec();
                LAUNCH(apply_g_kernel, warp_blocks(B), 128, st, B, n, 1, (int)r_below[j].kind, r_below[j].p, nullptr, nullptr,
                       bottom, a_minus[j]);
                if (pure_films) {
                    LAUNCH(clear_unexcited_kernel, nblocks(nv), kTpb, st, B, n, M, a_minus[j]);
                    mem.free(bottom);
                }
            }
        }
        zc* Tv = cur;

        // ---- 4. efficiencies, NaN fill, status
        LAUNCH(finalize_kernel, warp_blocks(B), 128, st, B, n, M, pol, pure_films ? 1 : 0, Rv, Tv, modes[0].q,
               modes[L + 1].q, k0, nI, nII, c.fail, reinterpret_cast<zc*>(d_out.R) + (long long)p0 * n,
               reinterpret_cast<zc*>(d_out.T) + (long long)p0 * n, d_out.DEr + (long long)p0 * n,
               d_out.DEt + (long long)p0 * n);
        LAUNCH(status_kernel, nblocks(B), kTpb, st, B, c.fail, eig_info, c.n_solve, c.n_lu, c.extra_solves,
               (int)grating.size(), d_out.status ? d_out.status + p0 : nullptr,
               d_out.eig_info ? d_out.eig_info + p0 : nullptr, d_out.n_eig ? d_out.n_eig + p0 : nullptr,
               d_out.n_dense_solve ? d_out.n_dense_solve + p0 : nullptr, d_out.n_lu ? d_out.n_lu + p0 : nullptr);
        if (fields && fields->layer_info)
            for (int k = 0; k < L; ++k)
                LAUNCH(zero_q_count_kernel, nblocks(B), kTpb, st, B, n, modes[k + 1].q, fields->layer_info + (size_t)p0 * L + k, L);
        if (fields) sample_fields(c, *fields, stack, pol, M, p0, modes, cap_W, cap_V, ld_einv, a_plus, a_minus, kx, k0,
                                  reinterpret_cast<zc*>(d_out.R) + (long long)p0 * n,
                                  reinterpret_cast<zc*>(d_out.T) + (long long)p0 * n);
        mem.release();
    }
    // A singular [[eps]] or [[1/eps]] (TM) fails every sample; checked once at the end.
    int lf = 0;
    RCWA_CUDA(cudaMemcpyAsync(&lf, layer_fail, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    if (lf) {
        // reference: the TM assembly solve throws NumericalFailure for every point
        const double nan = std::nan("");
        std::vector<double> nans((size_t)n_points * n * 2, nan);
        RCWA_CUDA(cudaMemcpyAsync(d_out.R, nans.data(), (size_t)n_points * n * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_out.T, nans.data(), (size_t)n_points * n * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_out.DEr, nans.data(), (size_t)n_points * n * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_out.DEt, nans.data(), (size_t)n_points * n * sizeof(double), cudaMemcpyHostToDevice, st));
        if (d_out.status) {
            std::vector<int> s(n_points, RCWA_SAMPLE_NUMERICAL);
            RCWA_CUDA(cudaMemcpyAsync(d_out.status, s.data(), n_points * sizeof(int), cudaMemcpyHostToDevice, st));
        }
        RCWA_CUDA(stream_wait(st));
    }
}

// ---------------------------------------------------------------- device-side point preparation

namespace {
__global__ void prepare_points_kernel(int N, const rcwa_point1d* __restrict__ pts, double nI, double* __restrict__ s,
                                      double* __restrict__ wl, int* __restrict__ bad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const double w = pts[p].wavelength, th = pts[p].theta_deg;
    if (!isfinite(w) || w <= 0.0 || !isfinite(th) || fabs(th) >= 90.0) atomicOr(bad, 1);
    wl[p] = w;
    s[p] = nI * sin(th * 3.141592653589793238462643383279502884 / 180.0);
}
}  // namespace

bool prepare_points_device(cudaStream_t st, const rcwa_point1d* d_points, int n_points, double nI, double* d_s,
                           double* d_wl) {
    DeviceScratch mem(st);
    int* bad = mem.zeros<int>(1);
    LAUNCH(prepare_points_kernel, nblocks(n_points), kTpb, st, n_points, d_points, nI, d_s, d_wl, bad);
    int h = 0;
    RCWA_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    return h == 0;
}

// One profile's coefficients for the C entry point rcwa_gpu_fourier_coefficients, validated like
// rcwa::fourier_coefficients_fft (include/stablercwa/fourier.hpp:49-63).
void fourier_coefficients_api(cudaStream_t st, const double* edges, const rcwa_complex* values, int K, double period,
                              int hmax, int method, int samples, rcwa_complex* out) {
    if (method != 0 && method != 1) throw EngineError{RCWA_EINVAL, "rcwa: invalid Fourier method"};
    if (method == 1 && (samples < 0 || samples > kMaxFFTSamples))
        throw EngineError{RCWA_EINVAL, "rcwa: fft_samples must be 0..4194304 (0 for automatic)"};
    if (hmax < 0 || (method == 1 && samples <= 2LL * hmax))
        throw EngineError{RCWA_EINVAL, "rcwa: FFT sample count must exceed 2*hmax"};
    if (!std::isfinite(period) || period <= 0 || K < 1 || !edges || !values || !out)
        throw EngineError{RCWA_EINVAL, "rcwa: FFT needs a positive period, K values and K+1 edges"};
    for (int j = 0; j <= K; ++j)
        if (!std::isfinite(edges[j]) || (j && edges[j] <= edges[j - 1]))
            throw EngineError{RCWA_EINVAL, "rcwa: FFT edges must be finite and strictly increasing"};
    if (std::abs((edges[K] - edges[0]) - period) > 1e-10 * period)
        throw EngineError{RCWA_EINVAL, "rcwa: FFT edges must span exactly one period"};
    std::vector<double> e(edges, edges + K + 1);
    std::vector<cd> v(K);
    for (int j = 0; j < K; ++j) {
        if (!std::isfinite(values[j].re) || !std::isfinite(values[j].im))
            throw EngineError{RCWA_EINVAL, "rcwa: FFT material values must be finite"};
        v[j] = cd{values[j].re, values[j].im};
    }
    DeviceScratch mem(st);
    zc* d = method == 0 ? closed_form_coefficients(st, mem, e, v, period, hmax)
                        : fft_coefficients_dev(st, mem, e, v, period, hmax, samples);
    RCWA_CUDA(cudaMemcpyAsync(out, d, (2 * (size_t)hmax + 1) * sizeof(zc), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
}

}  // namespace rcwa_gb300
