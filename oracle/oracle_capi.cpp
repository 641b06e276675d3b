// oracle_capi.cpp -- C entry points of the CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// Built into oracle/_build/liboracle.so by oracle/build.py. Loaded by tests/ (as the parity
// reference), by __graft_entry__.smoke() and by bench.py's CPU-baseline leg; never by the engine.
// The structs are the engine's public C ABI (include/stablercwa_gb300.h), so both sides read the
// same inputs.
#include <atomic>
#include <mutex>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../include/stablercwa_gb300.h"
#include "oracle_conical.hpp"
#include "oracle_rcwa2d.hpp"

using namespace oracle;

namespace {

cplx C(rcwa_complex z) { return {z.re, z.im}; }
rcwa_complex R(cplx z) { return {z.real(), z.imag()}; }

void put_error(char* err, size_t len, const std::string& msg) {
    if (!err || len == 0) return;
    std::strncpy(err, msg.c_str(), len - 1);
    err[len - 1] = '\0';
}

Stack1D to_stack(const rcwa_stack1d* s) {
    Stack1D out;
    out.nI = C(s->nI);
    out.nII = C(s->nII);
    out.period = s->period;
    for (int k = 0; k < s->n_layers; ++k) {
        const rcwa_layer1d& L = s->layers[k];
        Layer1D l;
        l.d = L.d;
        l.homogeneous = L.homogeneous != 0;
        l.n = C(L.n);
        if (!l.homogeneous && L.fourier_method != 0)
            throw InvalidArgument{"oracle: FFT-sampled coefficients are not restated here (the tests use the reference's outputs)"};
        if (!l.homogeneous) {
            for (int j = 0; j <= L.n_segments; ++j) l.edges.push_back(L.edges[j]);
            for (int j = 0; j < L.n_segments; ++j) l.n_values.push_back(C(L.n_values[j]));
        }
        out.layers.push_back(std::move(l));
    }
    return out;
}

r2d::Layer to_layer2d(const rcwa_layer2d& L) {
    r2d::Layer l;
    l.d = L.d;
    l.homogeneous = L.homogeneous != 0;
    l.n = C(L.n);
    if (!l.homogeneous) {
        for (int k = 0; k <= L.n_strips; ++k) l.y_edges.push_back(L.y_edges[k]);
        for (int k = 0; k < L.n_strips; ++k) {
            const rcwa_xprofile2d& xp = L.x_profiles[k];
            r2d::XProfile p;
            for (int j = 0; j <= xp.n_segments; ++j) p.edges.push_back(xp.edges[j]);
            for (int j = 0; j < xp.n_segments; ++j) p.n.push_back(C(xp.n_values[j]));
            l.strips.push_back(std::move(p));
        }
    }
    return l;
}

void put_mat(const Mat& m, rcwa_complex* out) {  // row-major, as the engine's operator export
    for (int i = 0; i < m.rows; ++i)
        for (int j = 0; j < m.cols; ++j) out[static_cast<std::size_t>(i) * m.cols + j] = R(m(i, j));
}

Mat to_mat(const rcwa_complex* p, int rows, int cols) {
    Mat m(rows, cols);
    for (std::size_t k = 0; k < m.a.size(); ++k) m.a[k] = C(p[k]);
    return m;
}

}  // namespace

extern "C" {

// Batched 1-D solve on the CPU: rcwa::sweep semantics (include/stablercwa/rcwa1d.hpp:1084-1091),
// points split over n_threads std::threads. Returns 0, or -1 with a message for invalid input.
int oracle_solve1d_batch(const rcwa_stack1d* stack, const rcwa_point1d* points, int n_points, int M, int pol,
                         int diagnostics, rcwa_result1d* out, int n_threads, char* err, size_t err_len) {
    Stack1D s;
    try {
        s = to_stack(stack);
    } catch (const InvalidArgument& e) {
        put_error(err, err_len, e.what.c_str());
        return -1;
    } catch (...) {
        put_error(err, err_len, "oracle: bad stack");
        return -1;
    }
    const int n = 2 * M + 1;
    std::atomic<int> next{0};
    std::atomic<int> failed{0};
    std::string first_error;
    std::mutex error_lock;
    const auto worker = [&]() {
        for (;;) {
            const int p = next.fetch_add(1);
            if (p >= n_points) return;
            try {
                const Result1D r = solve1d(s, points[p].wavelength, points[p].theta_deg, M, pol, diagnostics != 0);
                for (int j = 0; j < n; ++j) {
                    out->R[static_cast<std::size_t>(p) * n + j] = R(r.R[j]);
                    out->T[static_cast<std::size_t>(p) * n + j] = R(r.T[j]);
                    out->DEr[static_cast<std::size_t>(p) * n + j] = r.DEr[j];
                    out->DEt[static_cast<std::size_t>(p) * n + j] = r.DEt[j];
                }
                if (out->status) out->status[p] = !r.failed ? RCWA_SAMPLE_OK : (r.eig_info ? RCWA_SAMPLE_EIG_NOCONV : RCWA_SAMPLE_NUMERICAL);
                if (out->eig_info) out->eig_info[p] = r.eig_info;
                if (out->n_eig) out->n_eig[p] = r.n_eig;
                if (out->n_dense_solve) out->n_dense_solve[p] = r.n_dense_solve;
                if (out->max_eig_residual) out->max_eig_residual[p] = r.max_eig_residual;
            } catch (const InvalidArgument& e) {
                std::lock_guard<std::mutex> hold(error_lock);
                if (failed.fetch_add(1) == 0) first_error = e.what;
            }
        }
    };
    if (n_threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < n_threads; ++t) pool.emplace_back(worker);
        for (std::thread& t : pool) t.join();
    }
    if (failed.load()) {
        put_error(err, err_len, first_error);
        return -1;
    }
    return 0;
}

// Batched conical solve on the CPU: rcwa::sweep_conical (include/stablercwa/rcwa1d_conical.hpp:992-999).
int oracle_solve_conical_batch(const rcwa_stack1d* stack, const rcwa_point_conical* points, int n_points, int M,
                               rcwa_result_conical* out, int n_threads, char* err, size_t err_len) {
    Stack1D s;
    try {
        s = to_stack(stack);
    } catch (const InvalidArgument& e) {
        put_error(err, err_len, e.what.c_str());
        return -1;
    }
    const int n = 2 * M + 1;
    std::atomic<int> next{0};
    std::atomic<int> failed{0};
    std::string first_error;
    std::mutex error_lock;
    const auto worker = [&]() {
        for (;;) {
            const int p = next.fetch_add(1);
            if (p >= n_points) return;
            try {
                const ConicalResult r = solve_conical(s, points[p].wavelength, points[p].theta_deg, points[p].phi_deg, M);
                for (int j = 0; j < n; ++j) {
                    const size_t o = (static_cast<size_t>(p) * n + j) * 4;
                    const cplx jr[4] = {r.Jr[j].ss, r.Jr[j].sp, r.Jr[j].ps, r.Jr[j].pp};
                    const cplx jt[4] = {r.Jt[j].ss, r.Jt[j].sp, r.Jt[j].ps, r.Jt[j].pp};
                    for (int k = 0; k < 4; ++k) {
                        out->Jr[o + k] = R(jr[k]);
                        out->Jt[o + k] = R(jt[k]);
                        out->DEr[o + k] = r.DEr[j][k];
                        out->DEt[o + k] = r.DEt[j][k];
                    }
                    if (out->kx) out->kx[static_cast<size_t>(p) * n + j] = r.kx[j];
                    if (out->flux_r) out->flux_r[static_cast<size_t>(p) * n + j] = r.flux_r[j];
                    if (out->flux_t) out->flux_t[static_cast<size_t>(p) * n + j] = r.flux_t[j];
                }
                if (out->ky) out->ky[p] = r.ky;
                if (out->status) out->status[p] = !r.failed ? RCWA_SAMPLE_OK : (r.eig_info ? RCWA_SAMPLE_EIG_NOCONV : RCWA_SAMPLE_NUMERICAL);
                if (out->eig_info) out->eig_info[p] = r.eig_info;
                if (out->n_eig) out->n_eig[p] = r.n_eig;
                if (out->n_dense_solve) out->n_dense_solve[p] = r.n_dense_solve;
                if (out->n_schur) out->n_schur[p] = r.n_schur;
                if (out->min_abs_lambda) out->min_abs_lambda[p] = r.min_abs_lambda;
                if (out->degenerate_mode_warning) out->degenerate_mode_warning[p] = r.degenerate_mode_warning ? 1 : 0;
            } catch (const InvalidArgument& e) {
                std::lock_guard<std::mutex> hold(error_lock);
                if (failed.fetch_add(1) == 0) first_error = e.what;
            }
        }
    };
    if (n_threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < n_threads; ++t) pool.emplace_back(worker);
        for (std::thread& t : pool) t.join();
    }
    if (failed.load()) {
        put_error(err, err_len, first_error);
        return -1;
    }
    return 0;
}

// One eigensolve (include/stablercwa/eig_qr.hpp:1008-1124). vectors may be NULL.
int oracle_eig(int n, const rcwa_complex* a, double eps, int max_iter, rcwa_complex* values, rcwa_complex* vectors,
               int* info, int* sweeps) {
    const EigOut r = eig_qr(to_mat(a, n, n), eps, max_iter, vectors != nullptr);
    for (int j = 0; j < n; ++j) values[j] = R(r.values[j]);
    if (vectors && r.info == 0)
        for (std::size_t k = 0; k < r.vectors.a.size(); ++k) vectors[k] = R(r.vectors.a[k]);
    if (info) *info = r.info;
    if (sweeps) *sweeps = r.sweeps;
    return 0;
}

// Schur form with the accumulated transform: Z^H A Z = T (keep_transform in include/stablercwa/eig_qr.hpp:1106-1122).
int oracle_schur(int n, const rcwa_complex* a, rcwa_complex* z, rcwa_complex* t, int* info) {
    const EigOut r = eig_qr(to_mat(a, n, n), kEps, 30, false, true);
    for (std::size_t k = 0; k < r.Z.a.size(); ++k) z[k] = R(r.Z.a[k]);
    for (std::size_t k = 0; k < r.T.a.size(); ++k) t[k] = R(r.T.a[k]);
    if (info) *info = r.info;
    return 0;
}

// A X = B with partial-pivot LU (include/stablercwa/lu.hpp:427-436); singular -> 1 and X untouched.
int oracle_solve(int n, int nrhs, const rcwa_complex* a, const rcwa_complex* b, rcwa_complex* x, int* singular) {
    const LUF f = lu_factor(to_mat(a, n, n));
    if (singular) *singular = f.singular ? 1 : 0;
    if (f.singular) return 0;
    const Mat s = lu_solve(f, to_mat(b, n, nrhs));
    for (std::size_t k = 0; k < s.a.size(); ++k) x[k] = R(s.a[k]);
    return 0;
}

// C = A B (include/stablercwa/matrix.hpp:170-192)
int oracle_multiply(int m, int k, int n, const rcwa_complex* a, const rcwa_complex* b, rcwa_complex* c) {
    const Mat r = matmul(to_mat(a, m, k), to_mat(b, k, n));
    for (std::size_t q = 0; q < r.a.size(); ++q) c[q] = R(r.a[q]);
    return 0;
}

// Relative eigen-pair residual (include/stablercwa/eig.hpp:38-69)
double oracle_eig_residual(int n, const rcwa_complex* a, const rcwa_complex* values, const rcwa_complex* vectors) {
    CVec w(n);
    for (int j = 0; j < n; ++j) w[j] = C(values[j]);
    return eig_residual(to_mat(a, n, n), w, to_mat(vectors, n, n));
}

// TE/TM layer matrix the solve hands to the eigensolver (include/stablercwa/rcwa1d.hpp:1098-1110).
int oracle_layer_matrix(const rcwa_layer1d* layer, double period, double wavelength, double nI, double theta_deg,
                        int M, int pol, rcwa_complex* a) {
    rcwa_stack1d st{};
    st.period = period;
    st.n_layers = 1;
    st.layers = layer;
    Stack1D s;
    try {
        s = to_stack(&st);
    } catch (const InvalidArgument&) {
        return -1;
    }
    const CVec kx = r1::transverse_wavevectors(nI, theta_deg, wavelength, period, M);
    r1::Work w;
    try {
        const r1::LayerOp op = r1::assemble_layer(s.layers[0], period, kx, M, pol, w);
        for (std::size_t k = 0; k < op.a.a.size(); ++k) a[k] = R(op.a.a[k]);
    } catch (const r1::NumericalFailure&) {
        return -1;
    }
    return 0;
}

// Eps, Cx, Cy of one 2-D layer (include/stablercwa/rcwa2d_operators.hpp:325-429), N x N row-major each.
// factorization: RCWA_FACTORIZATION_LI or _LAURENT. Returns 0, or 1 where an inverse-rule block is singular.
int oracle_layer_operators2d(const rcwa_layer2d* layer, double Lx, double Ly, int M1, int M2, int factorization,
                             rcwa_complex* eps, rcwa_complex* cx, rcwa_complex* cy) {
    try {
        const r2d::Operators op = r2d::layer_operators(to_layer2d(*layer), Lx, Ly, M1, M2,
                                                       factorization == RCWA_FACTORIZATION_LAURENT);
        put_mat(op.eps, eps);
        put_mat(op.cx, cx);
        put_mat(op.cy, cy);
    } catch (const Singular&) {
        return 1;
    }
    return 0;
}

}  // extern "C"

namespace {

int solve2d_points(const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                   int factorization, const double* zs, int nz, rcwa_complex* fields, rcwa_result2d* out,
                   int n_threads, char* err, size_t err_len) {
    r2d::Stack st;
    st.nI = stack->nI;
    st.nII = C(stack->nII);
    st.Lx = stack->Lx;
    st.Ly = stack->Ly;
    for (int k = 0; k < stack->n_layers; ++k) st.layers.push_back(to_layer2d(stack->layers[k]));
    const int L = static_cast<int>(st.layers.size());
    std::vector<r2d::Operators> ops(static_cast<std::size_t>(L));
    bool singular = false;
    for (int k = 0; k < L; ++k) {
        if (st.layers[k].homogeneous) continue;
        try {
            ops[k] = r2d::layer_operators(st.layers[k], st.Lx, st.Ly, M1, M2, factorization == RCWA_FACTORIZATION_LAURENT);
        } catch (const Singular&) {
            singular = true;
        }
    }
    if (singular) {
        put_error(err, err_len, "oracle: an inverse-rule Toeplitz block is singular");
        return -1;
    }
    const int N = (2 * M1 + 1) * (2 * M2 + 1);
    std::atomic<int> next{0};
    const auto worker = [&]() {
        for (;;) {
            const int p = next.fetch_add(1);
            if (p >= n_points) return;
            const rcwa_point2d& pt = points[p];
            std::vector<double> depths(zs, zs + (fields ? nz : 0));
            CVec f;
            const r2d::Result r = r2d::solve2d(st, ops, pt.wavelength, pt.theta_deg, pt.phi_deg, M1, M2, C(pt.Es), C(pt.Ep),
                                               fields ? &depths : nullptr, fields ? &f : nullptr);
            if (fields)
                for (std::size_t k = 0; k < f.size(); ++k) fields[static_cast<std::size_t>(p) * f.size() + k] = R(f[k]);
            const std::size_t o = static_cast<std::size_t>(p) * N;
            for (int i = 0; i < N; ++i) {
                out->Kx[o + i] = r.Kx[i];
                out->Ky[o + i] = r.Ky[i];
                out->kzI[o + i] = R(r.kzI[i]);
                out->kzII[o + i] = R(r.kzII[i]);
                out->Ex_r[o + i] = R(r.Ex_r[i]);
                out->Ey_r[o + i] = R(r.Ey_r[i]);
                out->Ez_r[o + i] = R(r.Ez_r[i]);
                out->Ex_t[o + i] = R(r.Ex_t[i]);
                out->Ey_t[o + i] = R(r.Ey_t[i]);
                out->Ez_t[o + i] = R(r.Ez_t[i]);
                out->Rs[o + i] = R(r.Rs[i]);
                out->Rp[o + i] = R(r.Rp[i]);
                out->Ts[o + i] = R(r.Ts[i]);
                out->Tp[o + i] = R(r.Tp[i]);
                out->DEr[o + i] = r.DEr[i];
                out->DEt[o + i] = r.DEt[i];
                out->prop_r[o + i] = r.prop_r[i];
                out->prop_t[o + i] = r.prop_t[i];
            }
            out->status[p] = r.status;
            if (out->eig_info) out->eig_info[p] = r.eig_info;
            if (out->n_eig) out->n_eig[p] = r.n_eig;
            if (out->rayleigh_regions)
                for (int k = 0; k < L + 2; ++k) out->rayleigh_regions[static_cast<std::size_t>(p) * (L + 2) + k] = r.rayleigh[k];
        }
    };
    if (n_threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < n_threads; ++t) pool.emplace_back(worker);
        for (std::thread& t : pool) t.join();
    }
    return 0;
}

}  // namespace

extern "C" {

// Batched 2-D solve on the CPU: rcwa::solve2d per point (include/stablercwa/rcwa2d.hpp:1359), the operators
// formed once per stack, points split over n_threads std::threads. out's arrays as rcwa_result2d documents;
// n_dense_solve is not restated (left untouched). Returns 0, or -1 with a message.
int oracle_solve2d_batch(const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                         int factorization, rcwa_result2d* out, int n_threads, char* err, size_t err_len) {
    return solve2d_points(stack, points, n_points, M1, M2, factorization, nullptr, 0, nullptr, out, n_threads, err,
                          err_len);
}

// The same with the near-field harmonics at nz depths (include/stablercwa/rcwa2d_fields.hpp): fields holds,
// per point, 6 components (Ex, Ey, Ez, Hx, Hy, Hz) x N orders x nz depths, the depth index fastest.
int oracle_solve2d_fields(const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                          int factorization, const double* zs, int nz, rcwa_result2d* out, rcwa_complex* fields,
                          int n_threads, char* err, size_t err_len) {
    return solve2d_points(stack, points, n_points, M1, M2, factorization, zs, nz, fields, out, n_threads, err, err_len);
}

}  // extern "C"
