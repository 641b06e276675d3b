// stablercwa_gb300.hpp -- C++ drop-in for StableRCWA's solve entry points on the GB300 engine.
//
// Include it after the StableRCWA headers: it takes and returns the reference's own value types
// (stablercwa::rcwa::Stack, Result, ConicalResult, Stack2D, Result2D, Matrix, EigResult) and gives, in
// namespace stablercwa_gb300::rcwa, functions with the reference's signatures and semantics:
//   solve          include/stablercwa/rcwa1d.hpp:1077
//   sweep          include/stablercwa/rcwa1d.hpp:1084   (all points in one batched call)
//   solve_conical  include/stablercwa/rcwa1d_conical.hpp:985
//   sweep_conical  include/stablercwa/rcwa1d_conical.hpp:992
//   solve2d        include/stablercwa/rcwa2d.hpp:1359
// and, for the reference's own CPU solves, adapters for its plug-in hooks Options::custom_eig,
// custom_solve and custom_multiply (include/stablercwa/rcwa1d.hpp:122-136, rcwa2d_types.hpp:89-95):
//   options.custom_eig = stablercwa_gb300::gpu_eig();   (likewise gpu_solve(), gpu_multiply())
// Error behaviour follows the reference: invalid arguments throw std::invalid_argument with the
// reference's message, checked on the host before any device work; a numerical failure gives the
// reference's NaN results with eig_info (1-D, conical) or status and message (2-D); a CUDA failure
// (no device, out of device memory) throws std::runtime_error. Each host thread uses its own engine
// context (one CUDA stream), so the calls may be made from several threads at once, as the reference's
// are. Link with libstablercwa_gb300.so (the C ABI of stablercwa_gb300.h).
#pragma once

#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "stablercwa_gb300.h"

namespace stablercwa_gb300 {

namespace dropin_detail {

namespace ref = ::stablercwa::rcwa;
using cplx = ::stablercwa::cplx;

inline rcwa_complex to_c(cplx z) { return rcwa_complex{z.real(), z.imag()}; }
inline cplx from_c(rcwa_complex z) { return cplx{z.re, z.im}; }

// one engine context per host thread, created on first use on device 0
class ThreadContext {
public:
    ThreadContext() {
        rcwa_gpu_config cfg{0, 0};
        const int rc = rcwa_gpu_create(&cfg, &ctx_);
        if (rc != RCWA_OK) {
            ctx_ = nullptr;
            code_ = rc;
        }
    }
    ~ThreadContext() {
        if (ctx_) rcwa_gpu_destroy(ctx_);
    }
    ThreadContext(const ThreadContext&) = delete;
    ThreadContext& operator=(const ThreadContext&) = delete;
    rcwa_gpu_ctx* get() {
        if (!ctx_) throw std::runtime_error("stablercwa_gb300: no CUDA device (engine context error " + std::to_string(code_) + ")");
        return ctx_;
    }

private:
    rcwa_gpu_ctx* ctx_ = nullptr;
    int code_ = 0;
};

inline rcwa_gpu_ctx* context() {
    thread_local ThreadContext c;
    return c.get();
}

inline void check(int rc, rcwa_gpu_ctx* ctx) {
    if (rc == RCWA_OK) return;
    char buf[1024] = {0};
    if (ctx) rcwa_gpu_last_error(ctx, buf, sizeof buf);
    if (rc == RCWA_EINVAL) throw std::invalid_argument(buf);
    throw std::runtime_error(std::string("stablercwa_gb300: ") + buf + " (error " + std::to_string(rc) + ")");
}

inline void check_valid(int rc, const char* message) {
    if (rc == RCWA_OK) return;
    if (rc == RCWA_EINVAL) throw std::invalid_argument(message);
    throw std::runtime_error(std::string("stablercwa_gb300: ") + message);
}

// the hooks belong to the reference's CPU solve; the engine runs every step itself
template <class Opt>
inline void reject_hooks(const Opt& o) {
    if (o.custom_eig || o.custom_multiply || o.custom_solve)
        throw std::invalid_argument("stablercwa_gb300: custom_eig / custom_multiply / custom_solve are hooks of the CPU solve; "
                                    "the GPU solve does not call them");
}

inline rcwa_options options1d(const ref::Options& o) {
    reject_hooks(o);
    rcwa_options c;
    rcwa_options_default(&c);
    c.eig_method = static_cast<int>(o.eig);
    c.linear_solver = static_cast<int>(o.linear);
    c.homogeneous_fast_path = o.homogeneous_fast_path ? 1 : 0;
    c.diagnostics = o.diagnostics ? 1 : 0;
    return c;
}

// a Stack marshalled into the C structs (the vectors own what the pointers point at)
struct Stack1D {
    std::vector<rcwa_layer1d> layers;
    std::vector<std::vector<rcwa_complex>> values;
    rcwa_stack1d s{};
    explicit Stack1D(const ref::Stack& st) {
        layers.resize(st.layers.size());
        values.resize(st.layers.size());
        for (std::size_t k = 0; k < st.layers.size(); ++k) {
            const ref::Layer& L = st.layers[k];
            rcwa_layer1d& c = layers[k];
            c.d = L.d;
            c.homogeneous = L.homogeneous ? 1 : 0;
            c.n = to_c(L.n);
            for (const cplx& v : L.n_values) values[k].push_back(to_c(v));
            c.n_segments = L.homogeneous ? 0 : static_cast<int>(L.n_values.size());
            c.edges = L.edges.empty() ? nullptr : L.edges.data();
            c.n_values = values[k].empty() ? nullptr : values[k].data();
            c.fourier_method = static_cast<int>(L.fourier_method);
            c.fft_samples = L.fft_samples;
            // a grating whose edge count does not match its indices is rejected like the reference's check
            if (!L.homogeneous && L.edges.size() != L.n_values.size() + 1) c.n_segments = -1;
        }
        s.nI = to_c(st.nI);
        s.nII = to_c(st.nII);
        s.period = st.period;
        s.n_layers = static_cast<int>(layers.size());
        s.layers = layers.empty() ? nullptr : layers.data();
    }
};

struct Stack2D {
    std::vector<rcwa_layer2d> layers;
    std::vector<std::vector<rcwa_xprofile2d>> profiles;
    std::vector<std::vector<std::vector<rcwa_complex>>> values;
    rcwa_stack2d s{};
    explicit Stack2D(const ref::Stack2D& st) {
        const std::size_t L = st.layers.size();
        layers.resize(L);
        profiles.resize(L);
        values.resize(L);
        for (std::size_t k = 0; k < L; ++k) {
            const ref::Layer2D& src = st.layers[k];
            rcwa_layer2d& c = layers[k];
            c.d = src.d;
            c.homogeneous = src.homogeneous ? 1 : 0;
            c.n = to_c(src.n);
            c.n_strips = src.homogeneous ? 0 : static_cast<int>(src.x_profiles.size());
            c.y_edges = src.y_edges.empty() ? nullptr : src.y_edges.data();
            if (!src.homogeneous && src.y_edges.size() != src.x_profiles.size() + 1) c.n_strips = -1;
            values[k].resize(src.x_profiles.size());
            for (std::size_t p = 0; p < src.x_profiles.size(); ++p) {
                const ref::XProfile2D& xp = src.x_profiles[p];
                for (const cplx& v : xp.n_values) values[k][p].push_back(to_c(v));
                rcwa_xprofile2d x;
                x.n_segments = xp.edges.size() == xp.n_values.size() + 1 ? static_cast<int>(xp.n_values.size()) : -1;
                x.edges = xp.edges.empty() ? nullptr : xp.edges.data();
                x.n_values = values[k][p].empty() ? nullptr : values[k][p].data();
                profiles[k].push_back(x);
            }
            c.x_profiles = profiles[k].empty() ? nullptr : profiles[k].data();
        }
        s.nI = st.nI;
        s.nII = to_c(st.nII);
        s.Lx = st.Lx;
        s.Ly = st.Ly;
        s.n_layers = static_cast<int>(L);
        s.layers = layers.empty() ? nullptr : layers.data();
    }
};

inline double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace dropin_detail

namespace rcwa {

// rcwa::sweep (include/stablercwa/rcwa1d.hpp:1084): every point in one batched call
inline std::vector<::stablercwa::rcwa::Result> sweep(const ::stablercwa::rcwa::Stack& stack,
                                                     const std::vector<::stablercwa::rcwa::Point>& points, int M,
                                                     ::stablercwa::rcwa::Polarization pol,
                                                     const ::stablercwa::rcwa::Options& options = {}) {
    namespace d = dropin_detail;
    const auto t0 = std::chrono::steady_clock::now();
    const rcwa_options o = d::options1d(options);
    const d::Stack1D st(stack);
    std::vector<rcwa_point1d> pts(points.size());
    for (std::size_t p = 0; p < points.size(); ++p) pts[p] = rcwa_point1d{points[p].wavelength, points[p].theta_deg};
    char msg[512];
    const int polc = pol == ::stablercwa::rcwa::Polarization::TE ? RCWA_TE : RCWA_TM;
    d::check_valid(rcwa_validate_solve1d(&st.s, pts.data(), static_cast<int>(pts.size()), M, polc, msg, sizeof msg), msg);
    std::vector<::stablercwa::rcwa::Result> out(points.size());
    if (points.empty()) return out;
    const int n = 2 * M + 1, P = static_cast<int>(points.size());
    std::vector<rcwa_complex> R((std::size_t)P * n), T((std::size_t)P * n);
    std::vector<double> DEr((std::size_t)P * n), DEt((std::size_t)P * n), resid(P);
    std::vector<int> status(P), info(P), neig(P), nsolve(P);
    rcwa_result1d res{R.data(), T.data(), DEr.data(), DEt.data(), status.data(), info.data(), neig.data(), nsolve.data(),
                      resid.data()};
    rcwa_gpu_ctx* ctx = d::context();
    d::check(rcwa_gpu_solve1d_batch(ctx, &st.s, pts.data(), P, M, polc, &o, &res), ctx);
    const double total = d::seconds_since(t0) / P;
    for (int p = 0; p < P; ++p) {
        ::stablercwa::rcwa::Result& r = out[p];
        r.orders.resize(n);
        r.R.resize(n);
        r.T.resize(n);
        r.DEr.resize(n);
        r.DEt.resize(n);
        for (int j = 0; j < n; ++j) {
            r.orders[j] = j - M;
            r.R[j] = d::from_c(R[(std::size_t)p * n + j]);
            r.T[j] = d::from_c(T[(std::size_t)p * n + j]);
            r.DEr[j] = DEr[(std::size_t)p * n + j];
            r.DEt[j] = DEt[(std::size_t)p * n + j];
        }
        r.eig_info = info[p];
        r.n_eig = neig[p];
        r.n_dense_solve = nsolve[p];
        r.max_eig_residual = options.diagnostics ? resid[p] : 0.0;
        r.timing.total = total;
    }
    return out;
}

// rcwa::solve (include/stablercwa/rcwa1d.hpp:1077)
inline ::stablercwa::rcwa::Result solve(const ::stablercwa::rcwa::Stack& stack, double wavelength, double theta_deg, int M,
                                        ::stablercwa::rcwa::Polarization pol = ::stablercwa::rcwa::Polarization::TE,
                                        const ::stablercwa::rcwa::Options& options = {}) {
    ::stablercwa::rcwa::Point pt;
    pt.wavelength = wavelength;
    pt.theta_deg = theta_deg;
    return ::stablercwa_gb300::rcwa::sweep(stack, std::vector<::stablercwa::rcwa::Point>{pt}, M, pol, options)[0];
}

// rcwa::sweep_conical (include/stablercwa/rcwa1d_conical.hpp:992)
inline std::vector<::stablercwa::rcwa::ConicalResult> sweep_conical(const ::stablercwa::rcwa::Stack& stack,
                                                                    const std::vector<::stablercwa::rcwa::ConicalPoint>& points,
                                                                    int M, const ::stablercwa::rcwa::Options& options = {}) {
    namespace d = dropin_detail;
    namespace dc = ::stablercwa::rcwa::detail::conical;
    const auto t0 = std::chrono::steady_clock::now();
    const rcwa_options o = d::options1d(options);
    const d::Stack1D st(stack);
    std::vector<rcwa_point_conical> pts(points.size());
    for (std::size_t p = 0; p < points.size(); ++p)
        pts[p] = rcwa_point_conical{points[p].wavelength, points[p].theta_deg, points[p].phi_deg};
    char msg[512];
    d::check_valid(rcwa_validate_solve_conical(&st.s, pts.data(), static_cast<int>(pts.size()), M, msg, sizeof msg), msg);
    std::vector<::stablercwa::rcwa::ConicalResult> out(points.size());
    if (points.empty()) return out;
    const int n = 2 * M + 1, P = static_cast<int>(points.size());
    std::vector<rcwa_complex> Jr((std::size_t)P * n * 4), Jt((std::size_t)P * n * 4);
    std::vector<double> DEr((std::size_t)P * n * 4), DEt((std::size_t)P * n * 4), minl(P), kx((std::size_t)P * n), ky(P),
        fr((std::size_t)P * n), ft((std::size_t)P * n);
    std::vector<int> status(P), info(P), neig(P), nsolve(P), nschur(P), warn(P);
    rcwa_result_conical res{Jr.data(), Jt.data(), DEr.data(), DEt.data(), status.data(), info.data(), neig.data(),
                            nsolve.data(), nschur.data(), minl.data(), warn.data(), kx.data(), ky.data(), fr.data(),
                            ft.data()};
    rcwa_gpu_ctx* ctx = d::context();
    d::check(rcwa_gpu_solve_conical_batch(ctx, &st.s, pts.data(), P, M, &o, &res), ctx);
    const double total = d::seconds_since(t0) / P;
    const double kPi = 3.141592653589793238462643383279502884;
    const double nI = stack.nI.real();
    for (int p = 0; p < P; ++p) {
        ::stablercwa::rcwa::ConicalResult& r = out[p];
        const double theta = points[p].theta_deg * kPi / 180.0, phi = points[p].phi_deg * kPi / 180.0;
        r.orders.resize(n);
        r.kx.resize(n);
        r.phi_m_deg.resize(n);
        r.kzI.resize(n);
        r.kzII.resize(n);
        r.flux_r.resize(n);
        r.flux_t.resize(n);
        r.Jr.resize(n);
        r.Jt.resize(n);
        r.DEr.resize(n);
        r.DEt.resize(n);
        r.ky = ky[p];
        for (int j = 0; j < n; ++j) {
            const std::size_t q = (std::size_t)p * n + j;
            r.orders[j] = j - M;
            r.kx[j] = kx[q];
            // the azimuth of each order and kz in the two media, as the reference forms them
            // (include/stablercwa/rcwa1d_conical.hpp:724-747)
            const double kt = std::hypot(kx[q], r.ky);
            r.phi_m_deg[j] = kt <= 1e-14 ? points[p].phi_deg : std::atan2(r.ky, kx[q]) * 180.0 / kPi;
            r.kzI[j] = j == M ? dc::longitudinal0(stack.nI, nI, std::cos(theta)) : dc::longitudinal(stack.nI, kx[q], r.ky);
            r.kzII[j] = j == M ? dc::longitudinal0(stack.nII, nI, std::cos(theta)) : dc::longitudinal(stack.nII, kx[q], r.ky);
            r.flux_r[j] = fr[q];
            r.flux_t[j] = ft[q];
            const rcwa_complex* a = &Jr[q * 4];
            const rcwa_complex* b = &Jt[q * 4];
            r.Jr[j] = ::stablercwa::rcwa::Jones{d::from_c(a[0]), d::from_c(a[1]), d::from_c(a[2]), d::from_c(a[3])};
            r.Jt[j] = ::stablercwa::rcwa::Jones{d::from_c(b[0]), d::from_c(b[1]), d::from_c(b[2]), d::from_c(b[3])};
            r.DEr[j] = ::stablercwa::rcwa::JonesEfficiency{DEr[q * 4], DEr[q * 4 + 1], DEr[q * 4 + 2], DEr[q * 4 + 3]};
            r.DEt[j] = ::stablercwa::rcwa::JonesEfficiency{DEt[q * 4], DEt[q * 4 + 1], DEt[q * 4 + 2], DEt[q * 4 + 3]};
        }
        (void)phi;
        r.eig_info = info[p];
        r.n_eig = neig[p];
        r.n_dense_solve = nsolve[p];
        r.n_schur = nschur[p];
        r.min_abs_lambda = minl[p];
        r.degenerate_mode_warning = warn[p] != 0;
        r.timing.total = total;
    }
    return out;
}

// rcwa::solve_conical (include/stablercwa/rcwa1d_conical.hpp:985)
inline ::stablercwa::rcwa::ConicalResult solve_conical(const ::stablercwa::rcwa::Stack& stack, double wavelength,
                                                       double theta_deg, double phi_deg, int M,
                                                       const ::stablercwa::rcwa::Options& options = {}) {
    ::stablercwa::rcwa::ConicalPoint pt;
    pt.wavelength = wavelength;
    pt.theta_deg = theta_deg;
    pt.phi_deg = phi_deg;
    return ::stablercwa_gb300::rcwa::sweep_conical(stack, std::vector<::stablercwa::rcwa::ConicalPoint>{pt}, M, options)[0];
}

// rcwa::solve2d (include/stablercwa/rcwa2d.hpp:1359)
inline ::stablercwa::rcwa::Result2D solve2d(const ::stablercwa::rcwa::Stack2D& stack, double wavelength, double theta_deg,
                                            double phi_deg, int M1, int M2, const ::stablercwa::rcwa::Jones2D& jones,
                                            const ::stablercwa::rcwa::Options2D& options = {}) {
    namespace d = dropin_detail;
    using ::stablercwa::rcwa::Status2D;
    using cplx = ::stablercwa::cplx;
    const auto t0 = std::chrono::steady_clock::now();
    d::reject_hooks(options);
    rcwa_options o;
    rcwa_options_default(&o);
    o.eig_method = static_cast<int>(options.eig);
    o.homogeneous_fast_path = options.homogeneous_fast_path ? 1 : 0;
    o.diagnostics = options.diagnostics ? 1 : 0;
    const int fact =
        options.factorization == ::stablercwa::rcwa::Factorization2D::Li ? RCWA_FACTORIZATION_LI : RCWA_FACTORIZATION_LAURENT;
    // the reference's checks in its order (include/stablercwa/rcwa2d.hpp:1363-1386): the truncation, then the
    // geometry of each patterned layer by the reference's own check functions (its messages name the layer),
    // then the remaining arguments (rcwa2d.hpp:985-1013) by the engine's host-side check
    if (M1 < 0 || M2 < 0) throw std::invalid_argument("rcwa2d: \u622a\u65ad\u9636\u6570 M1\u3001M2 \u4e0d\u80fd\u4e3a\u8d1f");
    for (const ::stablercwa::rcwa::Layer2D& layer : stack.layers)
        if (!layer.homogeneous) {
            ::stablercwa::rcwa::detail2d::impl::check_geometry(stack.Lx, stack.Ly, M1, M2);
            ::stablercwa::rcwa::detail2d::impl::check_patterned(layer, stack.Lx, stack.Ly);
        }
    const d::Stack2D st(stack);
    const rcwa_point2d pt{wavelength, theta_deg, phi_deg, d::to_c(jones[0]), d::to_c(jones[1])};
    char msg[512];
    d::check_valid(rcwa_validate_solve2d(&st.s, &pt, 1, M1, M2, fact, msg, sizeof msg), msg);
    const int N = (2 * M1 + 1) * (2 * M2 + 1), L = static_cast<int>(stack.layers.size());
    ::stablercwa::rcwa::Result2D r;
    std::vector<rcwa_complex> c[12];
    for (auto& v : c) v.resize(N);
    std::vector<double> Kx(N), Ky(N), DEr(N), DEt(N);
    std::vector<unsigned char> pr(N), ptr_(N), regions(L + 2);
    int status = 0, info = 0, neig = 0, nsolve = 0;
    double resid = 0.0;
    rcwa_result2d res{Kx.data(), Ky.data(), c[0].data(), c[1].data(), c[2].data(), c[3].data(), c[4].data(),
                      c[5].data(), c[6].data(), c[7].data(), c[8].data(), c[9].data(), c[10].data(), c[11].data(),
                      DEr.data(), DEt.data(), pr.data(), ptr_.data(), &status, &info, &neig, &nsolve, &resid,
                      regions.data()};
    rcwa_gpu_ctx* ctx = d::context();
    d::check(rcwa_gpu_solve2d_batch(ctx, &st.s, &pt, 1, M1, M2, fact, &o, &res), ctx);
    const double kPi = 3.141592653589793238462643383279502884;
    const int n2 = 2 * M2 + 1;
    r.M1 = M1;
    r.M2 = M2;
    r.N = N;
    r.i0 = M1 * n2 + M2;
    r.k0 = 2.0 * kPi / wavelength;
    r.theta = theta_deg * kPi / 180.0;
    r.phi = phi_deg * kPi / 180.0;
    r.m.resize(N);
    r.n.resize(N);
    for (int i = 0; i < N; ++i) {
        r.m[i] = i / n2 - M1;
        r.n[i] = i % n2 - M2;
    }
    r.Kx.assign(Kx.begin(), Kx.end());
    r.Ky.assign(Ky.begin(), Ky.end());
    ::stablercwa::Vector* dst[12] = {&r.kzI, &r.kzII, &r.Ex_r, &r.Ey_r, &r.Ez_r, &r.Ex_t, &r.Ey_t, &r.Ez_t,
                                     &r.Rs,  &r.Rp,   &r.Ts,   &r.Tp};
    for (int k = 0; k < 12; ++k) {
        dst[k]->resize(N);
        for (int i = 0; i < N; ++i) (*dst[k])[i] = d::from_c(c[k][i]);
    }
    r.DEr.assign(DEr.begin(), DEr.end());
    r.DEt.assign(DEt.begin(), DEt.end());
    r.prop_r.assign(pr.begin(), pr.end());
    r.prop_t.assign(ptr_.begin(), ptr_.end());
    r.eig_info = info;
    r.n_eig = neig;
    r.n_dense_solve = nsolve;
    r.max_eig_residual = options.diagnostics ? resid : 0.0;
    if (status == RCWA_SAMPLE_RAYLEIGH) {
        // the regions and (m, n) orders with kz exactly 0 (report_rayleigh, include/stablercwa/rcwa2d.hpp:1012-1026)
        r.status = Status2D::RayleighAnomaly;
        std::string text = "Rayleigh anomaly:";
        const auto list = [&](const char* name, const std::vector<cplx>& kz) {
            std::string s;
            for (int i = 0; i < N; ++i)
                if (kz[i] == cplx{}) s += " (" + std::to_string(r.m[i]) + ", " + std::to_string(r.n[i]) + ")";
            if (!s.empty()) text += std::string(" ") + name + ":" + s + ";";
        };
        if (regions[0]) list("incident medium", r.kzI);
        if (regions[L + 1]) list("exit medium", r.kzII);
        for (int j = 0; j < L; ++j)
            if (regions[j + 1]) {
                std::vector<cplx> kz(N);
                const cplx nn = stack.layers[j].n;
                for (int i = 0; i < N; ++i) kz[i] = std::sqrt(nn * nn - r.Kx[i] * r.Kx[i] - r.Ky[i] * r.Ky[i]);
                list(("layer " + std::to_string(j + 1)).c_str(), kz);
            }
        r.message = text;
    } else if (status != RCWA_SAMPLE_OK) {
        r.status = Status2D::NumericalFailure;
        r.message = info ? "eigen-solver did not converge (eig_info " + std::to_string(info) + ")"
                         : std::string("singular system or NaN/Inf");
    }
    r.timing.total = d::seconds_since(t0);
    return r;
}

}  // namespace rcwa

// Options::custom_eig for the reference's CPU solve: the eigenproblem on the GPU (rcwa_gpu_eig_batch),
// eigenvectors normalised to unit 2-norm, info > 0 when an eigenvalue did not converge.
inline std::function<::stablercwa::EigResult(const ::stablercwa::Matrix&)> gpu_eig(int max_iter = 30,
                                                                                  double eps = 2.220446049250313e-16) {
    return [max_iter, eps](const ::stablercwa::Matrix& a) {
        namespace d = dropin_detail;
        if (a.rows() != a.cols()) throw std::invalid_argument("eig: the matrix must be square");
        const int n = a.rows();
        ::stablercwa::EigResult r;
        r.values.resize(n);
        r.vectors = ::stablercwa::Matrix(n, n);
        int info = 0, sweeps = 0;
        rcwa_gpu_ctx* ctx = d::context();
        d::check(rcwa_gpu_eig_batch(ctx, n, 1, reinterpret_cast<const rcwa_complex*>(a.data()), eps, max_iter,
                                    reinterpret_cast<rcwa_complex*>(r.values.data()),
                                    reinterpret_cast<rcwa_complex*>(r.vectors.data()), &info, &sweeps),
                 ctx);
        r.info = info;
        r.sweeps = sweeps;
        return r;
    };
}

// Options::custom_solve: A X = B by partial-pivot LU on the GPU; a singular A throws std::runtime_error,
// which the reference's solve turns into a numerical failure, like its own LU's zero pivot.
inline std::function<::stablercwa::Matrix(const ::stablercwa::Matrix&, const ::stablercwa::Matrix&)> gpu_solve() {
    return [](const ::stablercwa::Matrix& a, const ::stablercwa::Matrix& b) {
        namespace d = dropin_detail;
        if (a.rows() != a.cols() || b.rows() != a.rows()) throw std::invalid_argument("solve: shape mismatch");
        ::stablercwa::Matrix x(a.cols(), b.cols());
        int singular = 0;
        rcwa_gpu_ctx* ctx = d::context();
        d::check(rcwa_gpu_solve_batch(ctx, a.rows(), b.cols(), 1, reinterpret_cast<const rcwa_complex*>(a.data()),
                                      reinterpret_cast<const rcwa_complex*>(b.data()),
                                      reinterpret_cast<rcwa_complex*>(x.data()), &singular),
                 ctx);
        if (singular) throw std::runtime_error("stablercwa_gb300: singular matrix");
        return x;
    };
}

// Options::custom_multiply: C = A B on the GPU
inline std::function<::stablercwa::Matrix(const ::stablercwa::Matrix&, const ::stablercwa::Matrix&)> gpu_multiply() {
    return [](const ::stablercwa::Matrix& a, const ::stablercwa::Matrix& b) {
        namespace d = dropin_detail;
        if (a.cols() != b.rows()) throw std::invalid_argument("Matrix product: shape mismatch");
        ::stablercwa::Matrix c(a.rows(), b.cols());
        if (a.rows() == 0 || b.cols() == 0) return c;
        rcwa_gpu_ctx* ctx = d::context();
        d::check(rcwa_gpu_multiply_batch(ctx, a.rows(), a.cols(), b.cols(), 1, reinterpret_cast<const rcwa_complex*>(a.data()),
                                         reinterpret_cast<const rcwa_complex*>(b.data()),
                                         reinterpret_cast<rcwa_complex*>(c.data())),
                 ctx);
        return c;
    };
}

}  // namespace stablercwa_gb300
