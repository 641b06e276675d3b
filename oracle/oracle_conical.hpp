// oracle_conical.hpp -- CPU restatement of StableRCWA's conical-incidence solve (TEST INFRASTRUCTURE ONLY).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this file. It restates
// include/stablercwa/rcwa1d_conical.hpp (default options: homogeneous fast path, QR, LU partial
// pivoting) function by function; every function names the lines it follows. The dimension-free
// pieces (Op algebra, stack_on, propagation, linear_solve) come from oracle_rcwa1d.hpp.
#pragma once

#include <array>

#include "oracle_rcwa1d.hpp"

namespace oracle {

struct Jones {
    cplx ss, sp, ps, pp;
};
struct ConicalResult {
    std::vector<double> kx;
    double ky = 0.0;
    std::vector<double> phi_m_deg;
    CVec kzI, kzII;
    std::vector<double> flux_r, flux_t;
    std::vector<Jones> Jr, Jt;
    std::vector<std::array<double, 4>> DEr, DEt;  // ss, sp, ps, pp
    int eig_info = 0, n_eig = 0, n_dense_solve = 0, n_schur = 0;
    double min_abs_lambda = std::numeric_limits<double>::infinity();
    bool degenerate_mode_warning = false;
    bool failed = false;
};

namespace cn {

using r1::NumericalFailure;
using r1::Op;
using r1::SBlock;
using r1::Work;

constexpr double kDegenerateWarn = 1e-2;  // rcwa1d_conical.hpp:191

// kz = sqrt(n^2 - kx^2 - ky^2), Im >= 0, Re >= 0 when Im ~ 0 (rcwa1d_conical.hpp:195-203)
inline cplx longitudinal(cplx n, double kx, double ky) {
    const cplx z = n * n - kx * kx - ky * ky;
    if (z.imag() == 0.0) return z.real() >= 0.0 ? cplx{std::sqrt(z.real()), 0.0} : cplx{0.0, std::sqrt(-z.real())};
    cplx kz = std::sqrt(z);
    if (kz.imag() < 0.0) kz = -kz;
    if (std::fabs(kz.imag()) < 1e-12 && kz.real() < 0.0) kz = -kz;
    return kz;
}
// the zeroth order from the incidence cosine (rcwa1d_conical.hpp:251-258)
inline cplx longitudinal0(cplx n, double nI, double cosine) {
    const cplx z = (n - nI) * (n + nI) + (nI * cosine) * (nI * cosine);
    if (z.imag() == 0.0) return z.real() >= 0.0 ? cplx{std::sqrt(z.real()), 0.0} : cplx{0.0, std::sqrt(-z.real())};
    cplx kz = std::sqrt(z);
    if (kz.imag() < 0.0) kz = -kz;
    if (std::fabs(kz.imag()) < 1e-12 && kz.real() < 0.0) kz = -kz;
    return kz;
}

struct Region {
    bool analytic = false;
    CVec q, w, v;
    Mat W, V, G;
};

// s branch (w, v) = (1, q); t branch (w, v) = (kz/n, -i n) (rcwa1d_conical.hpp:259-283)
inline Region analytic_region(cplx n, const std::vector<double>& kx, double ky, double nI, double cosine) {
    const std::size_t orders = kx.size();
    Region r;
    r.analytic = true;
    r.q.resize(2 * orders);
    r.w.resize(2 * orders);
    r.v.resize(2 * orders);
    for (std::size_t j = 0; j < orders; ++j) {
        const cplx kz = 2 * j + 1 == orders ? longitudinal0(n, nI, cosine) : longitudinal(n, kx[j], ky);
        const cplx q{kz.imag(), -kz.real()};
        r.q[j] = q;
        r.q[orders + j] = q;
        r.w[j] = 1.0;
        r.v[j] = q;
        r.w[orders + j] = kz / n;
        r.v[orders + j] = cplx{n.imag(), -n.real()};
    }
    return r;
}

// rcwa1d_conical.hpp:286-291
inline bool is_uniform(const Layer1D& layer) {
    if (layer.homogeneous) return true;
    for (const cplx& n : layer.n_values)
        if (n != layer.n_values.front()) return false;
    return true;
}

struct Operators {
    Mat a, bc, inv_eps, c;
};
// A = Kx^2 - [[eps]], B C with B = Kx [[eps]]^{-1} Kx - I, C = [[1/eps]]^{-1} (rcwa1d_conical.hpp:301-336)
inline Operators assemble(const Layer1D& layer, double period, const std::vector<double>& kx, int M, Work& work) {
    const std::vector<double> one_edge{0.0, period};
    const std::vector<double>& edges = layer.homogeneous ? one_edge : layer.edges;
    CVec eps, inv;
    if (layer.homogeneous) {
        eps.push_back(layer.n * layer.n);
        inv.push_back(1.0 / (layer.n * layer.n));
    } else {
        for (const cplx& n : layer.n_values) {
            eps.push_back(n * n);
            inv.push_back(1.0 / (n * n));
        }
    }
    const int size = 2 * M + 1;
    Operators out;
    Mat e = r1::convolution_matrix(edges, eps, period, M);
    out.inv_eps = r1::linear_solve(e, Mat::eye(size), work);
    out.c = r1::linear_solve(r1::convolution_matrix(edges, inv, period, M), Mat::eye(size), work);
    Mat b = out.inv_eps;
    for (int j = 0; j < size; ++j) {
        cplx* bj = b.col(j);
        for (int i = 0; i < size; ++i) bj[i] = (kx[i] * bj[i]) * kx[j];
        bj[j] -= 1.0;
    }
    out.bc = matmul(b, out.c);
    for (cplx& z : e.a) z = -z;
    for (int j = 0; j < size; ++j) e(j, j) += cplx{kx[j] * kx[j], 0.0};
    out.a = std::move(e);
    return out;
}

// 2N modes from the two eigensolves, rotated to the (s, t) basis, columns normalised
// (rcwa1d_conical.hpp:341-411)
inline Region general_region(const EigOut& te, const EigOut& tm, const Operators& op, const std::vector<double>& kx,
                             double ky, const std::vector<double>& cs, const std::vector<double>& sn) {
    const int orders = static_cast<int>(kx.size());
    const int n = 2 * orders;
    Region r;
    r.q.resize(n);
    for (int j = 0; j < orders; ++j) {
        r.q[j] = r1::branch(std::sqrt(te.values[j] + ky * ky));
        r.q[orders + j] = r1::branch(std::sqrt(tm.values[j] + ky * ky));
    }
    const Mat cw = matmul(op.c, tm.vectors);
    Mat coupling;
    if (ky != 0.0) {
        Mat scaled = cw;
        for (int j = 0; j < orders; ++j) {
            cplx* sj = scaled.col(j);
            for (int m = 0; m < orders; ++m) sj[m] = (ky * kx[m]) * sj[m];
        }
        coupling = matmul(op.inv_eps, scaled);
    }
    r.W = Mat(n, n);
    r.V = Mat(n, n);
    const auto normalise = [&](int column) {
        cplx* wc = r.W.col(column);
        cplx* vc = r.V.col(column);
        double sum = 0.0;
        for (int i = 0; i < n; ++i) sum += std::norm(wc[i]) + std::norm(vc[i]);
        const double scale = std::sqrt(sum);
        if (!(scale > 0.0) || !std::isfinite(scale)) throw NumericalFailure{};
        for (int i = 0; i < n; ++i) {
            wc[i] = wc[i] / scale;
            vc[i] = vc[i] / scale;
        }
    };
    for (int j = 0; j < orders; ++j) {
        {
            const cplx q1 = r.q[j];
            const cplx fy = q1 * q1, gx = -(te.values[j] * q1), gy = -ky * q1;
            const cplx* w1 = te.vectors.col(j);
            cplx* wc = r.W.col(j);
            cplx* vc = r.V.col(j);
            for (int m = 0; m < orders; ++m) {
                const cplx ey = w1[m] * fy, hx = w1[m] * gx, hy = (kx[m] * w1[m]) * gy;
                wc[m] = cs[m] * ey;
                wc[orders + m] = sn[m] * ey;
                vc[m] = -(cs[m] * hx) - sn[m] * hy;
                vc[orders + m] = cs[m] * hy - sn[m] * hx;
            }
            normalise(j);
        }
        {
            const cplx q2 = r.q[orders + j], lambda2 = tm.values[j];
            const cplx* w2 = tm.vectors.col(j);
            const cplx* cwj = cw.col(j);
            const cplx* yj = ky != 0.0 ? coupling.col(j) : nullptr;
            cplx* wc = r.W.col(orders + j);
            cplx* vc = r.V.col(orders + j);
            for (int m = 0; m < orders; ++m) {
                const cplx ex = w2[m] * lambda2, ey = yj ? yj[m] : cplx{}, hy = -(cwj[m] * q2);
                wc[m] = cs[m] * ey - sn[m] * ex;
                wc[orders + m] = cs[m] * ex + sn[m] * ey;
                vc[m] = -(sn[m] * hy);
                vc[orders + m] = cs[m] * hy;
            }
            normalise(orders + j);
        }
    }
    return r;
}

inline double norm_1(const Mat& a) {
    double best = 0.0;
    for (int j = 0; j < a.cols; ++j) {
        double s = 0.0;
        for (int i = 0; i < a.rows; ++i) s += std::abs(a(i, j));
        best = std::max(best, s);
    }
    return best;
}

// principal square root of an upper triangular matrix, diagonal by diagonal (rcwa1d_conical.hpp:415-437)
inline Mat triangular_root(const Mat& t) {
    const int n = t.rows;
    if (!t.all_finite()) throw NumericalFailure{};
    Mat g(n, n);
    for (int i = 0; i < n; ++i) {
        g(i, i) = r1::branch(std::sqrt(t(i, i)));
        if (g(i, i) == cplx{} || !finite(g(i, i))) throw NumericalFailure{};
    }
    for (int gap = 1; gap < n; ++gap)
        for (int i = 0; i + gap < n; ++i) {
            const int j = i + gap;
            cplx v = t(i, j);
            for (int k = i + 1; k < j; ++k) v -= g(i, k) * g(k, j);
            const cplx den = g(i, i) + g(j, j);
            if (den == cplx{}) throw NumericalFailure{};
            g(i, j) = v / den;
        }
    if (!g.all_finite()) throw NumericalFailure{};
    Mat residual = matmul(g, g);
    for (std::size_t k = 0; k < residual.a.size(); ++k) residual.a[k] -= t.a[k];
    const double scale = norm_1(t), error = norm_1(residual);
    if (!residual.all_finite() || !std::isfinite(scale) || !std::isfinite(error) ||
        error > 1e-10 * std::max(scale, std::numeric_limits<double>::min()))
        throw NumericalFailure{};
    return g;
}

// exp of an upper triangular matrix: scaling and squaring with a Taylor series and exact diagonal
// (rcwa1d_conical.hpp:439-464)
inline Mat triangular_exp(const Mat& a) {
    const int n = a.rows;
    if (!a.all_finite()) throw NumericalFailure{};
    const double size = norm_1(a);
    if (!std::isfinite(size)) throw NumericalFailure{};
    const int scaling = size > .25 ? std::max(0, static_cast<int>(std::ceil(std::log2(size) + 2.))) : 0;
    if (scaling > 1020) throw NumericalFailure{};
    Mat b = a;
    const cplx f(std::ldexp(1., -scaling));
    for (cplx& z : b.a) z *= f;
    Mat e = Mat::eye(n), term = e;
    bool converged = n == 0;
    for (int k = 1; k <= 40 && !converged; ++k) {
        term = matmul(term, b);
        const cplx inv(1. / k);
        for (cplx& z : term.a) z *= inv;
        for (std::size_t q = 0; q < e.a.size(); ++q) e.a[q] += term.a[q];
        if (!e.all_finite() || !term.all_finite()) throw NumericalFailure{};
        converged = norm_1(term) <= kEps * std::max(1., norm_1(e));
    }
    if (!converged) throw NumericalFailure{};
    for (int i = 0; i < n; ++i) e(i, i) = std::exp(a(i, i) * std::ldexp(1., -scaling));
    for (int k = 0; k < scaling; ++k) {
        e = matmul(e, e);
        for (int i = 0; i < n; ++i) e(i, i) = std::exp(a(i, i) * std::ldexp(1., k + 1 - scaling));
        if (!e.all_finite()) throw NumericalFailure{};
    }
    return e;
}

// Schur basis of the full 2N operator for a near-degenerate layer (rcwa1d_conical.hpp:466-502)
inline Region schur_region(const Operators& op, const std::vector<double>& kx, double ky, const std::vector<double>& cs,
                           const std::vector<double>& sn, int& info) {
    const int N = static_cast<int>(kx.size()), n = 2 * N;
    Mat p(n, n), q(n, n), re(n, n), rv(n, n);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            const cplx id = i == j ? 1. : 0.;
            p(i, j) = ky * kx[i] * op.inv_eps(i, j);
            p(i, N + j) = id - kx[i] * op.inv_eps(i, j) * kx[j];
            p(N + i, j) = ky * ky * op.inv_eps(i, j) - id;
            p(N + i, N + j) = -ky * op.inv_eps(i, j) * kx[j];
            q(i, j) = ky * kx[i] * id;
            q(i, N + j) = -op.a(i, j);
            q(N + i, j) = ky * ky * id - op.c(i, j);
            q(N + i, N + j) = -ky * kx[i] * id;
        }
    for (int i = 0; i < N; ++i) {
        re(i, i) = -sn[i];
        re(i, N + i) = re(N + i, i) = cs[i];
        re(N + i, N + i) = sn[i];
        rv(i, i) = -cs[i];
        rv(i, N + i) = rv(N + i, i) = -sn[i];
        rv(N + i, N + i) = cs[i];
    }
    p = matmul(matmul(re, p), rv);
    q = matmul(matmul(rv, q), re);
    Mat h = matmul(p, q);
    if (!h.all_finite()) throw NumericalFailure{};
    EigOut e = eig_qr(h, kEps, 100, false, true);
    if (e.info != 0) {
        info = e.info;
        throw NumericalFailure{};
    }
    Region r;
    r.G = triangular_root(e.T);
    r.q.resize(n);
    for (int i = 0; i < n; ++i) r.q[i] = r.G(i, i);
    r.W = std::move(e.Z);
    r.V = matmul(q, r.W);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            cplx v = r.V(i, j);
            for (int k = 0; k < j; ++k) v -= r.V(i, k) * r.G(k, j);
            r.V(i, j) = v / r.G(j, j);
        }
    if (!r.V.all_finite()) throw NumericalFailure{};
    return r;
}

// rcwa1d_conical.hpp:513-533
inline SBlock diagonal_interface(const Region& up, const Region& low) {
    const std::size_t size = up.q.size();
    CVec tdd(size), rdu(size), rud(size), tuu(size);
    for (std::size_t j = 0; j < size; ++j) {
        const cplx w1 = up.w[j], v1 = up.v[j], w2 = low.w[j], v2 = low.v[j];
        const cplx a = w1 * v2, b = v1 * w2;
        const cplx inv = 1.0 / (a + b);
        tdd[j] = 2.0 * (w1 * v1) * inv;
        rdu[j] = (a - b) * inv;
        rud[j] = (b - a) * inv;
        tuu[j] = 2.0 * (w2 * v2) * inv;
    }
    SBlock s;
    s.Tdd = r1::diag_op(std::move(tdd));
    s.Rdu = r1::diag_op(std::move(rdu));
    s.Rud = r1::diag_op(std::move(rud));
    s.Tuu = r1::diag_op(std::move(tuu));
    return s;
}

// rcwa1d_conical.hpp:536-568
inline void interface_matching(const Region& up, const Region& low, Work& work, Mat& tp, Mat& tm) {
    Mat mm, nn;
    if (low.analytic) {
        CVec inv_w(low.w.size()), inv_v(low.v.size());
        for (std::size_t j = 0; j < inv_w.size(); ++j) {
            if (low.w[j] == cplx{} || low.v[j] == cplx{}) throw NumericalFailure{};
            inv_w[j] = 1.0 / low.w[j];
            inv_v[j] = 1.0 / low.v[j];
        }
        mm = scale_rows(up.W, inv_w);
        nn = scale_rows(up.V, inv_v);
    } else if (up.analytic) {
        mm = r1::linear_solve(low.W, Mat::diag(up.w), work);
        nn = r1::linear_solve(low.V, Mat::diag(up.v), work);
    } else {
        mm = r1::linear_solve(low.W, up.W, work);
        nn = r1::linear_solve(low.V, up.V, work);
    }
    tp = mm;
    for (std::size_t k = 0; k < tp.a.size(); ++k) tp.a[k] += nn.a[k];
    tm = std::move(mm);
    for (std::size_t k = 0; k < tm.a.size(); ++k) tm.a[k] -= nn.a[k];
    for (std::size_t k = 0; k < tp.a.size(); ++k) {
        tp.a[k] = 0.5 * tp.a[k];
        tm.a[k] = 0.5 * tm.a[k];
    }
}

inline SBlock interface_block(const Region& up, const Region& low, Work& work) {
    if (up.analytic && low.analytic) return diagonal_interface(up, low);
    const int n = static_cast<int>(up.q.size());
    Mat tp, tm;
    interface_matching(up, low, work, tp, tm);
    Mat tpi = r1::linear_solve(tp, Mat::eye(n), work);
    Mat rdu = matmul(tm, tpi);
    const Mat back = matmul(rdu, tm);
    for (std::size_t k = 0; k < tp.a.size(); ++k) tp.a[k] -= back.a[k];
    Mat rud = matmul(tpi, tm);
    for (cplx& z : rud.a) z = -z;
    SBlock s;
    s.Tdd = r1::dense_op(std::move(tp));
    s.Rdu = r1::dense_op(std::move(rdu));
    s.Rud = r1::dense_op(std::move(rud));
    s.Tuu = r1::dense_op(std::move(tpi));
    return s;
}

struct TopBlock {
    Op Rdu, Tuu;
    Mat tdd, rud;
};
// rcwa1d_conical.hpp:594-623
inline TopBlock top_interface_block(const Region& up, const Region& low, int M, Work& work) {
    const int n = static_cast<int>(up.q.size());
    const int column[2] = {M, n / 2 + M};
    TopBlock t;
    t.tdd = Mat(n, 2);
    t.rud = Mat(n, 2);
    if (up.analytic && low.analytic) {
        SBlock s = diagonal_interface(up, low);
        for (int k = 0; k < 2; ++k) {
            t.tdd(column[k], k) = s.Tdd.d[column[k]];
            t.rud(column[k], k) = s.Rud.d[column[k]];
        }
        t.Rdu = std::move(s.Rdu);
        t.Tuu = std::move(s.Tuu);
        return t;
    }
    Mat tp, tm;
    interface_matching(up, low, work, tp, tm);
    Mat tpi = r1::linear_solve(tp, Mat::eye(n), work);
    Mat rdu = matmul(tm, tpi);
    Mat tm_e(n, 2);
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < n; ++i) {
            tm_e(i, k) = tm(i, column[k]);
            t.tdd(i, k) = tp(i, column[k]);
        }
    const Mat back = matmul(rdu, tm_e);
    for (std::size_t q = 0; q < t.tdd.a.size(); ++q) t.tdd.a[q] -= back.a[q];
    t.rud = matmul(tpi, tm_e);
    for (cplx& z : t.rud.a) z *= cplx{-1.0, 0.0};
    t.Rdu = r1::dense_op(std::move(rdu));
    t.Tuu = r1::dense_op(std::move(tpi));
    return t;
}

// a x for a two-column x (rcwa1d_conical.hpp:626-634)
inline Mat apply(const Op& a, const Mat& x) {
    if (a.kind == Op::Dense) return matmul(a.m, x);
    Mat y(x.rows, x.cols);
    if (a.kind == Op::Diag)
        for (int k = 0; k < x.cols; ++k)
            for (int i = 0; i < x.rows; ++i) y(i, k) = a.d[i] * x(i, k);
    return y;
}

}  // namespace cn

// solve_conical (include/stablercwa/rcwa1d_conical.hpp:678-982), default options.
inline ConicalResult solve_conical(const Stack1D& stack, double wavelength, double theta_deg, double phi_deg, int M) {
    using namespace cn;
    r1::check_setup(stack.period, wavelength, stack.nI, theta_deg, M, 0);
    if (!std::isfinite(phi_deg)) throw InvalidArgument{"rcwa: azimuth angle must be finite"};
    r1::check_index(stack.nII);
    if (stack.nII.imag() != 0.0) throw InvalidArgument{"rcwa: conical incidence needs a real index in the exit medium"};
    for (const Layer1D& layer : stack.layers) r1::check_layer(layer, stack.period);

    const int orders = 2 * M + 1;
    const int n = 2 * orders;
    std::vector<const Layer1D*> layers;
    for (const Layer1D& layer : stack.layers)
        if (layer.d > 0.0) layers.push_back(&layer);
    const int layer_count = static_cast<int>(layers.size());
    const double k0 = 2.0 * kPi / wavelength;
    const double theta = theta_deg * kPi / 180.0, phi = phi_deg * kPi / 180.0;
    const double nI = stack.nI.real();

    ConicalResult result;
    const std::size_t count = orders;
    result.kx.resize(count);
    result.phi_m_deg.resize(count);
    result.kzI.resize(count);
    result.kzII.resize(count);
    result.flux_r.resize(count);
    result.flux_t.resize(count);
    result.Jr.resize(count);
    result.Jt.resize(count);
    result.DEr.resize(count);
    result.DEt.resize(count);
    const double sine = nI * std::sin(theta);
    const double ky = sine * std::sin(phi);
    const double flux_unit = nI * std::cos(theta);
    result.ky = ky;
    std::vector<double> cs(count), sn(count);
    for (int j = 0; j < orders; ++j) {
        const double kxj = sine * std::cos(phi) - (j - M) * wavelength / stack.period;
        const double kt = std::hypot(kxj, ky);
        result.kx[j] = kxj;
        if (kt <= 1e-14) {
            cs[j] = std::cos(phi);
            sn[j] = std::sin(phi);
            result.phi_m_deg[j] = phi_deg;
        } else {
            cs[j] = kxj / kt;
            sn[j] = ky / kt;
            result.phi_m_deg[j] = std::atan2(ky, kxj) * 180.0 / kPi;
        }
        result.kzI[j] = j == M ? longitudinal0(stack.nI, nI, std::cos(theta)) : longitudinal(stack.nI, kxj, ky);
        result.kzII[j] = j == M ? longitudinal0(stack.nII, nI, std::cos(theta)) : longitudinal(stack.nII, kxj, ky);
        result.flux_r[j] = result.kzI[j].real() / flux_unit;
        result.flux_t[j] = result.kzII[j].real() / flux_unit;
    }
    const std::vector<double>& kx = result.kx;
    Work work;
    try {
        std::vector<Region> modes(layer_count + 2);
        modes.front() = analytic_region(stack.nI, kx, ky, nI, std::cos(theta));
        modes.back() = analytic_region(stack.nII, kx, ky, nI, std::cos(theta));
        std::vector<int> eig_layers;
        bool pure_films = true;
        for (const Layer1D* layer : layers) pure_films = pure_films && is_uniform(*layer);
        for (int j = 0; j < layer_count; ++j) {
            const Layer1D& layer = *layers[j];
            if (is_uniform(layer)) {
                modes[j + 1] = analytic_region(layer.homogeneous ? layer.n : layer.n_values.front(), kx, ky, nI, std::cos(theta));
                for (int k = 0; k < orders; ++k)
                    if (modes[j + 1].q[k] == cplx{} && (!pure_films || k == M)) throw NumericalFailure{};
            } else {
                eig_layers.push_back(j);
            }
        }
        const int eig_count = static_cast<int>(eig_layers.size());
        std::vector<Operators> ops(eig_count);
        for (int i = 0; i < eig_count; ++i) {
            ops[i] = assemble(*layers[eig_layers[i]], stack.period, kx, M, work);
            if (!ops[i].a.all_finite() || !ops[i].bc.all_finite()) throw NumericalFailure{};
        }
        std::vector<EigOut> eigs(2 * eig_count);
        for (int t = 0; t < 2 * eig_count; ++t) eigs[t] = eig_qr(t % 2 == 0 ? ops[t / 2].a : ops[t / 2].bc);
        result.n_eig = 2 * eig_count;
        for (int t = 0; t < 2 * eig_count; ++t)
            if (eigs[t].info != 0 && result.eig_info == 0) result.eig_info = eigs[t].info;
        for (int t = 0; t < 2 * eig_count; ++t) {
            if (eigs[t].info != 0) continue;
            for (const cplx& value : eigs[t].values) result.min_abs_lambda = std::min(result.min_abs_lambda, std::abs(value));
        }
        const double ky_scale = std::fabs(ky) * std::sqrt(std::fabs(ky));
        if (ky != 0.0 && result.min_abs_lambda < kDegenerateWarn * ky_scale) result.degenerate_mode_warning = true;
        if (result.eig_info != 0) throw NumericalFailure{};
        for (int i = 0; i < eig_count; ++i) {
            double local_min = std::numeric_limits<double>::infinity();
            for (int t : {2 * i, 2 * i + 1})
                for (cplx value : eigs[t].values) local_min = std::min(local_min, std::abs(value));
            if (ky != 0.0 && local_min < kDegenerateWarn * ky_scale) {
                ++result.n_schur;
                ++result.n_eig;
                modes[eig_layers[i] + 1] = schur_region(ops[i], kx, ky, cs, sn, result.eig_info);
            } else {
                modes[eig_layers[i] + 1] = general_region(eigs[2 * i], eigs[2 * i + 1], ops[i], kx, ky, cs, sn);
            }
        }
        const int block_count = 2 * layer_count + 1;
        std::vector<Op> g(block_count);
        Op r;
        for (int b = block_count - 1; b >= 1; --b) {
            const int j = b / 2;
            SBlock block;
            if (b % 2 == 0) {
                block = interface_block(modes[j], modes[j + 1], work);
            } else if (modes[j + 1].G.rows != 0) {
                Mat a = modes[j + 1].G;
                const cplx f(-k0 * layers[j]->d);
                for (cplx& z : a.a) z *= f;
                Mat x = triangular_exp(a);
                block.Tdd = r1::dense_op(x);
                block.Tuu = r1::dense_op(std::move(x));
            } else {
                block = r1::propagation_block(modes[j + 1].q, layers[j]->d, k0, false);
            }
            r1::Seam seam = r1::stack_on(std::move(block), r, n, work);
            g[b] = std::move(seam.g);
            r = std::move(seam.r);
        }
        Mat up, down;
        {
            TopBlock top = top_interface_block(modes[0], modes[1], M, work);
            Op k = r1::op_mul(top.Rdu, r);
            down = std::move(top.tdd);
            if (k.kind == Op::Diag) {
                for (int c = 0; c < 2; ++c)
                    for (int j = 0; j < n; ++j) down(j, c) = down(j, c) / (1.0 - k.d[j]);
            } else if (k.kind == Op::Dense) {
                down = r1::linear_solve(r1::identity_minus(std::move(k.m)), down, work);
            }
            up = std::move(top.rud);
            const Mat back = apply(top.Tuu, apply(r, down));
            for (std::size_t q = 0; q < up.a.size(); ++q) up.a[q] += back.a[q];
            for (int b = 1; b < block_count; ++b) down = apply(g[b], down);
        }
        for (int j = 0; j < orders; ++j) {
            result.Jr[j] = Jones{up(j, 0), up(j, 1), -up(orders + j, 0), -up(orders + j, 1)};
            result.Jt[j] = Jones{down(j, 0), down(j, 1), down(orders + j, 0), down(orders + j, 1)};
        }
        if (pure_films)
            for (int j = 0; j < orders; ++j) {
                if (j == M) continue;
                for (Jones* a : {&result.Jr[j], &result.Jt[j]})
                    for (cplx* v : {&a->ss, &a->sp, &a->ps, &a->pp})
                        if (!finite(*v)) *v = cplx{};
            }
        for (int j = 0; j < orders; ++j)
            for (const Jones* a : {&result.Jr[j], &result.Jt[j]})
                if (!finite(a->ss) || !finite(a->sp) || !finite(a->ps) || !finite(a->pp)) throw NumericalFailure{};
        for (int j = 0; j < orders; ++j) {
            const Jones& a = result.Jr[j];
            const Jones& b = result.Jt[j];
            const double fr = result.flux_r[j], ft = result.flux_t[j];
            result.DEr[j] = {fr * std::norm(a.ss), fr * std::norm(a.sp), fr * std::norm(a.ps), fr * std::norm(a.pp)};
            result.DEt[j] = {ft * std::norm(b.ss), ft * std::norm(b.sp), ft * std::norm(b.ps), ft * std::norm(b.pp)};
            for (double v : result.DEr[j])
                if (!std::isfinite(v)) throw NumericalFailure{};
            for (double v : result.DEt[j])
                if (!std::isfinite(v)) throw NumericalFailure{};
        }
    } catch (const NumericalFailure&) {
        const double nan = std::numeric_limits<double>::quiet_NaN();
        const cplx z{nan, nan};
        result.Jr.assign(orders, Jones{z, z, z, z});
        result.Jt.assign(orders, Jones{z, z, z, z});
        result.DEr.assign(orders, {nan, nan, nan, nan});
        result.DEt.assign(orders, {nan, nan, nan, nan});
        result.failed = true;
    }
    result.n_dense_solve = work.n_solve;
    return result;
}

}  // namespace oracle
