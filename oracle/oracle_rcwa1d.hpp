// oracle_rcwa1d.hpp -- CPU restatement of StableRCWA's 1-D TE/TM solve (TEST INFRASTRUCTURE ONLY).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this file. It restates
// include/stablercwa/rcwa1d.hpp (the analytic-Fourier default path: homogeneous fast path, QR
// eigensolver, partial-pivot LU) step by step; every function names the lines it follows.
#pragma once

#include <string>

#include "oracle_dense.hpp"

namespace oracle {

struct Layer1D {
    double d = 0.0;
    bool homogeneous = true;
    cplx n = 1.0;
    std::vector<double> edges;
    CVec n_values;
};
struct Stack1D {
    cplx nI = 1.0, nII = 1.0;
    double period = 1.0;
    std::vector<Layer1D> layers;
};
struct Result1D {
    CVec R, T;
    std::vector<double> DEr, DEt;
    int eig_info = 0, n_eig = 0, n_dense_solve = 0;
    bool failed = false;
    double max_eig_residual = 0.0;
};

struct InvalidArgument {
    std::string what;
};

namespace r1 {

struct NumericalFailure {};

// include/stablercwa/rcwa1d.hpp:191-194
inline void check_index(cplx n) {
    if (!finite(n) || std::abs(n) == 0.0 || n.real() < 0.0 || n.imag() < 0.0)
        throw InvalidArgument{"rcwa: refractive index must be finite, nonzero, with Re n >= 0 and Im n >= 0"};
}
// include/stablercwa/rcwa1d.hpp:196-215 (analytic coefficients only)
inline void check_layer(const Layer1D& layer, double period) {
    if (!std::isfinite(layer.d) || layer.d < 0.0) throw InvalidArgument{"rcwa: layer thickness must be finite and >= 0"};
    if (layer.homogeneous) {
        check_index(layer.n);
        return;
    }
    const std::vector<double>& e = layer.edges;
    if (layer.n_values.empty() || e.size() != layer.n_values.size() + 1)
        throw InvalidArgument{"rcwa: a grating layer needs K indices and K+1 edges"};
    for (std::size_t j = 0; j < e.size(); ++j)
        if (!std::isfinite(e[j]) || (j > 0 && e[j] <= e[j - 1]))
            throw InvalidArgument{"rcwa: grating edges must be finite and strictly increasing"};
    if (std::fabs((e.back() - e.front()) - period) > 1e-10 * period)
        throw InvalidArgument{"rcwa: grating edges must span exactly one period"};
    for (const cplx& n : layer.n_values) check_index(n);
}
// include/stablercwa/rcwa1d.hpp:217-229
inline void check_setup(double period, double wavelength, cplx nI, double theta_deg, int M, int pol) {
    if (M < 0 || M > (std::numeric_limits<int>::max() - 1) / 4) throw InvalidArgument{"rcwa: invalid truncation order M"};
    if (pol != 0 && pol != 1) throw InvalidArgument{"rcwa: polarization must be TE or TM"};
    if (!std::isfinite(wavelength) || wavelength <= 0.0 || !std::isfinite(period) || period <= 0.0)
        throw InvalidArgument{"rcwa: wavelength and period must be finite and positive"};
    if (!std::isfinite(theta_deg) || std::fabs(theta_deg) >= 90.0)
        throw InvalidArgument{"rcwa: incidence angle must lie strictly between -90 and 90 degrees"};
    check_index(nI);
    if (nI.imag() != 0.0 || nI.real() <= 0.0) throw InvalidArgument{"rcwa: the incident medium must have a real positive index"};
}

// Analytic Fourier coefficients of a piecewise-constant profile, h = -hmax..hmax
// (include/stablercwa/rcwa1d.hpp:366-388).
inline CVec fourier_coefficients(const std::vector<double>& edges, const CVec& values, double period, int hmax) {
    CVec c(2 * hmax + 1);
    const std::size_t segments = values.size();
    CVec phase(edges.size());
    for (int h = -hmax; h <= hmax; ++h) {
        cplx sum{};
        if (h == 0) {
            for (std::size_t j = 0; j < segments; ++j) sum += values[j] * (edges[j + 1] - edges[j]) / period;
        } else {
            for (std::size_t k = 0; k < edges.size(); ++k) {
                const double arg = -2.0 * kPi * h * edges[k] / period;
                phase[k] = cplx{std::cos(arg), std::sin(arg)};
            }
            const double w = -2.0 * kPi * h;
            for (std::size_t j = 0; j < segments; ++j) {
                const cplx t = values[j] * (phase[j + 1] - phase[j]);
                sum += cplx{t.imag() / w, -t.real() / w};
            }
        }
        c[h + hmax] = sum;
    }
    return c;
}

// Toeplitz matrix (m, p) = c_{m-p} (include/stablercwa/rcwa1d.hpp:391-407)
inline Mat convolution_matrix(const std::vector<double>& edges, const CVec& values, double period, int M) {
    const CVec c = fourier_coefficients(edges, values, period, 2 * M);
    const int n = 2 * M + 1;
    Mat m(n, n);
    for (int col = 0; col < n; ++col)
        for (int row = 0; row < n; ++row) m(row, col) = c[row - col + 2 * M];
    return m;
}

// kx_m = nI sin(theta) - m lambda / period (include/stablercwa/rcwa1d.hpp:410-415)
inline CVec transverse_wavevectors(double nI, double theta_deg, double wavelength, double period, int M) {
    const double s = nI * std::sin(theta_deg * kPi / 180.0);
    CVec kx(2 * M + 1);
    for (int j = 0; j <= 2 * M; ++j) kx[j] = s - (j - M) * wavelength / period;
    return kx;
}

struct Work {
    int n_solve = 0;
};
inline Mat linear_solve(const Mat& a, const Mat& b, Work& w) {
    ++w.n_solve;
    try {
        return solve(a, b);
    } catch (const Singular&) {
        throw NumericalFailure{};
    }
}

struct LayerOp {
    Mat a, inv_eps;
};
// TE: A = Kx^2 - [[eps]]; TM: A = [[1/eps]]^{-1} (Kx [[eps]]^{-1} Kx - I) (include/stablercwa/rcwa1d.hpp:432-468)
inline LayerOp assemble_layer(const Layer1D& layer, double period, const CVec& kx, int M, int pol, Work& work) {
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
    LayerOp out;
    Mat e = convolution_matrix(edges, eps, period, M);
    if (pol == 0) {
        for (cplx& z : e.a) z = -z;
        for (int j = 0; j < size; ++j) e(j, j) += kx[j] * kx[j];
        out.a = std::move(e);
    } else {
        out.inv_eps = convolution_matrix(edges, inv, period, M);
        Mat b = scale_rows(linear_solve(e, Mat::diag(kx), work), kx);
        for (int j = 0; j < size; ++j) b(j, j) -= 1.0;
        out.a = linear_solve(out.inv_eps, b, work);
    }
    return out;
}

struct Modes {
    bool analytic = false;
    bool finite_zero_basis = false;
    CVec q, p;
    Mat W, V;
};

// include/stablercwa/rcwa1d.hpp:514-518
inline cplx branch(cplx q) {
    if (q.real() < 0.0) q = -q;
    if (q.real() < 1e-10 && q.imag() > 0.0) q = -q;
    return q;
}

// include/stablercwa/rcwa1d.hpp:522-544 (as_dense = false: the fast path)
inline Modes analytic_modes(cplx n, const CVec& kx, int pol, bool finite_zero_basis) {
    Modes m;
    m.analytic = true;
    m.finite_zero_basis = finite_zero_basis;
    const std::size_t size = kx.size();
    m.q.resize(size);
    m.p.resize(size);
    for (std::size_t j = 0; j < size; ++j) {
        cplx kz = std::sqrt(n * n - kx[j] * kx[j]);
        if (kz.imag() < 0.0) kz = -kz;
        if (std::fabs(kz.imag()) < 1e-12 && kz.real() < 0.0) kz = -kz;
        m.q[j] = cplx{kz.imag(), -kz.real()};
        const cplx basis_q = finite_zero_basis && m.q[j] == cplx{} ? cplx(1.0) : m.q[j];
        m.p[j] = pol == 0 ? basis_q : basis_q / (n * n);
    }
    return m;
}

// Zero / diagonal / dense operators (include/stablercwa/rcwa1d.hpp:549-629)
struct Op {
    enum Kind { Zero, Diag, Dense } kind = Zero;
    CVec d;
    Mat m;
};
inline Op diag_op(CVec v) {
    Op o;
    o.kind = Op::Diag;
    o.d = std::move(v);
    return o;
}
inline Op dense_op(Mat a) {
    Op o;
    o.kind = Op::Dense;
    o.m = std::move(a);
    return o;
}
inline Op op_mul(const Op& a, const Op& b) {
    if (a.kind == Op::Zero || b.kind == Op::Zero) return Op{};
    if (a.kind == Op::Diag && b.kind == Op::Diag) {
        CVec v(a.d.size());
        for (std::size_t i = 0; i < v.size(); ++i) v[i] = a.d[i] * b.d[i];
        return diag_op(std::move(v));
    }
    if (a.kind == Op::Diag) return dense_op(scale_rows(b.m, a.d));
    if (b.kind == Op::Diag) return dense_op(scale_cols(a.m, b.d));
    return dense_op(matmul(a.m, b.m));
}
inline Op op_add(Op a, const Op& b) {
    if (b.kind == Op::Zero) return a;
    if (a.kind == Op::Zero) return b;
    if (a.kind == Op::Diag && b.kind == Op::Diag) {
        for (std::size_t i = 0; i < a.d.size(); ++i) a.d[i] += b.d[i];
        return a;
    }
    if (a.kind == Op::Dense && b.kind == Op::Dense) {
        for (std::size_t k = 0; k < a.m.a.size(); ++k) a.m.a[k] += b.m.a[k];
        return a;
    }
    if (a.kind == Op::Dense) {
        for (int i = 0; i < a.m.rows; ++i) a.m(i, i) += b.d[i];
        return a;
    }
    Op out = b;
    for (int i = 0; i < out.m.rows; ++i) out.m(i, i) += a.d[i];
    return out;
}
inline CVec op_apply(const Op& a, const CVec& x) {
    if (a.kind == Op::Dense) return matvec(a.m, x);
    CVec y(x.size());
    if (a.kind == Op::Diag)
        for (std::size_t i = 0; i < y.size(); ++i) y[i] = a.d[i] * x[i];
    return y;
}
inline Mat op_to_dense(const Op& a, int n) {
    if (a.kind == Op::Dense) return a.m;
    if (a.kind == Op::Diag) return Mat::diag(a.d);
    return Mat(n, n);
}
inline Mat identity_minus(Mat m) {
    for (cplx& z : m.a) z = -z;
    for (int i = 0; i < m.rows; ++i) m(i, i) += 1.0;
    return m;
}

struct SBlock {
    Op Tdd, Rdu, Rud, Tuu;
};

// include/stablercwa/rcwa1d.hpp:644-661
inline SBlock diagonal_interface(const Modes& up, const Modes& low) {
    const std::size_t size = up.p.size();
    CVec tdd(size), rdu(size), rud(size), tuu(size);
    for (std::size_t j = 0; j < size; ++j) {
        const cplx p1 = up.p[j], p2 = low.p[j];
        const cplx inv = 1.0 / (p1 + p2);
        tdd[j] = 2.0 * p1 * inv;
        rdu[j] = (p2 - p1) * inv;
        rud[j] = (p1 - p2) * inv;
        tuu[j] = 2.0 * p2 * inv;
    }
    SBlock s;
    s.Tdd = diag_op(std::move(tdd));
    s.Rdu = diag_op(std::move(rdu));
    s.Rud = diag_op(std::move(rud));
    s.Tuu = diag_op(std::move(tuu));
    return s;
}

// include/stablercwa/rcwa1d.hpp:664-692
inline void interface_matching(const Modes& up, const Modes& low, Work& work, Mat& tp, Mat& tm) {
    const int n = static_cast<int>(up.q.size());
    Mat mm, nn;
    if (low.analytic) {
        mm = up.W;
        CVec inv_p(low.p.size());
        for (std::size_t j = 0; j < inv_p.size(); ++j) inv_p[j] = 1.0 / low.p[j];
        nn = scale_rows(up.V, inv_p);
    } else if (up.analytic) {
        mm = linear_solve(low.W, Mat::eye(n), work);
        nn = linear_solve(low.V, Mat::diag(up.p), work);
    } else {
        mm = linear_solve(low.W, up.W, work);
        nn = linear_solve(low.V, up.V, work);
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

// include/stablercwa/rcwa1d.hpp:694-712
inline SBlock interface_block(const Modes& up, const Modes& low, Work& work) {
    if (up.analytic && low.analytic) return diagonal_interface(up, low);
    const int n = static_cast<int>(up.q.size());
    Mat tp, tm;
    interface_matching(up, low, work, tp, tm);
    Mat tpi = linear_solve(tp, Mat::eye(n), work);
    Mat rdu = matmul(tm, tpi);
    const Mat back = matmul(rdu, tm);
    for (std::size_t k = 0; k < tp.a.size(); ++k) tp.a[k] -= back.a[k];
    Mat rud = matmul(tpi, tm);
    for (cplx& z : rud.a) z = -z;
    SBlock s;
    s.Tdd = dense_op(std::move(tp));
    s.Rdu = dense_op(std::move(rdu));
    s.Rud = dense_op(std::move(rud));
    s.Tuu = dense_op(std::move(tpi));
    return s;
}

struct TopBlock {
    Op Rdu, Tuu;
    CVec tdd, rud;
};
// include/stablercwa/rcwa1d.hpp:720-746
inline TopBlock top_interface_block(const Modes& up, const Modes& low, int M, Work& work) {
    const int n = static_cast<int>(up.q.size());
    TopBlock t;
    if (up.analytic && low.analytic) {
        SBlock s = diagonal_interface(up, low);
        t.tdd.assign(n, cplx{});
        t.rud.assign(n, cplx{});
        t.tdd[M] = s.Tdd.d[M];
        t.rud[M] = s.Rud.d[M];
        t.Rdu = std::move(s.Rdu);
        t.Tuu = std::move(s.Tuu);
        return t;
    }
    Mat tp, tm;
    interface_matching(up, low, work, tp, tm);
    Mat tpi = linear_solve(tp, Mat::eye(n), work);
    Mat rdu = matmul(tm, tpi);
    const CVec tm_e(tm.col(M), tm.col(M) + n);
    t.tdd.assign(tp.col(M), tp.col(M) + n);
    const CVec back = matvec(rdu, tm_e);
    for (int j = 0; j < n; ++j) t.tdd[j] -= back[j];
    t.rud = matvec(tpi, tm_e);
    for (cplx& v : t.rud) v = -v;
    t.Rdu = dense_op(std::move(rdu));
    t.Tuu = dense_op(std::move(tpi));
    return t;
}

// include/stablercwa/rcwa1d.hpp:751-784 (as_dense = false)
inline SBlock propagation_block(const CVec& q, double d, double k0, bool finite_zero_basis) {
    CVec x(q.size()), reflection(q.size());
    bool has_zero = false;
    for (std::size_t j = 0; j < x.size(); ++j) {
        if (finite_zero_basis && q[j] == cplx{}) {
            const double h = k0 * d;
            if (!std::isfinite(h)) throw NumericalFailure{};
            const double denominator = 1.0 + 0.5 * h;
            x[j] = 1.0 / denominator;
            reflection[j] = (0.5 * h) / denominator;
            has_zero = true;
        } else {
            x[j] = std::exp(-k0 * d * q[j]);
        }
    }
    SBlock s;
    s.Tdd = diag_op(x);
    s.Tuu = diag_op(std::move(x));
    if (has_zero) {
        s.Rdu = diag_op(reflection);
        s.Rud = diag_op(std::move(reflection));
    }
    return s;
}

struct Seam {
    Op g, r;
};
// g = (I - Rdu r)^{-1} Tdd, r' = Rud + Tuu r g (include/stablercwa/rcwa1d.hpp:791-808)
inline Seam stack_on(SBlock&& s, const Op& r, int n, Work& work) {
    Seam out;
    Op k = op_mul(s.Rdu, r);
    if (k.kind == Op::Zero) {
        out.g = std::move(s.Tdd);
    } else if (k.kind == Op::Diag) {
        for (cplx& v : k.d) v = 1.0 / (1.0 - v);
        out.g = op_mul(k, s.Tdd);
    } else {
        out.g = dense_op(linear_solve(identity_minus(std::move(k.m)), op_to_dense(s.Tdd, n), work));
    }
    out.r = op_add(std::move(s.Rud), op_mul(s.Tuu, op_mul(r, out.g)));
    return out;
}

}  // namespace r1

// The full solve (include/stablercwa/rcwa1d.hpp:853-1074) with default options: homogeneous fast
// path, EigMethod::QR, LinearSolver::LUPartial. Invalid input throws InvalidArgument.
inline Result1D solve1d(const Stack1D& stack, double wavelength, double theta_deg, int M, int pol,
                        bool diagnostics = false, double eig_eps = kEps, int eig_max_iter = 30) {
    using namespace r1;
    check_setup(stack.period, wavelength, stack.nI, theta_deg, M, pol);
    check_index(stack.nII);
    for (const Layer1D& layer : stack.layers) check_layer(layer, stack.period);

    const int n = 2 * M + 1;
    const int layer_count = static_cast<int>(stack.layers.size());
    const double k0 = 2.0 * kPi / wavelength;
    Result1D result;
    const CVec kx = transverse_wavevectors(stack.nI.real(), theta_deg, wavelength, stack.period, M);
    Work work;
    try {
        std::vector<Modes> modes(layer_count + 2);
        modes.front() = analytic_modes(stack.nI, kx, pol, false);
        modes.back() = analytic_modes(stack.nII, kx, pol, false);
        std::vector<int> eig_layers;
        bool pure_films = true;
        for (const Layer1D& layer : stack.layers) pure_films = pure_films && layer.homogeneous;
        for (int j = 0; j < layer_count; ++j) {
            const Layer1D& layer = stack.layers[j];
            if (layer.homogeneous) modes[j + 1] = analytic_modes(layer.n, kx, pol, true);
            else eig_layers.push_back(j);
        }
        const int eig_count = static_cast<int>(eig_layers.size());
        std::vector<LayerOp> ops(eig_count);
        for (int i = 0; i < eig_count; ++i) {
            ops[i] = assemble_layer(stack.layers[eig_layers[i]], stack.period, kx, M, pol, work);
            if (!ops[i].a.all_finite()) throw NumericalFailure{};
        }
        std::vector<EigOut> eigs(eig_count);
        for (int i = 0; i < eig_count; ++i) eigs[i] = eig_qr(ops[i].a, eig_eps, eig_max_iter);
        result.n_eig = eig_count;
        for (int i = 0; i < eig_count; ++i) {
            if (eigs[i].info != 0 && result.eig_info == 0) result.eig_info = eigs[i].info;
            if (diagnostics) {
                const double res = eigs[i].info == 0 ? eig_residual(ops[i].a, eigs[i].values, eigs[i].vectors)
                                                     : std::numeric_limits<double>::quiet_NaN();
                if (std::isnan(res) || std::isnan(result.max_eig_residual)) result.max_eig_residual = std::numeric_limits<double>::quiet_NaN();
                else result.max_eig_residual = std::max(result.max_eig_residual, res);
            }
        }
        if (result.eig_info != 0) throw NumericalFailure{};
        for (int i = 0; i < eig_count; ++i) {
            Modes& m = modes[eig_layers[i] + 1];
            m.q.resize(n);
            for (int j = 0; j < n; ++j) m.q[j] = branch(std::sqrt(eigs[i].values[j]));
            m.W = std::move(eigs[i].vectors);
            m.finite_zero_basis = true;
            CVec basis_q = m.q;
            for (cplx& q : basis_q)
                if (q == cplx{}) q = 1.0;
            if (pol == 0) m.V = scale_cols(m.W, basis_q);
            else m.V = scale_cols(matmul(ops[i].inv_eps, m.W), basis_q);
        }
        const int block_count = 2 * layer_count + 1;
        std::vector<Op> g(block_count);
        Op r;
        for (int b = block_count - 1; b >= 1; --b) {
            const int j = b / 2;
            SBlock block;
            if (b % 2 == 0) block = interface_block(modes[j], modes[j + 1], work);
            else block = propagation_block(modes[j + 1].q, stack.layers[j].d, k0, modes[j + 1].finite_zero_basis);
            Seam seam = stack_on(std::move(block), r, n, work);
            g[b] = std::move(seam.g);
            r = std::move(seam.r);
        }
        {
            TopBlock top = top_interface_block(modes[0], modes[1], M, work);
            Op k = op_mul(top.Rdu, r);
            CVec down = std::move(top.tdd);
            if (k.kind == Op::Diag) {
                for (int j = 0; j < n; ++j) down[j] = down[j] / (1.0 - k.d[j]);
            } else if (k.kind == Op::Dense) {
                Mat rhs(n, 1);
                for (int j = 0; j < n; ++j) rhs(j, 0) = down[j];
                const Mat sol = linear_solve(identity_minus(std::move(k.m)), rhs, work);
                down.assign(sol.col(0), sol.col(0) + n);
            }
            result.R = std::move(top.rud);
            const CVec back = op_apply(top.Tuu, op_apply(r, down));
            for (int j = 0; j < n; ++j) result.R[j] += back[j];
            for (int b = 1; b < block_count; ++b) down = op_apply(g[b], down);
            result.T = std::move(down);
        }
        if (pure_films)
            for (int j = 0; j < n; ++j) {
                if (j == M) continue;
                if (!finite(result.R[j])) result.R[j] = cplx{};
                if (!finite(result.T[j])) result.T[j] = cplx{};
            }
        for (int j = 0; j < n; ++j)
            if (!finite(result.R[j]) || !finite(result.T[j])) throw NumericalFailure{};
        const CVec& qI = modes.front().q;
        const CVec& qII = modes.back().q;
        const cplx den{-k0 * qI[M].imag(), k0 * qI[M].real()};
        result.DEr.resize(n);
        result.DEt.resize(n);
        for (int j = 0; j < n; ++j) {
            const cplx kIz{-k0 * qI[j].imag(), k0 * qI[j].real()};
            const cplx kIIz{-k0 * qII[j].imag(), k0 * qII[j].real()};
            result.DEr[j] = std::norm(result.R[j]) * (kIz / den).real();
            const cplx factor = pol == 0 ? kIIz / den : (kIIz / (stack.nII * stack.nII)) / (den / (stack.nI * stack.nI));
            result.DEt[j] = std::norm(result.T[j]) * factor.real();
            if (!std::isfinite(result.DEr[j]) || !std::isfinite(result.DEt[j])) throw NumericalFailure{};
        }
    } catch (const NumericalFailure&) {
        const double nan = std::numeric_limits<double>::quiet_NaN();
        result.R.assign(n, cplx{nan, nan});
        result.T.assign(n, cplx{nan, nan});
        result.DEr.assign(n, nan);
        result.DEt.assign(n, nan);
        result.failed = true;
    }
    result.n_dense_solve = work.n_solve;
    return result;
}

}  // namespace oracle
