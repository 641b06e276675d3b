// oracle_dense.hpp -- CPU restatement of StableRCWA's dense kernels (TEST INFRASTRUCTURE ONLY).
//
// This is the oracle, not the product: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may build, load or call anything under oracle/. It restates, in plain C++17, the
// reference's complex dense numerics on the RCWA hot path:
//   * the column-major complex matrix            (include/stablercwa/matrix.hpp:34-114)
//   * the GEMM with grouped zero skipping         (include/stablercwa/matrix.hpp:170-192)
//   * partial-pivot LU factor + solve             (include/stablercwa/lu.hpp:268-396, :233, :427)
//   * the CORTH + COMQR2 eigensolver (serial form) (include/stablercwa/eig_qr.hpp:231-961, :1008-1124)
// Each function below names the reference lines it follows. Parity with the reference is pinned by
// tests/golden (fixtures produced by the reference's own code) and checked in tests/test_oracle.py.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <vector>

namespace oracle {

using cplx = std::complex<double>;
using CVec = std::vector<cplx>;
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kEps = std::numeric_limits<double>::epsilon();

// |Re| + |Im| (include/stablercwa/matrix.hpp:34)
inline double abs1(cplx z) { return std::fabs(z.real()) + std::fabs(z.imag()); }
inline bool finite(cplx z) { return std::isfinite(z.real()) && std::isfinite(z.imag()); }

// Column-major complex matrix: element (i, j) at data[i + j*rows] (include/stablercwa/matrix.hpp:34-114).
struct Mat {
    int rows = 0, cols = 0;
    CVec a;
    Mat() = default;
    Mat(int r, int c) : rows(r), cols(c), a(static_cast<std::size_t>(r) * c) {}
    static Mat eye(int n) {
        Mat m(n, n);
        for (int i = 0; i < n; ++i) m(i, i) = 1.0;
        return m;
    }
    static Mat diag(const CVec& d) {
        Mat m(static_cast<int>(d.size()), static_cast<int>(d.size()));
        for (int i = 0; i < m.rows; ++i) m(i, i) = d[i];
        return m;
    }
    cplx& operator()(int i, int j) { return a[static_cast<std::size_t>(j) * rows + i]; }
    const cplx& operator()(int i, int j) const { return a[static_cast<std::size_t>(j) * rows + i]; }
    cplx* col(int j) { return a.data() + static_cast<std::size_t>(j) * rows; }
    const cplx* col(int j) const { return a.data() + static_cast<std::size_t>(j) * rows; }
    bool empty() const { return a.empty(); }
    bool all_finite() const {
        for (const cplx& z : a)
            if (!finite(z)) return false;
        return true;
    }
};

// Raised where the reference throws std::runtime_error for a zero pivot (include/stablercwa/lu.hpp:427-436).
struct Singular {};

// c += a*t with the product written out (include/stablercwa/matrix.hpp:126-136).
inline void add_col(cplx* c, const cplx* a, cplx t, int len) {
    const double tr = t.real(), ti = t.imag();
    for (int i = 0; i < len; ++i) {
        const double ar = a[i].real(), ai = a[i].imag();
        c[i] = cplx(c[i].real() + (ar * tr - ai * ti), c[i].imag() + (ar * ti + ai * tr));
    }
}

// C = A*B. Columns of C accumulate four columns of A at a time; a group of four zero coefficients
// of B is skipped, so a diagonal B costs O(n^2) (include/stablercwa/matrix.hpp:139-192 and the
// solver-local copy include/stablercwa/rcwa1d.hpp:299-357).
inline Mat matmul(const Mat& a, const Mat& b) {
    if (a.cols != b.rows) throw std::invalid_argument("matmul: shape");
    const int m = a.rows, n = b.cols, p = a.cols;
    Mat c(m, n);
    for (int j = 0; j < n; ++j) {
        cplx* cj = c.col(j);
        const cplx* bj = b.col(j);
        int k = 0;
        for (; k + 4 <= p; k += 4) {
            const cplx t[4] = {bj[k], bj[k + 1], bj[k + 2], bj[k + 3]};
            if (t[0] == cplx{} && t[1] == cplx{} && t[2] == cplx{} && t[3] == cplx{}) continue;
            const cplx* a0 = a.col(k);
            const cplx* a1 = a.col(k + 1);
            const cplx* a2 = a.col(k + 2);
            const cplx* a3 = a.col(k + 3);
            for (int i = 0; i < m; ++i) {
                double xr = cj[i].real(), xi = cj[i].imag();
                xr = xr + a0[i].real() * t[0].real() - a0[i].imag() * t[0].imag();
                xi = xi + a0[i].real() * t[0].imag() + a0[i].imag() * t[0].real();
                xr = xr + a1[i].real() * t[1].real() - a1[i].imag() * t[1].imag();
                xi = xi + a1[i].real() * t[1].imag() + a1[i].imag() * t[1].real();
                xr = xr + a2[i].real() * t[2].real() - a2[i].imag() * t[2].imag();
                xi = xi + a2[i].real() * t[2].imag() + a2[i].imag() * t[2].real();
                xr = xr + a3[i].real() * t[3].real() - a3[i].imag() * t[3].imag();
                xi = xi + a3[i].real() * t[3].imag() + a3[i].imag() * t[3].real();
                cj[i] = cplx(xr, xi);
            }
        }
        for (; k < p; ++k)
            if (bj[k] != cplx{}) add_col(cj, a.col(k), bj[k], m);
    }
    return c;
}

inline CVec matvec(const Mat& a, const CVec& x) {
    CVec y(a.rows);
    for (int k = 0; k < a.cols; ++k) {
        const cplx t = x[k];
        const cplx* ak = a.col(k);
        for (int i = 0; i < a.rows; ++i) y[i] += ak[i] * t;
    }
    return y;
}

inline Mat scale_rows(Mat a, const CVec& d) {
    for (int j = 0; j < a.cols; ++j)
        for (int i = 0; i < a.rows; ++i) a(i, j) *= d[i];
    return a;
}
inline Mat scale_cols(Mat a, const CVec& d) {
    for (int j = 0; j < a.cols; ++j)
        for (int i = 0; i < a.rows; ++i) a(i, j) *= d[j];
    return a;
}

// Smith division (include/stablercwa/lu.hpp:88-97).
inline cplx cdiv(cplx a, cplx b) {
    const double br = b.real(), bi = b.imag();
    if (std::fabs(br) >= std::fabs(bi)) {
        const double r = bi / br, d = br + bi * r;
        return {(a.real() + a.imag() * r) / d, (a.imag() - a.real() * r) / d};
    }
    const double r = br / bi, d = bi + br * r;
    return {(a.real() * r + a.imag()) / d, (a.imag() * r - a.real()) / d};
}
inline cplx cmul(cplx a, cplx b) {
    return {a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real()};
}

// Partial-pivot right-looking LU, P*A = L*U, LAPACK ipiv convention. The pivot is the first entry of
// largest std::abs at or below the diagonal; multipliers are formed as a*(1/pivot) unless 1/pivot
// overflows. A zero pivot marks the factor singular (include/stablercwa/lu.hpp:268-396). The
// reference panels the elimination by 32 columns, which changes only the order in which columns are
// visited, not the operations on any element (include/stablercwa/lu.hpp:14-17), so the textbook
// column sweep below performs the same arithmetic.
struct LUF {
    Mat lu;
    std::vector<int> perm;
    bool singular = false;
};
inline LUF lu_factor(Mat a) {
    const int n = a.rows;
    LUF f;
    f.perm.resize(n);
    for (int k = 0; k < n; ++k) f.perm[k] = k;
    for (int j = 0; j < n; ++j) {
        // bring column j up to date with steps 0..j-1 (swaps already applied to it below)
        cplx* c = a.col(j);
        for (int k = 0; k < j; ++k) {
            const cplx t = c[k];
            if (t == cplx{}) continue;
            const cplx* l = a.col(k);
            for (int i = k + 1; i < n; ++i)
                c[i] = cplx(c[i].real() - l[i].real() * t.real() + l[i].imag() * t.imag(),
                            c[i].imag() - l[i].real() * t.imag() - l[i].imag() * t.real());
        }
        int p = j;
        double best = std::abs(c[j]);
        for (int i = j + 1; i < n; ++i) {
            const double v = std::abs(c[i]);
            if (v > best) { best = v; p = i; }
        }
        f.perm[j] = p;
        if (p != j)
            for (int k = 0; k < n; ++k) std::swap(a(j, k), a(p, k));
        const cplx pivot = c[j];
        if (pivot == cplx{}) {
            f.singular = true;
            for (int i = j + 1; i < n; ++i) c[i] = cplx{};
            continue;
        }
        const cplx inv = cdiv(cplx(1.0, 0.0), pivot);
        if (finite(inv)) {
            for (int i = j + 1; i < n; ++i) c[i] = cmul(c[i], inv);
        } else {
            for (int i = j + 1; i < n; ++i) c[i] = cdiv(c[i], pivot);
        }
    }
    f.lu = std::move(a);
    return f;
}

// Solve A X = B from the factor (include/stablercwa/lu.hpp:233-266): row swaps, forward
// substitution with the unit-lower L, back substitution with U.
inline Mat lu_solve(const LUF& f, Mat b) {
    const int n = f.lu.rows;
    for (int j = 0; j < b.cols; ++j) {
        cplx* x = b.col(j);
        for (int k = 0; k < n; ++k)
            if (f.perm[k] != k) std::swap(x[k], x[f.perm[k]]);
        for (int k = 0; k < n; ++k) {
            const cplx t = x[k];
            if (t == cplx{}) continue;
            const cplx* l = f.lu.col(k);
            for (int i = k + 1; i < n; ++i)
                x[i] = cplx(x[i].real() - l[i].real() * t.real() + l[i].imag() * t.imag(),
                            x[i].imag() - l[i].real() * t.imag() - l[i].imag() * t.real());
        }
        for (int k = n - 1; k >= 0; --k) {
            const cplx* u = f.lu.col(k);
            x[k] = cdiv(x[k], u[k]);
            const cplx t = x[k];
            if (t == cplx{}) continue;
            for (int i = 0; i < k; ++i)
                x[i] = cplx(x[i].real() - u[i].real() * t.real() + u[i].imag() * t.imag(),
                            x[i].imag() - u[i].real() * t.imag() - u[i].imag() * t.real());
        }
    }
    return b;
}

// stablercwa::solve (include/stablercwa/lu.hpp:427-436): a zero pivot is a Singular failure.
inline Mat solve(const Mat& a, const Mat& b) {
    LUF f = lu_factor(a);
    if (f.singular) throw Singular{};
    return lu_solve(f, b);
}

// ------------------------------------------------------------------------------------------
// Eigensolver: EISPACK CORTH + COMQR2 as restated by include/stablercwa/eig_qr.hpp (serial path).

struct EigOut {
    CVec values;
    Mat vectors;       // 2-norm normalised columns
    Mat Z, T;          // kept only when keep_transform is set
    int info = 0;
    int sweeps = 0;
};

namespace eq {

// sum conj(u_k) a_k with four partial sums (include/stablercwa/eig_qr.hpp:65-84)
inline cplx dot_conj(const cplx* u, const cplx* a, int len) {
    double sr[4] = {0, 0, 0, 0}, si[4] = {0, 0, 0, 0};
    int k = 0;
    for (; k + 4 <= len; k += 4)
        for (int q = 0; q < 4; ++q) {
            const double ur = u[k + q].real(), ui = u[k + q].imag(), ar = a[k + q].real(), ai = a[k + q].imag();
            sr[q] += ur * ar + ui * ai;
            si[q] += ur * ai - ui * ar;
        }
    for (; k < len; ++k) {
        const double ur = u[k].real(), ui = u[k].imag(), ar = a[k].real(), ai = a[k].imag();
        sr[0] += ur * ar + ui * ai;
        si[0] += ur * ai - ui * ar;
    }
    return {(sr[0] + sr[1]) + (sr[2] + sr[3]), (si[0] + si[1]) + (si[2] + si[3])};
}
// y += t*x (include/stablercwa/eig_qr.hpp:87-96)
inline void axpy(cplx* y, cplx t, const cplx* x, int len) {
    const double tr = t.real(), ti = t.imag();
    for (int k = 0; k < len; ++k) {
        const double xr = x[k].real(), xi = x[k].imag();
        y[k] = cplx(y[k].real() + (tr * xr - ti * xi), y[k].imag() + (tr * xi + ti * xr));
    }
}
// x = t*x (include/stablercwa/eig_qr.hpp:99-107)
inline void scal(cplx* x, cplx t, int len) {
    const double tr = t.real(), ti = t.imag();
    for (int k = 0; k < len; ++k) {
        const double xr = x[k].real(), xi = x[k].imag();
        x[k] = cplx(tr * xr - ti * xi, tr * xi + ti * xr);
    }
}
inline int bexp(double m) {  // include/stablercwa/eig_qr.hpp:206-210
    int e = 0;
    if (m > 0.0 && std::isfinite(m)) std::frexp(m, &e);
    return e;
}
inline cplx scale2(cplx z, int e) { return {std::ldexp(z.real(), e), std::ldexp(z.imag(), e)}; }
// unit-modulus z/|z| and |z| (include/stablercwa/eig_qr.hpp:216-222)
inline cplx unit_phase(cplx z, double& modulus) {
    const int e = bexp(std::max(std::fabs(z.real()), std::fabs(z.imag())));
    z = scale2(z, -e);
    const double r = std::abs(z);
    modulus = std::ldexp(r, e);
    return z / r;
}
inline bool safe_magnitude(double m) { return m > 1e-140 && m < 1e140; }

// CORTH (include/stablercwa/eig_qr.hpp:231-272)
inline void hessenberg(Mat& a, CVec& ort) {
    const int n = a.rows;
    CVec work(n);
    for (int m = 1; m < n - 1; ++m) {
        cplx* x = a.col(m - 1);
        ort[m] = 0.0;
        double scale_x = 0.0;
        for (int i = m; i < n; ++i) scale_x += abs1(x[i]);
        if (scale_x == 0.0) continue;
        double h = 0.0;
        for (int i = n - 1; i >= m; --i) {
            ort[i] = x[i] / scale_x;
            h += std::norm(ort[i]);
        }
        double g = std::sqrt(h);
        const double f = std::abs(ort[m]);
        if (f == 0.0) {
            ort[m] = g;
            x[m] = scale_x;
        } else {
            h += f * g;
            g /= f;
            ort[m] *= 1.0 + g;
        }
        const cplx* u = ort.data();
        const int len = n - m;
        std::fill(work.begin(), work.end(), cplx{});
        for (int j = n - 1; j >= m; --j) {
            cplx* aj = a.col(j);
            axpy(aj + m, -dot_conj(u + m, aj + m, len) / h, u + m, len);
            axpy(work.data(), u[j], aj, n);
        }
        for (int i = 0; i < n; ++i) work[i] /= h;
        for (int j = m; j < n; ++j) axpy(a.col(j), -std::conj(u[j]), work.data(), n);
        ort[m] *= scale_x;
        x[m] *= -g;
    }
}

// Z = P_1 ... P_{n-2} (include/stablercwa/eig_qr.hpp:354-373)
inline Mat accumulate(const Mat& a, CVec& ort) {
    const int n = a.rows;
    Mat z = Mat::eye(n);
    for (int i = n - 2; i >= 1; --i) {
        if (ort[i] == cplx{} || a(i, i - 1) == cplx{}) continue;
        const int e = bexp(abs1(ort[i]));
        const cplx sub = scale2(a(i, i - 1), -e);
        ort[i] = scale2(ort[i], -e);
        for (int k = i + 1; k < n; ++k) ort[k] = scale2(a(k, i - 1), -e);
        const double minus_h = sub.real() * ort[i].real() + sub.imag() * ort[i].imag();
        const cplx* v = ort.data() + i;
        const int len = n - i;
        for (int j = i; j < n; ++j) {
            cplx* zj = z.col(j) + i;
            axpy(zj, dot_conj(v, zj, len) / minus_h, v, len);
        }
    }
    return z;
}

// include/stablercwa/eig_qr.hpp:427-439
inline void real_subdiagonal(Mat& h, Mat* z) {
    const int n = h.rows;
    for (int i = 1; i < n; ++i) {
        const cplx sub = h(i, i - 1);
        if (sub.imag() == 0.0) continue;
        double norm = 0.0;
        const cplx y = unit_phase(sub, norm);
        h(i, i - 1) = norm;
        for (int j = i; j < n; ++j) h(i, j) = std::conj(y) * h(i, j);
        scal(h.col(i), y, std::min(i + 1, n - 1) + 1);
        if (z) scal(z->col(i), y, n);
    }
}

struct Rot { double cr, ci, s; };

// include/stablercwa/eig_qr.hpp:450-464
inline Rot make_rotation(cplx* col, int j) {
    double xr = col[j].real(), xi = col[j].imag(), sub = col[j + 1].real();
    const double m = std::max({std::fabs(xr), std::fabs(xi), std::fabs(sub)});
    int e = 0;
    if (!safe_magnitude(m)) {
        e = bexp(m);
        xr = std::ldexp(xr, -e);
        xi = std::ldexp(xi, -e);
        sub = std::ldexp(sub, -e);
    }
    const double norm = std::sqrt(xr * xr + xi * xi + sub * sub);
    col[j] = e ? std::ldexp(norm, e) : norm;
    col[j + 1] = 0.0;
    return Rot{xr / norm, xi / norm, sub / norm};
}

// G_first..G_last applied from the left to one column (include/stablercwa/eig_qr.hpp:468-484)
inline void rotate_rows(cplx* col, const Rot* rot, int first, int last) {
    if (first > last) return;
    double yr = col[first - 1].real(), yi = col[first - 1].imag();
    for (int i = first; i <= last; ++i) {
        const Rot g = rot[i];
        const double zr = col[i].real(), zi = col[i].imag();
        col[i - 1] = cplx(g.cr * yr + g.ci * yi + g.s * zr, g.cr * yi - g.ci * yr + g.s * zi);
        const double tr = g.cr * zr - g.ci * zi - g.s * yr;
        const double ti = g.cr * zi + g.ci * zr - g.s * yi;
        yr = tr;
        yi = ti;
    }
    col[last] = cplx(yr, yi);
}

// (a, b) <- (c a + s b, conj(c) b - s a) on two columns (include/stablercwa/eig_qr.hpp:517-528)
inline void rotate_columns(cplx* a, cplx* b, int len, const Rot& g) {
    for (int k = 0; k < len; ++k) {
        const double yr = a[k].real(), yi = a[k].imag(), zr = b[k].real(), zi = b[k].imag();
        a[k] = cplx(g.cr * yr - g.ci * yi + g.s * zr, g.cr * yi + g.ci * yr + g.s * zi);
        b[k] = cplx(g.cr * zr + g.ci * zi - g.s * yr, g.cr * zi - g.ci * zr - g.s * yi);
    }
}

// include/stablercwa/eig_qr.hpp:535-544
inline cplx wilkinson_shift(cplx a, cplx b, double c, cplx d) {
    const cplx y = (a - d) / 2.0;
    const int e = bexp(std::max({abs1(b), std::fabs(c), abs1(y)}));
    const cplx x = scale2(b, -e) * std::ldexp(c, -e);
    if (x == cplx{}) return d;
    const cplx ys = scale2(y, -e);
    cplx zz = std::sqrt(ys * ys + x);
    if (ys.real() * zz.real() + ys.imag() * zz.imag() < 0.0) zz = -zz;
    return d - scale2(x / (ys + zz), e);
}

// One full QR step on the active block [l, en] (include/stablercwa/eig_qr.hpp:551-607, full = true).
inline void qr_step(Mat& h, Mat* z, int l, int en, std::vector<Rot>& rot) {
    const int n = h.rows;
    // chain: column j gets G_{l+1..j}, then G_{j+1} is formed from it
    for (int j = l; j <= en; ++j) {
        cplx* c = h.col(j);
        rotate_rows(c, rot.data(), l + 1, j);
        if (j < en) rot[j + 1] = make_rotation(c, j);
    }
    for (int j = en + 1; j < n; ++j) rotate_rows(h.col(j), rot.data(), l + 1, en);
    cplx phase{1.0, 0.0};
    const bool has_phase = h(en, en).imag() != 0.0;
    if (has_phase) {
        double norm = 0.0;
        phase = unit_phase(h(en, en), norm);
        h(en, en) = norm;
        for (int j = en + 1; j < n; ++j) h(en, j) = std::conj(phase) * h(en, j);
    }
    for (int j = l + 1; j <= en; ++j) {
        rotate_columns(h.col(j - 1), h.col(j), j + 1, rot[j]);
        if (z) rotate_columns(z->col(j - 1), z->col(j), n, rot[j]);
    }
    if (has_phase) {
        scal(h.col(en), phase, en + 1);
        if (z) scal(z->col(en), phase, n);
    }
}

// Back substitution on the Schur form, multiply by Z, normalise (include/stablercwa/eig_qr.hpp:886-961).
inline Mat schur_vectors(const Mat& t, const CVec& w, const Mat& z, double eps) {
    const int n = t.rows;
    double norm = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j; ++i) norm = std::max(norm, abs1(t(i, j)));
    const double rel = std::max(eps, kEps);
    double tiny = rel * norm;
    if (tiny == 0.0) tiny = std::numeric_limits<double>::min();
    constexpr double kQuotientMax = 1e300;
    constexpr double kShrink = 0x1p-512;
    Mat v(n, n);
    CVec x(n);
    for (int j = 0; j < n; ++j) {
        std::copy(t.col(j), t.col(j) + j, x.begin());
        x[j] = 1.0;
        for (int i = j - 1; i >= 0; --i) {
            cplx y = w[j] - w[i];
            if (y == cplx{}) {
                y = tiny;
            } else {
                const double floor_value = rel * std::max(abs1(w[j]), abs1(w[i]));
                if (abs1(y) < floor_value) y = floor_value;
            }
            for (int pass = 0; pass < 3 && abs1(x[i]) > abs1(y) * kQuotientMax; ++pass)
                for (int k = 0; k <= j; ++k) x[k] *= kShrink;
            x[i] /= y;
            const double tr = abs1(x[i]);
            if (tr != 0.0 && tr + 1.0 / tr <= tr)
                for (int k = 0; k <= j; ++k) x[k] /= tr;
            axpy(x.data(), x[i], t.col(i), i);
        }
        cplx* vj = v.col(j);
        for (int k = 0; k <= j; ++k) axpy(vj, x[k], z.col(k), n);
        double big = 0.0;
        for (int i = 0; i < n; ++i) big = std::max(big, std::max(std::fabs(vj[i].real()), std::fabs(vj[i].imag())));
        if (big == 0.0 || !std::isfinite(big)) continue;
        double ssq = 0.0;
        for (int i = 0; i < n; ++i) ssq += std::norm(vj[i] / big);
        const double inv = 1.0 / std::sqrt(ssq);
        for (int i = 0; i < n; ++i) vj[i] = (vj[i] / big) * inv;
    }
    return v;
}

}  // namespace eq

// eig_qr (include/stablercwa/eig_qr.hpp:1008-1124), serial path, vectors = true.
inline EigOut eig_qr(const Mat& a, double eps = kEps, int max_iter = 30, bool vectors = true, bool keep_transform = false) {
    const int n = a.rows;
    EigOut r;
    r.values.assign(n, cplx{});
    Mat h = a;
    Mat z;
    {
        CVec ort(n);
        eq::hessenberg(h, ort);
        z = eq::accumulate(h, ort);
    }
    for (int j = 0; j + 2 < n; ++j) std::fill(h.col(j) + j + 2, h.col(j) + n, cplx{});
    eq::real_subdiagonal(h, &z);
    cplx t{};
    int en = n - 1, its = 0;
    std::vector<eq::Rot> rot(n);
    CVec& w = r.values;
    while (en >= 0) {
        int l = en;
        for (; l > 0; --l)
            if (abs1(h(l, l - 1)) <= eps * (abs1(h(l - 1, l - 1)) + abs1(h(l, l)))) break;
        if (l == en) {
            w[en] = h(en, en) + t;
            h(en, en) = w[en];
            --en;
            its = 0;
            continue;
        }
        if (its == max_iter) {
            r.info = en + 1;
            break;
        }
        cplx s;
        if (its == 10 || its == 20)
            s = std::fabs(h(en, en - 1).real()) + (en >= 2 ? std::fabs(h(en - 1, en - 2).real()) : 0.0);
        else
            s = eq::wilkinson_shift(h(en - 1, en - 1), h(en - 1, en), h(en, en - 1).real(), h(en, en));
        for (int i = 0; i <= en; ++i) h(i, i) -= s;
        t += s;
        ++its;
        ++r.sweeps;
        eq::qr_step(h, &z, l, en, rot);
    }
    if (r.info != 0) {
        for (int i = 0; i <= en; ++i) {
            h(i, i) += t;
            w[i] = h(i, i);
        }
        for (int j = en; j + 1 < n; ++j) h(j + 1, j) = 0.0;
        if (keep_transform) {
            r.Z = std::move(z);
            r.T = std::move(h);
        }
        return r;
    }
    for (int j = 0; j + 1 < n; ++j) h(j + 1, j) = 0.0;
    if (vectors) r.vectors = eq::schur_vectors(h, w, z, eps);
    if (keep_transform) {
        r.Z = std::move(z);
        r.T = std::move(h);
    }
    return r;
}

// max_j ||A v_j - l_j v_j|| / (||A||_F ||v_j||) (include/stablercwa/eig.hpp:38-69), plain sums.
inline double eig_residual(const Mat& a, const CVec& values, const Mat& v) {
    const int n = a.rows;
    if (n == 0) return 0.0;
    double fro = 0.0;
    for (const cplx& z : a.a) fro += std::norm(z);
    fro = std::sqrt(fro);
    const Mat av = matmul(a, v);
    double worst = 0.0;
    for (int j = 0; j < n; ++j) {
        double dn = 0.0, vn = 0.0;
        for (int i = 0; i < n; ++i) {
            dn += std::norm(av(i, j) - values[j] * v(i, j));
            vn += std::norm(v(i, j));
        }
        const double val = (std::sqrt(dn) / fro) / std::sqrt(vn);
        if (std::isnan(val)) return val;
        worst = std::max(worst, val);
    }
    return worst;
}

}  // namespace oracle
