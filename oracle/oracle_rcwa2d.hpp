// oracle_rcwa2d.hpp -- CPU restatement of StableRCWA's 2-D (crossed-grating) solve (TEST INFRASTRUCTURE ONLY).
//
// This is the oracle, not the product: only tests/ may build, load or call it. It restates, in plain
// C++17 on top of oracle_dense.hpp, rcwa::solve2d (include/stablercwa/rcwa2d.hpp:1042-1347, :1359) with
// the layer operators of include/stablercwa/rcwa2d_operators.hpp:
//   * Fourier coefficients, Toeplitz blocks and Li's factorisation (Eps, Cx, Cy; or Laurent's rule), in the
//     reference's own arithmetic (its phase arguments, its accumulation order), so the operators can be
//     pinned against the reference's frozen operator tables;
//   * the modes of the homogeneous regions (closed form, W = I) and of the structured layers (H = P Q, the
//     CORTH + COMQR2 eigensolver of oracle_dense.hpp, q = branch(sqrt(lambda)), V = Q W / q);
//   * the reflection recursion from the exit medium up, with every interface in the reference's direct form
//     (r' = A+^-1 A-, A+- = (I + r) Nn +- (I - r) Mm; rcwa2d.hpp:738-790), the propagation blocks, the top
//     interface solved directly (K d = 2 e; rcwa2d.hpp:871-896) and the amplitudes carried back down;
//   * the efficiencies, the z components and the s/p amplitudes (rcwa2d.hpp:1226-1262), Rayleigh checks;
//   * the near-field harmonics at given depths (include/stablercwa/rcwa2d_fields.hpp:17-43: the layer
//     amplitudes a+ at each layer's top and a- at its bottom, the regions' plane waves, hz and Ez from the
//     tangential fields, H = -i h), with the reference's rule for which region a depth belongs to.
// The reference keeps block-diagonal operators of homogeneous regions in O(N) form and switches between
// S-block and direct forms by case; here every matrix is dense and every interface direct: the same
// algebra, so results agree with the reference's to rounding, not bit for bit. Parity with the reference
// is pinned by tests/golden/rcwa2d_cases.jsonl.gz (its frozen tables and its own solve2d outputs) in
// tests/test_oracle2d.py.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "oracle_dense.hpp"

namespace oracle {
namespace r2d {

// ------------------------------------------------------------------ geometry and results

struct XProfile {
    std::vector<double> edges;  // one more than values, spanning one x period
    CVec n;                     // refractive index of each segment
};

struct Layer {
    double d = 0.0;
    bool homogeneous = true;
    cplx n{1.0, 0.0};
    std::vector<double> y_edges;  // patterned: strips along y
    std::vector<XProfile> strips;
};

struct Stack {
    double nI = 1.0;
    cplx nII{1.0, 0.0};
    double Lx = 1.0, Ly = 1.0;
    std::vector<Layer> layers;
};

enum Status { kOk = 0, kNumerical = 1, kEigNoConv = 2, kRayleigh = 3 };

struct Result {
    int status = kOk, eig_info = 0, n_eig = 0;
    std::vector<double> Kx, Ky, DEr, DEt;
    CVec kzI, kzII, Ex_r, Ey_r, Ez_r, Ex_t, Ey_t, Ez_t, Rs, Rp, Ts, Tp;
    std::vector<unsigned char> prop_r, prop_t, rayleigh;  // rayleigh: regions 0 .. L+1
};

struct Operators {
    Mat eps, cx, cy;
};

// ------------------------------------------------------------------ Fourier operators

// Python's float %: the sign of b, +0 for an exact multiple (rcwa2d_operators.hpp:133-145)
inline double py_mod(double a, double b) {
    double r = std::fmod(a, b);
    if (r != 0.0) {
        if ((b < 0.0) != (r < 0.0)) r += b;
    } else {
        r = std::copysign(0.0, b);
    }
    return r;
}

// The contribution of segment [x0, x1] of period P to harmonic h: (x1 - x0)/P for h = 0, else
// (e(x1) - e(x0)) / (-2 pi i h) with e(x) = exp(-2 pi i h x / P), the phase argument formed as
// (-2 pi (h x)) / P (rcwa2d_operators.hpp:67-74, :97-120).
inline cplx edge_phase(double x, int h, double period) {
    const double arg = (-2.0 * kPi * (static_cast<double>(h) * x)) / period;
    return {std::cos(arg), std::sin(arg)};
}
inline cplx segment_term(cplx d, int h) {  // d / (i w), w = -2 pi h
    const double w = -2.0 * kPi * static_cast<double>(h);
    return {d.imag() / w, -d.real() / w};
}

// c[h + hmax], h = -hmax..hmax, of a piecewise-constant profile (rcwa2d_operators.hpp:78-95)
inline CVec fourier(const std::vector<double>& edges, const CVec& v, double period, int hmax) {
    CVec c(static_cast<std::size_t>(2 * hmax + 1));
    cplx mean{};
    for (std::size_t j = 0; j < v.size(); ++j) mean += v[j] * (edges[j + 1] - edges[j]);
    c[static_cast<std::size_t>(hmax)] = mean / period;
    for (int h = -hmax; h <= hmax; ++h) {
        if (h == 0) continue;
        cplx sum{};
        cplx prev = edge_phase(edges[0], h, period);
        for (std::size_t j = 0; j < v.size(); ++j) {
            const cplx next = edge_phase(edges[j + 1], h, period);
            sum += v[j] * (next - prev);
            prev = next;
        }
        c[static_cast<std::size_t>(h + hmax)] = segment_term(sum, h);
    }
    return c;
}

// Weights w(k, h + hmax) of every segment of one edge list (rcwa2d_operators.hpp:105-120)
inline Mat segment_weights(const std::vector<double>& edges, int hmax, double period) {
    const int K = static_cast<int>(edges.size()) - 1;
    Mat w(K, 2 * hmax + 1);
    for (int k = 0; k < K; ++k) w(k, hmax) = (edges[k + 1] - edges[k]) / period;
    for (int h = -hmax; h <= hmax; ++h) {
        if (h == 0) continue;
        for (int k = 0; k < K; ++k) w(k, h + hmax) = segment_term(edge_phase(edges[k + 1], h, period) - edge_phase(edges[k], h, period), h);
    }
    return w;
}

// (2M+1)-order Toeplitz block, (i, j) = c[i - j + 2M] (rcwa2d_operators.hpp:99-107)
inline Mat toeplitz(const CVec& c, int M) {
    const int n = 2 * M + 1;
    Mat t(n, n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) t(i, j) = c[static_cast<std::size_t>(i - j + 2 * M)];
    return t;
}

// out[h] = sum_k w(k, h) mats[k], k ascending (rcwa2d_operators.hpp:290-306)
inline std::vector<Mat> weighted(const Mat& w, const std::vector<Mat>& mats) {
    std::vector<Mat> out;
    for (int h = 0; h < w.cols; ++h) {
        Mat acc(mats[0].rows, mats[0].cols);
        for (std::size_t k = 0; k < mats.size(); ++k) {
            const cplx wk = w(static_cast<int>(k), h);
            for (std::size_t t = 0; t < acc.a.size(); ++t) acc.a[t] += wk * mats[k].a[t];
        }
        out.push_back(std::move(acc));
    }
    return out;
}

// Harmonic index of (m, n): (m + M1)(2 M2 + 1) + (n + M2). x-first blocks: blocks[n - n' + 2 M2](m, m');
// y-first blocks: blocks[m - m' + 2 M1](n, n') (rcwa2d_operators.hpp:208-249).
inline Mat assemble(const std::vector<Mat>& blocks, int M1, int M2, bool x_first) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2;
    Mat out(N, N);
    for (int a = 0; a < n1; ++a)
        for (int b = 0; b < n2; ++b)
            for (int ap = 0; ap < n1; ++ap)
                for (int bp = 0; bp < n2; ++bp)
                    out(a * n2 + b, ap * n2 + bp) = x_first ? blocks[static_cast<std::size_t>(b - bp + 2 * M2)](a, ap)
                                                            : blocks[static_cast<std::size_t>(a - ap + 2 * M1)](b, bp);
    return out;
}

// eps = n^2 of a strip's x profile at x, the profile repeating with period Lx from its first edge
// (rcwa2d_operators.hpp:162-171)
inline cplx eps_at(const XProfile& p, double x, double Lx) {
    const double xx = p.edges[0] + py_mod(x - p.edges[0], Lx);
    const long k = static_cast<long>(std::upper_bound(p.edges.begin(), p.edges.end(), xx) - p.edges.begin()) - 1;
    const long last = static_cast<long>(p.n.size()) - 1;
    const cplx n = p.n[static_cast<std::size_t>(std::min(std::max(k, 0L), last))];
    return n * n;
}

// The column boundaries: every strip edge mod Lx plus 0 and Lx, unique, rounded half-even to 12
// decimals, unique again, kept inside [-1e-12, Lx + 1e-12], 0 and Lx restored (rcwa2d_operators.hpp:178-192)
inline std::vector<double> column_cuts(const std::vector<XProfile>& strips, double Lx) {
    std::vector<double> c;
    for (const XProfile& p : strips)
        for (double e : p.edges) c.push_back(py_mod(e, Lx));
    c.push_back(0.0);
    c.push_back(Lx);
    const auto uniq = [](std::vector<double>& v) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    };
    uniq(c);
    for (double& x : c) x = std::rint(x * 1e12) / 1e12;
    uniq(c);
    std::vector<double> kept;
    for (double x : c)
        if (x >= -1e-12 && x <= Lx + 1e-12) kept.push_back(x);
    if (kept.empty() || kept.front() > 1e-12) kept.insert(kept.begin(), 0.0);
    if (kept.back() < Lx - 1e-12) kept.push_back(Lx);
    return kept;
}

inline CVec squares(const CVec& n) {
    CVec e(n.size());
    for (std::size_t j = 0; j < n.size(); ++j) e[j] = n[j] * n[j];
    return e;
}

// Eps, Cx, Cy of one layer (rcwa2d_operators.hpp:325-429); homogeneous layers give n^2 I three times.
// Throws Singular where an inverse-rule Toeplitz block is singular.
inline Operators layer_operators(const Layer& L, double Lx, double Ly, int M1, int M2, bool laurent) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2;
    Operators out;
    if (L.homogeneous) {
        out.eps = Mat(N, N);
        for (int i = 0; i < N; ++i) out.eps(i, i) = L.n * L.n;
        out.cx = out.cy = out.eps;
        return out;
    }
    const int K = static_cast<int>(L.strips.size());
    const Mat wy = segment_weights(L.y_edges, 2 * M2, Ly);
    std::vector<Mat> blocks;
    for (int k = 0; k < K; ++k) blocks.push_back(toeplitz(fourier(L.strips[k].edges, squares(L.strips[k].n), Lx, 2 * M1), M1));
    out.eps = assemble(weighted(wy, blocks), M1, M2, true);
    if (laurent) {
        out.cx = out.cy = out.eps;
        return out;
    }
    blocks.clear();
    for (int k = 0; k < K; ++k) {
        CVec inv = squares(L.strips[k].n);
        for (cplx& z : inv) z = cplx{1.0, 0.0} / z;
        blocks.push_back(solve(toeplitz(fourier(L.strips[k].edges, inv, Lx, 2 * M1), M1), Mat::eye(n1)));
    }
    out.cx = assemble(weighted(wy, blocks), M1, M2, true);
    const std::vector<double> cuts = column_cuts(L.strips, Lx);
    const int Kx = static_cast<int>(cuts.size()) - 1;
    const Mat wx = segment_weights(cuts, 2 * M1, Lx);
    blocks.clear();
    for (int j = 0; j < Kx; ++j) {
        const double xm = 0.5 * (cuts[j] + cuts[j + 1]);
        CVec col(static_cast<std::size_t>(K));
        for (int k = 0; k < K; ++k) col[k] = cplx{1.0, 0.0} / eps_at(L.strips[k], xm, Lx);
        blocks.push_back(solve(toeplitz(fourier(L.y_edges, col, Ly, 2 * M2), M2), Mat::eye(n2)));
    }
    out.cy = assemble(weighted(wx, blocks), M1, M2, false);
    return out;
}

// ------------------------------------------------------------------ modes

// Square-root branch (rcwa2d.hpp:360-364): negate when Re q < 0, then when Re q < 1e-10 and Im q > 0.
inline cplx branch(cplx q) {
    if (q.real() < 0.0) q = -q;
    if (q.real() < 1e-10 && q.imag() > 0.0) q = -q;
    return q;
}

// kz / k0 = sqrt(n^2 - Kx^2 - Ky^2) with Im >= 0 (rcwa2d.hpp:368-373)
inline cplx kz_over_k0(cplx n, double Kx, double Ky) {
    const cplx s = n * n - Kx * Kx - Ky * Ky;
    cplx kz = std::sqrt(s);
    if (kz.imag() < 0.0) kz = -kz;
    return kz;
}

// One region's modes, dense: tangential E = W [a+ e^(-k0 q (z - top)) + a- e^(-k0 q (bottom - z))],
// tangential H = V [-a+ ... + a- ...] (rcwa2d.hpp:375-384)
struct Modes {
    CVec q;
    Mat W, V;
    Mat Ei;  // structured layers: Eps^-1 (the near field's Ez)
};

// A homogeneous region (rcwa2d.hpp:386-410): W = I, q = branch(-i kz) twice, V = Qb / q with
// Qb = [[Kx Ky, n^2 - Kx^2], [Ky^2 - n^2, -Ky Kx]] per order
inline Modes homogeneous_modes(cplx n, const std::vector<double>& Kx, const std::vector<double>& Ky, const CVec& kz) {
    const int N = static_cast<int>(Kx.size());
    Modes m;
    m.q.resize(2 * static_cast<std::size_t>(N));
    m.W = Mat::eye(2 * N);
    m.V = Mat(2 * N, 2 * N);
    const cplx n2 = n * n;
    for (int i = 0; i < N; ++i) {
        const cplx q1 = branch(cplx{kz[i].imag(), -kz[i].real()});
        m.q[i] = m.q[N + i] = q1;
        m.V(i, i) = cplx{Kx[i] * Ky[i], 0.0} / q1;
        m.V(i, N + i) = (n2 - Kx[i] * Kx[i]) / q1;
        m.V(N + i, i) = (Ky[i] * Ky[i] - n2) / q1;
        m.V(N + i, N + i) = cplx{-Ky[i] * Kx[i], 0.0} / q1;
    }
    return m;
}

// A structured layer (rcwa2d.hpp:412-537): with Ei = Eps^-1 and Kx, Ky diagonal,
//   P = [[Kx Ei Ky, I - Kx Ei Kx], [Ky Ei Ky - I, -Ky Ei Kx]],  Q = [[Kx Ky, Cy - Kx^2], [Ky^2 - Cx, -Ky Kx]],
// H = P Q, H W = W diag(lambda), q = branch(sqrt(lambda)), V = Q W / q. Returns the eigensolver's info.
inline int structured_modes(const Operators& op, const std::vector<double>& Kx, const std::vector<double>& Ky, Modes& m) {
    const int N = static_cast<int>(Kx.size()), n = 2 * N;
    m.Ei = solve(op.eps, Mat::eye(N));
    const Mat& Ei = m.Ei;
    Mat P(n, n), Q(n, n);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            const cplx e = Ei(i, j);
            const double delta = i == j ? 1.0 : 0.0;
            P(i, j) = e * Kx[i] * Ky[j];
            P(i, N + j) = delta - e * Kx[i] * Kx[j];
            P(N + i, j) = e * Ky[i] * Ky[j] - delta;
            P(N + i, N + j) = -(e * Ky[i] * Kx[j]);
            Q(i, N + j) = op.cy(i, j) - (i == j ? Kx[i] * Kx[i] : 0.0);
            Q(N + i, j) = -op.cx(i, j) + (i == j ? Ky[i] * Ky[i] : 0.0);
        }
    for (int i = 0; i < N; ++i) {
        Q(i, i) = Kx[i] * Ky[i];
        Q(N + i, N + i) = -(Ky[i] * Kx[i]);
    }
    const EigOut e = eig_qr(matmul(P, Q));
    if (e.info != 0) return e.info;
    m.q.resize(static_cast<std::size_t>(n));
    for (int j = 0; j < n; ++j) m.q[j] = branch(std::sqrt(e.values[j]));
    m.W = e.vectors;
    m.V = matmul(Q, m.W);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) m.V(i, j) /= m.q[j];
    return 0;
}

// ------------------------------------------------------------------ the recursion

inline Mat plus_identity(Mat a, double s) {  // s I + a
    for (int i = 0; i < a.rows; ++i) a(i, i) += s;
    return a;
}
inline Mat neg(Mat a) {
    for (cplx& z : a.a) z = -z;
    return a;
}
inline Mat add(Mat a, const Mat& b, double s = 1.0) {  // a + s b
    for (std::size_t t = 0; t < a.a.size(); ++t) a.a[t] += s * b.a[t];
    return a;
}

// The step that carries the down-going amplitudes across one block, top to bottom.
struct Step {
    bool propagation = false;
    CVec x;        // propagation: diag(exp(-k0 q d))
    Mat tm, nn, rp;  // interface: down' = Tm (I + r') down + Nn down
};

// Interface (up | low) stacked on the reflection r below it, direct form (rcwa2d.hpp:738-790):
// Mm = W_low^-1 W_up, Nn = V_low^-1 V_up, A+- = (I + r) Nn +- (I - r) Mm, r' = A+^-1 A-, Tm = (Mm - Nn) / 2.
inline Mat interface_on(const Modes& up, const Modes& low, const Mat& r, Step& step) {
    const Mat mm = solve(low.W, up.W), nn = solve(low.V, up.V);
    const Mat pn = add(nn, matmul(r, nn)), qm = add(mm, matmul(r, mm), -1.0);
    const Mat rp = solve(add(pn, qm), add(pn, qm, -1.0));
    step.propagation = false;
    step.tm = add(mm, nn, -1.0);
    for (cplx& z : step.tm.a) z *= 0.5;
    step.nn = nn;
    step.rp = rp;
    return rp;
}

// Propagation through a layer of thickness d: Rdu = Rud = 0, Tdd = Tuu = X, so r' = X r X (rcwa2d.hpp:618-633)
inline Mat propagation_on(const CVec& q, double d, double k0, const Mat& r, Step& step) {
    step.propagation = true;
    step.x.resize(q.size());
    for (std::size_t i = 0; i < q.size(); ++i) step.x[i] = std::exp(-k0 * q[i] * d);
    Mat out = r;
    for (int j = 0; j < r.cols; ++j)
        for (int i = 0; i < r.rows; ++i) out(i, j) = step.x[i] * r(i, j) * step.x[j];
    return out;
}

inline CVec carry(const Step& s, const CVec& v) {
    if (s.propagation) {
        CVec out(v.size());
        for (std::size_t i = 0; i < v.size(); ++i) out[i] = s.x[i] * v[i];
        return out;
    }
    CVec u = matvec(s.rp, v);
    for (std::size_t i = 0; i < u.size(); ++i) u[i] += v[i];
    CVec out = matvec(s.tm, u);
    const CVec w = matvec(s.nn, v);
    for (std::size_t i = 0; i < out.size(); ++i) out[i] += w[i];
    return out;
}

// ------------------------------------------------------------------ the solve

inline bool finite_vec(const CVec& v) {
    for (const cplx& z : v)
        if (!finite(z)) return false;
    return true;
}

// rcwa::solve2d for one point (rcwa2d.hpp:1042-1347, :1359). ops[j] are layer j's operators (ignored for
// homogeneous layers).
inline void near_fields(const Stack& st, const std::vector<Modes>& modes, const std::vector<CVec>& a_plus,
                        const std::vector<CVec>& a_minus, const CVec& inc, const CVec& R, const CVec& T,
                        const Result& res, double k0, int i0, const std::vector<double>& zs, CVec& fields);

// rcwa::solve2d for one point (rcwa2d.hpp:1042-1347, :1359). ops[j] are layer j's operators (ignored for
// homogeneous layers). With zs, fields receives the near-field harmonics (6 components Ex, Ey, Ez, Hx, Hy, Hz
// x N orders x zs.size() depths, last index fastest), NaN where the solve failed.
inline Result solve2d(const Stack& st, const std::vector<Operators>& ops, double wavelength, double theta_deg,
                      double phi_deg, int M1, int M2, cplx Es, cplx Ep, const std::vector<double>* zs = nullptr,
                      CVec* fields = nullptr) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2, L = static_cast<int>(st.layers.size());
    const double nI = st.nI, k0 = 2.0 * kPi / wavelength;
    const double th = theta_deg * (kPi / 180.0), ph = phi_deg * (kPi / 180.0);
    const double cos_th = std::cos(th), sin_th = std::sin(th), cos_ph = std::cos(ph), sin_ph = std::sin(ph);
    Result res;
    res.Kx.resize(N);
    res.Ky.resize(N);
    res.kzI.resize(N);
    res.kzII.resize(N);
    res.prop_r.resize(N);
    res.prop_t.resize(N);
    res.rayleigh.assign(static_cast<std::size_t>(L) + 2, 0);
    std::vector<int> mm(N), nn(N);
    for (int a = 0; a < n1; ++a)
        for (int b = 0; b < n2; ++b) {
            const int i = a * n2 + b, m = a - M1, n = b - M2;
            mm[i] = m;
            nn[i] = n;
            res.Kx[i] = nI * sin_th * cos_ph - m * wavelength / st.Lx;
            res.Ky[i] = nI * sin_th * sin_ph - n * wavelength / st.Ly;
            res.kzI[i] = kz_over_k0(nI, res.Kx[i], res.Ky[i]);
            res.kzII[i] = kz_over_k0(st.nII, res.Kx[i], res.Ky[i]);
            res.prop_r[i] = res.kzI[i].real() > 1e-12;
            res.prop_t[i] = res.kzII[i].real() > 1e-12;
        }
    const auto fail = [&](int status) {
        const double nan = std::nan("");
        res.status = status;
        for (CVec* v : {&res.Ex_r, &res.Ey_r, &res.Ez_r, &res.Ex_t, &res.Ey_t, &res.Ez_t, &res.Rs, &res.Rp, &res.Ts, &res.Tp})
            v->assign(N, cplx{nan, nan});
        res.DEr.assign(N, nan);
        res.DEt.assign(N, nan);
        if (fields) fields->assign(6 * static_cast<std::size_t>(N) * (zs ? zs->size() : 0), cplx{nan, nan});
        return res;
    };
    // Rayleigh anomalies: an order with kz exactly 0 in a homogeneous region (rcwa2d.hpp:1094-1112)
    std::vector<CVec> kz_layer(static_cast<std::size_t>(L));
    bool rayleigh = false;
    const auto mark = [&](const CVec& kz, int region) {
        for (const cplx& z : kz)
            if (z == cplx{}) {
                res.rayleigh[region] = 1;
                rayleigh = true;
            }
    };
    mark(res.kzI, 0);
    mark(res.kzII, L + 1);
    for (int j = 0; j < L; ++j) {
        if (!st.layers[j].homogeneous) continue;
        kz_layer[j].resize(N);
        for (int i = 0; i < N; ++i) kz_layer[j][i] = kz_over_k0(st.layers[j].n, res.Kx[i], res.Ky[i]);
        mark(kz_layer[j], j + 1);
    }
    if (rayleigh) return fail(kRayleigh);
    try {
        // modes: region 0 the incident medium, j + 1 layer j, L + 1 the exit medium
        std::vector<Modes> modes(static_cast<std::size_t>(L) + 2);
        modes[0] = homogeneous_modes(nI, res.Kx, res.Ky, res.kzI);
        modes[L + 1] = homogeneous_modes(st.nII, res.Kx, res.Ky, res.kzII);
        for (int j = 0; j < L; ++j) {
            if (st.layers[j].homogeneous) {
                modes[j + 1] = homogeneous_modes(st.layers[j].n, res.Kx, res.Ky, kz_layer[j]);
                continue;
            }
            ++res.n_eig;
            const int info = structured_modes(ops[j], res.Kx, res.Ky, modes[j + 1]);
            if (info != 0) {
                res.eig_info = info;
                return fail(kEigNoConv);
            }
            if (!modes[j + 1].W.all_finite() || !modes[j + 1].V.all_finite()) return fail(kNumerical);
        }
        // incident vector: the (0, 0) order's Ex, Ey (rcwa2d.hpp:1166-1170)
        const int i0 = M1 * n2 + M2;
        CVec inc(2 * static_cast<std::size_t>(N));
        inc[i0] = -Es * sin_ph + Ep * cos_th * cos_ph;
        inc[N + i0] = Es * cos_ph + Ep * cos_th * sin_ph;
        // blocks 2j: the interface between regions j and j + 1; 2j + 1: propagation in layer j; stacked from
        // the exit medium (r = 0) up to block 1, block 0 (the top interface) solved directly
        const int blocks = 2 * L + 1;
        std::vector<Step> steps(static_cast<std::size_t>(blocks));
        std::vector<Mat> r_below(static_cast<std::size_t>(L));  // the reflection under each layer
        Mat r(2 * N, 2 * N);
        for (int b = blocks - 1; b >= 1; --b) {
            const int j = b / 2;
            if (b % 2 == 0) {
                r = interface_on(modes[j], modes[j + 1], r, steps[b]);
            } else {
                if (fields) r_below[j] = r;
                r = propagation_on(modes[j + 1].q, st.layers[j].d, k0, r, steps[b]);
            }
        }
        // top: e + R = W (I + r) d, V_I (e - R) = V (I - r) d  =>  [W (I + r) + V_I^-1 V (I - r)] d = 2 e
        const Modes& low = modes[1];
        const Mat wp = matmul(low.W, plus_identity(r, 1.0));
        const Mat vq = matmul(low.V, plus_identity(neg(r), 1.0));
        Mat rhs(2 * N, 1);
        for (int i = 0; i < 2 * N; ++i) rhs(i, 0) = 2.0 * inc[i];
        const Mat dmat = solve(add(wp, solve(modes[0].V, vq)), rhs);
        CVec down(dmat.a);
        CVec R = matvec(wp, down);
        for (int i = 0; i < 2 * N; ++i) R[i] -= inc[i];
        std::vector<CVec> a_plus(static_cast<std::size_t>(L)), a_minus(static_cast<std::size_t>(L));
        for (int b = 1; b < blocks; ++b) {
            const bool propagation = b % 2 != 0;
            if (fields && propagation) a_plus[b / 2] = down;  // at the layer's top
            down = carry(steps[b], down);
            if (fields && propagation) a_minus[b / 2] = matvec(r_below[b / 2], down);  // at its bottom
        }
        const CVec& T = down;
        if (!finite_vec(R) || !finite_vec(T)) return fail(kNumerical);
        // efficiencies and s/p amplitudes (rcwa2d.hpp:1226-1262)
        const auto efficiency = [&](const CVec& F, const CVec& kz, double sign, CVec& Ex, CVec& Ey, CVec& Ez,
                                    std::vector<double>& de) {
            Ex.assign(F.begin(), F.begin() + N);
            Ey.assign(F.begin() + N, F.end());
            Ez.assign(N, cplx{});
            de.assign(N, 0.0);
            for (int i = 0; i < N; ++i) {
                if (!(kz[i].real() > 1e-12)) continue;
                Ez[i] = -sign * (res.Kx[i] * Ex[i] + res.Ky[i] * Ey[i]) / kz[i];
                const double E2 = std::norm(Ex[i]) + std::norm(Ey[i]) + std::norm(Ez[i]);
                de[i] = kz[i].real() * E2 / (nI * cos_th);
            }
        };
        const auto spol = [&](const CVec& Ex, const CVec& Ey, const CVec& kz, cplx n_med, double sign, CVec& s, CVec& p) {
            s.resize(N);
            p.resize(N);
            for (int i = 0; i < N; ++i) {
                const double kt = std::hypot(res.Kx[i], res.Ky[i]);
                const cplx cth = std::abs(kz[i]) > 1e-12 ? kz[i] / n_med : cplx{1.0, 0.0};
                if (kt > 1e-12) {
                    s[i] = (-res.Ky[i] * Ex[i] + res.Kx[i] * Ey[i]) / kt;
                    p[i] = sign * (res.Kx[i] * Ex[i] + res.Ky[i] * Ey[i]) / (kt * cth);
                } else {
                    s[i] = -sin_ph * Ex[i] + cos_ph * Ey[i];
                    p[i] = sign * (cos_ph * Ex[i] + sin_ph * Ey[i]) / cth;
                }
            }
        };
        efficiency(R, res.kzI, -1.0, res.Ex_r, res.Ey_r, res.Ez_r, res.DEr);
        efficiency(T, res.kzII, +1.0, res.Ex_t, res.Ey_t, res.Ez_t, res.DEt);
        spol(res.Ex_r, res.Ey_r, res.kzI, cplx{nI, 0.0}, -1.0, res.Rs, res.Rp);
        spol(res.Ex_t, res.Ey_t, res.kzII, st.nII, +1.0, res.Ts, res.Tp);
        for (int i = 0; i < N; ++i)
            if (!std::isfinite(res.DEr[i]) || !std::isfinite(res.DEt[i]) || !finite(res.Rs[i]) || !finite(res.Rp[i]) ||
                !finite(res.Ts[i]) || !finite(res.Tp[i]))
                return fail(kNumerical);
        if (fields) {
            near_fields(st, modes, a_plus, a_minus, inc, R, T, res, k0, i0, *zs, *fields);
            if (!finite_vec(*fields)) return fail(kNumerical);
        }
    } catch (const Singular&) {
        return fail(kNumerical);
    }
    return res;
}

// The six near-field harmonics at each depth (include/stablercwa/rcwa2d_fields.hpp:17-43). z runs down from
// the top surface (z = 0) to z_bot, the sum of the thicknesses. A depth belongs to the incident region when
// z < 0, to the exit region when z > z_bot (or when there are no layers), else to the first layer with
// z <= z_top + d + 1e-12, its distance from the layer's top clamped to [0, d]. Per region:
//   incident:  F = inc e^(-k0 q z) + R e^(k0 q z), G = V_I (-inc e^(-k0 q z) + R e^(k0 q z)), the incident term
//              only on the (0, 0) order's two entries (where inc is non-zero), Ei = 1 / nI^2;
//   exit:      F = T e^(-k0 q (z - z_bot)), G = -V_II F, Ei = 1 / nII^2;
//   layer:     F = W (a+ e^(-k0 q zl) + a- e^(-k0 q (d - zl))), G = V (-a+ ... + a- ...), Ei = Eps^-1 (1 / n^2
//              for a homogeneous layer);
// then Ex, Ey = F's halves, hx, hy = G's halves, hz = i (Ky Ex - Kx Ey), Ez = i Ei (Ky hx - Kx hy),
// (Hx, Hy, Hz) = -i (hx, hy, hz).
inline void near_fields(const Stack& st, const std::vector<Modes>& modes, const std::vector<CVec>& a_plus,
                        const std::vector<CVec>& a_minus, const CVec& inc, const CVec& R, const CVec& T,
                        const Result& res, double k0, int i0, const std::vector<double>& zs, CVec& fields) {
    const int N = static_cast<int>(res.Kx.size()), L = static_cast<int>(st.layers.size());
    const std::size_t nz = zs.size();
    fields.assign(6 * static_cast<std::size_t>(N) * nz, cplx{});
    std::vector<double> top(static_cast<std::size_t>(L));
    double zbot = 0.0;
    for (int j = 0; j < L; ++j) {
        top[j] = zbot;
        zbot += st.layers[j].d;
    }
    const cplx I{0.0, 1.0};
    for (std::size_t iz = 0; iz < nz; ++iz) {
        const double z = zs[iz];
        int region = -1;  // -1 incident, L exit, else the layer
        if (z < 0.0) region = -1;
        else if (L == 0 || z > zbot) region = L;
        else {
            region = L;
            for (int j = 0; j < L; ++j)
                if (z <= top[j] + st.layers[j].d + 1e-12) {
                    region = j;
                    break;
                }
        }
        CVec F(2 * static_cast<std::size_t>(N)), u(2 * static_cast<std::size_t>(N));
        const Mat* Vm = nullptr;
        const Mat* Eim = nullptr;
        cplx inv_eps{};
        if (region < 0) {
            const Modes& m = modes[0];
            for (int i = 0; i < 2 * N; ++i) {
                const cplx up = R[i] * std::exp(k0 * m.q[i] * z);
                F[i] = up;
                u[i] = up;
            }
            for (int i : {i0, N + i0}) {
                const cplx dn = inc[i] * std::exp(-k0 * m.q[i] * z);
                F[i] += dn;
                u[i] -= dn;
            }
            Vm = &m.V;
            inv_eps = cplx{1.0, 0.0} / (cplx{st.nI, 0.0} * st.nI);
        } else if (region == L) {
            const Modes& m = modes[L + 1];
            for (int i = 0; i < 2 * N; ++i) {
                F[i] = T[i] * std::exp(-k0 * m.q[i] * (z - zbot));
                u[i] = -F[i];
            }
            Vm = &m.V;
            inv_eps = cplx{1.0, 0.0} / (st.nII * st.nII);
        } else {
            const Modes& m = modes[region + 1];
            const double d = st.layers[region].d, zl = std::min(std::max(z - top[region], 0.0), d);
            CVec w(2 * static_cast<std::size_t>(N));
            for (int i = 0; i < 2 * N; ++i) {
                const cplx ep = a_plus[region][i] * std::exp(-k0 * m.q[i] * zl);
                const cplx em = a_minus[region][i] * std::exp(-k0 * m.q[i] * (d - zl));
                w[i] = ep + em;
                u[i] = em - ep;
            }
            F = matvec(m.W, w);
            Vm = &m.V;
            if (st.layers[region].homogeneous) inv_eps = cplx{1.0, 0.0} / (st.layers[region].n * st.layers[region].n);
            else Eim = &m.Ei;
        }
        const CVec G = matvec(*Vm, u);
        CVec t(static_cast<std::size_t>(N));
        for (int i = 0; i < N; ++i) t[i] = res.Ky[i] * G[i] - res.Kx[i] * G[N + i];
        const CVec ez = Eim ? matvec(*Eim, t) : t;
        for (int i = 0; i < N; ++i) {
            const cplx hz = I * (res.Ky[i] * F[i] - res.Kx[i] * F[N + i]);
            const cplx vals[6] = {F[i], F[N + i], I * (Eim ? ez[i] : inv_eps * ez[i]), -I * G[i], -I * G[N + i], -I * hz};
            for (int c = 0; c < 6; ++c) fields[(static_cast<std::size_t>(c) * N + i) * nz + iz] = vals[c];
        }
    }
}

}  // namespace r2d
}  // namespace oracle
