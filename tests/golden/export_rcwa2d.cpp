// Golden-fixture exporter for the 2-D (crossed-grating) solve.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_rcwa2d_reference.cpp in place (main() renamed) and its
// data file tests/rcwa2d_core_fixture.inc, so the frozen tables of both (Kx, Ky, kz, field amplitudes,
// s/p amplitudes and efficiencies per order, Rayleigh failures, and the Eps / Cx / Cy operators) come
// from the reference itself. A few further structures with more layers and larger orders are built
// here; for every case the reference's own rcwa::solve2d result is written beside the table. One
// JSON object per line.
#define main stablercwa_reference_rcwa2d_test_main
#include "test_rcwa2d_reference.cpp"
#undef main
#include "rcwa2d_core_fixture.inc"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>

namespace {

// shortest decimal that reads back to the same double
void put_d(std::FILE* f, double v) {
    if (std::isnan(v)) { std::fprintf(f, "\"nan\""); return; }
    if (std::isinf(v)) { std::fprintf(f, v > 0 ? "\"inf\"" : "\"-inf\""); return; }
    char buf[40];
    for (int prec = 15; prec <= 17; ++prec) {
        std::snprintf(buf, sizeof buf, "%.*g", prec, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::fputs(buf, f);
}
void put_c(std::FILE* f, cplx z) {
    std::fputc('[', f);
    put_d(f, z.real());
    std::fputc(',', f);
    put_d(f, z.imag());
    std::fputc(']', f);
}
void put_cvec(std::FILE* f, const char* key, const Vector& v) {
    std::fprintf(f, "\"%s\":[", key);
    for (std::size_t i = 0; i < v.size(); ++i) {
        if (i) std::fputc(',', f);
        put_c(f, v[i]);
    }
    std::fputc(']', f);
}
void put_rvec(std::FILE* f, const char* key, const RealVector& v) {
    std::fprintf(f, "\"%s\":[", key);
    for (std::size_t i = 0; i < v.size(); ++i) {
        if (i) std::fputc(',', f);
        put_d(f, v[i]);
    }
    std::fputc(']', f);
}
// interleaved (re, im) doubles, count complex values
void put_pairs(std::FILE* f, const char* key, const double* p, int count) {
    std::fprintf(f, "\"%s\":[", key);
    for (int i = 0; i < count; ++i) {
        if (i) std::fputc(',', f);
        put_c(f, cplx{p[2 * i], p[2 * i + 1]});
    }
    std::fputc(']', f);
}
void put_reals(std::FILE* f, const char* key, const double* p, int count) {
    std::fprintf(f, "\"%s\":[", key);
    for (int i = 0; i < count; ++i) {
        if (i) std::fputc(',', f);
        put_d(f, p[i]);
    }
    std::fputc(']', f);
}

void put_stack(std::FILE* f, const rcwa::Stack2D& s) {
    std::fprintf(f, "\"stack\":{\"nI\":");
    put_d(f, s.nI);
    std::fprintf(f, ",\"nII\":");
    put_c(f, s.nII);
    std::fprintf(f, ",\"Lx\":");
    put_d(f, s.Lx);
    std::fprintf(f, ",\"Ly\":");
    put_d(f, s.Ly);
    std::fprintf(f, ",\"layers\":[");
    for (std::size_t k = 0; k < s.layers.size(); ++k) {
        const rcwa::Layer2D& L = s.layers[k];
        std::fprintf(f, "%s{\"d\":", k ? "," : "");
        put_d(f, L.d);
        if (L.homogeneous) {
            std::fprintf(f, ",\"n\":");
            put_c(f, L.n);
        } else {
            std::fprintf(f, ",\"y_edges\":[");
            for (std::size_t j = 0; j < L.y_edges.size(); ++j) {
                if (j) std::fputc(',', f);
                put_d(f, L.y_edges[j]);
            }
            std::fprintf(f, "],\"x_profiles\":[");
            for (std::size_t p = 0; p < L.x_profiles.size(); ++p) {
                const rcwa::XProfile2D& xp = L.x_profiles[p];
                std::fprintf(f, "%s{\"edges\":[", p ? "," : "");
                for (std::size_t j = 0; j < xp.edges.size(); ++j) {
                    if (j) std::fputc(',', f);
                    put_d(f, xp.edges[j]);
                }
                std::fprintf(f, "],\"n_values\":[");
                for (std::size_t j = 0; j < xp.n_values.size(); ++j) {
                    if (j) std::fputc(',', f);
                    put_c(f, xp.n_values[j]);
                }
                std::fprintf(f, "]}");
            }
            std::fprintf(f, "]");
        }
        std::fprintf(f, "}");
    }
    std::fprintf(f, "]}");
}

// Regions whose exact kz == 0 makes the reference report a Rayleigh anomaly, with their (m, n),
// found with the reference's own kz (rcwa2d.hpp:1099-1113): "incident", "exit", "layer<j>" (1-based).
void put_rayleigh(std::FILE* f, const rcwa::Stack2D& s, const rcwa::Result2D& r) {
    std::fprintf(f, "\"rayleigh\":[");
    bool first = true;
    auto region = [&](const char* name, int layer, cplx n) {
        std::string orders;
        for (int i = 0; i < r.N; ++i) {
            const cplx kz = rcwa::detail2d::kz_over_k0(n, r.Kx[i], r.Ky[i]);
            if (kz != cplx{}) continue;
            orders += (orders.empty() ? "" : ",") + std::string("[") + std::to_string(r.m[i]) + "," + std::to_string(r.n[i]) + "]";
        }
        if (orders.empty()) return;
        std::fprintf(f, "%s{\"region\":\"%s\",\"layer\":%d,\"orders\":[%s]}", first ? "" : ",", name, layer, orders.c_str());
        first = false;
    };
    region("incident", -1, cplx{s.nI, 0.0});
    region("exit", -1, s.nII);
    for (std::size_t j = 0; j < s.layers.size(); ++j)
        if (s.layers[j].homogeneous) region("layer", static_cast<int>(j), s.layers[j].n);
    std::fprintf(f, "]");
}

void put_result(std::FILE* f, const rcwa::Result2D& r, bool full) {
    std::fprintf(f, "\"ref\":{\"status\":%d,\"eig_info\":%d,\"n_eig\":%d,\"n_dense_solve\":%d,",
                 static_cast<int>(r.status), r.eig_info, r.n_eig, r.n_dense_solve);
    if (full) {
        put_rvec(f, "Kx", r.Kx); std::fputc(',', f);
        put_rvec(f, "Ky", r.Ky); std::fputc(',', f);
        put_cvec(f, "kzI", r.kzI); std::fputc(',', f);
        put_cvec(f, "kzII", r.kzII); std::fputc(',', f);
        put_cvec(f, "Ex_r", r.Ex_r); std::fputc(',', f);
        put_cvec(f, "Ey_r", r.Ey_r); std::fputc(',', f);
        put_cvec(f, "Ez_r", r.Ez_r); std::fputc(',', f);
        put_cvec(f, "Ex_t", r.Ex_t); std::fputc(',', f);
        put_cvec(f, "Ey_t", r.Ey_t); std::fputc(',', f);
        put_cvec(f, "Ez_t", r.Ez_t); std::fputc(',', f);
        std::fprintf(f, "\"prop_r\":[");
        for (std::size_t i = 0; i < r.prop_r.size(); ++i) std::fprintf(f, "%s%d", i ? "," : "", r.prop_r[i] ? 1 : 0);
        std::fprintf(f, "],\"prop_t\":[");
        for (std::size_t i = 0; i < r.prop_t.size(); ++i) std::fprintf(f, "%s%d", i ? "," : "", r.prop_t[i] ? 1 : 0);
        std::fprintf(f, "],");
    }
    put_cvec(f, "Rs", r.Rs); std::fputc(',', f);
    put_cvec(f, "Rp", r.Rp); std::fputc(',', f);
    put_cvec(f, "Ts", r.Ts); std::fputc(',', f);
    put_cvec(f, "Tp", r.Tp); std::fputc(',', f);
    put_rvec(f, "DEr", r.DEr); std::fputc(',', f);
    put_rvec(f, "DEt", r.DEt);
    std::fprintf(f, "}");
}

struct Case {
    std::string name, source;
    rcwa::Stack2D stack;
    double wavelength, theta, phi;
    int M1, M2;
    rcwa::Jones2D jones;
    bool laurent;
};

void put_head(std::FILE* f, const Case& c) {
    std::fprintf(f, "{\"name\":\"%s\",\"source\":\"%s\",", c.name.c_str(), c.source.c_str());
    put_stack(f, c.stack);
    std::fprintf(f, ",\"wavelength\":");
    put_d(f, c.wavelength);
    std::fprintf(f, ",\"theta\":");
    put_d(f, c.theta);
    std::fprintf(f, ",\"phi\":");
    put_d(f, c.phi);
    std::fprintf(f, ",\"M1\":%d,\"M2\":%d,\"jones\":[", c.M1, c.M2);
    put_c(f, c.jones[0]);
    std::fputc(',', f);
    put_c(f, c.jones[1]);
    std::fprintf(f, "],\"laurent\":%d,", c.laurent ? 1 : 0);
}

rcwa::Result2D run(const Case& c) {
    rcwa::Options2D o;
    o.factorization = c.laurent ? rcwa::Factorization2D::Laurent : rcwa::Factorization2D::Li;
    return rcwa::solve2d(c.stack, c.wavelength, c.theta, c.phi, c.M1, c.M2, c.jones, o);
}

// ---- the reference's frozen tables (tests/rcwa2d_reference.inc, checked by tests/test_rcwa2d_reference.cpp:75-110)
void export_reference_case(std::FILE* f, const Rcwa2dRefCase& rc) {
    Case c{std::string("ref_") + std::to_string(rc.id) + "_" + rc.name, "tests/rcwa2d_reference.inc",
           rcwa2d_ref_stack(rc.id), rc.wavelength, rc.theta_deg, rc.phi_deg, rc.M1, rc.M2,
           {cplx{rc.jones[0], rc.jones[1]}, cplx{rc.jones[2], rc.jones[3]}}, rc.laurent != 0};
    const rcwa::Result2D r = run(c);
    put_head(f, c);
    std::fprintf(f, "\"table_status\":%d,", rc.status == 0 ? 0 : 2);
    if (rc.status == 0) {
        const int N = rc.count;
        std::vector<double> Kx(N), Ky(N), DEr(N), DEt(N);
        std::vector<double> kzI(2 * N), kzII(2 * N), fld[10];
        for (auto& v : fld) v.resize(2 * N);
        std::vector<int> pr(N), pt(N);
        for (int i = 0; i < N; ++i) {
            const Rcwa2dRefOrder& o = rc.orders[i];
            Kx[i] = o.Kx; Ky[i] = o.Ky; DEr[i] = o.DEr; DEt[i] = o.DEt; pr[i] = o.prop_r; pt[i] = o.prop_t;
            kzI[2 * i] = o.kzI[0]; kzI[2 * i + 1] = o.kzI[1];
            kzII[2 * i] = o.kzII[0]; kzII[2 * i + 1] = o.kzII[1];
            const double* src[10] = {o.Ex_r, o.Ey_r, o.Ez_r, o.Ex_t, o.Ey_t, o.Ez_t, o.Rs, o.Rp, o.Ts, o.Tp};
            for (int k = 0; k < 10; ++k) { fld[k][2 * i] = src[k][0]; fld[k][2 * i + 1] = src[k][1]; }
        }
        static const char* names[10] = {"Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"};
        std::fprintf(f, "\"table\":{\"m\":[");
        for (int i = 0; i < N; ++i) std::fprintf(f, "%s%d", i ? "," : "", rc.orders[i].m);
        std::fprintf(f, "],\"n\":[");
        for (int i = 0; i < N; ++i) std::fprintf(f, "%s%d", i ? "," : "", rc.orders[i].n);
        std::fprintf(f, "],");
        put_reals(f, "Kx", Kx.data(), N); std::fputc(',', f);
        put_reals(f, "Ky", Ky.data(), N); std::fputc(',', f);
        put_pairs(f, "kzI", kzI.data(), N); std::fputc(',', f);
        put_pairs(f, "kzII", kzII.data(), N); std::fputc(',', f);
        for (int k = 0; k < 10; ++k) { put_pairs(f, names[k], fld[k].data(), N); std::fputc(',', f); }
        put_reals(f, "DEr", DEr.data(), N); std::fputc(',', f);
        put_reals(f, "DEt", DEt.data(), N);
        std::fprintf(f, ",\"prop_r\":[");
        for (int i = 0; i < N; ++i) std::fprintf(f, "%s%d", i ? "," : "", pr[i] ? 1 : 0);
        std::fprintf(f, "],\"prop_t\":[");
        for (int i = 0; i < N; ++i) std::fprintf(f, "%s%d", i ? "," : "", pt[i] ? 1 : 0);
        std::fprintf(f, "],\"atol\":");
        put_d(f, rc.far_atol);
        std::fprintf(f, ",\"rtol\":");
        put_d(f, rc.far_rtol);
        std::fprintf(f, "},");
    } else {
        std::fprintf(f, "\"table_failure\":{\"count\":%d,\"orders\":[", rc.failure_count);
        for (int i = 0; i < rc.failure_count; ++i)
            std::fprintf(f, "%s[%d,%d]", i ? "," : "", rc.failure_orders[i][0], rc.failure_orders[i][1]);
        std::fprintf(f, "]},");
    }
    std::fprintf(f, "\"operators\":[");
    for (int k = 0; k < rc.operator_count; ++k) {
        const Rcwa2dRefOperators& o = rc.operators[k];
        std::fprintf(f, "%s{\"layer\":%d,\"N\":%d,", k ? "," : "", o.layer, o.N);
        put_pairs(f, "eps", o.eps, o.N * o.N); std::fputc(',', f);
        put_pairs(f, "cx", o.cx, o.N * o.N); std::fputc(',', f);
        put_pairs(f, "cy", o.cy, o.N * o.N);
        std::fprintf(f, "}");
    }
    std::fprintf(f, "],");
    put_rayleigh(f, c.stack, r);
    std::fputc(',', f);
    put_result(f, r, false);
    std::fprintf(f, "}\n");
}

// ---- the core fixture (tests/rcwa2d_core_fixture.inc, checked by tests/test_rcwa2d.cpp:263-300)
void export_core_case(std::FILE* f, const CoreRefCase& cc) {
    Case c;
    c.name = std::string("core_") + std::to_string(cc.id) + "_" + cc.name;
    c.source = "tests/rcwa2d_core_fixture.inc";
    c.stack.nI = cc.nI;
    c.stack.nII = cplx{cc.nII_re, cc.nII_im};
    c.stack.Lx = cc.Lx;
    c.stack.Ly = cc.Ly;
    c.wavelength = cc.wavelength;
    c.theta = cc.theta_deg;
    c.phi = cc.phi_deg;
    c.M1 = cc.M1;
    c.M2 = cc.M2;
    c.jones = {cplx{cc.jones[0], cc.jones[1]}, cplx{cc.jones[2], cc.jones[3]}};
    c.laurent = std::string(cc.name).find("laurent") != std::string::npos;
    for (int j = 0; j < cc.layer_count; ++j) {
        const CoreRefLayer& L = cc.layers[j];
        if (L.homogeneous) {
            c.stack.layers.push_back(rcwa::Layer2D::uniform(L.d, cplx{L.n_re, L.n_im}, L.name));
            continue;
        }
        std::vector<double> ye(L.y_edges, L.y_edges + L.K + 1);
        std::vector<rcwa::XProfile2D> rows;
        const double* xe = L.x_edges;
        const double* nv = L.n_values;
        for (int k = 0; k < L.K; ++k) {
            rcwa::XProfile2D row;
            row.edges.assign(xe, xe + L.x_count[k] + 1);
            for (int s = 0; s < L.x_count[k]; ++s) row.n_values.push_back(cplx{nv[2 * s], nv[2 * s + 1]});
            xe += L.x_count[k] + 1;
            nv += 2 * L.x_count[k];
            rows.push_back(std::move(row));
        }
        c.stack.layers.push_back(rcwa::Layer2D::patterned(L.d, std::move(ye), std::move(rows), L.name));
    }
    const rcwa::Result2D r = run(c);
    put_head(f, c);
    const int N = cc.N;
    std::fprintf(f, "\"table_status\":%d,", cc.status == 0 ? 0 : 2);
    if (cc.status == 0) {
        std::fprintf(f, "\"table\":{");
        put_reals(f, "Kx", cc.Kx, N); std::fputc(',', f);
        put_reals(f, "Ky", cc.Ky, N); std::fputc(',', f);
        put_pairs(f, "kzI", cc.kzI, N); std::fputc(',', f);
        put_pairs(f, "kzII", cc.kzII, N); std::fputc(',', f);
        const double* src[10] = {cc.Ex_r, cc.Ey_r, cc.Ez_r, cc.Ex_t, cc.Ey_t, cc.Ez_t, cc.Rs, cc.Rp, cc.Ts, cc.Tp};
        static const char* names[10] = {"Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"};
        for (int k = 0; k < 10; ++k) { put_pairs(f, names[k], src[k], N); std::fputc(',', f); }
        put_reals(f, "DEr", cc.DEr, N); std::fputc(',', f);
        put_reals(f, "DEt", cc.DEt, N);
        std::fprintf(f, ",\"atol\":1e-09,\"rtol\":1e-09},");
    }
    std::fprintf(f, "\"operators\":[");
    bool first = true;
    for (int j = 0; j < cc.layer_count; ++j) {
        const CoreRefLayer& L = cc.layers[j];
        if (L.homogeneous || !L.eps) continue;
        std::fprintf(f, "%s{\"layer\":%d,\"N\":%d,", first ? "" : ",", j, N);
        put_pairs(f, "eps", L.eps, N * N); std::fputc(',', f);
        put_pairs(f, "cx", L.cx, N * N); std::fputc(',', f);
        put_pairs(f, "cy", L.cy, N * N);
        std::fprintf(f, "}");
        first = false;
    }
    std::fprintf(f, "],");
    put_rayleigh(f, c.stack, r);
    std::fputc(',', f);
    put_result(f, r, false);
    std::fprintf(f, "}\n");
}

// ---- further structures (no frozen table; the reference's solve2d is the only authority)

rcwa::XProfile2D row(double Lx, double x0, double x1, cplx n_in, cplx n_out) {
    rcwa::XProfile2D p;
    if (x1 <= x0) {
        p.edges = {0.0, Lx};
        p.n_values = {n_out};
    } else {
        p.edges = {0.0, x0, x1, Lx};
        p.n_values = {n_out, n_in, n_out};
    }
    return p;
}

// circular pillar of radius r centred in the cell, staircased into K equal y-strips
rcwa::Layer2D circle_layer(double d, double Lx, double Ly, double r, int K, cplx n_in, cplx n_out) {
    std::vector<double> ye(K + 1);
    std::vector<rcwa::XProfile2D> rows;
    for (int k = 0; k <= K; ++k) ye[k] = Ly * k / K;
    ye[K] = Ly;
    for (int k = 0; k < K; ++k) {
        const double yc = 0.5 * (ye[k] + ye[k + 1]) - 0.5 * Ly;
        const double w2 = r * r - yc * yc;
        const double w = w2 > 0 ? std::sqrt(w2) : 0.0;
        rows.push_back(row(Lx, 0.5 * Lx - w, 0.5 * Lx + w, n_in, n_out));
    }
    return rcwa::Layer2D::patterned(d, ye, rows);
}

// rectangle w x h centred in the cell
rcwa::Layer2D rect_layer(double d, double Lx, double Ly, double w, double h, cplx n_in, cplx n_out) {
    const std::vector<double> ye = {0.0, 0.5 * (Ly - h), 0.5 * (Ly + h), Ly};
    std::vector<rcwa::XProfile2D> rows = {row(Lx, 0, 0, n_in, n_out), row(Lx, 0.5 * (Lx - w), 0.5 * (Lx + w), n_in, n_out),
                                          row(Lx, 0, 0, n_in, n_out)};
    return rcwa::Layer2D::patterned(d, ye, rows);
}

std::vector<Case> generated_cases() {
    std::vector<Case> out;
    const double P = 0.8;
    auto base = [&](const std::string& name) {
        Case c;
        c.name = name;
        c.source = "generated";
        c.stack.nI = 1.0;
        c.stack.nII = cplx{1.46, 0.0};
        c.stack.Lx = P;
        c.stack.Ly = P;
        c.wavelength = 0.7;
        c.theta = 0.0;
        c.phi = 0.0;
        c.M1 = c.M2 = 3;
        c.jones = {cplx{1.0, 0.0}, cplx{0.0, 0.0}};
        c.laurent = false;
        return c;
    };
    // three patterned layers between five films, normal incidence, s polarisation
    const auto pillars = [&](Case& c) {
        auto& L = c.stack.layers;
        L.push_back(rcwa::Layer2D::uniform(0.12, 1.7));
        L.push_back(circle_layer(0.2, P, P, 0.3 * P, 8, 2.0, 1.0));
        L.push_back(rcwa::Layer2D::uniform(0.08, 1.45));
        L.push_back(rect_layer(0.15, P, P, 0.5 * P, 0.35 * P, 2.0, 1.0));
        L.push_back(rcwa::Layer2D::uniform(0.1, 2.1));
        L.push_back(rcwa::Layer2D::uniform(0.06, 1.38));
        L.push_back(circle_layer(0.1, P, P, 0.22 * P, 8, 2.0, 1.0));
        L.push_back(rcwa::Layer2D::uniform(0.15, 1.9));
    };
    {
        Case c = base("pillars_films_normal");
        pillars(c);
        out.push_back(c);
    }
    {
        Case c = base("pillars_films_oblique");
        pillars(c);
        c.theta = 23.0;
        c.phi = 37.0;
        c.wavelength = 0.83;
        c.jones = {cplx{0.6, 0.2}, cplx{0.7745966692414834, 0.0}};
        out.push_back(c);
    }
    {
        // patterned layers touching each other and both half-spaces; absorbing pillar; Laurent rule
        Case c = base("adjacent_patterned_laurent");
        c.laurent = true;
        c.M1 = 2;
        c.M2 = 3;
        c.stack.Ly = 0.9;
        c.theta = 31.0;
        c.phi = -12.0;
        c.jones = {cplx{0.0, 0.0}, cplx{1.0, 0.0}};
        auto& L = c.stack.layers;
        L.push_back(rect_layer(0.11, P, 0.9, 0.4 * P, 0.6 * 0.9, cplx{1.8, 0.05}, 1.0));
        L.push_back(circle_layer(0.09, P, 0.9, 0.25 * P, 6, 2.3, 1.2));
        L.push_back(rect_layer(0.13, P, 0.9, 0.7 * P, 0.3 * 0.9, 1.6, 1.0));
        out.push_back(c);
    }
    {
        // the same stack with the Li rule and films between, absorbing exit medium
        Case c = base("adjacent_patterned_li");
        c.M1 = 3;
        c.M2 = 2;
        c.stack.Lx = 0.7;
        c.stack.nII = cplx{1.5, 0.02};
        c.theta = 12.0;
        c.phi = 71.0;
        c.jones = {cplx{0.5, 0.5}, cplx{0.0, 0.7071067811865476}};
        auto& L = c.stack.layers;
        L.push_back(rect_layer(0.11, 0.7, P, 0.4 * 0.7, 0.6 * P, cplx{1.8, 0.05}, 1.0));
        L.push_back(circle_layer(0.09, 0.7, P, 0.25 * 0.7, 6, 2.3, 1.2));
        L.push_back(rcwa::Layer2D::uniform(0.0, 1.7));
        L.push_back(rcwa::Layer2D::uniform(0.05, cplx{1.6, 0.01}));
        L.push_back(rect_layer(0.13, 0.7, P, 0.6 * 0.7, 0.3 * P, 1.6, 1.0));
        out.push_back(c);
    }
    {
        // larger truncation: N = 169, 2N = 338
        Case c = base("pillars_films_m6");
        pillars(c);
        c.M1 = c.M2 = 6;
        c.theta = 8.0;
        c.phi = 15.0;
        c.wavelength = 0.9;
        out.push_back(c);
    }
    {
        // only films: the 2x2 block-diagonal path end to end
        Case c = base("films_only");
        c.M1 = 2;
        c.M2 = 1;
        c.theta = 40.0;
        c.phi = 20.0;
        c.jones = {cplx{0.8, 0.0}, cplx{0.6, 0.0}};
        c.stack.layers = {rcwa::Layer2D::uniform(0.2, 1.9), rcwa::Layer2D::uniform(0.1, cplx{1.3, 0.02}),
                          rcwa::Layer2D::uniform(0.3, 2.4)};
        out.push_back(c);
    }
    return out;
}

void export_generated(std::FILE* f, const Case& c) {
    const rcwa::Result2D r = run(c);
    put_head(f, c);
    std::fprintf(f, "\"operators\":[],");
    put_rayleigh(f, c.stack, r);
    std::fputc(',', f);
    put_result(f, r, true);
    std::fprintf(f, "}\n");
}

// ---- cases described in a text file (the seeded benchmark structures, written by make_golden.py):
//   case <name> <wavelength> <theta> <phi> <M1> <M2> <Es re> <Es im> <Ep re> <Ep im> <laurent>
//   stack <nI> <nII re> <nII im> <Lx> <Ly>
//   uniform <d> <n re> <n im>
//   patterned <d> <K> <y_0> ... <y_K>        followed by K lines
//   profile <S> <x_0> ... <x_S> <n_0 re> <n_0 im> ... <n_{S-1} re> <n_{S-1} im>
//   end
std::vector<Case> read_cases(const char* path) {
    std::vector<Case> out;
    std::ifstream in(path);
    std::string word;
    auto num = [&] { std::string t; in >> t; return std::strtod(t.c_str(), nullptr); };
    while (in >> word) {
        if (word != "case") throw std::runtime_error("case expected");
        Case c;
        c.source = "benchmark";
        in >> c.name;
        c.wavelength = num(); c.theta = num(); c.phi = num();
        in >> c.M1 >> c.M2;
        const double a = num(), b = num(), d = num(), e = num();
        c.jones = {cplx{a, b}, cplx{d, e}};
        int laurent = 0;
        in >> laurent;
        c.laurent = laurent != 0;
        in >> word;
        c.stack.nI = num();
        const double r = num(), i = num();
        c.stack.nII = cplx{r, i};
        c.stack.Lx = num(); c.stack.Ly = num();
        while (in >> word && word != "end") {
            if (word == "uniform") {
                const double th = num(), nr = num(), ni = num();
                c.stack.layers.push_back(rcwa::Layer2D::uniform(th, cplx{nr, ni}));
            } else {
                const double th = num();
                int K = 0;
                in >> K;
                std::vector<double> ye(K + 1);
                for (double& y : ye) y = num();
                std::vector<rcwa::XProfile2D> rows;
                for (int k = 0; k < K; ++k) {
                    in >> word;
                    int S = 0;
                    in >> S;
                    std::vector<double> xe(S + 1);
                    for (double& x : xe) x = num();
                    std::vector<cplx> nv(S);
                    for (cplx& v : nv) { const double vr = num(), vi = num(); v = cplx{vr, vi}; }
                    rows.push_back(rcwa::XProfile2D{xe, nv});
                }
                c.stack.layers.push_back(rcwa::Layer2D::patterned(th, ye, rows));
            }
        }
        out.push_back(c);
    }
    return out;
}

// every case solved by the reference on its own thread (solve2d is reentrant), written in input order
void export_listed(std::FILE* f, const std::vector<Case>& cases) {
    std::vector<rcwa::Result2D> res(cases.size());
    std::vector<std::thread> th;
    for (std::size_t k = 0; k < cases.size(); ++k) th.emplace_back([&, k] { res[k] = run(cases[k]); });
    for (std::thread& t : th) t.join();
    for (std::size_t k = 0; k < cases.size(); ++k) {
        put_head(f, cases[k]);
        std::fprintf(f, "\"operators\":[],");
        put_rayleigh(f, cases[k].stack, res[k]);
        std::fputc(',', f);
        put_result(f, res[k], false);
        std::fprintf(f, "}\n");
    }
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    if (argc > 3 && std::string(argv[2]) == "--cases") {
        export_listed(f, read_cases(argv[3]));
    } else {
        for (int i = 0; i < kRcwa2dRefCaseCount; ++i) export_reference_case(f, kRcwa2dRefCases[i]);
        for (int i = 0; i < kCoreRefCaseCount; ++i) export_core_case(f, kCoreRefCases[i]);
        for (const Case& c : generated_cases()) export_generated(f, c);
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
