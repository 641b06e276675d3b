// Golden-fixture exporter for the conical-incidence solve.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_rcwa1d_conical.cpp in place (main() renamed), so the ten
// reference Jones tables of tests/conical_reference.inc and their structures (conical_ref_stack),
// and the degenerate-layer (Schur branch) cases of test_degenerate_modes, come from the reference
// itself. For every case it writes the structure, incidence, table (when the reference holds one)
// and the reference's own rcwa::solve_conical result, one JSON object per line.
#define main stablercwa_reference_conical_test_main
#include "test_rcwa1d_conical.cpp"
#undef main

#include <cstdio>
#include <string>

namespace {

void put_c(std::FILE* f, cplx z) {
    if (std::isnan(z.real()) || std::isnan(z.imag())) std::fprintf(f, "[\"nan\",\"nan\"]");
    else std::fprintf(f, "[%.17g,%.17g]", z.real(), z.imag());
}
void put_d(std::FILE* f, double v) {
    if (std::isnan(v)) std::fprintf(f, "\"nan\"");
    else if (std::isinf(v)) std::fprintf(f, "\"inf\"");
    else std::fprintf(f, "%.17g", v);
}

void put_stack(std::FILE* f, const rcwa::Stack& s) {
    std::fprintf(f, "{\"nI\":");
    put_c(f, s.nI);
    std::fprintf(f, ",\"nII\":");
    put_c(f, s.nII);
    std::fprintf(f, ",\"period\":%.17g,\"layers\":[", s.period);
    for (std::size_t k = 0; k < s.layers.size(); ++k) {
        const rcwa::Layer& L = s.layers[k];
        std::fprintf(f, "%s{\"d\":%.17g,", k ? "," : "", L.d);
        if (L.homogeneous) {
            std::fprintf(f, "\"n\":");
            put_c(f, L.n);
        } else {
            std::fprintf(f, "\"edges\":[");
            for (std::size_t j = 0; j < L.edges.size(); ++j) std::fprintf(f, "%s%.17g", j ? "," : "", L.edges[j]);
            std::fprintf(f, "],\"n_values\":[");
            for (std::size_t j = 0; j < L.n_values.size(); ++j) {
                if (j) std::fprintf(f, ",");
                put_c(f, L.n_values[j]);
            }
            std::fprintf(f, "]");
        }
        std::fprintf(f, "}");
    }
    std::fprintf(f, "]}");
}

void put_case(std::FILE* f, const std::string& name, const char* source, const rcwa::Stack& s, double wl, double th,
              double ph, int M, const ConicalRefCase* table) {
    const rcwa::ConicalResult r = rcwa::solve_conical(s, wl, th, ph, M);
    std::fprintf(f, "{\"name\":\"%s\",\"source\":\"%s\",\"stack\":", name.c_str(), source);
    put_stack(f, s);
    std::fprintf(f, ",\"wavelength\":%.17g,\"theta\":%.17g,\"phi\":%.17g,\"M\":%d,", wl, th, ph, M);
    if (table) {
        std::fprintf(f, "\"table\":{\"jr\":[");
        for (int i = 0; i < table->count; ++i) {
            std::fprintf(f, "%s[", i ? "," : "");
            for (int k = 0; k < 8; ++k) std::fprintf(f, "%s%.17g", k ? "," : "", table->orders[i].jr[k]);
            std::fprintf(f, "]");
        }
        std::fprintf(f, "],\"jt\":[");
        for (int i = 0; i < table->count; ++i) {
            std::fprintf(f, "%s[", i ? "," : "");
            for (int k = 0; k < 8; ++k) std::fprintf(f, "%s%.17g", k ? "," : "", table->orders[i].jt[k]);
            std::fprintf(f, "]");
        }
        std::fprintf(f, "]},");
    }
    std::fprintf(f, "\"ref\":{\"Jr\":[");
    for (std::size_t j = 0; j < r.Jr.size(); ++j) {
        std::fprintf(f, "%s[", j ? "," : "");
        put_c(f, r.Jr[j].ss); std::fprintf(f, ","); put_c(f, r.Jr[j].sp); std::fprintf(f, ",");
        put_c(f, r.Jr[j].ps); std::fprintf(f, ","); put_c(f, r.Jr[j].pp);
        std::fprintf(f, "]");
    }
    std::fprintf(f, "],\"Jt\":[");
    for (std::size_t j = 0; j < r.Jt.size(); ++j) {
        std::fprintf(f, "%s[", j ? "," : "");
        put_c(f, r.Jt[j].ss); std::fprintf(f, ","); put_c(f, r.Jt[j].sp); std::fprintf(f, ",");
        put_c(f, r.Jt[j].ps); std::fprintf(f, ","); put_c(f, r.Jt[j].pp);
        std::fprintf(f, "]");
    }
    std::fprintf(f, "],\"DEr\":[");
    for (std::size_t j = 0; j < r.DEr.size(); ++j) {
        std::fprintf(f, "%s[", j ? "," : "");
        put_d(f, r.DEr[j].ss); std::fprintf(f, ","); put_d(f, r.DEr[j].sp); std::fprintf(f, ",");
        put_d(f, r.DEr[j].ps); std::fprintf(f, ","); put_d(f, r.DEr[j].pp);
        std::fprintf(f, "]");
    }
    std::fprintf(f, "],\"DEt\":[");
    for (std::size_t j = 0; j < r.DEt.size(); ++j) {
        std::fprintf(f, "%s[", j ? "," : "");
        put_d(f, r.DEt[j].ss); std::fprintf(f, ","); put_d(f, r.DEt[j].sp); std::fprintf(f, ",");
        put_d(f, r.DEt[j].ps); std::fprintf(f, ","); put_d(f, r.DEt[j].pp);
        std::fprintf(f, "]");
    }
    std::fprintf(f, "],\"kx\":[");
    for (std::size_t j = 0; j < r.kx.size(); ++j) std::fprintf(f, "%s%.17g", j ? "," : "", r.kx[j]);
    std::fprintf(f, "],\"flux_r\":[");
    for (std::size_t j = 0; j < r.flux_r.size(); ++j) std::fprintf(f, "%s%.17g", j ? "," : "", r.flux_r[j]);
    std::fprintf(f, "],\"flux_t\":[");
    for (std::size_t j = 0; j < r.flux_t.size(); ++j) std::fprintf(f, "%s%.17g", j ? "," : "", r.flux_t[j]);
    std::fprintf(f, "],\"ky\":%.17g,\"eig_info\":%d,\"n_eig\":%d,\"n_dense_solve\":%d,\"n_schur\":%d,\"min_abs_lambda\":",
                 r.ky, r.eig_info, r.n_eig, r.n_dense_solve, r.n_schur);
    put_d(f, r.min_abs_lambda);
    std::fprintf(f, ",\"degenerate_mode_warning\":%s}}\n", r.degenerate_mode_warning ? "true" : "false");
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    // the ten reference Jones tables (tests/test_rcwa1d_conical.cpp:231-276, tests/conical_reference.inc)
    for (const ConicalRefCase& c : kConicalRefCases)
        put_case(f, std::string("ref_") + std::to_string(c.id), "tests/test_rcwa1d_conical.cpp:235", conical_ref_stack(c.id),
                 c.wavelength, c.theta_deg, c.phi_deg, c.M, &c);
    // degenerate layer: an eigenvalue of A crosses zero with ky != 0 -> Schur propagation
    // (tests/test_rcwa1d_conical.cpp:1360-1400)
    {
        const rcwa::Stack s = conical_ref_stack(1);
        const double theta = 40.0, phi = 25.0;
        const int M = 8;
        const auto count = [&](double wavelength) { return negative_eigenvalues(s, wavelength, theta, phi, M); };
        const double t0 = bisect_step(count, 0.9, 1.05);
        put_case(f, "schur_at_crossing", "tests/test_rcwa1d_conical.cpp:1374", s, t0, theta, phi, M, nullptr);
        put_case(f, "schur_above", "tests/test_rcwa1d_conical.cpp:1404", s, t0 * (1.0 + 1e-6), theta, phi, M, nullptr);
        put_case(f, "schur_below", "tests/test_rcwa1d_conical.cpp:1404", s, t0 * (1.0 - 1e-6), theta, phi, M, nullptr);
        put_case(f, "schur_window_outside", "tests/test_rcwa1d_conical.cpp:1413", s, t0 * (1.0 + 1e-3), theta, phi, M, nullptr);
        rcwa::Stack mixed = s;
        mixed.layers.push_back(rcwa::Layer::uniform(.2, 1.7));
        mixed.layers.push_back(rcwa::Layer::grating(.1, {0., .15, mixed.period}, {1.8, 1.1}));
        put_case(f, "schur_mixed_stack", "tests/test_rcwa1d_conical.cpp:1385", mixed, t0, theta, phi, M, nullptr);
        rcwa::Stack thick = s;
        thick.layers[0].d = 20.;
        put_case(f, "schur_thick_layer", "tests/test_rcwa1d_conical.cpp:1397", thick, t0, theta, phi, M, nullptr);
    }
    // structures of the test file without a table: trapezoid and four-ridge stacks, a film stack
    put_case(f, "trapezoid3_conical", "tests/test_rcwa1d_conical.cpp:86", trapezoid_stack(3), 1.053, 50.0, 30.0, 10, nullptr);
    put_case(f, "ridges_conical", "tests/test_rcwa1d_conical.cpp:104", ridges_stack(), 0.94, 22.0, 35.0, 20, nullptr);
    {
        rcwa::Stack films;
        films.nI = 1.0;
        films.nII = 1.5;
        films.period = 0.7;
        films.layers = {rcwa::Layer::uniform(0.3, cplx(1.9, 0.02)), rcwa::Layer::uniform(0.0, 2.5),
                        rcwa::Layer::uniform(0.2, 1.4)};
        put_case(f, "pure_films_conical", "tests/test_rcwa1d_conical.cpp:1708", films, 0.8, 35.0, 40.0, 5, nullptr);
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
