// Golden-fixture exporter for the 1-D TE/TM solve.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_rcwa1d.cpp in place, with its main() renamed, so that the
// test structures (grating_stack, mdg_stack, random_stack_N, ...) and the golden efficiency tables
// (kGratingTE, kRandom3Der, ...) are taken from the reference itself rather than retyped. For every
// case it writes the structure, the incidence, the table from the reference's tests, and the result
// of the reference's own rcwa::solve (17 significant digits) as one JSON object per line.
#define main stablercwa_reference_test_main
#include "test_rcwa1d.cpp"
#undef main

#include <cstdio>
#include <string>

namespace {

void put_c(std::FILE* f, cplx z) { std::fprintf(f, "[%.17g,%.17g]", z.real(), z.imag()); }

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

void put_result(std::FILE* f, const rcwa::Result& r) {
    const auto cvec = [&](const char* key, const Vector& v) {
        std::fprintf(f, "\"%s\":[", key);
        for (std::size_t j = 0; j < v.size(); ++j) {
            if (j) std::fprintf(f, ",");
            if (std::isnan(v[j].real())) std::fprintf(f, "[\"nan\",\"nan\"]");
            else put_c(f, v[j]);
        }
        std::fprintf(f, "],");
    };
    const auto rvec = [&](const char* key, const RealVector& v) {
        std::fprintf(f, "\"%s\":[", key);
        for (std::size_t j = 0; j < v.size(); ++j) {
            if (std::isnan(v[j])) std::fprintf(f, "%s\"nan\"", j ? "," : "");
            else std::fprintf(f, "%s%.17g", j ? "," : "", v[j]);
        }
        std::fprintf(f, "],");
    };
    std::fprintf(f, "{");
    cvec("R", r.R);
    cvec("T", r.T);
    rvec("DEr", r.DEr);
    rvec("DEt", r.DEt);
    std::fprintf(f, "\"eig_info\":%d,\"n_eig\":%d,\"n_dense_solve\":%d}", r.eig_info, r.n_eig, r.n_dense_solve);
}

void put_case(std::FILE* f, const std::string& name, const char* source, const rcwa::Stack& s, double wl, double th,
              int M, Polarization pol, const std::vector<double>* der, const std::vector<double>* det) {
    const rcwa::Result r = rcwa::solve(s, wl, th, M, pol);
    std::fprintf(f, "{\"name\":\"%s\",\"source\":\"%s\",\"stack\":", name.c_str(), source);
    put_stack(f, s);
    std::fprintf(f, ",\"wavelength\":%.17g,\"theta\":%.17g,\"M\":%d,\"pol\":\"%s\",", wl, th, M,
                 pol == Polarization::TE ? "TE" : "TM");
    if (der && det) {
        std::fprintf(f, "\"table\":{\"der\":[");
        for (std::size_t j = 0; j < der->size(); ++j) std::fprintf(f, "%s%.17g", j ? "," : "", (*der)[j]);
        std::fprintf(f, "],\"det\":[");
        for (std::size_t j = 0; j < det->size(); ++j) std::fprintf(f, "%s%.17g", j ? "," : "", (*det)[j]);
        std::fprintf(f, "]},");
    }
    std::fprintf(f, "\"ref\":");
    put_result(f, r);
    std::fprintf(f, "}\n");
}

template <std::size_t N>
void table_case(std::FILE* f, const char* name, const char* source, const rcwa::Stack& s, double wl, double th, int M,
                Polarization pol, const OrderRef (&table)[N]) {
    std::vector<double> der(2 * M + 1, 0.0), det(2 * M + 1, 0.0);
    for (const OrderRef& row : table) {
        der[row.order + M] = row.der;
        det[row.order + M] = row.det;
    }
    put_case(f, name, source, s, wl, th, M, pol, &der, &det);
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    const auto TE = Polarization::TE, TM = Polarization::TM;
    // Per-order tables of test_reference_tables (tests/test_rcwa1d.cpp:606-636).
    table_case(f, "grating_TE", "tests/test_rcwa1d.cpp:619", grating_stack(), 1.053, 66.36, 12, TE, kGratingTE);
    table_case(f, "grating_TM", "tests/test_rcwa1d.cpp:620", grating_stack(), 1.053, 66.36, 12, TM, kGratingTM);
    table_case(f, "lossy_TE", "tests/test_rcwa1d.cpp:621", grating_stack(true), 1.053, 42.0, 14, TE, kLossyTE);
    table_case(f, "lossy_TM", "tests/test_rcwa1d.cpp:622", grating_stack(true), 1.053, 42.0, 14, TM, kLossyTM);
    table_case(f, "mdg_TE", "tests/test_rcwa1d.cpp:623", mdg_stack(), 1.053, 66.36, 20, TE, kMdgTE);
    table_case(f, "mdg_TM", "tests/test_rcwa1d.cpp:624", mdg_stack(), 1.053, 66.36, 20, TM, kMdgTM);
    table_case(f, "multilayer_TE", "tests/test_rcwa1d.cpp:625", multilayer_stack(), 0.83, 27.0, 12, TE, kMultilayerTE);
    table_case(f, "multilayer_TM", "tests/test_rcwa1d.cpp:626", multilayer_stack(), 0.83, 27.0, 12, TM, kMultilayerTM);
    table_case(f, "ridges_silver_TE", "tests/test_rcwa1d.cpp:627", ridges_on_silver(), 0.8, 23.0, 50, TE, kRidgesSilver50TE);
    table_case(f, "ridges_silver_TM", "tests/test_rcwa1d.cpp:628", ridges_on_silver(), 0.8, 23.0, 50, TM, kRidgesSilver50TM);
    table_case(f, "silver_glass_TE", "tests/test_rcwa1d.cpp:630", silver_on_glass(), 0.8, 30.0, 15, TE, kSilverGlassTE);
    table_case(f, "silver_glass_TM", "tests/test_rcwa1d.cpp:631", silver_on_glass(), 0.8, 30.0, 15, TM, kSilverGlassTM);
    table_case(f, "silver_bulk_TE", "tests/test_rcwa1d.cpp:632", silver_on_silver(), 0.8, 30.0, 15, TE, kSilverBulkTE);
    table_case(f, "silver_bulk_TM", "tests/test_rcwa1d.cpp:633", silver_on_silver(), 0.8, 30.0, 15, TM, kSilverBulkTM);
    // Random stacks of test_random_stacks (tests/test_rcwa1d.cpp:1572-1626).
    for (const RandomCase& c : kRandomCases) {
        const std::vector<double> der(c.der, c.der + 2 * c.M + 1), det(c.det, c.det + 2 * c.M + 1);
        put_case(f, "random_" + std::to_string(c.id), "tests/test_rcwa1d.cpp:1572", c.stack(), c.wavelength, c.theta,
                 c.M, c.pol, &der, &det);
    }
    // Structures without a table: the reference's own solve is the golden value.
    for (Polarization pol : {TE, TM}) {
        const char* p = pol == TE ? "TE" : "TM";
        put_case(f, std::string("ridges_mirror_M30_") + p, "tests/test_rcwa1d.cpp:414", ridges_on_mirror(),
                 kRidgesWavelength, kRidgesTheta, 30, pol, nullptr, nullptr);
        put_case(f, std::string("trapezoid4_") + p, "tests/test_rcwa1d.cpp:373", trapezoid_stack(4), 1.053, 66.36, 15,
                 pol, nullptr, nullptr);
    }
    // Exact Rayleigh anomalies: exact q == 0 in a finite film (tests/test_rcwa1d.cpp:1834-1866).
    {
        const rcwa::Layer grating = rcwa::Layer::grating(0.3, {0.0, 0.3, 1.0}, {1.5, 1.0});
        const auto make = [](std::vector<rcwa::Layer> layers, cplx nII) {
            rcwa::Stack s;
            s.nI = 1.0;
            s.nII = nII;
            s.period = 1.0;
            s.layers = std::move(layers);
            return s;
        };
        const rcwa::Stack cases[] = {
            make({rcwa::Layer::uniform(0.2, 2.0), grating}, 1.5),
            make({grating, rcwa::Layer::uniform(0.2, 2.0)}, 1.5),
            make({grating, rcwa::Layer::uniform(0.1, 1.7), rcwa::Layer::uniform(0.2, 2.0), rcwa::Layer::uniform(0.1, 1.7)}, 1.5),
            make({rcwa::Layer::uniform(0.0, 2.0), grating}, 1.5),
        };
        const char* names[] = {"film_on_grating", "film_below", "film_buried", "film_zero_thickness"};
        for (int k = 0; k < 4; ++k)
            for (Polarization pol : {TE, TM})
                put_case(f, std::string("rayleigh_") + names[k] + (pol == TE ? "_TE" : "_TM"),
                         "tests/test_rcwa1d.cpp:1847", cases[k], 1.0, 0.0, 6, pol, nullptr, nullptr);
        // Closed-form cutoff film (tests/test_rcwa1d.cpp:1868-1895): R = 1/2 (TE), 1/17 (TM).
        const double kx = 2.0 * std::sin(30.0 * kPi / 180.0);
        rcwa::Stack cutoff;
        cutoff.nI = cutoff.nII = 2.0;
        cutoff.period = 1.0;
        cutoff.layers = {rcwa::Layer::uniform(1.0 / (kPi * std::sqrt(4.0 - kx * kx)), kx)};
        put_case(f, "cutoff_TE", "tests/test_rcwa1d.cpp:1869", cutoff, 1.0, 30.0, 0, TE, nullptr, nullptr);
        put_case(f, "cutoff_TM", "tests/test_rcwa1d.cpp:1869", cutoff, 1.0, 30.0, 0, TM, nullptr, nullptr);
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
