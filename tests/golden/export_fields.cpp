// Golden-fixture exporter for the planar near fields.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It calls the
// reference's own rcwa::solve_with_fields and rcwa::field_at (include/stablercwa/rcwa1d_fields.hpp) on
// the structures of tests/test_rcwa_public_fields.cpp (mixed and Schur stacks, compiled in place with
// main() renamed) and on a few more (the README configuration, a film stack, an absorbing multi-grating
// stack), at depths in the incident medium, inside every layer, on interfaces and in the exit medium.
// One JSON object per line: structure, point, depths, and the six harmonic field components.
#define main stablercwa_reference_public_fields_test_main
#include "test_rcwa_public_fields.cpp"
#undef main

#include <cstdio>
#include <cstdlib>
#include <string>

namespace {

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

void put_stack(std::FILE* f, const rc::Stack& s) {
    std::fprintf(f, "\"stack\":{\"nI\":");
    put_c(f, s.nI);
    std::fprintf(f, ",\"nII\":");
    put_c(f, s.nII);
    std::fprintf(f, ",\"period\":");
    put_d(f, s.period);
    std::fprintf(f, ",\"layers\":[");
    for (std::size_t k = 0; k < s.layers.size(); ++k) {
        const rc::Layer& L = s.layers[k];
        std::fprintf(f, "%s{\"d\":", k ? "," : "");
        put_d(f, L.d);
        if (L.homogeneous) {
            std::fprintf(f, ",\"n\":");
            put_c(f, L.n);
        } else {
            std::fprintf(f, ",\"edges\":[");
            for (std::size_t j = 0; j < L.edges.size(); ++j) {
                if (j) std::fputc(',', f);
                put_d(f, L.edges[j]);
            }
            std::fprintf(f, "],\"n_values\":[");
            for (std::size_t j = 0; j < L.n_values.size(); ++j) {
                if (j) std::fputc(',', f);
                put_c(f, L.n_values[j]);
            }
            std::fprintf(f, "]");
        }
        std::fprintf(f, "}");
    }
    std::fprintf(f, "]}");
}

// depths: the incident medium, each layer's top, middle and bottom, the interface +-1e-9, the exit medium
RealVector depths_for(const rc::Stack& s) {
    RealVector zs = {-0.37, -1e-9, 0.0};
    double z = 0.0;
    for (const rc::Layer& L : s.layers) {
        zs.push_back(z + 0.31 * L.d);
        zs.push_back(z + 0.5 * L.d);
        z += L.d;
        zs.push_back(z);
        zs.push_back(z + 1e-9);
    }
    zs.push_back(z + 0.2);
    zs.push_back(z + 1.3);
    return zs;
}

void fields_case(std::FILE* f, const std::string& name, const rc::Stack& s, double wl, double th, int M, rc::Polarization pol,
                 const RealVector* depths = nullptr) {
    const RealVector zs = depths ? *depths : depths_for(s);
    const auto res = rc::solve_with_fields(s, wl, th, M, pol);
    std::fprintf(f, "{\"kind\":\"planar\",\"name\":\"%s\",", name.c_str());
    put_stack(f, s);
    std::fprintf(f, ",\"wavelength\":");
    put_d(f, wl);
    std::fprintf(f, ",\"theta\":");
    put_d(f, th);
    std::fprintf(f, ",\"M\":%d,\"pol\":\"%s\",\"available\":%d,\"zs\":[", M, pol == rc::Polarization::TE ? "TE" : "TM",
                 res.fields.available() ? 1 : 0);
    for (std::size_t k = 0; k < zs.size(); ++k) {
        if (k) std::fputc(',', f);
        put_d(f, zs[k]);
    }
    std::fprintf(f, "],\"kxm\":[");
    for (std::size_t k = 0; k < res.fields.metadata().kxm.size(); ++k) {
        if (k) std::fputc(',', f);
        put_d(f, res.fields.metadata().kxm[k].real());
    }
    std::fprintf(f, "],\"DEr\":[");
    for (std::size_t k = 0; k < res.result.DEr.size(); ++k) {
        if (k) std::fputc(',', f);
        put_d(f, res.result.DEr[k]);
    }
    std::fprintf(f, "]");
    if (res.fields.available()) {
        const rc::HarmonicFields h = rc::field_at(res, zs);
        std::fprintf(f, ",\"fields\":[");
        for (int c = 0; c < 6; ++c) {
            std::fprintf(f, "%s[", c ? "," : "");
            const Matrix& m = h.components[c];
            for (int j = 0; j < m.rows(); ++j) {
                std::fprintf(f, "%s[", j ? "," : "");
                for (int iz = 0; iz < m.cols(); ++iz) {
                    if (iz) std::fputc(',', f);
                    put_c(f, m(j, iz));
                }
                std::fputc(']', f);
            }
            std::fputc(']', f);
        }
        std::fputc(']', f);
    }
    std::fprintf(f, "}\n");
}

void put_harmonics(std::FILE* f, const rc::HarmonicFields& h) {
    std::fprintf(f, ",\"fields\":[");
    for (int c = 0; c < 6; ++c) {
        std::fprintf(f, "%s[", c ? "," : "");
        const Matrix& m = h.components[c];
        for (int j = 0; j < m.rows(); ++j) {
            std::fprintf(f, "%s[", j ? "," : "");
            for (int iz = 0; iz < m.cols(); ++iz) {
                if (iz) std::fputc(',', f);
                put_c(f, m(j, iz));
            }
            std::fputc(']', f);
        }
        std::fputc(']', f);
    }
    std::fputc(']', f);
}

// rcwa::solve_conical_with_fields + field_at(result, zs, jones) (include/stablercwa/rcwa1d_conical_fields.hpp)
void conical_case(std::FILE* f, const std::string& name, const rc::Stack& s, double wl, double th, double ph, int M,
                  rc::JonesVector jones, const RealVector& zs) {
    const auto res = rc::solve_conical_with_fields(s, wl, th, ph, M);
    std::fprintf(f, "{\"kind\":\"conical\",\"name\":\"%s\",", name.c_str());
    put_stack(f, s);
    std::fprintf(f, ",\"wavelength\":");
    put_d(f, wl);
    std::fprintf(f, ",\"theta\":");
    put_d(f, th);
    std::fprintf(f, ",\"phi\":");
    put_d(f, ph);
    std::fprintf(f, ",\"M\":%d,\"jones\":[", M);
    put_c(f, jones[0]);
    std::fputc(',', f);
    put_c(f, jones[1]);
    std::fprintf(f, "],\"available\":%d,\"n_schur\":%d,\"zs\":[", res.fields.available() ? 1 : 0, res.result.n_schur);
    for (std::size_t k = 0; k < zs.size(); ++k) {
        if (k) std::fputc(',', f);
        put_d(f, zs[k]);
    }
    std::fprintf(f, "],\"kxm\":[");
    for (std::size_t k = 0; k < res.fields.metadata().kxm.size(); ++k) {
        if (k) std::fputc(',', f);
        put_d(f, res.fields.metadata().kxm[k].real());
    }
    std::fprintf(f, "],\"ky\":");
    put_d(f, res.fields.metadata().ky);
    std::fprintf(f, ",\"DEr_ss\":[");
    for (std::size_t k = 0; k < res.result.DEr.size(); ++k) {
        if (k) std::fputc(',', f);
        put_d(f, res.result.DEr[k].ss);
    }
    std::fprintf(f, "]");
    if (res.fields.available()) put_harmonics(f, rc::field_at(res, zs, jones));
    std::fprintf(f, "}\n");
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    for (auto pol : {rc::Polarization::TE, rc::Polarization::TM}) {
        const char* p = pol == rc::Polarization::TE ? "TE" : "TM";
        // tests/test_rcwa_public_fields.cpp:27-38
        fields_case(f, std::string("mixed_") + p, mixed_stack(), .83, 27., 3, pol);
        // the unsorted, repeated and far depths of test_sampling_order_interfaces_and_ownership (:57)
        const RealVector far{.083, -.12, .42, .2, .2 + 5e-13, .42 + 5e-13, .083, .245, 0., 100., -100.};
        fields_case(f, std::string("mixed_far_") + p, mixed_stack(), .83, 27., 3, pol, &far);
        fields_case(f, std::string("schur_") + p, schur_stack(), 1.053, 66.36, 6, pol);
        // the README configuration (README.md:87-94)
        rc::Stack readme;
        readme.nI = 1.0; readme.nII = 1.46; readme.period = 0.574;
        readme.layers = {rc::Layer::grating(0.38, {0., 0.172, 0.574}, {1.46, 1.0}), rc::Layer::uniform(0.115, 1.96)};
        fields_case(f, std::string("readme_M20_") + p, readme, 1.053, 66.36, 20, pol);
        // films only (every order but the incident one unexcited)
        rc::Stack films;
        films.nI = 1.0; films.nII = 1.5; films.period = 0.7;
        films.layers = {rc::Layer::uniform(0.3, cplx(1.9, 0.02)), rc::Layer::uniform(0.0, 2.5), rc::Layer::uniform(0.2, 1.4)};
        fields_case(f, std::string("films_") + p, films, 0.8, 35., 4, pol);
        // absorbing gratings around a film, oblique
        rc::Stack multi;
        multi.nI = 1.0; multi.nII = cplx(1.52, 0.0); multi.period = 0.9;
        multi.layers = {rc::Layer::grating(0.15, {-0.1, 0.2, 0.55, 0.8}, {cplx(2.2, 0.05), 1.0, 1.6}),
                        rc::Layer::uniform(0.07, cplx(1.45, 0.01)),
                        rc::Layer::grating(0.21, {0.0, 0.33, 0.9}, {1.3, cplx(2.0, 0.02)})};
        fields_case(f, std::string("multi_grating_") + p, multi, 0.95, -18., 12, pol);
    }
    // conical near fields: tests/test_rcwa_public_fields.cpp:96-104, :207-216, :229-247
    {
        const rc::JonesVector jones{{cplx(.3, .2), cplx(-.7, .5)}};
        const RealVector zs{.083, -.12, .42, .2, .2 + 5e-13, .42 + 5e-13, .083, .245, 0., 100., -100.,
                            -1e-9, .2 - 1e-9, .2 + 1e-9, .29 - 1e-9, .29 + 1e-9, .42 - 1e-9, .42 + 1e-9, .51};
        conical_case(f, "conical_mixed_jones", mixed_stack(), .83, 27., 31., 3, jones, zs);
        conical_case(f, "conical_mixed_s", mixed_stack(), .83, 27., 31., 3, {{1.0, 0.0}}, zs);
        conical_case(f, "conical_mixed_phi0_p", mixed_stack(), .83, 27., 0., 3, {{0.0, 1.0}}, zs);
        auto zero_added = mixed_stack();
        zero_added.layers.insert(zero_added.layers.begin(), rc::Layer::uniform(0., 4.));
        zero_added.layers.insert(zero_added.layers.begin() + 2, rc::Layer::uniform(0., 2.));
        conical_case(f, "conical_zero_layers", zero_added, .83, 27., 31., 3, jones, zs);
        RealVector through(33);
        for (std::size_t j = 0; j < through.size(); ++j) through[j] = .38 * static_cast<double>(j) / 32.;
        for (double z : {-.2, .0001, .19, .38 + 1e-9, .45, .495, .7}) through.push_back(z);
        conical_case(f, "conical_schur_M8", schur_stack(), .980484673140678, 40., 25., 8, jones, through);
        auto thick = mixed_stack();
        thick.layers[1] = rc::Layer::uniform(1000., cplx(1.8, .7));
        conical_case(f, "conical_thick_absorber", thick, .83, 27., 31., 3, jones,
                     {-1000., 0., .2, 100.2, 500.2, 1000.29, 1000.42, 2000.});
        rc::Stack films;
        films.nI = 1.0; films.nII = 1.5; films.period = 0.7;
        films.layers = {rc::Layer::uniform(0.3, cplx(1.9, 0.02)), rc::Layer::uniform(0.2, 1.4)};
        conical_case(f, "conical_films", films, 0.8, 35., 20., 4, {{cplx(0.5, 0.5), 1.0}}, depths_for(films));
        rc::Stack multi;
        multi.nI = 1.0; multi.nII = 1.52; multi.period = 0.9;
        multi.layers = {rc::Layer::grating(0.15, {-0.1, 0.2, 0.55, 0.8}, {cplx(2.2, 0.05), 1.0, 1.6}),
                        rc::Layer::uniform(0.07, cplx(1.45, 0.01)),
                        rc::Layer::grating(0.21, {0.0, 0.33, 0.9}, {1.3, cplx(2.0, 0.02)})};
        conical_case(f, "conical_multi_grating", multi, 0.95, -18., 63., 12, {{0.0, 1.0}}, depths_for(multi));
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
