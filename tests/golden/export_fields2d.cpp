// Golden-fixture exporter for the 2-D (crossed-grating) near fields.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_rcwa2d_fields.cpp in place (main() renamed), and writes, from
// the reference's rcwa::solve2d_with_fields + rcwa::field_at (include/stablercwa/rcwa2d_fields.hpp):
//   - every successful case of tests/rcwa2d_reference.inc at its frozen depths, with the frozen harmonics
//     of the Python authority and their tolerances beside the C++ reference's own values;
//   - the test's problems A, B, C (films, absorbers, 5 um thick layers) at depths on both sides of every
//     interface, inside every layer and in both outer regions;
//   - the depth list of its test_depth_semantics, the all-zero-thickness stack of test_edge_stacks, and a
//     zero-thickness layer between two layers.
// One JSON object per line.
#define main stablercwa_reference_rcwa2d_fields_test_main
#include "test_rcwa2d_fields.cpp"
#undef main

#include <cstdio>
#include <cstdlib>
#include <string>

namespace {

void fx_d(std::FILE* f, double v) {
    if (std::isnan(v)) { std::fprintf(f, "\"nan\""); return; }
    if (std::isinf(v)) { std::fprintf(f, v > 0 ? "\"inf\"" : "\"-inf\""); return; }
    char buf[40];
    for (int prec = 15; prec <= 17; ++prec) {
        std::snprintf(buf, sizeof buf, "%.*g", prec, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::fputs(buf, f);
}
void fx_c(std::FILE* f, cplx z) {
    std::fputc('[', f);
    fx_d(f, z.real());
    std::fputc(',', f);
    fx_d(f, z.imag());
    std::fputc(']', f);
}

void fx_stack(std::FILE* f, const rcwa::Stack2D& s) {
    std::fprintf(f, "\"stack\":{\"nI\":");
    fx_d(f, s.nI);
    std::fprintf(f, ",\"nII\":");
    fx_c(f, s.nII);
    std::fprintf(f, ",\"Lx\":");
    fx_d(f, s.Lx);
    std::fprintf(f, ",\"Ly\":");
    fx_d(f, s.Ly);
    std::fprintf(f, ",\"layers\":[");
    for (std::size_t k = 0; k < s.layers.size(); ++k) {
        const rcwa::Layer2D& L = s.layers[k];
        std::fprintf(f, "%s{\"d\":", k ? "," : "");
        fx_d(f, L.d);
        if (L.homogeneous) {
            std::fprintf(f, ",\"n\":");
            fx_c(f, L.n);
        } else {
            std::fprintf(f, ",\"y_edges\":[");
            for (std::size_t j = 0; j < L.y_edges.size(); ++j) {
                if (j) std::fputc(',', f);
                fx_d(f, L.y_edges[j]);
            }
            std::fprintf(f, "],\"x_profiles\":[");
            for (std::size_t p = 0; p < L.x_profiles.size(); ++p) {
                const rcwa::XProfile2D& xp = L.x_profiles[p];
                std::fprintf(f, "%s{\"edges\":[", p ? "," : "");
                for (std::size_t j = 0; j < xp.edges.size(); ++j) {
                    if (j) std::fputc(',', f);
                    fx_d(f, xp.edges[j]);
                }
                std::fprintf(f, "],\"n_values\":[");
                for (std::size_t j = 0; j < xp.n_values.size(); ++j) {
                    if (j) std::fputc(',', f);
                    fx_c(f, xp.n_values[j]);
                }
                std::fprintf(f, "]}");
            }
            std::fprintf(f, "]");
        }
        std::fprintf(f, "}");
    }
    std::fprintf(f, "]}");
}

// components[c][j][iz]
void fx_harmonics(std::FILE* f, const char* key, const rcwa::HarmonicFields& h) {
    std::fprintf(f, ",\"%s\":[", key);
    for (int c = 0; c < 6; ++c) {
        std::fprintf(f, "%s[", c ? "," : "");
        const Matrix& m = h.components[c];
        for (int j = 0; j < m.rows(); ++j) {
            std::fprintf(f, "%s[", j ? "," : "");
            for (int iz = 0; iz < m.cols(); ++iz) {
                if (iz) std::fputc(',', f);
                fx_c(f, m(j, iz));
            }
            std::fputc(']', f);
        }
        std::fputc(']', f);
    }
    std::fputc(']', f);
}

// One solve2d_with_fields + field_at; frozen (optional) holds the Python authority's harmonics [iz][j][c]
void fx_case(std::FILE* f, const std::string& name, const rcwa::Stack2D& s, double wl, double th, double ph, int M1, int M2,
             const rcwa::Jones2D& jones, bool laurent, const RealVector& zs, const Rcwa2dRefCase* frozen) {
    rcwa::Options2D options;
    options.factorization = laurent ? rcwa::Factorization2D::Laurent : rcwa::Factorization2D::Li;
    const rcwa::FieldResult2D run = rcwa::solve2d_with_fields(s, wl, th, ph, M1, M2, jones, options);
    std::fprintf(f, "{\"name\":\"%s\",", name.c_str());
    fx_stack(f, s);
    std::fprintf(f, ",\"wavelength\":");
    fx_d(f, wl);
    std::fprintf(f, ",\"theta\":");
    fx_d(f, th);
    std::fprintf(f, ",\"phi\":");
    fx_d(f, ph);
    std::fprintf(f, ",\"M1\":%d,\"M2\":%d,\"laurent\":%d,\"jones\":[", M1, M2, laurent ? 1 : 0);
    fx_c(f, jones[0]);
    std::fputc(',', f);
    fx_c(f, jones[1]);
    std::fprintf(f, "],\"status\":%d,\"available\":%d,\"zs\":[", static_cast<int>(run.result.status), run.fields.available() ? 1 : 0);
    for (std::size_t k = 0; k < zs.size(); ++k) {
        if (k) std::fputc(',', f);
        fx_d(f, zs[k]);
    }
    std::fprintf(f, "],\"DEr\":[");
    for (std::size_t k = 0; k < run.result.DEr.size(); ++k) {
        if (k) std::fputc(',', f);
        fx_d(f, run.result.DEr[k]);
    }
    std::fprintf(f, "]");
    if (run.fields.available()) fx_harmonics(f, "fields", rcwa::field_at(run, zs));
    if (frozen) {
        std::fprintf(f, ",\"near_atol\":");
        fx_d(f, frozen->near_atol);
        std::fprintf(f, ",\"near_rtol\":");
        fx_d(f, frozen->near_rtol);
        std::fprintf(f, ",\"frozen\":[");
        for (int c = 0; c < 6; ++c) {
            std::fprintf(f, "%s[", c ? "," : "");
            for (int j = 0; j < frozen->count; ++j) {
                std::fprintf(f, "%s[", j ? "," : "");
                for (int k = 0; k < frozen->depth_count; ++k) {
                    if (k) std::fputc(',', f);
                    const double* v = frozen->depths[k].columns[j].c[c];
                    fx_c(f, cplx{v[0], v[1]});
                }
                std::fputc(']', f);
            }
            std::fputc(']', f);
        }
        std::fputc(']', f);
    }
    std::fprintf(f, "}\n");
}

RealVector straddle(const rcwa::Stack2D& s) {
    RealVector zs{-0.4, -1e-9};
    double z = 0.0;
    for (const rcwa::Layer2D& L : s.layers) {
        zs.push_back(z + 1e-9);
        zs.push_back(z + 0.37 * L.d);
        z += L.d;
        zs.push_back(z - 1e-9);
        zs.push_back(z);
    }
    zs.push_back(z + 1e-9);
    zs.push_back(z + 0.45);
    return zs;
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    // the frozen Python harmonics of tests/rcwa2d_reference.inc (test_frozen_harmonics, test_rcwa2d_fields.cpp:292-324)
    for (int i = 0; i < kRcwa2dRefCaseCount; ++i) {
        const Rcwa2dRefCase& c = kRcwa2dRefCases[i];
        if (c.status != 0 || c.depth_count == 0) continue;
        RealVector zs;
        for (int k = 0; k < c.depth_count; ++k) zs.push_back(c.depths[k].z);
        const rcwa::Jones2D jones = {cplx{c.jones[0], c.jones[1]}, cplx{c.jones[2], c.jones[3]}};
        fx_case(f, std::string("ref_") + c.name, rcwa2d_ref_stack(c.id), c.wavelength, c.theta_deg, c.phi_deg, c.M1, c.M2, jones,
                c.laurent != 0, zs, &c);
    }
    // problems A, B, C (test_rcwa2d_fields.cpp:199-249)
    const Problem pa = problem_a(), pb = problem_b(), pc = problem_c();
    fx_case(f, "problem_a", pa.stack, pa.wavelength, pa.theta, pa.phi, pa.M1, pa.M2, pa.jones, false, straddle(pa.stack), nullptr);
    fx_case(f, "problem_b", pb.stack, pb.wavelength, pb.theta, pb.phi, pb.M1, pb.M2, pb.jones, false, straddle(pb.stack), nullptr);
    fx_case(f, "problem_c", pc.stack, pc.wavelength, pc.theta, pc.phi, pc.M1, pc.M2, pc.jones, false, straddle(pc.stack), nullptr);
    fx_case(f, "problem_b_laurent", pb.stack, pb.wavelength, pb.theta, pb.phi, pb.M1, pb.M2, pb.jones, true, straddle(pb.stack),
            nullptr);
    // the depth list of test_depth_semantics (:1558-1559) at M1 = M2 = 1
    fx_case(f, "problem_a_depths", pa.stack, pa.wavelength, pa.theta, pa.phi, 1, 1, pa.jones, false,
            {0.5, -0.2, 0.1, 0.1, 0.9, 0.35, -0.2, 0.0, 0.1, 0.3, 0.725, 0.2}, nullptr);
    // all layers of zero thickness (test_edge_stacks, :1694-1724)
    {
        rcwa::Stack2D s;
        s.nI = 1.0;
        s.nII = 1.9;
        s.Lx = s.Ly = 0.9;
        s.layers = {rcwa::Layer2D::uniform(0.0, 2.8), rcwa::Layer2D::uniform(0.0, 1.6)};
        fx_case(f, "all_zero_thickness", s, 1.053, 40.0, 20.0, 1, 1, {cplx{0.6, 0.0}, cplx{0.0, 0.8}}, false,
                {-1e-9, 0.0, 5e-13, 0.3}, nullptr);
    }
    // a zero-thickness layer first and between two layers of problem A
    {
        rcwa::Stack2D s = pa.stack;
        s.layers.insert(s.layers.begin(), rcwa::Layer2D::uniform(0.0, 2.2));
        s.layers.insert(s.layers.begin() + 2, rcwa::Layer2D::uniform(0.0, 1.3));
        fx_case(f, "problem_a_zero_layers", s, pa.wavelength, pa.theta, pa.phi, 2, 2, pa.jones, false,
                {-0.1, 0.0, 1e-13, 0.15, 0.3, 0.3 + 1e-13, 0.35, 0.415, 0.6, 0.725, 0.9}, nullptr);
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
