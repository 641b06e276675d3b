// Golden-fixture exporter for real-space field slices and phase maps.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_rcwa2d_fields.cpp in place (main() renamed) for its frozen slice
// fixture (tests/rcwa2d_fields_fixture.inc: x-z and y-z slices, absolute and incident phases and masks of the
// Python authority) and writes, from the reference's own rcwa::field_at, field_slice, field_map and
// phase_data (include/stablercwa/rcwa_fields.hpp, rcwa_phase.hpp):
//   kind "slice2d": per frozen case and plane the harmonics at the frozen depths, the reference's slice, its
//                   absolute and incident phase maps per component, and the frozen Python arrays;
//   kind "phase":   phase_data of 1-D, conical and 2-D grids under every reference kind, unwrap axis and a
//                   large floor, with the input grid, so the phase step is compared on identical inputs.
// One JSON object per line.
#define main stablercwa_reference_rcwa2d_fields_test_main
#include "test_rcwa2d_fields.cpp"
#undef main

#include <cstdio>
#include <cstdlib>
#include <string>

namespace {

void px_d(std::FILE* f, double v) {
    if (std::isnan(v)) { std::fprintf(f, "\"nan\""); return; }
    if (std::isinf(v)) { std::fprintf(f, v > 0 ? "\"inf\"" : "\"-inf\""); return; }
    char buf[40];
    for (int prec = 15; prec <= 17; ++prec) {
        std::snprintf(buf, sizeof buf, "%.*g", prec, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::fputs(buf, f);
}
void px_c(std::FILE* f, cplx z) {
    std::fputc('[', f);
    px_d(f, z.real());
    std::fputc(',', f);
    px_d(f, z.imag());
    std::fputc(']', f);
}
void px_reals(std::FILE* f, const char* key, const double* p, std::size_t count) {
    std::fprintf(f, ",\"%s\":[", key);
    for (std::size_t i = 0; i < count; ++i) {
        if (i) std::fputc(',', f);
        px_d(f, p[i]);
    }
    std::fputc(']', f);
}
void px_cplx(std::FILE* f, const char* key, const cplx* p, std::size_t count) {
    std::fprintf(f, ",\"%s\":[", key);
    for (std::size_t i = 0; i < count; ++i) {
        if (i) std::fputc(',', f);
        px_c(f, p[i]);
    }
    std::fputc(']', f);
}
void px_mask(std::FILE* f, const char* key, const std::vector<bool>& m) {
    std::fprintf(f, ",\"%s\":\"", key);
    for (bool b : m) std::fputc(b ? '1' : '0', f);
    std::fputc('"', f);
}

// harmonics [c][j][iz] flattened
void px_harmonics(std::FILE* f, const rcwa::HarmonicFields& h) {
    std::vector<cplx> v;
    for (int c = 0; c < 6; ++c)
        for (int j = 0; j < h.components[c].rows(); ++j)
            for (int iz = 0; iz < h.components[c].cols(); ++iz) v.push_back(h.components[c](j, iz));
    px_cplx(f, "harmonics", v.data(), v.size());
}
// slice [c][iz][it] flattened (the Matrix [nt, nz] column-major data of each component)
template <class Grid>
void px_grid(std::FILE* f, const char* key, const Grid& g) {
    std::vector<cplx> v;
    for (int c = 0; c < 6; ++c) {
        const Matrix& m = g.components[c];
        v.insert(v.end(), m.data(), m.data() + static_cast<std::size_t>(m.rows()) * static_cast<std::size_t>(m.cols()));
    }
    px_cplx(f, key, v.data(), v.size());
}

void px_phase(std::FILE* f, const char* prefix, const rcwa::PhaseGrid& p) {
    const std::string k = prefix;
    px_reals(f, (k + "_phase").c_str(), p.phase.data(), p.phase.size());
    px_mask(f, (k + "_mask").c_str(), p.mask);
}

void slice_case(std::FILE* f, const Rcwa2dFieldsCase& fc) {
    Rcwa2dRefCase c{};
    rcwa::Stack2D stack;
    rcwa::Jones2D jones{cplx{1.0, 0.0}, cplx{0.0, 0.0}};
    double wavelength, theta, phi;
    int M1, M2;
    rcwa::Options2D options;
    const bool big = fc.id == 22;
    if (big) {  // case 9's geometry at M1 = M2 = 12 (test_frozen_slices, test_rcwa2d_fields.cpp:409-412)
        c = rcwa2d_ref_case(9);
        stack = rcwa2d_ref_stack(9);
        wavelength = c.wavelength; theta = c.theta_deg; phi = c.phi_deg; M1 = 12; M2 = 12;
    } else {
        c = rcwa2d_ref_case(fc.id);
        stack = rcwa2d_ref_stack(fc.id);
        jones = {cplx{c.jones[0], c.jones[1]}, cplx{c.jones[2], c.jones[3]}};
        wavelength = c.wavelength; theta = c.theta_deg; phi = c.phi_deg; M1 = c.M1; M2 = c.M2;
        options.factorization = c.laurent ? rcwa::Factorization2D::Laurent : rcwa::Factorization2D::Li;
    }
    const rcwa::FieldResult2D run = rcwa::solve2d_with_fields(stack, wavelength, theta, phi, M1, M2, jones, options);
    const RealVector zs(fc.z, fc.z + fc.nz);
    const rcwa::HarmonicFields h = rcwa::field_at(run, zs);
    const auto& meta = run.fields.metadata();
    for (int plane = 0; plane < 2; ++plane) {
        const Rcwa2dFieldsSlice& ref = plane == 0 ? fc.xz : fc.yz;
        const rcwa::SlicePlane sp = plane == 0 ? rcwa::SlicePlane::XZ : rcwa::SlicePlane::YZ;
        const rcwa::FieldGridSlice slice = rcwa::field_slice(h, sp, fc.nt, ref.fixed);
        std::fprintf(f, "{\"kind\":\"slice2d\",\"name\":\"%s_%s\",\"id\":%d,\"plane\":%d,\"nt\":%d,\"nz\":%d,\"N\":%d,\"at\":", fc.name,
                     plane == 0 ? "xz" : "yz", fc.id, plane, fc.nt, fc.nz, run.result.N);
        px_d(f, ref.fixed);
        std::fprintf(f, ",\"period\":");
        px_d(f, plane == 0 ? stack.Lx : stack.Ly);
        std::fprintf(f, ",\"near_atol\":");
        px_d(f, fc.near_atol);
        std::fprintf(f, ",\"near_rtol\":");
        px_d(f, fc.near_rtol);
        std::fprintf(f, ",\"wavelength\":");
        px_d(f, wavelength);
        std::fprintf(f, ",\"theta\":");
        px_d(f, theta);
        std::fprintf(f, ",\"phi\":");
        px_d(f, phi);
        std::fprintf(f, ",\"M1\":%d,\"M2\":%d,\"laurent\":%d,\"jones\":[", M1, M2, options.factorization == rcwa::Factorization2D::Laurent);
        px_c(f, jones[0]);
        std::fputc(',', f);
        px_c(f, jones[1]);
        std::fputc(']', f);
        px_reals(f, "zs", zs.data(), zs.size());
        std::vector<double> kx, ky, kz0(1);
        for (std::size_t j = 0; j < meta.kxm.size(); ++j) {
            kx.push_back(meta.kxm[j].real());
            ky.push_back(meta.kyn[j]);
        }
        px_reals(f, "kx", kx.data(), kx.size());
        px_reals(f, "ky", ky.data(), ky.size());
        const std::size_t i0 = static_cast<std::size_t>(run.result.i0);
        const double kin[3] = {meta.kxm[i0].real(), meta.kyn[i0], meta.kzI[i0].real()};
        px_reals(f, "incident_k", kin, 3);
        px_reals(f, "x", slice.x.data(), slice.x.size());
        px_reals(f, "y", slice.y.data(), slice.y.size());
        if (plane == 0) px_harmonics(f, h);  // the y-z line of the same case uses the x-z line's harmonics
        px_grid(f, "slice", slice);
        for (int comp = 0; comp < 6; ++comp) {
            rcwa::PhaseOptions absolute, incident;
            incident.reference = rcwa::PhaseReference::Incident;
            const auto component = static_cast<rcwa::FieldComponent>(comp);
            px_phase(f, ("abs" + std::to_string(comp)).c_str(), rcwa::phase_data(slice, component, absolute));
            px_phase(f, ("inc" + std::to_string(comp)).c_str(), rcwa::phase_data(slice, component, incident));
        }
        const std::size_t total = 6 * static_cast<std::size_t>(fc.nz) * fc.nt;
        std::vector<cplx> frozen(total);
        for (std::size_t k = 0; k < total; ++k) frozen[k] = cplx{ref.fields[2 * k], ref.fields[2 * k + 1]};
        px_cplx(f, "frozen_slice", frozen.data(), total);
        px_reals(f, "frozen_phase_absolute", ref.phase_absolute, total);
        px_reals(f, "frozen_phase_incident", ref.phase_incident, total);
        std::fprintf(f, ",\"frozen_mask\":\"%.*s\",\"frozen_comparison\":\"%.*s\"}\n", static_cast<int>(total), ref.phase_mask,
                     static_cast<int>(total), ref.comparison_mask);
    }
}

// phase_data of one grid under several options, with the grid itself (kind "phase")
template <class Grid>
void phase_case(std::FILE* f, const std::string& name, const Grid& grid, const std::vector<double>& x, const std::vector<double>& y,
                const double kin[3]) {
    const std::size_t nt = x.size(), nz = grid.z.size();
    std::fprintf(f, "{\"kind\":\"phase\",\"name\":\"%s\",\"nt\":%zu,\"nz\":%zu", name.c_str(), nt, nz);
    px_reals(f, "x", x.data(), nt);
    px_reals(f, "y", y.data(), nt);
    px_reals(f, "z", grid.z.data(), nz);
    px_reals(f, "incident_k", kin, 3);
    px_grid(f, "grid", grid);
    // custom reference: a horizontal row (broadcast over z), complex with a zero to force masks
    Matrix row(static_cast<int>(nt), 1);
    for (std::size_t it = 0; it < nt; ++it) row(static_cast<int>(it), 0) = it == 1 ? cplx{} : std::polar(1.5, 0.3 * static_cast<double>(it));
    std::vector<cplx> rowv(row.data(), row.data() + nt);
    px_cplx(f, "custom_row", rowv.data(), nt);
    struct Opt { const char* key; rcwa::PhaseReference ref; rcwa::PhaseUnwrap unwrap; double floor; };
    const Opt opts[] = {{"abs_none", rcwa::PhaseReference::Absolute, rcwa::PhaseUnwrap::None, 1e-6},
                        {"abs_both", rcwa::PhaseReference::Absolute, rcwa::PhaseUnwrap::Both, 1e-6},
                        {"inc_x", rcwa::PhaseReference::Incident, rcwa::PhaseUnwrap::X, 1e-6},
                        {"inc_z", rcwa::PhaseReference::Incident, rcwa::PhaseUnwrap::Z, 1e-6},
                        {"custom_both", rcwa::PhaseReference::Custom, rcwa::PhaseUnwrap::Both, 1e-6},
                        {"abs_floor", rcwa::PhaseReference::Absolute, rcwa::PhaseUnwrap::Both, 0.35}};
    for (int comp = 0; comp < 6; ++comp)
        for (const Opt& o : opts) {
            rcwa::PhaseOptions po;
            po.reference = o.ref;
            po.unwrap = o.unwrap;
            po.phase_floor = o.floor;
            if (o.ref == rcwa::PhaseReference::Custom) po.custom_reference = row;
            const rcwa::PhaseGrid p = rcwa::phase_data(grid, static_cast<rcwa::FieldComponent>(comp), po);
            px_phase(f, (std::string(o.key) + std::to_string(comp)).c_str(), p);
            px_reals(f, (std::string(o.key) + std::to_string(comp) + "_amplitude").c_str(), p.amplitude.data(), p.amplitude.size());
        }
    std::fprintf(f, "}\n");
}

rcwa::Stack planar_mixed() {  // mixed_stack() of tests/test_rcwa_public_fields.cpp:28-33
    rcwa::Stack s;
    s.nI = 1.2; s.nII = 1.4; s.period = .6;
    s.layers = {rcwa::Layer::grating(.2, {0., .21, .6}, {1.7, 1.}), rcwa::Layer::uniform(.09, cplx(1.46, .03)),
                rcwa::Layer::grating(.13, {0., .12, .6}, {1.1, cplx(1.9, .07)})};
    return s;
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    for (int i = 0; i < kRcwa2dFieldsCaseCount; ++i) slice_case(f, kRcwa2dFieldsCases[i]);
    RealVector zs;
    for (int k = 0; k <= 12; ++k) zs.push_back(-0.2 + 0.06 * k);
    {   // 1-D planar TM, x-z map with 41 points
        const auto res = rcwa::solve_with_fields(planar_mixed(), .83, 27., 6, rcwa::Polarization::TM);
        const rcwa::FieldGridXZ g = rcwa::field_map(res, zs, 21);
        const auto& m = res.fields.metadata();
        const double kin[3] = {m.kxm[6].real(), m.ky, m.kzI[6].real()};
        phase_case(f, "planar_tm_map", g, g.x, std::vector<double>(g.x.size(), g.y), kin);
    }
    {   // conical, x-z map at y = 0.11 with a Jones vector
        const auto res = rcwa::solve_conical_with_fields(planar_mixed(), .83, 27., 31., 5);
        const rcwa::FieldGridXZ g = rcwa::field_map(res, zs, 17, .11, {{cplx(.3, .2), cplx(-.7, .5)}});
        const auto& m = res.fields.metadata();
        const double kin[3] = {m.kxm[5].real(), m.ky, m.kzI[5].real()};
        phase_case(f, "conical_map", g, g.x, std::vector<double>(g.x.size(), g.y), kin);
    }
    {   // 2-D problem A, y-z slice at x = 0.21
        const Problem pa = problem_a();
        const rcwa::FieldResult2D run = solve(pa);
        RealVector z2;
        for (int k = 0; k <= 12; ++k) z2.push_back(-0.3 + 0.1 * k);
        const rcwa::FieldGridSlice g = rcwa::field_slice(run, z2, rcwa::SlicePlane::YZ, 19, 0.21);
        const auto& m = run.fields.metadata();
        const std::size_t i0 = static_cast<std::size_t>(run.result.i0);
        const double kin[3] = {m.kxm[i0].real(), m.kyn[i0], m.kzI[i0].real()};
        phase_case(f, "problem_a_yz", g, g.x, g.y, kin);
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
