// Golden-fixture exporter for the FFT-sampled Fourier coefficients and the solves that use them.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_fft.cpp in place (main() renamed) and writes, from the
// reference's own functions: rcwa::fourier_coefficients_fft on the profiles of test_fft.cpp's
// coefficients() (and a few larger sample counts), the closed-form coefficients for comparison, and
// rcwa::solve / rcwa::solve_conical on the FFT stacks of its solvers() plus a larger grating. One JSON
// object per line.
#define main stablercwa_reference_fft_test_main
#include "test_fft.cpp"
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
void put_cvec(std::FILE* f, const char* key, const Vector& v) {
    std::fprintf(f, "\"%s\":[", key);
    for (std::size_t i = 0; i < v.size(); ++i) {
        if (i) std::fputc(',', f);
        put_c(f, v[i]);
    }
    std::fputc(']', f);
}
void put_rvec(std::FILE* f, const char* key, const std::vector<double>& v) {
    std::fprintf(f, "\"%s\":[", key);
    for (std::size_t i = 0; i < v.size(); ++i) {
        if (i) std::fputc(',', f);
        put_d(f, v[i]);
    }
    std::fputc(']', f);
}

void coeff_case(std::FILE* f, const std::string& name, const std::vector<double>& edges, const Vector& values,
                double period, int hmax, int samples) {
    const Vector c = rc::fourier_coefficients_fft(edges, values, period, hmax, samples);
    const Vector a = rc::detail::fourier_coefficients(edges, values, period, hmax);
    std::fprintf(f, "{\"kind\":\"coeff\",\"name\":\"%s\",", name.c_str());
    put_rvec(f, "edges", edges);
    std::fputc(',', f);
    put_cvec(f, "values", values);
    std::fprintf(f, ",\"period\":");
    put_d(f, period);
    std::fprintf(f, ",\"hmax\":%d,\"samples\":%d,", hmax, samples);
    put_cvec(f, "fft", c);
    std::fputc(',', f);
    put_cvec(f, "analytic", a);
    std::fprintf(f, "}\n");
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
            std::fputc(',', f);
            put_rvec(f, "edges", L.edges);
            std::fputc(',', f);
            put_cvec(f, "n_values", L.n_values);
            std::fprintf(f, ",\"fourier_method\":%d,\"fft_samples\":%d", L.fourier_method == rc::FourierMethod::FFT ? 1 : 0,
                         L.fft_samples);
        }
        std::fprintf(f, "}");
    }
    std::fprintf(f, "]}");
}

void solve_case(std::FILE* f, const std::string& name, const rc::Stack& s, double wl, double th, int M, rc::Polarization pol) {
    const rc::Result r = rc::solve(s, wl, th, M, pol);
    std::fprintf(f, "{\"kind\":\"solve\",\"name\":\"%s\",", name.c_str());
    put_stack(f, s);
    std::fprintf(f, ",\"wavelength\":");
    put_d(f, wl);
    std::fprintf(f, ",\"theta\":");
    put_d(f, th);
    std::fprintf(f, ",\"M\":%d,\"pol\":\"%s\",\"ref\":{", M, pol == rc::Polarization::TE ? "TE" : "TM");
    put_cvec(f, "R", r.R);
    std::fputc(',', f);
    put_cvec(f, "T", r.T);
    std::fputc(',', f);
    put_rvec(f, "DEr", r.DEr);
    std::fputc(',', f);
    put_rvec(f, "DEt", r.DEt);
    std::fprintf(f, ",\"eig_info\":%d,\"n_dense_solve\":%d}}\n", r.eig_info, r.n_dense_solve);
}

void conical_case(std::FILE* f, const std::string& name, const rc::Stack& s, double wl, double th, double ph, int M) {
    const rc::ConicalResult r = rc::solve_conical(s, wl, th, ph, M);
    std::fprintf(f, "{\"kind\":\"conical\",\"name\":\"%s\",", name.c_str());
    put_stack(f, s);
    std::fprintf(f, ",\"wavelength\":");
    put_d(f, wl);
    std::fprintf(f, ",\"theta\":");
    put_d(f, th);
    std::fprintf(f, ",\"phi\":");
    put_d(f, ph);
    std::fprintf(f, ",\"M\":%d,\"ref\":{\"Jr\":[", M);
    for (std::size_t j = 0; j < r.Jr.size(); ++j) {
        std::fprintf(f, "%s[", j ? "," : "");
        put_c(f, r.Jr[j].ss); std::fputc(',', f); put_c(f, r.Jr[j].sp); std::fputc(',', f);
        put_c(f, r.Jr[j].ps); std::fputc(',', f); put_c(f, r.Jr[j].pp);
        std::fputc(']', f);
    }
    std::fprintf(f, "],\"Jt\":[");
    for (std::size_t j = 0; j < r.Jt.size(); ++j) {
        std::fprintf(f, "%s[", j ? "," : "");
        put_c(f, r.Jt[j].ss); std::fputc(',', f); put_c(f, r.Jt[j].sp); std::fputc(',', f);
        put_c(f, r.Jt[j].ps); std::fputc(',', f); put_c(f, r.Jt[j].pp);
        std::fputc(']', f);
    }
    std::fprintf(f, "],\"eig_info\":%d}}\n", r.eig_info);
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    // coefficients() of tests/test_fft.cpp:36-47
    for (double origin : {0., -.3, .2, 1.2}) {
        const std::vector<double> edges{origin, origin + .3125, origin + .7, origin + 1.};
        const Vector values{{2.3, .4}, {1.1, -.2}, {3., .1}};
        for (int N : {9, 17, 60, 257, 8192})
            coeff_case(f, "origin" + std::to_string(origin) + "_N" + std::to_string(N), edges, values, 1., 4, N);
    }
    coeff_case(f, "boundary_at_midpoint", {0., .5 / 9, 1.}, {4., 1.}, 1., 4, 9);
    coeff_case(f, "constant_one_sample", {0., 1.}, {{2., .3}}, 1., 0, 1);
    for (int N : {64, 256, 1024}) coeff_case(f, "convergence_N" + std::to_string(N), {-.3, -.05, .7}, {{2., .3}, {1., -.1}}, 1., 4, N);
    // larger sample counts and truncations (the automatic count for M = 60 and the maximum)
    {
        const std::vector<double> edges{0.0, 0.1779940, 0.3050, 0.574};
        const Vector values{cplx(2.1, 0.0) * cplx(2.1, 0.0), {1.0, 0.0}, cplx(1.46, 0.01) * cplx(1.46, 0.01)};
        coeff_case(f, "grating_M60_auto", edges, values, 0.574, 120, rc::resolve_fft_samples(60));
        coeff_case(f, "grating_max_samples", edges, values, 0.574, 120, rc::kMaxFFTSamples);
        coeff_case(f, "grating_odd_samples", edges, values, 0.574, 40, 1000003);
    }
    // solvers() of tests/test_fft.cpp:84-146
    rc::Stack analytic;
    analytic.period = .9; analytic.nI = 1.2; analytic.nII = 1.5;
    analytic.layers = {rc::Layer::grating(.2, {-.1, .125, .8}, {cplx(2., .02), 1.2}), rc::Layer::uniform(.12, {1.7, .05})};
    auto sampled = analytic;
    sampled.layers[0].fourier_method = rc::FourierMethod::FFT;
    sampled.layers[0].fft_samples = 65536;
    solve_case(f, "sampled65536_TE", sampled, .83, 27., 3, rc::Polarization::TE);
    solve_case(f, "sampled65536_TM", sampled, .83, 27., 3, rc::Polarization::TM);
    conical_case(f, "sampled65536_conical", sampled, .83, 27., 41., 3);
    sampled.layers[0].fft_samples = 257;
    sampled.layers.push_back(rc::Layer::grating(.09, {0., .3, .9}, {1.7, 1.2}, rc::FourierMethod::FFT, 1009));
    solve_case(f, "two_fft_layers_TM_a", sampled, .83, 27., 3, rc::Polarization::TM);
    solve_case(f, "two_fft_layers_TM_b", sampled, .91, -15., 3, rc::Polarization::TM);
    {
        rc::Stack big;
        big.period = 0.574; big.nI = 1.0; big.nII = 1.46;
        big.layers = {rc::Layer::grating(0.38, {0.0, 0.172, 0.574}, {1.46, 1.0}, rc::FourierMethod::FFT, 0),
                      rc::Layer::uniform(0.115, 1.96),
                      rc::Layer::grating(0.2, {-0.05, 0.1, 0.3, 0.524}, {cplx(2.0, 0.01), 1.3, 1.8}, rc::FourierMethod::FFT, 4096)};
        solve_case(f, "grating_auto_M20_TE", big, 1.053, 66.36, 20, rc::Polarization::TE);
        solve_case(f, "grating_auto_M20_TM", big, 1.053, 66.36, 20, rc::Polarization::TM);
        conical_case(f, "grating_auto_M12_conical", big, 1.053, 40.0, 25.0, 12);
    }
    // derived epsilon overflow: a numerical failure (tests/test_fft.cpp:119-131)
    {
        auto overflow = analytic;
        overflow.layers[0].fourier_method = rc::FourierMethod::FFT;
        overflow.layers[0].fft_samples = 17;
        overflow.layers[0].n_values[0] = 1e200;
        solve_case(f, "overflow_TE", overflow, .83, 27., 3, rc::Polarization::TE);
        solve_case(f, "overflow_TM", overflow, .83, 27., 3, rc::Polarization::TM);
        overflow.layers[0].n_values[0] = 1e-200;
        solve_case(f, "underflow_TE", overflow, .83, 27., 3, rc::Polarization::TE);
        solve_case(f, "underflow_TM", overflow, .83, 27., 3, rc::Polarization::TM);
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
