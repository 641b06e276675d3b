// Golden-fixture exporter for the JSON request front end.
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). For every request
// below (valid requests of the three modes, and invalid ones covering each check of the reference's request
// reader) it writes the reference's own reply, rcwa::solve_json_reply (include/stablercwa/rcwa_json.hpp),
// as {"name", "indent", "request", "reply"}. The structures are those of tests/test_rcwa_json.cpp
// (example, lossy, pure films, silver, Rayleigh, trapezoid) and of the periodic2d example in the header.
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "stablercwa/rcwa_json.hpp"

namespace {

const char* kExample = R"("stack": {"nI": 1.0, "nII": 1.46, "period": 0.574, "layers": [{"d": 0.38, "edges": [0.0, 0.1722, 0.574], "n_values": [1.46, 1.0]}, {"d": 0.115, "n": [1.96, 0.0]}]})";
const char* kLossy = R"("stack": {"nI": 1.2, "nII": [1.5, 0.0], "period": 0.9, "layers": [{"d": 0.23, "edges": [0.0, 0.21, 0.47, 0.9], "n_values": [[1.7, 0.0], [1.0, 0.0], [2.1, 0.05]]}, {"d": 0.19, "n": [1.4, 0.02]}, {"d": 0.31, "edges": [-0.12, 0.17, 0.78], "n_values": [1.0, [1.9, 0.3]]}]})";
const char* kLossyAbsorbingExit = R"("stack": {"nI": 1.2, "nII": [1.5, 0.04], "period": 0.9, "layers": [{"d": 0.23, "edges": [0.0, 0.21, 0.47, 0.9], "n_values": [1.7, 1.0, [2.1, 0.05]]}, {"d": 0.19, "n": [1.4, 0.02]}, {"d": 0.31, "edges": [-0.12, 0.17, 0.78], "n_values": [1.0, [1.9, 0.3]]}]})";
const char* kFilms = R"("stack": {"nI": 1.0, "nII": 1.52, "period": 1.0, "layers": [{"d": 0.1, "n": 2.3}, {"d": 0.2, "n": 1.38}, {"d": 0.05, "n": [1.7, 0.3]}]})";
const char* kSilver = R"("stack": {"nI": 1.0, "nII": [0.079095, 5.42875], "period": 0.6, "layers": [{"d": 0.1, "edges": [-0.1, 0.15, 0.5], "n_values": [[0.079095, 5.42875], 1.0]}]})";
const char* kRayleigh = R"("stack": {"nI": 1.0, "nII": 2.0, "period": 0.5747, "layers": [{"d": 0.38, "edges": [-0.086205, 0.086205, 0.488495], "n_values": [1.45, 1.0]}]})";
const char* kTrapezoid = R"("stack": {"nI": 1.0, "nII": 1.46, "period": 0.574, "layers": [{"d": 0.095, "edges": [0.0, 0.23247, 0.34153, 0.574], "n_values": [1.0, 1.46, 1.0]}, {"d": 0.095, "edges": [0.0, 0.21453, 0.35947, 0.574], "n_values": [1.0, 1.46, 1.0]}, {"d": 0.095, "edges": [0.0, 0.19659, 0.37741, 0.574], "n_values": [1.0, 1.46, 1.0]}, {"d": 0.095, "edges": [0.0, 0.17865, 0.39535, 0.574], "n_values": [1.0, 1.46, 1.0]}, {"d": 0.115306, "n": 1.96}]})";
const char* kFFT = R"("stack": {"nI": 1.0, "nII": 1.46, "period": 0.574, "layers": [{"d": 0.38, "edges": [0.0, 0.1722, 0.574], "n_values": [1.46, 1.0], "fourier_method": "fft", "fft_samples": 4096}, {"d": 0.115, "n": 1.96}]})";
const char* kPillar = R"("stack": {"nI": 1.0, "nII": 1.46, "Lx": 0.8, "Ly": 0.8, "layers": [{"d": 0.3, "y_edges": [0.0, 0.25, 0.55, 0.8], "x_profiles": [{"edges": [0.0, 0.8], "n_values": [1.0]}, {"edges": [0.0, 0.25, 0.55, 0.8], "n_values": [1.0, 1.8, 1.0]}, {"edges": [0.0, 0.8], "n_values": [1.0]}]}, {"d": 0.115, "n": [1.96, 0.0]}]})";
const char* kPillarAbs = R"("stack": {"nI": 1.2, "nII": [1.5, 0.03], "Lx": 0.62, "Ly": 0.93, "layers": [{"d": 0.1, "n": [1.65, 0.12]}, {"d": 0.28, "y_edges": [0.0, 0.3, 0.7, 0.93], "x_profiles": [{"edges": [0.0, 0.62], "n_values": [1.0]}, {"edges": [0.0, 0.2, 0.46, 0.62], "n_values": [1.0, [1.8, 0.13], 1.0]}, {"edges": [0.0, 0.62], "n_values": [1.0]}]}, {"d": 0.0, "n": 1.3}, {"d": 0.2, "n": 1.9}]})";

std::string planar(const char* stack, const std::string& rest) { return std::string("{\"mode\": \"planar\", ") + stack + ", " + rest + "}"; }
std::string conical(const char* stack, const std::string& rest) { return std::string("{\"mode\": \"conical\", ") + stack + ", " + rest + "}"; }
std::string grid2d(const char* stack, const std::string& rest) { return std::string("{\"mode\": \"periodic2d\", ") + stack + ", " + rest + "}"; }

void put(std::FILE* f, const std::string& s) {
    std::string out;
    stablercwa::json::detail::append_string(out, s.data(), s.size());
    std::fputs(out.c_str(), f);
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    std::vector<std::pair<std::string, std::string>> cases = {
        // ---- valid requests
        {"planar_readme_te", planar(kExample, R"("M": 20, "polarization": "TE", "wavelength": 1.053, "theta_deg": 66.36)")},
        {"planar_readme_tm_sweep", planar(kExample, R"("M": 20, "polarization": "TM", "points": [{"wavelength": 1.053, "theta_deg": 66.36}, {"wavelength": 0.9, "theta_deg": 10.0}, {"wavelength": 1.2, "theta_deg": -35.0}], "options": {"diagnostics": true, "threads": 4})")},
        {"planar_lossy_te", planar(kLossyAbsorbingExit, R"("M": 12, "polarization": "TE", "points": [{"wavelength": 0.83, "theta_deg": 27.0}, {"wavelength": 1.1, "theta_deg": 5.0}])")},
        {"planar_films_tm", planar(kFilms, R"("M": 5, "polarization": "TM", "points": [{"wavelength": 0.8, "theta_deg": 35.0}, {"wavelength": 0.55, "theta_deg": 0.0}])")},
        {"planar_silver_tm", planar(kSilver, R"("M": 15, "polarization": "TM", "wavelength": 0.633, "theta_deg": 20.0)")},
        {"planar_rayleigh_sweep", planar(kRayleigh, R"("M": 8, "polarization": "TE", "points": [{"wavelength": 0.6, "theta_deg": 10.0}, {"wavelength": 0.5747, "theta_deg": 0.0}, {"wavelength": 0.61, "theta_deg": 0.0}])")},
        {"planar_fft", planar(kFFT, R"("M": 10, "polarization": "TE", "wavelength": 1.053, "theta_deg": 40.0, "options": {"eig": "qr", "linear": "lu", "homogeneous_fast_path": true, "parallel_layers": true, "backend": "builtin"})")},
        {"planar_trapezoid_indent", planar(kTrapezoid, R"("M": 25, "polarization": "TE", "points": [{"wavelength": 1.0, "theta_deg": 30.0}])")},
        {"conical_lossy", conical(kLossy, R"("M": 6, "points": [{"wavelength": 0.83, "theta_deg": 27.0, "phi_deg": 31.0}, {"wavelength": 0.95, "theta_deg": 12.0}])")},
        {"conical_example_angles", conical(kExample, R"("M": 8, "wavelength": 1.053, "theta_deg": 40.0, "phi_deg": 25.0, "input": {"psi_deg": 45.0, "delta_deg": 90.0})")},
        {"conical_lossy_jones", conical(kLossy, R"("M": 5, "points": [{"wavelength": 0.83, "theta_deg": 27.0, "phi_deg": -61.0}], "input": {"jones": [[0.3, 0.2], [-0.7, 0.5]]})")},
        {"conical_films_normal", conical(kFilms, R"("M": 3, "points": [{"wavelength": 0.8, "theta_deg": 0.0, "phi_deg": 0.0}, {"wavelength": 0.7, "theta_deg": 20.0, "phi_deg": 45.0}], "input": {"psi_deg": 90.0})")},
        {"periodic2d_pillar", grid2d(kPillar, R"("M": 3, "My": 3, "points": [{"wavelength": 1.053, "theta_deg": 42.0, "phi_deg": -25.0}, {"wavelength": 0.9, "theta_deg": 10.0}], "input": {"psi_deg": 90.0, "delta_deg": 0.0})")},
        {"periodic2d_absorbing_laurent", grid2d(kPillarAbs, R"("M": 2, "My": 1, "wavelength": 0.83, "theta_deg": 27.0, "phi_deg": -61.0, "input": {"jones": [[0.6, 0.0], [0.0, 0.8]]}, "options": {"factorization": "laurent", "diagnostics": true})")},
        {"periodic2d_rayleigh", grid2d(kPillar, R"("M": 2, "My": 2, "points": [{"wavelength": 0.8, "theta_deg": 0.0}, {"wavelength": 0.85, "theta_deg": 5.0}], "input": {"psi_deg": 30.0})")},
        {"periodic2d_indent", grid2d(kPillarAbs, R"("M": 1, "My": 2, "points": [{"wavelength": 0.75, "theta_deg": 15.0, "phi_deg": 10.0}], "input": {"psi_deg": 0.0})")},
        // ---- invalid requests (where, and the message of each check)
        {"bad_syntax", R"({"mode": "planar",)"},
        {"bad_top_array", "[1, 2]"},
        {"bad_duplicate_key", R"({"mode": "planar", "mode": "planar"})"},
        {"bad_huge_number", R"({"mode": "planar", "M": 1e999})"},
        {"bad_leading_zero", R"({"mode": "planar", "M": 020})"},
        {"bad_no_mode", R"({"M": 3})"},
        {"bad_mode", R"({"mode": "spherical"})"},
        {"bad_unknown_key", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "colour": 1)")},
        {"bad_planar_phi", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "phi_deg": 3.0)")},
        {"bad_planar_input", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0})")},
        {"bad_stack_type", R"({"mode": "planar", "stack": 3, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_stack_key", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [], "Lx": 1.0}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_nI_absorbing", R"({"mode": "planar", "stack": {"nI": [1.0, 0.1], "nII": 1.5, "period": 1.0, "layers": []}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_nI_negative", R"({"mode": "planar", "stack": {"nI": -1.0, "nII": 1.5, "period": 1.0, "layers": []}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_conical_nII", conical(kLossyAbsorbingExit, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_period", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 0.0, "layers": []}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_layers_type", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": {}}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_layer_mixed", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "n": 1.5, "edges": [0.0, 1.0]}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_layer_no_index", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "n": 1.5}, {"d": 0.2}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_layer_d", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": -0.1, "n": 1.5}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_edges_order", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 0.4, 1.0], "n_values": [1.0, 2.0, 1.5]}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_edges_span", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 0.9], "n_values": [1.0, 2.0]}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_edges_missing", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "n_values": [1.0, 2.0]}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_segments", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 1.0], "n_values": [1.0, 2.0, 3.0]}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_n_value", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 1.0], "n_values": [1.0, [2.0, -0.1]]}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_n_shape", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": [1.5, 0.0, 1.0], "period": 1.0, "layers": []}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_fourier_method", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 1.0], "n_values": [1.0, 2.0], "fourier_method": "dft"}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_fft_samples", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 1.0], "n_values": [1.0, 2.0], "fourier_method": "fft", "fft_samples": -1}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_fft_too_few", R"({"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": [{"d": 0.1, "edges": [0.0, 0.5, 1.0], "n_values": [1.0, 2.0], "fourier_method": "fft", "fft_samples": 12}]}, "M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0})"},
        {"bad_M_negative", planar(kExample, R"("M": -1, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_M_huge", planar(kExample, R"("M": 9000, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_M_text", planar(kExample, R"("M": "20", "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_M_fraction", planar(kExample, R"("M": 2.5, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_conical_M", conical(kExample, R"("M": 4096, "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_polarization", planar(kExample, R"("M": 3, "polarization": "TX", "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_no_polarization", planar(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_points_both", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "points": [])")},
        {"bad_points_none", planar(kExample, R"("M": 3, "polarization": "TE")")},
        {"bad_points_empty", planar(kExample, R"("M": 3, "polarization": "TE", "points": [])")},
        {"bad_point_type", planar(kExample, R"("M": 3, "polarization": "TE", "points": [{"wavelength": 1.0, "theta_deg": 0.0}, 7])")},
        {"bad_theta", planar(kExample, R"("M": 3, "polarization": "TE", "points": [{"wavelength": 1.0, "theta_deg": 90.0}])")},
        {"bad_wavelength", planar(kExample, R"("M": 3, "polarization": "TE", "points": [{"wavelength": -1.0, "theta_deg": 0.0}])")},
        {"bad_point_phi", planar(kExample, R"("M": 3, "polarization": "TE", "points": [{"wavelength": 1.0, "theta_deg": 0.0, "phi_deg": 1.0}])")},
        {"bad_point_key", planar(kExample, R"("M": 3, "polarization": "TE", "points": [{"lambda": 1.0, "theta_deg": 0.0}])")},
        {"bad_point_missing", planar(kExample, R"("M": 3, "polarization": "TE", "points": [{"wavelength": 1.0}])")},
        {"bad_options_type", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": [])")},
        {"bad_options_key", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"speed": 1})")},
        {"bad_options_eig", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"eig": "jacobi"})")},
        {"bad_options_linear", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"linear": "cholesky"})")},
        {"bad_options_threads", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"threads": 0})")},
        {"bad_options_threads_fraction", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"threads": 1.5})")},
        {"bad_options_diagnostics", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"diagnostics": "yes"})")},
        {"bad_options_backend", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"backend": "mkl"})")},
        {"bad_options_backend_name", planar(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": {"backend": "cuda"})")},
        {"bad_conical_polarization", conical(kExample, R"("M": 3, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_input_both", conical(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 1.0, "jones": [1.0, 0.0]})")},
        {"bad_input_zero", conical(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0, "input": {"jones": [0.0, [0.0, 0.0]]})")},
        {"bad_input_length", conical(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0, "input": {"jones": [1.0, 0.0, 0.0]})")},
        {"bad_input_no_psi", conical(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0, "input": {"delta_deg": 1.0})")},
        {"bad_input_psi_text", conical(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": "s"})")},
        {"bad_conical_phi", conical(kExample, R"("M": 3, "wavelength": 1.0, "theta_deg": 0.0, "phi_deg": "east")")},
        {"bad_2d_polarization", grid2d(kPillar, R"("M": 2, "My": 2, "polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0})")},
        {"bad_2d_period", grid2d(kPillar, R"("M": 2, "My": 2, "period": 1.0, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0})")},
        {"bad_2d_stack_period", R"({"mode": "periodic2d", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": []}, "M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}})"},
        {"bad_2d_no_My", grid2d(kPillar, R"("M": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0})")},
        {"bad_2d_M_large", grid2d(kPillar, R"("M": 1024, "My": 0, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0})")},
        {"bad_2d_harmonics", grid2d(kPillar, R"("M": 20, "My": 30, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0})")},
        {"bad_2d_no_input", grid2d(kPillar, R"("M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0)")},
        {"bad_2d_linear", grid2d(kPillar, R"("M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}, "options": {"linear": "lu"})")},
        {"bad_2d_factorization", grid2d(kPillar, R"("M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}, "options": {"factorization": "fft"})")},
        {"bad_2d_profiles_count", R"({"mode": "periodic2d", "stack": {"nI": 1.0, "nII": 1.5, "Lx": 1.0, "Ly": 1.0, "layers": [{"d": 0.1, "y_edges": [0.0, 0.5, 1.0], "x_profiles": [{"edges": [0.0, 1.0], "n_values": [1.5]}]}]}, "M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}})"},
        {"bad_2d_profile_span", R"({"mode": "periodic2d", "stack": {"nI": 1.0, "nII": 1.5, "Lx": 1.0, "Ly": 1.0, "layers": [{"d": 0.1, "y_edges": [0.0, 1.0], "x_profiles": [{"edges": [0.0, 0.9], "n_values": [1.5]}]}]}, "M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}})"},
        {"bad_2d_y_order", R"({"mode": "periodic2d", "stack": {"nI": 1.0, "nII": 1.5, "Lx": 1.0, "Ly": 1.0, "layers": [{"d": 0.1, "y_edges": [0.0, 0.6, 0.6, 1.0], "x_profiles": [{"edges": [0.0, 1.0], "n_values": [1.5]}, {"edges": [0.0, 1.0], "n_values": [1.5]}, {"edges": [0.0, 1.0], "n_values": [1.5]}]}]}, "M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}})"},
        {"bad_2d_Lx", R"({"mode": "periodic2d", "stack": {"nI": 1.0, "nII": 1.5, "Lx": -1.0, "Ly": 1.0, "layers": []}, "M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}})"},
        {"bad_2d_layer_key", R"({"mode": "periodic2d", "stack": {"nI": 1.0, "nII": 1.5, "Lx": 1.0, "Ly": 1.0, "layers": [{"d": 0.1, "n": 1.5, "name": "film"}]}, "M": 2, "My": 2, "wavelength": 1.0, "theta_deg": 0.0, "input": {"psi_deg": 0.0}})"},
    };
    for (const auto& c : cases) {
        const int indent = c.first.find("indent") != std::string::npos ? 2 : -1;
        const stablercwa::rcwa::JsonReply r = stablercwa::rcwa::solve_json_reply(c.second, indent);
        std::fprintf(f, "{\"name\": \"%s\", \"indent\": %d, \"request\": ", c.first.c_str(), indent);
        put(f, c.second);
        std::fprintf(f, ", \"reply\": ");
        put(f, r.text);
        std::fprintf(f, "}\n");
    }
    if (f != stdout) std::fclose(f);
    return 0;
}
