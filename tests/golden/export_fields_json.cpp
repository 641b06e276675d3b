// Golden-fixture exporter for the near-field protocol (rcwa::solve_fields_json_reply,
// include/stablercwa/rcwa_fields_json.hpp).
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). Every request below is
// answered by the reference into a fresh directory under a temporary root; the fixture line holds the request
// (with OUTPUT_DIR standing for the directory), the reply (directory path replaced by OUTPUT_DIR) and, when the
// reply is ok, the published NPY arrays read back: fields [6, nz, n] as [re, im] pairs, phase [2, 6, nz, n]
// (NaN as "nan"), the mask as a '0'/'1' string, the coordinate files. One JSON object per line.
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

#include "stablercwa/rcwa_fields_json.hpp"

namespace {

namespace fs = std::filesystem;

void put(std::FILE* f, const std::string& s) {
    std::string out;
    stablercwa::json::detail::append_string(out, s.data(), s.size());
    std::fputs(out.c_str(), f);
}
void put_d(std::FILE* f, double v) {
    std::string out;
    if (std::isnan(v)) out = "\"nan\"";
    else stablercwa::json::detail::append_double(out, v);
    std::fputs(out.c_str(), f);
}

std::string replace_all(std::string s, const std::string& from, const std::string& to) {
    for (std::size_t at = s.find(from); at != std::string::npos; at = s.find(from, at + to.size())) s.replace(at, from.size(), to);
    return s;
}

// the data bytes of an NPY file (after the header)
std::vector<char> npy_data(const fs::path& path) {
    std::ifstream in(path, std::ios::binary);
    std::vector<char> bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    const std::size_t header = static_cast<unsigned char>(bytes[8]) | (static_cast<unsigned char>(bytes[9]) << 8);
    return std::vector<char>(bytes.begin() + 10 + header, bytes.end());
}
void put_doubles(std::FILE* f, const char* key, const fs::path& path) {
    const std::vector<char> b = npy_data(path);
    std::fprintf(f, ",\"%s\":[", key);
    for (std::size_t k = 0; k * 8 < b.size(); ++k) {
        double v;
        std::memcpy(&v, &b[k * 8], 8);
        if (k) std::fputc(',', f);
        put_d(f, v);
    }
    std::fputc(']', f);
}
void put_complex(std::FILE* f, const char* key, const fs::path& path) {
    const std::vector<char> b = npy_data(path);
    std::fprintf(f, ",\"%s\":[", key);
    for (std::size_t k = 0; k * 16 < b.size(); ++k) {
        double re, im;
        std::memcpy(&re, &b[k * 16], 8);
        std::memcpy(&im, &b[k * 16 + 8], 8);
        std::fprintf(f, "%s[", k ? "," : "");
        put_d(f, re);
        std::fputc(',', f);
        put_d(f, im);
        std::fputc(']', f);
    }
    std::fputc(']', f);
}
void put_bytes(std::FILE* f, const char* key, const fs::path& path) {
    const std::vector<char> b = npy_data(path);
    std::fprintf(f, ",\"%s\":\"", key);
    for (char c : b) std::fputc(c ? '1' : '0', f);
    std::fputc('"', f);
}

const char* kMixed = R"("stack": {"nI": 1.2, "nII": 1.4, "period": 0.6, "layers": [{"d": 0.2, "edges": [0.0, 0.21, 0.6], "n_values": [1.7, 1.0]}, {"d": 0.09, "n": [1.46, 0.03]}, {"d": 0.13, "edges": [0.0, 0.12, 0.6], "n_values": [1.1, [1.9, 0.07]]}]})";
const char* kExample = R"("stack": {"nI": 1.0, "nII": 1.46, "period": 0.574, "layers": [{"d": 0.38, "edges": [0.0, 0.1722, 0.574], "n_values": [1.46, 1.0]}, {"d": 0.0, "n": 1.7}, {"d": 0.115, "n": [1.96, 0.0]}]})";
const char* kSchur = R"("stack": {"nI": 1.0, "nII": 1.46, "period": 0.574, "layers": [{"d": 0.38, "edges": [0.0, 0.1722, 0.574], "n_values": [1.46, 1.0]}, {"d": 0.115, "n": 1.96}]})";
const char* kRayleigh = R"("stack": {"nI": 1.0, "nII": 2.0, "period": 0.5747, "layers": [{"d": 0.38, "edges": [-0.086205, 0.086205, 0.488495], "n_values": [1.45, 1.0]}]})";
const char* kPillar = R"("stack": {"nI": 1.0, "nII": 1.46, "Lx": 0.8, "Ly": 0.8, "layers": [{"d": 0.3, "y_edges": [0.0, 0.25, 0.55, 0.8], "x_profiles": [{"edges": [0.0, 0.8], "n_values": [1.0]}, {"edges": [0.0, 0.25, 0.55, 0.8], "n_values": [1.0, 1.8, 1.0]}, {"edges": [0.0, 0.8], "n_values": [1.0]}]}, {"d": 0.115, "n": [1.96, 0.0]}]})";
const char* kPillarAbs = R"("stack": {"nI": 1.2, "nII": [1.5, 0.03], "Lx": 0.62, "Ly": 0.93, "layers": [{"d": 0.1, "n": [1.65, 0.12]}, {"d": 0.28, "y_edges": [0.0, 0.3, 0.7, 0.93], "x_profiles": [{"edges": [0.0, 0.62], "n_values": [1.0]}, {"edges": [0.0, 0.2, 0.46, 0.62], "n_values": [1.0, [1.8, 0.13], 1.0]}, {"edges": [0.0, 0.62], "n_values": [1.0]}]}, {"d": 0.0, "n": 1.3}, {"d": 0.2, "n": 1.9}]})";

std::string request(const std::string& solve, const std::string& sampling, const std::string& id = "case") {
    return "{\"solve\": " + solve + ", \"sampling\": " + sampling + ", \"output_dir\": \"OUTPUT_DIR\", \"request_id\": \"" + id + "\"}";
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    char tmpl[] = "/tmp/stablercwa_fields_XXXXXX";
    const fs::path root = mkdtemp(tmpl);
    const std::string z1 = R"([-0.2, 0.0, 0.1, 0.25, 0.2, 0.42, 0.6])";
    struct Case {
        std::string name, text;
        bool pre_create = false;
    };
    std::vector<Case> cases = {
        {"planar_tm", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 6, "polarization": "TM", "wavelength": 0.83, "theta_deg": 27.0})",
                              "{\"z\": " + z1 + R"(, "nx": 16})")},
        {"planar_te_zero_layer", request(std::string("{\"mode\": \"planar\", ") + kExample + R"(, "M": 10, "polarization": "TE", "points": [{"wavelength": 1.053, "theta_deg": 30.0}]})",
                                         R"({"z": [-0.1, 0.19, 0.38, 0.45, 0.7], "nx": 12, "y": 0})")},
        {"conical_angles", request(std::string("{\"mode\": \"conical\", ") + kMixed + R"(, "M": 5, "wavelength": 0.83, "theta_deg": 27.0, "phi_deg": 31.0, "input": {"psi_deg": 45.0, "delta_deg": 90.0}})",
                                   "{\"z\": " + z1 + R"(, "nx": 10, "y": 0.11})")},
        {"conical_schur_jones", request(std::string("{\"mode\": \"conical\", ") + kSchur + R"(, "M": 8, "wavelength": 0.980484673140678, "theta_deg": 40.0, "phi_deg": 25.0, "input": {"jones": [[0.3, 0.2], [-0.7, 0.5]]}})",
                                        R"({"z": [-0.05, 0.0, 0.1, 0.2, 0.3, 0.38, 0.45, 0.6], "nx": 9})")},
        {"periodic2d_xz", request(std::string("{\"mode\": \"periodic2d\", ") + kPillar + R"(, "M": 2, "My": 2, "wavelength": 1.053, "theta_deg": 42.0, "phi_deg": -25.0, "input": {"psi_deg": 90.0}})",
                                  R"({"z": [-0.2, 0.05, 0.15, 0.3, 0.35, 0.6], "plane": "xz", "nt": 12, "at": 0.3})")},
        {"periodic2d_yz", request(std::string("{\"mode\": \"periodic2d\", ") + kPillarAbs + R"(, "M": 2, "My": 1, "wavelength": 0.83, "theta_deg": 27.0, "phi_deg": -61.0, "input": {"jones": [[0.6, 0.0], [0.0, 0.8]]}, "options": {"factorization": "laurent"}})",
                                  R"({"z": [-0.1, 0.05, 0.2, 0.38, 0.45, 0.7], "plane": "yz", "nt": 10, "at": 0.21})")},
        // requests that publish nothing
        {"exists", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 3, "polarization": "TE", "wavelength": 0.83, "theta_deg": 27.0})",
                           R"({"z": [0.1], "nx": 4})"), true},
        {"planar_y", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 3, "polarization": "TE", "wavelength": 0.83, "theta_deg": 27.0})",
                             R"({"z": [0.1], "nx": 4, "y": 0.5})")},
        {"conical_no_input", request(std::string("{\"mode\": \"conical\", ") + kMixed + R"(, "M": 3, "wavelength": 0.83, "theta_deg": 27.0})",
                                     R"({"z": [0.1], "nx": 4})")},
        {"two_points", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 3, "polarization": "TE", "points": [{"wavelength": 0.83, "theta_deg": 27.0}, {"wavelength": 0.9, "theta_deg": 2.0}]})",
                               R"({"z": [0.1], "nx": 4})")},
        {"plane_name", request(std::string("{\"mode\": \"periodic2d\", ") + kPillar + R"(, "M": 1, "My": 1, "wavelength": 1.0, "theta_deg": 10.0, "input": {"psi_deg": 0.0}})",
                               R"({"z": [0.1], "plane": "xy", "nt": 4})")},
        {"sampling_nx", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 3, "polarization": "TE", "wavelength": 0.83, "theta_deg": 27.0})",
                                R"({"z": [0.1], "nx": 0})")},
        {"sampling_empty", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 3, "polarization": "TE", "wavelength": 0.83, "theta_deg": 27.0})",
                                   R"({"z": [], "nx": 4})")},
        {"sampling_key", request(std::string("{\"mode\": \"periodic2d\", ") + kPillar + R"(, "M": 1, "My": 1, "wavelength": 1.0, "theta_deg": 10.0, "input": {"psi_deg": 0.0}})",
                                 R"({"z": [0.1], "plane": "xz", "nt": 4, "nx": 3})")},
        {"no_request_id", request(std::string("{\"mode\": \"planar\", ") + kMixed + R"(, "M": 3, "polarization": "TE", "wavelength": 0.83, "theta_deg": 27.0})",
                                  R"({"z": [0.1], "nx": 4})", "")},
        {"planar_failure", request(std::string("{\"mode\": \"planar\", ") + kRayleigh + R"(, "M": 8, "polarization": "TE", "wavelength": 0.5747, "theta_deg": 0.0})",
                                   R"({"z": [0.1], "nx": 4})")},
        {"periodic2d_rayleigh", request(std::string("{\"mode\": \"periodic2d\", ") + kPillar + R"(, "M": 2, "My": 2, "wavelength": 0.8, "theta_deg": 0.0, "input": {"psi_deg": 30.0}})",
                                        R"({"z": [0.1], "plane": "xz", "nt": 4})")},
    };
    int k = 0;
    for (const Case& c : cases) {
        const fs::path dir = root / ("case" + std::to_string(k++));
        if (c.pre_create) fs::create_directory(dir);
        const std::string text = replace_all(c.text, "OUTPUT_DIR", dir.string());
        const stablercwa::rcwa::JsonReply r = stablercwa::rcwa::solve_fields_json_reply(text);
        std::fprintf(f, "{\"name\":\"%s\",\"pre_create\":%d,\"ok\":%d,\"request\":", c.name.c_str(), c.pre_create ? 1 : 0, r.ok ? 1 : 0);
        put(f, c.text);
        std::fprintf(f, ",\"reply\":");
        put(f, replace_all(r.text, dir.string(), "OUTPUT_DIR"));
        if (r.ok) {
            put_complex(f, "fields", dir / "fields.npy");
            put_doubles(f, "phase", dir / "phase.npy");
            put_bytes(f, "phase_mask", dir / "phase_mask.npy");
            put_doubles(f, "x", dir / "x.npy");
            put_doubles(f, "z", dir / "z.npy");
            if (fs::exists(dir / "t.npy")) {
                put_doubles(f, "t", dir / "t.npy");
                put_doubles(f, "y", dir / "y.npy");
            }
        }
        std::fprintf(f, "}\n");
    }
    fs::remove_all(root);
    if (f != stdout) std::fclose(f);
    return 0;
}
