// json_front.cpp -- the JSON request front end (rcwa::solve_json_reply, include/stablercwa/rcwa_json.hpp:1287-1312):
// one JSON request (planar, conical or periodic2d, one or many incidence points) in, one JSON reply out, run
// either as one batched call on a context or as one request per point on the serving loop.
//
// Request validation follows the reference's reader (rcwa_json.hpp:214-800): unknown keys are errors, every
// error carries the path of the offending field (stack.layers[1].n_values[0], points[2].theta_deg, ...) and
// the reference's message text. The reply has the reference's field order; its numbers are the engine's
// results written with the shortest round-trip decimal, so reading them back gives the engine's doubles
// bit for bit. Where this engine differs from the reference the reply says so instead of guessing: the
// options the engine does not implement (eig "lr", linear "lu_nopivot"/"qr", homogeneous_fast_path false,
// backend "mkl") are request errors naming the option; per-point timing is the call's wall time shared over
// its points (context) or the request's own run time (serving loop); max_solve_backward_error is 0.
//
// The front end is a client of the C ABI (rcwa_gpu_solve1d_batch, rcwa_gpu_solve_conical_batch,
// rcwa_gpu_solve2d_batch, rcwa_gpu_server_submit / wait).
#include <algorithm>
#include <chrono>
#include <filesystem>
#include <fstream>
#include <random>
#include <stdexcept>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/stablercwa_gb300.h"
#include "json_text.h"

namespace rcwa_gb300 {
namespace jfront {
namespace {

using cd = std::complex<double>;
using jtext::Value;
using jtext::Writer;

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr int kVersion = 1;
constexpr int kMaxThreads = 256;
constexpr int kMax2dHarmonics = 2048;
constexpr int kMaxMatrixOrder = 16384;
constexpr int kMaxFFTSamples = 4194304;

struct RequestError {
    std::string message, where;
};
[[noreturn]] void fail(const std::string& where, const std::string& message) { throw RequestError{message, where}; }

// ------------------------------------------------------------------ paths and typed reads

std::string shown_key(const std::string& key) {
    if (key.size() <= 48) return key;
    std::size_t cut = 48;
    while (cut > 0 && (static_cast<unsigned char>(key[cut]) & 0xC0) == 0x80) --cut;
    return key.substr(0, cut) + "...";
}
std::string child(const std::string& path, const std::string& key) { return path.empty() ? key : path + "." + key; }
std::string child(const std::string& path, std::size_t index) { return path + "[" + std::to_string(index) + "]"; }

void check_keys(const Value& object, const std::string& path, std::initializer_list<const char*> allowed) {
    for (const std::string& key : object.keys) {
        bool known = false;
        for (const char* name : allowed) known = known || key == name;
        if (known) continue;
        std::string list;
        for (const char* name : allowed) {
            if (!list.empty()) list += "、";
            list += name;
        }
        fail(child(path, shown_key(key)), "不认识的键（这里可以写：" + list + "）");
    }
}
const Value& member(const Value& object, const char* key, const std::string& path) {
    const Value* v = object.find(key);
    if (!v) fail(child(path, key), "缺少这一项");
    return *v;
}
void need_object(const Value& v, const std::string& where) {
    if (!v.is_object()) fail(where, "应当是一个对象 {…}");
}
void need_array(const Value& v, const std::string& where) {
    if (!v.is_array()) fail(where, "应当是一个数组 […]");
}
double number(const Value& v, const std::string& where) {
    if (!v.is_number()) fail(where, "应当是一个数");
    return v.number;
}
int integer(const Value& v, const std::string& where) {
    int out = 0;
    if (!v.to_int(out)) fail(where, "应当是一个整数");
    return out;
}
bool truth(const Value& v, const std::string& where) {
    if (!v.is_bool()) fail(where, "应当是 true 或 false");
    return v.boolean;
}
std::string text(const Value& v, const std::string& where) {
    if (!v.is_string()) fail(where, "应当是一个字符串");
    return v.text;
}
cd complex_number(const Value& v, const std::string& where) {
    if (v.is_number()) return cd{v.number, 0.0};
    if (!v.is_array() || v.size() != 2 || !v.at(0).is_number() || !v.at(1).is_number())
        fail(where, "应当是一个实数，或者 [实部, 虚部]");
    return cd{v.at(0).number, v.at(1).number};
}
bool finite(cd z) { return std::isfinite(z.real()) && std::isfinite(z.imag()); }
void check_index(cd n, const std::string& where) {
    if (!finite(n) || std::abs(n) == 0.0 || n.real() < 0.0 || n.imag() < 0.0)
        fail(where, "折射率不能是零，实部、虚部都不能是负的（吸收介质写成 [n, k]，k > 0）");
}

// ------------------------------------------------------------------ the request

struct Layer1 {
    double d = 0.0;
    bool homogeneous = true;
    cd n{1.0, 0.0};
    std::vector<double> edges;
    std::vector<cd> values;
    int fourier_method = 0, fft_samples = 0;
};
struct Stack1 {
    cd nI{1.0, 0.0}, nII{1.0, 0.0};
    double period = 1.0;
    std::vector<Layer1> layers;
};
struct Layer2 {
    double d = 0.0;
    bool homogeneous = true;
    cd n{1.0, 0.0};
    std::vector<double> y_edges;
    std::vector<std::vector<double>> x_edges;
    std::vector<std::vector<cd>> x_values;
};
struct Stack2 {
    double nI = 1.0;
    cd nII{1.0, 0.0};
    double Lx = 1.0, Ly = 1.0;
    std::vector<Layer2> layers;
};
struct PointSpec {
    double wavelength = 1.0, theta_deg = 0.0, phi_deg = 0.0;
};
enum class Mode { Planar, Conical, Periodic2D };
enum class Input { None, Angles, Jones };

struct Request {
    Mode mode = Mode::Planar;
    Stack1 stack;
    Stack2 stack2d;
    int M = 0, My = 0;
    int polarization = RCWA_TE;
    std::vector<PointSpec> points;
    bool points_array = false;
    int threads = 0;
    bool diagnostics = false;
    bool laurent = false;
    Input input = Input::None;
    double psi_deg = 0.0, delta_deg = 0.0;
    cd Es, Ep;
};

// the engine implements eig "qr", linear "lu" and the homogeneous fast path only
[[noreturn]] void unsupported(const std::string& where, const std::string& what) {
    fail(where, "GPU 引擎没有实现 " + what + "（只实现了 QR 本征分解、按列选主元 LU 与均匀层快速路径）");
}

// rcwa::resolve_fft_samples's checks (include/stablercwa/fourier.hpp:26-41)
void check_fft_samples(int M, int samples, const std::string& where) {
    if (M > (kMaxFFTSamples - 1) / 4) fail(where, "rcwa: FFT truncation requires more than 4194304 samples");
    if (samples == 0) {
        const long long target = std::max(8192LL, 64LL * (2LL * M + 1));
        if (target > kMaxFFTSamples) fail(where, "rcwa: automatic FFT exceeds 4194304 samples");
        return;
    }
    if (samples <= 4 * M) fail(where, "rcwa: fft_samples must be at least 4*M+1");
}

// rcwa_json.hpp:307-364
Layer1 read_layer(const Value& v, const std::string& path, double period) {
    need_object(v, path);
    check_keys(v, path, {"d", "n", "edges", "n_values", "fourier_method", "fft_samples"});
    Layer1 layer;
    layer.d = number(member(v, "d", path), child(path, "d"));
    if (!std::isfinite(layer.d) || layer.d < 0.0) fail(child(path, "d"), "层厚不能是负的");
    const Value* n = v.find("n");
    const Value* edges = v.find("edges");
    const Value* values = v.find("n_values");
    if (n && (edges || values)) fail(path, "均匀层只写 n，光栅层只写 edges 和 n_values，两种写法不能混在一层里");
    if (!n && !edges && !values) fail(path, "缺少折射率：均匀层写 n，光栅层写 edges 和 n_values");
    if (n) {
        layer.n = complex_number(*n, child(path, "n"));
        check_index(layer.n, child(path, "n"));
    } else {
        const std::string ep = child(path, "edges"), vp = child(path, "n_values");
        if (!edges) fail(ep, "光栅层还要写 edges（一个周期内的分段边界）");
        if (!values) fail(vp, "光栅层还要写 n_values（各段的折射率）");
        need_array(*edges, ep);
        need_array(*values, vp);
        layer.homogeneous = false;
        for (std::size_t j = 0; j < edges->size(); ++j) layer.edges.push_back(number(edges->at(j), child(ep, j)));
        for (std::size_t j = 0; j < values->size(); ++j) {
            layer.values.push_back(complex_number(values->at(j), child(vp, j)));
            check_index(layer.values.back(), child(vp, j));
        }
        const std::vector<double>& e = layer.edges;
        if (layer.values.empty() || e.size() != layer.values.size() + 1)
            fail(vp, "段数对不上：K 段折射率要配 K+1 个边界（现在是 " + std::to_string(layer.values.size()) + " 段折射率、" +
                         std::to_string(e.size()) + " 个边界）");
        for (std::size_t j = 0; j < e.size(); ++j)
            if (!std::isfinite(e[j]) || (j > 0 && e[j] <= e[j - 1])) fail(child(ep, j), "分段边界必须严格递增");
        if (std::abs((e.back() - e.front()) - period) > 1e-10 * period)
            fail(ep, "分段边界的首尾必须正好相差一个周期（stack.period）");
    }
    if (const Value* method = v.find("fourier_method")) {
        const std::string where = child(path, "fourier_method");
        const std::string name = text(*method, where);
        if (name == "analytic") layer.fourier_method = 0;
        else if (name == "fft") layer.fourier_method = 1;
        else fail(where, "只能是 \"analytic\" 或 \"fft\"");
    }
    if (const Value* samples = v.find("fft_samples")) {
        const std::string where = child(path, "fft_samples");
        layer.fft_samples = integer(*samples, where);
        if (layer.fft_samples < 0 || layer.fft_samples > kMaxFFTSamples) fail(where, "FFT 采样数必须为 0..4194304（0 表示自动选择）");
    }
    return layer;
}

Stack1 read_stack(const Value& v, bool conical) {
    const std::string path = "stack";
    need_object(v, path);
    check_keys(v, path, {"nI", "nII", "period", "layers"});
    Stack1 s;
    s.nI = complex_number(member(v, "nI", path), "stack.nI");
    check_index(s.nI, "stack.nI");
    if (s.nI.imag() != 0.0 || s.nI.real() <= 0.0) fail("stack.nI", "入射介质必须无吸收，折射率是正实数");
    s.nII = complex_number(member(v, "nII", path), "stack.nII");
    check_index(s.nII, "stack.nII");
    if (conical && s.nII.imag() != 0.0) fail("stack.nII", "圆锥入射要求出射介质的折射率是实数");
    s.period = number(member(v, "period", path), "stack.period");
    if (!std::isfinite(s.period) || s.period <= 0.0) fail("stack.period", "周期必须是正数");
    const Value& layers = member(v, "layers", path);
    need_array(layers, "stack.layers");
    for (std::size_t i = 0; i < layers.size(); ++i) s.layers.push_back(read_layer(layers.at(i), child("stack.layers", i), s.period));
    return s;
}

PointSpec read_point(const Value& v, const std::string& path, bool azimuth) {
    PointSpec p;
    p.wavelength = number(member(v, "wavelength", path), child(path, "wavelength"));
    if (!std::isfinite(p.wavelength) || p.wavelength <= 0.0) fail(child(path, "wavelength"), "波长必须是正数");
    p.theta_deg = number(member(v, "theta_deg", path), child(path, "theta_deg"));
    if (!std::isfinite(p.theta_deg) || std::abs(p.theta_deg) >= 90.0)
        fail(child(path, "theta_deg"), "入射角必须严格在 -90 度与 90 度之间");
    if (azimuth)
        if (const Value* phi = v.find("phi_deg")) {
            p.phi_deg = number(*phi, child(path, "phi_deg"));
            if (!std::isfinite(p.phi_deg)) fail(child(path, "phi_deg"), "方位角必须是有限的数");
        }
    return p;
}

const char* planar_phi_message() { return "planar 模式没有方位角；方位角不为零的入射请用 conical 模式"; }

// rcwa_json.hpp:427-453
void read_points(const Value& root, Request& rq) {
    const Value* points = root.find("points");
    const bool single = root.contains("wavelength") || root.contains("theta_deg") || root.contains("phi_deg");
    if (points && single) fail("points", "入射点只能用一种写法：points 数组，或者写在最外层的 wavelength、theta_deg");
    if (!points && !single) fail("points", "缺少入射点：写 points 数组，或者把 wavelength、theta_deg 写在最外层");
    const bool azimuth = rq.mode != Mode::Planar;
    if (!points) {
        rq.points.push_back(read_point(root, "", azimuth));
        return;
    }
    rq.points_array = true;
    need_array(*points, "points");
    if (points->size() == 0) fail("points", "至少要有一个入射点");
    for (std::size_t k = 0; k < points->size(); ++k) {
        const std::string path = child("points", k);
        const Value& item = points->at(k);
        need_object(item, path);
        if (azimuth) {
            check_keys(item, path, {"wavelength", "theta_deg", "phi_deg"});
        } else {
            if (item.contains("phi_deg")) fail(child(path, "phi_deg"), planar_phi_message());
            check_keys(item, path, {"wavelength", "theta_deg"});
        }
        rq.points.push_back(read_point(item, path, azimuth));
    }
}

void read_backend(const Value& v) {
    const Value* backend = v.find("backend");
    if (!backend) return;
    const std::string name = text(*backend, "options.backend");
    if (name == "builtin") return;
    if (name != "mkl") fail("options.backend", "只能是 \"builtin\"（默认）或 \"mkl\"");
    fail("options.backend", "这个程序编译时没有编入 oneMKL 后端（STABLERCWA_WITH_MKL），不能用 \"mkl\"；请去掉这一项或写 \"builtin\"");
}

void read_common_options(const Value& v, Request& rq) {
    if (const Value* fast = v.find("homogeneous_fast_path"))
        if (!truth(*fast, "options.homogeneous_fast_path")) unsupported("options.homogeneous_fast_path", "homogeneous_fast_path = false");
    if (const Value* layers = v.find("parallel_layers")) (void)truth(*layers, "options.parallel_layers");
    if (const Value* diagnostics = v.find("diagnostics")) rq.diagnostics = truth(*diagnostics, "options.diagnostics");
    if (const Value* threads = v.find("threads")) {
        rq.threads = integer(*threads, "options.threads");
        if (rq.threads < 1 || rq.threads > kMaxThreads)
            fail("options.threads", "线程数应当在 1 到 " + std::to_string(kMaxThreads) + " 之间");
    }
}

void read_eig(const Value& v) {
    if (const Value* method = v.find("eig")) {
        const std::string name = text(*method, "options.eig");
        if (name == "lr") unsupported("options.eig", "LR 本征分解（\"lr\"）");
        if (name != "qr") fail("options.eig", "只能是 \"qr\" 或 \"lr\"");
    }
}

// rcwa_json.hpp:495-528
void read_options(const Value& v, Request& rq) {
    need_object(v, "options");
    check_keys(v, "options", {"backend", "eig", "linear", "homogeneous_fast_path", "parallel_layers", "diagnostics", "threads"});
    read_backend(v);
    read_eig(v);
    if (const Value* solver = v.find("linear")) {
        const std::string name = text(*solver, "options.linear");
        if (name == "lu_nopivot" || name == "qr") unsupported("options.linear", "\"" + name + "\" 线性求解");
        if (name != "lu") fail("options.linear", "只能是 \"lu\"、\"lu_nopivot\" 或 \"qr\"");
    }
    read_common_options(v, rq);
}

// rcwa_json.hpp:531-552
void read_input(const Value& v, Request& rq) {
    need_object(v, "input");
    check_keys(v, "input", {"psi_deg", "delta_deg", "jones"});
    if (const Value* jones = v.find("jones")) {
        if (v.contains("psi_deg") || v.contains("delta_deg")) fail("input", "入射偏振只能用一种写法：psi_deg（和 delta_deg），或者 jones");
        if (!jones->is_array() || jones->size() != 2) fail("input.jones", "应当是两个分量 [Es, Ep]（s 在前）");
        rq.Es = complex_number(jones->at(0), "input.jones[0]");
        rq.Ep = complex_number(jones->at(1), "input.jones[1]");
        const double norm = std::hypot(std::abs(rq.Es), std::abs(rq.Ep));
        if (!(norm > 0.0) || !std::isfinite(norm)) fail("input.jones", "入射 Jones 矢量不能是零矢量");
        rq.input = Input::Jones;
        return;
    }
    if (!v.contains("psi_deg")) fail("input.psi_deg", "缺少这一项（入射偏振写 psi_deg，或者改写 jones）");
    rq.psi_deg = number(*v.find("psi_deg"), "input.psi_deg");
    if (const Value* delta = v.find("delta_deg")) rq.delta_deg = number(*delta, "input.delta_deg");
    if (!std::isfinite(rq.psi_deg)) fail("input.psi_deg", "必须是有限的数");
    if (!std::isfinite(rq.delta_deg)) fail("input.delta_deg", "必须是有限的数");
    rq.input = Input::Angles;
}

// ---- periodic2d (rcwa_json.hpp:558-735)

std::vector<double> read_edge_numbers(const Value& v, const std::string& path) {
    need_array(v, path);
    std::vector<double> e;
    for (std::size_t j = 0; j < v.size(); ++j) e.push_back(number(v.at(j), child(path, j)));
    return e;
}
void check_edges_2d(const std::vector<double>& e, const std::string& path, double period, const char* name) {
    for (std::size_t j = 0; j < e.size(); ++j)
        if (!std::isfinite(e[j]) || (j > 0 && e[j] <= e[j - 1])) fail(child(path, j), "分段边界必须严格递增");
    if (std::abs((e.back() - e.front()) - period) > 1e-9 * period)
        fail(path, std::string("分段边界的首尾必须正好相差一个周期（stack.") + name + "）");
}

Layer2 read_layer_2d(const Value& v, const std::string& path, double Lx, double Ly) {
    need_object(v, path);
    check_keys(v, path, {"d", "n", "y_edges", "x_profiles"});
    Layer2 layer;
    layer.d = number(member(v, "d", path), child(path, "d"));
    if (!std::isfinite(layer.d) || layer.d < 0.0) fail(child(path, "d"), "层厚不能是负的");
    const Value* n = v.find("n");
    const Value* y_edges = v.find("y_edges");
    const Value* profiles = v.find("x_profiles");
    if (n && (y_edges || profiles)) fail(path, "均匀层只写 n，结构层只写 y_edges 和 x_profiles，两种写法不能混在一层里");
    if (!n && !y_edges && !profiles) fail(path, "缺少折射率：均匀层写 n，结构层写 y_edges 和 x_profiles");
    if (n) {
        layer.n = complex_number(*n, child(path, "n"));
        check_index(layer.n, child(path, "n"));
        return layer;
    }
    const std::string yp = child(path, "y_edges"), xp = child(path, "x_profiles");
    if (!y_edges) fail(yp, "结构层还要写 y_edges（y 方向的分段边界）");
    if (!profiles) fail(xp, "结构层还要写 x_profiles（每个 y 分段里沿 x 的折射率剖面）");
    layer.homogeneous = false;
    layer.y_edges = read_edge_numbers(*y_edges, yp);
    need_array(*profiles, xp);
    if (profiles->size() == 0 || layer.y_edges.size() != profiles->size() + 1)
        fail(xp, "段数对不上：K 个 x 剖面要配 K+1 个 y 边界（现在是 " + std::to_string(profiles->size()) + " 个 x 剖面、" +
                     std::to_string(layer.y_edges.size()) + " 个 y 边界）");
    check_edges_2d(layer.y_edges, yp, Ly, "Ly");
    for (std::size_t k = 0; k < profiles->size(); ++k) {
        const std::string rp = child(xp, k);
        const Value& item = profiles->at(k);
        need_object(item, rp);
        check_keys(item, rp, {"edges", "n_values"});
        const std::string ep = child(rp, "edges"), np = child(rp, "n_values");
        std::vector<double> e = read_edge_numbers(member(item, "edges", rp), ep);
        const Value& values = member(item, "n_values", rp);
        need_array(values, np);
        std::vector<cd> nv;
        for (std::size_t j = 0; j < values.size(); ++j) {
            nv.push_back(complex_number(values.at(j), child(np, j)));
            check_index(nv.back(), child(np, j));
        }
        if (nv.empty() || e.size() != nv.size() + 1)
            fail(np, "段数对不上：K 段折射率要配 K+1 个边界（现在是 " + std::to_string(nv.size()) + " 段折射率、" +
                         std::to_string(e.size()) + " 个边界）");
        check_edges_2d(e, ep, Lx, "Lx");
        layer.x_edges.push_back(std::move(e));
        layer.x_values.push_back(std::move(nv));
    }
    return layer;
}

Stack2 read_stack_2d(const Value& v) {
    need_object(v, "stack");
    if (v.contains("period")) fail("stack.period", "periodic2d 模式没有 period：x、y 方向的周期写成 Lx、Ly（period 是一维的写法）");
    check_keys(v, "stack", {"nI", "nII", "Lx", "Ly", "layers"});
    Stack2 s;
    const cd nI = complex_number(member(v, "nI", "stack"), "stack.nI");
    check_index(nI, "stack.nI");
    if (nI.imag() != 0.0 || nI.real() <= 0.0) fail("stack.nI", "入射介质必须无吸收，折射率是正实数");
    s.nI = nI.real();
    s.nII = complex_number(member(v, "nII", "stack"), "stack.nII");
    check_index(s.nII, "stack.nII");
    s.Lx = number(member(v, "Lx", "stack"), "stack.Lx");
    if (!std::isfinite(s.Lx) || s.Lx <= 0.0) fail("stack.Lx", "周期必须是正数");
    s.Ly = number(member(v, "Ly", "stack"), "stack.Ly");
    if (!std::isfinite(s.Ly) || s.Ly <= 0.0) fail("stack.Ly", "周期必须是正数");
    const Value& layers = member(v, "layers", "stack");
    need_array(layers, "stack.layers");
    for (std::size_t i = 0; i < layers.size(); ++i) s.layers.push_back(read_layer_2d(layers.at(i), child("stack.layers", i), s.Lx, s.Ly));
    return s;
}

void read_options_2d(const Value& v, Request& rq) {
    need_object(v, "options");
    if (v.contains("linear")) fail("options.linear", "二维不适用：二维求解没有 linear 选项（它是一维的线性求解器选项）");
    check_keys(v, "options", {"backend", "eig", "factorization", "homogeneous_fast_path", "parallel_layers", "diagnostics", "threads"});
    read_backend(v);
    read_eig(v);
    if (const Value* rule = v.find("factorization")) {
        const std::string name = text(*rule, "options.factorization");
        if (name == "li") rq.laurent = false;
        else if (name == "laurent") rq.laurent = true;
        else fail("options.factorization", "只能是 \"li\" 或 \"laurent\"");
    }
    read_common_options(v, rq);
}

void check_truncation_2d(int order, const char* name) {
    const long long max_order = (kMax2dHarmonics - 1) / 2;
    if (order < 0 || order > max_order)
        fail(name, std::string("截断阶数不能是负的，也不能超过 ") + std::to_string(max_order) + "（总谐波数 (2M+1)(2My+1) 不得超过 " +
                       std::to_string(kMax2dHarmonics) + "）");
}

Request read_request_2d(const Value& root) {
    Request rq;
    rq.mode = Mode::Periodic2D;
    if (root.contains("polarization"))
        fail("polarization", "periodic2d 模式不用 polarization：入射偏振写在 input 里（psi_deg、delta_deg 或 jones）");
    if (root.contains("period")) fail("period", "periodic2d 模式没有 period：x、y 方向的周期写成 stack.Lx、stack.Ly");
    check_keys(root, "", {"mode", "stack", "M", "My", "points", "wavelength", "theta_deg", "phi_deg", "input", "options"});
    rq.stack2d = read_stack_2d(member(root, "stack", ""));
    rq.M = integer(member(root, "M", ""), "M");
    check_truncation_2d(rq.M, "M");
    rq.My = integer(member(root, "My", ""), "My");
    check_truncation_2d(rq.My, "My");
    const long long harmonics = (2LL * rq.M + 1) * (2LL * rq.My + 1);
    if (harmonics > kMax2dHarmonics)
        fail("My", "总谐波数 N = (2M+1)(2My+1) = " + std::to_string(harmonics) + " 超过了上限 " + std::to_string(kMax2dHarmonics));
    read_points(root, rq);
    const Value* input = root.find("input");
    if (!input) fail("input", "缺少这一项：二维必须指定入射偏振，写 psi_deg（和 delta_deg），或者 jones");
    read_input(*input, rq);
    if (rq.input == Input::Angles) {  // jones_from_angles_2d (include/stablercwa/rcwa2d_types.hpp:104-107)
        const double psi = rq.psi_deg * kPi / 180.0, delta = rq.delta_deg * kPi / 180.0;
        rq.Es = std::sin(psi) * std::exp(cd{0.0, 1.0} * delta);
        rq.Ep = cd{std::cos(psi), 0.0};
    }
    if (const Value* options = root.find("options")) read_options_2d(*options, rq);
    return rq;
}

// rcwa_json.hpp:739-800
Request read_request(const Value& root) {
    if (!root.is_object()) fail("", "请求的最外层应当是一个对象 {…}");
    Request rq;
    const std::string mode = text(member(root, "mode", ""), "mode");
    if (mode == "conical") rq.mode = Mode::Conical;
    else if (mode == "periodic2d") return read_request_2d(root);
    else if (mode != "planar")
        fail("mode", "只能是 \"planar\"（平面内入射，TE 或 TM）、\"conical\"（圆锥入射）或 \"periodic2d\"（二维交叉光栅）");
    const bool conical = rq.mode == Mode::Conical;
    if (conical) {
        if (root.contains("polarization"))
            fail("polarization", "conical 模式不用 polarization：入射偏振写在 input 里；不写 input 时给出各级的 Jones 矩阵");
        check_keys(root, "", {"mode", "stack", "M", "points", "wavelength", "theta_deg", "phi_deg", "input", "options"});
    } else {
        if (root.contains("phi_deg")) fail("phi_deg", planar_phi_message());
        if (root.contains("input")) fail("input", "planar 模式的入射偏振由 polarization 指定；input 只用于 conical 模式");
        check_keys(root, "", {"mode", "stack", "M", "polarization", "points", "wavelength", "theta_deg", "options"});
    }
    rq.stack = read_stack(member(root, "stack", ""), conical);
    rq.M = integer(member(root, "M", ""), "M");
    const int max_order = (kMaxMatrixOrder / (conical ? 2 : 1) - 1) / 2;
    if (rq.M < 0 || rq.M > max_order)
        fail("M", "截断阶数不能是负的，也不能超过 " + std::to_string(max_order) + "（再大，单个稠密矩阵就超过 4 GiB）");
    for (std::size_t j = 0; j < rq.stack.layers.size(); ++j) {
        const Layer1& L = rq.stack.layers[j];
        if (!L.homogeneous && L.fourier_method == 1)
            check_fft_samples(rq.M, L.fft_samples, child(child("stack.layers", j), "fft_samples"));
    }
    if (!conical) {
        const std::string name = text(member(root, "polarization", ""), "polarization");
        if (name == "TE") rq.polarization = RCWA_TE;
        else if (name == "TM") rq.polarization = RCWA_TM;
        else fail("polarization", "只能是 \"TE\" 或 \"TM\"");
    }
    read_points(root, rq);
    if (conical)
        if (const Value* input = root.find("input")) read_input(*input, rq);
    if (const Value* options = root.find("options")) read_options(*options, rq);
    return rq;
}

Request parse_request(const std::string& request) {
    Value root;
    try {
        root = jtext::parse(request);
    } catch (const jtext::ParseError& e) {
        fail("", "请求不是合法的 JSON（第 " + std::to_string(e.line) + " 行第 " + std::to_string(e.column) + " 列，字节偏移 " +
                     std::to_string(e.offset) + "）：" + e.reason);
    }
    return read_request(root);
}

// ------------------------------------------------------------------ C structs of the request

struct Marshal1 {
    std::vector<std::vector<rcwa_complex>> values;
    std::vector<rcwa_layer1d> layers;
    rcwa_stack1d st{};
    explicit Marshal1(const Stack1& s) {
        for (const Layer1& L : s.layers) {
            values.emplace_back();
            for (const cd& z : L.values) values.back().push_back({z.real(), z.imag()});
        }
        for (std::size_t k = 0; k < s.layers.size(); ++k) {
            const Layer1& L = s.layers[k];
            rcwa_layer1d l{};
            l.d = L.d;
            l.homogeneous = L.homogeneous ? 1 : 0;
            l.n = {L.n.real(), L.n.imag()};
            l.n_segments = static_cast<int>(L.values.size());
            l.edges = L.edges.empty() ? nullptr : L.edges.data();
            l.n_values = values[k].empty() ? nullptr : values[k].data();
            l.fourier_method = L.fourier_method;
            l.fft_samples = L.fft_samples;
            layers.push_back(l);
        }
        st.nI = {s.nI.real(), s.nI.imag()};
        st.nII = {s.nII.real(), s.nII.imag()};
        st.period = s.period;
        st.n_layers = static_cast<int>(layers.size());
        st.layers = layers.empty() ? nullptr : layers.data();
    }
};

struct Marshal2 {
    std::vector<std::vector<std::vector<rcwa_complex>>> values;
    std::vector<std::vector<rcwa_xprofile2d>> rows;
    std::vector<rcwa_layer2d> layers;
    rcwa_stack2d st{};
    explicit Marshal2(const Stack2& s) {
        for (const Layer2& L : s.layers) {
            values.emplace_back();
            for (const auto& row : L.x_values) {
                values.back().emplace_back();
                for (const cd& z : row) values.back().back().push_back({z.real(), z.imag()});
            }
        }
        for (std::size_t k = 0; k < s.layers.size(); ++k) {
            rows.emplace_back();
            const Layer2& L = s.layers[k];
            for (std::size_t r = 0; r < L.x_values.size(); ++r)
                rows.back().push_back({static_cast<int>(L.x_values[r].size()), L.x_edges[r].data(), values[k][r].data()});
        }
        for (std::size_t k = 0; k < s.layers.size(); ++k) {
            const Layer2& L = s.layers[k];
            rcwa_layer2d l{};
            l.d = L.d;
            l.homogeneous = L.homogeneous ? 1 : 0;
            l.n = {L.n.real(), L.n.imag()};
            l.n_strips = static_cast<int>(L.x_values.size());
            l.y_edges = L.y_edges.empty() ? nullptr : L.y_edges.data();
            l.x_profiles = rows[k].empty() ? nullptr : rows[k].data();
            layers.push_back(l);
        }
        st.nI = s.nI;
        st.nII = {s.nII.real(), s.nII.imag()};
        st.Lx = s.Lx;
        st.Ly = s.Ly;
        st.n_layers = static_cast<int>(layers.size());
        st.layers = layers.empty() ? nullptr : layers.data();
    }
};

// ------------------------------------------------------------------ results of every point

struct Planar {
    std::vector<rcwa_complex> R, T;
    std::vector<double> DEr, DEt, resid;
    std::vector<int> status, info, neig, nsolve;
    rcwa_result1d view(std::size_t p, int n) {
        return rcwa_result1d{&R[p * n], &T[p * n], &DEr[p * n], &DEt[p * n], &status[p], &info[p], &neig[p], &nsolve[p], &resid[p]};
    }
    Planar(std::size_t P, int n) : R(P * n), T(P * n), DEr(P * n), DEt(P * n), resid(P), status(P), info(P), neig(P), nsolve(P) {}
};
struct Conical {
    std::vector<rcwa_complex> Jr, Jt;
    std::vector<double> DEr, DEt, minl, kx, ky, fr, ft;
    std::vector<int> status, info, neig, nsolve, nschur, warn;
    rcwa_result_conical view(std::size_t p, int n) {
        return rcwa_result_conical{&Jr[p * n * 4], &Jt[p * n * 4], &DEr[p * n * 4], &DEt[p * n * 4], &status[p], &info[p], &neig[p],
                                   &nsolve[p], &nschur[p], &minl[p], &warn[p], &kx[p * n], &ky[p], &fr[p * n], &ft[p * n]};
    }
    Conical(std::size_t P, int n)
        : Jr(P * n * 4), Jt(P * n * 4), DEr(P * n * 4), DEt(P * n * 4), minl(P), kx(P * n), ky(P), fr(P * n), ft(P * n), status(P),
          info(P), neig(P), nsolve(P), nschur(P), warn(P) {}
};
struct Grid2 {
    std::vector<double> Kx, Ky, DEr, DEt, resid;
    std::vector<rcwa_complex> kzI, kzII, Ex_r, Ey_r, Ez_r, Ex_t, Ey_t, Ez_t, Rs, Rp, Ts, Tp;
    std::vector<unsigned char> prop_r, prop_t, regions;
    std::vector<int> status, info, neig, nsolve;
    int regions_per = 0;
    rcwa_result2d view(std::size_t p, int N) {
        rcwa_result2d r{};
        r.Kx = &Kx[p * N];
        r.Ky = &Ky[p * N];
        r.kzI = &kzI[p * N];
        r.kzII = &kzII[p * N];
        r.Ex_r = &Ex_r[p * N];
        r.Ey_r = &Ey_r[p * N];
        r.Ez_r = &Ez_r[p * N];
        r.Ex_t = &Ex_t[p * N];
        r.Ey_t = &Ey_t[p * N];
        r.Ez_t = &Ez_t[p * N];
        r.Rs = &Rs[p * N];
        r.Rp = &Rp[p * N];
        r.Ts = &Ts[p * N];
        r.Tp = &Tp[p * N];
        r.DEr = &DEr[p * N];
        r.DEt = &DEt[p * N];
        r.prop_r = &prop_r[p * N];
        r.prop_t = &prop_t[p * N];
        r.status = &status[p];
        r.eig_info = &info[p];
        r.n_eig = &neig[p];
        r.n_dense_solve = &nsolve[p];
        r.max_eig_residual = &resid[p];
        r.rayleigh_regions = &regions[p * regions_per];
        return r;
    }
    Grid2(std::size_t P, int N, int n_layers)
        : Kx(P * N), Ky(P * N), DEr(P * N), DEt(P * N), resid(P), kzI(P * N), kzII(P * N), Ex_r(P * N), Ey_r(P * N), Ez_r(P * N),
          Ex_t(P * N), Ey_t(P * N), Ez_t(P * N), Rs(P * N), Rp(P * N), Ts(P * N), Tp(P * N), prop_r(P * N), prop_t(P * N),
          regions(P * (n_layers + 2)), status(P), info(P), neig(P), nsolve(P), regions_per(n_layers + 2) {}
};

// Where the solves run: one batched call on a context, or one request per point on the serving loop.
struct Runner {
    rcwa_gpu_ctx* ctx = nullptr;
    rcwa_gpu_server* server = nullptr;
    std::vector<double> seconds;  // per point

    [[noreturn]] void engine_error(int rc) const {
        std::string message;
        if (ctx) {
            char buf[1024] = "";
            rcwa_gpu_last_error(ctx, buf, sizeof buf);
            message = buf;
        }
        if (rc == RCWA_EINVAL) fail("", "求解器不接受这组参数：" + message);
        if (rc == RCWA_ENOMEM) fail("M", "内存不够：截断阶数 M 太大");
        fail("", "求解时出错：rcwa_gb300 error " + std::to_string(rc) + (message.empty() ? "" : "：" + message));
    }

    template <class Batch, class Submit>
    void run(std::size_t P, Batch&& batch, Submit&& request_of) {
        seconds.assign(P, 0.0);
        if (ctx) {
            const auto t0 = std::chrono::steady_clock::now();
            const int rc = batch();
            if (rc != RCWA_OK) engine_error(rc);
            const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            for (double& s : seconds) s = wall / static_cast<double>(P);
            return;
        }
        std::vector<unsigned long long> tickets(P);
        for (std::size_t p = 0; p < P; ++p) {
            const rcwa_request rq = request_of(p);
            const int rc = rcwa_gpu_server_submit(server, &rq, &tickets[p]);
            if (rc != RCWA_OK) {
                for (std::size_t q = 0; q < p; ++q) rcwa_gpu_server_wait(server, tickets[q], -1, nullptr, nullptr);
                engine_error(rc);
            }
        }
        int first_error = RCWA_OK;
        for (std::size_t p = 0; p < P; ++p) {
            rcwa_response resp{};
            request_of.collect(p, tickets[p], resp);
            if (resp.code != RCWA_OK && first_error == RCWA_OK) first_error = resp.code;
            seconds[p] = resp.finish_s - resp.start_s;
        }
        if (first_error != RCWA_OK) engine_error(first_error);
    }
};

// ------------------------------------------------------------------ reply

void write_complex_array(Writer& w, const rcwa_complex* v, std::size_t n) {
    w.begin_array(true);
    for (std::size_t j = 0; j < n; ++j) w.complex(v[j].re, v[j].im);
    w.end_array();
}
void write_complex_array(Writer& w, const std::vector<cd>& v) {
    w.begin_array(true);
    for (const cd& z : v) w.complex(z.real(), z.imag());
    w.end_array();
}
void write_real_array(Writer& w, const double* v, std::size_t n) {
    w.begin_array(true);
    for (std::size_t j = 0; j < n; ++j) w.value(v[j]);
    w.end_array();
}

void write_head(Writer& w, const Request& rq) {
    w.begin_object();
    w.key("ok");
    w.value(true);
    w.key("version");
    w.value(kVersion);
    w.key("mode");
    w.value(rq.mode == Mode::Periodic2D ? "periodic2d" : rq.mode == Mode::Conical ? "conical" : "planar");
    w.key("M");
    w.value(rq.M);
    if (rq.mode == Mode::Periodic2D) {
        w.key("My");
        w.value(rq.My);
        w.key("orders");
        w.begin_array(true);
        for (int m = -rq.M; m <= rq.M; ++m)
            for (int n = -rq.My; n <= rq.My; ++n) {
                w.begin_array(true);
                w.value(m);
                w.value(n);
                w.end_array();
            }
        w.end_array();
    } else {
        w.key("orders");
        w.begin_array(true);
        for (int m = -rq.M; m <= rq.M; ++m) w.value(m);
        w.end_array();
    }
    w.key("threads");
    w.value(rq.threads > 0 ? rq.threads : 1);
    w.key("results");
    w.begin_array();
}

// eig_info .. timing (rcwa_json.hpp:930-957); timing: the point's share of the run
void write_bookkeeping(Writer& w, int info, int neig, int nsolve, double resid, double seconds) {
    w.key("eig_info");
    w.value(info);
    w.key("n_eig");
    w.value(neig);
    w.key("n_dense_solve");
    w.value(nsolve);
    w.key("max_eig_residual");
    w.value(resid);
    w.key("max_solve_backward_error");
    w.value(0.0);
    w.key("timing");
    w.begin_object(true);
    w.key("total");
    w.value(seconds);
    w.key("eig");
    w.value(0.0);
    w.key("linear");
    w.value(0.0);
    w.key("product");
    w.value(0.0);
    w.end_object();
}

double sum(const double* v, std::size_t n) {
    double s = 0.0;
    for (std::size_t j = 0; j < n; ++j) s += v[j];
    return s;
}

// ------------------------------------------------------------------ near-field protocol (rcwa_fields_json.hpp)
//
// {"solve": <one-point request>, "sampling": {...}, "output_dir": "...", "request_id": "..."}: the one point is
// solved with its fields, the x-z map (1-D: nx points at y) or the x-z / y-z slice (2-D: nt points at `at`)
// is formed on the device at the requested depths, with its absolute and incident-referenced phase maps
// (floor 1e-6, no unwrapping), and written as NPY files into a new directory published by one rename.

constexpr std::size_t kFieldsMaxSamples = 4000000;

struct FieldsRequest {
    Request solve;
    std::vector<double> z;
    int nx = 0, nt = 0;
    double y = 0.0, at = 0.0;
    int plane = RCWA_SLICE_XZ;
    std::filesystem::path output_dir;
    std::string id;
};

struct FieldsJob {
    const FieldsRequest* fr = nullptr;
    std::vector<rcwa_complex> harmonics;  // 6 x n x nz
    std::vector<int> layer_info;          // per layer (1-D and conical)
    double solve_seconds = 0.0;
};

// rcwa_fields_json.hpp:68-151
FieldsRequest read_fields_request(const Value& root) {
    need_object(root, "");
    check_keys(root, "", {"solve", "sampling", "output_dir", "request_id"});
    FieldsRequest fr;
    fr.solve = read_request(member(root, "solve", ""));
    if (fr.solve.points.size() != 1) fail("solve.points", "fields 协议每次只接受一个入射点");
    if (fr.solve.mode == Mode::Conical && fr.solve.input == Input::None)
        fail("solve.input", "圆锥场采样必须指定入射 Jones 或偏振角");
    const Value& sampling = member(root, "sampling", "");
    need_object(sampling, "sampling");
    if (fr.solve.mode == Mode::Periodic2D) {
        check_keys(sampling, "sampling", {"z", "plane", "nt", "at"});
        const std::string plane = text(member(sampling, "plane", "sampling"), "sampling.plane");
        if (plane == "xz") fr.plane = RCWA_SLICE_XZ;
        else if (plane == "yz") fr.plane = RCWA_SLICE_YZ;
        else fail("sampling.plane", "只能是 \"xz\"（固定 y，沿 x）或 \"yz\"（固定 x，沿 y）");
        fr.nt = integer(member(sampling, "nt", "sampling"), "sampling.nt");
        if (fr.nt < 1) fail("sampling.nt", "必须是正整数");
        const Value& depths = member(sampling, "z", "sampling");
        need_array(depths, "sampling.z");
        if (depths.size() == 0 || depths.size() > kFieldsMaxSamples / static_cast<std::size_t>(fr.nt))
            fail("sampling", "采样网格为空或超过 4000000 个点");
        for (std::size_t j = 0; j < depths.size(); ++j) {
            fr.z.push_back(number(depths.at(j), child("sampling.z", j)));
            if (!std::isfinite(fr.z.back())) fail(child("sampling.z", j), "必须是有限的数");
        }
        if (const Value* at = sampling.find("at")) {
            fr.at = number(*at, "sampling.at");
            if (!std::isfinite(fr.at)) fail("sampling.at", "必须是有限的数");
        }
    } else {
        check_keys(sampling, "sampling", {"z", "nx", "y"});
        fr.nx = integer(member(sampling, "nx", "sampling"), "sampling.nx");
        if (fr.nx < 1) fail("sampling.nx", "必须是正整数");
        const Value& depths = member(sampling, "z", "sampling");
        need_array(depths, "sampling.z");
        if (depths.size() == 0 || depths.size() > kFieldsMaxSamples / static_cast<std::size_t>(fr.nx))
            fail("sampling", "采样网格为空或超过 4000000 个点");
        for (std::size_t j = 0; j < depths.size(); ++j) fr.z.push_back(number(depths.at(j), child("sampling.z", j)));
        if (const Value* y = sampling.find("y")) fr.y = number(*y, "sampling.y");
        if (fr.solve.mode != Mode::Conical && fr.y != 0.0) fail("sampling.y", "planar 场采样的 y 必须是 0");
    }
    const std::string path = text(member(root, "output_dir", ""), "output_dir");
    if (path.empty() || path.find('\0') != std::string::npos) fail("output_dir", "输出目录不能为空或含 NUL");
    fr.output_dir = std::filesystem::absolute(std::filesystem::u8path(path)).lexically_normal();
    if (fr.output_dir.filename().empty()) fail("output_dir", "必须是本次新建的子目录");
    fr.id = text(member(root, "request_id", ""), "request_id");
    if (fr.id.empty() || fr.id.size() > 128) fail("request_id", "必须是 1 到 128 字节的本次请求标记");
    return fr;
}

// A temporary sibling directory, renamed onto the requested one when everything is written; removed otherwise.
class DirectoryOutput {
public:
    explicit DirectoryOutput(const std::filesystem::path& final_path) : final_(final_path) {
        namespace fs = std::filesystem;
        if (fs::exists(final_)) throw std::invalid_argument("fields 输出目录已存在，拒绝覆盖历史文件");
        if (!fs::is_directory(final_.parent_path())) throw std::invalid_argument("fields 输出目录的父目录不存在");
        std::random_device random;
        for (int attempt = 0; attempt < 20; ++attempt) {
            temporary_ = final_.parent_path() /
                         fs::u8path(final_.filename().u8string() + ".tmp-" + std::to_string(random()) + "-" + std::to_string(random()));
            if (fs::create_directory(temporary_)) {
                owned_ = true;
                return;
            }
        }
        throw std::runtime_error("fields 不能建立临时输出目录");
    }
    ~DirectoryOutput() {
        if (owned_) {
            std::error_code ignored;
            std::filesystem::remove_all(temporary_, ignored);
        }
    }
    DirectoryOutput(const DirectoryOutput&) = delete;
    DirectoryOutput& operator=(const DirectoryOutput&) = delete;
    std::filesystem::path file(const char* name) const { return temporary_ / name; }
    void publish() {
        if (std::filesystem::exists(final_)) throw std::runtime_error("fields 输出目录在发布前已存在");
        std::filesystem::rename(temporary_, final_);
        owned_ = false;
    }

private:
    std::filesystem::path final_, temporary_;
    bool owned_ = false;
};

// NPY version 1.0: magic, header length, the dict padded so the data starts on a 64-byte boundary, then the
// little-endian data in C order.
void write_npy(const std::filesystem::path& path, const char* dtype, const std::vector<std::size_t>& shape, const void* data,
               std::size_t bytes) {
    std::string tuple = "(";
    for (std::size_t d : shape) tuple += std::to_string(d) + ", ";
    tuple += ")";
    std::string header = std::string("{'descr': '") + dtype + "', 'fortran_order': False, 'shape': " + tuple + ", }";
    header.append((64 - (10 + header.size() + 1) % 64) % 64, ' ');
    header += '\n';
    const unsigned char prefix[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, static_cast<unsigned char>(header.size() & 255),
                                      static_cast<unsigned char>(header.size() >> 8)};
    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    if (!out) throw std::runtime_error("NPY: cannot create output file");
    out.write(reinterpret_cast<const char*>(prefix), sizeof prefix);
    out.write(header.data(), static_cast<std::streamsize>(header.size()));
    out.write(static_cast<const char*>(data), static_cast<std::streamsize>(bytes));  // the supported hosts (x86-64, aarch64) are little-endian
    out.close();
    if (!out) throw std::runtime_error("NPY: writing output failed");
}

void write_shape(Writer& w, const std::vector<std::size_t>& shape) {
    w.begin_array(true);
    for (std::size_t d : shape) w.value(static_cast<long long>(d));
    w.end_array();
}
void write_file(Writer& w, const char* key, const char* name, const char* dtype, const std::vector<std::size_t>& shape) {
    w.key(key);
    w.begin_object(true);
    w.key("name");
    w.value(name);
    w.key("dtype");
    w.value(dtype);
    w.key("shape");
    write_shape(w, shape);
    w.end_object();
}

// Everything after the far-field result: slice, phases, files, manifest (rcwa_fields_json.hpp:156-301, :303-459).
// kx, ky: the physical wavevector of each harmonic; kinc: real (kx, ky, kz) of the incident order; layers:
// (original index, effective index, z_top, z_bottom, finite-zero modes, Schur) per stack layer.
struct LayerRow {
    long long original;
    int effective;
    double z_top, z_bottom;
    int finite_zero;
    bool schur;
};
void fields_tail(Writer& w, rcwa_gpu_ctx* ctx, FieldsJob& fj, const std::vector<double>& kx, const std::vector<double>& ky,
                 const double kinc[3], double period, double norm_E, double norm_H, const std::vector<LayerRow>& layers) {
    using Clock = std::chrono::steady_clock;
    const FieldsRequest& fr = *fj.fr;
    const bool two_d = fr.solve.mode == Mode::Periodic2D;
    const int n = static_cast<int>(kx.size()), nz = static_cast<int>(fr.z.size());
    const int nt = two_d ? fr.nt : fr.nx;
    const int plane = two_d ? fr.plane : RCWA_SLICE_XZ;
    const double at = two_d ? fr.at : fr.y;
    DirectoryOutput output(fr.output_dir);
    auto started = Clock::now();
    std::vector<rcwa_complex> grid((std::size_t)6 * nz * nt);
    int rc = rcwa_gpu_field_slice(ctx, fj.harmonics.data(), n, nz, kx.data(), ky.data(), plane, nt, period, at, grid.data());
    if (rc == RCWA_ENUMERIC) throw std::runtime_error("fields 采样产生非有限复场，拒绝发布");
    if (rc != RCWA_OK) throw std::runtime_error("fields 采样失败：rcwa_gb300 error " + std::to_string(rc));
    for (const rcwa_complex& v : grid)
        if (!std::isfinite(v.re) || !std::isfinite(v.im)) throw std::runtime_error("fields 采样产生非有限复场，拒绝发布");
    const double sample_seconds = std::chrono::duration<double>(Clock::now() - started).count();
    std::vector<double> t(nt), x(nt), y(nt);
    for (int it = 0; it < nt; ++it) {
        t[it] = (static_cast<double>(it) / nt) * period;
        x[it] = plane == RCWA_SLICE_XZ ? t[it] : at;
        y[it] = plane == RCWA_SLICE_XZ ? at : t[it];
    }
    const std::size_t plane_size = static_cast<std::size_t>(nz) * nt;
    std::vector<double> phase(2 * 6 * plane_size), amplitude(plane_size);
    std::vector<unsigned char> mask(2 * 6 * plane_size);
    started = Clock::now();
    for (int reference = 0; reference < 2; ++reference)
        for (int c = 0; c < 6; ++c) {
            const std::size_t off = (static_cast<std::size_t>(reference) * 6 + c) * plane_size;
            rc = rcwa_gpu_phase_data(ctx, &grid[c * plane_size], nt, nz, reference == 0 ? RCWA_PHASE_ABSOLUTE : RCWA_PHASE_INCIDENT,
                                     kinc, x.data(), y.data(), fr.z.data(), nullptr, 1e-6, RCWA_UNWRAP_NONE, &phase[off],
                                     amplitude.data(), &mask[off], nullptr);
            if (rc != RCWA_OK) throw std::runtime_error("fields 相位计算失败：rcwa_gb300 error " + std::to_string(rc));
        }
    const double phase_seconds = std::chrono::duration<double>(Clock::now() - started).count();
    started = Clock::now();
    const std::size_t sz = static_cast<std::size_t>(nz), snt = static_cast<std::size_t>(nt);
    write_npy(output.file("fields.npy"), "<c16", {6, sz, snt}, grid.data(), grid.size() * sizeof(rcwa_complex));
    write_npy(output.file("phase.npy"), "<f8", {2, 6, sz, snt}, phase.data(), phase.size() * sizeof(double));
    write_npy(output.file("phase_mask.npy"), "|u1", {2, 6, sz, snt}, mask.data(), mask.size());
    if (two_d) {
        write_npy(output.file("t.npy"), "<f8", {snt}, t.data(), snt * sizeof(double));
        write_npy(output.file("x.npy"), "<f8", {snt}, x.data(), snt * sizeof(double));
        write_npy(output.file("y.npy"), "<f8", {snt}, y.data(), snt * sizeof(double));
    } else {
        write_npy(output.file("x.npy"), "<f8", {snt}, x.data(), snt * sizeof(double));
    }
    write_npy(output.file("z.npy"), "<f8", {sz}, fr.z.data(), sz * sizeof(double));
    const double write_seconds = std::chrono::duration<double>(Clock::now() - started).count();

    w.key("protocol");
    w.value("stablercwa-fields");
    w.key("field_data");
    w.begin_object();
    w.key("version");
    w.value(1);
    w.key("producer");
    w.value("stablercwa.cpp.rcwa_fields");
    w.key("request_id");
    w.value(fr.id);
    w.key("directory");
    w.value(fr.output_dir.u8string());
    w.key("layout");
    w.value("C");
    w.key("shape");
    write_shape(w, {sz, snt});
    w.key("components");
    w.begin_array(true);
    for (const char* name : {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"}) w.value(name);
    w.end_array();
    if (two_d) {
        w.key("slice");
        w.begin_object(true);
        w.key("plane");
        w.value(plane == RCWA_SLICE_XZ ? "xz" : "yz");
        w.key("at");
        w.value(at);
        w.key("period");
        w.value(period);
        w.end_object();
        w.key("harmonics");
        w.begin_object(true);
        w.key("M");
        w.value(fr.solve.M);
        w.key("My");
        w.value(fr.solve.My);
        w.key("N");
        w.value(static_cast<long long>(n));
        w.end_object();
    } else {
        w.key("y");
        w.value(fr.y);
    }
    w.key("phase");
    w.begin_object(true);
    w.key("references");
    w.begin_array(true);
    w.value("absolute");
    w.value("incident");
    w.end_array();
    w.key("floor");
    w.value(1e-6);
    w.key("unwrap");
    w.value("none");
    w.key("unit");
    w.value("rad");
    w.key("mask_true");
    w.value("undefined");
    w.end_object();
    w.key("normalization");
    w.begin_object(true);
    w.key("E");
    w.value(norm_E);
    w.key("H");
    w.value(norm_H);
    w.key("H_convention");
    w.value("Z0 H_physical");
    w.end_object();
    w.key("files");
    w.begin_object();
    write_file(w, "fields", "fields.npy", "<c16", {6, sz, snt});
    write_file(w, "phase", "phase.npy", "<f8", {2, 6, sz, snt});
    write_file(w, "phase_mask", "phase_mask.npy", "|u1", {2, 6, sz, snt});
    if (two_d) {
        write_file(w, "t", "t.npy", "<f8", {snt});
        write_file(w, "x", "x.npy", "<f8", {snt});
        write_file(w, "y", "y.npy", "<f8", {snt});
    } else {
        write_file(w, "x", "x.npy", "<f8", {snt});
    }
    write_file(w, "z", "z.npy", "<f8", {sz});
    w.end_object();
    w.key("layers");
    w.begin_array();
    for (const LayerRow& L : layers) {
        w.begin_object(true);
        w.key("original_index");
        w.value(L.original);
        w.key("effective_index");
        w.value(L.effective);
        w.key("z_top");
        w.value(L.z_top);
        w.key("z_bottom");
        w.value(L.z_bottom);
        w.key("finite_zero_modes");
        w.value(L.finite_zero);
        w.key("schur");
        w.value(L.schur);
        w.end_object();
    }
    w.end_array();
    w.key("timing");
    w.begin_object(true);
    w.key("solve");
    w.value(fj.solve_seconds);
    w.key("sample");
    w.value(sample_seconds);
    w.key("phase");
    w.value(phase_seconds);
    w.key("write");
    w.value(write_seconds);
    w.end_object();
    w.end_object();
    w.end_object();
    output.publish();
}

// z_top / z_bottom per stack layer, effective indices skipping zero thickness when skip_zero
template <class Layers>
std::vector<LayerRow> layer_rows(const Layers& layers, bool skip_zero, const std::vector<int>& info, bool info_is_schur) {
    std::vector<LayerRow> rows;
    double z = 0.0;
    int effective = 0;
    for (std::size_t j = 0; j < layers.size(); ++j) {
        LayerRow r{};
        r.original = static_cast<long long>(j);
        r.effective = skip_zero && layers[j].d == 0.0 ? -1 : effective++;
        r.z_top = z;
        z += layers[j].d;
        r.z_bottom = z;
        const int v = j < info.size() ? info[j] : 0;
        r.finite_zero = info_is_schur ? 0 : v;
        r.schur = info_is_schur && v != 0;
        rows.push_back(r);
    }
    return rows;
}

std::string run_planar(const Request& rq, Runner& run, int indent, FieldsJob* fj = nullptr) {
    const int n = 2 * rq.M + 1;
    const std::size_t P = rq.points.size();
    Marshal1 m(rq.stack);
    Planar res(P, n);
    rcwa_options o;
    rcwa_options_default(&o);
    o.diagnostics = rq.diagnostics ? 1 : 0;
    std::vector<rcwa_point1d> pts(P);
    for (std::size_t p = 0; p < P; ++p) pts[p] = {rq.points[p].wavelength, rq.points[p].theta_deg};
    struct Req {
        const Request& rq;
        Marshal1& m;
        Planar& res;
        const rcwa_options& o;
        int n;
        rcwa_request operator()(std::size_t p) const {
            rcwa_request r{};
            r.kind = RCWA_REQ_1D;
            r.stack1d = &m.st;
            r.wavelength = rq.points[p].wavelength;
            r.theta_deg = rq.points[p].theta_deg;
            r.M = rq.M;
            r.polarization = rq.polarization;
            r.options = o;
            return r;
        }
        rcwa_gpu_server* server = nullptr;
        void collect(std::size_t p, unsigned long long t, rcwa_response& resp) const {
            rcwa_result1d v = res.view(p, n);
            rcwa_gpu_server_wait(server, t, -1, &resp, &v);
        }
    } req{rq, m, res, o, n, run.server};
    run.run(P, [&] {
        rcwa_result1d v = res.view(0, n);
        if (fj) {  // one point with its fields at the requested depths
            const int nz = static_cast<int>(fj->fr->z.size());
            fj->harmonics.resize((std::size_t)6 * n * nz);
            fj->layer_info.assign(std::max<std::size_t>(1, rq.stack.layers.size()), 0);
            return rcwa_gpu_solve1d_fields(run.ctx, &m.st, pts.data(), 1, rq.M, rq.polarization, &o, fj->fr->z.data(), nz, &v,
                                           fj->harmonics.data(), fj->layer_info.data());
        }
        return rcwa_gpu_solve1d_batch(run.ctx, &m.st, pts.data(), static_cast<int>(P), rq.M, rq.polarization, &o, &v);
    }, req);
    if (fj && res.status[0] != RCWA_SAMPLE_OK) throw std::logic_error("rcwa: planar field context is unavailable");
    Writer w(indent);
    write_head(w, rq);
    for (std::size_t p = 0; p < P; ++p) {
        w.begin_object();
        w.key("wavelength");
        w.value(rq.points[p].wavelength);
        w.key("theta_deg");
        w.value(rq.points[p].theta_deg);
        w.key("R");
        write_complex_array(w, &res.R[p * n], n);
        w.key("T");
        write_complex_array(w, &res.T[p * n], n);
        w.key("DEr");
        write_real_array(w, &res.DEr[p * n], n);
        w.key("DEt");
        write_real_array(w, &res.DEt[p * n], n);
        w.key("R_total");
        w.value(sum(&res.DEr[p * n], n));
        w.key("T_total");
        w.value(sum(&res.DEt[p * n], n));
        write_bookkeeping(w, res.info[p], res.neig[p], res.nsolve[p], rq.diagnostics ? res.resid[p] : 0.0, run.seconds[p]);
        w.end_object();
    }
    w.end_array();
    if (fj) {
        // metadata of the planar fields (rcwa1d_fields.hpp:55-103): kxm = k0 kx, ky = 0, kzI from the incident mode
        const PointSpec& pt = rq.points[0];
        const double k0 = 2.0 * kPi / pt.wavelength, nI = rq.stack.nI.real();
        const double s0 = nI * std::sin(pt.theta_deg * kPi / 180.0);
        std::vector<double> kx(n), ky(n, 0.0);
        for (int j = 0; j < n; ++j) kx[j] = k0 * (s0 - (j - rq.M) * pt.wavelength / rq.stack.period);
        const double kinc[3] = {kx[rq.M], 0.0, k0 * std::sqrt((nI - s0) * (nI + s0))};
        const bool te = rq.polarization == RCWA_TE;
        fj->solve_seconds = run.seconds[0];
        fields_tail(w, run.ctx, *fj, kx, ky, kinc, rq.stack.period, te ? 1.0 : 1.0 / nI, te ? nI : 1.0,
                    layer_rows(rq.stack.layers, false, fj->layer_info, false));
        return w.take();
    }
    w.end_object();
    return w.take();
}

// kz of a homogeneous medium for the conical orders (rcwa1d_conical.hpp:195-203, :251-258)
cd longitudinal(cd n, double kx, double ky) {
    const cd z = n * n - kx * kx - ky * ky;
    if (z.imag() == 0.0) return z.real() >= 0.0 ? cd{std::sqrt(z.real()), 0.0} : cd{0.0, std::sqrt(-z.real())};
    cd kz = std::sqrt(z);
    if (kz.imag() < 0.0) kz = -kz;
    if (std::abs(kz.imag()) < 1e-12 && kz.real() < 0.0) kz = -kz;
    return kz;
}
cd longitudinal0(cd n, double nI, double cosine) {
    const cd z = (n - nI) * (n + nI) + (nI * cosine) * (nI * cosine);
    if (z.imag() == 0.0) return z.real() >= 0.0 ? cd{std::sqrt(z.real()), 0.0} : cd{0.0, std::sqrt(-z.real())};
    cd kz = std::sqrt(z);
    if (kz.imag() < 0.0) kz = -kz;
    if (std::abs(kz.imag()) < 1e-12 && kz.real() < 0.0) kz = -kz;
    return kz;
}

std::string run_conical(const Request& rq, Runner& run, int indent, FieldsJob* fj = nullptr) {
    const int n = 2 * rq.M + 1;
    const std::size_t P = rq.points.size();
    Marshal1 m(rq.stack);
    Conical res(P, n);
    rcwa_options o;
    rcwa_options_default(&o);
    std::vector<rcwa_point_conical> pts(P);
    for (std::size_t p = 0; p < P; ++p) pts[p] = {rq.points[p].wavelength, rq.points[p].theta_deg, rq.points[p].phi_deg};
    struct Req {
        const Request& rq;
        Marshal1& m;
        Conical& res;
        const rcwa_options& o;
        int n;
        rcwa_gpu_server* server;
        rcwa_request operator()(std::size_t p) const {
            rcwa_request r{};
            r.kind = RCWA_REQ_CONICAL;
            r.stack1d = &m.st;
            r.wavelength = rq.points[p].wavelength;
            r.theta_deg = rq.points[p].theta_deg;
            r.phi_deg = rq.points[p].phi_deg;
            r.M = rq.M;
            r.options = o;
            return r;
        }
        void collect(std::size_t p, unsigned long long t, rcwa_response& resp) const {
            rcwa_result_conical v = res.view(p, n);
            rcwa_gpu_server_wait(server, t, -1, &resp, &v);
        }
    } req{rq, m, res, o, n, run.server};
    run.run(P, [&] {
        rcwa_result_conical v = res.view(0, n);
        if (fj) {  // one point with its fields, for the request's input polarization
            const int nz = static_cast<int>(fj->fr->z.size());
            fj->harmonics.resize((std::size_t)6 * n * nz);
            fj->layer_info.assign(std::max<std::size_t>(1, rq.stack.layers.size()), 0);
            cd Es = rq.Es, Ep = rq.Ep;
            if (rq.input == Input::Angles) {
                const double psi = rq.psi_deg * kPi / 180.0, delta = rq.delta_deg * kPi / 180.0;
                Es = std::sin(psi) * cd{std::cos(delta), std::sin(delta)};
                Ep = cd{std::cos(psi), 0.0};
            }
            const rcwa_complex jones[2] = {{Es.real(), Es.imag()}, {Ep.real(), Ep.imag()}};
            return rcwa_gpu_solve_conical_fields(run.ctx, &m.st, pts.data(), 1, rq.M, &o, jones, fj->fr->z.data(), nz, &v,
                                                 fj->harmonics.data(), fj->layer_info.data());
        }
        return rcwa_gpu_solve_conical_batch(run.ctx, &m.st, pts.data(), static_cast<int>(P), rq.M, &o, &v);
    }, req);
    if (fj && res.status[0] != RCWA_SAMPLE_OK) throw std::logic_error("rcwa: conical field context is unavailable");

    const double nI = rq.stack.nI.real();
    Writer w(indent);
    write_head(w, rq);
    for (std::size_t p = 0; p < P; ++p) {
        const PointSpec& pt = rq.points[p];
        const double* kx = &res.kx[p * n];
        const double ky = res.ky[p];
        const double cos_th = std::cos(pt.theta_deg * kPi / 180.0);
        std::vector<double> phi_m(n);
        std::vector<cd> kzI(n), kzII(n);
        for (int j = 0; j < n; ++j) {  // rcwa1d_conical.hpp:730-746
            const double kt = std::hypot(kx[j], ky);
            phi_m[j] = kt <= 1e-14 ? pt.phi_deg : std::atan2(ky, kx[j]) * 180.0 / kPi;
            kzI[j] = j == rq.M ? longitudinal0(rq.stack.nI, nI, cos_th) : longitudinal(rq.stack.nI, kx[j], ky);
            kzII[j] = j == rq.M ? longitudinal0(rq.stack.nII, nI, cos_th) : longitudinal(rq.stack.nII, kx[j], ky);
        }
        const auto J = [&](const std::vector<rcwa_complex>& a, int j, int k) {
            const rcwa_complex z = a[(p * n + j) * 4 + k];
            return cd{z.re, z.im};
        };
        w.begin_object();
        w.key("wavelength");
        w.value(pt.wavelength);
        w.key("theta_deg");
        w.value(pt.theta_deg);
        w.key("phi_deg");
        w.value(pt.phi_deg);
        w.key("kx");
        write_real_array(w, kx, n);
        w.key("ky");
        w.value(ky);
        w.key("phi_m_deg");
        write_real_array(w, phi_m.data(), n);
        w.key("kzI");
        write_complex_array(w, kzI);
        w.key("kzII");
        write_complex_array(w, kzII);
        w.key("flux_r");
        write_real_array(w, &res.fr[p * n], n);
        w.key("flux_t");
        write_real_array(w, &res.ft[p * n], n);
        for (const char* key : {"Jr", "Jt"}) {
            const std::vector<rcwa_complex>& a = key[1] == 'r' ? res.Jr : res.Jt;
            w.key(key);
            w.begin_array(true);
            for (int j = 0; j < n; ++j) {
                w.begin_array(true);
                for (int k = 0; k < 4; ++k) w.complex(J(a, j, k).real(), J(a, j, k).imag());
                w.end_array();
            }
            w.end_array();
        }
        for (const char* key : {"DEr_channels", "DEt_channels"}) {
            const std::vector<double>& a = key[2] == 'r' ? res.DEr : res.DEt;
            w.key(key);
            w.begin_array(true);
            for (int j = 0; j < n; ++j) write_real_array(w, &a[(p * n + j) * 4], 4);
            w.end_array();
        }
        // flux_unitarity (rcwa1d_conical.hpp:155-169)
        cd u[4] = {};
        for (int j = 0; j < n; ++j)
            for (int side = 0; side < 2; ++side) {
                const std::vector<rcwa_complex>& a = side == 0 ? res.Jr : res.Jt;
                const double f = side == 0 ? res.fr[p * n + j] : res.ft[p * n + j];
                const cd ss = J(a, j, 0), sp = J(a, j, 1), ps = J(a, j, 2), pp = J(a, j, 3);
                u[0] += f * (std::norm(ss) + std::norm(ps));
                u[1] += f * (std::conj(ss) * sp + std::conj(ps) * pp);
                u[2] += f * (std::conj(sp) * ss + std::conj(pp) * ps);
                u[3] += f * (std::norm(sp) + std::norm(pp));
            }
        w.key("flux_unitarity");
        w.begin_array(true);
        for (const cd& z : u) w.complex(z.real(), z.imag());
        w.end_array();
        if (rq.input != Input::None) {  // ConicalResult::for_input / for_angles (rcwa1d_conical.hpp:116-153)
            cd Es = rq.Es, Ep = rq.Ep;
            if (rq.input == Input::Angles) {
                const double psi = rq.psi_deg * kPi / 180.0, delta = rq.delta_deg * kPi / 180.0;
                Es = std::sin(psi) * cd{std::cos(delta), std::sin(delta)};
                Ep = cd{std::cos(psi), 0.0};
            }
            const double norm = std::hypot(std::abs(Es), std::abs(Ep));
            if (!(norm > 0.0) || !std::isfinite(norm)) fail("", "求解器不接受这组参数：rcwa: the input Jones vector must be finite and nonzero");
            Es /= norm;
            Ep /= norm;
            std::vector<cd> Rs(n), Rp(n), Ts(n), Tp(n);
            std::vector<double> DEr(n), DEt(n), DErs(n), DErp(n), DEts(n), DEtp(n);
            for (int j = 0; j < n; ++j) {
                Rs[j] = J(res.Jr, j, 0) * Es + J(res.Jr, j, 1) * Ep;
                Rp[j] = J(res.Jr, j, 2) * Es + J(res.Jr, j, 3) * Ep;
                Ts[j] = J(res.Jt, j, 0) * Es + J(res.Jt, j, 1) * Ep;
                Tp[j] = J(res.Jt, j, 2) * Es + J(res.Jt, j, 3) * Ep;
                DErs[j] = res.fr[p * n + j] * std::norm(Rs[j]);
                DErp[j] = res.fr[p * n + j] * std::norm(Rp[j]);
                DEts[j] = res.ft[p * n + j] * std::norm(Ts[j]);
                DEtp[j] = res.ft[p * n + j] * std::norm(Tp[j]);
                DEr[j] = DErs[j] + DErp[j];
                DEt[j] = DEts[j] + DEtp[j];
            }
            w.key("polarized");
            w.begin_object();
            w.key("jones_in");
            w.begin_array(true);
            w.complex(Es.real(), Es.imag());
            w.complex(Ep.real(), Ep.imag());
            w.end_array();
            const std::pair<const char*, const std::vector<cd>*> amps[] = {{"Rs", &Rs}, {"Rp", &Rp}, {"Ts", &Ts}, {"Tp", &Tp}};
            for (const auto& a : amps) {
                w.key(a.first);
                write_complex_array(w, *a.second);
            }
            const std::pair<const char*, const std::vector<double>*> effs[] = {
                {"DEr", &DEr}, {"DEt", &DEt}, {"DEr_s", &DErs}, {"DEr_p", &DErp}, {"DEt_s", &DEts}, {"DEt_p", &DEtp}};
            for (const auto& e : effs) {
                w.key(e.first);
                write_real_array(w, e.second->data(), n);
            }
            w.key("R_total");
            w.value(sum(DEr.data(), n));
            w.key("T_total");
            w.value(sum(DEt.data(), n));
            w.end_object();
        }
        write_bookkeeping(w, res.info[p], res.neig[p], res.nsolve[p], 0.0, run.seconds[p]);
        w.key("n_schur");
        w.value(res.nschur[p]);
        w.key("min_abs_lambda");
        w.value(res.minl[p]);
        w.key("degenerate_mode_warning");
        w.value(res.warn[p] != 0);
        w.end_object();
    }
    w.end_array();
    if (fj) {
        // metadata of the conical fields (rcwa1d_conical_fields.hpp:52-97): kxm = k0 kx, ky = k0 ky
        const PointSpec& pt = rq.points[0];
        const double k0 = 2.0 * kPi / pt.wavelength, nI = rq.stack.nI.real();
        std::vector<double> kx(n), ky(n, k0 * res.ky[0]);
        for (int j = 0; j < n; ++j) kx[j] = k0 * res.kx[j];
        const cd kz0 = longitudinal0(rq.stack.nI, nI, std::cos(pt.theta_deg * kPi / 180.0));
        const double kinc[3] = {kx[rq.M], k0 * res.ky[0], (k0 * kz0).real()};
        fj->solve_seconds = run.seconds[0];
        fields_tail(w, run.ctx, *fj, kx, ky, kinc, rq.stack.period, 1.0, nI, layer_rows(rq.stack.layers, true, fj->layer_info, true));
        return w.take();
    }
    w.end_object();
    return w.take();
}

// kz/k0 in a homogeneous 2-D region (rcwa2d.hpp:376-381) and the index as the Rayleigh message prints it
// (format_index, rcwa2d.hpp:1019-1024)
cd kz_over_k0(cd n, double Kx, double Ky) {
    cd kz = std::sqrt(n * n - Kx * Kx - Ky * Ky);
    if (kz.imag() < 0.0) kz = -kz;
    return kz;
}
std::string format_index(cd n) {
    char buf[96];
    if (n.imag() == 0.0) std::snprintf(buf, sizeof buf, "%.10g", n.real());
    else std::snprintf(buf, sizeof buf, "(%.10g%+.10gj)", n.real(), n.imag());
    return buf;
}

// Result2D::message of a failed point (rcwa2d.hpp:1027-1037, :1101-1113, :1174, :1229)
std::string message_2d(const Request& rq, Grid2& g, std::size_t p, int N) {
    const int st = g.status[p];
    if (st == RCWA_SAMPLE_OK) return "";
    if (st == RCWA_SAMPLE_RAYLEIGH) {
        const int n2 = 2 * rq.My + 1;
        std::string message;
        const auto report = [&](const std::string& where, cd n, const std::vector<cd>& kz) {
            std::string labels;
            for (int i = 0; i < N; ++i) {
                if (kz[i] != cd{}) continue;
                if (!labels.empty()) labels += ", ";
                labels += "(" + std::to_string(i / n2 - rq.M) + ", " + std::to_string(i % n2 - rq.My) + ")";
            }
            if (labels.empty()) return;
            if (!message.empty()) message += "；";
            message += where + "（n=" + format_index(n) + "）的 (m, n) = " + labels + " 级恰好沿界面掠射（kz=0，Rayleigh 异常点），无法求解";
        };
        std::vector<cd> kzI(N), kzII(N);
        for (int i = 0; i < N; ++i) {
            kzI[i] = {g.kzI[p * N + i].re, g.kzI[p * N + i].im};
            kzII[i] = {g.kzII[p * N + i].re, g.kzII[p * N + i].im};
        }
        report("入射区", cd{rq.stack2d.nI, 0.0}, kzI);
        report("出射区", rq.stack2d.nII, kzII);
        for (std::size_t j = 0; j < rq.stack2d.layers.size(); ++j) {
            const Layer2& L = rq.stack2d.layers[j];
            if (!L.homogeneous) continue;
            std::vector<cd> kz(N);
            for (int i = 0; i < N; ++i) kz[i] = kz_over_k0(L.n, g.Kx[p * N + i], g.Ky[p * N + i]);
            report("第" + std::to_string(j + 1) + "层", L.n, kz);
        }
        return message + "。请把入射角、方位角或周期略作改动（例如入射角改动 0.01°）后重算。";
    }
    if (g.info[p] != 0) return "数值失败：本征迭代未收敛（eig_info = " + std::to_string(g.info[p]) + "）";
    return "数值失败：求解中出现奇异的线性方程组或 NaN/Inf";
}

std::string run_periodic2d(const Request& rq, Runner& run, int indent, FieldsJob* fj = nullptr) {
    const int N = (2 * rq.M + 1) * (2 * rq.My + 1);
    const std::size_t P = rq.points.size();
    Marshal2 m(rq.stack2d);
    Grid2 g(P, N, static_cast<int>(rq.stack2d.layers.size()));
    rcwa_options o;
    rcwa_options_default(&o);
    o.diagnostics = rq.diagnostics ? 1 : 0;
    const int fact = rq.laurent ? RCWA_FACTORIZATION_LAURENT : RCWA_FACTORIZATION_LI;
    std::vector<rcwa_point2d> pts(P);
    for (std::size_t p = 0; p < P; ++p)
        pts[p] = {rq.points[p].wavelength, rq.points[p].theta_deg, rq.points[p].phi_deg, {rq.Es.real(), rq.Es.imag()},
                  {rq.Ep.real(), rq.Ep.imag()}};
    struct Req {
        const Request& rq;
        Marshal2& m;
        Grid2& g;
        const rcwa_options& o;
        const std::vector<rcwa_point2d>& pts;
        int N, fact;
        rcwa_gpu_server* server;
        rcwa_request operator()(std::size_t p) const {
            rcwa_request r{};
            r.kind = RCWA_REQ_2D;
            r.stack2d = &m.st;
            r.wavelength = pts[p].wavelength;
            r.theta_deg = pts[p].theta_deg;
            r.phi_deg = pts[p].phi_deg;
            r.M1 = rq.M;
            r.M2 = rq.My;
            r.factorization = fact;
            r.Es = pts[p].Es;
            r.Ep = pts[p].Ep;
            r.options = o;
            return r;
        }
        void collect(std::size_t p, unsigned long long t, rcwa_response& resp) const {
            rcwa_result2d v = g.view(p, N);
            rcwa_gpu_server_wait(server, t, -1, &resp, &v);
        }
    } req{rq, m, g, o, pts, N, fact, run.server};
    run.run(P, [&] {
        rcwa_result2d v = g.view(0, N);
        if (fj) {
            const int nz = static_cast<int>(fj->fr->z.size());
            fj->harmonics.resize((std::size_t)6 * N * nz);
            return rcwa_gpu_solve2d_fields(run.ctx, &m.st, pts.data(), 1, rq.M, rq.My, fact, &o, fj->fr->z.data(), nz, &v,
                                           fj->harmonics.data());
        }
        return rcwa_gpu_solve2d_batch(run.ctx, &m.st, pts.data(), static_cast<int>(P), rq.M, rq.My, fact, &o, &v);
    }, req);
    if (fj && g.status[0] != RCWA_SAMPLE_OK) {  // rcwa_fields_json.hpp:313-314
        const std::string why = message_2d(rq, g, 0, N);
        throw std::runtime_error(why.empty() ? std::string("fields 求解失败") : why);
    }

    Writer w(indent);
    write_head(w, rq);
    for (std::size_t p = 0; p < P; ++p) {
        const bool solved = g.status[p] == RCWA_SAMPLE_OK;
        const auto reals = [&](const char* key, const std::vector<double>& v) {
            w.key(key);
            w.begin_array(true);
            for (int i = 0; i < N; ++i)
                if (solved) w.value(v[p * N + i]);
                else w.null();
            w.end_array();
        };
        const auto complexes = [&](const char* key, const std::vector<rcwa_complex>& v) {
            w.key(key);
            w.begin_array(true);
            for (int i = 0; i < N; ++i) {
                if (solved) {
                    w.complex(v[p * N + i].re, v[p * N + i].im);
                } else {
                    w.begin_array(true);
                    w.null();
                    w.null();
                    w.end_array();
                }
            }
            w.end_array();
        };
        const auto flags = [&](const char* key, const std::vector<unsigned char>& v) {
            w.key(key);
            w.begin_array(true);
            for (int i = 0; i < N; ++i) w.value(v[p * N + i] != 0 ? 1 : 0);
            w.end_array();
        };
        w.begin_object();
        w.key("wavelength");
        w.value(rq.points[p].wavelength);
        w.key("theta_deg");
        w.value(rq.points[p].theta_deg);
        w.key("phi_deg");
        w.value(rq.points[p].phi_deg);
        w.key("status");
        w.value(g.status[p] == RCWA_SAMPLE_OK ? "ok" : g.status[p] == RCWA_SAMPLE_RAYLEIGH ? "rayleigh_anomaly" : "numerical_failure");
        w.key("message");
        w.value(message_2d(rq, g, p, N));
        reals("Kx", g.Kx);
        reals("Ky", g.Ky);
        complexes("kzI", g.kzI);
        complexes("kzII", g.kzII);
        complexes("Rs", g.Rs);
        complexes("Rp", g.Rp);
        complexes("Ts", g.Ts);
        complexes("Tp", g.Tp);
        complexes("Ex_r", g.Ex_r);
        complexes("Ey_r", g.Ey_r);
        complexes("Ez_r", g.Ez_r);
        complexes("Ex_t", g.Ex_t);
        complexes("Ey_t", g.Ey_t);
        complexes("Ez_t", g.Ez_t);
        reals("DEr", g.DEr);
        reals("DEt", g.DEt);
        flags("prop_r", g.prop_r);
        flags("prop_t", g.prop_t);
        w.key("eig_info");
        w.value(g.info[p]);
        w.key("n_eig");
        w.value(g.neig[p]);
        w.key("n_dense_solve");
        w.value(g.nsolve[p]);
        w.key("max_eig_residual");
        w.value(rq.diagnostics ? g.resid[p] : 0.0);
        w.key("max_solve_backward_error");
        w.value(0.0);
        w.key("timing");
        w.begin_object(true);
        w.key("total");
        w.value(run.seconds[p]);
        w.key("operators");
        w.value(0.0);
        w.key("eig");
        w.value(0.0);
        w.key("linear");
        w.value(0.0);
        w.key("product");
        w.value(0.0);
        w.end_object();
        w.end_object();
    }
    w.end_array();
    if (fj) {
        // metadata of the 2-D fields (rcwa2d_fields.hpp:138-177): kxm = k0 Kx, kyn = k0 Ky, |E_inc| = |Jones|
        const PointSpec& pt = rq.points[0];
        const double k0 = 2.0 * kPi / pt.wavelength;
        std::vector<double> kx(N), ky(N);
        for (int i = 0; i < N; ++i) {
            kx[i] = k0 * g.Kx[i];
            ky[i] = k0 * g.Ky[i];
        }
        const int i0 = rq.M * (2 * rq.My + 1) + rq.My;
        const cd kz0{g.kzI[i0].re, g.kzI[i0].im};
        const double kinc[3] = {kx[i0], ky[i0], (k0 * kz0).real()};
        const double jn = std::hypot(std::abs(rq.Es), std::abs(rq.Ep));
        fj->solve_seconds = run.seconds[0];
        const double period = fj->fr->plane == RCWA_SLICE_XZ ? rq.stack2d.Lx : rq.stack2d.Ly;
        fields_tail(w, run.ctx, *fj, kx, ky, kinc, period, jn, rq.stack2d.nI * jn,
                    layer_rows(rq.stack2d.layers, false, std::vector<int>{}, false));
        return w.take();
    }
    w.end_object();
    return w.take();
}

std::string error_reply(const std::string& message, const std::string& where, int indent) {
    Writer w(indent);
    w.begin_object();
    w.key("ok");
    w.value(false);
    w.key("error");
    w.value(message);
    w.key("where");
    w.value(where);
    w.end_object();
    return w.take();
}

// The whole answer; never throws.
std::string answer(const char* request, int indent, Runner* run, bool& ok) {
    ok = false;
    try {
        try {
            const Request rq = parse_request(request ? std::string(request) : std::string());
            if (!run) {  // validation only
                ok = true;
                return "";
            }
            std::string reply = rq.mode == Mode::Periodic2D ? run_periodic2d(rq, *run, indent)
                                : rq.mode == Mode::Conical  ? run_conical(rq, *run, indent)
                                                            : run_planar(rq, *run, indent);
            ok = true;
            return reply;
        } catch (const RequestError& e) {
            return error_reply(e.message, e.where, indent);
        } catch (const std::bad_alloc&) {
            return error_reply("内存不够", "", indent);
        } catch (const std::exception& e) {
            return error_reply(std::string("求解时出错：") + e.what(), "", indent);
        }
    } catch (...) {
    }
    return "{\"ok\": false, \"error\": \"out of memory\", \"where\": \"\"}";
}

// rcwa::solve_fields_json_reply (rcwa_fields_json.hpp:462-474); never throws
std::string answer_fields(const char* request, int indent, rcwa_gpu_ctx* ctx, bool& ok) {
    ok = false;
    try {
        try {
            Value root;
            try {
                root = jtext::parse(request ? std::string(request) : std::string());
            } catch (const jtext::ParseError& e) {
                throw std::invalid_argument("json: " + e.reason + " at offset " + std::to_string(e.offset) + " (line " +
                                            std::to_string(e.line) + ", column " + std::to_string(e.column) + ")");
            }
            const FieldsRequest fr = read_fields_request(root);
            if (!ctx) {  // validation only
                ok = true;
                return "";
            }
            Runner run;
            run.ctx = ctx;
            FieldsJob fj;
            fj.fr = &fr;
            std::string reply = fr.solve.mode == Mode::Periodic2D ? run_periodic2d(fr.solve, run, indent, &fj)
                                : fr.solve.mode == Mode::Conical  ? run_conical(fr.solve, run, indent, &fj)
                                                                  : run_planar(fr.solve, run, indent, &fj);
            ok = true;
            return reply;
        } catch (const RequestError& e) {
            return error_reply(e.message, e.where, indent);
        } catch (const std::exception& e) {
            return error_reply(e.what(), "fields", indent);
        }
    } catch (...) {
    }
    return "{\"ok\": false, \"error\": \"fields 未识别的求解或输出错误\", \"where\": \"fields\"}";
}

int hand_out(const std::string& text, bool ok, char** reply, int* ok_out) {
    char* p = static_cast<char*>(std::malloc(text.size() + 1));
    if (!p) return RCWA_ENOMEM;
    std::memcpy(p, text.c_str(), text.size() + 1);
    *reply = p;
    if (ok_out) *ok_out = ok ? 1 : 0;
    return RCWA_OK;
}

}  // namespace
}  // namespace jfront
}  // namespace rcwa_gb300

extern "C" {

int rcwa_gpu_solve_json(rcwa_gpu_ctx* ctx, const char* request, int indent, char** reply, int* ok) {
    if (!ctx || !reply) return RCWA_EINVAL;
    rcwa_gb300::jfront::Runner run;
    run.ctx = ctx;
    bool good = false;
    const std::string text = rcwa_gb300::jfront::answer(request, indent, &run, good);
    return rcwa_gb300::jfront::hand_out(text, good, reply, ok);
}

int rcwa_gpu_server_solve_json(rcwa_gpu_server* server, const char* request, int indent, char** reply, int* ok) {
    if (!server || !reply) return RCWA_EINVAL;
    rcwa_gb300::jfront::Runner run;
    run.server = server;
    bool good = false;
    const std::string text = rcwa_gb300::jfront::answer(request, indent, &run, good);
    return rcwa_gb300::jfront::hand_out(text, good, reply, ok);
}

int rcwa_json_validate(const char* request, int indent, char** reply, int* ok) {
    if (!reply) return RCWA_EINVAL;
    bool good = false;
    const std::string text = rcwa_gb300::jfront::answer(request, indent, nullptr, good);
    return rcwa_gb300::jfront::hand_out(text, good, reply, ok);
}

int rcwa_fields_json_validate(const char* request, int indent, char** reply, int* ok) {
    if (!reply) return RCWA_EINVAL;
    bool good = false;
    const std::string text = rcwa_gb300::jfront::answer_fields(request, indent, nullptr, good);
    return rcwa_gb300::jfront::hand_out(text, good, reply, ok);
}

int rcwa_gpu_solve_fields_json(rcwa_gpu_ctx* ctx, const char* request, int indent, char** reply, int* ok) {
    if (!ctx || !reply) return RCWA_EINVAL;
    bool good = false;
    const std::string text = rcwa_gb300::jfront::answer_fields(request, indent, ctx, good);
    return rcwa_gb300::jfront::hand_out(text, good, reply, ok);
}

void rcwa_json_free(char* reply) { std::free(reply); }

}  // extern "C"
