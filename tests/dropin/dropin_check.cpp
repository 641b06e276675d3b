// Drop-in check (test program): include/stablercwa_gb300.hpp against the reference's own entry points.
// Built by tests/test_dropin.py against the StableRCWA headers and libstablercwa_gb300.so. For every
// invalid input below, stablercwa_gb300::rcwa::{solve, solve_conical, solve2d} must throw the same
// exception type with the same message as stablercwa::rcwa::{solve, solve_conical, solve2d}; with a
// valid input and no CUDA device the drop-in must throw std::runtime_error (never a wrong result).
// With a device present (argument "device") it also compares efficiencies with the reference's.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <typeinfo>

#include "stablercwa/stablercwa.hpp"
#include "stablercwa_gb300.hpp"

namespace ref = stablercwa::rcwa;
namespace gb = stablercwa_gb300::rcwa;
using stablercwa::cplx;

static int failures = 0;

struct Outcome {
    std::string kind, what;
};

static Outcome run(const std::function<void()>& f) {
    try {
        f();
        return {"ok", ""};
    } catch (const std::invalid_argument& e) {
        return {"invalid_argument", e.what()};
    } catch (const std::runtime_error& e) {
        return {"runtime_error", e.what()};
    } catch (const std::exception& e) {
        return {typeid(e).name(), e.what()};
    }
}

static void same(const char* name, const std::function<void()>& a, const std::function<void()>& b) {
    const Outcome x = run(a), y = run(b);
    const bool ok = x.kind == "invalid_argument" && x.kind == y.kind && x.what == y.what;
    std::printf("%s %s: reference [%s] %s | drop-in [%s] %s\n", ok ? "PASS" : "FAIL", name, x.kind.c_str(), x.what.c_str(),
                y.kind.c_str(), y.what.c_str());
    failures += ok ? 0 : 1;
}

static ref::Stack readme_stack() {
    ref::Stack s;
    s.nI = 1.0;
    s.nII = 1.46;
    s.period = 0.574;
    s.layers.push_back(ref::Layer::grating(0.38, {0.0, 0.172, 0.574}, {1.46, 1.0}));
    s.layers.push_back(ref::Layer::uniform(0.115, 1.96));
    return s;
}

static ref::Stack2D pillar_stack() {
    ref::Stack2D s;
    s.nI = 1.0;
    s.nII = 1.46;
    s.Lx = s.Ly = 0.8;
    ref::XProfile2D air{{0.0, 0.8}, {1.0}}, mid{{0.0, 0.2, 0.6, 0.8}, {1.0, 2.0, 1.0}};
    s.layers.push_back(ref::Layer2D::patterned(0.2, {0.0, 0.2, 0.6, 0.8}, {air, mid, air}));
    s.layers.push_back(ref::Layer2D::uniform(0.1, 1.7));
    return s;
}

int main(int argc, char** argv) {
    const bool device = argc > 1 && std::strcmp(argv[1], "device") == 0;
    using P = ref::Polarization;
    // ---- 1-D: one fault per case, the reference's check order decides the message
    struct Case1 {
        const char* name;
        std::function<void(ref::Stack&, double&, double&, int&)> edit;
    };
    const Case1 cases1[] = {
        {"period <= 0", [](ref::Stack& s, double&, double&, int&) { s.period = 0.0; }},
        {"wavelength NaN", [](ref::Stack&, double& wl, double&, int&) { wl = std::nan(""); }},
        {"theta = 90", [](ref::Stack&, double&, double& th, int&) { th = 90.0; }},
        {"negative M", [](ref::Stack&, double&, double&, int& M) { M = -1; }},
        {"absorbing incident medium", [](ref::Stack& s, double&, double&, int&) { s.nI = cplx{1.0, 0.1}; }},
        {"gain in a film", [](ref::Stack& s, double&, double&, int&) { s.layers[1].n = cplx{1.5, -0.01}; }},
        {"negative thickness", [](ref::Stack& s, double&, double&, int&) { s.layers[1].d = -0.1; }},
        {"edges not increasing", [](ref::Stack& s, double&, double&, int&) { s.layers[0].edges = {0.0, 0.3, 0.2}; }},
        {"edges not one period", [](ref::Stack& s, double&, double&, int&) { s.layers[0].edges = {0.0, 0.172, 0.5}; }},
        {"index count", [](ref::Stack& s, double&, double&, int&) { s.layers[0].n_values = {1.46}; }},
        {"zero exit index", [](ref::Stack& s, double&, double&, int&) { s.nII = 0.0; }},
        {"FFT samples too few",
         [](ref::Stack& s, double&, double&, int&) {
             s.layers[0].fourier_method = ref::FourierMethod::FFT;
             s.layers[0].fft_samples = 16;
         }},
    };
    for (const Case1& c : cases1) {
        for (P pol : {P::TE, P::TM}) {
            ref::Stack s = readme_stack();
            double wl = 1.053, th = 66.36;
            int M = 20;
            c.edit(s, wl, th, M);
            const std::string name = std::string("solve ") + c.name + (pol == P::TE ? " TE" : " TM");
            same(name.c_str(), [&] { ref::solve(s, wl, th, M, pol); }, [&] { gb::solve(s, wl, th, M, pol); });
        }
    }
    // ---- conical
    {
        ref::Stack s = readme_stack();
        s.nII = cplx{1.46, 0.01};
        same("solve_conical absorbing exit medium", [&] { ref::solve_conical(s, 1.053, 30.0, 20.0, 10); },
             [&] { gb::solve_conical(s, 1.053, 30.0, 20.0, 10); });
        ref::Stack t = readme_stack();
        same("solve_conical theta = -90", [&] { ref::solve_conical(t, 1.053, -90.0, 20.0, 10); },
             [&] { gb::solve_conical(t, 1.053, -90.0, 20.0, 10); });
    }
    // ---- 2-D
    {
        const ref::Jones2D j = ref::jones_from_angles_2d(90.0);
        ref::Stack2D s = pillar_stack();
        s.Lx = -1.0;
        same("solve2d negative period", [&] { ref::solve2d(s, 0.7, 0.0, 0.0, 2, 2, j); },
             [&] { gb::solve2d(s, 0.7, 0.0, 0.0, 2, 2, j); });
        ref::Stack2D t = pillar_stack();
        same("solve2d negative M1", [&] { ref::solve2d(t, 0.7, 0.0, 0.0, -1, 2, j); },
             [&] { gb::solve2d(t, 0.7, 0.0, 0.0, -1, 2, j); });
        ref::Stack2D u = pillar_stack();
        u.layers[0].y_edges = {0.0, 0.2, 0.6, 0.7};
        same("solve2d y edges not one period", [&] { ref::solve2d(u, 0.7, 0.0, 0.0, 2, 2, j); },
             [&] { gb::solve2d(u, 0.7, 0.0, 0.0, 2, 2, j); });
    }
    // ---- a valid solve
    if (!device) {
        const Outcome o = run([] { gb::solve(readme_stack(), 1.053, 66.36, 20); });
        const bool ok = o.kind == "runtime_error";
        std::printf("%s valid solve without a device: [%s] %s\n", ok ? "PASS" : "FAIL", o.kind.c_str(), o.what.c_str());
        failures += ok ? 0 : 1;
        const Outcome h = run([] {
            ref::Options opt;
            opt.custom_eig = stablercwa_gb300::gpu_eig();
            ref::solve(readme_stack(), 1.053, 66.36, 20, P::TE, opt);
        });
        const bool hok = h.kind == "ok" || h.kind == "runtime_error";
        std::printf("%s custom_eig hook without a device: [%s] %s\n", hok ? "PASS" : "FAIL", h.kind.c_str(), h.what.c_str());
        failures += hok ? 0 : 1;
    } else {
        const ref::Result a = ref::solve(readme_stack(), 1.053, 66.36, 20);
        const ref::Result b = gb::solve(readme_stack(), 1.053, 66.36, 20);
        double d = 0.0;
        for (std::size_t k = 0; k < a.DEr.size(); ++k)
            d = std::fmax(d, std::fmax(std::fabs(a.DEr[k] - b.DEr[k]), std::fabs(a.DEt[k] - b.DEt[k])));
        const bool ok = d <= 1e-10 && a.n_eig == b.n_eig;
        std::printf("%s README structure on the device: max |dDE| %.2e\n", ok ? "PASS" : "FAIL", d);
        failures += ok ? 0 : 1;
    }
    std::printf("%d failures\n", failures);
    return failures == 0 ? 0 : 1;
}
