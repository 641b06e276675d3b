// ref_solve1d.cpp -- runs StableRCWA's own rcwa::sweep on a case read from stdin (TEST INFRASTRUCTURE).
//
// Built only where the StableRCWA sources exist (oracle/build.py --ref compiles it against the
// reference headers in place into oracle/_ref/). Input (whitespace separated):
//   M pol threads n_points nI_re nII_re nII_im period n_layers
//   per layer: d homogeneous(1|0) then n_re n_im, or K then K+1 edges and K (re im) indices
//   per point: wavelength theta_deg
// Output: per point one line with 2M+1 DEr values then 2M+1 DEt values (17 significant digits).
#include <cstdio>
#include <iostream>
#include <vector>

#include "stablercwa/rcwa1d.hpp"

namespace rcwa = stablercwa::rcwa;
using stablercwa::cplx;

int main() {
    int M, pol, threads, n_points, n_layers;
    double nIr, nIIr, nIIi, period;
    if (!(std::cin >> M >> pol >> threads >> n_points >> nIr >> nIIr >> nIIi >> period >> n_layers)) return 2;
    rcwa::Stack s;
    s.nI = nIr;
    s.nII = cplx(nIIr, nIIi);
    s.period = period;
    for (int k = 0; k < n_layers; ++k) {
        double d;
        int hom;
        std::cin >> d >> hom;
        if (hom) {
            double re, im;
            std::cin >> re >> im;
            s.layers.push_back(rcwa::Layer::uniform(d, cplx(re, im)));
        } else {
            int K;
            std::cin >> K;
            std::vector<double> e(K + 1);
            std::vector<cplx> v(K);
            for (double& x : e) std::cin >> x;
            for (cplx& x : v) {
                double re, im;
                std::cin >> re >> im;
                x = cplx(re, im);
            }
            s.layers.push_back(rcwa::Layer::grating(d, e, v));
        }
    }
    std::vector<rcwa::Point> pts(n_points);
    for (auto& p : pts) std::cin >> p.wavelength >> p.theta_deg;
    stablercwa::set_num_threads(threads);
    const auto res = rcwa::sweep(s, pts, M, pol ? rcwa::Polarization::TM : rcwa::Polarization::TE);
    for (const auto& r : res) {
        for (double v : r.DEr) std::printf("%.17g ", v);
        for (double v : r.DEt) std::printf("%.17g ", v);
        std::printf("\n");
    }
    return 0;
}
