// Golden-fixture exporter for the general complex eigensolver (CORTH + COMQR2).
//
// Built and run only where the StableRCWA sources are present (see make_golden.py). It compiles the
// reference's own test program tests/test_eig_qr.cpp in place (main() renamed) so the matrices are
// the ones its tests use (rcwa_te_matrix, random_complex, companion, ...). For each matrix it writes
// the entries, and the reference eig_qr's eigenvalues, info and sweep count (one JSON object per line).
#define main stablercwa_reference_eig_test_main
#include "test_eig_qr.cpp"
#undef main

#include <cstdio>
#include <string>

namespace {

void put_c(std::FILE* f, cplx z) { std::fprintf(f, "[%.17g,%.17g]", z.real(), z.imag()); }

void put_case(std::FILE* f, const std::string& name, const char* source, const Matrix& a, int max_iter = 30) {
    EigOptions opt;
    opt.max_iter = max_iter;
    const EigResult r = eig_qr(a, opt);
    const int n = a.rows();
    std::fprintf(f, "{\"name\":\"%s\",\"source\":\"%s\",\"n\":%d,\"max_iter\":%d,\"a\":[", name.c_str(), source, n, max_iter);
    for (int k = 0; k < n * n; ++k) {
        if (k) std::fprintf(f, ",");
        put_c(f, a.data()[k]);
    }
    std::fprintf(f, "],\"values\":[");
    for (int k = 0; k < n; ++k) {
        if (k) std::fprintf(f, ",");
        put_c(f, r.values[k]);
    }
    const double res = r.info == 0 ? ::eig_residual(a, r) : -1.0;
    std::fprintf(f, "],\"info\":%d,\"sweeps\":%d,\"residual\":%.17g}\n", r.info, r.sweeps, res);
}

}  // namespace

int main(int argc, char** argv) {
    std::FILE* f = argc > 1 ? std::fopen(argv[1], "w") : stdout;
    if (!f) return 2;
    const double fill = 0.4, lop = 0.61, st = 0.2;   // test_rcwa_like (tests/test_eig_qr.cpp:711-716)
    for (int n : {41}) {
        put_case(f, "rcwa_te_lossless_" + std::to_string(n), "tests/test_eig_qr.cpp:718", rcwa_te_matrix(n, 1.5, 1.0, fill, lop, st));
        put_case(f, "rcwa_te_lossy_" + std::to_string(n), "tests/test_eig_qr.cpp:732", rcwa_te_matrix(n, cplx(1.8, 0.13), 1.0, fill, lop, st));
        put_case(f, "rcwa_te_metal_" + std::to_string(n), "tests/test_eig_qr.cpp:732", rcwa_te_matrix(n, cplx(0.08, 5.43), 1.0, fill, lop, st));
    }
    put_case(f, "rcwa_te_littrow_41", "tests/test_eig_qr.cpp:770", rcwa_te_matrix(41, 1.5, 1.0, fill, lop, 0.3));
    for (int n : {6, 30}) put_case(f, "random_complex_" + std::to_string(n), "tests/test_eig_qr.cpp:785", random_complex(n, 700 + n));
    put_case(f, "random_real_40", "tests/test_eig_qr.cpp:510", random_real(40, 77));
    {
        const Vector d{1.0, 1.0, 1.0, 2.0, 3.0, 3.0};   // tests/test_eig_qr.cpp:532-541
        const Matrix q = random_unitary(6, 501);
        put_case(f, "semisimple_repeated", "tests/test_eig_qr.cpp:532", hermitian_part(q * Matrix::diagonal(d) * adjoint(q)));
    }
    {
        Matrix a(5, 5);                                 // tests/test_eig_qr.cpp:544-551
        a(0, 0) = a(1, 1) = a(2, 2) = 2.0;
        a(0, 1) = a(1, 2) = 1.0;
        a(3, 3) = 5.0;
        a(4, 4) = -1.0;
        put_case(f, "jordan_upper", "tests/test_eig_qr.cpp:544", a);
    }
    put_case(f, "companion_roots", "tests/test_eig_qr.cpp:404",
             companion(Vector{1.0, 2.0, 3.0, cplx(0, 1), cplx(0, -1), cplx(-2, 0.5), 0.25}));
    {
        const Matrix a = random_complex(20, 1001);      // tests/test_eig_qr.cpp:957-1000
        for (int max_iter = 1; max_iter <= 4; ++max_iter)
            put_case(f, "not_converged_maxiter" + std::to_string(max_iter), "tests/test_eig_qr.cpp:964", a, max_iter);
    }
    {
        Matrix a(12, 12);                                // tests/test_eig_qr.cpp:990-1000 (cyclic P (+) B, max_iter 10)
        const Matrix b = random_complex(4, 1002);
        for (int i = 1; i < 8; ++i) a(i, i - 1) = 1.0;
        a(0, 7) = 1.0;
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 4; ++i) a(8 + i, 8 + j) = b(i, j);
        put_case(f, "partial_cyclic_maxiter10", "tests/test_eig_qr.cpp:990", a, 10);
    }
    put_case(f, "uniform_layer_normal_incidence_25", "tests/test_eig_qr.cpp:625", uniform_layer_matrix(25, 1.5, 0.61));
    if (f != stdout) std::fclose(f);
    return 0;
}
