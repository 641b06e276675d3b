// Runs the Hermitian eigensolver's kernels (stablercwa_gb300/csrc/eig.cuh: herm_tridiag_one, herm_ql_kernel,
// herm_apply_real_kernel, herm_apply_kernel) and the general solver's eig_one on the CPU through
// tests/emu/cuda_runtime.h and checks the eigenpairs: residual ||A v - lambda v|| / (||A||_F ||v||) <= 1e-13,
// and orthonormal columns for the Hermitian solver. The group of G lanes is G std::threads, and so is each
// 32-row CTA of herm_apply_real_kernel; the QL and complex rotation kernels run one emulated thread at a
// time. Exit status 0 and a final "OK" line when every case passes. Test infrastructure only.
#include <barrier>
#include <cmath>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

#include "cuda_runtime.h"

thread_local dim3e threadIdx;
static std::barrier<>* bar;
static int group_size;
static double dslot[256];
static int islot[256];
void emu_sync() { bar->arrive_and_wait(); }
double emu_shfl_xor(double v, int o) {
    const int l = threadIdx.x;
    dslot[l] = v;
    bar->arrive_and_wait();
    const double r = dslot[l ^ o];
    bar->arrive_and_wait();
    return r;
}
int emu_shfl_xor_i(int v, int o) {
    const int l = threadIdx.x;
    islot[l] = v;
    bar->arrive_and_wait();
    const int r = islot[l ^ o];
    bar->arrive_and_wait();
    return r;
}
unsigned emu_ballot(int p) {
    const int l = threadIdx.x;
    islot[l] = p;
    bar->arrive_and_wait();
    unsigned b = 0;
    const int w0 = (l / 32) * 32;
    for (int k = w0; k < group_size && k < w0 + 32; ++k)
        if (islot[k]) b |= 1u << (k - w0);
    bar->arrive_and_wait();
    return b;
}

#include "../../stablercwa_gb300/csrc/eig.cuh"

using namespace rcwa_gb300;

static int failures = 0;
// the shared reduction slots of a CTA form (G > 32 lanes: herm_reduce_block_kernel's red and ired)
static double cta_red[8];
static int cta_ired[8];

// herm_apply_real_kernel for one matrix: each CTA (32 rows) as 32 threads meeting at one barrier, since the
// warp stages the rotation log through shared memory
static void apply_real(int n, double* Y, const zc* ws, const int* info) {
    for (int by = 0; by * kHermRows < n; ++by) {
        blockIdx.x = 0;
        blockIdx.y = by;
        group_size = kHermRows;
        std::barrier<> b(kHermRows);
        bar = &b;
        std::vector<std::thread> th;
        for (int l = 0; l < kHermRows; ++l)
            th.emplace_back([&, l] {
                threadIdx.x = l;
                herm_apply_real_kernel(n, 1, Y, ws, info);
            });
        for (auto& x : th) x.join();
    }
    blockIdx.y = 0;
}

template <int G>
void run(int n, const std::vector<zc>& a, const char* tag, bool real_form, bool smem_ql) {
    group_size = G;
    std::barrier<> b(G);
    bar = &b;
    std::vector<zc> V((size_t)n * n), W(n), ws(eig_workspace_elems(n));
    int info = -7;
    std::vector<std::thread> th;
    for (int l = 0; l < G; ++l)
        th.emplace_back([&, l] {
            threadIdx.x = l;
            herm_tridiag_one<G>(n, a.data(), V.data(), ws.data(), G > 32 ? cta_red : nullptr, G > 32 ? cta_ired : nullptr);
        });
    for (auto& t : th) t.join();
    unsigned long long rot = 0;
    threadIdx.x = 0;
    blockIdx.x = 0;
    blockIdx.y = 0;
    blockDim.x = smem_ql ? kHermQlThreads : 128;
    // the real form's log is fixed point, the complex form's doubles
    if (smem_ql && real_form)
        herm_ql_kernel<true, true>(n, 1, W.data(), &info, ws.data(), 2.220446049250313e-16, 30, &rot);
    else if (smem_ql)
        herm_ql_kernel<true, false>(n, 1, W.data(), &info, ws.data(), 2.220446049250313e-16, 30, &rot);
    else if (real_form)
        herm_ql_kernel<false, true>(n, 1, W.data(), &info, ws.data(), 2.220446049250313e-16, 30, &rot);
    else
        herm_ql_kernel<false, false>(n, 1, W.data(), &info, ws.data(), 2.220446049250313e-16, 30, &rot);
    const int* tail = reinterpret_cast<const int*>(ws.data() + 3LL * n * n);
    if (info != 0 || tail[1] != 0) {
        std::printf("FAIL %s n=%d: info %d overflow %d\n", tag, n, info, tail[1]);
        ++failures;
        return;
    }
    if (real_form) {
        std::vector<double> Y((size_t)n * n);
        apply_real(n, Y.data(), ws.data(), &info);
        std::vector<zc> Q = V;  // Z = Q Y, the product zdgemm_kernel forms on the device
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                zc acc{0.0, 0.0};
                for (int k = 0; k < n; ++k) acc = acc + Q[(size_t)k * n + i] * Y[(size_t)j * n + k];
                V[(size_t)j * n + i] = acc;
            }
    } else {
        blockDim.x = 128;
        for (int r = 0; r < n; ++r) {
            blockIdx.x = 0;
            threadIdx.x = r;
            herm_apply_kernel(n, 1, V.data(), ws.data(), &info);
        }
    }
    blockIdx.y = 0;
    double fro = 0.0;
    for (const zc& z : a) fro += norm2(z);
    fro = std::sqrt(fro);
    double worst = 0.0, orth = 0.0;
    for (int j = 0; j < n; ++j) {
        double dn = 0.0, vn = 0.0;
        for (int i = 0; i < n; ++i) {
            zc acc{0.0, 0.0};
            for (int k = 0; k < n; ++k) acc = acc + a[(size_t)k * n + i] * V[(size_t)j * n + k];
            dn += norm2(acc - W[j] * V[(size_t)j * n + i]);
            vn += norm2(V[(size_t)j * n + i]);
        }
        worst = std::fmax(worst, std::sqrt(dn) / (std::fmax(fro, 1e-300) * std::sqrt(vn)));
        for (int k = 0; k < n; ++k) {
            zc dot{0.0, 0.0};
            for (int i = 0; i < n; ++i) dot = dot + conj(V[(size_t)j * n + i]) * V[(size_t)k * n + i];
            orth = std::fmax(orth, zabs(dot - zc{j == k ? 1.0 : 0.0, 0.0}));
        }
    }
    const bool ok = worst <= 1e-13 && orth <= 1e-13 * std::sqrt((double)std::max(n, 1));
    std::printf("%s %s G=%d n=%d rotations %llu residual %.2e orth %.2e%s\n", ok ? "pass" : "FAIL", tag, G, n, rot, worst,
                orth, real_form ? "" : " (complex rotations)");
    if (!ok) ++failures;
}

// herm_q62 (a rotation coefficient to round(x 2^62), integer operations only) against long-double rounding
// on random values of every magnitude and on the edges: +-0, subnormals, values below 2^-63, ties, +-1 and
// one ulp above 1 (saturated to 2^62 - 1), and the limbs of herm_fixed_entry recombined.
void check_q62() {
    std::mt19937_64 rng(3);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::uniform_int_distribution<int> ex(-80, 0);
    std::vector<double> xs = {0.0, -0.0, 5e-324, -5e-324, 2.2e-308, 1e-300, 0x1p-63, 0x1p-64, 0x1.8p-63, -0x1.8p-63,
                              0x1p-62, 0x1.4p-62, 0.5, -0.5, 0.75, 1.0, -1.0, std::nextafter(1.0, 2.0),
                              -std::nextafter(1.0, 2.0), std::nextafter(1.0, 0.0), -std::nextafter(1.0, 0.0)};
    for (int k = 0; k < 200000; ++k) xs.push_back(std::ldexp(u(rng), ex(rng)));
    int bad = 0;
    for (double x : xs) {
        const long double lim = 4611686018427387903.0L;  // 2^62 - 1
        long double want = std::fabs((long double)x) * 4611686018427387904.0L;  // |x| 2^62
        want = want >= lim ? lim : std::floor(want + 0.5L);                  // half away from zero
        if (x < 0) want = -want;
        const long long got = herm_q62(x);
        if ((long double)got != want) {
            if (++bad <= 3) std::printf("herm_q62(%a) = %lld, want %.0Lf\n", x, got, want);
        }
        const int4 e = herm_fixed_entry(-x, x);  // S = q62(x), M = q62(x)
        const long long s = (long long)e.x * 2147483648LL + e.y, m = (long long)e.z * 2147483648LL + e.w;
        if (s != got || m != got || e.y < 0 || e.w < 0) {
            if (++bad <= 3) std::printf("herm_fixed_entry limbs of %a do not recombine\n", x);
        }
    }
    std::printf("%s q62 conversions %zu mismatches %d\n", bad ? "FAIL" : "pass", xs.size(), bad);
    if (bad) ++failures;
}

// herm_apply_real_kernel alone on synthetic sweeps of ~1.05 n^2 random rotations (c = +-1 and s = +-1
// among them), logged with herm_fixed_entry as the QL kernel logs them, against the same rotations applied
// in long double: max |Y - exact| <= 2e-16 and orthogonality <= 4e-16 n^(1/2) (the entries leave rounded to
// doubles).
void run_rotations(int n, unsigned seed) {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> ang(-3.14159, 3.14159);
    std::vector<zc> ws(eig_workspace_elems(n));
    zc* base = ws.data();
    int2* table = reinterpret_cast<int2*>(reinterpret_cast<double*>(base) + 2 * n);
    int4* log = reinterpret_cast<int4*>(base + (long long)n * n);
    int* tail = reinterpret_cast<int*>(base + 3LL * n * n);
    std::vector<double> cs;
    std::vector<int2> sweeps;
    long long pos = 0;
    const long long target = (long long)(1.05 * n * n);
    while (n > 1) {
        int l = (int)(rng() % n), m = (int)(rng() % n);
        if (l > m) std::swap(l, m);
        if (m == l) continue;
        if (pos + (m - l) > target) break;
        sweeps.push_back(make_int2(l, m - 1));
        for (int i = m - 1; i >= l; --i) {
            const double th = ang(rng);
            double c = std::cos(th), s = std::sin(th);
            switch (rng() % 50) {
                case 0: c = 1.0, s = 0.0; break;
                case 1: c = -1.0, s = 0.0; break;
                case 2: c = 0.0, s = 1.0; break;
                case 3: c = 0.0, s = -1.0; break;
                default: break;
            }
            cs.push_back(c);
            cs.push_back(s);
            log[pos++] = herm_fixed_entry(c, s);
        }
    }
    for (size_t k = 0; k < sweeps.size(); ++k) table[k] = sweeps[k];
    tail[0] = (int)sweeps.size();
    tail[1] = 0;
    int info = 0;
    std::vector<double> Y((size_t)n * n);
    apply_real(n, Y.data(), ws.data(), &info);
    std::vector<long double> X((size_t)n * n, 0.0L);  // column-major, as Y
    for (int i = 0; i < n; ++i) X[(size_t)i * n + i] = 1.0L;
    size_t p = 0;
    for (const int2& f : sweeps)
        for (int i = f.y; i >= f.x; --i, p += 2) {
            const long double c = cs[p], s = cs[p + 1];
            for (int r = 0; r < n; ++r) {
                const long double a = X[(size_t)i * n + r], b = X[(size_t)(i + 1) * n + r];
                X[(size_t)(i + 1) * n + r] = s * a + c * b;
                X[(size_t)i * n + r] = c * a - s * b;
            }
        }
    double err = 0.0, orth = 0.0;
    for (size_t k = 0; k < Y.size(); ++k) err = std::fmax(err, (double)std::fabs((long double)Y[k] - X[k]));
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            long double d = 0.0L;
            for (int r = 0; r < n; ++r) d += (long double)Y[(size_t)a * n + r] * Y[(size_t)b * n + r];
            orth = std::fmax(orth, (double)std::fabs(d - (a == b ? 1.0L : 0.0L)));
        }
    const bool ok = err <= 2e-16 && orth <= 4e-16 * std::sqrt((double)n);
    std::printf("%s rotations n=%d count %zu max |Y - exact| %.2e orth %.2e\n", ok ? "pass" : "FAIL", n, cs.size() / 2,
                err, orth);
    if (!ok) ++failures;
}

// The tridiagonalisation (herm_tridiag_one), then divide and conquer on (d, e) (herm_dc_one) for Y and the
// eigenvalues, and X = Q Y on the host; residual and orthonormality as run().
template <int G>
void run_dc(int n, const std::vector<zc>& a, const char* tag) {
    group_size = G;
    std::barrier<> b(G);
    bar = &b;
    std::vector<zc> Q((size_t)n * n), W(n), ws(eig_workspace_elems(n));
    std::vector<double> Y((size_t)n * n, -7.0);
    int info = -7;
    {
        std::vector<std::thread> th;
        for (int l = 0; l < G; ++l)
            th.emplace_back([&, l] {
                threadIdx.x = l;
                herm_tridiag_one<G>(n, a.data(), Q.data(), ws.data(), nullptr, nullptr);
            });
        for (auto& t : th) t.join();
    }
    {
        std::vector<std::thread> th;
        for (int l = 0; l < G; ++l)
            th.emplace_back([&, l] {
                threadIdx.x = l;
                herm_dc_one<G>(n, ws.data(), Y.data(), W.data(), &info, 2.220446049250313e-16, 30);
            });
        for (auto& t : th) t.join();
    }
    if (info != 0) {
        std::printf("FAIL dc %s n=%d: info %d\n", tag, n, info);
        ++failures;
        return;
    }
    std::vector<zc> V((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            zc acc{0.0, 0.0};
            for (int k = 0; k < n; ++k) acc = acc + Q[(size_t)k * n + i] * Y[(size_t)j * n + k];
            V[(size_t)j * n + i] = acc;
        }
    double fro = 0.0;
    for (const zc& z : a) fro += norm2(z);
    fro = std::sqrt(fro);
    double worst = 0.0, orth = 0.0;
    for (int j = 0; j < n; ++j) {
        double dn = 0.0, vn = 0.0;
        for (int i = 0; i < n; ++i) {
            zc acc{0.0, 0.0};
            for (int k = 0; k < n; ++k) acc = acc + a[(size_t)k * n + i] * V[(size_t)j * n + k];
            dn += norm2(acc - W[j] * V[(size_t)j * n + i]);
            vn += norm2(V[(size_t)j * n + i]);
        }
        worst = std::fmax(worst, std::sqrt(dn) / (std::fmax(fro, 1e-300) * std::sqrt(vn)));
        for (int k = 0; k < n; ++k) {
            zc dot{0.0, 0.0};
            for (int i = 0; i < n; ++i) dot = dot + conj(V[(size_t)j * n + i]) * V[(size_t)k * n + i];
            orth = std::fmax(orth, zabs(dot - zc{j == k ? 1.0 : 0.0, 0.0}));
        }
    }
    const bool ok = worst <= 1e-13 && orth <= 1e-13 * std::sqrt((double)std::max(n, 1));
    std::printf("%s dc %s G=%d n=%d residual %.2e orth %.2e\n", ok ? "pass" : "FAIL", tag, G, n, worst, orth);
    if (!ok) ++failures;
}

// The blocked reduction (herm_panel_one per panel, the trailing update and the back-transformation as
// plain host products, standing in for the device's batched products), then the same QL and rotation
// kernels as run(), and X = Q Y applied panel by panel from the stored reflectors and T V^H.
template <int G>
void run_blocked(int n, const std::vector<zc>& a, const char* tag) {
    group_size = G;
    std::barrier<> b(G);
    bar = &b;
    const int nb = kHermNb, P = herm_panel_count(n), pnb = P * nb;
    std::vector<zc> V((size_t)n * n), W(n), ws(eig_workspace_elems(n)), pan(herm_panel_elems(n)), vall((size_t)n * n),
        mall((size_t)pnb * n);
    for (int p = 0; p < P; ++p) {
        const int k0 = p * nb;
        std::vector<std::thread> th;
        for (int l = 0; l < G; ++l)
            th.emplace_back([&, l] {
                threadIdx.x = l;
                herm_panel_one<G>(n, k0, a.data(), ws.data(), pan.data(), vall.data(), mall.data(), pnb);
            });
        for (auto& t : th) t.join();
        if (k0 + nb < n - 1) {  // A(t0:, t0:) -= [V W](t0:, :) Bt(:, t0:)
            const int t0 = k0 + nb;
            const zc* VW = pan.data();
            const zc* Bt = pan.data() + 2LL * nb * n;
            for (int c = t0; c < n; ++c)
                for (int r = t0; r < n; ++r) {
                    zc acc{0.0, 0.0};
                    for (int q = 0; q < 2 * nb; ++q) acc = acc + VW[(size_t)q * n + r] * Bt[(size_t)c * 2 * nb + q];
                    ws[(size_t)c * n + r] = ws[(size_t)c * n + r] - acc;
                }
        }
    }
    int info = -7;
    unsigned long long rot = 0;
    threadIdx.x = 0;
    blockIdx.x = 0;
    blockIdx.y = 0;
    blockDim.x = kHermQlThreads;
    herm_ql_kernel<true, true>(n, 1, W.data(), &info, ws.data(), 2.220446049250313e-16, 30, &rot);
    const int* tail = reinterpret_cast<const int*>(ws.data() + 3LL * n * n);
    if (info != 0 || tail[1] != 0) {
        std::printf("FAIL blocked %s n=%d: info %d overflow %d\n", tag, n, info, tail[1]);
        ++failures;
        return;
    }
    std::vector<double> Y((size_t)n * n);
    apply_real(n, Y.data(), ws.data(), &info);
    for (size_t i = 0; i < Y.size(); ++i) V[i] = zc{Y[i], 0.0};
    for (int p = P - 1; p >= 0; --p) {  // X(r0:, :) -= V_p (M_p X(r0:, :))
        const int k0 = p * nb, nbp = std::min(nb, n - 1 - k0), r0 = k0 + 1;
        std::vector<zc> U((size_t)nb * n, zc{0.0, 0.0});
        for (int c = 0; c < n; ++c)
            for (int q = 0; q < nbp; ++q) {
                zc acc{0.0, 0.0};
                for (int r = r0; r < n; ++r) acc = acc + mall[(size_t)r * pnb + k0 + q] * V[(size_t)c * n + r];
                U[(size_t)c * nb + q] = acc;
            }
        for (int c = 0; c < n; ++c)
            for (int r = r0; r < n; ++r) {
                zc acc{0.0, 0.0};
                for (int q = 0; q < nbp; ++q) acc = acc + vall[(size_t)(k0 + q) * n + r] * U[(size_t)c * nb + q];
                V[(size_t)c * n + r] = V[(size_t)c * n + r] - acc;
            }
    }
    double fro = 0.0;
    for (const zc& z : a) fro += norm2(z);
    fro = std::sqrt(fro);
    double worst = 0.0, orth = 0.0;
    for (int j = 0; j < n; ++j) {
        double dn = 0.0, vn = 0.0;
        for (int i = 0; i < n; ++i) {
            zc acc{0.0, 0.0};
            for (int k = 0; k < n; ++k) acc = acc + a[(size_t)k * n + i] * V[(size_t)j * n + k];
            dn += norm2(acc - W[j] * V[(size_t)j * n + i]);
            vn += norm2(V[(size_t)j * n + i]);
        }
        worst = std::fmax(worst, std::sqrt(dn) / (std::fmax(fro, 1e-300) * std::sqrt(vn)));
        for (int k = 0; k < n; ++k) {
            zc dot{0.0, 0.0};
            for (int i = 0; i < n; ++i) dot = dot + conj(V[(size_t)j * n + i]) * V[(size_t)k * n + i];
            orth = std::fmax(orth, zabs(dot - zc{j == k ? 1.0 : 0.0, 0.0}));
        }
    }
    const bool ok = worst <= 1e-13 && orth <= 1e-13 * std::sqrt((double)std::max(n, 1));
    std::printf("%s blocked %s G=%d n=%d panels %d rotations %llu residual %.2e orth %.2e\n", ok ? "pass" : "FAIL", tag, G,
                n, P, rot, worst, orth);
    if (!ok) ++failures;
}

// Layer matrices of a lossless binary grating (ridge index nr, groove ng, ridge fill f of the period,
// lambda / period = lp, sin(theta) = st) at order n = 2M + 1, as the engine forms them: TE the Hermitian
// Kx^2 - [[eps]]; TM the pencil matrix L^-1 (Kx E Kx - I) L^-H with E the Hermitian part of [[eps]]^-1,
// [[1/eps]] = L L^H and L^-1 formed explicitly; coefficients made exactly conjugate-symmetric first.
static std::vector<zc> grating_coefficients(int M, double f, zc v_ridge, zc v_groove) {
    const int H = 2 * M;
    std::vector<zc> c(2 * H + 1);
    for (int h = 0; h <= H; ++h) {
        zc w;
        if (h == 0) {
            w = v_ridge * f + v_groove * (1.0 - f);
        } else {  // (1/P) integral of the profile exp(-2 pi i h x / P): ridge on [0, f P), groove after
            const double t = 2.0 * 3.14159265358979323846 * h;
            const zc e{std::cos(t * f), -std::sin(t * f)};  // exp(-i t f)
            const zc one{1.0, 0.0};
            const zc ridge = (e - one) * zc{0.0, 1.0 / t};   // (exp(-i t f) - 1) / (-i t)
            const zc groove = (one - e) * zc{0.0, 1.0 / t};
            w = v_ridge * ridge + v_groove * groove;
        }
        c[H + h] = w;
        c[H - h] = conj(w);
    }
    return c;
}

static std::vector<zc> inverse(int n, std::vector<zc> a) {  // Gauss-Jordan, partial pivoting, column-major
    std::vector<zc> x((size_t)n * n, zc{0.0, 0.0});
    for (int i = 0; i < n; ++i) x[(size_t)i * n + i] = zc{1.0, 0.0};
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (zabs(a[(size_t)k * n + i]) > zabs(a[(size_t)k * n + p])) p = i;
        for (int j = 0; j < n; ++j) {
            std::swap(a[(size_t)j * n + k], a[(size_t)j * n + p]);
            std::swap(x[(size_t)j * n + k], x[(size_t)j * n + p]);
        }
        const zc piv = a[(size_t)k * n + k];
        const zc r = zinv(piv);
        for (int j = 0; j < n; ++j) {
            a[(size_t)j * n + k] = a[(size_t)j * n + k] * r;
            x[(size_t)j * n + k] = x[(size_t)j * n + k] * r;
        }
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            const zc m = a[(size_t)k * n + i];
            if (m.re == 0.0 && m.im == 0.0) continue;
            for (int j = 0; j < n; ++j) {
                a[(size_t)j * n + i] = a[(size_t)j * n + i] - m * a[(size_t)j * n + k];
                x[(size_t)j * n + i] = x[(size_t)j * n + i] - m * x[(size_t)j * n + k];
            }
        }
    }
    return x;
}

static std::vector<zc> matmul(int n, const std::vector<zc>& a, const std::vector<zc>& b) {
    std::vector<zc> c((size_t)n * n, zc{0.0, 0.0});
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
            const zc bkj = b[(size_t)j * n + k];
            for (int i = 0; i < n; ++i) c[(size_t)j * n + i] = c[(size_t)j * n + i] + a[(size_t)k * n + i] * bkj;
        }
    return c;
}

static std::vector<zc> grating_matrix(int M, bool tm, double nr, double ng, double f, double lp, double st) {
    const int n = 2 * M + 1, H = 2 * M;
    const std::vector<zc> ce = grating_coefficients(M, f, zc{nr * nr, 0.0}, zc{ng * ng, 0.0});
    std::vector<zc> E((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) E[(size_t)j * n + i] = ce[i - j + H];
    std::vector<double> kx(n);
    for (int i = 0; i < n; ++i) kx[i] = st - (i - M) * lp;
    if (!tm) {
        for (auto& z : E) z = zc{-z.re, -z.im};
        for (int i = 0; i < n; ++i) E[(size_t)i * n + i].re += kx[i] * kx[i];
        return E;
    }
    const std::vector<zc> ci = grating_coefficients(M, f, zc{1.0 / (nr * nr), 0.0}, zc{1.0 / (ng * ng), 0.0});
    std::vector<zc> L((size_t)n * n, zc{0.0, 0.0});
    for (int j = 0; j < n; ++j)
        for (int i = j; i < n; ++i) L[(size_t)j * n + i] = ci[i - j + H];
    for (int j = 0; j < n; ++j) {  // right-looking Cholesky, as toeplitz_cholesky_kernel
        const double piv = std::sqrt(L[(size_t)j * n + j].re);
        L[(size_t)j * n + j] = zc{piv, 0.0};
        for (int i = j + 1; i < n; ++i) L[(size_t)j * n + i] = L[(size_t)j * n + i] * (1.0 / piv);
        for (int k = j + 1; k < n; ++k)
            for (int i = k; i < n; ++i)
                L[(size_t)k * n + i] = L[(size_t)k * n + i] - L[(size_t)j * n + i] * conj(L[(size_t)j * n + k]);
    }
    const std::vector<zc> Li = inverse(n, L);
    std::vector<zc> LiH((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) LiH[(size_t)j * n + i] = conj(Li[(size_t)i * n + j]);
    const std::vector<zc> Ei = inverse(n, E);
    std::vector<zc> B((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            const zc a = Ei[(size_t)j * n + i], b = Ei[(size_t)i * n + j];
            const zc h{0.5 * (a.re + b.re), 0.5 * (a.im - b.im)};
            B[(size_t)j * n + i] = h * (kx[i] * kx[j]) - zc{i == j ? 1.0 : 0.0, 0.0};
        }
    return matmul(n, Li, matmul(n, B, LiH));
}

// the general solver (CORTH + COMQR2, eig_one) with G lanes or a CTA of G threads per matrix
template <int G>
void run_general(int n, const std::vector<zc>& a, const char* tag) {
    group_size = G;
    std::barrier<> b(G);
    bar = &b;
    std::vector<zc> V((size_t)n * n), W(n), ws(eig_workspace_elems(n));
    int info = -7, sweeps = 0;
    static double red[8];
    static int ired[8];
    std::vector<std::thread> th;
    for (int l = 0; l < G; ++l)
        th.emplace_back([&, l] {
            threadIdx.x = l;
            eig_one<G>(n, a.data(), W.data(), V.data(), &info, &sweeps, ws.data(), 2.220446049250313e-16, 30, nullptr, red,
                       ired);
        });
    for (auto& t : th) t.join();
    double fro = 0.0;
    for (const zc& z : a) fro += norm2(z);
    fro = std::sqrt(fro);
    double worst = 0.0;
    for (int j = 0; j < n; ++j) {
        double dn = 0.0, vn = 0.0;
        for (int i = 0; i < n; ++i) {
            zc acc{0.0, 0.0};
            for (int k = 0; k < n; ++k) acc = acc + a[(size_t)k * n + i] * V[(size_t)j * n + k];
            dn += norm2(acc - W[j] * V[(size_t)j * n + i]);
            vn += norm2(V[(size_t)j * n + i]);
        }
        worst = std::fmax(worst, std::sqrt(dn) / (std::fmax(fro, 1e-300) * std::sqrt(vn)));
    }
    const bool ok = info == 0 && worst <= 1e-13;
    std::printf("%s general %s G=%d n=%d sweeps %d residual %.2e\n", ok ? "pass" : "FAIL", tag, G, n, sweeps, worst);
    if (!ok) ++failures;
}

int main() {
    std::setvbuf(stdout, nullptr, _IONBF, 0);
    std::mt19937_64 rng(11);
    std::normal_distribution<double> nd;
    check_q62();
    for (int n : {2, 8, 121, 301}) run_rotations(n, 5u + (unsigned)n);  // the fixed-point rotation product alone
    for (int n : {1, 2, 3, 9, 33, 61}) {
        std::vector<zc> r((size_t)n * n), t((size_t)n * n), d((size_t)n * n, zc{0.0, 0.0});
        for (int j = 0; j < n; ++j)
            for (int i = 0; i <= j; ++i) {
                const zc v{nd(rng), i == j ? 0.0 : nd(rng)};
                r[(size_t)j * n + i] = v;
                r[(size_t)i * n + j] = conj(v);
            }
        // a lossless grating's TE layer matrix Kx^2 - [[eps]] (repeated eigenvalues at kx0 = 0)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int h = i - j;
                const double kx = (i - n / 2) * 0.61;
                const zc c = h == 0 ? zc{2.2, 0.0} : zc{0.6 * std::sin(0.9 * h) / h, 0.6 * (1 - std::cos(0.9 * h)) / h};
                t[(size_t)j * n + i] = (i == j ? zc{kx * kx, 0.0} : zc{0.0, 0.0}) - c;
            }
        for (int i = 0; i < n; ++i) d[(size_t)i * n + i] = zc{(double)(i % 3), 0.0};  // repeated, already diagonal
        run<4>(n, r, "random", true, true);
        run<16>(n, r, "random", true, false);
        run<32>(n, t, "toeplitz", true, true);
        run<8>(n, t, "toeplitz", false, true);
        run<4>(n, d, "diagonal", true, true);
    }
    for (int n : {1, 2, 5, 9, 16, 17, 33, 61, 121, 162}) {  // divide and conquer, incl. repeated eigenvalues
        std::vector<zc> r((size_t)n * n), t((size_t)n * n), d((size_t)n * n, zc{0.0, 0.0}), t0((size_t)n * n);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i <= j; ++i) {
                const zc v{nd(rng), i == j ? 0.0 : nd(rng)};
                r[(size_t)j * n + i] = v;
                r[(size_t)i * n + j] = conj(v);
            }
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int h = i - j;
                const double kx = (i - n / 2) * 0.61, kx0 = (i - n / 2) * 0.61 + 0.3;
                const zc c = h == 0 ? zc{2.2, 0.0} : zc{0.6 * std::sin(0.9 * h) / h, 0.6 * (1 - std::cos(0.9 * h)) / h};
                const zc c0 = h == 0 ? zc{2.2, 0.0} : zc{0.6 * std::sin(0.9 * h) / h, 0.0};  // symmetric: degenerate at kx0
                t[(size_t)j * n + i] = (i == j ? zc{kx0 * kx0, 0.0} : zc{0.0, 0.0}) - c;
                t0[(size_t)j * n + i] = (i == j ? zc{kx * kx, 0.0} : zc{0.0, 0.0}) - c0;
            }
        for (int i = 0; i < n; ++i) d[(size_t)i * n + i] = zc{(double)(i % 3), 0.0};
        // Wilkinson's W+ (pairs of eigenvalues equal to many digits) and glued copies of one small
        // tridiagonal (clusters of nearly equal eigenvalues)
        std::vector<zc> wk((size_t)n * n, zc{0.0, 0.0}), gl((size_t)n * n, zc{0.0, 0.0});
        for (int i = 0; i < n; ++i) {
            wk[(size_t)i * n + i] = zc{std::fabs(i - (n - 1) / 2.0), 0.0};
            gl[(size_t)i * n + i] = zc{1.0 + 0.5 * std::sin((double)(i % 6)), 0.0};
            if (i + 1 < n) {
                wk[(size_t)(i + 1) * n + i] = wk[(size_t)i * n + i + 1] = zc{1.0, 0.0};
                const double off = (i % 6 == 5) ? 1e-10 : 0.7;
                gl[(size_t)(i + 1) * n + i] = gl[(size_t)i * n + i + 1] = zc{off, 0.0};
            }
        }
        run<32>(n, t0, "toeplitz-symmetric", true, true);  // the QL kernel on the clustered spectra too
        run<16>(n, wk, "wilkinson", true, true);
        run<16>(n, gl, "glued", true, false);
        run_dc<16>(n, r, "random");
        run_dc<8>(n, t, "toeplitz");
        run_dc<32>(n, t0, "toeplitz-symmetric");
        run_dc<4>(n, d, "diagonal");
        run_dc<16>(n, wk, "wilkinson");
        run_dc<16>(n, gl, "glued");
    }
    for (int n : {64, 65, 97, 121}) {  // the blocked form: full and partial last panels
        std::vector<zc> r((size_t)n * n), t((size_t)n * n);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i <= j; ++i) {
                const zc v{nd(rng), i == j ? 0.0 : nd(rng)};
                r[(size_t)j * n + i] = v;
                r[(size_t)i * n + j] = conj(v);
            }
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int h = i - j;
                const double kx = (i - n / 2) * 0.61;
                const zc c = h == 0 ? zc{2.2, 0.0} : zc{0.6 * std::sin(0.9 * h) / h, 0.6 * (1 - std::cos(0.9 * h)) / h};
                t[(size_t)j * n + i] = (i == j ? zc{kx * kx, 0.0} : zc{0.0, 0.0}) - c;
            }
        run_blocked<16>(n, r, "random");
        run_blocked<8>(n, t, "toeplitz");
    }
    {  // order 301 (M = 150), high index contrast: the CTA form a lone solve takes (128 threads), and the
       // blocked form with a warp (a few hundred matrices) or 16 lanes (thousands) per matrix
        const std::vector<zc> tm_si = grating_matrix(150, true, 3.48, 1.0, 0.37, 0.6, 0.5);
        const std::vector<zc> te_si = grating_matrix(150, false, 3.48, 1.0, 0.37, 0.6, 0.5);
        const std::vector<zc> tm_ge = grating_matrix(150, true, 4.0, 1.0, 0.5, 1.3, std::sin(85.0 * 3.14159265358979323846 / 180.0));
        run<128>(301, tm_si, "tm-pencil-n3.48", true, true);
        run_blocked<32>(301, te_si, "te-n3.48");
        run_blocked<16>(301, tm_ge, "tm-pencil-n4.0-grazing");
    }
    for (int n : {1, 2, 5, 17, 30}) {
        std::vector<zc> g((size_t)n * n);
        for (auto& z : g) z = zc{nd(rng), nd(rng)};
        run_general<4>(n, g, "random");
        run_general<32>(n, g, "random");
        run_general<64>(n, g, "random");
    }
    if (failures) {
        std::printf("%d FAILED\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
