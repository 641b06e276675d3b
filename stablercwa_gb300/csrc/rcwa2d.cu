// rcwa2d.cu -- batched 2-D (crossed-grating) solve: rcwa::solve2d over many points of one stack
// (include/stablercwa/rcwa2d.hpp:1042-1413).
//
// Per call: the Fourier operators Eps, Cx, Cy of every patterned layer (they depend on the geometry
// only) and Ei = Eps^-1 are built once on the device. Per chunk of B points, every step below is a
// batched launch over the chunk:
//   modes      homogeneous regions in 2x2 block-diagonal form; patterned layers H = P Q assembled
//              with two GEMMs each, one eigensolve launch over all patterned layers x samples, V = Q W / q;
//   bottom-up  the total reflection r below each block, Zero / block-diagonal / dense with the
//              reference's three branches (stack_on, direct_bd_over_dense, direct_dense);
//   top block  the incident interface solved for the (0,0) order only;
//   top-down   the downward amplitudes pushed through the stored steps;
//   outputs    field amplitudes, efficiencies and s/p amplitudes per order.
// The kinematics (Kx, Ky, kz, the Rayleigh check, prop flags) are evaluated on the host exactly as
// the reference does, so the branch a point takes is the reference's.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "rcwa2d_kernels.cuh"
#include "smatrix.cuh"

namespace rcwa_gb300 {
namespace {

// ============================================================== host: geometry and Fourier data

// A layer's geometry as host vectors (strip k spans y_edges[k]..y_edges[k+1] and holds the x profile
// strip_edges[k] / strip_n[k]).
struct HostLayer {
    double d = 0.0;
    bool homog = true;
    cd n{1.0, 0.0};
    std::vector<double> y_edges;
    std::vector<std::vector<double>> strip_edges;
    std::vector<std::vector<cd>> strip_n;
};

inline cd to_cd(const rcwa_complex& z) { return cd{z.re, z.im}; }

HostLayer host_layer(const rcwa_layer2d& L) {
    HostLayer h;
    h.d = L.d;
    h.homog = L.homogeneous != 0;
    h.n = to_cd(L.n);
    if (!h.homog) {
        h.y_edges.assign(L.y_edges, L.y_edges + L.n_strips + 1);
        for (int k = 0; k < L.n_strips; ++k) {
            const rcwa_xprofile2d& p = L.x_profiles[k];
            h.strip_edges.emplace_back(p.edges, p.edges + p.n_segments + 1);
            std::vector<cd> nv(p.n_segments);
            for (int s = 0; s < p.n_segments; ++s) nv[s] = to_cd(p.n_values[s]);
            h.strip_n.push_back(std::move(nv));
        }
    }
    return h;
}

LayerFourier2D layer_fourier(cudaStream_t st, DeviceScratch& mem, const HostLayer& L, double Lx, double Ly, int M1,
                             int M2, bool li) {
    return layer_fourier2d(st, mem, L.y_edges, L.strip_edges, L.strip_n, Lx, Ly, M1, M2, li);
}

zc* upload(DeviceScratch& mem, cudaStream_t st, const std::vector<cd>& v) {
    zc* d = mem.get<zc>(v.size());
    if (!v.empty()) RCWA_CUDA(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(zc), cudaMemcpyHostToDevice, st));
    return d;
}
template <class T>
T* upload_raw(DeviceScratch& mem, cudaStream_t st, const T* src, size_t count) {
    T* d = mem.get<T>(count);
    if (count) RCWA_CUDA(cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, st));
    return d;
}

struct DevOps {
    zc *eps = nullptr, *cx = nullptr, *cy = nullptr;
};

// Eps, Cx, Cy of one patterned layer on the device from its device Fourier data (consumed and freed);
// a singular inverse-rule Toeplitz matrix or a non-finite operator sets *d_flag.
DevOps device_operators(cudaStream_t st, DeviceScratch& mem, LayerFourier2D F, int M1, int M2, bool li, int* d_flag) {
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2;
    const long long NN = (long long)N * N;
    DevOps o;
    o.eps = mem.get<zc>(NN);
    LAUNCH(op_eps_kernel, nblocks(NN), kTpb, st, M1, M2, F.K, F.wy, F.ce, o.eps);
    if (!li) {
        o.cx = o.eps;
        o.cy = o.eps;
    } else {
        zc* tx = mem.get<zc>((size_t)F.K * n1 * n1);
        zc* invx = mem.get<zc>((size_t)F.K * n1 * n1);
        int* sing = mem.zeros<int>(F.K);
        LAUNCH(toeplitz_batch_kernel, nblocks((long long)F.K * n1 * n1), kTpb, st, F.K, M1, F.ci, tx);
        launch_lu_solve(st, n1, n1, F.K, tx, (long long)n1 * n1, tx, (long long)n1 * n1, RHS_IDENTITY, nullptr, 0, invx,
                        (long long)n1 * n1, sing);
        LAUNCH(any_set_kernel, nblocks(F.K), kTpb, st, F.K, sing, d_flag);
        o.cx = mem.get<zc>(NN);
        LAUNCH(op_cx_kernel, nblocks(NN), kTpb, st, M1, M2, F.K, F.wy, invx, o.cx);

        zc* ty = mem.get<zc>((size_t)F.Kx * n2 * n2);
        zc* invy = mem.get<zc>((size_t)F.Kx * n2 * n2);
        int* sing_y = mem.zeros<int>(F.Kx);
        LAUNCH(toeplitz_batch_kernel, nblocks((long long)F.Kx * n2 * n2), kTpb, st, F.Kx, M2, F.cyc, ty);
        launch_lu_solve(st, n2, n2, F.Kx, ty, (long long)n2 * n2, ty, (long long)n2 * n2, RHS_IDENTITY, nullptr, 0, invy,
                        (long long)n2 * n2, sing_y);
        LAUNCH(any_set_kernel, nblocks(F.Kx), kTpb, st, F.Kx, sing_y, d_flag);
        o.cy = mem.get<zc>(NN);
        LAUNCH(op_cy_kernel, nblocks(NN), kTpb, st, M1, M2, F.Kx, F.wx, invy, o.cy);
        for (void* p : {(void*)tx, (void*)invx, (void*)sing, (void*)ty, (void*)invy, (void*)sing_y}) mem.free(p);
    }
    free_layer_fourier2d(mem, F);
    for (zc* m : {o.eps, o.cx, o.cy}) LAUNCH(any_nonfinite_kernel, nblocks(NN), kTpb, st, NN, m, d_flag);
    return o;
}

// ============================================================== host: kinematics (rcwa2d.hpp:1074-1113)

// kz/k0 = sqrt(n^2 - Kx^2 - Ky^2), Im < 0 flipped (kz_over_k0, rcwa2d.hpp:376-381)
cd kz_over_k0(cd n, double Kx, double Ky) {
    const cd s = n * n - Kx * Kx - Ky * Ky;
    cd kz = std::sqrt(s);
    if (kz.imag() < 0.0) kz = -kz;
    return kz;
}

struct Point2D {
    double k0, th, ph, cos_th, sin_th, cos_ph, sin_ph;
    cd e_x, e_y;  // incident Ex, Ey of the (0,0) order
};

Point2D point_setup(const rcwa_point2d& p) {
    Point2D q;
    q.k0 = 2.0 * kPiD / p.wavelength;
    q.th = p.theta_deg * (kPiD / 180.0);
    q.ph = p.phi_deg * (kPiD / 180.0);
    q.cos_th = std::cos(q.th);
    q.sin_th = std::sin(q.th);
    q.cos_ph = std::cos(q.ph);
    q.sin_ph = std::sin(q.ph);
    const cd Es = to_cd(p.Es), Ep = to_cd(p.Ep);
    q.e_x = -Es * q.sin_ph + Ep * q.cos_th * q.cos_ph;
    q.e_y = Es * q.cos_ph + Ep * q.cos_th * q.sin_ph;
    return q;
}

// ============================================================== device regions and steps

struct Region {
    bool homog = true;
    zc* q = nullptr;   // B x 2N
    zc* vb = nullptr;  // B x 4N (homogeneous)
    zc* W = nullptr;   // B x n x n (patterned)
    zc* V = nullptr;
};

enum RKind { R_ZERO = 0, R_BD = 1, R_DENSE = 2 };
struct RState {
    RKind kind = R_ZERO;
    zc* p = nullptr;
    bool owned = false;  // freed when replaced (otherwise a step owns it)
};

enum SKind { S_NONE = 0, S_BDMAT = 1, S_IFACE_DENSE = 2, S_IFACE_BD = 3 };
struct Step {
    SKind kind = S_NONE;
    zc *bd = nullptr, *tm = nullptr, *nn = nullptr, *rp = nullptr;
};

void replace_r(DeviceScratch& mem, RState& r, RState next) {
    if (r.owned && r.p) mem.free(r.p);
    r = next;
}

// The field harmonics of one chunk (sample_field_2d, include/stablercwa/rcwa2d_fields.hpp:282-320): depths
// grouped like field_region_2d (:117-124: z < 0 region I, z > z_bot region II, else the first layer with
// z <= z_top + d + 1e-12, zero-thickness layers included), S and D per layer group, W S and V D for
// patterned layers (block-diagonal V for homogeneous ones), the six components, Ez through Ei = Eps^-1
// or 1/eps. The result goes to out (device, B x 6 x N x nz); failed samples get NaN.
struct Capture2D {
    std::vector<zc*> W, V;            // retained modes of the patterned layers
    std::vector<RState> r_below;      // reflection below each layer (deep copies)
    std::vector<zc*> a_plus, a_minus;  // B x 2N per layer
};

void sample_fields2d(Batch& c, const std::vector<double>& zs, const std::vector<HostLayer>& layers, double nI, cd nII,
                     int N, int i0, const std::vector<Region>& reg, const Capture2D& cap, const std::vector<int>& patterned,
                     const std::vector<zc*>& Ei, const zc* inc, const zc* R, const zc* T, const double* dKx, const double* dKy,
                     const double* dk0, zc* out) {
    const cudaStream_t st = c.st;
    DeviceScratch& mem = *c.mem;
    const int B = c.B, n = 2 * N, L = (int)layers.size(), nz = (int)zs.size();
    const long long nn = (long long)n * n;
    std::vector<double> ztop(L);
    double z = 0.0;
    for (int j = 0; j < L; ++j) {
        ztop[j] = z;
        z += layers[j].d;
    }
    const double zb = z;
    std::vector<std::vector<int>> groups(L + 2);  // 0 region I, 1 region II, 2 + j layer j
    for (int iz = 0; iz < nz; ++iz) {
        const double zz = zs[iz];
        int g = 1;
        if (zz < 0.0) {
            g = 0;
        } else if (!(zz > zb)) {
            for (int j = 0; j < L; ++j)
                if (zz <= ztop[j] + layers[j].d + 1e-12) {
                    g = 2 + j;
                    break;
                }
        }
        groups[g].push_back(iz);
    }
    std::vector<int> ei_of(L, -1);
    for (size_t k = 0; k < patterned.size(); ++k) ei_of[patterned[k]] = (int)k;
    zc* scale = mem.get<zc>(1);
    for (int g = 0; g < L + 2; ++g) {
        const std::vector<int>& cols = groups[g];
        if (cols.empty()) continue;
        const int cnt = (int)cols.size();
        const long long tot = (long long)B * n * cnt, totN = (long long)B * N * cnt;
        std::vector<double> local(cnt);
        for (int k = 0; k < cnt; ++k) local[k] = g >= 2 ? zs[cols[k]] - ztop[g - 2] : zs[cols[k]];
        double* d_z = mem.get<double>(cnt);
        int* d_cols = mem.get<int>(cnt);
        RCWA_CUDA(cudaMemcpyAsync(d_z, local.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(d_cols, cols.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, st));
        zc* F = mem.get<zc>(tot);
        zc* G = mem.get<zc>(tot);
        const zc* ei = nullptr;
        cd ie{0.0, 0.0};
        if (g < 2) {
            const Region& m = g == 0 ? reg[0] : reg[L + 1];
            LAUNCH(fields2d_region_kernel, nblocks(totN), kTpb, st, B, N, i0, cnt, d_z, g == 0 ? -1 : -2, zb, dk0, m.q, m.vb,
                   inc, g == 0 ? R : T, F, G);
            ie = g == 0 ? cd{1.0 / (nI * nI), 0.0} : cd{1.0, 0.0} / (nII * nII);
        } else {
            const int j = g - 2;
            const Region& m = reg[j + 1];
            zc* S = mem.get<zc>(tot);
            zc* D = mem.get<zc>(tot);
            LAUNCH(fields2d_layer_kernel, nblocks(tot), kTpb, st, B, n, cnt, d_z, layers[j].d, dk0, cap.a_plus[j],
                   cap.a_minus[j], m.q, S, D);
            if (m.homog) {
                RCWA_CUDA(cudaMemcpyAsync(F, S, tot * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                LAUNCH(bd_rows_kernel, nblocks(totN), kTpb, st, B, N, cnt, m.vb, D, G);
                ie = cd{1.0, 0.0} / (layers[j].n * layers[j].n);
            } else {
                launch_zgemm(st, n, cnt, n, B, cap.W[j], n, nn, S, n, (long long)n * cnt, nullptr, 0, F, n, (long long)n * cnt,
                             1.0, 0.0);
                launch_zgemm(st, n, cnt, n, B, cap.V[j], n, nn, D, n, (long long)n * cnt, nullptr, 0, G, n, (long long)n * cnt,
                             1.0, 0.0);
                ei = Ei[ei_of[j]];
            }
            mem.free(S);
            mem.free(D);
        }
        zc* t = mem.get<zc>(totN);
        LAUNCH(fields2d_out_kernel, nblocks(totN), kTpb, st, B, N, cnt, nz, d_cols, dKx, dKy, F, G, t, out);
        if (ei) {
            zc* e = mem.get<zc>(totN);
            launch_zgemm(st, N, cnt, N, B, ei, N, 0, t, N, (long long)N * cnt, nullptr, 0, e, N, (long long)N * cnt, 1.0, 0.0);
            LAUNCH(fields2d_ez_kernel, nblocks(totN), kTpb, st, B, N, cnt, nz, d_cols, e, nullptr, out);
            RCWA_CUDA(stream_wait(st));
            mem.free(e);
        } else {
            const zc hs{ie.real(), ie.imag()};
            RCWA_CUDA(cudaMemcpyAsync(scale, &hs, sizeof(zc), cudaMemcpyHostToDevice, st));
            LAUNCH(fields2d_ez_kernel, nblocks(totN), kTpb, st, B, N, cnt, nz, d_cols, t, scale, out);
            RCWA_CUDA(stream_wait(st));  // the host values of this group end here
        }
        for (void* p : {(void*)F, (void*)G, (void*)t, (void*)d_z, (void*)d_cols}) mem.free(p);
    }
    mem.free(scale);
    LAUNCH(nan_fields2d_kernel, nblocks((long long)B * 6 * N * nz), kTpb, st, B, 6LL * N * nz, c.fail, out);
}

}  // namespace

// ============================================================== validation (rcwa2d.hpp:928-1006, rcwa2d_operators.hpp:252-320)

namespace {
[[noreturn]] void invalid2d(const std::string& what) { throw EngineError{RCWA_EINVAL, "rcwa2d: " + what}; }
bool finite_c(const rcwa_complex& z) { return std::isfinite(z.re) && std::isfinite(z.im); }
void check_index_2d(const rcwa_complex& n, const char* what) {
    if (!finite_c(n) || std::abs(to_cd(n)) == 0.0 || n.re < 0.0 || n.im < 0.0)
        invalid2d(std::string(what) + " must be finite, nonzero, with Re n >= 0 and Im n >= 0");
}
void check_edge_list(const double* e, int count, double period, const char* what) {
    if (!e || count < 2) invalid2d(std::string(what) + " need at least two entries");
    for (int j = 0; j < count; ++j)
        if (!std::isfinite(e[j]) || (j > 0 && e[j] <= e[j - 1]))
            invalid2d(std::string(what) + " must be finite and strictly increasing");
    if (std::abs((e[count - 1] - e[0]) - period) > 1e-9 * period) invalid2d(std::string(what) + " must span exactly one period");
}
}  // namespace

void validate2d(const rcwa_stack2d& stack, const rcwa_point2d* points, int n_points, int M1, int M2, int factorization) {
    const long long limit = ((std::numeric_limits<int>::max)() - 1) / 4;
    if (M1 < 0 || M2 < 0 || M1 > limit || M2 > limit || (2LL * M1 + 1) * (2LL * M2 + 1) > limit)
        invalid2d("invalid truncation order M1, M2");
    if (factorization != RCWA_FACTORIZATION_LI && factorization != RCWA_FACTORIZATION_LAURENT)
        invalid2d("unknown factorization");
    if (!std::isfinite(stack.Lx) || stack.Lx <= 0.0 || !std::isfinite(stack.Ly) || stack.Ly <= 0.0)
        invalid2d("wavelength and periods must be finite and positive");
    if (!std::isfinite(stack.nI) || stack.nI <= 0.0) invalid2d("the incident medium must have a real positive index");
    check_index_2d(stack.nII, "exit-medium index");
    if (stack.n_layers < 0 || (stack.n_layers > 0 && !stack.layers)) invalid2d("layers missing");
    for (int j = 0; j < stack.n_layers; ++j) {
        const rcwa_layer2d& L = stack.layers[j];
        if (!std::isfinite(L.d) || L.d < 0.0) invalid2d("layer thickness must be finite and >= 0");
        if (L.homogeneous) {
            check_index_2d(L.n, "layer index");
            continue;
        }
        if (L.n_strips < 1 || !L.x_profiles || !L.y_edges) invalid2d("a patterned layer needs K x-profiles and K+1 y-edges");
        check_edge_list(L.y_edges, L.n_strips + 1, stack.Ly, "y-edges");
        for (int k = 0; k < L.n_strips; ++k) {
            const rcwa_xprofile2d& p = L.x_profiles[k];
            if (p.n_segments < 1 || !p.n_values || !p.edges) invalid2d("an x-profile needs K indices and K+1 edges");
            check_edge_list(p.edges, p.n_segments + 1, stack.Lx, "x-edges");
            for (int s = 0; s < p.n_segments; ++s) {
                check_index_2d(p.n_values[s], "profile index");
                const cd n = to_cd(p.n_values[s]), eps = n * n;
                if (!std::isfinite(eps.real()) || !std::isfinite(eps.imag())) invalid2d("epsilon = n^2 overflows");
                if (eps == cd{}) invalid2d("epsilon = n^2 is zero");
                const cd inv = cd{1.0, 0.0} / eps;
                if (!std::isfinite(inv.real()) || !std::isfinite(inv.imag())) invalid2d("1/epsilon overflows");
            }
        }
    }
    for (int p = 0; p < n_points; ++p) {
        const rcwa_point2d& q = points[p];
        if (!std::isfinite(q.wavelength) || q.wavelength <= 0.0) invalid2d("wavelength and periods must be finite and positive");
        if (!std::isfinite(q.theta_deg) || std::abs(q.theta_deg) >= 90.0)
            invalid2d("incidence angle must lie strictly between -90 and 90 degrees");
        if (!std::isfinite(q.phi_deg)) invalid2d("azimuth angle must be finite");
        if (!finite_c(q.Es) || !finite_c(q.Ep)) invalid2d("the Jones vector must be finite");
    }
}

void layer_operators2d(cudaStream_t st, const rcwa_layer2d& layer, double Lx, double Ly, int M1, int M2,
                       int factorization, rcwa_complex* eps, rcwa_complex* cx, rcwa_complex* cy, int* singular) {
    rcwa_stack2d one{1.0, rcwa_complex{1.0, 0.0}, Lx, Ly, 1, &layer};
    validate2d(one, nullptr, 0, M1, M2, factorization);
    const int N = (2 * M1 + 1) * (2 * M2 + 1);
    const size_t NN = (size_t)N * N;
    if (layer.homogeneous) {  // n^2 I three times (rcwa2d_operators.hpp:333-343)
        const cd e = to_cd(layer.n) * to_cd(layer.n);
        for (rcwa_complex* m : {eps, cx, cy}) {
            if (!m) continue;
            std::memset(m, 0, NN * sizeof(rcwa_complex));
            for (int i = 0; i < N; ++i) m[(size_t)i * N + i] = rcwa_complex{e.real(), e.imag()};
        }
        if (singular) *singular = 0;
        return;
    }
    DeviceScratch mem(st);
    const bool li = factorization == RCWA_FACTORIZATION_LI;
    int* flag = mem.zeros<int>(1);
    const DevOps o = device_operators(st, mem, layer_fourier(st, mem, host_layer(layer), Lx, Ly, M1, M2, li), M1, M2, li, flag);
    if (eps) RCWA_CUDA(cudaMemcpyAsync(eps, o.eps, NN * sizeof(zc), cudaMemcpyDeviceToHost, st));
    if (cx) RCWA_CUDA(cudaMemcpyAsync(cx, o.cx, NN * sizeof(zc), cudaMemcpyDeviceToHost, st));
    if (cy) RCWA_CUDA(cudaMemcpyAsync(cy, o.cy, NN * sizeof(zc), cudaMemcpyDeviceToHost, st));
    int h_flag = 0;
    RCWA_CUDA(cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    if (singular) *singular = h_flag;
}

// ============================================================== the solve

void solve2d_host(cudaStream_t st, const rcwa_stack2d& stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                  int factorization, const Options& opt, const rcwa_result2d& out, size_t chunk_bytes,
                  const FieldSpec* fields) {
    const Fp64ProductsGuard fp64_products;
    const int n1 = 2 * M1 + 1, n2 = 2 * M2 + 1, N = n1 * n2, n = 2 * N;
    const long long NN = (long long)N * N, nn = (long long)n * n;
    const int L = stack.n_layers;
    const int i0 = M1 * n2 + M2;
    const double nI = stack.nI;
    const cd nII = to_cd(stack.nII);
    const bool li = factorization == RCWA_FACTORIZATION_LI;

    std::vector<HostLayer> layers;
    for (int j = 0; j < L; ++j) layers.push_back(host_layer(stack.layers[j]));
    std::vector<int> patterned;  // layer indices with dense modes
    for (int j = 0; j < L; ++j)
        if (!layers[j].homog) patterned.push_back(j);
    const int P = (int)patterned.size();

    // ---- kinematics and the Rayleigh check, every point (host, the reference's arithmetic)
    std::vector<Point2D> pt(n_points);
    std::vector<int> valid;
    std::vector<double> hKx((size_t)n_points * N), hKy((size_t)n_points * N);
    std::vector<cd> hkzI((size_t)n_points * N), hkzII((size_t)n_points * N);
    const int n_regions = L + 2;
    for (int p = 0; p < n_points; ++p) {
        pt[p] = point_setup(points[p]);
        const Point2D& q = pt[p];
        const double wl = points[p].wavelength;
        bool rayleigh = false;
        std::vector<unsigned char> reg(n_regions, 0);
        for (int a = 0; a < n1; ++a)
            for (int b = 0; b < n2; ++b) {
                const size_t i = (size_t)a * n2 + b, k = (size_t)p * N + i;
                const int m = a - M1, nn_ = b - M2;
                hKx[k] = nI * q.sin_th * q.cos_ph - m * wl / stack.Lx;
                hKy[k] = nI * q.sin_th * q.sin_ph - nn_ * wl / stack.Ly;
                hkzI[k] = kz_over_k0(cd{nI, 0.0}, hKx[k], hKy[k]);
                hkzII[k] = kz_over_k0(nII, hKx[k], hKy[k]);
                if (hkzI[k] == cd{}) reg[0] = 1;
                if (hkzII[k] == cd{}) reg[L + 1] = 1;
                for (int j = 0; j < L; ++j)
                    if (layers[j].homog && kz_over_k0(layers[j].n, hKx[k], hKy[k]) == cd{}) reg[j + 1] = 1;
            }
        for (unsigned char r : reg) rayleigh = rayleigh || r;
        if (out.rayleigh_regions) std::memcpy(out.rayleigh_regions + (size_t)p * n_regions, reg.data(), n_regions);
        if (rayleigh) {
            out.status[p] = RCWA_SAMPLE_RAYLEIGH;
            if (out.eig_info) out.eig_info[p] = 0;
            if (out.n_eig) out.n_eig[p] = 0;
            if (out.n_dense_solve) out.n_dense_solve[p] = 0;
        } else {
            valid.push_back(p);
        }
        if (out.max_eig_residual) out.max_eig_residual[p] = 0.0;
    }
    std::memcpy(out.Kx, hKx.data(), hKx.size() * sizeof(double));
    std::memcpy(out.Ky, hKy.data(), hKy.size() * sizeof(double));
    std::memcpy(out.kzI, hkzI.data(), hkzI.size() * sizeof(cd));
    std::memcpy(out.kzII, hkzII.data(), hkzII.size() * sizeof(cd));
    for (size_t k = 0; k < hkzI.size(); ++k) {
        out.prop_r[k] = hkzI[k].real() > 1e-12;
        out.prop_t[k] = hkzII[k].real() > 1e-12;
    }
    const double nan = std::numeric_limits<double>::quiet_NaN();
    auto nan_point = [&](int p) {
        const rcwa_complex cn{nan, nan};
        for (rcwa_complex* a : {out.Ex_r, out.Ey_r, out.Ez_r, out.Ex_t, out.Ey_t, out.Ez_t, out.Rs, out.Rp, out.Ts, out.Tp})
            for (int i = 0; i < N; ++i) a[(size_t)p * N + i] = cn;
        for (int i = 0; i < N; ++i) {
            out.DEr[(size_t)p * N + i] = nan;
            out.DEt[(size_t)p * N + i] = nan;
        }
    };
    const int nz = fields ? (int)fields->zs.size() : 0;
    const size_t fper = (size_t)6 * N * nz;  // field values per point
    auto nan_fields = [&](int p) {
        if (nz == 0) return;
        zc* f = fields->out + (size_t)p * fper;
        for (size_t k = 0; k < fper; ++k) f[k] = zc{nan, nan};
    };
    for (int p = 0; p < n_points; ++p)
        if (out.status[p] == RCWA_SAMPLE_RAYLEIGH) {
            nan_point(p);
            nan_fields(p);
        }
    if (valid.empty()) return;

    DeviceScratch call_mem(st);  // per-call data: operators and Ei

    // ---- operators and Ei = Eps^-1 of every patterned layer, once per call
    int* op_flag = call_mem.zeros<int>(1);
    std::vector<DevOps> ops(P);
    std::vector<zc*> Ei(P);
    for (int k = 0; k < P; ++k) {
        const HostLayer& hl = layers[patterned[k]];
        ops[k] = device_operators(st, call_mem, layer_fourier(st, call_mem, hl, stack.Lx, stack.Ly, M1, M2, li), M1, M2, li,
                                  op_flag);
        int* sing = call_mem.zeros<int>(1);
        Ei[k] = call_mem.get<zc>(NN);
        zc* tmp = call_mem.get<zc>(NN);
        launch_lu_solve(st, N, N, 1, ops[k].eps, NN, tmp, NN, RHS_IDENTITY, nullptr, 0, Ei[k], NN, sing);
        LAUNCH(any_set_kernel, 1, 32, st, 1, sing, op_flag);
        LAUNCH(any_nonfinite_kernel, nblocks(NN), kTpb, st, NN, Ei[k], op_flag);
        call_mem.free(tmp);
        call_mem.free(sing);
    }
    int h_op_flag = 0;
    RCWA_CUDA(cudaMemcpyAsync(&h_op_flag, op_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    if (h_op_flag) {  // operators or Ei singular / non-finite: every point fails (rcwa2d.hpp:412-418, :1394-1403)
        for (int p : valid) {
            out.status[p] = RCWA_SAMPLE_NUMERICAL;
            if (out.eig_info) out.eig_info[p] = 0;
            if (out.n_eig) out.n_eig[p] = P;
            if (out.n_dense_solve) out.n_dense_solve[p] = 0;
            if (out.max_eig_residual) out.max_eig_residual[p] = 0.0;
            nan_point(p);
            nan_fields(p);
        }
        return;
    }

    // ---- chunk size from a per-point estimate of the device working set
    double per_point = 16.0 * (double)nn * (5.0 * P + 3.0 * (L + 1) + 8.0) + 64.0 * N * (L + 8);
    if (nz > 0)  // retained W, V and reflections, amplitudes, the field output and one depth group's buffers
        per_point += 16.0 * ((double)nn * (2.0 * P + L) + 4.0 * n * L + 12.0 * (double)N * nz);
    const int B_max = (int)std::max(1.0, std::min((double)valid.size(), (double)chunk_bytes / per_point));

    for (size_t start = 0; start < valid.size(); start += B_max) {
        const int B = (int)std::min<size_t>(B_max, valid.size() - start);
        const int* idx = valid.data() + start;
        DeviceScratch mem(st);  // everything of this chunk, released when the chunk ends
        // per-point host data of the chunk
        std::vector<double> cKx((size_t)B * N), cKy((size_t)B * N), ck0(B), cnic(B), csin(B), ccos(B);
        std::vector<cd> ckzI((size_t)B * N), ckzII((size_t)B * N), ce2((size_t)2 * B);
        for (int b = 0; b < B; ++b) {
            const int p = idx[b];
            std::memcpy(&cKx[(size_t)b * N], &hKx[(size_t)p * N], N * sizeof(double));
            std::memcpy(&cKy[(size_t)b * N], &hKy[(size_t)p * N], N * sizeof(double));
            std::memcpy(&ckzI[(size_t)b * N], &hkzI[(size_t)p * N], N * sizeof(cd));
            std::memcpy(&ckzII[(size_t)b * N], &hkzII[(size_t)p * N], N * sizeof(cd));
            ck0[b] = pt[p].k0;
            cnic[b] = nI * pt[p].cos_th;
            csin[b] = pt[p].sin_ph;
            ccos[b] = pt[p].cos_ph;
            ce2[2 * b] = pt[p].e_x;
            ce2[2 * b + 1] = pt[p].e_y;
        }
        double* dKx = upload_raw(mem, st, cKx.data(), cKx.size());
        double* dKy = upload_raw(mem, st, cKy.data(), cKy.size());
        double* dk0 = upload_raw(mem, st, ck0.data(), ck0.size());
        double* dnic = upload_raw(mem, st, cnic.data(), cnic.size());
        double* dsin = upload_raw(mem, st, csin.data(), csin.size());
        double* dcos = upload_raw(mem, st, ccos.data(), ccos.size());
        zc* dkzI = upload(mem, st, ckzI);
        zc* dkzII = upload(mem, st, ckzII);
        zc* de2 = upload(mem, st, ce2);
        int* fail = mem.zeros<int>(B);
        int* eig_info = mem.zeros<int>(B);
        double* resid = mem.zeros<double>(B);
        Batch c{st, &mem, B, n, 0, fail, nullptr};

        // ---- modes of every region
        std::vector<Region> reg(n_regions);
        auto homog_region = [&](Region& r, const zc* kz, cd idx_n) {
            r.homog = true;
            r.q = mem.get<zc>((size_t)B * n);
            r.vb = mem.get<zc>((size_t)B * 4 * N);
            const cd n2c = idx_n * idx_n;
            LAUNCH(homog_modes_kernel, nblocks((long long)B * N), kTpb, st, B, N, kz, zc{n2c.real(), n2c.imag()}, dKx, dKy,
                   r.q, r.vb);
        };
        homog_region(reg[0], dkzI, cd{nI, 0.0});
        homog_region(reg[L + 1], dkzII, nII);
        for (int j = 0; j < L; ++j) {
            if (!layers[j].homog) continue;
            std::vector<cd> kz((size_t)B * N);
            for (int b = 0; b < B; ++b)
                for (int i = 0; i < N; ++i)
                    kz[(size_t)b * N + i] = kz_over_k0(layers[j].n, cKx[(size_t)b * N + i], cKy[(size_t)b * N + i]);
            zc* dkz = upload(mem, st, kz);
            homog_region(reg[j + 1], dkz, layers[j].n);
            mem.free(dkz);
        }

        if (P > 0) {
            // H = P Q of every patterned layer, then one eigensolve launch over layers x points
            zc* Hall = mem.get<zc>((size_t)P * B * nn);
            for (int k = 0; k < P; ++k) {
                zc* pc1 = mem.get<zc>((size_t)B * 2 * NN);
                zc* pc2 = mem.get<zc>((size_t)B * 2 * NN);
                zc* q12 = mem.get<zc>((size_t)B * NN);
                zc* q21 = mem.get<zc>((size_t)B * NN);
                LAUNCH(pc_kernel, nblocks((long long)B * NN), kTpb, st, B, N, Ei[k], dKx, dKy, pc1, pc2);
                LAUNCH(q_blocks_kernel, nblocks((long long)B * NN), kTpb, st, B, N, ops[k].cx, ops[k].cy, dKx, dKy, q12, q21);
                zc* t1 = mem.get<zc>((size_t)B * 2 * NN);
                zc* t2 = mem.get<zc>((size_t)B * 2 * NN);
                launch_zgemm(st, n, N, N, B, pc2, n, 2 * NN, q21, N, NN, nullptr, 0, t1, n, 2 * NN, 1.0, 0.0);
                launch_zgemm(st, n, N, N, B, pc1, n, 2 * NN, q12, N, NN, nullptr, 0, t2, n, 2 * NN, 1.0, 0.0);
                LAUNCH(h_assemble_kernel, nblocks((long long)B * 2 * NN), kTpb, st, B, N, t1, t2, pc1, pc2, dKx, dKy,
                       Hall + (size_t)k * B * nn);
                for (zc* p : {pc1, pc2, q12, q21, t1, t2}) mem.free(p);
            }
            const long long PB = (long long)P * B;
            zc* wall = mem.get<zc>((size_t)PB * n);
            zc* Wall = mem.get<zc>((size_t)PB * nn);
            int* info = mem.zeros<int>(PB);
            zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(n, (int)PB) / sizeof(zc)) + 1);
            launch_eig(st, n, (int)PB, Hall, nn, wall, Wall, info, nullptr, ws, opt.eps, opt.max_iter, opt.eig_group);
            mem.free(ws);
            if (opt.diagnostics) {  // eig_residual of each H (rcwa2d.hpp:497)
                zc* av = mem.get<zc>((size_t)PB * nn);
                launch_zgemm(st, n, n, n, (int)PB, Hall, n, nn, Wall, n, nn, nullptr, 0, av, n, nn, 1.0, 0.0);
                for (int k = 0; k < P; ++k)
                    LAUNCH(eig_residual_kernel, warp_blocks(B), 128, st, B, n, Hall + (size_t)k * B * nn,
                           av + (size_t)k * B * nn, Wall + (size_t)k * B * nn, wall + (size_t)k * B * n, info + (size_t)k * B,
                           resid);
                mem.free(av);
            }
            mem.free(Hall);
            LAUNCH(eig_info_layers_kernel, nblocks(B), kTpb, st, B, P, info, eig_info, fail);
            zc* qall = mem.get<zc>((size_t)PB * n);
            LAUNCH(q_from_values_kernel, nblocks(PB * n), kTpb, st, PB * n, wall, qall);
            mem.free(wall);
            mem.free(info);
            zc* Vall = mem.get<zc>((size_t)PB * nn);
            for (int k = 0; k < P; ++k) {
                zc* W = Wall + (size_t)k * B * nn;
                zc* V = Vall + (size_t)k * B * nn;
                zc* q12 = mem.get<zc>((size_t)B * NN);
                zc* q21 = mem.get<zc>((size_t)B * NN);
                LAUNCH(q_blocks_kernel, nblocks((long long)B * NN), kTpb, st, B, N, ops[k].cx, ops[k].cy, dKx, dKy, q12, q21);
                zc* top = mem.get<zc>((size_t)B * N * n);
                zc* bot = mem.get<zc>((size_t)B * N * n);
                launch_zgemm(st, N, n, N, B, q12, N, NN, W + N, n, nn, nullptr, 0, top, N, (long long)N * n, 1.0, 0.0);
                launch_zgemm(st, N, n, N, B, q21, N, NN, W, n, nn, nullptr, 0, bot, N, (long long)N * n, 1.0, 0.0);
                LAUNCH(v_assemble_kernel, nblocks((long long)B * N * n), kTpb, st, B, N, top, bot, W,
                       qall + (size_t)k * B * n, dKx, dKy, V);
                for (zc* p : {q12, q21, top, bot}) mem.free(p);
                LAUNCH(finite_check_kernel, nblocks((long long)B * nn), kTpb, st, B, nn, W, fail);
                LAUNCH(finite_check_kernel, nblocks((long long)B * nn), kTpb, st, B, nn, V, fail);
                Region& r = reg[patterned[k] + 1];
                r.homog = false;
                r.q = qall + (size_t)k * B * n;
                r.W = W;
                r.V = V;
            }
            // Wall / Vall / qall stay allocated until the chunk ends; the per-layer views are released with them
            (void)Vall;
        }
        Capture2D cap;
        if (nz > 0) {  // the interface above a layer consumes its W and V; the field sampler needs them after
            cap.W.assign(L, nullptr);
            cap.V.assign(L, nullptr);
            cap.r_below.assign(L, RState{});
            cap.a_plus.assign(L, nullptr);
            cap.a_minus.assign(L, nullptr);
            for (int j : patterned) {
                cap.W[j] = c.dense();
                cap.V[j] = c.dense();
                RCWA_CUDA(cudaMemcpyAsync(cap.W[j], reg[j + 1].W, (size_t)B * nn * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                RCWA_CUDA(cudaMemcpyAsync(cap.V[j], reg[j + 1].V, (size_t)B * nn * sizeof(zc), cudaMemcpyDeviceToDevice, st));
            }
        }

        // ---- bottom-up (rcwa2d.hpp:1176-1197)
        const int blocks = 2 * L + 1;
        std::vector<Step> steps(blocks);
        RState r;
        for (int b = blocks - 1; b >= 1; --b) {
            const int j = b / 2;
            if (b % 2 == 0) {
                const Region& up = reg[j];
                Region& low = reg[j + 1];
                if (up.homog && low.homog) {
                    if (r.kind != R_DENSE) {
                        zc* rout = mem.get<zc>((size_t)B * 4 * N);
                        zc* gt = mem.get<zc>((size_t)B * 4 * N);
                        LAUNCH(iface_bd_kernel, nblocks((long long)B * N), kTpb, st, B, N, up.vb, low.vb,
                               r.kind == R_BD ? r.p : nullptr, rout, gt);
                        steps[b] = Step{S_BDMAT, gt};
                        replace_r(mem, r, RState{R_BD, rout, true});
                    } else {  // direct_bd_over_dense (rcwa2d.hpp:791-809)
                        zc* vnn = mem.get<zc>((size_t)B * 4 * N);
                        zc* np1 = mem.get<zc>((size_t)B * 4 * N);
                        zc* nm1 = mem.get<zc>((size_t)B * 4 * N);
                        zc* tmb = mem.get<zc>((size_t)B * 4 * N);
                        LAUNCH(bd_over_dense_prep_kernel, nblocks((long long)B * N), kTpb, st, B, N, up.vb, low.vb, vnn, np1,
                               nm1, tmb);
                        zc* ap = c.dense();
                        zc* am = c.dense();
                        LAUNCH(rmul_bd_kernel, nblocks((long long)B * n * N), kTpb, st, B, N, r.p, nm1, 0, np1, ap);
                        LAUNCH(rmul_bd_kernel, nblocks((long long)B * n * N), kTpb, st, B, N, r.p, np1, 0, nm1, am);
                        zc* x = solve(c, ap, true, RHS_DENSE, am);
                        for (zc* p : {ap, am, np1, nm1}) mem.free(p);
                        Step s;
                        s.kind = S_IFACE_BD;
                        s.tm = tmb;
                        s.nn = vnn;
                        s.rp = x;
                        steps[b] = s;
                        replace_r(mem, r, RState{R_DENSE, x, false});
                    }
                } else {
                    // interface_matching (rcwa2d.hpp:600-611)
                    zc *mm = nullptr, *vn = nullptr;
                    if (low.homog) {
                        mm = c.dense();
                        RCWA_CUDA(cudaMemcpyAsync(mm, up.W, (size_t)B * nn * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                        vn = c.dense();
                        LAUNCH(apply_rows_bd_kernel, nblocks((long long)B * N * n), kTpb, st, B, N, n, low.vb, 3, up.V,
                               nullptr, vn);
                    } else if (up.homog) {
                        mm = solve(c, low.W, true, RHS_IDENTITY, nullptr);
                        zc* rhs = mem.zeros<zc>((size_t)B * nn);
                        LAUNCH(bd_to_dense_kernel, nblocks((long long)B * N), kTpb, st, B, N, up.vb, rhs);
                        vn = solve(c, low.V, true, RHS_DENSE, rhs);
                        mem.free(rhs);
                    } else {
                        mm = solve(c, low.W, true, RHS_DENSE, up.W);
                        vn = solve(c, low.V, true, RHS_DENSE, up.V);
                    }
                    // direct_dense (rcwa2d.hpp:753-789)
                    zc* ap = c.dense();
                    zc* am = c.dense();
                    if (r.kind == R_ZERO) {
                        RCWA_CUDA(cudaMemcpyAsync(ap, vn, (size_t)B * nn * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                        RCWA_CUDA(cudaMemcpyAsync(am, mm, (size_t)B * nn * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                    } else if (r.kind == R_BD) {
                        LAUNCH(apply_rows_bd_kernel, nblocks((long long)B * N * n), kTpb, st, B, N, n, r.p, 1, vn, nullptr, ap);
                        LAUNCH(apply_rows_bd_kernel, nblocks((long long)B * N * n), kTpb, st, B, N, n, r.p, 2, mm, nullptr, am);
                    } else {
                        gemm(c, r.p, nn, vn, vn, 1.0, 1.0, ap);   // Nn + r Nn
                        gemm(c, r.p, nn, mm, mm, -1.0, 1.0, am);  // Mm - r Mm
                    }
                    LAUNCH(sum_diff_kernel, nblocks((long long)B * nn), kTpb, st, (long long)B * nn, ap, am);
                    zc* x = solve(c, ap, true, RHS_DENSE, am);
                    mem.free(ap);
                    mem.free(am);
                    LAUNCH(half_diff_kernel, nblocks((long long)B * nn), kTpb, st, (long long)B * nn, mm, vn);
                    Step s;
                    s.kind = S_IFACE_DENSE;
                    s.tm = mm;
                    s.nn = vn;
                    s.rp = x;
                    steps[b] = s;
                    replace_r(mem, r, RState{R_DENSE, x, false});
                }
                // the modes below this interface are no longer needed (rcwa2d.hpp:1184-1187)
                if (!low.homog) {
                    low.W = nullptr;
                    low.V = nullptr;
                }
            } else {
                // propagation in layer j (propagation_block + stack_on, rcwa2d.hpp:612-627, :706-713)
                const Region& rg = reg[j + 1];
                if (nz > 0) {  // the reflection below layer j's bottom (rcwa2d.hpp:1202)
                    RState& rb = cap.r_below[j];
                    rb.kind = r.kind;
                    if (r.kind != R_ZERO) {
                        const size_t cnt = r.kind == R_DENSE ? (size_t)B * nn : (size_t)B * 4 * N;
                        rb.p = mem.get<zc>(cnt);
                        rb.owned = true;
                        RCWA_CUDA(cudaMemcpyAsync(rb.p, r.p, cnt * sizeof(zc), cudaMemcpyDeviceToDevice, st));
                    }
                }
                zc* gt = mem.get<zc>((size_t)B * 4 * N);
                if (r.kind != R_DENSE) {
                    zc* rout = mem.get<zc>((size_t)B * 4 * N);
                    LAUNCH(prop_bd_kernel, nblocks((long long)B * N), kTpb, st, B, N, rg.q, layers[j].d, dk0,
                           r.kind == R_BD ? r.p : nullptr, rout, gt, nullptr);
                    replace_r(mem, r, RState{R_BD, rout, true});
                } else {
                    zc* xv = c.vec();
                    LAUNCH(prop_bd_kernel, nblocks((long long)B * N), kTpb, st, B, N, rg.q, layers[j].d, dk0, nullptr,
                           nullptr, gt, xv);
                    zc* rout = c.dense();
                    LAUNCH(prop_dense_kernel, nblocks((long long)B * nn), kTpb, st, B, n, xv, r.p, rout);
                    mem.free(xv);
                    replace_r(mem, r, RState{R_DENSE, rout, true});
                }
                steps[b] = Step{S_BDMAT, gt};
            }
        }

        // ---- top block (rcwa2d.hpp:826-910, direct form)
        zc* inc = c.vec();
        LAUNCH(incident_kernel, nblocks((long long)B * n), kTpb, st, B, N, i0, de2, inc);
        zc* down = nullptr;
        zc* R = c.vec();
        {
            const Region& up = reg[0];
            const Region& low = reg[1];
            if (up.homog && low.homog) {
                if (r.kind != R_DENSE) {
                    down = c.vec();
                    LAUNCH(top_bd_kernel, nblocks((long long)B * N), kTpb, st, B, N, up.vb, low.vb,
                           r.kind == R_BD ? r.p : nullptr, inc, down, R);
                } else {
                    zc* tdd = mem.get<zc>((size_t)B * 4 * N);
                    zc* rdu = mem.get<zc>((size_t)B * 4 * N);
                    zc* rud = mem.get<zc>((size_t)B * 4 * N);
                    zc* tuu = mem.get<zc>((size_t)B * 4 * N);
                    LAUNCH(iface_blocks_kernel, nblocks((long long)B * N), kTpb, st, B, N, up.vb, low.vb, tdd, rdu, rud, tuu);
                    zc* mat = c.dense();
                    LAUNCH(apply_rows_bd_kernel, nblocks((long long)B * N * n), kTpb, st, B, N, n, rdu, 0, r.p, nullptr, mat);
                    LAUNCH(identity_minus_kernel, nblocks((long long)B * nn), kTpb, st, B, n, mat, nullptr, 1);
                    zc* rhs = c.vec();
                    LAUNCH(bd_apply_vec_kernel, nblocks((long long)B * N), kTpb, st, B, N, tdd, inc, rhs);
                    down = solve(c, mat, true, RHS_DENSE, rhs, 1);
                    zc* back = c.vec();
                    LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, r.p, down, nullptr, back, 1.0, 0.0);
                    LAUNCH(top_bd_finish_kernel, nblocks((long long)B * N), kTpb, st, B, N, rud, tuu, inc, back, R);
                    for (zc* p : {tdd, rdu, rud, tuu, mat, rhs, back}) mem.free(p);
                }
            } else {
                zc *wp = low.W, *vq = low.V;
                bool own = false;
                if (r.kind == R_BD) {
                    wp = c.dense();
                    vq = c.dense();
                    LAUNCH(rmul_bd_kernel, nblocks((long long)B * n * N), kTpb, st, B, N, low.W, r.p, 1, nullptr, wp);
                    LAUNCH(rmul_bd_kernel, nblocks((long long)B * n * N), kTpb, st, B, N, low.V, r.p, 2, nullptr, vq);
                    own = true;
                } else if (r.kind == R_DENSE) {
                    wp = gemm(c, low.W, nn, r.p, low.W, 1.0, 1.0);   // W + W r
                    vq = gemm(c, low.V, nn, r.p, low.V, -1.0, 1.0);  // V - V r
                    own = true;
                }
                zc* kmat = c.dense();
                LAUNCH(apply_rows_bd_kernel, nblocks((long long)B * N * n), kTpb, st, B, N, n, up.vb, 3, vq, wp, kmat);
                zc* rhs = c.vec();
                LAUNCH(scale_vec_kernel, nblocks((long long)B * n), kTpb, st, (long long)B * n, inc, 2.0, rhs);
                down = solve(c, kmat, true, RHS_DENSE, rhs, 1);
                LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, wp, down, inc, R, 1.0, -1.0);
                mem.free(kmat);
                mem.free(rhs);
                if (own) {
                    mem.free(wp);
                    mem.free(vq);
                }
            }
        }
        replace_r(mem, r, RState{});

        // ---- top-down (rcwa2d.hpp:1210-1219)
        for (int b = 1; b < blocks; ++b) {
            Step& s = steps[b];
            const int jl = b / 2;
            if (nz > 0 && b % 2 != 0) {  // amplitude at the layer's top (rcwa2d.hpp:1221)
                cap.a_plus[jl] = c.vec();
                RCWA_CUDA(cudaMemcpyAsync(cap.a_plus[jl], down, (size_t)B * n * sizeof(zc), cudaMemcpyDeviceToDevice, st));
            }
            zc* y = c.vec();
            if (s.kind == S_BDMAT) {
                LAUNCH(bd_apply_vec_kernel, nblocks((long long)B * N), kTpb, st, B, N, s.bd, down, y);
            } else {
                zc* u = c.vec();
                LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, s.rp, down, down, u, 1.0, 1.0);  // (I + r') v
                if (s.kind == S_IFACE_DENSE) {
                    zc* w = c.vec();
                    LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, s.nn, down, nullptr, w, 1.0, 0.0);
                    LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, s.tm, u, w, y, 1.0, 1.0);
                    mem.free(w);
                } else {
                    LAUNCH(iface_bd_step_kernel, nblocks((long long)B * N), kTpb, st, B, N, s.tm, s.nn, u, down, y);
                }
                mem.free(u);
            }
            mem.free(down);
            down = y;
            for (zc* p : {s.bd, s.tm, s.nn, s.rp})
                if (p) mem.free(p);
            s = Step{};
            if (nz > 0 && b % 2 != 0) {  // the reflection below applied at the layer's bottom (rcwa2d.hpp:1224-1225)
                const RState& rb = cap.r_below[jl];
                zc* am = c.vec();
                if (rb.kind == R_ZERO)
                    RCWA_CUDA(cudaMemsetAsync(am, 0, (size_t)B * n * sizeof(zc), st));
                else if (rb.kind == R_BD)
                    LAUNCH(bd_apply_vec_kernel, nblocks((long long)B * N), kTpb, st, B, N, rb.p, down, am);
                else
                    LAUNCH(matvec_kernel, warp_blocks(B), 128, st, B, n, 1, rb.p, down, nullptr, am, 1.0, 0.0);
                cap.a_minus[jl] = am;
            }
        }

        // ---- outputs (rcwa2d.hpp:1225-1270)
        Outputs2D o;
        zc** zs[10] = {&o.Ex_r, &o.Ey_r, &o.Ez_r, &o.Ex_t, &o.Ey_t, &o.Ez_t, &o.Rs, &o.Rp, &o.Ts, &o.Tp};
        for (zc** z : zs) *z = mem.get<zc>((size_t)B * N);
        o.DEr = mem.get<double>((size_t)B * N);
        o.DEt = mem.get<double>((size_t)B * N);
        LAUNCH(finalize2d_kernel, nblocks((long long)B * N), kTpb, st, B, N, R, down, dKx, dKy, dkzI, dkzII, nI,
               zc{nII.real(), nII.imag()}, dnic, dsin, dcos, o, fail);
        LAUNCH(nan_fill2d_kernel, nblocks((long long)B * N), kTpb, st, B, N, o, fail);
        std::vector<zc> hfields;
        if (nz > 0) {
            zc* fout = mem.get<zc>((size_t)B * fper);
            RCWA_CUDA(cudaMemsetAsync(fout, 0, (size_t)B * fper * sizeof(zc), st));
            sample_fields2d(c, fields->zs, layers, nI, nII, N, i0, reg, cap, patterned, Ei, inc, R, down, dKx, dKy, dk0, fout);
            hfields.resize((size_t)B * fper);
            RCWA_CUDA(cudaMemcpyAsync(hfields.data(), fout, (size_t)B * fper * sizeof(zc), cudaMemcpyDeviceToHost, st));
        }

        std::vector<cd> hz[10];
        for (auto& v : hz) v.resize((size_t)B * N);
        std::vector<double> hder((size_t)B * N), hdet((size_t)B * N), hres(B);
        std::vector<int> hfail(B), hinfo(B);
        for (int k = 0; k < 10; ++k)
            RCWA_CUDA(cudaMemcpyAsync(hz[k].data(), *zs[k], (size_t)B * N * sizeof(zc), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(hder.data(), o.DEr, (size_t)B * N * sizeof(double), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(hdet.data(), o.DEt, (size_t)B * N * sizeof(double), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(hfail.data(), fail, B * sizeof(int), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(hinfo.data(), eig_info, B * sizeof(int), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(hres.data(), resid, B * sizeof(double), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(stream_wait(st));
        rcwa_complex* dst[10] = {out.Ex_r, out.Ey_r, out.Ez_r, out.Ex_t, out.Ey_t, out.Ez_t, out.Rs, out.Rp, out.Ts, out.Tp};
        const int n_solve = P + c.n_solve;  // Ei per layer (rcwa2d.hpp:420) plus the chunk's dense solves
        for (int b = 0; b < B; ++b) {
            const int p = idx[b];
            for (int k = 0; k < 10; ++k)
                std::memcpy(dst[k] + (size_t)p * N, hz[k].data() + (size_t)b * N, N * sizeof(zc));
            std::memcpy(out.DEr + (size_t)p * N, hder.data() + (size_t)b * N, N * sizeof(double));
            std::memcpy(out.DEt + (size_t)p * N, hdet.data() + (size_t)b * N, N * sizeof(double));
            out.status[p] = hinfo[b] != 0 ? RCWA_SAMPLE_EIG_NOCONV : (hfail[b] ? RCWA_SAMPLE_NUMERICAL : RCWA_SAMPLE_OK);
            if (out.eig_info) out.eig_info[p] = hinfo[b];
            if (out.n_eig) out.n_eig[p] = P;
            if (out.n_dense_solve) out.n_dense_solve[p] = hinfo[b] != 0 ? P : n_solve;
            if (out.max_eig_residual) out.max_eig_residual[p] = opt.diagnostics ? hres[b] : 0.0;
            if (nz > 0) std::memcpy(fields->out + (size_t)p * fper, hfields.data() + (size_t)b * fper, fper * sizeof(zc));
        }
    }
}

}  // namespace rcwa_gb300
