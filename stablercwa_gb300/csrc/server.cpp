// server.cpp -- the serving request loop declared in include/stablercwa_gb300.h.
//
// Worker slots, each a host thread with its own engine context (and so its own CUDA stream), take
// requests from queues bucketed by matrix order. Admission charges each request its estimated
// device footprint against the server's HBM budget: a free slot takes the oldest request if it
// fits, otherwise the oldest request of another bucket that fits (backfilling), unless the oldest
// request has already waited longer than max_bypass_ms, in which case the slot waits for memory to
// be released. A request alone on the device is always admitted. Requests on different slots run
// concurrently, so work arriving while others are on the device overlaps with them. A slot that takes a
// request also takes the queued requests that differ from it only in the point (same kind, stack, orders,
// polarization or factorization, and options: the same structure at other wavelengths, angles or Jones
// vectors), up to max_batch of them while they fit the budget, and solves them in one batched call.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <new>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/stablercwa_gb300.h"

namespace rcwa_gb300 {
void preload_eig_cluster_kernel();  // eig_cluster.cu
}

namespace {

using Clock = std::chrono::steady_clock;

// ------------------------------------------------------------------ owned copies of a request

struct Owned1D {
    std::vector<rcwa_layer1d> layers;
    std::vector<std::vector<double>> edges;
    std::vector<std::vector<rcwa_complex>> values;
    rcwa_stack1d stack{};
    int gratings = 0;

    void copy(const rcwa_stack1d& s) {
        stack = s;
        const int L = std::max(0, s.n_layers);
        layers.assign(s.layers, s.layers + L);
        edges.resize(L);
        values.resize(L);
        for (int k = 0; k < L; ++k) {
            const rcwa_layer1d& l = s.layers[k];
            if (!l.homogeneous && l.n_segments > 0 && l.edges && l.n_values) {
                edges[k].assign(l.edges, l.edges + l.n_segments + 1);
                values[k].assign(l.n_values, l.n_values + l.n_segments);
                ++gratings;
            }
        }
        for (int k = 0; k < L; ++k) {
            layers[k].edges = edges[k].empty() ? nullptr : edges[k].data();
            layers[k].n_values = values[k].empty() ? nullptr : values[k].data();
        }
        stack.layers = layers.empty() ? nullptr : layers.data();
    }
};

struct Owned2D {
    std::vector<rcwa_layer2d> layers;
    std::vector<std::vector<double>> y_edges;
    std::vector<std::vector<rcwa_xprofile2d>> rows;
    std::vector<std::vector<std::vector<double>>> x_edges;
    std::vector<std::vector<std::vector<rcwa_complex>>> n_values;
    rcwa_stack2d stack{};
    int patterned = 0;

    void copy(const rcwa_stack2d& s) {
        stack = s;
        const int L = std::max(0, s.n_layers);
        layers.assign(s.layers, s.layers + L);
        y_edges.resize(L);
        rows.resize(L);
        x_edges.resize(L);
        n_values.resize(L);
        for (int k = 0; k < L; ++k) {
            const rcwa_layer2d& l = s.layers[k];
            if (l.homogeneous || l.n_strips <= 0 || !l.y_edges || !l.x_profiles) continue;
            ++patterned;
            y_edges[k].assign(l.y_edges, l.y_edges + l.n_strips + 1);
            rows[k].assign(l.x_profiles, l.x_profiles + l.n_strips);
            x_edges[k].resize(l.n_strips);
            n_values[k].resize(l.n_strips);
            for (int r = 0; r < l.n_strips; ++r) {
                const rcwa_xprofile2d& p = l.x_profiles[r];
                if (p.n_segments > 0 && p.edges && p.n_values) {
                    x_edges[k][r].assign(p.edges, p.edges + p.n_segments + 1);
                    n_values[k][r].assign(p.n_values, p.n_values + p.n_segments);
                }
            }
        }
        for (int k = 0; k < L; ++k) {
            for (size_t r = 0; r < rows[k].size(); ++r) {
                rows[k][r].edges = x_edges[k][r].empty() ? nullptr : x_edges[k][r].data();
                rows[k][r].n_values = n_values[k][r].empty() ? nullptr : n_values[k][r].data();
            }
            layers[k].y_edges = y_edges[k].empty() ? nullptr : y_edges[k].data();
            layers[k].x_profiles = rows[k].empty() ? nullptr : rows[k].data();
        }
        stack.layers = layers.empty() ? nullptr : layers.data();
    }
};

// ------------------------------------------------------------------ result storage per kind

template <class T>
void put(T* dst, const std::vector<T>& src) {
    if (dst && !src.empty()) std::memcpy(dst, src.data(), src.size() * sizeof(T));
}
template <class T>
void put1(T* dst, T v) {
    if (dst) *dst = v;
}

struct Res1D {
    std::vector<rcwa_complex> R, T;
    std::vector<double> DEr, DEt;
    int status = 0, eig_info = 0, n_eig = 0, n_dense = 0, n_lu = 0;
    double resid = 0;
    rcwa_result1d view(int n) {
        R.resize(n);
        T.resize(n);
        DEr.resize(n);
        DEt.resize(n);
        return rcwa_result1d{R.data(), T.data(), DEr.data(), DEt.data(), &status, &eig_info, &n_eig, &n_dense, &resid, &n_lu};
    }
    void out(rcwa_result1d* o) const {
        put(o->R, R);
        put(o->T, T);
        put(o->DEr, DEr);
        put(o->DEt, DEt);
        put1(o->status, status);
        put1(o->eig_info, eig_info);
        put1(o->n_eig, n_eig);
        put1(o->n_dense_solve, n_dense);
        put1(o->max_eig_residual, resid);
        put1(o->n_lu, n_lu);
    }
};

struct ResConical {
    std::vector<rcwa_complex> Jr, Jt;
    std::vector<double> DEr, DEt, kx, flux_r, flux_t;
    int status = 0, eig_info = 0, n_eig = 0, n_dense = 0, n_schur = 0, warn = 0, n_lu = 0;
    double min_abs = 0, ky = 0;
    rcwa_result_conical view(int n) {
        Jr.resize(4 * n);
        Jt.resize(4 * n);
        DEr.resize(4 * n);
        DEt.resize(4 * n);
        kx.resize(n);
        flux_r.resize(n);
        flux_t.resize(n);
        return rcwa_result_conical{Jr.data(), Jt.data(), DEr.data(), DEt.data(), &status, &eig_info, &n_eig, &n_dense,
                                   &n_schur, &min_abs, &warn, kx.data(), &ky, flux_r.data(), flux_t.data(), &n_lu};
    }
    void out(rcwa_result_conical* o) const {
        put(o->Jr, Jr);
        put(o->Jt, Jt);
        put(o->DEr, DEr);
        put(o->DEt, DEt);
        put1(o->status, status);
        put1(o->eig_info, eig_info);
        put1(o->n_eig, n_eig);
        put1(o->n_dense_solve, n_dense);
        put1(o->n_schur, n_schur);
        put1(o->min_abs_lambda, min_abs);
        put1(o->degenerate_mode_warning, warn);
        put1(o->n_lu, n_lu);
        put(o->kx, kx);
        put1(o->ky, ky);
        put(o->flux_r, flux_r);
        put(o->flux_t, flux_t);
    }
};

struct Res2D {
    std::vector<double> Kx, Ky, DEr, DEt;
    std::vector<rcwa_complex> c[12];  // kzI, kzII, Ex_r, Ey_r, Ez_r, Ex_t, Ey_t, Ez_t, Rs, Rp, Ts, Tp
    std::vector<unsigned char> prop_r, prop_t, regions;
    int status = 0, eig_info = 0, n_eig = 0, n_dense = 0;
    double resid = 0;
    rcwa_result2d view(int N, int L) {
        for (auto* v : {&Kx, &Ky, &DEr, &DEt}) v->resize(N);
        for (auto& v : c) v.resize(N);
        prop_r.resize(N);
        prop_t.resize(N);
        regions.resize(L + 2);
        rcwa_result2d r{};
        r.Kx = Kx.data();
        r.Ky = Ky.data();
        rcwa_complex** z[12] = {&r.kzI, &r.kzII, &r.Ex_r, &r.Ey_r, &r.Ez_r, &r.Ex_t, &r.Ey_t, &r.Ez_t, &r.Rs, &r.Rp, &r.Ts, &r.Tp};
        for (int k = 0; k < 12; ++k) *z[k] = c[k].data();
        r.DEr = DEr.data();
        r.DEt = DEt.data();
        r.prop_r = prop_r.data();
        r.prop_t = prop_t.data();
        r.status = &status;
        r.eig_info = &eig_info;
        r.n_eig = &n_eig;
        r.n_dense_solve = &n_dense;
        r.max_eig_residual = &resid;
        r.rayleigh_regions = regions.data();
        return r;
    }
    void out(rcwa_result2d* o) const {
        put(o->Kx, Kx);
        put(o->Ky, Ky);
        rcwa_complex* z[12] = {o->kzI, o->kzII, o->Ex_r, o->Ey_r, o->Ez_r, o->Ex_t, o->Ey_t, o->Ez_t, o->Rs, o->Rp, o->Ts, o->Tp};
        for (int k = 0; k < 12; ++k) put(z[k], c[k]);
        put(o->DEr, DEr);
        put(o->DEt, DEt);
        put(o->prop_r, prop_r);
        put(o->prop_t, prop_t);
        put1(o->status, status);
        put1(o->eig_info, eig_info);
        put1(o->n_eig, n_eig);
        put1(o->n_dense_solve, n_dense);
        put1(o->max_eig_residual, resid);
        put(o->rayleigh_regions, regions);
    }
};

struct Job {
    unsigned long long ticket = 0;
    rcwa_request req{};
    std::string key;  // everything but the point: requests with equal keys can share one batched call
    int batch = 1;    // requests in the call that solved this one
    Owned1D s1;
    Owned2D s2;
    int order = 0;
    int bucket = 0;
    double footprint = 0;
    Clock::time_point submitted;
    double submit_s = 0, start_s = 0, finish_s = 0;
    int slot = -1, code = RCWA_OK;
    bool done = false;
    Res1D r1;
    ResConical rc;
    Res2D r2;
};

// Device bytes one solve holds at its peak, from the engines' own working-set estimates: the
// eigensolver workspace and the dense operators of the S-matrix recursion at the algebra order n.
double footprint_of(const Job& j) {
    const double z = 16.0;
    switch (j.req.kind) {
        case RCWA_REQ_1D: {
            const double n = 2.0 * j.req.M + 1;
            return z * n * n * (3.0 * (j.s1.stack.n_layers + 1) + 12.0) + (1 << 20);
        }
        case RCWA_REQ_CONICAL: {
            const double N = 2.0 * j.req.M + 1, n = 2 * N;
            return z * (n * n * 16.0 + N * N * 12.0 * j.s1.gratings + n * 8.0 * (j.s1.stack.n_layers + 2)) +
                   2.0 * z * (3 * N * N + 4 * N + 8) * std::max(1, j.s1.gratings) + (1 << 20);
        }
        default: {
            const double N = (2.0 * j.req.M1 + 1) * (2.0 * j.req.M2 + 1), n = 2 * N;
            return z * n * n * (5.0 * j.s2.patterned + 3.0 * (j.s2.stack.n_layers + 1) + 8.0) + (1 << 20);
        }
    }
}

// The batching key: kind, orders, polarization / factorization, options and the stack's contents, as bytes
// (field by field, so no padding enters).
template <class T>
void add_bytes(std::string& k, const T& v) {
    k.append(reinterpret_cast<const char*>(&v), sizeof v);
}
template <class T>
void add_array(std::string& k, const T* p, size_t n) {
    if (p && n) k.append(reinterpret_cast<const char*>(p), n * sizeof(T));
}
std::string key_of(const Job& j) {
    std::string k;
    const rcwa_request& r = j.req;
    add_bytes(k, r.kind);
    add_bytes(k, r.M);
    add_bytes(k, r.polarization);
    add_bytes(k, r.M1);
    add_bytes(k, r.M2);
    add_bytes(k, r.factorization);
    add_bytes(k, r.options.eig_method);
    add_bytes(k, r.options.linear_solver);
    add_bytes(k, r.options.homogeneous_fast_path);
    add_bytes(k, r.options.diagnostics);
    add_bytes(k, r.options.eig_max_iter);
    add_bytes(k, r.options.eig_eps);
    if (r.kind == RCWA_REQ_2D) {
        const rcwa_stack2d& s = j.s2.stack;
        add_bytes(k, s.nI);
        add_bytes(k, s.nII);
        add_bytes(k, s.Lx);
        add_bytes(k, s.Ly);
        add_bytes(k, s.n_layers);
        for (int l = 0; l < s.n_layers; ++l) {
            const rcwa_layer2d& L = j.s2.layers[l];
            add_bytes(k, L.d);
            add_bytes(k, L.homogeneous);
            add_bytes(k, L.n);
            add_bytes(k, L.n_strips);
            add_array(k, j.s2.y_edges[l].data(), j.s2.y_edges[l].size());
            for (size_t q = 0; q < j.s2.rows[l].size(); ++q) {
                add_bytes(k, j.s2.rows[l][q].n_segments);
                add_array(k, j.s2.x_edges[l][q].data(), j.s2.x_edges[l][q].size());
                add_array(k, j.s2.n_values[l][q].data(), j.s2.n_values[l][q].size());
            }
        }
    } else {
        const rcwa_stack1d& s = j.s1.stack;
        add_bytes(k, s.nI);
        add_bytes(k, s.nII);
        add_bytes(k, s.period);
        add_bytes(k, s.n_layers);
        for (int l = 0; l < s.n_layers; ++l) {
            const rcwa_layer1d& L = j.s1.layers[l];
            add_bytes(k, L.d);
            add_bytes(k, L.homogeneous);
            add_bytes(k, L.n);
            add_bytes(k, L.n_segments);
            add_bytes(k, L.fourier_method);
            add_bytes(k, L.fft_samples);
            add_array(k, j.s1.edges[l].data(), j.s1.edges[l].size());
            add_array(k, j.s1.values[l].data(), j.s1.values[l].size());
        }
    }
    return k;
}

int order_of(const rcwa_request& r) {
    if (r.kind == RCWA_REQ_1D) return 2 * r.M + 1;
    if (r.kind == RCWA_REQ_CONICAL) return 2 * (2 * r.M + 1);
    return 2 * (2 * r.M1 + 1) * (2 * r.M2 + 1);
}

int bucket_of(int order) {
    int b = 0;
    while ((1 << b) < order && b < 30) ++b;
    return b;
}

// With lazy module loading (the CUDA default) a kernel is loaded at its first launch, and a load may
// synchronise the context: on a busy server it then waits for every running solve, however long, and
// each slot whose request meets a kernel for the first time stalls behind the longest one. Small solves of
// each kind on one context before the slots start load the kernels the requests use (once per process);
// the cluster eigensolver, which only orders >= 384 reach, is loaded directly.
void warm_up(rcwa_gpu_ctx* ctx) {
    static std::once_flag once;
    std::call_once(once, [ctx] {
        const double e1[3] = {0.0, 0.3, 1.0}, e2[3] = {0.0, 0.55, 1.0};
        const rcwa_complex v1[2] = {{1.5, 0.0}, {1.0, 0.0}}, v2[2] = {{1.6, 0.01}, {1.0, 0.0}};
        rcwa_layer1d L[3] = {};
        L[0].d = 0.2;
        L[0].n_segments = 2;
        L[0].edges = e1;
        L[0].n_values = v1;
        L[1].d = 0.1;
        L[1].homogeneous = 1;
        L[1].n = {2.0, 0.0};
        L[2] = L[0];
        L[2].edges = e2;
        L[2].n_values = v2;
        for (int lossy = 0; lossy < 2; ++lossy) {
            const rcwa_stack1d st{{1.0, 0.0}, {1.46, 0.0}, 1.0, lossy ? 3 : 2, L};
            for (int M : {20, 60}) {
                Res1D r;
                rcwa_result1d v = r.view(2 * M + 1);
                const rcwa_point1d p{0.7, 10.0};
                for (int pol = 0; pol < 2; ++pol) rcwa_gpu_solve1d_batch(ctx, &st, &p, 1, M, pol, nullptr, &v);
            }
            for (int M : {10, 40}) {
                ResConical r;
                rcwa_result_conical v = r.view(2 * M + 1);
                const rcwa_point_conical p{0.7, 10.0, 20.0};
                rcwa_gpu_solve_conical_batch(ctx, &st, &p, 1, M, nullptr, &v);
            }
        }
        const double ye[4] = {0.0, 0.3, 0.7, 1.0}, xe0[2] = {0.0, 1.0}, xe1[3] = {0.0, 0.4, 1.0};
        const rcwa_complex xv0[1] = {{1.0, 0.0}}, xv1[2] = {{2.0, 0.0}, {1.0, 0.0}};
        const rcwa_xprofile2d rows[3] = {{1, xe0, xv0}, {2, xe1, xv1}, {1, xe0, xv0}};
        rcwa_layer2d L2[2] = {};
        L2[0].d = 0.2;
        L2[0].n_strips = 3;
        L2[0].y_edges = ye;
        L2[0].x_profiles = rows;
        L2[1].d = 0.1;
        L2[1].homogeneous = 1;
        L2[1].n = {1.8, 0.0};
        const rcwa_stack2d st2{1.0, {1.5, 0.0}, 1.0, 1.0, 2, L2};
        for (int M : {2, 5}) {
            const int N = (2 * M + 1) * (2 * M + 1);
            Res2D r;
            rcwa_result2d v = r.view(N, 2);
            const rcwa_point2d p{0.7, 10.0, 20.0, {1.0, 0.0}, {0.0, 0.0}};
            rcwa_gpu_solve2d_batch(ctx, &st2, &p, 1, M, M, 0, nullptr, &v);
        }
        rcwa_gb300::preload_eig_cluster_kernel();
    });
}

}  // namespace

struct rcwa_gpu_server {
    int device = 0;
    std::vector<rcwa_gpu_ctx*> ctxs;
    std::vector<std::thread> workers;
    std::mutex m;
    std::condition_variable cv_work, cv_done, cv_idle;
    int waiters = 0;  // threads inside rcwa_gpu_server_wait (destroy lets them leave before freeing)
    std::map<int, std::deque<Job*>> buckets;
    std::map<unsigned long long, std::unique_ptr<Job>> jobs;
    double budget = 0, in_use = 0;
    int running = 0;
    std::chrono::milliseconds max_bypass{2000};
    int max_batch = 256;
    bool stop = false;
    unsigned long long next_ticket = 1;
    Clock::time_point t0 = Clock::now();

    double now_s() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    // under the lock: the next request a free slot may start and the queued requests that can share its
    // call (equal keys, while they fit the budget), or an empty batch
    std::vector<Job*> pick_batch() {
        std::vector<Job*> batch;
        Job* lead = pick();
        if (!lead) return batch;
        batch.push_back(lead);
        double room = budget - in_use - lead->footprint;
        if (max_batch > 1) {
            std::deque<Job*>& q = buckets[lead->bucket];
            for (auto it = q.begin(); it != q.end() && (int)batch.size() < max_batch;) {
                if ((*it)->key == lead->key && (*it)->footprint <= room) {
                    room -= (*it)->footprint;
                    batch.push_back(*it);
                    it = q.erase(it);
                } else {
                    ++it;
                }
            }
        }
        return batch;
    }

    // under the lock: the next request a free slot may start, or null
    Job* pick() {
        Job* oldest = nullptr;
        for (auto& kv : buckets)
            if (!kv.second.empty() && (!oldest || kv.second.front()->ticket < oldest->ticket)) oldest = kv.second.front();
        if (!oldest) return nullptr;
        const double room = budget - in_use;
        Job* chosen = nullptr;
        if (running == 0 || oldest->footprint <= room) {
            chosen = oldest;
        } else if (Clock::now() - oldest->submitted < max_bypass) {
            for (auto& kv : buckets) {
                if (kv.second.empty()) continue;
                Job* f = kv.second.front();
                if (f->footprint <= room && (!chosen || f->ticket < chosen->ticket)) chosen = f;
            }
        }
        if (chosen) buckets[chosen->bucket].pop_front();
        return chosen;
    }

    void run(Job& j, rcwa_gpu_ctx* ctx) {
        rcwa_options o = j.req.options;
        if (j.req.kind == RCWA_REQ_1D) {
            const rcwa_point1d p{j.req.wavelength, j.req.theta_deg};
            rcwa_result1d v = j.r1.view(2 * j.req.M + 1);
            j.code = rcwa_gpu_solve1d_batch(ctx, &j.s1.stack, &p, 1, j.req.M, j.req.polarization, &o, &v);
        } else if (j.req.kind == RCWA_REQ_CONICAL) {
            const rcwa_point_conical p{j.req.wavelength, j.req.theta_deg, j.req.phi_deg};
            rcwa_result_conical v = j.rc.view(2 * j.req.M + 1);
            j.code = rcwa_gpu_solve_conical_batch(ctx, &j.s1.stack, &p, 1, j.req.M, &o, &v);
        } else {
            const rcwa_point2d p{j.req.wavelength, j.req.theta_deg, j.req.phi_deg, j.req.Es, j.req.Ep};
            rcwa_result2d v = j.r2.view((2 * j.req.M1 + 1) * (2 * j.req.M2 + 1), j.s2.stack.n_layers);
            j.code = rcwa_gpu_solve2d_batch(ctx, &j.s2.stack, &p, 1, j.req.M1, j.req.M2, j.req.factorization, &o, &v);
        }
    }

    // Several requests of one key in one call: the points side by side, the results copied back to each.
    void run_batch(std::vector<Job*>& b, rcwa_gpu_ctx* ctx) {
        const int P = (int)b.size();
        const rcwa_request& r0 = b[0]->req;
        rcwa_options o = r0.options;
        int code = RCWA_OK;
        if (r0.kind == RCWA_REQ_1D) {
            const int n = 2 * r0.M + 1;
            std::vector<rcwa_point1d> pts(P);
            std::vector<rcwa_complex> R((size_t)P * n), T((size_t)P * n);
            std::vector<double> DEr((size_t)P * n), DEt((size_t)P * n), resid(P);
            std::vector<int> st(P), info(P), neig(P), nds(P), nlu(P);
            for (int p = 0; p < P; ++p) pts[p] = rcwa_point1d{b[p]->req.wavelength, b[p]->req.theta_deg};
            rcwa_result1d v{R.data(), T.data(), DEr.data(), DEt.data(), st.data(), info.data(), neig.data(), nds.data(),
                            resid.data(), nlu.data()};
            code = rcwa_gpu_solve1d_batch(ctx, &b[0]->s1.stack, pts.data(), P, r0.M, r0.polarization, &o, &v);
            for (int p = 0; p < P; ++p) {
                Res1D& h = b[p]->r1;
                h.view(n);
                std::copy_n(R.begin() + (size_t)p * n, n, h.R.begin());
                std::copy_n(T.begin() + (size_t)p * n, n, h.T.begin());
                std::copy_n(DEr.begin() + (size_t)p * n, n, h.DEr.begin());
                std::copy_n(DEt.begin() + (size_t)p * n, n, h.DEt.begin());
                h.status = st[p];
                h.eig_info = info[p];
                h.n_eig = neig[p];
                h.n_dense = nds[p];
                h.n_lu = nlu[p];
                h.resid = resid[p];
            }
        } else if (r0.kind == RCWA_REQ_CONICAL) {
            const int n = 2 * r0.M + 1;
            std::vector<rcwa_point_conical> pts(P);
            std::vector<rcwa_complex> Jr((size_t)P * n * 4), Jt((size_t)P * n * 4);
            std::vector<double> DEr((size_t)P * n * 4), DEt((size_t)P * n * 4), kx((size_t)P * n), fr((size_t)P * n),
                ft((size_t)P * n), ky(P), minl(P);
            std::vector<int> st(P), info(P), neig(P), nds(P), nsch(P), warn(P), nlu(P);
            for (int p = 0; p < P; ++p)
                pts[p] = rcwa_point_conical{b[p]->req.wavelength, b[p]->req.theta_deg, b[p]->req.phi_deg};
            rcwa_result_conical v{Jr.data(), Jt.data(), DEr.data(), DEt.data(), st.data(), info.data(), neig.data(),
                                  nds.data(), nsch.data(), minl.data(), warn.data(), kx.data(), ky.data(), fr.data(),
                                  ft.data(), nlu.data()};
            code = rcwa_gpu_solve_conical_batch(ctx, &b[0]->s1.stack, pts.data(), P, r0.M, &o, &v);
            for (int p = 0; p < P; ++p) {
                ResConical& h = b[p]->rc;
                h.view(n);
                std::copy_n(Jr.begin() + (size_t)p * n * 4, n * 4, h.Jr.begin());
                std::copy_n(Jt.begin() + (size_t)p * n * 4, n * 4, h.Jt.begin());
                std::copy_n(DEr.begin() + (size_t)p * n * 4, n * 4, h.DEr.begin());
                std::copy_n(DEt.begin() + (size_t)p * n * 4, n * 4, h.DEt.begin());
                std::copy_n(kx.begin() + (size_t)p * n, n, h.kx.begin());
                std::copy_n(fr.begin() + (size_t)p * n, n, h.flux_r.begin());
                std::copy_n(ft.begin() + (size_t)p * n, n, h.flux_t.begin());
                h.status = st[p];
                h.eig_info = info[p];
                h.n_eig = neig[p];
                h.n_dense = nds[p];
                h.n_schur = nsch[p];
                h.warn = warn[p];
                h.n_lu = nlu[p];
                h.min_abs = minl[p];
                h.ky = ky[p];
            }
        } else {
            const int N = (2 * r0.M1 + 1) * (2 * r0.M2 + 1), L = b[0]->s2.stack.n_layers;
            std::vector<rcwa_point2d> pts(P);
            std::vector<double> Kx((size_t)P * N), Ky((size_t)P * N), DEr((size_t)P * N), DEt((size_t)P * N), resid(P);
            std::vector<rcwa_complex> c[12];
            for (auto& x : c) x.resize((size_t)P * N);
            std::vector<unsigned char> pr((size_t)P * N), pt((size_t)P * N), reg((size_t)P * (L + 2));
            std::vector<int> st(P), info(P), neig(P), nds(P);
            for (int p = 0; p < P; ++p)
                pts[p] = rcwa_point2d{b[p]->req.wavelength, b[p]->req.theta_deg, b[p]->req.phi_deg, b[p]->req.Es, b[p]->req.Ep};
            rcwa_result2d v{};
            v.Kx = Kx.data();
            v.Ky = Ky.data();
            rcwa_complex** z[12] = {&v.kzI, &v.kzII, &v.Ex_r, &v.Ey_r, &v.Ez_r, &v.Ex_t, &v.Ey_t, &v.Ez_t, &v.Rs, &v.Rp, &v.Ts, &v.Tp};
            for (int q = 0; q < 12; ++q) *z[q] = c[q].data();
            v.DEr = DEr.data();
            v.DEt = DEt.data();
            v.prop_r = pr.data();
            v.prop_t = pt.data();
            v.status = st.data();
            v.eig_info = info.data();
            v.n_eig = neig.data();
            v.n_dense_solve = nds.data();
            v.max_eig_residual = resid.data();
            v.rayleigh_regions = reg.data();
            code = rcwa_gpu_solve2d_batch(ctx, &b[0]->s2.stack, pts.data(), P, r0.M1, r0.M2, r0.factorization, &o, &v);
            for (int p = 0; p < P; ++p) {
                Res2D& h = b[p]->r2;
                h.view(N, L);
                std::copy_n(Kx.begin() + (size_t)p * N, N, h.Kx.begin());
                std::copy_n(Ky.begin() + (size_t)p * N, N, h.Ky.begin());
                std::copy_n(DEr.begin() + (size_t)p * N, N, h.DEr.begin());
                std::copy_n(DEt.begin() + (size_t)p * N, N, h.DEt.begin());
                for (int q = 0; q < 12; ++q) std::copy_n(c[q].begin() + (size_t)p * N, N, h.c[q].begin());
                std::copy_n(pr.begin() + (size_t)p * N, N, h.prop_r.begin());
                std::copy_n(pt.begin() + (size_t)p * N, N, h.prop_t.begin());
                std::copy_n(reg.begin() + (size_t)p * (L + 2), L + 2, h.regions.begin());
                h.status = st[p];
                h.eig_info = info[p];
                h.n_eig = neig[p];
                h.n_dense = nds[p];
                h.resid = resid[p];
            }
        }
        for (Job* j : b) {
            j->code = code;
            j->batch = P;
        }
    }

    void worker(int slot) {
        cudaSetDevice(device);
        for (;;) {
            std::vector<Job*> b;
            {
                std::unique_lock<std::mutex> lk(m);
                cv_work.wait(lk, [&] { return stop || !(b = pick_batch()).empty(); });
                if (b.empty()) return;
                const double t = now_s();
                for (Job* j : b) {
                    in_use += j->footprint;
                    j->slot = slot;
                    j->start_s = t;
                }
                ++running;
            }
            if (b.size() == 1) {
                run(*b[0], ctxs[slot]);
            } else {
                try {
                    run_batch(b, ctxs[slot]);
                } catch (const std::bad_alloc&) {
                    for (Job* j : b) j->code = RCWA_ENOMEM;
                }
            }
            {
                std::lock_guard<std::mutex> lk(m);
                const double t = now_s();
                for (Job* j : b) {
                    in_use -= j->footprint;
                    j->finish_s = t;
                    j->done = true;
                }
                --running;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

extern "C" {

int rcwa_gpu_server_create(const rcwa_server_config* config, rcwa_gpu_server** out) {
    if (!out) return RCWA_EINVAL;
    *out = nullptr;
    const int slots = config && config->slots > 0 ? config->slots : 32;
    if (slots > 1024) return RCWA_EINVAL;
    std::unique_ptr<rcwa_gpu_server> s;
    try {
        s.reset(new rcwa_gpu_server());
    } catch (const std::bad_alloc&) {
        return RCWA_ENOMEM;
    }
    s->device = config ? config->device : 0;
    if (config && config->max_bypass_ms > 0) s->max_bypass = std::chrono::milliseconds(config->max_bypass_ms);
    if (config && config->max_batch > 0) s->max_batch = config->max_batch;
    for (int k = 0; k < slots; ++k) {
        rcwa_gpu_config c{s->device, 0};
        rcwa_gpu_ctx* ctx = nullptr;
        const int rc = rcwa_gpu_create(&c, &ctx);
        if (rc != RCWA_OK) {
            for (rcwa_gpu_ctx* p : s->ctxs) rcwa_gpu_destroy(p);
            return rc;
        }
        s->ctxs.push_back(ctx);
    }
    if (config && config->hbm_budget) {
        s->budget = (double)config->hbm_budget;
    } else {
        size_t free_b = 0, total = 0;
        cudaSetDevice(s->device);
        s->budget = cudaMemGetInfo(&free_b, &total) == cudaSuccess ? 0.8 * (double)free_b : 8.0 * (1 << 30);
    }
    warm_up(s->ctxs[0]);
    for (int k = 0; k < slots; ++k) s->workers.emplace_back(&rcwa_gpu_server::worker, s.get(), k);
    *out = s.release();
    return RCWA_OK;
}

void rcwa_gpu_server_destroy(rcwa_gpu_server* s) {
    if (!s) return;
    {
        // requests still queued are cancelled: their waiters wake with RCWA_ECANCELLED
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
        for (auto& kv : s->buckets)
            for (Job* j : kv.second) {
                j->code = RCWA_ECANCELLED;
                j->done = true;
            }
        s->buckets.clear();
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    for (std::thread& t : s->workers) t.join();  // requests already running finish and wake their waiters
    {
        std::unique_lock<std::mutex> lk(s->m);
        s->cv_done.notify_all();
        s->cv_idle.wait(lk, [&] { return s->waiters == 0; });
    }
    for (rcwa_gpu_ctx* c : s->ctxs) rcwa_gpu_destroy(c);
    delete s;
}

int rcwa_gpu_server_submit(rcwa_gpu_server* s, const rcwa_request* r, unsigned long long* ticket) {
    if (!s || !r || !ticket) return RCWA_EINVAL;
    if (r->kind == RCWA_REQ_2D ? !r->stack2d : (r->kind == RCWA_REQ_1D || r->kind == RCWA_REQ_CONICAL ? !r->stack1d : true))
        return RCWA_EINVAL;
    std::unique_ptr<Job> j;
    try {
        j.reset(new Job());
        j->req = *r;
        if (r->kind == RCWA_REQ_2D) {
            if (r->stack2d->n_layers < 0 || (r->stack2d->n_layers > 0 && !r->stack2d->layers)) return RCWA_EINVAL;
            j->s2.copy(*r->stack2d);
            j->req.stack2d = &j->s2.stack;
            j->req.stack1d = nullptr;
            if (r->M1 < 0 || r->M2 < 0 || r->M1 > 64 || r->M2 > 64) return RCWA_EINVAL;
        } else {
            if (r->stack1d->n_layers < 0 || (r->stack1d->n_layers > 0 && !r->stack1d->layers)) return RCWA_EINVAL;
            j->s1.copy(*r->stack1d);
            j->req.stack1d = &j->s1.stack;
            j->req.stack2d = nullptr;
            if (r->M < 0 || r->M > 4096) return RCWA_EINVAL;
        }
    } catch (const std::bad_alloc&) {
        return RCWA_ENOMEM;
    }
    j->order = order_of(j->req);
    j->bucket = bucket_of(j->order);
    j->footprint = footprint_of(*j);
    try {
        j->key = key_of(*j);
    } catch (const std::bad_alloc&) {
        return RCWA_ENOMEM;
    }
    {
        std::lock_guard<std::mutex> lk(s->m);
        if (s->stop) return RCWA_ECANCELLED;
        j->ticket = s->next_ticket++;
        j->submitted = Clock::now();
        j->submit_s = s->now_s();
        *ticket = j->ticket;
        s->buckets[j->bucket].push_back(j.get());
        s->jobs[j->ticket] = std::move(j);
    }
    s->cv_work.notify_one();
    return RCWA_OK;
}

int rcwa_gpu_server_wait(rcwa_gpu_server* s, unsigned long long ticket, int timeout_ms, rcwa_response* resp, void* result) {
    if (!s) return RCWA_EINVAL;
    std::unique_ptr<Job> j;
    {
        std::unique_lock<std::mutex> lk(s->m);
        if (s->jobs.find(ticket) == s->jobs.end()) return RCWA_EINVAL;
        // the job is looked up again on every wake-up: another thread waiting on the same ticket may have
        // taken (and freed) it meanwhile
        const auto ready = [&] {
            const auto it = s->jobs.find(ticket);
            return it == s->jobs.end() || it->second->done;
        };
        ++s->waiters;
        bool finished = true;
        if (timeout_ms < 0) s->cv_done.wait(lk, ready);
        else finished = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
        if (--s->waiters == 0 && s->stop) s->cv_idle.notify_all();
        if (!finished) return RCWA_ETIMEOUT;
        const auto it = s->jobs.find(ticket);
        if (it == s->jobs.end()) return RCWA_EINVAL;  // released by a concurrent wait on the same ticket
        j = std::move(it->second);
        s->jobs.erase(it);
    }
    if (resp) *resp = rcwa_response{j->code, j->slot, j->submit_s, j->start_s, j->finish_s, j->footprint, j->batch};
    if (result) {
        if (j->req.kind == RCWA_REQ_1D) j->r1.out(static_cast<rcwa_result1d*>(result));
        else if (j->req.kind == RCWA_REQ_CONICAL) j->rc.out(static_cast<rcwa_result_conical*>(result));
        else j->r2.out(static_cast<rcwa_result2d*>(result));
    }
    return j->code == RCWA_ECANCELLED ? RCWA_ECANCELLED : RCWA_OK;
}

}  // extern "C"
