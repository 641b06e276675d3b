// capi.cu -- the C ABI of libstablercwa_gb300.so (declared in include/stablercwa_gb300.h).
//
// Every entry point validates its arguments the way the reference does before any work, runs on
// the context's stream under the context's lock, and turns engine errors into return codes with a
// message kept in the context.
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

struct rcwa_gpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex lock;
    std::string last_error;
    size_t workspace_limit = 0;
    bool timing = false;
    rcwa_gb300::KernelTimer timer;
    cudaStream_t stream2 = nullptr;  // second stream of the both-polarization call, created on first use
    cudaEvent_t fork = nullptr, join = nullptr;
};

namespace {

using namespace rcwa_gb300;

std::mutex g_create_lock;
std::string g_create_error;

int fail(rcwa_gpu_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

template <class F>
int guarded(rcwa_gpu_ctx* ctx, F&& body) {
    if (!ctx) return RCWA_EINVAL;
    std::lock_guard<std::mutex> hold(ctx->lock);
    struct TimerScope {
        explicit TimerScope(rcwa_gpu_ctx* c) { current_timer() = c->timing ? &c->timer : nullptr; }
        ~TimerScope() { current_timer() = nullptr; }
    } scope(ctx);
    try {
        RCWA_CUDA(cudaSetDevice(ctx->device));
        body();
        return RCWA_OK;
    } catch (const EngineError& e) {
        return fail(ctx, e.code, e.message);
    } catch (const std::bad_alloc&) {
        return fail(ctx, RCWA_ENOMEM, "host allocation failed");
    }
}

Options to_options(const rcwa_options* o) {
    Options opt;
    if (!o) return opt;
    if (o->eig_method != 0) throw EngineError{RCWA_EUNSUPPORTED, "rcwa: only the QR eigensolver (EigMethod::QR) is implemented"};
    if (o->linear_solver != 0)
        throw EngineError{RCWA_EUNSUPPORTED, "rcwa: only partial-pivot LU (LinearSolver::LUPartial) is implemented"};
    if (!o->homogeneous_fast_path)
        throw EngineError{RCWA_EUNSUPPORTED, "rcwa: homogeneous_fast_path = false is not implemented"};
    if (o->eig_max_iter < 1) throw EngineError{RCWA_EINVAL, "eig_qr: max_iter must be >= 1"};
    if (!(o->eig_eps >= 0.0) || !std::isfinite(o->eig_eps)) throw EngineError{RCWA_EINVAL, "eig_qr: eps must be finite and >= 0"};
    opt.diagnostics = o->diagnostics != 0;
    opt.max_iter = o->eig_max_iter;
    opt.eps = o->eig_eps;
    if (const char* g = std::getenv("RCWA_GB300_EIG_GROUP")) opt.eig_group = std::atoi(g);
    return opt;
}

size_t chunk_bytes(const rcwa_gpu_ctx* ctx) {
    if (ctx->workspace_limit) return ctx->workspace_limit;
    size_t free_b = 0, total = 0;
    if (cudaMemGetInfo(&free_b, &total) != cudaSuccess) return size_t(8) << 30;
    return std::min<size_t>(free_b / 2, size_t(48) << 30);
}

// Device bytes a 2-D call may hold: free memory plus what the stream-ordered pool caches unused.
size_t chunk_bytes2d(const rcwa_gpu_ctx* ctx) {
    if (ctx->workspace_limit) return ctx->workspace_limit;
    size_t free_b = 0, total = 0;
    if (cudaMemGetInfo(&free_b, &total) != cudaSuccess) return size_t(8) << 30;
    size_t cached = 0;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        uint64_t reserved = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
            cached = (size_t)(reserved - used);
    }
    return (size_t)(0.8 * (double)(free_b + cached));
}

// Both polarizations of the same points: TE on the context's stream, TM on a second stream driven from
// a second host thread. The two sweeps share nothing but the prepared points, so their kernels
// overlap on the device. Results: TE block first, then the TM block, in every array of d_out.
void solve_both(rcwa_gpu_ctx* ctx, const rcwa_stack1d& stack, const double* ds, const double* dw, int n_points, int M,
                const Options& opt, const rcwa_result1d& d_out) {
    const cudaStream_t st = ctx->stream;
    if (!ctx->stream2) {
        RCWA_CUDA(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
        RCWA_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
        RCWA_CUDA(cudaEventCreateWithFlags(&ctx->join, cudaEventDisableTiming));
    }
    RCWA_CUDA(cudaEventRecord(ctx->fork, st));
    RCWA_CUDA(cudaStreamWaitEvent(ctx->stream2, ctx->fork, 0));
    const int n = 2 * M + 1;
    const size_t pn = (size_t)n_points * n;
    rcwa_result1d te = d_out, tm = d_out;
    tm.R = d_out.R + pn;
    tm.T = d_out.T + pn;
    tm.DEr = d_out.DEr + pn;
    tm.DEt = d_out.DEt + pn;
    tm.status = d_out.status ? d_out.status + n_points : nullptr;
    tm.eig_info = d_out.eig_info ? d_out.eig_info + n_points : nullptr;
    tm.n_eig = d_out.n_eig ? d_out.n_eig + n_points : nullptr;
    tm.n_dense_solve = d_out.n_dense_solve ? d_out.n_dense_solve + n_points : nullptr;
    tm.n_lu = d_out.n_lu ? d_out.n_lu + n_points : nullptr;
    tm.max_eig_residual = d_out.max_eig_residual ? d_out.max_eig_residual + n_points : nullptr;
    const size_t cb = chunk_bytes(ctx) / 2;
    std::exception_ptr tm_error;
    std::thread worker([&] {
        try {
            RCWA_CUDA(cudaSetDevice(ctx->device));
            current_timer() = ctx->timing ? &ctx->timer : nullptr;
            solve1d_device(ctx->stream2, stack, ds, dw, n_points, M, RCWA_TM, opt, tm, cb);
        } catch (...) {
            tm_error = std::current_exception();
        }
        current_timer() = nullptr;
    });
    std::exception_ptr te_error;
    try {
        solve1d_device(st, stack, ds, dw, n_points, M, RCWA_TE, opt, te, cb);
    } catch (...) {
        te_error = std::current_exception();
    }
    worker.join();
    RCWA_CUDA(cudaEventRecord(ctx->join, ctx->stream2));
    RCWA_CUDA(cudaStreamWaitEvent(st, ctx->join, 0));
    if (te_error) std::rethrow_exception(te_error);
    if (tm_error) std::rethrow_exception(tm_error);
}

void check_result_ptrs(const rcwa_result1d* out) {
    if (!out || !out->R || !out->T || !out->DEr || !out->DEt)
        throw EngineError{RCWA_EINVAL, "rcwa: result arrays R, T, DEr, DEt are required"};
}

template <class T>
void copy_back(T* host, const T* dev, size_t count, cudaStream_t st) {
    if (host && dev && count) RCWA_CUDA(cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, st));
}

}  // namespace

extern "C" {

int rcwa_gpu_abi_version(void) { return RCWA_GB300_ABI_VERSION; }

void rcwa_options_default(rcwa_options* o) {
    if (!o) return;
    o->eig_method = 0;
    o->linear_solver = 0;
    o->homogeneous_fast_path = 1;
    o->diagnostics = 0;
    o->eig_max_iter = 30;
    o->eig_eps = DBL_EPSILON;
}

long long rcwa_gpu_launch_count(void) { return launch_count(); }

long long rcwa_gpu_eig_rotations(void) {
    try {
        return take_rotation_count();
    } catch (...) {
        return -1;
    }
}

int rcwa_gpu_create(const rcwa_gpu_config* config, rcwa_gpu_ctx** out) {
    std::lock_guard<std::mutex> hold(g_create_lock);
    if (!out) return RCWA_EINVAL;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return RCWA_ECUDA;
    }
    const int dev = config ? config->device : 0;
    if (dev < 0 || dev >= count) {
        g_create_error = "device ordinal out of range";
        return RCWA_EINVAL;
    }
    auto* ctx = new rcwa_gpu_ctx();
    ctx->device = dev;
    ctx->workspace_limit = config ? config->workspace_limit : 0;
    if ((e = cudaSetDevice(dev)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        g_create_error = cudaGetErrorString(e);
        delete ctx;
        return RCWA_ECUDA;
    }
    // keep stream-ordered allocations cached in the device pool between calls, and never let the pool hand
    // one stream memory that another stream freed with work still pending (it would make the second stream
    // wait for the first: contexts on separate streams, as the serving loop's slots are, would serialise)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        int no = 0;
        cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
    *out = ctx;
    return RCWA_OK;
}

void rcwa_gpu_destroy(rcwa_gpu_ctx* ctx) {
    if (!ctx) return;
    {
        std::lock_guard<std::mutex> hold(ctx->lock);
        cudaSetDevice(ctx->device);
        stream_wait(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        if (ctx->stream2) {
            stream_wait(ctx->stream2);
            cudaStreamDestroy(ctx->stream2);
        }
        if (ctx->fork) cudaEventDestroy(ctx->fork);
        if (ctx->join) cudaEventDestroy(ctx->join);
    }
    delete ctx;
}

int rcwa_gpu_last_error(const rcwa_gpu_ctx* ctx, char* buffer, size_t size) {
    if (!buffer || size == 0) return RCWA_EINVAL;
    const std::string& msg = ctx ? ctx->last_error : g_create_error;
    std::strncpy(buffer, msg.c_str(), size - 1);
    buffer[size - 1] = '\0';
    return RCWA_OK;
}

void* rcwa_gpu_stream(rcwa_gpu_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

int rcwa_gpu_set_kernel_timing(rcwa_gpu_ctx* ctx, int enable) {
    return guarded(ctx, [&] {
        ctx->timer.collect();
        ctx->timing = enable != 0;
        if (ctx->timing) {
            if (!ctx->timer.base) RCWA_CUDA(cudaEventCreate(&ctx->timer.base));
            RCWA_CUDA(cudaEventRecord(ctx->timer.base, ctx->stream));
            RCWA_CUDA(cudaEventSynchronize(ctx->timer.base));
            for (auto& v : ctx->timer.spans) v.clear();
        }
    });
}

int rcwa_gpu_kernel_busy(rcwa_gpu_ctx* ctx, const char* kind, double* milliseconds) {
    return guarded(ctx, [&] {
        if (!kind || !milliseconds) throw EngineError{RCWA_EINVAL, "kernel_busy: null argument"};
        int k = -1;
        if (!std::strcmp(kind, "eig")) k = TK_EIG;
        if (!std::strcmp(kind, "lu")) k = TK_LU;
        if (!std::strcmp(kind, "gemm")) k = TK_GEMM;
        if (k < 0) throw EngineError{RCWA_EINVAL, "kernel_busy: kind must be eig, lu or gemm"};
        *milliseconds = ctx->timer.busy_ms(k);
    });
}

int rcwa_gpu_kernel_time(rcwa_gpu_ctx* ctx, const char* kind, double* milliseconds, long long* launches) {
    return guarded(ctx, [&] {
        if (!kind || !milliseconds) throw EngineError{RCWA_EINVAL, "kernel_time: null argument"};
        int k = -1;
        if (!std::strcmp(kind, "eig")) k = TK_EIG;
        if (!std::strcmp(kind, "lu")) k = TK_LU;
        if (!std::strcmp(kind, "gemm")) k = TK_GEMM;
        if (k < 0) throw EngineError{RCWA_EINVAL, "kernel_time: kind must be eig, lu or gemm"};
        ctx->timer.collect();
        *milliseconds = ctx->timer.ms[k];
        if (launches) *launches = ctx->timer.count[k];
        ctx->timer.ms[k] = 0.0;
        ctx->timer.count[k] = 0;
    });
}

int rcwa_gpu_synchronize(rcwa_gpu_ctx* ctx) {
    return guarded(ctx, [&] { RCWA_CUDA(stream_wait(ctx->stream)); });
}

int rcwa_gpu_solve1d_batch(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point1d* points, int n_points, int M,
                           int polarization, const rcwa_options* options, rcwa_result1d* out) {
    return guarded(ctx, [&] {
        if (!stack || (n_points > 0 && !points) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
        check_result_ptrs(out);
        const bool both = polarization == RCWA_TE_TM;
        validate1d(*stack, points, n_points, M, both ? RCWA_TE : polarization);
        if (both) validate1d(*stack, points, n_points, M, RCWA_TM);
        const Options opt = to_options(options);
        if (n_points == 0) return;
        const cudaStream_t st = ctx->stream;
        const int n = 2 * M + 1;
        const int sweeps = both ? 2 : 1;
        // s = nI sin(theta) with the host libm, the reference's own expression (rcwa1d.hpp:411)
        std::vector<double> hs(n_points), hw(n_points);
        const double kPi = 3.141592653589793238462643383279502884;
        for (int p = 0; p < n_points; ++p) {
            hs[p] = stack->nI.re * std::sin(points[p].theta_deg * kPi / 180.0);
            hw[p] = points[p].wavelength;
        }
        DeviceScratch mem(st);
        double* ds = mem.get<double>(n_points);
        double* dw = mem.get<double>(n_points);
        RCWA_CUDA(cudaMemcpyAsync(ds, hs.data(), n_points * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dw, hw.data(), n_points * sizeof(double), cudaMemcpyHostToDevice, st));
        const size_t nv = (size_t)n_points * n * sweeps, np = (size_t)n_points * sweeps;
        rcwa_result1d d{};
        d.R = reinterpret_cast<rcwa_complex*>(mem.get<zc>(nv));
        d.T = reinterpret_cast<rcwa_complex*>(mem.get<zc>(nv));
        d.DEr = mem.get<double>(nv);
        d.DEt = mem.get<double>(nv);
        d.status = mem.get<int>(np);
        d.eig_info = mem.get<int>(np);
        d.n_eig = mem.get<int>(np);
        d.n_dense_solve = mem.get<int>(np);
        d.max_eig_residual = opt.diagnostics ? mem.zeros<double>(np) : nullptr;
        d.n_lu = out->n_lu ? mem.get<int>(np) : nullptr;
        if (both) solve_both(ctx, *stack, ds, dw, n_points, M, opt, d);
        else solve1d_device(st, *stack, ds, dw, n_points, M, polarization, opt, d, chunk_bytes(ctx));
        copy_back(out->R, d.R, nv, st);
        copy_back(out->T, d.T, nv, st);
        copy_back(out->DEr, d.DEr, nv, st);
        copy_back(out->DEt, d.DEt, nv, st);
        copy_back(out->status, d.status, np, st);
        copy_back(out->eig_info, d.eig_info, np, st);
        copy_back(out->n_eig, d.n_eig, np, st);
        copy_back(out->n_dense_solve, d.n_dense_solve, np, st);
        if (out->n_lu) copy_back(out->n_lu, d.n_lu, np, st);
        if (opt.diagnostics) copy_back(out->max_eig_residual, d.max_eig_residual, np, st);
        RCWA_CUDA(stream_wait(st));
    });
}

int rcwa_gpu_field_slice(rcwa_gpu_ctx* ctx, const rcwa_complex* harmonics, int n, int nz, const double* kx,
                         const double* ky, int plane, int nt, double period, double at, rcwa_complex* out) {
    return guarded(ctx, [&] { field_slice_api(ctx->stream, harmonics, n, nz, kx, ky, plane, nt, period, at, out); });
}

int rcwa_gpu_phase_data(rcwa_gpu_ctx* ctx, const rcwa_complex* field, int nt, int nz, int reference,
                        const double* incident_k, const double* x, const double* y, const double* z,
                        const rcwa_complex* custom, double phase_floor, int unwrap, double* phase, double* amplitude,
                        unsigned char* mask, rcwa_complex* reference_out) {
    return guarded(ctx, [&] {
        phase_data_api(ctx->stream, field, nt, nz, reference, incident_k, x, y, z, custom, phase_floor, unwrap, phase,
                       amplitude, mask, reference_out);
    });
}

int rcwa_gpu_fourier_coefficients(rcwa_gpu_ctx* ctx, const double* edges, const rcwa_complex* values, int K,
                                  double period, int hmax, int method, int samples, rcwa_complex* out) {
    return guarded(ctx, [&] { fourier_coefficients_api(ctx->stream, edges, values, K, period, hmax, method, samples, out); });
}

namespace {
void solve2d_entry(rcwa_gpu_ctx* ctx, const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                   int factorization, const rcwa_options* options, rcwa_result2d* out, const FieldSpec* fs) {
    if (!stack || n_points < 0 || (n_points > 0 && !points)) throw EngineError{RCWA_EINVAL, "rcwa2d: stack and points are required"};
    if (!out || !out->Kx || !out->Ky || !out->kzI || !out->kzII || !out->Ex_r || !out->Ey_r || !out->Ez_r || !out->Ex_t ||
        !out->Ey_t || !out->Ez_t || !out->Rs || !out->Rp || !out->Ts || !out->Tp || !out->DEr || !out->DEt ||
        !out->prop_r || !out->prop_t || !out->status)
        throw EngineError{RCWA_EINVAL, "rcwa2d: every result array but the optional ones is required"};
    validate2d(*stack, points, n_points, M1, M2, factorization);
    const Options opt = to_options(options);
    if (n_points == 0) return;
    solve2d_host(ctx->stream, *stack, points, n_points, M1, M2, factorization, opt, *out, chunk_bytes2d(ctx), fs);
}
}  // namespace

int rcwa_gpu_solve2d_batch(rcwa_gpu_ctx* ctx, const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points,
                           int M1, int M2, int factorization, const rcwa_options* options, rcwa_result2d* out) {
    return guarded(ctx, [&] { solve2d_entry(ctx, stack, points, n_points, M1, M2, factorization, options, out, nullptr); });
}

int rcwa_gpu_solve2d_fields(rcwa_gpu_ctx* ctx, const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points,
                            int M1, int M2, int factorization, const rcwa_options* options, const double* zs, int nz,
                            rcwa_result2d* out, rcwa_complex* fields) {
    return guarded(ctx, [&] {
        if (nz < 0 || (nz > 0 && (!zs || !fields))) throw EngineError{RCWA_EINVAL, "rcwa2d: null argument"};
        FieldSpec fs;
        fs.zs.assign(zs, zs + nz);
        for (int k = 0; k < nz; ++k)
            if (!std::isfinite(zs[k])) throw EngineError{RCWA_EINVAL, "rcwa2d: field depths must be finite"};
        fs.out = reinterpret_cast<zc*>(fields);
        solve2d_entry(ctx, stack, points, n_points, M1, M2, factorization, options, out, nz > 0 ? &fs : nullptr);
    });
}

int rcwa_gpu_layer_operators2d(rcwa_gpu_ctx* ctx, const rcwa_layer2d* layer, double Lx, double Ly, int M1, int M2,
                               int factorization, rcwa_complex* eps, rcwa_complex* cx, rcwa_complex* cy, int* singular) {
    return guarded(ctx, [&] {
        if (!layer) throw EngineError{RCWA_EINVAL, "rcwa2d: layer is required"};
        layer_operators2d(ctx->stream, *layer, Lx, Ly, M1, M2, factorization, eps, cx, cy, singular);
    });
}

namespace {
// rcwa_gpu_solve_conical_batch and, with fs, rcwa_gpu_solve_conical_fields (fs->out: host fields)
void conical_batch(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point_conical* points, int n_points, int M,
                   const rcwa_options* options, rcwa_result_conical* out, const FieldSpec* fs) {
    if (!stack || (n_points > 0 && !points) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
    if (!out || !out->Jr || !out->Jt || !out->DEr || !out->DEt)
        throw EngineError{RCWA_EINVAL, "rcwa: result arrays Jr, Jt, DEr, DEt are required"};
    validate_conical(*stack, points, n_points, M);
    const Options opt = to_options(options);
    if (n_points == 0) return;
    const cudaStream_t st = ctx->stream;
    const int n = 2 * M + 1;
    // the incidence trigonometry with the host libm, the reference's own expressions
    // (include/stablercwa/rcwa1d_conical.hpp:704-730)
    const double kPi = 3.141592653589793238462643383279502884;
    const double nI = stack->nI.re;
    std::vector<double> h(6 * (size_t)n_points);
    for (int p = 0; p < n_points; ++p) {
        const double theta = points[p].theta_deg * kPi / 180.0, phi = points[p].phi_deg * kPi / 180.0;
        const double sine = nI * std::sin(theta);
        h[0 * (size_t)n_points + p] = sine * std::cos(phi);
        h[1 * (size_t)n_points + p] = sine * std::sin(phi);
        h[2 * (size_t)n_points + p] = std::cos(phi);
        h[3 * (size_t)n_points + p] = std::sin(phi);
        h[4 * (size_t)n_points + p] = std::cos(theta);
        h[5 * (size_t)n_points + p] = points[p].wavelength;
    }
    DeviceScratch mem(st);
    double* dh = mem.get<double>(h.size());
    RCWA_CUDA(cudaMemcpyAsync(dh, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    const ConicalPointsDev P{dh, dh + n_points, dh + 2 * (size_t)n_points, dh + 3 * (size_t)n_points,
                             dh + 4 * (size_t)n_points, dh + 5 * (size_t)n_points};
    const size_t nv = (size_t)n_points * n;
    rcwa_result_conical d{};
    d.Jr = reinterpret_cast<rcwa_complex*>(mem.get<zc>(nv * 4));
    d.Jt = reinterpret_cast<rcwa_complex*>(mem.get<zc>(nv * 4));
    d.DEr = mem.get<double>(nv * 4);
    d.DEt = mem.get<double>(nv * 4);
    d.status = mem.get<int>(n_points);
    d.eig_info = mem.get<int>(n_points);
    d.n_eig = mem.get<int>(n_points);
    d.n_dense_solve = mem.get<int>(n_points);
    d.n_lu = out->n_lu ? mem.get<int>(n_points) : nullptr;
    d.n_schur = mem.get<int>(n_points);
    d.min_abs_lambda = mem.get<double>(n_points);
    d.degenerate_mode_warning = mem.get<int>(n_points);
    d.kx = mem.get<double>(nv);
    d.ky = mem.get<double>(n_points);
    d.flux_r = mem.get<double>(nv);
    d.flux_t = mem.get<double>(nv);
    FieldSpec dfs;
    const size_t nf = fs ? (size_t)n_points * 6 * n * fs->zs.size() : 0;
    const size_t ni = fs && fs->layer_info ? (size_t)n_points * stack->n_layers : 0;
    if (fs) {
        dfs.zs = fs->zs;
        dfs.jones = fs->jones;
        dfs.out = nf > 0 ? mem.get<zc>(nf) : nullptr;
        dfs.layer_info = ni > 0 ? mem.zeros<int>(ni) : nullptr;
    }
    solve_conical_device(st, *stack, P, n_points, M, opt, d, chunk_bytes(ctx), fs && (nf > 0 || ni > 0) ? &dfs : nullptr);
    if (nf > 0) copy_back(fs->out, dfs.out, nf, st);
    if (ni > 0) copy_back(fs->layer_info, dfs.layer_info, ni, st);
    copy_back(out->Jr, d.Jr, nv * 4, st);
    copy_back(out->Jt, d.Jt, nv * 4, st);
    copy_back(out->DEr, d.DEr, nv * 4, st);
    copy_back(out->DEt, d.DEt, nv * 4, st);
    copy_back(out->status, d.status, n_points, st);
    copy_back(out->eig_info, d.eig_info, n_points, st);
    copy_back(out->n_eig, d.n_eig, n_points, st);
    copy_back(out->n_dense_solve, d.n_dense_solve, n_points, st);
    if (out->n_lu) copy_back(out->n_lu, d.n_lu, n_points, st);
    copy_back(out->n_schur, d.n_schur, n_points, st);
    copy_back(out->min_abs_lambda, d.min_abs_lambda, n_points, st);
    copy_back(out->degenerate_mode_warning, d.degenerate_mode_warning, n_points, st);
    copy_back(out->kx, d.kx, nv, st);
    copy_back(out->ky, d.ky, n_points, st);
    copy_back(out->flux_r, d.flux_r, nv, st);
    copy_back(out->flux_t, d.flux_t, nv, st);
    RCWA_CUDA(stream_wait(st));
}
}  // namespace

int rcwa_gpu_solve_conical_batch(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point_conical* points,
                                 int n_points, int M, const rcwa_options* options, rcwa_result_conical* out) {
    return guarded(ctx, [&] { conical_batch(ctx, stack, points, n_points, M, options, out, nullptr); });
}

int rcwa_gpu_solve_conical_fields(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point_conical* points,
                                  int n_points, int M, const rcwa_options* options, const rcwa_complex* jones,
                                  const double* zs, int nz, rcwa_result_conical* out, rcwa_complex* fields,
                                  int* layer_info) {
    return guarded(ctx, [&] {
        if (nz < 0 || (nz > 0 && (!zs || !fields)) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
        FieldSpec fs;
        fs.zs.assign(zs, zs + nz);
        for (int k = 0; k < nz; ++k)
            if (!std::isfinite(zs[k])) throw EngineError{RCWA_EINVAL, "rcwa: field depths must be finite"};
        if (jones) {  // rcwa::normalized_jones (include/stablercwa/rcwa_fields.hpp:218-230)
            fs.jones.resize(2 * (size_t)n_points);
            for (int p = 0; p < n_points; ++p) {
                std::complex<double> v[2] = {{jones[2 * p].re, jones[2 * p].im}, {jones[2 * p + 1].re, jones[2 * p + 1].im}};
                double scale = 0.0;
                for (const auto& x : v) {
                    if (!std::isfinite(x.real()) || !std::isfinite(x.imag()))
                        throw EngineError{RCWA_EINVAL, "rcwa: Jones input must be finite and nonzero"};
                    scale = std::max(scale, std::max(std::abs(x.real()), std::abs(x.imag())));
                }
                if (scale == 0.0) throw EngineError{RCWA_EINVAL, "rcwa: Jones input must be finite and nonzero"};
                for (auto& x : v) x /= scale;
                const double norm = std::sqrt(std::norm(v[0]) + std::norm(v[1]));
                for (auto& x : v) x /= norm;
                fs.jones[2 * p] = v[0];
                fs.jones[2 * p + 1] = v[1];
            }
        }
        fs.out = reinterpret_cast<zc*>(fields);
        fs.layer_info = layer_info;  // host here; conical_batch stages it on the device
        conical_batch(ctx, stack, points, n_points, M, options, out, &fs);
    });
}

int rcwa_gpu_solve1d_fields(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point1d* points, int n_points,
                            int M, int polarization, const rcwa_options* options, const double* zs, int nz,
                            rcwa_result1d* out, rcwa_complex* fields, int* layer_info) {
    return guarded(ctx, [&] {
        if (!stack || (n_points > 0 && !points) || n_points < 0 || nz < 0 || (nz > 0 && (!zs || !fields)))
            throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
        check_result_ptrs(out);
        validate1d(*stack, points, n_points, M, polarization);
        for (int k = 0; k < nz; ++k)
            if (!std::isfinite(zs[k])) throw EngineError{RCWA_EINVAL, "rcwa: field depths must be finite"};
        const Options opt = to_options(options);
        if (n_points == 0) return;
        const cudaStream_t st = ctx->stream;
        const int n = 2 * M + 1;
        std::vector<double> hs(n_points), hw(n_points);
        const double kPi = 3.141592653589793238462643383279502884;
        for (int p = 0; p < n_points; ++p) {
            hs[p] = stack->nI.re * std::sin(points[p].theta_deg * kPi / 180.0);
            hw[p] = points[p].wavelength;
        }
        DeviceScratch mem(st);
        double* ds = mem.get<double>(n_points);
        double* dw = mem.get<double>(n_points);
        RCWA_CUDA(cudaMemcpyAsync(ds, hs.data(), n_points * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dw, hw.data(), n_points * sizeof(double), cudaMemcpyHostToDevice, st));
        const size_t nv = (size_t)n_points * n, nf = (size_t)n_points * 6 * n * nz;
        rcwa_result1d d{};
        d.R = reinterpret_cast<rcwa_complex*>(mem.get<zc>(nv));
        d.T = reinterpret_cast<rcwa_complex*>(mem.get<zc>(nv));
        d.DEr = mem.get<double>(nv);
        d.DEt = mem.get<double>(nv);
        d.status = mem.get<int>(n_points);
        d.eig_info = mem.get<int>(n_points);
        d.n_eig = mem.get<int>(n_points);
        d.n_dense_solve = mem.get<int>(n_points);
        d.n_lu = out->n_lu ? mem.get<int>(n_points) : nullptr;
        FieldSpec fs;
        fs.zs.assign(zs, zs + nz);
        fs.out = nz > 0 ? mem.get<zc>(nf) : nullptr;
        const size_t ni = (size_t)n_points * stack->n_layers;
        if (layer_info && ni > 0) fs.layer_info = mem.zeros<int>(ni);
        solve1d_device(st, *stack, ds, dw, n_points, M, polarization, opt, d, chunk_bytes(ctx),
                       nz > 0 || fs.layer_info ? &fs : nullptr);
        if (fs.layer_info) copy_back(layer_info, fs.layer_info, ni, st);
        copy_back(out->R, d.R, nv, st);
        copy_back(out->T, d.T, nv, st);
        copy_back(out->DEr, d.DEr, nv, st);
        copy_back(out->DEt, d.DEt, nv, st);
        copy_back(out->status, d.status, n_points, st);
        copy_back(out->eig_info, d.eig_info, n_points, st);
        copy_back(out->n_eig, d.n_eig, n_points, st);
        copy_back(out->n_dense_solve, d.n_dense_solve, n_points, st);
        if (out->n_lu) copy_back(out->n_lu, d.n_lu, n_points, st);
        if (nz > 0) copy_back(reinterpret_cast<zc*>(fields), fs.out, nf, st);
        RCWA_CUDA(stream_wait(st));
    });
}

int rcwa_gpu_solve1d_batch_dev(rcwa_gpu_ctx* ctx, const rcwa_stack1d* stack, const rcwa_point1d* d_points, int n_points,
                               int M, int polarization, const rcwa_options* options, rcwa_result1d* d_out) {
    return guarded(ctx, [&] {
        if (!stack || (n_points > 0 && !d_points) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
        check_result_ptrs(d_out);
        const bool both = polarization == RCWA_TE_TM;
        validate1d(*stack, nullptr, 0, M, both ? RCWA_TE : polarization);
        if (both) validate1d(*stack, nullptr, 0, M, RCWA_TM);
        const Options opt = to_options(options);
        if (n_points == 0) return;
        const cudaStream_t st = ctx->stream;
        DeviceScratch mem(st);
        double* ds = mem.get<double>(n_points);
        double* dw = mem.get<double>(n_points);
        if (!prepare_points_device(st, d_points, n_points, stack->nI.re, ds, dw))
            throw EngineError{RCWA_EINVAL, "rcwa: every point needs a finite positive wavelength and |theta| < 90 degrees"};
        if (!both) {
            solve1d_device(st, *stack, ds, dw, n_points, M, polarization, opt, *d_out, chunk_bytes(ctx));
            return;
        }
        solve_both(ctx, *stack, ds, dw, n_points, M, opt, *d_out);
    });
}

int rcwa_gpu_eig_batch_dev(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* d_a, double eps, int max_iter,
                           rcwa_complex* d_values, rcwa_complex* d_vectors, int* d_info, int* d_sweeps) {
    return guarded(ctx, [&] {
        if (n < 0 || batch < 0) throw EngineError{RCWA_EINVAL, "eig: negative size"};
        if (max_iter < 1) throw EngineError{RCWA_EINVAL, "eig_qr: max_iter must be >= 1"};
        if (!(eps >= 0.0) || !std::isfinite(eps)) throw EngineError{RCWA_EINVAL, "eig_qr: eps must be finite and >= 0"};
        if (n == 0 || batch == 0) return;
        if (!d_a || !d_values || !d_vectors || !d_info) throw EngineError{RCWA_EINVAL, "eig: null argument"};
        DeviceScratch mem(ctx->stream);
        zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(n, batch) / sizeof(zc)) + 1);
        int group = 0;
        if (const char* g = std::getenv("RCWA_GB300_EIG_GROUP")) group = std::atoi(g);
        launch_eig(ctx->stream, n, batch, reinterpret_cast<const zc*>(d_a), (long long)n * n,
                   reinterpret_cast<zc*>(d_values), reinterpret_cast<zc*>(d_vectors), d_info, d_sweeps, ws, eps, max_iter,
                   group);
    });
}

namespace {
void check_eig_args(int n, int batch, double eps, int max_iter) {
    if (n < 0 || batch < 0) throw EngineError{RCWA_EINVAL, "eig: negative size"};
    if (max_iter < 1) throw EngineError{RCWA_EINVAL, "eig_qr: max_iter must be >= 1"};
    if (!(eps >= 0.0) || !std::isfinite(eps)) throw EngineError{RCWA_EINVAL, "eig_qr: eps must be finite and >= 0"};
}
int eig_group_from_env() {
    const char* g = std::getenv("RCWA_GB300_EIG_GROUP");
    return g ? std::atoi(g) : 0;
}
}  // namespace

int rcwa_gpu_eig_hermitian_batch_dev(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* d_a, double eps,
                                     int max_iter, rcwa_complex* d_values, rcwa_complex* d_vectors, int* d_info) {
    return guarded(ctx, [&] {
        check_eig_args(n, batch, eps, max_iter);
        if (n == 0 || batch == 0) return;
        if (!d_a || !d_values || !d_vectors || !d_info) throw EngineError{RCWA_EINVAL, "eig: null argument"};
        DeviceScratch mem(ctx->stream);
        zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(n, batch) / sizeof(zc)) + 1);
        launch_eig_herm(ctx->stream, n, batch, reinterpret_cast<const zc*>(d_a), (long long)n * n,
                        reinterpret_cast<zc*>(d_values), reinterpret_cast<zc*>(d_vectors), d_info, ws, eps, max_iter,
                        eig_group_from_env());
    });
}

int rcwa_gpu_eig_hermitian_batch(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* a, double eps, int max_iter,
                                 rcwa_complex* values, rcwa_complex* vectors, int* info) {
    return guarded(ctx, [&] {
        check_eig_args(n, batch, eps, max_iter);
        if (n == 0 || batch == 0) return;
        if (!a || !values || !vectors || !info) throw EngineError{RCWA_EINVAL, "eig: null argument"};
        const size_t nn = (size_t)n * n * batch;
        for (size_t k = 0; k < nn; ++k)
            if (!std::isfinite(a[k].re) || !std::isfinite(a[k].im))
                throw EngineError{RCWA_EINVAL, "eig_qr: matrix has non-finite entries"};
        const cudaStream_t st = ctx->stream;
        DeviceScratch mem(st);
        zc* da = mem.get<zc>(nn);
        zc* dw = mem.get<zc>((size_t)n * batch);
        zc* dv = mem.get<zc>(nn);
        int* di = mem.get<int>(batch);
        zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(n, batch) / sizeof(zc)) + 1);
        RCWA_CUDA(cudaMemcpyAsync(da, a, nn * sizeof(zc), cudaMemcpyHostToDevice, st));
        launch_eig_herm(st, n, batch, da, (long long)n * n, dw, dv, di, ws, eps, max_iter, eig_group_from_env());
        RCWA_CUDA(cudaMemcpyAsync(values, dw, (size_t)n * batch * sizeof(zc), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(vectors, dv, nn * sizeof(zc), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(cudaMemcpyAsync(info, di, batch * sizeof(int), cudaMemcpyDeviceToHost, st));
        RCWA_CUDA(stream_wait(st));
    });
}

int rcwa_gpu_eig_batch(rcwa_gpu_ctx* ctx, int n, int batch, const rcwa_complex* a, double eps, int max_iter,
                       rcwa_complex* values, rcwa_complex* vectors, int* info, int* sweeps) {
    return guarded(ctx, [&] {
        if (n < 0 || batch < 0) throw EngineError{RCWA_EINVAL, "eig: negative size"};
        if (max_iter < 1) throw EngineError{RCWA_EINVAL, "eig_qr: max_iter must be >= 1"};
        if (!(eps >= 0.0) || !std::isfinite(eps)) throw EngineError{RCWA_EINVAL, "eig_qr: eps must be finite and >= 0"};
        if (n == 0 || batch == 0) return;
        if (!a || !values || !vectors || !info) throw EngineError{RCWA_EINVAL, "eig: null argument"};
        const size_t nn = (size_t)n * n * batch;
        for (size_t k = 0; k < nn; ++k)
            if (!std::isfinite(a[k].re) || !std::isfinite(a[k].im))
                throw EngineError{RCWA_EINVAL, "eig_qr: matrix has non-finite entries"};
        const cudaStream_t st = ctx->stream;
        DeviceScratch mem(st);
        zc* da = mem.get<zc>(nn);
        zc* dw = mem.get<zc>((size_t)n * batch);
        zc* dv = mem.get<zc>(nn);
        int* di = mem.get<int>(batch);
        int* dsw = mem.get<int>(batch);
        zc* ws = mem.get<zc>((size_t)(eig_workspace_bytes(n, batch) / sizeof(zc)) + 1);
        RCWA_CUDA(cudaMemcpyAsync(da, a, nn * sizeof(zc), cudaMemcpyHostToDevice, st));
        int group = 0;
        if (const char* g = std::getenv("RCWA_GB300_EIG_GROUP")) group = std::atoi(g);
        launch_eig(st, n, batch, da, (long long)n * n, dw, dv, di, dsw, ws, eps, max_iter, group);
        copy_back(reinterpret_cast<zc*>(values), dw, (size_t)n * batch, st);
        copy_back(reinterpret_cast<zc*>(vectors), dv, nn, st);
        copy_back(info, di, batch, st);
        copy_back(sweeps, dsw, batch, st);
        RCWA_CUDA(stream_wait(st));
    });
}

int rcwa_gpu_solve_batch(rcwa_gpu_ctx* ctx, int n, int nrhs, int batch, const rcwa_complex* a, const rcwa_complex* b,
                         rcwa_complex* x, int* singular) {
    return guarded(ctx, [&] {
        if (n < 0 || nrhs < 0 || batch < 0) throw EngineError{RCWA_EINVAL, "solve: negative size"};
        if (n == 0 || nrhs == 0 || batch == 0) return;
        if (!a || !b || !x || !singular) throw EngineError{RCWA_EINVAL, "solve: null argument"};
        const cudaStream_t st = ctx->stream;
        const size_t na = (size_t)n * n * batch, nb = (size_t)n * nrhs * batch;
        DeviceScratch mem(st);
        zc* da = mem.get<zc>(na);
        zc* db = mem.get<zc>(nb);
        int* ds = mem.zeros<int>(batch);
        RCWA_CUDA(cudaMemcpyAsync(da, a, na * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(db, b, nb * sizeof(zc), cudaMemcpyHostToDevice, st));
        launch_lu_solve(st, n, nrhs, batch, da, (long long)n * n, da, (long long)n * n, RHS_DENSE, db, (long long)n * nrhs,
                        db, (long long)n * nrhs, ds);
        copy_back(reinterpret_cast<zc*>(x), db, nb, st);
        copy_back(singular, ds, batch, st);
        RCWA_CUDA(stream_wait(st));
    });
}

namespace {
int validated(char* message, size_t size, const std::function<void()>& check) {
    try {
        check();
        if (message && size) message[0] = '\0';
        return RCWA_OK;
    } catch (const EngineError& e) {
        if (message && size) {
            std::strncpy(message, e.message.c_str(), size - 1);
            message[size - 1] = '\0';
        }
        return e.code;
    } catch (const std::bad_alloc&) {
        return RCWA_ENOMEM;
    }
}
}  // namespace

int rcwa_validate_solve1d(const rcwa_stack1d* stack, const rcwa_point1d* points, int n_points, int M, int polarization,
                          char* message, size_t size) {
    return validated(message, size, [&] {
        if (!stack || (n_points > 0 && !points) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
        validate1d(*stack, points, n_points, M, polarization);
    });
}

int rcwa_validate_solve_conical(const rcwa_stack1d* stack, const rcwa_point_conical* points, int n_points, int M,
                                char* message, size_t size) {
    return validated(message, size, [&] {
        if (!stack || (n_points > 0 && !points) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
        validate_conical(*stack, points, n_points, M);
    });
}

int rcwa_validate_solve2d(const rcwa_stack2d* stack, const rcwa_point2d* points, int n_points, int M1, int M2,
                          int factorization, char* message, size_t size) {
    return validated(message, size, [&] {
        if (!stack || (n_points > 0 && !points) || n_points < 0) throw EngineError{RCWA_EINVAL, "rcwa2d: null argument"};
        validate2d(*stack, points, n_points, M1, M2, factorization);
    });
}

int rcwa_gpu_autotune_eig(rcwa_gpu_ctx* ctx, int hermitian, int n, int batch, const rcwa_complex* d_a, int* form,
                          double* milliseconds) {
    return guarded(ctx, [&] {
        if (n < 1 || batch < 1 || !d_a) throw EngineError{RCWA_EINVAL, "autotune: positive order and batch and a matrix array"};
        double ms = 0.0;
        const int f = autotune_eig(ctx->stream, hermitian ? 1 : 0, n, batch, reinterpret_cast<const zc*>(d_a),
                                   (long long)n * n, &ms);
        if (form) *form = f;
        if (milliseconds) *milliseconds = ms;
    });
}

int rcwa_gpu_autotune_set(int hermitian, int n, int batch, int form) {
    const bool ok_form = form == -1 || form == 4 || form == 8 || form == 16 || form == 32 || form == 64 || form == 128 ||
                         form == 256;
    if (n < 1 || batch < 1 || !ok_form || (form == -1 && hermitian)) return RCWA_EINVAL;
    set_tuned_eig_form(hermitian ? 1 : 0, n, batch, form);
    return RCWA_OK;
}

int rcwa_gpu_autotune_table(char* buffer, size_t size) {
    try {
        const std::string t = autotune_table_text();
        if (buffer && size) {
            std::strncpy(buffer, t.c_str(), size - 1);
            buffer[size - 1] = '\0';
        }
        return (int)t.size();
    } catch (...) {
        return RCWA_ENOMEM;
    }
}

int rcwa_gpu_gemm_info(int* tensor_cores, int* slices, int* stuck) {
    try {
        if (tensor_cores) *tensor_cores = tc_gemm_enabled() ? 1 : 0;
        if (slices) *slices = tc_gemm_slices();
        if (stuck) *stuck = tc_gemm_error();
        return RCWA_OK;
    } catch (const EngineError& e) {
        return e.code;
    }
}

int rcwa_gpu_multiply_batch(rcwa_gpu_ctx* ctx, int m, int k, int n, int batch, const rcwa_complex* a,
                            const rcwa_complex* b, rcwa_complex* c) {
    return guarded(ctx, [&] {
        if (m < 0 || k < 0 || n < 0 || batch < 0) throw EngineError{RCWA_EINVAL, "multiply: negative size"};
        if (m == 0 || n == 0 || batch == 0) return;
        if (!a || !b || !c) throw EngineError{RCWA_EINVAL, "multiply: null argument"};
        const cudaStream_t st = ctx->stream;
        const size_t na = (size_t)m * k * batch, nb = (size_t)k * n * batch, nc = (size_t)m * n * batch;
        DeviceScratch mem(st);
        zc* da = mem.get<zc>(na);
        zc* db = mem.get<zc>(nb);
        zc* dc = mem.get<zc>(nc);
        RCWA_CUDA(cudaMemcpyAsync(da, a, na * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(db, b, nb * sizeof(zc), cudaMemcpyHostToDevice, st));
        launch_zgemm(st, m, n, k, batch, da, m, (long long)m * k, db, k, (long long)k * n, nullptr, 0, dc, m,
                     (long long)m * n, 1.0, 0.0);
        copy_back(reinterpret_cast<zc*>(c), dc, nc, st);
        RCWA_CUDA(stream_wait(st));
    });
}

}  // extern "C"
