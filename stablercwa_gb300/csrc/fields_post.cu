// fields_post.cu -- real-space slices of field harmonics and their phase maps on the GPU: the engine
// behind rcwa::field_map / field_slice (detail::reconstruct_field_grid / reconstruct_field_slice,
// include/stablercwa/rcwa_fields.hpp:326-385) and rcwa::phase_data (include/stablercwa/rcwa_phase.hpp:229-271).
//
// Slice: the carrier exp(-i (kx_j x + ky_j y)) is formed once per (point, harmonic), then every output
// value (component, depth, point) is one thread's sum over the harmonics. Phase: amplitude, phase and
// reference per grid value in one pass, the finite amplitude peak by an atomic max on the bit pattern
// (non-negative doubles order like their bits), the mask against floor * peak, then the np.unwrap-style
// line unwrapping with one thread per row (horizontal) or column (depth).
#include <cmath>
#include <vector>

#include "smatrix.cuh"

namespace rcwa_gb300 {
namespace {

// carrier C[j * nt + it] = exp(-i (kx_j x_it + ky_j y_it)), t_it = (it / nt) period (rcwa_fields.hpp:193-204)
__global__ void slice_carrier_kernel(int n, int nt, const double* __restrict__ kx, const double* __restrict__ ky, int plane,
                                     double period, double at, zc* __restrict__ C, int* __restrict__ bad) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n * nt) return;
    const int j = (int)(idx / nt), it = (int)(idx - (long long)j * nt);
    const double t = ((double)it / nt) * period;
    const double x = plane == 0 ? t : at, y = plane == 0 ? at : t;
    const double a = kx[j] * x + ky[j] * y;
    double s, c;
    sincos(a, &s, &c);
    const zc v{c, -s};
    if (!zfinite(v)) *bad = 1;
    C[idx] = v;
}

// out[(c * nz + iz) * nt + it] = sum_j C[j][it] H[(c * n + j) * nz + iz]
__global__ void slice_sum_kernel(int n, int nz, int nt, const zc* __restrict__ C, const zc* __restrict__ H,
                                 zc* __restrict__ out, int* __restrict__ bad) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)nz * nt;
    if (idx >= 6 * per) return;
    const int c = (int)(idx / per);
    const long long r = idx - c * per;
    const int iz = (int)(r / nt), it = (int)(r - (long long)iz * nt);
    const zc* h = H + (long long)c * n * nz + iz;
    zc acc{0.0, 0.0};
    for (int j = 0; j < n; ++j) acc = zfma(C[(long long)j * nt + it], h[(long long)j * nz], acc);
    if (!zfinite(acc)) *bad = 1;
    out[idx] = acc;
}

__device__ __forceinline__ bool finite_ref(zc z) { return isfinite(z.re) && isfinite(z.im); }

// amplitude |f|, the reference (incident carrier or custom), phase arg(f conj(ref)) or arg(f), and the
// peak of the finite amplitudes (rcwa_phase.hpp:246-261, incident_reference :190-214)
__global__ void phase_prep_kernel(int nt, int nz, const zc* __restrict__ f, int ref_kind, const zc* __restrict__ custom,
                                  double kx0, double ky0, double kz0, const double* __restrict__ x, const double* __restrict__ y,
                                  const double* __restrict__ z, zc* __restrict__ ref, double* __restrict__ amp,
                                  double* __restrict__ phase, unsigned long long* __restrict__ peak_bits, int* __restrict__ bad) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nt * nz) return;
    const int iz = (int)(idx / nt), it = (int)(idx - (long long)iz * nt);
    const zc v = f[idx];
    const double a = hypot(v.re, v.im);
    amp[idx] = a;
    if (isfinite(a)) atomicMax(peak_bits, (unsigned long long)__double_as_longlong(a));
    zc w = v;
    if (ref_kind != 0) {
        zc rv;
        if (ref_kind == 1) {
            const double arg = (-kx0 * x[it] - ky0 * y[it]) + kz0 * z[iz];
            if (!isfinite(arg)) *bad = 1;
            double s, c;
            sincos(arg, &s, &c);
            rv = zc{c, s};
        } else {
            rv = custom[idx];
        }
        ref[idx] = rv;
        w = v * zc{rv.re, -rv.im};
    }
    phase[idx] = atan2(w.im, w.re);
}

__global__ void phase_mask_kernel(long long size, const zc* __restrict__ f, const double* __restrict__ amp,
                                  const zc* __restrict__ ref, double floor_, const unsigned long long* __restrict__ peak_bits,
                                  unsigned char* __restrict__ mask) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= size) return;
    const double peak = __longlong_as_double((long long)*peak_bits);
    bool m = !finite_ref(f[idx]) || amp[idx] <= floor_ * peak;
    if (ref) m = m || !finite_ref(ref[idx]) || hypot(ref[idx].re, ref[idx].im) == 0.0;
    mask[idx] = m ? 1 : 0;
}

// np.unwrap (period 2 pi, discontinuity pi) along one line; a masked value ends the run
// (unwrap_phase_line, rcwa_phase.hpp:94-113)
__device__ void unwrap_line(double* v, const unsigned char* mask, long long start, long long stride, int length) {
    const double kPi = 3.141592653589793238462643383279502884;
    bool active = false;
    double previous = 0.0, correction = 0.0;
    long long index = start;
    for (int j = 0; j < length; ++j, index += stride) {
        if (mask[index]) {
            active = false;
            correction = 0.0;
            continue;
        }
        const double original = v[index];
        if (active) {
            const double delta = original - previous;
            double wrapped = fmod(delta + kPi, 2.0 * kPi);
            if (wrapped < 0.0) wrapped += 2.0 * kPi;
            wrapped -= kPi;
            if (wrapped == -kPi && delta > 0.0) wrapped = kPi;
            if (fabs(delta) >= kPi) correction += wrapped - delta;
            v[index] = original + correction;
        }
        previous = original;
        active = true;
    }
}

__global__ void unwrap_rows_kernel(int nt, int nz, double* __restrict__ phase, const unsigned char* __restrict__ mask) {
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    if (iz < nz) unwrap_line(phase, mask, (long long)iz * nt, 1, nt);
}
__global__ void unwrap_cols_kernel(int nt, int nz, double* __restrict__ phase, const unsigned char* __restrict__ mask) {
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it < nt) unwrap_line(phase, mask, it, nt, nz);
}
__global__ void phase_nan_kernel(long long size, double* __restrict__ phase, const unsigned char* __restrict__ mask) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < size && mask[idx]) phase[idx] = __longlong_as_double(0x7ff8000000000000LL);
}

}  // namespace

void field_slice_api(cudaStream_t st, const rcwa_complex* harmonics, int n, int nz, const double* kx, const double* ky,
                     int plane, int nt, double period, double at, rcwa_complex* out) {
    // argument checks of slice_coordinates / slice_period (rcwa_fields.hpp:181-204)
    if (plane != RCWA_SLICE_XZ && plane != RCWA_SLICE_YZ) throw EngineError{RCWA_EINVAL, "rcwa: invalid slice plane"};
    if (nt <= 0) throw EngineError{RCWA_EINVAL, "rcwa: slice nt must be positive"};
    if (!std::isfinite(at)) throw EngineError{RCWA_EINVAL, "rcwa: slice coordinate must be finite"};
    if (!std::isfinite(period) || !(period > 0.0))
        throw EngineError{RCWA_EINVAL, "rcwa: slice period must be positive and finite"};
    if (n < 0 || nz < 0 || (n > 0 && (!kx || !ky)) || (n > 0 && nz > 0 && !harmonics) || (nz > 0 && !out))
        throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
    if (nz == 0) return;
    DeviceScratch mem(st);
    const size_t nh = (size_t)6 * n * nz, no = (size_t)6 * nz * nt;
    zc* H = mem.get<zc>(nh);
    double* dkx = mem.get<double>(n);
    double* dky = mem.get<double>(n);
    zc* C = mem.get<zc>((size_t)n * nt);
    zc* O = mem.get<zc>(no);
    int* bad = mem.zeros<int>(2);
    if (n > 0) {
        RCWA_CUDA(cudaMemcpyAsync(H, harmonics, nh * sizeof(zc), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dkx, kx, n * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dky, ky, n * sizeof(double), cudaMemcpyHostToDevice, st));
        LAUNCH(slice_carrier_kernel, nblocks((long long)n * nt), kTpb, st, n, nt, dkx, dky, plane, period, at, C, bad);
    }
    LAUNCH(slice_sum_kernel, nblocks((long long)no), kTpb, st, n, nz, nt, C, H, O, bad + 1);
    int hb[2] = {0, 0};
    RCWA_CUDA(cudaMemcpyAsync(hb, bad, sizeof hb, cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(cudaMemcpyAsync(out, O, no * sizeof(zc), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    if (hb[0]) throw EngineError{RCWA_ENUMERIC, "rcwa: field carrier produced nonfinite values"};
    if (hb[1]) throw EngineError{RCWA_ENUMERIC, "rcwa: field reconstruction produced nonfinite values"};
}

void phase_data_api(cudaStream_t st, const rcwa_complex* field, int nt, int nz, int reference, const double* incident_k,
                    const double* x, const double* y, const double* z, const rcwa_complex* custom, double phase_floor,
                    int unwrap, double* phase, double* amplitude, unsigned char* mask, rcwa_complex* reference_out) {
    // scalar_phase_data's checks (rcwa_phase.hpp:232-237) and those of incident_reference (:121-143, :204-214)
    if (!std::isfinite(phase_floor) || phase_floor < 0.0)
        throw EngineError{RCWA_EINVAL, "rcwa: phase_floor must be finite and nonnegative"};
    if (unwrap < RCWA_UNWRAP_NONE || unwrap > RCWA_UNWRAP_BOTH) throw EngineError{RCWA_EINVAL, "rcwa: unsupported phase unwrap axis"};
    if (reference < RCWA_PHASE_ABSOLUTE || reference > RCWA_PHASE_CUSTOM)
        throw EngineError{RCWA_EINVAL, "rcwa: unsupported phase reference"};
    if (nt < 0 || nz < 0) throw EngineError{RCWA_EINVAL, "rcwa: phase grid sizes must be nonnegative"};
    const long long size = (long long)nt * nz;
    if (size > 0 && (!field || !phase || !amplitude || !mask)) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
    if (reference == RCWA_PHASE_INCIDENT) {
        if (!incident_k || !std::isfinite(incident_k[0]) || !std::isfinite(incident_k[1]) || !std::isfinite(incident_k[2]))
            throw EngineError{RCWA_EINVAL, "rcwa: incident reference wavevector is unavailable"};
        if (size > 0 && (!x || !y || !z)) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
    }
    if (reference == RCWA_PHASE_CUSTOM && size > 0 && !custom) throw EngineError{RCWA_EINVAL, "rcwa: null argument"};
    if (size == 0) return;
    DeviceScratch mem(st);
    zc* f = mem.get<zc>(size);
    RCWA_CUDA(cudaMemcpyAsync(f, field, size * sizeof(zc), cudaMemcpyHostToDevice, st));
    zc* ref = reference != RCWA_PHASE_ABSOLUTE ? mem.get<zc>(size) : nullptr;
    zc* cus = nullptr;
    double *dx = nullptr, *dy = nullptr, *dz = nullptr;
    if (reference == RCWA_PHASE_CUSTOM) {
        cus = mem.get<zc>(size);
        RCWA_CUDA(cudaMemcpyAsync(cus, custom, size * sizeof(zc), cudaMemcpyHostToDevice, st));
    } else if (reference == RCWA_PHASE_INCIDENT) {
        dx = mem.get<double>(nt);
        dy = mem.get<double>(nt);
        dz = mem.get<double>(nz);
        RCWA_CUDA(cudaMemcpyAsync(dx, x, nt * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dy, y, nt * sizeof(double), cudaMemcpyHostToDevice, st));
        RCWA_CUDA(cudaMemcpyAsync(dz, z, nz * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    double* amp = mem.get<double>(size);
    double* ph = mem.get<double>(size);
    unsigned char* mk = mem.get<unsigned char>(size);
    unsigned long long* peak = mem.zeros<unsigned long long>(1);
    int* bad = mem.zeros<int>(1);
    const double k0x = incident_k ? incident_k[0] : 0.0, k0y = incident_k ? incident_k[1] : 0.0,
                 k0z = incident_k ? incident_k[2] : 0.0;
    LAUNCH(phase_prep_kernel, nblocks(size), kTpb, st, nt, nz, f, reference, cus, k0x, k0y, k0z, dx, dy, dz, ref, amp, ph, peak,
           bad);
    int hbad = 0;
    RCWA_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
    if (hbad) throw EngineError{RCWA_EINVAL, "rcwa: incident reference coordinates must be finite and representable"};
    LAUNCH(phase_mask_kernel, nblocks(size), kTpb, st, size, f, amp, ref, phase_floor, peak, mk);
    if (unwrap == RCWA_UNWRAP_X || unwrap == RCWA_UNWRAP_BOTH) LAUNCH(unwrap_rows_kernel, nblocks(nz, 128), 128, st, nt, nz, ph, mk);
    if (unwrap == RCWA_UNWRAP_Z || unwrap == RCWA_UNWRAP_BOTH) LAUNCH(unwrap_cols_kernel, nblocks(nt, 128), 128, st, nt, nz, ph, mk);
    LAUNCH(phase_nan_kernel, nblocks(size), kTpb, st, size, ph, mk);
    RCWA_CUDA(cudaMemcpyAsync(phase, ph, size * sizeof(double), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(cudaMemcpyAsync(amplitude, amp, size * sizeof(double), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(cudaMemcpyAsync(mask, mk, size, cudaMemcpyDeviceToHost, st));
    if (reference_out && ref) RCWA_CUDA(cudaMemcpyAsync(reference_out, ref, size * sizeof(zc), cudaMemcpyDeviceToHost, st));
    RCWA_CUDA(stream_wait(st));
}

}  // namespace rcwa_gb300
