// gemm_tc.cu -- batched complex FP64 GEMM on the tensor cores (tcgen05, sm_103a), accurate to FP64.
//
// C = s_ab A B + s_c C0 with A m x k, B k x n complex double, any batch. The product is emulated with
// the Ozaki scheme (Ozaki, Ogita, Oishi and Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication", Numer. Algorithms 59, 2012) on
// bf16 tensor-core products:
//   * the complex product is one real product of twice the size: rows 2i and 2i+1 of A^ are
//     [Re A(i,:), -Im A(i,:)] and [Im A(i,:), Re A(i,:)], and B^ = [Re B; Im B], so (A^ B^)(2i, j) and
//     (A^ B^)(2i+1, j) are the real and imaginary parts of C(i, j);
//   * every row of A^ is scaled by a power of two 2^ea(i) taken from its largest entry, every column of
//     B^ by 2^eb(j), and each scaled entry y in (-1, 1) is split into S signed integer digits,
//     y = 2^-7 (d_1 + 2^-8 d_2 + ... + 2^-8(S-1) d_S), |d_s| <= 128: each digit is exact in bf16;
//   * the digit products d_s e_t are exact (<= 2^14) and a tensor-core sum of up to 1024 of them stays
//     an integer below 2^24, exact in the FP32 accumulator. Digit pairs (s, t) with s + t <= S + 1 are
//     kept (the dropped ones lie below 2^-8S of the product's scale); pairs of one diagonal s + t share
//     a scale factor 2^(-14 - 8 (s + t - 2)), so up to 1024 / K of them accumulate in one exact FP32
//     tensor-memory accumulator (a "group") before it is added, exactly, into an int64 per element.
// Per element the result is exact up to the digit truncation (relative 2^-8S of max|A(i,:)| max|B(:,j)|
// times k) and one final rounding: FP64-level accuracy with S = 7.
//
// Kernels. The split kernels write the digit planes in HBM as bf16 rows with K contiguous (K-major for
// both operands). The product kernel gives each CTA one 128 x 128 tile of C^ of one matrix: one warp
// issues TMA loads (128-byte swizzle, boxes of 128 rows x 64 K) into a 4-stage shared-memory ring; one
// thread issues tcgen05.mma (M = 128, N = 128, K = 16, bf16 in, FP32 out) into one of two 128-column
// tensor-memory accumulators; eight warps read each finished group out of tensor memory (tcgen05.ld) and
// add it, as an integer at its diagonal's weight, into one int64 per element while the next group
// accumulates in the other buffer, then convert once, apply 2^(ea + eb), pair the real and imaginary rows
// and write C. Every mbarrier wait is bounded: on
// expiry the kernel records an error, drains its own copies and products, frees its tensor memory and
// returns without writing C.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "engine.h"

namespace rcwa_gb300 {
namespace {

constexpr int kTileM = 128, kTileN = 128, kTileK = 64;  // K per stage: 64 bf16 = one 128-byte swizzle row
constexpr int kStages = 4;
constexpr int kStageBytes = (kTileM + kTileN) * kTileK * 2;  // 32 KB
constexpr int kTmemCols = 256;                                // two accumulators of 128 columns
constexpr int kThreads = 320;                                 // producer, MMA, 8 epilogue warps
constexpr int kMaxGroups = 160;
constexpr int kMaxSlices = 8;
constexpr unsigned kWaitLimit = 1u << 22;  // try_wait rounds before a wait is declared stuck

// One accumulation group: digit pairs (i, d - i) for i in [i0, i0 + ni), K blocks [kb0, kb0 + nkb).
struct Plan {
    int n_groups;
    int S;
    int s0;  // the int64 accumulator holds the product in units of 2^(-14 - s0) (diagonal d enters times 2^(s0 - 8 (d - 2)))
    unsigned g[kMaxGroups];  // d | i0 << 4 | ni << 8 | kb0 << 12 | nkb << 22
};
__host__ __device__ inline int g_d(unsigned v) { return v & 15; }
__host__ __device__ inline int g_i0(unsigned v) { return (v >> 4) & 15; }
__host__ __device__ inline int g_ni(unsigned v) { return (v >> 8) & 15; }
__host__ __device__ inline int g_kb0(unsigned v) { return (v >> 12) & 1023; }
__host__ __device__ inline int g_nkb(unsigned v) { return (v >> 22) & 1023; }

// ---------------------------------------------------------------- PTX wrappers

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of bar: false when the CTA is aborting or the wait ran out (which
// starts the abort and records it in *err).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* err) {
    for (unsigned it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && *abort_flag) return false;
        if (it >= kWaitLimit) {
            *abort_flag = 1;
            atomicOr(err, 1);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor of a K-major tile written by TMA with the 128-byte swizzle: rows of
// 128 bytes, 8-row atoms 1024 bytes apart (stride byte offset), descriptor version 1 (bits 46-48)
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)2 << 61);
}

// instruction descriptor: D f32, A and B bf16, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTileN >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// ---------------------------------------------------------------- digit split

// A row of A or column of B holding a non-finite entry gets this exponent: its digits come out zero and
// the epilogue writes NaN for every element of C it touches (any such product is non-finite in FP64 too).
constexpr int kNonFinite = 1 << 20;

// The split kernels use no FP64 arithmetic: the FP64 pipe of this GPU runs 1/32 of the FP32 rate, and
// conversions between FP64 and 64-bit integers run there too. Magnitudes are compared as the bit patterns
// of |x| (ordered like the values), and a value is brought to fixed point from its exponent and mantissa.
constexpr unsigned long long kMagInf = 0x7FF0000000000000ull;
// |x| as a comparable bit pattern; kMagInf for inf and NaN
__device__ __forceinline__ unsigned long long mag_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    return b >= kMagInf ? kMagInf : b;
}

// the scale exponent of a row or column from its largest magnitude's bits: max = f 2^e with f in [0.5, 1);
// kNonFinite when the row or column holds a non-finite entry, 0 when it is zero
__device__ __forceinline__ int scale_exponent(unsigned long long mb) {
    if (mb >= kMagInf) return kNonFinite;
    if (mb == 0) return 0;
    const int be = (int)(mb >> 52);
    if (be == 0) {  // a subnormal maximum (the FP64 path: rare)
        int e;
        frexp(__longlong_as_double((long long)mb), &e);
        return e;
    }
    return be - 1022;
}

// Y = x 2^(62 - e) rounded to the nearest integer (ties to even), for |x| < 2^e: |Y| < 2^62
__device__ __forceinline__ long long fixed62(double x, int e) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7FF);
    if (be == 0) {
        if ((b << 1) == 0) return 0;
        return __double2ll_rn(ldexp(x, 62 - e));  // subnormal: the FP64 path
    }
    const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = be - 1075 + 62 - e;  // |Y| = mant 2^sh; |x| < 2^e keeps sh <= 9
    unsigned long long m = 0;
    if (sh >= 0) {
        m = mant << sh;
    } else if (sh > -64) {
        const int r = -sh;
        const unsigned long long rem = mant & ((1ull << r) - 1ull), half = 1ull << (r - 1);
        m = mant >> r;
        if (rem > half || (rem == half && (m & 1ull))) ++m;
    }
    return (b >> 63) ? -(long long)m : (long long)m;
}

// x 2^e2 as the nearest double (ties to even), for |x| < 2^63, from integer operations only: the FP64 pipe
// of this GPU runs 1/32 of the FP32 rate, so the epilogue's conversions would otherwise dominate the tile.
// False when the result is not a normal double (the caller converts in FP64 then).
__device__ __forceinline__ bool i64_ldexp_bits(long long x, int e2, unsigned long long& bits) {
    if (x == 0) {
        bits = 0;
        return true;
    }
    const unsigned long long sign = x < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long u = x < 0 ? 0ull - (unsigned long long)x : (unsigned long long)x;
    const int msb = 63 - __clzll((long long)u);
    int ex = msb + e2;
    unsigned long long mant;
    if (msb > 52) {
        const int r = msb - 52;
        const unsigned long long rem = u & ((1ull << r) - 1ull), half = 1ull << (r - 1);
        mant = u >> r;
        if (rem > half || (rem == half && (mant & 1ull))) ++mant;
        if (mant >> 53) {
            mant >>= 1;
            ++ex;
        }
    } else {
        mant = u << (52 - msb);
    }
    if (ex < -1022 || ex > 1023) return false;
    bits = sign | ((unsigned long long)(ex + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull);
    return true;
}

// c as an integer count of 2^e2 units (nearest, ties to even), for adding C0 into the accumulator; false when
// c is subnormal, not finite, or at least 2^61 units (the caller adds in FP64 then)
__device__ __forceinline__ bool double_to_units(double c, int e2, long long& t) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(c);
    const int be = (int)((b >> 52) & 0x7FF);
    if (be == 0) {
        t = 0;
        return (b << 1) == 0;
    }
    if (be == 0x7FF) return false;
    const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = (be - 1075) - e2;  // c = mant 2^(be - 1075)
    unsigned long long m = 0;
    if (sh >= 0) {
        if (sh > 8) return false;
        m = mant << sh;
    } else if (sh > -64) {
        const int r = -sh;
        const unsigned long long rem = mant & ((1ull << r) - 1ull), half = 1ull << (r - 1);
        m = mant >> r;
        if (rem > half || (rem == half && (m & 1ull))) ++m;
    }
    t = (b >> 63) ? -(long long)m : (long long)m;
    return true;
}

// bf16 bit pattern of a small integer (exact for |d| <= 256), from integer operations
__device__ __forceinline__ uint16_t bf16_int(long long d) {
    if (d == 0) return 0;
    const unsigned sign = d < 0 ? 0x8000u : 0u;
    const unsigned a = (unsigned)(d < 0 ? -d : d);
    const int p = 31 - __clz((int)a);  // a = 1.f 2^p
    return (uint16_t)(sign | ((unsigned)(p + 127) << 7) | ((a << (7 - p)) & 0x7Fu));
}

// The S digits of x 2^-e (|x 2^-e| < 1), integer arithmetic: Y = x 2^(62 - e) is the value to 62 fractional
// bits (an int64 below 2^62, so adding the rounding half never overflows); digit s (from 0) is Y rounded at
// bit 55 - 8 s and taken out of Y before the next, so each lies in [-128, 128] and carries weight
// 2^(-7 - 8 s); an eighth digit is the remainder itself, in units of 2^-63. A non-finite x (whose row or
// column then carries kNonFinite) gives zero digits.
__device__ __forceinline__ void split_digits(double x, int e, int S, uint16_t* dg) {
    if (mag_bits(x) >= kMagInf || e == kNonFinite) {
        for (int s = 0; s < S; ++s) dg[s] = 0;
        return;
    }
    long long Y = fixed62(x, e);
#pragma unroll 1
    for (int s = 0; s < S; ++s) {
        const int sh = 55 - 8 * s;
        long long d;
        if (sh > 0) {
            d = (Y + (1LL << (sh - 1))) >> sh;
            Y -= d * (1LL << sh);
        } else {
            d = Y * (1LL << -sh);
            Y = 0;
        }
        dg[s] = bf16_int(d);
    }
}

__device__ __forceinline__ void store_digits(double x, int e, int S, uint16_t* out, long long plane_stride) {
    if (mag_bits(x) >= kMagInf || e == kNonFinite) {
        for (int s = 0; s < S; ++s) out[s * plane_stride] = 0;
        return;
    }
    long long Y = fixed62(x, e);
#pragma unroll 1
    for (int s = 0; s < S; ++s) {
        const int sh = 55 - 8 * s;
        long long d;
        if (sh > 0) {
            d = (Y + (1LL << (sh - 1))) >> sh;
            Y -= d * (1LL << sh);
        } else {
            d = Y * (1LL << -sh);
            Y = 0;
        }
        out[s * plane_stride] = bf16_int(d);
    }
}

// A (m x k, column-major, lda) of matrix blockIdx.y -> S planes of A^ (2m rows x Kp, K contiguous) and
// ea[i]; one CTA per 32 rows of A. Complex B (real_b = 0): rows 2i, 2i+1 = [Re A(i,:), -Im A(i,:)] and
// [Im A(i,:), Re A(i,:)] over K = 2k; real B (real_b = 1): rows [Re A(i,:)] and [Im A(i,:)] over K = k.
// A is read through a shared-memory tile (coalesced along the rows) and written row by row.
__global__ void __launch_bounds__(256) tc_split_a_kernel(int m, int k, int Kp, int S, int real_b, const zc* __restrict__ A,
                                                         int lda, long long a_stride, uint16_t* __restrict__ out,
                                                         int* __restrict__ ea) {
    const long long b = blockIdx.y;
    const int i0 = blockIdx.x * 32, t = threadIdx.x, il = t & 31, w = t >> 5;
    const zc* As = A + b * a_stride;
    __shared__ unsigned long long smax[8][32];
    __shared__ int sexp[32];
    __shared__ zc tile[32][33];
    unsigned long long mx = 0;
    if (i0 + il < m)
        for (int kk = w; kk < k; kk += 8) {
            const zc v = As[(long long)kk * lda + i0 + il];
            mx = max(mx, max(mag_bits(v.re), mag_bits(v.im)));
        }
    smax[w][il] = mx;
    __syncthreads();
    if (w == 0) {
        for (int q = 1; q < 8; ++q) mx = max(mx, smax[q][il]);
        sexp[il] = scale_exponent(mx);
        if (i0 + il < m) ea[b * m + i0 + il] = sexp[il];
    }
    __syncthreads();
    const long long rows = 2LL * m, plane = rows * Kp;
    uint16_t* o = out + b * S * plane;
    const int kin = real_b ? k : 2 * k;  // K of the product before padding
    for (int kc = 0; kc < k; kc += 32) {
        for (int q = w; q < 32; q += 8) {
            const int kk = kc + q, i = i0 + il;
            tile[il][q] = (kk < k && i < m) ? As[(long long)kk * lda + i] : zc{0.0, 0.0};
        }
        __syncthreads();
        // each value is split once: Re A(i, kk) goes to row 2i at kk and row 2i+1 at k + kk, Im A(i, kk) to row
        // 2i+1 at kk and, negated digit by digit (the negated digits sum exactly to -Im A), to row 2i at k + kk
        for (int idx = t; idx < 64 * 32; idx += 256) {
            const int vi = idx >> 5, c = idx & 31, kk = kc + c;
            const int il2 = vi >> 1, im_part = vi & 1, i = i0 + il2;
            if (i >= m || kk >= k) continue;
            const zc v = tile[il2][c];
            uint16_t dg[kMaxSlices];
            split_digits(im_part ? v.im : v.re, sexp[il2], S, dg);
            uint16_t* first = o + (2LL * i + im_part) * Kp + kk;
            for (int s2 = 0; s2 < S; ++s2) first[s2 * plane] = dg[s2];
            if (!real_b) {
                uint16_t* second = o + (2LL * i + (1 - im_part)) * Kp + k + kk;
                for (int s2 = 0; s2 < S; ++s2)
                    second[s2 * plane] = im_part && dg[s2] ? (uint16_t)(dg[s2] ^ 0x8000u) : dg[s2];
            }
        }
        __syncthreads();
    }
    for (int idx = t; idx < 64 * (Kp - kin); idx += 256) {  // zero padding of K
        const int rr = idx / (Kp - kin), kk = kin + idx - rr * (Kp - kin);
        const int i = i0 + (rr >> 1), part = rr & 1;
        if (i >= m) continue;
        uint16_t* cell = o + (2LL * i + part) * Kp + kk;
        for (int s2 = 0; s2 < S; ++s2) cell[s2 * plane] = 0;
    }
}

// B (k x n, column-major, ldb) -> S planes of B^t (n rows x Kp) and eb[j]; one warp per column. Complex B:
// [Re B(:, j); Im B(:, j)]; real B (Br, double): B(:, j).
__global__ void __launch_bounds__(128) tc_split_b_kernel(int n, int k, int Kp, int S, int batch, const zc* __restrict__ B,
                                                         const double* __restrict__ Br, int ldb, long long b_stride,
                                                         uint16_t* __restrict__ out, int* __restrict__ eb) {
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (long long)batch * n) return;
    const long long b = gw / n;
    const int j = (int)(gw - b * n), lane = threadIdx.x & 31;
    unsigned long long mx = 0;
    if (Br) {
        const double* col = Br + b * b_stride + (long long)j * ldb;
        for (int kk = lane; kk < k; kk += 32) mx = max(mx, mag_bits(col[kk]));
    } else {
        const zc* col = B + b * b_stride + (long long)j * ldb;
        for (int kk = lane; kk < k; kk += 32) mx = max(mx, max(mag_bits(col[kk].re), mag_bits(col[kk].im)));
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = scale_exponent(mx);
    if (lane == 0) eb[b * n + j] = e;
    const long long plane = (long long)n * Kp;
    uint16_t* o = out + b * S * plane + (long long)j * Kp;
    for (int kk = lane; kk < Kp; kk += 32) {
        double x;
        if (Br) {
            x = kk < k ? Br[b * b_stride + (long long)j * ldb + kk] : 0.0;
        } else {
            const zc* col = B + b * b_stride + (long long)j * ldb;
            x = kk < k ? col[kk].re : (kk < 2 * k ? col[kk - k].im : 0.0);
        }
        store_digits(x, e, S, o + kk, plane);
    }
}

// ---------------------------------------------------------------- the product

// One element of C from its int64 accumulator ac (units of 2^(e - 14 - s0)), e = ea + eb: s_ab = +-1 and
// s_c in {0, 1} (unit_scales) without FP64 arithmetic (C0's part joins as an integer count of the same unit,
// one rounding to double by integer operations), anything else in FP64; NaN for a non-finite row or column.
__device__ __forceinline__ double finish_element(long long ac, int e, int s0, bool neg, bool unit_scales, const double* C0d,
                                                 long long off2, double s_ab, double s_c) {
    if (e >= kNonFinite / 2) return __longlong_as_double(0x7FF8000000000000LL);
    const int e2 = e - 14 - s0;
    long long a = neg ? -ac : ac;
    bool fast = unit_scales;
    if (fast && C0d) {
        long long t;
        fast = double_to_units(C0d[off2], e2, t);
        a += t;
    }
    unsigned long long bits;
    if (fast && i64_ldexp_bits(a, e2, bits)) return __longlong_as_double((long long)bits);
    double out = s_ab * ldexp((double)ac, e2);
    if (C0d) out = fma(s_c, C0d[off2], out);
    return out;
}

struct SharedState {
    uint64_t full[kStages], empty[kStages], tfull[2], tempty[2], drain;
    uint32_t tmem_base;
    int abort_flag;
};

__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, const __grid_constant__ Plan plan,
                   int m, int n, int batch0, int a_bcast, int b_bcast, const int* __restrict__ ea, const int* __restrict__ eb,
                   const zc* C0, long long c0_stride, zc* C, int ldc, long long c_stride, double s_ab, double s_c,
                   const int* __restrict__ skip, int skip_value, int* __restrict__ err) {
    const int lb = blockIdx.z;  // matrix within this chunk
    if (skip && skip[batch0 + lb] == skip_value) return;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    SharedState* ss = reinterpret_cast<SharedState*>(smem + kStages * kStageBytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kTileM, n0 = blockIdx.x * kTileN;
    const int S = plan.S;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&ss->full[s], 1);
            mbar_init(&ss->empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&ss->tfull[s], 1);
            mbar_init(&ss->tempty[s], 8);
        }
        mbar_init(&ss->drain, 1);
        ss->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ss->tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ss->tmem_base;
    volatile int* abort_flag = &ss->abort_flag;
    const int za = a_bcast ? 0 : lb, zb = b_bcast ? 0 : lb;

    if (warp == 0) {
        // ---- TMA producer
        if (lane == 0) {
            int it = 0;
            int issued[kStages];
            for (int s = 0; s < kStages; ++s) issued[s] = -1;
            bool ok = true;
            for (int gi = 0; gi < plan.n_groups && ok; ++gi) {
                const unsigned g = plan.g[gi];
                const int d = g_d(g);
                for (int p = 0; p < g_ni(g) && ok; ++p) {
                    const int i = g_i0(g) + p, j = d - i;
                    for (int kb = g_kb0(g); kb < g_kb0(g) + g_nkb(g); ++kb, ++it) {
                        const int st = it % kStages, ph = (it / kStages) & 1;
                        if (!mbar_wait(&ss->empty[st], ph ^ 1, abort_flag, err)) {
                            ok = false;
                            break;
                        }
                        unsigned char* sa = smem + st * kStageBytes;
                        mbar_expect_tx(&ss->full[st], kStageBytes);
                        tma_load_3d(sa, &map_a, kb * kTileK, m0, za * S + i - 1, &ss->full[st]);
                        tma_load_3d(sa + kTileM * kTileK * 2, &map_b, kb * kTileK, n0, zb * S + j - 1, &ss->full[st]);
                        issued[st] = it;
                    }
                }
            }
            if (!ok) {
                // drain: wait (bounded) for the copies this thread started into each stage
                for (int s = 0; s < kStages; ++s) {
                    if (issued[s] < 0) continue;
                    const int ph = (issued[s] / kStages) & 1;
                    for (unsigned r = 0; r < kWaitLimit && !mbar_try_wait(&ss->full[s], ph); ++r) {
                    }
                }
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            bool any = false;
            for (int gi = 0; gi < plan.n_groups && ok; ++gi) {
                const unsigned g = plan.g[gi];
                const int buf = gi & 1;
                if (!mbar_wait(&ss->tempty[buf], ((gi >> 1) & 1) ^ 1, abort_flag, err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t d_tmem = tmem + buf * kTileN;
                uint32_t acc = 0;
                for (int p = 0; p < g_ni(g) && ok; ++p) {
                    for (int kb = 0; kb < g_nkb(g); ++kb, ++it) {
                        const int st = it % kStages, ph = (it / kStages) & 1;
                        if (!mbar_wait(&ss->full[st], ph, abort_flag, err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t a_addr = smem_u32(smem + st * kStageBytes);
                        const uint32_t b_addr = a_addr + kTileM * kTileK * 2;
#pragma unroll
                        for (int kk = 0; kk < kTileK / 16; ++kk) {
                            mma_bf16(d_tmem, smem_desc_sw128(a_addr + kk * 32), smem_desc_sw128(b_addr + kk * 32), acc);
                            acc = 1;
                        }
                        any = true;
                        mma_commit(&ss->empty[st]);  // the stage is free once these products have read it
                    }
                }
                if (ok) mma_commit(&ss->tfull[buf]);
            }
            if (!ok && any) {
                // drain: every product issued so far completes before the accumulators are freed
                mma_commit(&ss->drain);
                for (unsigned r = 0; r < kWaitLimit && !mbar_try_wait(&ss->drain, 0); ++r) {
                }
            }
        }
    } else {
        // ---- epilogue: warps 2..9; lane quarter q of tensor memory, column half h
        const int q = warp & 3, h = (warp - 2) >> 2;
        // Every group sum is an integer below 2^24 (exact in the FP32 accumulator). They are added into one
        // int64 per element in units of 2^(-14 - s0): diagonal d enters times 2^(s0 - 8 (d - 2)), exactly
        // while that shift is >= 0, else rounded right (half a unit per group at most); s0 = 47 - log2(Kp)
        // keeps the whole sum below 2^62, so the unit is 2^-53 of the row-and-column scale for K = 256.
        // Integer sums are exact in any order; the element is then (double) acc 2^(ea + eb - 14 - s0), one
        // rounding.
        long long acc[64];
#pragma unroll
        for (int c = 0; c < 64; ++c) acc[c] = 0;
        bool ok = true;
        for (int gi = 0; gi < plan.n_groups; ++gi) {
            const int buf = gi & 1;
            ok = mbar_wait(&ss->tfull[buf], (gi >> 1) & 1, abort_flag, err);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            tc_fence_after();
            const int d = g_d(plan.g[gi]);
            const int sh = plan.s0 - 8 * (d - 2);
            const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + buf * kTileN + h * 64;
            const int lsh = sh >= 0 ? sh : 0, rsh = sh >= 0 ? 0 : -sh;  // one of them is zero
            const long long half = rsh ? (1LL << (rsh - 1)) : 0LL;
#pragma unroll
            for (int c16 = 0; c16 < 4; ++c16) {
                float v[16];
                tmem_ld16(base + c16 * 16, v);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    acc[c16 * 16 + j] += (((long long)__float2int_rn(v[j]) << lsh) + half) >> rsh;
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ss->tempty[buf]);
        }
        if (ok && !*abort_flag) {
            // Each lane writes its own row's part of C: row r of C^ is the real (r even) or imaginary part of
            // row r / 2 of C, so a warp's 32 lanes store 32 consecutive doubles of a column. With s_ab = +-1
            // and s_c in {0, 1} (every product of the solves) the element is formed without FP64 arithmetic:
            // C0's part joins the accumulator as an integer count of the same unit, and the sum is rounded
            // once to a double by integer operations; anything else takes the FP64 path.
            const int r = m0 + q * 32 + lane;  // row of A^
            const int i = r >> 1, part = r & 1;
            const int er = (i < m) ? ea[(long long)(a_bcast ? 0 : batch0 + lb) * m + i] : 0;
            const int* ebs = eb + (long long)(b_bcast ? 0 : batch0 + lb) * n;
            double* Cd = reinterpret_cast<double*>(C + (long long)(batch0 + lb) * c_stride);
            const double* C0d = C0 && s_c != 0.0 ? reinterpret_cast<const double*>(C0 + (long long)(batch0 + lb) * c0_stride)
                                                 : nullptr;
            const bool unit_scales = (s_ab == 1.0 || s_ab == -1.0) && (C0d == nullptr || s_c == 1.0);
            const bool neg = s_ab < 0.0;
            // The accumulators go to shared memory first (the stage ring is idle once the last group has
            // landed; column-major by thread, so a warp's accesses are conflict-free), which keeps the
            // conversion loop below out of the registers that hold them.
            long long* sacc = reinterpret_cast<long long*>(smem);
            const int et = threadIdx.x - 64;
#pragma unroll
            for (int c = 0; c < 64; ++c) sacc[c * 256 + et] = acc[c];
            if (i < m) {
#pragma unroll 2
                for (int c = 0; c < 64; ++c) {
                    const int col = n0 + h * 64 + c;
                    if (col >= n) break;
                    const long long ac = sacc[c * 256 + et];
                    const int e = er + ebs[col];
                    const long long off2 = 2 * ((long long)col * ldc + i) + part;
                    Cd[off2] = finish_element(ac, e, plan.s0, neg, unit_scales, C0d, off2, s_ab, s_c);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// ---------------------------------------------------------------- the slice-resident product
//
// The same product with each operand tile loaded once per K block instead of once per digit pair: a CTA
// computes a 128 x 64 tile of C^; per K block of 64 the producer loads the S slices of B's 64 rows (one B
// stage, S x 8 KB, double-buffered) and then the S slices of A's 128 rows one after another (a 4-deep
// ring of 16 KB), and A slice s meets every B slice t with s + t <= S - 1 (0-based) while it is resident:
// 4 MMAs (M 128, N 64, K 16) per pair into the tensor-memory accumulator of its diagonal s + t (S
// accumulators of 64 columns). 168 KB of operand tiles feed 28 pairs per K block for S = 7, against 32 KB
// per pair in the kernel above: about 2.7x fewer bytes per MMA. Every accumulator sums at most S pairs over
// K chunks of 128 (S x 128 x 2^14 <= 2^24, exact in FP32); after each chunk the eight epilogue warps add
// the S accumulators into their int64 registers at each diagonal's weight (the same units as above) while
// the MMA warp waits for them, then the last chunk's sums are converted as above.
constexpr int kTileNr = 64;                                   // columns of C^ per CTA
constexpr int kBStage = kMaxSlices * kTileNr * kTileK * 2;     // one K block of every B slice: 64 KB
constexpr int kATile = kTileM * kTileK * 2;                    // one A slice tile: 16 KB
constexpr int kARing = 4;
constexpr int kChunkKb = 2;                                    // K blocks per exact accumulation chunk
constexpr uint32_t kIdescN64 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTileNr >> 3) << 17) |
                               ((uint32_t)(kTileM >> 4) << 24);

__device__ __forceinline__ void mma_bf16_n64(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdescN64), "r"(accumulate)
        : "memory");
}

struct SharedStateR {
    uint64_t afull[kARing], aempty[kARing], bfull[2], bempty[2], tfull, tempty, drain;
    uint32_t tmem_base;
    int abort_flag;
};

__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_resident_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int S,
                            int s0, int kblocks, int m, int n, int batch0, int a_bcast, int b_bcast,
                            const int* __restrict__ ea, const int* __restrict__ eb, const zc* C0, long long c0_stride,
                            zc* C, int ldc, long long c_stride, double s_ab, double s_c, const int* __restrict__ skip,
                            int skip_value, int* __restrict__ err) {
    const int lb = blockIdx.z;
    if (skip && skip[batch0 + lb] == skip_value) return;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* bst = smem;                    // 2 B stages
    unsigned char* ast = smem + 2 * kBStage;      // the A ring
    SharedStateR* ss = reinterpret_cast<SharedStateR*>(ast + kARing * kATile);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kTileM, n0 = blockIdx.x * kTileNr;
    const int nchunks = (kblocks + kChunkKb - 1) / kChunkKb;

    if (threadIdx.x == 0) {
        for (int r = 0; r < kARing; ++r) {
            mbar_init(&ss->afull[r], 1);
            mbar_init(&ss->aempty[r], 1);
        }
        for (int r = 0; r < 2; ++r) {
            mbar_init(&ss->bfull[r], 1);
            mbar_init(&ss->bempty[r], 1);
        }
        mbar_init(&ss->tfull, 1);
        mbar_init(&ss->tempty, 8);
        mbar_init(&ss->drain, 1);
        ss->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ss->tmem_base)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ss->tmem_base;
    volatile int* abort_flag = &ss->abort_flag;
    const int za = a_bcast ? 0 : lb, zb = b_bcast ? 0 : lb;

    if (warp == 0) {
        // ---- TMA producer: per K block one B stage (all slices), then the A slices through the ring
        if (lane == 0) {
            bool ok = true;
            int ai = 0, bi = 0;
            int aissued[kARing], bissued[2];
            for (int r = 0; r < kARing; ++r) aissued[r] = -1;
            bissued[0] = bissued[1] = -1;
            for (int kb = 0; kb < kblocks && ok; ++kb) {
                const int b = bi & 1, bph = (bi >> 1) & 1;
                if (!mbar_wait(&ss->bempty[b], bph ^ 1, abort_flag, err)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(&ss->bfull[b], (uint32_t)(S * kTileNr * kTileK * 2));
                for (int t = 0; t < S; ++t)
                    tma_load_3d(bst + b * kBStage + t * (kTileNr * kTileK * 2), &map_b, kb * kTileK, n0, zb * S + t,
                                &ss->bfull[b]);
                bissued[b] = bi;
                ++bi;
                for (int sl = 0; sl < S; ++sl, ++ai) {
                    const int r = ai % kARing, aph = (ai / kARing) & 1;
                    if (!mbar_wait(&ss->aempty[r], aph ^ 1, abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&ss->afull[r], (uint32_t)kATile);
                    tma_load_3d(ast + r * kATile, &map_a, kb * kTileK, m0, za * S + sl, &ss->afull[r]);
                    aissued[r] = ai;
                }
            }
            if (!ok) {  // drain: wait (bounded) for the copies this thread started
                for (int r = 0; r < kARing; ++r) {
                    if (aissued[r] < 0) continue;
                    const int ph = (aissued[r] / kARing) & 1;
                    for (unsigned it = 0; it < kWaitLimit && !mbar_try_wait(&ss->afull[r], ph); ++it) {
                    }
                }
                for (int r = 0; r < 2; ++r) {
                    if (bissued[r] < 0) continue;
                    const int ph = (bissued[r] >> 1) & 1;
                    for (unsigned it = 0; it < kWaitLimit && !mbar_try_wait(&ss->bfull[r], ph); ++it) {
                    }
                }
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            bool ok = true, any = false;
            int ai = 0, bi = 0;
            for (int c = 0; c < nchunks && ok; ++c) {
                if (!mbar_wait(&ss->tempty, (c & 1) ^ 1, abort_flag, err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int kb0 = c * kChunkKb, kb1 = min(kblocks, kb0 + kChunkKb);
                for (int kb = kb0; kb < kb1 && ok; ++kb) {
                    const int b = bi & 1, bph = (bi >> 1) & 1;
                    if (!mbar_wait(&ss->bfull[b], bph, abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t b_base = smem_u32(bst + b * kBStage);
                    for (int sl = 0; sl < S; ++sl, ++ai) {
                        const int r = ai % kARing, aph = (ai / kARing) & 1;
                        if (!mbar_wait(&ss->afull[r], aph, abort_flag, err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t a_addr = smem_u32(ast + r * kATile);
                        for (int t = 0; t + sl < S; ++t) {
                            const uint32_t b_addr = b_base + t * (kTileNr * kTileK * 2);
                            const uint32_t d_tmem = tmem + (uint32_t)((sl + t) * kTileNr);
#pragma unroll
                            for (int kk = 0; kk < kTileK / 16; ++kk) {
                                const uint32_t acc = (kb == kb0 && sl == 0 && kk == 0) ? 0u : 1u;
                                mma_bf16_n64(d_tmem, smem_desc_sw128(a_addr + kk * 32), smem_desc_sw128(b_addr + kk * 32),
                                             acc);
                            }
                        }
                        any = true;
                        mma_commit(&ss->aempty[r]);  // the A tile is free once these products have read it
                    }
                    if (!ok) break;
                    mma_commit(&ss->bempty[b]);
                    ++bi;
                }
                if (ok) mma_commit(&ss->tfull);
            }
            if (!ok && any) {
                mma_commit(&ss->drain);
                for (unsigned it = 0; it < kWaitLimit && !mbar_try_wait(&ss->drain, 0); ++it) {
                }
            }
        }
    } else {
        // ---- epilogue: warps 2..9; lane quarter q of tensor memory, column half h (32 of the 64 columns)
        const int q = warp & 3, h = (warp - 2) >> 2;
        long long acc[32];
#pragma unroll
        for (int cc = 0; cc < 32; ++cc) acc[cc] = 0;
        bool ok = true;
        for (int c = 0; c < nchunks; ++c) {
            ok = mbar_wait(&ss->tfull, c & 1, abort_flag, err);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            tc_fence_after();
            for (int dg = 0; dg < S; ++dg) {  // diagonal dg = s + t enters at 2^(s0 - 8 dg)
                const int sh = s0 - 8 * dg;
                const int lsh = sh >= 0 ? sh : 0, rsh = sh >= 0 ? 0 : -sh;
                const long long half = rsh ? (1LL << (rsh - 1)) : 0LL;
                const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(dg * kTileNr + h * 32);
#pragma unroll
                for (int c16 = 0; c16 < 2; ++c16) {
                    float v[16];
                    tmem_ld16(base + c16 * 16, v);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        acc[c16 * 16 + j] += (((long long)__float2int_rn(v[j]) << lsh) + half) >> rsh;
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ss->tempty);
        }
        if (ok && !*abort_flag) {
            const int r = m0 + q * 32 + lane;  // row of A^
            const int i = r >> 1, part = r & 1;
            const int er = (i < m) ? ea[(long long)(a_bcast ? 0 : batch0 + lb) * m + i] : 0;
            const int* ebs = eb + (long long)(b_bcast ? 0 : batch0 + lb) * n;
            double* Cd = reinterpret_cast<double*>(C + (long long)(batch0 + lb) * c_stride);
            const double* C0d = C0 && s_c != 0.0 ? reinterpret_cast<const double*>(C0 + (long long)(batch0 + lb) * c0_stride)
                                                 : nullptr;
            const bool unit_scales = (s_ab == 1.0 || s_ab == -1.0) && (C0d == nullptr || s_c == 1.0);
            const bool neg = s_ab < 0.0;
            long long* sacc = reinterpret_cast<long long*>(ast);  // the A ring is idle after the last chunk
            const int et = threadIdx.x - 64;
#pragma unroll
            for (int cc = 0; cc < 32; ++cc) sacc[cc * 256 + et] = acc[cc];
            if (i < m) {
#pragma unroll 2
                for (int cc = 0; cc < 32; ++cc) {
                    const int col = n0 + h * 32 + cc;
                    if (col >= n) break;
                    const long long off2 = 2 * ((long long)col * ldc + i) + part;
                    Cd[off2] = finish_element(sacc[cc * 256 + et], er + ebs[col], s0, neg, unit_scales, C0d, off2, s_ab, s_c);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

// ---------------------------------------------------------------- host side

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(f);
    });
    if (!fn) throw EngineError{RCWA_ECUDA, "tensor-core GEMM: cuTensorMapEncodeTiled is not available"};
    return fn;
}

// digit planes (planes x rows x Kp bf16, K contiguous) as a 3-D tensor map with 64 x box_rows boxes
CUtensorMap plane_map(const uint16_t* base, long long rows, int Kp, long long planes, int box_rows = kTileM) {
    CUtensorMap map;
    const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)rows * Kp * 2};
    const cuuint32_t box[3] = {(cuuint32_t)kTileK, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<uint16_t*>(base), dims, strides,
                                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw EngineError{RCWA_ECUDA, "tensor-core GEMM: tensor map encoding failed"};
    return map;
}

// The groups, smallest contributions first: diagonal d = S + 1 down to 2, K in chunks of at most 1024,
// at most 1024 / (chunk length) digit pairs per group so every group's sum is exact in FP32.
Plan make_plan(int S, int kblocks) {
    Plan p{};
    p.S = S;
    int lg = 0;
    while ((1 << lg) < kblocks * kTileK) ++lg;
    p.s0 = 47 - lg;
    const int chunk_kb = 1024 / kTileK;
    for (int d = S + 1; d >= 2; --d) {
        const int lo = std::max(1, d - S), hi = std::min(S, d - 1);
        for (int kb0 = 0; kb0 < kblocks; kb0 += chunk_kb) {
            const int nkb = std::min(chunk_kb, kblocks - kb0);
            const int per = std::max(1, 1024 / (nkb * kTileK));
            for (int i0 = lo; i0 <= hi; i0 += per) {
                if (p.n_groups >= kMaxGroups) throw EngineError{RCWA_EUNSUPPORTED, "tensor-core GEMM: K too large"};
                const int ni = std::min(per, hi - i0 + 1);
                p.g[p.n_groups++] = (unsigned)d | (unsigned)i0 << 4 | (unsigned)ni << 8 | (unsigned)kb0 << 12 |
                                    (unsigned)nkb << 22;
            }
        }
    }
    return p;
}

int* error_flag() { return static_cast<int*>(device_word(1, sizeof(int))); }

}  // namespace

// the slice-resident kernel when RCWA_GB300_TC_KERNEL=resident. Not the default: it moves 2.7x fewer bytes
// from L2 per MMA but measured slower (4096 products of order 121: 9.8 ms against 8.8 ms; tensor pipe 17 %
// against 22 %): its tiles are half as wide, so twice the CTAs pay the per-tile setup and epilogue, and its
// single set of accumulators makes the MMAs wait for every chunk's drain. A persistent form that overlaps
// one tile's epilogue with the next tile's products is what it needs.
bool tc_gemm_resident() {
    static const bool on = [] {
        const char* e = std::getenv("RCWA_GB300_TC_KERNEL");
        return e && std::strcmp(e, "resident") == 0;
    }();
    return on;
}

int tc_gemm_slices() {
    static const int s = [] {
        const char* e = std::getenv("RCWA_GB300_TC_SLICES");
        const int v = e ? std::atoi(e) : 7;
        return std::min(kMaxSlices, std::max(2, v));
    }();
    return s;
}

bool tc_gemm_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("RCWA_GB300_GEMM");
        return !(e && std::strcmp(e, "fp64") == 0);
    }();
    return on;
}

namespace {
thread_local int g_fp64_guards = 0;
}
Fp64ProductsGuard::Fp64ProductsGuard() { ++g_fp64_guards; }
Fp64ProductsGuard::~Fp64ProductsGuard() { --g_fp64_guards; }
bool Fp64ProductsGuard::active() { return g_fp64_guards > 0; }

int tc_gemm_error() {
    int h = 0;
    RCWA_CUDA(cudaMemcpy(&h, error_flag(), sizeof(int), cudaMemcpyDeviceToHost));
    return h;
}

namespace {

// C = s_ab A B + s_c C0 with B complex (B) or real (Br)
void tc_product(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride, const zc* B,
                const double* Br, int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc,
                long long c_stride, double s_ab, double s_c, const int* skip, int skip_value) {
    if (batch <= 0 || m <= 0 || n <= 0) return;
    const bool resident = tc_gemm_resident();
    const int smem_bytes = resident ? 2 * kBStage + kARing * kATile + 1024 + (int)sizeof(SharedStateR) + 64
                                    : kStages * kStageBytes + 1024 + (int)sizeof(SharedState) + 64;
    if (resident) ensure_smem_optin(reinterpret_cast<const void*>(tc_gemm_resident_kernel), smem_bytes);
    else ensure_smem_optin(reinterpret_cast<const void*>(tc_gemm_kernel), smem_bytes);
    const int real_b = Br != nullptr;
    const int S = tc_gemm_slices();
    const int kin = real_b ? k : 2 * k;
    const int Kp = ((kin + kTileK - 1) / kTileK) * kTileK;
    const Plan plan = make_plan(S, Kp / kTileK);
    const bool a_bcast = a_stride == 0, b_bcast = b_stride == 0;
    const long long a_bytes = (long long)S * 2 * m * Kp * 2, b_bytes = (long long)S * n * Kp * 2;
    // matrices per pass: digit planes of at most ~1 GiB
    const long long per = (a_bcast ? 0 : a_bytes) + (b_bcast ? 0 : b_bytes) + 1;
    const int chunk = (int)std::max(1LL, std::min<long long>(batch, (1LL << 30) / per));
    int* err = error_flag();

    uint16_t *pa = nullptr, *pb = nullptr;
    int *dea = nullptr, *deb = nullptr;
    const int na = a_bcast ? 1 : chunk, nb = b_bcast ? 1 : chunk;
    RCWA_CUDA(cudaMallocAsync(&pa, (size_t)a_bytes * na, st));
    RCWA_CUDA(cudaMallocAsync(&pb, (size_t)b_bytes * nb, st));
    RCWA_CUDA(cudaMallocAsync(&dea, sizeof(int) * (size_t)m * (a_bcast ? 1 : batch), st));
    RCWA_CUDA(cudaMallocAsync(&deb, sizeof(int) * (size_t)n * (b_bcast ? 1 : batch), st));
    const CUtensorMap map_a = plane_map(pa, 2LL * m, Kp, (long long)na * S);
    const CUtensorMap map_b = plane_map(pb, n, Kp, (long long)nb * S, resident ? kTileNr : kTileN);
    if (a_bcast) {
        tc_split_a_kernel<<<dim3((m + 31) / 32, 1), 256, 0, st>>>(m, k, Kp, S, real_b, A, lda, 0, pa, dea);
        ++launch_count();
    }
    if (b_bcast) {
        tc_split_b_kernel<<<(unsigned)((n * 32LL + 127) / 128), 128, 0, st>>>(n, k, Kp, S, 1, B, Br, ldb, 0, pb, deb);
        ++launch_count();
    }
    for (int b0 = 0; b0 < batch; b0 += chunk) {
        const int cb = std::min(chunk, batch - b0);
        if (!a_bcast) {
            tc_split_a_kernel<<<dim3((m + 31) / 32, cb), 256, 0, st>>>(m, k, Kp, S, real_b, A + (long long)b0 * a_stride, lda,
                                                                        a_stride, pa, dea + (long long)b0 * m);
            ++launch_count();
        }
        if (!b_bcast) {
            tc_split_b_kernel<<<(unsigned)((cb * (long long)n * 32 + 127) / 128), 128, 0, st>>>(
                n, k, Kp, S, cb, B ? B + (long long)b0 * b_stride : nullptr, Br ? Br + (long long)b0 * b_stride : nullptr,
                ldb, b_stride, pb, deb + (long long)b0 * n);
            ++launch_count();
        }
        if (resident) {
            const dim3 grid((n + kTileNr - 1) / kTileNr, (2 * m + kTileM - 1) / kTileM, cb);
            tc_gemm_resident_kernel<<<grid, kThreads, smem_bytes, st>>>(map_a, map_b, S, plan.s0, Kp / kTileK, m, n, b0,
                                                                        a_bcast, b_bcast, dea, deb, C0, c0_stride, C, ldc,
                                                                        c_stride, s_ab, s_c, skip, skip_value, err);
        } else {
            const dim3 grid((n + kTileN - 1) / kTileN, (2 * m + kTileM - 1) / kTileM, cb);
            tc_gemm_kernel<<<grid, kThreads, smem_bytes, st>>>(map_a, map_b, plan, m, n, b0, a_bcast, b_bcast, dea, deb, C0,
                                                               c0_stride, C, ldc, c_stride, s_ab, s_c, skip, skip_value, err);
        }
        ++launch_count();
        RCWA_CUDA(cudaGetLastError());
    }
    RCWA_CUDA(cudaFreeAsync(pa, st));
    RCWA_CUDA(cudaFreeAsync(pb, st));
    RCWA_CUDA(cudaFreeAsync(dea, st));
    RCWA_CUDA(cudaFreeAsync(deb, st));
}

}  // namespace

void launch_zgemm_tc(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                     const zc* B, int ldb, long long b_stride, const zc* C0, long long c0_stride, zc* C, int ldc,
                     long long c_stride, double s_ab, double s_c, const int* skip, int skip_value) {
    tc_product(st, m, n, k, batch, A, lda, a_stride, B, nullptr, ldb, b_stride, C0, c0_stride, C, ldc, c_stride, s_ab, s_c,
               skip, skip_value);
}

void launch_zdgemm_tc(cudaStream_t st, int m, int n, int k, int batch, const zc* A, int lda, long long a_stride,
                      const double* B, int ldb, long long b_stride, zc* C, int ldc, long long c_stride, const int* skip,
                      int skip_value) {
    tc_product(st, m, n, k, batch, A, lda, a_stride, nullptr, B, ldb, b_stride, nullptr, 0, C, ldc, c_stride, 1.0, 0.0,
               skip, skip_value);
}

}  // namespace rcwa_gb300
