// Host stand-ins for the CUDA names the eigensolver kernels use, so that tests/emu/herm_emu.cpp can run
// those kernels on the CPU: every emulated thread of one group or CTA is a std::thread, barriers and
// shuffles meet at one std::barrier, shared arrays are statics shared by the emulated threads of the
// one block in flight. Test infrastructure only; it emulates semantics, not performance.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#define __host__
#define __device__
#define __forceinline__ inline
#define __global__
#define __launch_bounds__(x)
#define __align__(x) alignas(x)
#define __restrict__
#define __shared__ static
#define RCWA_DYN_SMEM(T, name) static T name[64 * 1024]

using std::max;
using std::min;
struct dim3e {
    unsigned x, y = 0, z = 0;
};
extern thread_local dim3e threadIdx;
inline dim3e blockIdx{0}, blockDim{32};
struct int2 {
    int x, y;
};
struct double2 {
    double x, y;
};
struct int4 {
    int x, y, z, w;
};
inline int4 make_int4(int a, int b, int c, int d) { return {a, b, c, d}; }
inline double2 make_double2(double a, double b) { return {a, b}; }
inline int2 make_int2(int a, int b) { return {a, b}; }
inline double __longlong_as_double(long long v) {
    double d;
    std::memcpy(&d, &v, 8);
    return d;
}
inline long long __double_as_longlong(double d) {
    long long v;
    std::memcpy(&v, &d, 8);
    return v;
}

void emu_sync();
double emu_shfl_xor(double v, int o);
int emu_shfl_xor_i(int v, int o);
unsigned emu_ballot(int pred);
inline void __syncwarp(unsigned = 0xffffffffu) { emu_sync(); }
inline void __syncthreads() { emu_sync(); }
inline double __shfl_xor_sync(unsigned, double v, int o, int = 32) { return emu_shfl_xor(v, o); }
inline int __shfl_xor_sync(unsigned, int v, int o, int = 32) { return emu_shfl_xor_i(v, o); }
inline unsigned __ballot_sync(unsigned, int pred) { return emu_ballot(pred); }
inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
    const unsigned long long o = *p;  // the harness runs the kernels that count one thread at a time
    *p += v;
    return o;
}
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
