// launch.cuh -- launch geometry helpers and the counted launch macro shared by the engine's kernels.
#pragma once

#include "engine.h"

namespace rcwa_gb300 {
namespace {

constexpr int kTpb = 256;
inline unsigned nblocks(long long total, int tpb = kTpb) {
    return static_cast<unsigned>((total + tpb - 1) / tpb > 0 ? (total + tpb - 1) / tpb : 1);
}
inline unsigned warp_blocks(long long warps) { return static_cast<unsigned>((warps * 32 + 127) / 128); }

}  // namespace
}  // namespace rcwa_gb300

// every kernel launch of the engine goes through LAUNCH: it is counted (launch_count) and checked
#define LAUNCH(kernel, grid, block, st, ...)                      \
    do {                                                         \
        kernel<<<(grid), (block), 0, (st)>>>(__VA_ARGS__);       \
        ++launch_count();                                        \
        RCWA_CUDA(cudaGetLastError());                           \
    } while (0)
