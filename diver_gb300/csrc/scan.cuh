// Exclusive prefix sum of int32 counts into int64 offsets (three phases over
// tiles of SCAN_TILE counts: per-tile sums, a scan of the tile sums, per-tile
// scans).  The kernels are defined in traverse.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dv {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void scan_tile_sums(const int* __restrict__ in, long long n, long long* __restrict__ tile_sum);
__global__ void scan_tile_prefix(long long* __restrict__ tile_sum, long long tiles);
__global__ void scan_tiles(const int* __restrict__ in, long long n, const long long* __restrict__ tile_prefix,
                           int64_t* __restrict__ out);

}  // namespace dv
