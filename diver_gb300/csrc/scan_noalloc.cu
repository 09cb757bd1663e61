// Allocation-free form of the segment-offset prefix sum.
//
// dv_exclusive_scan needs a small scratch buffer for its per-tile sums, which
// the caller allocates.  Some callers cannot do that: a renderer embedded in a
// host application whose device memory is owned by another allocator (a game
// engine or a framework's caching pool that forbids raw cudaMalloc), code that
// runs where allocation is not allowed or too slow (inside a real-time frame
// loop with a fixed memory budget, or while a CUDA graph is being captured),
// and plugins loaded into a process that must not grow its device footprint
// per call.  This entry point takes only its inputs and outputs; its scratch
// is a fixed-size array in this library's own device memory.
//
// Limits and rules:
//   - at most DV_SCAN_STATIC_MAX_TILES tiles of 2048 counts, i.e. 8,388,608
//     counts per call; larger n is rejected with DV_ERR_OVERFLOW before any
//     launch;
//   - the array (32 KiB) exists on every device that loads the library and
//     stays allocated until the process exits;
//   - the first call on a device with n > 0 looks up the array's device
//     address (a one-time set-up per device, made with that device current);
//     make that first call before any stream capture.  The address is cached
//     for the process: after cudaDeviceReset (or any teardown of the device's
//     primary context) the library must not be called on that device again;
//   - n = 0 only writes offsets[0] = 0 and needs no set-up;
//   - all calls share the one array: calls whose work overlaps on the GPU
//     (different streams, or different host threads on the same device) race
//     on it and must be serialised by the caller;
//   - nothing in the array needs clearing between calls: every tile sum is
//     written before it is read, so the previous call's contents never leak
//     into the result.
#include "common.cuh"
#include "scan.cuh"

#include <mutex>

namespace {

constexpr long long DV_SCAN_STATIC_MAX_TILES = 4096;
constexpr int DV_MAX_DEVICES = 64;

// Per-tile sums of the allocation-free scan (host code must not use this
// name as a pointer: it is a host-side stand-in for the device symbol).
static __device__ __align__(256) long long g_scan_tile_sums[DV_SCAN_STATIC_MAX_TILES];

std::mutex g_setup_mutex;
long long* g_scratch_on_device[DV_MAX_DEVICES] = {};

// Device address of g_scan_tile_sums on the current device (set up once per device).
int static_scratch(long long** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DV_ERR_CUDA;
  if (dev < 0 || dev >= DV_MAX_DEVICES) return DV_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_on_device[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scan_tile_sums) != cudaSuccess || p == nullptr) return DV_ERR_CUDA;
    g_scratch_on_device[dev] = static_cast<long long*>(p);
  }
  *out = g_scratch_on_device[dev];
  return DV_OK;
}

}  // namespace

using namespace dv;

extern "C" {

long long dv_exclusive_scan_static_max(void) { return DV_SCAN_STATIC_MAX_TILES * SCAN_TILE; }

int dv_exclusive_scan_static(const int* counts, long long n, int64_t* offsets, void* stream) {
  DV_CHECK(n >= 0 && offsets, DV_ERR_ARG);
  if (n > DV_SCAN_STATIC_MAX_TILES * SCAN_TILE) return DV_ERR_OVERFLOW;
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    if (cudaMemsetAsync(offsets, 0, sizeof(int64_t), st) != cudaSuccess) return DV_ERR_CUDA;
    return DV_OK;
  }
  DV_CHECK(counts, DV_ERR_ARG);
  long long* tile_sum = nullptr;
  const int st_setup = static_scratch(&tile_sum);
  if (st_setup != DV_OK) return st_setup;
  const long long tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  scan_tile_sums<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(counts, n, tile_sum);
  scan_tile_prefix<<<1, SCAN_THREADS, 0, st>>>(tile_sum, tiles);
  scan_tiles<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(counts, n, tile_sum, offsets);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
