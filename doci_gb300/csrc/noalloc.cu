// noalloc.cu -- doci_multidot_noalloc: the projections of doci_multidot with
// no device allocation at all.
//
// Some callers cannot let a library call cudaMalloc/cudaMallocAsync: a
// process that has pre-reserved the GPU's memory in its own pool (a serving
// loop that keeps many Davidson states resident, or a framework's caching
// allocator) can see such an allocation fail or fragment its pool, and a
// latency-critical loop cannot afford the device-wide synchronisation an
// allocation or a free may trigger.  This entry point serves them: the caller
// passes inputs and outputs, and the per-block partial sums go to a fixed
// file-scope device array instead of stream-ordered scratch.
//
// The array is part of this library's device image: every GPU that loads the
// library holds it (kScratchDoubles doubles = 256 KiB) until the process
// exits.  All calls share it, so calls that overlap on the GPU (on different
// streams, or from different host threads without ordering) race on it.
// Every slot a call reads is written earlier in the same call, so nothing
// needs clearing between calls.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"
#include "vec.h"

namespace doci {
namespace {

constexpr int kMaxBlocks = 1024;  // partial-sum rows: grid blocks of the reduction
constexpr int kMaxM = 32;         // projections per call
constexpr int kScratchDoubles = kMaxBlocks * kMaxM;

static __device__ __align__(256) double g_multidot_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (host code cannot use the symbol itself as a device pointer) and
// kept for the life of the process: a cudaDeviceReset reloads the device image
// elsewhere, so the entry point is not for use on a device after a reset.
int scratch_address(double **out) {
  int dev = 0;
  DOCI_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return DOCI_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    DOCI_CUDA(cudaGetSymbolAddress(&p, g_multidot_scratch));
    g_scratch_addr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[dev];
  return DOCI_OK;
}

}  // namespace
}  // namespace doci

using namespace doci;

extern "C" int doci_multidot_noalloc(const void *d_V, int64_t ld, int m, const void *d_w, int64_t n, int precision,
                                     double *d_out, void *stream) {
  if (!d_V || !d_w || !d_out || m < 1 || n < 0 || ld < n) return DOCI_ERR_INVALID;
  if (precision != DOCI_FP64 && precision != DOCI_FP32) return DOCI_ERR_INVALID;
  if (m > kMaxM) return DOCI_ERR_SCRATCH_LIMIT;
  // the partial-sum buffer the projection pass needs: a counter and the
  // results (36 doubles; the counter starts at zero with the array and every
  // pass resets it) and m partials per block
  if (36 + static_cast<int64_t>(vec_reduction_blocks()) * m > kScratchDoubles) return DOCI_ERR_SCRATCH_LIMIT;
  double *scratch = nullptr;
  const int s0 = scratch_address(&scratch);
  if (s0 != DOCI_OK) return s0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int s = precision == DOCI_FP64
                    ? vec_multidot<double>(static_cast<const double *>(d_V), static_cast<size_t>(ld), m,
                                           static_cast<const double *>(d_w), static_cast<size_t>(n), scratch, st)
                    : vec_multidot<float>(static_cast<const float *>(d_V), static_cast<size_t>(ld), m,
                                          static_cast<const float *>(d_w), static_cast<size_t>(n), scratch, st, true);
  if (s != DOCI_OK) return s;
  return vec_reduce(scratch, m, d_out, st);
}
