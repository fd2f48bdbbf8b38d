// Dependency-count export for callers that cannot allocate device memory.
//
// sw_get_dependency_counts stages the per-(cell, direction) counts in a buffer it
// obtains from cudaMalloc for the duration of the call.  Some callers cannot allow
// that: a host framework whose device memory is owned by its own pool allocator (an
// ECS engine that sized its GPU budget up front), code that must not trigger the
// implicit device synchronisation cudaMalloc/cudaFree can cause, and processes whose
// allocation calls are intercepted or capped.  sw_get_dependency_counts_noalloc does
// the same work but stages the counts in a file-scope __device__ array of fixed size,
// so the call itself allocates nothing.
//
// The array (kNoAllocScratchBytes, 16 MiB) lives in every GPU context that loads this
// library, until the process exits.  Host code cannot use the array's name as a
// device address (it names a host-side stand-in), so the first call on each device
// looks the address up with cudaGetSymbolAddress while that device is current; make
// that first call before any stream capture.  The address stays valid while the
// device's primary context lives: a caller that resets the device (cudaDeviceReset)
// must not call this entry point again in the same process.  All calls share the one
// array and it keeps the last call's contents, so each call clears the part it uses
// first; calls that overlap on the GPU (two handles on two streams at once) race on it.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/subsweep_gpu.h"
#include "launch.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
uint8_t* g_scratch_address[kMaxDevices];  // device address of the array, per device

// The handle's error message for a failed CUDA call, naming this entry point.
sw_status cuda_failure(sw_handle* h, cudaError_t e, const char* where) {
  char msg[256];
  snprintf(msg, sizeof(msg), "dependency counts (noalloc): %s: %s", where, cudaGetErrorString(e));
  return swh::handle_fail(h, e == cudaErrorMemoryAllocation ? SW_ERR_OOM : SW_ERR_CUDA, msg);
}

}  // namespace

extern "C" sw_status sw_get_dependency_counts_noalloc(sw_handle* h, int32_t level, uint8_t* counts) {
  swh::HandleView v;
  if (!swh::handle_view(h, &v) || !counts) return SW_ERR_INVALID_ARG;
  swh::handle_clear_error(h);
  if (level < 0 || level >= v.num_levels) return swh::handle_fail(h, SW_ERR_INVALID_ARG, "level out of range");
  const size_t need = (size_t)v.num_cells * (size_t)v.num_directions;
  if (need > kNoAllocScratchBytes) {
    char msg[200];
    snprintf(msg, sizeof(msg),
             "sw_get_dependency_counts_noalloc: %zu cells x directions exceed its fixed %zu-byte scratch array",
             need, kNoAllocScratchBytes);
    return swh::handle_fail(h, SW_ERR_INVALID_ARG, msg);
  }
  if (v.device < 0 || v.device >= kMaxDevices)
    return swh::handle_fail(h, SW_ERR_UNSUPPORTED, "device ordinal above the scratch table");
  if (v.p->num_spaces > 1)
    return swh::handle_fail(h, SW_ERR_UNSUPPORTED,
                            "sw_get_dependency_counts_noalloc: a handle split into task spaces (use "
                            "sw_get_dependency_counts)");
  // the handle's device is current during the call; the caller's device afterwards
  swh::DeviceScope device_scope(v.device);
  if (device_scope.status != cudaSuccess) return cuda_failure(h, device_scope.status, "select device");
  cudaError_t e = cudaSuccess;
  uint8_t* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[v.device]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_failure(h, e, "address of the scratch array");
      g_scratch_address[v.device] = static_cast<uint8_t*>(ptr);
    }
    scratch = g_scratch_address[v.device];
  }
  // inactive cells' entries are not written by the counting kernel: start from zero
  e = cudaMemsetAsync(scratch, 0, need, v.stream);
  if (e == cudaSuccess) e = v.ops->init_counts(*v.p, level, scratch, false, v.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts, scratch, need, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return cuda_failure(h, e, "count kernel and copy");
  return SW_OK;
}
