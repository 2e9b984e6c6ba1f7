// Allocation-free variant of pdq_lml_fixed_grid.
//
// Some callers cannot call cudaMalloc: plugin hosts that only hand over the
// input and output buffers of a call (a custom-call interface without a
// scratch operand), or latency-critical loops that forbid allocation.  This entry
// point serves them by using a scratch array that lives in the library
// itself: a file-scope __device__ array of PDQ_LML_STATIC_SCRATCH_BYTES
// (32 MiB).  Every GPU on which the library is loaded holds the array until
// the process exits.
//
// The array's name is only a host-side stand-in in host code; the kernel
// gets the device address, obtained once per device with that device current
// by cudaGetSymbolAddress.  That set-up happens on the first call on each
// device, so the first call should come before any stream capture.
// Every call shares the one array: calls whose launches overlap on the GPU
// race on it.  Nothing needs clearing between calls: the covariance plan at
// the head of the array is reused only when its key (a sentinel, a validity
// flag set last, and the grid, prior, precision and noise levels) matches the
// call's, which a zero-initialised or stale array cannot do by accident, and
// every other scratch entry is written before it is read.
#include <cuda_runtime.h>

#include <mutex>

#include "pdq_nvtx.h"
#include "pdq.h"

namespace {

constexpr size_t kStaticScratchBytes = PDQ_LML_STATIC_SCRATCH_BYTES;

static __device__ __align__(256) unsigned char g_lml_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_lml_scratch on the current device (set up once per device).
cudaError_t static_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_lml_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" pdq_status pdq_lml_fixed_grid_static(const pdq_config* config, const pdq_lml_args* args, void* stream) {
  pdq::NvtxRange nvtx_range("pdq_lml_fixed_grid_static");
  if (args == nullptr) return PDQ_ERROR_INVALID_VALUE;
  size_t need = 0;
  const pdq_status st =
      pdq_lml_workspace_size(config, args->num_instances, args->num_steps, args->save_every, &need);
  if (st != PDQ_SUCCESS) return st;
  if (need > kStaticScratchBytes) return PDQ_ERROR_STATIC_SCRATCH;
  void* scratch = nullptr;
  if (static_scratch(&scratch) != cudaSuccess) return PDQ_ERROR_CUDA;
  return pdq_lml_fixed_grid(config, args, scratch, kStaticScratchBytes, stream);
}
