// d4_dispersion_noalloc: the dispersion call for callers that cannot
// allocate device memory.  Its workspace is a fixed array compiled into the
// library image instead of a caller buffer; see the header for the rules.
#include <mutex>

#include "d4_common.cuh"
#include "d4_kernels.cuh"

namespace {

constexpr size_t kScratchBytes = D4_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The shared scratch.  Device code in this file could name it directly; host
// code only ever sees a stand-in symbol, so the device address is looked up
// with cudaGetSymbolAddress once per device (with that device current).
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_scratch on the current device, looked up on first use.
int scratch_address(void **addr) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return D4_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return D4_ERR_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || p == nullptr)
      return D4_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *addr = g_scratch_addr[dev];
  return D4_OK;
}

}  // namespace

extern "C" int d4_dispersion_noalloc(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                                     const d4_batch_t *batch, const d4_params_t *params,
                                     uint32_t flags, int32_t n_slots, const d4_outputs_t *out,
                                     int32_t check_status, void *stream) {
  if (!batch || n_slots <= 0 || batch->n_struct <= 0 || batch->n_pad <= 0)
    return D4_ERR_ARGUMENT;
  // Reject problems that do not fit before touching the device.
  const size_t need = d4_workspace_size(batch->n_struct, batch->n_pad, n_slots, flags);
  if (need == 0) return D4_ERR_ARGUMENT;
  if (need > kScratchBytes) return D4_ERR_WORKSPACE;
  void *scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != D4_OK) return rc;
  // The call clears what must start at zero (status word, accumulators) on
  // the stream before its kernels read them.
  rc = d4_dispersion(tables, cfg, batch, params, flags, n_slots, scratch, kScratchBytes, out,
                     stream);
  if (rc != D4_OK || !check_status) return rc;
  return d4_read_status(scratch, stream);
}
