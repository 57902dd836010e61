// Per-stage CUDA-event timing and the FMA throughput probe.
#include <vector>

#include "d4_common.cuh"
#include "d4_kernels.cuh"
#include "d4_tc.cuh"

namespace d4 {
namespace {

struct Timing {
  bool on = false;
  int max_calls = 0;
  int call = -1;
  std::vector<cudaEvent_t> ev;  // [max_calls][ST_COUNT][2]
  cudaEvent_t last = nullptr;
};

thread_local Timing g_t;

const char *kStageNames[ST_COUNT] = {
    "prep", "cn", "eeq", "weights", "pair_fwd", "atm", "pair_atm_bwd",
    "eeq_adjoint", "pair_cn_bwd", "finish",
};

cudaEvent_t *slot(int stage, int which) {
  if (!g_t.on || g_t.call < 0 || g_t.call >= g_t.max_calls) return nullptr;
  return &g_t.ev[((size_t)g_t.call * ST_COUNT + stage) * 2 + which];
}

}  // namespace

void timing_next_call() {
  if (g_t.on) ++g_t.call;
}

void stage_begin(int stage, cudaStream_t st) {
  if (cudaEvent_t *e = slot(stage, 0)) cudaEventRecord(*e, st);
}

void stage_end(int stage, cudaStream_t st) {
  if (cudaEvent_t *e = slot(stage, 1)) {
    cudaEventRecord(*e, st);
    g_t.last = *e;
  }
}

// Dependent FMA chains on 8 accumulators per thread.
template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, double *sink) {
  T a[8];
  const T m = (T)0.999999;
  const T add = (T)1e-7;
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (T)(threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, add);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  sink[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}

// One thread waits, with the library's bounded wait loop, for an mbarrier
// phase that nothing completes (initialised for one arrival, none made).
__global__ void selftest_wait_kernel(int32_t *result, unsigned long long limit_ns) {
  __shared__ __align__(8) unsigned long long bar;
  const uint32_t mbar = tc::smem_u32(&bar);
  tc::mbar_init(mbar, 1);
  *result = tc::mbar_wait(mbar, 0u, limit_ns) ? D4_OK : D4_ERR_DEVICE_TIMEOUT;
}

}  // namespace d4

extern "C" {

int d4_selftest_wait(int32_t *d_result, uint64_t limit_ns, void *stream) {
  if (!d_result || limit_ns > 1000000000ull) return D4_ERR_ARGUMENT;
  d4::selftest_wait_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(
      d_result, (unsigned long long)limit_ns);
  return cudaGetLastError() == cudaSuccess ? D4_OK : D4_ERR_CUDA;
}

int d4_timing_begin(int32_t max_calls) {
  using namespace d4;
  if (max_calls <= 0) return D4_ERR_ARGUMENT;
  for (cudaEvent_t e : g_t.ev) cudaEventDestroy(e);
  g_t.ev.assign((size_t)max_calls * ST_COUNT * 2, nullptr);
  for (auto &e : g_t.ev)
    if (cudaEventCreate(&e) != cudaSuccess) return D4_ERR_CUDA;
  g_t.on = true;
  g_t.max_calls = max_calls;
  g_t.call = -1;
  g_t.last = nullptr;
  return D4_OK;
}

int d4_timing_end(float *ms_per_stage, int32_t n_stage, int32_t *n_calls) {
  using namespace d4;
  if (!g_t.on) return D4_ERR_ARGUMENT;
  int rc = D4_OK;
  if (g_t.last && cudaEventSynchronize(g_t.last) != cudaSuccess) rc = D4_ERR_CUDA;
  const int calls = g_t.call + 1 < g_t.max_calls ? g_t.call + 1 : g_t.max_calls;
  for (int s = 0; s < n_stage && s < ST_COUNT; ++s) {
    float tot = 0.0f;
    for (int k = 0; k < calls; ++k) {
      cudaEvent_t a = g_t.ev[((size_t)k * ST_COUNT + s) * 2];
      cudaEvent_t b = g_t.ev[((size_t)k * ST_COUNT + s) * 2 + 1];
      float ms = 0.0f;
      if (cudaEventQuery(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
        tot += ms;
      else
        cudaGetLastError();  // stage not recorded in this call
    }
    if (ms_per_stage) ms_per_stage[s] = tot;
  }
  if (n_calls) *n_calls = calls;
  for (cudaEvent_t e : g_t.ev) cudaEventDestroy(e);
  g_t.ev.clear();
  g_t.on = false;
  g_t.call = -1;
  g_t.last = nullptr;
  return rc;
}

int32_t d4_stage_count(void) { return d4::ST_COUNT; }

const char *d4_stage_name(int32_t stage) {
  return (stage >= 0 && stage < d4::ST_COUNT) ? d4::kStageNames[stage] : "";
}

int d4_probe_fma(int32_t fp64, int32_t n_blocks, int32_t iters, double *d_sink,
                 float *ms_out, void *stream) {
  if (n_blocks <= 0 || iters <= 0 || !d_sink || !ms_out) return D4_ERR_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return D4_ERR_CUDA;
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return D4_ERR_CUDA;
  }
  cudaEventRecord(a, st);
  if (fp64)
    d4::fma_probe_kernel<double><<<n_blocks, 256, 0, st>>>(iters, d_sink);
  else
    d4::fma_probe_kernel<float><<<n_blocks, 256, 0, st>>>(iters, d_sink);
  cudaEventRecord(b, st);
  const cudaError_t e = cudaEventSynchronize(b);
  cudaEventElapsedTime(ms_out, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return e == cudaSuccess ? D4_OK : D4_ERR_CUDA;
}

}  // extern "C"
