// C ABI entry points (include/tad_dftd4_gb300.h).
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <utility>
#include <vector>

#include "d4_common.cuh"
#include "d4_kernels.cuh"

namespace d4 {

// (device, kernel) -> dynamic shared-memory limit already set
void ensure_smem_impl(const void *func, size_t bytes) {
  static std::mutex mu;
  static std::vector<std::pair<std::pair<int, const void *>, size_t>> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  for (auto &e : done)
    if (e.first.first == dev && e.first.second == func) {
      if (bytes > e.second) {
        cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        e.second = bytes;
      }
      return;
    }
  cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  done.push_back({{dev, func}, bytes});
}

}  // namespace d4

namespace {
thread_local char g_cuda_error[256] = "";

int check_cuda(cudaError_t e) {
  if (e == cudaSuccess) return D4_OK;
  snprintf(g_cuda_error, sizeof(g_cuda_error), "%s: %s", cudaGetErrorName(e),
           cudaGetErrorString(e));
  return D4_ERR_CUDA;
}

bool tables_ok(const d4_tables_t *t) {
  return t && t->alpha && t->refcovcn && t->refc && t->refq && t->gam && t->zeff &&
         t->r4r2 && t->cov_d3 && t->en && t->eeq_chi && t->eeq_eta && t->eeq_kcn &&
         t->eeq_rad && t->freq_weights && t->n_ref_elem > 0 && t->n_elem >= t->n_ref_elem &&
         t->n_ref_elem <= d4::MAX_ELEM_ID;
}
}  // namespace

extern "C" {

int d4_abi_version(void) { return D4_ABI_VERSION; }

const char *d4_status_string(int status) {
  switch (status) {
    case D4_OK: return "ok";
    case D4_ERR_ARGUMENT: return "invalid argument";
    case D4_ERR_WORKSPACE: return "workspace too small";
    case D4_ERR_CUDA: return "CUDA error";
    case D4_ERR_ELEMENT: return "atomic number outside the element tables";
    case D4_ERR_EEQ_SINGULAR: return "EEQ matrix is not positive definite";
    case D4_ERR_NONFINITE: return "non-finite position or charge";
    case D4_ERR_TOO_MANY_ELEMENTS: return "more distinct elements than D4S slots";
    case D4_ERR_DEVICE_TIMEOUT: return "on-device wait for the tensor cores timed out";
    default: return "unknown status";
  }
}

const char *d4_last_cuda_error(void) { return g_cuda_error; }

int d4_prepare_alpha(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                     const double *d_refalpha, const double *d_refascale,
                     const double *d_refscount, const int64_t *d_refsys,
                     const double *d_secscale, const double *d_secalpha, int32_t n_sec,
                     const double *d_refh, double *d_alpha_out, void *stream) {
  if (!tables || !cfg || !d_refalpha || !d_refascale || !d_refscount || !d_refsys ||
      !d_secscale || !d_secalpha || !d_refh || !d_alpha_out || n_sec <= 0 ||
      !tables->gam || !tables->zeff || tables->n_ref_elem <= 0)
    return D4_ERR_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  d4::launch_prepare_alpha(*tables, *cfg, d_refalpha, d_refascale, d_refscount, d_refsys,
                           d_secscale, d_secalpha, n_sec, d_refh, d_alpha_out, st);
  return check_cuda(cudaGetLastError());
}

size_t d4_workspace_size(int32_t n_struct, int32_t n_pad, int32_t n_slots, uint32_t flags) {
  if (n_struct <= 0 || n_pad <= 0 || n_slots <= 0) return 0;
  return d4::carve_workspace(nullptr, n_struct, n_pad, n_slots, flags).bytes;
}

int d4_dispersion(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                  const d4_batch_t *batch, const d4_params_t *params, uint32_t flags,
                  int32_t n_slots, void *d_workspace, size_t workspace_bytes,
                  const d4_outputs_t *out, void *stream) {
  if (!tables_ok(tables) || !cfg || !batch || !params || !out || !d_workspace)
    return D4_ERR_ARGUMENT;
  if (batch->n_struct <= 0 || batch->n_pad <= 0 || batch->n_struct > 65535 || n_slots <= 0)
    return D4_ERR_ARGUMENT;
  if (!batch->d_numbers || !batch->d_positions || !batch->d_charge || !out->d_energy)
    return D4_ERR_ARGUMENT;
  if ((flags & D4_FLAG_GRADIENT) && !out->d_gradient) return D4_ERR_ARGUMENT;
  if ((flags & D4_FLAG_CHARGES_IN) && !batch->d_charges_in) return D4_ERR_ARGUMENT;
  if ((flags & D4_FLAG_PARAM_GRAD) && (!out->d_param_grad || !(flags & D4_FLAG_GRADIENT)))
    return D4_ERR_ARGUMENT;
  if (cfg->kind != D4_MODEL_D4 && cfg->kind != D4_MODEL_D4S) return D4_ERR_ARGUMENT;
  if (cfg->kind == D4_MODEL_D4S && !tables->wfpair) return D4_ERR_ARGUMENT;
  if (cfg->kind == D4_MODEL_D4 && n_slots != 1) return D4_ERR_ARGUMENT;
  // D3-family two-body damping and exact C9 run on the plain FP64 kernels;
  // the zero and modified-zero damping need the pairwise radii; no
  // quadrupole-quadrupole (s10) term beside them (damping/functions.py:352-356)
  const int damp = params->damping;
  if (damp < D4_DAMP_RATIONAL || damp > D4_DAMP_OP) return D4_ERR_ARGUMENT;
  if ((flags & D4_FLAG_MIXED) && (damp != D4_DAMP_RATIONAL || (flags & D4_FLAG_EXACT_C9)))
    return D4_ERR_ARGUMENT;
  if ((damp == D4_DAMP_ZERO || damp == D4_DAMP_MZERO) && !batch->d_rvdw_in)
    return D4_ERR_ARGUMENT;
  if (damp != D4_DAMP_RATIONAL && params->has_s10) return D4_ERR_ARGUMENT;
  d4::Workspace w = d4::carve_workspace(d_workspace, batch->n_struct, batch->n_pad, n_slots,
                                        flags);
  if (workspace_bytes < w.bytes) return D4_ERR_WORKSPACE;
  d4::Ctx c{};
  c.tab = *tables;
  c.cfg = *cfg;
  c.par = *params;
  c.numbers = batch->d_numbers;
  c.positions = batch->d_positions;
  c.charge = batch->d_charge;
  c.charges_in = batch->d_charges_in;
  c.r4r2_in = batch->d_r4r2_in;
  c.weights = batch->d_energy_weights;
  c.rvdw_in = batch->d_rvdw_in;
  c.B = batch->n_struct;
  c.N = batch->n_pad;
  c.S = n_slots;
  c.flags = flags;
  c.w = w;
  c.out = *out;
  const d4_params_t &pp = *params;
  c.pf = {(float)pp.s6,        (float)pp.s8,         (float)pp.s10,    (float)pp.a1,
          (float)pp.a2,        (float)pp.s9,         (float)(pp.alp / 3.0),
          (float)pp.cut_disp2, (float)pp.cut_disp3,  (float)pp.cut_cn, (float)pp.cut_cn_eeq,
          (float)pp.kcn,       (float)pp.k4,         (float)pp.k5,     (float)pp.k6,
          (float)pp.cn_eeq_max, (float)cfg->wf,        (float)cfg->ga};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (flags & D4_FLAG_MIXED)
    d4::launch_mixed(c, st);
  else
    d4::launch_fp64(c, st);
  return check_cuda(cudaGetLastError());
}

int d4_properties(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                  const d4_batch_t *batch, const d4_params_t *params, void *d_workspace,
                  size_t workspace_bytes, const d4_properties_t *out, void *stream) {
  if (!tables_ok(tables) || !cfg || !batch || !params || !out || !d_workspace)
    return D4_ERR_ARGUMENT;
  if (batch->n_struct <= 0 || batch->n_pad <= 0 || batch->n_struct > 65535) return D4_ERR_ARGUMENT;
  if (!batch->d_numbers || !batch->d_positions || !batch->d_charge) return D4_ERR_ARGUMENT;
  if (cfg->kind != D4_MODEL_D4) return D4_ERR_ARGUMENT;
  d4::Workspace w = d4::carve_workspace(d_workspace, batch->n_struct, batch->n_pad, 1, 0);
  if (workspace_bytes < w.bytes) return D4_ERR_WORKSPACE;
  d4::Ctx c{};
  c.tab = *tables;
  c.cfg = *cfg;
  c.par = *params;
  c.numbers = batch->d_numbers;
  c.positions = batch->d_positions;
  c.charge = batch->d_charge;
  c.r4r2_in = batch->d_r4r2_in;
  c.B = batch->n_struct;
  c.N = batch->n_pad;
  c.S = 1;
  c.flags = 0;
  c.w = w;
  c.out = d4_outputs_t{};
  c.out.d_cn = out->d_cn;
  const d4_params_t &pp = *params;
  c.pf = {(float)pp.s6,        (float)pp.s8,         (float)pp.s10,    (float)pp.a1,
          (float)pp.a2,        (float)pp.s9,         (float)(pp.alp / 3.0),
          (float)pp.cut_disp2, (float)pp.cut_disp3,  (float)pp.cut_cn, (float)pp.cut_cn_eeq,
          (float)pp.kcn,       (float)pp.k4,         (float)pp.k5,     (float)pp.k6,
          (float)pp.cn_eeq_max, (float)cfg->wf,        (float)cfg->ga};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  d4::launch_properties(c, out->d_c6, out->d_alpha, out->d_charges, st);
  return check_cuda(cudaGetLastError());
}

int d4_status_async(void *d_workspace, int32_t *h_status, void *stream) {
  if (!d_workspace || !h_status) return D4_ERR_ARGUMENT;
  d4::Workspace w = d4::carve_workspace(d_workspace, 1, 1, 1, 0);
  return check_cuda(cudaMemcpyAsync(h_status, w.status, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    static_cast<cudaStream_t>(stream)));
}

int d4_eeq_residuals(void *d_workspace, int32_t n_struct, float *h_out, void *stream) {
  if (!d_workspace || !h_out || n_struct <= 0) return D4_ERR_ARGUMENT;
  d4::Workspace w = d4::carve_workspace(d_workspace, n_struct, 1, 1, 0);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = check_cuda(cudaMemcpyAsync(h_out, w.eeq_final, sizeof(float) * 2 * (size_t)n_struct,
                                      cudaMemcpyDeviceToHost, st));
  if (rc != D4_OK) return rc;
  return check_cuda(cudaStreamSynchronize(st));
}

int d4_read_status(void *d_workspace, void *stream) {
  if (!d_workspace) return D4_ERR_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int status = 0;
  d4::Workspace w = d4::carve_workspace(d_workspace, 1, 1, 1, 0);
  int rc = check_cuda(cudaMemcpyAsync(&status, w.status, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (rc != D4_OK) return rc;
  rc = check_cuda(cudaStreamSynchronize(st));
  if (rc != D4_OK) return rc;
  rc = check_cuda(cudaMemsetAsync(w.status, 0, sizeof(int), st));
  if (rc != D4_OK) return rc;
  return status;
}

}  // extern "C"
