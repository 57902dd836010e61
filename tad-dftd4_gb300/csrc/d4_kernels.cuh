// Host-side launchers of the kernel families.
#pragma once

#include <mutex>

#include "d4_common.cuh"

namespace d4 {

enum Stage {
  ST_PREP = 0,
  ST_CN,
  ST_EEQ,
  ST_WEIGHTS,
  ST_PAIR_FWD,
  ST_ATM,
  ST_PAIR_ATM_BWD,
  ST_EEQ_ADJ,
  ST_PAIR_CN_BWD,
  ST_FINISH,
  ST_COUNT
};

// The library's second stream of a device (high priority, non-blocking) and
// the events that order it against the caller's stream; created on first use
// (nullptr if the runtime refuses them: callers then stay on one stream).
// Enqueue sequences that use the events hold side_stream_mutex().
struct SideStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, panel = nullptr, bulk[2] = {nullptr, nullptr}, done = nullptr;
  bool ok = false, tried = false;
};
SideStream *side_stream_for_device();
std::mutex &side_stream_mutex();

// Stage timing hooks (no-ops unless d4_timing_begin was called).
void stage_begin(int stage, cudaStream_t st);
void stage_end(int stage, cudaStream_t st);
void timing_next_call();

int launch_fp64(const Ctx &c, cudaStream_t st);
int launch_mixed(const Ctx &c, cudaStream_t st);
void launch_eeq_big(const Ctx &c, cudaStream_t st, bool adjoint);
void launch_pair_fwd_tc(const Ctx &c, cudaStream_t st);  // D4, precision form (d4_c6tc.cu)
bool pair_atm_bwd_tc_ok(const Ctx &c);
void launch_pair_atm_bwd_tc(const Ctx &c, cudaStream_t st);
void launch_atm_exact(const Ctx &c, cudaStream_t st);  // exact C9, FP64 (d4_exact.cu)
int launch_properties(const Ctx &c, double *c6out, double *alpha_out, double *q_out,
                      cudaStream_t st);

// stages shared by the FP64 method and the precision form (d4_fp64.cu)
void launch_prep(const Ctx &c, cudaStream_t st);
void launch_prep_memsets(const Ctx &c, cudaStream_t st);  // the memsets of launch_prep
void launch_cn(const Ctx &c, cudaStream_t st);
void launch_weights(const Ctx &c, cudaStream_t st);
void launch_charges_in(const Ctx &c, cudaStream_t st);
void launch_finish(const Ctx &c, cudaStream_t st);
int launch_prepare_alpha(const d4_tables_t &tab, const d4_model_cfg_t &cfg,
                         const double *refalpha, const double *refascale,
                         const double *refscount, const int64_t *refsys,
                         const double *secscale, const double *secalpha, int n_sec,
                         const double *refh, double *out, cudaStream_t st);

}  // namespace d4
