// Host-side launchers of the kernel families.
#pragma once

#include "d4_common.cuh"

namespace d4 {

int launch_fp64(const Ctx &c, cudaStream_t st);
int launch_prepare_alpha(const d4_tables_t &tab, const d4_model_cfg_t &cfg,
                         const double *refalpha, const double *refascale,
                         const double *refscount, const int64_t *refsys,
                         const double *secscale, const double *secalpha, int n_sec,
                         const double *refh, double *out, cudaStream_t st);

}  // namespace d4
