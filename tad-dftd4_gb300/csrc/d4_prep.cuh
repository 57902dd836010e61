// Per-structure set-up shared by the FP64 method and the precision form
// (d4_fp64.cu: prep_kernel; d4_mixed.cu: prep_tables_kernel).
#pragma once

#include "d4_common.cuh"

namespace d4 {

// Structures padded beyond this size have their N x N pair accumulators
// cleared by memsets instead of by the prep kernel.
constexpr int PREP_ZERO_MAX_N = 256;

// n_eff, input validation, D4S element slots, zeroing of accumulators of
// structure b, by one CTA of 256 threads (all of which call it).
static __device__ __forceinline__ void prep_structure(const Ctx &c, int b) {
  const int N = c.N;
  const int64_t *Z = c.numbers + (size_t)b * N;
  __shared__ int s_neff, s_first;
  __shared__ int s_present[MAX_ELEM_ID];
  __shared__ int s_slot_of[MAX_ELEM_ID];
  if (threadIdx.x == 0) {
    s_neff = 0;
    s_first = N;
    c.w.eeq_final[2 * b] = 0.f;  // stays 0 where no refinement runs
    c.w.eeq_final[2 * b + 1] = 0.f;
  }
  for (int e = threadIdx.x; e < MAX_ELEM_ID; e += blockDim.x) s_present[e] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int64_t z = Z[i];
    if (z == 0) continue;
    if (z < 0 || z >= c.tab.n_ref_elem || z >= MAX_ELEM_ID) {
      set_status(c.w.status, D4_ERR_ELEMENT);
      continue;
    }
    atomicMax(&s_neff, i + 1);
    atomicMin(&s_first, i);
    s_present[z] = 1;
    const double *r = c.positions + ((size_t)b * N + i) * 3;
    if (!isfinite(r[0]) || !isfinite(r[1]) || !isfinite(r[2]))
      set_status(c.w.status, D4_ERR_NONFINITE);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!isfinite(c.charge[b])) set_status(c.w.status, D4_ERR_NONFINITE);
    int ns = 0;
    if (c.cfg.kind == D4_MODEL_D4S) {
      for (int e = 0; e < MAX_ELEM_ID; ++e) {
        s_slot_of[e] = s_present[e] ? ns : 0;
        if (s_present[e]) {
          if (ns < c.S) c.w.slot_elem[b * MAX_ELEM_ID + ns] = e;
          ++ns;
        }
      }
      if (ns > c.S) set_status(c.w.status, D4_ERR_TOO_MANY_ELEMENTS);
      if (ns == 0) ns = 1;
    } else {
      for (int e = 0; e < MAX_ELEM_ID; ++e) s_slot_of[e] = 0;
      c.w.slot_elem[b * MAX_ELEM_ID] = 0;
      ns = 1;
    }
    c.w.n_slots[b] = ns < c.S ? ns : c.S;
    c.w.n_eff[b] = s_neff;
  }
  __syncthreads();
  const int n = s_neff;
  // FP32 positions are taken relative to the first real atom
  const double *p0 = c.positions + ((size_t)b * N + (s_first < N ? s_first : 0)) * 3;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const size_t a = (size_t)b * N + i;
    const int64_t z = Z[i];
    const bool ok = z > 0 && z < c.tab.n_ref_elem && z < MAX_ELEM_ID;
    int s = ok ? s_slot_of[z] : 0;
    c.w.z[a] = ok ? (int)z : 0;
    c.w.w32[a] = c.weights ? (float)c.weights[a] : 1.0f;
    c.w.slot[a] = s < c.S ? s : c.S - 1;
    c.w.e3[a] = 0.0;
    if (ok) {
      const double *p = c.positions + 3 * a;
      const double dx = p[0] - p0[0], dy = p[1] - p0[1], dz = p[2] - p0[2];
      const double sr = sqrt(atom_r4r2(c, a, z));
      c.w.pos32[a] = make_float4((float)dx, (float)dy, (float)dz, (float)sr);
      if (c.w.pos32lo)  // low parts (positions and sqrt(r4r2)) of the double-float copies
        c.w.pos32lo[a] = make_float4((float)(dx - (double)(float)dx),
                                     (float)(dy - (double)(float)dy),
                                     (float)(dz - (double)(float)dz),
                                     (float)(sr - (double)(float)sr));
      c.w.aux32[a] = make_float4((float)c.tab.cov_d3[z], (float)c.tab.en[z],
                                 (float)c.tab.eeq_rad[z], 0.f);
    } else {
      c.w.pos32[a] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (c.w.pos32lo) c.w.pos32lo[a] = make_float4(0.f, 0.f, 0.f, 0.f);
      c.w.aux32[a] = make_float4(1.f, 0.f, 1.f, 0.f);
    }
  }
  // index of every real atom among the real atoms (EEQ matrix rows)
  if (threadIdx.x < 32) {
    int base = 0;
    for (int i0 = 0; i0 < N; i0 += 32) {
      const int i = i0 + threadIdx.x;
      const int64_t z = i < N ? Z[i] : 0;
      const bool real = i < N && z > 0 && z < c.tab.n_ref_elem && z < MAX_ELEM_ID;
      const unsigned mask = __ballot_sync(0xffffffffu, real);
      const int k = base + __popc(mask & ((1u << threadIdx.x) - 1u));
      if (i < N) c.w.cidx[(size_t)b * N + i] = real ? k : -1;
      if (real && c.w.ridx) c.w.ridx[(size_t)b * N + k] = i;
      base += __popc(mask);
    }
    if (threadIdx.x == 0 && c.w.n_real) c.w.n_real[b] = base;
  }
  if (threadIdx.x < D4_PARAM_GRAD_STRIDE) c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + threadIdx.x] = 0.0;
  if (b == 0 && threadIdx.x < NFREQ)
    c.w.fw32[threadIdx.x] = (float)(THOPI * c.tab.freq_weights[threadIdx.x]);
  if (c.w.pr_S && c.N <= PREP_ZERO_MAX_N) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int i = t / n, j = t % n;
      const size_t o = ((size_t)b * N + i) * N + j;
      c.w.pr_S[o] = 0.0;
      c.w.pr_P[o] = 0.0;
    }
  }
  // (the register-tiled ATM stores every pair sum of a structure it covers
  // with one CTA, so those structures need no zeroing)
  if (c.w.prS32 && c.N <= PREP_ZERO_MAX_N && !(c.atm_tiled && atm_tiled_ctas(n, c.B) == 1)) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int i = t / n, j = t % n;
      const size_t o = ((size_t)b * N + i) * N + j;
      c.w.prS32[o] = 0.f;
      c.w.prP32[o] = 0.f;
    }
  }
}

}  // namespace d4
