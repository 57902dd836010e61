// FP64 kernels of the plain DFT-D4 method: CN, EEQ, weights, fused C6 +
// rational two-body term, ATM three-body term and the hand-written adjoint.
//
// Layout: structure b, atom i live at b * N + i (zero-padded batch).  Pair
// quantities live in dense per-structure N x N blocks, only the leading
// n_eff x n_eff part of which is touched.  Every "atom-owned" kernel maps one
// warp to one atom i and loops its lanes over partners j, so per-atom sums
// need no atomics.  The ATM kernel maps a CTA to a tile of pairs (j, k) and
// loops over the third atom i < j.
#include <float.h>

#include "d4_common.cuh"
#include "d4_kernels.cuh"
#include "d4_prep.cuh"

namespace d4 {

// ---------------------------------------------------------------- prep

// n_eff, input validation, D4S element slots, zeroing of accumulators.
__global__ void __launch_bounds__(256) prep_kernel(Ctx c) { prep_structure(c, blockIdx.x); }

// ---------------------------------------------------------------- CN

// D4 coordination number (EN weighted, cut_cn) and the EEQ coordination
// number (plain count, cut_cn_eeq, smooth cap) in one pass over the pairs.
// A pair whose FP32 estimate of x exceeds 9 (1/2 erfc(x) < 1e-36) is dropped
// before any FP64 work.  The surviving partners of the warp's
// atom are queued in shared memory and evaluated 32 at a time, so the FP64
// instructions run with full warps.
__global__ void __launch_bounds__(256) cn_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_q[8][64];
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int zi = c.w.z[ai];
  if (i >= n || zi == 0) {
    if (lane == 0) {
      c.w.cn[ai] = 0.0;
      c.w.cnq[ai] = 0.0;
      c.w.dcnq[ai] = 0.0;
      if (c.out.d_cn) c.out.d_cn[ai] = 0.0;
    }
    return;
  }
  const double *P = c.positions + (size_t)b * N * 3;
  const double xi = P[3 * i], yi = P[3 * i + 1], zi3 = P[3 * i + 2];
  const double rci = c.tab.cov_d3[zi], eni = c.tab.en[zi];
  const float4 *P32 = c.w.pos32 + (size_t)b * N;
  const float4 *X32 = c.w.aux32 + (size_t)b * N;
  const float4 pi32 = P32[i];
  const float rci32 = X32[i].x, kcn32 = (float)c.par.kcn;
  double s_d4 = 0.0, s_q4 = 0.0;
  int queued = 0;
  auto evaluate = [&](int j) {
    const int zj = c.w.z[(size_t)b * N + j];
    const double dx = xi - P[3 * j], dy = yi - P[3 * j + 1], dz = zi3 - P[3 * j + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    const double r0 = rci + c.tab.cov_d3[zj];
    const double cf = erf_count(r, r0, c.par.kcn);
    if (r <= c.par.cut_cn) s_d4 += en_factor(eni, c.tab.en[zj], c.par.k4, c.par.k5, c.par.k6) * cf;
    if (r <= c.par.cut_cn_eeq) s_q4 += cf;
  };
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    bool keep = false;
    if (j < n && j != i && c.w.z[(size_t)b * N + j] != 0) {
      const float4 pj32 = P32[j];
      const float ex = pi32.x - pj32.x, ey = pi32.y - pj32.y, ez = pi32.z - pj32.z;
      const float r32 = sqrtf(ex * ex + ey * ey + ez * ez);
      keep = kcn32 * (r32 / (rci32 + X32[j].x) - 1.0f) <= 9.0f;  // erfc(9) / 2 < 1e-36
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) s_q[warp][queued + __popc(m & ((1u << lane) - 1u))] = j;
    queued += __popc(m);
    __syncwarp();
    if (queued >= 32) {
      evaluate(s_q[warp][lane]);
      queued -= 32;
      __syncwarp();
      if (lane < queued) s_q[warp][lane] = s_q[warp][32 + lane];
      __syncwarp();
    }
  }
  if (lane < queued) evaluate(s_q[warp][lane]);
  s_d4 = warp_sum(s_d4);
  s_q4 = warp_sum(s_q4);
  if (lane == 0) {
    c.w.cn[ai] = s_d4;
    const double m = c.par.cn_eeq_max;
    // log(1 + e^m) - log(1 + e^(m - cn)) as log1p(expm1(cn) / (1 + e^(cn - m))):
    // the same function without the cancellation of the two logarithms, so
    // that nearly isolated atoms (cn << 1) keep a relative accuracy (the EEQ
    // right-hand side takes sqrt(cn), which magnifies absolute noise there)
    c.w.cnq[ai] = log1p(expm1(s_q4) / (1.0 + exp(s_q4 - m)));
    c.w.dcnq[ai] = 1.0 / (1.0 + exp(s_q4 - m));
    if (c.out.d_cn) c.out.d_cn[ai] = s_d4;
  }
}

// ---------------------------------------------------------------- EEQ

// Row-oriented triangular solves with one warp.  L is packed lower.
// forward: L z = v (in place); backward: L^T x = z (in place).
template <int NRHS>
__device__ void warp_forward_solve(const double *L, double *v, int ldv, int m) {
  const int lane = threadIdx.x & 31;
  for (int i = 0; i < m; ++i) {
    const double *row = L + tri_index(i, 0);
    double s[NRHS];
#pragma unroll
    for (int r = 0; r < NRHS; ++r) s[r] = 0.0;
    for (int k = lane; k < i; k += 32) {
      const double l = row[k];
#pragma unroll
      for (int r = 0; r < NRHS; ++r) s[r] += l * v[r * ldv + k];
    }
#pragma unroll
    for (int r = 0; r < NRHS; ++r) s[r] = warp_sum(s[r]);
    if (lane == 0) {
      const double inv = 1.0 / row[i];
#pragma unroll
      for (int r = 0; r < NRHS; ++r) v[r * ldv + i] = (v[r * ldv + i] - s[r]) * inv;
    }
    __syncwarp();
  }
}

template <int NRHS>
__device__ void warp_backward_solve(const double *L, double *v, int ldv, int m) {
  const int lane = threadIdx.x & 31;
  for (int i = m - 1; i >= 0; --i) {
    double s[NRHS];
#pragma unroll
    for (int r = 0; r < NRHS; ++r) s[r] = 0.0;
    for (int k = i + 1 + lane; k < m; k += 32) {
      const double l = L[tri_index(k, i)];
#pragma unroll
      for (int r = 0; r < NRHS; ++r) s[r] += l * v[r * ldv + k];
    }
#pragma unroll
    for (int r = 0; r < NRHS; ++r) s[r] = warp_sum(s[r]);
    if (lane == 0) {
      const double inv = 1.0 / L[tri_index(i, i)];
#pragma unroll
      for (int r = 0; r < NRHS; ++r) v[r * ldv + i] = (v[r * ldv + i] - s[r]) * inv;
    }
    __syncwarp();
  }
}

// EEQ charges of one structure per CTA: build the (real-atom) Coulomb matrix
// in packed form, Cholesky-factorise it, solve for A^-1 b and A^-1 1, apply
// the total-charge constraint.  The factor is kept in the workspace for the
// adjoint solve.  ``SMEM``: factorise in shared memory, else in place in the
// workspace.
template <bool SMEM>
__global__ void __launch_bounds__(256) eeq_kernel(Ctx c) {
  extern __shared__ double s_dyn[];
  const int b = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_m;
  __shared__ double s_inv;
  // shared scratch: idx[N] (int), vectors rhs[2*N]
  int *s_idx = reinterpret_cast<int *>(s_dyn);
  double *vec = s_dyn + (N + 1) / 2 + 1;  // 2 * N doubles
  double *L = SMEM ? vec + 2 * N : c.w.eeq_L + (size_t)b * ((size_t)N * (N + 1) / 2);
  const int m = compact_real_atoms(c, b, n, s_idx, &s_m);
  const double *P = c.positions + (size_t)b * N * 3;
  const int *Zb = c.w.z + (size_t)b * N;
  const size_t tri_m = (size_t)m * (m + 1) / 2;
  // build
  for (size_t t = threadIdx.x; t < tri_m; t += blockDim.x) {
    // invert t -> (ii, jj) with jj <= ii
    int ii = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (tri_index(ii + 1, 0) <= t) ++ii;
    while (tri_index(ii, 0) > t) --ii;
    const int jj = (int)(t - tri_index(ii, 0));
    const int ia = s_idx[ii], ja = s_idx[jj];
    const int za = Zb[ia], zb = Zb[ja];
    double v;
    if (ii == jj) {
      v = c.tab.eeq_eta[za] + SQRT_2_OVER_PI / c.tab.eeq_rad[za];
    } else {
      const double dx = P[3 * ia] - P[3 * ja], dy = P[3 * ia + 1] - P[3 * ja + 1],
                   dz = P[3 * ia + 2] - P[3 * ja + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const double ra = c.tab.eeq_rad[za], rb = c.tab.eeq_rad[zb];
      const double g = 1.0 / sqrt(ra * ra + rb * rb);
      v = erf(g * r) / r;
    }
    L[t] = v;
  }
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const int ia = s_idx[k];
    const int z = Zb[ia];
    const double cq = c.w.cnq[(size_t)b * N + ia];
    const double sq = cq > 0.0 ? sqrt(cq) : 0.0;
    vec[k] = -c.tab.eeq_chi[z] + c.tab.eeq_kcn[z] * sq;
    vec[N + k] = 1.0;
  }
  __syncthreads();
  // right-looking Cholesky, packed lower
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int k = 0; k < m; ++k) {
    if (threadIdx.x == 0) {
      double d = L[tri_index(k, k)];
      if (!(d > 0.0)) {
        set_status(c.w.status, D4_ERR_EEQ_SINGULAR);
        d = 1.0;
      }
      d = sqrt(d);
      L[tri_index(k, k)] = d;
      s_inv = 1.0 / d;
    }
    __syncthreads();
    const double inv = s_inv;
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) L[tri_index(i, k)] *= inv;
    __syncthreads();
    for (int i = k + 1 + warp; i < m; i += nw) {
      const double lik = L[tri_index(i, k)];
      double *row = L + tri_index(i, 0);
      for (int j = k + 1 + lane; j <= i; j += 32) row[j] -= lik * L[tri_index(j, k)];
    }
    __syncthreads();
  }
  if (warp == 0) {
    warp_forward_solve<2>(L, vec, N, m);
    warp_backward_solve<2>(L, vec, N, m);
  }
  __syncthreads();
  if (warp == 0) {
    double sx = 0.0, sy = 0.0;
    for (int k = lane; k < m; k += 32) {
      sx += vec[k];
      sy += vec[N + k];
    }
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    if (lane == 0) {
      const double lam = m > 0 ? (sx - c.charge[b]) / sy : 0.0;
      c.w.eeq_sum[2 * b] = sy;
      c.w.eeq_sum[2 * b + 1] = lam;
      s_inv = lam;
    }
  }
  __syncthreads();
  const double lam = s_inv;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    c.w.q[(size_t)b * N + i] = 0.0;
    c.w.eeq_y[(size_t)b * N + i] = 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const size_t a = (size_t)b * N + s_idx[k];
    c.w.q[a] = vec[k] - lam * vec[N + k];
    c.w.eeq_y[a] = vec[N + k];
  }
  if (SMEM) {
    double *G = c.w.eeq_L + (size_t)b * ((size_t)N * (N + 1) / 2);
    for (size_t t = threadIdx.x; t < tri_m; t += blockDim.x) G[t] = L[t];
  }
}

// Adjoint of the constrained EEQ solve: w = A^-1 g - nu A^-1 1 with
// sum(w) = 0, g = dE/dq.  Then dE/d(raw EEQ CN) = w kcn / (2 sqrt(cn)) dcap.
__global__ void __launch_bounds__(256) eeq_adjoint_kernel(Ctx c) {
  extern __shared__ double s_dyn[];
  const int b = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_m;
  __shared__ double s_nu;
  int *s_idx = reinterpret_cast<int *>(s_dyn);
  double *vec = s_dyn + (N + 1) / 2 + 1;
  const int m = compact_real_atoms(c, b, n, s_idx, &s_m);
  const double *L = c.w.eeq_L + (size_t)b * ((size_t)N * (N + 1) / 2);
  for (int k = threadIdx.x; k < m; k += blockDim.x) vec[k] = c.w.dEdq[(size_t)b * N + s_idx[k]];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    warp_forward_solve<1>(L, vec, N, m);
    warp_backward_solve<1>(L, vec, N, m);
    double su = 0.0;
    for (int k = lane; k < m; k += 32) su += vec[k];
    su = warp_sum(su);
    if (lane == 0) s_nu = m > 0 ? su / c.w.eeq_sum[2 * b] : 0.0;
  }
  __syncthreads();
  const double nu = s_nu;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    c.w.eeq_w[(size_t)b * N + i] = 0.0;
    c.w.dEdcnq[(size_t)b * N + i] = 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const size_t a = (size_t)b * N + s_idx[k];
    const double w = vec[k] - nu * c.w.eeq_y[a];
    c.w.eeq_w[a] = w;
    const double cq = c.w.cnq[a];
    const int z = c.w.z[a];
    c.w.dEdcnq[a] = cq > 0.0 ? w * c.tab.eeq_kcn[z] * 0.5 / sqrt(cq) * c.w.dcnq[a] : 0.0;
  }
}

// ---------------------------------------------------------------- weights

constexpr int WU = 4;  // (atom, slot) units per warp of weights_kernel

// Charge-scaled Gaussian weights of every reference and the weighted
// polarisabilities A_i(w) = sum_r gw_ir alpha_{Z_i r}(w), at the charges q
// and at q = 0, with their derivatives.  A warp handles four units (atom,
// D4S slot): in phase 1 lane 8u + r computes reference r of unit u (lanes
// 8u + 7 idle), in phase 2 the lanes cover the 4 x 23 (unit, frequency)
// outputs, reading the per-reference values from shared memory.
__global__ void __launch_bounds__(256) weights_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int N = c.N;
  const int S = c.S;
  __shared__ double s_w[8][WU][5][NREF];
  const int u = lane >> 3, r = lane & 7;
  const int unit = (blockIdx.x * 8 + warp) * WU + u;  // = atom * S + slot
  const int i = unit / S, s = unit % S;
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  const bool d4s = c.cfg.kind == D4_MODEL_D4S;
  const int n = c.w.n_eff[b];
  const int nslot = c.w.n_slots[b];
  const size_t ai = (size_t)b * N + (i < N ? i : 0);
  const int zi = (i < N) ? c.w.z[ai] : 0;
  const bool live = i < N && i < n && zi != 0 && s < nslot;
  // ---- phase 1: references
  double e = 0.0, de = 0.0, refcn = -1e300;
  int refc = 0;
  double z = 0.0, dz = 0.0, z0 = 0.0;
  if (live && r < NREF) {
    const double cn = c.w.cn[ai];
    const double wf = d4s ? c.tab.wfpair[zi * c.tab.n_elem + c.w.slot_elem[b * MAX_ELEM_ID + s]]
                          : c.cfg.wf;
    refc = (int)c.tab.refc[zi * NREF + r];
    refcn = c.tab.refcovcn[zi * NREF + r];
    const double dcn = cn - refcn;
    if (refc > 0) {
      if (!d4s) {  // model/d4.py:177-194
        const double tmp = exp(-dcn * dcn);
        // tmp^wf: the default wf = 6 by products (within a few ulp of pow)
        const bool six = wf == 6.0;
        double p1;
        if (six) {
          const double t2 = tmp * tmp;
          p1 = t2 * t2 * t2;
        } else {
          p1 = pow(tmp, wf);
        }
        if (refc == 1) {
          e = p1;
          de = -2.0 * wf * dcn * p1;
        } else if (refc == 3) {
          const double p2 = six ? p1 * p1 : pow(tmp, 2.0 * wf);
          const double p3 = six ? p2 * p1 : pow(tmp, 3.0 * wf);
          e = p1 + p2 + p3;
          de = -2.0 * wf * dcn * (p1 + 2.0 * p2 + 3.0 * p3);
        } else {
          e = tmp;
          de = -2.0 * dcn * tmp;
        }
      } else {  // model/d4s.py:191-213
        const double tmp = exp(-dcn * dcn * wf);
        const double dtmp = -2.0 * wf * dcn * tmp;
        if (refc == 3) {
          const double t2 = tmp * tmp, t3 = t2 * tmp;
          e = tmp + t2 + t3;
          de = dtmp * (1.0 + 2.0 * tmp + 3.0 * t2);
        } else {
          e = tmp;
          de = dtmp;
        }
      }
      const double zeff = (double)c.tab.zeff[zi];
      const double gam = c.tab.gam[zi] * c.cfg.gc;
      const double qref = c.tab.refq[zi * NREF + r] + zeff;
      double dz0;
      zeta_and_deriv(gam, qref, c.w.q[ai] + zeff, c.cfg.ga, DBL_EPSILON, &z, &dz);
      zeta_and_deriv(gam, qref, 0.0 + zeff, c.cfg.ga, DBL_EPSILON, &z0, &dz0);
    }
  }
  // sums over the 8-lane group of this unit
  double norm = e, dnorm = de, maxcn = refcn;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    norm += __shfl_xor_sync(0xffffffffu, norm, o);
    dnorm += __shfl_xor_sync(0xffffffffu, dnorm, o);
    maxcn = fmax(maxcn, __shfl_xor_sync(0xffffffffu, maxcn, o));
  }
  if (r < NREF) {
    double gq = 0.0, g0 = 0.0, dgq_dcn = 0.0, dgq_dq = 0.0, dg0_dcn = 0.0;
    if (live && refc > 0) {
      double gw = e / norm;
      double dgw = (de - gw * dnorm) / norm;
      if (isnan(gw) || gw > DBL_MAX) {  // utils.py:208-224, model/d4.py:209-217
        gw = (refcn == maxcn) ? 1.0 : 0.0;
        dgw = 0.0;
      }
      gq = z * gw;
      g0 = z0 * gw;
      dgq_dcn = z * dgw;
      dgq_dq = dz * gw;
      dg0_dcn = z0 * dgw;
    }
    s_w[warp][u][0][r] = gq;
    s_w[warp][u][1][r] = g0;
    s_w[warp][u][2][r] = dgq_dcn;
    s_w[warp][u][3][r] = dgq_dq;
    s_w[warp][u][4][r] = dg0_dcn;
  }
  __syncwarp();
  // ---- phase 2: frequencies
  for (int o = lane; o < WU * NFREQ; o += 32) {
    const int uu = o / NFREQ, w = o % NFREQ;
    const int unit2 = (blockIdx.x * 8 + warp) * WU + uu;
    const int i2 = unit2 / S, s2 = unit2 % S;
    if (i2 >= N) continue;
    const size_t a2 = (size_t)b * N + i2;
    const int z2 = c.w.z[a2];
    const size_t off = (a2 * S + s2) * NFREQ + w;
    double a = 0.0, a0 = 0.0, da_dcn = 0.0, da_dq = 0.0, da0_dcn = 0.0;
    if (z2 != 0) {
      const double *alpha = c.tab.alpha + (size_t)z2 * NREF * NFREQ + w;
#pragma unroll
      for (int rr = 0; rr < NREF; ++rr) {
        const double al = alpha[rr * NFREQ];
        a += s_w[warp][uu][0][rr] * al;
        a0 += s_w[warp][uu][1][rr] * al;
        da_dcn += s_w[warp][uu][2][rr] * al;
        da_dq += s_w[warp][uu][3][rr] * al;
        da0_dcn += s_w[warp][uu][4][rr] * al;
      }
    }
    c.w.A[off] = a;
    c.w.A0[off] = a0;
    if (grad) {
      c.w.dA_dcn[off] = da_dcn;
      c.w.dA_dq[off] = da_dq;
      c.w.dA0_dcn[off] = da0_dcn;
    }
  }
}

// ---------------------------------------------------------------- pairs

// One order n of a D3-family two-body damping (damping/functions.py:308-484):
// t = f_n / r^n and its derivatives with respect to r and to the damping
// parameters.  ``rv`` is the pair's van der Waals radius (zero and
// modified-zero damping), ``R0`` = a1 sqrt(3 r4r2_i r4r2_j) + a2 (optimised
// power), ``rs`` the order's radius scaling, ``pw`` its exponent (alp for
// n = 6, alp + 2 for n = 8; bet for the optimised power).
struct DampD3 {
  double t, dr, dR0, drs, dalp, dbet;
};

__device__ __forceinline__ DampD3 damp_d3(int kind, int n, double r, double R0, double rv,
                                          double rs, double pw, double bet) {
  DampD3 d{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double rn = r * r;
  rn = rn * rn * rn;
  if (n == 8) rn *= r * r;
  if (kind == D4_DAMP_ZERO) {
    // f = 1 / (1 + 6 u^p), u = rs r / rv (the reference's argument order)
    const double u = rs * r / rv;
    const double up = pow(u, pw);
    const double f = 1.0 / (1.0 + 6.0 * up);
    d.t = f / rn;
    const double dfdu = -6.0 * f * f * (u > 0.0 ? pw * up / u : 0.0);
    d.dr = dfdu * (rs / rv) / rn - n * d.t / r;
    d.drs = dfdu * (r / rv) / rn;
    d.dalp = u > 0.0 ? -6.0 * f * f * up * log(u) / rn : 0.0;
  } else if (kind == D4_DAMP_MZERO) {
    // f = 1 / (1 + 6 u^-p), u = r / (rs rv) + bet rv
    const double u = r / (rs * rv) + bet * rv;
    const double um = pow(u, -pw);
    const double f = 1.0 / (1.0 + 6.0 * um);
    d.t = f / rn;
    const double dfdu = 6.0 * pw * um / u * f * f;
    d.dr = dfdu / (rs * rv) / rn - n * d.t / r;
    d.drs = -dfdu * r / (rs * rs * rv) / rn;
    d.dbet = dfdu * rv / rn;
    d.dalp = 6.0 * um * log(u) * f * f / rn;
  } else {  // D4_DAMP_OP: r^bet / (r^bet r^n + R0^bet r^n) = 1 / (r^n (1 + (R0/r)^bet))
    const double x = R0 / r;
    const double v = pow(x, bet);
    const double h = 1.0 / (1.0 + v);
    d.t = h / rn;
    d.dr = d.t / r * (bet * v * h - n);
    d.dR0 = -d.t * bet * v * h / R0;
    d.dbet = -d.t * v * h * log(x);
  }
  return d;
}

// Fused C6 + rational (BJ) two-body energy, its direct gradient and its C6
// adjoint, and the per-pair tables the ATM kernel consumes.  One warp per
// atom i; lanes over partners j.  C6 is never stored.
__global__ void __launch_bounds__(256) pair_fwd_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  __shared__ double s_wa[8][NFREQ];
  __shared__ double s_wa0[8][NFREQ];
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int zi = c.w.z[ai];
  const int n = c.w.n_eff[b];
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  if (i >= n || zi == 0) {
    if (lane == 0) {
      c.out.d_energy[ai] = 0.0;
      if (grad) {
        c.out.d_gradient[3 * ai] = 0.0;
        c.out.d_gradient[3 * ai + 1] = 0.0;
        c.out.d_gradient[3 * ai + 2] = 0.0;
      }
    }
    if (grad && lane < NFREQ)
      for (int s = 0; s < c.S; ++s) c.w.G[(ai * c.S + s) * NFREQ + lane] = 0.0;
    return;
  }
  const d4_params_t &p = c.par;
  const double *P = c.positions + (size_t)b * N * 3;
  const double xi = P[3 * i], yi = P[3 * i + 1], zi3 = P[3 * i + 2];
  const double r4i = atom_r4r2(c, ai, zi);
  const double wi = atom_weight(c, ai);
  const int nslot = c.w.n_slots[b];
  const int slot_i = c.w.slot[ai];
  const double *fw = c.tab.freq_weights;
  double e_acc = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
  // s6, s8, s10, a1, a2, -, alp, rs6, rs8, bet (slots of d_param_grad)
  double pg[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double *rvdw_row = c.rvdw_in ? c.rvdw_in + ai * N : nullptr;
  for (int s = 0; s < nslot; ++s) {
    if (lane < NFREQ) {
      const size_t o = (ai * c.S + s) * NFREQ + lane;
      s_wa[warp][lane] = THOPI * fw[lane] * c.w.A[o];
      s_wa0[warp][lane] = THOPI * fw[lane] * c.w.A0[o];
    }
    __syncwarp();
    double gacc[NFREQ];
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) gacc[w] = 0.0;
    for (int j = lane; j < n; j += 32) {
      const size_t aj = (size_t)b * N + j;
      const int zj = c.w.z[aj];
      if (j == i || zj == 0 || c.w.slot[aj] != s) continue;
      const double dx = xi - P[3 * j], dy = yi - P[3 * j + 1], dz = zi3 - P[3 * j + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      const double r = sqrt(r2);
      const double *Aj = c.w.A + (aj * c.S + slot_i) * NFREQ;
      const double *A0j = c.w.A0 + (aj * c.S + slot_i) * NFREQ;
      double c6 = 0.0, c60 = 0.0;
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) {
        c6 += s_wa[warp][w] * Aj[w];
        c60 += s_wa0[warp][w] * A0j[w];
      }
      const double qq = 3.0 * r4i * atom_r4r2(c, aj, zj);
      const double sqq = sqrt(qq);
      const double R0 = p.a1 * sqq + p.a2;
      const size_t pij = ((size_t)b * N + i) * N + j;
      c.w.pr_r[pij] = r;
      c.w.pr_ir[pij] = 1.0 / r;
      c.w.pr_L[pij] = log(R0 / r);
      c.w.pr_c[pij] = sqrt(c60);
      if (c.w.pr_da1) {
        c.w.pr_da1[pij] = sqq / R0;
        c.w.pr_da2[pij] = 1.0 / R0;
      }
      if (r <= p.cut_disp2 && p.damping != D4_DAMP_RATIONAL) {
        // D3-family damping: e = s6 c6 t6 + s8 c8 t8 (dispersion2,
        // dispersion/twobody.py:147-182), derivatives of -e as below
        const double rv = rvdw_row ? rvdw_row[j] : 0.0;
        const bool zero_kind = p.damping != D4_DAMP_OP;
        const DampD3 d6 = damp_d3(p.damping, 6, r, R0, rv, p.rs6,
                                  zero_kind ? p.alp : p.bet, p.bet);
        double e = p.s6 * c6 * d6.t;
        double dEdr = -p.s6 * c6 * d6.dr;
        double K = -p.s6 * d6.t;
        double gR0 = -p.s6 * c6 * d6.dR0, grs6 = -p.s6 * c6 * d6.drs, grs8 = 0.0;
        double galp = -p.s6 * c6 * d6.dalp, gbet = -p.s6 * c6 * d6.dbet;
        pg[0] += -wi * c6 * d6.t;
        if (p.has_s8) {
          const double c8 = c6 * qq;
          const DampD3 d8 = damp_d3(p.damping, 8, r, R0, rv, p.rs8,
                                    zero_kind ? p.alp + 2.0 : p.bet, p.bet);
          e += p.s8 * c8 * d8.t;
          dEdr += -p.s8 * c8 * d8.dr;
          K += -p.s8 * qq * d8.t;
          gR0 += -p.s8 * c8 * d8.dR0;
          grs8 += -p.s8 * c8 * d8.drs;
          galp += -p.s8 * c8 * d8.dalp;
          gbet += -p.s8 * c8 * d8.dbet;
          pg[1] += -wi * c8 * d8.t;
        }
        e_acc += -0.5 * e;
        const double phi = 0.5 * (wi + atom_weight(c, aj));
        dEdr *= phi;
        K *= phi;
        pg[3] += wi * 0.5 * gR0 * sqq;
        pg[4] += wi * 0.5 * gR0;
        pg[6] += wi * 0.5 * galp;
        pg[7] += wi * 0.5 * grs6;
        pg[8] += wi * 0.5 * grs8;
        pg[9] += wi * 0.5 * gbet;
        const double f = dEdr / r;
        gx += f * dx;
        gy += f * dy;
        gz += f * dz;
        if (grad) {
#pragma unroll
          for (int w = 0; w < NFREQ; ++w) gacc[w] += K * Aj[w];
        }
      } else if (r <= p.cut_disp2) {
        const double r6 = r2 * r2 * r2, R02 = R0 * R0, R06 = R02 * R02 * R02;
        const double t6 = 1.0 / (r6 + R06);
        double e = p.s6 * c6 * t6;
        double dEdr = 6.0 * p.s6 * c6 * (r6 / r) * t6 * t6;
        double K = -p.s6 * t6;
        // dt_n/dR0 = -n R0^(n-1) t_n^2 ; dR0/da1 = sqq, dR0/da2 = 1
        double dE_dR0 = p.s6 * c6 * 6.0 * (R06 / R0) * t6 * t6;
        pg[0] += -wi * c6 * t6;
        if (p.has_s8) {
          const double r8 = r6 * r2, R08 = R06 * R02;
          const double t8 = 1.0 / (r8 + R08);
          const double c8 = c6 * qq;
          e += p.s8 * c8 * t8;
          dEdr += 8.0 * p.s8 * c8 * (r8 / r) * t8 * t8;
          K += -p.s8 * qq * t8;
          dE_dR0 += p.s8 * c8 * 8.0 * (R08 / R0) * t8 * t8;
          pg[1] += -wi * c8 * t8;
        }
        if (p.has_s10) {
          const double r10 = r6 * r2 * r2, R010 = R06 * R02 * R02;
          const double t10 = 1.0 / (r10 + R010);
          const double c10 = c6 * qq * qq * 49.0 / 40.0;
          e += p.s10 * c10 * t10;
          dEdr += 10.0 * p.s10 * c10 * (r10 / r) * t10 * t10;
          K += -p.s10 * qq * qq * 49.0 / 40.0 * t10;
          dE_dR0 += p.s10 * c10 * 10.0 * (R010 / R0) * t10 * t10;
          pg[2] += -wi * c10 * t10;
        }
        e_acc += -0.5 * e;
        // The pair energy e_ij = e_ji goes half to i, half to j, so the
        // weighted sum holds it with (w_i + w_j) / 2 per visit of (i, j)
        // and (j, i); dEdr and K above are the unit-weight derivatives of
        // e_ij + e_ji.  Parameter derivatives take atom i's share only.
        const double phi = 0.5 * (wi + atom_weight(c, aj));
        dEdr *= phi;
        K *= phi;
        pg[3] += wi * 0.5 * dE_dR0 * sqq;
        pg[4] += wi * 0.5 * dE_dR0;
        const double f = dEdr / r;
        gx += f * dx;
        gy += f * dy;
        gz += f * dz;
        if (grad) {
#pragma unroll
          for (int w = 0; w < NFREQ; ++w) gacc[w] += K * Aj[w];
        }
      }
    }
    if (grad) {
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) {
        const double g = warp_sum(gacc[w]);
        if (lane == w) c.w.G[(ai * c.S + s) * NFREQ + w] = THOPI * fw[w] * g;
      }
    }
    __syncwarp();
  }
  if (grad && lane < NFREQ)
    for (int s = nslot; s < c.S; ++s) c.w.G[(ai * c.S + s) * NFREQ + lane] = 0.0;
  e_acc = warp_sum(e_acc);
  gx = warp_sum(gx);
  gy = warp_sum(gy);
  gz = warp_sum(gz);
  if (c.flags & D4_FLAG_PARAM_GRAD) {
    const int npg = p.damping != D4_DAMP_RATIONAL ? 10 : 5;
#pragma unroll
    for (int k = 0; k < 10; ++k)
      if (k < npg) pg[k] = warp_sum(pg[k]);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 0], 0.5 * pg[0]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 1], 0.5 * pg[1]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 2], 0.5 * pg[2]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 3], pg[3]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 4], pg[4]);
      if (npg > 5) {
#pragma unroll
        for (int k = 6; k < 10; ++k) atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + k], pg[k]);
      }
    }
  }
  if (lane == 0) {
    c.out.d_energy[ai] = e_acc;
    if (grad) {
      c.out.d_gradient[3 * ai] = gx;
      c.out.d_gradient[3 * ai + 1] = gy;
      c.out.d_gradient[3 * ai + 2] = gz;
    }
  }
}

// ---------------------------------------------------------------- ATM

// Axilrod-Teller-Muto energy over triples i < j < k.  A CTA owns a tile of
// pairs (j, k) -- 8 rows j (one per warp) by 32 columns k (one per lane) --
// and loops over i < j.  Everything a triple needs is a per-pair scalar:
// r, 1/r, log(R0/r), sqrt(C6(q=0)).  With GRAD, it accumulates per pair
// S = dE/d(r^2) and P = sum of mask-weighted triple energies (upper entry
// [min][max]), from which pair kernel B builds forces and dE/dC6.
template <bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(256) atm_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  const int ntk = (N + 31) / 32;
  const int jb = blockIdx.x / ntk, kb = blockIdx.x % ntk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j0 = jb * 8, k0 = kb * 32;
  if (j0 >= n || k0 + 31 <= j0) return;  // empty tile (block-uniform)
  const int j = j0 + warp, k = k0 + lane;
  const int *Zb = c.w.z + (size_t)b * N;
  const bool pair_ok = j < n && k < n && k > j && Zb[j] != 0 && Zb[k] != 0;
  const double cut = c.par.cut_disp3;
  const double alp3 = c.par.alp / 3.0;
  const double s9 = c.par.s9;
  const size_t base = (size_t)b * N * N;
  double rjk = 1.0, irjk = 0.0, Ljk = 0.0, cjk = 0.0;
  if (pair_ok) {
    const size_t o = base + (size_t)j * N + k;
    rjk = c.w.pr_r[o];
    irjk = c.w.pr_ir[o];
    Ljk = c.w.pr_L[o];
    cjk = c.w.pr_c[o];
  }
  const double zjk = rjk * rjk;
  const bool mjk = rjk <= cut;
  const double wj = pair_ok ? atom_weight(c, (size_t)b * N + j) : 0.0;
  const double wk = pair_ok ? atom_weight(c, (size_t)b * N + k) : 0.0;
  double Sjk = 0.0, Pjk = 0.0, Ej = 0.0, Ek = 0.0;
  double g_s9 = 0.0, g_alp = 0.0, g_a1 = 0.0, g_a2 = 0.0;
  double da1jk = 0.0, da2jk = 0.0;
  if (PGRAD && pair_ok) {
    const size_t o = base + (size_t)j * N + k;
    da1jk = c.w.pr_da1[o];
    da2jk = c.w.pr_da2[o];
  }
  __shared__ double red[2][3][8][32];
  const int i_end = min(j0 + 8, n) - 1;  // i < j <= j0 + 7
  for (int i = 0; i < i_end; ++i) {
    double sij = 0.0, pij = 0.0, ei = 0.0, sik = 0.0, pik = 0.0;
    if (pair_ok && i < j && Zb[i] != 0) {
      const size_t oij = base + (size_t)i * N + j;
      const size_t oik = base + (size_t)i * N + k;
      const double rij = c.w.pr_r[oij], rik = c.w.pr_r[oik];
      const double irij = c.w.pr_ir[oij], irik = c.w.pr_ir[oik];
      const double x = rij * rij, y = rik * rik, z = zjk;
      const bool mij = rij <= cut, mik = rik <= cut;
      const int wcount = (mij & mik) + (mij & mjk) + (mik & mjk);
      if (wcount > 0) {
        const double ir1 = irij * irik * irjk;
        const double ir2 = ir1 * ir1;
        const double ir3 = ir1 * ir2;
        const double A = x + z - y, Bv = x - z + y, Cv = -x + z + y;
        const double sfac = A * Bv * Cv;
        const double ang = ir3 * (0.375 * sfac * ir2 + 1.0);
        const double Lsum = c.w.pr_L[oij] + c.w.pr_L[oik] + Ljk;
        const double ta = exp(alp3 * Lsum);
        const double fd = 1.0 / (1.0 + 6.0 * ta);
        const double c9 = c.w.pr_c[oij] * c.w.pr_c[oik] * cjk;
        const double e = s9 * c9 * fd * ang;
        const double sixth = e * (1.0 / 6.0);
        const double mi = (double)(mjk * (mij + mik));
        const double mj = (double)(mik * (mij + mjk));
        const double mk = (double)(mij * (mik + mjk));
        ei = sixth * mi;
        Ej += sixth * mj;
        Ek += sixth * mk;
        if (GRAD) {
          // weight of this triple in sum_x w_x E_x (wcount / 3 for unit weights)
          const double wgt =
              (atom_weight(c, (size_t)b * N + i) * mi + wj * mj + wk * mk) * (1.0 / 6.0);
          // de/d(r^2): see the derivation in the module notes
          const double K = s9 * c9;
          const double dfl = 6.0 * alp3 * ta * fd * fd;  // df / d ln r_xy
          const double Q = -(5.0 * ang - 2.0 * ir3);
          const double U = K * fd * 0.375 * ir2 * ir3;
          const double V = 0.5 * K * (fd * Q + ang * dfl);
          const double BC = Bv * Cv, AC = A * Cv, AB = A * Bv;
          const double dex = U * (BC + AC - AB) + V * irij * irij;
          const double dey = U * (-BC + AC + AB) + V * irik * irik;
          const double dez = U * (BC - AC + AB) + V * irjk * irjk;
          sij = wgt * dex;
          sik = wgt * dey;
          Sjk += wgt * dez;
          const double we = wgt * e;
          pij = we;
          pik = we;
          Pjk += we;
          if (PGRAD) {
            // e = s9 c9 f ang, f = 1 / (1 + 6 exp(alp/3 sum log(R0/r)))
            const double base_e = c9 * fd * ang;
            const double dfdL = -6.0 * fd * fd * ta;  // df / d(alp/3 * Lsum)
            g_s9 += wgt * base_e;
            g_alp += wgt * s9 * c9 * ang * dfdL * Lsum * (1.0 / 3.0);
            const double dfa = wgt * s9 * c9 * ang * dfdL * alp3;
            g_a1 += dfa * (c.w.pr_da1[oij] + c.w.pr_da1[oik] + da1jk);
            g_a2 += dfa * (c.w.pr_da2[oij] + c.w.pr_da2[oik] + da2jk);
          }
        }
      }
    }
    // (i, j) and E_i: reduce over the lanes of this warp
    if (GRAD) {
      sij = warp_sum(sij);
      pij = warp_sum(pij);
    }
    ei = warp_sum(ei);
    if (lane == 0 && i < j && j < n) {
      if (ei != 0.0) atomicAdd(&c.w.e3[(size_t)b * N + i], ei);
      if (GRAD && (sij != 0.0 || pij != 0.0)) {
        const size_t oij = base + (size_t)i * N + j;
        atomicAdd(&c.w.pr_S[oij], sij);
        atomicAdd(&c.w.pr_P[oij], pij);
      }
    }
    if (GRAD) {
      // (i, k): reduce over the warps of the CTA through shared memory
      const int buf = i & 1;
      red[buf][0][warp][lane] = sik;
      red[buf][1][warp][lane] = pik;
      __syncthreads();
      if (warp == 0 && k < n) {
        double ss = 0.0, pp = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) {
          ss += red[buf][0][w][lane];
          pp += red[buf][1][w][lane];
        }
        if (ss != 0.0 || pp != 0.0) {
          const size_t oik = base + (size_t)i * N + k;
          atomicAdd(&c.w.pr_S[oik], ss);
          atomicAdd(&c.w.pr_P[oik], pp);
        }
      }
    }
  }
  if (GRAD && pair_ok && (Sjk != 0.0 || Pjk != 0.0)) {
    const size_t o = base + (size_t)j * N + k;
    atomicAdd(&c.w.pr_S[o], Sjk);
    atomicAdd(&c.w.pr_P[o], Pjk);
  }
  Ej = warp_sum(Ej);
  if (lane == 0 && j < n && Ej != 0.0) atomicAdd(&c.w.e3[(size_t)b * N + j], Ej);
  if (PGRAD) {
    g_s9 = warp_sum(g_s9);
    g_alp = warp_sum(g_alp);
    g_a1 = warp_sum(g_a1);
    g_a2 = warp_sum(g_a2);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 3], g_a1);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 4], g_a2);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 5], g_s9);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 6], g_alp);
    }
  }
  __syncthreads();
  red[0][2][warp][lane] = Ek;
  __syncthreads();
  if (warp == 0 && k < n) {
    double ek = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) ek += red[0][2][w][lane];
    if (ek != 0.0) atomicAdd(&c.w.e3[(size_t)b * N + k], ek);
  }
}

// ATM forces from S, the ATM adjoint of C6(q = 0), the chain rule to
// dE/dCN and dE/dq per atom, and the final atom energy E2 + E3.
__global__ void __launch_bounds__(256) pair_atm_bwd_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x = blockIdx.x * 8 + warp;
  const int N = c.N;
  if (x >= N) return;
  const size_t ax = (size_t)b * N + x;
  const int zx = c.w.z[ax];
  const int n = c.w.n_eff[b];
  if (x >= n || zx == 0) {
    if (lane == 0) {
      c.w.dEdcn[ax] = 0.0;
      c.w.dEdq[ax] = 0.0;
    }
    if (lane < NFREQ)
      for (int s = 0; s < c.S; ++s) c.w.G0[(ax * c.S + s) * NFREQ + lane] = 0.0;
    return;
  }
  const double *P = c.positions + (size_t)b * N * 3;
  const double px = P[3 * x], py = P[3 * x + 1], pz = P[3 * x + 2];
  const int nslot = c.w.n_slots[b];
  const int slot_x = c.w.slot[ax];
  const size_t base = (size_t)b * N * N;
  const double *fw = c.tab.freq_weights;
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int s = 0; s < nslot; ++s) {
    double gacc[NFREQ];
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) gacc[w] = 0.0;
    for (int y = lane; y < n; y += 32) {
      const size_t ay = (size_t)b * N + y;
      if (y == x || c.w.z[ay] == 0 || c.w.slot[ay] != s) continue;
      const int lo = min(x, y), hi = max(x, y);
      const size_t o = base + (size_t)lo * N + hi;
      const double S = c.w.pr_S[o];
      const double Pv = c.w.pr_P[o];
      gx += 2.0 * S * (px - P[3 * y]);
      gy += 2.0 * S * (py - P[3 * y + 1]);
      gz += 2.0 * S * (pz - P[3 * y + 2]);
      if (Pv != 0.0) {
        const double cc = c.w.pr_c[base + (size_t)x * N + y];
        const double D = Pv / (2.0 * cc * cc);
        const double *A0y = c.w.A0 + (ay * c.S + slot_x) * NFREQ;
#pragma unroll
        for (int w = 0; w < NFREQ; ++w) gacc[w] += D * A0y[w];
      }
    }
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) {
      const double g = warp_sum(gacc[w]);
      if (lane == w) {
        double g0 = THOPI * fw[w] * g;
        if (c.w.gax)  // exact C9: the adjoint of a_x (D4) or of the slot averages (D4S)
          g0 += c.cfg.kind == D4_MODEL_D4S ? c.w.gbar[((size_t)b * c.S + s) * NFREQ + w]
                                           : c.w.gax[ax * NFREQ + w];
        c.w.G0[(ax * c.S + s) * NFREQ + w] = g0;
      }
    }
  }
  if (lane < NFREQ)
    for (int s = nslot; s < c.S; ++s) c.w.G0[(ax * c.S + s) * NFREQ + lane] = 0.0;
  gx = warp_sum(gx);
  gy = warp_sum(gy);
  gz = warp_sum(gz);
  if (c.w.f3x) {  // exact C9: the ATM force of atom x from its own warp
    gx += c.w.f3x[3 * ax];
    gy += c.w.f3x[3 * ax + 1];
    gz += c.w.f3x[3 * ax + 2];
  }
  __syncwarp();
  // chain rule to CN and q
  double dcn = 0.0, dq = 0.0;
  for (int s = 0; s < nslot; ++s) {
    if (lane < NFREQ) {
      const size_t o = (ax * c.S + s) * NFREQ + lane;
      dcn += c.w.G[o] * c.w.dA_dcn[o] + c.w.G0[o] * c.w.dA0_dcn[o];
      dq += c.w.G[o] * c.w.dA_dq[o];
    }
  }
  dcn = warp_sum(dcn);
  dq = warp_sum(dq);
  if (lane == 0) {
    c.w.dEdcn[ax] = dcn;
    c.w.dEdq[ax] = dq;
    c.out.d_gradient[3 * ax] += gx;
    c.out.d_gradient[3 * ax + 1] += gy;
    c.out.d_gradient[3 * ax + 2] += gz;
    c.out.d_energy[ax] += c.w.e3[ax];
  }
}

// Forces through the D4 CN, the EEQ CN and the EEQ Coulomb matrix.
__global__ void __launch_bounds__(256) pair_cn_bwd_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int zi = c.w.z[ai];
  const int n = c.w.n_eff[b];
  if (i >= n || zi == 0) return;
  const bool eeq = (c.flags & D4_FLAG_CHARGES_IN) == 0;
  const d4_params_t &p = c.par;
  const double *P = c.positions + (size_t)b * N * 3;
  const double xi = P[3 * i], yi = P[3 * i + 1], zi3 = P[3 * i + 2];
  const double rci = c.tab.cov_d3[zi], eni = c.tab.en[zi], radi = c.tab.eeq_rad[zi];
  const double gcn_i = c.w.dEdcn[ai];
  const double gq_i = eeq ? c.w.dEdcnq[ai] : 0.0;
  const double wi = eeq ? c.w.eeq_w[ai] : 0.0, qi = c.w.q[ai];
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int j = lane; j < n; j += 32) {
    const size_t aj = (size_t)b * N + j;
    const int zj = c.w.z[aj];
    if (j == i || zj == 0) continue;
    const double dx = xi - P[3 * j], dy = yi - P[3 * j + 1], dz = zi3 - P[3 * j + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    const double r0 = rci + c.tab.cov_d3[zj];
    const double dcf = erf_count_dr(r, r0, p.kcn);
    double dEdr = 0.0;
    if (r <= p.cut_cn) dEdr += (gcn_i + c.w.dEdcn[aj]) * en_factor(eni, c.tab.en[zj], p.k4, p.k5, p.k6) * dcf;
    if (eeq) {
      if (r <= p.cut_cn_eeq) dEdr += (gq_i + c.w.dEdcnq[aj]) * dcf;
      const double radj = c.tab.eeq_rad[zj];
      const double g = 1.0 / sqrt(radi * radi + radj * radj);
      const double gr = g * r;
      const double dA = (2.0 * g * INV_SQRT_PI * exp(-gr * gr) * r - erf(gr)) / (r * r);
      dEdr -= (wi * c.w.q[aj] + c.w.eeq_w[aj] * qi) * dA;
    }
    const double f = dEdr / r;
    gx += f * dx;
    gy += f * dy;
    gz += f * dz;
  }
  gx = warp_sum(gx);
  gy = warp_sum(gy);
  gz = warp_sum(gz);
  if (lane == 0) {
    c.out.d_gradient[3 * ai] += gx;
    c.out.d_gradient[3 * ai + 1] += gy;
    c.out.d_gradient[3 * ai + 2] += gz;
  }
}

// Energy-only finish: E = E2 + E3; optional outputs.
__global__ void finish_kernel(Ctx c) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)c.B * c.N;
  if (t >= total) return;
  if (!(c.flags & D4_FLAG_GRADIENT)) c.out.d_energy[t] += c.w.e3[t];
  if (c.out.d_charges) c.out.d_charges[t] = c.w.q[t];
  if (c.out.d_cn_eeq) c.out.d_cn_eeq[t] = c.w.cnq[t];
}

// Copy charges given by the caller into the workspace.
__global__ void charges_in_kernel(Ctx c) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)c.B * c.N;
  if (t >= total) return;
  c.w.q[t] = c.w.z[t] != 0 ? c.charges_in[t] : 0.0;
}

// Parameter gradients per structure: two-body terms from pair_fwd_kernel,
// s9 / alp / ATM radii from atm_kernel.
__global__ void param_grad_finish_kernel(Ctx c) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < D4_PARAM_GRAD_STRIDE * c.B) c.out.d_param_grad[t] = c.w.pgrad[t];
}

// ---------------------------------------------------------------- alpha

__global__ void prepare_alpha_kernel(d4_tables_t tab, d4_model_cfg_t cfg,
                                     const double *refalpha, const double *refascale,
                                     const double *refscount, const int64_t *refsys,
                                     const double *secscale, const double *secalpha,
                                     int n_sec, const double *refh, double *out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = tab.n_ref_elem * NREF * NFREQ;
  if (t >= total) return;
  const int w = t % NFREQ;
  const int er = t / NFREQ;  // element * NREF + ref
  const int64_t s = refsys[er];
  double zeta = 0.0;
  if (s > 0 && s < n_sec) {
    const double zeff = (double)tab.zeff[s];
    const double gam = tab.gam[s] * cfg.gc;
    double dz;
    zeta_and_deriv(gam, zeff, refh[er] + zeff, cfg.ga, DBL_EPSILON, &zeta, &dz);
  }
  const int ss = (s > 0 && s < n_sec) ? (int)s : 0;
  const double aiw = secscale[ss] * secalpha[ss * NFREQ + w] * zeta;
  const double h = refalpha[t] - refscount[er] * aiw;
  const double a = refascale[er] * h;
  out[t] = a > 0.0 ? a : 0.0;
}

// ---------------------------------------------------------------- launch

int launch_fp64(const Ctx &c, cudaStream_t st) {
  const int B = c.B, N = c.N;
  const dim3 atoms((N + 7) / 8, B);
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  const bool eeq = (c.flags & D4_FLAG_CHARGES_IN) == 0;
  timing_next_call();
  stage_begin(ST_PREP, st);
  launch_prep(c, st);
  stage_end(ST_PREP, st);
  stage_begin(ST_CN, st);
  cn_kernel<<<atoms, 256, 0, st>>>(c);
  stage_end(ST_CN, st);
  const size_t vec_bytes = (size_t)8 * ((N + 1) / 2 + 1 + 2 * N);
  const size_t tri_bytes = (size_t)8 * ((size_t)N * (N + 1) / 2);
  stage_begin(ST_EEQ, st);
  if (eeq) {
    if (vec_bytes + tri_bytes <= 220 * 1024) {
      ensure_smem(eeq_kernel<true>, (int)(vec_bytes + tri_bytes));
      eeq_kernel<true><<<B, 256, vec_bytes + tri_bytes, st>>>(c);
    } else {
      ensure_smem(eeq_kernel<false>, (int)vec_bytes);
      eeq_kernel<false><<<B, 256, vec_bytes, st>>>(c);
    }
  } else {
    const size_t total = (size_t)B * N;
    charges_in_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c);
  }
  stage_end(ST_EEQ, st);
  stage_begin(ST_WEIGHTS, st);
  const dim3 units(((size_t)N * c.S + 8 * WU - 1) / (8 * WU), B);
  weights_kernel<<<units, 256, 0, st>>>(c);
  stage_end(ST_WEIGHTS, st);
  stage_begin(ST_PAIR_FWD, st);
  pair_fwd_kernel<<<atoms, 256, 0, st>>>(c);
  stage_end(ST_PAIR_FWD, st);
  const dim3 tiles(((N + 7) / 8) * ((N + 31) / 32), B);
  stage_begin(ST_ATM, st);
  if (c.flags & D4_FLAG_EXACT_C9) {
    launch_atm_exact(c, st);
  } else if (grad) {
    if (c.flags & D4_FLAG_PARAM_GRAD)
      atm_kernel<true, true><<<tiles, 256, 0, st>>>(c);
    else
      atm_kernel<true, false><<<tiles, 256, 0, st>>>(c);
  } else {
    atm_kernel<false, false><<<tiles, 256, 0, st>>>(c);
  }
  stage_end(ST_ATM, st);
  if (grad) {
    stage_begin(ST_PAIR_ATM_BWD, st);
    pair_atm_bwd_kernel<<<atoms, 256, 0, st>>>(c);
    stage_end(ST_PAIR_ATM_BWD, st);
    if (eeq) {
      stage_begin(ST_EEQ_ADJ, st);
      ensure_smem(eeq_adjoint_kernel, (int)vec_bytes);
      eeq_adjoint_kernel<<<B, 256, vec_bytes, st>>>(c);
      stage_end(ST_EEQ_ADJ, st);
    }
    stage_begin(ST_PAIR_CN_BWD, st);
    pair_cn_bwd_kernel<<<atoms, 256, 0, st>>>(c);
    stage_end(ST_PAIR_CN_BWD, st);
  }
  stage_begin(ST_FINISH, st);
  const size_t total = (size_t)B * N;
  finish_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c);
  if (c.flags & D4_FLAG_PARAM_GRAD)
    param_grad_finish_kernel<<<(D4_PARAM_GRAD_STRIDE * B + 255) / 256, 256, 0, st>>>(c);
  stage_end(ST_FINISH, st);
  return 0;
}

// get_properties (disp.py:149-197) of the D4 model: the atom-resolved C6 at
// the EEQ charges for every pair including i = j (model/d4.py:268-289; rows
// and columns of padding atoms 0), the static polarisabilities
// alpha_i = sum_r w_ir alpha_ir(0) (model/base.py:286-302), i.e. A_i at the
// first frequency, and the charges.  Warp per row i, lanes over j; the C6
// sums run in the order of pair_fwd_kernel.
__global__ void __launch_bounds__(256) props_kernel(Ctx c, double *c6out, double *alpha_out,
                                                    double *q_out) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  __shared__ double s_wa[8][NFREQ];
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int n = c.w.n_eff[b];
  const bool ri = i < n && c.w.z[ai] != 0;
  if (lane < NFREQ)
    s_wa[warp][lane] = ri ? THOPI * c.tab.freq_weights[lane] * c.w.A[ai * NFREQ + lane] : 0.0;
  __syncwarp();
  if (c6out) {
    double *row = c6out + ai * N;
    for (int j = lane; j < N; j += 32) {
      const size_t aj = (size_t)b * N + j;
      double v = 0.0;
      if (ri && j < n && c.w.z[aj] != 0) {
        const double *Aj = c.w.A + aj * NFREQ;
#pragma unroll
        for (int w = 0; w < NFREQ; ++w) v += s_wa[warp][w] * Aj[w];
      }
      row[j] = v;
    }
  }
  if (lane == 0) {
    if (alpha_out) alpha_out[ai] = ri ? c.w.A[ai * NFREQ] : 0.0;
    if (q_out) q_out[ai] = c.w.q[ai];
  }
}

int launch_properties(const Ctx &c, double *c6out, double *alpha_out, double *q_out,
                      cudaStream_t st) {
  const int B = c.B, N = c.N;
  const dim3 atoms((N + 7) / 8, B);
  launch_prep(c, st);
  cn_kernel<<<atoms, 256, 0, st>>>(c);
  const size_t vec_bytes = (size_t)8 * ((N + 1) / 2 + 1 + 2 * N);
  const size_t tri_bytes = (size_t)8 * ((size_t)N * (N + 1) / 2);
  if (vec_bytes + tri_bytes <= 220 * 1024) {
    ensure_smem(eeq_kernel<true>, (int)(vec_bytes + tri_bytes));
    eeq_kernel<true><<<B, 256, vec_bytes + tri_bytes, st>>>(c);
  } else {
    ensure_smem(eeq_kernel<false>, (int)vec_bytes);
    eeq_kernel<false><<<B, 256, vec_bytes, st>>>(c);
  }
  launch_weights(c, st);
  props_kernel<<<atoms, 256, 0, st>>>(c, c6out, alpha_out, q_out);
  return 0;
}

void launch_prep(const Ctx &c, cudaStream_t st) {
  launch_prep_memsets(c, st);
  prep_kernel<<<c.B, 256, 0, st>>>(c);
}

void launch_prep_memsets(const Ctx &c, cudaStream_t st) {
  cudaMemsetAsync(c.w.status, 0, sizeof(int), st);
  if (c.N > PREP_ZERO_MAX_N) {  // the pair accumulators of large structures: plain memsets
    const size_t bnn = (size_t)c.B * c.N * c.N;
    if (c.w.pr_S) cudaMemsetAsync(c.w.pr_S, 0, 8 * bnn, st);
    if (c.w.pr_P) cudaMemsetAsync(c.w.pr_P, 0, 8 * bnn, st);
    if (c.w.prS32) cudaMemsetAsync(c.w.prS32, 0, 4 * bnn, st);
    if (c.w.prP32) cudaMemsetAsync(c.w.prP32, 0, 4 * bnn, st);
  }
  if (c.w.atm_cnt) cudaMemsetAsync(c.w.atm_cnt, 0, 8 * 2 * (size_t)c.B, st);
}

void launch_cn(const Ctx &c, cudaStream_t st) {
  cn_kernel<<<dim3((c.N + 7) / 8, c.B), 256, 0, st>>>(c);
}

void launch_weights(const Ctx &c, cudaStream_t st) {
  const dim3 units(((size_t)c.N * c.S + 8 * WU - 1) / (8 * WU), c.B);
  weights_kernel<<<units, 256, 0, st>>>(c);
}

void launch_charges_in(const Ctx &c, cudaStream_t st) {
  const size_t total = (size_t)c.B * c.N;
  charges_in_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c);
}

void launch_finish(const Ctx &c, cudaStream_t st) {
  const size_t total = (size_t)c.B * c.N;
  finish_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c);
  if (c.flags & D4_FLAG_PARAM_GRAD)
    param_grad_finish_kernel<<<(D4_PARAM_GRAD_STRIDE * c.B + 255) / 256, 256, 0, st>>>(c);
}

int launch_prepare_alpha(const d4_tables_t &tab, const d4_model_cfg_t &cfg,
                         const double *refalpha, const double *refascale,
                         const double *refscount, const int64_t *refsys,
                         const double *secscale, const double *secalpha, int n_sec,
                         const double *refh, double *out, cudaStream_t st) {
  const int total = tab.n_ref_elem * NREF * NFREQ;
  prepare_alpha_kernel<<<(total + 255) / 256, 256, 0, st>>>(tab, cfg, refalpha, refascale,
                                                            refscount, refsys, secscale,
                                                            secalpha, n_sec, refh, out);
  return 0;
}

}  // namespace d4
