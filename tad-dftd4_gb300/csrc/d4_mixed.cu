// Precision form of the D4 path: FP32 coordination numbers, reference
// weights, pair and triple arithmetic with compensated accumulation, FP32
// Cholesky of the EEQ matrix recovered by FP64 iterative refinement; FP64 for
// the EEQ matrix and residuals and the final per-atom / per-structure
// reductions.
//
// Shared stages (prep, finish) are the FP64 ones.
#include <float.h>

#include "d4_common.cuh"
#include "d4_chol.cuh"
#include "d4_kernels.cuh"
#include "d4_prep.cuh"

namespace d4 {

constexpr float INV_SQRT_PI_F = 0.564189583547756f;
constexpr int ATM_CTA_TRIPLES = 300000;  // target triples per ATM CTA
constexpr int ATM_THREADS = 1024;       // 32 warps: one CTA per SM (shared memory)
constexpr int ATM_THREADS_PGRAD = 512;  // the parameter-gradient variant needs more registers

// ---------------------------------------------------------------- weights

// threads of tables32_kernel: the largest of its tables, 128 x 7 x 23
constexpr int TABLES32_THREADS = ((MAX_ELEM_ID * NREF * NFREQ + 255) / 256) * 256;
static_assert(TABLES32_THREADS >= MAX_ELEM_ID * MAX_ELEM_ID && TABLES32_THREADS >= ERF_TAB,
              "tables32_kernel covers every table");

// FP32 tables of the precision form, rebuilt on every call (20k values):
// alpha32 [128][7][23]; ref32 [128][7] = (refcovcn, refq + zeff, Gaussians
// per reference, zeta at q = 0 evaluated in FP64); el32 [128] = (zeff,
// gam * gc); the erf nodes and 1/sqrt(rad_a^2 + rad_b^2) per element pair as
// double-floats for the EEQ matrix.  Rows of elements without references are
// zero.
static __device__ __forceinline__ void tables32_entry(const Ctx &c, int t) {
  const int nz = c.tab.n_ref_elem < MAX_ELEM_ID ? c.tab.n_ref_elem : MAX_ELEM_ID;
  if (t < MAX_ELEM_ID * NREF * NFREQ) {
    const int z = t / (NREF * NFREQ);
    const dfl a = z < nz ? df_from(c.tab.alpha[t]) : dfl{0.f, 0.f};
    c.w.alpha32[t] = a.hi;
    c.w.alpha32lo[t] = a.lo;
  }
  if (t < NFREQ) {
    const dfl f = df_from(sqrt(THOPI * c.tab.freq_weights[t]));
    c.w.sfw[t] = make_float2(f.hi, f.lo);
  }
  if (t < MAX_ELEM_ID * NREF) {
    const int z = t / NREF;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    float z0lo = 0.f;
    if (z < nz && z < c.tab.n_elem) {
      const double zeff = (double)c.tab.zeff[z];
      const double qref = c.tab.refq[t] + zeff;
      double z0, dz0;
      zeta_and_deriv(c.tab.gam[z] * c.cfg.gc, qref, zeff, c.cfg.ga, DBL_EPSILON, &z0, &dz0);
      const dfl zz = df_from(z0);
      v = make_float4((float)c.tab.refcovcn[t], (float)qref, (float)c.tab.refc[t], zz.hi);
      z0lo = zz.lo;
    }
    c.w.ref32[t] = v;
    c.w.z0lo[t] = z0lo;
  }
  if (t < MAX_ELEM_ID) {
    float2 e = make_float2(0.f, 0.f);
    if (t < nz && t < c.tab.n_elem)
      e = make_float2((float)c.tab.zeff[t], (float)(c.tab.gam[t] * c.cfg.gc));
    c.w.el32[t] = e;
    dfl d = {0.f, 0.f};
    if (t < c.tab.n_elem) d = df_from(c.tab.eeq_eta[t] + SQRT_2_OVER_PI / c.tab.eeq_rad[t]);
    c.w.eeq_diag[t] = make_float2(d.hi, d.lo);
  }
  if (t < ERF_TAB) {  // nodes of the double-float erf
    const double x0 = (double)t / (double)ERF_SCALE;
    const dfl e = df_from(erf(x0)), d = df_from(2.0 / sqrt(M_PI) * exp(-x0 * x0));
    c.w.erf_tab[t] = make_float4(e.hi, e.lo, d.hi, d.lo);
  }
  if (t < MAX_ELEM_ID * MAX_ELEM_ID) {  // R0, qq, R0^6, R0^8 of the table r4r2 values
    const int za = t / MAX_ELEM_ID, zb = t % MAX_ELEM_ID;
    float4 A = make_float4(0.f, 0.f, 0.f, 0.f), Bq = A;
    if (za < c.tab.n_elem && zb < c.tab.n_elem) {
      const double qq = 3.0 * c.tab.r4r2[za] * c.tab.r4r2[zb];
      const double R0 = c.par.a1 * sqrt(qq) + c.par.a2;
      const double R02 = R0 * R0, R06 = R02 * R02 * R02;
      const dfl r0 = df_from(R0), q = df_from(qq), r6 = df_from(R06), r8 = df_from(R06 * R02);
      A = make_float4(r0.hi, r0.lo, q.hi, q.lo);
      Bq = make_float4(r6.hi, r6.lo, r8.hi, r8.lo);
    }
    c.w.pairA[t] = A;
    c.w.pairB[t] = Bq;
  }
  if (t < MAX_ELEM_ID * MAX_ELEM_ID) {  // CN pair constants in FP64, kept as double-floats
    // (an FP32 rounding of them would shift every pair of an element pair the
    // same way: a bias that adds up over the structure instead of averaging out)
    const int za = t / MAX_ELEM_ID, zb = t % MAX_ELEM_ID;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (za < c.tab.n_elem && zb < c.tab.n_elem && za > 0 && zb > 0) {
      const dfl a = df_from(1.0 / (c.tab.cov_d3[za] + c.tab.cov_d3[zb]));
      const dfl e = df_from(en_factor(c.tab.en[za], c.tab.en[zb], c.par.k4, c.par.k5, c.par.k6));
      v = make_float4(a.hi, a.lo, e.hi, e.lo);
    }
    c.w.cnpair[t] = v;
  }
  if (t < MAX_ELEM_ID * MAX_ELEM_ID) {  // 1 / sqrt(rad_a^2 + rad_b^2)
    const int za = t / MAX_ELEM_ID, zb = t % MAX_ELEM_ID;
    dfl g = {0.f, 0.f};
    if (za < c.tab.n_elem && zb < c.tab.n_elem) {
      const double ra = c.tab.eeq_rad[za], rb = c.tab.eeq_rad[zb];
      g = df_from(1.0 / sqrt(ra * ra + rb * rb));
    }
    c.w.igam[t] = make_float2(g.hi, g.lo);
  }
}

// The per-structure set-up (prep_structure: CTAs 0 .. B-1) and the per-call
// FP32 tables (the other CTAs) in one launch: neither needs the other.
__global__ void __launch_bounds__(256) prep_tables_kernel(Ctx c) {
  if ((int)blockIdx.x < c.B)
    prep_structure(c, blockIdx.x);
  else
    tables32_entry(c, ((int)blockIdx.x - c.B) * 256 + threadIdx.x);
}

// transposed index of (structure b, atom i, slot s, frequency w)
__device__ __forceinline__ size_t a32_index(int b, int i, int s, int w, int N, int S) {
  return (((size_t)b * S + s) * NFREQ + w) * N + i;
}

// Charge-scaled Gaussian reference weights and the weighted polarisabilities
// A_i(w) = sum_r gw_ir zeta_ir alpha_{Z_i r}(w) at q and at q = 0, with their
// CN / q derivatives, in FP32 (model/d4.py:103-228, model/d4s.py:109-248).
// One thread per (atom, slot); lanes over consecutive atoms, so that the
// transposed A32 / A032 rows are stored coalesced.
//
// The Gaussian exponents c k dcn_r^2 are taken relative to the nearest
// reference (smallest c dcn^2), whose first Gaussian becomes exp(0) = 1:
// the normalised weight is the same as the reference's e_r / sum e_r and the
// norm cannot underflow.  Where the
// reference's FP64 norm underflows (every |dcn| > 11) it falls back to the
// reference of largest refcovcn (model/d4.py:209-217), which is then also
// the nearest one, so both give the same weights.
//
// The nearest reference's weight is never rounded: near 1 it would be
// 1 - t with t spread over many decades, and FP32 rounds most such values
// the same way (up to 1), so the weights of every atom would sum to slightly
// more than 1 -- a bias that C6 ~ w_i w_j turns into a relative energy
// shift of ~1e-8 shared by the whole structure.  A is assembled as
// zeta_n alpha_n + sum_{r != n} gw_r (zeta_r alpha_r - zeta_n alpha_n), the
// first term as a double-float, the corrections in FP32 (exact in the limit
// of one reference, no value near 1 rounded).
__global__ void __launch_bounds__(128) weights_mixed_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int S = c.S, N = c.N;
  const int s = blockIdx.x % S;
  const int i = (blockIdx.x / S) * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int zi = c.w.z[ai];
  const bool grad = c.w.dA32 != nullptr;
  const bool live = i < c.w.n_eff[b] && zi != 0 && s < c.w.n_slots[b];
  // gq / g0: coefficients of the corrections (gw_r zeta_r for r != n,
  // -G zeta_n with G = sum_{r != n} gw_r for the nearest reference n);
  // zn / z0n: zeta of n at q and at q = 0 (double-floats) times weight 1
  float gq[NREF], g0[NREF], dgc[NREF], dgq[NREF], dg0[NREF];
  int rn = 0;
  float zn = 0.f, z0n = 0.f, z0nl = 0.f;
#pragma unroll
  for (int r = 0; r < NREF; ++r) gq[r] = g0[r] = dgc[r] = dgq[r] = dg0[r] = 0.f;
  if (live) {
    const bool d4s = c.cfg.kind == D4_MODEL_D4S;
    // FP64 set-up per reference (a few FP64 instructions per atom): the CN
    // offsets, the exponent differences to the nearest reference and q - q_ref
    // are rounded to FP32 only after the cancellations.
    const double cn = c.w.cn[ai];
    const double q = c.w.q[ai];
    const double wf = d4s ? c.tab.wfpair[zi * c.tab.n_elem + c.w.slot_elem[b * MAX_ELEM_ID + s]]
                          : c.cfg.wf;
    const float4 *R = c.w.ref32 + zi * NREF;
    const float *Z0L = c.w.z0lo + zi * NREF;
    float4 rv[NREF];
    float dcn[NREF], cf[NREF], ua[NREF], zq[NREF];
    double y64[NREF];
    double best = INFINITY;
    // charge scaling argument gam gc (q - q_ref) / (q + zeff) in FP64, rounded
    // once (an FP32-rounded gam would bias every atom of the element alike)
    const double qmod64 = q + (double)c.tab.zeff[zi];
    const double gam64 = c.tab.gam[zi] * c.cfg.gc;
    // one FP64 division per atom (GB300 runs FP64 at 1/64 of the FP32 rate)
    const double gq64 = qmod64 > 0.0 ? gam64 / qmod64 : 0.0;
#pragma unroll
    for (int r = 0; r < NREF; ++r) {
      rv[r] = R[r];
      const int refc = (int)rv[r].z;
      dcn[r] = cf[r] = ua[r] = zq[r] = 0.f;
      y64[r] = 0.0;
      if (refc <= 0) continue;  // no such reference: nothing below reads these
      const double d = cn - c.tab.refcovcn[zi * NREF + r];
      // D4: wf for 1 or 3 Gaussians, 1 otherwise; D4S: wf
      const double cfr = (d4s || refc == 1 || refc == 3) ? wf : 1.0;
      y64[r] = cfr * d * d;
      dcn[r] = (float)d;
      cf[r] = (float)cfr;
      // zeta(q) = exp(-ga expm1(u)) with the outer exponential in FP64,
      // rounded once: FP32 expf carries a mean relative error of ~+5e-9,
      // which C6 ~ zeta_i zeta_j would double into a bias shared by every pair
      // of the structure (expm1f's error is scaled down by u ~ 0.1 there)
      const double u64 = gq64 * (q - c.tab.refq[zi * NREF + r]);
      ua[r] = (float)u64;
      zq[r] = (float)exp(-c.cfg.ga * (double)expm1f((float)u64));
      if (y64[r] < best) {
        best = y64[r];
        rn = r;
      }
    }
    if (best < INFINITY) {
      float e[NREF], de[NREF];
      float norm = 0.f, dnorm = 0.f;
#pragma unroll
      for (int r = 0; r < NREF; ++r) {
        e[r] = de[r] = 0.f;
        const int refc = (int)rv[r].z;
        if (refc <= 0) continue;
        const float x1 = (float)(y64[r] - best);  // >= 0, 0 for the nearest reference
        const float y = (float)y64[r];
        const float t1 = expf(-x1);
        float ee = t1, dd = t1;
        if (refc == 3) {
          const float t2 = expf(-(y + x1)), t3 = expf(-(2.f * y + x1));
          ee = t1 + t2 + t3;
          dd = t1 + 2.f * t2 + 3.f * t3;
        }
        e[r] = ee;
        de[r] = -2.f * cf[r] * dcn[r] * dd;
        norm += ee;
        dnorm += de[r];
      }
      const float inorm = 1.0f / norm;
      const float2 el = c.w.el32[zi];
      const float qmod = (float)q + el.x;
      const float ga = c.pf.ga, gam = el.y;
      float G = 0.f;  // sum of the other references' weights
#pragma unroll
      for (int r = 0; r < NREF; ++r) {
        if ((int)rv[r].z <= 0) continue;
        const float gw = e[r] * inorm;
        const float dgw = (de[r] - gw * dnorm) * inorm;
        float z, dz;
        if (qmod > 0.f) {
          // model/base.py:308-335 as exp(-ga expm1(gam (q - q_ref) / (q + zeff)))
          const float em1 = expm1f(ua[r]);
          z = zq[r];
          dz = -ga * z * (1.f + em1) * gam * rv[r].y / (qmod * qmod);
        } else {
          z = expf(ga);
          dz = 0.f;
        }
        const float z0 = rv[r].w, z0l = Z0L[r];  // zeta(q = 0) as a double-float
        if (r == rn) {
          zn = z;
          z0n = z0;
          z0nl = z0l;
        } else {
          G += gw;
          gq[r] = z * gw;
          g0[r] = fmaf(z0l, gw, z0 * gw);
        }
        dgc[r] = z * dgw;
        dgq[r] = dz * gw;
        dg0[r] = fmaf(z0l, dgw, z0 * dgw);
      }
#pragma unroll
      for (int r = 0; r < NREF; ++r)  // static indices: the arrays stay in registers
        if (r == rn) {
          gq[r] = -G * zn;
          g0[r] = -G * (z0n + z0nl);
        }
    }
  }
  // A'(w) = sqrt((3/pi) w_w) A(w): the Casimir-Polder weight is folded into
  // A so that C6 = sum_w A'_i A'_j carries no rounded weight; alpha and the
  // scale are double-floats, the nearest reference's term zeta_n alpha_n is
  // a double-float, and the corrections are FP32 sums (no bias shared by all
  // atoms of an element)
  const float *al = c.w.alpha32 + (size_t)zi * NREF * NFREQ;
  const float *all = c.w.alpha32lo + (size_t)zi * NREF * NFREQ;
  for (int w = 0; w < NFREQ; ++w) {
    float a = 0.f, a0 = 0.f, da_dcn = 0.f, da_dq = 0.f, da0_dcn = 0.f;
    float al_ = 0.f, al0 = 0.f;
#pragma unroll
    for (int r = 0; r < NREF; ++r) {
      const float v = al[r * NFREQ + w], vl = all[r * NFREQ + w];
      a = fmaf(gq[r], v, a);
      al_ = fmaf(gq[r], vl, al_);
      a0 = fmaf(g0[r], v, a0);
      al0 = fmaf(g0[r], vl, al0);
      da_dcn = fmaf(dgc[r], v, da_dcn);
      da_dq = fmaf(dgq[r], v, da_dq);
      da0_dcn = fmaf(dg0[r], v, da0_dcn);
    }
    // the nearest reference's term, exact products as double-floats
    const float vn = al[rn * NFREQ + w], vnl = all[rn * NFREQ + w];
    const float bh = zn * vn, b0h = z0n * vn;
    const dfl A = df_two_sum(bh, a);
    const float Al = A.lo + (fmaf(zn, vn, -bh) + fmaf(zn, vnl, al_));
    const dfl A0 = df_two_sum(b0h, a0);
    const float A0l = A0.lo + (fmaf(z0n, vn, -b0h) + fmaf(z0nl, vn, fmaf(z0n, vnl, al0)));
    const float2 f = c.w.sfw[w];
    const size_t t = a32_index(b, i, s, w, N, S);
    c.w.A32[t] = fmaf(A.hi, f.x, fmaf(A.hi, f.y, Al * f.x));
    c.w.A032[t] = fmaf(A0.hi, f.x, fmaf(A0.hi, f.y, A0l * f.x));
    if (grad) {
      float *d = c.w.dA32 + 3 * ((ai * S + s) * NFREQ + w);
      d[0] = da_dcn * f.x;
      d[1] = da_dq * f.x;
      d[2] = da0_dcn * f.x;
    }
  }
}


// ---------------------------------------------------------------- CN

// D4 and EEQ coordination numbers in FP32 (precision form): the counting
// function as 1/2 erfc(x) (no cancellation for small counts) with
// x = kcn (r / r0 - 1) from 1/r0 as a double-float per element pair, the EN
// factor as a double-float per element pair (no FP32-rounded constant), and
// compensated per-lane sums; FP64 per-atom totals and the smooth EEQ cap in
// FP64.
__global__ void __launch_bounds__(256) cn_mixed_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int zi = c.w.z[ai];
  if (lane == 0) c.w.atm_rowmax[ai] = 0u;  // the pair kernels raise it
  if (i >= n || zi == 0) {
    if (lane == 0) {
      c.w.cn[ai] = 0.0;
      c.w.cnq[ai] = 0.0;
      c.w.dcnq[ai] = 0.0;
      if (c.out.d_cn) c.out.d_cn[ai] = 0.0;
    }
    return;
  }
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 *PL = c.w.pos32lo + (size_t)b * N;
  const float4 pi = P[i], li = PL[i];
  const float kcn = c.pf.kcn;
  const float cut_cn = c.pf.cut_cn, cut_q = c.pf.cut_q;
  const float4 *CP = c.w.cnpair + (size_t)zi * MAX_ELEM_ID;
  Acc32 s_d4, s_q;
  for (int j = lane; j < n; j += 32) {
    const int zj = c.w.z[(size_t)b * N + j];
    if (j == i || zj == 0) continue;
    const float4 pj = P[j];
    const float4 cp = CP[zj];
    const float3 d = pos_diff(pi, li, pj, PL[j]);
    const float dx = d.x, dy = d.y, dz = d.z;
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float x = kcn * fmaf(r, cp.y, fmaf(r, cp.x, -1.0f));  // kcn (r / r0 - 1)
    if (x > 9.0f) continue;  // erfc(9) / 2 < 1e-36
    const float cf = 0.5f * erfcf(x);
    if (r <= cut_cn) s_d4.add(fmaf(cf, cp.z, cf * cp.w));
    if (r <= cut_q) s_q.add(cf);
  }
  // FP32 warp reductions of the compensated per-lane sums (hi and lo apart)
  const Acc32 d4a = warp_sum_acc(s_d4), qa = warp_sum_acc(s_q);
  if (lane == 0) {
    const float q = qa.hi + qa.lo;
    const float m = c.pf.cn_max;
    const double d4 = d4a.value();
    c.w.cn[ai] = d4;
    // log(1 + e^m) - log(1 + e^(m - q)) = log1p(expm1(q) / (1 + e^(q - m))):
    // no cancellation, FP32 relative accuracy also for small q (the EEQ
    // right-hand side takes its square root, which is steep near 0).  Its
    // FP32 rounding differs from atom to atom and averages out in the
    // energies; the FP64 form would cost an FP64 pass per atom.
    const float t = 1.0f + expf(q - m);
    c.w.cnq[ai] = (double)log1pf(expm1f(q) / t);
    c.w.dcnq[ai] = (double)(1.0f / t);
    if (c.out.d_cn) c.out.d_cn[ai] = d4;
  }
}

// ---------------------------------------------------------------- pairs

// Fused C6 + BJ two-body term in FP32, the per-pair ATM table (float4:
// r^2, 1/r^2, (R0/r)^(alp/3), sqrt(C6(q=0)) / r^3), the direct gradient and
// the C6 adjoint.  One warp per atom i, lanes over partners j.
template <bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(256, 2) pair_fwd_mixed_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  __shared__ float s_wa[8][NFREQ];
  __shared__ float s_wa0[8][NFREQ];
  if (i >= N) return;
  const size_t ai = (size_t)b * N + i;
  const int zi = c.w.z[ai];
  const int n = c.w.n_eff[b];
  if (i >= n || zi == 0) {
    if (lane == 0) {
      c.out.d_energy[ai] = 0.0;
      if (GRAD) {
        c.out.d_gradient[3 * ai] = 0.0;
        c.out.d_gradient[3 * ai + 1] = 0.0;
        c.out.d_gradient[3 * ai + 2] = 0.0;
      }
    }
    if (GRAD && lane < NFREQ)
      for (int s = 0; s < c.S; ++s) c.w.G32[(ai * c.S + s) * NFREQ + lane] = 0.f;
    return;
  }
  const d4_params_t &p = c.par;
  const float s6 = c.pf.s6, s8 = c.pf.s8, s10 = c.pf.s10;
  const float cut2 = c.pf.cut2;
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 *PL = c.w.pos32lo + (size_t)b * N;
  const float4 pi = P[i], li = PL[i];
  const float wi = c.w.w32[ai];
  const int nslot = c.w.n_slots[b];
  const int slot_i = c.w.slot[ai];
  float4 *T = c.w.ptf + (size_t)ai * N;
  float4 *Tda = PGRAD ? c.w.ptf_da + (size_t)ai * N : nullptr;
  // R0 = a1 sqrt(qq) + a2, qq = 3 r4r2_i r4r2_j, R0^6 and R0^8 as
  // double-floats, so that no FP32 rounding of a per-element-pair constant
  // biases every pair of that element pair the same way: from the per-call
  // element-pair table, or (per-atom r4r2 given) per pair from u_i = a1
  // sqrt(3) s_i, v_i = sqrt(3) s_i (FP64 per atom) and s_j = pos32.w + pos32lo.w
  const bool tabled = c.r4r2_in == nullptr;
  // compensated sums of c6 t6 (with (s10/s6) c10 t10 folded in) and of
  // c8 t8; s6 and s8 are applied in FP64 at the end (one FP32 sum of both
  // orders, with s8/s6 as a double-float, measured 4x less accurate)
  const double sref = p.s6 != 0.0 ? p.s6 : 1.0;
  const dfl rho10 = df_from(p.has_s10 ? p.s10 / sref : 0.0);
  const float rho6 = p.s6 != 0.0 ? 1.f : 0.f;
  Acc32 e_acc, e8_acc, gx, gy, gz;
  float pg[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float r2mx = 0.f;  // largest r^2 of this atom's pairs (the ATM's far-atom test)
  for (int s = 0; s < nslot; ++s) {
    if (lane < NFREQ) {  // A' already carries sqrt((3/pi) w): C6 = sum_w A'_i A'_j
      const size_t o = a32_index(b, i, s, lane, N, c.S);
      s_wa[warp][lane] = c.w.A32[o];
      s_wa0[warp][lane] = c.w.A032[o];
    }
    __syncwarp();
    float gacc[NFREQ];
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) gacc[w] = 0.f;
    for (int j = lane; j < n; j += 32) {
      const size_t aj = (size_t)b * N + j;
      const int zj = c.w.z[aj];
      if (j == i || zj == 0 || c.w.slot[aj] != s) continue;
      const float4 pj = P[j];
      const float3 d = pos_diff(pi, li, pj, PL[j]);
      const float dx = d.x, dy = d.y, dz = d.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      const float ir = __frcp_rn(sqrtf(r2));  // correctly rounded: no bias in the ATM records
      const float r = r2 * ir;
      const float *Aj = c.w.A32 + a32_index(b, j, slot_i, 0, N, c.S);
      const float *A0j = c.w.A032 + a32_index(b, j, slot_i, 0, N, c.S);
      float c6 = 0.f, c60 = 0.f;
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) {
        c6 = fmaf(s_wa[warp][w], Aj[(size_t)w * N], c6);
        c60 = fmaf(s_wa0[warp][w], A0j[(size_t)w * N], c60);
      }
      dfl R0d, qqd, R06d, R08d;
      if (tabled) {  // per element pair, from the table r4r2 values
        const float4 A = c.w.pairA[zi * MAX_ELEM_ID + zj], Bq = c.w.pairB[zi * MAX_ELEM_ID + zj];
        R0d = {A.x, A.y};
        qqd = {A.z, A.w};
        R06d = {Bq.x, Bq.y};
        R08d = {Bq.z, Bq.w};
      } else {  // per-atom r4r2 given (rare): FP64 per pair
        const double si = (double)pi.w + (double)li.w, sj = (double)pj.w + (double)PL[j].w;
        const double qq = 3.0 * si * si * sj * sj;
        const double R0 = p.a1 * sqrt(qq) + p.a2;
        const double R02 = R0 * R0, R06 = R02 * R02 * R02;
        R0d = df_from(R0);
        qqd = df_from(qq);
        R06d = df_from(R06);
        R08d = df_from(R06 * R02);
      }
      const float R0 = R0d.hi, sqq = sqrtf(qqd.hi);
      const float lnR0r = logf(R0 * ir) + R0d.lo / R0;
      const float ir2 = __frcp_rn(r2);
      T[j] = make_float4(r2, ir2, expf(c.pf.alp3 * lnR0r), sqrtf(c60) * (ir * ir2));
      r2mx = fmaxf(r2mx, r2);
      if (PGRAD) Tda[j] = make_float4(sqq / R0, 1.0f / R0, lnR0r, 0.f);
      if (r <= cut2) {
        const float r6 = r2 * r2 * r2, R02 = R0 * R0, R06 = R06d.hi;
        const float t6 = 1.0f / ((r6 + R06) + R06d.lo);
        float eterm = rho6 * c6 * t6;
        float dEdr = 6.0f * s6 * c6 * (r6 * ir) * t6 * t6;
        float K = -s6 * t6;
        float dE_dR0 = 6.0f * s6 * c6 * (R06 / R0) * t6 * t6;
        pg[0] -= wi * c6 * t6;
        if (p.has_s8) {
          const float r8 = r6 * r2, R08 = R08d.hi, qq = qqd.hi;
          const float t8 = 1.0f / ((r8 + R08) + R08d.lo);
          const float c8 = fmaf(c6, qqd.hi, c6 * qqd.lo);
          const float e8 = c8 * t8;
          e8_acc.add(e8);
          dEdr += 8.0f * s8 * c8 * (r8 * ir) * t8 * t8;
          K -= s8 * qq * t8;
          dE_dR0 += 8.0f * s8 * c8 * (R08 / R0) * t8 * t8;
          pg[1] -= wi * c8 * t8;
        }
        if (p.has_s10) {  // rare: FP32 powers
          const float qq = sqq * sqq;
          const float r10 = r6 * r2 * r2, R010 = R06 * R02 * R02;
          const float t10 = 1.0f / (r10 + R010);
          const float q2 = qq * qq * (49.0f / 40.0f);
          const float c10 = c6 * q2;
          const float e10 = c10 * t10;
          eterm = fmaf(rho10.hi, e10, fmaf(rho10.lo, e10, eterm));
          dEdr += 10.0f * s10 * c10 * (r10 * ir) * t10 * t10;
          K -= s10 * q2 * t10;
          dE_dR0 += 10.0f * s10 * c10 * (R010 / R0) * t10 * t10;
          pg[2] -= wi * c10 * t10;
        }
        e_acc.add(eterm);
        const float phi = 0.5f * (wi + c.w.w32[aj]);
        dEdr *= phi;
        K *= phi;
        pg[3] += wi * 0.5f * dE_dR0 * sqq;
        pg[4] += wi * 0.5f * dE_dR0;
        const float f = dEdr * ir;
        gx.add(f * dx);
        gy.add(f * dy);
        gz.add(f * dz);
        if (GRAD) {
#pragma unroll
          for (int w = 0; w < NFREQ; ++w) gacc[w] = fmaf(K, Aj[(size_t)w * N], gacc[w]);
        }
      }
    }
    if (GRAD) {
      const float mine = warp_reduce_scatter32(gacc);  // lane w: sum of gacc[w]
      if (lane < NFREQ) c.w.G32[(ai * c.S + s) * NFREQ + lane] = mine;  // dE/dA'_i
    }
    __syncwarp();
  }
  if (GRAD && lane < NFREQ)
    for (int s = nslot; s < c.S; ++s) c.w.G32[(ai * c.S + s) * NFREQ + lane] = 0.f;
  const Acc32 ea = warp_sum_acc(e_acc), ea8 = warp_sum_acc(e8_acc);
  r2mx = warp_maxf(r2mx);
  if (lane == 0 && r2mx > 0.f) atomicMax(&c.w.atm_rowmax[ai], __float_as_uint(r2mx));
  if (PGRAD) {
    float v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = warp_sumf(pg[k]);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 0], 0.5 * (double)v[0]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 1], 0.5 * (double)v[1]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 2], 0.5 * (double)v[2]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 3], (double)v[3]);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 4], (double)v[4]);
    }
  }
  if (GRAD) {
    const Acc32 g0 = warp_sum_acc(gx), g1 = warp_sum_acc(gy), g2 = warp_sum_acc(gz);
    if (lane == 0) {
      c.out.d_gradient[3 * ai] = g0.value();
      c.out.d_gradient[3 * ai + 1] = g1.value();
      c.out.d_gradient[3 * ai + 2] = g2.value();
    }
  }
  if (lane == 0)
    c.out.d_energy[ai] = -0.5 * (sref * ea.value() + (p.has_s8 ? p.s8 * ea8.value() : 0.0));
}

// ---------------------------------------------------------------- launch order

// Structures by decreasing size (n_eff), ties by index: the per-structure
// kernels (EEQ solves, shared-memory ATM) take structure sorder[blockIdx],
// so that the largest structures start first and the small ones fill the
// last wave (longest-processing-time-first).  One CTA, bitonic sort of
// (size, index) keys in shared memory; batches above SORDER_MAX keep index
// order.
__global__ void __launch_bounds__(1024) size_order_kernel(Ctx c) {
  extern __shared__ unsigned long long s_ord[];
  const int B = c.B;
  const int tid = threadIdx.x;
  if (B > SORDER_MAX) {
    for (int t = tid; t < B; t += blockDim.x) c.w.sorder[t] = t;
    return;
  }
  int P = 1;
  while (P < B) P <<= 1;
  for (int t = tid; t < P; t += blockDim.x) {
    const unsigned key = t < B ? 0x7FFFFFFFu - (unsigned)c.w.n_eff[t] : 0xFFFFFFFFu;
    s_ord[t] = ((unsigned long long)key << 32) | (unsigned)t;
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = tid; t < P; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const unsigned long long a = s_ord[t], bb = s_ord[u];
          if ((a > bb) == ((t & k) == 0)) {
            s_ord[t] = bb;
            s_ord[u] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int t = tid; t < B; t += blockDim.x) c.w.sorder[t] = (int)(s_ord[t] & 0xFFFFFFFFu);
}

// ---------------------------------------------------------------- ATM

// 2^x on the special-function unit (ex2.approx.ftz: relative error about
// 2^-22, results below 2^-126 flushed to 0); the ATM damping
// 1 / (1 + 6 * 2^x) needs no more.
__device__ __forceinline__ float sfu_exp2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 1 / x to the SFU's ~1 ulp (x >= 1 here: the ATM damping)
__device__ __forceinline__ float sfu_rcp(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ int tri_u(int j, int k, int n) {  // j < k, upper triangle
  return j * n - j * (j + 1) / 2 + (k - j - 1);
}

// Number of CTAs that share one structure's triples.
__device__ __forceinline__ int atm_ctas(int n) {
  const long long work = (long long)n * n * n / 6;
  const long long per = (long long)ATM_CTA_TRIPLES;
  const int K = (int)((work + per - 1) / per);
  return K < 1 ? 1 : (K > ATM_KMAX ? ATM_KMAX : K);
}

// Accumulation target of the per-pair / per-atom ATM adjoints.  SMEM: the
// upper triangle of the structure in shared memory (flushed to both halves
// of the global pair arrays).  Global: FP32 atomics on the upper half only
// (j < k in every call), mirrored by atm_mirror_kernel afterwards.
template <bool SMEM>
struct AtmAcc {
  float *sS, *sP, *sE;  // shared (SMEM): upper triangle and atoms
  float *gS, *gP;       // global pair blocks [N][N]
  double *gE;           // atom energies
  double escale;        // s9 / 6: energies arrive in units of (triple energy without s9) / 6
  int n, N;
  __device__ __forceinline__ void pair(int j, int k, float S, float P) const {
    if (SMEM) {
      const int t = tri_u(j, k, n);
      atomicAdd(&sS[t], S);
      atomicAdd(&sP[t], P);
    } else {
      atomicAdd(&gS[(size_t)j * N + k], S);
      atomicAdd(&gP[(size_t)j * N + k], P);
    }
  }
  __device__ __forceinline__ void energy(int x, float e) const {
    if (SMEM)
      atomicAdd(&sE[x], e);
    else
      atomicAdd(&gE[x], (double)e * escale);
  }
  // what = 0: dE/d(r^2) of the pair (j, k), 1: its weighted energy, 2:
  // energy of atom j
  __device__ __forceinline__ void one(int j, int k, int what, float v) const {
    if (SMEM) {
      float *dst = what == 2 ? &sE[j] : (what == 1 ? sP : sS) + tri_u(j, k, n);
      atomicAdd(dst, v);
    } else if (what == 2) {
      atomicAdd(&gE[j], (double)v * escale);
    } else {
      atomicAdd((what == 1 ? gP : gS) + (size_t)j * N + k, v);
    }
  }
};

// Warp sums of three values, scattered: lanes 0-7 receive the sum of a,
// lanes 8-15 of b, lanes 16-23 of c (24-31: 0).  Two halving exchanges
// (xor 16, xor 8) and three butterfly steps: 6 shuffles instead of 15.
__device__ __forceinline__ float warp_sum3_scatter(float a, float b, float c) {
  const int lane = threadIdx.x & 31;
  const bool up16 = (lane & 16) != 0, up8 = (lane & 8) != 0;
  float k0 = up16 ? c : a, k1 = up16 ? 0.f : b;
  const float s0 = up16 ? a : c, s1 = up16 ? b : 0.f;
  k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
  k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
  float k = up8 ? k1 : k0;
  k += __shfl_xor_sync(0xffffffffu, up8 ? k0 : k1, 8);
  k += __shfl_xor_sync(0xffffffffu, k, 4);
  k += __shfl_xor_sync(0xffffffffu, k, 2);
  k += __shfl_xor_sync(0xffffffffu, k, 1);
  return k;
}

// ATM triple (i, j, k) of the precision form from its three pair records
// (r^2, 1/r^2, (R0/r)^(alp/3), sqrt(C6(q=0)) / r^3) of the pairs ij, ik,
// jk (x, y, z = their r^2).  With R = r_ij r_ik r_jk, the angular factor is
// w / R^3, w = 1 + 3/8 (x - y + z)(x + y - z)(y + z - x) / R^2, and C9 / R^3
// is the product Q of the records' fourth entries, so the energy without s9
// is eu = Q fd w with fd = 1 / (1 + 6 prod (R0/r)^(alp/3)) (the reference's
// damping, model/d4.py three-body term through damping/atm.py).  dex, dey,
// dez: d eu / d(x, y, z); qwg = Q w fd (1 - fd), for the parameter gradients.
struct AtmTri {
  float eu, dex, dey, dez, qwg;
};

// EZ6: ez arrives multiplied by 6 (a caller that holds the (j, k) record for
// many triples scales it once).
template <bool GRAD, bool EZ6 = false>
__device__ __forceinline__ AtmTri atm_triple(float x, float ix2, float ex, float qx, float y,
                                             float iy2, float ey, float qy, float z, float iz2,
                                             float ez, float qz, float alp3h) {
  AtmTri r;
  const float ir2 = ix2 * (iy2 * iz2);
  const float h = 0.375f * ir2;
  const float u = x - y;
  const float A = u + z, Bv = (x + y) - z, Cv = z - u;
  const float AB = A * Bv;
  const float w = fmaf(AB * Cv, h, 1.0f);
  // (rounding 1 + 6 prod drops its small values at distant triples alike;
  // measured on 16000 atoms the three-body energy stays within 1e-8 Eh of
  // the FP64 reference, and a Newton-corrected fd costs 3 % of the kernel)
  const float fd = EZ6 ? sfu_rcp(fmaf(ex, ey * ez, 1.0f))
                      : sfu_rcp(fmaf(6.0f, ex * (ey * ez), 1.0f));
  const float Q = qx * (qy * qz);
  const float cq = Q * fd;
  r.eu = cq * w;
  if (GRAD) {
    // U = 3/8 C9 fd / R^5, V = C9 / (2 R^3) (fd (2 - 5 w) + w alp/3 fd (1 - fd))
    //   = C9 fd / R^3 (1 + w (alp/6 (1 - fd) - 5/2))
    const float U = cq * h;
    const float V = cq * fmaf(w, fmaf(-alp3h, fd, alp3h - 2.5f), 1.0f);
    const float AC = A * Cv, BC = Bv * Cv;
    const float Sg = AB + AC + BC;
    r.dex = fmaf(U, fmaf(-2.0f, AB, Sg), V * ix2);
    r.dey = fmaf(U, fmaf(-2.0f, BC, Sg), V * iy2);
    r.dez = fmaf(U, fmaf(-2.0f, AC, Sg), V * iz2);
    r.qwg = Q * w * fmaf(-fd, fd, fd);
  } else {
    r.dex = r.dey = r.dez = r.qwg = 0.f;
  }
  return r;
}

// Constant inputs of the ATM triple loop of one structure.
struct AtmIn {
  const int *Zb;
  bool gaps;  // padding atoms below the last real one
  const float4 *T, *Tda;
  const float *W;
  float cut2, alp3, s9, s9m;
  bool weighted;
  int N;
};

// Parameter-gradient partial sums of one warp.
struct AtmPg {
  float s9 = 0.f, alp = 0.f, a1 = 0.f, a2 = 0.f;
};

// One task of the ATM loop: the pair (j, k = kc + lane) held by the lanes,
// the third atom i < j running from i0 in steps of istep.  Triple energy
// without s9 (applied at the flush, SMEM) or with it (global).
template <bool SMEM, bool GRAD, bool PGRAD>
__device__ __forceinline__ void atm_task(const AtmIn &in, const AtmAcc<SMEM> &acc, int n, int j,
                                         int kc, int i0, int istep, AtmPg &pg) {
  const int lane = threadIdx.x & 31;
  const int N = in.N;
  const float cut2 = in.cut2, alp3 = in.alp3, s9 = in.s9, s9m = in.s9m;
  const float4 *T = in.T;
  const float *W = in.W;
  const int k = kc + lane;
  const bool kok = k < n && in.Zb[k] != 0;
  const float4 pjk = kok ? T[(size_t)j * N + k] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float zjk = pjk.x, izjk = pjk.y, ejk6 = 6.0f * pjk.z, qjk = pjk.w;
  const float alp3h = 0.5f * alp3;
  const bool mjk = kok && zjk <= cut2;
  float4 dajk = make_float4(0.f, 0.f, 0.f, 0.f);
  if (PGRAD && kok) dajk = in.Tda[(size_t)j * N + k];
  const float wj = W[j];
  const float wk = kok ? W[k] : 0.f;
  float Sjk = 0.f, Pjk = 0.f, Ej = 0.f, Ek = 0.f;
  float kept = 0.f;  // pending (i, j) / E_i value of this lane
  int kept_i = -1, nred = 0;
  const size_t step = (size_t)istep * N;
  const float4 *Tij = T + (size_t)i0 * N + j;
  const float4 *Tik = T + (size_t)i0 * N + (kok ? k : j);
  for (int i = i0; i < j; i += istep, Tij += step, Tik += step) {
    if (in.gaps && in.Zb[i] == 0) continue;
    const float4 pij = *Tij;
    float sij = 0.f, pe = 0.f, ei = 0.f;
    if (kok) {
      const float4 pik = *Tik;
      const bool mij = pij.x <= cut2, mik = pik.x <= cut2;
      if ((int)mij + (int)mik + (int)mjk >= 2) {
        const AtmTri tr = atm_triple<GRAD, true>(pij.x, pij.y, pij.z, pij.w, pik.x, pik.y,
                                                 pik.z, pik.w, zjk, izjk, ejk6, qjk, alp3h);
        const float eu = tr.eu;  // triple energy without s9
        const float e = s9m * eu;
        float wgt;
        // atom energies in units of e/6 (exact multiples; s9/6 is applied in
        // FP64 when they leave the kernel, so no rounded 1/3 biases them)
        if (mij & mik & mjk) {
          const float e2 = eu + eu;
          ei = e2;
          Ej += e2;
          Ek += e2;
          wgt = ((in.weighted ? W[i] : 1.f) + wj + wk) * (1.0f / 3.0f);
        } else {
          const float fij = mij, fik = mik, fjk = mjk;
          const float mi = fjk * (fij + fik), mj = fik * (fij + fjk), mk = fij * (fik + fjk);
          ei = eu * mi;
          Ej += eu * mj;
          Ek += eu * mk;
          wgt = ((in.weighted ? W[i] : 1.f) * mi + wj * mj + wk * mk) * (1.0f / 6.0f);
        }
        if (GRAD) {
          const float ws = wgt * s9m;
          sij = ws * tr.dex;
          Sjk = fmaf(ws, tr.dez, Sjk);
          const float we = wgt * e;
          pe = we;
          Pjk += we;
          acc.pair(i, k, ws * tr.dey, we);
          if (PGRAD) {
            const float4 daij = in.Tda[(size_t)i * N + j];
            const float4 daik = in.Tda[(size_t)i * N + k];
            const float lsum = daij.z + daik.z + dajk.z;
            // d fd / d(alp/3 sum log(R0/r)) = -fd (1 - fd)
            pg.s9 += wgt * eu;
            pg.alp -= wgt * s9 * tr.qwg * lsum * (1.0f / 3.0f);
            const float dfa = -wgt * s9 * tr.qwg * alp3;
            pg.a1 += dfa * (daij.x + daik.x + dajk.x);
            pg.a2 += dfa * (daij.y + daik.y + dajk.y);
          }
        }
      }
    }
    // (i, j) and E_i: the three warp sums in one reduce-scatter (lanes
    // 0-7: dE/d(r_ij^2), 8-15: weighted energy of (i, j), 16-23: E_i); lane
    // u % 8 of each group keeps the value of the u-th reduction, and the 24
    // kept values are accumulated together every 8 reductions
    if (GRAD) {
      const float v = warp_sum3_scatter(sij, pe, ei);
      if ((lane & 7) == (nred & 7)) {
        kept = v;
        kept_i = i;
      }
      if ((++nred & 7) == 0) {
        if (lane < 24 && kept_i >= 0 && kept != 0.f) acc.one(kept_i, j, lane >> 3, kept);
        kept_i = -1;
      }
    } else {
      ei = warp_sumf(ei);
      if (lane == 0 && ei != 0.f) acc.energy(i, ei);
    }
  }
  if (GRAD && lane < 24 && kept_i >= 0 && kept != 0.f) acc.one(kept_i, j, lane >> 3, kept);
  if (GRAD && kok && (Sjk != 0.f || Pjk != 0.f)) acc.pair(j, k, Sjk, Pjk);
  const float ej = warp_sumf(Ej);
  if (lane == 0 && ej != 0.f) acc.energy(j, ej);
  if (kok && Ek != 0.f) acc.energy(k, Ek);
}

// Whether the ATM of structure b runs over neighbour triples (centre-atom
// enumeration, atm_sparse_kernel) instead of all triples i < j < k: when
// every centre's neighbour list fits the kernel's shared memory and the
// centre-pair visits, sum_j deg_j (deg_j - 1) / 2, are fewer than half the
// n (n - 1) (n - 2) / 6 triples.  Counts come from atm_nbr_kernel; only
// structures of the global-accumulation path (N > 234) have them.
__device__ __forceinline__ bool atm_sparse_mode(const Ctx &c, int b, int n) {
  if (c.w.atm_cnt == nullptr) return false;
  const unsigned long long visits = c.w.atm_cnt[2 * b], dmax = c.w.atm_cnt[2 * b + 1];
  const unsigned long long nn = (unsigned long long)n;
  const unsigned long long all = nn * (nn - 1) * (nn - 2) / 6;
  return dmax <= (unsigned long long)ATM_SPARSE_DMAX && 2 * visits < all;
}

// CTAs per structure of the global-accumulation ATM (large structures):
// about ATM_BIG_TRIPLES triples each, at most ATM_BIG_KMAX.
constexpr long long ATM_BIG_TRIPLES = 250000;
constexpr int ATM_BIG_KMAX = 1024;
__host__ __device__ inline int atm_ctas_big(int n) {
  const long long work = (long long)n * n * n / 6;
  const long long K = (work + ATM_BIG_TRIPLES - 1) / ATM_BIG_TRIPLES;
  return K < 1 ? 1 : (K > ATM_BIG_KMAX ? ATM_BIG_KMAX : (int)K);
}

// ATM energy and adjoint over triples i < j < k of one structure.  A warp
// takes a task (j, 32 consecutive k > j) and loops over i: lanes hold the
// (j, k) pair record in registers and read the (i, j) (broadcast) and (i, k)
// (coalesced 128-bit) records.  A pair record holds r^2, 1/r^2,
// (R0/r)^(alp/3) and sqrt(C6(q=0)) / r^3, so the damping factor and
// C9 / (r_ij r_ik r_jk)^3 are two products each (atm_triple).
//   SMEM (n <= 234): K <= 8 CTAs share a structure, interleaving i; per-pair
//     dE/d(r^2) and mask-weighted triple energies accumulate in shared memory
//     without the s9 factor, applied when a CTA flushes them (FP32 global
//     atomics, both triangle halves).
//   Global (large structures): up to 1024 CTAs per structure, the tasks
//     (j, k-chunk) dealt round-robin over all their warps, i running over
//     all i < j; FP32 global atomics on the upper half.
template <bool SMEM, bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(PGRAD ? ATM_THREADS_PGRAD : ATM_THREADS)
    atm_mixed_kernel(Ctx c) {
  extern __shared__ float s_acc[];
  const int b = SMEM ? c.w.sorder[blockIdx.y] : (int)blockIdx.y;
  const int cta = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  if (n < 3) return;
  const int K = SMEM ? atm_ctas(n) : atm_ctas_big(n);
  if (cta >= K) return;
  if (!SMEM && atm_sparse_mode(c, b, n)) return;  // the neighbour-triple kernel takes it
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int P = n * (n - 1) / 2;
  AtmAcc<SMEM> acc;
  acc.n = n;
  acc.N = N;
  acc.sS = s_acc;
  acc.sP = s_acc + P;
  acc.sE = s_acc + 2 * P;
  acc.gS = GRAD ? c.w.prS32 + (size_t)b * N * N : nullptr;
  acc.gP = GRAD ? c.w.prP32 + (size_t)b * N * N : nullptr;
  acc.gE = c.w.e3 + (size_t)b * N;
  acc.escale = c.par.s9 / 6.0;
  if (SMEM) {
    for (int t = threadIdx.x; t < 2 * P + n; t += blockDim.x) s_acc[t] = 0.f;
    __syncthreads();
  }
  AtmIn in;
  in.Zb = c.w.z + (size_t)b * N;
  in.gaps = c.w.n_real[b] != n;
  in.T = c.w.ptf + (size_t)b * N * N;
  in.Tda = PGRAD ? c.w.ptf_da + (size_t)b * N * N : nullptr;
  in.W = c.w.w32 + (size_t)b * N;
  in.cut2 = c.pf.cut3 * c.pf.cut3;
  in.alp3 = c.pf.alp3;
  in.s9 = c.pf.s9;
  in.s9m = SMEM ? 1.f : c.pf.s9;  // SMEM: s9 is applied at the flush
  in.weighted = c.weights != nullptr;
  in.N = N;
  AtmPg pg;
  if (SMEM) {
    // tasks (j, chunk of 32 k > j) in j-major order, dealt round-robin to
    // the warps; a warp walks straight to its next task (no division)
    int j = 1, jbase = 0, nch = (n - 2 + 31) >> 5;  // row j: tasks jbase .. jbase + nch
    for (int t = warp;; t += nwarps) {
      while (j < n - 1 && t >= jbase + nch) {
        jbase += nch;
        ++j;
        nch = (n - 1 - j + 31) >> 5;
      }
      if (j >= n - 1) break;
      if (in.gaps && in.Zb[j] == 0) continue;
      atm_task<SMEM, GRAD, PGRAD>(in, acc, n, j, j + 1 + 32 * (t - jbase), cta, K, pg);
    }
  } else {
    const int NC = (n + 31) / 32;  // chunk slots per row j
    const long long slots = (long long)n * NC;
    const int G = K * nwarps;
    for (long long sl = (long long)cta * nwarps + warp; sl < slots; sl += G) {
      const int j = (int)(sl / NC), ch = (int)(sl % NC);
      const int kc = j + 1 + 32 * ch;
      if (j < 1 || j >= n - 1 || kc >= n || in.Zb[j] == 0) continue;
      atm_task<SMEM, GRAD, PGRAD>(in, acc, n, j, kc, 0, 1, pg);
    }
  }
  if (PGRAD) {
    pg.s9 = warp_sumf(pg.s9);
    pg.alp = warp_sumf(pg.alp);
    pg.a1 = warp_sumf(pg.a1);
    pg.a2 = warp_sumf(pg.a2);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 3], (double)pg.a1);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 4], (double)pg.a2);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 5], (double)pg.s9);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 6], (double)pg.alp);
    }
  }
  if (SMEM) {
    const float s9 = c.pf.s9;
    __syncthreads();
    for (int j = warp; j < n; j += nwarps) {
      for (int k = j + 1 + lane; k < n; k += 32) {
        const int t = tri_u(j, k, n);
        if (GRAD) {
          const float sv = acc.sS[t] * s9, pv = acc.sP[t] * s9;
          if (sv != 0.f || pv != 0.f) {
            const size_t base = (size_t)b * N * N;
            atomicAdd(&c.w.prS32[base + (size_t)j * N + k], sv);
            atomicAdd(&c.w.prP32[base + (size_t)j * N + k], pv);
            atomicAdd(&c.w.prS32[base + (size_t)k * N + j], sv);
            atomicAdd(&c.w.prP32[base + (size_t)k * N + j], pv);
          }
        }
      }
    }
    for (int x = threadIdx.x; x < n; x += blockDim.x) {
      const float ev = acc.sE[x];
      if (ev != 0.f) atomicAdd(&c.w.e3[(size_t)b * N + x], (double)ev * acc.escale);
    }
  }
}

// ---------------------------------------------------------------- ATM, register-tiled

// Shared-memory ATM (n <= 234) for structures with no padding below the
// last real atom and unit atom weights.  A triple whose three pairs lie
// inside the three-body cutoff has attribution weight 1, and the atom
// energies follow from the pair sums, E_x = sum_y P(x, y) (each triple
// reaches x through two pairs; the same total as the per-triple attribution
// eu / 3 per atom).  Triples with a pair beyond the cutoff are only possible
// where one of the three atoms is "far" (its largest pair r^2, recorded by
// the pair kernels, exceeds the cutoff): steps and tasks that touch a far
// atom run the masked variant, which weights each triple by
// (f_ij f_ik + f_ij f_jk + f_ik f_jk) / 3 (f: pair inside the cutoff; 1, 1/3
// or 0) and corrects the atom energies of the 1/3 triples, whose pair sums
// alone do not give the reference attribution (in these units the atom of
// both inside pairs gets 0, the other two eu each, while the pair sums give
// each 2 eu / 3): -2 eu / 3 to the common atom and +eu / 3 to the other two,
// accumulated beside the row sums.
//
// A warp task is a tile of AT_C = 8 consecutive middle atoms j (j0 .. j0+7)
// and a chunk of 8 outer atoms k > j.  Lane (q, l) = (lane / 8, lane % 8)
// takes k = kc + l and keeps the eight (j, k) pair records and their
// dE/dr^2 and energy sums in registers; the four lane groups q walk the
// inner atoms i < j in step (group q takes every fourth i of the CTA's
// sequence).  Per i a lane reads the (i, k) record and the eight (i, j)
// records (one row segment per group), evaluates eight triples, adds its
// (i, k) sums to shared memory once, and the group reduce-scatters its
// sixteen (i, j) sums over its eight lanes.  8 x 8 tiles keep the triples
// evaluated outside i < j < k at ~22 % for sizes 8..200 (8 x 32: ~50 %).
// The triple arithmetic is that of atm_task with unit atom weights.
// Structures outside these conditions run atm_task in the same kernel.
constexpr int AT_C = 8;             // middle atoms per task (and outer atoms per chunk)
constexpr int AT_THREADS = 512;     // 16 warps at 128 registers, no spills (measured on
                                    // batch512: 768 threads at 80 registers spill and run
                                    // 13 % slower, 640 at 96 registers 10 % slower)
constexpr int AT_TASKS_MAX = 900;   // tiles x chunks for n <= 237 (30 x 30)
constexpr int AT_FAR_WORDS = 8;     // far-atom bits for n <= 256
__host__ __device__ inline size_t atm_tiled_smem_bytes(int N) {
  return atm_smem_bytes(N) + sizeof(int) * AT_TASKS_MAX;
}

// tri_u(i, x, n) = tri_row(i, n) + x for x > i
__device__ __forceinline__ int tri_row(int i, int n) { return i * n - i * (i + 1) / 2 - i - 1; }

// Halving exchanges over the lane bits H, H/2, ... (STEPS of them): v[p]
// for p < NV >> STEPS ends as the sum over the 2^STEPS lanes that differ in
// those bits of the value with index p + (NV/2) bit(H) + (NV/4) bit(H/2) + ...
template <int NV, int H, int STEPS>
__device__ __forceinline__ void lane_halving(float (&v)[NV]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < STEPS; ++s) {
    const int m = NV >> (s + 1), h = H >> s;
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int q = 0; q < m; ++q) {
      const float keep = up ? v[q + m] : v[q];
      const float send = up ? v[q] : v[q + m];
      v[q] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
}

// Per-structure state of the tiled ATM: shared accumulators, the far-atom
// bit set, the cutoff and the damping exponent.
struct AtTile {
  const float4 *__restrict__ T;
  float *sS, *sP, *sE;
  const unsigned *far;  // bit x: atom x has a pair beyond the three-body cutoff
  float cut2, alp3h;
  int n, N;
  __device__ __forceinline__ bool is_far(int x) const {
    return x < n && ((far[x >> 5] >> (x & 31)) & 1u) != 0u;
  }
};

// One step of a tile task: inner atom i of this lane's group.  GUARD: some
// (i, j) of the step are not pairs (i >= j, j beyond the structure, i
// beyond the task's range).  MASK: a far atom takes part, so each triple
// carries its cutoff weight and the 1/3 triples their energy corrections.
template <bool GRAD, bool GUARD, bool MASK>
__device__ __forceinline__ void atm_tile_step(const AtTile &a, int j0, int jend, int k, bool kok,
                                              int i, const float (&zjk)[AT_C],
                                              const float (&izjk)[AT_C],
                                              const float (&ejk)[AT_C],
                                              const float (&qjk)[AT_C], float (&Sjk)[AT_C],
                                              float (&Pjk)[AT_C]) {
  const int l = threadIdx.x & 7;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const bool iok = !GUARD || i < jend - 1;
  const float4 *Ti = a.T + (size_t)(iok ? i : 0) * a.N;
  const bool lk = iok && kok && k > i;
  const float4 pik = lk ? Ti[k] : zero4;
  const bool fik = !MASK || pik.x <= a.cut2;
  float Sik = 0.f, Pik = 0.f;
  constexpr int NV = GRAD ? 2 * AT_C : AT_C;
  float v[NV];  // (i, j) sums: dE/dr^2 (GRAD) then energies
#pragma unroll
  for (int t = 0; t < AT_C; ++t) {
    float4 pij;
    if (GUARD) {
      const int jt = j0 + t;
      const bool ok = iok && jt > i && jt < jend;
      pij = ok ? Ti[ok ? jt : 0] : zero4;
    } else {
      pij = Ti[j0 + t];
    }
    bool fij = true, fjk = true;
    float qij = pij.w;
    if (MASK) {  // cutoff weight 1, 1/3 or 0, folded into C9 / R^3
      fij = pij.x <= a.cut2;
      fjk = zjk[t] <= a.cut2;
      const int m = (int)fij + (int)fik + (int)fjk;
      qij *= m == 3 ? 1.f : (m == 2 ? (1.0f / 3.0f) : 0.f);
    }
    const AtmTri tr = atm_triple<GRAD, true>(pij.x, pij.y, pij.z, qij, pik.x, pik.y, pik.z,
                                             pik.w, zjk[t], izjk[t], ejk[t], qjk[t], a.alp3h);
    if (MASK && !(fij & fik & fjk) && tr.eu != 0.f) {
      // a 1/3 triple: -2 eu_w to the atom of both inside pairs, +eu_w to the others
      atomicAdd(&a.sE[i], fjk ? tr.eu : -2.f * tr.eu);
      atomicAdd(&a.sE[j0 + t], fik ? tr.eu : -2.f * tr.eu);
      atomicAdd(&a.sE[k], fij ? tr.eu : -2.f * tr.eu);
    }
    Pik += tr.eu;
    Pjk[t] += tr.eu;
    if (GRAD) {
      Sik += tr.dey;
      Sjk[t] += tr.dez;
      v[t] = tr.dex;
      v[AT_C + t] = tr.eu;
    } else {
      v[t] = tr.eu;
    }
  }
  const int rb = tri_row(i, a.n);
  if (lk) {
    if (GRAD) atomicAdd(&a.sS[rb + k], Sik);
    atomicAdd(&a.sP[rb + k], Pik);
  }
  // group sums over the eight lanes: lane l keeps values NV/8 l .. NV/8 l + NV/8 - 1
  lane_halving<NV, 4, 3>(v);
#pragma unroll
  for (int p = 0; p < NV / 8; ++p) {
    const int idx = (NV / 8) * l + p;
    const int jt = j0 + idx % AT_C;
    if (!GUARD || (iok && jt > i && jt < jend && v[p] != 0.f))
      atomicAdd(&((GRAD && idx < AT_C) ? a.sS : a.sP)[rb + jt], v[p]);
  }
}

// The steps of a task over inner atoms i, i running from ib in steps of st4
// while i < ilim: the masked step where a far atom takes part
// (warp-uniform: any of the four groups' i), the plain one elsewhere.
template <bool GRAD, bool GUARD>
__device__ __forceinline__ int atm_tile_steps(const AtTile &a, bool any_far, bool task_far,
                                              int ib, int ilim, int st4, int istep, int j0,
                                              int jend, int k, bool kok,
                                              const float (&zjk)[AT_C],
                                              const float (&izjk)[AT_C],
                                              const float (&ejk)[AT_C],
                                              const float (&qjk)[AT_C], float (&Sjk)[AT_C],
                                              float (&Pjk)[AT_C]) {
  const int i_off = ((threadIdx.x & 31) >> 3) * istep;
  for (; ib < ilim; ib += st4) {
    const int i = ib + i_off;
    if (any_far && (task_far || __any_sync(0xffffffffu, a.is_far(i))))
      atm_tile_step<GRAD, GUARD, true>(a, j0, jend, k, kok, i, zjk, izjk, ejk, qjk, Sjk, Pjk);
    else
      atm_tile_step<GRAD, GUARD, false>(a, j0, jend, k, kok, i, zjk, izjk, ejk, qjk, Sjk, Pjk);
  }
  return ib;
}

template <bool GRAD>
__device__ __forceinline__ void atm_tile_task(const AtTile &a, bool any_far, int j0, int kc,
                                              int i0, int istep) {
  const int lane = threadIdx.x & 31;
  const int q = lane >> 3;
  const int n = a.n;
  const int k = kc + (lane & 7);
  const bool kok = k < n;
  float zjk[AT_C], izjk[AT_C], ejk[AT_C], qjk[AT_C], Sjk[AT_C], Pjk[AT_C];
#pragma unroll
  for (int t = 0; t < AT_C; ++t) {
    const int jt = j0 + t;
    const bool ok = kok && jt < k;  // then also jt <= n - 2
    const float4 r = ok ? a.T[(size_t)jt * a.N + k] : make_float4(0.f, 0.f, 0.f, 0.f);
    zjk[t] = r.x;
    izjk[t] = r.y;
    ejk[t] = 6.0f * r.z;  // prescaled for atm_triple<., true>
    qjk[t] = r.w;  // 0 also zeroes every product of a (j, k) that is not a pair
    Sjk[t] = 0.f;
    Pjk[t] = 0.f;
  }
  const int jend = min(j0 + AT_C, n - 1);  // middle atoms j0 .. jend - 1
  // a far middle or outer atom makes every step of the task a masked one
  bool task_far = false;
  if (any_far) {
    bool mine = a.is_far(k);
#pragma unroll
    for (int t = 0; t < AT_C; ++t) mine |= a.is_far(j0 + t);
    task_far = __any_sync(0xffffffffu, mine);
  }
  // group q takes i = i0 + (4 s + q) istep, s = 0, 1, ...
  const int st4 = 4 * istep;
  int ib = i0;  // i of group 0 in this step
  if (j0 + AT_C <= n - 1) {
    // plain steps while all four groups' i are below j0: ib + 3 istep < j0
    const int ilim = j0 - 3 * istep;
    ib = atm_tile_steps<GRAD, false>(a, any_far, task_far, ib, ilim, st4, istep, j0, jend, k,
                                     kok, zjk, izjk, ejk, qjk, Sjk, Pjk);
  }
  atm_tile_steps<GRAD, true>(a, any_far, task_far, ib, jend - 1, st4, istep, j0, jend, k, kok,
                             zjk, izjk, ejk, qjk, Sjk, Pjk);
  // (j, k) sums of the four groups: group q keeps values NV/4 q .. NV/4 q + NV/4 - 1
  constexpr int NV = GRAD ? 2 * AT_C : AT_C;
  float v[NV];
#pragma unroll
  for (int t = 0; t < AT_C; ++t) {
    if (GRAD) {
      v[t] = Sjk[t];
      v[AT_C + t] = Pjk[t];
    } else {
      v[t] = Pjk[t];
    }
  }
  lane_halving<NV, 16, 2>(v);
#pragma unroll
  for (int p = 0; p < NV / 4; ++p) {
    const int idx = (NV / 4) * q + p;
    const int jt = j0 + idx % AT_C;
    if (kok && jt < k && v[p] != 0.f)
      atomicAdd(&((GRAD && idx < AT_C) ? a.sS : a.sP)[tri_u(jt, k, n)], v[p]);
  }
}

template <bool GRAD>
__global__ void __launch_bounds__(AT_THREADS, 1) atm_tiled_kernel(Ctx c) {
  extern __shared__ float s_acc[];
  __shared__ int s_next, s_ntask, s_any_far;
  __shared__ unsigned s_far[AT_FAR_WORDS];
  const int b = c.w.sorder[blockIdx.y];
  const int cta = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  if (n < 3) return;
  const int K = atm_tiled_ctas(n, c.B);
  if (cta >= K) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int P = n * (n - 1) / 2;
  float *sS = s_acc, *sP = s_acc + P, *sE = s_acc + 2 * P;
  int *s_task = reinterpret_cast<int *>(s_acc + 2 * P + n);
  const float cut2 = c.pf.cut3 * c.pf.cut3;
  const bool tiled = c.w.n_real[b] == n;
  for (int t = threadIdx.x; t < 2 * P + n; t += blockDim.x) s_acc[t] = 0.f;
  if (threadIdx.x == 0) s_any_far = 0;
  if (warp < AT_FAR_WORDS) {  // far atoms: largest pair r^2 beyond the cutoff
    const int x = 32 * warp + lane;
    const bool far = x < n && __uint_as_float(c.w.atm_rowmax[(size_t)b * N + x]) > cut2;
    const unsigned m = __ballot_sync(0xffffffffu, far);
    if (lane == 0) s_far[warp] = m;
  }
  const int NT = (n - 2 + AT_C - 1) / AT_C;  // tiles of middle atoms 1 .. n - 2
  if (tiled && threadIdx.x < NT) {
    // task table: tiles from the last (longest i range) to the first, the
    // chunks of eight outer atoms of each in order
    auto nch = [&](int ti) { return (n - 1 - (1 + AT_C * ti) + AT_C - 1) / AT_C; };
    const int ti = threadIdx.x;
    int off = 0;
    for (int u = NT - 1; u > ti; --u) off += nch(u);
    for (int ch = 0; ch < nch(ti); ++ch) s_task[off + ch] = (ti << 8) | ch;
    if (ti == 0) {
      s_ntask = off + nch(0);
      s_next = nwarps;
    }
  }
  __syncthreads();
  if (threadIdx.x < AT_FAR_WORDS && s_far[threadIdx.x] != 0u) s_any_far = 1;
  __syncthreads();
  const float4 *T = c.w.ptf + (size_t)b * N * N;
  if (tiled) {
    AtTile a;
    a.T = T;
    a.sS = sS;
    a.sP = sP;
    a.sE = sE;
    a.far = s_far;
    a.cut2 = cut2;
    a.alp3h = 0.5f * c.pf.alp3;
    a.n = n;
    a.N = N;
    const bool any_far = s_any_far != 0;
    const int ntask = s_ntask;
    for (int task = warp; task < ntask;) {
      const int e = s_task[task];
      const int j0 = 1 + AT_C * (e >> 8);
      atm_tile_task<GRAD>(a, any_far, j0, j0 + 1 + AT_C * (e & 255), cta, K);
      int nx = 0;
      if (lane == 0) nx = atomicAdd(&s_next, 1);
      task = __shfl_sync(0xffffffffu, nx, 0);
    }
  } else {
    AtmAcc<true> acc;
    acc.n = n;
    acc.N = N;
    acc.sS = sS;
    acc.sP = sP;
    acc.sE = sE;
    acc.gS = acc.gP = nullptr;
    acc.gE = nullptr;
    acc.escale = c.par.s9 / 6.0;
    AtmIn in;
    in.Zb = c.w.z + (size_t)b * N;
    in.gaps = c.w.n_real[b] != n;
    in.T = T;
    in.Tda = nullptr;
    in.W = c.w.w32 + (size_t)b * N;
    in.cut2 = cut2;
    in.alp3 = c.pf.alp3;
    in.s9 = c.pf.s9;
    in.s9m = 1.f;
    in.weighted = false;
    in.N = N;
    AtmPg pg;
    int j = 1, jbase = 0, nch = (n - 2 + 31) >> 5;
    for (int t = warp;; t += nwarps) {
      while (j < n - 1 && t >= jbase + nch) {
        jbase += nch;
        ++j;
        nch = (n - 1 - j + 31) >> 5;
      }
      if (j >= n - 1) break;
      if (in.gaps && in.Zb[j] == 0) continue;
      atm_task<true, GRAD, false>(in, acc, n, j, j + 1 + 32 * (t - jbase), cta, K, pg);
    }
  }
  __syncthreads();
  // Flush: the upper half of the pair sums row by row (lanes over k > j),
  // then the lower half row by row (lanes over j < k), both coalesced in
  // global memory; a structure with one CTA stores, several CTAs add.  The
  // tiled path's atom energies are the row sums of P: the part over y > x
  // in the first pass (parked in sE), the part over y < x in the second.
  const float s9 = c.pf.s9;
  float *gS = GRAD ? c.w.prS32 + (size_t)b * N * N : nullptr;
  float *gP = GRAD ? c.w.prP32 + (size_t)b * N * N : nullptr;
  const bool solo = K == 1;
  const double escale = c.par.s9 / 6.0;
  for (int j = warp; j < n; j += nwarps) {
    const int rb = tri_row(j, n);
    float er = 0.f;
    for (int k = j + 1 + lane; k < n; k += 32) {
      const float pv = sP[rb + k];
      er += pv;
      if (GRAD) {
        const float sv = sS[rb + k];
        float *ds = gS + (size_t)j * N + k, *dp = gP + (size_t)j * N + k;
        if (solo) {
          *ds = sv * s9;
          *dp = pv * s9;
        } else if (sv != 0.f || pv != 0.f) {
          atomicAdd(ds, sv * s9);
          atomicAdd(dp, pv * s9);
        }
      }
    }
    if (tiled) {
      er = warp_sumf(er);
      if (lane == 0) sE[j] += er;  // beside the 1/3-triple corrections
    }
  }
  __syncthreads();
  for (int k = warp; k < n; k += nwarps) {
    float ec = 0.f;
    for (int j = lane; j < k; j += 32) {
      const int t = tri_u(j, k, n);
      const float pv = sP[t];
      ec += pv;
      if (GRAD) {
        const float sv = sS[t];
        float *ds = gS + (size_t)k * N + j, *dp = gP + (size_t)k * N + j;
        if (solo) {
          *ds = sv * s9;
          *dp = pv * s9;
        } else if (sv != 0.f || pv != 0.f) {
          atomicAdd(ds, sv * s9);
          atomicAdd(dp, pv * s9);
        }
      }
    }
    if (tiled) {
      ec = warp_sumf(ec);
      const float ev = ec + sE[k];  // E_k = sum_y P(k, y)
      if (lane == 0 && ev != 0.f) atomicAdd(&c.w.e3[(size_t)b * N + k], (double)ev * escale);
    }
  }
  if (!tiled)
    for (int x = threadIdx.x; x < n; x += blockDim.x) {
      const float ev = sE[x];
      if (ev != 0.f) atomicAdd(&c.w.e3[(size_t)b * N + x], (double)ev * escale);
    }
}

// Lower half of the ATM pair accumulators from the upper half (global
// accumulation), 32 x 32 tiles through shared memory.
__global__ void atm_mirror_kernel(Ctx c) {
  __shared__ float sS[32][33], sP[32][33];
  const int b = blockIdx.z;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  const int ti = blockIdx.y, tj = blockIdx.x;  // source tile (rows ti, columns tj), tj >= ti
  if (tj < ti || ti * 32 >= n || tj * 32 >= n) return;
  float *S = c.w.prS32 + (size_t)b * N * N;
  float *P = c.w.prP32 + (size_t)b * N * N;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += blockDim.x >> 5) {
    const int i = ti * 32 + r, j = tj * 32 + tx;
    const bool ok = i < n && j < n && j > i;
    sS[r][tx] = ok ? S[(size_t)i * N + j] : 0.f;
    sP[r][tx] = ok ? P[(size_t)i * N + j] : 0.f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += blockDim.x >> 5) {
    const int i = tj * 32 + r, j = ti * 32 + tx;  // destination (i > j)
    if (i < n && j < n && i > j) {
      S[(size_t)i * N + j] = sS[tx][r];
      P[(size_t)i * N + j] = sP[tx][r];
    }
  }
}

// ---------------------------------------------------------------- ATM over neighbour triples

// Neighbour lists of the ATM (global-accumulation structures): for every
// real atom j the real atoms k != j with r_jk <= disp3, ascending, taken
// from the r^2 of the pair records; the per-structure counts decide between
// the two ATM variants (atm_sparse_mode).  One warp per atom, ballot
// compaction.
__global__ void __launch_bounds__(256) atm_nbr_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + warp;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  if (j >= N) return;
  const size_t bN = (size_t)b * N;
  if (j >= n || c.w.z[bN + j] == 0) {
    if (lane == 0) c.w.nbr_deg[bN + j] = 0;
    return;
  }
  const float cut2 = c.pf.cut3 * c.pf.cut3;
  const float4 *T = c.w.ptf + (bN + j) * N;
  int *L = c.w.nbr + (bN + j) * N;
  const int *Z = c.w.z + bN;
  int base = 0;
  for (int k0 = 0; k0 < n; k0 += 32) {
    const int k = k0 + lane;
    bool ok = false;
    if (k < n && k != j && Z[k] != 0) ok = T[k].x <= cut2;
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok) L[base + __popc(m & ((1u << lane) - 1u))] = k;
    base += __popc(m);
  }
  if (lane == 0) {
    c.w.nbr_deg[bN + j] = base;
    const unsigned long long d = (unsigned long long)base;
    atomicAdd(&c.w.atm_cnt[2 * b], d * (d > 0 ? d - 1 : 0) / 2);
    atomicMax(&c.w.atm_cnt[2 * b + 1], d);
  }
}

// Centre order of the neighbour-triple ATM: the real atoms of a structure
// sorted by the Z-order (Morton) code of their positions on a 1024^3 grid
// over the structure's bounding box, so that CTAs running at the same time
// work on nearby centres and share their neighbourhoods' pair records in L2.
// One CTA per structure: bitonic sort of (code << 32 | atom) keys in shared
// memory (padding last); n <= ATM_ORDER_MAX, else index order.
__device__ __forceinline__ unsigned spread_bits10(unsigned v) {  // 10 bits -> every third bit
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void __launch_bounds__(1024) atm_order_kernel(Ctx c) {
  extern __shared__ unsigned long long s_key[];
  __shared__ float s_lo[3][32], s_hi[3][32];
  const int b = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  const size_t bN = (size_t)b * N;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (n > ATM_ORDER_MAX) {
    for (int t = tid; t < n; t += blockDim.x) c.w.atm_order[bN + t] = t;
    return;
  }
  int P = 1;
  while (P < n) P <<= 1;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int t = tid; t < n; t += blockDim.x) {
    if (c.w.z[bN + t] == 0) continue;
    const float4 p = c.w.pos32[bN + t];
    const float v[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], v[d]);
      hi[d] = fmaxf(hi[d], v[d]);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
    if (lane == 0) {
      s_lo[d][warp] = lo[d];
      s_hi[d][warp] = hi[d];
    }
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = FLT_MAX;
    hi[d] = -FLT_MAX;
    for (int w = 0; w < nw; ++w) {
      lo[d] = fminf(lo[d], s_lo[d][w]);
      hi[d] = fmaxf(hi[d], s_hi[d][w]);
    }
  }
  for (int t = tid; t < P; t += blockDim.x) {
    unsigned code = 0xFFFFFFFFu;  // padding and beyond n: last
    if (t < n && c.w.z[bN + t] != 0) {
      const float4 p = c.w.pos32[bN + t];
      const float v[3] = {p.x, p.y, p.z};
      unsigned q[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float ext = hi[d] - lo[d];
        const float f = ext > 0.f ? (v[d] - lo[d]) / ext : 0.f;
        q[d] = (unsigned)fminf(fmaxf(f * 1024.f, 0.f), 1023.f);
      }
      code = (spread_bits10(q[0]) << 2) | (spread_bits10(q[1]) << 1) | spread_bits10(q[2]);
    }
    s_key[t] = ((unsigned long long)code << 32) | (unsigned)t;
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = tid; t < P; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const unsigned long long a = s_key[t], bb = s_key[u];
          if ((a > bb) == ((t & k) == 0)) {
            s_key[t] = bb;
            s_key[u] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int t = tid; t < n; t += blockDim.x) c.w.atm_order[bN + t] = (int)(s_key[t] & 0xFFFFFFFFu);
}

constexpr int ATM_SPARSE_THREADS = 512;

// ATM energy and adjoint over the neighbour triples of one centre atom j
// (one CTA): every pair (i, k), i < k, of atoms within disp3 of j is a triple
// whose sides r_ij and r_jk are inside the cutoff.  Each unordered triple is
// taken once: with r_ik > disp3 its centre is unique; with all three sides
// inside, only at the centre of smallest index (j < i).  The arithmetic, the
// reference's per-atom attribution (threebody.py:153-163; here [ij] = [jk]
// = 1) and the adjoint are those of atm_task.
// Shared memory per list entry a (atom L[a]): the (j, L[a]) pair record, the
// entry's dE/d(r^2) and weighted-energy sums of the pair (j, L[a]) and its
// energy (units of e/6, s9 applied at the flush).  The (i, k) pair sums go
// to the global upper-half accumulators directly; atm_mirror_kernel fills
// the lower half afterwards.
template <bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(ATM_SPARSE_THREADS, 2) atm_sparse_kernel(Ctx c) {
  extern __shared__ float4 s_rec[];  // [ATM_SPARSE_DMAX] records, then L, S, P, E
  int *s_L = reinterpret_cast<int *>(s_rec + ATM_SPARSE_DMAX);
  float *s_S = reinterpret_cast<float *>(s_L + ATM_SPARSE_DMAX);
  float *s_P = s_S + ATM_SPARSE_DMAX;
  float *s_E = s_P + ATM_SPARSE_DMAX;
  __shared__ float s_red[ATM_SPARSE_THREADS / 32];
  const int b = blockIdx.y;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  if ((int)blockIdx.x >= n || n < 3 || !atm_sparse_mode(c, b, n)) return;
  const size_t bN = (size_t)b * N;
  const int j = c.w.atm_order[bN + blockIdx.x];  // centres in spatial order
  if (c.w.z[bN + j] == 0) return;
  const int d = c.w.nbr_deg[bN + j];  // <= ATM_SPARSE_DMAX in sparse mode
  if (d < 2) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const float4 *T = c.w.ptf + bN * N;
  const float4 *Tda = PGRAD ? c.w.ptf_da + bN * N : nullptr;
  const int *L = c.w.nbr + (bN + j) * N;
  for (int t = threadIdx.x; t < d; t += blockDim.x) {
    const int k = L[t];
    s_L[t] = k;
    s_rec[t] = T[(size_t)j * N + k];
    s_S[t] = 0.f;
    s_P[t] = 0.f;
    s_E[t] = 0.f;
  }
  __syncthreads();
  const float *W = c.w.w32 + bN;
  const bool weighted = c.weights != nullptr;
  const float cut2 = c.pf.cut3 * c.pf.cut3, alp3 = c.pf.alp3, s9 = c.pf.s9;
  const float alp3h = 0.5f * alp3;
  float *gS = GRAD ? c.w.prS32 + bN * N : nullptr;
  float *gP = GRAD ? c.w.prP32 + bN * N : nullptr;
  const float wj = W[j];
  float Ej = 0.f;
  AtmPg pg;
  for (int a = warp; a < d - 1; a += nwarps) {
    const int i = s_L[a];
    const float4 pij = s_rec[a];
    const float wi = weighted ? W[i] : 1.f;
    const float4 *Ti = T + (size_t)i * N;
    const bool later = j < i;  // j is the smallest atom of every triple of this row
    float sij = 0.f, pe = 0.f, ei = 0.f;
    float4 daij = make_float4(0.f, 0.f, 0.f, 0.f);
    if (PGRAD) daij = Tda[(size_t)j * N + i];
    for (int e = a + 1 + lane; e < d; e += 32) {
      const int k = s_L[e];
      const float4 pik = Ti[k];
      const bool mik = pik.x <= cut2;
      if (mik && !later) continue;  // counted at its smallest atom
      const float4 pjk = s_rec[e];
      const AtmTri tr = atm_triple<GRAD>(pij.x, pij.y, pij.z, pij.w, pik.x, pik.y, pik.z,
                                         pik.w, pjk.x, pjk.y, pjk.z, pjk.w, alp3h);
      const float eu = tr.eu;  // triple energy without s9
      const float wk = weighted ? W[k] : 1.f;
      float wgt;
      if (mik) {  // all sides inside: e/3 to each atom
        const float e2 = eu + eu;
        ei += e2;
        Ej += e2;
        atomicAdd(&s_E[e], e2);
        wgt = (wi + wj + wk) * (1.0f / 3.0f);
      } else {  // r_ik outside: e/6 to i and to k, nothing to the centre
        ei += eu;
        atomicAdd(&s_E[e], eu);
        wgt = (wi + wk) * (1.0f / 6.0f);
      }
      if (GRAD) {
        const float ws = wgt * s9;
        const float we = ws * eu;
        sij = fmaf(ws, tr.dex, sij);
        pe += we;
        atomicAdd(&s_S[e], ws * tr.dez);
        atomicAdd(&s_P[e], we);
        atomicAdd(&gS[(size_t)i * N + k], ws * tr.dey);  // i < k: upper half
        atomicAdd(&gP[(size_t)i * N + k], we);
        if (PGRAD) {
          const float4 daik = Tda[(size_t)i * N + k];
          const float4 dajk = Tda[(size_t)j * N + k];
          const float lsum = daij.z + daik.z + dajk.z;
          pg.s9 += wgt * eu;
          pg.alp -= wgt * s9 * tr.qwg * lsum * (1.0f / 3.0f);
          const float dfa = -wgt * s9 * tr.qwg * alp3;
          pg.a1 += dfa * (daij.x + daik.x + dajk.x);
          pg.a2 += dfa * (daij.y + daik.y + dajk.y);
        }
      }
    }
    ei = warp_sumf(ei);
    if (GRAD) {
      sij = warp_sumf(sij);
      pe = warp_sumf(pe);
    }
    if (lane == 0) {
      if (ei != 0.f) atomicAdd(&s_E[a], ei);
      if (GRAD && (sij != 0.f || pe != 0.f)) {
        atomicAdd(&s_S[a], sij);
        atomicAdd(&s_P[a], pe);
      }
    }
  }
  if (PGRAD) {
    pg.s9 = warp_sumf(pg.s9);
    pg.alp = warp_sumf(pg.alp);
    pg.a1 = warp_sumf(pg.a1);
    pg.a2 = warp_sumf(pg.a2);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 3], (double)pg.a1);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 4], (double)pg.a2);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 5], (double)pg.s9);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 6], (double)pg.alp);
    }
  }
  Ej = warp_sumf(Ej);
  if (lane == 0) s_red[warp] = Ej;
  __syncthreads();
  const double escale = c.par.s9 / 6.0;
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < nwarps; ++w) t += s_red[w];
    if (t != 0.f) atomicAdd(&c.w.e3[bN + j], (double)t * escale);
  }
  for (int t = threadIdx.x; t < d; t += blockDim.x) {
    const int k = s_L[t];
    const float ev = s_E[t];
    if (ev != 0.f) atomicAdd(&c.w.e3[bN + k], (double)ev * escale);
    if (GRAD) {
      const float sv = s_S[t], pv = s_P[t];
      if (sv != 0.f || pv != 0.f) {
        const size_t o = j < k ? (size_t)j * N + k : (size_t)k * N + j;  // upper half
        atomicAdd(&gS[o], sv);
        atomicAdd(&gP[o], pv);
      }
    }
  }
}

// ATM forces, C6(q=0) adjoint, chain rule to dE/dCN and dE/dq, E2 + E3.
__global__ void __launch_bounds__(256) pair_atm_bwd_mixed_kernel(Ctx c) {
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
      c.w.adj32[ax] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 *PL = c.w.pos32lo + (size_t)b * N;
  const float4 px = P[x], lx = PL[x];
  const int nslot = c.w.n_slots[b];
  const int slot_x = c.w.slot[ax];
  const size_t base = (size_t)b * N * N;
  const float4 *T = c.w.ptf + base + (size_t)x * N;
  Acc32 gx, gy, gz;
  Acc32 dcn_acc, dq_acc;
  for (int s = 0; s < nslot; ++s) {
    float gacc[NFREQ];
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) gacc[w] = 0.f;
    for (int y = lane; y < n; y += 32) {
      const size_t ay = (size_t)b * N + y;
      if (y == x || c.w.z[ay] == 0 || c.w.slot[ay] != s) continue;
      const size_t o = base + (size_t)x * N + y;
      const float S = c.w.prS32[o];
      const float Pv = c.w.prP32[o];
      const float3 d = pos_diff(px, lx, P[y], PL[y]);
      gx.add(2.0f * S * d.x);
      gy.add(2.0f * S * d.y);
      gz.add(2.0f * S * d.z);
      if (Pv != 0.f) {
        const float cw = T[y].w;  // sqrt(C6(q=0)) / r^3: C6(q=0) = w^2 r^6
        const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
        const float D = Pv / (2.0f * (cw * cw) * (r2 * r2 * r2));
        const float *A0y = c.w.A032 + a32_index(b, y, slot_x, 0, N, c.S);
#pragma unroll
        for (int w = 0; w < NFREQ; ++w) gacc[w] = fmaf(D, A0y[(size_t)w * N], gacc[w]);
      }
    }
    const float mine = warp_reduce_scatter32(gacc);  // lane w: sum of gacc[w]
    // chain rule to CN and q for this slot (lane = frequency)
    if (lane < NFREQ) {
      const size_t o = (ax * c.S + s) * NFREQ + lane;
      const float g0w = mine;  // dE/dA'0_x
      const float gw = c.w.G32[o];
      const float *d = c.w.dA32 + 3 * o;
      dcn_acc.add(gw * d[0]);
      dcn_acc.add(g0w * d[2]);
      dq_acc.add(gw * d[1]);
    }
  }
  const Acc32 g0 = warp_sum_acc(gx), g1 = warp_sum_acc(gy), g2 = warp_sum_acc(gz);
  const Acc32 dcn = warp_sum_acc(dcn_acc), dq = warp_sum_acc(dq_acc);
  if (lane == 0) {
    c.w.dEdcn[ax] = dcn.value();
    c.w.dEdq[ax] = dq.value();
    c.w.adj32[ax] = make_float4(dcn.hi + dcn.lo, 0.f, (float)c.w.q[ax], 0.f);
    c.out.d_gradient[3 * ax] += g0.value();
    c.out.d_gradient[3 * ax + 1] += g1.value();
    c.out.d_gradient[3 * ax + 2] += g2.value();
    c.out.d_energy[ax] += c.w.e3[ax];
  }
}

// Forces through the D4 CN, the EEQ CN and the EEQ Coulomb matrix (FP32).
__global__ void __launch_bounds__(256) pair_cn_bwd_mixed_kernel(Ctx c) {
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
  const float kcn = c.pf.kcn;
  const float cut_cn = c.pf.cut_cn, cut_q = c.pf.cut_q;
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 *X = c.w.aux32 + (size_t)b * N;
  const float4 *D = c.w.adj32 + (size_t)b * N;
  const float4 *PL = c.w.pos32lo + (size_t)b * N;
  const float4 pi = P[i], li = PL[i], xi = X[i], di = D[i];
  const float4 *CP = c.w.cnpair + (size_t)zi * MAX_ELEM_ID;
  Acc32 gx, gy, gz;
  for (int j = lane; j < n; j += 32) {
    const size_t aj = (size_t)b * N + j;
    const int zj = c.w.z[aj];
    if (j == i || zj == 0) continue;
    const float4 pj = P[j], xj = X[j], dj = D[j];
    const float4 cp = CP[zj];
    const float3 d = pos_diff(pi, li, pj, PL[j]);
    const float dx = d.x, dy = d.y, dz = d.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ir = rsqrtf(r2);
    const float r = r2 * ir;
    float dEdr = 0.f;
    const float xx = kcn * fmaf(r, cp.y, fmaf(r, cp.x, -1.0f));  // kcn (r / r0 - 1)
    if (xx < 9.0f) {
      const float dcf = -kcn * cp.x * INV_SQRT_PI_F * __expf(-xx * xx);
      if (r <= cut_cn) dEdr += (di.x + dj.x) * (cp.z + cp.w) * dcf;
      if (eeq && r <= cut_q) dEdr += (di.y + dj.y) * dcf;
    }
    if (eeq) {
      const float g = rsqrtf(xi.z * xi.z + xj.z * xj.z);
      const float gr = g * r;
      const float dA = (2.0f * g * INV_SQRT_PI_F * __expf(-gr * gr) * r - erff(gr)) * ir * ir;
      dEdr -= (di.w * dj.z + dj.w * di.z) * dA;
    }
    const float f = dEdr * ir;
    gx.add(f * dx);
    gy.add(f * dy);
    gz.add(f * dz);
  }
  const Acc32 g0 = warp_sum_acc(gx), g1 = warp_sum_acc(gy), g2 = warp_sum_acc(gz);
  if (lane == 0) {
    c.out.d_gradient[3 * ai] += g0.value();
    c.out.d_gradient[3 * ai + 1] += g1.value();
    c.out.d_gradient[3 * ai + 2] += g2.value();
  }
}

// ---------------------------------------------------------------- EEQ

// Dense EEQ Coulomb matrix of the real atoms as the double-float pair of
// FP32 matrices hi + lo (compact order, leading dimension N), the operator of
// the FP64-accurate refinement residuals:
//   A_kl = erf(r_kl / g_kl) / r_kl (k != l),  A_kk = eta + sqrt(2/pi) / rad,
// g_kl = sqrt(rad_k^2 + rad_l^2) (tad_multicharge's EEQ, restated).  Off the
// diagonal all of it runs in double-float on the FP32 pipe: positions as
// pos32 + pos32lo, r^2 from them, 1/r by df_rsqrt, erf by df_erf, with
// 1/g and the diagonal from per-element tables; no FP64 instruction.
// Persistent blocks loop over the 32 x 32 tiles of the lower triangles of
// all structures; a tile and its mirror are both stored coalesced (the
// mirror through shared memory).  The lower tiles' hi part also goes to the
// multi-CTA factorisation's matrix F (row stride eeq_ldf(N)), which reads
// nothing above the diagonal.
__global__ void __launch_bounds__(256) eeq_build_df_kernel(Ctx c) {
  __shared__ float4 s_erf[ERF_TAB];
  __shared__ float s_hi[32][33], s_lo[32][33];
  for (int k = threadIdx.x; k < ERF_TAB; k += blockDim.x) s_erf[k] = c.w.erf_tab[k];
  __syncthreads();
  const int N = c.N;
  const int NF = eeq_ldf(N);
  const int T = (N + 31) / 32;
  const int tp = T * (T + 1) / 2;
  const size_t total = (size_t)c.B * tp;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (size_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = (int)(t / tp);
    const int r = (int)(t % tp);
    int ti = (int)((sqrtf(8.f * (float)r + 1.f) - 1.f) * 0.5f);
    while ((ti + 1) * (ti + 2) / 2 <= r) ++ti;
    while (ti > 0 && ti * (ti + 1) / 2 > r) --ti;
    const int tj = r - ti * (ti + 1) / 2;
    const int m = c.w.n_real[b];
    if (ti * 32 >= m) continue;  // uniform over the block
    const size_t bN = (size_t)b * N;
    float *Hi = c.w.eeq_hi + bN * N;
    float *Lo = c.w.eeq_lo + bN * N;
    float *F = c.w.eeq_F + bN * NF;
    const int l = tj * 32 + tx;
    int zl = 0;
    float4 pl = make_float4(0.f, 0.f, 0.f, 0.f), pll = pl;
    if (l < m) {
      const int al = c.w.ridx[bN + l];
      zl = c.w.z[bN + al];
      pl = c.w.pos32[bN + al];
      pll = c.w.pos32lo[bN + al];
    }
#pragma unroll 1
    for (int kk = 0; kk < 4; ++kk) {
      const int rr = ty + 8 * kk;
      const int k = ti * 32 + rr;
      dfl v = {0.f, 0.f};
      if (k < m && l < m) {
        const int ak = c.w.ridx[bN + k];
        const int zk = c.w.z[bN + ak];
        if (k == l) {
          const float2 d = c.w.eeq_diag[zk];
          v = dfl{d.x, d.y};
        } else {
          const float4 pk = c.w.pos32[bN + ak], pkl = c.w.pos32lo[bN + ak];
          const dfl dx = df_add(dfl{pk.x, pkl.x}, dfl{-pl.x, -pll.x});
          const dfl dy = df_add(dfl{pk.y, pkl.y}, dfl{-pl.y, -pll.y});
          const dfl dz = df_add(dfl{pk.z, pkl.z}, dfl{-pl.z, -pll.z});
          const dfl r2 = df_add(df_add(df_sq(dx), df_sq(dy)), df_sq(dz));
          const dfl ir = df_rsqrt(r2);
          const float2 g = c.w.igam[zk * MAX_ELEM_ID + zl];
          const dfl x = df_mul(df_mul(r2, ir), dfl{g.x, g.y});
          v = df_mul(df_erf(x, s_erf), ir);
        }
        Hi[(size_t)k * N + l] = v.hi;
        Lo[(size_t)k * N + l] = v.lo;
        F[(size_t)k * NF + l] = v.hi;  // the factorisation's input (lower part)
      }
      s_hi[rr][tx] = v.hi;
      s_lo[rr][tx] = v.lo;
    }
    if (ti != tj) {
      __syncthreads();
#pragma unroll 1
      for (int kk = 0; kk < 4; ++kk) {
        const int rr = ty + 8 * kk;
        const int l2 = tj * 32 + rr, k2 = ti * 32 + tx;
        if (l2 < m && k2 < m) {
          Hi[(size_t)l2 * N + k2] = s_hi[tx][rr];
          Lo[(size_t)l2 * N + k2] = s_lo[tx][rr];
        }
      }
    }
    __syncthreads();
  }
}

// Shared-memory layout of the mixed EEQ kernels (in floats):
//   idx      int[Nr]          compact index -> atom (Nr = N rounded up to 4)
//   X        float2[2N]       solution (two right-hand sides), double-float
//   BB       float2[2N]       right-hand sides (b, 1), double-float
//   vf       float[2N]        FP32 residual / correction
//   (16-byte aligned from here)
//   PT       float[32 * ldp]  transposed panel of the factorisation (SMEM only)
//   L        float[N(N+1)/2]  FP32 factor (SMEM only; the adjoint has no PT)

constexpr int EEQ_REFINE_MAX = 8;
constexpr int EEQ_THREADS = 256;
constexpr float EEQ_RESIDUAL_TOL = 1e-10f;

// acc + (h + lo) x for a double-float x; acc is left unnormalised (its low
// part collects the rounding errors; a row has at most a few hundred terms
// per lane).
__device__ __forceinline__ dfl df_acc_prod(dfl acc, float h, float lo, float2 x) {
  const float p = h * x.x;
  const float e = fmaf(h, x.y, fmaf(lo, x.x, fmaf(h, x.x, -p)));
  const dfl s = df_two_sum(acc.hi, p);
  return {s.hi, acc.lo + (s.lo + e)};
}

__device__ __forceinline__ dfl df_warp_sum(dfl a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, a.hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, a.lo, o);
    const dfl s = df_two_sum(a.hi, oh);
    a = df_fast(s.hi, s.lo + (a.lo + ol));
  }
  return a;
}

// Residual r = BB - (hi + lo) X for ``nr`` right-hand sides, in double-float
// (FP64-accurate, on the FP32 pipe): a warp takes four rows at a time, lanes
// over columns (coalesced), so that 32 independent loads per lane are in
// flight (one row at a time left the warp waiting on L2 latency row after
// row).  r is rounded to FP32 into vf, the right-hand side of the next
// correction; returns max |r| over the block.
__device__ float eeq_residual_df(const float *Hi, const float *Lo, const float2 *X,
                                 const float2 *BB, float *vf, int m, int N, int nr,
                                 float *s_red) {
  constexpr int RW = 4;  // rows per warp pass
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  float mx = 0.f;
  for (int k0 = warp * RW; k0 < m; k0 += nw * RW) {
    dfl a0[RW], a1[RW];
#pragma unroll
    for (int q = 0; q < RW; ++q) a0[q] = a1[q] = dfl{0.f, 0.f};
    for (int l0 = lane; l0 < m; l0 += 128) {
      float h[RW][4], lo[RW][4];
#pragma unroll
      for (int q = 0; q < RW; ++q) {
        const int k = k0 + q;
        const float *hr = Hi + (size_t)(k < m ? k : 0) * N, *lr = Lo + (size_t)(k < m ? k : 0) * N;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + 32 * u;
          const bool ok = k < m && l < m;
          h[q][u] = ok ? hr[l] : 0.f;
          lo[q][u] = ok ? lr[l] : 0.f;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int l = l0 + 32 * u;
        if (l < m) {
          const float2 x0 = X[l];
          const float2 x1 = nr == 2 ? X[N + l] : make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 0; q < RW; ++q) {
            a0[q] = df_acc_prod(a0[q], h[q][u], lo[q][u], x0);
            if (nr == 2) a1[q] = df_acc_prod(a1[q], h[q][u], lo[q][u], x1);
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RW; ++q) {
      const int k = k0 + q;
      const dfl s0 = df_warp_sum(a0[q]);
      const dfl s1 = nr == 2 ? df_warp_sum(a1[q]) : dfl{0.f, 0.f};
      if (lane == 0 && k < m) {
        const dfl r0 = df_add(dfl{BB[k].x, BB[k].y}, df_neg(s0));
        vf[k] = r0.hi;
        mx = fmaxf(mx, fabsf(r0.hi));
        if (nr == 2) {
          const dfl r1 = df_add(dfl{BB[N + k].x, BB[N + k].y}, df_neg(s1));
          vf[N + k] = r1.hi;
          mx = fmaxf(mx, fabsf(r1.hi));
        }
      }
    }
  }
  if (lane == 0) s_red[warp] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    float v = 0.f;
    for (int w = 0; w < nw; ++w) v = fmaxf(v, s_red[w]);
    s_red[32] = v;
  }
  __syncthreads();
  const float out = s_red[32];
  __syncthreads();
  return out;
}

// FP32 factor + double-float refinement: X (nr columns) <- A^-1 BB to an
// FP64-level residual below 1e-10.  Returns the last residual max |r|
// (uniform over the block).
__device__ float eeq_refined_solve(const float *L, const float *Hi, const float *Lo, float2 *X,
                                   const float2 *BB, float *vf, int m, int N, int nr,
                                   float *s_red) {
  for (int t = threadIdx.x; t < m * nr; t += blockDim.x) {
    const int o = (t / m) * N + t % m;
    X[o] = make_float2(0.f, 0.f);
    vf[o] = BB[o].x;
  }
  __syncthreads();
  float res = 0.f;
  for (int it = 0; it < EEQ_REFINE_MAX; ++it) {
    fwd_solve_blocked(L, vf, N, m, nr);
    bwd_solve_blocked(L, vf, N, m, nr);
    for (int t = threadIdx.x; t < m * nr; t += blockDim.x) {
      const int o = (t / m) * N + t % m;
      const dfl s = df_add(dfl{X[o].x, X[o].y}, dfl{vf[o], 0.f});
      X[o] = make_float2(s.hi, s.lo);
    }
    __syncthreads();
    res = eeq_residual_df(Hi, Lo, X, BB, vf, m, N, nr, s_red);
    if (res < EEQ_RESIDUAL_TOL) break;
  }
  return res;
}

template <bool SMEM>
__global__ void __launch_bounds__(EEQ_THREADS, 2) eeq_mixed_kernel(Ctx c) {
  extern __shared__ float4 s_dyn4[];
  float *s_f = reinterpret_cast<float *>(s_dyn4);
  const int b = c.w.sorder[blockIdx.x];  // largest structures first
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_m;
  __shared__ float s_red[33];
  __shared__ double s_lam;
  const int Nr = eeq_round4(N);
  int *s_idx = reinterpret_cast<int *>(s_f);
  float2 *X = reinterpret_cast<float2 *>(s_f + Nr);
  float2 *BB = X + 2 * N;
  float *vf = reinterpret_cast<float *>(BB + 2 * N);
  const size_t NN2 = (size_t)N * (N + 1) / 2;
  const int ldp = chol_panel_ld(N);
  float *PT = SMEM ? s_f + eeq_mixed_vec_floats(N) : nullptr;
  float *L = SMEM ? PT + PB * ldp : c.w.eeq_L32 + (size_t)b * NN2;
  const float *Hi = c.w.eeq_hi + (size_t)b * N * N;
  const float *Lo = c.w.eeq_lo + (size_t)b * N * N;
  const int m = compact_real_atoms(c, b, n, s_idx, &s_m);
  const int *Zb = c.w.z + (size_t)b * N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  // The Coulomb matrix of the structure in double-float (the arithmetic of
  // eeq_build_df_kernel, which builds it for the multi-CTA solve): the FP32
  // factor input straight into L, the hi / lo rows (both triangles) to global
  // memory for the refinement residuals.  The structure's atoms are staged in
  // the panel buffer, idle until the factorisation; a warp takes every
  // (EEQ_THREADS / 32)-th row, lanes over its columns.
  {
    static_assert(SMEM, "the matrix is built into the shared-memory factor");
    float4 *sp = reinterpret_cast<float4 *>(PT);  // positions (hi), then (lo), then Z
    float4 *spl = sp + m;
    int *sz = reinterpret_cast<int *>(spl + m);
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
      const size_t a = (size_t)b * N + s_idx[k];
      sp[k] = c.w.pos32[a];
      spl[k] = c.w.pos32lo[a];
      sz[k] = c.w.z[a];
    }
    __syncthreads();
    float *Hw = c.w.eeq_hi + (size_t)b * N * N;
    float *Lw = c.w.eeq_lo + (size_t)b * N * N;
    const float4 *etab = c.w.erf_tab;
    for (int k = warp; k < m; k += nw) {
      const float4 pk = sp[k], pkl = spl[k];
      const int zk = sz[k];
      float *lrow = L + tri_index(k, 0);
      for (int l = lane; l <= k; l += 32) {
        dfl v;
        if (l == k) {
          const float2 d = c.w.eeq_diag[zk];
          v = dfl{d.x, d.y};
        } else {
          const float4 pl = sp[l], pll = spl[l];
          const dfl dx = df_add(dfl{pk.x, pkl.x}, dfl{-pl.x, -pll.x});
          const dfl dy = df_add(dfl{pk.y, pkl.y}, dfl{-pl.y, -pll.y});
          const dfl dz = df_add(dfl{pk.z, pkl.z}, dfl{-pl.z, -pll.z});
          const dfl r2 = df_add(df_add(df_sq(dx), df_sq(dy)), df_sq(dz));
          const dfl ir = df_rsqrt(r2);
          const float2 g = c.w.igam[zk * MAX_ELEM_ID + sz[l]];
          const dfl x = df_mul(df_mul(r2, ir), dfl{g.x, g.y});
          v = df_mul(df_erf(x, etab), ir);
          Hw[(size_t)l * N + k] = v.hi;  // the upper triangle (strided)
          Lw[(size_t)l * N + k] = v.lo;
        }
        lrow[l] = v.hi;
        Hw[(size_t)k * N + l] = v.hi;
        Lw[(size_t)k * N + l] = v.lo;
      }
    }
  }
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const int ia = s_idx[k];
    const int z = Zb[ia];
    const double cq = c.w.cnq[(size_t)b * N + ia];
    const double sq = cq > 0.0 ? sqrt(cq) : 0.0;
    const dfl bk = df_from(-c.tab.eeq_chi[z] + c.tab.eeq_kcn[z] * sq);
    BB[k] = make_float2(bk.hi, bk.lo);
    BB[N + k] = make_float2(1.f, 0.f);
  }
  __syncthreads();
  chol_blocked(L, PT, ldp, m, &s_bad);
  if (threadIdx.x == 0 && s_bad) set_status(c.w.status, D4_ERR_EEQ_SINGULAR);
  const float res = eeq_refined_solve(L, Hi, Lo, X, BB, vf, m, N, 2, s_red);
  if (threadIdx.x == 0) c.w.eeq_final[2 * b] = res;
  if (warp == 0) {
    double sx = 0.0, sy = 0.0;
    for (int k = lane; k < m; k += 32) {
      sx += (double)X[k].x + (double)X[k].y;
      sy += (double)X[N + k].x + (double)X[N + k].y;
    }
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    if (lane == 0) {
      const double lam = m > 0 ? (sx - c.charge[b]) / sy : 0.0;
      c.w.eeq_sum[2 * b] = sy;
      c.w.eeq_sum[2 * b + 1] = lam;
      s_lam = lam;
    }
  }
  __syncthreads();
  const double lam = s_lam;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    c.w.q[(size_t)b * N + i] = 0.0;
    c.w.eeq_y[(size_t)b * N + i] = 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const size_t a = (size_t)b * N + s_idx[k];
    const double x0 = (double)X[k].x + (double)X[k].y;
    const double x1 = (double)X[N + k].x + (double)X[N + k].y;
    c.w.q[a] = x0 - lam * x1;
    c.w.eeq_y[a] = x1;
  }
  if (SMEM) {
    float *G = c.w.eeq_L32 + (size_t)b * NN2;
    const size_t tri_m = (size_t)m * (m + 1) / 2;
    for (size_t t = threadIdx.x; t < tri_m; t += blockDim.x) G[t] = L[t];
  }
}

// Adjoint: A u = dE/dq by the FP32 factor + double-float refinement,
// w = u - nu y.  SMEM: the factor is staged in shared memory.
template <bool SMEM>
__global__ void __launch_bounds__(EEQ_THREADS, 2) eeq_adjoint_mixed_kernel(Ctx c) {
  extern __shared__ float4 s_dyn4[];
  float *s_f = reinterpret_cast<float *>(s_dyn4);
  const int b = c.w.sorder[blockIdx.x];  // largest structures first
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_m;
  __shared__ float s_red[33];
  __shared__ double s_nu;
  const int Nr = eeq_round4(N);
  int *s_idx = reinterpret_cast<int *>(s_f);
  float2 *X = reinterpret_cast<float2 *>(s_f + Nr);
  float2 *BB = X + 2 * N;
  float *vf = reinterpret_cast<float *>(BB + 2 * N);
  const size_t NN2 = (size_t)N * (N + 1) / 2;
  const float *Lg = c.w.eeq_L32 + (size_t)b * NN2;
  const float *Hi = c.w.eeq_hi + (size_t)b * N * N;
  const float *Lo = c.w.eeq_lo + (size_t)b * N * N;
  const int m = compact_real_atoms(c, b, n, s_idx, &s_m);
  const float *L = Lg;
  if (SMEM) {
    float *Ls = s_f + eeq_mixed_vec_floats(N);
    const size_t tri_m = (size_t)m * (m + 1) / 2;
    for (size_t t = threadIdx.x; t < tri_m; t += blockDim.x) Ls[t] = Lg[t];
    L = Ls;
  }
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const dfl g = df_from(c.w.dEdq[(size_t)b * N + s_idx[k]]);
    BB[k] = make_float2(g.hi, g.lo);
  }
  __syncthreads();
  const float res = eeq_refined_solve(L, Hi, Lo, X, BB, vf, m, N, 1, s_red);
  if (threadIdx.x == 0) c.w.eeq_final[2 * b + 1] = res;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    double su = 0.0;
    for (int k = lane; k < m; k += 32) su += (double)X[k].x + (double)X[k].y;
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
    const double w = (double)X[k].x + (double)X[k].y - nu * c.w.eeq_y[a];
    c.w.eeq_w[a] = w;
    const double cq = c.w.cnq[a];
    const int z = c.w.z[a];
    const double dq = cq > 0.0 ? w * c.tab.eeq_kcn[z] * 0.5 / sqrt(cq) * c.w.dcnq[a] : 0.0;
    c.w.dEdcnq[a] = dq;
    c.w.adj32[a].y = (float)dq;
    c.w.adj32[a].w = (float)w;
  }
}

// ---------------------------------------------------------------- launch

// persistent grid of the EEQ build: 4 blocks per SM, at most one per tile
static unsigned build_blocks(const Ctx &c) {
  static int sms[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int &n = sms[dev & 63];
  if (n == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n = v > 0 ? v : 1;
  }
  const size_t T = (size_t)(c.N + 31) / 32;
  const size_t tiles = (size_t)c.B * T * (T + 1) / 2;
  const size_t want = (size_t)4 * n;
  return (unsigned)(tiles < want ? (tiles > 0 ? tiles : 1) : want);
}

template <bool SMEM, bool GRAD, bool PGRAD>
static void launch_atm(const Ctx &c, cudaStream_t st, size_t smem) {
  if (SMEM)
    ensure_smem(atm_mixed_kernel<SMEM, GRAD, PGRAD>, (int)smem);
  const int threads = PGRAD ? ATM_THREADS_PGRAD : ATM_THREADS;
  const int K = SMEM ? ATM_KMAX : atm_ctas_big(c.N);
  if (!SMEM) {
    atm_nbr_kernel<<<dim3((c.N + 7) / 8, c.B), 256, 0, st>>>(c);
    int P = 1;
    while (P < c.N && P < ATM_ORDER_MAX) P <<= 1;
    const int osm = 8 * P;
    ensure_smem(atm_order_kernel, osm);
    atm_order_kernel<<<c.B, 1024, osm, st>>>(c);
  }
  atm_mixed_kernel<SMEM, GRAD, PGRAD><<<dim3(K, c.B), threads, smem, st>>>(c);
  if (!SMEM) {  // neighbour-triple variant; returns at once for dense structures
    const int sp = ATM_SPARSE_DMAX * (16 + 4 * 4);
    ensure_smem(atm_sparse_kernel<GRAD, PGRAD>, sp);
    atm_sparse_kernel<GRAD, PGRAD><<<dim3(c.N, c.B), ATM_SPARSE_THREADS, sp, st>>>(c);
  }
  if (!SMEM && GRAD) {
    const int T = (c.N + 31) / 32;
    atm_mirror_kernel<<<dim3(T, T, c.B), 256, 0, st>>>(c);
  }
}

int launch_mixed(const Ctx &c_in, cudaStream_t st) {
  Ctx c = c_in;
  const int B = c.B, N = c.N;
  const dim3 atoms((N + 7) / 8, B);
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  const bool pgrad = (c.flags & D4_FLAG_PARAM_GRAD) != 0;
  const bool eeq = (c.flags & D4_FLAG_CHARGES_IN) == 0;
  const bool atm_tiled = atm_smem_fits(N) && !pgrad && c.weights == nullptr;
  c.atm_tiled = atm_tiled ? 1 : 0;  // (the prep skips zeroing what that kernel stores)
  timing_next_call();
  stage_begin(ST_PREP, st);
  launch_prep_memsets(c, st);
  prep_tables_kernel<<<B + TABLES32_THREADS / 256, 256, 0, st>>>(c);
  {
    int P = 1;
    while (P < B && P < SORDER_MAX) P <<= 1;
    const int osm = 8 * P;
    if (osm > 48 * 1024)
      ensure_smem(size_order_kernel, osm);
    size_order_kernel<<<1, 1024, osm, st>>>(c);
  }
  stage_end(ST_PREP, st);
  stage_begin(ST_CN, st);
  cn_mixed_kernel<<<atoms, 256, 0, st>>>(c);
  stage_end(ST_CN, st);
  const size_t vec_bytes = 4 * eeq_mixed_vec_floats(N);
  const size_t tri_bytes = (size_t)4 * ((size_t)N * (N + 1) / 2);
  const size_t pt_bytes = (size_t)4 * PB * chol_panel_ld(N);
  const bool eeq_smem = eeq_small_fits(N);
  stage_begin(ST_EEQ, st);
  if (eeq) {
    if (!eeq_smem) eeq_build_df_kernel<<<build_blocks(c), 256, 0, st>>>(c);
    if (eeq_smem) {  // builds its matrix itself
      ensure_smem(eeq_mixed_kernel<true>, (int)(vec_bytes + pt_bytes + tri_bytes));
      eeq_mixed_kernel<true><<<B, EEQ_THREADS, vec_bytes + pt_bytes + tri_bytes, st>>>(c);
    } else {
      launch_eeq_big(c, st, false);
    }
  } else {
    launch_charges_in(c, st);
  }
  stage_end(ST_EEQ, st);
  stage_begin(ST_WEIGHTS, st);
  weights_mixed_kernel<<<dim3((unsigned)(((N + 127) / 128) * c.S), B), 128, 0, st>>>(c);
  stage_end(ST_WEIGHTS, st);
  stage_begin(ST_PAIR_FWD, st);
  if (c.cfg.kind == D4_MODEL_D4)  // C6 on the tensor cores
    launch_pair_fwd_tc(c, st);
  else if (pgrad)
    pair_fwd_mixed_kernel<true, true><<<atoms, 256, 0, st>>>(c);
  else if (grad)
    pair_fwd_mixed_kernel<true, false><<<atoms, 256, 0, st>>>(c);
  else
    pair_fwd_mixed_kernel<false, false><<<atoms, 256, 0, st>>>(c);
  stage_end(ST_PAIR_FWD, st);
  // ATM: shared-memory accumulation when the largest structure fits
  const size_t atm_smem = atm_smem_bytes(N);
  const bool atm_sm = atm_smem_fits(N);
  stage_begin(ST_ATM, st);
  if (atm_tiled) {  // register-tiled triples
    const size_t sm = atm_tiled_smem_bytes(N);
    if (grad) {
      ensure_smem(atm_tiled_kernel<true>, (int)sm);
      atm_tiled_kernel<true><<<dim3(ATM_KMAX, B), AT_THREADS, sm, st>>>(c);
    } else {
      ensure_smem(atm_tiled_kernel<false>, (int)sm);
      atm_tiled_kernel<false><<<dim3(ATM_KMAX, B), AT_THREADS, sm, st>>>(c);
    }
  } else if (atm_sm) {
    if (pgrad)
      launch_atm<true, true, true>(c, st, atm_smem);
    else if (grad)
      launch_atm<true, true, false>(c, st, atm_smem);
    else
      launch_atm<true, false, false>(c, st, atm_smem);
  } else {
    if (pgrad)
      launch_atm<false, true, true>(c, st, 0);
    else if (grad)
      launch_atm<false, true, false>(c, st, 0);
    else
      launch_atm<false, false, false>(c, st, 0);
  }
  stage_end(ST_ATM, st);
  if (grad) {
    stage_begin(ST_PAIR_ATM_BWD, st);
    if (pair_atm_bwd_tc_ok(c))  // C6(q=0) adjoint on the tensor cores
      launch_pair_atm_bwd_tc(c, st);
    else
      pair_atm_bwd_mixed_kernel<<<atoms, 256, 0, st>>>(c);
    stage_end(ST_PAIR_ATM_BWD, st);
    if (eeq) {
      stage_begin(ST_EEQ_ADJ, st);
      if (eeq_smem) {
        ensure_smem(eeq_adjoint_mixed_kernel<true>, (int)(vec_bytes + tri_bytes));
        eeq_adjoint_mixed_kernel<true><<<B, EEQ_THREADS, vec_bytes + tri_bytes, st>>>(c);
      } else {
        launch_eeq_big(c, st, true);
      }
      stage_end(ST_EEQ_ADJ, st);
    }
    stage_begin(ST_PAIR_CN_BWD, st);
    pair_cn_bwd_mixed_kernel<<<atoms, 256, 0, st>>>(c);
    stage_end(ST_PAIR_CN_BWD, st);
  }
  stage_begin(ST_FINISH, st);
  launch_finish(c, st);
  stage_end(ST_FINISH, st);
  return 0;
}

}  // namespace d4
