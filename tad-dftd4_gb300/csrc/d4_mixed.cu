// Precision form of the D4 path: FP32 pair and triple arithmetic with
// compensated accumulation, FP32 Cholesky of the EEQ matrix recovered by FP64
// iterative refinement, FP64 for coordination numbers, reference weights,
// residuals and the final per-atom / per-structure reductions.
//
// Shared stages (prep, CN, weights, finish) are the FP64 ones.  The CN kernel
// skips pairs whose counting function is exactly zero in FP64, so it costs
// little; the weights are per atom.
#include <float.h>

#include "d4_common.cuh"
#include "d4_kernels.cuh"

namespace d4 {

constexpr float INV_SQRT_PI_F = 0.564189583547756f;
constexpr float SQRT3_F = 1.7320508075688772f;
constexpr int ATM_CTA_TRIPLES = 300000;  // target triples per ATM CTA
constexpr int ATM_KMAX = 8;                   // CTAs per structure at most
constexpr int ATM_THREADS = 1024;       // 32 warps: one CTA per SM (shared memory)
constexpr int ATM_THREADS_PGRAD = 512;  // the parameter-gradient variant needs more registers

// ---------------------------------------------------------------- convert

// FP32 copies of the weighted polarisabilities, transposed to
// [b][slot][frequency][atom] so that lanes over partner atoms load
// consecutive addresses.
__global__ void mixed_convert_kernel(Ctx c) {
  const size_t nA = (size_t)c.B * c.N * c.S * NFREQ;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const int N = c.N, S = c.S;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nA; t += stride) {
    // t indexes the transposed layout: ((b * S + s) * 23 + w) * N + i
    const int i = (int)(t % N);
    const size_t r = t / N;
    const int w = (int)(r % NFREQ);
    const size_t bs = r / NFREQ;
    const int s = (int)(bs % S);
    const size_t b = bs / S;
    const size_t src = (((b * N + i) * S) + s) * NFREQ + w;
    c.w.A32[t] = (float)c.w.A[src];
    c.w.A032[t] = (float)c.w.A0[src];
    if (c.w.dA32) {
      c.w.dA32[3 * src] = (float)c.w.dA_dcn[src];
      c.w.dA32[3 * src + 1] = (float)c.w.dA_dq[src];
      c.w.dA32[3 * src + 2] = (float)c.w.dA0_dcn[src];
    }
  }
}

// transposed index of (structure b, atom i, slot s, frequency w)
__device__ __forceinline__ size_t a32_index(int b, int i, int s, int w, int N, int S) {
  return (((size_t)b * S + s) * NFREQ + w) * N + i;
}

// ---------------------------------------------------------------- CN

// D4 and EEQ coordination numbers in FP32 (precision form): the counting
// function as 1/2 erfc(x) (no cancellation for small counts), compensated
// per-lane sums, FP64 per-atom totals and the smooth EEQ cap in FP64.
__global__ void __launch_bounds__(256) cn_mixed_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  const int N = c.N;
  const int n = c.w.n_eff[b];
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
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 *X = c.w.aux32 + (size_t)b * N;
  const float4 pi = P[i], xi = X[i];
  const float kcn = c.pf.kcn, k4 = c.pf.k4, k5 = c.pf.k5, k6 = c.pf.k6;
  const float cut_cn = c.pf.cut_cn, cut_q = c.pf.cut_q;
  Acc32 s_d4, s_q;
  for (int j = lane; j < n; j += 32) {
    if (j == i || c.w.z[(size_t)b * N + j] == 0) continue;
    const float4 pj = P[j], xj = X[j];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float x = kcn * (r / (xi.x + xj.x) - 1.0f);
    if (x > 9.0f) continue;  // erfc(9) / 2 < 1e-36
    const float cf = 0.5f * erfcf(x);
    if (r <= cut_cn) {
      const float t = fabsf(xi.y - xj.y) + k5;
      s_d4.add(k4 * __expf(-(t * t) / k6) * cf);
    }
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
    // right-hand side takes its square root, which is steep near 0)
    const float t = 1.0f + expf(q - m);
    c.w.cnq[ai] = (double)log1pf(expm1f(q) / t);
    c.w.dcnq[ai] = (double)(1.0f / t);
    if (c.out.d_cn) c.out.d_cn[ai] = d4;
  }
}

// ---------------------------------------------------------------- pairs

// Fused C6 + BJ two-body term in FP32, the per-pair ATM table (float4:
// r, 1/r, log(R0/r), sqrt(C6(q=0))), the direct gradient and the C6
// adjoint.  One warp per atom i, lanes over partners j.
template <bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(256) pair_fwd_mixed_kernel(Ctx c) {
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
  const float a1 = c.pf.a1, a2 = c.pf.a2, cut2 = c.pf.cut2;
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 pi = P[i];
  const float wi = c.w.w32[ai];
  const int nslot = c.w.n_slots[b];
  const int slot_i = c.w.slot[ai];
  float4 *T = c.w.ptf + (size_t)ai * N;
  float4 *Tda = PGRAD ? c.w.ptf_da + (size_t)ai * N : nullptr;
  const float alp3_log2e = c.pf.alp3 * 1.4426950408889634f;
  Acc32 e_acc, gx, gy, gz;
  float pg[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  const float fw_l = lane < NFREQ ? c.w.fw32[lane] : 0.f;  // (3/pi) w_lane
  for (int s = 0; s < nslot; ++s) {
    if (lane < NFREQ) {
      const size_t o = a32_index(b, i, s, lane, N, c.S);
      s_wa[warp][lane] = fw_l * c.w.A32[o];
      s_wa0[warp][lane] = fw_l * c.w.A032[o];
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
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      const float ir = rsqrtf(r2);
      const float r = r2 * ir;
      const float *Aj = c.w.A32 + a32_index(b, j, slot_i, 0, N, c.S);
      const float *A0j = c.w.A032 + a32_index(b, j, slot_i, 0, N, c.S);
      float c6 = 0.f, c60 = 0.f;
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) {
        c6 = fmaf(s_wa[warp][w], Aj[(size_t)w * N], c6);
        c60 = fmaf(s_wa0[warp][w], A0j[(size_t)w * N], c60);
      }
      const float sqq = SQRT3_F * pi.w * pj.w;  // sqrt(3 r4r2_i r4r2_j)
      const float qq = sqq * sqq;
      const float R0 = fmaf(a1, sqq, a2);
      const float lnR0r = logf(R0 * ir);
      T[j] = make_float4(r2, ir, alp3_log2e * lnR0r, sqrtf(c60));
      if (PGRAD) Tda[j] = make_float4(sqq / R0, 1.0f / R0, lnR0r, 0.f);
      if (r <= cut2) {
        const float r6 = r2 * r2 * r2, R02 = R0 * R0, R06 = R02 * R02 * R02;
        const float t6 = 1.0f / (r6 + R06);
        float e = s6 * c6 * t6;
        float dEdr = 6.0f * s6 * c6 * (r6 * ir) * t6 * t6;
        float K = -s6 * t6;
        float dE_dR0 = 6.0f * s6 * c6 * (R06 / R0) * t6 * t6;
        pg[0] -= wi * c6 * t6;
        if (p.has_s8) {
          const float r8 = r6 * r2, R08 = R06 * R02;
          const float t8 = 1.0f / (r8 + R08);
          const float c8 = c6 * qq;
          e += s8 * c8 * t8;
          dEdr += 8.0f * s8 * c8 * (r8 * ir) * t8 * t8;
          K -= s8 * qq * t8;
          dE_dR0 += 8.0f * s8 * c8 * (R08 / R0) * t8 * t8;
          pg[1] -= wi * c8 * t8;
        }
        if (p.has_s10) {
          const float r10 = r6 * r2 * r2, R010 = R06 * R02 * R02;
          const float t10 = 1.0f / (r10 + R010);
          const float q2 = qq * qq * (49.0f / 40.0f);
          const float c10 = c6 * q2;
          e += s10 * c10 * t10;
          dEdr += 10.0f * s10 * c10 * (r10 * ir) * t10 * t10;
          K -= s10 * q2 * t10;
          dE_dR0 += 10.0f * s10 * c10 * (R010 / R0) * t10 * t10;
          pg[2] -= wi * c10 * t10;
        }
        e_acc.add(-0.5f * e);
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
      float mine = 0.f;
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) {
        const float g = warp_sumf(gacc[w]);
        if (lane == w) mine = g;
      }
      if (lane < NFREQ) c.w.G32[(ai * c.S + s) * NFREQ + lane] = fw_l * mine;
    }
    __syncwarp();
  }
  if (GRAD && lane < NFREQ)
    for (int s = nslot; s < c.S; ++s) c.w.G32[(ai * c.S + s) * NFREQ + lane] = 0.f;
  const Acc32 ea = warp_sum_acc(e_acc);
  if (PGRAD) {
    float v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = warp_sumf(pg[k]);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * 8 + 0], 0.5 * (double)v[0]);
      atomicAdd(&c.w.pgrad[b * 8 + 1], 0.5 * (double)v[1]);
      atomicAdd(&c.w.pgrad[b * 8 + 2], 0.5 * (double)v[2]);
      atomicAdd(&c.w.pgrad[b * 8 + 3], (double)v[3]);
      atomicAdd(&c.w.pgrad[b * 8 + 4], (double)v[4]);
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
  if (lane == 0) c.out.d_energy[ai] = ea.value();
}

// ---------------------------------------------------------------- ATM

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

// Accumulation target of the per-pair / per-atom ATM adjoints.  Pair
// values go to both (j, k) and (k, j) so that the backward pair kernel reads
// rows.
template <bool SMEM>
struct AtmAcc {
  float *sS, *sP, *sE;  // shared (SMEM): upper triangle and atoms
  float *gS, *gP;       // global pair blocks [N][N]
  double *gE;           // atom energies
  int n, N;
  __device__ __forceinline__ void pair(int j, int k, float S, float P) const {
    if (SMEM) {
      const int t = tri_u(j, k, n);
      atomicAdd(&sS[t], S);
      atomicAdd(&sP[t], P);
    } else {
      atomicAdd(&gS[(size_t)j * N + k], S);
      atomicAdd(&gP[(size_t)j * N + k], P);
      atomicAdd(&gS[(size_t)k * N + j], S);
      atomicAdd(&gP[(size_t)k * N + j], P);
    }
  }
  __device__ __forceinline__ void energy(int x, float e) const {
    if (SMEM)
      atomicAdd(&sE[x], e);
    else
      atomicAdd(&gE[x], (double)e);
  }
};

// ATM energy and adjoint over triples i < j < k of one structure.  K CTAs
// share a structure (the third atom i is interleaved over them).  A warp
// takes a task (j, 32 consecutive k > j) and loops over i: lanes hold the
// (j, k) pair record in registers and read the (i, j) (broadcast) and (i, k)
// (coalesced 128-bit) records.  A pair record holds r^2, 1/r,
// alp/3 log2(R0/r) and sqrt(C6(q=0)), so the damping is one exp2 and C9 two
// products.  Per-pair dE/d(r^2) and mask-weighted triple energies
// accumulate in shared memory (SMEM, n <= 234) without the s9 factor, which
// is applied once when a CTA flushes them (FP32 global atomics, both
// triangle halves); larger structures accumulate straight into global
// memory.
template <bool SMEM, bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(PGRAD ? ATM_THREADS_PGRAD : ATM_THREADS)
    atm_mixed_kernel(Ctx c) {
  extern __shared__ float s_acc[];
  const int b = blockIdx.y;
  const int cta = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  if (n < 3) return;
  const int K = atm_ctas(n);
  if (cta >= K) return;
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
  if (SMEM) {
    for (int t = threadIdx.x; t < 2 * P + n; t += blockDim.x) s_acc[t] = 0.f;
    __syncthreads();
  }
  const int *Zb = c.w.z + (size_t)b * N;
  const float4 *T = c.w.ptf + (size_t)b * N * N;
  const float4 *Tda = PGRAD ? c.w.ptf_da + (size_t)b * N * N : nullptr;
  const float cut2 = c.pf.cut3 * c.pf.cut3;
  const float alp3 = c.pf.alp3;
  const float s9 = c.pf.s9;
  const float s9m = SMEM ? 1.f : s9;  // SMEM: s9 is applied at the flush
  const bool weighted = c.weights != nullptr;
  const float *W = c.w.w32 + (size_t)b * N;
  const size_t step = (size_t)K * N;
  float g_s9 = 0.f, g_alp = 0.f, g_a1 = 0.f, g_a2 = 0.f;
  int task = 0;
  for (int j = 1; j < n - 1; ++j) {
    for (int kc = j + 1; kc < n; kc += 32, ++task) {
      if (task % nwarps != warp || Zb[j] == 0) continue;
      const int k = kc + lane;
      const bool kok = k < n && Zb[k] != 0;
      const float4 pjk = kok ? T[(size_t)j * N + k] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float zjk = pjk.x, irjk = pjk.y, Ljk = pjk.z, cjk = pjk.w;
      const bool mjk = kok && zjk <= cut2;
      float4 dajk = make_float4(0.f, 0.f, 0.f, 0.f);
      if (PGRAD && kok) dajk = Tda[(size_t)j * N + k];
      const float wj = W[j];
      const float wk = kok ? W[k] : 0.f;
      float Sjk = 0.f, Pjk = 0.f, Ej = 0.f, Ek = 0.f;
      const float4 *Tij = T + (size_t)cta * N + j;
      const float4 *Tik = T + (size_t)cta * N + (kok ? k : j);
      for (int i = cta; i < j; i += K, Tij += step, Tik += step) {
        if (Zb[i] == 0) continue;
        const float4 pij = *Tij;
        float sij = 0.f, pe = 0.f, ei = 0.f;
        if (kok) {
          const float4 pik = *Tik;
          const bool mij = pij.x <= cut2, mik = pik.x <= cut2;
          if ((int)mij + (int)mik + (int)mjk >= 2) {
            const float x = pij.x, y = pik.x, z = zjk;
            const float ir1 = pij.y * irjk * pik.y;
            const float ir2 = ir1 * ir1;
            const float ir3 = ir1 * ir2;
            const float u = x - y, v = x + y;
            const float A = u + z, Bv = v - z, Cv = z - u;
            const float sfac = A * Bv * Cv;
            const float ang = ir3 * fmaf(0.375f * sfac, ir2, 1.0f);
            const float ta = exp2f(pij.z + pik.z + Ljk);
            const float fd = __fdividef(1.0f, fmaf(6.0f, ta, 1.0f));
            const float c9 = pij.w * pik.w * cjk;
            const float eu = c9 * fd * ang;  // triple energy without s9
            const float e = s9m * eu;
            float wgt;
            if (mij & mik & mjk) {
              const float third = e * (1.0f / 3.0f);
              ei = third;
              Ej += third;
              Ek += third;
              wgt = ((weighted ? W[i] : 1.f) + wj + wk) * (1.0f / 3.0f);
            } else {
              const float fij = mij, fik = mik, fjk = mjk;
              const float mi = fjk * (fij + fik), mj = fik * (fij + fjk), mk = fij * (fik + fjk);
              const float sixth = e * (1.0f / 6.0f);
              ei = sixth * mi;
              Ej += sixth * mj;
              Ek += sixth * mk;
              wgt = ((weighted ? W[i] : 1.f) * mi + wj * mj + wk * mk) * (1.0f / 6.0f);
            }
            if (GRAD) {
              const float kc9 = s9m * c9;
              const float dfl = alp3 * fd * (1.0f - fd);  // = 6 alp/3 ta fd^2
              const float Q = 2.0f * ir3 - 5.0f * ang;
              const float U = 0.375f * kc9 * fd * ir2 * ir3;
              const float V = 0.5f * kc9 * fmaf(fd, Q, ang * dfl);
              const float BC = Bv * Cv, AC = A * Cv, AB = A * Bv;
              const float dex = fmaf(U, BC + AC - AB, V * pij.y * pij.y);
              const float dey = fmaf(U, AC + AB - BC, V * pik.y * pik.y);
              const float dez = fmaf(U, BC + AB - AC, V * irjk * irjk);
              sij = wgt * dex;
              Sjk = fmaf(wgt, dez, Sjk);
              const float we = wgt * e;
              pe = we;
              Pjk += we;
              acc.pair(i, k, wgt * dey, we);
              if (PGRAD) {
                const float4 daij = Tda[(size_t)i * N + j];
                const float4 daik = Tda[(size_t)i * N + k];
                const float lsum = daij.z + daik.z + dajk.z;
                const float dfd = -fd * (1.0f - fd);  // d fd / d(alp/3 sum log(R0/r))
                g_s9 += wgt * eu;
                g_alp += wgt * s9 * c9 * ang * dfd * lsum * (1.0f / 3.0f);
                const float dfa = wgt * s9 * c9 * ang * dfd * alp3;
                g_a1 += dfa * (daij.x + daik.x + dajk.x);
                g_a2 += dfa * (daij.y + daik.y + dajk.y);
              }
            }
          }
        }
        // (i, j) and E_i: one value per warp
        if (GRAD) {
          sij = warp_sumf(sij);
          pe = warp_sumf(pe);
        }
        ei = warp_sumf(ei);
        if (lane == 0) {
          if (ei != 0.f) acc.energy(i, ei);
          if (GRAD && (sij != 0.f || pe != 0.f)) acc.pair(i, j, sij, pe);
        }
      }
      if (GRAD && kok && (Sjk != 0.f || Pjk != 0.f)) acc.pair(j, k, Sjk, Pjk);
      const float ej = warp_sumf(Ej);
      if (lane == 0 && ej != 0.f) acc.energy(j, ej);
      if (kok && Ek != 0.f) acc.energy(k, Ek);
    }
  }
  if (PGRAD) {
    g_s9 = warp_sumf(g_s9);
    g_alp = warp_sumf(g_alp);
    g_a1 = warp_sumf(g_a1);
    g_a2 = warp_sumf(g_a2);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * 8 + 3], (double)g_a1);
      atomicAdd(&c.w.pgrad[b * 8 + 4], (double)g_a2);
      atomicAdd(&c.w.pgrad[b * 8 + 5], (double)g_s9);
      atomicAdd(&c.w.pgrad[b * 8 + 6], (double)g_alp);
    }
  }
  if (SMEM) {
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
      const float ev = acc.sE[x] * s9;
      if (ev != 0.f) atomicAdd(&c.w.e3[(size_t)b * N + x], (double)ev);  // once per atom
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
  const float4 px = P[x];
  const int nslot = c.w.n_slots[b];
  const int slot_x = c.w.slot[ax];
  const size_t base = (size_t)b * N * N;
  const float4 *T = c.w.ptf + base + (size_t)x * N;
  const float fw_l = lane < NFREQ ? c.w.fw32[lane] : 0.f;  // (3/pi) w_lane
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
      const float4 py = P[y];
      gx.add(2.0f * S * (px.x - py.x));
      gy.add(2.0f * S * (px.y - py.y));
      gz.add(2.0f * S * (px.z - py.z));
      if (Pv != 0.f) {
        const float cc = T[y].w;
        const float D = Pv / (2.0f * cc * cc);
        const float *A0y = c.w.A032 + a32_index(b, y, slot_x, 0, N, c.S);
#pragma unroll
        for (int w = 0; w < NFREQ; ++w) gacc[w] = fmaf(D, A0y[(size_t)w * N], gacc[w]);
      }
    }
    float mine = 0.f;
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) {
      const float g = warp_sumf(gacc[w]);
      if (lane == w) mine = g;
    }
    // chain rule to CN and q for this slot (lane = frequency)
    if (lane < NFREQ) {
      const size_t o = (ax * c.S + s) * NFREQ + lane;
      const float g0w = fw_l * mine;
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
  const float kcn = c.pf.kcn, k4 = c.pf.k4, k5 = c.pf.k5, k6 = c.pf.k6;
  const float cut_cn = c.pf.cut_cn, cut_q = c.pf.cut_q;
  const float4 *P = c.w.pos32 + (size_t)b * N;
  const float4 *X = c.w.aux32 + (size_t)b * N;
  const float4 *D = c.w.adj32 + (size_t)b * N;
  const float4 pi = P[i], xi = X[i], di = D[i];
  Acc32 gx, gy, gz;
  for (int j = lane; j < n; j += 32) {
    const size_t aj = (size_t)b * N + j;
    if (j == i || c.w.z[aj] == 0) continue;
    const float4 pj = P[j], xj = X[j], dj = D[j];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ir = rsqrtf(r2);
    const float r = r2 * ir;
    float dEdr = 0.f;
    const float r0 = xi.x + xj.x;
    const float xx = kcn * (r / r0 - 1.0f);
    if (xx < 9.0f) {
      const float dcf = -kcn / r0 * INV_SQRT_PI_F * __expf(-xx * xx);
      if (r <= cut_cn) {
        const float t = fabsf(xi.y - xj.y) + k5;
        dEdr += (di.x + dj.x) * k4 * __expf(-(t * t) / k6) * dcf;
      }
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

// FP64 reciprocal square root: FP32 estimate refined by two Newton steps
// y <- y (3 - a y^2) / 2 (quadratic convergence: 2^-22 -> 2^-44 -> below
// one FP64 ulp), for a > 0 in the FP32 range.
__device__ __forceinline__ double rsqrt_newton(double a) {
  double y = (double)rsqrtf((float)a);
  y = y * (1.5 - 0.5 * a * y * y);
  y = y * (1.5 - 0.5 * a * y * y);
  return y;
}

// Dense FP64 EEQ matrix of the real atoms (rows / columns in the order of
// ``cidx``, leading dimension N).  One thread per lower-triangle entry,
// mirrored; all structures at once.  erf(x) is exactly 1.0 in FP64 for
// x > 6.5, where the entry is 1/r.
__global__ void eeq_build_mixed_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n * (n + 1) / 2) return;
  int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while (tri_index(i + 1, 0) <= t) ++i;
  while (i > 0 && tri_index(i, 0) > t) --i;
  const int j = (int)(t - tri_index(i, 0));
  const size_t ai = (size_t)b * N + i, aj = (size_t)b * N + j;
  const int ci = c.w.cidx[ai], cj = c.w.cidx[aj];
  if (ci < 0 || cj < 0) return;
  const int zi = c.w.z[ai], zj = c.w.z[aj];
  double *A = c.w.eeq_A64 + (size_t)b * N * N;
  if (i == j) {
    A[(size_t)ci * N + ci] = c.tab.eeq_eta[zi] + SQRT_2_OVER_PI / c.tab.eeq_rad[zi];
    return;
  }
  const double *pi = c.positions + 3 * ai, *pj = c.positions + 3 * aj;
  const double dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
  const double r2 = dx * dx + dy * dy + dz * dz;
  const double ir = rsqrt_newton(r2);
  const double ra = c.tab.eeq_rad[zi], rb = c.tab.eeq_rad[zj];
  const double x = r2 * ir * rsqrt_newton(ra * ra + rb * rb);
  const double v = (x > 6.5 ? 1.0 : erf(x)) * ir;
  A[(size_t)ci * N + cj] = v;
  A[(size_t)cj * N + ci] = v;
}

// Shared-memory layout of the mixed EEQ kernels (in doubles):
//   idx      int[N]               (N/2 + 1 doubles)
//   x        double[2N]           solution (two right-hand sides)
//   rx       double[2N]           FP64 residual
//   bb       double[2N]           right-hand sides (b, 1) in FP64
//   vf       float[2N]            FP32 correction (N doubles)
//   invd     float[N]             reciprocal diagonal of the factor
//   L        float[N(N+1)/2]      FP32 factor (SMEM only)
__host__ __device__ inline size_t eeq_mixed_vec_doubles(int N) {
  return (size_t)(N + 1) / 2 + 1 + 6 * (size_t)N + (size_t)N + (size_t)(N + 1) / 2 + 1;
}

constexpr int PB = 32;  // panel width of the blocked factorisation and solves

// Blocked right-looking Cholesky (panels of 32 columns) of the packed lower
// m x m FP32 matrix L, in place; invd receives 1 / L_kk.  Three barriers per
// panel.  A non-positive pivot sets *bad and continues with pivot 1.
__device__ void chol_blocked(float *L, float *invd, int m, int *bad) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  for (int k0 = 0; k0 < m; k0 += PB) {
    const int kb = min(PB, m - k0);
    if (warp == 0) {  // diagonal block: lane r owns row k0 + r
      for (int cc = 0; cc < kb; ++cc) {
        float d = L[tri_index(k0 + cc, k0 + cc)];
        if (!(d > 0.f)) {
          if (lane == 0) *bad = 1;
          d = 1.f;
        }
        d = sqrtf(d);
        const float inv = 1.0f / d;
        __syncwarp();
        if (lane == 0) {
          L[tri_index(k0 + cc, k0 + cc)] = d;
          invd[k0 + cc] = inv;
        }
        float lrc = 0.f;
        if (lane > cc && lane < kb) {
          lrc = L[tri_index(k0 + lane, k0 + cc)] * inv;
          L[tri_index(k0 + lane, k0 + cc)] = lrc;
        }
        __syncwarp();
        if (lane > cc && lane < kb) {
          float *row = L + tri_index(k0 + lane, 0);
          for (int c2 = cc + 1; c2 <= lane; ++c2)
            row[k0 + c2] = fmaf(-lrc, L[tri_index(k0 + c2, k0 + cc)], row[k0 + c2]);
        }
        __syncwarp();
      }
    }
    __syncthreads();
    // panel below the block: rows solve against the block's transpose
    for (int i = k0 + kb + tid; i < m; i += nt) {
      float *row = L + tri_index(i, 0);
      for (int cc = 0; cc < kb; ++cc) {
        float v = row[k0 + cc];
        const float *lc = L + tri_index(k0 + cc, 0);
        for (int c2 = 0; c2 < cc; ++c2) v = fmaf(-row[k0 + c2], lc[k0 + c2], v);
        row[k0 + cc] = v * invd[k0 + cc];
      }
    }
    __syncthreads();
    // trailing update of the lower triangle right of the panel
    const int t0 = k0 + kb;
    const int nrem = m - t0;
    const int ntri = nrem * (nrem + 1) / 2;
    for (int t = tid; t < ntri; t += nt) {
      int ii = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
      while ((ii + 1) * (ii + 2) / 2 <= t) ++ii;
      while (ii > 0 && ii * (ii + 1) / 2 > t) --ii;
      const int jj = t - ii * (ii + 1) / 2;
      const float *ri = L + tri_index(t0 + ii, 0) + k0;
      const float *rj = L + tri_index(t0 + jj, 0) + k0;
      float acc = 0.f;
      for (int cc = 0; cc < kb; ++cc) acc = fmaf(ri[cc], rj[cc], acc);
      L[tri_index(t0 + ii, t0 + jj)] -= acc;
    }
    __syncthreads();
  }
}

// Blocked solves with the packed factor (all threads of the block call
// them): forward L z = v, backward L^T x = z, ``nr`` right-hand sides of
// leading dimension ldv.  Within a 32-row block the recurrence runs on one
// warp with shuffles; the rest of the rows are updated by all threads.
__device__ void fwd_solve_blocked(const float *L, const float *invd, float *v, int ldv, int m,
                                  int nr) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  for (int k0 = 0; k0 < m; k0 += PB) {
    const int kb = min(PB, m - k0);
    if (warp == 0) {
      float x0 = lane < kb ? v[k0 + lane] : 0.f;
      float x1 = (nr == 2 && lane < kb) ? v[ldv + k0 + lane] : 0.f;
      for (int cc = 0; cc < kb; ++cc) {
        const float inv = invd[k0 + cc];
        const float xc0 = __shfl_sync(0xffffffffu, x0, cc) * inv;
        const float xc1 = __shfl_sync(0xffffffffu, x1, cc) * inv;
        if (lane == cc) {
          x0 = xc0;
          x1 = xc1;
        } else if (lane > cc && lane < kb) {
          const float l = L[tri_index(k0 + lane, k0 + cc)];
          x0 = fmaf(-l, xc0, x0);
          x1 = fmaf(-l, xc1, x1);
        }
      }
      if (lane < kb) {
        v[k0 + lane] = x0;
        if (nr == 2) v[ldv + k0 + lane] = x1;
      }
    }
    __syncthreads();
    const int rows = m - k0 - kb;
    for (int t = tid; t < rows * nr; t += nt) {
      const int r = t / rows, i = k0 + kb + t % rows;
      const float *row = L + tri_index(i, 0) + k0;
      const float *xv = v + r * ldv + k0;
      float acc = 0.f;
      for (int cc = 0; cc < kb; ++cc) acc = fmaf(row[cc], xv[cc], acc);
      v[r * ldv + i] -= acc;
    }
    __syncthreads();
  }
}

__device__ void bwd_solve_blocked(const float *L, const float *invd, float *v, int ldv, int m,
                                  int nr) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  if (m <= 0) return;
  for (int k0 = ((m - 1) / PB) * PB; k0 >= 0; k0 -= PB) {
    const int kb = min(PB, m - k0);
    if (warp == 0) {
      float x0 = lane < kb ? v[k0 + lane] : 0.f;
      float x1 = (nr == 2 && lane < kb) ? v[ldv + k0 + lane] : 0.f;
      for (int cc = kb - 1; cc >= 0; --cc) {
        const float inv = invd[k0 + cc];
        const float xc0 = __shfl_sync(0xffffffffu, x0, cc) * inv;
        const float xc1 = __shfl_sync(0xffffffffu, x1, cc) * inv;
        if (lane == cc) {
          x0 = xc0;
          x1 = xc1;
        } else if (lane < cc) {
          const float l = L[tri_index(k0 + cc, k0 + lane)];
          x0 = fmaf(-l, xc0, x0);
          x1 = fmaf(-l, xc1, x1);
        }
      }
      if (lane < kb) {
        v[k0 + lane] = x0;
        if (nr == 2) v[ldv + k0 + lane] = x1;
      }
    }
    __syncthreads();
    for (int t = tid; t < k0 * nr; t += nt) {
      const int r = t / k0, i = t % k0;
      const float *xv = v + r * ldv + k0;
      float acc = 0.f;
      for (int cc = 0; cc < kb; ++cc) acc = fmaf(L[tri_index(k0 + cc, i)], xv[cc], acc);
      v[r * ldv + i] -= acc;
    }
    __syncthreads();
  }
}

constexpr int EEQ_REFINE_MAX = 8;
constexpr double EEQ_RESIDUAL_TOL = 1e-10;

// rx = bb - A x for ``nr`` right-hand sides; one warp per row of the dense
// FP64 matrix (coalesced).  Returns max |rx| over the block.
__device__ double eeq_residual(const double *A64, const double *x, const double *bb, double *rx,
                               int m, int N, int nr, double *s_red) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double mx = 0.0;
  for (int k = warp; k < m; k += nw) {
    const double *row = A64 + (size_t)k * N;
    double a0 = 0.0, a1 = 0.0;
    for (int l = lane; l < m; l += 32) {
      const double a = row[l];
      a0 += a * x[l];
      if (nr == 2) a1 += a * x[N + l];
    }
    a0 = warp_sum(a0);
    if (nr == 2) a1 = warp_sum(a1);
    if (lane == 0) {
      const double r0 = bb[k] - a0;
      rx[k] = r0;
      mx = fmax(mx, fabs(r0));
      if (nr == 2) {
        const double r1 = bb[N + k] - a1;
        rx[N + k] = r1;
        mx = fmax(mx, fabs(r1));
      }
    }
  }
  if (lane == 0) s_red[warp] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < nw; ++w) v = fmax(v, s_red[w]);
    s_red[32] = v;
  }
  __syncthreads();
  const double out = s_red[32];
  __syncthreads();
  return out;
}

// FP32 factor + FP64 refinement: x (nr columns) <- A^-1 bb.
__device__ void eeq_refined_solve(const float *L, const float *invd, const double *A64,
                                  double *x, double *rx, const double *bb, float *vf, int m,
                                  int N, int nr, double *s_red) {
  for (int t = threadIdx.x; t < m * nr; t += blockDim.x) {
    const int r = t / m, k = t % m;
    x[r * N + k] = 0.0;
    rx[r * N + k] = bb[r * N + k];
  }
  __syncthreads();
  for (int it = 0; it < EEQ_REFINE_MAX; ++it) {
    for (int t = threadIdx.x; t < m * nr; t += blockDim.x) {
      const int r = t / m, k = t % m;
      vf[r * N + k] = (float)rx[r * N + k];
    }
    __syncthreads();
    fwd_solve_blocked(L, invd, vf, N, m, nr);
    bwd_solve_blocked(L, invd, vf, N, m, nr);
    for (int t = threadIdx.x; t < m * nr; t += blockDim.x) {
      const int r = t / m, k = t % m;
      x[r * N + k] += (double)vf[r * N + k];
    }
    __syncthreads();
    if (eeq_residual(A64, x, bb, rx, m, N, nr, s_red) < EEQ_RESIDUAL_TOL) break;
  }
}

template <bool SMEM>
__global__ void __launch_bounds__(512) eeq_mixed_kernel(Ctx c) {
  extern __shared__ double s_dyn[];
  const int b = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_m;
  __shared__ double s_red[33];
  int *s_idx = reinterpret_cast<int *>(s_dyn);
  double *x = s_dyn + (N + 1) / 2 + 1;
  double *rx = x + 2 * N;
  double *bb = rx + 2 * N;
  float *vf = reinterpret_cast<float *>(bb + 2 * N);
  float *invd = vf + 2 * N;
  const size_t NN2 = (size_t)N * (N + 1) / 2;
  float *L = SMEM ? invd + N + 2 : c.w.eeq_L32 + (size_t)b * NN2;
  const double *A64 = c.w.eeq_A64 + (size_t)b * N * N;
  const int m = compact_real_atoms(c, b, n, s_idx, &s_m);
  const int *Zb = c.w.z + (size_t)b * N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  // FP32 copy of the lower triangle, one warp per row
  for (int ii = warp; ii < m; ii += nw) {
    const double *row = A64 + (size_t)ii * N;
    float *lrow = L + tri_index(ii, 0);
    for (int jj = lane; jj <= ii; jj += 32) lrow[jj] = (float)row[jj];
  }
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const int ia = s_idx[k];
    const int z = Zb[ia];
    const double cq = c.w.cnq[(size_t)b * N + ia];
    const double sq = cq > 0.0 ? sqrt(cq) : 0.0;
    bb[k] = -c.tab.eeq_chi[z] + c.tab.eeq_kcn[z] * sq;
    bb[N + k] = 1.0;
  }
  __syncthreads();
  chol_blocked(L, invd, m, &s_bad);
  if (threadIdx.x == 0 && s_bad) set_status(c.w.status, D4_ERR_EEQ_SINGULAR);
  eeq_refined_solve(L, invd, A64, x, rx, bb, vf, m, N, 2, s_red);
  if (warp == 0) {
    double sx = 0.0, sy = 0.0;
    for (int k = lane; k < m; k += 32) {
      sx += x[k];
      sy += x[N + k];
    }
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    if (lane == 0) {
      const double lam = m > 0 ? (sx - c.charge[b]) / sy : 0.0;
      c.w.eeq_sum[2 * b] = sy;
      c.w.eeq_sum[2 * b + 1] = lam;
      s_red[32] = lam;
    }
  }
  __syncthreads();
  const double lam = s_red[32];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    c.w.q[(size_t)b * N + i] = 0.0;
    c.w.eeq_y[(size_t)b * N + i] = 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const size_t a = (size_t)b * N + s_idx[k];
    c.w.q[a] = x[k] - lam * x[N + k];
    c.w.eeq_y[a] = x[N + k];
  }
  if (SMEM) {
    float *G = c.w.eeq_L32 + (size_t)b * NN2;
    const size_t tri_m = (size_t)m * (m + 1) / 2;
    for (size_t t = threadIdx.x; t < tri_m; t += blockDim.x) G[t] = L[t];
  }
}

// Adjoint: A u = dE/dq by the FP32 factor + FP64 refinement, w = u - nu y.
__global__ void __launch_bounds__(512) eeq_adjoint_mixed_kernel(Ctx c) {
  extern __shared__ double s_dyn[];
  const int b = blockIdx.x;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  __shared__ int s_m;
  __shared__ double s_red[33];
  int *s_idx = reinterpret_cast<int *>(s_dyn);
  double *x = s_dyn + (N + 1) / 2 + 1;
  double *rx = x + 2 * N;
  double *bb = rx + 2 * N;
  float *vf = reinterpret_cast<float *>(bb + 2 * N);
  float *invd = vf + 2 * N;
  const size_t NN2 = (size_t)N * (N + 1) / 2;
  const float *L = c.w.eeq_L32 + (size_t)b * NN2;
  const double *A64 = c.w.eeq_A64 + (size_t)b * N * N;
  const int m = compact_real_atoms(c, b, n, s_idx, &s_m);
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    bb[k] = c.w.dEdq[(size_t)b * N + s_idx[k]];
    invd[k] = 1.0f / L[tri_index(k, k)];
  }
  __syncthreads();
  eeq_refined_solve(L, invd, A64, x, rx, bb, vf, m, N, 1, s_red);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    double su = 0.0;
    for (int k = lane; k < m; k += 32) su += x[k];
    su = warp_sum(su);
    if (lane == 0) s_red[32] = m > 0 ? su / c.w.eeq_sum[2 * b] : 0.0;
  }
  __syncthreads();
  const double nu = s_red[32];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    c.w.eeq_w[(size_t)b * N + i] = 0.0;
    c.w.dEdcnq[(size_t)b * N + i] = 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const size_t a = (size_t)b * N + s_idx[k];
    const double w = x[k] - nu * c.w.eeq_y[a];
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

template <bool SMEM, bool GRAD, bool PGRAD>
static void launch_atm(const Ctx &c, cudaStream_t st, size_t smem) {
  if (SMEM)
    cudaFuncSetAttribute(atm_mixed_kernel<SMEM, GRAD, PGRAD>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int threads = PGRAD ? ATM_THREADS_PGRAD : ATM_THREADS;
  atm_mixed_kernel<SMEM, GRAD, PGRAD><<<dim3(ATM_KMAX, c.B), threads, smem, st>>>(c);
}

int launch_mixed(const Ctx &c, cudaStream_t st) {
  const int B = c.B, N = c.N;
  const dim3 atoms((N + 7) / 8, B);
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  const bool pgrad = (c.flags & D4_FLAG_PARAM_GRAD) != 0;
  const bool eeq = (c.flags & D4_FLAG_CHARGES_IN) == 0;
  timing_next_call();
  stage_begin(ST_PREP, st);
  launch_prep(c, st);
  stage_end(ST_PREP, st);
  stage_begin(ST_CN, st);
  cn_mixed_kernel<<<atoms, 256, 0, st>>>(c);
  stage_end(ST_CN, st);
  const size_t vec_bytes = 8 * eeq_mixed_vec_doubles(N);
  const size_t tri_bytes = (size_t)4 * ((size_t)N * (N + 1) / 2);
  const bool eeq_smem = vec_bytes + tri_bytes <= 220 * 1024;
  stage_begin(ST_EEQ, st);
  if (eeq) {
    eeq_build_mixed_kernel<<<dim3((unsigned)(((size_t)N * (N + 1) / 2 + 255) / 256), B), 256, 0,
                             st>>>(c);
    if (eeq_smem) {
      cudaFuncSetAttribute(eeq_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(vec_bytes + tri_bytes));
      eeq_mixed_kernel<true><<<B, 512, vec_bytes + tri_bytes, st>>>(c);
    } else {
      cudaFuncSetAttribute(eeq_mixed_kernel<false>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vec_bytes);
      eeq_mixed_kernel<false><<<B, 512, vec_bytes, st>>>(c);
    }
  } else {
    launch_charges_in(c, st);
  }
  stage_end(ST_EEQ, st);
  stage_begin(ST_WEIGHTS, st);
  launch_weights(c, st);
  const size_t BN = (size_t)B * N;
  size_t conv_blocks = (BN * c.S * NFREQ + 255) / 256;
  if (conv_blocks > 65535) conv_blocks = 65535;
  mixed_convert_kernel<<<(unsigned)conv_blocks, 256, 0, st>>>(c);
  stage_end(ST_WEIGHTS, st);
  stage_begin(ST_PAIR_FWD, st);
  if (pgrad)
    pair_fwd_mixed_kernel<true, true><<<atoms, 256, 0, st>>>(c);
  else if (grad)
    pair_fwd_mixed_kernel<true, false><<<atoms, 256, 0, st>>>(c);
  else
    pair_fwd_mixed_kernel<false, false><<<atoms, 256, 0, st>>>(c);
  stage_end(ST_PAIR_FWD, st);
  // ATM: shared-memory accumulation when the largest structure fits
  const size_t atm_smem = (size_t)4 * ((size_t)N * (N - 1) + N);
  const bool atm_sm = atm_smem <= 220 * 1024;
  stage_begin(ST_ATM, st);
  if (atm_sm) {
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
    pair_atm_bwd_mixed_kernel<<<atoms, 256, 0, st>>>(c);
    stage_end(ST_PAIR_ATM_BWD, st);
    if (eeq) {
      stage_begin(ST_EEQ_ADJ, st);
      cudaFuncSetAttribute(eeq_adjoint_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)vec_bytes);
      eeq_adjoint_mixed_kernel<<<B, 512, vec_bytes, st>>>(c);
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
