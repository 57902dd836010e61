// Precision form, D4 model: the C6 contraction on the tensor cores, fused
// with the BJ two-body term.
//
// C6_ij = sum_w A'_i(w) A'_j(w) (model/d4.py:268-289 through
// utils.py:33-94; A' = weighted reference polarisabilities times
// sqrt((3/pi) w_w)) and C6_ij at q = 0 are, per structure, the products of
// an n x 23 matrix with its transpose.  A CTA takes 128 atoms i of one
// structure (the MMA's M) and walks over the partners j in chunks of 32 (its
// N): tcgen05 kind::tf32 MMAs form the 128 x 32 tiles of C6 and C6(q=0) in
// tensor memory, one thread issuing them.  The products are exact: every
// row of A' is cut into three 9-bit integer digits under a power-of-two row
// scale, and the tensor cores sum digit products class by class (integers
// below 2^24, exact in their FP32 accumulators; K = 23 padded to 24, three
// k-steps, six digit products per k-step); the epilogue combines the three
// class sums in FP32.  The epilogue reads the tiles back with tcgen05.ld
// (thread = atom i, two threads per atom for the two column halves) and
// evaluates the rational damping, the energy, the direct gradient, the C6
// adjoint dE/dA'_i and the ATM pair record of every pair (i, j) -- the C6
// matrices never reach global memory.  Everything after the contraction is
// the arithmetic of pair_fwd_mixed_kernel (the D4S model keeps that kernel:
// its C6 does not factorise into one product).
#include <float.h>

#include "d4_common.cuh"
#include "d4_kernels.cuh"
#include "d4_tc.cuh"

namespace d4 {

constexpr int TC_M = 128;       // atoms i per CTA (MMA M, tensor-memory lanes)
constexpr int TC_NJ = 32;       // partners j per chunk (MMA N)
constexpr int TC_K = 24;        // frequencies, 23 padded to three k-steps of 8
constexpr int TC_THREADS = 256; // two threads per atom i (column halves of a chunk)
constexpr int TC_LBO = 128;     // bytes between core matrices along K
constexpr int TC_SBO = (TC_K / 4) * 128;  // bytes between groups of 8 rows
constexpr int TC_COLS = 256;    // tensor memory: 3 digit classes x 32 columns per matrix,
                                // C6 at +0, C6(q=0) at +96
constexpr int TC_NRED = 38;     // per-atom partial values combined between halves

// byte offset of element (row r, k) in the canonical K-major layout
__device__ __forceinline__ int kmaj_off(int r, int k) {
  return (r >> 3) * TC_SBO + (k >> 2) * TC_LBO + (r & 7) * 16 + (k & 3) * 4;
}

struct TcSmem {
  float a[2][3][TC_M * TC_K];    // A operands: matrix (A', A0'), digit, canonical layout
  float bm[2][3][TC_NJ * TC_K];  // B operands of the chunk
  float aj[TC_NJ][TC_K];         // A'_j in FP32 (C6 adjoint)
  float sa[2][TC_M];             // row scales 2^(e - 9) of the A rows
  float sb[2][TC_NJ];            // and of the chunk's rows
  float4 pj[TC_NJ], lj[TC_NJ];
  int zj[TC_NJ];
  float wj[TC_NJ];
  unsigned long long mbar;
  uint32_t tmem;
};

// 2^e > x for every x of a row with maximum mx (frexp exponent; 0 for 0).
__device__ __forceinline__ int row_exponent(float mx) {
  int e = 0;
  frexpf(mx, &e);
  return mx > 0.f ? e : 0;
}

// x = 2^e (d1 2^-9 + d2 2^-18 + d3 2^-27) with integer digits (round to
// nearest at each step, so |d2|, |d3| <= 256); every step is exact in FP32.
// The digits go to byte offset ``off`` of the three planes.
__device__ __forceinline__ void store_digits(float *p1, float *p2, float *p3, int off, float x,
                                             int e) {
  const float y = ldexpf(x, 9 - e);
  const float d1 = rintf(y);
  const float r1 = (y - d1) * 512.f;
  const float d2 = rintf(r1);
  const float d3 = rintf((r1 - d2) * 512.f);
  *reinterpret_cast<float *>(reinterpret_cast<char *>(p1) + off) = d1;
  *reinterpret_cast<float *>(reinterpret_cast<char *>(p2) + off) = d2;
  *reinterpret_cast<float *>(reinterpret_cast<char *>(p3) + off) = d3;
}

size_t pair_fwd_tc_smem() { return sizeof(TcSmem); }

template <bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(TC_THREADS, 2) pair_fwd_tc_kernel(Ctx c) {
  extern __shared__ __align__(128) unsigned char s_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(s_raw);
  const int b = blockIdx.y;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  const int i0 = blockIdx.x * TC_M;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;
  const int row = quad * 32 + lane;  // tensor-memory lane of this thread
  // A tile of m <= 64 (32) atoms holds each atom in 2 (4) rows of the MMA's
  // 128, so that 4 (8) threads share an atom's partners instead of 2 and no
  // lane idles: copies of MR = 128 / D rows, thread column group cg of 2 D
  // (warp-uniform: a copy spans whole lane quadrants)
  const int mt = n - i0;  // atoms of the tile (if fewer than TC_M; <= 0: padding only)
  const int D = (mt <= 0 || mt > 64) ? 1 : (mt <= 32 ? 4 : 2);
  const int MR = TC_M / D;
  const int cg = half * D + row / MR;
  const int i = i0 + row % MR;
  const size_t bN = (size_t)b * N;
  const size_t ai = bN + i;
  const int zi = (i < n) ? c.w.z[ai] : 0;
  const bool real = zi != 0;
  // partners j of this CTA: chunks [ch0, ch1) of 32; with several CTAs per
  // tile (gridDim.z > 1, large structures) the outputs were zeroed by the
  // launcher and every CTA adds its partial sums atomically
  const int nsplit = gridDim.z;
  const int nch = (n + TC_NJ - 1) / TC_NJ;
  const int ch0 = (int)((long long)blockIdx.z * nch / nsplit);
  const int ch1 = (int)((long long)(blockIdx.z + 1) * nch / nsplit);
  if (nsplit > 1 && (i0 >= n || ch0 >= ch1)) return;
  if (i0 >= n) {  // a tile of padding only (D = 1)
    if (half == 0 && i < N) {
      c.out.d_energy[ai] = 0.0;
      if (GRAD) {
        c.out.d_gradient[3 * ai] = 0.0;
        c.out.d_gradient[3 * ai + 1] = 0.0;
        c.out.d_gradient[3 * ai + 2] = 0.0;
        for (int w = 0; w < NFREQ; ++w) c.w.G32[ai * NFREQ + w] = 0.f;
      }
    }
    return;
  }
  if (nsplit == 1)  // atoms i0 + MR .. i0 + 127 of a duplicated tile: padding
    for (int a = MR + tid; a < TC_M && i0 + a < N; a += TC_THREADS) {
      const size_t ap = bN + i0 + a;
      c.out.d_energy[ap] = 0.0;
      if (GRAD) {
        c.out.d_gradient[3 * ap] = 0.0;
        c.out.d_gradient[3 * ap + 1] = 0.0;
        c.out.d_gradient[3 * ap + 2] = 0.0;
        for (int w = 0; w < NFREQ; ++w) c.w.G32[ap * NFREQ + w] = 0.f;
      }
    }
  const uint32_t mbar = tc::smem_u32(&S.mbar);
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(&S.tmem), TC_COLS);
  if (tid == 0) tc::mbar_init(mbar, 1);
  // A operands: A'(w) and A0'(w) of the tile's atoms as digits under a
  // power-of-two scale per row and matrix
  const float *A32 = c.w.A32 + bN * NFREQ;  // [w][N] of structure b (one slot)
  const float *A032 = c.w.A032 + bN * NFREQ;
  __shared__ int s_ea[2][TC_M];
  {
    const int m = tid / TC_M, r = tid % TC_M;  // 256 threads: one per (matrix, row)
    const int ii = i0 + r % MR;
    const float *src = m == 0 ? A32 : A032;
    float mx = 0.f;
    if (ii < n && c.w.z[bN + ii] != 0)
      for (int k = 0; k < NFREQ; ++k) mx = fmaxf(mx, src[(size_t)k * N + ii]);
    const int e = row_exponent(mx);
    s_ea[m][r] = e;
    S.sa[m][r] = ldexpf(1.f, e - 9);
  }
  __syncthreads();
  for (int t = tid; t < 2 * TC_M * TC_K; t += TC_THREADS) {
    const int m = t / (TC_M * TC_K), rk = t % (TC_M * TC_K);
    const int r = rk % TC_M, k = rk / TC_M;
    const int ii = i0 + r % MR;
    float v = 0.f;
    if (k < NFREQ && ii < n && c.w.z[bN + ii] != 0)
      v = (m == 0 ? A32 : A032)[(size_t)k * N + ii];
    store_digits(S.a[m][0], S.a[m][1], S.a[m][2], kmaj_off(r, k), v, s_ea[m][r]);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;

  const d4_params_t &p = c.par;
  const float s6 = c.pf.s6, s8 = c.pf.s8, s10 = c.pf.s10;
  const float cut2 = c.pf.cut2;
  const float4 *P = c.w.pos32 + bN;
  const float4 *PL = c.w.pos32lo + bN;
  const float4 pi = real ? P[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 li = real ? PL[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float wi = real ? c.w.w32[ai] : 0.f;
  float4 *Tt = c.w.ptf + bN * N;  // written transposed: T[j][i], coalesced over i
  float4 *Tdat = PGRAD ? c.w.ptf_da + bN * N : nullptr;
  const float alp3 = c.pf.alp3;
  const bool tabled = c.r4r2_in == nullptr;
  const double sref = p.s6 != 0.0 ? p.s6 : 1.0;
  const dfl rho10 = df_from(p.has_s10 ? p.s10 / sref : 0.0);
  const float rho6 = p.s6 != 0.0 ? 1.f : 0.f;
  Acc32 e_acc, e8_acc, gx, gy, gz;
  float pg[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float gacc[NFREQ];
#pragma unroll
  for (int w = 0; w < NFREQ; ++w) gacc[w] = 0.f;
  float r2mx = 0.f;  // largest r^2 of this thread's pairs (the ATM's far-atom test)

  constexpr uint32_t IDESC = tc::idesc_tf32(TC_M, TC_NJ);
  const uint32_t a_base = tc::smem_u32(&S.a[0][0]);
  const uint32_t b_base = tc::smem_u32(&S.bm[0][0]);
  const uint32_t t_lane = (uint32_t)(quad * 32) << 16;
  uint32_t parity = 0;
  bool timed_out = false;
  const bool test_timeout = (c.flags & D4_FLAG_TEST_TIMEOUT) != 0;
  for (int j0 = ch0 * TC_NJ; j0 < ch1 * TC_NJ; j0 += TC_NJ) {
    // B operands (digits under per-row scales) and partner data of the chunk
    __shared__ int s_eb[2][TC_NJ];
    if (tid < 2 * TC_NJ) {
      const int m = tid / TC_NJ, r = tid % TC_NJ;
      const int jj = j0 + r;
      const float *src = m == 0 ? A32 : A032;
      float mx = 0.f;
      if (jj < n && c.w.z[bN + jj] != 0)
        for (int k = 0; k < NFREQ; ++k) mx = fmaxf(mx, src[(size_t)k * N + jj]);
      const int e = row_exponent(mx);
      s_eb[m][r] = e;
      S.sb[m][r] = ldexpf(1.f, e - 9);
    }
    __syncthreads();
    for (int t = tid; t < 2 * TC_NJ * TC_K; t += TC_THREADS) {
      const int m = t / (TC_NJ * TC_K), rk = t % (TC_NJ * TC_K);
      const int r = rk % TC_NJ, k = rk / TC_NJ;
      const int jj = j0 + r;
      float v = 0.f;
      if (k < NFREQ && jj < n && c.w.z[bN + jj] != 0)
        v = (m == 0 ? A32 : A032)[(size_t)k * N + jj];
      store_digits(S.bm[m][0], S.bm[m][1], S.bm[m][2], kmaj_off(r, k), v, s_eb[m][r]);
      if (m == 0) S.aj[r][k] = v;
    }
    if (tid < TC_NJ) {
      const int jj = j0 + tid;
      const bool ok = jj < n;
      S.pj[tid] = ok ? P[jj] : make_float4(0.f, 0.f, 0.f, 0.f);
      S.lj[tid] = ok ? PL[jj] : make_float4(0.f, 0.f, 0.f, 0.f);
      S.zj[tid] = ok ? c.w.z[bN + jj] : 0;
      S.wj[tid] = ok ? c.w.w32[bN + jj] : 0.f;
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      // matrix m (0: C6 from A', 1: C6(q=0) from A0') into columns 96 m:
      // class 0 (d1 d1) at +0, class 1 (d1 d2 + d2 d1) at +32, class 2
      // (d1 d3 + d2 d2 + d3 d1) at +64, each over the three k-steps
      constexpr int AP = TC_M * TC_K * 4, BP = TC_NJ * TC_K * 4;  // plane bytes
      constexpr int cls_of[6] = {0, 1, 1, 2, 2, 2};
      constexpr int da_of[6] = {0, 0, 1, 0, 1, 2};
      constexpr int db_of[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
      for (int m = 0; m < 2; ++m) {
#pragma unroll
        for (int pr = 0; pr < 6; ++pr) {
          const uint32_t d = tmem + 96u * m + 32u * cls_of[pr];
          const uint32_t ab = a_base + (3 * m + da_of[pr]) * AP;
          const uint32_t bb = b_base + (3 * m + db_of[pr]) * BP;
          const bool first = pr == 0 || pr == 1 || pr == 3;
#pragma unroll
          for (int s = 0; s < TC_K / 8; ++s)
            tc::mma_tf32(d, tc::desc_kmajor(ab + 2 * TC_LBO * s, TC_LBO, TC_SBO),
                         tc::desc_kmajor(bb + 2 * TC_LBO * s, TC_LBO, TC_SBO), IDESC,
                         !(first && s == 0));
        }
      }
      tc::commit(mbar);
    }
    // (test hook: the first wait of a D4_FLAG_TEST_TIMEOUT call counts as
    // timed out; the drain below then waits for these MMAs for real)
    const bool done = (test_timeout && j0 == ch0 * TC_NJ) ? false : tc::mbar_wait(mbar, parity);
    parity ^= 1u;
    if (__syncthreads_or(!done)) {
      timed_out = true;
      break;
    }
    tc::fence_after_sync();
    // this thread's columns: ncol = 16 / D from cbeg, in blocks of 8 (D = 4:
    // half of one block)
    const int ncol = 16 / D, cbeg = cg * ncol;
#pragma unroll 1
    for (int u = 0; u < (ncol + 7) / 8; ++u) {
      const int c0 = (cbeg + 8 * u) & ~7;
      const int qlo = cbeg + 8 * u - c0, qhi = qlo + (ncol < 8 ? ncol : 8);
      float c6v[8], c60v[8];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        uint32_t va[8], vb[8], vc[8];
        tc::tmem_ld8(tmem + t_lane + 96 * m + c0, va);
        tc::tmem_ld8(tmem + t_lane + 96 * m + 32 + c0, vb);
        tc::tmem_ld8(tmem + t_lane + 96 * m + 64 + c0, vc);
        tc::tmem_ld_wait();
        const float sc = S.sa[m][row];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float t = fmaf(__uint_as_float(vc[q]), 1.f / 512.f, __uint_as_float(vb[q]));
          const float v = fmaf(t, 1.f / 512.f, __uint_as_float(va[q])) * (sc * S.sb[m][c0 + q]);
          if (m == 0)
            c6v[q] = v;
          else
            c60v[q] = v;
        }
      }
      if (!real) continue;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int r = c0 + q;
        const int j = j0 + r;
        const int zj = S.zj[r];
        if (q < qlo || q >= qhi || j >= n || j == i || zj == 0) continue;
        const float4 pj = S.pj[r];
        const float3 dv = pos_diff(pi, li, pj, S.lj[r]);
        const float dx = dv.x, dy = dv.y, dz = dv.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float ir = __frcp_rn(sqrtf(r2));  // correctly rounded: no bias in the ATM records
        const float rr = r2 * ir;
        const float c6 = c6v[q];
        const float c60 = c60v[q];
        dfl R0d, qqd, R06d, R08d;
        if (tabled) {
          const float4 A = c.w.pairA[zi * MAX_ELEM_ID + zj], Bq = c.w.pairB[zi * MAX_ELEM_ID + zj];
          R0d = {A.x, A.y};
          qqd = {A.z, A.w};
          R06d = {Bq.x, Bq.y};
          R08d = {Bq.z, Bq.w};
        } else {
          const double si = (double)pi.w + (double)li.w;
          const double sj = (double)pj.w + (double)S.lj[r].w;
          const double qq = 3.0 * si * si * sj * sj;
          const double R0 = p.a1 * sqrt(qq) + p.a2;
          const double R02 = R0 * R0, R06 = R02 * R02 * R02;
          R0d = df_from(R0);
          qqd = df_from(qq);
          R06d = df_from(R06);
          R08d = df_from(R06 * R02);
        }
        const float R0 = R0d.hi, sqq = sqrtf(qqd.hi);
        const float iR0 = __frcp_rn(R0);
        // log(R0 / r) and (R0 / r)^(alp/3) of the ATM damping through logf /
        // expf (SFU estimates bias the three-body energy by ~1e-6 relative;
        // exp2f keeps a mean relative error of ~-3e-8, expf ~+5e-9, and every
        // triple multiplies three of these factors)
        const float lnR0r = logf(R0 * ir) + R0d.lo * iR0;
        const float ir2 = __frcp_rn(r2);
        Tt[(size_t)j * N + i] = make_float4(r2, ir2, expf(alp3 * lnR0r),
                                            sqrtf(fmaxf(c60, 0.f)) * (ir * ir2));
        r2mx = fmaxf(r2mx, r2);
        if (PGRAD)
          Tdat[(size_t)j * N + i] = make_float4(sqq * iR0, iR0, lnR0r, 0.f);
        if (rr <= cut2) {
          const float r6 = r2 * r2 * r2, R02 = R0 * R0, R06 = R06d.hi;
          const float t6 = __frcp_rn((r6 + R06) + R06d.lo);
          float eterm = rho6 * c6 * t6;
          float dEdr = 6.0f * s6 * c6 * (r6 * ir) * t6 * t6;
          float K = -s6 * t6;
          float dE_dR0 = 6.0f * s6 * c6 * (R06 * iR0) * t6 * t6;
          pg[0] -= wi * c6 * t6;
          if (p.has_s8) {
            const float r8 = r6 * r2, R08 = R08d.hi, qq = qqd.hi;
            const float t8 = __frcp_rn((r8 + R08) + R08d.lo);
            const float c8 = fmaf(c6, qqd.hi, c6 * qqd.lo);
            e8_acc.add(c8 * t8);
            dEdr += 8.0f * s8 * c8 * (r8 * ir) * t8 * t8;
            K -= s8 * qq * t8;
            dE_dR0 += 8.0f * s8 * c8 * (R08 * iR0) * t8 * t8;
            pg[1] -= wi * c8 * t8;
          }
          if (p.has_s10) {
            const float qq = sqq * sqq;
            const float r10 = r6 * r2 * r2, R010 = R06 * R02 * R02;
            const float t10 = __frcp_rn(r10 + R010);
            const float q2 = qq * qq * (49.0f / 40.0f);
            const float c10 = c6 * q2;
            const float e10 = c10 * t10;
            eterm = fmaf(rho10.hi, e10, fmaf(rho10.lo, e10, eterm));
            dEdr += 10.0f * s10 * c10 * (r10 * ir) * t10 * t10;
            K -= s10 * q2 * t10;
            dE_dR0 += 10.0f * s10 * c10 * (R010 * iR0) * t10 * t10;
            pg[2] -= wi * c10 * t10;
          }
          e_acc.add(eterm);
          const float phi = 0.5f * (wi + S.wj[r]);
          dEdr *= phi;
          K *= phi;
          pg[3] += wi * 0.5f * dE_dR0 * sqq;
          pg[4] += wi * 0.5f * dE_dR0;
          const float f = dEdr * ir;
          gx.add(f * dx);
          gy.add(f * dy);
          gz.add(f * dz);
          if (GRAD) {
            const float4 *aj4 = reinterpret_cast<const float4 *>(S.aj[r]);
#pragma unroll
            for (int w4 = 0; w4 < TC_K / 4; ++w4) {
              const float4 a4 = aj4[w4];
              gacc[4 * w4] = fmaf(K, a4.x, gacc[4 * w4]);
              gacc[4 * w4 + 1] = fmaf(K, a4.y, gacc[4 * w4 + 1]);
              gacc[4 * w4 + 2] = fmaf(K, a4.z, gacc[4 * w4 + 2]);
              if (4 * w4 + 3 < NFREQ) gacc[4 * w4 + 3] = fmaf(K, a4.w, gacc[4 * w4 + 3]);
            }
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();  // chunk buffers and tensor memory are free again
  }
  if (real && r2mx > 0.f) atomicMax(&c.w.atm_rowmax[ai], __float_as_uint(r2mx));
  if (timed_out) {
    // an MMA batch did not complete in time: report it, give the tensor
    // cores one more bounded wait, release the tensor memory and leave
    if (tid == 0) set_status(c.w.status, D4_ERR_DEVICE_TIMEOUT);
    tc::mbar_wait(mbar, parity ^ 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
      tc::fence_after_sync();
      tc::tmem_free(tmem, TC_COLS);
    }
    return;
  }
  // combine the 2 D column groups of every atom in the group-0 thread (A
  // operand area reused: the last MMA batch has completed; (2 D - 1) x 38 x
  // MR floats <= 8512)
  float *red = &S.a[0][0][0];
  const int ra = row % MR;
  if (cg != 0) {
    float v[TC_NRED] = {e_acc.hi, e_acc.lo, e8_acc.hi, e8_acc.lo, gx.hi, gx.lo, gy.hi, gy.lo,
                        gz.hi,    gz.lo,    pg[0],     pg[1],     pg[2], pg[3], pg[4]};
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) v[15 + w] = gacc[w];
    float *o = red + (size_t)(cg - 1) * TC_NRED * MR + ra;
#pragma unroll
    for (int k = 0; k < TC_NRED; ++k) o[k * MR] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_free(tmem, TC_COLS);
  }
  if (cg != 0) return;
  for (int g = 0; g < 2 * D - 1; ++g) {
    const float *o = red + (size_t)g * TC_NRED * MR + ra;
    auto merge = [&](Acc32 &a, int k) {
      a.add(o[k * MR]);
      a.lo += o[(k + 1) * MR];
    };
    merge(e_acc, 0);
    merge(e8_acc, 2);
    merge(gx, 4);
    merge(gy, 6);
    merge(gz, 8);
#pragma unroll
    for (int k = 0; k < 5; ++k) pg[k] += o[(10 + k) * MR];
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) gacc[w] += o[(15 + w) * MR];
  }
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
  if (i >= N) return;
  if (nsplit > 1) {  // partial sums of this CTA's partners
    if (!real) return;
    if (GRAD) {
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) atomicAdd(&c.w.G32[ai * NFREQ + w], gacc[w]);
      atomicAdd(&c.out.d_gradient[3 * ai], gx.value());
      atomicAdd(&c.out.d_gradient[3 * ai + 1], gy.value());
      atomicAdd(&c.out.d_gradient[3 * ai + 2], gz.value());
    }
    atomicAdd(&c.out.d_energy[ai],
              -0.5 * (sref * e_acc.value() + (p.has_s8 ? p.s8 * e8_acc.value() : 0.0)));
    return;
  }
  if (!real) {
    c.out.d_energy[ai] = 0.0;
    if (GRAD) {
      c.out.d_gradient[3 * ai] = 0.0;
      c.out.d_gradient[3 * ai + 1] = 0.0;
      c.out.d_gradient[3 * ai + 2] = 0.0;
      for (int w = 0; w < NFREQ; ++w) c.w.G32[ai * NFREQ + w] = 0.f;
    }
    return;
  }
  if (GRAD) {
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) c.w.G32[ai * NFREQ + w] = gacc[w];  // dE/dA'_i
    c.out.d_gradient[3 * ai] = gx.value();
    c.out.d_gradient[3 * ai + 1] = gy.value();
    c.out.d_gradient[3 * ai + 2] = gz.value();
  }
  c.out.d_energy[ai] =
      -0.5 * (sref * e_acc.value() + (p.has_s8 ? p.s8 * e8_acc.value() : 0.0));
}

// Few tiles (large structures): the partners of a tile are split over
// several CTAs so that every SM gets about four CTAs.
static int pair_tc_splits(const Ctx &c) {
  static int sms[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int &nsm = sms[dev & 63];
  if (nsm == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    nsm = v > 0 ? v : 1;
  }
  const long long tiles = (long long)((c.N + TC_M - 1) / TC_M) * c.B;
  const long long want = 4LL * nsm;
  if (tiles >= want) return 1;
  const long long chunks = (c.N + TC_NJ - 1) / TC_NJ;
  const long long s = (want + tiles - 1) / tiles;
  return (int)(s < chunks ? s : chunks);
}

void launch_pair_fwd_tc(const Ctx &c, cudaStream_t st) {
  const int nsplit = pair_tc_splits(c);
  const dim3 grid((c.N + TC_M - 1) / TC_M, c.B, nsplit);
  const int smem = (int)sizeof(TcSmem);
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  const bool pgrad = (c.flags & D4_FLAG_PARAM_GRAD) != 0;
  if (nsplit > 1) {  // the CTAs of a tile accumulate atomically
    const size_t bn = (size_t)c.B * c.N;
    cudaMemsetAsync(c.out.d_energy, 0, 8 * bn, st);
    if (grad) {
      cudaMemsetAsync(c.out.d_gradient, 0, 24 * bn, st);
      cudaMemsetAsync(c.w.G32, 0, 4 * NFREQ * bn, st);
    }
  }
  if (pgrad) {
    ensure_smem(pair_fwd_tc_kernel<true, true>, smem);
    pair_fwd_tc_kernel<true, true><<<grid, TC_THREADS, smem, st>>>(c);
  } else if (grad) {
    ensure_smem(pair_fwd_tc_kernel<true, false>, smem);
    pair_fwd_tc_kernel<true, false><<<grid, TC_THREADS, smem, st>>>(c);
  } else {
    ensure_smem(pair_fwd_tc_kernel<false, false>, smem);
    pair_fwd_tc_kernel<false, false><<<grid, TC_THREADS, smem, st>>>(c);
  }
}

}  // namespace d4

namespace d4 {

// ---------------------------------------------------------------- ATM / C6(q=0) adjoint

// ATM forces, the C6(q=0) adjoint and the chain rule to dE/dCN and dE/dq of
// the D4 precision form (the work of pair_atm_bwd_mixed_kernel), with the
// C6(q=0) adjoint on the tensor cores:
//   G0_x(w) = sum_y D_xy A0'_y(w),  D_xy = P_xy / (2 C6(q=0)_xy),
// P_xy = the weighted triple energies of the pair, C6(q=0)_xy = c_xy^2 from
// the pair record.  A CTA takes 128 atoms x (thread x) and walks the
// partners y in chunks of 32: the threads read S_xy, P_xy and c_xy (pair
// arrays are symmetric, read as row y so that the reads are coalesced over
// x), add 2 S_xy (r_x - r_y) to the force on x and write D_xy into the MMA's
// A operand; one thread issues the M=128, N=32 (frequencies, 23 used), K=32
// products into tensor memory.  Split products hi = tf32(v), lo = tf32(v -
// hi), three MMAs (lo hi, hi lo, hi hi) per k-step: this adjoint only feeds
// forces, whose bar (1e-6 Eh/Bohr) the few-1e-7 relative accuracy meets.
constexpr int BW_THREADS = 256;               // two threads per atom (halves of a chunk)
constexpr int BW_K = 32;                      // partners per chunk (MMA K)
constexpr int BW_SBO = (BW_K / 4) * 128;      // 1024 bytes between groups of 8 rows
constexpr int BW_COLS = 32;                   // tensor memory: G0 (32 frequencies)

__device__ __forceinline__ int kmaj32_off(int r, int k) {
  return (r >> 3) * BW_SBO + (k >> 2) * TC_LBO + (r & 7) * 16 + (k & 3) * 4;
}

struct BwSmem {
  float a[2][TC_M * BW_K];  // D hi / lo (rows x, K = partners)
  float bm[2][32 * BW_K];   // A0' hi / lo (rows = frequencies, K = partners)
  float4 py[BW_K], ly[BW_K];
  int zy[BW_K];
  unsigned long long mbar;
  uint32_t tmem;
};

__device__ __forceinline__ void split_tf32(float *hi, float *lo, int off, float v) {
  const float h = tc::to_tf32(v);
  *reinterpret_cast<float *>(reinterpret_cast<char *>(hi) + off) = h;
  *reinterpret_cast<float *>(reinterpret_cast<char *>(lo) + off) = tc::to_tf32(v - h);
}

__global__ void __launch_bounds__(BW_THREADS) pair_atm_bwd_tc_kernel(Ctx c) {
  extern __shared__ __align__(128) unsigned char s_raw[];
  BwSmem &S = *reinterpret_cast<BwSmem *>(s_raw);
  const int b = blockIdx.y;
  const int N = c.N;
  const int n = c.w.n_eff[b];
  const int x0 = blockIdx.x * TC_M;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (TC_M - 1), half = tid >> 7;
  const int x = x0 + row;
  const size_t bN = (size_t)b * N;
  const size_t ax = bN + x;
  const bool real = x < n && c.w.z[ax] != 0;
  // partners of this CTA: chunks [ch0, ch1); with several CTAs per tile
  // (gridDim.z > 1) they add G0 and the forces atomically and
  // pair_atm_bwd_finish_kernel applies the chain rule
  const int nsplit = gridDim.z;
  const int nch = (n + BW_K - 1) / BW_K;
  const int ch0 = (int)((long long)blockIdx.z * nch / nsplit);
  const int ch1 = (int)((long long)(blockIdx.z + 1) * nch / nsplit);
  if (nsplit > 1 && (x0 >= n || ch0 >= ch1)) return;
  if (x0 >= n) {  // a tile of padding only
    if (half == 0 && x < N) {
      c.w.dEdcn[ax] = 0.0;
      c.w.dEdq[ax] = 0.0;
      c.w.adj32[ax] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  const uint32_t mbar = tc::smem_u32(&S.mbar);
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(&S.tmem), BW_COLS);
  if (tid == 0) tc::mbar_init(mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  const float4 *P = c.w.pos32 + bN;
  const float4 *PL = c.w.pos32lo + bN;
  const float4 px = real ? P[x] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 lx = real ? PL[x] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float *Sxy = c.w.prS32 + bN * N;
  const float *Pxy = c.w.prP32 + bN * N;
  const float4 *T = c.w.ptf + bN * N;
  const float *A032 = c.w.A032 + bN * NFREQ;  // [w][N] of structure b
  constexpr uint32_t IDESC = tc::idesc_tf32(TC_M, 32);
  const uint32_t a_base = tc::smem_u32(&S.a[0][0]);
  const uint32_t b_base = tc::smem_u32(&S.bm[0][0]);
  Acc32 gx, gy, gz;
  uint32_t parity = 0;
  bool timed_out = false, issued = false;
  for (int y0 = ch0 * BW_K; y0 < ch1 * BW_K; y0 += BW_K) {
    if (tid < BW_K) {
      const int y = y0 + tid;
      const bool ok = y < n;
      S.py[tid] = ok ? P[y] : make_float4(0.f, 0.f, 0.f, 0.f);
      S.ly[tid] = ok ? PL[y] : make_float4(0.f, 0.f, 0.f, 0.f);
      S.zy[tid] = ok ? c.w.z[bN + y] : 0;
    }
    for (int t = tid; t < 32 * BW_K; t += BW_THREADS) {  // B: A0'_y(w), rows w
      const int w = t / BW_K, q = t % BW_K;
      const int y = y0 + q;
      const float v = (w < NFREQ && y < n && c.w.z[bN + y] != 0) ? A032[(size_t)w * N + y] : 0.f;
      split_tf32(S.bm[0], S.bm[1], kmaj32_off(w, q), v);
    }
    __syncthreads();
    {
      constexpr int QH = BW_K / 2;
      const int q0 = half * QH;
      float sv[QH], pv[QH], cv[QH];  // cv: record w = sqrt(C6(q=0)) / r^3
#pragma unroll
      for (int u = 0; u < QH; ++u) {  // all loads of the half chunk first
        const int q = q0 + u, y = y0 + q;
        const bool ok = real && y < n && y != x && S.zy[q] != 0;
        const size_t o = (size_t)(ok ? y : 0) * N + x;  // the pair arrays are symmetric
        sv[u] = ok ? Sxy[o] : 0.f;
        pv[u] = ok ? Pxy[o] : 0.f;
        cv[u] = ok ? T[o].w : 0.f;
      }
#pragma unroll
      for (int u = 0; u < QH; ++u) {
        const int q = q0 + u;
        float D = 0.f;
        if (sv[u] != 0.f || pv[u] != 0.f) {
          const float3 d = pos_diff(px, lx, S.py[q], S.ly[q]);
          gx.add(2.0f * sv[u] * d.x);
          gy.add(2.0f * sv[u] * d.y);
          gz.add(2.0f * sv[u] * d.z);
          if (pv[u] != 0.f) {  // D = P / (2 C6(q=0)), C6(q=0) = w^2 r^6
            const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
            D = pv[u] / (2.0f * (cv[u] * cv[u]) * (r2 * r2 * r2));
          }
        }
        split_tf32(S.a[0], S.a[1], kmaj32_off(row, q), D);
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      constexpr int AP = TC_M * BW_K * 4, BP = 32 * BW_K * 4;
#pragma unroll
      for (int pr = 0; pr < 3; ++pr) {
        const uint32_t ab = a_base + (pr == 0 ? AP : 0), bb = b_base + (pr == 1 ? BP : 0);
#pragma unroll
        for (int s = 0; s < BW_K / 8; ++s)
          tc::mma_tf32(tmem, tc::desc_kmajor(ab + 2 * TC_LBO * s, TC_LBO, BW_SBO),
                       tc::desc_kmajor(bb + 2 * TC_LBO * s, TC_LBO, BW_SBO), IDESC,
                       (issued || pr > 0 || s > 0) ? 1u : 0u);
      }
      tc::commit(mbar);
    }
    issued = true;
    const bool done = tc::mbar_wait(mbar, parity);
    parity ^= 1u;
    if (__syncthreads_or(!done)) {
      timed_out = true;
      break;
    }
  }
  if (timed_out) {
    if (tid == 0) set_status(c.w.status, D4_ERR_DEVICE_TIMEOUT);
    tc::mbar_wait(mbar, parity ^ 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
      tc::fence_after_sync();
      tc::tmem_free(tmem, BW_COLS);
    }
    return;
  }
  tc::fence_after_sync();
  uint32_t g0[32];
  if (half == 0) {
    uint32_t (&lo16)[16] = *reinterpret_cast<uint32_t(*)[16]>(&g0[0]);
    uint32_t (&hi16)[16] = *reinterpret_cast<uint32_t(*)[16]>(&g0[16]);
    const uint32_t t_lane = (uint32_t)(warp * 32) << 16;
    tc::tmem_ld16(tmem + t_lane, lo16);
    tc::tmem_ld16(tmem + t_lane + 16, hi16);
    tc::tmem_ld_wait();
  }
  // the second half's force partial sums, through the (now free) A operand
  float *red = &S.a[0][0];
  if (half == 1) {
    red[0 * TC_M + row] = gx.hi;
    red[1 * TC_M + row] = gx.lo;
    red[2 * TC_M + row] = gy.hi;
    red[3 * TC_M + row] = gy.lo;
    red[4 * TC_M + row] = gz.hi;
    red[5 * TC_M + row] = gz.lo;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_free(tmem, BW_COLS);
  }
  if (half == 1) return;
  gx.add(red[0 * TC_M + row]);
  gx.lo += red[1 * TC_M + row];
  gy.add(red[2 * TC_M + row]);
  gy.lo += red[3 * TC_M + row];
  gz.add(red[4 * TC_M + row]);
  gz.lo += red[5 * TC_M + row];
  if (x >= N) return;
  if (nsplit > 1) {  // partial sums of this CTA's partners
    if (!real) return;
#pragma unroll
    for (int w = 0; w < NFREQ; ++w) atomicAdd(&c.w.G032[ax * NFREQ + w], __uint_as_float(g0[w]));
    atomicAdd(&c.out.d_gradient[3 * ax], gx.value());
    atomicAdd(&c.out.d_gradient[3 * ax + 1], gy.value());
    atomicAdd(&c.out.d_gradient[3 * ax + 2], gz.value());
    return;
  }
  if (!real) {
    c.w.dEdcn[ax] = 0.0;
    c.w.dEdq[ax] = 0.0;
    c.w.adj32[ax] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  if (!issued) {  // a structure with no partners: G0 = 0
#pragma unroll
    for (int w = 0; w < 32; ++w) g0[w] = 0u;
  }
  // chain rule to CN and q (one slot): dE/dCN = sum_w G dA/dCN + G0 dA0/dCN,
  // dE/dq = sum_w G dA/dq
  Acc32 dcn, dq;
  const float *G = c.w.G32 + ax * NFREQ;
  const float *dA = c.w.dA32 + ax * NFREQ * 3;
#pragma unroll
  for (int w = 0; w < NFREQ; ++w) {
    const float gw = G[w];
    dcn.add(gw * dA[3 * w]);
    dcn.add(__uint_as_float(g0[w]) * dA[3 * w + 2]);
    dq.add(gw * dA[3 * w + 1]);
  }
  c.w.dEdcn[ax] = dcn.value();
  c.w.dEdq[ax] = dq.value();
  c.w.adj32[ax] = make_float4(dcn.hi + dcn.lo, 0.f, (float)c.w.q[ax], 0.f);
  c.out.d_gradient[3 * ax] += gx.value();
  c.out.d_gradient[3 * ax + 1] += gy.value();
  c.out.d_gradient[3 * ax + 2] += gz.value();
  c.out.d_energy[ax] += c.w.e3[ax];
}

// Chain rule of the split tensor-core adjoint (thread per atom): dE/dCN and
// dE/dq from G (pair kernel) and the accumulated G0, and E2 + E3.
__global__ void __launch_bounds__(256) pair_atm_bwd_finish_kernel(Ctx c) {
  const int b = blockIdx.y;
  const int N = c.N;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= N) return;
  const size_t ax = (size_t)b * N + x;
  const int n = c.w.n_eff[b];
  if (x >= n || c.w.z[ax] == 0) {
    c.w.dEdcn[ax] = 0.0;
    c.w.dEdq[ax] = 0.0;
    c.w.adj32[ax] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  Acc32 dcn, dq;
  const float *G = c.w.G32 + ax * NFREQ;
  const float *G0 = c.w.G032 + ax * NFREQ;
  const float *dA = c.w.dA32 + ax * NFREQ * 3;
#pragma unroll
  for (int w = 0; w < NFREQ; ++w) {
    const float gw = G[w];
    dcn.add(gw * dA[3 * w]);
    dcn.add(G0[w] * dA[3 * w + 2]);
    dq.add(gw * dA[3 * w + 1]);
  }
  c.w.dEdcn[ax] = dcn.value();
  c.w.dEdq[ax] = dq.value();
  c.w.adj32[ax] = make_float4(dcn.hi + dcn.lo, 0.f, (float)c.w.q[ax], 0.f);
  c.out.d_energy[ax] += c.w.e3[ax];
}

// Whether the tensor-core adjoint runs: the D4 model (one slot).
bool pair_atm_bwd_tc_ok(const Ctx &c) { return c.cfg.kind == D4_MODEL_D4 && c.S == 1; }

void launch_pair_atm_bwd_tc(const Ctx &c, cudaStream_t st) {
  const int smem = (int)sizeof(BwSmem);
  ensure_smem(pair_atm_bwd_tc_kernel, smem);
  // few tiles (large structures): a tile's partners are split over several
  // CTAs so that every SM gets about four
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (long long)((c.N + TC_M - 1) / TC_M) * c.B;
  const long long want = 4LL * (nsm > 0 ? nsm : 1);
  const long long chunks = (c.N + BW_K - 1) / BW_K;
  int nsplit = 1;
  if (tiles < want) {
    const long long sp = (want + tiles - 1) / tiles;
    nsplit = (int)(sp < chunks ? sp : chunks);
  }
  if (nsplit > 1) {
    cudaMemsetAsync(c.w.G032, 0, (size_t)4 * NFREQ * c.B * c.N, st);
    pair_atm_bwd_tc_kernel<<<dim3((c.N + TC_M - 1) / TC_M, c.B, nsplit), BW_THREADS, smem, st>>>(c);
    pair_atm_bwd_finish_kernel<<<dim3((c.N + 255) / 256, c.B), 256, 0, st>>>(c);
  } else {
    pair_atm_bwd_tc_kernel<<<dim3((c.N + TC_M - 1) / TC_M, c.B), BW_THREADS, smem, st>>>(c);
  }
}

}  // namespace d4
