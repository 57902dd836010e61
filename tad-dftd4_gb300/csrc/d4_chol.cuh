// Blocked FP32 Cholesky factorisation and triangular solves of packed
// symmetric positive definite matrices held by one CTA (shared or global
// memory), used by the EEQ solves of the precision form.
#pragma once

#include "d4_common.cuh"

namespace d4 {

constexpr int PB = 32;  // panel width of the blocked factorisation and solves
constexpr unsigned FULL = 0xffffffffu;

// Diagonal 32 x 32 block (rows / columns k0 .. k0+kb-1) of the packed lower
// matrix L, by one warp, in registers: the Cholesky factor (lane r holds row
// r; rows beyond the matrix are padded with the identity), then the inverse
// of the factor (lane c computes column c), which replaces the block in
// place: the panel and the triangular solves only need the inverse.  A
// non-positive pivot sets *bad and goes on with pivot 1.
static __device__ void chol_diag_block(float *L, int k0, int kb, int *bad) {
  const int r = threadIdx.x & 31;
  const bool live = r < kb;
  float *row = L + tri_index(k0 + (live ? r : 0), k0);
  float a[PB];
#pragma unroll
  for (int j = 0; j < PB; ++j) a[j] = live ? (j <= r ? row[j] : 0.f) : (j == r ? 1.f : 0.f);
#pragma unroll
  for (int c = 0; c < PB; ++c) {
    float d = __shfl_sync(FULL, a[c], c);
    if (!(d > 0.f)) {
      if (r == 0) *bad = 1;
      d = 1.f;
    }
    const float inv = rsqrtf(d);
    if (r == c) a[c] = d * inv;
    else if (r > c) a[c] *= inv;
#pragma unroll
    for (int j = 0; j < PB; ++j) {
      if (j > c) {
        const float lj = __shfl_sync(FULL, a[c], j);
        if (r >= j) a[j] = fmaf(-a[c], lj, a[j]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < PB; ++j)
    if (live && j <= r) row[j] = a[j];
  __syncwarp();
  // inverse: X[rr][c] = -(sum_{k=c}^{rr-1} L[rr][k] X[k][c]) / L[rr][rr]; x = column c
  const int c = r;
  float x[PB];
#pragma unroll
  for (int rr = 0; rr < PB; ++rr) {
    x[rr] = 0.f;
    if (rr < kb) {
      const float *lr = L + tri_index(k0 + rr, k0);
      float acc0 = 0.f, acc1 = 0.f;
#pragma unroll
      for (int k = 0; k < rr; ++k) {
        if (k & 1) acc1 = fmaf(lr[k], x[k], acc1);
        else acc0 = fmaf(lr[k], x[k], acc0);
      }
      const float dii = 1.0f / lr[rr];
      x[rr] = rr == c ? dii : (rr > c ? -(acc0 + acc1) * dii : 0.f);
    }
  }
  __syncwarp();
#pragma unroll
  for (int rr = 0; rr < PB; ++rr)
    if (rr < kb && rr >= c) L[tri_index(k0 + rr, k0 + c)] = x[rr];
  __syncwarp();
}

// (ti, tj), tj <= ti, of the t-th tile of a packed lower triangle of tiles
static __device__ __forceinline__ void tri_tile(int t, int &ti, int &tj) {
  ti = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
  while (ti > 0 && ti * (ti + 1) / 2 > t) --ti;
  tj = t - ti * (ti + 1) / 2;
}

// Blocked right-looking Cholesky (panels of 32 columns) of the packed lower
// m x m FP32 matrix L, in place, except that each diagonal block holds the
// inverse of its factor.  Per panel: the diagonal block by warp 0 in
// registers, the panel L21 = A21 X^T (X the block inverse; one warp per row,
// lane = column), and the trailing update A22 -= L21 L21^T.  With a panel
// buffer PT (shared memory, 32 x ldp) the panel is also stored transposed and
// the update runs on 8 x 8 register tiles read as float4 (64 FMAs per four
// 16-byte loads); without it (PT == nullptr) on 4 x 4 tiles read from the
// packed rows.
static __device__ void chol_blocked(float *L, float *PT, int ldp, int m, int *bad) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  const int nw = nt >> 5;
  for (int k0 = 0; k0 < m; k0 += PB) {
    const int kb = min(PB, m - k0);
    if (warp == 0) chol_diag_block(L, k0, kb, bad);
    __syncthreads();
    const int t0 = k0 + kb;
    // panel: row i of L21 solves L11 x = A21[i]^T, i.e. x = X A21[i]^T
    for (int i = t0 + warp; i < m; i += nw) {
      float *row = L + tri_index(i, k0);
      float v = 0.f;
      if (lane < kb) {
        const float *xc = L + tri_index(k0 + lane, k0);
        for (int cc = 0; cc <= lane; ++cc) v = fmaf(row[cc], xc[cc], v);
      }
      __syncwarp();
      if (lane < kb) {
        row[lane] = v;
        if (PT) PT[lane * ldp + (i - t0)] = v;
      }
    }
    __syncthreads();
    const int nrem = m - t0;
    if (PT) {
      const int T8 = (nrem + 7) >> 3;
      const int ntile = T8 * (T8 + 1) / 2;
      for (int t = tid; t < ntile; t += nt) {
        int ti, tj;
        tri_tile(t, ti, tj);
        const int i0 = 8 * ti, j0 = 8 * tj;  // relative to t0
        float acc[8][8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[q][u] = 0.f;
        for (int cc = 0; cc < kb; ++cc) {
          const float4 *p = reinterpret_cast<const float4 *>(PT + cc * ldp);
          const float4 xa = p[i0 >> 2], xb = p[(i0 >> 2) + 1];
          const float4 ya = p[j0 >> 2], yb = p[(j0 >> 2) + 1];
          const float x[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
          const float y[8] = {ya.x, ya.y, ya.z, ya.w, yb.x, yb.y, yb.z, yb.w};
#pragma unroll
          for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[q][u] = fmaf(x[q], y[u], acc[q][u]);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int i = t0 + i0 + q;
          if (i < m) {
            float *ri = L + tri_index(i, 0);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int j = t0 + j0 + u;
              if (j <= i) ri[j] -= acc[q][u];
            }
          }
        }
      }
    } else {
      const int T4 = (nrem + 3) >> 2;
      const int ntile = T4 * (T4 + 1) / 2;
      for (int t = tid; t < ntile; t += nt) {
        int ti, tj;
        tri_tile(t, ti, tj);
        const int i0 = t0 + 4 * ti, j0 = t0 + 4 * tj;
        size_t ri[4], rj[4];  // offsets of the panel segments of rows i0+q, j0+q
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          ri[q] = tri_index(min(i0 + q, m - 1), k0);
          rj[q] = tri_index(min(j0 + q, m - 1), k0);
        }
        float acc[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q][u] = 0.f;
        for (int cc = 0; cc < kb; ++cc) {
          float x[4], y[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            x[q] = L[ri[q] + cc];
            y[q] = L[rj[q] + cc];
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[q][u] = fmaf(x[q], y[u], acc[q][u]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int i = i0 + q, j = j0 + u;
            if (i < m && j <= i) L[tri_index(i, j)] -= acc[q][u];
          }
      }
    }
    __syncthreads();
  }
}

// Blocked solves with the packed factor whose diagonal blocks hold their
// inverses (all threads of the block call them): forward L z = v, backward
// L^T x = z, ``nr`` <= 2 right-hand sides of leading dimension ldv.  Per
// 32-row block: a 32 x 32 product with the block inverse (warp w handles
// right-hand side w), then the update of the other rows by all threads.
static __device__ void fwd_solve_blocked(const float *L, float *v, int ldv, int m, int nr) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  for (int k0 = 0; k0 < m; k0 += PB) {
    const int kb = min(PB, m - k0);
    if (warp < nr) {
      float *vr = v + warp * ldv + k0;
      float z = 0.f;
      if (lane < kb) {
        const float *xr = L + tri_index(k0 + lane, k0);
        for (int cc = 0; cc <= lane; ++cc) z = fmaf(xr[cc], vr[cc], z);
      }
      __syncwarp();
      if (lane < kb) vr[lane] = z;
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

static __device__ void bwd_solve_blocked(const float *L, float *v, int ldv, int m, int nr) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  if (m <= 0) return;
  for (int k0 = ((m - 1) / PB) * PB; k0 >= 0; k0 -= PB) {
    const int kb = min(PB, m - k0);
    if (warp < nr) {
      float *vr = v + warp * ldv + k0;
      float z = 0.f;
      if (lane < kb)
        for (int cc = lane; cc < kb; ++cc) z = fmaf(L[tri_index(k0 + cc, k0 + lane)], vr[cc], z);
      __syncwarp();
      if (lane < kb) vr[lane] = z;
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

}  // namespace d4
