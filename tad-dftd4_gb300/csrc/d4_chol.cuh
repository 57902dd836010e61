// Blocked FP32 Cholesky factorisation and triangular solves of packed
// symmetric positive definite matrices held by one CTA (shared or global
// memory), used by the EEQ solves of the precision form.
#pragma once

#include "d4_common.cuh"

namespace d4 {

constexpr int PB = 32;  // panel width of the blocked factorisation and solves
constexpr unsigned FULL = 0xffffffffu;

// Diagonal 32 x 32 block (rows / columns k0 .. k0+kb-1) of the packed lower
// matrix L: the Cholesky factor by one warp, in registers (lane r holds row
// r; rows beyond the matrix are padded with the identity).  Per column c the
// pivot comes by a shuffle; the scaled column goes through shared memory
// (double-buffered, one __syncwarp) and is read back as float4 broadcasts,
// eight loads instead of one shuffle per entry below the pivot (~4.9k cycles
// per block against ~8.8k).  The update is unconditional: the entries above
// a lane's diagonal collect values that are never read, since the column
// value of a row above the pivot is forced to zero.  A non-positive pivot
// sets *bad and goes on with pivot 1.
static __device__ void chol_diag_factor(float *L, int k0, int kb, int *bad) {
  __shared__ __align__(16) float s_col[2][PB];
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
    const float lc = r == c ? d * inv : (r > c ? a[c] * inv : 0.f);
    a[c] = lc;
    if (c + 1 < PB) {
      float *col = s_col[c & 1];
      col[r] = lc;
      __syncwarp();
      const float4 *c4 = reinterpret_cast<const float4 *>(col);
#pragma unroll
      for (int q = (c + 1) >> 2; q < PB / 4; ++q) {
        const float4 v = c4[q];
        const float lv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (4 * q + e > c) a[4 * q + e] = fmaf(-lc, lv[e], a[4 * q + e]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < PB; ++j)
    if (live && j <= r) row[j] = a[j];
}

// The inverse X of the factored diagonal block, which replaces it in place
// (the panel and the triangular solves only need the inverse), by all warps
// of the CTA (Q x warps >= 32; every thread calls it): warp w forms the
// columns w, w + nw, ... by forward substitution down the column, lane r =
// row r, X[r][c] = (delta_rc - sum_{k<r} L[r][k] X[k][c]) / L[r][r]; the
// columns of a warp advance together, the finished value of row k reaching
// the other lanes by a shuffle.  (One warp forming all 32 columns took ~12k
// cycles per block, three times the factorisation; eight warps take ~2.7k.
// Sixteen warps take Q = 2: with four slots per warp, two of them empty,
// the shuffles alone doubled the time.)
template <int Q>
static __device__ void chol_diag_inverse(float *L, int k0, int kb) {
  const int w = threadIdx.x >> 5, r = threadIdx.x & 31, nw = blockDim.x >> 5;
  const bool live = r < kb;
  const float *lr = L + tri_index(k0 + (live ? r : 0), k0);
  const float dinv = live ? 1.0f / lr[r] : 1.f;
  float sq[Q], xr[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) sq[q] = xr[q] = 0.f;
#pragma unroll 1
  for (int k = 0; k < kb; ++k) {
    float xk[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int cq = w + nw * q;
      const float mine = r == cq ? dinv : (r > cq ? -sq[q] * dinv : 0.f);
      if (r == k) xr[q] = mine;
      xk[q] = __shfl_sync(FULL, mine, k);
    }
    const float lrk = (live && r > k) ? lr[k] : 0.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) sq[q] = fmaf(lrk, xk[q], sq[q]);
  }
  __syncthreads();  // every warp has read the factor
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cq = w + nw * q;
    if (cq < PB && live && r >= cq) L[tri_index(k0 + r, k0 + cq)] = xr[q];
  }
}

// chol_diag_inverse with the column slots per warp that the CTA's size needs
static __device__ __forceinline__ void chol_diag_inverse_cta(float *L, int k0, int kb) {
  if (blockDim.x >= 512)
    chol_diag_inverse<2>(L, k0, kb);
  else
    chol_diag_inverse<4>(L, k0, kb);
}

// (ti, tj), tj <= ti, of the t-th tile of a packed lower triangle of tiles
static __device__ __forceinline__ void tri_tile(int t, int &ti, int &tj) {
  ti = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
  while (ti > 0 && ti * (ti + 1) / 2 > t) --ti;
  tj = t - ti * (ti + 1) / 2;
}

// A22 -= L21 L21^T for the rows / columns t0 .. m-1 of the packed matrix,
// from the panel PT (transposed, 32 x ldp), in TS x TS register tiles of
// the lower triangle (one tile per thread at a time, read as float4).
template <int TS>
static __device__ __forceinline__ void chol_update_tiles(float *L, const float *PT, int ldp,
                                                         int m, int t0, int kb) {
  const int nrem = m - t0;
  const int T = (nrem + TS - 1) / TS;
  const int ntile = T * (T + 1) / 2;
  for (int t = threadIdx.x; t < ntile; t += blockDim.x) {
    int ti, tj;
    tri_tile(t, ti, tj);
    const int i0 = TS * ti, j0 = TS * tj;  // relative to t0
    float acc[TS][TS];
#pragma unroll
    for (int q = 0; q < TS; ++q)
#pragma unroll
      for (int u = 0; u < TS; ++u) acc[q][u] = 0.f;
    for (int cc = 0; cc < kb; ++cc) {
      const float4 *p = reinterpret_cast<const float4 *>(PT + cc * ldp);
      float x[TS], y[TS];
#pragma unroll
      for (int h = 0; h < TS / 4; ++h) {
        const float4 xa = p[(i0 >> 2) + h], ya = p[(j0 >> 2) + h];
        x[4 * h] = xa.x;
        x[4 * h + 1] = xa.y;
        x[4 * h + 2] = xa.z;
        x[4 * h + 3] = xa.w;
        y[4 * h] = ya.x;
        y[4 * h + 1] = ya.y;
        y[4 * h + 2] = ya.z;
        y[4 * h + 3] = ya.w;
      }
#pragma unroll
      for (int q = 0; q < TS; ++q)
#pragma unroll
        for (int u = 0; u < TS; ++u) acc[q][u] = fmaf(x[q], y[u], acc[q][u]);
    }
#pragma unroll
    for (int q = 0; q < TS; ++q) {
      const int i = t0 + i0 + q;
      if (i < m) {
        float *ri = L + tri_index(i, 0);
#pragma unroll
        for (int u = 0; u < TS; ++u) {
          const int j = t0 + j0 + u;
          if (j <= i) ri[j] -= acc[q][u];
        }
      }
    }
  }
}

// Blocked right-looking Cholesky (panels of 32 columns) of the packed lower
// m x m FP32 matrix L, in place, except that each diagonal block holds the
// inverse of its factor.  Per panel: the diagonal block (factor by warp 0,
// inverse by all warps), the panel L21 = A21 X^T (X the block inverse; one
// warp per row, lane = column), and the trailing update A22 -= L21 L21^T.
// The panel buffer PT (shared memory, 32 x ldp) holds the panel transposed,
// so that the update runs on register tiles read as float4 (8 x 8: 64 FMAs
// per four 16-byte loads; 4 x 4 once the trailing matrix is small).
static __device__ void chol_blocked(float *L, float *PT, int ldp, int m, int *bad) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  const int nw = nt >> 5;
  for (int k0 = 0; k0 < m; k0 += PB) {
    const int kb = min(PB, m - k0);
    if (warp == 0) chol_diag_factor(L, k0, kb, bad);
    __syncthreads();
    chol_diag_inverse_cta(L, k0, kb);
    __syncthreads();
    const int t0 = k0 + kb;
    // panel: row i of L21 solves L11 x = A21[i]^T, i.e. x = X A21[i]^T; the
    // lane's row of X stays in registers, the row of A21 is read broadcast,
    // four independent partial sums
    if (t0 < m) {
      float xr[PB];
      const float *xc = L + tri_index(k0 + (lane < kb ? lane : 0), k0);
#pragma unroll
      for (int cc = 0; cc < PB; ++cc) xr[cc] = (lane < kb && cc <= lane) ? xc[cc] : 0.f;
      for (int i = t0 + warp; i < m; i += nw) {
        float *row = L + tri_index(i, k0);
        float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
#pragma unroll
        for (int cc = 0; cc < PB; cc += 4) {
          const float r0 = cc < kb ? row[cc] : 0.f, r1 = cc + 1 < kb ? row[cc + 1] : 0.f;
          const float r2 = cc + 2 < kb ? row[cc + 2] : 0.f, r3 = cc + 3 < kb ? row[cc + 3] : 0.f;
          v0 = fmaf(r0, xr[cc], v0);
          v1 = fmaf(r1, xr[cc + 1], v1);
          v2 = fmaf(r2, xr[cc + 2], v2);
          v3 = fmaf(r3, xr[cc + 3], v3);
        }
        const float v = (v0 + v1) + (v2 + v3);
        __syncwarp();
        if (lane < kb) {
          row[lane] = v;
          PT[lane * ldp + (i - t0)] = v;
        }
      }
    }
    __syncthreads();
    // trailing update: 8 x 8 register tiles while they keep at least half of
    // the threads busy, else 4 x 4 (four times as many tiles)
    const int nrem = m - t0;
    const int T8 = (nrem + 7) >> 3;
    if (2 * (T8 * (T8 + 1) / 2) >= nt)
      chol_update_tiles<8>(L, PT, ldp, m, t0, kb);
    else
      chol_update_tiles<4>(L, PT, ldp, m, t0, kb);
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
      const float *xr = L + tri_index(k0 + (lane < kb ? lane : 0), k0);
      float z0 = 0.f, z1 = 0.f, z2 = 0.f, z3 = 0.f;
#pragma unroll
      for (int cc = 0; cc < PB; cc += 4) {
        const bool ok = lane < kb;
        z0 = fmaf(ok && cc <= lane ? xr[cc] : 0.f, cc < kb ? vr[cc] : 0.f, z0);
        z1 = fmaf(ok && cc + 1 <= lane ? xr[cc + 1] : 0.f, cc + 1 < kb ? vr[cc + 1] : 0.f, z1);
        z2 = fmaf(ok && cc + 2 <= lane ? xr[cc + 2] : 0.f, cc + 2 < kb ? vr[cc + 2] : 0.f, z2);
        z3 = fmaf(ok && cc + 3 <= lane ? xr[cc + 3] : 0.f, cc + 3 < kb ? vr[cc + 3] : 0.f, z3);
      }
      const float z = (z0 + z1) + (z2 + z3);
      __syncwarp();
      if (lane < kb) vr[lane] = z;
    }
    __syncthreads();
    const int rows = m - k0 - kb;
    for (int t = tid; t < rows * nr; t += nt) {
      const int r = t / rows, i = k0 + kb + t % rows;
      const float *row = L + tri_index(i, 0) + k0;
      const float *xv = v + r * ldv + k0;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
      for (int cc = 0; cc < PB; cc += 4) {
        if (cc < kb) a0 = fmaf(row[cc], xv[cc], a0);
        if (cc + 1 < kb) a1 = fmaf(row[cc + 1], xv[cc + 1], a1);
        if (cc + 2 < kb) a2 = fmaf(row[cc + 2], xv[cc + 2], a2);
        if (cc + 3 < kb) a3 = fmaf(row[cc + 3], xv[cc + 3], a3);
      }
      v[r * ldv + i] -= (a0 + a1) + (a2 + a3);
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
      float z0 = 0.f, z1 = 0.f, z2 = 0.f, z3 = 0.f;
      const int cl = lane < kb ? lane : 0;
#pragma unroll
      for (int cc = 0; cc < PB; cc += 4) {
        // column `lane` of the block inverse: rows cc >= lane
        const bool o0 = lane < kb && cc >= lane && cc < kb;
        const bool o1 = lane < kb && cc + 1 >= lane && cc + 1 < kb;
        const bool o2 = lane < kb && cc + 2 >= lane && cc + 2 < kb;
        const bool o3 = lane < kb && cc + 3 >= lane && cc + 3 < kb;
        z0 = fmaf(o0 ? L[tri_index(k0 + cc, k0 + cl)] : 0.f, o0 ? vr[cc] : 0.f, z0);
        z1 = fmaf(o1 ? L[tri_index(k0 + cc + 1, k0 + cl)] : 0.f, o1 ? vr[cc + 1] : 0.f, z1);
        z2 = fmaf(o2 ? L[tri_index(k0 + cc + 2, k0 + cl)] : 0.f, o2 ? vr[cc + 2] : 0.f, z2);
        z3 = fmaf(o3 ? L[tri_index(k0 + cc + 3, k0 + cl)] : 0.f, o3 ? vr[cc + 3] : 0.f, z3);
      }
      const float z = (z0 + z1) + (z2 + z3);
      __syncwarp();
      if (lane < kb) vr[lane] = z;
    }
    __syncthreads();
    for (int t = tid; t < k0 * nr; t += nt) {
      const int r = t / k0, i = t % k0;
      const float *xv = v + r * ldv + k0;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
      for (int cc = 0; cc < PB; cc += 4) {
        if (cc < kb) a0 = fmaf(L[tri_index(k0 + cc, i)], xv[cc], a0);
        if (cc + 1 < kb) a1 = fmaf(L[tri_index(k0 + cc + 1, i)], xv[cc + 1], a1);
        if (cc + 2 < kb) a2 = fmaf(L[tri_index(k0 + cc + 2, i)], xv[cc + 2], a2);
        if (cc + 3 < kb) a3 = fmaf(L[tri_index(k0 + cc + 3, i)], xv[cc + 3], a3);
      }
      v[r * ldv + i] -= (a0 + a1) + (a2 + a3);
    }
    __syncthreads();
  }
}

}  // namespace d4
