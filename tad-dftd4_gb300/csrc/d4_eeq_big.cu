// Multi-CTA EEQ solve of the precision form, for structures too large for
// one CTA's shared memory (N > 290): blocked right-looking FP32 Cholesky of
// the dense matrix in panels of 128 columns, blocked triangular solves and
// double-float refinement residuals, every stage spread over all SMs.
//
//   factor (per panel k0):  diag   one CTA per structure: Cholesky of the
//                                  128 x 128 diagonal block (chol_blocked in
//                                  shared memory), stored over the block with
//                                  the inverses of its 32 x 32 diagonal blocks
//                          panel   L21 L11^T = A21 by block substitution,
//                                  64-row tiles
//                          syrk    A22 -= L21 L21^T, 128 x 128 lower tiles
//                                  on the tensor cores (tcgen05, split TF32)
//   inverse (once):         the 512 x 512 diagonal blocks of the factor
//                          are inverted (block forward substitution over
//                          their panels, 128 x 128 products) and stored with
//                          their transposes above the diagonal
//   solve  (per iteration): forward and backward sweeps in 512-row steps
//                          (products with the block inverses, GEMV updates
//                          off the diagonal), then x += v and the
//                          double-float residual of (hi + lo) x, whose max
//                          |r| per structure decides whether later
//                          iterations run.
//
// Rows and columns are in compact order (real atoms only, ``ridx``); the
// structures of a batch are processed together (grid y), each up to its own
// size n_real[b].
#include <float.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "d4_chol.cuh"
#include "d4_common.cuh"
#include "d4_kernels.cuh"
#include "d4_tc.cuh"

namespace d4 {

constexpr int BNB = 128;  // panel width
constexpr float BIG_TOL = 1e-10f;

__device__ __forceinline__ bool big_skip(const Ctx &c, int b, int it) {
  return it > 0 && __uint_as_float(c.w.eeq_res[b * EEQ_BIG_REFINE + it - 1]) < BIG_TOL;
}

// ---------------------------------------------------------------- factor

// Diagonal block [k0, k0 + kb) of structure b: Cholesky in shared memory
// (chol_blocked), written back over the block in the form the panel solve
// works from: the factor below the 32 x 32 diagonal blocks and the inverses
// of those blocks in their place.  The full inverse of the block, which the
// sweeps need, is formed after the factorisation for all panels at once
// (eeq_big_pinv_kernel), off the factorisation's critical path.
__global__ void __launch_bounds__(512) eeq_big_diag_kernel(Ctx c, int k0) {
  extern __shared__ float4 s_dyn4[];
  float *P = reinterpret_cast<float *>(s_dyn4);  // packed kb x kb
  const int ldp = chol_panel_ld(BNB);
  float *PT = P + ((BNB * (BNB + 1) / 2 + 3) & ~3);  // 32 x ldp
  __shared__ int s_bad;
  const int b = blockIdx.x;
  const int m = c.w.n_real[b];
  if (k0 >= m) return;
  const int kb = min(BNB, m - k0);
  const int N = c.N;
  const int NF = eeq_ldf(N);
  float *F = c.w.eeq_F + (size_t)b * N * NF;
  const int tid = threadIdx.x;
  if (tid == 0) s_bad = 0;
  // 512 threads: warp w takes rows w, w + 16, ...; lane l columns l, l + 32,
  // ...: all of a thread's loads are issued before its first store
  const int warp = tid >> 5, lane = tid & 31;
  {
    float v[BNB / 16][4];
#pragma unroll
    for (int s = 0; s < BNB / 16; ++s) {
      const int i = warp + 16 * s;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = lane + 32 * q;
        v[s][q] = (i < kb && j <= i) ? __ldcg(F + (size_t)(k0 + i) * NF + k0 + j) : 0.f;
      }
    }
#pragma unroll
    for (int s = 0; s < BNB / 16; ++s) {
      const int i = warp + 16 * s;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = lane + 32 * q;
        if (i < kb && j <= i) P[tri_index(i, j)] = v[s][q];
      }
    }
  }
  __syncthreads();
  chol_blocked(P, PT, ldp, kb, &s_bad);
  if (tid == 0 && s_bad) set_status(c.w.status, D4_ERR_EEQ_SINGULAR);
#pragma unroll
  for (int s = 0; s < BNB / 16; ++s) {
    const int i = warp + 16 * s;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = lane + 32 * q;
      if (i < kb && j <= i) F[(size_t)(k0 + i) * NF + k0 + j] = P[tri_index(i, j)];
    }
  }
}

size_t eeq_big_diag_smem() {
  const size_t p = (BNB * (BNB + 1) / 2 + 3) & ~3;
  return 4 * (p + (size_t)32 * chol_panel_ld(BNB));
}

// Full inverse X of every panel's diagonal block (grid: panels x
// structures), from the diagonal kernel's form: block forward substitution
// (X_cc = D_c^-1, X_rc = -D_r^-1 sum_k L_rk X_kc), written over the block
// (lower part).  The block sweeps and the 512-block inverses use it.
__global__ void __launch_bounds__(512) eeq_big_pinv_kernel(Ctx c) {
  extern __shared__ float4 s_dyn4[];
  float *P = reinterpret_cast<float *>(s_dyn4);  // packed kb x kb
  const int ldp = chol_panel_ld(BNB);
  float *PT = P + ((BNB * (BNB + 1) / 2 + 3) & ~3);  // T scratch, 32 x ldp
  float *Xs = PT + 32 * ldp;                         // dense [BNB][BNB + 1]
  const int k0 = blockIdx.x * BNB, b = blockIdx.y;
  const int m = c.w.n_real[b];
  if (k0 >= m) return;
  const int kb = min(BNB, m - k0);
  const int N = c.N;
  const int NF = eeq_ldf(N);
  float *F = c.w.eeq_F + (size_t)b * N * NF;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int tri = kb * (kb + 1) / 2;
  for (int t = tid; t < tri; t += nt) {
    int i, j;
    tri_tile(t, i, j);
    P[t] = F[(size_t)(k0 + i) * NF + k0 + j];
  }
  __syncthreads();
  constexpr int LX = BNB + 1;
  // X = 0, diagonal 32-blocks = their inverses (held by P)
  for (int t = tid; t < BNB * BNB; t += nt) {
    const int i = t / BNB, j = t % BNB;
    Xs[i * LX + j] = (i < kb && j <= i && (i >> 5) == (j >> 5)) ? P[tri_index(i, j)] : 0.f;
  }
  __syncthreads();
  const int nbk = (kb + 31) >> 5;
  for (int rb = 1; rb < nbk; ++rb) {
    const int r0 = rb * 32, rows = min(32, kb - r0), cols = r0;
    // T[r][c] = sum_{k in [c's block, r0)} L[r0 + r][k] X[k][c]
    for (int t = tid; t < rows * cols; t += nt) {
      const int r = t / cols, cc = t % cols;
      const float *lr = P + tri_index(r0 + r, 0);
      float acc = 0.f;
      for (int k = (cc >> 5) << 5; k < r0; ++k) acc = fmaf(lr[k], Xs[k * LX + cc], acc);
      PT[r * ldp + cc] = acc;
    }
    __syncthreads();
    // X[r0 + r][c] = -sum_{r' <= r} D^-1[r][r'] T[r'][c]
    for (int t = tid; t < rows * cols; t += nt) {
      const int r = t / cols, cc = t % cols;
      float acc = 0.f;
      for (int q = 0; q <= r; ++q) acc = fmaf(P[tri_index(r0 + r, r0 + q)], PT[q * ldp + cc], acc);
      Xs[(r0 + r) * LX + cc] = -acc;
    }
    __syncthreads();
  }
  for (int t = tid; t < kb * kb; t += nt) {
    const int i = t / kb, j = t % kb;
    if (j <= i) F[(size_t)(k0 + i) * NF + k0 + j] = Xs[i * LX + j];
  }
}

size_t eeq_big_pinv_smem() {
  const size_t p = (BNB * (BNB + 1) / 2 + 3) & ~3;
  return 4 * (p + (size_t)32 * chol_panel_ld(BNB) + (size_t)BNB * (BNB + 1));
}

// Split panel operands of the trailing updates: the rows of L21 as TF32
// pairs hi = tf32(v), lo = tf32(v - hi), in 128-row blocks (relative to the
// first trailing row), each block 8 chunks of 16 columns, each chunk a hi and
// a lo plane of 128 rows x 16 values in the canonical K-major layout of the
// MMA (LBO 128 bytes, SBO 512 bytes), so that a trailing-update CTA copies
// its operands as contiguous 8 KB planes.  Two buffers, alternating with the
// panel's parity (the look-ahead writes panel p + 1 while panel p is read).
constexpr int SY_KC = 16;                       // K per chunk of the trailing update
constexpr int SY_LBO = 128;                     // bytes between core matrices along K
constexpr int SY_SBO = (SY_KC / 4) * SY_LBO;    // bytes between groups of 8 rows
constexpr int SY_PLANE = (BNB / 8) * SY_SBO;    // bytes of one 128 x 16 plane (8192)
constexpr int SY_NCH = BNB / SY_KC;             // chunks per panel
static_assert(EEQ_BNB == BNB && (size_t)SY_NCH * 2 * SY_PLANE == EEQ_OPND_BLOCK,
              "operand block layout");

__device__ __forceinline__ unsigned char *opnd_block(const Ctx &c, int par, int b, int rb) {
  return c.w.eeq_P + (((size_t)par * c.B + b) * eeq_nblk(c.N) + rb) * EEQ_OPND_BLOCK;
}

// Panel rows [t0 + 64 blockIdx.x, +64): L21 solves L21 L11^T = A21, by
// block substitution over the panel's 32-column blocks with the diagonal
// kernel's form of L11 (factor below the 32 x 32 diagonal blocks, their
// inverses D^-1 on them):  Y_c = (A_c - sum_{k < c} Y_k L_ck^T) D_c^-T.
// Written to F and, split, to the operand buffer ``par``.  Thread tile 2
// rows x 4 columns of the current 32-column block; L11 transposed and the
// rows transposed in shared memory.
constexpr int PN_LLT = BNB + 4, PN_LAT = 64 + 2;
__global__ void __launch_bounds__(256, 1) eeq_big_panel_kernel(Ctx c, int k0, int par) {
  extern __shared__ float4 s_dyn4[];
  float *LT = reinterpret_cast<float *>(s_dyn4);  // LT[k][col] = L11[col][k], 0 for k > col
  float *AT = LT + BNB * PN_LLT;                   // AT[cc][row] = A21[row][cc], then L21
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  if (k0 >= m) return;
  const int kb = min(BNB, m - k0);
  const int t0 = k0 + kb;
  const int r0 = t0 + 64 * blockIdx.x;
  if (r0 >= m || kb != BNB) return;
  const int N = c.N;
  const int NF = eeq_ldf(N);
  float *F = c.w.eeq_F + (size_t)b * N * NF;
  const int tid = threadIdx.x;
  // Past the early returns the panel is full (kb = BNB: a shorter panel is
  // the structure's last, with no rows below it).  L11 and the 64 rows of
  // A21 arrive as 16-byte loads, eight in flight per thread before any is
  // stored; the lanes of a warp take consecutive columns of L11 (rows of
  // A21), so that the transposed stores hit consecutive banks.
  for (int s0 = 0; s0 < BNB * BNB / 4 / 256; s0 += 8) {
    float4 v[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const int f = tid + 256 * (s0 + s), col = f & (BNB - 1), kg = f >> 7;
      v[s] = __ldcg(reinterpret_cast<const float4 *>(F + (size_t)(k0 + col) * NF + k0 + 4 * kg));
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const int f = tid + 256 * (s0 + s), col = f & (BNB - 1), kg = f >> 7;
      const float e[4] = {v[s].x, v[s].y, v[s].z, v[s].w};
#pragma unroll
      for (int q = 0; q < 4; ++q) LT[(4 * kg + q) * PN_LLT + col] = 4 * kg + q <= col ? e[q] : 0.f;
    }
  }
  {
    float4 v[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const int f = tid + 256 * s, row = f & 63, cg = f >> 6;
      const int i = r0 + row;
      v[s] = i < m ? __ldcg(reinterpret_cast<const float4 *>(F + (size_t)i * NF + k0 + 4 * cg))
                   : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const int f = tid + 256 * s, row = f & 63, cg = f >> 6;
      AT[(4 * cg) * PN_LAT + row] = v[s].x;
      AT[(4 * cg + 1) * PN_LAT + row] = v[s].y;
      AT[(4 * cg + 2) * PN_LAT + row] = v[s].z;
      AT[(4 * cg + 3) * PN_LAT + row] = v[s].w;
    }
  }
  __syncthreads();
  // rows 2 ty, 2 ty + 1; columns 4 tx .. + 3 of a block: warp w owns rows
  // 8 w .. 8 w + 7 from here on, so that only its own lanes synchronise
  const int ty = tid >> 3, tx = tid & 7;
  const int nb32 = (kb + 31) >> 5;
  for (int cb = 0; cb < nb32; ++cb) {
    const int c0 = 32 * cb + 4 * tx;
    float acc[2][4];
#pragma unroll
    for (int v = 0; v < 2; ++v)
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[v][u] = 0.f;
    // sum_{k < 32 cb} Y_k L_ck^T (Y of the earlier blocks is in AT)
#pragma unroll 4
    for (int k = 0; k < 32 * cb; ++k) {
      const float2 y = *reinterpret_cast<const float2 *>(AT + k * PN_LAT + 2 * ty);
      const float4 l = *reinterpret_cast<const float4 *>(LT + k * PN_LLT + c0);
      const float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        acc[0][u] = fmaf(y.x, lv[u], acc[0][u]);
        acc[1][u] = fmaf(y.y, lv[u], acc[1][u]);
      }
    }
    // Z_c = A_c - that, in place (each entry read and written by its thread)
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float *z = AT + (c0 + u) * PN_LAT + 2 * ty;
      z[0] -= acc[0][u];
      z[1] -= acc[1][u];
    }
    __syncwarp();
    // Y_c = Z_c D_c^-T: Y[r][c] = sum_q Z[r][q] D^-1[c][q] (LT is 0 above)
    float y[2][4];
#pragma unroll
    for (int v = 0; v < 2; ++v)
#pragma unroll
      for (int u = 0; u < 4; ++u) y[v][u] = 0.f;
#pragma unroll 4
    for (int q = 32 * cb; q < 32 * cb + 32; ++q) {
      const float2 zr = *reinterpret_cast<const float2 *>(AT + q * PN_LAT + 2 * ty);
      const float4 l = *reinterpret_cast<const float4 *>(LT + q * PN_LLT + c0);
      const float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        y[0][u] = fmaf(zr.x, lv[u], y[0][u]);
        y[1][u] = fmaf(zr.y, lv[u], y[1][u]);
      }
    }
    __syncwarp();  // every lane has read Z_c
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float *z = AT + (c0 + u) * PN_LAT + 2 * ty;
      z[0] = y[0][u];
      z[1] = y[1][u];
    }
    __syncwarp();
  }
  // L21 rows to F (the warp's own rows, lanes over 4-column groups) and,
  // split, to the operands of the trailing update (only full panels have one)
  const bool split = kb == BNB;
  const int warp = tid >> 5, lane = tid & 31;
  const int col = 4 * lane;
  for (int rr = 8 * warp; rr < 8 * warp + 8; ++rr) {
    const int i = r0 + rr;
    if (i >= m || col >= kb) continue;
    float v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = AT[(col + e) * PN_LAT + rr];
    *reinterpret_cast<float4 *>(F + (size_t)i * NF + k0 + col) = make_float4(v[0], v[1], v[2], v[3]);
    if (split) {
      const int q = i - t0, r = q & (BNB - 1);
      unsigned char *dst = opnd_block(c, par, b, q / BNB) + (size_t)(col / SY_KC) * 2 * SY_PLANE +
                           (r >> 3) * SY_SBO + ((col % SY_KC) >> 2) * SY_LBO + (r & 7) * 16;
      float h[4], l[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        h[e] = tc::to_tf32(v[e]);
        l[e] = tc::to_tf32(v[e] - h[e]);
      }
      *reinterpret_cast<float4 *>(dst) = make_float4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<float4 *>(dst + SY_PLANE) = make_float4(l[0], l[1], l[2], l[3]);
    }
  }
}

size_t eeq_big_panel_smem() { return 4 * ((size_t)BNB * PN_LLT + (size_t)BNB * PN_LAT); }

// Trailing update A22 -= L21 L21^T of the lower 128 x 128 tiles (ti >= tj)
// right of the panel, on the tensor cores.  One CTA (128 threads) per tile:
//  - the split operands of the tile's two row blocks (written by the panel
//    kernel) arrive in chunks of 16 columns -- four 8 KB planes (A hi, A lo,
//    B hi, B lo) -- by 16-byte asynchronous copies, double-buffered: the
//    copies of chunk k + 1 are in flight while the tensor cores work on k;
//  - one thread issues tcgen05 kind::tf32 MMAs (M = N = 128: lo hi, hi lo,
//    hi hi per k-step of 8) into a 128-column tensor-memory accumulator;
//  - the tile goes from tensor memory to shared memory (thread = row,
//    negated) and every row is added to the matrix by one bulk reduction
//    (cp.reduce.async.bulk .add.f32, performed at L2: no read of the matrix
//    into the SM).  Diagonal tiles update their upper half too, which no
//    later step reads; rows beyond the structure are skipped, columns
//    beyond it receive sums of padding (never read).
// The split products keep the update at about FP32 accuracy (a few 1e-7
// relative), which the FP64 refinement of the solves absorbs.
constexpr int SY_STAGE = 4 * SY_PLANE;          // A hi, A lo, B hi, B lo of one chunk
constexpr int SY_COLS = 128;                    // tensor memory: the 128 x 128 tile
constexpr int SY_TLD = BNB + 4;                 // row stride (floats) of the staged tile
constexpr int SY_SMEM =
    (2 * SY_STAGE > 4 * BNB * SY_TLD) ? 2 * SY_STAGE : 4 * BNB * SY_TLD;

// Which tiles a launch updates (tile coordinates relative to the trailing
// matrix): every lower tile, only the first tile column (the next panel's
// columns, on the factorisation's critical path), or every tile right of it.
enum SyrkTiles : int { SYRK_ALL = 0, SYRK_FIRST_COLUMN = 1, SYRK_REST = 2 };

__global__ void __launch_bounds__(BNB) eeq_big_syrk_kernel(Ctx c, int k0, int tiles, int par) {
  extern __shared__ __align__(1024) unsigned char s_raw[];
  __shared__ unsigned long long s_mbar;
  __shared__ uint32_t s_tmem;
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  if (k0 + BNB >= m) return;  // no trailing matrix (a last, partial panel has none)
  const int t0 = k0 + BNB;
  int ti, tj;
  if (tiles == SYRK_FIRST_COLUMN) {
    ti = blockIdx.x;
    tj = 0;
  } else {
    tri_tile(blockIdx.x, ti, tj);
    if (tiles == SYRK_REST) {
      ++ti;
      ++tj;
    }
  }
  const int i0 = t0 + BNB * ti, j0 = t0 + BNB * tj;
  if (i0 >= m) return;
  const int N = c.N;
  const int NF = eeq_ldf(N);
  float *F = c.w.eeq_F + (size_t)b * N * NF;
  const unsigned char *PA = opnd_block(c, par, b, ti);
  const unsigned char *PB = opnd_block(c, par, b, tj);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t mbar = tc::smem_u32(&s_mbar);
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(&s_tmem), SY_COLS);
  if (tid == 0) tc::mbar_init(mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  constexpr uint32_t IDESC = tc::idesc_tf32(BNB, BNB);
  // chunk ch -> stage st: 32 KB, 16 bytes per thread and step
  auto issue = [&](int ch, int st) {
    unsigned char *dst = s_raw + st * SY_STAGE;
#pragma unroll
    for (int q = 0; q < SY_STAGE / (16 * BNB); ++q) {
      const int byte = (q * BNB + tid) * 16;
      const int plane = byte / SY_PLANE, off = byte % SY_PLANE;  // A hi, A lo, B hi, B lo
      const unsigned char *src =
          (plane < 2 ? PA : PB) + ((size_t)ch * 2 + (plane & 1)) * SY_PLANE + off;
      tc::cp_async16(dst + byte, src);
    }
    tc::cp_async_commit();
  };
  issue(0, 0);
  bool timed_out = false;
  int last = -1;  // last chunk whose MMAs were committed (uniform over the CTA)
  for (int ch = 0; ch < SY_NCH; ++ch) {
    // stage (ch + 1) & 1 was read by the MMAs of chunk ch - 1
    if (ch > 0) {
      const bool done = tc::mbar_wait(mbar, (uint32_t)((ch - 1) & 1));
      if (__syncthreads_or(!done)) {
        timed_out = true;
        break;
      }
    }
    if (ch + 1 < SY_NCH) {
      issue(ch + 1, (ch + 1) & 1);
      tc::cp_async_wait<1>();
    } else {
      tc::cp_async_wait<0>();
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t base = tc::smem_u32(s_raw + (ch & 1) * SY_STAGE);
#pragma unroll
      for (int pr = 0; pr < 3; ++pr) {  // lo hi, hi lo, hi hi
        const uint32_t ab = base + (pr == 0 ? SY_PLANE : 0);
        const uint32_t bb = base + 2 * SY_PLANE + (pr == 1 ? SY_PLANE : 0);
#pragma unroll
        for (int s8 = 0; s8 < SY_KC / 8; ++s8)
          tc::mma_tf32(tmem, tc::desc_kmajor(ab + 2 * SY_LBO * s8, SY_LBO, SY_SBO),
                       tc::desc_kmajor(bb + 2 * SY_LBO * s8, SY_LBO, SY_SBO), IDESC,
                       (ch > 0 || pr > 0 || s8 > 0) ? 1u : 0u);
      }
      tc::commit(mbar);
    }
    last = ch;
  }
  tc::cp_async_wait<0>();  // nothing of ours may land in shared memory after we leave
  const bool last_done = !timed_out && tc::mbar_wait(mbar, (uint32_t)(last & 1));
  if (__syncthreads_or(!last_done)) {
    if (tid == 0) set_status(c.w.status, D4_ERR_DEVICE_TIMEOUT);
    // one more bounded wait for the last committed MMAs, then release
    if (last >= 0) tc::mbar_wait(mbar, (uint32_t)(last & 1));
  } else {
    // tensor memory -> shared tile (thread = row, negated) -> one bulk
    // reduction per row into the matrix
    tc::fence_after_sync();
    float *T = reinterpret_cast<float *>(s_raw);
    const uint32_t t_lane = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int cc = 0; cc < BNB; cc += 16) {
      uint32_t v[16];
      tc::tmem_ld16(tmem + t_lane + cc, v);
      tc::tmem_ld_wait();
#pragma unroll
      for (int u = 0; u < 16; u += 4)
        *reinterpret_cast<float4 *>(T + tid * SY_TLD + cc + u) =
            make_float4(-__uint_as_float(v[u]), -__uint_as_float(v[u + 1]),
                        -__uint_as_float(v[u + 2]), -__uint_as_float(v[u + 3]));
    }
    const int i = i0 + tid;
    if (i < m) {
      tc::fence_async_smem();
      const int ncol = min(BNB, NF - j0);  // a multiple of 4: NF and j0 are
      tc::bulk_reduce_add_f32(F + (size_t)i * NF + j0, T + tid * SY_TLD, (uint32_t)(4 * ncol));
      tc::bulk_commit();
      tc::bulk_wait_read();
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_free(tmem, SY_COLS);
  }
}

size_t eeq_big_syrk_smem() { return (size_t)SY_SMEM; }

// ---------------------------------------------------------------- solves

// Right-hand sides and starting point: x = 0, v = FP32 rounding of b.
// Forward: b = (-chi + kcn sqrt(cn_q), 1); adjoint: b = dE/dq.
__global__ void eeq_big_rhs_kernel(Ctx c, int adjoint) {
  const int b = blockIdx.y;
  const int N = c.N;
  const int m = c.w.n_real[b];
  if (blockIdx.x == 0 && threadIdx.x < EEQ_BIG_REFINE) c.w.eeq_res[b * EEQ_BIG_REFINE + threadIdx.x] = 0u;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const size_t ia = (size_t)b * N + c.w.ridx[(size_t)b * N + k];
  const size_t o = (size_t)b * 2 * N + k;
  dfl v;
  if (adjoint) {
    v = df_from(c.w.dEdq[ia]);
  } else {
    const int z = c.w.z[ia];
    const double cq = c.w.cnq[ia];
    v = df_from(-c.tab.eeq_chi[z] + c.tab.eeq_kcn[z] * (cq > 0.0 ? sqrt(cq) : 0.0));
    c.w.eeq_B[o + N] = make_float2(1.f, 0.f);
    c.w.eeq_X[o + N] = make_float2(0.f, 0.f);
    c.w.eeq_V[o + N] = 1.f;
  }
  c.w.eeq_B[o] = make_float2(v.hi, v.lo);
  c.w.eeq_X[o] = make_float2(0.f, 0.f);
  c.w.eeq_V[o] = v.hi;
}

// ---------------------------------------------------------------- block inverses

// Inverses of the 512 x 512 diagonal blocks of the factor (four panels
// each), so that the triangular sweeps advance 512 rows per step with plain
// matrix-vector products.  Xd[b][s] (row-major, lower) is built by block
// forward substitution over the panels of block s:
//   W_rr = X_rr (the panel inverses the factorisation left on F's diagonal),
//   W_rc = -X_rr sum_{j=c}^{r-1} L_rj W_jc   (r = 1..3, c < r).
// Rows and columns beyond the structure's size are zero.
constexpr int SBP = EEQ_SB / BNB;  // panels per block

__device__ __forceinline__ float *xd_block(const Ctx &c, int b, int sblk) {
  return c.w.eeq_Xd + ((size_t)b * eeq_nsb(c.N) + sblk) * EEQ_SB * EEQ_SB;
}

__global__ void __launch_bounds__(256) eeq_blkinv_init_kernel(Ctx c) {
  const int sblk = blockIdx.x, b = blockIdx.y;
  const int m = c.w.n_real[b];
  const int s0 = sblk * EEQ_SB;
  if (s0 >= m) return;
  const int N = c.N;
  const int NF = eeq_ldf(N);
  const float *F = c.w.eeq_F + (size_t)b * N * NF;
  float *X = xd_block(c, b, sblk);
  for (int t = threadIdx.x; t < EEQ_SB * EEQ_SB; t += blockDim.x) {
    const int i = t / EEQ_SB, j = t % EEQ_SB;
    const int gi = s0 + i, gj = s0 + j;
    const bool diag = (i / BNB) == (j / BNB) && j <= i && gi < m;
    X[t] = diag ? F[(size_t)gi * NF + gj] : 0.f;
  }
}

// Sub-block row r of every block: one CTA per (block, column sub-block cc < r)
// forms T = sum_j L_rj W_jc (K = 128 (r - cc)) and then W_rc = -X_rr T, both
// as 128 x 128 products with 8 x 8 register tiles (256 threads).
constexpr int IK = 16;
__global__ void __launch_bounds__(256) eeq_blkinv_step_kernel(Ctx c, int r) {
  extern __shared__ float4 s_dyn4[];
  float *As = reinterpret_cast<float *>(s_dyn4);  // [IK][BNB + 4]: A^T chunk
  float *Bs = As + IK * (BNB + 4);                 // [IK][BNB + 4]: B chunk
  float *Ts = Bs + IK * (BNB + 4);                 // [BNB][BNB + 4]: T
  constexpr int LD = BNB + 4;
  const int b = blockIdx.y;
  const int sblk = blockIdx.x / r, cc = blockIdx.x % r;
  const int m = c.w.n_real[b];
  const int s0 = sblk * EEQ_SB;
  if (s0 + r * BNB >= m) return;  // sub-block row r does not exist
  const int N = c.N;
  const int NF = eeq_ldf(N);
  const float *F = c.w.eeq_F + (size_t)b * N * NF;
  float *X = xd_block(c, b, sblk);
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int lrow = tid >> 1, lcol = (tid & 1) * 8;
  const int gr0 = s0 + r * BNB;  // first global row of sub-block row r
  float acc[8][8];
#pragma unroll
  for (int q = 0; q < 8; ++q)
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[q][u] = 0.f;
  // T = sum_j L[r][j] W[j][cc]: A = L rows gr0.., columns s0 + 128 j ..; B = W rows 128 j..
  for (int j = cc; j < r; ++j) {
    for (int k0 = 0; k0 < BNB; k0 += IK) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int kk = lcol + q;
        const int gi = gr0 + lrow, gk = s0 + j * BNB + k0 + kk;
        As[kk * LD + lrow] = (gi < m && gk < m) ? F[(size_t)gi * NF + gk] : 0.f;
        Bs[kk * LD + lrow] = X[(size_t)(j * BNB + k0 + kk) * EEQ_SB + cc * BNB + lrow];
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < IK; ++kk) {
        const float4 a0 = *reinterpret_cast<const float4 *>(&As[kk * LD + 8 * ty]);
        const float4 a1 = *reinterpret_cast<const float4 *>(&As[kk * LD + 8 * ty + 4]);
        const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[kk * LD + 8 * tx]);
        const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[kk * LD + 8 * tx + 4]);
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[q][u] = fmaf(av[q], bv[u], acc[q][u]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int q = 0; q < 8; ++q)
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      Ts[(8 * ty + q) * LD + 8 * tx + u] = acc[q][u];
      acc[q][u] = 0.f;
    }
  __syncthreads();
  // W[r][cc] = -X_rr T (X_rr: Xd's diagonal sub-block r)
  for (int k0 = 0; k0 < BNB; k0 += IK) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int kk = lcol + q;
      As[kk * LD + lrow] = X[(size_t)(r * BNB + lrow) * EEQ_SB + r * BNB + k0 + kk];
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < IK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4 *>(&As[kk * LD + 8 * ty]);
      const float4 a1 = *reinterpret_cast<const float4 *>(&As[kk * LD + 8 * ty + 4]);
      const float4 b0 = *reinterpret_cast<const float4 *>(&Ts[(k0 + kk) * LD + 8 * tx]);
      const float4 b1 = *reinterpret_cast<const float4 *>(&Ts[(k0 + kk) * LD + 8 * tx + 4]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[q][u] = fmaf(av[q], bv[u], acc[q][u]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int i = r * BNB + 8 * ty + q;
    const bool rok = s0 + i < m;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = cc * BNB + 8 * tx + u;
      X[(size_t)i * EEQ_SB + j] = (rok && s0 + j < m) ? -acc[q][u] : 0.f;
    }
  }
}

size_t eeq_blkinv_smem() { return 4 * ((size_t)2 * IK * (BNB + 4) + (size_t)BNB * (BNB + 4)); }

// After the steps: the upper triangle of every block (zero until here)
// receives the transpose of its lower triangle, so that the backward sweep
// reads X_s^T by rows as the forward sweep reads X_s.  One CTA per pair of
// 32 x 32 tiles (lower tile (ti, tj), ti >= tj, and its mirror), through
// shared memory; grid (136, blocks, structures).
constexpr int MIR_TILES = (EEQ_SB / 32) * (EEQ_SB / 32 + 1) / 2;
__global__ void __launch_bounds__(256) eeq_blkinv_mirror_kernel(Ctx c) {
  __shared__ float t[32][33];
  const int b = blockIdx.z, sblk = blockIdx.y;
  const int m = c.w.n_real[b];
  if (sblk * EEQ_SB >= m) return;
  int ti, tj;
  tri_tile(blockIdx.x, ti, tj);
  float *X = xd_block(c, b, sblk);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) t[r][tx] = X[(size_t)(32 * ti + r) * EEQ_SB + 32 * tj + tx];
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int gi = 32 * tj + r, gk = 32 * ti + tx;
    if (gk > gi) X[(size_t)gi * EEQ_SB + gk] = t[tx][r];
  }
}

// ---------------------------------------------------------------- sweeps

// Diagonal block s of a sweep, nr right-hand sides, warp per output row i:
// forward dst_i = sum_{k <= i} X_s[i][k] src_k, backward
// dst_i = sum_{k >= i} X_s^T[i][k] src_k -- both from row i of the block
// (X_s below the diagonal, X_s^T above it).  A lane's sixteen loads of the
// row are issued before the first product.
__global__ void __launch_bounds__(256, 1) eeq_sweep_diag_kernel(Ctx c, int sblk, int it, int trans,
                                                                int nr, int src_y) {
  __shared__ float s_v[2][EEQ_SB];
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  const int s0 = sblk * EEQ_SB;
  if (s0 >= m || big_skip(c, b, it)) return;
  const int kb = min(EEQ_SB, m - s0);
  const int N = c.N;
  const float *src = (src_y ? c.w.eeq_Y : c.w.eeq_V) + (size_t)b * 2 * N;
  float *dst = (src_y ? c.w.eeq_V : c.w.eeq_Y) + (size_t)b * 2 * N;
  const float *X = xd_block(c, b, sblk);
  for (int t = threadIdx.x; t < 2 * EEQ_SB; t += blockDim.x) {
    const int r = t / EEQ_SB, k = t % EEQ_SB;
    s_v[r][k] = (r < nr && k < kb) ? src[(size_t)r * N + s0 + k] : 0.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);  // output index
  if (i >= kb) return;
  const float *row = X + (size_t)i * EEQ_SB;
  const int k_lo = trans ? i : 0, k_hi = trans ? kb - 1 : i;
  float x[EEQ_SB / 32];
#pragma unroll
  for (int t = 0; t < EEQ_SB / 32; ++t) {
    const int k = lane + 32 * t;
    x[t] = (k >= k_lo && k <= k_hi) ? row[k] : 0.f;
  }
  float a0 = 0.f, a1 = 0.f;
#pragma unroll
  for (int t = 0; t < EEQ_SB / 32; ++t) {
    const int k = lane + 32 * t;
    a0 = fmaf(x[t], s_v[0][k], a0);
    a1 = fmaf(x[t], s_v[1][k], a1);
  }
  a0 = warp_sumf(a0);
  if (nr == 2) a1 = warp_sumf(a1);
  if (lane == 0) {
    dst[s0 + i] = a0;
    if (nr == 2) dst[N + s0 + i] = a1;
  }
}

// Forward sweep update below block s: V_i -= F[i][blk] . Y_blk.  Four rows
// per warp, lane l over the block's columns 4 l + 128 t (16-byte loads: the
// rows of F and the block start are 16-byte aligned): a lane's sixteen
// matrix loads and the old V entries of its rows are issued together (one
// round trip), Y_blk is staged in shared memory once per CTA.
constexpr int BL_ROWS = 4;
__global__ void __launch_bounds__(256, 2) eeq_sweep_below_kernel(Ctx c, int sblk, int it, int nr) {
  __shared__ __align__(16) float s_y[2][EEQ_SB];
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  const int s0 = sblk * EEQ_SB;
  if (s0 >= m || big_skip(c, b, it)) return;
  const int kb = min(EEQ_SB, m - s0);
  const int i0 = s0 + kb + (blockIdx.x * 8 + (threadIdx.x >> 5)) * BL_ROWS;
  if (s0 + kb + blockIdx.x * 8 * BL_ROWS >= m) return;  // the whole CTA is past the end
  const int N = c.N;
  const float *Yg = c.w.eeq_Y + (size_t)b * 2 * N + s0;
  for (int t = threadIdx.x; t < 2 * EEQ_SB; t += blockDim.x) {
    const int r = t / EEQ_SB, k = t % EEQ_SB;
    s_y[r][k] = (r < nr && k < kb) ? Yg[(size_t)r * N + k] : 0.f;
  }
  __syncthreads();
  if (i0 >= m) return;
  const int lane = threadIdx.x & 31;
  const int NF = eeq_ldf(N);
  const float *base = c.w.eeq_F + (size_t)b * N * NF + (size_t)i0 * NF + s0;
  float *V = c.w.eeq_V + (size_t)b * 2 * N;
  constexpr int NT = EEQ_SB / 128;  // float4 steps per row
  float4 x[BL_ROWS][NT];
#pragma unroll
  for (int r = 0; r < BL_ROWS; ++r)
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int k = 4 * lane + 128 * t;  // k < kb keeps k + 3 inside the row's NF columns
      float4 v = (i0 + r < m && k < kb)
                     ? *reinterpret_cast<const float4 *>(base + (size_t)r * NF + k)
                     : make_float4(0.f, 0.f, 0.f, 0.f);
      if (k + 3 >= kb) {  // columns from kb on hold no data of this call
        if (k + 1 >= kb) v.y = 0.f;
        if (k + 2 >= kb) v.z = 0.f;
        v.w = 0.f;
      }
      x[r][t] = v;
    }
  const bool own = lane < BL_ROWS && i0 + lane < m;  // lane r writes row i0 + r
  const float v0 = own ? V[i0 + lane] : 0.f;
  const float v1 = own && nr == 2 ? V[N + i0 + lane] : 0.f;
  float o0 = 0.f, o1 = 0.f;
#pragma unroll
  for (int r = 0; r < BL_ROWS; ++r) {
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int k = 4 * lane + 128 * t;  // s_y is 0 from kb on
      const float4 y0 = *reinterpret_cast<const float4 *>(&s_y[0][k]);
      const float4 y1 = *reinterpret_cast<const float4 *>(&s_y[1][k]);
      a0 = fmaf(x[r][t].x, y0.x, fmaf(x[r][t].y, y0.y, fmaf(x[r][t].z, y0.z, fmaf(x[r][t].w, y0.w, a0))));
      a1 = fmaf(x[r][t].x, y1.x, fmaf(x[r][t].y, y1.y, fmaf(x[r][t].z, y1.z, fmaf(x[r][t].w, y1.w, a1))));
    }
    a0 = warp_sumf(a0);
    if (nr == 2) a1 = warp_sumf(a1);
    if (lane == r) {
      o0 = a0;
      o1 = a1;
    }
  }
  if (own) {
    V[i0 + lane] = v0 - o0;
    if (nr == 2) V[N + i0 + lane] = v1 - o1;
  }
}

// Backward sweep update above block s: Y_i -= sum_k F[s0 + k][i] V_{s0+k}
// for i < s0.  A CTA takes 64 columns i (lane l: i and i + 1 from 2 l, one
// 8-byte load per row, coalesced over i) and splits the block's rows k over
// its eight warps (64 each, sixteen loads in flight per lane); the warps'
// partial sums meet in shared memory.
constexpr int AB_COLS = 64;
__global__ void __launch_bounds__(256, 2) eeq_sweep_above_kernel(Ctx c, int sblk, int it, int nr) {
  __shared__ float s_v[2][EEQ_SB];
  __shared__ float2 s_part[2][8][AB_COLS / 2];
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  const int s0 = sblk * EEQ_SB;
  if (s0 >= m || big_skip(c, b, it)) return;
  const int kb = min(EEQ_SB, m - s0);
  const int N = c.N;
  const float *V = c.w.eeq_V + (size_t)b * 2 * N;
  float *Y = c.w.eeq_Y + (size_t)b * 2 * N;
  for (int t = threadIdx.x; t < 2 * EEQ_SB; t += blockDim.x) {
    const int r = t / EEQ_SB, k = t % EEQ_SB;
    s_v[r][k] = (r < nr && k < kb) ? V[(size_t)r * N + s0 + k] : 0.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * AB_COLS + 2 * lane;  // i + 1 < s0 with i (s0 is even)
  float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
  if (i < s0) {
    const int NF = eeq_ldf(N);
    const float *col = c.w.eeq_F + (size_t)b * N * NF + (size_t)s0 * NF + i;
    const int kbeg = (EEQ_SB / 8) * w;
#pragma unroll
    for (int h = 0; h < EEQ_SB / 8; h += 16) {
      float2 x[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const int k = kbeg + h + t;
        x[t] = k < kb ? *reinterpret_cast<const float2 *>(col + (size_t)k * NF)
                      : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const int k = kbeg + h + t;
        a0.x = fmaf(x[t].x, s_v[0][k], a0.x);
        a0.y = fmaf(x[t].y, s_v[0][k], a0.y);
        a1.x = fmaf(x[t].x, s_v[1][k], a1.x);
        a1.y = fmaf(x[t].y, s_v[1][k], a1.y);
      }
    }
  }
  s_part[0][w][lane] = a0;
  s_part[1][w][lane] = a1;
  __syncthreads();
  if (w == 0 && i < s0) {
    float2 t0 = make_float2(0.f, 0.f), t1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      t0.x += s_part[0][q][lane].x;
      t0.y += s_part[0][q][lane].y;
      t1.x += s_part[1][q][lane].x;
      t1.y += s_part[1][q][lane].y;
    }
    Y[i] -= t0.x;
    Y[i + 1] -= t0.y;
    if (nr == 2) {
      Y[N + i] -= t1.x;
      Y[N + i + 1] -= t1.y;
    }
  }
}

// x += v (double-float).
__global__ void eeq_big_update_kernel(Ctx c, int it, int nr) {
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m || big_skip(c, b, it)) return;
  const int N = c.N;
  for (int r = 0; r < nr; ++r) {
    const size_t o = (size_t)b * 2 * N + (size_t)r * N + k;
    const float2 x = c.w.eeq_X[o];
    const dfl s = df_add(dfl{x.x, x.y}, dfl{c.w.eeq_V[o], 0.f});
    c.w.eeq_X[o] = make_float2(s.hi, s.lo);
  }
}

// r = b - (hi + lo) x in double-float; v <- FP32 r and the structure's max
// |r| of this iteration.  RS_ROWS rows per warp (every x entry read serves
// them all), lanes over columns, the loads of the next 128 columns in
// flight while the current ones are summed.  VEC (rows 16-byte aligned: N a
// multiple of four): lane l takes columns 4 l .. 4 l + 3 of each 128 as one
// float4 per row and plane; else columns l, l + 32, l + 64, l + 96.
constexpr int RS_ROWS = 2;
template <int NR, bool VEC>
__global__ void __launch_bounds__(256, 3) eeq_big_residual_kernel(Ctx c, int it) {
  const int b = blockIdx.y;
  const int m = c.w.n_real[b];
  if (big_skip(c, b, it)) return;
  const int k0 = (blockIdx.x * 8 + (threadIdx.x >> 5)) * RS_ROWS;
  if (k0 >= m) return;
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  const float *hr = c.w.eeq_hi + (size_t)b * N * N + (size_t)k0 * N;
  const float *lr = c.w.eeq_lo + (size_t)b * N * N + (size_t)k0 * N;
  const float2 *X = c.w.eeq_X + (size_t)b * 2 * N;
  dfl acc[RS_ROWS][NR];
#pragma unroll
  for (int r = 0; r < RS_ROWS; ++r)
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[r][q] = {0.f, 0.f};
  // column of element u (0..3) of the lane in the 128-column step at l0
  auto col = [&](int l0, int u) { return VEC ? l0 + 4 * lane + u : l0 + lane + 32 * u; };
  auto load = [&](float (&hh)[RS_ROWS][4], float (&ll)[RS_ROWS][4], int l0) {
#pragma unroll
    for (int r = 0; r < RS_ROWS; ++r) {
      const bool rok = k0 + r < m;
      if (VEC) {
        const int l = col(l0, 0);
        const bool ok = rok && l < m;
        const float4 h4 = ok ? *reinterpret_cast<const float4 *>(hr + (size_t)r * N + l)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 l4 = ok ? *reinterpret_cast<const float4 *>(lr + (size_t)r * N + l)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        hh[r][0] = h4.x, hh[r][1] = h4.y, hh[r][2] = h4.z, hh[r][3] = h4.w;
        ll[r][0] = l4.x, ll[r][1] = l4.y, ll[r][2] = l4.z, ll[r][3] = l4.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = col(l0, u);
          const bool ok = rok && l < m;
          hh[r][u] = ok ? hr[(size_t)r * N + l] : 0.f;
          ll[r][u] = ok ? lr[(size_t)r * N + l] : 0.f;
        }
      }
    }
  };
  auto sum = [&](const float (&hh)[RS_ROWS][4], const float (&ll)[RS_ROWS][4], int l0) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int l = col(l0, u);
      if (l < m) {
#pragma unroll
        for (int q = 0; q < NR; ++q) {
          const float2 x = X[(size_t)q * N + l];
#pragma unroll
          for (int r = 0; r < RS_ROWS; ++r) {
            const float p = hh[r][u] * x.x;
            const float e = fmaf(hh[r][u], x.y, fmaf(ll[r][u], x.x, fmaf(hh[r][u], x.x, -p)));
            const dfl s = df_two_sum(acc[r][q].hi, p);
            acc[r][q] = {s.hi, acc[r][q].lo + (s.lo + e)};
          }
        }
      }
    }
  };
  float h[2][RS_ROWS][4], lo[2][RS_ROWS][4];
  load(h[0], lo[0], 0);
  for (int l0 = 0; l0 < m; l0 += 256) {
    load(h[1], lo[1], l0 + 128);
    sum(h[0], lo[0], l0);
    load(h[0], lo[0], l0 + 256);
    sum(h[1], lo[1], l0 + 128);
  }
  float mx = 0.f;
#pragma unroll
  for (int r = 0; r < RS_ROWS; ++r)
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      dfl a = acc[r][q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, a.hi, o);
        const float ol = __shfl_xor_sync(0xffffffffu, a.lo, o);
        const dfl s = df_two_sum(a.hi, oh);
        a = df_fast(s.hi, s.lo + (a.lo + ol));
      }
      const int k = k0 + r;
      if (lane == 0 && k < m) {
        const float2 bb = c.w.eeq_B[(size_t)b * 2 * N + (size_t)q * N + k];
        const dfl res = df_add(dfl{bb.x, bb.y}, df_neg(a));
        c.w.eeq_V[(size_t)b * 2 * N + (size_t)q * N + k] = res.hi;
        mx = fmaxf(mx, fabsf(res.hi));
      }
    }
  if (lane == 0) atomicMax(&c.w.eeq_res[b * EEQ_BIG_REFINE + it], __float_as_uint(mx));
}

// Charges (forward) or the adjoint charges (adjoint) from the solutions;
// FP64 sums.  Grid (FIN_CTAS, structures): every CTA forms the structure's
// sums itself (same order, same values), CTA 0 records them, and each CTA
// writes its share of the atoms (real atoms by their compact index,
// padding slots zeroed -- disjoint sets, so the CTAs never write the same
// entry).
constexpr int FIN_CTAS = 16;
__global__ void __launch_bounds__(1024) eeq_big_finish_kernel(Ctx c, int adjoint) {
  __shared__ double s_a[32], s_b[32];
  __shared__ double s_par;
  const int b = blockIdx.y;
  const bool lead = blockIdx.x == 0;
  const int N = c.N;
  const int m = c.w.n_real[b];
  const float2 *X = c.w.eeq_X + (size_t)b * 2 * N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  double sa = 0.0, sb = 0.0;
  for (int k = tid; k < m; k += blockDim.x) {
    sa += (double)X[k].x + (double)X[k].y;
    if (!adjoint) sb += (double)X[N + k].x + (double)X[N + k].y;
  }
  sa = warp_sum(sa);
  sb = warp_sum(sb);
  if (lane == 0) {
    s_a[warp] = sa;
    s_b[warp] = sb;
  }
  __syncthreads();
  if (tid == 0) {
    // final refinement residual: that of the first iteration below the
    // tolerance (later iterations were skipped), else of the last one
    float fin = 0.f;
    for (int it = 0; it < EEQ_BIG_REFINE; ++it) {
      fin = __uint_as_float(c.w.eeq_res[b * EEQ_BIG_REFINE + it]);
      if (fin < BIG_TOL) break;
    }
    if (lead) c.w.eeq_final[2 * b + (adjoint ? 1 : 0)] = fin;
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      ta += s_a[w];
      tb += s_b[w];
    }
    if (adjoint) {
      s_par = m > 0 ? ta / c.w.eeq_sum[2 * b] : 0.0;
    } else {
      const double lam = m > 0 ? (ta - c.charge[b]) / tb : 0.0;
      if (lead) {
        c.w.eeq_sum[2 * b] = tb;
        c.w.eeq_sum[2 * b + 1] = lam;
      }
      s_par = lam;
    }
  }
  __syncthreads();
  const double par = s_par;
  const int g0 = blockIdx.x * blockDim.x + tid, gs = gridDim.x * blockDim.x;
  for (int i = g0; i < N; i += gs) {
    if (c.w.cidx[(size_t)b * N + i] >= 0) continue;  // a real atom: written below
    if (adjoint) {
      c.w.eeq_w[(size_t)b * N + i] = 0.0;
      c.w.dEdcnq[(size_t)b * N + i] = 0.0;
    } else {
      c.w.q[(size_t)b * N + i] = 0.0;
      c.w.eeq_y[(size_t)b * N + i] = 0.0;
    }
  }
  for (int k = g0; k < m; k += gs) {
    const size_t a = (size_t)b * N + c.w.ridx[(size_t)b * N + k];
    const double x0 = (double)X[k].x + (double)X[k].y;
    if (adjoint) {
      const double w = x0 - par * c.w.eeq_y[a];
      c.w.eeq_w[a] = w;
      const double cq = c.w.cnq[a];
      const int z = c.w.z[a];
      const double dq = cq > 0.0 ? w * c.tab.eeq_kcn[z] * 0.5 / sqrt(cq) * c.w.dcnq[a] : 0.0;
      c.w.dEdcnq[a] = dq;
      c.w.adj32[a].y = (float)dq;
      c.w.adj32[a].w = (float)w;
    } else {
      const double x1 = (double)X[N + k].x + (double)X[N + k].y;
      c.w.q[a] = x0 - par * x1;
      c.w.eeq_y[a] = x1;
    }
  }
}

// ---------------------------------------------------------------- launch

// The library's second stream per device (see SideStream): the multi-CTA
// factorisation's look-ahead runs on it.
static std::mutex g_side_mutex;
static SideStream g_side[64];

std::mutex &side_stream_mutex() { return g_side_mutex; }

SideStream *side_stream_for_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(g_side_mutex);
  SideStream &ss = g_side[dev & 63];
  if (!ss.tried) {
    ss.tried = true;
    int lo = 0, hi = 0;
    bool ok = cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess &&
              cudaStreamCreateWithPriority(&ss.s, cudaStreamNonBlocking, hi) == cudaSuccess;
    cudaEvent_t *evs[5] = {&ss.fork, &ss.panel, &ss.bulk[0], &ss.bulk[1], &ss.done};
    for (cudaEvent_t *e : evs)
      ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
    ss.ok = ok;
    if (!ok) cudaGetLastError();  // clear the failed call's error
  }
  return ss.ok ? &ss : nullptr;
}

// Look-ahead of the factorisation.  The chain diagonal block -> panel ->
// update of the next panel's columns is the critical path; it runs on a
// high-priority stream of the library (one per device) while the caller's
// stream carries the bulk of each trailing update, so that panel p + 1 is
// factored while the columns right of it still receive panel p's update.
// Events order the two streams:
//   critical  diag(p), panel(p), record PANEL, wait BULK(p - 1),
//             syrk(p, first column)            [columns of panel p + 1]
//   caller    wait PANEL, syrk(p, rest), record BULK(p)   [columns >= p + 2]
// BULK(p - 1) covers panel p + 1's columns, so the critical stream waits for
// it before adding panel p's update to them (both read-modify-write those
// tiles); diag(p + 1) and panel(p + 1) touch no column that syrk(p, rest)
// writes.  The two events of BULK alternate with the parity of p.  Calls
// that enqueue this schedule are serialised by a mutex (the events are
// shared); the caller's stream waits for the critical stream at the end,
// so the schedule also holds inside a stream capture.
static void launch_factor(const Ctx &c, cudaStream_t st) {
  const int B = c.B, N = c.N;
  const int npan = (N + BNB - 1) / BNB;
  ensure_smem(eeq_big_diag_kernel, (int)eeq_big_diag_smem());
  ensure_smem(eeq_big_panel_kernel, (int)eeq_big_panel_smem());
  ensure_smem(eeq_big_syrk_kernel, (int)eeq_big_syrk_smem());
  SideStream *la = npan > 2 ? side_stream_for_device() : nullptr;
  if (!la) {
    for (int p = 0; p < npan; ++p) {
      const int k0 = p * BNB;
      eeq_big_diag_kernel<<<B, 512, eeq_big_diag_smem(), st>>>(c, k0);
      const int rest = N - k0 - BNB;
      if (rest <= 0) break;
      eeq_big_panel_kernel<<<dim3((rest + 63) / 64, B), 256, eeq_big_panel_smem(), st>>>(c, k0,
                                                                                       p & 1);
      const int T = (rest + BNB - 1) / BNB;
      eeq_big_syrk_kernel<<<dim3(T * (T + 1) / 2, B), BNB, eeq_big_syrk_smem(), st>>>(
          c, k0, SYRK_ALL, p & 1);
    }
    return;
  }
  std::lock_guard<std::mutex> lock(side_stream_mutex());
  cudaStream_t cs = la->s;
  cudaEventRecord(la->fork, st);
  cudaStreamWaitEvent(cs, la->fork, 0);
  bool bulk_prev = false;  // whether BULK(p - 1) was recorded
  for (int p = 0; p < npan; ++p) {
    const int k0 = p * BNB;
    eeq_big_diag_kernel<<<B, 512, eeq_big_diag_smem(), cs>>>(c, k0);
    const int rest = N - k0 - BNB;
    if (rest <= 0) break;
    eeq_big_panel_kernel<<<dim3((rest + 63) / 64, B), 256, eeq_big_panel_smem(), cs>>>(c, k0,
                                                                                     p & 1);
    const int T = (rest + BNB - 1) / BNB;
    bool bulk_now = false;
    if (T > 1) {
      cudaEventRecord(la->panel, cs);
      cudaStreamWaitEvent(st, la->panel, 0);
      eeq_big_syrk_kernel<<<dim3((T - 1) * T / 2, B), BNB, eeq_big_syrk_smem(), st>>>(
          c, k0, SYRK_REST, p & 1);
      cudaEventRecord(la->bulk[p & 1], st);
      bulk_now = true;
    }
    if (bulk_prev) cudaStreamWaitEvent(cs, la->bulk[(p - 1) & 1], 0);
    eeq_big_syrk_kernel<<<dim3(T, B), BNB, eeq_big_syrk_smem(), cs>>>(c, k0, SYRK_FIRST_COLUMN,
                                                                      p & 1);
    bulk_prev = bulk_now;
  }
  cudaEventRecord(la->done, cs);
  cudaStreamWaitEvent(st, la->done, 0);
}

// Whether every structure's refinement residual of iteration ``it`` is below
// the tolerance, read on the host (one small copy and a wait for the
// stream).  A failed copy or wait answers no, and the device-side skips
// decide as before.
static bool converged_on_host(const Ctx &c, cudaStream_t st, int it) {
  std::vector<unsigned> res((size_t)c.B * EEQ_BIG_REFINE);
  if (cudaMemcpyAsync(res.data(), c.w.eeq_res, 4 * res.size(), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return false;
  for (int b = 0; b < c.B; ++b) {
    float r;
    std::memcpy(&r, &res[(size_t)b * EEQ_BIG_REFINE + it], 4);
    if (!(r < BIG_TOL)) return false;
  }
  return true;
}

// Forward (adjoint = 0: factorisation, two right-hand sides, charges) or
// adjoint (reuses the factor; one right-hand side dE/dq) multi-CTA EEQ.
// Refinement iterations after the second are launched only while some
// structure still needs them: for large structures (eight 512-blocks or
// more, where an iteration is ~130 launches) the host reads the residuals
// after the second and each later iteration, unless the stream is being
// captured into a graph or the call sets D4_FLAG_NO_HOST_WAIT; otherwise
// every iteration is launched and the converged structures skip it on the
// device.
void launch_eeq_big(const Ctx &c, cudaStream_t st, bool adjoint) {
  const int B = c.B, N = c.N;
  if (!adjoint) launch_factor(c, st);  // F: the lower part of hi, from the build kernel
  const int nsb = eeq_nsb(N);
  if (!adjoint) {  // inverses of the 128- and 512-blocks, kept for the adjoint solve
    ensure_smem(eeq_big_pinv_kernel, (int)eeq_big_pinv_smem());
    eeq_big_pinv_kernel<<<dim3((N + BNB - 1) / BNB, B), 512, eeq_big_pinv_smem(), st>>>(c);
    eeq_blkinv_init_kernel<<<dim3(nsb, B), 256, 0, st>>>(c);
    ensure_smem(eeq_blkinv_step_kernel, (int)eeq_blkinv_smem());
    for (int r = 1; r < SBP; ++r)
      eeq_blkinv_step_kernel<<<dim3(nsb * r, B), 256, eeq_blkinv_smem(), st>>>(c, r);
    eeq_blkinv_mirror_kernel<<<dim3(MIR_TILES, nsb, B), 256, 0, st>>>(c);
  }
  const int nr = adjoint ? 1 : 2;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusActive;
  const bool host_check =
      nsb >= 8 && cap == cudaStreamCaptureStatusNone && !(c.flags & D4_FLAG_NO_HOST_WAIT);
  eeq_big_rhs_kernel<<<dim3((N + 255) / 256, B), 256, 0, st>>>(c, adjoint ? 1 : 0);
  for (int it = 0; it < EEQ_BIG_REFINE; ++it) {
    if (host_check && it >= 2 && converged_on_host(c, st, it - 1)) break;
    // V = L^-T L^-1 V: forward sweep into Y, backward sweep into V
    for (int sb = 0; sb < nsb; ++sb) {
      eeq_sweep_diag_kernel<<<dim3(EEQ_SB / 8, B), 256, 0, st>>>(c, sb, it, 0, nr, 0);
      const int rest = N - (sb + 1) * EEQ_SB;
      if (rest > 0)
        eeq_sweep_below_kernel<<<dim3((rest + 8 * BL_ROWS - 1) / (8 * BL_ROWS), B), 256, 0, st>>>(
            c, sb, it, nr);
    }
    for (int sb = nsb - 1; sb >= 0; --sb) {
      eeq_sweep_diag_kernel<<<dim3(EEQ_SB / 8, B), 256, 0, st>>>(c, sb, it, 1, nr, 1);
      const int s0 = sb * EEQ_SB;
      if (s0 > 0)
        eeq_sweep_above_kernel<<<dim3((s0 + AB_COLS - 1) / AB_COLS, B), 256, 0, st>>>(c, sb, it,
                                                                                     nr);
    }
    eeq_big_update_kernel<<<dim3((N + 255) / 256, B), 256, 0, st>>>(c, it, nr);
    const dim3 rg((N + 8 * RS_ROWS - 1) / (8 * RS_ROWS), B);
    if (N % 4 == 0) {
      if (nr == 2) eeq_big_residual_kernel<2, true><<<rg, 256, 0, st>>>(c, it);
      else eeq_big_residual_kernel<1, true><<<rg, 256, 0, st>>>(c, it);
    } else {
      if (nr == 2) eeq_big_residual_kernel<2, false><<<rg, 256, 0, st>>>(c, it);
      else eeq_big_residual_kernel<1, false><<<rg, 256, 0, st>>>(c, it);
    }
  }
  eeq_big_finish_kernel<<<dim3(FIN_CTAS, B), 1024, 0, st>>>(c, adjoint ? 1 : 0);
}

}  // namespace d4
