// Shared device-side definitions for the DFT-D4 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tad_dftd4_gb300.h"

namespace d4 {

constexpr int NREF = D4_NREF;
constexpr int NFREQ = D4_NFREQ;
constexpr int MAX_ELEM_ID = 128;  // element ids are < 128 in every table
constexpr int ERF_TAB = 1537;     // erf table nodes k / 256, k <= 1536 (x0 <= 6)
constexpr float ERF_SCALE = 256.f;
constexpr double THOPI = 3.0 / 3.141592653589793238462643383279502884197;  // utils.py:50
constexpr double SQRT_2_OVER_PI = 0.79788456080286535587989211986876;
constexpr double INV_SQRT_PI = 0.56418958354775628694807945156077;

// Workspace carved out of one caller-provided buffer.  The same function
// computes the layout for d4_workspace_size and d4_dispersion.
// ---------------------------------------------------------------- EEQ sizes

// Shared memory of the one-CTA EEQ kernels of the precision form (floats):
// vectors (compact index, double-float solution and right-hand sides, FP32
// residual), the transposed panel PT[32][ldp] and the packed factor.
__host__ __device__ inline int eeq_round4(int n) { return (n + 3) & ~3; }
__host__ __device__ inline size_t eeq_mixed_vec_floats(int N) {  // multiple of 4 (16 bytes)
  return ((size_t)eeq_round4(N) + 10 * (size_t)N + 3) & ~(size_t)3;
}
// Leading dimension of the transposed panel PT[32][ldp] of chol_blocked:
// rows of at most N - 32 entries, rounded up to 8 (the 8-wide tiles read up
// to there) plus 4 (16-byte rows, spread banks).
__host__ __device__ inline int chol_panel_ld(int N) {
  const int n = N > 40 ? N - 32 : 8;
  return ((n + 7) & ~7) + 4;
}
__host__ __device__ inline size_t eeq_small_bytes(int N) {
  return 4 * (eeq_mixed_vec_floats(N) + (size_t)32 * chol_panel_ld(N) +
              (size_t)N * (N + 1) / 2);
}
// Structures padded to N are solved by one CTA each when everything fits in
// shared memory (N <= 290), else by the multi-CTA path.
__host__ __device__ inline bool eeq_small_fits(int N) { return eeq_small_bytes(N) <= 220 * 1024; }
constexpr int EEQ_BIG_REFINE = 4;  // refinement iterations of the multi-CTA path at most
constexpr int EEQ_SB = 512;        // diagonal blocks inverted for the multi-CTA solves
__host__ __device__ inline int eeq_nsb(int N) { return (N + EEQ_SB - 1) / EEQ_SB; }
constexpr int EEQ_BNB = 128;       // panel width of the multi-CTA factorisation
__host__ __device__ inline int eeq_nblk(int N) { return (N + EEQ_BNB - 1) / EEQ_BNB; }
// Row stride (floats) of the multi-CTA factor: 16-byte rows for bulk copies.
__host__ __device__ inline int eeq_ldf(int N) { return (N + 3) & ~3; }
// Bytes of one row block's split panel operands: 8 chunks of 16 columns,
// hi and lo planes of 128 rows x 16 TF32 values in the MMA's K-major layout.
constexpr size_t EEQ_OPND_BLOCK = (size_t)8 * 2 * 8192;

// ---------------------------------------------------------------- ATM sizes

// The precision-form ATM accumulates a structure's pair adjoints in shared
// memory (upper triangle + atoms, FP32) when the padded size allows it
// (N <= 234); larger structures accumulate in global memory and get
// neighbour lists for the neighbour-triple variant.
__host__ __device__ inline size_t atm_smem_bytes(int N) {
  return (size_t)4 * ((size_t)N * (N - 1) + N);
}
__host__ __device__ inline bool atm_smem_fits(int N) { return atm_smem_bytes(N) <= 220 * 1024; }
// Batches up to this many structures get a size-ordered launch order.
constexpr int SORDER_MAX = 16384;

// Largest neighbour count of a centre atom in the neighbour-triple ATM.
constexpr int ATM_SPARSE_DMAX = 2048;
// Structures up to this size get their ATM centres in spatial (Z-) order
// (one shared-memory sort per structure); larger ones keep index order.
constexpr int ATM_ORDER_MAX = 16384;


struct Workspace {
  int *status;      // [1]
  float *eeq_final; // [B][2] final EEQ refinement residual (forward, adjoint); fixed offset
  int *n_eff;       // [B]   highest real atom index + 1
  int *n_slots;     // [B]   distinct-element slots (D4S), 1 for D4
  int *z;           // [B*N] validated atomic numbers (0: padding or invalid)
  int *slot;        // [B*N] slot of each atom's element in its structure
  int *slot_elem;   // [B*MAX_ELEM_ID] element of each slot
  double *cn;       // [B*N] D4 coordination number
  double *cnq;      // [B*N] capped EEQ coordination number
  double *dcnq;     // [B*N] d(capped)/d(raw)
  double *q;        // [B*N] atomic charges
  double *eeq_y;    // [B*N] A^-1 1
  double *eeq_w;    // [B*N] adjoint charges
  double *eeq_sum;  // [B*2] (sum y, lambda)
  double *dEdcn;    // [B*N]
  double *dEdq;     // [B*N]
  double *dEdcnq;   // [B*N] dE/d(raw EEQ CN)
  double *e3;       // [B*N] ATM energy (accumulated atomically)
  double *pgrad;    // [B*D4_PARAM_GRAD_STRIDE] parameter gradients (atomics)
  double *A;        // [B*N*S*23] weighted polarisabilities at q
  double *A0;       // [B*N*S*23] at q = 0
  double *dA_dcn;   // [B*N*S*23]
  double *dA_dq;    // [B*N*S*23]
  double *dA0_dcn;  // [B*N*S*23]
  double *G;        // [B*N*S*23] dE/dA
  double *G0;       // [B*N*S*23] dE/dA0
  double *pr_r;     // [B*N*N] distance
  double *pr_ir;    // [B*N*N] 1/distance
  double *pr_L;     // [B*N*N] log(R0/r) of the ATM damping
  double *pr_c;     // [B*N*N] sqrt(C6 at q = 0)
  double *pr_S;     // [B*N*N] dE_ATM/d(r^2) (atomics)
  double *pr_P;     // [B*N*N] sum of weighted triple energies (atomics)
  double *pr_da1;   // [B*N*N] d log R0 / d a1 (parameter gradients only)
  double *pr_da2;   // [B*N*N] d log R0 / d a2 (parameter gradients only)
  // exact C9 (D4_FLAG_EXACT_C9, FP64 method only)
  double *ax;       // [B*N*23] polarisabilities a_i(iw) of the exact C9
  double *gax;      // [B*N*23] dE/da_i(iw)
  double *gbar;     // [B*S*23] D4S: slot sums of dE/da over the structure's atoms / nat
  double *f3x;      // [B*N*3] ATM part of dE/dR
  double *eeq_L;    // [B*N*(N+1)/2] packed Cholesky factor (FP64 method) or
                    // packed FP64 EEQ matrix (precision form)
  float4 *pos32;    // [B*N] positions relative to the structure's first slot, FP32,
                    // with sqrt(r4r2) in .w (both methods)
  float4 *aux32;    // [B*N] (cov_d3, en, eeq_rad, 0) in FP32 (both methods)
  int *cidx;        // [B*N] index among the real atoms of the structure, -1 padding
  float *w32;       // [B*N] energy weights of the differentiated sum (1 by default)
  float *fw32;      // [23] (3/pi) times the Casimir-Polder weights, FP32
  // precision form only
  float4 *adj32;    // [B*N] (dE/dCN, dE/dCN_EEQ, q, EEQ adjoint w) in FP32
  float *prS32;     // [B*N*N] ATM dE/d(r^2), FP32 accumulation
  float *prP32;     // [B*N*N] ATM weighted triple energies, FP32 accumulation
  float *eeq_hi;    // [B*N*N] dense EEQ matrix of the real atoms (compact order) as the
  float *eeq_lo;    //         double-float hi + lo
  int *ridx;        // [B*N] atom index of the k-th real atom
  int *n_real;      // [B] real atoms
  float4 *pos32lo;  // [B*N] low parts of the positions: pos32 + pos32lo = r - r_first
  float4 *erf_tab;  // [ERF_TAB] (erf(x0) hi, lo, 2/sqrt(pi) exp(-x0^2) hi, lo), x0 = k/256
  float2 *igam;     // [MAX_ELEM_ID^2] 1/sqrt(rad_a^2 + rad_b^2) as double-float
  float2 *eeq_diag; // [MAX_ELEM_ID] eta + sqrt(2/pi)/rad as double-float
  float *A32;       // [B*S*23*N] (transposed: atoms contiguous per frequency)
  float *A032;      // [B*S*23*N]
  float *dA32;      // [B*N*S*23*3] (dA/dCN, dA/dq, dA0/dCN) per atom, slot, frequency
  float *alpha32;   // [MAX_ELEM_ID*7*23] reference polarisabilities (double-float hi
  float *alpha32lo; //                     and lo parts)
  float *z0lo;      // [MAX_ELEM_ID*7] low part of zeta at q = 0 (hi in ref32.w)
  float2 *sfw;      // [32] sqrt((3/pi) w) of the Casimir-Polder weights, double-float
  float4 *pairA;    // [MAX_ELEM_ID^2] (R0, qq) per element pair, double-floats (hi, lo, hi, lo)
  float4 *pairB;    // [MAX_ELEM_ID^2] (R0^6, R0^8) per element pair, double-floats
  float4 *cnpair;   // [MAX_ELEM_ID^2] (1 / (rcov_a + rcov_b), k4 exp(-(|en_a - en_b| + k5)^2
                    //  / k6)) per element pair, double-floats (hi, lo, hi, lo)
  float4 *ref32;    // [MAX_ELEM_ID*7] (refcovcn, refq + zeff, Gaussians, zeta at q = 0)
  float2 *el32;     // [MAX_ELEM_ID] (zeff, gam * gc)
  float *G32;       // [B*N*S*23] dE/dA
  float *G032;      // [B*N*S*23] dE/dA0
  float4 *ptf;      // [B*N*N] (r^2, 1/r^2, (R0/r)^(alp/3), sqrt(C6(q=0)) / r^3)
  float4 *ptf_da;   // [B*N*N] (d log R0/d a1, d log R0/d a2, log(R0/r), 0)
  float *eeq_L32;   // [B*N*(N+1)/2] packed FP32 Cholesky factor (one-CTA path)
  float *eeq_F;     // [B][N][eeq_ldf(N)] dense FP32 factor, block inverses on the diagonal
  unsigned char *eeq_P;  // [2][B][eeq_nblk(N)] split panel operands (EEQ_OPND_BLOCK each)
  float *eeq_V;     // [B*2*N] FP32 residual / correction (multi-CTA)
  float2 *eeq_X;    // [B*2*N] double-float solution (multi-CTA)
  float2 *eeq_B;    // [B*2*N] double-float right-hand sides (multi-CTA)
  unsigned *eeq_res;  // [B*EEQ_BIG_REFINE] max |residual| per iteration (float bits)
  float *eeq_Y;     // [B*2*N] FP32 intermediate of the triangular sweeps (multi-CTA)
  float *eeq_Xd;    // [B*nsb*512*512] inverses of the 512-diagonal blocks of the factor
  int *nbr;         // [B*N*N] ATM neighbour lists: row j = atoms within disp3 of j, ascending
  int *nbr_deg;     // [B*N] neighbours per atom
  unsigned long long *atm_cnt;  // [B*2] (sum_j deg_j (deg_j - 1) / 2, max_j deg_j)
  int *atm_order;   // [B*N] atoms in Z-order of their positions (centre order of the
                    // neighbour-triple ATM)
  int *sorder;      // [B] structures by decreasing n_eff (launch order of the
                    // per-structure kernels of the precision form)
  unsigned *atm_rowmax;  // [B*N] largest r^2 over the real pairs of each atom (FP32
                         // bits; zeroed by the CN kernel, raised by the pair kernels of
                         // the precision form)
  size_t bytes;
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Raise a kernel's dynamic shared-memory limit once per device and size:
// cudaFuncSetAttribute costs microseconds of host time, which every call of
// the library would otherwise pay again (d4_api.cu).
void ensure_smem_impl(const void *func, size_t bytes);
template <typename F>
inline void ensure_smem(F *func, size_t bytes) {
  ensure_smem_impl(reinterpret_cast<const void *>(func), bytes);
}

// Layout of the workspace; ``base == nullptr`` only measures it.
inline Workspace carve_workspace(void *base, int B, int N, int S, uint32_t flags) {
  Workspace w{};
  size_t off = 0;
  char *p = static_cast<char *>(base);
  auto take = [&](size_t bytes) -> void * {
    off = align_up(off, 256);
    void *r = p ? p + off : nullptr;
    off += bytes;
    return r;
  };
  const size_t BN = (size_t)B * N;
  const size_t BNS23 = BN * S * NFREQ;
  const size_t BNN = BN * N;
  const bool grad = (flags & D4_FLAG_GRADIENT) != 0;
  const bool mixed = (flags & D4_FLAG_MIXED) != 0;
  w.status = (int *)take(sizeof(int) * 4);
  w.eeq_final = (float *)take(sizeof(float) * 2 * (size_t)B);  // at byte 256 for every B
  w.n_eff = (int *)take(sizeof(int) * B);
  w.n_slots = (int *)take(sizeof(int) * B);
  w.z = (int *)take(sizeof(int) * BN);
  w.slot = (int *)take(sizeof(int) * BN);
  w.slot_elem = (int *)take(sizeof(int) * B * MAX_ELEM_ID);
  w.cn = (double *)take(8 * BN);
  w.cnq = (double *)take(8 * BN);
  w.dcnq = (double *)take(8 * BN);
  w.q = (double *)take(8 * BN);
  w.eeq_y = (double *)take(8 * BN);
  w.eeq_w = (double *)take(8 * BN);
  w.eeq_sum = (double *)take(8 * 2 * B);
  w.dEdcn = (double *)take(8 * BN);
  w.dEdq = (double *)take(8 * BN);
  w.dEdcnq = (double *)take(8 * BN);
  w.e3 = (double *)take(8 * BN);
  w.pgrad = (double *)take(8 * (size_t)D4_PARAM_GRAD_STRIDE * B);
  w.A = mixed ? nullptr : (double *)take(8 * BNS23);
  w.A0 = mixed ? nullptr : (double *)take(8 * BNS23);
  w.dA_dcn = (grad && !mixed) ? (double *)take(8 * BNS23) : nullptr;
  w.dA_dq = (grad && !mixed) ? (double *)take(8 * BNS23) : nullptr;
  w.dA0_dcn = (grad && !mixed) ? (double *)take(8 * BNS23) : nullptr;
  w.G = (grad && !mixed) ? (double *)take(8 * BNS23) : nullptr;
  w.G0 = (grad && !mixed) ? (double *)take(8 * BNS23) : nullptr;
  w.pr_r = mixed ? nullptr : (double *)take(8 * BNN);
  w.pr_ir = mixed ? nullptr : (double *)take(8 * BNN);
  w.pr_L = mixed ? nullptr : (double *)take(8 * BNN);
  w.pr_c = mixed ? nullptr : (double *)take(8 * BNN);
  w.pr_S = (grad && !mixed) ? (double *)take(8 * BNN) : nullptr;
  w.pr_P = (grad && !mixed) ? (double *)take(8 * BNN) : nullptr;
  const bool pgrad = (flags & D4_FLAG_PARAM_GRAD) != 0;
  w.pr_da1 = (pgrad && !mixed) ? (double *)take(8 * BNN) : nullptr;
  w.pr_da2 = (pgrad && !mixed) ? (double *)take(8 * BNN) : nullptr;
  const bool exact = (flags & D4_FLAG_EXACT_C9) != 0 && !mixed;
  w.ax = exact ? (double *)take(8 * BN * NFREQ) : nullptr;
  w.gax = (exact && grad) ? (double *)take(8 * BN * NFREQ) : nullptr;
  w.gbar = (exact && grad) ? (double *)take(8 * (size_t)B * S * NFREQ) : nullptr;
  w.f3x = (exact && grad) ? (double *)take(8 * BN * 3) : nullptr;
  w.eeq_L = mixed ? nullptr : (double *)take(8 * (size_t)B * ((size_t)N * (N + 1) / 2));
  w.pos32 = (float4 *)take(16 * BN);
  w.aux32 = (float4 *)take(16 * BN);
  w.cidx = (int *)take(sizeof(int) * BN);
  w.w32 = (float *)take(sizeof(float) * BN);
  w.fw32 = (float *)take(sizeof(float) * 32);
  if (mixed) {
    w.adj32 = (float4 *)take(16 * BN);
    w.sorder = (int *)take(sizeof(int) * (size_t)B);
    w.atm_rowmax = (unsigned *)take(sizeof(unsigned) * BN);
    w.prS32 = grad ? (float *)take(4 * BNN) : nullptr;
    w.prP32 = grad ? (float *)take(4 * BNN) : nullptr;
    w.eeq_hi = (float *)take(4 * BNN);
    w.eeq_lo = (float *)take(4 * BNN);
    w.ridx = (int *)take(sizeof(int) * BN);
    w.n_real = (int *)take(sizeof(int) * B);
    w.pos32lo = (float4 *)take(16 * BN);
    w.erf_tab = (float4 *)take(16 * (size_t)ERF_TAB);
    w.igam = (float2 *)take(8 * (size_t)MAX_ELEM_ID * MAX_ELEM_ID);
    w.eeq_diag = (float2 *)take(8 * (size_t)MAX_ELEM_ID);
    w.A32 = (float *)take(4 * BNS23);
    w.A032 = (float *)take(4 * BNS23);
    w.dA32 = grad ? (float *)take(4 * 3 * BNS23) : nullptr;
    w.alpha32 = (float *)take(4 * (size_t)MAX_ELEM_ID * NREF * NFREQ);
    w.alpha32lo = (float *)take(4 * (size_t)MAX_ELEM_ID * NREF * NFREQ);
    w.z0lo = (float *)take(4 * (size_t)MAX_ELEM_ID * NREF);
    w.sfw = (float2 *)take(8 * 32);
    w.pairA = (float4 *)take(16 * (size_t)MAX_ELEM_ID * MAX_ELEM_ID);
    w.pairB = (float4 *)take(16 * (size_t)MAX_ELEM_ID * MAX_ELEM_ID);
    w.cnpair = (float4 *)take(16 * (size_t)MAX_ELEM_ID * MAX_ELEM_ID);
    w.ref32 = (float4 *)take(16 * (size_t)MAX_ELEM_ID * NREF);
    w.el32 = (float2 *)take(8 * (size_t)MAX_ELEM_ID);
    w.G32 = grad ? (float *)take(4 * BNS23) : nullptr;
    w.G032 = grad ? (float *)take(4 * BNS23) : nullptr;
    w.ptf = (float4 *)take(16 * BNN);
    w.ptf_da = pgrad ? (float4 *)take(16 * BNN) : nullptr;
    if (eeq_small_fits(N)) {
      w.eeq_L32 = (float *)take(4 * (size_t)B * ((size_t)N * (N + 1) / 2));
    } else {
      w.eeq_F = (float *)take(4 * BN * eeq_ldf(N));
      w.eeq_P = (unsigned char *)take(2 * (size_t)B * eeq_nblk(N) * EEQ_OPND_BLOCK);
      w.eeq_V = (float *)take(4 * 2 * BN);
      w.eeq_X = (float2 *)take(8 * 2 * BN);
      w.eeq_B = (float2 *)take(8 * 2 * BN);
      w.eeq_res = (unsigned *)take(4 * (size_t)B * EEQ_BIG_REFINE);
      w.eeq_Y = (float *)take(4 * 2 * BN);
      w.eeq_Xd = (float *)take(4 * (size_t)B * eeq_nsb(N) * EEQ_SB * EEQ_SB);
    }
    if (!atm_smem_fits(N)) {
      w.nbr = (int *)take(sizeof(int) * BNN);
      w.nbr_deg = (int *)take(sizeof(int) * BN);
      w.atm_cnt = (unsigned long long *)take(8 * 2 * (size_t)B);
      w.atm_order = (int *)take(sizeof(int) * BN);
    }
  }
  w.bytes = align_up(off, 256);
  return w;
}

// FP32 copies of the parameters, converted once on the host so that no
// kernel thread spends FP64-pipe cycles on setup.
struct ParamsF {
  float s6, s8, s10, a1, a2, s9, alp3;
  float cut2, cut3, cut_cn, cut_q, kcn, k4, k5, k6, cn_max;
  float wf, ga;  // model weighting factor and charge-scaling height
};

// Everything a kernel needs, passed by value.
struct Ctx {
  ParamsF pf;
  d4_tables_t tab;
  d4_model_cfg_t cfg;
  d4_params_t par;
  const int64_t *numbers;
  const double *positions;
  const double *charge;
  const double *charges_in;
  const double *r4r2_in;
  const double *weights;
  const double *rvdw_in;  // [B*N*N] pairwise radii of the zero / modified-zero damping
  int B, N, S;
  uint32_t flags;
  int atm_tiled;  // the register-tiled ATM runs (set by the precision form's launcher)
  Workspace w;
  d4_outputs_t out;
};


// ---------------------------------------------------------------- helpers

constexpr int ATM_KMAX = 8;  // CTAs per structure at most (ATM kernels of the precision form)

// CTAs of the register-tiled ATM for a structure of n atoms in a batch of B:
// 1.2M triples per CTA for batches of 512 structures and more (measured on
// batch512 at 512 threads: 600000 -> 12 % slower, 900000 -> 3 %, 1800000 ->
// 13 %: fewer CTAs per structure mean fewer masked edge steps per task and
// fewer flushes, until the largest structures' CTAs set the makespan), fewer
// for smaller batches so that they still fill the GPU.
__host__ __device__ inline int atm_tiled_ctas(int n, int B) {
  const long long per = B >= 512 ? 1200000 : (B <= 64 ? 75000 : 1200000LL * B / 512);
  const long long work = (long long)n * n * n / 6;
  const int K = (int)((work + per - 1) / per);
  return K < 1 ? 1 : (K > ATM_KMAX ? ATM_KMAX : K);
}

__device__ __forceinline__ double atom_r4r2(const Ctx &c, size_t a, int64_t z) {
  return c.r4r2_in ? c.r4r2_in[a] : c.tab.r4r2[z];
}

__device__ __forceinline__ double atom_weight(const Ctx &c, size_t a) {
  return c.weights ? c.weights[a] : 1.0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void set_status(int *status, int code) {
  atomicCAS(status, 0, code);
}

// Error-function counting function of the CN, 1/2 (1 + erf(-x)) with
// x = k (r/r0 - 1), evaluated as 1/2 erfc(x): the same function without the
// cancellation of 1 + erf(-x) for x >> 1, where the far pairs of a nearly
// isolated atom make up its whole (tiny) coordination number.
__device__ __forceinline__ double erf_count(double r, double r0, double k) {
  return 0.5 * erfc(k * (r / r0 - 1.0));
}

// Its derivative with respect to r.
__device__ __forceinline__ double erf_count_dr(double r, double r0, double k) {
  const double x = k * (r / r0 - 1.0);
  return -k / r0 * INV_SQRT_PI * exp(-x * x);
}

// EN weighting of the D4 CN: k4 exp(-(|en_i - en_j| + k5)^2 / k6).
__device__ __forceinline__ double en_factor(double eni, double enj, double k4, double k5,
                                            double k6) {
  const double t = fabs(eni - enj) + k5;
  return k4 * exp(-(t * t) / k6);
}

// Charge-scaling function zeta (model/base.py:308-335) and d zeta / d qmod.
__device__ __forceinline__ void zeta_and_deriv(double gam, double qref, double qmod,
                                               double ga, double eps, double *z,
                                               double *dz) {
  if (qmod > 0.0) {
    const double den = qmod - eps;
    const double scale = exp(gam * (1.0 - qref / den));
    const double zz = exp(ga * (1.0 - scale));
    *z = zz;
    *dz = -ga * zz * scale * gam * qref / (den * den);
  } else {
    *z = exp(ga);
    *dz = 0.0;
  }
}

__host__ __device__ inline size_t tri_index(int i, int j) {  // packed lower, j <= i
  return (size_t)i * (i + 1) / 2 + j;
}

// r_i - r_j from the FP32 positions relative to the structure's first atom
// (pos32) and their low parts (pos32lo): the high parts of nearby atoms
// subtract exactly, the low parts restore what rounding the absolute
// positions to FP32 lost (about 4e-6 Bohr at 60 Bohr from the origin).
__device__ __forceinline__ float3 pos_diff(const float4 &pi, const float4 &li, const float4 &pj,
                                          const float4 &lj) {
  return make_float3((pi.x - pj.x) + (li.x - lj.x), (pi.y - pj.y) + (li.y - lj.y),
                     (pi.z - pj.z) + (li.z - lj.z));
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Warp sums of up to 32 per-lane values, scattered: lane L receives the
// sum over the warp of in[L] (0 for L >= NV).  Five halving exchanges
// (16 + 8 + 4 + 2 + 1 shuffles) instead of NV full butterflies (5 NV).
template <int NV>
__device__ __forceinline__ float warp_reduce_scatter32(const float (&in)[NV]) {
  const int lane = threadIdx.x & 31;
  float v[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) v[q] = q < NV ? in[q] : 0.f;
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int q = 0; q < h; ++q) {
      const float keep = up ? v[q + h] : v[q];
      const float send = up ? v[q] : v[q + h];
      v[q] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
  return v[0];
}

// Compensated FP32 accumulator (Knuth two-sum): value = hi + lo.
struct Acc32 {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float t = hi + x;
    const float bp = t - hi;
    lo += (hi - (t - bp)) + (x - bp);
    hi = t;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Compensated warp reduction of Acc32 partial sums: every shuffle step adds
// the high parts with a two-sum and carries the rounding error into the low
// parts (FP32 only).  All lanes receive the total.
__device__ __forceinline__ Acc32 warp_sum_acc(Acc32 a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, a.hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, a.lo, o);
    const float t = a.hi + h2;
    const float bp = t - a.hi;
    const float err = (a.hi - (t - bp)) + (h2 - bp);
    a.hi = t;
    a.lo = a.lo + l2 + err;
  }
  return a;
}

// Real atoms of structure b compacted into s_idx[0..m).  Returns m.

// ---------------------------------------------------------------- double-float

// A double-float value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi) / 2: about 48 significant bits on the FP32 pipe.  Built
// from the error-free transformations TwoSum (Knuth), FastTwoSum (Dekker,
// |a| >= |b|) and the FMA product error fma(a, b, -a b).
struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dfl df_fast(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const dfl s = df_two_sum(a.hi, b.hi);
  return df_fast(s.hi, s.lo + (a.lo + b.lo));
}

__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast(p, e);
}

__device__ __forceinline__ dfl df_sq(dfl a) {
  const float p = a.hi * a.hi;
  const float e = fmaf(2.f * a.hi, a.lo, fmaf(a.hi, a.hi, -p));
  return df_fast(p, e);
}

__device__ __forceinline__ dfl df_from(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// 1/sqrt(a), a > 0 and normal: the FP32 estimate y and one Newton step
// y (1 + (1 - a y^2) / 2) whose residual 1 - a y^2 is formed in double-float
// (y^2 is exact as yy + yye; 1 - t.hi is exact since t.hi is within 2^-21
// of 1).  The relative error goes from ~2^-22 to ~2^-43.
__device__ __forceinline__ dfl df_rsqrt(dfl a) {
  const float y = rsqrtf(a.hi);
  const float yy = y * y;
  const dfl t = df_mul(a, dfl{yy, fmaf(y, y, -yy)});
  const float e = (1.0f - t.hi) - t.lo;
  return df_fast(y, 0.5f * y * e);
}

// erf(x) for x >= 0 in double-float, by Taylor expansion around the nearest
// node x0 = k / 256 (|h| = |x - x0| <= 1/512):
//   erf(x0 + h) = erf(x0) + D [h - x0 h^2 + (2 x0^2 - 1)/3 h^3
//                 - x0 (2 x0^2 - 3)/6 h^4 + (4 x0^4 - 12 x0^2 + 3)/30 h^5 + ...]
// with D = 2/sqrt(pi) exp(-x0^2) (the n-th derivative of erf is D times a
// Hermite polynomial).  erf(x0) and D come from the table as double-floats,
// D h is formed in double-float, the h^2 tail (|tail| < 2e-6) in FP32; the
// omitted h^6 term is below 1e-15.  Absolute error about 5e-13; erf = 1 from
// x = 6 on (erfc(6) = 2e-17).
__device__ __forceinline__ dfl df_erf(dfl x, const float4 *tab) {
  if (x.hi >= 6.0f) return {1.0f, 0.0f};
  // clamped: a NaN argument (coincident atoms) must not index outside the table
  const int k = min(max(__float2int_rn(x.hi * ERF_SCALE), 0), ERF_TAB - 1);
  const float x0 = (float)k * (1.0f / ERF_SCALE);
  const float hh = x.hi - x0;  // exact (Sterbenz)
  const float4 t = tab[k];
  const float p = t.z * hh;
  const float e = fmaf(t.z, x.lo, fmaf(t.w, hh, fmaf(t.z, hh, -p)));
  const float h = hh + x.lo;
  const float x02 = x0 * x0;
  const float c3 = (2.f * x02 - 1.f) * (1.f / 3.f);
  const float c4 = -x0 * (2.f * x02 - 3.f) * (1.f / 6.f);
  const float c5 = (4.f * x02 * x02 - 12.f * x02 + 3.f) * (1.f / 30.f);
  const float tail = t.z * h * h * fmaf(h, fmaf(h, fmaf(h, c5, c4), c3), -x0);
  const dfl s = df_two_sum(t.x, p);
  return df_fast(s.hi, s.lo + (t.y + e + tail));
}

__device__ inline int compact_real_atoms(const Ctx &c, int b, int n, int *s_idx, int *s_tmp) {
  // serial prefix by warp 0 is enough for n <= a few thousand
  if (threadIdx.x < 32) {
    int base = 0;
    for (int i0 = 0; i0 < n; i0 += 32) {
      const int i = i0 + threadIdx.x;
      const bool real = i < n && c.w.z[(size_t)b * c.N + i] != 0;
      const unsigned mask = __ballot_sync(0xffffffffu, real);
      if (real) s_idx[base + __popc(mask & ((1u << threadIdx.x) - 1u))] = i;
      base += __popc(mask);
    }
    if (threadIdx.x == 0) *s_tmp = base;
  }
  __syncthreads();
  return *s_tmp;
}

}  // namespace d4
