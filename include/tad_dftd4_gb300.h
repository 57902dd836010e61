/*
 * tad_dftd4_gb300.h -- C ABI of the GB300 DFT-D4 dispersion library.
 *
 * The library evaluates the DFT-D4 dispersion energy (atom-resolved) and its
 * gradient for a zero-padded batch of structures, on one CUDA device.  It is
 * the compiled replacement for tad-dftd4's ``dftd4()`` path
 * (``src/tad_dftd4/disp.py:44-146``): coordination number, EEQ charges,
 * Gaussian reference weights with charge scaling, C6 by Casimir-Polder
 * integration, the rational (BJ) two-body term and the ATM three-body term.
 *
 * Conventions (the same as the reference):
 *  - ``numbers`` holds atomic numbers, 0 marks a padding slot;
 *  - positions are in Bohr, energies in Hartree, gradients in Eh/Bohr;
 *  - arrays are C-contiguous, batch-major: numbers[b * n_pad + i].
 *
 * Memory: nothing is allocated by the library.  Every device buffer
 * (element tables, workspace, outputs) is owned by the caller; the workspace
 * size comes from ``d4_workspace_size``.  All pointers named ``d_*`` or
 * documented as "device" are device pointers.  ``stream`` is a
 * ``cudaStream_t`` passed as ``void*``; work is enqueued on it and every
 * call returns without synchronising, with one exception: for structures
 * padded beyond 3584 atoms the precision form's EEQ solves wait once each
 * for ``stream`` (after their second refinement iteration, to launch a
 * third only if a residual asks for it), unless the stream is being
 * captured or the call sets D4_FLAG_NO_HOST_WAIT.  Calls on different
 * streams with different workspaces are independent.
 *
 * Errors: every entry point returns a ``d4_status`` code.  Input problems
 * that can only be seen on the device (atomic number outside the tables,
 * a non-positive EEQ pivot, non-finite input) are reported through the
 * ``status`` word of the workspace; read it with ``d4_read_status`` after
 * the stream has been synchronised.  The status word is the first int32 of
 * the workspace (byte offset D4_STATUS_OFFSET), so a caller that cannot
 * synchronise (a captured CUDA graph) may copy it asynchronously instead; it
 * is cleared at the start of every call.
 */
#ifndef TAD_DFTD4_GB300_H
#define TAD_DFTD4_GB300_H

#define D4_STATUS_OFFSET 0 /* byte offset of the device status word in a workspace */

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define D4_ABI_VERSION 2
#define D4_NREF 7   /* reference systems per element (reference/d4/params.py) */
#define D4_NFREQ 23 /* imaginary frequencies of the Casimir-Polder grid (utils.py:52-80) */

typedef enum d4_status {
  D4_OK = 0,
  D4_ERR_ARGUMENT = 1,         /* null pointer, bad size or flag */
  D4_ERR_WORKSPACE = 2,        /* workspace smaller than d4_workspace_size() */
  D4_ERR_CUDA = 3,             /* a CUDA launch failed; see d4_last_cuda_error() */
  D4_ERR_ELEMENT = 4,          /* atomic number outside the element tables */
  D4_ERR_EEQ_SINGULAR = 5,     /* EEQ matrix not positive definite */
  D4_ERR_NONFINITE = 6,        /* non-finite position or charge */
  D4_ERR_TOO_MANY_ELEMENTS = 7, /* D4S: more distinct elements than slots */
  D4_ERR_DEVICE_TIMEOUT = 8     /* an on-device wait for the tensor cores ran out */
} d4_status;

/* Model variants (tad_dftd4.model): D4Model and D4SModel. */
typedef enum d4_model_kind { D4_MODEL_D4 = 0, D4_MODEL_D4S = 1 } d4_model_kind;

/* Flags for d4_dispersion. */
#define D4_FLAG_GRADIENT 1u    /* also compute dE/dR (d_gradient must be set) */
#define D4_FLAG_CHARGES_IN 2u  /* use batch->d_charges_in instead of the EEQ solve */
#define D4_FLAG_MIXED 4u       /* precision form: FP32 pair/triple maths, FP64 sums */
#define D4_FLAG_PARAM_GRAD 8u  /* also compute the parameter gradient (d_param_grad) */
#define D4_FLAG_EXACT_C9 16u   /* ATM with exact C9 = (3/pi) sum_w w a_i a_j a_k
                                  (D4ATMExact, dispersion/threebody.py:276-302,
                                  dispersion/d4.py:67-84) instead of
                                  sqrt(C6 C6 C6); plain FP64 method only */
#define D4_FLAG_NO_HOST_WAIT 32u /* never wait for the stream inside the call:
                                    the multi-CTA EEQ launches all its
                                    refinement iterations and converged
                                    structures skip them on the device (no
                                    reference counterpart) */

/* Test hook of the timeout handling: the tensor-core pair kernel of the
   precision form treats the first wait for its MMAs as timed out and takes
   its error path (status D4_ERR_DEVICE_TIMEOUT, a bounded wait for the MMAs
   in flight, tensor memory released, early return).  Results of such a call
   are incomplete; the next call is unaffected. */
#define D4_FLAG_TEST_TIMEOUT 0x80000000u

/* Entries per structure of d_param_grad: dE_b / d(s6, s8, s10, a1, a2, s9,
   alp, rs6, rs8, bet), then two unused entries. */
#define D4_PARAM_GRAD_STRIDE 12

/* Two-body damping functions (damping/functions.py).  RATIONAL is the
   Becke-Johnson damping dftd4() uses; the others are the D3-family damping
   functions a caller can pass as ``damping_function`` (plain FP64 method). */
typedef enum d4_damping_kind {
  D4_DAMP_RATIONAL = 0, /* 1 / (r^n + (a1 sqrt(3 r4r2_i r4r2_j) + a2)^n), 262-305 */
  D4_DAMP_ZERO = 1,     /* f / r^n, f = 1 / (1 + 6 (rs_n r / rvdw)^alp_n), 308-378 */
  D4_DAMP_MZERO = 2,    /* f / r^n, f = 1 / (1 + 6 (r / (rs_n rvdw) + bet rvdw)^-alp_n), 381-434 */
  D4_DAMP_OP = 3        /* r^bet / (r^n (r^bet + R0^bet)), 437-484 */
} d4_damping_kind;

/*
 * Element tables, device pointers.  Row 0 is the dummy element.  The first
 * group has ``n_ref_elem`` rows (104 in tad-dftd4), the second ``n_elem``
 * rows (119).  ``alpha`` is produced by d4_prepare_alpha().
 */
typedef struct d4_tables {
  int32_t n_ref_elem;
  int32_t n_elem;
  const double *alpha;        /* [n_ref_elem][7][23] reference polarisabilities */
  const double *refcovcn;     /* [n_ref_elem][7] reference coordination numbers */
  const int64_t *refc;        /* [n_ref_elem][7] Gaussians per reference (0, 1, 3) */
  const double *refq;         /* [n_ref_elem][7] reference charges for the weights */
  const double *gam;          /* [n_elem] chemical hardness (before the gc factor) */
  const int64_t *zeff;        /* [n_elem] effective nuclear charge */
  const double *r4r2;         /* [n_elem] sqrt(0.5 * <r4>/<r2> * sqrt(Z)) */
  const double *cov_d3;       /* [n_elem] D3 covalent radii (Bohr) */
  const double *en;           /* [n_elem] Pauling electronegativities */
  const double *eeq_chi;      /* [n_elem] EEQ electronegativity */
  const double *eeq_eta;      /* [n_elem] EEQ chemical hardness */
  const double *eeq_kcn;      /* [n_elem] EEQ CN scaling */
  const double *eeq_rad;      /* [n_elem] EEQ charge width (Bohr) */
  const double *wfpair;       /* [n_elem][n_elem] D4S weighting factors */
  const double *freq_weights; /* [23] Casimir-Polder quadrature weights */
} d4_tables_t;

/* Charge-scaling and weighting constants of a model (model/base.py:57-59). */
typedef struct d4_model_cfg {
  int32_t kind; /* d4_model_kind */
  double ga;    /* 3.0 */
  double gc;    /* 2.0 */
  double wf;    /* 6.0 (D4; D4S takes wfpair) */
} d4_model_cfg_t;

/* Damping parameters and cutoffs (damping/parameters/base.py:48-85, cutoff.py). */
typedef struct d4_params {
  double s6, s8, s10, a1, a2, s9, alp;
  int32_t has_s8;  /* 0: no dipole-quadrupole term (reference gating, functions.py:144) */
  int32_t has_s10; /* 1: add the s10 term (twobody.py:184-197) */
  double cut_disp2;  /* two-body cutoff, inclusive (60) */
  double cut_disp3;  /* three-body cutoff on r_ij and r_jk (40) */
  double cut_cn;     /* D4 CN cutoff (30) */
  double cut_cn_eeq; /* EEQ CN cutoff (25) */
  double cn_eeq_max; /* smooth EEQ CN cap (8) */
  double kcn, k4, k5, k6; /* CN counting constants (defaults.py:41-50) */
  /* two-body damping (added in ABI version 2; zero-initialised = rational) */
  int32_t damping;   /* d4_damping_kind */
  int32_t reserved;
  double rs6, rs8;   /* zero / modified-zero damping radius scalings */
  double bet;        /* modified-zero / optimised-power damping exponent */
} d4_params_t;

/* A zero-padded batch (device pointers). */
typedef struct d4_batch {
  int32_t n_struct; /* B */
  int32_t n_pad;    /* N, padded atoms per structure */
  const int64_t *d_numbers;  /* [B][N] */
  const double *d_positions; /* [B][N][3] */
  const double *d_charge;    /* [B] total charges */
  const double *d_charges_in; /* [B][N] atomic charges, read with D4_FLAG_CHARGES_IN */
  const double *d_r4r2_in;    /* [B][N] per-atom r4r2 values, or NULL for the table */
  const double *d_energy_weights; /* [B][N] weights w of the differentiated quantity
                                     sum_i w_i E_i, or NULL for all ones */
  const double *d_rvdw_in; /* [B][N][N] pairwise van der Waals radii, required by the
                              zero and modified-zero damping (ABI version 2) */
} d4_batch_t;

/* Outputs (device pointers; optional ones may be NULL). */
typedef struct d4_outputs {
  double *d_energy;   /* [B][N] atom-resolved energy (required) */
  double *d_gradient; /* [B][N][3] dE/dR, written with D4_FLAG_GRADIENT */
  double *d_charges;  /* [B][N] EEQ charges (optional) */
  double *d_cn;       /* [B][N] D4 coordination numbers (optional) */
  double *d_param_grad; /* [B][D4_PARAM_GRAD_STRIDE], D4_FLAG_PARAM_GRAD */
  double *d_cn_eeq;   /* [B][N] capped EEQ coordination numbers (optional) */
} d4_outputs_t;

/* Library ABI version (D4_ABI_VERSION). */
int d4_abi_version(void);

/* Human-readable text for a status code (static storage). */
const char *d4_status_string(int status);

/* Text of the last CUDA error seen by this thread ("" if none). */
const char *d4_last_cuda_error(void);

/*
 * Reference polarisabilities alpha_{e,r}(i w) for every element, written to
 * ``d_alpha_out`` [n_ref_elem][7][23].  Follows model/base.py:367-418: the
 * secondary-system polarisability scaled by the charge-scaling function of
 * its reference charge ``d_refh`` is subtracted from the free reference
 * value, clipped at zero.  Replaces the per-call ``_get_alpha`` of
 * BaseModel (called from model/base.py:151 and model/d4.py:306).
 */
int d4_prepare_alpha(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                     const double *d_refalpha,  /* [n_ref_elem][7][23] */
                     const double *d_refascale, /* [n_ref_elem][7] */
                     const double *d_refscount, /* [n_ref_elem][7] */
                     const int64_t *d_refsys,   /* [n_ref_elem][7] */
                     const double *d_secscale,  /* [n_sec] */
                     const double *d_secalpha,  /* [n_sec][23] */
                     int32_t n_sec,
                     const double *d_refh,      /* [n_ref_elem][7] */
                     double *d_alpha_out, void *stream);

/*
 * Bytes of workspace needed by d4_dispersion for B structures of N padded
 * atoms.  ``n_slots`` is 1 for D4 and the largest number of distinct
 * elements in one structure for D4S.
 */
size_t d4_workspace_size(int32_t n_struct, int32_t n_pad, int32_t n_slots, uint32_t flags);

/*
 * Atom-resolved DFT-D4 energy (and gradient) of a padded batch.  Replaces
 * ``tad_dftd4.dftd4`` (disp.py:44-146) / ``Disp.calculate``
 * (dispersion/base.py:285-431) with the terms registered by ``dftd4``:
 * ``TwoBodyTerm`` with rational damping at the EEQ charges
 * (dispersion/twobody.py:60-201) and ``D4ATMApprox`` at q = 0
 * (dispersion/threebody.py:54-163, 210-256, 311-321).  The gradient is the
 * derivative of the total energy, through CN, charges, weights, C6, damping
 * and ATM, as autograd gives in the reference.
 */
int d4_dispersion(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                  const d4_batch_t *batch, const d4_params_t *params,
                  uint32_t flags, int32_t n_slots, void *d_workspace,
                  size_t workspace_bytes, const d4_outputs_t *out, void *stream);

/* Outputs of d4_properties (device pointers; any may be NULL). */
typedef struct d4_properties {
  double *d_cn;      /* [B][N] D4 coordination numbers */
  double *d_charges; /* [B][N] EEQ charges */
  double *d_c6;      /* [B][N][N] atom-resolved C6 at the charges, padding rows/columns 0 */
  double *d_alpha;   /* [B][N] static polarisabilities */
} d4_properties_t;

/*
 * Properties of the D4 model for a padded batch, plain FP64 method: the D4
 * coordination numbers, the EEQ charges, the atom-resolved C6 coefficients
 * at those charges and the static polarisabilities.  Replaces
 * ``tad_dftd4.get_properties`` (disp.py:149-197: cn_d4, get_eeq_charges,
 * D4Model.weight_references / get_atomic_c6 (model/d4.py:103-289) /
 * get_polarizabilities (model/base.py:286-302)).  ``cfg->kind`` must be
 * D4_MODEL_D4; the workspace is d4_workspace_size(B, N, 1, 0) bytes.
 */
int d4_properties(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                  const d4_batch_t *batch, const d4_params_t *params, void *d_workspace,
                  size_t workspace_bytes, const d4_properties_t *out, void *stream);

/*
 * Copy the device status word of a workspace to the host (synchronous on
 * ``stream``) and clear it.  Returns a d4_status.
 */
int d4_read_status(void *d_workspace, void *stream);

/*
 * Final residuals max |A x - b| of the EEQ refinement of the last
 * d4_dispersion call that used this workspace, per structure: h_out[2 b]
 * for the charges (forward), h_out[2 b + 1] for the adjoint solve of a
 * gradient call.  Precision form only: its FP32 factorisation is refined in
 * double-float until the residual is below 1e-10 (or the iteration limit);
 * the entries stay 0 where no refinement ran (plain FP64 method, given
 * charges, energy-only calls for the adjoint).  ``n_struct`` is the batch
 * size of that call.  Synchronous on ``stream``.  (No reference counterpart:
 * the reference solves the EEQ system directly in its working precision.)
 */
int d4_eeq_residuals(void *d_workspace, int32_t n_struct, float *h_out, void *stream);

/*
 * Queue a copy of the device status word of a workspace into ``h_status``
 * (host memory that stays valid until the copy has run; page-locked for the
 * copy to be asynchronous) behind the work already on ``stream``, without
 * waiting.  Returns D4_OK or D4_ERR_CUDA.  (No reference counterpart: the
 * host layer uses it to read an autograd forward's status later.)
 */
int d4_status_async(void *d_workspace, int32_t *h_status, void *stream);

/*
 * Kernel timing.  Between d4_timing_begin and d4_timing_end, every
 * d4_dispersion call on this host thread records a pair of CUDA events
 * around each of its kernels, on the stream it launches them on (at most
 * ``max_calls`` calls are recorded).  d4_timing_end waits for the last event
 * and writes the summed milliseconds of each stage to ``ms_per_stage``
 * (``n_stage`` entries, see d4_stage_name) and the number of recorded calls
 * to ``n_calls``.
 */
int d4_timing_begin(int32_t max_calls);
int d4_timing_end(float *ms_per_stage, int32_t n_stage, int32_t *n_calls);
int32_t d4_stage_count(void);
const char *d4_stage_name(int32_t stage);

/*
 * Arithmetic-throughput probe: ``n_blocks`` CTAs of 256 threads run
 * ``iters`` dependent-chain FMA iterations on 8 independent accumulators in
 * FP64 (``fp64`` != 0) or FP32 and write one value per thread to
 * ``d_sink`` (n_blocks * 256 doubles).  The elapsed time of the launch (CUDA
 * events) goes to ``ms_out``; the flop count is
 * n_blocks * 256 * iters * 8 * 2.  Used to measure the FP32 / FP64 peak
 * that bounds the pair and triple kernels.
 */
int d4_probe_fma(int32_t fp64, int32_t n_blocks, int32_t iters, double *d_sink,
                 float *ms_out, void *stream);

/*
 * Self-test of the bounded waits every tensor-core kernel uses: one CTA
 * initialises an mbarrier that nothing arrives on and waits for it with the
 * library's wait loop, limited to ``limit_ns`` nanoseconds of the GPU's
 * global timer; the outcome (D4_ERR_DEVICE_TIMEOUT when the limit ran out,
 * as it must) goes to ``*d_result`` (device int).  No counterpart in the
 * reference.
 */
int d4_selftest_wait(int32_t *d_result, uint64_t limit_ns, void *stream);

/*
 * Allocation-free variant of d4_dispersion.  This entry point has no
 * counterpart in the reference (tad-dftd4 allocates tensors on every call).
 *
 * It is meant for callers that cannot call cudaMalloc: code running where
 * device allocation is forbidden or unsafe, such as inside a host callback
 * or a real-time loop with a fixed memory budget, a plugin that must not
 * touch its host application's allocator, or a process whose memory pool is
 * managed by someone else.  Instead of a caller-provided workspace it uses
 * one file-scope device array of D4_NOALLOC_SCRATCH_BYTES (32 MiB) that is
 * part of the library image: every GPU that loads the library holds it until
 * the process exits.  The caller still provides all inputs and outputs.
 *
 * Limits and rules:
 *  - the problem must fit: d4_workspace_size(B, N, n_slots, flags) must not
 *    exceed D4_NOALLOC_SCRATCH_BYTES (with gradients that is, e.g., 12
 *    structures of 200 atoms or one structure of about 700 atoms); larger
 *    problems are rejected with D4_ERR_WORKSPACE before any work is queued;
 *  - all calls share the one array, and it keeps the last call's contents
 *    (everything a call needs zeroed it clears itself): calls whose work
 *    overlaps on the GPU -- different streams without ordering, or
 *    different host threads on one device -- race and corrupt each other;
 *  - the first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture starts;
 *  - with ``check_status`` != 0 the call waits for ``stream`` and returns the
 *    device status (as d4_read_status would); otherwise it returns without
 *    waiting and device-side input errors are not reported.
 * No cudaMalloc, cudaFree or allocating library routine is called.
 */
#define D4_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int d4_dispersion_noalloc(const d4_tables_t *tables, const d4_model_cfg_t *cfg,
                          const d4_batch_t *batch, const d4_params_t *params,
                          uint32_t flags, int32_t n_slots, const d4_outputs_t *out,
                          int32_t check_status, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TAD_DFTD4_GB300_H */
