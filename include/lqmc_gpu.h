/*
 * lqmc_gpu.h -- C ABI of liblqmc_gpu.so, the GB300 (sm_103a) engine for the DQMC sweep
 * hot path of KieDani/LatticeQMC (package `lqmc`).
 *
 * The reference is pure Python; its "interface" for this path is the LatticeQMC solver
 * (lqmc/lqmc.py).  Each entry point below replaces one piece of it; the Python facade in
 * latticeqmc_gb300/ binds these symbols with ctypes and keeps the reference's API
 * (HubbardModel / Configuration / LatticeQMC / measure / measure_betas).
 *
 * Conventions
 *   - Every function returns 0 (LQMC_OK) or a negative LQMC_ERR_* code; no exception or
 *     abort crosses the ABI.  lqmc_last_error() gives a message for the last failure.
 *   - Plain pointers and sizes only.  Matrices are float64, row-major (C order), n x n.
 *     The Hubbard-Stratonovich field crosses the ABI in the reference's (n_sites,
 *     time_steps) int8 layout (lqmc/configuration.py:89) and is held on the device as
 *     [slice][site] so that one time slice is contiguous.
 *   - Host buffers in, host buffers out: the handle owns every device buffer it uses
 *     (allocated in lqmc_set_chains, freed in lqmc_destroy).
 *   - lqmc_sweep is asynchronous on the given stream (NULL = the default stream);
 *     lqmc_get_* synchronise that stream.
 *   - A handle is not thread-safe: use one host thread per handle.
 *   - Algorithm mode, precision and RNG are fixed at lqmc_create.
 */
#ifndef LQMC_GPU_H
#define LQMC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LQMC_ABI_VERSION 1

/* return codes */
#define LQMC_OK 0
#define LQMC_ERR_INVALID -1      /* bad argument (size, index, null pointer, ...)      */
#define LQMC_ERR_CUDA -2         /* a CUDA runtime call failed                          */
#define LQMC_ERR_STATE -3        /* call out of order (e.g. sweep before set_chains)   */
#define LQMC_ERR_UNSUPPORTED -4  /* combination not built (e.g. compat + mixed)         */
#define LQMC_ERR_NUMERIC -5      /* a chain reported non-finite G or a zero pivot       */
#define LQMC_ERR_NOMEM -6        /* device allocation failed                            */

/* algorithm modes */
#define LQMC_MODE_COMPAT 0   /* replays lqmc.py:301-347 arithmetic, defects included     */
#define LQMC_MODE_DQMC 1     /* textbook DQMC, QR/UDV stabilised                          */
#define LQMC_MODE_DET 2      /* the reference's determinant mode (lqmc.py:236-299): every
                                ratio from det M of the flipped configuration, unstabilised
                                products; float64, shared-memory kernel, a slow check path */

/* precisions */
#define LQMC_PREC_FP64 0     /* every floating-point operation in float64                */
#define LQMC_PREC_MIXED 1    /* float32 G, wraps and delayed updates; FP64 stabilisation */
#define LQMC_PREC_FP64E 2    /* float64 G and updates; every dense product a float64-accurate
                                GEMM emulated on the tcgen05 BF16 tensor cores (operands as
                                56-bit fixed point in 8 balanced base-128 digits, exact FP32
                                accumulation in tensor memory); FP64 Householder panels     */

/* uniform-draw sources */
#define LQMC_RNG_REPLAY 0    /* caller uploads the uniforms (e.g. numpy's stream)        */
#define LQMC_RNG_PHILOX 1    /* Philox4x64-10 on the device, keyed by (seed, chain)      */

/* sweep orders (dqmc mode, tiled kernel) */
#define LQMC_ORDER_DOWN 0        /* every sweep l = L-1 .. 0, the reference's order; the right
                                    stack of UDT factors is rebuilt at the start of each sweep */
#define LQMC_ORDER_ALTERNATE 1   /* sweeps alternate down and up; each direction's products
                                    serve the next sweep, so the stack is built from scratch only
                                    after the field is set; the end-of-sweep G is at tau = 0
                                    (down) or tau = beta (up), both equal to G(0)             */

/* per-chain status bits (lqmc_get_status) */
#define LQMC_STATUS_NONFINITE 1   /* NaN/Inf found in G                                  */
#define LQMC_STATUS_SINGULAR 2    /* zero pivot in an LU factorisation                   */
#define LQMC_STATUS_DRIFT 4       /* stabilisation residual above the drift threshold    */
#define LQMC_STATUS_TIMEOUT 8     /* a bounded device-side wait (tensor-core pipeline) ran
                                     out; the chain's results since then are not valid     */

/* observable vector layout returned by lqmc_get_observables (per chain), float64:
 *   [0] number of measurements       [1] sum of kinetic energy   [2] sum of potential energy
 *   [3] sum of mean double occupancy [4] sum of mean density     [5..7] reserved
 *   [8 .. 8+N)        per-site density sums
 *   [8+N .. 8+2N)     per-site double-occupancy sums
 *   [8+2N .. 8+2N+N^2)        <n_i n_j> sums
 *   [8+2N+N^2 .. 8+2N+2N^2)   <S^z_i S^z_j> sums                                         */
#define LQMC_OBS_HEADER 8
#define LQMC_OBS_LEN(n) (LQMC_OBS_HEADER + 2 * (n) + 2 * (n) * (n))

/* per-chain diagnostics layout (lqmc_get_diagnostics), float64:
 *   [0] accepted flips (cumulative)  [1] attempted flips (cumulative)
 *   [2] max stabilisation residual max|G_wrapped - G_scratch| of the last launch
 *   [3] log|det G_up|  [4] log|det G_dn|  [5] sign det G_up  [6] sign det G_dn
 *   [7] sweeps done (cumulative; the philox sweep counter)
 *   [8..12] SM clock cycles of the last lqmc_sweep spent per phase (thread 0 of the chain's
 *   CTA): [8] from-scratch recompute of G, [9] site updates, [10] wraps, [11] stabilisation
 *   refreshes, [12] measurements; tiled kernel only, cycles inside those phases spent in
 *   [13] Householder QR, [14] forming Q and T of the UDT factors, [15] LU solves,
 *   [16] splitting operands of emulated float64 GEMMs, [17] their tensor-core loops
 *   (including [18]), [18] their epilogues (reading and combining the accumulators),
 *   [19] the delayed-update flushes G -= X Y^T, [20] waiting at the per-site cluster barrier.
 *   [21] alternating sweep order: 0 = no products kept (the next sweep builds them and goes
 *   down), 1 = the next sweep goes up, 2 = the next sweep goes down; reset to 0 when the field
 *   or the chain state is set.  [22..23] reserved.                                             */
#define LQMC_DIAG_LEN 24

typedef struct lqmc_params {
    int32_t mode;          /* LQMC_MODE_*                                                  */
    int32_t precision;     /* LQMC_PREC_*                                                  */
    int32_t rng;           /* LQMC_RNG_*                                                   */
    int32_t stab_every;    /* slices between from-scratch refreshes (dqmc); 0 -> 10        */
    int32_t delay;         /* delayed-update depth k of the tiled kernel; 0 -> 24 fp64e, 16
                              fp64, 32 mixed (X, Y move to global memory rather than shrink k) */
    int32_t record;        /* 1: keep per-site accept decisions of the last lqmc_sweep    */
    uint64_t seed;         /* Philox key word 0 (LQMC_RNG_PHILOX)                          */
    int32_t device;        /* CUDA device ordinal                                          */
    int32_t engine;        /* LQMC_ENGINE_*: which sweep kernel runs the chains            */
    int32_t debug;         /* LQMC_DEBUG_* bits; 0 in production                           */
    int32_t fp64e_native;  /* LQMC_FP64E_NATIVE_* bits: product categories the fp64e engine
                              keeps in native float64 (0: all on the tensor cores)            */
    int32_t measure_tau;   /* 1: measured sweeps also accumulate the unequal-time G(tau_l, 0)
                              of every slice (LQMC_MODE_DQMC only; lqmc_get_green_tau)      */
    int32_t sweep_order;   /* LQMC_ORDER_*; LQMC_ORDER_ALTERNATE runs every chain on the tiled
                              kernel (LQMC_MODE_DQMC only)                                    */
    int32_t oz_stages;     /* LQMC_PREC_FP64E: stage buffers of the emulated GEMM's copy / MMA
                              ring, 1 .. 3 (0: three where they fit, else two, else one)     */
    int32_t reserved[1];
} lqmc_params;

/* product categories of the fp64e engine (lqmc_params.fp64e_native) */
#define LQMC_FP64E_NATIVE_WRAP 1     /* the two products of every slice wrap                  */
#define LQMC_FP64E_NATIVE_STACK 2    /* B-chain products of the UDT stacks                    */
#define LQMC_FP64E_NATIVE_UDT 4      /* blocked QR updates, Q and T of the UDT factors        */
#define LQMC_FP64E_NATIVE_GREEN 8    /* U_R^T U_L, T_R T_L^T and U_L Z of the stable inverse   */
#define LQMC_FP64E_NATIVE_UPDATE 16  /* delayed rank-k updates G -= X Y^T                     */
#define LQMC_FP64E_NATIVE_LU 32      /* trailing updates of the stabilised inverse's LU
                                        factorisation (emulated, they are equilibrated along k
                                        and leave a larger stabilisation residual)             */
#define LQMC_FP64E_NATIVE_LU_RHS 64  /* the LU solve's updates of its right-hand side          */

/* debug bits (lqmc_params.debug), for testing the failure paths */
#define LQMC_DEBUG_STALL_TC_WAIT 1  /* emulated-GEMM kernel: the first tensor-core step issues
                                       no copies, so its bounded wait runs out (about a second)
                                       and the chain reports LQMC_STATUS_TIMEOUT              */

/* sweep kernels (lqmc_params.engine) */
#define LQMC_ENGINE_AUTO 0   /* shared-memory kernel for fp64 and n <= 128, else tiled        */
#define LQMC_ENGINE_SMEM 1   /* one CTA per chain, G in shared memory (fp64, n <= 128)        */
#define LQMC_ENGINE_TILED 2  /* one CTA per chain, matrices in global memory, tiled GEMMs     */

typedef struct lqmc_handle lqmc_handle;

/* Create a handle.  Replaces the solver construction LatticeQMC.__init__
 * (lqmc/lqmc.py:16-79) minus the model set-up, which stays on the host. */
int lqmc_create(const lqmc_params* params, lqmc_handle** out);

/* Define the batch of independent Markov chains (on-device replacement of the walker pool,
 * lqmc/multiprocessing.py:252-289).  Chain c has n_sites[c] sites and n_slices[c] time
 * slices; exp_k[c] = expm(-dtau K) (lqmc/lqmc.py:106), exp_k_inv[c] = its inverse used by
 * the wrap (compat: numpy inv(exp_k); dqmc: expm(+dtau K)), kinetic[c] = K
 * (lqmc/hubbard.py:91-110, used by the energy measurement), exp_consts[4c..4c+3] =
 * {exp(2 lambda), exp(-2 lambda), exp(-lambda), exp(lambda)} (lqmc/lqmc.py:105, :149-154,
 * :313-323) and u[c] the interaction.  Allocates every device buffer. */
int lqmc_set_chains(lqmc_handle* h, int32_t n_chains, const int32_t* n_sites,
                    const int32_t* n_slices, const double* const* exp_k,
                    const double* const* exp_k_inv, const double* const* kinetic,
                    const double* exp_consts, const double* u);

/* Upload / download the HS field of one chain, (n_sites, n_slices) int8 in {-1, +1}
 * (Configuration.config, lqmc/configuration.py:86-136). */
int lqmc_set_field(lqmc_handle* h, int32_t chain, const int8_t* field);
int lqmc_get_field(lqmc_handle* h, int32_t chain, int8_t* field);

/* Replay mode: the uniforms chain `chain` consumes in its next lqmc_sweep call, in sweep
 * order (per sweep: l = L-1..0, i = 0..N-1), n_sweeps * N * L doubles.  Replaces the
 * np.random.rand() draw per site (lqmc/lqmc.py:317). */
int lqmc_set_uniforms(lqmc_handle* h, int32_t chain, const double* uniforms, size_t count);

/* Replay mode, every chain at once: the concatenation over chains (in chain order) of each
 * chain's n_sweeps * N * L uniforms, count = n_sweeps * sum(N * L).  One host-to-device copy
 * for the whole batch; same meaning as lqmc_set_uniforms per chain. */
int lqmc_set_uniforms_all(lqmc_handle* h, const double* uniforms, size_t count);

/* Run n_sweeps sweeps of every chain (lqmc/lqmc.py:301-347 per sweep; warmup_loop /
 * measure_loop, :349-375).  measure != 0 accumulates G and the Wick observables after
 * every sweep.  Asynchronous on `stream` (a cudaStream_t, NULL = default stream). */
int lqmc_sweep(lqmc_handle* h, int32_t n_sweeps, int32_t measure, void* stream);

/* Green's functions after the last sweep, (2, N, N): the value _update_step returns
 * (lqmc/lqmc.py:347). */
int lqmc_get_green(lqmc_handle* h, int32_t chain, double* green);

/* G of every chain after the last sweep, concatenated in chain order ((2, N, N) each);
 * one device-to-host copy for the whole batch. */
int lqmc_get_green_all(lqmc_handle* h, double* green);

/* Accumulated sum of G over measured sweeps, (2, N, N), and the number of measurements;
 * sum / count is what measure_loop returns (lqmc/lqmc.py:356-375). */
int lqmc_get_green_sum(lqmc_handle* h, int32_t chain, double* green_sum, int64_t* count);

/* Accumulated Wick observables, LQMC_OBS_LEN(N) doubles (layout above). */
int lqmc_get_observables(lqmc_handle* h, int32_t chain, double* obs);

/* Clear the measurement accumulators of every chain. */
int lqmc_reset_measurements(lqmc_handle* h);

/* Per-site accept decisions of the last lqmc_sweep (params.record = 1), int8
 * [n_sweeps][L][N] in sweep order (step = L-1-l); the decisions the reference logs per site
 * (lqmc/lqmc.py:317, :335). */
int lqmc_get_decisions(lqmc_handle* h, int32_t chain, int8_t* decisions, size_t count);

/* Per-chain diagnostics, LQMC_DIAG_LEN doubles (layout above). */
int lqmc_get_diagnostics(lqmc_handle* h, int32_t chain, double* diag);

/* Resume a chain from a checkpoint: restore its diagnostics (LQMC_DIAG_LEN doubles as
 * lqmc_get_diagnostics returned them; [7] is the sweep counter that keys the Philox stream),
 * its sum of G ((2, N, N)) and its observable sums (LQMC_OBS_LEN(N); [0] is the measurement
 * count).  Each pointer may be NULL to keep the current values.  Together with
 * lqmc_set_field this restores everything the next sweep depends on: G is recomputed from
 * the field at the start of every sweep.  No reference counterpart (the reference's runs
 * cannot be resumed); serves the per-chain checkpoint / resume of long beta / U scans. */
int lqmc_set_chain_state(lqmc_handle* h, int32_t chain, const double* diag, const double* green_sum,
                         const double* obs);

/* Unequal-time Green's function (params.measure_tau = 1): the sum over the measured sweeps
 * of G_sigma(tau_l, 0) = B_{l-1} ... B_0 (1 + B_{L-1} ... B_0)^-1, B_l = exp(V_sigma(l))
 * exp(-dtau K), for l = 0 .. L-1 (tau_l = l dtau), of the field each measured sweep ends
 * with; float64 [2][L][N][N]; divide by the measurement count (observables[0]).
 * G(tau, 0) = <c_i(tau) c_j^+(0)>, i.e. minus the imaginary-time Green's function that
 * lqmc/tools.py:182-200 (compute_pole_gf_tau) gives at U = 0.  The end-of-sweep G that
 * lqmc_get_green_sum accumulates is the equal-time G at tau_1 (the slice boundary above
 * slice 0): per sample G(tau_1, 0) = G_sweep B_0.  Stabilised: recomputed from UDT factors
 * of B(tau, 0) and B(beta, tau) at every multiple of stab_every and propagated one slice at
 * a time in between.  No reference counterpart in the solver (it measures only the
 * equal-time G, lqmc/lqmc.py:356-375). */
int lqmc_get_green_tau(lqmc_handle* h, int32_t chain, double* green_tau_sum);

/* Restore a chain's G(tau) sum ([2][L][N][N], as lqmc_get_green_tau returned it), for
 * checkpoint / resume. */
int lqmc_set_green_tau(lqmc_handle* h, int32_t chain, const double* green_tau_sum);

/* Per-chain LQMC_STATUS_* bit masks, n_chains int32 (0 = healthy). */
int lqmc_get_status(lqmc_handle* h, int32_t* status);

/* Device kernel launches issued by the last lqmc_sweep call. */
int lqmc_get_launch_count(lqmc_handle* h, int64_t* launches);

/* Message for the last failure on this handle (or for a failed lqmc_create when h == NULL). */
const char* lqmc_last_error(const lqmc_handle* h);

/* Release the handle and every device buffer it owns. */
void lqmc_destroy(lqmc_handle* h);

/* LQMC_ABI_VERSION of the loaded library. */
int lqmc_abi_version(void);

/* ---------------------------------------------------------------------------------------
 * Allocation-free sweep of one chain.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc -- applications whose device memory belongs to their
 * own allocator or arena (a host code that hands this library a fixed set of buffers), and
 * time-stepping loops that cannot afford the device-wide synchronisation cudaMalloc and
 * cudaFree may imply.
 *
 * The caller passes every input and output as DEVICE pointers it already owns; the scratch
 * the dqmc sweep needs (the UDT stacks of the stabilised B-chain products and the chain
 * descriptor) lives in one static device array of LQMC_STATIC_SCRATCH_BYTES (4 MiB) inside
 * the library, which every GPU that loads the library keeps until the process exits.
 *
 * Limits: mode dqmc, precision fp64, 1 <= n_sites <= LQMC_STATIC_MAX_SITES (64),
 * n_slices >= 1, 1 <= stab_every, and (2 ceil(n_slices / stab_every) + 4) * slot doubles
 * plus 512 bytes must fit in the array, slot = 2 n^2 + n + 1 rounded up to a multiple of 4
 * (e.g. n = 64 allows up to 29 chunks, n = 16 up to 490).  Larger sizes are rejected with
 * LQMC_ERR_INVALID and a message in error_message.
 *
 * Every call shares the one array, which keeps the previous call's contents (the sweep
 * writes every scratch value before reading it, so nothing needs clearing): calls that
 * overlap on the GPU -- on different streams, or from different host threads -- race and
 * must be serialised by the caller.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) for that device.  Asynchronous on `stream` (NULL =
 * default stream); results are valid once the stream has been synchronised.
 * --------------------------------------------------------------------------------------- */
#define LQMC_STATIC_SCRATCH_BYTES (4u << 20)
#define LQMC_STATIC_MAX_SITES 64

typedef struct lqmc_static_chain {
    int32_t n_sites;
    int32_t n_slices;
    int32_t stab_every;
    int32_t rng;               /* LQMC_RNG_REPLAY (uniforms given) or LQMC_RNG_PHILOX       */
    uint64_t seed;             /* philox key word 0                                         */
    int32_t chain_id;          /* philox key word 1                                         */
    int32_t measure;           /* != 0: accumulate green_sum and obs after every sweep      */
    double exp_consts[4];      /* exp(2 lambda), exp(-2 lambda), exp(-lambda), exp(lambda)  */
    double u;                  /* Hubbard U                                                 */
    const double* exp_k;       /* device, n x n: expm(-dtau K)                              */
    const double* exp_k_t;     /* device, its transpose                                     */
    const double* exp_k_inv;   /* device, n x n: expm(+dtau K)                              */
    const double* exp_k_inv_t; /* device, its transpose                                     */
    const double* kinetic;     /* device, n x n: K                                          */
    int8_t* field;             /* device, [n_slices][n_sites], +-1, updated in place        */
    const double* uniforms;    /* device, replay: n_sweeps * n_sites * n_slices; else NULL  */
    double* green;             /* device out, (2, n, n): G after the last sweep             */
    double* green_sum;         /* device in/out, (2, n, n) measurement sum                  */
    double* obs;               /* device in/out, LQMC_OBS_LEN(n)                            */
    double* diag;              /* device in/out, LQMC_DIAG_LEN (zero before the first call) */
    int32_t* status;           /* device in/out, LQMC_STATUS_* bits                         */
    char* error_message;       /* optional host buffer for a message on failure             */
    size_t error_capacity;
} lqmc_static_chain;

/* Run n_sweeps dqmc sweeps of the chain described by *chain without allocating memory. */
int lqmc_sweep_static(const lqmc_static_chain* chain, int32_t n_sweeps, void* stream);

/* ---- the emulated float64 GEMM on its own --------------------------------------------------
 * No counterpart in the reference (its products are numpy's np.dot, lqmc/lqmc.py:182, :342-345):
 * one product through the emulated float64 GEMM of the fp64e sweep kernel -- eight BF16 digit
 * slices per operand on the tcgen05 tensor cores, the same single-CTA pipeline and staging as a
 * chain's CTA in the sweep -- so that it can be checked against float64 and timed on its own.
 * Host arrays, row-major: C (m x n, ldc) = op(A) op(B), A(i, p) = trans_a ? a[p lda + i] :
 * a[i lda + p], B(p, j) = trans_b ? b[j ldb + p] : b[p ldb + j]; with LQMC_GEMM_SUBTRACT,
 * C -= the product instead; row_scale / col_scale (optional, m / n values) scale the product's
 * rows / columns first.  stages: 1 .. 3 stage buffers.  cycles (optional, 3 values): SM clock
 * cycles of operand splitting, of the whole product pipeline, and of the accumulator drain
 * (one epilogue warp).  Returns LQMC_OK, LQMC_ERR_INVALID, LQMC_ERR_CUDA, LQMC_ERR_NOMEM, or
 * LQMC_ERR_NUMERIC when a bounded wait of the pipeline ran out (C is then not valid).
 * Allocates and synchronises: a check and measurement tool, not a hot-path call. */
#define LQMC_GEMM_SUBTRACT 1     /* C -= op(A) op(B)                                            */
#define LQMC_GEMM_KSCALE 2       /* equilibrate along k (the LU's trailing updates use this)    */
#define LQMC_GEMM_PRESPLIT_A 4   /* split A in a separate pass first (as the constant operands) */
#define LQMC_GEMM_PRESPLIT_B 8
int lqmc_emulated_gemm(int32_t m, int32_t n, int32_t k, const double* a, int32_t lda,
                       int32_t trans_a, const double* b, int32_t ldb, int32_t trans_b,
                       double* c, int32_t ldc, const double* row_scale, const double* col_scale,
                       int32_t flags, int32_t stages, int32_t device, double* cycles);

#ifdef __cplusplus
}
#endif
#endif /* LQMC_GPU_H */
