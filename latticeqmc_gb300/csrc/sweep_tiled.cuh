// Persistent dqmc sweep kernel for large lattices and for mixed precision: a cluster of two
// CTAs per Markov chain, one per spin, every n x n matrix in global memory (L2-resident for
// tens of chains at N = 256), dense products through the block-tiled GEMM of
// block_gemm.cuh or the emulated float64 GEMM of ozaki_tc.cuh.  The spins only meet in
// the acceptance ratio R = R_up R_dn of each site, whose two factors the CTAs exchange
// through distributed shared memory under one cluster barrier per site, and in the
// measurements.
//
// Template parameter T is the precision of G, of the wraps, of the rank-1 updates and of
// the B-chain products (float: the mixed-precision engine; double: the plain FP64 engine).
// The pre-pivoted Householder QR of the UDT chain product and the LU solve of the
// stabilised inverse are float64 in both.  Same algorithm, sweep order and uniform stream
// as the dqmc path of sweep_fp64.cu (lqmc/lqmc.py:301-347 with the defects fixed):
//   ratio R = (1 + D_up (1 - G_up,ii)) (1 + D_dn (1 - G_dn,ii)), accept if u <= R
//   G' = G - (D/R) G[:, i] (e_i - G[i, :])                 rank-1 update
//   G <- e^{+dtau K} e^{-V_l} G e^{V_l} e^{-dtau K}         wrap from slice l to l-1
//   refresh every stab_every slices from the UDT right stack and left product.
//
// This header holds the kernel template; each precision is instantiated in a translation
// unit of its own (sweep_tiled_f64.cu, sweep_tiled_f32.cu, sweep_tiled_f64e.cu) so that the
// three compile in parallel, and sweep_tiled.cu holds the host-side sizing and dispatch.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "block_fp64.cuh"
#include "block_gemm.cuh"
#include "chain_desc.h"
#include "lqmc_gpu.h"
#include "ozaki_tc.cuh"
#include "philox.cuh"

namespace lqmc {
namespace {

using namespace blk;

__host__ __device__ constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// Per-chain global work layout of the tiled kernel (bytes from desc.work): one block per
// spin (its CTA's G, GEMM temporaries, float64 QR / LU buffers, emulated-GEMM slices), then
// the UDT slots of both spins.
template <typename T>
struct TiledLayout {
    size_t nn, g, z, s, oz, oz_ea, xy, spin_block, slot, total, g_slots;
    // xy_delay > 0: the spin blocks also hold the delayed-update buffers X, Y (n x (k + 1));
    // alt: the alternating sweep order keeps a left product at every chunk boundary (n_chunks
    // slots per spin) instead of a ping-pong pair
    __host__ __device__ TiledLayout(int n, int n_chunks, bool emu = false, int xy_delay = 0,
                                    bool alt = false) {
        nn = (size_t)n * n;
        g = 0;                                              // G of the spin       (T)
        z = g + align256(nn * sizeof(T));                   // Z0, Z1 GEMM temps   (T)
        s = z + align256(2 * nn * sizeof(T));               // S0, S1 QR / LU      (double)
        oz = s + align256(2 * nn * sizeof(double));         // emulated GEMM slices (bf16)
        // the largest product of the kernel has m, n, k <= n_sites
        const size_t oz_bytes = emu ? align256(ozt::slice_elems(n, n, n) * 2) : 0;
        oz_ea = oz + oz_bytes;                              // emulated GEMM exponents (int)
        xy = oz_ea + (emu ? align256(2 * (size_t)n * sizeof(int)) : 0);
        spin_block = xy + (xy_delay > 0 ? align256(2 * (size_t)n * (xy_delay + 1) * sizeof(T)) : 0);
        g_slots = 2 * spin_block;
        slot = align256(2 * nn * sizeof(T) + (size_t)(n + 1) * sizeof(double));
        const int n_slots = alt ? (4 * n_chunks > 2 * n_chunks + 4 ? 4 * n_chunks : 2 * n_chunks + 4)
                                : 2 * n_chunks + 4;
        total = g_slots + (size_t)n_slots * slot;
    }
};

// The constant operands of the emulated GEMMs, split once per handle and shared by every
// chain with the same e^{-dtau K} and e^{+dtau K}: e^{-dtau K} as A, its transpose as A,
// e^{+dtau K} as A (row blocks of kBM), e^{-dtau K} as B and e^{+dtau K} as B (column blocks of
// kBN), then the five exponent vectors (n ints each).  Byte offsets from the region's start.
struct PresplitLayout {
    size_t a, b, e, total;
    __host__ __device__ PresplitLayout(int n) {
        a = align256((size_t)ozt::kSlices * ozt::rows_pad(n, ozt::kBM) * ozt::kpad(n) * 2);
        b = align256((size_t)ozt::kSlices * ozt::rows_pad(n, ozt::kBN) * ozt::kpad(n) * 2);
        e = 3 * a + 2 * b;
        total = e + align256(5 * (size_t)n * sizeof(int));
    }
    // operands 0..2 are A operands (a bytes each), 3..4 B operands (b bytes each)
    __host__ __device__ size_t slices(int i) const { return i < 3 ? (size_t)i * a : 3 * a + (size_t)(i - 3) * b; }
};

template <typename T>
struct TSmem {
    int spin;         // the spin this CTA owns (its cluster rank)
    T* g;             // G of that spin
    double* peer_gii; // the partner CTA's gii buffer (distributed shared memory)
    double* peer_xv;  // the partner CTA's xv[0] (its xv[1] follows)
    T* z0;
    T* z1;
    double* s0;
    double* s1;
    unsigned char* slots;
    size_t slot_bytes;
    double* xv[2];
    double* yv[2];
    double* ev;
    double* nrm;
    double* tau;
    double* dv;       // site updates: the running diagonal of X Y^T (udt: the new d)
    int* order;
    double* sv;
    T* ev_t;      // exp_v of the current slice in precision T
    T* iev_t;     // its inverse
    T* xt[2];     // rank-1 update vectors in precision T
    T* yt[2];
    T* stage;
    T* dx;        // delayed updates: X (n x (kd + 1)), G_eff = G - X Y^T
    T* dy;        // Y (n x (kd + 1))
    double* gii;  // by site parity p = i & 1: [2 p + spin] ratio factors R_sigma of both
                  // spins, [4 + p] this spin's update coefficient D / R, [6 + p] the uniform
    long long* sub;   // clock cycles (thread 0): [0] Householder QR, [1] Q and T formation,
                      // [2] LU solve, [3..5] emulated GEMMs, [6] update flushes, [7] site barrier
    ozt::Workspace oz;    // emulated float64 GEMM: slice buffers, exponents, staging, TMEM state
    double* panel;    // blocked LU panel, n x (panel_width + 1); overlays stage, dx, dy
    int* piv;         // [kPanel] panel pivots
    double* stage64;  // float64 GEMM staging of the LU (float kernel; same region as stage)
    int native;       // LQMC_FP64E_NATIVE_* categories kept in native float64 (EMU kernel)
    ozt::Presplit pre[5];   // EMU: e^{-dtau K} as A, its transpose as A, e^{+dtau K} as A,
                            // e^{-dtau K} as B, e^{+dtau K} as B (indices kPreK .. kPreKinvB)
};

enum { kPreK = 0, kPreKT = 1, kPreKinv = 2, kPreKB = 3, kPreKinvB = 4, kNumPre = 5 };

template <typename T> __device__ __forceinline__ T* slot_U(const TSmem<T>& sm, int idx, size_t nn) {
    return reinterpret_cast<T*>(sm.slots + (size_t)idx * sm.slot_bytes);
}
template <typename T> __device__ __forceinline__ T* slot_T(const TSmem<T>& sm, int idx, size_t nn) {
    return slot_U(sm, idx, nn) + nn;
}
template <typename T> __device__ __forceinline__ double* slot_d(const TSmem<T>& sm, int idx, size_t nn) {
    return reinterpret_cast<double*>(slot_U(sm, idx, nn) + 2 * nn);
}

// Product categories whose emulated GEMMs are inlined at their call sites (a mask of
// LQMC_FP64E_NATIVE_* bits): the most frequent ones (the wraps -- inside the out-of-line
// wrap_t --, the delayed-update flushes and the B-chain products); every other site calls the
// single out-of-line copy.  Calling out of line from the kernel body makes it keep more live
// values across calls (255 registers and spills with no category inlined, none with these).
#ifndef LQMC_OZ_INLINE_CATS
#define LQMC_OZ_INLINE_CATS (LQMC_FP64E_NATIVE_WRAP | LQMC_FP64E_NATIVE_UPDATE | LQMC_FP64E_NATIVE_STACK)
#endif
constexpr int kInlineCats = LQMC_OZ_INLINE_CATS;

// Dense product of the tiled kernel: the block-tiled SIMT GEMM, or with EMU the float64
// GEMM emulated on the tcgen05 BF16 tensor cores (ozaki_tc.cuh), unless the product's
// category (LQMC_FP64E_NATIVE_* bit) is kept in native float64 for this chain.
template <typename T, bool EMU, int Cat, bool TA, bool TB, typename TAIn, typename TBIn>
__device__ __forceinline__ void gemm_t(TSmem<T>& sm, T* c, int ldc, const TAIn* a, int lda,
                                       const TBIn* b, int ldb, int m, int n, int k,
                                       GemmOpt<T> o = GemmOpt<T>(), int pa = -1, int pb = -1) {
    if constexpr (EMU) {
        if (sm.native & Cat) tile_gemm<T, TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.stage64, o);
        else if constexpr ((Cat & kInlineCats) != 0)
            ozt::oz_gemm_tc_impl<TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.oz, o,
                                         pa >= 0 ? &sm.pre[pa] : nullptr, pb >= 0 ? &sm.pre[pb] : nullptr);
        else ozt::oz_gemm_tc<TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.oz, o,
                                     pa >= 0 ? &sm.pre[pa] : nullptr, pb >= 0 ? &sm.pre[pb] : nullptr);
    } else {
        tile_gemm<T, TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.stage, o);
    }
}

template <typename T> __device__ __forceinline__ const T* mat_expk(const ChainDesc& d);
template <> __device__ __forceinline__ const double* mat_expk<double>(const ChainDesc& d) { return d.expk; }
template <> __device__ __forceinline__ const float* mat_expk<float>(const ChainDesc& d) { return d.expk_f; }
template <typename T> __device__ __forceinline__ const T* mat_expkinv(const ChainDesc& d);
template <> __device__ __forceinline__ const double* mat_expkinv<double>(const ChainDesc& d) { return d.expkinv; }
template <> __device__ __forceinline__ const float* mat_expkinv<float>(const ChainDesc& d) { return d.expkinv_f; }

// exp_v of slice l, sigma (lqmc.py:149-154) in float64 and in T, and its inverse in T
template <typename T>
__device__ __forceinline__ void load_ev_t(const ChainDesc& d, TSmem<T>& sm, int l, int sigma) {
    const int8_t* f = d.field + (size_t)l * d.n;
    for (int j = threadIdx.x; j < d.n; j += kNT) {
        const bool pos = sigma * f[j] > 0;
        sm.ev[j] = pos ? d.c[2] : d.c[3];
        sm.ev_t[j] = (T)(pos ? d.c[2] : d.c[3]);
        sm.iev_t[j] = (T)(pos ? d.c[3] : d.c[2]);
    }
}

// Householder QR of one panel of a column-major matrix (element (i, j) at s[j n + i], so
// that every column is contiguous in global memory): columns jb .. jb+b-1, rows jb .. n-1,
// each reflector applied only to the later columns of the panel (the trailing columns are
// updated by the caller in compact WY form).  Same convention as blk::householder_qr:
// beta = -sign(alpha) |x|, tau = (beta - alpha) / beta, v = x / (alpha - beta) with v_0 = 1
// implicit, R's diagonal entry beta stored in place.  Returns the number of reflectors with
// tau != 0.
__device__ int householder_panel_cm(double* s, double* tau, int n, int jb, int b, double* sv) {
    const int lane = lane_id();
    int nrefl = 0;
    for (int j = jb; j < jb + b; ++j) {
        double* cj = s + (size_t)j * n;
        if (warp_id() == 0) {
            double ss = 0.0;
#pragma unroll 4
            for (int i = j + 1 + lane; i < n; i += 32) { const double v = cj[i]; ss = fma(v, v, ss); }
            ss = warp_sum(ss);
            if (lane == 0) {
                const double alpha = cj[j];
                const double xnorm = sqrt(ss);
                if (xnorm == 0.0) {
                    tau[j] = 0.0;
                } else {
                    const double beta = -copysign(hypot(alpha, xnorm), alpha);
                    tau[j] = (beta - alpha) / beta;
                    sv[kNW] = alpha - beta;
                    sv[kNW + 1] = beta;
                }
            }
        }
        __syncthreads();
        const double t = tau[j];
        if (t == 0.0) continue;
        ++nrefl;
        const double den = sv[kNW];
        for (int i = j + 1 + threadIdx.x; i < n; i += kNT) cj[i] = cj[i] / den;
        __syncthreads();
        // a warp updates kCols later columns of the panel at once (their loads in flight
        // together); per column the same operations in the same order as one at a time
        constexpr int kCols = 4;
        for (int k0 = j + 1 + warp_id() * kCols; k0 < jb + b; k0 += kNW * kCols) {
            const int nc = min(kCols, jb + b - k0);
            double acc[kCols];
#pragma unroll
            for (int c = 0; c < kCols; ++c) acc[c] = 0.0;
#pragma unroll 2
            for (int i = j + 1 + lane; i < n; i += 32) {
                const double v = cj[i];
#pragma unroll
                for (int c = 0; c < kCols; ++c)
                    if (c < nc) acc[c] = fma(v, s[(size_t)(k0 + c) * n + i], acc[c]);
            }
            double wk[kCols];
#pragma unroll
            for (int c = 0; c < kCols; ++c) {
                acc[c] = warp_sum(acc[c]);
                wk[c] = (c < nc) ? t * (s[(size_t)(k0 + c) * n + j] + acc[c]) : 0.0;
            }
            for (int i = j + lane; i < n; i += 32) {
                const double vi = (i == j) ? 1.0 : cj[i];
#pragma unroll
                for (int c = 0; c < kCols; ++c) {
                    if (c < nc) {
                        double* ck = s + (size_t)(k0 + c) * n;
                        ck[i] = fma(-vi, wk[c], ck[i]);
                    }
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) cj[j] = sv[kNW + 1];
        __syncthreads();
    }
    return nrefl;
}

// Explicit V of the panel at jb (rows jb .. n-1, b columns; unit diagonal, zeros above),
// column-major with leading dimension n - jb: v[c (n - jb) + i] = V(i, c).
__device__ void panel_v(double* v, const double* s, int n, int jb, int b) {
    const int rows = n - jb;
    for (int e = threadIdx.x; e < rows * b; e += kNT) {
        const int c = e / rows, i = e % rows;
        v[e] = (i < c) ? 0.0 : (i == c ? 1.0 : s[(size_t)(jb + c) * n + jb + i]);
    }
    __syncthreads();
}

// T factor of the compact WY form H_jb ... H_{jb+b-1} = I - V T V^T (LAPACK dlarft, forward,
// columnwise): T(i, i) = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) (V^T V)(0:i, i).  gram is V^T V
// and tf the b x b row-major T (b <= 64: one warp, lane r owns rows r and r + 32; a row only
// reads its own earlier entries).
__device__ void wy_t_factor(double* tf, const double* gram, const double* tau, int b) {
    if (warp_id() == 0) {
        const int lane = lane_id();
        for (int i = 0; i < b; ++i) {
            for (int r = lane; r < b; r += 32) {
                double v = 0.0;
                if (r < i) {
                    for (int q = r; q < i; ++q) v = fma(tf[r * b + q], gram[q * b + i], v);
                    v *= -tau[i];
                } else if (r == i) {
                    v = tau[i];
                }
                tf[r * b + i] = v;
            }
            __syncwarp();
        }
    }
    __syncthreads();
}

#ifndef LQMC_QR_BLOCK_MAX
#define LQMC_QR_BLOCK_MAX 64
#endif

// scratch doubles of udt_absorb_t for panel width bw: the panels' T factors and V, V T, V^T C
__device__ __forceinline__ size_t qr_scratch(int n, int bw) {
    return (size_t)((n - 2) / bw + 1) * bw * bw + 3 * (size_t)n * bw;
}

// panel width of the blocked QR: the widest <= LQMC_QR_BLOCK_MAX (at most 64, the limit of
// wy_t_factor) whose scratch fits in the n^2 of S1
__device__ __forceinline__ int qr_block(int n) {
    int bw = min(min(LQMC_QR_BLOCK_MAX, 64), max(1, n / 4));
    while (bw > 1 && qr_scratch(n, bw) > (size_t)n * n) --bw;
    return bw;
}

// Solve W Z = R in place (both n x n, row-major, global memory) by a blocked right-looking
// bytes of the GEMM staging region: the kernel's own GEMM (tiled T, or emulated with
// `stages` tensor-core stage buffers), and in the float kernel also the float64 tiled GEMM of
// the LU
__host__ __device__ constexpr size_t stage_region_bytes(bool fp32, bool emu, int stages) {
    size_t b = fp32 ? tile_gemm_smem<float>() : tile_gemm_smem<double>();
    if (emu && ozt::stage_bytes(stages) > b) b = ozt::stage_bytes(stages);
    if (fp32 && tile_gemm_smem<double>() > b) b = tile_gemm_smem<double>();
    return b;
}

// An emulated-GEMM CTA owns all 512 TMEM columns of its SM: its shared memory is kept above
// half of the SM's so that no second CTA can be resident there.
constexpr size_t kEmuMinSmem = 120 * 1024;

// LU with partial pivoting: each 32-column panel is factorised in shared memory (pivot =
// first maximal |entry|, as LAPACK), its row interchanges applied across W and R, and the
// trailing submatrix and R updated with tiled float64 GEMMs; then blocked back substitution.
// `panel` is shared memory of n * (panel_width(n) + 1) doubles, `stage` the GEMM staging
// buffer.  Returns log|det W|, sign(det W) and a zero-pivot flag like blk::lu_solve.
constexpr int kPanel = 32;   // widest panel

__host__ __device__ constexpr int panel_width(int n) { return n <= 256 ? 32 : (n <= 512 ? 16 : 8); }

// EMU_W / EMU_R: the factorisation's trailing updates / the right-hand side's updates on the
// emulated GEMM (else the float64 tiled GEMM)
template <bool EMU_W, bool EMU_R>
__device__ void lu_solve_blocked(TSmem<double>& sm, double* w, double* rhs, int n, double* panel,
                                 int* piv, double* sv, double* logabs, double* sgn, int* singular) {
    const int lane = lane_id();
    const int P = panel_width(n), LD = P + 1;
    double la = 0.0, sg = 1.0;
    int sing = 0;
    for (int jb = 0; jb < n; jb += P) {
        const int nb = min(P, n - jb), rows = n - jb;
        // load the panel W[jb:n, jb:jb+nb] into shared memory: panel[r * LD + c]
        for (int r = warp_id(); r < rows; r += kNW)
            for (int c = lane; c < nb; c += 32) panel[r * LD + c] = w[(size_t)(jb + r) * n + jb + c];
        __syncthreads();
        // unblocked LU with partial pivoting inside the panel
        for (int c = 0; c < nb; ++c) {
            if (warp_id() == 0) {
                double best = -1.0;
                int bi = rows;
                for (int r = c + lane; r < rows; r += 32) {
                    const double v = fabs(panel[r * LD + c]);
                    if (v > best) { best = v; bi = r; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
                if (lane == 0) piv[c] = (bi < rows) ? bi : c;
            }
            __syncthreads();
            const int p = piv[c];
            if (p != c) {
                for (int k = threadIdx.x; k < nb; k += kNT) {
                    const double t = panel[c * LD + k];
                    panel[c * LD + k] = panel[p * LD + k];
                    panel[p * LD + k] = t;
                }
                sg = -sg;
            }
            __syncthreads();
            const double pv = panel[c * LD + c];
            if (pv == 0.0) sing = 1;
            la += log(fabs(pv));
            if (pv < 0.0) sg = -sg;
            for (int r = c + 1 + threadIdx.x; r < rows; r += kNT) panel[r * LD + c] /= pv;
            __syncthreads();
            for (int r = c + 1 + warp_id(); r < rows; r += kNW) {
                const double l = panel[r * LD + c];
                for (int k = c + 1 + lane; k < nb; k += 32) panel[r * LD + k] = fma(-l, panel[c * LD + k], panel[r * LD + k]);
            }
            __syncthreads();
        }
        // store the factored panel and apply its interchanges to the other columns of W and to R
        for (int r = warp_id(); r < rows; r += kNW)
            for (int c = lane; c < nb; c += 32) w[(size_t)(jb + r) * n + jb + c] = panel[r * LD + c];
        for (int c = 0; c < nb; ++c) {
            const int p = piv[c];
            if (p == c) continue;
            double* ra = w + (size_t)(jb + c) * n;
            double* rb = w + (size_t)(jb + p) * n;
            for (int k = threadIdx.x; k < n; k += kNT) {
                if (k >= jb && k < jb + nb) continue;
                const double t = ra[k]; ra[k] = rb[k]; rb[k] = t;
            }
            double* qa = rhs + (size_t)(jb + c) * n;
            double* qb = rhs + (size_t)(jb + p) * n;
            for (int k = threadIdx.x; k < n; k += kNT) {
                const double t = qa[k]; qa[k] = qb[k]; qb[k] = t;
            }
            __syncthreads();
        }
        __syncthreads();
        // U12 = L11^-1 W[jb:jb+nb, jb+nb:n] and R1 = L11^-1 R[jb:jb+nb, :] (unit lower, by columns)
        const int rest = n - jb - nb;
        for (int k = threadIdx.x; k < rest + n; k += kNT) {
            double* col = (k < rest) ? (w + (size_t)jb * n + jb + nb + k) : (rhs + (size_t)jb * n + (k - rest));
            for (int r = 1; r < nb; ++r) {
                double v = col[(size_t)r * n];
                for (int q = 0; q < r; ++q) v = fma(-panel[r * LD + q], col[(size_t)q * n], v);
                col[(size_t)r * n] = v;
            }
        }
        __syncthreads();
        if (rest > 0) {
            GemmOpt<double> o;
            o.subtract = true;
            o.kscale = true;
            // W22 -= L21 U12 ; R2 -= L21 R1
            gemm_t<double, EMU_W, 0, false, false>(sm, w + (size_t)(jb + nb) * n + jb + nb, n,
                                                w + (size_t)(jb + nb) * n + jb, n,
                                                w + (size_t)jb * n + jb + nb, n, rest, rest, nb, o);
            gemm_t<double, EMU_R, 0, false, false>(sm, rhs + (size_t)(jb + nb) * n, n,
                                                w + (size_t)(jb + nb) * n + jb, n,
                                                rhs + (size_t)jb * n, n, rest, n, nb, o);
        }
    }
    // back substitution with U, 32-row blocks from the bottom
    for (int jb = ((n - 1) / P) * P; jb >= 0; jb -= P) {
        const int nb = min(P, n - jb);
        // R1 = U11^-1 R1 (upper, by columns)
        for (int k = threadIdx.x; k < n; k += kNT) {
            double* col = rhs + (size_t)jb * n + k;
            for (int r = nb - 1; r >= 0; --r) {
                const double* ur = w + (size_t)(jb + r) * n + jb;
                double v = col[(size_t)r * n];
                for (int q = r + 1; q < nb; ++q) v = fma(-ur[q], col[(size_t)q * n], v);
                col[(size_t)r * n] = v / ur[r];
            }
        }
        __syncthreads();
        if (jb > 0) {
            GemmOpt<double> o;
            o.subtract = true;
            o.kscale = true;
            // R0 -= U01 R1
            gemm_t<double, EMU_R, 0, false, false>(sm, rhs, n, w + jb, n, rhs + (size_t)jb * n, n, jb, n, nb, o);
        }
    }
    *logabs = la;
    *sgn = sg;
    *singular = sing;
}

// The LU of the stabilised inverse works in float64 on S0 / S1.  With T = double its
// trailing updates use the kernel's GEMM (tiled or emulated); with T = float they use a
// float64 tiled GEMM on the separate float64 staging buffer.
template <typename T, bool EMU>
__device__ void lu_solve_dispatch(TSmem<T>& sm, int n, double* la, double* sw, int* sing);

template <>
__device__ void lu_solve_dispatch<double, false>(TSmem<double>& sm, int n, double* la, double* sw, int* sing) {
    lu_solve_blocked<false, false>(sm, sm.s0, sm.s1, n, sm.panel, sm.piv, sm.sv, la, sw, sing);
}
// The stabilised matrix is graded in its rows and columns, so L21 and U12 (and U01, R1 of the
// back substitution) carry mirrored grading along the contraction index; the emulated
// products of the LU are therefore equilibrated along k (GemmOpt::kscale), which keeps their
// accuracy relative to each row / column.  LQMC_FP64E_NATIVE_LU keeps them in float64.
template <>
__device__ void lu_solve_dispatch<double, true>(TSmem<double>& sm, int n, double* la, double* sw, int* sing) {
    const bool nw = sm.native & LQMC_FP64E_NATIVE_LU, nr = sm.native & LQMC_FP64E_NATIVE_LU_RHS;
    if (nw && nr) lu_solve_blocked<false, false>(sm, sm.s0, sm.s1, n, sm.panel, sm.piv, sm.sv, la, sw, sing);
    else if (nw) lu_solve_blocked<false, true>(sm, sm.s0, sm.s1, n, sm.panel, sm.piv, sm.sv, la, sw, sing);
    else if (nr) lu_solve_blocked<true, false>(sm, sm.s0, sm.s1, n, sm.panel, sm.piv, sm.sv, la, sw, sing);
    else lu_solve_blocked<true, true>(sm, sm.s0, sm.s1, n, sm.panel, sm.piv, sm.sv, la, sw, sing);
}
template <>
__device__ void lu_solve_dispatch<float, false>(TSmem<float>& sm, int n, double* la, double* sw, int* sing) {
    // a float64 view of the workspace pointers for the float64 LU
    TSmem<double> d;
    d.stage = sm.stage64;
    d.oz = sm.oz;
    lu_solve_blocked<false, false>(d, sm.s0, sm.s1, n, sm.panel, sm.piv, sm.sv, la, sw, sing);
}

// Float64 GEMM of the QR: the emulated tensor-core GEMM, or the float64 tiled GEMM on the
// (shared) staging buffer.
template <typename T, bool EMU, bool TA, bool TB>
__device__ __forceinline__ void gemm64(TSmem<T>& sm, double* c, int ldc, const double* a, int lda,
                                       const double* b, int ldb, int m, int n, int k,
                                       GemmOpt<double> o = GemmOpt<double>()) {
    if constexpr (EMU) {
        if (sm.native & LQMC_FP64E_NATIVE_UDT) tile_gemm<double, TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.stage64, o);
        else ozt::oz_gemm_tc<TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.oz, o);
    } else {
        tile_gemm<double, TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, sm.stage64, o);
    }
}

// UDT of Z diag(d_old) T_old (pre-pivoted QR, QR in float64).  z row-major; U is written
// column-major (uc[k n + i] = U[i][k]), T row-major.  Returns det sign of U.
//
// Blocked Householder QR: each panel of qr_block(n) columns is factorised column by column,
// then the trailing columns are updated in compact WY form C -= (V T^T)(V^T C) with GEMMs.
// Q = Q_0 Q_1 ... is accumulated backwards with GEMMs (Q_p = I - V_p T_p V_p^T), and
// T_new = diag(1 / d) R P^T T_old is one GEMM.  Scratch: S1 (the panels' T factors, V, V T
// and the V^T C products) and Z0 (P^T T_old); z is dead once copied.
template <typename T, bool EMU>
__device__ double udt_absorb_t(const ChainDesc& d, TSmem<T>& sm, const T* z, const double* d_old,
                               const T* t_old, T* u_new, double* d_new, T* t_new) {
    const int n = d.n, lane = lane_id();
    // column norms of Z diag(d_old): lanes over columns (contiguous rows of z)
    for (int k = threadIdx.x; k < n; k += kNT) {
        double acc = 0.0;
#pragma unroll 8
        for (int i = 0; i < n; ++i) { const double v = (double)z[(size_t)i * n + k]; acc = fma(v, v, acc); }
        const double dk = d_old ? fabs(d_old[k]) : 1.0;
        sm.nrm[k] = sqrt(acc) * dk;
    }
    __syncthreads();
    // descending order of the norms (ties by index, NaN last), compared as integer keys
    for (int k = threadIdx.x; k < n; k += kNT) {
        const long long v = isnan(sm.nrm[k]) ? -1ll : __double_as_longlong(sm.nrm[k]);
        int rank = 0;
        for (int j = 0; j < n; ++j) {
            const long long w = isnan(sm.nrm[j]) ? -1ll : __double_as_longlong(sm.nrm[j]);
            rank += (w > v) || (w == v && j < k);
        }
        sm.order[rank] = k;
    }
    __syncthreads();
    double* s = sm.s0;   // column-major
    for (int i = warp_id(); i < n; i += kNW)
        for (int r = lane; r < n; r += 32) {
            const int src = sm.order[r];
            s[(size_t)r * n + i] = (double)z[(size_t)i * n + src] * (d_old ? d_old[src] : 1.0);
        }
    __syncthreads();
    const long long t0 = clock64();
    const int bw = qr_block(n);
    double* tstore = sm.s1;                       // panels' T factors, bw x bw each
    double* vbuf = tstore + (size_t)((n - 2) / bw + 1) * bw * bw;   // V of a panel, column-major
    double* ubuf = vbuf + (size_t)n * bw;         // V T^T (QR) or V T (Q), row-major
    double* ybuf = ubuf + (size_t)n * bw;         // V^T V, V^T C, V^T Q
    int nrefl = 0, npan = 0;
    for (int jb = 0; jb < n - 1; jb += bw, ++npan) {
        const int b = min(bw, n - 1 - jb), rows = n - jb, nc = n - jb - b;
        nrefl += householder_panel_cm(s, sm.tau, n, jb, b, sm.sv);
        panel_v(vbuf, s, n, jb, b);
        double* tf = tstore + (size_t)npan * bw * bw;
        gemm64<T, EMU, false, true>(sm, ybuf, b, vbuf, rows, vbuf, rows, b, b, rows);   // V^T V
        wy_t_factor(tf, ybuf, sm.tau + jb, b);
        if (nc > 0) {
            // U = V T^T;  Y = V^T C;  C -= U Y  (as C^T -= Y^T U^T on the column-major s)
            gemm64<T, EMU, true, true>(sm, ubuf, b, vbuf, rows, tf, b, rows, b, b);
            double* ct = s + (size_t)(jb + b) * n + jb;
            gemm64<T, EMU, false, true>(sm, ybuf, nc, vbuf, rows, ct, n, b, nc, rows);
            GemmOpt<double> o;
            o.subtract = true;
            gemm64<T, EMU, true, true>(sm, ct, n, ybuf, nc, ubuf, b, nc, rows, b, o);
        }
    }
    const long long t1 = clock64();
    if (threadIdx.x == 0) sm.sub[0] += t1 - t0;
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double di = s[(size_t)i * n + i];
        sm.dv[i] = di;
        d_new[i] = di;
        sm.xt[0][i] = (T)(1.0 / di);
    }
    // Q, backwards: Q[jb:, jb:] -= (V T)(V^T Q[jb:, jb:])
    for (int k = warp_id(); k < n; k += kNW)
        for (int i = lane; i < n; i += 32) u_new[(size_t)k * n + i] = (i == k) ? T(1) : T(0);
    __syncthreads();
    T* yq = reinterpret_cast<T*>(ybuf);
    for (int p = npan - 1; p >= 0; --p) {
        const int jb = p * bw, b = min(bw, n - 1 - jb), rows = n - jb;
        panel_v(vbuf, s, n, jb, b);
        gemm64<T, EMU, true, false>(sm, ubuf, b, vbuf, rows, tstore + (size_t)p * bw * bw, b, rows, b, b);
        T* q2 = u_new + (size_t)jb * n + jb;
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_UDT, false, true>(sm, yq, rows, vbuf, rows, q2, n, b, rows, rows);
        GemmOpt<T> o;
        o.subtract = true;
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_UDT, true, true>(sm, q2, n, yq, rows, (const double*)ubuf, b, rows, rows, b, o);
    }
    // T_new = diag(1 / d) R (P^T T_old): R's strict lower part (the reflectors) cleared, the
    // rows of T_old gathered in the pivot order
    for (int k = warp_id(); k < n; k += kNW)
        for (int i = k + 1 + lane; i < n; i += 32) s[(size_t)k * n + i] = 0.0;
    T* tg = sm.z0;
    for (int k = warp_id(); k < n; k += kNW) {
        const int src = sm.order[k];
        for (int c = lane; c < n; c += 32)
            tg[(size_t)k * n + c] = t_old ? t_old[(size_t)src * n + c] : (src == c ? T(1) : T(0));
    }
    __syncthreads();
    {
        GemmOpt<T> o;
        o.rs = sm.xt[0];
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_UDT, true, false>(sm, t_new, n, (const double*)s, n, (const T*)tg, n, n, n, n, o);
    }
    __syncthreads();
    if (threadIdx.x == 0) sm.sub[1] += clock64() - t1;
    return (nrefl & 1) ? -1.0 : 1.0;
}

// G = (1 + U_R D_R T_R T_L^T D_L U_L^T)^-1; ul == nullptr: identity left product.
// U_R, U_L column-major (uc[k n + i] = U[i][k]), T_R, T_L row-major.
template <typename T, bool EMU>
__device__ double green_udt_t(const ChainDesc& d, TSmem<T>& sm, const T* ur, const double* dr,
                              const T* tr, double sign_r, const T* ul, const double* dl,
                              const T* tl, double sign_l, T* g, bool residual, double* logdet,
                              double* sgn, int* singular) {
    const int n = d.n, lane = lane_id();
    double* dbr = sm.xv[0];
    double* dsr = sm.xv[1];
    double* dbl = sm.yv[0];
    double* dsl = sm.yv[1];
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double a = dr[i], b = fmax(fabs(a), 1.0);
        dbr[i] = b;
        dsr[i] = a / b;
        if (ul) {
            const double c = dl[i], e = fmax(fabs(c), 1.0);
            dbl[i] = e;
            dsl[i] = c / e;
        } else {
            dbl[i] = 1.0;
            dsl[i] = 1.0;
        }
    }
    if (ul) {
        // X = U_R^T U_L: A(i,p) = U_R[p][i] = ur[i n + p]; B(p,j) = U_L[p][j] = ul[j n + p]
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_GREEN, false, true>(sm, sm.z0, n, ur, n, ul, n, n, n, n);
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_GREEN, false, true>(sm, sm.z1, n, tr, n, tl, n, n, n, n);   // Y = T_R T_L^T
    }
    __syncthreads();
    for (int i = warp_id(); i < n; i += kNW)
        for (int j = lane; j < n; j += 32) {
            const size_t e = (size_t)i * n + j;
            const double x = ul ? (double)sm.z0[e] : (double)ur[e];   // U_R^T[i][j] = ur[i n + j]
            const double y = ul ? (double)sm.z1[e] : (double)tr[e];
            sm.s0[e] = x / dbr[i] / dbl[j] + dsr[i] * y * dsl[j];
            sm.s1[e] = (double)ur[e] / dbr[i];
        }
    __syncthreads();
    double la, sw;
    int sing;
    const long long t0 = clock64();
    double* zz = sm.s1;   // Z = M^-1 D_Rb^-1 U_R^T
    bool by_inverse = false;
    if constexpr (EMU) by_inverse = !(sm.native & LQMC_FP64E_NATIVE_LU_RHS);
    if constexpr (!EMU) {
        lu_solve_dispatch<T, EMU>(sm, n, &la, &sw, &sing);
    } else if (by_inverse) {
        // With emulated products the right-hand side D_Rb^-1 U_R^T (rows graded by 1 / dbr,
        // down to ~1e-30) is not pushed through the substitutions, whose intermediate rows
        // would cancel against the fixed-point rounding of their larger neighbours.  M itself
        // is O(1) and well conditioned: its inverse comes from the LU with an identity
        // right-hand side, and Z = M^-1 (D_Rb^-1 U_R^T) is one product in which every term
        // of an output is at most its largest term.
        T* rhs = sm.z1;
        for (int i = warp_id(); i < n; i += kNW)
            for (int j = lane; j < n; j += 32) {
                const size_t e = (size_t)i * n + j;
                rhs[e] = sm.s1[e];
                sm.s1[e] = (i == j) ? 1.0 : 0.0;
            }
        __syncthreads();
        lu_solve_dispatch<T, EMU>(sm, n, &la, &sw, &sing);
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_GREEN, false, false>(sm, sm.s0, n, sm.s1, n, (const T*)rhs, n, n, n, n);
        zz = sm.s0;
    } else {
        lu_solve_dispatch<T, EMU>(sm, n, &la, &sw, &sing);
    }
    if (threadIdx.x == 0) sm.sub[2] += clock64() - t0;
    if (sing) *singular = 1;
    double res = 0.0, m = 0.0;
    if (ul) {
        for (int i = warp_id(); i < n; i += kNW)
            for (int j = lane; j < n; j += 32) zz[(size_t)i * n + j] /= dbl[i];
        __syncthreads();
        // G = U_L Z: A(i,p) = U_L[i][p] = ul[p n + i]
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_GREEN, true, false>(sm, sm.z0, n, ul, n, zz, n, n, n, n);
        for (int i = warp_id(); i < n; i += kNW)
            for (int j = lane; j < n; j += 32) {
                const size_t e = (size_t)i * n + j;
                if (residual) m = fmax(m, fabs((double)sm.z0[e] - (double)g[e]));
                g[e] = sm.z0[e];
            }
    } else {
        for (int i = warp_id(); i < n; i += kNW)
            for (int j = lane; j < n; j += 32) {
                const size_t e = (size_t)i * n + j;
                if (residual) m = fmax(m, fabs(zz[e] - (double)g[e]));
                g[e] = (T)zz[e];
            }
    }
    if (residual) res = block_max(m, sm.sv);
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += kNT) part += log(dbr[i]) + log(dbl[i]);
    const double tot = block_sum(part, sm.sv);
    __syncthreads();
    *logdet = -(tot + la);
    *sgn = sign_r * sw * sign_l;
    return res;
}

// UDT of the right product through chunk c, R_c = B_{hi-1} ... B_lo R_{c-1} (slices lo..hi-1
// of the chunk), R_{c-1} from slot `in` (-1: identity), into slot `out`.
template <typename T, bool EMU>
__device__ void right_chunk_t(const ChainDesc& d, TSmem<T>& sm, int s, int c, int in, int out) {
    const int n = d.n, sigma = s ? -1 : 1;
    const size_t nn = (size_t)n * n;
    const T* ek = mat_expk<T>(d);
    const int lo = c * d.stab_every, hi = min(lo + d.stab_every, d.L);
    const int lane = lane_id();
    T* za = sm.z0;
    T* zb = sm.z1;
    for (int l = lo; l < hi; ++l) {
        load_ev_t<T>(d, sm, l, sigma);
        __syncthreads();
        GemmOpt<T> o;
        o.rs = sm.ev_t;
        if (l == lo && in < 0) {
            // e^V e^{-dtau K}: the first factor itself
            for (int i = warp_id(); i < n; i += kNW)
                for (int j = lane; j < n; j += 32)
                    zb[(size_t)i * n + j] = sm.ev_t[i] * ek[(size_t)i * n + j];
            __syncthreads();
        } else if (l == lo) {
            // B(p, j) = U[p][j] = uc[j n + p] (column-major slot)
            gemm_t<T, EMU, LQMC_FP64E_NATIVE_STACK, false, true>(sm, zb, n, ek, n, slot_U(sm, in, nn), n, n, n, n, o,
                                                                 kPreK);
        } else {
            // e^V e^{-dtau K} Z
            gemm_t<T, EMU, LQMC_FP64E_NATIVE_STACK, false, false>(sm, zb, n, ek, n, za, n, n, n, n, o, kPreK);
        }
        T* t = za; za = zb; zb = t;
    }
    const double sg = udt_absorb_t<T, EMU>(d, sm, za, in >= 0 ? slot_d(sm, in, nn) : nullptr,
                                      in >= 0 ? slot_T(sm, in, nn) : nullptr, slot_U(sm, out, nn),
                                      slot_d(sm, out, nn), slot_T(sm, out, nn));
    if (threadIdx.x == 0) slot_d(sm, out, nn)[n] = sg;
    __syncthreads();
}

// Right stack R_0 .. R_{K-1} of spin s from scratch (slots s K + c) and G = (1 + R_{K-1})^-1.
template <typename T, bool EMU>
__device__ void right_stack_t(const ChainDesc& d, TSmem<T>& sm, int s, double* logdet, double* sgn,
                              int* singular) {
    const int n = d.n;
    const size_t nn = (size_t)n * n;
    for (int c = 0; c < d.n_chunks; ++c)
        right_chunk_t<T, EMU>(d, sm, s, c, c ? s * d.n_chunks + c - 1 : -1, s * d.n_chunks + c);
    const int top = s * d.n_chunks + d.n_chunks - 1;
    green_udt_t<T, EMU>(d, sm, slot_U(sm, top, nn), slot_d(sm, top, nn), slot_T(sm, top, nn),
                   slot_d(sm, top, nn)[n], nullptr, nullptr, nullptr, 1.0, sm.g, false, logdet,
                   sgn, singular);
}

// UDT of the transposed left product through slices lo..hi-1, C^T = B_lo^T ... B_{hi-1}^T L_in
// (L_in from slot `in`; -1: identity), into slot `out`.
template <typename T, bool EMU>
__device__ void left_step_t(const ChainDesc& d, TSmem<T>& sm, int s, int in, int out, int lo,
                            int hi) {
    const int n = d.n, sigma = s ? -1 : 1;
    const size_t nn = (size_t)n * n;
    const bool first = in < 0;
    const T* ek = mat_expk<T>(d);
    T* za = sm.z0;
    T* zb = sm.z1;
    const int lane = lane_id();
    for (int l = hi - 1; l >= lo; --l) {
        load_ev_t<T>(d, sm, l, sigma);
        __syncthreads();
        if (l == hi - 1) {
            // za = e^V U (U column-major in the slot; identity on the first chunk)
            const T* u = first ? nullptr : slot_U(sm, in, nn);
            for (int k = warp_id(); k < n; k += kNW)
                for (int i = lane; i < n; i += 32)
                    za[(size_t)i * n + k] = first ? (i == k ? sm.ev_t[i] : T(0))
                                                  : sm.ev_t[i] * u[(size_t)k * n + i];
        } else {
            for (int i = warp_id(); i < n; i += kNW)
                for (int j = lane; j < n; j += 32)
                    za[(size_t)i * n + j] = sm.ev_t[i] * za[(size_t)i * n + j];
        }
        // e^{-dtau K}^T (e^V Z)
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_STACK, true, false>(sm, zb, n, ek, n, za, n, n, n, n, GemmOpt<T>(), kPreKT);
        T* t = za; za = zb; zb = t;
    }
    const double sg = udt_absorb_t<T, EMU>(d, sm, za, first ? nullptr : slot_d(sm, in, nn),
                                      first ? nullptr : slot_T(sm, in, nn), slot_U(sm, out, nn),
                                      slot_d(sm, out, nn), slot_T(sm, out, nn));
    if (threadIdx.x == 0) slot_d(sm, out, nn)[n] = sg;
    __syncthreads();
}

// Wrap across slice l.  Down (from slice l to l - 1): G <- B_l^-1 G B_l =
// e^{+dtau K} e^{-V_l} G e^{V_l} e^{-dtau K}.  Up (from slice l - 1 to l, the alternating
// order's upward sweep): G <- B_l G B_l^-1 = e^{V_l} e^{-dtau K} G e^{+dtau K} e^{-V_l}.  Both
// directions share the two product call sites; not inlined into the kernel.
template <typename T, bool EMU>
__device__ __noinline__ void wrap_t(const ChainDesc& d, TSmem<T>& sm, int l, bool up = false) {
    const int n = d.n;
    load_ev_t<T>(d, sm, l, sm.spin ? -1 : 1);
    __syncthreads();
    T* g = sm.g;
    GemmOpt<T> o1, o2;
    if (up) {
        o1.rs = sm.ev_t;
        o2.cs = sm.iev_t;
    } else {
        for (int i = warp_id(); i < n; i += kNW)
            for (int j = lane_id(); j < n; j += 32) g[(size_t)i * n + j] *= sm.iev_t[i];
        o1.cs = sm.ev_t;
    }
    gemm_t<T, EMU, LQMC_FP64E_NATIVE_WRAP, false, false>(sm, sm.z0, n, up ? mat_expk<T>(d) : mat_expkinv<T>(d),
                                                         n, g, n, n, n, n, o1, up ? kPreK : kPreKinv);
    gemm_t<T, EMU, LQMC_FP64E_NATIVE_WRAP, false, false>(sm, g, n, sm.z0, n, up ? mat_expkinv<T>(d) : mat_expk<T>(d),
                                                         n, n, n, n, o2, -1, up ? kPreKinvB : kPreKB);
}

// G <- G^T in place (through Z0)
template <typename T>
__device__ void transpose_green(TSmem<T>& sm, int n) {
    for (int i = warp_id(); i < n; i += kNW)
        for (int j = lane_id(); j < n; j += 32) sm.z0[(size_t)j * n + i] = sm.g[(size_t)i * n + j];
    __syncthreads();
    for (size_t e = threadIdx.x; e < (size_t)n * n; e += kNT) sm.g[e] = sm.z0[e];
    __syncthreads();
}

// One element global -> shared through the asynchronous copy unit (cp.async; completes on
// this thread's async_copy_wait_all).
template <typename T>
__device__ __forceinline__ void async_copy_elem(T* dst_smem, const T* src) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n"
                 :: "r"((unsigned)__cvta_generic_to_shared(dst_smem)), "l"(src), "n"(sizeof(T))
                 : "memory");
}
__device__ __forceinline__ void async_copy_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void async_copy_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Site updates of slice l, visited as step `step` of the sweep (the index of its uniforms and
// decisions: L - 1 - l going down, l going up), with delayed rank-k updates (k = d.delay): the
// accepted flips of the slice accumulate as G_eff = G - X Y^T with x = G_eff[:, i],
// y = (D/R)(e_i - G_eff[i, :]) (the Sherman-Morrison update of lqmc.py:318-331 with the defects
// fixed); every k flips, and at the end of the slice, G -= X Y^T as one GEMM per spin.
//
// The per-site critical path (ratio, cluster exchange, acceptance) reads only shared memory:
// the slice's uniforms (one Philox call per four sites, in parallel), its field values and
// G's diagonal are staged before the sites are visited (the diagonal again after every flush),
// and the row and column of G of site i + 1 are copied asynchronously while site i is decided.
template <typename T, bool EMU>
__device__ void update_slice_t(const ChainDesc& d, TSmem<T>& sm, int l, int step, int sw,
                               uint64_t sweep_id, int* accepted) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int n = d.n, L = d.L, kd = d.delay, ld = kd + 1, sp = sm.spin;
    T* g = sm.g;
    int8_t* f = d.field + (size_t)l * n;
    // staging buffers, free while sites are updated (they serve the QR otherwise)
    double* uni = sm.nrm;      // [n] the slice's uniforms
    double* gdiag = sm.tau;    // [n] diag(G) of this spin
    int* fv = sm.order;        // [n] the slice's field values at its start
    T* cnext = sm.xt[1];       // [n] G[:, i + 1]
    T* rnext = sm.yt[1];       // [n] G[i + 1, :]
    double* dsum = sm.dv;      // [n] (X Y^T)_jj of the pending updates, kept by row j's thread
    {
        const size_t base = (size_t)step * n;
        if (d.rng == LQMC_RNG_REPLAY) {
            for (int i = threadIdx.x; i < n; i += kNT) uni[i] = d.uniforms[(size_t)sw * n * L + base + i];
        } else {
            const uint64_t q0 = base >> 2, q1 = (base + n - 1) >> 2;
            for (uint64_t q = q0 + threadIdx.x; q <= q1; q += kNT) {
                double u4[4];
                philox_uniform4(d.seed, (uint64_t)d.chain_id, sweep_id, q, u4);
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const long long i = (long long)(4 * q + w) - (long long)base;
                    if (i >= 0 && i < n) uni[i] = u4[w];
                }
            }
        }
        for (int i = threadIdx.x; i < n; i += kNT) {
            fv[i] = f[i];
            gdiag[i] = (double)g[(size_t)i * n + i];
            dsum[i] = 0.0;
        }
        __syncthreads();
    }
    int m = 0;   // pending updates
    constexpr int kPer = 4;   // rows per thread: n <= kPer * kNT
    T colv[kPer], rowv[kPer];   // G[:, i] and G[i, :] of this spin for the site being decided
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int j = threadIdx.x + q * kNT;
        colv[q] = (j < n) ? g[(size_t)j * n] : T(0);
        rowv[q] = (j < n) ? g[j] : T(0);
    }
    for (int i = 0; i < n; ++i) {
        const int s_il = fv[i];
        const int par = 2 * (i & 1);
        if (threadIdx.x == 0) {
            // this spin's factor R_sigma = 1 + D_sigma (1 - G_eff,ii) and its update
            // coefficient D_sigma / R_sigma, once per CTA; the factors are exchanged.
            // G_eff,ii = G_ii - (X Y^T)_ii, the latter kept up to date by row i's thread
            const double gv = (double)((T)gdiag[i] - (T)dsum[i]);
            const double ep = s_il > 0 ? d.c[0] : d.c[1];
            const double em = s_il > 0 ? d.c[1] : d.c[0];
            const double dl = (sp ? em : ep) - 1.0;
            const double r = 1.0 + dl * (1.0 - gv);
            sm.gii[par + sp] = r;
            sm.peer_gii[par + sp] = r;
            sm.gii[4 + (i & 1)] = dl / r;
        }
        // the next site's row and column are in flight while this one is decided (each thread
        // copies and later reads only its own rows j)
        if (i + 1 < n) {
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const int j = threadIdx.x + q * kNT;
                if (j < n) {
                    async_copy_elem(cnext + j, g + (size_t)j * n + i + 1);
                    async_copy_elem(rnext + j, g + (size_t)(i + 1) * n + j);
                }
            }
        }
        async_copy_commit();
        const long long tb = clock64();
        cluster.sync();
        if (threadIdx.x == 0) sm.sub[7] += clock64() - tb;
        const double ratio = sm.gii[par] * sm.gii[par + 1];   // R_up R_dn, the same product in both CTAs
        const bool acc = (uni[i] <= ratio);
        if (sp == 0 && d.record && threadIdx.x == 0) d.decisions[((size_t)sw * L + step) * n + i] = acc ? 1 : 0;
        bool flushed = false;
        if (acc) {
            const T a = (T)sm.gii[4 + (i & 1)];
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const int j = threadIdx.x + q * kNT;
                if (j >= n) break;
                T cu = colv[q], rv = rowv[q];
                // unrolled so that the loads of several p (X and Y may live in global memory)
                // are in flight together; the FMA order per output is unchanged
#pragma unroll 4
                for (int p = 0; p < m; ++p) {
                    cu = fma(-sm.dx[(size_t)j * ld + p], sm.dy[(size_t)i * ld + p], cu);   // G_eff[j][i]
                    rv = fma(-sm.dx[(size_t)i * ld + p], sm.dy[(size_t)j * ld + p], rv);   // G_eff[i][j]
                }
                const T yn = ((j == i ? T(1) : T(0)) - rv) * a;
                sm.dx[(size_t)j * ld + m] = cu;
                sm.dy[(size_t)j * ld + m] = yn;
                dsum[j] = fma((double)cu, (double)yn, dsum[j]);
            }
            if (threadIdx.x == 0) {
                f[i] = (int8_t)(-s_il);   // both CTAs write the same value
                if (sp == 0) ++*accepted;
            }
            __syncthreads();
            if (++m == kd) {
                // the copies of the next row and column read G before this flush changes it
                async_copy_wait_all();
                const long long tf = clock64();
                GemmOpt<T> o;
                o.subtract = true;
                gemm_t<T, EMU, LQMC_FP64E_NATIVE_UPDATE, false, true>(sm, g, n, sm.dx, ld, sm.dy, ld, n, n, m, o);
                if (threadIdx.x == 0) sm.sub[6] += clock64() - tf;
                m = 0;
                flushed = true;
                for (int j = threadIdx.x; j < n; j += kNT) {
                    gdiag[j] = (double)g[(size_t)j * n + j];
                    dsum[j] = 0.0;
                }
                __syncthreads();
            }
        }
        async_copy_wait_all();
        if (i + 1 < n) {
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const int j = threadIdx.x + q * kNT;
                if (flushed) {   // G changed: the next row and column are read again
                    colv[q] = (j < n) ? g[(size_t)j * n + i + 1] : T(0);
                    rowv[q] = (j < n) ? g[(size_t)(i + 1) * n + j] : T(0);
                } else {
                    colv[q] = (j < n) ? cnext[j] : T(0);
                    rowv[q] = (j < n) ? rnext[j] : T(0);
                }
            }
        }
    }
    if (m > 0) {
        const long long tf = clock64();
        GemmOpt<T> o;
        o.subtract = true;
        gemm_t<T, EMU, LQMC_FP64E_NATIVE_UPDATE, false, true>(sm, g, n, sm.dx, ld, sm.dy, ld, n, n, m, o);
        if (threadIdx.x == 0) sm.sub[6] += clock64() - tf;
    }
    __syncthreads();
}

// Measurements of one sweep: each CTA adds its spin's part; the spin diagonals are
// exchanged through distributed shared memory for the terms that need both spins, which
// the spin-up CTA adds.  Entries both CTAs add to are accumulated atomically.
template <typename T>
__device__ void measure_t(const ChainDesc& d, TSmem<T>& sm) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int n = d.n, sp = sm.spin;
    const size_t nn = (size_t)n * n;
    const T* g = sm.g;
    double* obs = d.obs;
    for (int i = warp_id(); i < n; i += kNW)
        for (int j = lane_id(); j < n; j += 32) {
            const size_t e = (size_t)i * n + j;
            d.gsum[(size_t)sp * nn + e] += (double)g[e];
        }
    double* nv = sm.xv[sp];
    double* peer_nv = sm.peer_xv + (size_t)sp * n;
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double a = 1.0 - (double)g[(size_t)i * n + i];
        nv[i] = a;
        peer_nv[i] = a;
    }
    cluster.sync();
    const double* nu = sm.xv[0];
    const double* nd = sm.xv[1];
    double ek = 0.0, ep = 0.0, dc = 0.0, dn = 0.0;
    for (int j = warp_id(); j < n; j += kNW)
        for (int k = lane_id(); k < n; k += 32) {
            const double kv = d.kinetic[(size_t)j * n + k];
            if (kv != 0.0) ek += kv * (((j == k) ? 1.0 : 0.0) - (double)g[(size_t)k * n + j]);
        }
    if (sp == 0) {
        for (int i = threadIdx.x; i < n; i += kNT) {
            obs[LQMC_OBS_HEADER + i] += nu[i] + nd[i];
            obs[LQMC_OBS_HEADER + n + i] += nu[i] * nd[i];
            ep += (nu[i] - 0.5) * (nd[i] - 0.5);
            dc += nu[i] * nd[i];
            dn += nu[i] + nd[i];
        }
    }
    ek = block_sum(ek, sm.sv);
    ep = block_sum(ep, sm.sv);
    dc = block_sum(dc, sm.sv);
    dn = block_sum(dn, sm.sv);
    // entries both spins add to are added in a fixed order (spin up, cluster barrier, spin
    // down), so that the sums do not depend on which CTA gets there first
    double* onn = obs + LQMC_OBS_HEADER + 2 * n;
    double* osz = onn + nn;
    const double* ns = sm.xv[sp];
    for (int turn = 0; turn < 2; ++turn) {
        if (turn == sp) {
            if (threadIdx.x == 0) {
                obs[1] += ek;
                if (sp == 0) {
                    obs[0] += 1.0;
                    obs[2] += d.u * ep;
                    obs[3] += dc / n;
                    obs[4] += dn / n;
                }
            }
            for (int i = warp_id(); i < n; i += kNW)
                for (int j = lane_id(); j < n; j += 32) {
                    const size_t e = (size_t)i * n + j;
                    const double del = (i == j) ? 1.0 : 0.0;
                    const double same = ns[i] * ns[j] + (del - (double)g[(size_t)j * n + i]) * (double)g[e];
                    const double cross = sp == 0 ? nu[i] * nd[j] + nd[i] * nu[j] : 0.0;
                    onn[e] += same + cross;
                    osz[e] += 0.25 * (same - cross);
                }
        }
        cluster.sync();
    }
}

}  // namespace

template <typename T, bool EMU>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kNT, 1)
sweep_tiled_kernel(const ChainDesc* __restrict__ descs, int n_sweeps, int do_measure,
                   int sweep_base) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) double smem[];
    __shared__ ChainDesc d;
    __shared__ int accepted;
    __shared__ int singular;
    __shared__ long long sub[8];
    __shared__ ozt::Tc tcs;
    __shared__ double peer_resid;
    const int sp = (int)cluster.block_rank();   // spin of this CTA
    if (threadIdx.x == 0) {
        d = descs[blockIdx.x >> 1];
        accepted = 0;
        singular = 0;
        for (int k = 0; k < 8; ++k) sub[k] = 0;
        peer_resid = 0.0;
    }
    __syncthreads();
    if constexpr (EMU) {
        ozt::tc_setup(&tcs);   // TMEM columns and the pipeline's mbarriers
        if (threadIdx.x == 0 && (d.debug & LQMC_DEBUG_STALL_TC_WAIT) && d.diag[7] == 0.0) tcs.stall = 1;
    }
    const int n = d.n;
    const size_t nn = (size_t)n * n;
    const bool xy_global = (d.flags & kUpdatesInGlobal) != 0;
    TiledLayout<T> lay(n, d.n_chunks, EMU, xy_global ? d.delay : 0, d.order == LQMC_ORDER_ALTERNATE);
    unsigned char* w = reinterpret_cast<unsigned char*>(d.work);
    unsigned char* wb = w + (size_t)sp * lay.spin_block;   // this spin's block
    TSmem<T> sm;
    sm.spin = sp;
    sm.g = reinterpret_cast<T*>(wb + lay.g);
    sm.z0 = reinterpret_cast<T*>(wb + lay.z);
    sm.z1 = sm.z0 + nn;
    sm.s0 = reinterpret_cast<double*>(wb + lay.s);
    sm.s1 = sm.s0 + nn;
    sm.slots = w + lay.g_slots;
    sm.slot_bytes = lay.slot;
    sm.sub = sub;
    double* p = smem;
    sm.sv = p; p += kNW + 8;
    sm.xv[0] = p; p += n;
    sm.xv[1] = p; p += n;
    sm.yv[0] = p; p += n;
    sm.yv[1] = p; p += n;
    sm.ev = p; p += n;
    sm.nrm = p; p += n;
    sm.tau = p; p += n;
    sm.dv = p; p += n;
    sm.order = reinterpret_cast<int*>(p); p += n;
    p = smem + (((p - smem) + 3) & ~(ptrdiff_t)3);
    T* tp = reinterpret_cast<T*>(p);
    sm.ev_t = tp; tp += n;
    sm.iev_t = tp; tp += n;
    sm.xt[0] = tp; tp += n;
    sm.xt[1] = tp; tp += n;
    sm.yt[0] = tp; tp += n;
    sm.yt[1] = tp; tp += n;
    p = reinterpret_cast<double*>(tp);
    p = smem + (((p - smem) + 3) & ~(ptrdiff_t)3);
    sm.gii = p; p += 8;
    if (EMU) p = smem + (((p - smem) + 15) & ~(ptrdiff_t)15);   // 128-byte aligned stage
    sm.stage = reinterpret_cast<T*>(p);
    sm.oz.stage = reinterpret_cast<unsigned char*>(p);
    sm.oz.stages = d.oz_stages;
    sm.native = d.native;
    if constexpr (EMU) {
        const PresplitLayout pl(n);
        for (int i = 0; i < kNumPre; ++i) {
            sm.pre[i].slices = reinterpret_cast<const __nv_bfloat16*>(d.presplit + pl.slices(i));
            sm.pre[i].exps = reinterpret_cast<const int*>(d.presplit + pl.e) + i * n;
        }
    }
    sm.oz.tc = &tcs;
    sm.stage64 = p;   // the float64 LU staging (float kernel) shares the staging region
    const size_t stage_region = stage_region_bytes(sizeof(T) == 4, EMU, d.oz_stages);
    tp = sm.stage + stage_region / sizeof(T);
    sm.oz.slices = reinterpret_cast<__nv_bfloat16*>(wb + lay.oz);
    sm.oz.ea = reinterpret_cast<int*>(wb + lay.oz_ea);
    sm.oz.eb = sm.oz.ea + n;
    sm.oz.cycles = sub + 3;   // splitting, product loops, epilogues
    const size_t dsz = (size_t)n * (d.delay + 1);
    if (xy_global) {
        sm.dx = reinterpret_cast<T*>(wb + lay.xy);
        sm.dy = sm.dx + dsz;
    } else {
        sm.dx = tp; tp += dsz;
        sm.dy = tp; tp += dsz;
    }
    {
        // The LU panel overlays the GEMM staging and the delayed-update buffers: the panel is
        // live only between a panel load and the trailing-update GEMMs, and X / Y only
        // between refreshes.  The pivot list follows the larger of the two.
        sm.panel = p;
        const size_t rbytes = stage_region + (xy_global ? 0 : 2 * dsz * sizeof(T));
        const size_t pbytes = (size_t)n * (panel_width(n) + 1) * sizeof(double);
        unsigned char* q = reinterpret_cast<unsigned char*>(p) + (rbytes > pbytes ? rbytes : pbytes);
        q = reinterpret_cast<unsigned char*>(((uintptr_t)q + 15) & ~(uintptr_t)15);
        sm.piv = reinterpret_cast<int*>(q);
    }
    // the partner CTA's exchange buffers
    sm.peer_gii = cluster.map_shared_rank(sm.gii, (unsigned)(sp ^ 1));
    sm.peer_xv = cluster.map_shared_rank(sm.xv[0], (unsigned)(sp ^ 1));
    cluster.sync();   // both CTAs set up before any remote write

    double max_resid = 0.0, logdet = 0.0, sgn = 1.0;
    uint64_t sweep_id = (uint64_t)d.diag[7];
    long long ph[5] = {0, 0, 0, 0, 0};   // clock cycles per phase (thread 0)
    long long tc = clock64();
#define LQMC_PHASE(k)                       \
    do {                                    \
        __syncthreads();                    \
        const long long t_ = clock64();     \
        ph[k] += t_ - tc;                   \
        tc = t_;                            \
    } while (0)
    // sw indexes the call's uniforms and decisions: sweep_base + the sweep of this launch.
    // Alternating order (d.order): state 0 = no valid stacks (build the right stack from
    // scratch and sweep down), 1 = the next sweep goes up, 2 = the next sweep goes down on the
    // right products the up sweep left.
    const bool alt = d.order == LQMC_ORDER_ALTERNATE;
    const int K = d.n_chunks;
    int state = alt ? (int)d.diag[21] : 0;
    auto lslot = [&](int c) { return 2 * K + sp * K + c; };   // alternating: left product at boundary c s
    for (int sw = sweep_base; sw < sweep_base + n_sweeps; ++sw, ++sweep_id) {
        if (!(alt && state == 1)) {
            // ---- down: l = L-1 .. 0 (the reference's order) ----
            if (!(alt && state == 2)) right_stack_t<T, EMU>(d, sm, sp, &logdet, &sgn, &singular);
            LQMC_PHASE(0);
            int lp = 0;
            for (int c = K - 1; c >= 0; --c) {
                const int lo = c * d.stab_every, hi = min(lo + d.stab_every, d.L);
                for (int l = hi - 1; l >= lo; --l) {
                    update_slice_t<T, EMU>(d, sm, l, d.L - 1 - l, sw, sweep_id, &accepted);
                    LQMC_PHASE(1);
                    if (l > 0 || alt) wrap_t<T, EMU>(d, sm, l);
                    LQMC_PHASE(2);
                }
                if (c > 0) {
                    int ls;
                    if (alt) {
                        ls = lslot(c);
                        left_step_t<T, EMU>(d, sm, sp, c == K - 1 ? -1 : lslot(c + 1), ls, lo, hi);
                    } else {
                        const int in = 2 * K + 2 * sp + lp;
                        lp ^= 1;
                        ls = 2 * K + 2 * sp + lp;
                        left_step_t<T, EMU>(d, sm, sp, c == K - 1 ? -1 : in, ls, lo, hi);
                    }
                    const int rs = sp * K + c - 1;
                    const double r = green_udt_t<T, EMU>(
                        d, sm, slot_U(sm, rs, nn), slot_d(sm, rs, nn), slot_T(sm, rs, nn),
                        slot_d(sm, rs, nn)[n], slot_U(sm, ls, nn), slot_d(sm, ls, nn),
                        slot_T(sm, ls, nn), slot_d(sm, ls, nn)[n], sm.g, true, &logdet, &sgn, &singular);
                    max_resid = fmax(max_resid, r);
                    LQMC_PHASE(3);
                } else if (alt) {
                    // the bottom turn: G wrapped down to tau = 0 and refreshed as
                    // G(0) = (1 + B_{L-1} ... B_0)^-1 = ((1 + C^T)^-1)^T from the full left product
                    const int ls = lslot(0);
                    left_step_t<T, EMU>(d, sm, sp, K == 1 ? -1 : lslot(1), ls, lo, hi);
                    transpose_green<T>(sm, n);
                    const double r = green_udt_t<T, EMU>(
                        d, sm, slot_U(sm, ls, nn), slot_d(sm, ls, nn), slot_T(sm, ls, nn),
                        slot_d(sm, ls, nn)[n], nullptr, nullptr, nullptr, 1.0, sm.g, true, &logdet, &sgn,
                        &singular);
                    transpose_green<T>(sm, n);
                    max_resid = fmax(max_resid, r);
                    LQMC_PHASE(3);
                }
            }
            if (alt) state = 1;
        } else {
            // ---- up: l = 0 .. L-1; each slice is wrapped into before its sites are visited,
            // and each chunk's right product becomes the next down sweep's right stack ----
            for (int c = 0; c < K; ++c) {
                const int lo = c * d.stab_every, hi = min(lo + d.stab_every, d.L);
                for (int l = lo; l < hi; ++l) {
                    wrap_t<T, EMU>(d, sm, l, true);
                    LQMC_PHASE(2);
                    update_slice_t<T, EMU>(d, sm, l, l, sw, sweep_id, &accepted);
                    LQMC_PHASE(1);
                }
                const int rs = sp * K + c;
                right_chunk_t<T, EMU>(d, sm, sp, c, c ? rs - 1 : -1, rs);
                double r;
                if (c < K - 1) {
                    const int ls = lslot(c + 1);
                    r = green_udt_t<T, EMU>(d, sm, slot_U(sm, rs, nn), slot_d(sm, rs, nn), slot_T(sm, rs, nn),
                                            slot_d(sm, rs, nn)[n], slot_U(sm, ls, nn), slot_d(sm, ls, nn),
                                            slot_T(sm, ls, nn), slot_d(sm, ls, nn)[n], sm.g, true, &logdet,
                                            &sgn, &singular);
                } else {
                    // the top turn: G(beta) = (1 + B_{L-1} ... B_0)^-1 from the full right product
                    r = green_udt_t<T, EMU>(d, sm, slot_U(sm, rs, nn), slot_d(sm, rs, nn), slot_T(sm, rs, nn),
                                            slot_d(sm, rs, nn)[n], nullptr, nullptr, nullptr, 1.0, sm.g, true,
                                            &logdet, &sgn, &singular);
                }
                max_resid = fmax(max_resid, r);
                LQMC_PHASE(3);
            }
            state = 2;
        }
        __syncthreads();
        if (do_measure) measure_t<T>(d, sm);
        LQMC_PHASE(4);
        int bad = 0;
        for (size_t e = threadIdx.x; e < nn; e += kNT)
            if (!isfinite((double)sm.g[e])) bad = 1;
        bad = __syncthreads_or(bad);
        if (bad && threadIdx.x == 0) atomicOr(d.status, LQMC_STATUS_NONFINITE);
    }
#undef LQMC_PHASE
    for (size_t e = threadIdx.x; e < nn; e += kNT) d.green[(size_t)sp * nn + e] = (double)sm.g[e];
    // the spin-down CTA hands its residual to the spin-up CTA, which writes the diagnostics
    if (sp == 1 && threadIdx.x == 0) *cluster.map_shared_rank(&peer_resid, 0u) = max_resid;
    cluster.sync();
    if (threadIdx.x == 0) {
        d.diag[3 + sp] = logdet;
        d.diag[5 + sp] = sgn;
        if (singular) atomicOr(d.status, LQMC_STATUS_SINGULAR);
        if (sp == 0) {
            max_resid = fmax(max_resid, peer_resid);
            d.diag[0] += (double)accepted;
            d.diag[1] += (double)n_sweeps * n * d.L;
            d.diag[2] = max_resid;
            d.diag[7] += (double)n_sweeps;
            if (alt) d.diag[21] = (double)state;
            for (int k = 0; k < 5; ++k) d.diag[8 + k] = (double)ph[k];
            for (int k = 0; k < 8; ++k) d.diag[13 + k] = (double)sub[k];
            if (max_resid > d.drift_tol) atomicOr(d.status, LQMC_STATUS_DRIFT);
        }
    }
    if constexpr (EMU) {
        if (threadIdx.x == 0 && tcs.fail) atomicOr(d.status, LQMC_STATUS_TIMEOUT);
        ozt::tc_teardown(&tcs);
    }
}

template <typename T, bool EMU>
static cudaError_t launch_tiled(const ChainDesc* d_descs, int n_chains, size_t smem, int n_sweeps,
                                int measure, int sweep_base, cudaStream_t stream) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(sweep_tiled_kernel<T, EMU>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // two CTAs (one cluster) per chain
    sweep_tiled_kernel<T, EMU><<<2 * n_chains, kNT, smem, stream>>>(d_descs, n_sweeps, measure,
                                                                  sweep_base);
    return cudaGetLastError();
}

// The constant operands of every distinct e^{-dtau K} (PresplitLayout): block kNumPre g + i
// splits operand i of job g.  Runs once per handle, before the first sweep.
struct PresplitJob {
    const double* expk;
    const double* expkinv;
    unsigned char* out;
    int n;
};

static __global__ void __launch_bounds__(kNT) presplit_kernel(const PresplitJob* jobs) {
    __shared__ int scratch[ozt::kScratchStripes + 8 * kNT];
    const PresplitJob j = jobs[blockIdx.x / kNumPre];
    const int i = blockIdx.x % kNumPre, n = j.n;
    const PresplitLayout pl(n);
    __nv_bfloat16* slices = reinterpret_cast<__nv_bfloat16*>(j.out + pl.slices(i));
    int* exps = reinterpret_cast<int*>(j.out + pl.e) + i * n;
    if (i == kPreK) ozt::presplit(j.expk, n, true, false, n, n, slices, exps, scratch);
    else if (i == kPreKT) ozt::presplit(j.expk, n, true, true, n, n, slices, exps, scratch);
    else if (i == kPreKinv) ozt::presplit(j.expkinv, n, true, false, n, n, slices, exps, scratch);
    else if (i == kPreKB) ozt::presplit(j.expk, n, false, false, n, n, slices, exps, scratch);
    else ozt::presplit(j.expkinv, n, false, false, n, n, slices, exps, scratch);
}

}  // namespace lqmc
