// Float64-accurate GEMM on the 5th-generation (tcgen05) tensor cores for one CTA of
// blk::kNT threads (Ozaki-style operand splitting, exact integer slice products).
//
// Row i of op(A) is scaled by 2^-E_i (E_i = exponent just above its largest entry) and
// rounded to the nearest 55-bit fixed-point integer N = round(a 2^(55 - E_i)), |N| <= 2^55,
// which is written in kSlices = 8 balanced base-128 digits q_t in [-64, 64] (exact in
// bfloat16): N = sum_t q_t 2^(7 (7 - t)).  Columns of op(B) likewise with 2^-F_j.  Then
// C_ij = 2^(E_i + F_j - 61) sum_{d<8} 2^(7 (7 - d)) D_d with D_d = sum_{t+u=d} (A_t B_u)_ij,
// keeping the 36 leading digit pairs.  The operands carry 2^-56 of their row / column
// maximum, finer than float64's own rounding, and the rounding and the dropped pairs
// (t + u >= 8, below 2^-60) have either sign, so their errors do not accumulate
// systematically over k.  Each A_t B_u is a tcgen05.mma (kind::f16, BF16 x BF16 -> FP32,
// M = 128, K = 16) accumulating into the TMEM columns of diagonal d: the eight accumulators
// of a 128 x 32 output tile take 256 TMEM columns, two tiles the SM's 512.  The FP32 sums are exact
// integers while |D_d| <= 8 k 64^2 <= 2^23, i.e. for k <= kMaxK = 256 (the bound that also lets
// the epilogue combine digit pairs in int32); longer products are cut
// into chunks of kMaxK whose results are added in float64.  A row (column) holding a NaN or
// Inf gives NaN in its output row (column).
//
// Data movement: the split writes every slice directly in the tensor core's canonical
// K-major, no-swizzle layout (8 x 16-byte core matrices), grouped so that all eight slices
// of one (row block, 16-wide k step) are one contiguous block; B's slices of a 32-column block
// stack into one 256-row operand.  The product then runs as a warp-specialised pipeline over
// 128 x 32 output tiles (x k chunks of kMaxK):
//   warp 1 (one thread)   streams each k step of A (32 KB) and B (8 KB) into a ring of
//                         `stages` shared-memory stage buffers, two bulk asynchronous copies
//                         per stage completing on the stage's `full` mbarrier;
//   warp 0 (one thread)   issues the step's MMAs -- one per A digit t, A_t times the stacked
//                         B_0 .. B_{7-t} (N = 32 (8 - t)) -- into one of two TMEM accumulator
//                         buffers (the 8 diagonals of a tile take 256 columns), commits each
//                         step to the stage's `empty` mbarrier and each tile to `acc_full`;
//   warps 4..7            drain a finished buffer (warp w reads TMEM lanes 32 (w mod 4) ..)
//                         while the MMAs of the next tile fill the other, combine the digits
//                         in int64, convert to float64 with integer operations (the scale
//                         folded into the exponent) and write C, then release the buffer.
// Every wait is bounded: a wait that runs out sets Tc::fail, after which this and every later
// call return without issuing work; the kernel reports the flag as a status bit.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "block_fp64.cuh"
#include "block_gemm.cuh"

namespace lqmc {
namespace ozt {

using namespace blk;

constexpr int kSlices = 8;
constexpr int kBits = 7;
constexpr int kWidth = kSlices * kBits - 1;   // 55: the top digit absorbs the rounding carry
constexpr int kBM = 128, kBN = 32, kBK = 16;
constexpr int kTileA = kBM * kBK;             // bf16 elements of one slice tile of A (4 KB)
constexpr int kTileB = kBN * kBK;             // one slice tile of B (1 KB)
constexpr int kStepA = kSlices * kTileA;      // all slices of one (row block, k step)
constexpr int kStepB = kSlices * kTileB;
constexpr int kMaxK = 256;                    // exact FP32 diagonal sums (and the epilogue's
                                              // int32 digit pairs) up to this k
constexpr int kAccCols = kSlices * kBN;       // 256: the eight diagonals of one output tile
constexpr int kTmemCols = 2 * kAccCols;       // 512: two accumulator buffers, the whole TMEM
constexpr int kMaxStages = 3;                 // stage buffers of the copy / MMA ring
constexpr int kEpiWarp0 = 4;                  // warps 4..7 drain the accumulators (TMEM lane
                                              // quadrant = warp % 4); warp 0 issues the MMAs,
                                              // warp 1 the copies
constexpr int kNonFinite = 1 << 20;

// The epilogue drops the 12 low bits of the combined diagonals (so that the sum fits int64).
// 1 (default): round them to nearest (an error below 2^-50 of 2^(E_i + F_j), either sign, no
// bias); 0: floor them (below 2^-49, one-signed).  At 16x16, beta=8, stabilisation every 8
// slices, rounding lowered the fp64e engine's median stabilisation residual about 3x and its
// G error against float64 2-3x (16 chains, 6 sweeps).
#ifndef LQMC_OZ_ROUND_EPILOGUE
#define LQMC_OZ_ROUND_EPILOGUE 1
#endif
constexpr long long kLowRound = LQMC_OZ_ROUND_EPILOGUE ? (1ll << 11) : 0;
constexpr long long kWaitCycles = 2000000000ll;   // ~1 s of SM clock before a wait gives up

// shared-memory bytes of `stages` stage buffers (1 .. kMaxStages)
__host__ __device__ constexpr size_t stage_bytes(int stages) {
    return (size_t)stages * (kStepA + kStepB) * sizeof(__nv_bfloat16);
}

__host__ __device__ constexpr int kpad(int k) { return (k + kBK - 1) / kBK * kBK; }
__host__ __device__ constexpr int rows_pad(int m, int blk) { return (m + blk - 1) / blk * blk; }

// bf16 elements of the slice buffers of an (m x k) times (k x n) product
__host__ __device__ constexpr size_t slice_elems(int m, int n, int k) {
    return (size_t)kSlices * ((size_t)rows_pad(m, kBM) + rows_pad(n, kBN)) * kpad(k);
}

// element offset of (row r, k index q) inside one slice tile: core matrix (r / 8, q / 8) at
// (r / 8) * 128 + (q / 8) * 64 elements (SBO = 256 B, LBO = 128 B), 8 x 8 elements inside
__device__ __forceinline__ int core_offset(int r, int q) {
    return (r >> 3) * 128 + (q >> 3) * 64 + (r & 7) * 8 + (q & 7);
}

// per-CTA state of the tensor-core path (static shared memory of the kernel)
// The pipeline's barriers complete once per use; a waiter for the u-th completion (u >= 1)
// waits on parity (u - 1) & 1.  `steps` and `units` count the k steps and accumulation units
// (output tile x k chunk) of all earlier calls, so every role derives its parities from them.
struct Tc {
    unsigned long long full[kMaxStages];    // stage loaded (bulk-copy transaction count)
    unsigned long long empty[kMaxStages];   // the MMAs that read the stage have completed
    unsigned long long acc_full[2];         // accumulator buffer complete (MMA commit)
    unsigned long long acc_empty[2];        // accumulator buffer drained (one arrival per
                                            // epilogue warp)
    uint32_t tmem;               // TMEM base address (lane 0, first column)
    uint32_t steps;              // k steps of all earlier calls
    uint32_t units;              // accumulation units of all earlier calls
    int fail;                    // a wait ran out
    int stall;                   // test hook: the next step issues no copies (its wait runs out)
};

struct Workspace {
    __nv_bfloat16* slices;   // slice_elems(m, n, k) bf16, 16-byte aligned
    int* ea;                 // m
    int* eb;                 // n
    unsigned char* stage;    // stage_bytes(stages) of shared memory, 128-byte aligned
    int stages;              // 1 .. kMaxStages
    Tc* tc;
    long long* cycles;       // optional [3]: splitting, whole product pipeline, the epilogue
                             // warps' combine and write-out (first epilogue warp)
};

// An operand split once and reused (constant matrices): its slices in the tile layout of
// split_tiles (A: row blocks of kBM, B: column blocks of kBN) and its exponents.
struct Presplit {
    const __nv_bfloat16* slices;
    const int* exps;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// ---- TMEM and barrier set-up, once per kernel --------------------------------------------

// warp 0 allocates the 512 TMEM columns; all threads initialise after a barrier
__device__ inline void tc_setup(Tc* tc) {
    if (warp_id() == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tc->tmem)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < kMaxStages; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&tc->full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&tc->empty[i])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&tc->acc_full[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n"
                         :: "r"(smem_u32(&tc->acc_empty[b])), "r"(kNW - kEpiWarp0));
        }
        tc->steps = 0;
        tc->units = 0;
        tc->fail = 0;
        tc->stall = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// warp 0 frees the TMEM columns; every MMA has completed (each call waits for its last commit)
__device__ inline void tc_teardown(Tc* tc) {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp_id() == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                     :: "r"(tc->tmem), "r"(kTmemCols));
}

// bounded parity wait; false when about kWaitCycles passed without the phase completing, or
// when another role of the pipeline has already given up (fail != 0)
__device__ __forceinline__ bool bar_wait(unsigned long long* bar, uint32_t parity,
                                         const volatile int* fail = nullptr) {
    const uint32_t a = smem_u32(bar);
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
        if ((fail && *fail) || clock64() - t0 > kWaitCycles) return false;
    }
}

__device__ __forceinline__ void bar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" :: "r"(smem_u32(bar)) : "memory");
}

// ---- splitting ---------------------------------------------------------------------------

// biased exponent of v scaled by 2^off (0 for zero / subnormal, 0x7FF for NaN / Inf)
__device__ __forceinline__ int biased_exp(double v, int off) {
    const int be = (int)((__double_as_longlong(v) >> 52) & 0x7FF);
    return (be == 0 || be == 0x7FF) ? be : be + off;
}

// N = round(v 2^off 2^(55 - e)) for |v 2^off| < 2^e (ties away from zero), 0 for zero /
// non-finite
__device__ __forceinline__ long long fixed55(double v, int e, int off) {
    const long long bits = __double_as_longlong(v);
    const int be = (int)((bits >> 52) & 0x7FF);
    const bool zero = be == 0 || be == 0x7FF || e == kNonFinite;
    const unsigned long long mant = ((unsigned long long)bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    // v 2^(55 - e) = mant 2^(be - 1075 + 55 - e); |v| < 2^e bounds the left shift by 2.
    // Selects only (both shifts clamped to [0, 63]), so that the 8 elements of a unit interleave
    const int rs = 1075 - 55 + e - (be + off);
    const unsigned long long left = mant << min(max(-rs, 0), 63);
    const unsigned long long right = ((mant >> (min(max(rs, 1), 64) - 1)) + 1ull) >> 1;
    const unsigned long long mag = zero ? 0ull : (rs <= 0 ? left : right);
    return bits < 0 ? -(long long)mag : (long long)mag;
}

// Scratch offsets (ints) in the stage buffer: the exponent maxima of split_tiles (rows <=
// 1024), the k-scaling shifts, and the per-stripe maxima of a transposed split (<= kNT * 8).
constexpr int kMaxKscale = 1024;
constexpr int kScratchKA = 2048, kScratchKB = kScratchKA + kMaxKscale;
constexpr int kScratchStripes = kScratchKB + kMaxKscale;
static_assert((kScratchStripes + 8 * kNT) * sizeof(int) <= (kStepA + kStepB) * sizeof(__nv_bfloat16),
              "split scratch fits one stage buffer");

// Split X (rows x k), X(r, q) = trans ? x[q ld + r] : x[r ld + q], into the tile layout with
// row blocks of BLK rows: slice t of (row block rb, k step s) at
// ((rb * S + s) * kSlices + t) * BLK * kBK, S = kpad(k) / kBK.  Rows >= `rows` and k >= `k`
// are zero.  exps[r] = E_r.  `scratch` is shared memory of kScratchStripes + 8 kNT ints.
//
// The exponent pass keeps its maxima in registers and reduces them per warp (row-contiguous
// X) or through one shared-memory combine of per-stripe maxima (transposed X), without
// atomics; NaN or Inf (biased exponent 0x7FF) dominates and marks the row.  The digit pass
// reads 8 consecutive elements of memory per unit with independent loads, so many L2
// requests are in flight.
// kshift (optional, k ints): element (r, q) is split as X(r, q) 2^kshift[q] (exact).
template <int BLK>
__device__ __noinline__ void split_tiles(const double* x, int ld, bool trans, int rows, int k, int* exps,
                            __nv_bfloat16* dst, int* scratch, const int* kshift = nullptr) {
    const int kp = kpad(k), S = kp / kBK, rp = rows_pad(rows, BLK);
    if (!trans) {
        // a warp takes rpw rows at a time, lpr lanes per row (lanes read 8 consecutive k each,
        // lpr the fewest lanes that cover k, at most 32), and kRowSets such row sets at once:
        // every load of a warp's rows is in flight together, one reduction per row set
        constexpr int kRowSets = 4;
        const int lane = lane_id();
        const int lpr = k <= 8 ? 1 : k <= 16 ? 2 : k <= 32 ? 4 : k <= 64 ? 8 : k <= 128 ? 16 : 32;
        const int rpw = 32 / lpr, sub = lane / lpr, ql = lane % lpr;
        for (int r0 = warp_id() * rpw; r0 < rows; r0 += kNW * rpw * kRowSets) {
            int em[kRowSets];
#pragma unroll
            for (int t = 0; t < kRowSets; ++t) em[t] = 0;
            for (int q0 = 8 * ql; q0 < k; q0 += 8 * lpr) {
#pragma unroll
                for (int t = 0; t < kRowSets; ++t) {
                    const int r = r0 + t * kNW * rpw + sub;
                    if (r < rows) {
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                            if (q0 + c < k)
                                em[t] = max(em[t], biased_exp(x[(size_t)r * ld + q0 + c], kshift ? kshift[q0 + c] : 0));
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < kRowSets; ++t) {
                for (int o = lpr / 2; o > 0; o >>= 1) em[t] = max(em[t], __shfl_xor_sync(0xffffffffu, em[t], o));
                const int r = r0 + t * kNW * rpw + sub;
                if (ql == 0 && r < rows) scratch[r] = em[t];
            }
        }
    } else {
        // thread (group of 8 consecutive rows, stripe of k) keeps 8 maxima in registers while
        // it walks its stripe (a warp, 32 groups of one k, reads contiguous memory), four k of
        // the stripe per step so that their loads are in flight together; the stripes'
        // maxima are combined through shared memory
        int* part = scratch + kScratchStripes;
        const int g8 = (rows + 7) / 8, nq = max(1, kNT / g8);
        if (threadIdx.x < g8 * nq) {
            const int r0 = (threadIdx.x % g8) * 8, qs = threadIdx.x / g8;
            int em[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll 4
            for (int q = qs; q < k; q += nq) {
                const int off = kshift ? kshift[q] : 0;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (r0 + c < rows) em[c] = max(em[c], biased_exp(x[(size_t)q * ld + r0 + c], off));
            }
#pragma unroll
            for (int c = 0; c < 8; ++c)
                if (r0 + c < rows) part[qs * rows + r0 + c] = em[c];
        }
        __syncthreads();
        for (int r = threadIdx.x; r < rows; r += kNT) {
            int emax = 0;
            for (int qs = 0; qs < nq; ++qs) emax = max(emax, part[qs * rows + r]);
            scratch[r] = emax;
        }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < rows; r += kNT) {
        const int emax = scratch[r];
        exps[r] = (emax == 0x7FF) ? kNonFinite : (emax == 0 ? 0 : emax - 1022);
    }
    __syncthreads();
    // slices: one unit = one row and 8 consecutive k; consecutive threads take consecutive
    // rows, so each slice's 16-byte stores are contiguous within a core matrix
    const int groups = kp / 8;
#pragma unroll 2
    for (int u = threadIdx.x; u < rp * groups; u += kNT) {
        const int r = u % rp, g = u / rp, q0 = g * 8;
        const int e = (r < rows) ? exps[r] : 0;
        // balanced digits without a carry chain: N + kBias (64 in every base-128 digit) has
        // the plain 7-bit fields q_t + 64 (the top field, 8 bits, takes q_0 + 64 in [0, 128])
        constexpr long long kBias = 0x81020408102040ll;
        uint32_t flo[8], fhi[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int q = q0 + c;
            double v = 0.0;
            if (r < rows && q < k) v = trans ? x[(size_t)q * ld + r] : x[(size_t)r * ld + q];
            const int off = (kshift && q < k) ? kshift[q] : 0;
            const unsigned long long mb = (unsigned long long)(fixed55(v, e, off) + kBias);
            flo[c] = (uint32_t)(mb & ((1ull << 28) - 1));   // fields of digits 7 .. 4
            fhi[c] = (uint32_t)(mb >> 28);                  // fields of digits 3 .. 0
        }
        const int rb = r / BLK, rr = r % BLK, s = q0 / kBK;
        __nv_bfloat16* base = dst + ((size_t)(rb * S + s) * kSlices) * (BLK * kBK) + core_offset(rr, q0 % kBK);
#pragma unroll
        for (int t = 0; t < kSlices; ++t) {
            const int sh = kBits * (kSlices / 2 - 1 - (t & 3));
            const uint32_t mask = (t == 0) ? 0xFFu : 0x7Fu;
            uint32_t w[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t a0 = ((t < 4 ? fhi[2 * c] : flo[2 * c]) >> sh) & mask;
                const uint32_t a1 = ((t < 4 ? fhi[2 * c + 1] : flo[2 * c + 1]) >> sh) & mask;
                // field - 64 exactly in float (2^23 magic); at most 7 significant bits, so
                // its bfloat16 is the float's upper half: one byte permute packs two
                const float f0 = __uint_as_float(0x4B000000u | a0) - 8388672.0f;
                const float f1 = __uint_as_float(0x4B000000u | a1) - 8388672.0f;
                w[c] = __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
            }
            *reinterpret_cast<uint4*>(base + (size_t)t * (BLK * kBK)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}



// out[q] = largest biased exponent (zero and non-finite entries excluded) of X(:, q),
// X(r, q) = trans ? x[q ld + r] : x[r ld + q], r < rows, q < k
__device__ inline void k_exponent_max(const double* x, int ld, bool trans, int rows, int k, int* out) {
    for (int q = threadIdx.x; q < k; q += kNT) out[q] = 0;
    __syncthreads();
    if (trans) {
        const int lane = lane_id();
        for (int q = warp_id(); q < k; q += kNW) {
            int emax = 0;
            for (int r = lane; r < rows; r += 32) {
                const int be = biased_exp(x[(size_t)q * ld + r], 0);
                if (be != 0x7FF) emax = max(emax, be);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
            if (lane == 0) out[q] = emax;
        }
    } else {
        const int g8 = (k + 7) / 8;
        for (int u = threadIdx.x; u < rows * g8; u += kNT) {
            const int r = u / g8, q0 = (u % g8) * 8;
#pragma unroll
            for (int c = 0; c < 8; ++c)
                if (q0 + c < k) {
                    const int be = biased_exp(x[(size_t)r * ld + q0 + c], 0);
                    if (be != 0x7FF && be != 0) atomicMax(&out[q0 + c], be);
                }
        }
    }
    __syncthreads();
}

// Split a constant operand once: as A (TA: A(i, p) = a[p lda + i]) when as_a, else as B
// (TB: B(p, j) = b[j ldb + p]), of an (m x k) / (k x n) product; `slices` holds
// kSlices rows_pad(rows, kBM or kBN) kpad(k) bf16 and `exps` rows ints.  `scratch` is shared
// memory of at least rows ints.  Ends with the fences the bulk copies need.
__device__ inline void presplit(const double* x, int ld, bool as_a, bool transposed, int rows, int k,
                                __nv_bfloat16* slices, int* exps, int* scratch) {
    if (as_a) split_tiles<kBM>(x, ld, transposed, rows, k, exps, slices, scratch);
    else split_tiles<kBN>(x, ld, !transposed, rows, k, exps, slices, scratch);
    asm volatile("fence.proxy.async;\n" ::: "memory");
    __syncthreads();
}

// ---- tensor-core issue -------------------------------------------------------------------

// shared-memory matrix descriptor: K-major, no swizzle, LBO = 128 B (next core matrix in k),
// SBO = 256 B (next 8 rows), descriptor version 1
__device__ __forceinline__ unsigned long long smem_desc(uint32_t addr) {
    return (unsigned long long)((addr & 0x3FFFF) >> 4) | ((unsigned long long)(128 >> 4) << 16) |
           ((unsigned long long)(256 >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D F32, A and B BF16, both K-major, M = 128, N = nn
// (a multiple of 16 up to 256)
__host__ __device__ constexpr uint32_t idesc(int nn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nn >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, unsigned long long a, unsigned long long b,
                                    uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// 8 consecutive TMEM columns of this thread's lane (no wait)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// The epilogue stays off the float64 pipe (a few operations per clock per SM on this part:
// the hardware int64 -> float64 conversion runs there and made the drain ~10 % slower) and
// keeps its integer work short and branch-free.

// t * 2^s as float64, t != 0, |t| < 2^63: t rounded to 53 significant bits half away from
// zero (the 12 bits below t were already dropped, so ties carry no meaning), then scaled.
__device__ __forceinline__ double scaled_double(long long t, int s) {
    const unsigned long long sign = (unsigned long long)t & (1ull << 63);
    const unsigned long long a = t < 0 ? (unsigned long long)(-t) : (unsigned long long)t;
    const int nb = 64 - __clzll((long long)a);              // bit length, 1 .. 63
    const int shr = max(nb - 53, 0), shl = max(53 - nb, 0);
    const unsigned long long mant = ((a + ((1ull << shr) >> 1)) >> shr) << shl;
    const int be = nb - 1 + 1023 + s;
    if (be > 0 && be < 0x7FF - 1)
        // a rounding carry to 2^53 moves into the exponent field
        return __longlong_as_double((long long)(sign | (((unsigned long long)be << 52) + (mant - (1ull << 52)))));
    // subnormal or overflowing result: assemble at unit scale and let ldexp round
    const double unit = __longlong_as_double((long long)(sign | (((unsigned long long)(nb - 1 + 1023) << 52) +
                                                                  (mant - (1ull << 52)))));
    return ldexp(unit, s);
}

// The same conversion without branches for the result of one output: t * 2^s when it is a
// normal float64 (or 0 for t == 0); `special` is set when it is subnormal or overflows, to be
// redone with scaled_double.  Every operation is a select, so eight outputs interleave.
__device__ __forceinline__ double scaled_double_normal(long long t, int s, bool& special) {
    const unsigned long long sign = (unsigned long long)t & (1ull << 63);
    const unsigned long long a = t < 0 ? (unsigned long long)(-t) : (unsigned long long)t;
    const int nb = 64 - __clzll((long long)a);              // bit length, 0 .. 63
    const int shr = max(nb - 53, 0), shl = max(53 - nb, 0);
    const unsigned long long mant = ((a + ((1ull << shr) >> 1)) >> shr) << shl;
    const int be = nb - 1 + 1023 + s;
    special = (a != 0) && !(be > 0 && be < 0x7FF - 1);
    const long long bits = (long long)(sign | (((unsigned long long)be << 52) + (mant - (1ull << 52))));
    return a == 0 ? 0.0 : __longlong_as_double(bits);
}

// ---- the product -------------------------------------------------------------------------

// The fixed-point sums of 8 outputs of one row from their 8 diagonal accumulators r[d][x]
// (exact FP32 integers): T = sum_d D_d 2^(7 (7 - d)) / 2^12.  D_d sums d + 1 digit pairs of
// |q| <= 64 over the chunk's k, so |D_d| <= (d + 1) k 2^12: the first MAGIC diagonals are
// below 2^22 and convert by the 1.5 2^23 magic number on the FMA / ALU pipes, the others by
// F2I on the XU pipe.  Digit pairs combine in int32 (128 D + D' < 2^31 for k <= 256), then
// two int64 halves (each < 2^45); the 12 dropped low bits are 2^-60 of the largest sum.
// Straight-line code over the 8 outputs: their dependency chains interleave.
template <int MAGIC>
__device__ __forceinline__ void fixed_sums(const uint32_t (&r)[kSlices][8], long long (&tt)[8]) {
#pragma unroll
    for (int x = 0; x < 8; ++x) {
        int q[kSlices];
#pragma unroll
        for (int d = 0; d < kSlices; ++d)
            q[d] = d < MAGIC ? __float_as_int(__uint_as_float(r[d][x]) + 12582912.0f) - 0x4B400000
                             : __float2int_rn(__uint_as_float(r[d][x]));
        const int p0 = q[0] * (1 << kBits) + q[1];
        const int p1 = q[2] * (1 << kBits) + q[3];
        const int p2 = q[4] * (1 << kBits) + q[5];
        const int p3 = q[6] * (1 << kBits) + q[7];
        const long long hi = (long long)p0 * (1 << (2 * kBits)) + p1;
        const long long lo = (long long)p2 * (1 << (2 * kBits)) + p3;
        tt[x] = hi * (1ll << (kBits * kSlices / 2 - 12)) + ((lo + kLowRound) >> 12);
    }
}

// The drain of one unit by one epilogue warp: its 32 rows (this lane: row gi) of the 128 x 32
// tile whose accumulators start at TMEM address `acc` (lane quadrant included), 8 columns at a
// time: all 8 diagonals read before one wait, combined in int32 / int64, converted to float64
// with integer operations (t 2^s, t rounded to 53 bits half away from zero) and written to C.
// Each step is branch-free over the 8 outputs (the rare subnormal / overflowing results are
// redone after one test of the group), so that the single warp of each SM sub-partition has
// 8 independent chains to issue from.  Out of line: its many live registers stay out of the
// kernels that call the product inline.
static __device__ __noinline__ void drain_tile(double* c, int ldc, int m, int n, int gi, int j0, int c0,
                                               int cs, const int* ea, const int* eb, GemmOpt<double> opt,
                                               uint32_t acc) {
    const int lane = lane_id();
    const bool row_ok = gi < m;
    const bool read_c = opt.subtract || c0 > 0;
    const int ei = row_ok ? ea[gi] : 0;
    const double rsv = (row_ok && opt.rs) ? opt.rs[gi] : 1.0;
    // the tile's 32 column exponents (and column scales): one per lane, broadcast by shuffles
    const int jl = min(j0 + lane, n - 1);
    const int ej_lane = eb[jl];
    const double cs_lane = opt.cs ? opt.cs[jl] : 1.0;
    const int sbase = ei - 2 * kWidth + kBits * (kSlices - 1) + 12;
    const bool all_magic = cs * kBK <= kMaxK / 2;       // (7 + 1) k 2^12 <= 2^22
    static_assert(kMaxK <= 256, "int32 digit pairs and 4 magic-number diagonals assume k <= 256");
    double* const crow0 = c + (size_t)gi * ldc + j0;
    const bool vec = (((uintptr_t)crow0 & 15) == 0) && (ldc % 2 == 0);
#pragma unroll 1
    for (int grp = 0; grp < kBN / 8; ++grp) {
        const int jc = j0 + 8 * grp;
        if (jc >= n) break;   // uniform: columns beyond C (the rows differ per lane)
        uint32_t r[kSlices][8];
#pragma unroll
        for (int d = 0; d < kSlices; ++d) tmem_ld8(acc + (uint32_t)(d * kBN + 8 * grp), r[d]);
        double* crow = c + (size_t)gi * ldc + jc;
        const bool full8 = jc + 8 <= n;
        double old[8];
#pragma unroll
        for (int x = 0; x < 8; ++x) old[x] = 0.0;
        if (read_c && row_ok) {
            if (vec && full8) {
#pragma unroll
                for (int x = 0; x < 8; x += 2) {
                    const double2 v = *reinterpret_cast<const double2*>(crow + x);
                    old[x] = v.x;
                    old[x + 1] = v.y;
                }
            } else {
#pragma unroll
                for (int x = 0; x < 8; ++x) old[x] = (jc + x < n) ? crow[x] : 0.0;
            }
        }
        int sx[8];
#pragma unroll
        for (int x = 0; x < 8; ++x) sx[x] = __shfl_sync(0xffffffffu, ej_lane, 8 * grp + x);
        tmem_wait();
        long long tt[8];
        if (all_magic) fixed_sums<kSlices>(r, tt);
        else fixed_sums<kSlices / 2>(r, tt);
        double v[8];
        unsigned special = 0, nonfinite = 0;
#pragma unroll
        for (int x = 0; x < 8; ++x) {
            bool sp;
            v[x] = scaled_double_normal(tt[x], sbase + sx[x], sp);
            special |= (unsigned)sp << x;
            nonfinite |= (unsigned)(sx[x] == kNonFinite) << x;
        }
        if (ei == kNonFinite) nonfinite = 0xFFu;
        if (special | nonfinite) {   // rare: subnormal or overflowing results, NaN rows / columns
#pragma unroll 1
            for (int x = 0; x < 8; ++x) {
                if ((special >> x) & 1u) v[x] = scaled_double(tt[x], sbase + sx[x]);
                if ((nonfinite >> x) & 1u) v[x] = __longlong_as_double(0x7FF8000000000000ll);
            }
        }
        if (opt.rs) {
#pragma unroll
            for (int x = 0; x < 8; ++x) v[x] *= rsv;
        }
        if (opt.cs) {
#pragma unroll
            for (int x = 0; x < 8; ++x) v[x] *= __shfl_sync(0xffffffffu, cs_lane, 8 * grp + x);
        }
        if (opt.subtract) {
#pragma unroll
            for (int x = 0; x < 8; ++x) v[x] = old[x] - v[x];
        } else if (c0 > 0) {
#pragma unroll
            for (int x = 0; x < 8; ++x) v[x] = old[x] + v[x];
        }
        if (!row_ok) continue;
        if (vec && full8) {
#pragma unroll
            for (int x = 0; x < 8; x += 2)
                *reinterpret_cast<double2*>(crow + x) = make_double2(v[x], v[x + 1]);
        } else {
#pragma unroll
            for (int x = 0; x < 8; ++x)
                if (jc + x < n) crow[x] = v[x];
        }
    }
}

// C (m x n, ldc) = op(A) op(B) with float64 accuracy; epilogue as blk::tile_gemm (row /
// column scale, subtract).  A(i, p) = TA ? a[p lda + i] : a[i lda + p];
// B(p, j) = TB ? b[j ldb + p] : b[p ldb + j].
// pa / pb: op(A) / op(B) already split (same m, n, k); a / b are then not read.
// oz_gemm_tc_impl is the body, inlined where the caller asks for it (the most frequent
// products); oz_gemm_tc, below, is one out-of-line copy per (TA, TB) for every other call
// site: inlining all ~20 of them cost minutes of compilation and spilled registers.
template <bool TA, bool TB>
__device__ __forceinline__ void oz_gemm_tc_impl(double* c, int ldc, const double* a, int lda,
                                                const double* b, int ldb, int m, int n, int k,
                                                const Workspace ws, GemmOpt<double> opt,
                                                const Presplit* pa, const Presplit* pb) {
    Tc* tc = ws.tc;
    unsigned char* const stage = as_shared(ws.stage);
    // callers may have just written A or B; order earlier generic shared-memory use of the
    // stage before the asynchronous copies into it
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tc->fail || m <= 0 || n <= 0) return;
    if (k <= 0) {
        // empty sum: C = 0, or C unchanged when subtracting
        if (!opt.subtract)
            for (int e = threadIdx.x; e < m * n; e += kNT) c[(size_t)(e / n) * ldc + e % n] = 0.0;
        __syncthreads();
        return;
    }
    const int kp = kpad(k), S = kp / kBK;
    const __nv_bfloat16* sa = pa ? pa->slices : ws.slices;
    const __nv_bfloat16* sb = pb ? pb->slices : ws.slices + (size_t)kSlices * rows_pad(m, kBM) * kp;
    const int* ea = pa ? pa->exps : ws.ea;
    const int* eb = pb ? pb->exps : ws.eb;
    const long long t0 = clock64();
    int* scratch = reinterpret_cast<int*>(stage);   // the stage is idle while splitting
    const int* ksa = nullptr;
    const int* ksb = nullptr;
    if (opt.kscale && !pa && !pb && k <= kMaxKscale) {
        // equilibrate along k: A(:, p) 2^s_p and B(p, :) 2^-s_p (exact, the product is
        // unchanged) with s_p bringing column p of A to [1/2, 1), so that a grading of A's
        // columns mirrored in B's rows costs no relative accuracy
        int* ca = scratch + kScratchKA;
        int* cb = scratch + kScratchKB;
        k_exponent_max(a, lda, TA, m, k, ca);
        k_exponent_max(b, ldb, !TB, n, k, cb);
        for (int p = threadIdx.x; p < k; p += kNT) {
            int sft = 0;
            if (ca[p] > 0 && ca[p] < 0x7FF) {
                sft = 1022 - ca[p];
                if (cb[p] > 0 && (cb[p] - sft >= 0x7FF - 8 || cb[p] - sft <= 8)) sft = 0;
            }
            ca[p] = sft;
            cb[p] = -sft;
        }
        __syncthreads();
        ksa = ca;
        ksb = cb;
    }
    if (!pa) split_tiles<kBM>(a, lda, TA, m, k, ws.ea, ws.slices, scratch, ksa);
    if (!pb) split_tiles<kBN>(b, ldb, !TB, n, k, ws.eb, ws.slices + (size_t)kSlices * rows_pad(m, kBM) * kp,
                              scratch, ksb);
    // the slices were written through the generic proxy and are read by bulk copies; the
    // stage served as scratch and is next written by bulk copies
    asm volatile("fence.proxy.async;\n" ::: "memory");
    __syncthreads();
    const long long t1 = clock64();
    if (ws.cycles && threadIdx.x == 0) ws.cycles[0] += t1 - t0;

    // ---- the pipeline: units = (output tile, k chunk of kMaxK), tiles column-major -------
    const int stages = ws.stages;
    const uint32_t tmem = tc->tmem;
    const int tiles_m = rows_pad(m, kBM) / kBM, tiles_n = rows_pad(n, kBN) / kBN;
    const int chunk_steps = kMaxK / kBK, n_chunks = (S + chunk_steps - 1) / chunk_steps;
    const int n_units = tiles_m * tiles_n * n_chunks;
    const uint32_t step0 = tc->steps, unit0 = tc->units;
    const int w = warp_id(), lane = lane_id();
    volatile int* fail = &tc->fail;
    // unit u: tile (tm, tn), chunk steps [c0, c0 + cs)
    // (row-block-major order and an L2 evict_last hint on A's slices were measured at 16x16,
    // 64 chains: no gain, +1.5 % with the hint)
    auto unit_of = [&](int u, int& tm, int& tn, int& c0, int& cs) {
        const int tile = u / n_chunks, ch = u % n_chunks;
        tm = tile % tiles_m;
        tn = tile / tiles_m;
        c0 = ch * chunk_steps;
        cs = min(chunk_steps, S - c0);
    };
    constexpr uint32_t kStageBytes = (kStepA + kStepB) * 2;
    if (w == 1 && lane == 0) {
        // producer: one k step of A (all slices of a 128-row block) and of B (of a 32-column
        // block) per stage, two bulk copies completing on the stage's `full` barrier
        uint32_t g = step0;
        bool stall = tc->stall != 0;
        tc->stall = 0;
        for (int u = 0; u < n_units && !*fail; ++u) {
            int tm, tn, c0, cs;
            unit_of(u, tm, tn, c0, cs);
            for (int s = 0; s < cs; ++s, ++g) {
                const int i = g % stages;
                const uint32_t use = g / stages;
                if (use >= 1 && !bar_wait(&tc->empty[i], (use - 1) & 1, fail)) { *fail = 1; break; }
                if (stall) { stall = false; continue; }   // test hook: this stage never fills
                unsigned char* st = stage + (size_t)i * kStageBytes;
                expect_tx(&tc->full[i], kStageBytes);
                bulk_load(st, sa + (size_t)(tm * S + c0 + s) * kStepA, kStepA * 2, &tc->full[i]);
                bulk_load(st + kStepA * 2, sb + (size_t)(tn * S + c0 + s) * kStepB, kStepB * 2, &tc->full[i]);
            }
        }
        if (*fail) {
            // no copy may still be landing when the CTA moves on: wait (bounded) for the
            // last `stages` steps this thread issued
            for (uint32_t q = (g > step0 + stages ? g - stages : step0); q < g; ++q)
                bar_wait(&tc->full[q % stages], (q / stages) & 1);
        }
    } else if (w == 0 && lane == 0) {
        // MMA issue: per k step A_t times the stacked B_0 .. B_{7-t} (diagonals t .. 7 are the
        // contiguous columns [32 t, 256) of the unit's accumulator buffer), one MMA per t
        uint32_t g = step0;
        for (int u = 0; u < n_units && !*fail; ++u) {
            int tm, tn, c0, cs;
            unit_of(u, tm, tn, c0, cs);
            const uint32_t U = unit0 + u, b = U & 1, ub = U >> 1;
            if (ub >= 1 && !bar_wait(&tc->acc_empty[b], (ub - 1) & 1, fail)) { *fail = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t acc = tmem + b * kAccCols;
            bool ok = true;
            for (int s = 0; s < cs; ++s, ++g) {
                const int i = g % stages;
                if (!bar_wait(&tc->full[i], (g / stages) & 1, fail)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t st = smem_u32(stage + (size_t)i * kStageBytes);
#pragma unroll
                for (int t = 0; t < kSlices; ++t)
                    mma(acc + (uint32_t)(t * kBN), smem_desc(st + t * kTileA * 2), smem_desc(st + kStepA * 2),
                        idesc((kSlices - t) * kBN), (s > 0 || t > 0) ? 1u : 0u);
                commit(&tc->empty[i]);
            }
            if (!ok) { *fail = 1; break; }
            commit(&tc->acc_full[b]);
        }
    } else if (w >= kEpiWarp0) {
        // epilogue: warp w drains TMEM lanes 32 (w % 4) .. of the unit's buffer (its 32 rows of
        // the tile), 8 columns at a time: all 8 diagonals read before one wait, combined in
        // int64, converted to float64 with integer operations and written straight to C
        const int quad = w & 3;
        long long epi_cycles = 0;
        for (int u = 0; u < n_units; ++u) {
            int tm, tn, c0, cs;
            unit_of(u, tm, tn, c0, cs);
            const uint32_t U = unit0 + u, b = U & 1, ub = U >> 1;
            const int i0 = tm * kBM, j0 = tn * kBN;
            const int gi = i0 + 32 * quad + lane;          // this thread's row of C
            const bool row_ok = gi < m;
            const bool read_c = opt.subtract || c0 > 0;
            if (read_c && row_ok) {   // the row's old values, requested into L2 while the MMAs run
                asm volatile("prefetch.L2 [%0];\n" :: "l"(c + (size_t)gi * ldc + j0));
                if (j0 + 16 < n) asm volatile("prefetch.L2 [%0];\n" :: "l"(c + (size_t)gi * ldc + j0 + 16));
            }
            // every lane waits; the outcome is made uniform over the warp before the collective
            // TMEM loads
            const bool bad = __any_sync(0xffffffffu, !bar_wait(&tc->acc_full[b], ub & 1, fail));
            if (bad) {
                if (lane == 0) *fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const long long te = clock64();
            drain_tile(c, ldc, m, n, gi, j0, c0, cs, ea, eb, opt,
                       tmem + ((uint32_t)(32 * quad) << 16) + b * kAccCols);
            // every lane has read its accumulators before the buffer is handed back
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) bar_arrive(&tc->acc_empty[b]);
            epi_cycles += clock64() - te;
        }
        if (ws.cycles && w == kEpiWarp0 && lane == 0) ws.cycles[2] += epi_cycles;
    }
    // every role is done: C is written, the MMAs have completed (each unit's epilogue waited
    // for its commit), the copies have landed
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (threadIdx.x == 0) {
        uint32_t steps = 0;
        for (int u = 0; u < n_units; ++u) {
            int tm, tn, c0, cs;
            unit_of(u, tm, tn, c0, cs);
            steps += cs;
        }
        tc->steps = step0 + steps;
        tc->units = unit0 + n_units;
        if (ws.cycles) ws.cycles[1] += clock64() - t1;
    }
    __syncthreads();
}

template <bool TA, bool TB>
__device__ __noinline__ void oz_gemm_tc(double* c, int ldc, const double* a, int lda, const double* b,
                                        int ldb, int m, int n, int k, const Workspace ws,
                                        GemmOpt<double> opt = GemmOpt<double>(),
                                        const Presplit* pa = nullptr, const Presplit* pb = nullptr) {
    oz_gemm_tc_impl<TA, TB>(c, ldc, a, lda, b, ldb, m, n, k, ws, opt, pa, pb);
}

}  // namespace ozt
}  // namespace lqmc
