// Float64-accurate GEMM on the BF16 tensor cores for one CTA of blk::kNT threads.
//
// Ozaki-style splitting: every row i of op(A) is scaled by 2^-E_i (E_i = exponent just
// above its largest entry) and written as a 48-bit fixed-point integer
// F = trunc(|a| 2^(48 - E_i)), cut into kSlices = 8 slices of 6 bits (q_t in [-63, 63],
// exact in bfloat16).  Columns of op(B) likewise with 2^-F_j.  Then
//     C_ij = 2^(E_i + F_j - 54) sum_{d=0..7} 2^(6 (7 - d)) D_d,   D_d = sum_{t+u=d} (A_t B_u)_ij
// keeping the 36 leading slice pairs.  Each (A_t B_u) is a BF16 x BF16 -> FP32
// mma.sync.m16n8k16; the pairs of one diagonal d share an FP32 accumulator, which holds
// exact integers: over kChunk = 128 values of k, |D_d| <= 8 * 128 * 63^2 < 2^22.  Every
// chunk the eight sums are moved, exactly, into two int64 accumulators
//     H += sum_{d<4} D_d 2^(6 (3 - d)),   Lo += sum_{d>=4} D_d 2^(6 (7 - d))
// and the output is formed once as (double)H 2^24 + (double)Lo.  So the only roundings are
// the truncation of the operands at 2^-48 of their row / column maximum and that one final
// float64 addition; the float64 pipe sees three operations per output element.
// Splitting, the float32 -> int64 moves and the power-of-two scaling are integer / float32
// bit operations.
//
// A row (column) holding a NaN or Inf produces NaN in its output row (column).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "block_fp64.cuh"
#include "block_gemm.cuh"

namespace lqmc {
namespace ozk {

using namespace blk;

constexpr int kSlices = 8;
constexpr int kBits = 6;
constexpr int kWidth = kSlices * kBits;   // fixed-point bits of an operand
constexpr int kChunk = 128;               // k per exact float32 accumulation
constexpr int kTM = 64, kTN = 32, kTK = 16;
constexpr int kAPad = kTK + 8;            // bf16 row stride of the staged tiles
constexpr int kNonFinite = 1 << 20;       // exponent sentinel of a row with NaN / Inf

// bytes of shared-memory staging oz_gemm needs
constexpr size_t stage_bytes() {
    return (size_t)kSlices * (kTM + kTN) * kAPad * sizeof(__nv_bfloat16);
}

// rounded-up k stride of the slice buffers
__host__ __device__ constexpr int kpad(int k) { return (k + 15) / 16 * 16; }

// bf16 elements of the slice buffers for an (m x k) times (k x n) product
__host__ __device__ constexpr size_t slice_elems(int m, int n, int k) {
    return (size_t)kSlices * ((size_t)m + n) * kpad(k);
}

__device__ __forceinline__ int biased_exp(double v) {
    return (int)((__double_as_longlong(v) >> 52) & 0x7FF);
}

// bfloat16 bits of the small integer q (|q| < 2^8): float(q) by the 2^23 magic number,
// whose low 16 bits are zero for such q, then its top half; the sign is set separately.
__device__ __forceinline__ unsigned short bf16_of_small_int(int q, bool neg) {
    const float f = __int_as_float(0x4B000000 | q) - 8388608.0f;
    return (unsigned short)((__float_as_uint(f) >> 16) | (neg ? 0x8000u : 0u));
}

// q_t of one value for row / column exponent e (|v| < 2^e), all slices at once
__device__ __forceinline__ void split_value(double v, int e, __nv_bfloat16* out, size_t stride) {
    const long long bits = __double_as_longlong(v);
    const int be = (int)((bits >> 52) & 0x7FF);
    unsigned long long f = 0;
    if (be != 0 && be != 0x7FF && e != kNonFinite) {
        const unsigned long long mant = ((unsigned long long)bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        const int sh = (be - 1075) + kWidth - e;
        if (sh >= 0) f = (sh < 11) ? (mant << sh) : 0;           // cannot happen when |v| < 2^e
        else f = (-sh < 64) ? (mant >> (-sh)) : 0;
    }
    const bool neg = bits < 0;
    unsigned short* o = reinterpret_cast<unsigned short*>(out);
#pragma unroll
    for (int t = 0; t < kSlices; ++t) {
        const int q = (int)((f >> (kBits * (kSlices - 1 - t))) & ((1u << kBits) - 1));
        o[(size_t)t * stride] = bf16_of_small_int(q, neg);
    }
}

// integer value of an integer-valued float |x| < 2^22 (the 1.5 * 2^23 magic number)
__device__ __forceinline__ long long int_of_float(float x) {
    return (long long)(__float_as_int(x + 12582912.0f) - 0x4B400000);
}

// v * 2^s by exponent arithmetic when the result stays a normal number, else ldexp
__device__ __forceinline__ double scale_pow2(double v, int s) {
    const long long b = __double_as_longlong(v);
    const int be = (int)((b >> 52) & 0x7FF);
    if (be == 0 || be == 0x7FF) return v == 0.0 ? v : ldexp(v, s);
    const int ne = be + s;
    if (ne <= 0 || ne >= 0x7FF) return ldexp(v, s);
    return __longlong_as_double(b + ((long long)s << 52));
}

// op(A) (m x k): A(i, p) = TA ? a[p lda + i] : a[i lda + p].  Writes slices
// sa[(t m + i) kp + p] and row exponents ea[i].
template <bool TA>
__device__ void split_rows(const double* a, int lda, int m, int k, __nv_bfloat16* sa, int* ea) {
    const int lane = lane_id(), kp = kpad(k);
    for (int i = warp_id(); i < m; i += kNW) {
        int emax = 0, bad = 0;
        for (int p = lane; p < k; p += 32) {
            const double v = TA ? a[(size_t)p * lda + i] : a[(size_t)i * lda + p];
            const int be = biased_exp(v);
            if (be == 0x7FF) bad = 1;
            emax = max(emax, be);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
            bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        }
        const int e = bad ? kNonFinite : (emax == 0 ? 0 : emax - 1022);
        if (lane == 0) ea[i] = e;
        for (int p = lane; p < kp; p += 32) {
            const double v = (p < k) ? (TA ? a[(size_t)p * lda + i] : a[(size_t)i * lda + p]) : 0.0;
            split_value(v, e, sa + (size_t)i * kp + p, (size_t)m * kp);
        }
    }
}

// op(B) (k x n): B(p, j) = TB ? b[j ldb + p] : b[p ldb + j].  Writes slices
// sb[(t n + j) kp + p] (k contiguous per column) and column exponents eb[j].
template <bool TB>
__device__ void split_cols(const double* b, int ldb, int k, int n, __nv_bfloat16* sb, int* eb) {
    const int lane = lane_id(), kp = kpad(k);
    for (int j = warp_id(); j < n; j += kNW) {
        int emax = 0, bad = 0;
        for (int p = lane; p < k; p += 32) {
            const double v = TB ? b[(size_t)j * ldb + p] : b[(size_t)p * ldb + j];
            const int be = biased_exp(v);
            if (be == 0x7FF) bad = 1;
            emax = max(emax, be);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
            bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        }
        const int e = bad ? kNonFinite : (emax == 0 ? 0 : emax - 1022);
        if (lane == 0) eb[j] = e;
        for (int p = lane; p < kp; p += 32) {
            const double v = (p < k) ? (TB ? b[(size_t)j * ldb + p] : b[(size_t)p * ldb + j]) : 0.0;
            split_value(v, e, sb + (size_t)j * kp + p, (size_t)n * kp);
        }
    }
}

// words (2 bf16) of one k step staged per thread: A part then B part
constexpr int kWordsA = kSlices * kTM * (kTK / 2) / kNT;   // 16
constexpr int kWordsB = kSlices * kTN * (kTK / 2) / kNT;   // 8
static_assert(kSlices * kTM * (kTK / 2) % kNT == 0 && kSlices * kTN * (kTK / 2) % kNT == 0,
              "staging words must divide evenly over the block");

__device__ __forceinline__ void load_step(const __nv_bfloat16* sa, const __nv_bfloat16* sb, int m,
                                          int n, int kp, int i0, int j0, int p0,
                                          uint32_t (&buf)[kWordsA + kWordsB]) {
#pragma unroll
    for (int r = 0; r < kWordsA; ++r) {
        const int w = threadIdx.x + r * kNT;
        const int t = w / (kTM * (kTK / 2)), row = (w / (kTK / 2)) % kTM, q = w % (kTK / 2);
        buf[r] = (i0 + row < m)
                     ? *reinterpret_cast<const uint32_t*>(sa + ((size_t)t * m + i0 + row) * kp + p0 + 2 * q)
                     : 0u;
    }
#pragma unroll
    for (int r = 0; r < kWordsB; ++r) {
        const int w = threadIdx.x + r * kNT;
        const int t = w / (kTN * (kTK / 2)), row = (w / (kTK / 2)) % kTN, q = w % (kTK / 2);
        buf[kWordsA + r] = (j0 + row < n)
                               ? *reinterpret_cast<const uint32_t*>(sb + ((size_t)t * n + j0 + row) * kp + p0 + 2 * q)
                               : 0u;
    }
}

__device__ __forceinline__ void store_step(__nv_bfloat16* as, __nv_bfloat16* bs,
                                           const uint32_t (&buf)[kWordsA + kWordsB]) {
#pragma unroll
    for (int r = 0; r < kWordsA; ++r) {
        const int w = threadIdx.x + r * kNT;
        const int t = w / (kTM * (kTK / 2)), row = (w / (kTK / 2)) % kTM, q = w % (kTK / 2);
        *reinterpret_cast<uint32_t*>(as + ((size_t)t * kTM + row) * kAPad + 2 * q) = buf[r];
    }
#pragma unroll
    for (int r = 0; r < kWordsB; ++r) {
        const int w = threadIdx.x + r * kNT;
        const int t = w / (kTN * (kTK / 2)), row = (w / (kTK / 2)) % kTN, q = w % (kTK / 2);
        *reinterpret_cast<uint32_t*>(bs + ((size_t)t * kTN + row) * kAPad + 2 * q) = buf[kWordsA + r];
    }
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct Workspace {
    __nv_bfloat16* slices;   // slice_elems(m, n, k) bf16
    int* ea;                 // m
    int* eb;                 // n
    unsigned char* stage;    // stage_bytes() of shared memory
    long long* cycles;       // optional [2] clock cycles: splitting, tensor-core loop (thread 0)
};

// C (m x n, ldc) = op(A) op(B) with float64 accuracy (see the header comment); epilogue as
// blk::tile_gemm (row / column scale, subtract).
template <bool TA, bool TB>
__device__ void oz_gemm(double* c, int ldc, const double* a, int lda, const double* b, int ldb,
                        int m, int n, int k, const Workspace& ws, GemmOpt<double> opt = GemmOpt<double>()) {
    const int kp = kpad(k);
    __nv_bfloat16* sa = ws.slices;
    __nv_bfloat16* sb = ws.slices + (size_t)kSlices * m * kp;
    __syncthreads();   // callers may have just written A or B without a barrier
    const long long t0 = clock64();
    split_rows<TA>(a, lda, m, k, sa, ws.ea);
    split_cols<TB>(b, ldb, k, n, sb, ws.eb);
    __syncthreads();
    const long long t1 = clock64();
    if (ws.cycles && threadIdx.x == 0) ws.cycles[0] += t1 - t0;
    __nv_bfloat16* as = reinterpret_cast<__nv_bfloat16*>(ws.stage);       // [t][kTM][kAPad]
    __nv_bfloat16* bs = as + (size_t)kSlices * kTM * kAPad;                // [t][kTN][kAPad]
    const int lane = lane_id(), g = lane >> 2, tig = lane & 3;
    const int wm = warp_id() >> 1, wn = warp_id() & 1;                     // 4 x 2 warps
    const int tiles_m = (m + kTM - 1) / kTM, tiles_n = (n + kTN - 1) / kTN;
    for (int tile = 0; tile < tiles_m * tiles_n; ++tile) {
        const int i0 = (tile / tiles_n) * kTM, j0 = (tile % tiles_n) * kTN;
        long long hi[2][4], lo[2][4];
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) hi[x][y] = lo[x][y] = 0;
        for (int c0 = 0; c0 < kp; c0 += kChunk) {
            float acc[kSlices][2][4];
#pragma unroll
            for (int d = 0; d < kSlices; ++d)
#pragma unroll
                for (int x = 0; x < 2; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) acc[d][x][y] = 0.f;
            const int c1 = min(kp, c0 + kChunk);
            for (int p0 = c0; p0 < c1; p0 += kTK) {
                // the step's slice words: one batch of independent loads, then the stores
                uint32_t buf[kWordsA + kWordsB];
                load_step(sa, sb, m, n, kp, i0, j0, p0, buf);
                __syncthreads();
                store_step(as, bs, buf);
                __syncthreads();
#pragma unroll
                for (int t = 0; t < kSlices; ++t) {
                    const __nv_bfloat16* ar = as + ((size_t)t * kTM + wm * 16) * kAPad;
                    uint32_t af[4];
                    af[0] = *reinterpret_cast<const uint32_t*>(ar + (size_t)g * kAPad + tig * 2);
                    af[1] = *reinterpret_cast<const uint32_t*>(ar + (size_t)(g + 8) * kAPad + tig * 2);
                    af[2] = *reinterpret_cast<const uint32_t*>(ar + (size_t)g * kAPad + tig * 2 + 8);
                    af[3] = *reinterpret_cast<const uint32_t*>(ar + (size_t)(g + 8) * kAPad + tig * 2 + 8);
#pragma unroll
                    for (int u = 0; u < kSlices - t; ++u) {
#pragma unroll
                        for (int x = 0; x < 2; ++x) {
                            const __nv_bfloat16* br = bs + ((size_t)u * kTN + wn * 16 + x * 8 + g) * kAPad;
                            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(br + tig * 2);
                            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(br + tig * 2 + 8);
                            mma_bf16(acc[t + u][x], af, b0, b1);
                        }
                    }
                }
            }
            // move the exact float32 diagonal sums into the int64 accumulators
#pragma unroll
            for (int x = 0; x < 2; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) {
                    long long h = 0, l = 0;
#pragma unroll
                    for (int d = 0; d < kSlices / 2; ++d)
                        h += int_of_float(acc[d][x][y]) << (kBits * (kSlices / 2 - 1 - d));
#pragma unroll
                    for (int d = kSlices / 2; d < kSlices; ++d)
                        l += int_of_float(acc[d][x][y]) << (kBits * (kSlices - 1 - d));
                    hi[x][y] += h;
                    lo[x][y] += l;
                }
        }
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) {
                const int gi = i0 + wm * 16 + g + (y >= 2 ? 8 : 0);
                const int gj = j0 + wn * 16 + x * 8 + tig * 2 + (y & 1);
                if (gi >= m || gj >= n) continue;
                const int ei = ws.ea[gi], ej = ws.eb[gj];
                // total = hi 2^(6 S/2) + lo;  C = total 2^(E_i + F_j - 2W + 6 (S - 1))
                const double total = fma((double)hi[x][y], (double)(1ll << (kBits * (kSlices / 2))),
                                         (double)lo[x][y]);
                double v = (ei == kNonFinite || ej == kNonFinite)
                               ? __longlong_as_double(0x7FF8000000000000ll)
                               : scale_pow2(total, ei + ej - 2 * kWidth + kBits * (kSlices - 1));
                if (opt.rs) v = opt.rs[gi] * v;
                if (opt.cs) v = v * opt.cs[gj];
                double* dst = c + (size_t)gi * ldc + gj;
                *dst = opt.subtract ? *dst - v : v;
            }
    }
    __syncthreads();
    if (ws.cycles && threadIdx.x == 0) ws.cycles[1] += clock64() - t1;
}

}  // namespace ozk
}  // namespace lqmc
