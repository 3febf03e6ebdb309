// Block-cooperative tiled GEMM for one CTA of blk::kNT (256) threads.
//
// C (m x n) = op(A) (m x k) * op(B) (k x n), row-major, generic pointers (global or shared
// memory).  Square output tiles (128 in float, 64 in double) with 8 x 8 / 4 x 4 outputs per
// thread, k staged through shared memory 16 at a time.  Every output is one fma chain in increasing k starting from zero, so the
// result is independent of the tiling.  Inputs of another type (float / double) are
// converted when they are staged.  Epilogue options: scale rows (rs) and columns (cs) of
// the product, and subtract the product from C instead of overwriting it.  The call begins
// and ends with a block barrier, so operands written just before it are seen.
#pragma once
#include <cuda_runtime.h>

#include "block_fp64.cuh"

namespace lqmc {
namespace blk {

constexpr int kTileK = 16;

// p, a generic pointer into the kernel's dynamic shared memory, re-derived from that array so
// that accesses through it in a function that is not inlined compile to shared-memory
// instructions (the compiler cannot otherwise tell where a pointer argument points)
template <typename T>
__device__ __forceinline__ T* as_shared(T* p) {
    extern __shared__ __align__(16) unsigned char lqmc_dyn_smem[];
    const int off = (int)((unsigned)__cvta_generic_to_shared(p) -
                          (unsigned)__cvta_generic_to_shared(lqmc_dyn_smem));
    return reinterpret_cast<T*>(lqmc_dyn_smem + off);
}

// outputs per thread along each axis: 8 x 8 in float (128 x 128 tiles, 4 FMAs per shared
// load), 4 x 4 in double (64 x 64 tiles; the float64 pipe is the limit there)
template <typename T>
constexpr int tile_r() { return sizeof(T) == 4 ? 8 : 4; }
template <typename T>
constexpr int tile_dim() { return 16 * tile_r<T>(); }

// shared-memory bytes tile_gemm<T> needs for its staging buffers
template <typename T>
constexpr size_t tile_gemm_smem() {
    return (size_t)2 * kTileK * (tile_dim<T>() + 1) * sizeof(T);
}

template <typename T>
struct GemmOpt {
    const T* rs = nullptr;        // multiply row i of the product by rs[i]
    const T* cs = nullptr;        // multiply column j of the product by cs[j]
    bool subtract = false;        // C -= product (else C = product)
    bool kscale = false;          // emulated GEMM: equilibrate along k (ignored by tile_gemm)
};

// A(i, p) = TA ? a[p * lda + i] : a[i * lda + p];  B(p, j) = TB ? b[j * ldb + p] : b[p * ldb + j]
// Not inlined, like the emulated GEMM: one copy per (T, TA, TB) keeps the sweep kernel small.
template <typename T, bool TA, bool TB, typename TAIn, typename TBIn>
__device__ __noinline__ void tile_gemm(T* __restrict__ c, int ldc, const TAIn* a, int lda, const TBIn* b,
                                       int ldb, int m, int n, int k, T* stage, GemmOpt<T> opt = GemmOpt<T>()) {
    constexpr int R = tile_r<T>();
    constexpr int D = tile_dim<T>();
    stage = as_shared(stage);   // the staging buffer lies in dynamic shared memory
    T* as = stage;                         // [kTileK][D + 1], as[p][i] = A(i0 + i, p0 + p)
    T* bs = stage + kTileK * (D + 1);      // [kTileK][D + 1], bs[p][j] = B(p0 + p, j0 + j)
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int tiles_m = (m + D - 1) / D, tiles_n = (n + D - 1) / D;
    __syncthreads();   // callers may have just written A or B without a barrier
    for (int tile = 0; tile < tiles_m * tiles_n; ++tile) {
        const int i0 = (tile / tiles_n) * D, j0 = (tile % tiles_n) * D;
        T acc[R][R];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int s = 0; s < R; ++s) acc[r][s] = T(0);
        for (int p0 = 0; p0 < k; p0 += kTileK) {
            // load the step's elements as one batch of independent loads, then store them
            constexpr int kPerThread = kTileK * D / kNT;
            static_assert(kTileK * D % kNT == 0, "staging must divide evenly over the block");
            T va[kPerThread], vb[kPerThread];
#pragma unroll
            for (int r = 0; r < kPerThread; ++r) {
                const int e = threadIdx.x + r * kNT;
                // consecutive threads walk the contiguous index of each operand
                int i, p;
                if (TA) { p = e / D; i = e % D; } else { i = e / kTileK; p = e % kTileK; }
                const int gi = i0 + i, gp = p0 + p;
                va[r] = (gi < m && gp < k) ? (T)(TA ? a[(size_t)gp * lda + gi] : a[(size_t)gi * lda + gp]) : T(0);
                int q, j;
                if (TB) { j = e / kTileK; q = e % kTileK; } else { q = e / D; j = e % D; }
                const int gq = p0 + q, gj = j0 + j;
                vb[r] = (gq < k && gj < n) ? (T)(TB ? b[(size_t)gj * ldb + gq] : b[(size_t)gq * ldb + gj]) : T(0);
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kPerThread; ++r) {
                const int e = threadIdx.x + r * kNT;
                int i, p;
                if (TA) { p = e / D; i = e % D; } else { i = e / kTileK; p = e % kTileK; }
                as[p * (D + 1) + i] = va[r];
                int q, j;
                if (TB) { j = e / kTileK; q = e % kTileK; } else { q = e / D; j = e % D; }
                bs[q * (D + 1) + j] = vb[r];
            }
            __syncthreads();
            const int pk = min(kTileK, k - p0);
            for (int p = 0; p < pk; ++p) {
                T av[R], bv[R];
#pragma unroll
                for (int r = 0; r < R; ++r) av[r] = as[p * (D + 1) + ty + 16 * r];
#pragma unroll
                for (int s = 0; s < R; ++s) bv[s] = bs[p * (D + 1) + tx + 16 * s];
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int s = 0; s < R; ++s) acc[r][s] = fma(av[r], bv[s], acc[r][s]);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int gi = i0 + ty + 16 * r;
            if (gi >= m) continue;
#pragma unroll
            for (int s = 0; s < R; ++s) {
                const int gj = j0 + tx + 16 * s;
                if (gj >= n) continue;
                T v = acc[r][s];
                if (opt.rs) v = opt.rs[gi] * v;
                if (opt.cs) v = v * opt.cs[gj];
                T* dst = c + (size_t)gi * ldc + gj;
                *dst = opt.subtract ? *dst - v : v;
            }
        }
    }
    __syncthreads();
}

}  // namespace blk
}  // namespace lqmc
