// Block-cooperative tiled GEMM for one CTA of blk::kNT (256) threads.
//
// C (m x n) = op(A) (m x k) * op(B) (k x n), row-major, generic pointers (global or shared
// memory).  64 x 64 output tiles, 4 x 4 outputs per thread, k staged through shared memory
// 16 at a time.  Every output is one fma chain in increasing k starting from zero, so the
// result is independent of the tiling.  Inputs of another type (float / double) are
// converted when they are staged.  Epilogue options: scale rows (rs) and columns (cs) of
// the product, and subtract the product from C instead of overwriting it.
#pragma once
#include <cuda_runtime.h>

#include "block_fp64.cuh"

namespace lqmc {
namespace blk {

constexpr int kTile = 64;
constexpr int kTileK = 16;

// shared-memory bytes tile_gemm<T> needs for its staging buffers
template <typename T>
constexpr size_t tile_gemm_smem() {
    return (size_t)2 * kTileK * (kTile + 1) * sizeof(T);
}

template <typename T>
struct GemmOpt {
    const T* rs = nullptr;        // multiply row i of the product by rs[i]
    const T* cs = nullptr;        // multiply column j of the product by cs[j]
    bool subtract = false;        // C -= product (else C = product)
};

// A(i, p) = TA ? a[p * lda + i] : a[i * lda + p];  B(p, j) = TB ? b[j * ldb + p] : b[p * ldb + j]
template <typename T, bool TA, bool TB, typename TAIn, typename TBIn>
__device__ void tile_gemm(T* __restrict__ c, int ldc, const TAIn* a, int lda, const TBIn* b,
                          int ldb, int m, int n, int k, T* stage, GemmOpt<T> opt = GemmOpt<T>()) {
    T* as = stage;                              // [kTileK][kTile + 1], as[p][i] = A(i0 + i, p0 + p)
    T* bs = stage + kTileK * (kTile + 1);       // [kTileK][kTile + 1], bs[p][j] = B(p0 + p, j0 + j)
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int tiles_m = (m + kTile - 1) / kTile, tiles_n = (n + kTile - 1) / kTile;
    for (int tile = 0; tile < tiles_m * tiles_n; ++tile) {
        const int i0 = (tile / tiles_n) * kTile, j0 = (tile % tiles_n) * kTile;
        T acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int s = 0; s < 4; ++s) acc[r][s] = T(0);
        for (int p0 = 0; p0 < k; p0 += kTileK) {
            __syncthreads();
            for (int e = threadIdx.x; e < kTileK * kTile; e += kNT) {
                // A tile: element (i, p); consecutive threads walk the contiguous index
                int i, p;
                if (TA) { p = e / kTile; i = e % kTile; } else { i = e / kTileK; p = e % kTileK; }
                const int gi = i0 + i, gp = p0 + p;
                T va = T(0);
                if (gi < m && gp < k) va = (T)(TA ? a[(size_t)gp * lda + gi] : a[(size_t)gi * lda + gp]);
                as[p * (kTile + 1) + i] = va;
                int q, j;
                if (TB) { j = e / kTileK; q = e % kTileK; } else { q = e / kTile; j = e % kTile; }
                const int gq = p0 + q, gj = j0 + j;
                T vb = T(0);
                if (gq < k && gj < n) vb = (T)(TB ? b[(size_t)gj * ldb + gq] : b[(size_t)gq * ldb + gj]);
                bs[q * (kTile + 1) + j] = vb;
            }
            __syncthreads();
            const int pk = min(kTileK, k - p0);
            for (int p = 0; p < pk; ++p) {
                T av[4], bv[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) av[r] = as[p * (kTile + 1) + ty + 16 * r];
#pragma unroll
                for (int s = 0; s < 4; ++s) bv[s] = bs[p * (kTile + 1) + tx + 16 * s];
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int s = 0; s < 4; ++s) acc[r][s] = fma(av[r], bv[s], acc[r][s]);
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int gi = i0 + ty + 16 * r;
            if (gi >= m) continue;
#pragma unroll
            for (int s = 0; s < 4; ++s) {
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
