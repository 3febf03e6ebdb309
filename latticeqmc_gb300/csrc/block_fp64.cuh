// Block-cooperative float64 dense kernels for one Markov chain per CTA (n <= 128).
//
// Every routine is called by all kNT threads of the block.  Matrices are n x n row-major
// and may live in shared or global memory (generic pointers); routines that write in place
// keep every output in registers until the inputs it depends on are consumed, so no
// second buffer is needed.  Accumulations are sequential fma chains in index order.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lqmc {
namespace blk {

constexpr int kNT = 256;             // threads per CTA
constexpr int kNW = kNT / 32;        // warps per CTA
constexpr int kMaxRows = 4;          // rows per lane: n <= 128

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_id() { return threadIdx.x >> 5; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum / max; `red` is kNW doubles of shared memory.  Result on every thread.
__device__ __forceinline__ double block_sum(double v, double* red) {
    v = warp_sum(v);
    __syncthreads();
    if (lane_id() == 0) red[warp_id()] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kNW; ++w) t += red[w];
    return t;
}

__device__ __forceinline__ double block_max(double v, double* red) {
    v = warp_max(v);
    __syncthreads();
    if (lane_id() == 0) red[warp_id()] = v;
    __syncthreads();
    double t = red[0];
#pragma unroll
    for (int w = 1; w < kNW; ++w) t = fmax(t, red[w]);
    return t;
}

__device__ __forceinline__ void copy(double* dst, const double* src, int count) {
    for (int e = threadIdx.x; e < count; e += kNT) dst[e] = src[e];
}

__device__ __forceinline__ void set_identity(double* x, int n) {
    for (int e = threadIdx.x; e < n * n; e += kNT) x[e] = (e / n == e % n) ? 1.0 : 0.0;
}

// X <- A X in place (column-local).  at[m n + j] = A[j][m].
__device__ inline void gemm_left_inplace(double* x, const double* __restrict__ at, int n) {
    const int lane = lane_id();
    for (int k = warp_id(); k < n; k += kNW) {
        double acc[kMaxRows] = {0.0, 0.0, 0.0, 0.0};
        for (int m = 0; m < n; ++m) {
            const double xm = x[m * n + k];
            const double* a = at + m * n;
#pragma unroll
            for (int r = 0; r < kMaxRows; ++r) {
                const int j = lane + 32 * r;
                if (j < n) acc[r] = fma(a[j], xm, acc[r]);
            }
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < kMaxRows; ++r) {
            const int j = lane + 32 * r;
            if (j < n) x[j * n + k] = acc[r];
        }
        __syncwarp();
    }
}

// X <- X A in place (row-local).  a row-major.
__device__ inline void gemm_right_inplace(double* x, const double* __restrict__ a, int n) {
    const int lane = lane_id();
    for (int j = warp_id(); j < n; j += kNW) {
        double acc[kMaxRows] = {0.0, 0.0, 0.0, 0.0};
        const double* xr = x + j * n;
        for (int m = 0; m < n; ++m) {
            const double xm = xr[m];
            const double* ar = a + m * n;
#pragma unroll
            for (int r = 0; r < kMaxRows; ++r) {
                const int k = lane + 32 * r;
                if (k < n) acc[r] = fma(xm, ar[k], acc[r]);
            }
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < kMaxRows; ++r) {
            const int k = lane + 32 * r;
            if (k < n) x[j * n + k] = acc[r];
        }
        __syncwarp();
    }
}

// C = op(A) op(B), out of place.  TA: A stored transposed (C = A^T B); TB: C = A B^T.
template <bool TA, bool TB>
__device__ inline void gemm(double* __restrict__ c, const double* a, const double* b, int n) {
    const int lane = lane_id();
    for (int i = warp_id(); i < n; i += kNW) {
        double acc[kMaxRows] = {0.0, 0.0, 0.0, 0.0};
        for (int m = 0; m < n; ++m) {
            const double am = TA ? a[m * n + i] : a[i * n + m];
#pragma unroll
            for (int r = 0; r < kMaxRows; ++r) {
                const int j = lane + 32 * r;
                if (j < n) acc[r] = fma(am, TB ? b[j * n + m] : b[m * n + j], acc[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < kMaxRows; ++r) {
            const int j = lane + 32 * r;
            if (j < n) c[i * n + j] = acc[r];
        }
    }
}

// C = op(A) op(B), out of place, any n: the columns in blocks of 32 kMaxRows per warp row.
// For n <= 32 kMaxRows it performs the same fma chains as gemm<TA, TB>.
template <bool TA, bool TB>
__device__ inline void gemm_any(double* __restrict__ c, const double* a, const double* b, int n) {
    const int lane = lane_id();
    for (int j0 = 0; j0 < n; j0 += 32 * kMaxRows) {
        for (int i = warp_id(); i < n; i += kNW) {
            double acc[kMaxRows] = {0.0, 0.0, 0.0, 0.0};
            for (int m = 0; m < n; ++m) {
                const double am = TA ? a[m * n + i] : a[i * n + m];
#pragma unroll
                for (int r = 0; r < kMaxRows; ++r) {
                    const int j = j0 + lane + 32 * r;
                    if (j < n) acc[r] = fma(am, TB ? b[j * n + m] : b[m * n + j], acc[r]);
                }
            }
#pragma unroll
            for (int r = 0; r < kMaxRows; ++r) {
                const int j = j0 + lane + 32 * r;
                if (j < n) c[i * n + j] = acc[r];
            }
        }
    }
}

// Solve W Z = R in place by LU with partial pivoting (first maximal |pivot|, like LAPACK
// idamax).  On return rhs holds Z and w its LU factors.  Returns log|det W| through
// *logabs (thread-uniform) and sign(det W) through *sgn; *singular = 1 on a zero pivot.
// `sv` is scratch shared memory of at least kNW + 2 doubles.
__device__ inline void lu_solve(double* w, double* rhs, int n, double* sv, double* logabs,
                         double* sgn, int* singular) {
    const int lane = lane_id();
    int* spiv = reinterpret_cast<int*>(sv + kNW);
    double la = 0.0, sg = 1.0;
    int sing = 0;
    for (int j = 0; j < n; ++j) {
        if (warp_id() == 0) {
            double best = -1.0;
            int bi = n;
            for (int i = j + lane; i < n; i += 32) {
                const double v = fabs(w[i * n + j]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            // a column without a comparable entry (all NaN) keeps its own row: the index
            // stays in range and the NaN propagates to the status check
            if (lane == 0) *spiv = (bi < n) ? bi : j;
        }
        __syncthreads();
        const int p = *spiv;
        if (p != j) {
            for (int k = threadIdx.x; k < n; k += kNT) {
                double t = w[j * n + k]; w[j * n + k] = w[p * n + k]; w[p * n + k] = t;
                t = rhs[j * n + k]; rhs[j * n + k] = rhs[p * n + k]; rhs[p * n + k] = t;
            }
            sg = -sg;
        }
        __syncthreads();
        const double piv = w[j * n + j];
        if (piv == 0.0) sing = 1;
        la += log(fabs(piv));
        if (piv < 0.0) sg = -sg;
        for (int i = j + 1 + threadIdx.x; i < n; i += kNT) w[i * n + j] = w[i * n + j] / piv;
        __syncthreads();
        // trailing update of W (columns > j) and of every column of rhs
        const int rows = n - j - 1;
        const int cols = 2 * n - j - 1;
        for (int e = threadIdx.x; e < rows * cols; e += kNT) {
            const int i = j + 1 + e / cols;
            const int cc = e % cols;
            const double l = w[i * n + j];
            if (cc < n - j - 1) {
                const int k = j + 1 + cc;
                w[i * n + k] = fma(-l, w[j * n + k], w[i * n + k]);
            } else {
                const int k = cc - (n - j - 1);
                rhs[i * n + k] = fma(-l, rhs[j * n + k], rhs[i * n + k]);
            }
        }
        __syncthreads();
    }
    // back substitution
    for (int j = n - 1; j >= 0; --j) {
        const double piv = w[j * n + j];
        for (int k = threadIdx.x; k < n; k += kNT) rhs[j * n + k] = rhs[j * n + k] / piv;
        __syncthreads();
        for (int e = threadIdx.x; e < j * n; e += kNT) {
            const int i = e / n, k = e % n;
            rhs[i * n + k] = fma(-w[i * n + j], rhs[j * n + k], rhs[i * n + k]);
        }
        __syncthreads();
    }
    *logabs = la;
    *sgn = sg;
    *singular = sing;
}

// Householder QR in place (LAPACK convention beta = -sign(alpha) ||x||): R in the upper
// triangle, reflector vectors v (v_j = 1 implied) below it, tau[j] in `tau` (shared).
// Returns the number of non-trivial reflectors (det Q = (-1)^count).
// `sv` is scratch shared memory of at least kNW + 4 doubles.
__device__ inline int householder_qr(double* s, double* tau, int n, double* sv) {
    const int lane = lane_id();
    int nrefl = 0;
    for (int j = 0; j < n - 1; ++j) {
        if (warp_id() == 0) {
            double ss = 0.0;
            for (int i = j + 1 + lane; i < n; i += 32) { const double v = s[i * n + j]; ss = fma(v, v, ss); }
            ss = warp_sum(ss);
            if (lane == 0) {
                const double alpha = s[j * n + j];
                const double xnorm = sqrt(ss);
                if (xnorm == 0.0) {
                    tau[j] = 0.0;
                    sv[kNW] = 0.0;
                } else {
                    const double beta = -copysign(hypot(alpha, xnorm), alpha);
                    tau[j] = (beta - alpha) / beta;
                    sv[kNW] = alpha - beta;   // divisor of the reflector vector
                    sv[kNW + 1] = beta;
                }
            }
        }
        __syncthreads();
        const double t = tau[j];
        if (t == 0.0) continue;   // uniform across the block
        ++nrefl;
        const double den = sv[kNW];
        for (int i = j + 1 + threadIdx.x; i < n; i += kNT) s[i * n + j] = s[i * n + j] / den;
        __syncthreads();
        for (int k = j + 1 + warp_id(); k < n; k += kNW) {
            double acc = 0.0;
            for (int i = j + 1 + lane; i < n; i += 32) acc = fma(s[i * n + j], s[i * n + k], acc);
            acc = warp_sum(acc);
            const double wk = t * (s[j * n + k] + acc);
            for (int i = j + lane; i < n; i += 32) {
                const double vi = (i == j) ? 1.0 : s[i * n + j];
                s[i * n + k] = fma(-vi, wk, s[i * n + k]);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s[j * n + j] = sv[kNW + 1];
        __syncthreads();
    }
    return nrefl;
}

// Q = H_0 H_1 ... H_{n-2} from the reflectors householder_qr left in s / tau.
__device__ inline void householder_form_q(double* q, const double* s, const double* tau, int n) {
    const int lane = lane_id();
    set_identity(q, n);
    __syncthreads();
    for (int j = n - 2; j >= 0; --j) {
        const double t = tau[j];
        if (t == 0.0) continue;
        for (int k = j + warp_id(); k < n; k += kNW) {
            double acc = 0.0;
            for (int i = j + 1 + lane; i < n; i += 32) acc = fma(s[i * n + j], q[i * n + k], acc);
            acc = warp_sum(acc);
            const double wk = t * (q[j * n + k] + acc);
            for (int i = j + lane; i < n; i += 32) {
                const double vi = (i == j) ? 1.0 : s[i * n + j];
                q[i * n + k] = fma(-vi, wk, q[i * n + k]);
            }
        }
        __syncthreads();
    }
}

}  // namespace blk
}  // namespace lqmc
