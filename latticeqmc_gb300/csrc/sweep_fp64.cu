// Persistent float64 sweep kernel: one CTA per Markov chain, G_up / G_dn held in shared
// memory (n <= 90 with scratch, n <= 120 without), for both algorithm modes.
//
// Hot path of lqmc/lqmc.py:301-347 (fast sweep) restated per chain:
//   K1 ratio + accept      lqmc.py:313-317          every thread evaluates it redundantly
//   K2 rank-1 update       lqmc.py:318-333          block-wide, in place in shared memory
//   K3 slice wrap          lqmc.py:337-345          two in-place GEMMs (column-/row-local)
//   K4/K5 recompute of G   lqmc.py:156-185, :303-307
//        compat: unstabilised B-chain product + LU inverse (the reference's arithmetic)
//        dqmc:   pre-pivoted QR (UDT) chain product, right stack + left product,
//                refreshed every stab_every slices, with log|det G| and sign
//   K7 measurements        lqmc.py:356-375 (sum of G) + Wick observables
#include <cuda_runtime.h>
#include <stdint.h>

#include "block_fp64.cuh"
#include "chain_desc.h"
#include "philox.cuh"
#include "lqmc_gpu.h"

namespace lqmc {
namespace {

using namespace blk;

struct Smem {
    double* g[2];
    double* s0;
    double* s1;
    double* xv[2];
    double* yv[2];
    double* ev;
    double* nrm;
    double* tau;
    double* dv;
    int* order;
    double* sv;     // kNW + 8 scalars
};

__device__ __forceinline__ double* slot_u(const ChainDesc& d, int idx) { return d.work + (size_t)idx * d.slot; }
__device__ __forceinline__ double* slot_t(const ChainDesc& d, int idx) { return slot_u(d, idx) + d.n * d.n; }
__device__ __forceinline__ double* slot_d(const ChainDesc& d, int idx) { return slot_u(d, idx) + 2 * d.n * d.n; }
__device__ __forceinline__ double* slot_sign(const ChainDesc& d, int idx) { return slot_d(d, idx) + d.n; }
// right stack slot of spin s, chunk c; left ping-pong slot p of spin s
__device__ __forceinline__ int right_slot(const ChainDesc& d, int s, int c) { return s * d.n_chunks + c; }
__device__ __forceinline__ int left_slot(const ChainDesc& d, int s, int p) { return 2 * d.n_chunks + 2 * s + p; }

// ev[j] = exp(-sigma lambda s[j, l])  (lqmc.py:149-154), from the host-computed constants
__device__ __forceinline__ void load_ev(const ChainDesc& d, double* ev, int l, int sigma) {
    const int8_t* f = d.field + (size_t)l * d.n;
    for (int j = threadIdx.x; j < d.n; j += kNT) ev[j] = (sigma * f[j] > 0) ? d.c[2] : d.c[3];
}

// ---------------------------------------------------------------------------------------
// compat mode: the reference's arithmetic
// ---------------------------------------------------------------------------------------

// G_s = inv(1 + b_{L-1} ... b_0), b_l = exp_k diag(exp_v(l))   (lqmc.py:156-185, :303-307)
__device__ void compat_recompute(const ChainDesc& d, Smem& sm, int s, int* singular) {
    const int n = d.n, nn = n * n, sigma = s ? -1 : 1;
    double* x = sm.s1;
    double* b = sm.s0;
    load_ev(d, sm.ev, d.L - 1, sigma);
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) x[e] = __dmul_rn(d.expk[e], sm.ev[e % n]);
    __syncthreads();
    for (int l = d.L - 2; l >= 0; --l) {
        load_ev(d, sm.ev, l, sigma);
        __syncthreads();
        for (int e = threadIdx.x; e < nn; e += kNT) b[e] = __dmul_rn(d.expk[e], sm.ev[e % n]);
        __syncthreads();
        gemm_right_inplace(x, b, n);
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += kNT) x[i * n + i] = __dadd_rn(1.0, x[i * n + i]);
    set_identity(sm.g[s], n);
    __syncthreads();
    double la, sg;
    int sing;
    lu_solve(x, sm.g[s], n, sm.sv, &la, &sg, &sing);
    if (sing) *singular = 1;
    __syncthreads();
}

// G <- b G inv(b), b = diag(exp_v(l-1)) exp_k   (lqmc.py:339-345)
__device__ void compat_wrap(const ChainDesc& d, Smem& sm, int l_next) {
    const int n = d.n, nn = n * n;
    for (int s = 0; s < 2; ++s) {
        const int sigma = s ? -1 : 1;
        load_ev(d, sm.ev, l_next, sigma);
        __syncthreads();
        for (int e = threadIdx.x; e < nn; e += kNT) {
            const int m = e / n, j = e % n;
            sm.s0[e] = __dmul_rn(sm.ev[j], d.expkT[e]);            // b^T[m][j] = d_j expK[j][m]
            sm.s1[e] = __ddiv_rn(d.expkinv[e], sm.ev[j]);          // inv(b)[m][k] = expK^-1[m][k] / d_k
            (void)m;
        }
        __syncthreads();
        gemm_left_inplace(sm.g[s], sm.s0, n);
        __syncthreads();
        gemm_right_inplace(sm.g[s], sm.s1, n);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// det mode: the reference's slow path (lqmc.py:236-299), every ratio from determinants
// ---------------------------------------------------------------------------------------

// log|det W| and sign(det W) by LU with partial pivoting (first maximal |pivot|); W is
// overwritten.  *singular = 1 on a zero pivot.
__device__ void lu_logdet(double* w, int n, double* sv, double* logabs, double* sgn, int* singular) {
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
            if (lane == 0) *spiv = (bi < n) ? bi : j;   // all-NaN column: keep the row
        }
        __syncthreads();
        const int p = *spiv;
        if (p != j) {
            for (int k = threadIdx.x; k < n; k += kNT) {
                const double t = w[j * n + k]; w[j * n + k] = w[p * n + k]; w[p * n + k] = t;
            }
            sg = -sg;
        }
        __syncthreads();
        const double piv = w[j * n + j];
        if (piv == 0.0) sing = 1;
        la += log(fabs(piv));
        if (piv < 0.0) sg = -sg;
        const int rows = n - j - 1;
        for (int e = threadIdx.x; e < rows * rows; e += kNT) {
            const int i = j + 1 + e / rows, k = j + 1 + e % rows;
            w[i * n + k] = fma(-(w[i * n + j] / piv), w[j * n + k], w[i * n + k]);
        }
        __syncthreads();
    }
    *logabs = la;
    *sgn = sg;
    *singular |= sing;
}

// M_s = 1 + b_{l0-1} ... b_0 b_{L-1} ... b_{l0}, b_t = exp_k diag(exp_v(t)), the cyclic product
// of get_m(l0, sigma) (lqmc.py:156-185), factorised for its log|det| and sign
__device__ void det_m(const ChainDesc& d, Smem& sm, int l0, int s, double* la, double* sg, int* singular) {
    const int n = d.n, nn = n * n, L = d.L, sigma = s ? -1 : 1;
    double* x = sm.s1;
    double* b = sm.s0;
    for (int k = 0; k < L; ++k) {
        const int t = ((l0 - 1 - k) % L + L) % L;
        load_ev(d, sm.ev, t, sigma);
        __syncthreads();
        double* dst = k ? b : x;
        for (int e = threadIdx.x; e < nn; e += kNT) dst[e] = __dmul_rn(d.expk[e], sm.ev[e % n]);
        __syncthreads();
        if (k) {
            gemm_right_inplace(x, b, n);
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += kNT) x[i * n + i] = __dadd_rn(1.0, x[i * n + i]);
    __syncthreads();
    lu_logdet(x, n, sm.sv, la, sg, singular);
}

// One det-mode sweep (lqmc.py:236-259): flip, recompute det M_up det M_dn, accept with
// u <= new / old, else flip back.  la_old / sg_old carry the current configuration's
// log|det M| and sign per spin.
__device__ void det_sweep(const ChainDesc& d, Smem& sm, int sw, uint64_t sweep_id, double* la_old,
                          double* sg_old, int* accepted, int* singular) {
    const int n = d.n, L = d.L;
    for (int l = L - 1; l >= 0; --l) {
        int8_t* f = d.field + (size_t)l * n;
        const int step = L - 1 - l;
        for (int i = 0; i < n; ++i) {
            const int pos = step * n + i;
            if (threadIdx.x == 0) f[i] = (int8_t)(-f[i]);
            __syncthreads();
            double la[2], sg[2];
            det_m(d, sm, l, 0, &la[0], &sg[0], singular);
            det_m(d, sm, l, 1, &la[1], &sg[1], singular);
            double u;
            if (d.rng == LQMC_RNG_REPLAY) u = d.uniforms[(size_t)sw * n * L + pos];
            else u = philox_uniform(d.seed, (uint64_t)d.chain_id, sweep_id, (uint64_t)pos);
            const double ratio = (sg[0] * sg[1]) / (sg_old[0] * sg_old[1]) *
                                 exp((la[0] + la[1]) - (la_old[0] + la_old[1]));
            const bool acc = (u <= ratio);
            if (acc) {
                la_old[0] = la[0]; la_old[1] = la[1];
                sg_old[0] = sg[0]; sg_old[1] = sg[1];
            }
            if (threadIdx.x == 0) {
                if (acc) ++*accepted;
                else f[i] = (int8_t)(-f[i]);
                if (d.record) d.decisions[((size_t)sw * L + step) * n + i] = acc ? 1 : 0;
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------------------
// dqmc mode: UDT chain products
// ---------------------------------------------------------------------------------------

// z holds C U_old.  Writes the UDT of C U_old diag(d_old) T_old (pre-pivoted QR).
// d_old == nullptr / t_old == nullptr stand for ones / identity.  Returns det sign of U.
__device__ double udt_absorb(const ChainDesc& d, Smem& sm, double* z, double* s,
                             const double* d_old, const double* t_old,
                             double* u_new, double* d_new, double* t_new) {
    const int n = d.n, nn = n * n, lane = lane_id();
    if (d_old) {
        for (int e = threadIdx.x; e < nn; e += kNT) z[e] = z[e] * d_old[e % n];
        __syncthreads();
    }
    for (int k = warp_id(); k < n; k += kNW) {
        double acc = 0.0;
        for (int i = lane; i < n; i += 32) { const double v = z[i * n + k]; acc = fma(v, v, acc); }
        acc = warp_sum(acc);
        if (lane == 0) sm.nrm[k] = sqrt(acc);
    }
    __syncthreads();
    // rank by descending norm, ties by index; NaN sorts last so the ranks always form a
    // permutation of 0..n-1
    for (int k = threadIdx.x; k < n; k += kNT) {
        const double v = isnan(sm.nrm[k]) ? -1.0 : sm.nrm[k];
        int rank = 0;
        for (int j = 0; j < n; ++j) {
            const double w = isnan(sm.nrm[j]) ? -1.0 : sm.nrm[j];
            rank += (w > v) || (w == v && j < k);
        }
        sm.order[rank] = k;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int i = e / n, r = e % n;
        s[e] = z[i * n + sm.order[r]];
    }
    __syncthreads();
    const int nrefl = householder_qr(s, sm.tau, n, sm.sv);
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double di = s[i * n + i];
        sm.dv[i] = di;
        d_new[i] = di;
    }
    __syncthreads();
    householder_form_q(u_new, s, sm.tau, n);
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int i = e / n, k = e % n;
        if (k >= i) s[e] = s[e] / sm.dv[i];
    }
    __syncthreads();
    for (int i = warp_id(); i < n; i += kNW) {
        for (int c = lane; c < n; c += 32) {
            double acc = 0.0;
            for (int k = i; k < n; ++k) {
                const int src = sm.order[k];
                const double tv = t_old ? t_old[src * n + c] : (src == c ? 1.0 : 0.0);
                acc = fma(s[i * n + k], tv, acc);
            }
            t_new[i * n + c] = acc;
        }
    }
    __syncthreads();
    return (nrefl & 1) ? -1.0 : 1.0;
}

// G = (1 + U_R D_R T_R T_L^T D_L U_L^T)^-1 via the split D = D_big D_small.
// ul == nullptr: the left product is the identity.  Writes G into g; returns the
// residual max|G_new - G_old| when `residual`.
__device__ double green_udt(const ChainDesc& d, Smem& sm, const double* ur, const double* dr,
                            const double* tr, double sign_r, const double* ul,
                            const double* dl, const double* tl, double sign_l, double* g,
                            bool residual, double* logdet, double* sgn, int* singular) {
    const int n = d.n, nn = n * n;
    double* dbr = sm.xv[0];
    double* dsr = sm.xv[1];
    double* dbl = sm.yv[0];
    double* dsl = sm.yv[1];
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double a = dr[i];
        const double b = fmax(fabs(a), 1.0);
        dbr[i] = b;
        dsr[i] = a / b;
        if (ul) {
            const double c = dl[i];
            const double e = fmax(fabs(c), 1.0);
            dbl[i] = e;
            dsl[i] = c / e;
        } else {
            dbl[i] = 1.0;
            dsl[i] = 1.0;
        }
    }
    if (ul) {
        gemm<true, false>(sm.s0, ur, ul, n);   // X = U_R^T U_L
        gemm<false, true>(sm.s1, tr, tl, n);   // Y = T_R T_L^T
    } else {
        for (int e = threadIdx.x; e < nn; e += kNT) {
            const int i = e / n, j = e % n;
            sm.s0[e] = ur[j * n + i];
            sm.s1[e] = tr[e];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int i = e / n, j = e % n;
        sm.s0[e] = sm.s0[e] / dbr[i] / dbl[j] + dsr[i] * sm.s1[e] * dsl[j];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int i = e / n, j = e % n;
        sm.s1[e] = ur[j * n + i] / dbr[i];
    }
    __syncthreads();
    double la, sw;
    int sing;
    lu_solve(sm.s0, sm.s1, n, sm.sv, &la, &sw, &sing);
    if (sing) *singular = 1;
    const double* src = sm.s1;
    if (ul) {
        for (int e = threadIdx.x; e < nn; e += kNT) sm.s1[e] = sm.s1[e] / dbl[e / n];
        __syncthreads();
        gemm<false, false>(sm.s0, ul, sm.s1, n);
        __syncthreads();
        src = sm.s0;
    }
    double res = 0.0;
    if (residual) {
        double m = 0.0;
        for (int e = threadIdx.x; e < nn; e += kNT) m = fmax(m, fabs(src[e] - g[e]));
        res = block_max(m, sm.sv);
    }
    // log|det G| = -(sum log D_big_R + log|det W| + sum log D_big_L)
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += kNT) part += log(dbr[i]) + log(dbl[i]);
    const double tot = block_sum(part, sm.sv);
    for (int e = threadIdx.x; e < nn; e += kNT) g[e] = src[e];
    __syncthreads();
    *logdet = -(tot + la);
    *sgn = sign_r * sw * sign_l;
    return res;
}

__device__ void dqmc_right_stack(const ChainDesc& d, Smem& sm, int s, double* logdet,
                                 double* sgn, int* singular) {
    const int n = d.n, nn = n * n, sigma = s ? -1 : 1;
    for (int c = 0; c < d.n_chunks; ++c) {
        const int lo = c * d.stab_every;
        const int hi = min(lo + d.stab_every, d.L);
        if (c == 0) set_identity(sm.s0, n);
        else copy(sm.s0, slot_u(d, right_slot(d, s, c - 1)), nn);
        __syncthreads();
        for (int l = lo; l < hi; ++l) {
            gemm_left_inplace(sm.s0, d.expkT, n);          // expK Z
            load_ev(d, sm.ev, l, sigma);
            __syncthreads();
            for (int e = threadIdx.x; e < nn; e += kNT) sm.s0[e] = sm.ev[e / n] * sm.s0[e];
            __syncthreads();
        }
        const int prev = right_slot(d, s, c - 1), cur = right_slot(d, s, c);
        const double sg = udt_absorb(d, sm, sm.s0, sm.s1, c ? slot_d(d, prev) : nullptr,
                                     c ? slot_t(d, prev) : nullptr, slot_u(d, cur),
                                     slot_d(d, cur), slot_t(d, cur));
        if (threadIdx.x == 0) *slot_sign(d, cur) = sg;
        __syncthreads();
    }
    const int top = right_slot(d, s, d.n_chunks - 1);
    green_udt(d, sm, slot_u(d, top), slot_d(d, top), slot_t(d, top), *slot_sign(d, top),
              nullptr, nullptr, nullptr, 1.0, sm.g[s], false, logdet, sgn, singular);
}

// Left product of the chunk [lo, hi) on top of the left ping-pong slot `p_in`
// (first == true: start from the identity); result into slot 1 - p_in.
__device__ void dqmc_left_step(const ChainDesc& d, Smem& sm, int s, int p_in, bool first,
                               int lo, int hi) {
    const int n = d.n, nn = n * n, sigma = s ? -1 : 1;
    const int in = left_slot(d, s, p_in), out = left_slot(d, s, 1 - p_in);
    if (first) set_identity(sm.s0, n);
    else copy(sm.s0, slot_u(d, in), nn);
    __syncthreads();
    for (int l = hi - 1; l >= lo; --l) {
        load_ev(d, sm.ev, l, sigma);
        __syncthreads();
        for (int e = threadIdx.x; e < nn; e += kNT) sm.s0[e] = sm.ev[e / n] * sm.s0[e];
        __syncthreads();
        gemm_left_inplace(sm.s0, d.expk, n);            // expK^T (exp_v Z)
        __syncthreads();
    }
    const double sg = udt_absorb(d, sm, sm.s0, sm.s1, first ? nullptr : slot_d(d, in),
                                 first ? nullptr : slot_t(d, in), slot_u(d, out),
                                 slot_d(d, out), slot_t(d, out));
    if (threadIdx.x == 0) *slot_sign(d, out) = sg;
    __syncthreads();
}

// G <- exp(+dtau K) exp_v(l)^-1 G exp_v(l) exp(-dtau K)
__device__ void dqmc_wrap(const ChainDesc& d, Smem& sm, int l) {
    const int n = d.n, nn = n * n;
    for (int s = 0; s < 2; ++s) {
        const int sigma = s ? -1 : 1;
        load_ev(d, sm.ev, l, sigma);
        __syncthreads();
        double* g = sm.g[s];
        for (int e = threadIdx.x; e < nn; e += kNT) g[e] = (g[e] / sm.ev[e / n]) * sm.ev[e % n];
        __syncthreads();
        gemm_left_inplace(g, d.expkinvT, n);
        __syncthreads();
        gemm_right_inplace(g, d.expk, n);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// site updates of one time slice (both modes)
// ---------------------------------------------------------------------------------------
__device__ void update_slice(const ChainDesc& d, Smem& sm, int l, int sw, uint64_t sweep_id,
                             int* accepted) {
    const int n = d.n, nn = n * n, L = d.L;
    const int step = L - 1 - l;
    double* g0 = sm.g[0];
    double* g1 = sm.g[1];
    int8_t* f = d.field + (size_t)l * n;
    for (int i = 0; i < n; ++i) {
        const int pos = step * n + i;
        const int8_t s_il = f[i];
        double u;
        if (d.rng == LQMC_RNG_REPLAY) u = d.uniforms[(size_t)sw * n * L + pos];
        else u = philox_uniform(d.seed, (uint64_t)d.chain_id, sweep_id, (uint64_t)pos);
        const double gi0 = g0[i * n + i], gi1 = g1[i * n + i];
        const double ep = s_il > 0 ? d.c[0] : d.c[1];   // exp(+arg), arg = 2 lambda s
        const double em = s_il > 0 ? d.c[1] : d.c[0];   // exp(-arg)
        double ratio, a0, a1;
        if (d.mode == LQMC_MODE_COMPAT) {
            const double d_up = __dadd_rn(1.0, __dmul_rn(__dsub_rn(1.0, gi0), __dsub_rn(ep, 1.0)));
            const double d_dn = __dadd_rn(1.0, __dmul_rn(__dsub_rn(1.0, gi1), __dsub_rn(em, 1.0)));
            ratio = __dmul_rn(d_up, d_dn);
            a0 = __dsub_rn(em, 1.0);    // the reference's up-spin update uses exp(-arg) - 1
            a1 = __dsub_rn(ep, 1.0);
        } else {
            const double dl_up = __dsub_rn(ep, 1.0), dl_dn = __dsub_rn(em, 1.0);
            const double r_up = __dadd_rn(1.0, __dmul_rn(dl_up, __dsub_rn(1.0, gi0)));
            const double r_dn = __dadd_rn(1.0, __dmul_rn(dl_dn, __dsub_rn(1.0, gi1)));
            ratio = __dmul_rn(r_up, r_dn);
            a0 = __ddiv_rn(dl_up, r_up);
            a1 = __ddiv_rn(dl_dn, r_dn);
        }
        const bool acc = (u <= ratio);
        if (d.record && threadIdx.x == 0)
            d.decisions[((size_t)sw * L + step) * n + i] = acc ? 1 : 0;
        if (!acc) continue;
        const int j = threadIdx.x;
        if (j < n) {
            if (d.mode == LQMC_MODE_COMPAT) {
                // c = -(E-1) G[i,:], c_i += E-1, e = G[:,i] / (1 + c_i)   (lqmc.py:320-327)
                const double t0 = -a0, t1 = -a1;
                const double ci0 = __dadd_rn(__dmul_rn(t0, gi0), a0);
                const double ci1 = __dadd_rn(__dmul_rn(t1, gi1), a1);
                sm.yv[0][j] = (j == i) ? ci0 : __dmul_rn(t0, g0[i * n + j]);
                sm.yv[1][j] = (j == i) ? ci1 : __dmul_rn(t1, g1[i * n + j]);
                sm.xv[0][j] = __ddiv_rn(g0[j * n + i], __dadd_rn(1.0, ci0));
                sm.xv[1][j] = __ddiv_rn(g1[j * n + i], __dadd_rn(1.0, ci1));
            } else {
                // x = G[:,i], y = (Delta/R) (e_i - G[i,:])
                sm.xv[0][j] = g0[j * n + i];
                sm.xv[1][j] = g1[j * n + i];
                sm.yv[0][j] = __dmul_rn((j == i) ? __dadd_rn(-gi0, 1.0) : -g0[i * n + j], a0);
                sm.yv[1][j] = __dmul_rn((j == i) ? __dadd_rn(-gi1, 1.0) : -g1[i * n + j], a1);
            }
        }
        __syncthreads();
        if (d.mode == LQMC_MODE_COMPAT) {
            for (int e = threadIdx.x; e < nn; e += kNT) {
                const int r = e / n, c = e % n;
                g0[e] = __dsub_rn(g0[e], __dmul_rn(sm.xv[0][r], sm.yv[0][c]));
                g1[e] = __dsub_rn(g1[e], __dmul_rn(sm.xv[1][r], sm.yv[1][c]));
            }
        } else {
            for (int e = threadIdx.x; e < nn; e += kNT) {
                const int r = e / n, c = e % n;
                g0[e] = fma(-sm.xv[0][r], sm.yv[0][c], g0[e]);
                g1[e] = fma(-sm.xv[1][r], sm.yv[1][c], g1[e]);
            }
        }
        if (threadIdx.x == 0) {
            f[i] = (int8_t)(-s_il);
            ++*accepted;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// K7: measurements (lqmc.py:367-375 sums G; Wick observables on top)
// ---------------------------------------------------------------------------------------
__device__ void measure(const ChainDesc& d, Smem& sm) {
    const int n = d.n, nn = n * n;
    const double* g0 = sm.g[0];
    const double* g1 = sm.g[1];
    double* obs = d.obs;
    for (int e = threadIdx.x; e < nn; e += kNT) {
        d.gsum[e] += g0[e];
        d.gsum[nn + e] += g1[e];
    }
    double* nu = sm.xv[0];
    double* nd = sm.xv[1];
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double a = 1.0 - g0[i * n + i], b = 1.0 - g1[i * n + i];
        nu[i] = a;
        nd[i] = b;
        obs[LQMC_OBS_HEADER + i] += a + b;
        obs[LQMC_OBS_HEADER + n + i] += a * b;
    }
    __syncthreads();
    double ek = 0.0, ep = 0.0, dc = 0.0, dn = 0.0;
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int j = e / n, k = e % n;
        const double kv = d.kinetic[e];
        if (kv != 0.0) {
            const double del = (j == k) ? 1.0 : 0.0;
            ek += kv * ((del - g0[k * n + j]) + (del - g1[k * n + j]));
        }
    }
    for (int i = threadIdx.x; i < n; i += kNT) {
        ep += (nu[i] - 0.5) * (nd[i] - 0.5);
        dc += nu[i] * nd[i];
        dn += nu[i] + nd[i];
    }
    ek = block_sum(ek, sm.sv);
    ep = block_sum(ep, sm.sv);
    dc = block_sum(dc, sm.sv);
    dn = block_sum(dn, sm.sv);
    if (threadIdx.x == 0) {
        obs[0] += 1.0;
        obs[1] += ek;
        obs[2] += d.u * ep;
        obs[3] += dc / n;
        obs[4] += dn / n;
    }
    double* onn = obs + LQMC_OBS_HEADER + 2 * n;
    double* osz = onn + nn;
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int i = e / n, j = e % n;
        const double del = (i == j) ? 1.0 : 0.0;
        const double same = nu[i] * nu[j] + nd[i] * nd[j] + (del - g0[j * n + i]) * g0[e] +
                            (del - g1[j * n + i]) * g1[e];
        const double cross = nu[i] * nd[j] + nd[i] * nu[j];
        onn[e] += same + cross;
        osz[e] += 0.25 * (same - cross);
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------------------
// Unequal-time G(tau_l, 0) = B_{l-1} ... B_0 G(0) (dqmc mode's B_l = exp_v(l) exp_k)
// ---------------------------------------------------------------------------------------

// X = G(tau, 0) = B(tau, 0) (1 + B(beta, tau) B(tau, 0))^-1 from the UDT factors
// B(tau, 0) = U_R D_R T_R and B(beta, tau)^T = U_L D_L T_L.  With D = D_big D_small on each
// side and the equal-time matrix W = D_bigR^-1 U_R^T U_L D_bigL^-1 + D_smallR T_R T_L^T
// D_smallL, G(tau) = U_L D_bigL^-1 W^-1 D_bigR^-1 U_R^T, and G(tau, 0) = G(tau) B(tau, 0)
// = U_L D_bigL^-1 W^-1 D_smallR T_R: no factor above 1 is left outside the solve.
// ur == nullptr: B(tau, 0) is the identity (tau = 0), X = U_L D_bigL^-1 W^-1.
__device__ void green_tau_udt(const ChainDesc& d, Smem& sm, const double* ur, const double* dr,
                              const double* tr, const double* ul, const double* dl,
                              const double* tl, double* x, int* singular) {
    const int n = d.n, nn = n * n;
    double* dbr = sm.xv[0];
    double* dsr = sm.xv[1];
    double* dbl = sm.yv[0];
    double* dsl = sm.yv[1];
    for (int i = threadIdx.x; i < n; i += kNT) {
        const double a = ur ? dr[i] : 1.0, b = fmax(fabs(a), 1.0);
        dbr[i] = b;
        dsr[i] = a / b;
        const double c = dl[i], e = fmax(fabs(c), 1.0);
        dbl[i] = e;
        dsl[i] = c / e;
    }
    if (ur) {
        gemm_any<true, false>(sm.s0, ur, ul, n);   // U_R^T U_L
        gemm_any<false, true>(sm.s1, tr, tl, n);   // T_R T_L^T
    } else {
        for (int e = threadIdx.x; e < nn; e += kNT) {
            sm.s0[e] = ul[e];
            sm.s1[e] = tl[(e % n) * n + e / n];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) {
        const int i = e / n, j = e % n;
        sm.s0[e] = sm.s0[e] / dbr[i] / dbl[j] + dsr[i] * sm.s1[e] * dsl[j];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT)
        sm.s1[e] = ur ? dsr[e / n] * tr[e] : ((e / n == e % n) ? 1.0 : 0.0);
    __syncthreads();
    double la, sw;
    int sing;
    lu_solve(sm.s0, sm.s1, n, sm.sv, &la, &sw, &sing);
    if (sing) *singular = 1;
    for (int e = threadIdx.x; e < nn; e += kNT) sm.s1[e] = sm.s1[e] / dbl[e / n];
    __syncthreads();
    gemm_any<false, false>(x, ul, sm.s1, n);
    __syncthreads();
}

// z <- B_l z = exp_v(l) (exp_k z), through the scratch `tmp`
__device__ void tau_b_left(const ChainDesc& d, Smem& sm, double* z, double* tmp, int l, int sigma) {
    const int n = d.n, nn = n * n;
    __syncthreads();
    gemm_any<false, false>(tmp, d.expk, z, n);
    load_ev(d, sm.ev, l, sigma);
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) z[e] = sm.ev[e / n] * tmp[e];
    __syncthreads();
}

// z <- B_l^T z = exp_k^T (exp_v(l) z), through the scratch `tmp`
__device__ void tau_bt_left(const ChainDesc& d, Smem& sm, double* z, double* tmp, int l, int sigma) {
    const int n = d.n, nn = n * n;
    load_ev(d, sm.ev, l, sigma);
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += kNT) tmp[e] = sm.ev[e / n] * z[e];
    __syncthreads();
    gemm_any<true, false>(z, d.expk, tmp, n);
    __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(kNT, 1)
sweep_fp64_kernel(const ChainDesc* __restrict__ descs, int n_sweeps, int do_measure,
                  int sweep_base) {
    extern __shared__ __align__(16) double smem[];
    __shared__ ChainDesc d;
    __shared__ int accepted;
    __shared__ int singular;
    if (threadIdx.x == 0) {
        d = descs[blockIdx.x];
        accepted = 0;
        singular = 0;
    }
    __syncthreads();
    const int n = d.n, nn = n * n;
    Smem sm;
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
    p = smem + (((p - smem) + 3) & ~(ptrdiff_t)3);   // 32-byte multiple from the base
    double* gw = d.work + (size_t)(2 * d.n_chunks + 4) * d.slot;   // spill area after the slots
    if (d.flags & kGreenInGlobal) { sm.g[0] = gw; sm.g[1] = gw + nn; gw += 2 * nn; }
    else { sm.g[0] = p; sm.g[1] = p + nn; p += 2 * nn; }
    if (d.flags & kScratchInGlobal) { sm.s0 = gw; sm.s1 = gw + nn; }
    else { sm.s0 = p; sm.s1 = p + nn; }

    double max_resid = 0.0;
    double logdet[2] = {0.0, 0.0}, sgn[2] = {1.0, 1.0};
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
    double la_old[2] = {0.0, 0.0}, sg_old[2] = {1.0, 1.0};   // det mode
    // sw indexes the call's uniforms and decisions: sweep_base + the sweep of this launch
    for (int sw = sweep_base; sw < sweep_base + n_sweeps; ++sw, ++sweep_id) {
        if (d.mode == LQMC_MODE_DET) {
            // det M of the current configuration, recomputed when a launch starts as the
            // reference does when each of its loops starts (lqmc.py:261-266, :277-282)
            if (sw == sweep_base) {
                det_m(d, sm, 0, 0, &la_old[0], &sg_old[0], &singular);
                det_m(d, sm, 0, 1, &la_old[1], &sg_old[1], &singular);
            }
            LQMC_PHASE(0);
            det_sweep(d, sm, sw, sweep_id, la_old, sg_old, &accepted, &singular);
            LQMC_PHASE(1);
            // G = inv(get_m(0, sigma)) for the measurement (lqmc.py:293-295) and the output
            compat_recompute(d, sm, 0, &singular);
            compat_recompute(d, sm, 1, &singular);
            for (int s = 0; s < 2; ++s) {
                logdet[s] = -la_old[s];
                sgn[s] = sg_old[s];
            }
            LQMC_PHASE(0);
        } else if (d.mode == LQMC_MODE_COMPAT) {
            compat_recompute(d, sm, 0, &singular);
            compat_recompute(d, sm, 1, &singular);
            LQMC_PHASE(0);
            for (int l = d.L - 1; l >= 0; --l) {
                update_slice(d, sm, l, sw, sweep_id, &accepted);
                LQMC_PHASE(1);
                if (l > 0) compat_wrap(d, sm, l - 1);
                LQMC_PHASE(2);
            }
        } else {
            dqmc_right_stack(d, sm, 0, &logdet[0], &sgn[0], &singular);
            dqmc_right_stack(d, sm, 1, &logdet[1], &sgn[1], &singular);
            LQMC_PHASE(0);
            int lp[2] = {0, 0};
            for (int c = d.n_chunks - 1; c >= 0; --c) {
                const int lo = c * d.stab_every;
                const int hi = min(lo + d.stab_every, d.L);
                for (int l = hi - 1; l >= lo; --l) {
                    update_slice(d, sm, l, sw, sweep_id, &accepted);
                    LQMC_PHASE(1);
                    if (l > 0) dqmc_wrap(d, sm, l);
                    LQMC_PHASE(2);
                }
                if (c > 0) {
                    for (int s = 0; s < 2; ++s) {
                        const bool first = (c == d.n_chunks - 1);
                        dqmc_left_step(d, sm, s, lp[s], first, lo, hi);
                        lp[s] ^= 1;
                        const int rs = right_slot(d, s, c - 1), ls = left_slot(d, s, lp[s]);
                        const double r = green_udt(d, sm, slot_u(d, rs), slot_d(d, rs), slot_t(d, rs),
                                                   *slot_sign(d, rs), slot_u(d, ls), slot_d(d, ls),
                                                   slot_t(d, ls), *slot_sign(d, ls), sm.g[s], true,
                                                   &logdet[s], &sgn[s], &singular);
                        max_resid = fmax(max_resid, r);
                    }
                    LQMC_PHASE(3);
                }
            }
        }
        __syncthreads();
        if (do_measure) measure(d, sm);
        LQMC_PHASE(4);
#undef LQMC_PHASE
        // health check of G (NaN/Inf)
        int bad = 0;
        for (int e = threadIdx.x; e < 2 * nn; e += kNT) {
            const double v = (e < nn) ? sm.g[0][e] : sm.g[1][e - nn];
            if (!isfinite(v)) bad = 1;
        }
        bad = __syncthreads_or(bad);
        if (bad && threadIdx.x == 0) atomicOr(d.status, LQMC_STATUS_NONFINITE);
    }
    for (int e = threadIdx.x; e < nn; e += kNT) {
        d.green[e] = sm.g[0][e];
        d.green[nn + e] = sm.g[1][e];
    }
    if (threadIdx.x == 0) {
        d.diag[0] += (double)accepted;
        d.diag[1] += (double)n_sweeps * n * d.L;
        d.diag[2] = max_resid;
        d.diag[3] = logdet[0];
        d.diag[4] = logdet[1];
        d.diag[5] = sgn[0];
        d.diag[6] = sgn[1];
        d.diag[7] += (double)n_sweeps;
        for (int k = 0; k < 5; ++k) d.diag[8 + k] = (double)ph[k];
        if (singular) atomicOr(d.status, LQMC_STATUS_SINGULAR);
        if (max_resid > d.drift_tol) atomicOr(d.status, LQMC_STATUS_DRIFT);
    }
}

// bytes of dynamic shared memory the kernel needs for a chain of n sites with `flags`
size_t sweep_fp64_smem_bytes(int n, int flags) {
    size_t v = (size_t)(kNW + 8 + 9 * n);
    v = ((v + 3) & ~(size_t)3) * sizeof(double);
    if (!(flags & kGreenInGlobal)) v += 2 * (size_t)n * n * sizeof(double);
    if (!(flags & kScratchInGlobal)) v += 2 * (size_t)n * n * sizeof(double);
    return v;
}

cudaError_t launch_sweep_fp64(const ChainDesc* d_descs, int n_chains, size_t smem, int n_sweeps,
                              int measure, int sweep_base, cudaStream_t stream) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(sweep_fp64_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    sweep_fp64_kernel<<<n_chains, kNT, smem, stream>>>(d_descs, n_sweeps, measure, sweep_base);
    return cudaGetLastError();
}

// G(tau_l, 0) = B(tau_l, 0) (1 + B(beta, 0))^-1, l = 0 .. L-1, of the field the last sweep
// left, added to desc.gtau.  One CTA per (chain, spin); float64 for every engine.
//   1. B(beta, tau_c)^T, tau_c = c stab_every, c = nc-1 .. 0, as UDT factors (slot c),
//      built down from the top like the sweep's left products;
//   2. at every chunk start X = G(tau_c, 0) from the UDT factors of B(tau_c, 0) (ping-pong
//      slots nc, nc+1, built up from the bottom like the sweep's right stack) and of
//      B(beta, tau_c) (green_tau_udt); inside the chunk X <- B_l X slice by slice.
__global__ void __launch_bounds__(kNT, 1) green_tau_kernel(const ChainDesc* __restrict__ descs) {
    extern __shared__ __align__(16) double smem[];
    __shared__ ChainDesc d;
    __shared__ int singular;
    const int s = blockIdx.y, sigma = s ? -1 : 1;
    if (threadIdx.x == 0) {
        d = descs[blockIdx.x];
        singular = 0;
        const size_t nn = (size_t)d.n * d.n;
        const size_t per_spin = (size_t)(d.n_chunks + 2) * d.slot + nn +
                                ((d.tau_flags & kScratchInGlobal) ? 2 * nn : 0);
        d.work = d.tau_work + (size_t)s * per_spin;   // slot_u(d, k): this spin's slot k
    }
    __syncthreads();
    const int n = d.n, nn = n * n, L = d.L, nc = d.n_chunks, se = d.stab_every;
    Smem sm;
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
    sm.g[0] = sm.g[1] = nullptr;
    double* x = d.work + (size_t)(nc + 2) * d.slot;
    if (d.tau_flags & kScratchInGlobal) { sm.s0 = x + nn; sm.s1 = x + 2 * nn; }
    else { sm.s0 = p; sm.s1 = p + nn; }

    // 1. slot c <- UDT of B(beta, tau_c)^T = B_{lo}^T ... B_{L-1}^T
    for (int c = nc - 1; c >= 0; --c) {
        const int lo = c * se, hi = min(lo + se, L);
        const bool first = (c == nc - 1);
        if (first) set_identity(sm.s0, n);
        else copy(sm.s0, slot_u(d, c + 1), nn);
        for (int l = hi - 1; l >= lo; --l) tau_bt_left(d, sm, sm.s0, sm.s1, l, sigma);
        udt_absorb(d, sm, sm.s0, sm.s1, first ? nullptr : slot_d(d, c + 1),
                   first ? nullptr : slot_t(d, c + 1), slot_u(d, c), slot_d(d, c), slot_t(d, c));
    }
    // 2. X = G(tau_l, 0), recomputed at each chunk start and propagated up inside it
    double* acc = d.gtau + (size_t)s * L * nn;
    int rp = 0;
    for (int c = 0; c < nc; ++c) {
        const int lo = c * se, hi = min(lo + se, L);
        const int r = nc + rp;
        green_tau_udt(d, sm, c ? slot_u(d, r) : nullptr, slot_d(d, r), slot_t(d, r), slot_u(d, c),
                      slot_d(d, c), slot_t(d, c), x, &singular);
        for (int l = lo; l < hi; ++l) {
            for (int e = threadIdx.x; e < nn; e += kNT) acc[(size_t)l * nn + e] += x[e];
            if (l + 1 < hi) tau_b_left(d, sm, x, sm.s1, l, sigma);
        }
        if (c + 1 < nc) {
            // running product B(tau_hi, 0) = B_{hi-1} ... B_lo B(tau_lo, 0)
            const int in = nc + rp, out = nc + (rp ^ 1);
            __syncthreads();
            if (c == 0) set_identity(sm.s0, n);
            else copy(sm.s0, slot_u(d, in), nn);
            for (int l = lo; l < hi; ++l) tau_b_left(d, sm, sm.s0, sm.s1, l, sigma);
            udt_absorb(d, sm, sm.s0, sm.s1, c ? slot_d(d, in) : nullptr,
                       c ? slot_t(d, in) : nullptr, slot_u(d, out), slot_d(d, out), slot_t(d, out));
            rp ^= 1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && singular) atomicOr(d.status, LQMC_STATUS_SINGULAR);
}

// dynamic shared memory and per-chain float64 workspace (doubles) of green_tau_kernel
size_t green_tau_smem_bytes(int n, int tau_flags) {
    return sweep_fp64_smem_bytes(n, kGreenInGlobal | (tau_flags & kScratchInGlobal));
}

size_t green_tau_work_doubles(int n, int n_chunks, int slot, int tau_flags) {
    const size_t nn = (size_t)n * n;
    return 2 * ((size_t)(n_chunks + 2) * slot + nn + ((tau_flags & kScratchInGlobal) ? 2 * nn : 0));
}

cudaError_t launch_green_tau(const ChainDesc* d_descs, int n_chains, size_t smem, cudaStream_t stream) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(green_tau_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    green_tau_kernel<<<dim3(n_chains, 2), kNT, smem, stream>>>(d_descs);
    return cudaGetLastError();
}

}  // namespace lqmc

// ---------------------------------------------------------------------------------------
// Allocation-free single-chain entry point (lqmc_sweep_static, include/lqmc_gpu.h).
// The chain descriptor and the UDT scratch of the sweep live in one static device array;
// the unchanged sweep kernel runs on it.
// ---------------------------------------------------------------------------------------
#include <cstdio>
#include <mutex>

namespace {

constexpr size_t kStaticDescBytes = 512;   // ChainDesc slot at the start of the array
static_assert(sizeof(lqmc::ChainDesc) <= kStaticDescBytes, "descriptor slot too small");
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[LQMC_STATIC_SCRATCH_BYTES];

std::mutex g_static_mutex;
void* g_static_addr[kStaticMaxDevices];   // device address of g_static_scratch, per device

int static_fail(const lqmc_static_chain* c, int code, const char* msg) {
    if (c && c->error_message && c->error_capacity) {
        std::snprintf(c->error_message, c->error_capacity, "%s", msg);
    }
    return code;
}

}  // namespace

extern "C" int lqmc_sweep_static(const lqmc_static_chain* c, int32_t n_sweeps, void* stream) {
    if (!c) return LQMC_ERR_INVALID;
    if (n_sweeps < 0) return static_fail(c, LQMC_ERR_INVALID, "n_sweeps < 0");
    const int n = c->n_sites, L = c->n_slices;
    if (n < 1 || n > LQMC_STATIC_MAX_SITES || L < 1 || c->stab_every < 1)
        return static_fail(c, LQMC_ERR_INVALID,
                           "lqmc_sweep_static: needs 1 <= n_sites <= 64, n_slices >= 1, stab_every >= 1");
    if (c->rng != LQMC_RNG_REPLAY && c->rng != LQMC_RNG_PHILOX)
        return static_fail(c, LQMC_ERR_INVALID, "lqmc_sweep_static: unknown rng");
    if (!c->exp_k || !c->exp_k_t || !c->exp_k_inv || !c->exp_k_inv_t || !c->kinetic || !c->field ||
        !c->green || !c->green_sum || !c->obs || !c->diag || !c->status ||
        (c->rng == LQMC_RNG_REPLAY && !c->uniforms))
        return static_fail(c, LQMC_ERR_INVALID, "lqmc_sweep_static: null device pointer");
    const int stab = c->stab_every < L ? c->stab_every : L;
    const int chunks = (L + stab - 1) / stab;
    const size_t slot = ((size_t)2 * n * n + n + 1 + 3) / 4 * 4;
    const size_t need = kStaticDescBytes + (size_t)(2 * chunks + 4) * slot * sizeof(double);
    if (need > LQMC_STATIC_SCRATCH_BYTES) {
        char msg[200];
        std::snprintf(msg, sizeof(msg),
                      "lqmc_sweep_static: %zu bytes of scratch needed for n_sites=%d and %d "
                      "chunks; the static array holds %u", need, n, chunks,
                      (unsigned)LQMC_STATIC_SCRATCH_BYTES);
        return static_fail(c, LQMC_ERR_INVALID, msg);
    }
    if (n_sweeps == 0) return LQMC_OK;

    // set-up, once per device, with that device current: the array's device address
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return static_fail(c, LQMC_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kStaticMaxDevices) return static_fail(c, LQMC_ERR_CUDA, "device ordinal too large");
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_static_mutex);
        if (!g_static_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess || !p) return static_fail(c, LQMC_ERR_CUDA, cudaGetErrorString(e));
            g_static_addr[dev] = p;
        }
        base = static_cast<unsigned char*>(g_static_addr[dev]);
    }

    lqmc::ChainDesc d{};
    d.n = n;
    d.L = L;
    d.stab_every = stab;
    d.n_chunks = chunks;
    d.mode = LQMC_MODE_DQMC;
    d.rng = c->rng;
    d.record = 0;
    d.flags = 0;   // n <= 64: G and both scratch matrices fit in shared memory
    d.chain_id = c->chain_id;
    d.slot = (int32_t)slot;
    d.seed = c->seed;
    for (int k = 0; k < 4; ++k) d.c[k] = c->exp_consts[k];
    d.u = c->u;
    d.drift_tol = 1e-6;
    d.expk = c->exp_k;
    d.expkT = c->exp_k_t;
    d.expkinv = c->exp_k_inv;
    d.expkinvT = c->exp_k_inv_t;
    d.kinetic = c->kinetic;
    d.field = c->field;
    d.green = c->green;
    d.gsum = c->green_sum;
    d.obs = c->obs;
    d.diag = c->diag;
    d.work = reinterpret_cast<double*>(base + kStaticDescBytes);
    d.uniforms = c->uniforms;
    d.decisions = nullptr;
    d.status = c->status;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemcpyAsync(base, &d, sizeof(d), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return static_fail(c, LQMC_ERR_CUDA, cudaGetErrorString(e));
    e = lqmc::launch_sweep_fp64(reinterpret_cast<const lqmc::ChainDesc*>(base), 1,
                                lqmc::sweep_fp64_smem_bytes(n, 0), n_sweeps, c->measure ? 1 : 0, 0, st);
    if (e != cudaSuccess) return static_fail(c, LQMC_ERR_CUDA, cudaGetErrorString(e));
    return LQMC_OK;
}

