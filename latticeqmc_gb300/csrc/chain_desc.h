// Per-chain descriptor shared by the host (capi.cu) and the sweep kernels.
#pragma once
#include <stdint.h>

namespace lqmc {

// desc.flags bits
enum : int32_t {
    kGreenInGlobal = 1,    // G_up/G_dn live in desc.work instead of shared memory
    kScratchInGlobal = 2,  // the two n x n scratch buffers live in desc.work
    kUpdatesInGlobal = 4,  // tiled kernel: the delayed-update buffers X, Y live in desc.work
};

struct ChainDesc {
    int32_t n;            // sites
    int32_t L;            // time slices
    int32_t stab_every;   // slices per UDT chunk (dqmc)
    int32_t n_chunks;     // ceil(L / stab_every)
    int32_t mode;         // LQMC_MODE_*
    int32_t rng;          // LQMC_RNG_*
    int32_t record;       // keep accept decisions
    int32_t flags;        // kGreenInGlobal | kScratchInGlobal
    int32_t chain_id;     // philox key word 1
    int32_t slot;         // doubles per UDT slot (2 n^2 + n, padded)
    uint64_t seed;        // philox key word 0
    double c[4];          // exp(2 lam), exp(-2 lam), exp(-lam), exp(+lam)
    double u;             // Hubbard U (potential energy)
    double drift_tol;     // residual above which LQMC_STATUS_DRIFT is set
    const double* expk;       // expm(-dtau K), row-major
    const double* expkT;      // its transpose
    const double* expkinv;    // compat: inv(expk); dqmc: expm(+dtau K)
    const double* expkinvT;   // its transpose
    const double* kinetic;    // K
    int8_t* field;            // [L][n]
    double* green;            // [2][n][n] G after the last sweep
    double* gsum;             // [2][n][n] measurement sum of G
    double* obs;              // LQMC_OBS_LEN(n)
    double* diag;             // LQMC_DIAG_LEN
    double* work;             // UDT stacks, left products, spilled G / scratch
    const double* uniforms;   // replay: [n_sweeps][n L]
    int8_t* decisions;        // [n_sweeps][L][n] (record)
    int32_t* status;          // LQMC_STATUS_* bits
    const float* expk_f;      // float copies of expk / expkinv (mixed-precision engine)
    const float* expkinv_f;
    int32_t delay;            // tiled kernel: rank-k depth of the delayed updates (>= 1)
    int32_t oz_stages;        // tiled kernel, emulated GEMMs: tensor-core stage buffers (1 or 2)
    int32_t debug;            // LQMC_DEBUG_* bits
    int32_t native;           // LQMC_FP64E_NATIVE_* bits (emulated-GEMM kernel)
    double* gtau;             // [2][L][n][n] measurement sum of G(tau_l, 0), or null
    double* tau_work;         // per spin: (n_chunks + 1) UDT slots, then X (+ scratch)
    int32_t tau_flags;        // kScratchInGlobal: the G(tau) kernel's two scratch matrices
    int32_t tau_pad;
    const unsigned char* presplit;   // emulated-GEMM kernel: the split constant operands,
                                     // shared by the chains with the same e^{-dtau K}
    int32_t order;            // LQMC_ORDER_* (tiled kernel)
    int32_t order_pad;
};

}  // namespace lqmc
