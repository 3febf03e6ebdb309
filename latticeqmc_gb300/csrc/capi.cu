// C ABI of liblqmc_gpu.so (declared in include/lqmc_gpu.h): handle, device memory, launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "chain_desc.h"
#include "lqmc_gpu.h"

namespace lqmc {
size_t sweep_fp64_smem_bytes(int n, int flags);
cudaError_t launch_sweep_fp64(const ChainDesc* d_descs, int n_chains, size_t smem, int n_sweeps,
                              int measure, int sweep_base, cudaStream_t stream);
size_t green_tau_smem_bytes(int n, int tau_flags);
size_t green_tau_work_doubles(int n, int n_chunks, int slot, int tau_flags);
cudaError_t launch_green_tau(const ChainDesc* d_descs, int n_chains, size_t smem, cudaStream_t stream);
size_t sweep_tiled_smem_bytes(int n, bool fp32, int delay, bool emu, int stages, bool xy_global);
int sweep_tiled_delay_target(bool fp32, int requested, bool emu);
int sweep_tiled_delay(int n, bool fp32, int requested, size_t cap, bool emu, int stages);
size_t sweep_tiled_work_bytes(int n, int n_chunks, bool fp32, bool emu, int xy_delay, bool alt);
size_t sweep_tiled_presplit_bytes(int n);
cudaError_t launch_presplit(const void* d_jobs, int count, cudaStream_t stream);
size_t sweep_tiled_presplit_job_bytes();
void sweep_tiled_presplit_job(void* job, const double* expk, const double* expkinv,
                              unsigned char* out, int n);
cudaError_t launch_sweep_tiled(const ChainDesc* d_descs, int n_chains, size_t smem, int precision,
                               int n_sweeps, int measure, int sweep_base, cudaStream_t stream);
}  // namespace lqmc

using lqmc::ChainDesc;

namespace {

constexpr int kMaxSitesSmem = 128;    // one-CTA shared-memory kernel (both modes)
constexpr int kMaxSitesTiled = 1024;  // tiled kernel (dqmc mode): 4 rows per thread
constexpr int kMaxOzStages = 3;       // stage buffers of the emulated GEMM

// which sweep kernel runs a chain
enum Kind : int { kSmemFp64 = 0, kTiledFp64 = 1, kTiledFp32 = 2, kTiledFp64e = 3 };
constexpr size_t kAlign = 32;   // doubles (256 bytes) between device sub-buffers

std::string g_create_error;

struct Bucket {
    int kind = kSmemFp64;
    size_t smem = 0;
    size_t tau_smem = 0;   // green_tau_kernel (params.measure_tau)
    std::vector<int> chains;
    ChainDesc* d_descs = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct lqmc_handle {
    lqmc_params p{};
    std::string err;
    int n_chains = 0;
    std::vector<ChainDesc> desc;
    std::vector<char> field_set;
    double* d_uni = nullptr;           // [chain][sweep][n L], chain c at uni_cap * uni_off[c]
    size_t uni_cap = 0;                // sweeps of uniforms each chain's region holds
    std::vector<size_t> uni_off;       // prefix sums of n L
    size_t uni_total = 0;              // sum of n L
    std::vector<size_t> uni_count;     // uniforms uploaded and not yet consumed, per chain
    double* d_green = nullptr;         // [chain][2][n][n], contiguous
    std::vector<size_t> green_off;
    size_t green_total = 0;
    double* d_f64 = nullptr;
    int8_t* d_i8 = nullptr;
    int32_t* d_status = nullptr;
    int8_t* d_dec = nullptr;
    size_t dec_cap = 0;
    unsigned char* d_pre = nullptr;    // split constant operands of the emulated GEMMs
    std::vector<Bucket> buckets;
    cudaEvent_t fork = nullptr;
    cudaStream_t last_stream = nullptr;
    int last_sweeps = 0;
    int64_t launches = 0;
    bool descs_dirty = true;
};

namespace {

int fail(lqmc_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    else g_create_error = msg;
    return code;
}

int cuda_fail(lqmc_handle* h, cudaError_t e, const char* what) {
    return fail(h, LQMC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define LQMC_CK(h, call)                                      \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call); \
    } while (0)

void release(lqmc_handle* h) {
    for (auto& b : h->buckets) {
        if (b.d_descs) cudaFree(b.d_descs);
        if (b.stream) cudaStreamDestroy(b.stream);
        if (b.done) cudaEventDestroy(b.done);
    }
    h->buckets.clear();
    if (h->d_uni) cudaFree(h->d_uni);
    h->d_uni = nullptr;
    h->uni_cap = 0;
    if (h->d_green) cudaFree(h->d_green);
    h->d_green = nullptr;
    if (h->d_f64) cudaFree(h->d_f64);
    if (h->d_i8) cudaFree(h->d_i8);
    if (h->d_status) cudaFree(h->d_status);
    if (h->d_dec) cudaFree(h->d_dec);
    if (h->d_pre) cudaFree(h->d_pre);
    h->d_pre = nullptr;
    h->d_f64 = nullptr;
    h->d_i8 = nullptr;
    h->d_status = nullptr;
    h->d_dec = nullptr;
    h->dec_cap = 0;
    h->n_chains = 0;
    h->desc.clear();
}

int check_chain(lqmc_handle* h, int32_t chain) {
    if (!h) return LQMC_ERR_INVALID;
    if (h->n_chains == 0) return fail(h, LQMC_ERR_STATE, "no chains defined (call lqmc_set_chains)");
    if (chain < 0 || chain >= h->n_chains) return fail(h, LQMC_ERR_INVALID, "chain index out of range");
    return LQMC_OK;
}

int sync_last(lqmc_handle* h) {
    cudaError_t e = h->last_stream ? cudaStreamSynchronize(h->last_stream) : cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
    return LQMC_OK;
}

}  // namespace

extern "C" {

int lqmc_abi_version(void) { return LQMC_ABI_VERSION; }

int lqmc_create(const lqmc_params* params, lqmc_handle** out) {
    if (!params || !out) return fail(nullptr, LQMC_ERR_INVALID, "null argument");
    *out = nullptr;
    if (params->mode != LQMC_MODE_COMPAT && params->mode != LQMC_MODE_DQMC && params->mode != LQMC_MODE_DET)
        return fail(nullptr, LQMC_ERR_INVALID, "unknown mode");
    if (params->precision != LQMC_PREC_FP64 && params->precision != LQMC_PREC_MIXED &&
        params->precision != LQMC_PREC_FP64E)
        return fail(nullptr, LQMC_ERR_INVALID, "unknown precision");
    if (params->rng != LQMC_RNG_REPLAY && params->rng != LQMC_RNG_PHILOX)
        return fail(nullptr, LQMC_ERR_INVALID, "unknown rng");
    if (params->engine < LQMC_ENGINE_AUTO || params->engine > LQMC_ENGINE_TILED)
        return fail(nullptr, LQMC_ERR_INVALID, "unknown engine");
    if (params->engine == LQMC_ENGINE_SMEM && params->precision == LQMC_PREC_MIXED)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "the shared-memory kernel is float64 only");
    if (params->engine == LQMC_ENGINE_TILED && params->mode != LQMC_MODE_DQMC)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "compat and det modes run on the shared-memory kernel only");
    if (params->stab_every < 0 || params->delay < 0)
        return fail(nullptr, LQMC_ERR_INVALID, "negative stab_every or delay");
    if (params->precision != LQMC_PREC_FP64 && params->mode != LQMC_MODE_DQMC)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "compat and det modes replay float64 arithmetic only");
    if (params->engine == LQMC_ENGINE_SMEM && params->precision == LQMC_PREC_FP64E)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "the shared-memory kernel has no emulated GEMM");
    if (params->measure_tau != 0 && params->measure_tau != 1)
        return fail(nullptr, LQMC_ERR_INVALID, "measure_tau must be 0 or 1");
    if (params->measure_tau && params->mode != LQMC_MODE_DQMC)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "the unequal-time G is measured in dqmc mode only");
    if (params->oz_stages < 0 || params->oz_stages > kMaxOzStages)
        return fail(nullptr, LQMC_ERR_INVALID, "oz_stages out of range");
    if (params->sweep_order != LQMC_ORDER_DOWN && params->sweep_order != LQMC_ORDER_ALTERNATE)
        return fail(nullptr, LQMC_ERR_INVALID, "unknown sweep order");
    if (params->sweep_order == LQMC_ORDER_ALTERNATE && params->mode != LQMC_MODE_DQMC)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "the alternating sweep order is a dqmc-mode order");
    if (params->sweep_order == LQMC_ORDER_ALTERNATE && params->engine == LQMC_ENGINE_SMEM)
        return fail(nullptr, LQMC_ERR_UNSUPPORTED, "the alternating sweep order runs on the tiled kernel");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return fail(nullptr, LQMC_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    if (params->device < 0 || params->device >= ndev) return fail(nullptr, LQMC_ERR_INVALID, "device ordinal out of range");
    e = cudaSetDevice(params->device);
    if (e != cudaSuccess) return fail(nullptr, LQMC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    lqmc_handle* h = new lqmc_handle();
    h->p = *params;
    if (h->p.stab_every == 0) h->p.stab_every = 10;
    e = cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete h;
        return fail(nullptr, LQMC_ERR_CUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
    }
    *out = h;
    return LQMC_OK;
}

int lqmc_set_chains(lqmc_handle* h, int32_t n_chains, const int32_t* n_sites,
                    const int32_t* n_slices, const double* const* exp_k,
                    const double* const* exp_k_inv, const double* const* kinetic,
                    const double* exp_consts, const double* u) {
    if (!h) return LQMC_ERR_INVALID;
    if (n_chains <= 0 || !n_sites || !n_slices || !exp_k || !exp_k_inv || !kinetic || !exp_consts || !u)
        return fail(h, LQMC_ERR_INVALID, "lqmc_set_chains: null argument or n_chains <= 0");
    LQMC_CK(h, cudaSetDevice(h->p.device));
    for (int c = 0; c < n_chains; ++c) {
        if (n_sites[c] < 1 || n_slices[c] < 1)
            return fail(h, LQMC_ERR_INVALID, "chain " + std::to_string(c) + ": n_sites and n_slices must be >= 1");
        if (h->p.mode != LQMC_MODE_DQMC && n_sites[c] > kMaxSitesSmem)
            return fail(h, LQMC_ERR_UNSUPPORTED, "chain " + std::to_string(c) +
                        ": compat and det modes run on the shared-memory kernel, n_sites <= 128");
        if (h->p.engine == LQMC_ENGINE_SMEM && n_sites[c] > kMaxSitesSmem)
            return fail(h, LQMC_ERR_UNSUPPORTED, "chain " + std::to_string(c) +
                        ": the shared-memory kernel holds n_sites <= 128");
        if (n_sites[c] > kMaxSitesTiled)
            return fail(h, LQMC_ERR_UNSUPPORTED, "chain " + std::to_string(c) + ": n_sites > 1024");
        if (!exp_k[c] || !exp_k_inv[c] || !kinetic[c])
            return fail(h, LQMC_ERR_INVALID, "chain " + std::to_string(c) + ": null matrix");
    }
    release(h);
    int dev = h->p.device;
    int optin = 0;
    LQMC_CK(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t smem_cap = (size_t)optin - 1024;   // static shared memory of the kernel

    h->n_chains = n_chains;
    h->desc.assign(n_chains, ChainDesc{});
    h->field_set.assign(n_chains, 0);
    h->uni_count.assign(n_chains, 0);
    h->uni_off.assign(n_chains, 0);
    h->green_off.assign(n_chains, 0);
    h->uni_total = 0;
    h->green_total = 0;
    for (int c = 0; c < n_chains; ++c) {
        h->uni_off[c] = h->uni_total;
        h->uni_total += (size_t)n_sites[c] * n_slices[c];
        h->green_off[c] = h->green_total;
        h->green_total += 2 * (size_t)n_sites[c] * n_sites[c];
    }

    // layout of the float64 arena
    std::vector<size_t> off(n_chains);
    std::vector<size_t> smem(n_chains);
    std::vector<int> kind(n_chains);
    size_t total = 0, total_i8 = 0;
    std::vector<size_t> off_i8(n_chains);
    for (int c = 0; c < n_chains; ++c) {
        ChainDesc& d = h->desc[c];
        const int n = n_sites[c], L = n_slices[c];
        const size_t nn = (size_t)n * n;
        d.n = n;
        d.L = L;
        d.mode = h->p.mode;
        d.rng = h->p.rng;
        d.stab_every = std::min(h->p.stab_every, L);
        d.n_chunks = (h->p.mode == LQMC_MODE_DQMC) ? (L + d.stab_every - 1) / d.stab_every : 0;
        d.chain_id = c;
        d.seed = h->p.seed;
        d.slot = (int32_t)round_up(2 * nn + n + 1, 4);
        for (int k = 0; k < 4; ++k) d.c[k] = exp_consts[4 * c + k];
        d.u = u[c];
        d.drift_tol = 1e-6;
        d.debug = h->p.debug;
        d.native = h->p.fp64e_native;
        d.order = h->p.sweep_order;
        if (h->p.precision == LQMC_PREC_MIXED) kind[c] = kTiledFp32;
        else if (h->p.precision == LQMC_PREC_FP64E) kind[c] = kTiledFp64e;
        else if (h->p.engine == LQMC_ENGINE_TILED || h->p.sweep_order == LQMC_ORDER_ALTERNATE) kind[c] = kTiledFp64;
        else kind[c] = (n <= kMaxSitesSmem) ? kSmemFp64 : kTiledFp64;
        if (kind[c] == kSmemFp64 && h->p.engine == LQMC_ENGINE_SMEM && n > kMaxSitesSmem) {
            release(h);
            return fail(h, LQMC_ERR_UNSUPPORTED, "the shared-memory kernel holds n_sites <= 128");
        }
        size_t work = 0;
        if (kind[c] == kSmemFp64) {
            int flags = 0;
            if (lqmc::sweep_fp64_smem_bytes(n, flags) > smem_cap) flags = lqmc::kScratchInGlobal;
            if (lqmc::sweep_fp64_smem_bytes(n, flags) > smem_cap) flags |= lqmc::kGreenInGlobal;
            d.flags = flags;
            smem[c] = lqmc::sweep_fp64_smem_bytes(n, flags);
            work = (size_t)(2 * d.n_chunks + 4) * d.slot;
            if (flags & lqmc::kGreenInGlobal) work += 2 * nn;
            if (flags & lqmc::kScratchInGlobal) work += 2 * nn;
        } else {
            const bool f32 = kind[c] == kTiledFp32, emu = kind[c] == kTiledFp64e;
            d.flags = 0;
            // the delayed-update buffers in shared memory when the target depth fits there,
            // else in global memory.  Tensor-core stage buffers (fp64e): the requested count,
            // else three where they fit, else two, else one; a count that does not fit beside
            // the delayed-update buffers moves them to global memory (same depth) -- at 16x16
            // the deeper copy ring gains more (3 % of the sweep) than their shared-memory
            // residence.
            const int target = lqmc::sweep_tiled_delay_target(f32, h->p.delay, emu);
            d.oz_stages = 1;
            d.delay = lqmc::sweep_tiled_delay(n, f32, h->p.delay, smem_cap, emu, 1);
            bool xy_global = false;
            if (d.delay < target) {
                xy_global = true;
                d.delay = target;
                d.flags |= lqmc::kUpdatesInGlobal;
            }
            const int want = emu ? h->p.oz_stages : 0;
            for (int st = emu ? (want > 0 ? want : kMaxOzStages) : 1; st > 1; --st) {
                if (lqmc::sweep_tiled_smem_bytes(n, f32, d.delay, emu, st, xy_global) <= smem_cap) {
                    d.oz_stages = st;
                    break;
                }
                if (!xy_global && lqmc::sweep_tiled_smem_bytes(n, f32, target, emu, st, true) <= smem_cap) {
                    xy_global = true;
                    d.delay = target;
                    d.flags |= lqmc::kUpdatesInGlobal;
                    d.oz_stages = st;
                    break;
                }
                if (want > 0) {
                    release(h);
                    return fail(h, LQMC_ERR_UNSUPPORTED, "the requested stage buffers do not fit in shared memory");
                }
            }
            smem[c] = lqmc::sweep_tiled_smem_bytes(n, f32, d.delay, emu, d.oz_stages, xy_global);
            work = (lqmc::sweep_tiled_work_bytes(n, d.n_chunks, f32, emu, xy_global ? d.delay : 0,
                                                 d.order == LQMC_ORDER_ALTERNATE) + 7) / 8;
            if (smem[c] > smem_cap) { release(h); return fail(h, LQMC_ERR_UNSUPPORTED, "lattice too large for shared memory"); }
        }
        const size_t fcopy = (kind[c] == kTiledFp32) ? 2 * round_up((nn + 1) / 2, kAlign) : 0;
        size_t tau = 0;
        d.tau_flags = 0;
        if (h->p.measure_tau) {
            if (lqmc::green_tau_smem_bytes(n, 0) > smem_cap) d.tau_flags = lqmc::kScratchInGlobal;
            if (lqmc::green_tau_smem_bytes(n, d.tau_flags) > smem_cap) {
                release(h);
                return fail(h, LQMC_ERR_UNSUPPORTED, "lattice too large for the unequal-time G kernel");
            }
            tau = round_up(2 * (size_t)L * nn, kAlign) +
                  round_up(lqmc::green_tau_work_doubles(n, d.n_chunks, d.slot, d.tau_flags), kAlign);
        }
        const size_t need = round_up(nn, kAlign) * 5 + fcopy + round_up(2 * nn, kAlign) +
                            round_up(LQMC_OBS_LEN(n), kAlign) + round_up(LQMC_DIAG_LEN, kAlign) +
                            tau + round_up(work, kAlign);
        off[c] = total;
        total += need;
        off_i8[c] = total_i8;
        total_i8 += round_up((size_t)n * L, 256);
    }
    cudaError_t e = cudaMalloc(&h->d_f64, total * sizeof(double));
    if (e != cudaSuccess) { release(h); return fail(h, LQMC_ERR_NOMEM, "device allocation of " + std::to_string(total * 8) + " bytes failed"); }
    e = cudaMalloc(&h->d_green, h->green_total * sizeof(double));
    if (e != cudaSuccess) { release(h); return fail(h, LQMC_ERR_NOMEM, "device allocation of G failed"); }
    e = cudaMalloc(&h->d_i8, total_i8);
    if (e != cudaSuccess) { release(h); return fail(h, LQMC_ERR_NOMEM, "device allocation of the fields failed"); }
    e = cudaMalloc(&h->d_status, sizeof(int32_t) * n_chains);
    if (e != cudaSuccess) { release(h); return fail(h, LQMC_ERR_NOMEM, "device allocation of the status words failed"); }
    LQMC_CK(h, cudaMemset(h->d_f64, 0, total * sizeof(double)));
    LQMC_CK(h, cudaMemset(h->d_green, 0, h->green_total * sizeof(double)));
    LQMC_CK(h, cudaMemset(h->d_i8, 1, total_i8));
    LQMC_CK(h, cudaMemset(h->d_status, 0, sizeof(int32_t) * n_chains));

    std::vector<double> tmp;
    for (int c = 0; c < n_chains; ++c) {
        ChainDesc& d = h->desc[c];
        const int n = d.n;
        const size_t nn = (size_t)n * n;
        double* p = h->d_f64 + off[c];
        auto take = [&](size_t count) { double* r = p; p += round_up(count, kAlign); return r; };
        double* ek = take(nn);
        double* ekt = take(nn);
        double* eki = take(nn);
        double* ekit = take(nn);
        double* kin = take(nn);
        float* ekf = nullptr;
        float* ekif = nullptr;
        if (kind[c] == kTiledFp32) {
            ekf = reinterpret_cast<float*>(take((nn + 1) / 2));
            ekif = reinterpret_cast<float*>(take((nn + 1) / 2));
        }
        d.green = h->d_green + h->green_off[c];
        d.gsum = take(2 * nn);
        d.obs = take(LQMC_OBS_LEN(n));
        d.diag = take(LQMC_DIAG_LEN);
        d.gtau = nullptr;
        d.tau_work = nullptr;
        if (h->p.measure_tau) {
            d.gtau = take(2 * (size_t)d.L * nn);
            d.tau_work = take(lqmc::green_tau_work_doubles(n, d.n_chunks, d.slot, d.tau_flags));
        }
        d.work = p;
        d.expk = ek;
        d.expkT = ekt;
        d.expkinv = eki;
        d.expkinvT = ekit;
        d.kinetic = kin;
        d.field = h->d_i8 + off_i8[c];
        d.status = h->d_status + c;
        tmp.resize(nn);
        LQMC_CK(h, cudaMemcpy(ek, exp_k[c], nn * sizeof(double), cudaMemcpyHostToDevice));
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) tmp[(size_t)j * n + i] = exp_k[c][(size_t)i * n + j];
        LQMC_CK(h, cudaMemcpy(ekt, tmp.data(), nn * sizeof(double), cudaMemcpyHostToDevice));
        LQMC_CK(h, cudaMemcpy(eki, exp_k_inv[c], nn * sizeof(double), cudaMemcpyHostToDevice));
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) tmp[(size_t)j * n + i] = exp_k_inv[c][(size_t)i * n + j];
        LQMC_CK(h, cudaMemcpy(ekit, tmp.data(), nn * sizeof(double), cudaMemcpyHostToDevice));
        LQMC_CK(h, cudaMemcpy(kin, kinetic[c], nn * sizeof(double), cudaMemcpyHostToDevice));
        if (ekf) {
            std::vector<float> tf(nn);
            for (size_t e = 0; e < nn; ++e) tf[e] = (float)exp_k[c][e];
            LQMC_CK(h, cudaMemcpy(ekf, tf.data(), nn * sizeof(float), cudaMemcpyHostToDevice));
            for (size_t e = 0; e < nn; ++e) tf[e] = (float)exp_k_inv[c][e];
            LQMC_CK(h, cudaMemcpy(ekif, tf.data(), nn * sizeof(float), cudaMemcpyHostToDevice));
        }
        d.expk_f = ekf;
        d.expkinv_f = ekif;
    }

    // the emulated-GEMM chains' constant operands, split once and shared by every chain with
    // the same e^{-dtau K} and e^{+dtau K} (the same lattice and dtau)
    {
        std::vector<int> leader(n_chains, -1);
        std::vector<int> groups_of;   // leader chain of each group
        for (int c = 0; c < n_chains; ++c) {
            if (kind[c] != kTiledFp64e) continue;
            const size_t nn = (size_t)n_sites[c] * n_sites[c];
            for (int g : groups_of) {
                if (n_sites[g] == n_sites[c] && !std::memcmp(exp_k[g], exp_k[c], nn * sizeof(double)) &&
                    !std::memcmp(exp_k_inv[g], exp_k_inv[c], nn * sizeof(double))) {
                    leader[c] = g;
                    break;
                }
            }
            if (leader[c] < 0) {
                leader[c] = c;
                groups_of.push_back(c);
            }
        }
        if (!groups_of.empty()) {
            std::map<int, size_t> pre_off;
            size_t pre_total = 0;
            for (int g : groups_of) {
                pre_off[g] = pre_total;
                pre_total += round_up(lqmc::sweep_tiled_presplit_bytes(n_sites[g]), 256);
            }
            e = cudaMalloc(&h->d_pre, pre_total);
            if (e != cudaSuccess) { release(h); return fail(h, LQMC_ERR_NOMEM, "device allocation of the split constants failed"); }
            const size_t jb = lqmc::sweep_tiled_presplit_job_bytes();
            std::vector<unsigned char> jobs(jb * groups_of.size());
            for (size_t k = 0; k < groups_of.size(); ++k) {
                const int g = groups_of[k];
                lqmc::sweep_tiled_presplit_job(jobs.data() + k * jb, h->desc[g].expk, h->desc[g].expkinv,
                                               h->d_pre + pre_off[g], n_sites[g]);
            }
            void* d_jobs = nullptr;
            e = cudaMalloc(&d_jobs, jobs.size());
            if (e != cudaSuccess) { release(h); return fail(h, LQMC_ERR_NOMEM, "presplit job allocation failed"); }
            e = cudaMemcpy(d_jobs, jobs.data(), jobs.size(), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = lqmc::launch_presplit(d_jobs, (int)groups_of.size(), nullptr);
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
            cudaFree(d_jobs);
            if (e != cudaSuccess) { release(h); return cuda_fail(h, e, "splitting the constant operands"); }
            for (int c = 0; c < n_chains; ++c)
                if (leader[c] >= 0) h->desc[c].presplit = h->d_pre + pre_off[leader[c]];
        }
    }

    // buckets of equal shared-memory footprint, largest first
    // buckets of one kernel and one shared-memory footprint; the largest lattices first
    std::map<std::pair<int, size_t>, std::vector<int>> groups;
    for (int c = 0; c < n_chains; ++c) groups[{-h->desc[c].n, (size_t)kind[c]}].push_back(c);
    for (auto& kv : groups) {
        Bucket b;
        b.kind = (int)kv.first.second;
        b.smem = smem[kv.second[0]];
        b.chains = kv.second;
        if (h->p.measure_tau) b.tau_smem = lqmc::green_tau_smem_bytes(h->desc[b.chains[0]].n, h->desc[b.chains[0]].tau_flags);
        e = cudaMalloc(&b.d_descs, sizeof(ChainDesc) * b.chains.size());
        if (e != cudaSuccess) { h->buckets.push_back(b); release(h); return fail(h, LQMC_ERR_NOMEM, "descriptor allocation failed"); }
        e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming);
        h->buckets.push_back(b);
        if (e != cudaSuccess) { release(h); return cuda_fail(h, e, "bucket stream/event"); }
    }
    h->descs_dirty = true;
    return LQMC_OK;
}

int lqmc_set_field(lqmc_handle* h, int32_t chain, const int8_t* field) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!field) return fail(h, LQMC_ERR_INVALID, "null field");
    const ChainDesc& d = h->desc[chain];
    std::vector<int8_t> t((size_t)d.n * d.L);
    for (int i = 0; i < d.n; ++i)
        for (int l = 0; l < d.L; ++l) {
            const int8_t v = field[(size_t)i * d.L + l];
            if (v != 1 && v != -1) return fail(h, LQMC_ERR_INVALID, "field values must be +1 or -1");
            t[(size_t)l * d.n + i] = v;
        }
    {
        const int r = sync_last(h);
        if (r) return r;
    }
    LQMC_CK(h, cudaMemcpy(d.field, t.data(), t.size(), cudaMemcpyHostToDevice));
    // a new field invalidates the products the alternating order keeps between sweeps
    LQMC_CK(h, cudaMemset(d.diag + 21, 0, sizeof(double)));
    h->field_set[chain] = 1;
    return LQMC_OK;
}

int lqmc_get_field(lqmc_handle* h, int32_t chain, int8_t* field) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!field) return fail(h, LQMC_ERR_INVALID, "null field");
    if ((rc = sync_last(h))) return rc;
    const ChainDesc& d = h->desc[chain];
    std::vector<int8_t> t((size_t)d.n * d.L);
    LQMC_CK(h, cudaMemcpy(t.data(), d.field, t.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < d.n; ++i)
        for (int l = 0; l < d.L; ++l) field[(size_t)i * d.L + l] = t[(size_t)l * d.n + i];
    return LQMC_OK;
}

// Grow (or, with exact = true, resize) the uniform arena to `sweeps` sweeps per chain,
// keeping every chain's pending uniforms.
static int ensure_uniform_capacity(lqmc_handle* h, size_t sweeps, bool exact) {
    if (sweeps <= h->uni_cap && !(exact && sweeps != h->uni_cap)) return LQMC_OK;
    for (int c = 0; c < h->n_chains; ++c)
        if ((size_t)h->uni_count[c] > sweeps * h->desc[c].n * h->desc[c].L) sweeps = h->uni_cap;
    if (sweeps == h->uni_cap) return LQMC_OK;
    double* fresh = nullptr;
    cudaError_t e = cudaMalloc(&fresh, std::max<size_t>(1, sweeps * h->uni_total) * sizeof(double));
    if (e != cudaSuccess) return fail(h, LQMC_ERR_NOMEM, "uniform buffer allocation failed");
    for (int c = 0; c < h->n_chains; ++c) {
        if (h->uni_count[c]) {
            e = cudaMemcpy(fresh + sweeps * h->uni_off[c], h->d_uni + h->uni_cap * h->uni_off[c],
                           h->uni_count[c] * sizeof(double), cudaMemcpyDeviceToDevice);
            if (e != cudaSuccess) { cudaFree(fresh); return cuda_fail(h, e, "uniform buffer copy"); }
        }
    }
    if (h->d_uni) cudaFree(h->d_uni);
    h->d_uni = fresh;
    h->uni_cap = sweeps;
    for (int c = 0; c < h->n_chains; ++c) h->desc[c].uniforms = h->d_uni + sweeps * h->uni_off[c];
    h->descs_dirty = true;
    return LQMC_OK;
}

int lqmc_set_uniforms(lqmc_handle* h, int32_t chain, const double* uniforms, size_t count) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (h->p.rng != LQMC_RNG_REPLAY) return fail(h, LQMC_ERR_STATE, "uniforms are only uploaded in replay mode");
    if (!uniforms && count) return fail(h, LQMC_ERR_INVALID, "null uniforms");
    const ChainDesc& d = h->desc[chain];
    const size_t per = (size_t)d.n * d.L;
    if (count % per) return fail(h, LQMC_ERR_INVALID, "uniform count must be a multiple of n_sites * n_slices");
    if ((rc = sync_last(h))) return rc;
    h->uni_count[chain] = 0;
    if ((rc = ensure_uniform_capacity(h, count / per, false))) return rc;
    if (count)
        LQMC_CK(h, cudaMemcpy(h->d_uni + h->uni_cap * h->uni_off[chain], uniforms,
                              count * sizeof(double), cudaMemcpyHostToDevice));
    h->uni_count[chain] = count;
    return LQMC_OK;
}

int lqmc_set_uniforms_all(lqmc_handle* h, const double* uniforms, size_t count) {
    if (!h) return LQMC_ERR_INVALID;
    if (h->n_chains == 0) return fail(h, LQMC_ERR_STATE, "no chains defined (call lqmc_set_chains)");
    if (h->p.rng != LQMC_RNG_REPLAY) return fail(h, LQMC_ERR_STATE, "uniforms are only uploaded in replay mode");
    if (!uniforms || count == 0 || count % h->uni_total)
        return fail(h, LQMC_ERR_INVALID, "uniform count must be a positive multiple of sum(n_sites * n_slices)");
    int rc = sync_last(h);
    if (rc) return rc;
    const size_t sweeps = count / h->uni_total;
    for (int c = 0; c < h->n_chains; ++c) h->uni_count[c] = 0;
    if ((rc = ensure_uniform_capacity(h, sweeps, true))) return rc;
    // the arena layout [chain][sweep][n L] equals the concatenation the caller passes
    LQMC_CK(h, cudaMemcpy(h->d_uni, uniforms, count * sizeof(double), cudaMemcpyHostToDevice));
    for (int c = 0; c < h->n_chains; ++c) h->uni_count[c] = sweeps * h->desc[c].n * h->desc[c].L;
    return LQMC_OK;
}

int lqmc_sweep(lqmc_handle* h, int32_t n_sweeps, int32_t measure, void* stream_ptr) {
    if (!h) return LQMC_ERR_INVALID;
    if (h->n_chains == 0) return fail(h, LQMC_ERR_STATE, "no chains defined (call lqmc_set_chains)");
    if (n_sweeps < 0) return fail(h, LQMC_ERR_INVALID, "n_sweeps < 0");
    h->launches = 0;
    if (n_sweeps == 0) return LQMC_OK;
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    for (int c = 0; c < h->n_chains; ++c) {
        if (!h->field_set[c]) return fail(h, LQMC_ERR_STATE, "chain " + std::to_string(c) + ": field not set");
        if (h->p.rng == LQMC_RNG_REPLAY) {
            const size_t need = (size_t)n_sweeps * h->desc[c].n * h->desc[c].L;
            if (h->uni_count[c] < need)
                return fail(h, LQMC_ERR_STATE, "chain " + std::to_string(c) + ": fewer uniforms uploaded than the sweeps consume");
        }
    }
    int rec = h->p.record ? 1 : 0;
    if (rec) {
        size_t need = 0;
        for (auto& d : h->desc) need += round_up((size_t)n_sweeps * d.L * d.n, 256);
        if (need > h->dec_cap) {
            if (h->d_dec) cudaFree(h->d_dec);
            h->d_dec = nullptr;
            h->dec_cap = 0;
            cudaError_t e = cudaMalloc(&h->d_dec, need);
            if (e != cudaSuccess) return fail(h, LQMC_ERR_NOMEM, "decision buffer allocation failed");
            h->dec_cap = need;
        }
        size_t o = 0;
        for (auto& d : h->desc) {
            if (d.decisions != h->d_dec + o) h->descs_dirty = true;
            d.decisions = h->d_dec + o;
            o += round_up((size_t)n_sweeps * d.L * d.n, 256);
        }
    }
    for (auto& d : h->desc) {
        if (d.record != rec) { d.record = rec; h->descs_dirty = true; }
    }
    if (h->descs_dirty) {
        const int r = sync_last(h);
        if (r) return r;
        std::vector<ChainDesc> tmp;
        for (auto& b : h->buckets) {
            tmp.clear();
            for (int c : b.chains) tmp.push_back(h->desc[c]);
            LQMC_CK(h, cudaMemcpy(b.d_descs, tmp.data(), sizeof(ChainDesc) * tmp.size(), cudaMemcpyHostToDevice));
        }
        h->descs_dirty = false;
    }
    // with the unequal-time G measured, one sweep per launch, each followed by the G(tau)
    // kernel on the field and G it left; else one launch runs every sweep
    const bool tau = measure && h->p.measure_tau;
    const int per_launch = tau ? 1 : n_sweeps;
    auto launch = [&](Bucket& b, cudaStream_t st, int base) {
        cudaError_t e;
        const int nc = (int)b.chains.size();
        if (b.kind == kSmemFp64) {
            e = lqmc::launch_sweep_fp64(b.d_descs, nc, b.smem, per_launch, measure, base, st);
        } else {
            const int prec = b.kind == kTiledFp32 ? 1 : (b.kind == kTiledFp64e ? 2 : 0);
            e = lqmc::launch_sweep_tiled(b.d_descs, nc, b.smem, prec, per_launch, measure, base, st);
        }
        ++h->launches;
        if (e == cudaSuccess && tau) {
            e = lqmc::launch_green_tau(b.d_descs, nc, b.tau_smem, st);
            ++h->launches;
        }
        return e;
    };
    for (int base = 0; base < n_sweeps; base += per_launch) {
        if (h->buckets.size() == 1) {
            LQMC_CK(h, launch(h->buckets[0], stream, base));
        } else {
            LQMC_CK(h, cudaEventRecord(h->fork, stream));
            for (auto& b : h->buckets) {
                LQMC_CK(h, cudaStreamWaitEvent(b.stream, h->fork, 0));
                LQMC_CK(h, launch(b, b.stream, base));
                LQMC_CK(h, cudaEventRecord(b.done, b.stream));
                LQMC_CK(h, cudaStreamWaitEvent(stream, b.done, 0));
            }
        }
    }
    if (h->p.rng == LQMC_RNG_REPLAY)
        for (int c = 0; c < h->n_chains; ++c) h->uni_count[c] = 0;
    h->last_stream = stream;
    h->last_sweeps = n_sweeps;
    return LQMC_OK;
}

int lqmc_get_green(lqmc_handle* h, int32_t chain, double* green) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!green) return fail(h, LQMC_ERR_INVALID, "null output");
    if ((rc = sync_last(h))) return rc;
    const ChainDesc& d = h->desc[chain];
    LQMC_CK(h, cudaMemcpy(green, d.green, 2 * (size_t)d.n * d.n * sizeof(double), cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_get_green_all(lqmc_handle* h, double* green) {
    if (!h) return LQMC_ERR_INVALID;
    if (h->n_chains == 0) return fail(h, LQMC_ERR_STATE, "no chains defined (call lqmc_set_chains)");
    if (!green) return fail(h, LQMC_ERR_INVALID, "null output");
    int rc = sync_last(h);
    if (rc) return rc;
    LQMC_CK(h, cudaMemcpy(green, h->d_green, h->green_total * sizeof(double), cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_get_green_sum(lqmc_handle* h, int32_t chain, double* green_sum, int64_t* count) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if ((rc = sync_last(h))) return rc;
    const ChainDesc& d = h->desc[chain];
    if (green_sum)
        LQMC_CK(h, cudaMemcpy(green_sum, d.gsum, 2 * (size_t)d.n * d.n * sizeof(double), cudaMemcpyDeviceToHost));
    if (count) {
        double c = 0.0;
        LQMC_CK(h, cudaMemcpy(&c, d.obs, sizeof(double), cudaMemcpyDeviceToHost));
        *count = (int64_t)c;
    }
    return LQMC_OK;
}

int lqmc_get_observables(lqmc_handle* h, int32_t chain, double* obs) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!obs) return fail(h, LQMC_ERR_INVALID, "null output");
    if ((rc = sync_last(h))) return rc;
    const ChainDesc& d = h->desc[chain];
    LQMC_CK(h, cudaMemcpy(obs, d.obs, LQMC_OBS_LEN(d.n) * sizeof(double), cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_reset_measurements(lqmc_handle* h) {
    if (!h) return LQMC_ERR_INVALID;
    if (h->n_chains == 0) return fail(h, LQMC_ERR_STATE, "no chains defined");
    int rc = sync_last(h);
    if (rc) return rc;
    for (auto& d : h->desc) {
        LQMC_CK(h, cudaMemset(d.gsum, 0, 2 * (size_t)d.n * d.n * sizeof(double)));
        LQMC_CK(h, cudaMemset(d.obs, 0, LQMC_OBS_LEN(d.n) * sizeof(double)));
        if (d.gtau) LQMC_CK(h, cudaMemset(d.gtau, 0, 2 * (size_t)d.L * d.n * d.n * sizeof(double)));
    }
    return LQMC_OK;
}

int lqmc_get_decisions(lqmc_handle* h, int32_t chain, int8_t* decisions, size_t count) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!h->p.record) return fail(h, LQMC_ERR_STATE, "handle was created with record = 0");
    const ChainDesc& d = h->desc[chain];
    const size_t have = (size_t)h->last_sweeps * d.L * d.n;
    if (!decisions || count < have) return fail(h, LQMC_ERR_INVALID, "decision buffer too small");
    if ((rc = sync_last(h))) return rc;
    if (have) LQMC_CK(h, cudaMemcpy(decisions, d.decisions, have, cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_set_chain_state(lqmc_handle* h, int32_t chain, const double* diag, const double* green_sum,
                         const double* obs) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if ((rc = sync_last(h))) return rc;
    const ChainDesc& d = h->desc[chain];
    if (diag) {
        if (!(diag[7] >= 0.0) || diag[7] != (double)(int64_t)diag[7])
            return fail(h, LQMC_ERR_INVALID, "diagnostics[7] (sweep counter) must be a non-negative integer");
        LQMC_CK(h, cudaMemcpy(d.diag, diag, LQMC_DIAG_LEN * sizeof(double), cudaMemcpyHostToDevice));
        // the kept products are not part of a checkpoint: the next sweep rebuilds them
        LQMC_CK(h, cudaMemset(d.diag + 21, 0, sizeof(double)));
    }
    if (green_sum)
        LQMC_CK(h, cudaMemcpy(d.gsum, green_sum, 2 * (size_t)d.n * d.n * sizeof(double), cudaMemcpyHostToDevice));
    if (obs) {
        if (!(obs[0] >= 0.0)) return fail(h, LQMC_ERR_INVALID, "observables[0] (measurement count) must be >= 0");
        LQMC_CK(h, cudaMemcpy(d.obs, obs, LQMC_OBS_LEN(d.n) * sizeof(double), cudaMemcpyHostToDevice));
    }
    return LQMC_OK;
}

int lqmc_get_green_tau(lqmc_handle* h, int32_t chain, double* green_tau_sum) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!green_tau_sum) return fail(h, LQMC_ERR_INVALID, "null output");
    const ChainDesc& d = h->desc[chain];
    if (!d.gtau) return fail(h, LQMC_ERR_STATE, "the unequal-time G is not measured (params.measure_tau = 0)");
    if ((rc = sync_last(h))) return rc;
    LQMC_CK(h, cudaMemcpy(green_tau_sum, d.gtau, 2 * (size_t)d.L * d.n * d.n * sizeof(double),
                          cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_set_green_tau(lqmc_handle* h, int32_t chain, const double* green_tau_sum) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!green_tau_sum) return fail(h, LQMC_ERR_INVALID, "null input");
    const ChainDesc& d = h->desc[chain];
    if (!d.gtau) return fail(h, LQMC_ERR_STATE, "the unequal-time G is not measured (params.measure_tau = 0)");
    if ((rc = sync_last(h))) return rc;
    LQMC_CK(h, cudaMemcpy(d.gtau, green_tau_sum, 2 * (size_t)d.L * d.n * d.n * sizeof(double),
                          cudaMemcpyHostToDevice));
    return LQMC_OK;
}

int lqmc_get_diagnostics(lqmc_handle* h, int32_t chain, double* diag) {
    int rc = check_chain(h, chain);
    if (rc) return rc;
    if (!diag) return fail(h, LQMC_ERR_INVALID, "null output");
    if ((rc = sync_last(h))) return rc;
    LQMC_CK(h, cudaMemcpy(diag, h->desc[chain].diag, LQMC_DIAG_LEN * sizeof(double), cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_get_status(lqmc_handle* h, int32_t* status) {
    if (!h) return LQMC_ERR_INVALID;
    if (h->n_chains == 0) return fail(h, LQMC_ERR_STATE, "no chains defined");
    if (!status) return fail(h, LQMC_ERR_INVALID, "null output");
    int rc = sync_last(h);
    if (rc) return rc;
    LQMC_CK(h, cudaMemcpy(status, h->d_status, sizeof(int32_t) * h->n_chains, cudaMemcpyDeviceToHost));
    return LQMC_OK;
}

int lqmc_get_launch_count(lqmc_handle* h, int64_t* launches) {
    if (!h || !launches) return LQMC_ERR_INVALID;
    *launches = h->launches;
    return LQMC_OK;
}

const char* lqmc_last_error(const lqmc_handle* h) {
    return h ? h->err.c_str() : g_create_error.c_str();
}

void lqmc_destroy(lqmc_handle* h) {
    if (!h) return;
    cudaSetDevice(h->p.device);
    cudaDeviceSynchronize();
    release(h);
    if (h->fork) cudaEventDestroy(h->fork);
    delete h;
}

}  // extern "C"
