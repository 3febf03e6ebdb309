// Host side of the tiled sweep kernel: shared-memory and global-work sizing, and the
// dispatch over the three precision instantiations (each compiled in its own translation
// unit, sweep_tiled_{f64,f32,f64e}.cu).
#include "sweep_tiled.cuh"

namespace lqmc {

cudaError_t launch_sweep_tiled_f64(const ChainDesc* d_descs, int n_chains, size_t smem,
                                   int n_sweeps, int measure, int sweep_base, cudaStream_t stream);
cudaError_t launch_sweep_tiled_f32(const ChainDesc* d_descs, int n_chains, size_t smem,
                                   int n_sweeps, int measure, int sweep_base, cudaStream_t stream);
cudaError_t launch_sweep_tiled_f64e(const ChainDesc* d_descs, int n_chains, size_t smem,
                                    int n_sweeps, int measure, int sweep_base, cudaStream_t stream);

// bytes of dynamic shared memory / per-chain global work of the tiled kernel
size_t sweep_tiled_smem_bytes(int n, bool fp32, int delay, bool emu, int stages, bool xy_global) {
    size_t v = (size_t)(kNW + 8 + 9 * n);
    v = (v + 3) & ~(size_t)3;                                   // doubles
    const size_t ts = fp32 ? 4 : 8;
    const size_t tvec = 6 * (size_t)n * ts;                     // T vectors, bytes
    v += ((tvec + 7) / 8 + 3) & ~(size_t)3;
    v += 8;                                                     // gii
    const size_t rbytes = stage_region_bytes(fp32, emu, stages) + (xy_global ? 0 : 2 * (size_t)n * (delay + 1) * ts);
    const size_t pbytes = (size_t)n * (panel_width(n) + 1) * sizeof(double);
    size_t total = v * sizeof(double) + (rbytes > pbytes ? rbytes : pbytes) + 16 + kPanel * sizeof(int);
    if (emu) {
        total += 128;   // stage alignment
        if (total < kEmuMinSmem) total = kEmuMinSmem;
    }
    return total;
}

// delayed-update depth wanted: requested, or 32 in fp32, 24 with emulated GEMMs, 16 in fp64
int sweep_tiled_delay_target(bool fp32, int requested, bool emu) {
    return requested > 0 ? requested : (fp32 ? 32 : (emu ? 24 : 16));
}

// largest delayed-update depth <= the target whose buffers fit `cap` in shared memory
int sweep_tiled_delay(int n, bool fp32, int requested, size_t cap, bool emu, int stages) {
    int k = sweep_tiled_delay_target(fp32, requested, emu);
    while (k > 1 && sweep_tiled_smem_bytes(n, fp32, k, emu, stages, false) > cap) --k;
    return k;
}

size_t sweep_tiled_work_bytes(int n, int n_chunks, bool fp32, bool emu, int xy_delay, bool alt) {
    return fp32 ? TiledLayout<float>(n, n_chunks, false, xy_delay, alt).total
                : TiledLayout<double>(n, n_chunks, emu, xy_delay, alt).total;
}

size_t sweep_tiled_presplit_bytes(int n) { return PresplitLayout(n).total; }

// split the constant operands of `count` jobs (device array) on `stream`
cudaError_t launch_presplit(const void* d_jobs, int count, cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    presplit_kernel<<<kNumPre * count, kNT, 0, stream>>>(static_cast<const PresplitJob*>(d_jobs));
    return cudaGetLastError();
}

size_t sweep_tiled_presplit_job_bytes() { return sizeof(PresplitJob); }

void sweep_tiled_presplit_job(void* job, const double* expk, const double* expkinv,
                              unsigned char* out, int n) {
    PresplitJob* j = static_cast<PresplitJob*>(job);
    j->expk = expk;
    j->expkinv = expkinv;
    j->out = out;
    j->n = n;
}

// precision: 0 float64, 1 float32 (mixed), 2 float64 with emulated tensor-core GEMMs
cudaError_t launch_sweep_tiled(const ChainDesc* d_descs, int n_chains, size_t smem, int precision,
                               int n_sweeps, int measure, int sweep_base, cudaStream_t stream) {
    if (precision == 1)
        return launch_sweep_tiled_f32(d_descs, n_chains, smem, n_sweeps, measure, sweep_base, stream);
    if (precision == 2)
        return launch_sweep_tiled_f64e(d_descs, n_chains, smem, n_sweeps, measure, sweep_base, stream);
    return launch_sweep_tiled_f64(d_descs, n_chains, smem, n_sweeps, measure, sweep_base, stream);
}

}  // namespace lqmc
