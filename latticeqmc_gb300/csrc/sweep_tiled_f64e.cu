// Tiled sweep kernel instantiated for float64 G with every dense product an emulated float64
// GEMM on the tcgen05 tensor cores.
#include "sweep_tiled.cuh"

namespace lqmc {

cudaError_t launch_sweep_tiled_f64e(const ChainDesc* d_descs, int n_chains, size_t smem,
                                    int n_sweeps, int measure, int sweep_base, cudaStream_t stream) {
    return launch_tiled<double, true>(d_descs, n_chains, smem, n_sweeps, measure, sweep_base, stream);
}

}  // namespace lqmc
