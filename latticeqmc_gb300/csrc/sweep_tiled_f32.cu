// Tiled sweep kernel instantiated for float32 G, wraps, updates and B-chain (mixed).
#include "sweep_tiled.cuh"

namespace lqmc {

cudaError_t launch_sweep_tiled_f32(const ChainDesc* d_descs, int n_chains, size_t smem,
                                   int n_sweeps, int measure, int sweep_base, cudaStream_t stream) {
    return launch_tiled<float, false>(d_descs, n_chains, smem, n_sweeps, measure, sweep_base, stream);
}

}  // namespace lqmc
