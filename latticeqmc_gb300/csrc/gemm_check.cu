// lqmc_emulated_gemm: one product C = op(A) op(B) through the emulated float64 GEMM of the
// fp64e sweep kernel (ozaki_tc.cuh), run by one CTA of the same shape and shared-memory
// staging as a chain's CTA in the sweep.  It lets the product be checked against float64
// on its own and timed on its own (SM clock cycles of its phases).
#include <cuda_runtime.h>

#include <vector>

#include "lqmc_gpu.h"
#include "ozaki_tc.cuh"

namespace lqmc {
namespace {

struct GemmJob {
    int m, n, k, lda, ldb, ldc, ta, tb, flags, stages;
    const double* a;
    const double* b;
    double* c;
    const double* rs;
    const double* cs;
    __nv_bfloat16* slices;       // fresh operands
    __nv_bfloat16* pre_a;        // A split in a separate pass (LQMC_GEMM_PRESPLIT_A)
    __nv_bfloat16* pre_b;        // B split in a separate pass (LQMC_GEMM_PRESPLIT_B)
    int* ea;
    int* eb;
    int* pre_ea;
    int* pre_eb;
    long long* out;              // [0] fail flag, [1..3] cycles: split, pipeline, drain
};

template <bool TA, bool TB>
__device__ void run_job(const GemmJob& j, ozt::Workspace ws) {
    blk::GemmOpt<double> o;
    o.rs = j.rs;
    o.cs = j.cs;
    o.subtract = (j.flags & LQMC_GEMM_SUBTRACT) != 0;
    o.kscale = (j.flags & LQMC_GEMM_KSCALE) != 0;
    int* scratch = reinterpret_cast<int*>(blk::as_shared(ws.stage));
    ozt::Presplit pa, pb;
    if (j.flags & LQMC_GEMM_PRESPLIT_A) {
        ozt::split_tiles<ozt::kBM>(j.a, j.lda, TA, j.m, j.k, j.pre_ea, j.pre_a, scratch);
        pa.slices = j.pre_a;
        pa.exps = j.pre_ea;
    }
    if (j.flags & LQMC_GEMM_PRESPLIT_B) {
        ozt::split_tiles<ozt::kBN>(j.b, j.ldb, !TB, j.n, j.k, j.pre_eb, j.pre_b, scratch);
        pb.slices = j.pre_b;
        pb.exps = j.pre_eb;
    }
    asm volatile("fence.proxy.async;\n" ::: "memory");
    __syncthreads();
    ozt::oz_gemm_tc<TA, TB>(j.c, j.ldc, j.a, j.lda, j.b, j.ldb, j.m, j.n, j.k, ws, o,
                            (j.flags & LQMC_GEMM_PRESPLIT_A) ? &pa : nullptr,
                            (j.flags & LQMC_GEMM_PRESPLIT_B) ? &pb : nullptr);
}

__global__ void __launch_bounds__(blk::kNT, 1) emulated_gemm_kernel(GemmJob j) {
    extern __shared__ __align__(128) unsigned char gemm_smem[];
    __shared__ ozt::Tc tc;
    __shared__ long long cyc[3];
    if (threadIdx.x < 3) cyc[threadIdx.x] = 0;
    ozt::tc_setup(&tc);
    ozt::Workspace ws;
    ws.slices = j.slices;
    ws.ea = j.ea;
    ws.eb = j.eb;
    ws.stage = reinterpret_cast<unsigned char*>(((uintptr_t)gemm_smem + 127) & ~(uintptr_t)127);
    ws.stages = j.stages;
    ws.tc = &tc;
    ws.cycles = cyc;
    if (j.ta && j.tb) run_job<true, true>(j, ws);
    else if (j.ta) run_job<true, false>(j, ws);
    else if (j.tb) run_job<false, true>(j, ws);
    else run_job<false, false>(j, ws);
    __syncthreads();
    if (threadIdx.x == 0) {
        j.out[0] = tc.fail;
        for (int i = 0; i < 3; ++i) j.out[1 + i] = cyc[i];
    }
    ozt::tc_teardown(&tc);
}

}  // namespace
}  // namespace lqmc

extern "C" int lqmc_emulated_gemm(int32_t m, int32_t n, int32_t k, const double* a, int32_t lda,
                                  int32_t trans_a, const double* b, int32_t ldb, int32_t trans_b,
                                  double* c, int32_t ldc, const double* row_scale,
                                  const double* col_scale, int32_t flags, int32_t stages,
                                  int32_t device, double* cycles) {
    using namespace lqmc;
    if (m <= 0 || n <= 0 || k <= 0 || m > 4096 || n > 4096 || k > 4096 || !a || !b || !c)
        return LQMC_ERR_INVALID;
    if (stages < 1 || stages > ozt::kMaxStages) return LQMC_ERR_INVALID;
    const size_t a_rows = trans_a ? (size_t)k : (size_t)m, a_cols = trans_a ? (size_t)m : (size_t)k;
    const size_t b_rows = trans_b ? (size_t)n : (size_t)k, b_cols = trans_b ? (size_t)k : (size_t)n;
    if ((size_t)lda < a_cols || (size_t)ldb < b_cols || ldc < n) return LQMC_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LQMC_ERR_CUDA;
    const size_t na = a_rows * lda, nb = b_rows * ldb, nc = (size_t)m * ldc;
    const size_t n_slices = ozt::slice_elems(m, n, k);
    const size_t n_pre_a = (size_t)ozt::kSlices * ozt::rows_pad(m, ozt::kBM) * ozt::kpad(k);
    const size_t n_pre_b = (size_t)ozt::kSlices * ozt::rows_pad(n, ozt::kBN) * ozt::kpad(k);
    // one allocation: A, B, C, scales (doubles), slices (bf16), exponents (ints), result
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t o_a = take(na * 8), o_b = take(nb * 8), o_c = take(nc * 8), o_rs = take((size_t)m * 8),
                 o_cs = take((size_t)n * 8), o_sl = take(n_slices * 2), o_pa = take(n_pre_a * 2),
                 o_pb = take(n_pre_b * 2), o_e = take((size_t)2 * (m + n) * 4), o_out = take(4 * 8);
    unsigned char* d = nullptr;
    if (cudaMalloc(&d, off) != cudaSuccess) return LQMC_ERR_NOMEM;
    int rc = LQMC_OK;
    std::vector<long long> out(4, 0);
    do {
        if (cudaMemcpy(d + o_a, a, na * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d + o_b, b, nb * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d + o_c, c, nc * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            (row_scale && cudaMemcpy(d + o_rs, row_scale, (size_t)m * 8, cudaMemcpyHostToDevice) != cudaSuccess) ||
            (col_scale && cudaMemcpy(d + o_cs, col_scale, (size_t)n * 8, cudaMemcpyHostToDevice) != cudaSuccess)) {
            rc = LQMC_ERR_CUDA;
            break;
        }
        GemmJob j{};
        j.m = m; j.n = n; j.k = k; j.lda = lda; j.ldb = ldb; j.ldc = ldc;
        j.ta = trans_a; j.tb = trans_b; j.flags = flags; j.stages = stages;
        j.a = reinterpret_cast<const double*>(d + o_a);
        j.b = reinterpret_cast<const double*>(d + o_b);
        j.c = reinterpret_cast<double*>(d + o_c);
        j.rs = row_scale ? reinterpret_cast<const double*>(d + o_rs) : nullptr;
        j.cs = col_scale ? reinterpret_cast<const double*>(d + o_cs) : nullptr;
        j.slices = reinterpret_cast<__nv_bfloat16*>(d + o_sl);
        j.pre_a = reinterpret_cast<__nv_bfloat16*>(d + o_pa);
        j.pre_b = reinterpret_cast<__nv_bfloat16*>(d + o_pb);
        int* e = reinterpret_cast<int*>(d + o_e);
        j.ea = e;
        j.eb = e + m;
        j.pre_ea = e + m + n;
        j.pre_eb = e + 2 * m + n;
        j.out = reinterpret_cast<long long*>(d + o_out);
        const size_t smem = ozt::stage_bytes(stages) + 128;
        if (cudaFuncSetAttribute(emulated_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess) {
            rc = LQMC_ERR_CUDA;
            break;
        }
        emulated_gemm_kernel<<<1, blk::kNT, smem>>>(j);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
            rc = LQMC_ERR_CUDA;
            break;
        }
        if (cudaMemcpy(c, d + o_c, nc * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(out.data(), d + o_out, 4 * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = LQMC_ERR_CUDA;
            break;
        }
        if (out[0]) rc = LQMC_ERR_NUMERIC;   // a bounded wait of the pipeline ran out
        if (cycles)
            for (int i = 0; i < 3; ++i) cycles[i] = (double)out[1 + i];
    } while (false);
    cudaFree(d);
    return rc;
}
