// k_map32.cu -- batched persistent kernel instantiations, FP32-shifted.
#include "batch_kernels.cuh"

namespace erlbm {

namespace {

template <int Q, int NPT>
cudaError_t go(const BatchGeo &g, const BatchRun *runs, int n_runs, int *counter, BatchResult *res, const double *aos,
               int grid, int block, size_t smem, int dbl, cudaStream_t s)
{
    auto k = k_batch<PrecShifted32, Q, NPT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, block, smem, s>>>(g, runs, n_runs, counter, res, aos, dbl);
    return cudaGetLastError();
}

template <int Q, int NPT>
int occ(int block, size_t smem)
{
    auto k = k_batch<PrecShifted32, Q, NPT>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace

int launch_batch_fp32(int q, int npt, const BatchGeo &g, const BatchRun *runs, int n_runs, int *counter,
                      BatchResult *res, const double *aos, int grid, int block, size_t smem, int dbl,
                      cudaStream_t s)
{
    cudaError_t e;
    if (q == 19 && npt == 1) e = go<19, 1>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else if (q == 19 && npt == 2) e = go<19, 2>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else if (q == 9 && npt == 1) e = go<9, 1>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else if (q == 9 && npt == 2) e = go<9, 2>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else if (q == 9 && npt == 4) e = go<9, 4>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else if (q == 19 && npt == 4) e = go<19, 4>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else if (q == 9 && npt == 8) e = go<9, 8>(g, runs, n_runs, counter, res, aos, grid, block, smem, dbl, s);
    else return -1;
    return e == cudaSuccess ? 0 : -3;
}

int batch_occupancy_fp32(int q, int npt, int block, size_t smem)
{
    if (q == 19 && npt == 1) return occ<19, 1>(block, smem);
    if (q == 19 && npt == 2) return occ<19, 2>(block, smem);
    if (q == 19 && npt == 4) return occ<19, 4>(block, smem);
    if (q == 9 && npt == 1) return occ<9, 1>(block, smem);
    if (q == 9 && npt == 2) return occ<9, 2>(block, smem);
    if (q == 9 && npt == 4) return occ<9, 4>(block, smem);
    if (q == 9 && npt == 8) return occ<9, 8>(block, smem);
    return 0;
}

int batch_occupancy_fp64(int q, int npt, int block, size_t smem);

int batch_occupancy(int prec, int q, int npt, int block, size_t smem)
{
    return prec == 0 ? batch_occupancy_fp64(q, npt, block, smem) : batch_occupancy_fp32(q, npt, block, smem);
}

size_t batch_smem(int prec, int q, int nb, int block, int dbl)
{
    if (prec == 0)
        return q == 9 ? batch_smem_bytes<PrecExact64, 9>(nb, block, dbl)
                      : batch_smem_bytes<PrecExact64, 19>(nb, block, dbl);
    return q == 9 ? batch_smem_bytes<PrecShifted32, 9>(nb, block, dbl)
                  : batch_smem_bytes<PrecShifted32, 19>(nb, block, dbl);
}


int launch_slot_server_fp32(const SlotRing &ring, int max_nb, int grid, int block, size_t smem, int dbl,
                            cudaStream_t s)
{
    auto k = k_slot_server<PrecShifted32, 19, 1>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return -3;
    // every resident loop asks for the largest shared-memory carveout: an SM runs CTAs of kernels with
    // one carveout at a time, so loops with different ones would keep each other off the SMs
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return -3;
    k<<<grid, block, smem, s>>>(ring, max_nb, dbl);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int slot_server_occupancy_fp32(int block, size_t smem)
{
    auto k = k_slot_server<PrecShifted32, 19, 1>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
            cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace erlbm
