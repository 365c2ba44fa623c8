// k_team64.cu -- the server's resident team loop over plain FP64 lattices (compiled with --fmad=false,
// the rounding of k_fp64.cu, so that a run gives the stream lane's bits).
#include "team_lane.cuh"

namespace erlbm {

// Dynamic shared memory the FP64 loop reserves and does not use: more than half an SM's, so that no
// SM holds two of its CTAs (an SM's FP64 pipes are the loop's bound, and two CTAs on one SM while
// another has none would halve them), but small enough that a slot loop's CTA still fits beside one.
constexpr int TEAM64_SPREAD_SMEM = 116 * 1024;

int launch_team_server_fp64(const TeamRing &r, int grid, cudaStream_t s)
{
    if (grid < 2 || grid > TEAM_MAX_GRID) return -1;
    // the slot loops' carveout (largest shared memory), so that the resident loops share SMs
    if (cudaFuncSetAttribute(team::k_team_server<PrecExact64>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaFuncSetAttribute(team::k_team_server<PrecExact64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             TEAM64_SPREAD_SMEM) != cudaSuccess)
        return -3;
    team::k_team_server<PrecExact64><<<grid, team_threads<PrecExact64>(), TEAM64_SPREAD_SMEM, s>>>(r);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int team_server_occupancy_fp64()
{
    int n = 0;
    if (cudaFuncSetAttribute(team::k_team_server<PrecExact64>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaFuncSetAttribute(team::k_team_server<PrecExact64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             TEAM64_SPREAD_SMEM) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, team::k_team_server<PrecExact64>, team_threads<PrecExact64>(),
                                                      TEAM64_SPREAD_SMEM) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

namespace {
__global__ void k_team_clock(long long *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *out = team::now_ns();
}
}  // namespace

int launch_team_clock(long long *out, cudaStream_t s)
{
    k_team_clock<<<1, 32, 0, s>>>(out);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace erlbm
