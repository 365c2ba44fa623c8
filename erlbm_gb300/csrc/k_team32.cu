// k_team32.cu -- the server's resident team loop over FP32-shifted lattices (compiled like k_fp32.cu,
// so that a run gives the stream lane's bits).
#include "team_lane.cuh"

namespace erlbm {

int launch_team_server_fp32(const TeamRing &r, int grid, cudaStream_t s)
{
    if (grid < 2 || grid > TEAM_MAX_GRID) return -1;
    // the slot loops' carveout (largest shared memory), so that the resident loops share SMs
    if (cudaFuncSetAttribute(team::k_team_server<PrecShifted32>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return -3;
    team::k_team_server<PrecShifted32><<<grid, team_threads<PrecShifted32>(), 0, s>>>(r);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int team_server_occupancy_fp32()
{
    int n = 0;
    if (cudaFuncSetAttribute(team::k_team_server<PrecShifted32>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, team::k_team_server<PrecShifted32>, team_threads<PrecShifted32>(), 0) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace erlbm
