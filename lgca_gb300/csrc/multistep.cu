// Temporally blocked step: several steps per pass over global memory.
#include "internal.cuh"

namespace lgca_gpu {

bool multistep_supported(int, const PlaneGeom &, int) { return false; }

cudaError_t launch_multistep(int, int, const MultiStepArgs &, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // namespace lgca_gpu
