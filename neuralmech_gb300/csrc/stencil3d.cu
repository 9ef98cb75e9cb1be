// 3D time-step kernel of the acoustic wave path (sm_103a): not built yet.
#include "common.cuh"
#include "internal.h"

namespace wfd {

bool step3d_available() { return false; }

cudaError_t launch_step3d(int, int, const CUtensorMap&, const CUtensorMap&, const CUtensorMap&,
                          const StepArgs&, cudaStream_t) {
    return cudaErrorNotSupported;
}

size_t step3d_smem_bytes(int, int) { return 0; }

}  // namespace wfd
