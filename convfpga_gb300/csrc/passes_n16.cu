// Pass-kernel launchers for cubes of size 16 (see pass_launch.cuh).
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"

namespace convgpu {
template cudaError_t launch_size<16>(const PassReq &);
template cudaError_t prepare_size<16>();
}  // namespace convgpu
