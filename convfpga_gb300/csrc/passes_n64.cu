// Pass-kernel launchers for cubes of size 64 (see pass_launch.cuh).
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"

namespace convgpu {
template cudaError_t launch_size<64>(const PassReq &);
template cudaError_t prepare_size<64>();
}  // namespace convgpu
