// Launcher of the L2-staged fused x + y pass for N = 256 (xyl2.cuh): scratch ring and
// dependency counters (grow-only, per process), counters cleared on the stream before
// every launch, one persistent grid of as many CTAs as fit.
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"
#include "xyl2.cuh"

#include <algorithm>

namespace convgpu {

// Clears the dependency counters on the stream. A kernel, not cudaMemsetAsync: a memset
// may be queued on a copy engine behind the host pipeline's large transfers.
__global__ void k_xyl2_clear(unsigned *c, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    c[i] = 0u;
}

namespace {
struct Scratch {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    const cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};
Scratch g_ring, g_ctr;
}  // namespace

void release_xy_l2() {
  g_ring.release();
  g_ctr.release();
}

// x then y transform of `nplanes` consecutive 256 x 256 planes, src -> dst (may be the
// same), inverse transforms with `inverse`, dst scaled by `scale`. The scratch ring and
// counters are shared by all calls: calls that overlap on the GPU (different streams)
// must not both run this pass. Returns cudaErrorNotSupported when the operands cannot be
// described by tensor maps.
cudaError_t launch_xy_l2(const float2 *src, float2 *dst, int nplanes, bool inverse, float scale, const float2 *tw512,
                         unsigned *status, cudaStream_t s) {
  if (nplanes <= 0) return cudaSuccess;
  if ((reinterpret_cast<uintptr_t>(dst) & 15u) != 0) return cudaErrorNotSupported;
  constexpr size_t plane = 256ull * 256 * sizeof(float2);
  cudaError_t e = g_ring.ensure(plane * kXyL2Ring);
  if (e != cudaSuccess) return e;
  const size_t cbytes = (2ull * nplanes + 2) * sizeof(unsigned);
  if ((e = g_ctr.ensure(std::max<size_t>(cbytes, 64 << 10))) != cudaSuccess) return e;
  CUtensorMap msrc, mscr;
  if (!encode_rows_map(&msrc, src, 256, (long long)nplanes * 256, kXyL2Cols)) return cudaErrorNotSupported;
  if (!encode_cube_map(&mscr, g_ring.p, 256, kXyL2Ring, 1, kXyL2Cols)) return cudaErrorNotSupported;
  auto kern = inverse ? k_xy_l2<true> : k_xy_l2<false>;
  static bool done[2] = {false, false};
  if ((e = set_smem_once(kern, kXyL2Smem, done[inverse ? 1 : 0])) != cudaSuccess) return e;
  static int per_sm[2] = {0, 0}, sms = 0;
  int &ps = per_sm[inverse ? 1 : 0];
  if (ps == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, (const void *)kern, kXyL2Threads, kXyL2Smem) !=
            cudaSuccess ||
        ps <= 0) {
      cudaGetLastError();
      ps = 1;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const long long ncount = (long long)(cbytes / sizeof(unsigned));
  k_xyl2_clear<<<(unsigned)std::min<long long>((ncount + 255) / 256, 64), 256, 0, s>>>(
      reinterpret_cast<unsigned *>(g_ctr.p), ncount);
  const long long items = 2LL * nplanes * kXyL2Items;
  const unsigned grid = (unsigned)std::min<long long>(items, (long long)ps * sms);
  kern<<<grid, kXyL2Threads, kXyL2Smem, s>>>(msrc, mscr, reinterpret_cast<float2 *>(g_ring.p), dst, nplanes, scale,
                                             tw512, reinterpret_cast<unsigned *>(g_ctr.p), status, kXyL2Lag,
                                             kXyL2Ring);
  return cudaGetLastError();
}

}  // namespace convgpu
