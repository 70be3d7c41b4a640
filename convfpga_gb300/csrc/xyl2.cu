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

// The scratch ring (allocated once, never moved) and the kernels' attributes. With
// max_planes > 0 also the process's own dependency counters (grow-only: reallocated when
// a launch needs more, so graphs bring their own counters).
static cudaError_t xy_l2_setup(long long max_planes, int &per_sm, int &sms) {
  constexpr size_t plane = 256ull * 256 * sizeof(float2);
  cudaError_t e = g_ring.ensure(plane * kXyL2Ring);
  if (e != cudaSuccess) return e;
  const size_t cbytes = (2ull * max_planes + 2) * sizeof(unsigned);
  if (max_planes > 0 && (e = g_ctr.ensure(std::max<size_t>(cbytes, 64 << 10))) != cudaSuccess) return e;
  static bool done[2] = {false, false};
  if ((e = set_smem_once(k_xy_l2<false>, kXyL2Smem, done[0])) != cudaSuccess) return e;
  if ((e = set_smem_once(k_xy_l2<true>, kXyL2Smem, done[1])) != cudaSuccess) return e;
  static int ps = 0, nsm = 0;
  if (ps == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, (const void *)k_xy_l2<false>, kXyL2Threads, kXyL2Smem) !=
            cudaSuccess ||
        ps <= 0) {
      cudaGetLastError();
      ps = 1;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
  }
  per_sm = ps;
  sms = nsm;
  return cudaSuccess;
}

cudaError_t prepare_xy_l2() {
  int ps, sms;
  return xy_l2_setup(0, ps, sms);
}

size_t xy_l2_counter_bytes(int ncubes) { return (2ull * 256 * ncubes + 2) * sizeof(unsigned); }

bool encode_xy_table_map(CUtensorMap *m, const void *cube) {
  return encode_rows_map(m, cube, 256, 256LL * 256, kXyL2Cols);
}

static cudaError_t launch_common(const CUtensorMap *msrc_or_null, const CUtensorMap *rmaps, float2 *const *dsts,
                                 float2 *dst, int nplanes, bool inverse, float scale, const float2 *tw512,
                                 unsigned *status, unsigned *ctr, cudaStream_t s) {
  int ps, sms;
  cudaError_t e = xy_l2_setup(ctr ? 0 : nplanes, ps, sms);
  if (e != cudaSuccess) return e;
  if (!ctr) ctr = reinterpret_cast<unsigned *>(g_ctr.p);
  CUtensorMap mscr;
  if (!encode_cube_map(&mscr, g_ring.p, 256, kXyL2Ring, 1, kXyL2Cols)) return cudaErrorNotSupported;
  const CUtensorMap &msrc = msrc_or_null ? *msrc_or_null : mscr;  // unused in table mode
  auto kern = inverse ? k_xy_l2<true> : k_xy_l2<false>;
  const long long ncount = 2LL * nplanes + 2;
  k_xyl2_clear<<<(unsigned)std::min<long long>((ncount + 255) / 256, 64), 256, 0, s>>>(ctr, ncount);
  const long long items = 2LL * nplanes * kXyL2Items;
  const unsigned grid = (unsigned)std::min<long long>(items, (long long)ps * sms);
  kern<<<grid, kXyL2Threads, kXyL2Smem, s>>>(msrc, mscr, reinterpret_cast<float2 *>(g_ring.p), dst, nplanes, scale,
                                             tw512, ctr, status, kXyL2Lag, kXyL2Ring, rmaps, dsts);
  return cudaGetLastError();
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
  CUtensorMap msrc;
  if (!encode_rows_map(&msrc, src, 256, (long long)nplanes * 256, kXyL2Cols)) return cudaErrorNotSupported;
  return launch_common(&msrc, nullptr, nullptr, dst, nplanes, inverse, scale, tw512, status, nullptr, s);
}

// The same over `ncubes` 256^3 cubes at unrelated addresses: rmaps[i] (device memory,
// from encode_xy_table_map) describes the rows of source cube i, dsts[i] is its output
// base. ctr: the caller's counters, xy_l2_counter_bytes(ncubes) bytes of device memory.
// Call prepare_xy_l2() first when the launch is captured in a graph.
cudaError_t launch_xy_l2_table(const CUtensorMap *rmaps, float2 *const *dsts, int ncubes, bool inverse, float scale,
                               const float2 *tw512, unsigned *status, unsigned *ctr, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  if (!ctr) return cudaErrorInvalidValue;
  return launch_common(nullptr, rmaps, dsts, nullptr, 256 * ncubes, inverse, scale, tw512, status, ctr, s);
}

}  // namespace convgpu
