// Launchers of the L2-staged fused x + y pass for N = 128, 256 and 512 (xyl2.cuh) and of its
// tensor-core form for N = 256 (xyl2_tc.cuh): scratch ring per size and dependency counters
// (grow-only, per process), counters cleared on the stream before every launch, one
// persistent grid of as many CTAs as fit.
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"
#include "xyl2.cuh"
#include "xyl2_tc.cuh"

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
Scratch g_ring[3], g_ctr;  // scratch rings of N = 256, 128 and 512; the process's counters
}  // namespace

void release_xy_l2() {
  for (auto &r : g_ring) r.release();
  g_ctr.release();
}

// The size's scratch ring (allocated once, never moved) and the kernels' attributes.
// With max_planes > 0 also the process's own dependency counters (grow-only: reallocated
// when a launch needs more, so graphs bring their own counters).
template <int N>
static cudaError_t xy_l2_setup(long long max_planes, int &per_sm, int &sms, Scratch *&ring) {
  using Cfg = XyL2Cfg<N>;
  constexpr size_t plane = (size_t)N * N * sizeof(float2);
  ring = &g_ring[N == 256 ? 0 : (N == 128 ? 1 : 2)];
  cudaError_t e = ring->ensure(plane * Cfg::RING);
  if (e != cudaSuccess) return e;
  const size_t cbytes = (2ull * max_planes + 2) * sizeof(unsigned);
  if (max_planes > 0 && (e = g_ctr.ensure(std::max<size_t>(cbytes, 64 << 10))) != cudaSuccess) return e;
  constexpr int smem = xyl2_smem<N>();
  static int done[4] = {0, 0, 0, 0};
  if ((e = set_smem_once(k_xy_l2<N, false, false>, smem, done[0])) != cudaSuccess) return e;
  if ((e = set_smem_once(k_xy_l2<N, true, false>, smem, done[1])) != cudaSuccess) return e;
  if ((e = set_smem_once(k_xy_l2<N, false, true>, smem, done[2])) != cudaSuccess) return e;
  if ((e = set_smem_once(k_xy_l2<N, true, true>, smem, done[3])) != cudaSuccess) return e;
  static int ps = 0, nsm = 0;
  if (ps == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, (const void *)k_xy_l2<N, false, false>, kXyL2Threads,
                                                      smem) !=
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

cudaError_t prepare_xy_l2(int n) {
  int ps, sms;
  Scratch *ring;
  if (n == 256) return xy_l2_setup<256>(0, ps, sms, ring);
  if (n == 128) return xy_l2_setup<128>(0, ps, sms, ring);
  if (n == 512) return xy_l2_setup<512>(0, ps, sms, ring);
  return cudaErrorInvalidValue;
}

size_t xy_l2_counter_bytes(int n, int ncubes) { return (2ull * n * ncubes + 2) * sizeof(unsigned); }

// The source rows map of the pass: 2D rows (box {N, C}) for N <= 256; for N = 512 rows
// viewed as (256, 2, rows) with box {256, 2, C}, since a box is at most 256 long.
static bool encode_xy_rows(CUtensorMap *m, const void *src, int n, long long rows) {
  if (n == 256) return encode_rows_map(m, src, 256, rows, XyL2Cfg<256>::C);
  if (n == 128) return encode_rows_map(m, src, 128, rows, XyL2Cfg<128>::C);
  if (n == 512) return encode_rows512_map(m, src, rows, XyL2Cfg<512>::C);
  return false;
}

bool encode_xy_table_map(CUtensorMap *m, const void *cube, int n) {
  return encode_xy_rows(m, cube, n, (long long)n * n);
}

template <int N>
static cudaError_t launch_common(const CUtensorMap *msrc_or_null, const CUtensorMap *rmaps, float2 *const *dsts,
                                 float2 *dst, int nplanes, bool inverse, float scale, const float2 *tw512,
                                 unsigned *status, unsigned *ctr, cudaStream_t s) {
  using Cfg = XyL2Cfg<N>;
  int ps, sms;
  Scratch *ring;
  cudaError_t e = xy_l2_setup<N>(ctr ? 0 : nplanes, ps, sms, ring);
  if (e != cudaSuccess) return e;
  if (!ctr) ctr = reinterpret_cast<unsigned *>(g_ctr.p);
  CUtensorMap mscr;
  if (!encode_cube_map(&mscr, ring->p, N, Cfg::RING, 1, Cfg::C)) return cudaErrorNotSupported;
  const CUtensorMap &msrc = msrc_or_null ? *msrc_or_null : mscr;  // unused in table mode
  auto kern = rmaps ? (inverse ? k_xy_l2<N, true, true> : k_xy_l2<N, false, true>)
                    : (inverse ? k_xy_l2<N, true, false> : k_xy_l2<N, false, false>);
  const long long ncount = 2LL * nplanes + 2;
  k_xyl2_clear<<<(unsigned)std::min<long long>((ncount + 255) / 256, 64), 256, 0, s>>>(ctr, ncount);
  const long long items = 2LL * nplanes * (N / Cfg::C);
  const unsigned grid = (unsigned)std::min<long long>(items, (long long)ps * sms);
  kern<<<grid, kXyL2Threads, xyl2_smem<N>(), s>>>(msrc, mscr, reinterpret_cast<float2 *>(ring->p), dst, nplanes,
                                                   scale, tw512, ctr, status, Cfg::LAG, rmaps, dsts);
  return cudaGetLastError();
}

// x then y transform of `nplanes` consecutive N x N planes (N = 128, 256 or 512), src -> dst
// (may be the same), inverse transforms with `inverse`, dst scaled by `scale`. The
// scratch ring and counters are shared by all calls: calls that overlap on the GPU
// (different streams) must not both run this pass. Returns cudaErrorNotSupported when the
// operands cannot be described by tensor maps.
cudaError_t launch_xy_l2(int n, const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                         const float2 *tw512, unsigned *status, cudaStream_t s) {
  if (nplanes <= 0) return cudaSuccess;
  if ((reinterpret_cast<uintptr_t>(dst) & 15u) != 0) return cudaErrorNotSupported;
  CUtensorMap msrc;
  if (!encode_xy_rows(&msrc, src, n, (long long)nplanes * n)) return cudaErrorNotSupported;
  switch (n) {
    case 256: return launch_common<256>(&msrc, nullptr, nullptr, dst, nplanes, inverse, scale, tw512, status, nullptr, s);
    case 128: return launch_common<128>(&msrc, nullptr, nullptr, dst, nplanes, inverse, scale, tw512, status, nullptr, s);
    case 512: return launch_common<512>(&msrc, nullptr, nullptr, dst, nplanes, inverse, scale, tw512, status, nullptr, s);
    default: return cudaErrorNotSupported;
  }
}

// Tensor-core (split-TF32, tcgen05) form of launch_xy_l2 for N = 256: same ring, counters
// and schedule, every 256-point transform on the tensor cores. The engine's twiddle buffer
// (tw512) must carry the tcgen05 constant block.
cudaError_t launch_xy_l2_tc(const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                            const float2 *tw512, unsigned *status, cudaStream_t s) {
  using Cfg = XyL2Cfg<256>;
  if (nplanes <= 0) return cudaSuccess;
  if ((reinterpret_cast<uintptr_t>(dst) & 15u) != 0) return cudaErrorNotSupported;
  CUtensorMap msrc;
  if (!encode_rows_map(&msrc, src, 256, (long long)nplanes * 256, Cfg::C)) return cudaErrorNotSupported;
  int ps, sms;
  Scratch *ring;
  cudaError_t e = xy_l2_setup<256>(nplanes, ps, sms, ring);
  if (e != cudaSuccess) return e;
  static int done[2] = {0, 0};
  for (int i = 0; i < 2; ++i) {
    if (done[i]) continue;
    auto kern = i ? k_xy_l2_tc<true> : k_xy_l2_tc<false>;
    if ((e = set_smem_once(kern, kXyTcSmem, done[i])) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  cudaSharedmemCarveoutMaxShared)) != cudaSuccess)
      return e;
  }
  // CTAs per SM from the footprint: shared memory (the kernel plus the driver's reserve
  // per block) against the SM's, at most the kXyTcMinBlocks the register budget was
  // compiled for. (Without a carveout preference the occupancy query returned 1 for this
  // kernel; ncu reports 5 as the shared-memory limit of the launch.) Any number is correct:
  // the schedule needs no co-residency.
  static int per_sm = 0;
  if (per_sm == 0) {
    int dev = 0, smem_sm = 0, reserve = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    per_sm = std::max(1, std::min(kXyTcMinBlocks, smem_sm / (kXyTcSmem + reserve)));
  }
  unsigned *ctr = reinterpret_cast<unsigned *>(g_ctr.p);
  const long long ncount = 2LL * nplanes + 2;
  k_xyl2_clear<<<(unsigned)std::min<long long>((ncount + 255) / 256, 64), 256, 0, s>>>(ctr, ncount);
  const long long items = 2LL * nplanes * (256 / Cfg::C);
  const unsigned grid = (unsigned)std::min<long long>(items, (long long)per_sm * sms);
  auto kern = inverse ? k_xy_l2_tc<true> : k_xy_l2_tc<false>;
  kern<<<grid, kXyTcThreads, kXyTcSmem, s>>>(msrc, reinterpret_cast<float2 *>(ring->p), dst, nplanes, scale,
                                             tw512, ctr, status, Cfg::LAG);
  return cudaGetLastError();
}

// The same over `ncubes` N^3 cubes at unrelated addresses: rmaps[i] (device memory, from
// encode_xy_table_map) describes the rows of source cube i, dsts[i] is its output base.
// ctr: the caller's counters, xy_l2_counter_bytes(n, ncubes) bytes of device memory. Call
// prepare_xy_l2(n) first when the launch is captured in a graph.
cudaError_t launch_xy_l2_table(int n, const CUtensorMap *rmaps, float2 *const *dsts, int ncubes, bool inverse,
                               float scale, const float2 *tw512, unsigned *status, unsigned *ctr, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  if (!ctr) return cudaErrorInvalidValue;
  switch (n) {
    case 256: return launch_common<256>(nullptr, rmaps, dsts, nullptr, 256 * ncubes, inverse, scale, tw512, status, ctr, s);
    case 128: return launch_common<128>(nullptr, rmaps, dsts, nullptr, 128 * ncubes, inverse, scale, tw512, status, ctr, s);
    case 512: return launch_common<512>(nullptr, rmaps, dsts, nullptr, 512 * ncubes, inverse, scale, tw512, status, ctr, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace convgpu
