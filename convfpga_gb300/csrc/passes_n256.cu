// Pass-kernel launchers for cubes of size 256 (see pass_launch.cuh), including the
// tensor-core split-precision kernels (tc.cuh), which exist for this size only.
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"
#include "tc.cuh"

#include <algorithm>

namespace convgpu {
template cudaError_t launch_size<256>(const PassReq &);
template cudaError_t prepare_size<256>();

template <class P, int OP>
static cudaError_t launch_tc256(int axis, PassArgs a, int nvol, cudaStream_t s) {
  constexpr int N = 256;
  if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
  if (axis == 0) {
    if constexpr (OP == OP_FWD || OP == OP_INV) {
      constexpr int XC = 16;
      constexpr int smem = 128 + XC * N * 8 + XC * 272 * 8 + N * 8;
      CUtensorMap m;
      const long long rows = (long long)nvol * N * N;
      if (!encode_rows_map(&m, a.src, N, rows, XC)) return cudaErrorNotSupported;
      auto kern = k_rows_tma_tc256<P, OP>;
      static int done = 0;
      cudaError_t e = set_smem_once(kern, smem, done);
      if (e != cudaSuccess) return e;
      kern<<<(unsigned)(rows / XC), 256, smem, s>>>(m, a);
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }
  constexpr int smem = tma_pass_smem_bytes<N, 16, OP>();
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  CUtensorMap msrc, mfilt;
  if (!encode_cube_map(&msrc, a.src, N, (long long)nvol * N, axis, 16)) return cudaErrorNotSupported;
  if (HAS_F) {
    const long long fplanes = a.filt_vol_elems ? (long long)nvol * N : (long long)N;
    if (!encode_cube_map(&mfilt, a.filt, N, fplanes, axis, 16)) return cudaErrorNotSupported;
  } else {
    mfilt = msrc;
  }
  auto kern = k_strided_tma_tc256<P, OP>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, smem, done);
  if (e != cudaSuccess) return e;
  a.vol_elems = 256LL * 256 * 256;
  a.groups_x = 256 / 16;
  a.groups_per_vol = 256 * (256 / 16);
  a.axis_stride = axis == 1 ? 256 : 256LL * 256;
  a.plane_pitch = axis == 1 ? 256LL * 256 : 256;
  const long long blocks = (long long)nvol * a.groups_per_vol;
  kern<<<(unsigned)blocks, 256, smem, s>>>(msrc, mfilt, a, axis);
  return cudaGetLastError();
}

template <class P>
static cudaError_t launch_tc256_op(int op, int axis, const PassArgs &a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_tc256<P, OP_FWD>(axis, a, nvol, s);
    case OP_INV: return launch_tc256<P, OP_INV>(axis, a, nvol, s);
    case OP_CONV: return launch_tc256<P, OP_CONV>(axis, a, nvol, s);
    case OP_CONV_FZ: return launch_tc256<P, OP_CONV_FZ>(axis, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

// Tensor-core pass of a 256^3 batch; cudaErrorNotSupported when tensor maps cannot
// describe the operands (the caller then runs the FP32 kernels).
cudaError_t launch_tc256_entry(const PassReq &r, int bf16x3) {
  return bf16x3 ? launch_tc256_op<PrecBf16x3>(r.op, r.axis, r.a, r.nvol, r.s)
                : launch_tc256_op<PrecTf32x3>(r.op, r.axis, r.a, r.nvol, r.s);
}
}  // namespace convgpu

#include "xy256.cuh"

namespace convgpu {

// Fused x + y pass over `nplanes` consecutive 256 x 256 planes (see xy256.cuh).
// cudaErrorNotSupported when the operands cannot be described by a tensor map.
cudaError_t launch_xy256(const float2 *src, float2 *dst, int nplanes, bool inverse, float scale, const float2 *tw512,
                         unsigned int *status, cudaStream_t s) {
  if (nplanes <= 0) return cudaSuccess;
  if ((reinterpret_cast<uintptr_t>(dst) & 15u) != 0) return cudaErrorNotSupported;
  CUtensorMap m;
  if (!encode_rows_map(&m, src, 256, (long long)nplanes * 256, kXyRows)) return cudaErrorNotSupported;
  auto kern = inverse ? k_xy256<true> : k_xy256<false>;
  static int done[2] = {0, 0};
  cudaError_t e = set_smem_once(kern, kXySmem, done[inverse ? 1 : 0]);
  if (e != cudaSuccess) return e;
  static int max_clusters[2] = {0, 0};
  int &mc = max_clusters[inverse ? 1 : 0];
  if (mc == 0) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(kXyCluster * 64, 1, 1);
    cfg.blockDim = dim3(kXyThreads, 1, 1);
    cfg.dynamicSmemBytes = kXySmem;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (const void *)kern, &cfg) != cudaSuccess || n <= 0) {
      cudaGetLastError();
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      n = std::max(1, sms / kXyCluster);
    }
    mc = n;
  }
  const int clusters = std::min(mc, nplanes);
  kern<<<clusters * kXyCluster, kXyThreads, kXySmem, s>>>(m, dst, nplanes, scale, tw512, status);
  return cudaGetLastError();
}

}  // namespace convgpu
