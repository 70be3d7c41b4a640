// Launchers of the tcgen05 split-TF32 pass kernels for 512^3 cubes (tc05.cuh, k_tc05_512):
// 4 pencils of 512 per CTA (x pass: 4 rows, one box {256, 2, 4}; y / z passes: 4 columns x
// 512 positions, two boxes of 256), 5 CTAs per SM, as the N = 256 kernels with 8 pencils.
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"
#include "tc05.cuh"

namespace convgpu {

template <int OP>
static cudaError_t launch_tc05_512(int axis, PassArgs a, int nvol, cudaStream_t s) {
  constexpr int N = 512, P = 4;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  constexpr int smem = T5Geom<8>::kSmem;
  if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
  if (axis == 0) {
    if constexpr (OP == OP_FWD || OP == OP_INV) {
      CUtensorMap m;
      const long long rows = (long long)nvol * N * N;
      if (!encode_rows512_map(&m, a.src, rows, P)) return cudaErrorNotSupported;
      auto kern = k_tc05_512<OP, true>;
      static int done = 0;
      cudaError_t e = set_smem_once(kern, smem, done);
      if (e != cudaSuccess) return e;
      kern<<<(unsigned)(rows / P), T5Geom<8>::kThreads, smem, s>>>(m, m, a, 0);
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }
  CUtensorMap msrc, mfilt;
  if (!encode_cube_map(&msrc, a.src, N, (long long)nvol * N, axis, P)) return cudaErrorNotSupported;
  if (HAS_F) {
    const long long fplanes = a.filt_vol_elems ? (long long)nvol * N : (long long)N;
    if (!encode_cube_map(&mfilt, a.filt, N, fplanes, axis, P)) return cudaErrorNotSupported;
  } else {
    mfilt = msrc;
  }
  auto kern = k_tc05_512<OP, false>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, smem, done);
  if (e != cudaSuccess) return e;
  a.vol_elems = (long long)N * N * N;
  a.groups_x = N / P;
  a.groups_per_vol = N * (N / P);
  a.axis_stride = axis == 1 ? N : (long long)N * N;
  a.plane_pitch = axis == 1 ? (long long)N * N : N;
  const long long blocks = (long long)nvol * a.groups_per_vol;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, T5Geom<8>::kThreads, smem, s>>>(msrc, mfilt, a, axis);
  return cudaGetLastError();
}

// tcgen05 pass of a 512^3 batch; r.a.tw512 must carry the constant block
// (tc05_init_consts). cudaErrorNotSupported when tensor maps cannot describe the
// operands (the caller then runs the FP32 kernels).
cudaError_t launch_tc05_512_entry(const PassReq &r) {
  switch (r.op) {
    case OP_FWD: return launch_tc05_512<OP_FWD>(r.axis, r.a, r.nvol, r.s);
    case OP_INV: return launch_tc05_512<OP_INV>(r.axis, r.a, r.nvol, r.s);
    case OP_CONV: return launch_tc05_512<OP_CONV>(r.axis, r.a, r.nvol, r.s);
    case OP_CONV_FZ: return launch_tc05_512<OP_CONV_FZ>(r.axis, r.a, r.nvol, r.s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace convgpu
