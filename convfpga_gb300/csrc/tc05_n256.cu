// Launchers of the tcgen05 split-TF32 pass kernels for 256^3 cubes (tc05.cuh). Same
// tensor maps and grids as the FP32 TMA kernels of this size: the x pass takes 16 rows
// per CTA (box {256, 16}), the y / z passes 16 columns x 256 positions per CTA.
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"
#include "tc05.cuh"

namespace convgpu {

template <int SW, int OP>
static cudaError_t launch_tc05(int axis, PassArgs a, int nvol, cudaStream_t s) {
  constexpr int N = 256;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
  if (axis == 0) {
    if constexpr (OP == OP_FWD || OP == OP_INV) {
      CUtensorMap m;
      const long long rows = (long long)nvol * N * N;
      if (!encode_rows_map(&m, a.src, N, rows, 16)) return cudaErrorNotSupported;
      auto kern = k_tc05_256<SW, OP, true>;
      static bool done = false;
      cudaError_t e = set_smem_once(kern, kT5Smem, done);
      if (e != cudaSuccess) return e;
      kern<<<(unsigned)(rows / 16), kT5Threads, kT5Smem, s>>>(m, m, a, 0);
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }
  CUtensorMap msrc, mfilt;
  if (!encode_cube_map(&msrc, a.src, N, (long long)nvol * N, axis, 16)) return cudaErrorNotSupported;
  if (HAS_F) {
    const long long fplanes = a.filt_vol_elems ? (long long)nvol * N : (long long)N;
    if (!encode_cube_map(&mfilt, a.filt, N, fplanes, axis, 16)) return cudaErrorNotSupported;
  } else {
    mfilt = msrc;
  }
  auto kern = k_tc05_256<SW, OP, false>;
  static bool done = false;
  cudaError_t e = set_smem_once(kern, kT5Smem, done);
  if (e != cudaSuccess) return e;
  a.vol_elems = 256LL * 256 * 256;
  a.groups_x = 256 / 16;
  a.groups_per_vol = 256 * (256 / 16);
  a.axis_stride = axis == 1 ? 256 : 256LL * 256;
  a.plane_pitch = axis == 1 ? 256LL * 256 : 256;
  const long long blocks = (long long)nvol * a.groups_per_vol;
  kern<<<(unsigned)blocks, kT5Threads, kT5Smem, s>>>(msrc, mfilt, a, axis);
  return cudaGetLastError();
}

template <int SW>
static cudaError_t launch_tc05_op(int op, int axis, const PassArgs &a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_tc05<SW, OP_FWD>(axis, a, nvol, s);
    case OP_INV: return launch_tc05<SW, OP_INV>(axis, a, nvol, s);
    case OP_CONV: return launch_tc05<SW, OP_CONV>(axis, a, nvol, s);
    case OP_CONV_FZ: return launch_tc05<SW, OP_CONV_FZ>(axis, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

// tcgen05 pass of a 256^3 batch; swizzle selects the operand layout (0: none,
// 1: 128-byte swizzle). cudaErrorNotSupported when tensor maps cannot describe the
// operands (the caller then runs the FP32 kernels).
cudaError_t launch_tc05_entry(const PassReq &r, int swizzle) {
  return swizzle ? launch_tc05_op<1>(r.op, r.axis, r.a, r.nvol, r.s) : launch_tc05_op<0>(r.op, r.axis, r.a, r.nvol, r.s);
}

}  // namespace convgpu
