// Launchers of the tcgen05 split-TF32 pass kernels for 256^3 cubes (tc05.cuh): the x
// pass takes P = 8 rows per CTA (box {256, 8}), the y / z passes 8 columns x 256
// positions per CTA (5 CTAs per SM).
#define CONVGPU_PASS_LAUNCH_IMPL
#include "pass_launch.cuh"
#include "tc05.cuh"

namespace convgpu {

template <int P, int OP>
static cudaError_t launch_tc05(int axis, PassArgs a, int nvol, cudaStream_t s) {
  constexpr int N = 256;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
  if (axis == 0) {
    if constexpr (OP == OP_FWD || OP == OP_INV) {
      CUtensorMap m;
      const long long rows = (long long)nvol * N * N;
      if (!encode_rows_map(&m, a.src, N, rows, P)) return cudaErrorNotSupported;
      auto kern = k_tc05_256<P, OP, true>;
      static int done = 0;
      cudaError_t e = set_smem_once(kern, T5Geom<P>::kSmem, done);
      if (e != cudaSuccess) return e;
      kern<<<(unsigned)(rows / P), T5Geom<P>::kThreads, T5Geom<P>::kSmem, s>>>(m, m, a, 0);
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
  auto kern = k_tc05_256<P, OP, false>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, T5Geom<P>::kSmem, done);
  if (e != cudaSuccess) return e;
  a.vol_elems = 256LL * 256 * 256;
  a.groups_x = 256 / P;
  a.groups_per_vol = 256 * (256 / P);
  a.axis_stride = axis == 1 ? 256 : 256LL * 256;
  a.plane_pitch = axis == 1 ? 256LL * 256 : 256;
  const long long blocks = (long long)nvol * a.groups_per_vol;
  kern<<<(unsigned)blocks, T5Geom<P>::kThreads, T5Geom<P>::kSmem, s>>>(msrc, mfilt, a, axis);
  return cudaGetLastError();
}

template <int P>
static cudaError_t launch_tc05_op(int op, int axis, const PassArgs &a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_tc05<P, OP_FWD>(axis, a, nvol, s);
    case OP_INV: return launch_tc05<P, OP_INV>(axis, a, nvol, s);
    case OP_CONV: return launch_tc05<P, OP_CONV>(axis, a, nvol, s);
    case OP_CONV_FZ: return launch_tc05<P, OP_CONV_FZ>(axis, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

// tcgen05 pass of a 256^3 batch; r.a.tw512 must carry the constant block
// (tc05_init_consts). cudaErrorNotSupported when tensor maps cannot describe the
// operands (the caller then runs the FP32 kernels).
cudaError_t launch_tc05_entry(const PassReq &r) { return launch_tc05_op<8>(r.op, r.axis, r.a, r.nvol, r.s); }

// Writes the tcgen05 constant block behind the 512 twiddles of `tw` (a buffer of at
// least kTwiddleBufBytes bytes) and waits for it.
cudaError_t tc05_init_consts(float2 *tw, cudaStream_t s) {
  k_tc05_consts<<<1, 256, 0, s>>>(reinterpret_cast<unsigned char *>(tw) + kT5ConstOffset, tw);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

}  // namespace convgpu
