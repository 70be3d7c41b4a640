// Instantiation and launch of the per-axis pass kernels, one shape per cube size.
//
// The shapes (radix list, elements per thread E, pencils per CTA) replace the
// reference's compile-time FFT size (kernels/common/conv_config.h.in:8-11): every
// supported N (16..512, the reference's LOG_FFT_SIZE range 4..9) is compiled in and
// chosen at run time.
#include <cuda_runtime.h>

#include "engine_internal.h"
#include "passes.cuh"

namespace convgpu {

template <int N>
struct Shape;
// E: elements per thread; XC: rows per CTA in the x pass; SC: columns per CTA in the
// y / z passes (SC*8 bytes per contiguous global run).
template <>
struct Shape<16> {
  static constexpr int E = 4, XC = 32, SC = 16;
  using Plan = Radices<4, 4>;
};
template <>
struct Shape<32> {
  static constexpr int E = 8, XC = 32, SC = 32;
  using Plan = Radices<8, 4>;
};
template <>
struct Shape<64> {
  static constexpr int E = 8, XC = 16, SC = 32;
  using Plan = Radices<8, 8>;
};
template <>
struct Shape<128> {
  static constexpr int E = 16, XC = 16, SC = 32;
  using Plan = Radices<16, 8>;
};
template <>
struct Shape<256> {
  static constexpr int E = 16, XC = 8, SC = 16;
  using Plan = Radices<16, 16>;
};
template <>
struct Shape<512> {
  static constexpr int E = 16, XC = 4, SC = 16;
  using Plan = Radices<16, 16, 2>;
};

template <int N, bool CONTIG, int OP>
static cudaError_t launch_shape(PassArgs a, int nvol, cudaStream_t s) {
  using S = Shape<N>;
  constexpr int E = S::E;
  constexpr int COLS = CONTIG ? S::XC : S::SC;
  constexpr int threads = COLS * (N / E);
  constexpr int smem = pass_smem_bytes<N, E, COLS, CONTIG>();
  auto kern = k_axis_pass<N, E, COLS, CONTIG, OP, typename S::Plan>;
  static bool attr_done = false;  // per template instance; set once per process
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  long long blocks;
  if constexpr (CONTIG) {
    blocks = (long long)nvol * N * N / COLS;
  } else {
    blocks = (long long)nvol * a.groups_per_vol;
  }
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, threads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N, bool CONTIG>
static cudaError_t launch_op(int op, PassArgs a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_shape<N, CONTIG, OP_FWD>(a, nvol, s);
    case OP_INV: return launch_shape<N, CONTIG, OP_INV>(a, nvol, s);
    case OP_CONV:
      if constexpr (!CONTIG) return launch_shape<N, CONTIG, OP_CONV>(a, nvol, s);
      break;
    case OP_CONV_FZ:
      if constexpr (!CONTIG) return launch_shape<N, CONTIG, OP_CONV_FZ>(a, nvol, s);
      break;
    default: break;
  }
  return cudaErrorInvalidValue;
}

template <int N>
static cudaError_t launch_n(int axis, int op, PassArgs a, int nvol, cudaStream_t s) {
  constexpr int SC = Shape<N>::SC;
  a.vol_elems = (long long)N * N * N;
  a.groups_x = N / SC;
  if (axis == 0) return launch_op<N, true>(op, a, nvol, s);
  a.groups_per_vol = N * (N / SC);
  if (axis == 1) {
    a.axis_stride = N;
    a.plane_pitch = (long long)N * N;
  } else {
    a.axis_stride = (long long)N * N;
    a.plane_pitch = N;
  }
  return launch_op<N, false>(op, a, nvol, s);
}

cudaError_t launch_axis_pass(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                             long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                             cudaStream_t s) {
  PassArgs a{};
  a.src = src;
  a.dst = dst;
  a.filt = filt;
  a.tw512 = tw512;
  a.filt_vol_elems = filt_vol_elems;
  a.scale = scale;
  if (nvol <= 0) return cudaSuccess;
  if ((op == OP_CONV || op == OP_CONV_FZ) && axis != 2) return cudaErrorInvalidValue;
  switch (n) {
    case 16: return launch_n<16>(axis, op, a, nvol, s);
    case 32: return launch_n<32>(axis, op, a, nvol, s);
    case 64: return launch_n<64>(axis, op, a, nvol, s);
    case 128: return launch_n<128>(axis, op, a, nvol, s);
    case 256: return launch_n<256>(axis, op, a, nvol, s);
    case 512: return launch_n<512>(axis, op, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t probe_kernel_image() {
  cudaFuncAttributes fa;
  return cudaFuncGetAttributes(&fa, (const void *)k_axis_pass<16, Shape<16>::E, Shape<16>::SC, false, OP_FWD,
                                                              Shape<16>::Plan>);
}

}  // namespace convgpu
