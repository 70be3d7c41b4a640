// Instantiation and launch of the per-axis pass kernels, one shape per cube size.
//
// The shapes (radix list, elements per thread E, pencils per CTA) replace the
// reference's compile-time FFT size (kernels/common/conv_config.h.in:8-11): every
// supported N (16..512, the reference's LOG_FFT_SIZE range 4..9) is compiled in and
// chosen at run time.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "engine_internal.h"
#include "passes.cuh"
#include "tc.cuh"

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

// ------------------------------------------------------------------ TMA descriptors
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q{};
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// Tensor map over `nplanes` consecutive N x N planes of complex64 (8-byte elements),
// dims (x, y, plane) = (N, N, nplanes); box {cols, 1 or nbox, nbox or 1}.
static bool encode_cube_map(CUtensorMap *m, const void *base, int n, long long nplanes, int axis, int cols) {
  auto enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15u) != 0 || nplanes > 0x7fffffffLL) return false;
  const cuuint32_t nbox = (cuuint32_t)(n > 256 ? 256 : n);
  cuuint64_t dims[3] = {(cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)nplanes};
  cuuint64_t strides[2] = {(cuuint64_t)n * 8, (cuuint64_t)n * n * 8};
  cuuint32_t box[3] = {(cuuint32_t)cols, axis == 1 ? nbox : 1u, axis == 1 ? 1u : nbox};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void *>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Tensor map over `rows` rows of N complex64: dims (x, row) = (N, rows), box
// {min(N,256), xc}.
static bool encode_rows_map(CUtensorMap *m, const void *base, int n, long long rows, int xc) {
  auto enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15u) != 0 || rows > 0x7fffffffLL) return false;
  cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)n * 8};
  cuuint32_t box[2] = {(cuuint32_t)(n > 256 ? 256 : n), (cuuint32_t)xc};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void *>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int N, int OP>
static cudaError_t launch_rows_tma(PassArgs a, int nvol, cudaStream_t s) {
  using S = Shape<N>;
  constexpr int E = S::E;
  constexpr int XC = S::XC;
  constexpr int threads = XC * (N / E);
  constexpr int smem = tma_rows_smem_bytes<N, XC>();
  if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
  const long long rows = (long long)nvol * N * N;
  CUtensorMap msrc;
  if (!encode_rows_map(&msrc, a.src, N, rows, XC)) return cudaErrorNotSupported;
  auto kern = k_rows_tma<N, E, XC, OP, typename S::Plan>;
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  const long long blocks = rows / XC;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, threads, smem, s>>>(msrc, a);
  return cudaGetLastError();
}

// Strided pass through the TMA kernel. Returns cudaErrorNotSupported when the
// operands cannot be described by tensor maps (unaligned pointers), so the caller can
// use the register-gather kernel instead.
template <int N, int OP>
static cudaError_t launch_tma(int axis, PassArgs a, int nvol, cudaStream_t s) {
  using S = Shape<N>;
  constexpr int E = S::E;
  constexpr int COLS = S::SC;
  constexpr int threads = COLS * (N / E);
  constexpr int smem = tma_pass_smem_bytes<N, COLS, OP>();
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
  CUtensorMap msrc, mfilt;
  if (!encode_cube_map(&msrc, a.src, N, (long long)nvol * N, axis, COLS)) return cudaErrorNotSupported;
  if (HAS_F) {
    const long long fplanes = a.filt_vol_elems ? (long long)nvol * N : (long long)N;
    if (!encode_cube_map(&mfilt, a.filt, N, fplanes, axis, COLS)) return cudaErrorNotSupported;
  } else {
    mfilt = msrc;
  }
  auto kern = k_strided_tma<N, E, COLS, OP, typename S::Plan>;
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  const long long blocks = (long long)nvol * a.groups_per_vol;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, threads, smem, s>>>(msrc, mfilt, a, axis);
  return cudaGetLastError();
}

template <int N>
static cudaError_t launch_tma_op(int axis, int op, PassArgs a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_tma<N, OP_FWD>(axis, a, nvol, s);
    case OP_INV: return launch_tma<N, OP_INV>(axis, a, nvol, s);
    case OP_CONV: return launch_tma<N, OP_CONV>(axis, a, nvol, s);
    case OP_CONV_FZ: return launch_tma<N, OP_CONV_FZ>(axis, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

static bool g_use_tma = true;
void set_tma_enabled(bool on) { g_use_tma = on; }

unsigned int *device_status_address() {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_device_status) != cudaSuccess) return nullptr;
  return static_cast<unsigned int *>(p);
}

unsigned int read_and_clear_device_status() {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_device_status, sizeof(v)) != cudaSuccess) return ~0u;
  const unsigned int zero = 0;
  cudaMemcpyToSymbol(g_device_status, &zero, sizeof(zero));
  return v;
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
  if (axis == 0) {
    if (g_use_tma && (op == OP_FWD || op == OP_INV)) {
      cudaError_t e = op == OP_FWD ? launch_rows_tma<N, OP_FWD>(a, nvol, s) : launch_rows_tma<N, OP_INV>(a, nvol, s);
      if (e != cudaErrorNotSupported) return e;
    }
    return launch_op<N, true>(op, a, nvol, s);
  }
  a.groups_per_vol = N * (N / SC);
  if (axis == 1) {
    a.axis_stride = N;
    a.plane_pitch = (long long)N * N;
  } else {
    a.axis_stride = (long long)N * N;
    a.plane_pitch = N;
  }
  if (g_use_tma) {
    cudaError_t e = launch_tma_op<N>(axis, op, a, nvol, s);
    if (e != cudaErrorNotSupported) return e;
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

// ------------------------------------------------------------------ table mode
bool encode_table_map(CUtensorMap *m, const void *cube, int n, int kind) {
  auto go = [&](auto shape) {
    using S = decltype(shape);
    if (kind == 0) return encode_rows_map(m, cube, n, (long long)n * n, S::XC);
    return encode_cube_map(m, cube, n, n, kind, S::SC);
  };
  switch (n) {
    case 16: return go(Shape<16>{});
    case 32: return go(Shape<32>{});
    case 64: return go(Shape<64>{});
    case 128: return go(Shape<128>{});
    case 256: return go(Shape<256>{});
    case 512: return go(Shape<512>{});
    default: return false;
  }
}

template <int N, int OP>
static cudaError_t launch_table_n(int axis, PassArgs a, int nvol, cudaStream_t s) {
  using S = Shape<N>;
  constexpr int E = S::E;
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof(dummy));
  if (axis == 0) {
    if constexpr (OP == OP_FWD || OP == OP_INV) {
      constexpr int XC = S::XC;
      constexpr int smem = tma_rows_smem_bytes<N, XC>();
      auto kern = k_rows_tma<N, E, XC, OP, typename S::Plan>;  // attributes: prepare_table_launches
      kern<<<(unsigned)((long long)nvol * N * N / XC), XC * (N / E), smem, s>>>(dummy, a);
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }
  constexpr int COLS = S::SC;
  constexpr int smem = tma_pass_smem_bytes<N, COLS, OP>();
  auto kern = k_strided_tma<N, E, COLS, OP, typename S::Plan>;  // attributes: prepare_table_launches
  a.groups_x = N / COLS;
  a.groups_per_vol = N * (N / COLS);
  a.axis_stride = axis == 1 ? N : (long long)N * N;
  a.plane_pitch = axis == 1 ? (long long)N * N : N;
  kern<<<(unsigned)((long long)nvol * a.groups_per_vol), COLS * (N / E), smem, s>>>(dummy, dummy, a, axis);
  return cudaGetLastError();
}

template <int N>
static cudaError_t prepare_table_n() {
  using S = Shape<N>;
  constexpr int E = S::E, XC = S::XC, COLS = S::SC;
  cudaError_t e = cudaSuccess;
  auto set = [&](auto kern, int smem) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  };
  set(k_rows_tma<N, E, XC, OP_FWD, typename S::Plan>, tma_rows_smem_bytes<N, XC>());
  set(k_rows_tma<N, E, XC, OP_INV, typename S::Plan>, tma_rows_smem_bytes<N, XC>());
  set(k_strided_tma<N, E, COLS, OP_FWD, typename S::Plan>, tma_pass_smem_bytes<N, COLS, OP_FWD>());
  set(k_strided_tma<N, E, COLS, OP_INV, typename S::Plan>, tma_pass_smem_bytes<N, COLS, OP_INV>());
  set(k_strided_tma<N, E, COLS, OP_CONV, typename S::Plan>, tma_pass_smem_bytes<N, COLS, OP_CONV>());
  set(k_strided_tma<N, E, COLS, OP_CONV_FZ, typename S::Plan>, tma_pass_smem_bytes<N, COLS, OP_CONV_FZ>());
  return e;
}

cudaError_t prepare_table_launches(int n) {
  switch (n) {
    case 16: return prepare_table_n<16>();
    case 32: return prepare_table_n<32>();
    case 64: return prepare_table_n<64>();
    case 128: return prepare_table_n<128>();
    case 256: return prepare_table_n<256>();
    case 512: return prepare_table_n<512>();
    default: return cudaErrorInvalidValue;
  }
}

template <int N>
static cudaError_t launch_table_op(int axis, int op, PassArgs a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_table_n<N, OP_FWD>(axis, a, nvol, s);
    case OP_INV: return launch_table_n<N, OP_INV>(axis, a, nvol, s);
    case OP_CONV: return launch_table_n<N, OP_CONV>(axis, a, nvol, s);
    case OP_CONV_FZ: return launch_table_n<N, OP_CONV_FZ>(axis, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_axis_pass_table(int n, int axis, int op, const CUtensorMap *maps, const CUtensorMap *fmaps,
                                   float2 *const *dsts, int nvol, float scale, const float2 *tw512,
                                   cudaStream_t s) {
  if (nvol <= 0) return cudaSuccess;
  if ((op == OP_CONV || op == OP_CONV_FZ) && (axis != 2 || !fmaps)) return cudaErrorInvalidValue;
  PassArgs a{};
  a.tw512 = tw512;
  a.scale = scale;
  a.vol_elems = (long long)n * n * n;
  a.filt_vol_elems = (long long)n * n * n;
  a.maps = maps;
  a.fmaps = fmaps;
  a.dsts = dsts;
  switch (n) {
    case 16: return launch_table_op<16>(axis, op, a, nvol, s);
    case 32: return launch_table_op<32>(axis, op, a, nvol, s);
    case 64: return launch_table_op<64>(axis, op, a, nvol, s);
    case 128: return launch_table_op<128>(axis, op, a, nvol, s);
    case 256: return launch_table_op<256>(axis, op, a, nvol, s);
    case 512: return launch_table_op<512>(axis, op, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

// ------------------------------------------------------------------ tensor-core path
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
      static bool attr_done = false;
      if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_done = true;
      }
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
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  const long long blocks = (long long)nvol * a.groups_per_vol;
  kern<<<(unsigned)blocks, 256, smem, s>>>(msrc, mfilt, a, axis);
  return cudaGetLastError();
}

template <class P>
static cudaError_t launch_tc256_op(int op, int axis, PassArgs a, int nvol, cudaStream_t s) {
  switch (op) {
    case OP_FWD: return launch_tc256<P, OP_FWD>(axis, a, nvol, s);
    case OP_INV: return launch_tc256<P, OP_INV>(axis, a, nvol, s);
    case OP_CONV: return launch_tc256<P, OP_CONV>(axis, a, nvol, s);
    case OP_CONV_FZ: return launch_tc256<P, OP_CONV_FZ>(axis, a, nvol, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_axis_pass_tc(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                                long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                cudaStream_t s, int prec) {
  // The tensor-core kernels cover N = 256 (two radix-16 stages per axis); other sizes,
  // and operands that tensor maps cannot describe, run the FP32 kernels.
  if (n != 256 || nvol <= 0 || !g_use_tma)
    return launch_axis_pass(n, axis, op, src, dst, filt, filt_vol_elems, nvol, scale, tw512, s);
  if ((op == OP_CONV || op == OP_CONV_FZ) && axis != 2) return cudaErrorInvalidValue;
  PassArgs a{};
  a.src = src;
  a.dst = dst;
  a.filt = filt;
  a.tw512 = tw512;
  a.filt_vol_elems = filt_vol_elems;
  a.scale = scale;
  a.vol_elems = 256LL * 256 * 256;
  a.groups_x = 256 / 16;
  a.groups_per_vol = 256 * (256 / 16);
  a.axis_stride = axis == 1 ? 256 : 256LL * 256;
  a.plane_pitch = axis == 1 ? 256LL * 256 : 256;
  const cudaError_t e = prec == kTcBf16x3 ? launch_tc256_op<PrecBf16x3>(op, axis, a, nvol, s)
                                           : launch_tc256_op<PrecTf32x3>(op, axis, a, nvol, s);
  if (e == cudaErrorNotSupported)
    return launch_axis_pass(n, axis, op, src, dst, filt, filt_vol_elems, nvol, scale, tw512, s);
  return e;
}

cudaError_t probe_kernel_image() {
  cudaFuncAttributes fa;
  return cudaFuncGetAttributes(&fa, (const void *)k_axis_pass<16, Shape<16>::E, Shape<16>::SC, false, OP_FWD,
                                                              Shape<16>::Plan>);
}

}  // namespace convgpu
