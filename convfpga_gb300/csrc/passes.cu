// Dispatch of the per-axis passes: tensor-map encoding, the device status word, the
// per-size plan table (shape variant per pass kind) and the entry points the runtime
// calls. The kernels of each cube size are instantiated in passes_n<N>.cu.
//
// Every supported N (16..512, the reference's LOG_FFT_SIZE range 4..9,
// kernels/CMakeLists.txt:31-32) is compiled in and chosen at run time.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "engine_internal.h"
#include "pass_launch.cuh"

namespace convgpu {

// Word 0: the device status word (kStatus* bits, OR-ed in by kernels whose bounded wait
// gave up). Word 1: the dependency-wait limit that tests may lower (tma.cuh:
// dep_wait_limit; 0 = every wait's own limit). Kernels get the address of word 0.
__device__ unsigned int g_device_words[2] = {0u, 0u};

extern template cudaError_t launch_size<16>(const PassReq &);
extern template cudaError_t launch_size<32>(const PassReq &);
extern template cudaError_t launch_size<64>(const PassReq &);
extern template cudaError_t launch_size<128>(const PassReq &);
extern template cudaError_t launch_size<256>(const PassReq &);
extern template cudaError_t launch_size<512>(const PassReq &);
extern template cudaError_t prepare_size<16>();
extern template cudaError_t prepare_size<32>();
extern template cudaError_t prepare_size<64>();
extern template cudaError_t prepare_size<128>();
extern template cudaError_t prepare_size<256>();
extern template cudaError_t prepare_size<512>();

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

// Tensor map over `nplanes` consecutive planes of n rows of `width` complex64 values
// (8-byte elements), dims (x, y, plane) = (width, n, nplanes); box {cols, 1 or nbox,
// nbox or 1}.
bool encode_pitched_map(CUtensorMap *m, const void *base, int width, int n, long long nplanes, int axis, int cols) {
  auto enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15u) != 0 || nplanes > 0x7fffffffLL || (width & 1)) return false;
  const cuuint32_t nbox = (cuuint32_t)(n > 256 ? 256 : n);
  cuuint64_t dims[3] = {(cuuint64_t)width, (cuuint64_t)n, (cuuint64_t)nplanes};
  cuuint64_t strides[2] = {(cuuint64_t)width * 8, (cuuint64_t)width * n * 8};
  cuuint32_t box[3] = {(cuuint32_t)cols, axis == 1 ? nbox : 1u, axis == 1 ? 1u : nbox};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void *>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Tensor map over `nplanes` consecutive N x N planes of complex64 (8-byte elements),
// dims (x, y, plane) = (N, N, nplanes); box {cols, 1 or nbox, nbox or 1}.
bool encode_cube_map(CUtensorMap *m, const void *base, int n, long long nplanes, int axis, int cols) {
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
bool encode_rows_map(CUtensorMap *m, const void *base, int n, long long rows, int xc) {
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

// Tensor map over `rows` rows of 512 complex64 viewed as (x, half, row) = (256, 2, rows),
// box {256, 2, xc}: one load lands xc whole rows, each contiguous in shared memory (a
// 2D box is at most 256 wide).
bool encode_rows512_map(CUtensorMap *m, const void *base, long long rows, int xc) {
  auto enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15u) != 0 || rows > 0x7fffffffLL) return false;
  cuuint64_t dims[3] = {256, 2, (cuuint64_t)rows};
  cuuint64_t strides[2] = {256 * 8, 512 * 8};
  cuuint32_t box[3] = {256, 2, (cuuint32_t)xc};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void *>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Box shapes of shape variant 0 (the variant table-mode launches use).
static void v0_shape(int n, int &xc, int &sc) {
  switch (n) {
    case 16: xc = Shape<16, 0>::XC, sc = Shape<16, 0>::SC; break;
    case 32: xc = Shape<32, 0>::XC, sc = Shape<32, 0>::SC; break;
    case 64: xc = Shape<64, 0>::XC, sc = Shape<64, 0>::SC; break;
    case 128: xc = Shape<128, 0>::XC, sc = Shape<128, 0>::SC; break;
    case 256: xc = Shape<256, 0>::XC, sc = Shape<256, 0>::SC; break;
    default: xc = Shape<512, 0>::XC, sc = Shape<512, 0>::SC; break;
  }
}

bool encode_table_map(CUtensorMap *m, const void *cube, int n, int kind) {
  int xc, sc;
  v0_shape(n, xc, sc);
  if (kind == 0) return encode_rows_map(m, cube, n, (long long)n * n, xc);
  return encode_cube_map(m, cube, n, n, kind, sc);
}

// ------------------------------------------------------------------ status word
unsigned int *device_status_address() {
  constexpr int kMaxDev = 64;
  static std::atomic<unsigned int *> cache[kMaxDev];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
  unsigned int *p = cache[dev].load();
  if (!p) {
    void *q = nullptr;
    if (cudaGetSymbolAddress(&q, g_device_words) != cudaSuccess) return nullptr;
    p = static_cast<unsigned int *>(q);
    cache[dev].store(p);
  }
  return p;
}

unsigned int read_and_clear_device_status() {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_device_words, sizeof(v)) != cudaSuccess) return ~0u;
  const unsigned int zero = 0;
  cudaMemcpyToSymbol(g_device_words, &zero, sizeof(zero));
  return v;
}

cudaError_t set_dependency_wait_limit(int probes) {
  const unsigned int v = probes < 0 ? 0u : (unsigned int)probes + 1u;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(g_device_words, &v, sizeof(v), sizeof(unsigned int));
  if (e != cudaSuccess) return e;
  return cudaDeviceSynchronize();
}

// ------------------------------------------------------------------ plan table
static bool g_use_tma = true;
void set_tma_enabled(bool on) { g_use_tma = on; }

static std::atomic<int> g_variant[6][kPassKinds];

static int size_index(int n) {
  switch (n) {
    case 16: return 0;
    case 32: return 1;
    case 64: return 2;
    case 128: return 3;
    case 256: return 4;
    case 512: return 5;
    default: return -1;
  }
}

int pass_kind(int axis, int op) {
  if (axis == 0) return kKindRows;
  if (op == OP_CONV) return kKindConv;
  if (op == OP_CONV_FZ) return kKindConvFz;
  return kKindStrided;
}

void set_pass_variant(int n, int kind, int variant) {
  const int i = size_index(n);
  if (i >= 0 && kind >= 0 && kind < kPassKinds)
    g_variant[i][kind].store(kind == kKindXy ? (variant < 0 ? 0 : (variant > 2 ? 2 : variant)) : (variant ? 1 : 0));
}

int get_pass_variant(int n, int kind) {
  const int i = size_index(n);
  return (i >= 0 && kind >= 0 && kind < kPassKinds) ? g_variant[i][kind].load() : 0;
}

static cudaError_t dispatch(int n, const PassReq &r) {
  switch (n) {
    case 16: return launch_size<16>(r);
    case 32: return launch_size<32>(r);
    case 64: return launch_size<64>(r);
    case 128: return launch_size<128>(r);
    case 256: return launch_size<256>(r);
    case 512: return launch_size<512>(r);
    default: return cudaErrorInvalidValue;
  }
}

static PassArgs make_args(int n, const float2 *src, float2 *dst, const float2 *filt, long long filt_vol_elems,
                          float scale, const float2 *tw512) {
  PassArgs a{};
  a.src = src;
  a.dst = dst;
  a.filt = filt;
  a.tw512 = tw512;
  a.filt_vol_elems = filt_vol_elems;
  a.scale = scale;
  a.vol_elems = (long long)n * n * n;
  a.status = device_status_address();
  return a;
}

// ------------------------------------------------------------------ entry points
cudaError_t launch_axis_pass_variant(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                                     long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                     cudaStream_t s, int variant) {
  if (nvol <= 0) return cudaSuccess;
  if ((op == OP_CONV || op == OP_CONV_FZ) && axis != 2) return cudaErrorInvalidValue;
  if (size_index(n) < 0) return cudaErrorInvalidValue;
  PassReq r{};
  r.mode = g_use_tma ? kModeTma : kModeGather;
  r.axis = axis;
  r.op = op;
  r.nvol = nvol;
  r.nplanes = nvol * n;
  r.variant = variant;
  r.a = make_args(n, src, dst, filt, filt_vol_elems, scale, tw512);
  r.s = s;
  return dispatch(n, r);
}

cudaError_t launch_axis_pass(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                             long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                             cudaStream_t s) {
  return launch_axis_pass_variant(n, axis, op, src, dst, filt, filt_vol_elems, nvol, scale, tw512, s,
                                  get_pass_variant(n, pass_kind(axis, op)));
}

cudaError_t launch_axis_pass_planes(int n, int axis, int op, const float2 *src, float2 *dst, int nplanes, float scale,
                                    const float2 *tw512, cudaStream_t s) {
  if (nplanes <= 0) return cudaSuccess;
  if (axis > 1 || (op != OP_FWD && op != OP_INV) || size_index(n) < 0) return cudaErrorInvalidValue;
  PassReq r{};
  r.mode = g_use_tma ? kModeTma : kModeGather;
  r.axis = axis;
  r.op = op;
  r.nvol = (nplanes + n - 1) / n;
  r.nplanes = nplanes;
  r.variant = get_pass_variant(n, pass_kind(axis, op));
  r.a = make_args(n, src, dst, nullptr, 0, scale, tw512);
  r.s = s;
  return dispatch(n, r);
}

cudaError_t prepare_table_launches(int n) {
  switch (n) {
    case 16: return prepare_size<16>();
    case 32: return prepare_size<32>();
    case 64: return prepare_size<64>();
    case 128: return prepare_size<128>();
    case 256: return prepare_size<256>();
    case 512: return prepare_size<512>();
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_axis_pass_table(int n, int axis, int op, const CUtensorMap *maps, const CUtensorMap *fmaps,
                                   float2 *const *dsts, int nvol, float scale, const float2 *tw512,
                                   cudaStream_t s) {
  if (nvol <= 0) return cudaSuccess;
  if ((op == OP_CONV || op == OP_CONV_FZ) && (axis != 2 || !fmaps)) return cudaErrorInvalidValue;
  if (size_index(n) < 0) return cudaErrorInvalidValue;
  PassReq r{};
  r.mode = kModeTable;
  r.axis = axis;
  r.op = op;
  r.nvol = nvol;
  r.nplanes = nvol * n;
  r.a = make_args(n, nullptr, nullptr, nullptr, (long long)n * n * n, scale, tw512);
  r.a.maps = maps;
  r.a.fmaps = fmaps;
  r.a.dsts = dsts;
  r.s = s;
  return dispatch(n, r);
}

cudaError_t launch_axis_pass_real(int n, const float *src, float2 *dst, int nvol, const float2 *tw512,
                                  cudaStream_t s) {
  if (nvol <= 0) return cudaSuccess;
  if (size_index(n) < 0) return cudaErrorInvalidValue;
  PassReq r{};
  r.mode = kModeGather;
  r.axis = 0;
  r.op = OP_FWD;
  r.nvol = nvol;
  r.nplanes = nvol * n;
  r.variant = get_pass_variant(n, kKindRows);
  r.real_src = true;
  r.a = make_args(n, reinterpret_cast<const float2 *>(src), dst, nullptr, 0, 1.f, tw512);
  r.s = s;
  return dispatch(n, r);
}

cudaError_t launch_axis_pass_half(int n, int axis, int op, const void *src, float2 *dst, const float2 *filt,
                                  long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                  cudaStream_t s) {
  if (nvol <= 0) return cudaSuccess;
  if (size_index(n) < 0 || half_pitch(n) == 0 || !g_use_tma) return cudaErrorNotSupported;
  PassReq r{};
  r.mode = kModeTma;
  r.axis = axis;
  r.op = op;
  r.nvol = nvol;
  r.nplanes = nvol * n;
  r.variant = get_pass_variant(n, kKindRows);
  r.real_src = axis == 0;
  r.half = half_pitch(n);
  r.a = make_args(n, reinterpret_cast<const float2 *>(src), dst, filt, filt_vol_elems, scale, tw512);
  r.s = s;
  return dispatch(n, r);
}

int half_spectrum_pitch(int n) { return half_pitch(n); }

cudaError_t launch_axis_pass_tc(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                                long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                cudaStream_t s, int prec) {
  // The tensor-core kernels cover N = 256 (two radix-16 stages per axis, TF32x3 on tcgen05
  // or mma.sync, BF16x3 on mma.sync) and N = 512 in TF32x3 (a radix-2 step around two
  // 256-point tcgen05 transforms); other sizes and precisions, and operands that tensor
  // maps cannot describe, run the FP32 kernels.
  const bool tc512 = n == 512 && prec == kTcTf32x3;
  if ((n != 256 && !tc512) || nvol <= 0 || !g_use_tma)
    return launch_axis_pass(n, axis, op, src, dst, filt, filt_vol_elems, nvol, scale, tw512, s);
  if ((op == OP_CONV || op == OP_CONV_FZ) && axis != 2) return cudaErrorInvalidValue;
  PassReq r{};
  r.mode = kModeTma;
  r.axis = axis;
  r.op = op;
  r.nvol = nvol;
  r.nplanes = nvol * n;
  r.a = make_args(n, src, dst, filt, filt_vol_elems, scale, tw512);
  r.s = s;
  // split TF32: tcgen05 kernels (plan kind kKindTc, variant 0) or mma.sync (variant 1);
  // BF16x3: mma.sync
  const cudaError_t e = tc512 ? launch_tc05_512_entry(r)
                        : (prec == kTcTf32x3 && get_pass_variant(n, kKindTc) == 0)
                            ? launch_tc05_entry(r)
                            : launch_tc256_entry(r, prec == kTcBf16x3 ? 1 : 0);
  if (e == cudaErrorNotSupported)
    return launch_axis_pass(n, axis, op, src, dst, filt, filt_vol_elems, nvol, scale, tw512, s);
  return e;
}

cudaError_t launch_xy_pass(int n, const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                           const float2 *tw512, cudaStream_t s, int variant) {
  if (!g_use_tma) return cudaErrorNotSupported;
  if (n == 128 || n == 512)
    return variant == 1 ? launch_xy_l2(n, src, dst, nplanes, inverse, scale, tw512, device_status_address(), s)
                        : cudaErrorNotSupported;
  if (n != 256) return cudaErrorNotSupported;
  if (variant == 2) return launch_xy256(src, dst, nplanes, inverse, scale, tw512, device_status_address(), s);
  return launch_xy_l2(256, src, dst, nplanes, inverse, scale, tw512, device_status_address(), s);
}

cudaError_t launch_xy_l2_tc_pass(int n, const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                                 const float2 *tw512, cudaStream_t s) {
  if (n != 256 || !g_use_tma) return cudaErrorNotSupported;
  return launch_xy_l2_tc(src, dst, nplanes, inverse, scale, tw512, device_status_address(), s);
}

cudaError_t probe_kernel_image() {
  // A trivial launch-free query on one kernel of this library's image.
  return prepare_size<16>();
}

}  // namespace convgpu
