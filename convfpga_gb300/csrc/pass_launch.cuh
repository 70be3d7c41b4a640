// Launchers of the per-axis pass kernels for one cube size N, templated on N and
// instantiated once per size in passes_n<N>.cu (so the sizes compile in parallel).
//
// Each size has two shape variants (radix list, elements per thread, pencils / rows per
// CTA); a run-time plan table (set by the autotuner, recorded in the plan cache) picks
// one per pass kind. The shapes replace the reference's synthesis-time FFT size and
// fixed 8-points-per-cycle engine (kernels/common/conv_config.h.in:8-11).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "herm.cuh"
#include "passes.cuh"

namespace convgpu {

// E: elements per thread; XC: rows per CTA (x pass); SC: columns per CTA (y / z passes).
template <int N, int V>
struct Shape;
template <> struct Shape<16, 0> { static constexpr int E = 4, XC = 32, SC = 16; using Plan = Radices<4, 4>; };
template <> struct Shape<16, 1> { static constexpr int E = 4, XC = 64, SC = 16; using Plan = Radices<4, 4>; };
template <> struct Shape<32, 0> { static constexpr int E = 8, XC = 32, SC = 32; using Plan = Radices<8, 4>; };
template <> struct Shape<32, 1> { static constexpr int E = 8, XC = 16, SC = 16; using Plan = Radices<4, 8>; };
template <> struct Shape<64, 0> { static constexpr int E = 8, XC = 16, SC = 32; using Plan = Radices<8, 8>; };
template <> struct Shape<64, 1> { static constexpr int E = 16, XC = 16, SC = 16; using Plan = Radices<16, 4>; };
template <> struct Shape<128, 0> { static constexpr int E = 16, XC = 16, SC = 32; using Plan = Radices<16, 8>; };
template <> struct Shape<128, 1> { static constexpr int E = 16, XC = 8, SC = 16; using Plan = Radices<8, 16>; };
template <> struct Shape<256, 0> { static constexpr int E = 16, XC = 8, SC = 16; using Plan = Radices<16, 16>; };
template <> struct Shape<256, 1> { static constexpr int E = 16, XC = 16, SC = 8; using Plan = Radices<16, 16>; };
template <> struct Shape<512, 0> { static constexpr int E = 16, XC = 4, SC = 16; using Plan = Radices<16, 16, 2>; };
template <> struct Shape<512, 1> { static constexpr int E = 16, XC = 8, SC = 8; using Plan = Radices<16, 16, 2>; };

// One pass launch request.
struct PassReq {
  int mode;     // kModeTma (TMA kernels, register-gather kernels if maps are impossible),
                // kModeTable (table-mode TMA), kModeGather (register-gather kernels)
  int axis;     // 0 x, 1 y, 2 z
  int op;       // OP_FWD, OP_INV, OP_CONV, OP_CONV_FZ
  int nvol;     // cubes (z pass); the x / y passes use nplanes
  int nplanes;  // x / y passes: planes of N*N points to transform (a cube is N planes)
  int variant;  // shape variant 0 / 1
  bool real_src;  // x pass of real rows (a.src holds floats): k_rows_real
  int half;       // Hermitian half-spectrum layout of pitch half_pitch(N) (herm.cuh), else 0
  PassArgs a;
  cudaStream_t s;
};
constexpr int kModeTma = 0, kModeTable = 1, kModeGather = 2;

// Tensor-map encoders (passes.cu). Return false when the operand cannot be described.
bool encode_cube_map(CUtensorMap *m, const void *base, int n, long long nplanes, int axis, int cols);
bool encode_rows_map(CUtensorMap *m, const void *base, int n, long long rows, int xc);
bool encode_rows512_map(CUtensorMap *m, const void *base, long long rows, int xc);
// As encode_cube_map over planes of N rows of `width` complex values (row pitch = width).
bool encode_pitched_map(CUtensorMap *m, const void *base, int width, int n, long long nplanes, int axis, int cols);

template <int N>
cudaError_t launch_size(const PassReq &r);
template <int N>
cudaError_t prepare_size();

#ifdef CONVGPU_PASS_LAUNCH_IMPL

template <class K>
static cudaError_t set_smem_once(K kern, int smem, int &done) {
  // `done` holds the device (+1) the limit was last set on: attributes belong to a
  // device's context, so a process that moves to another device sets them again.
  int dev = 0;
  cudaGetDevice(&dev);
  if (done == dev + 1) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) done = dev + 1;
  return e;
}

// Register-gather kernels (shape variant 0): any 8-byte aligned operands.
template <int N, bool CONTIG, int OP>
static cudaError_t launch_gather(PassArgs a, int nvol, int nplanes, cudaStream_t s) {
  using S = Shape<N, 0>;
  constexpr int E = S::E;
  constexpr int COLS = CONTIG ? S::XC : S::SC;
  constexpr int smem = pass_smem_bytes<N, E, COLS, CONTIG>();
  auto kern = k_axis_pass<N, E, COLS, CONTIG, OP, typename S::Plan>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, smem, done);
  if (e != cudaSuccess) return e;
  a.groups_x = N / S::SC;
  a.groups_per_vol = N * (N / S::SC);
  // x / y passes: nplanes planes (a plane is N rows, or N / SC y-tiles); z pass: cubes
  const long long blocks = CONTIG ? (long long)nplanes * N / COLS
                                  : (OP == OP_FWD || OP == OP_INV) && a.axis_stride == N
                                        ? (long long)nplanes * (N / S::SC)
                                        : (long long)nvol * a.groups_per_vol;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, COLS * (N / E), smem, s>>>(a);
  return cudaGetLastError();
}

// TMA x pass. Returns cudaErrorNotSupported when a tensor map cannot be built.
template <int N, int V, int OP>
static cudaError_t launch_rows(const PassReq &r) {
  using S = Shape<N, V>;
  constexpr int E = S::E, XC = S::XC;
  constexpr int smem = tma_rows_smem_bytes<N, XC>();
  auto kern = k_rows_tma<N, E, XC, OP, typename S::Plan>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, smem, done);
  if (e != cudaSuccess) return e;
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  if (r.mode != kModeTable) {
    if ((reinterpret_cast<uintptr_t>(r.a.dst) & 15u) != 0) return cudaErrorNotSupported;
    if (!encode_rows_map(&m, r.a.src, N, (long long)r.nplanes * N, XC)) return cudaErrorNotSupported;
  }
  const long long blocks = r.mode == kModeTable ? (long long)r.nvol * N * N / XC : (long long)r.nplanes * N / XC;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, XC * (N / E), smem, r.s>>>(m, r.a);
  return cudaGetLastError();
}

// TMA y / z pass. Returns cudaErrorNotSupported when a tensor map cannot be built.
template <int N, int V, int OP>
static cudaError_t launch_strided(const PassReq &r) {
  using S = Shape<N, V>;
  constexpr int E = S::E, COLS = S::SC;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  constexpr int smem = tma_pass_smem_bytes<N, COLS, OP>();
  auto kern = k_strided_tma<N, E, COLS, OP, typename S::Plan>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, smem, done);
  if (e != cudaSuccess) return e;
  PassArgs a = r.a;
  a.groups_x = N / COLS;
  a.groups_per_vol = N * (N / COLS);
  a.axis_stride = r.axis == 1 ? N : (long long)N * N;
  a.plane_pitch = r.axis == 1 ? (long long)N * N : N;
  CUtensorMap msrc, mfilt;
  std::memset(&msrc, 0, sizeof(msrc));
  std::memset(&mfilt, 0, sizeof(mfilt));
  if (r.mode != kModeTable) {
    if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
    const long long planes = r.axis == 1 ? (long long)r.nplanes : (long long)r.nvol * N;
    if (!encode_cube_map(&msrc, a.src, N, planes, r.axis, COLS)) return cudaErrorNotSupported;
    if (HAS_F) {
      const long long fplanes = a.filt_vol_elems ? (long long)r.nvol * N : (long long)N;
      if (!encode_cube_map(&mfilt, a.filt, N, fplanes, r.axis, COLS)) return cudaErrorNotSupported;
    }
  }
  const long long blocks = (r.axis == 1 && r.mode != kModeTable) ? (long long)r.nplanes * (N / COLS)
                                                                  : (long long)r.nvol * a.groups_per_vol;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, COLS * (N / E), smem, r.s>>>(msrc, mfilt, a, r.axis);
  return cudaGetLastError();
}

template <int N, int V>
static cudaError_t launch_tma_variant(const PassReq &r) {
  if (r.axis == 0) {
    if (r.op == OP_FWD) return launch_rows<N, V, OP_FWD>(r);
    if (r.op == OP_INV) return launch_rows<N, V, OP_INV>(r);
    return cudaErrorInvalidValue;
  }
  switch (r.op) {
    case OP_FWD: return launch_strided<N, V, OP_FWD>(r);
    case OP_INV: return launch_strided<N, V, OP_INV>(r);
    case OP_CONV: return launch_strided<N, V, OP_CONV>(r);
    case OP_CONV_FZ: return launch_strided<N, V, OP_CONV_FZ>(r);
    default: return cudaErrorInvalidValue;
  }
}

template <int N>
static cudaError_t launch_gather_op(const PassReq &r) {
  PassArgs a = r.a;
  a.vol_elems = (long long)N * N * N;
  if (r.axis == 0) {
    if (r.op == OP_FWD) return launch_gather<N, true, OP_FWD>(a, r.nvol, r.nplanes, r.s);
    if (r.op == OP_INV) return launch_gather<N, true, OP_INV>(a, r.nvol, r.nplanes, r.s);
    return cudaErrorInvalidValue;
  }
  a.axis_stride = r.axis == 1 ? N : (long long)N * N;
  a.plane_pitch = r.axis == 1 ? (long long)N * N : N;
  switch (r.op) {
    case OP_FWD: return launch_gather<N, false, OP_FWD>(a, r.nvol, r.nplanes, r.s);
    case OP_INV: return launch_gather<N, false, OP_INV>(a, r.nvol, r.nplanes, r.s);
    case OP_CONV: return launch_gather<N, false, OP_CONV>(a, r.nvol, r.nplanes, r.s);
    case OP_CONV_FZ: return launch_gather<N, false, OP_CONV_FZ>(a, r.nvol, r.nplanes, r.s);
    default: return cudaErrorInvalidValue;
  }
}

// x pass of real rows (shape variant V's radix plan and rows per CTA).
template <int N, int V>
static cudaError_t launch_rows_real(const PassReq &r) {
  using S = Shape<N, V>;
  constexpr int E = S::E, XC = S::XC;
  constexpr int smem = pass_smem_bytes<N, E, XC, true>();
  auto kern = k_rows_real<N, E, XC, typename S::Plan>;
  static int done = 0;
  cudaError_t e = set_smem_once(kern, smem, done);
  if (e != cudaSuccess) return e;
  const long long blocks = (long long)r.nplanes * N / XC;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, XC * (N / E), smem, r.s>>>(r.a);
  return cudaGetLastError();
}

// Passes over Hermitian half spectra (herm.cuh), N >= 64, shape variant 1's radix plan and
// columns: the real filter's x pass storing the first W = half_pitch(N) values of every row
// (axis 0), its y / z passes over that width (OP_FWD), and the paired fused z pass of the
// signals against it (axis 2, OP_CONV).
template <int N>
static cudaError_t launch_half(const PassReq &r) {
  if constexpr (half_pitch(N) == 0) {
    return cudaErrorNotSupported;
  } else {
    using S = Shape<N, 1>;
    constexpr int E = S::E, COLS = S::SC, W = half_pitch(N);
    static_assert(W % COLS == 0 && (N / 2) % COLS == 0 && (COLS + 2) * 8 % 16 == 0, "half-layout tiles");
    PassArgs a = r.a;
    if ((reinterpret_cast<uintptr_t>(a.dst) & 15u) != 0) return cudaErrorNotSupported;
    if (r.axis == 0) {
      if (!r.real_src || r.op != OP_FWD) return cudaErrorInvalidValue;
      PassReq q = r;
      q.a.out_cols = W;
      return r.variant ? launch_rows_real<N, 1>(q) : launch_rows_real<N, 0>(q);
    }
    if (r.op == OP_FWD) {
      auto kern = k_strided_tma<N, E, COLS, OP_FWD, typename S::Plan>;
      constexpr int smem = tma_pass_smem_bytes<N, COLS, OP_FWD>();
      static int done = 0;
      cudaError_t e = set_smem_once(kern, smem, done);
      if (e != cudaSuccess) return e;
      CUtensorMap m;
      if (!encode_pitched_map(&m, a.src, W, N, (long long)r.nvol * N, r.axis, COLS)) return cudaErrorNotSupported;
      a.vol_elems = (long long)N * N * W;
      a.groups_x = W / COLS;
      a.groups_per_vol = N * a.groups_x;
      a.axis_stride = r.axis == 1 ? W : (long long)N * W;
      a.plane_pitch = r.axis == 1 ? (long long)N * W : W;
      const long long blocks = (long long)r.nvol * a.groups_per_vol;
      if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
      kern<<<(unsigned)blocks, COLS * (N / E), smem, r.s>>>(m, m, a, r.axis);
      return cudaGetLastError();
    }
    if (r.op == OP_CONV && r.axis == 2) {
      auto kern = k_zconv_half<N, E, COLS, typename S::Plan>;
      constexpr int smem = zconv_half_smem_bytes<N, COLS>();
      static int done = 0;
      cudaError_t e = set_smem_once(kern, smem, done);
      if (e != cudaSuccess) return e;
      CUtensorMap ms, mh;
      const long long fplanes = a.filt_vol_elems ? (long long)r.nvol * N : (long long)N;
      if (!encode_cube_map(&ms, a.src, N, (long long)r.nvol * N, 2, COLS) ||
          !encode_pitched_map(&mh, a.filt, W, N, fplanes, 2, COLS + 2))
        return cudaErrorNotSupported;
      a.vol_elems = (long long)N * N * N;
      const long long blocks = (long long)r.nvol * N * (N / 2 / COLS);
      if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
      kern<<<(unsigned)blocks, 2 * COLS * (N / E), smem, r.s>>>(ms, mh, a);
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }
}

template <int N>
cudaError_t launch_size(const PassReq &r) {
  if (r.half) return launch_half<N>(r);
  if (r.real_src) return r.variant ? launch_rows_real<N, 1>(r) : launch_rows_real<N, 0>(r);
  if (r.mode == kModeGather) return launch_gather_op<N>(r);
  if (r.mode == kModeTable) return launch_tma_variant<N, 0>(r);  // tables are encoded with variant 0
  const cudaError_t e = r.variant ? launch_tma_variant<N, 1>(r) : launch_tma_variant<N, 0>(r);
  if (e != cudaErrorNotSupported) return e;
  return launch_gather_op<N>(r);
}

template <int N, int V>
static cudaError_t prepare_variant() {
  using S = Shape<N, V>;
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

// Sets the shared-memory attributes of every TMA kernel of size N (both variants), so
// launches can later be captured into graphs.
template <int N>
cudaError_t prepare_size() {
  cudaError_t e = prepare_variant<N, 0>();
  if (e == cudaSuccess) e = prepare_variant<N, 1>();
  return e;
}

#endif  // CONVGPU_PASS_LAUNCH_IMPL

}  // namespace convgpu

namespace convgpu {
// Tensor-core pass for N = 256 (passes_n256.cu); bf16x3 selects BF16x3 over TF32x3.
cudaError_t launch_tc256_entry(const PassReq &r, int bf16x3);
cudaError_t launch_tc05_entry(const PassReq &r);
// tcgen05 split-TF32 pass for N = 512 (tc05_n512.cu).
cudaError_t launch_tc05_512_entry(const PassReq &r);
// L2-staged fused x + y pass for N = 128, 256 or 512 (xyl2.cu, xyl2.cuh).
cudaError_t launch_xy_l2(int n, const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                         const float2 *tw512, unsigned *status, cudaStream_t s);
// Its tensor-core (split-TF32, tcgen05) form for N = 256 (xyl2.cu, xyl2_tc.cuh).
cudaError_t launch_xy_l2_tc(const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                            const float2 *tw512, unsigned *status, cudaStream_t s);
// Fused x + y pass for N = 256 on 8-CTA clusters (passes_n256.cu, xy256.cuh).
cudaError_t launch_xy256(const float2 *src, float2 *dst, int nplanes, bool inverse, float scale, const float2 *tw512,
                         unsigned int *status, cudaStream_t s);
}  // namespace convgpu
