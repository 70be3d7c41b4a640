// Per-axis FFT pass kernels for complex64 cubes (x fastest: idx = z*N*N + y*N + x).
//
// One launch transforms every pencil of one axis of a batch of cubes in place (or from
// src to dst). The reference builds each 3D transform from three streaming 1D engines
// joined by an on-chip plane transpose and a DDR round-trip transpose
// (kernels/conv3D.cl:71-420: fft3da, transpose, fft3db, transpose3D, fft3dc, store).
// Here each axis is one pass over HBM:
//   - x pass: pencils are contiguous rows; a CTA owns COLS consecutive rows.
//   - y / z passes: pencils are strided (N or N*N elements); a CTA owns COLS adjacent
//     x-columns of one plane, so every global access is a run of COLS*8 contiguous bytes.
// The transposes disappear: strided pencils are gathered straight into registers.
//
// Fused ops (Op):
//   FWD      forward transform.
//   INV      unnormalised backward transform, results multiplied by `scale`.
//   CONV     forward z transform, pointwise product with a filter spectrum read at the
//            same positions (conv3D / comp_mult: kernels/conv3D.cl:517-570,
//            kernels/fft/fft_8.cl:180-185), backward z transform. The spectrum never
//            leaves registers.
//   CONV_FZ  as CONV, but the filter operand is only x/y transformed: its z transform
//            is computed in the same kernel (per-signal filters: saves one filter pass).
#pragma once

#include <cstdint>

#include "fft_core.cuh"
#include "tma.cuh"

namespace convgpu {

enum PassOp : int { OP_FWD = 0, OP_INV = 1, OP_CONV = 2, OP_CONV_FZ = 3 };

struct PassArgs {
  const float2 *src;
  float2 *dst;
  const float2 *filt;      // CONV / CONV_FZ only
  const float2 *tw512;     // tw512[j] = exp(-2*pi*i*j/512), j < 512 (FP64-generated)
  long long vol_elems;     // N^3
  long long filt_vol_elems;  // 0: one filter for all volumes; N^3: one per volume
  long long axis_stride;   // elements between consecutive pencil positions (strided passes)
  long long plane_pitch;   // strided: element offset per group row (N*N for y, N for z)
  int groups_per_vol;      // CTAs per volume
  int groups_x;            // strided: N / COLS
  float scale;             // INV / CONV: output scale
  // Table mode of the TMA kernels (null otherwise): per-volume tensor maps of the source
  // and filter operands (each map covers one cube) and per-volume destination bases, so
  // one launch serves cubes at unrelated addresses.
  const CUtensorMap *maps;
  const CUtensorMap *fmaps;
  float2 *const *dsts;
  // Device status word: kernels OR in kStatus* bits when a bounded wait gives up.
  unsigned int *status;
  // x pass of real rows only: values stored per row, at that row pitch (0: all N). The
  // Hermitian half spectrum of a real filter keeps the first half_pitch(N) (herm.cuh).
  int out_cols;
};

// Shared-memory slot of pencil position n for the two layouts.
template <int COLS>
struct ColSlot {  // strided passes: position-major, columns contiguous (conflict-free)
  int c;
  __device__ __forceinline__ int operator()(int n) const { return n * COLS + c; }
};
template <int N>
struct RowSlot {  // x pass: pencil-major, one 8-byte pad every 16 slots
  int base;
  __device__ __forceinline__ int operator()(int n) const { return base + n + (n >> 4); }
};
template <int N>
constexpr int row_pitch() { return N + N / 16; }
// x pass of N = 256 in an unpadded row: the low 4 bits of the position XOR-swizzled by
// bits 4..7, which makes the Stockham exchange of a 16 x 16 row transform free of bank
// conflicts in the row's own N slots (the tile a TMA row load lands in).
struct SwzRow {
  int base;
  __device__ __forceinline__ int operator()(int n) const { return base + (n ^ ((n >> 4) & 15)); }
};

// Barrier between the exchange's writes and reads: the whole CTA, or only the warp when
// every pencil's threads and shared-memory slots belong to one warp (WARP).
template <bool WARP>
__device__ __forceinline__ void exchange_sync() {
  if constexpr (WARP)
    __syncwarp();
  else
    __syncthreads();
}

template <int N, int E, int NS, bool WARP, class SIdx, class TW, int R, int... Rest>
__device__ __forceinline__ void run_stages(float2 (&v)[E], int t, const TW &tw, float2 *sm, const SIdx &sidx) {
  constexpr int T = N / E;
  constexpr bool last = sizeof...(Rest) == 0;
  stockham_stage<N, E, R, NS, last>(v, t, tw, sm, sidx);
  if constexpr (!last) {
    exchange_sync<WARP>();
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sm[sidx(t + e * T)];
    exchange_sync<WARP>();
    run_stages<N, E, NS * R, WARP, SIdx, TW, Rest...>(v, t, tw, sm, sidx);
  }
}

// WARP: the caller guarantees that each pencil's T threads lie in one warp and that no
// other warp touches its slots, so the exchange needs only warp barriers.
template <int N, int E, bool WARP = false, class SIdx, class TW, int... Rs>
__device__ __forceinline__ void fft_forward(float2 (&v)[E], int t, const TW &tw, float2 *sm, const SIdx &sidx,
                                            Radices<Rs...>) {
  (void)PlanCheck<N, E, Radices<Rs...>>::stages;
  run_stages<N, E, 1, WARP, SIdx, TW, Rs...>(v, t, tw, sm, sidx);
}

template <int E>
__device__ __forceinline__ void swap_all(float2 (&v)[E]) {
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = cswap(v[e]);
}

// Dynamic shared memory: N twiddles, then the exchange buffer.
template <int N, int E, int COLS, bool CONTIG>
constexpr int pass_smem_bytes() {
  return (N + (CONTIG ? COLS * row_pitch<N>() : COLS * N)) * 8;
}

template <int N, int E, int COLS, bool CONTIG, int OP, class Plan>
__global__ void __launch_bounds__(COLS *(N / E)) k_axis_pass(PassArgs a) {
  constexpr int T = N / E;
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *sm = smem + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * (512 / N)];

  int t, c;
  long long base, fbase, es;
  if constexpr (CONTIG) {
    t = threadIdx.x % T;
    c = threadIdx.x / T;
    const long long row = (long long)blockIdx.x * COLS + c;
    base = row * N;
    const long long vol = row / ((long long)N * N);
    fbase = vol * a.filt_vol_elems + (row % ((long long)N * N)) * N;
    es = 1;
  } else {
    c = threadIdx.x % COLS;
    t = threadIdx.x / COLS;
    const long long vol = blockIdx.x / a.groups_per_vol;
    const int r = blockIdx.x % a.groups_per_vol;
    const long long outer = (long long)(r / a.groups_x) * a.plane_pitch + (long long)(r % a.groups_x) * COLS + c;
    base = vol * a.vol_elems + outer;
    fbase = vol * a.filt_vol_elems + outer;
    es = a.axis_stride;
  }
  auto sidx = [&]() {
    if constexpr (CONTIG) return RowSlot<N>{c * row_pitch<N>()};
    else return ColSlot<COLS>{c};
  }();

  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = a.src[base + (long long)(t + e * T) * es];
  __syncthreads();  // twiddle table ready

  if constexpr (OP == OP_FWD) {
    fft_forward<N, E>(v, t, tw, sm, sidx, Plan{});
  } else if constexpr (OP == OP_INV) {
    swap_all(v);
    fft_forward<N, E>(v, t, tw, sm, sidx, Plan{});
    swap_all(v);
    if (a.scale != 1.0f) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * a.scale, v[e].y * a.scale);
    }
  } else {
    float2 f[E];
#pragma unroll
    for (int e = 0; e < E; ++e) f[e] = a.filt[fbase + (long long)(t + e * T) * es];
    if constexpr (OP == OP_CONV_FZ) {
      fft_forward<N, E>(f, t, tw, sm, sidx, Plan{});
      __syncthreads();
    }
    fft_forward<N, E>(v, t, tw, sm, sidx, Plan{});
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = cmul(v[e], f[e]);
    __syncthreads();
    swap_all(v);
    fft_forward<N, E>(v, t, tw, sm, sidx, Plan{});
    swap_all(v);
    if (a.scale != 1.0f) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * a.scale, v[e].y * a.scale);
    }
  }

#pragma unroll
  for (int e = 0; e < E; ++e) a.dst[base + (long long)(t + e * T) * es] = v[e];
}

// x pass of real rows (real filters): a.src holds N floats per row; each value enters the
// transform as (x, 0). Same radix plan and exchange layout as k_rows_tma, so the result
// equals the complex x pass of the same data with zero imaginary parts, bit for bit. With
// a.out_cols it stores only the first out_cols values of each row, at that pitch.
template <int N, int E, int XC, class Plan>
__global__ void __launch_bounds__(XC *(N / E)) k_rows_real(PassArgs a) {
  constexpr int T = N / E;
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *sm = smem + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * (512 / N)];
  const int t = threadIdx.x % T, c = threadIdx.x / T;
  const long long row = (long long)blockIdx.x * XC + c;
  const float *src = reinterpret_cast<const float *>(a.src) + row * N;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = make_float2(src[t + e * T], 0.f);
  __syncthreads();  // twiddle table ready
  fft_forward<N, E>(v, t, tw, sm, RowSlot<N>{c * row_pitch<N>()}, Plan{});
  const int w = a.out_cols ? a.out_cols : N;
  float2 *dst = a.dst + row * w + t;
#pragma unroll
  for (int e = 0; e < E; ++e)
    if (t + e * T < w) dst[e * T] = v[e];
}

// Dynamic shared memory of the TMA-fed x pass: barrier slot, the unpadded row tile (TMA
// target), the padded exchange buffer, then N twiddles.
template <int N, int XC>
constexpr int tma_rows_smem_bytes() {
  return 128 + XC * N * 8 + XC * row_pitch<N>() * 8 + N * 8;
}

// Slot of element n of tile row c as TMA lands it: boxes are at most 256 wide, so a
// 512-point row arrives as two half-tiles [half][row][256].
template <int N, int XC>
__device__ __forceinline__ int rowtile_idx(int c, int n) {
  if constexpr (N <= 256) return c * N + n;
  else return ((n >> 8) * XC + c) * 256 + (n & 255);
}

// Dynamic shared memory of the TMA-fed strided pass: barrier (128 B slot), the signal
// tile, the filter tile (fused z ops), then N twiddles.
template <int N, int COLS, int OP>
constexpr int tma_pass_smem_bytes() {
  return 128 + N * COLS * 8 * ((OP == OP_CONV || OP == OP_CONV_FZ) ? 2 : 1) + N * 8;
}

// y / z pass fed by TMA. One CTA owns COLS adjacent x-columns of one plane (y pass,
// axis 1) or one row (z pass, axis 2): thread 0 loads the whole N x COLS tile (and the
// matching filter tile for the fused z ops) with cp.async.bulk.tensor into shared memory,
// position-major with columns contiguous -- exactly the ColSlot layout the Stockham
// stages exchange through, so the tile buffer doubles as the exchange buffer. The
// filter operand never occupies registers; CONV_FZ transforms it in place in its tile.
// Boxes are at most 256 long, so N = 512 takes two loads per tile.
template <int N, int E, int COLS, int OP, class Plan>
__global__ void __launch_bounds__(COLS *(N / E)) k_strided_tma(const __grid_constant__ CUtensorMap msrc,
                                                              const __grid_constant__ CUtensorMap mfilt,
                                                              PassArgs a, int axis) {
  constexpr int T = N / E;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  constexpr int TILE = N * COLS;
  constexpr int NBOX = N > 256 ? 256 : N;
  constexpr int NLOADS = N / NBOX;
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tile = reinterpret_cast<float2 *>(smraw + 128);
  float2 *ftile = tile + TILE;
  float2 *tw = HAS_F ? ftile + TILE : tile + TILE;
  // bar: the signal tile; fbar: the filter tile. CONV_FZ issues the filter first and
  // transforms it while the signal lands; CONV needs the filter only for the product, so
  // it lands during the signal's transform.
  const uint32_t bar = smem_u32(smraw), fbar = bar + 8;

  const int vol = blockIdx.x / a.groups_per_vol;
  const int r = blockIdx.x % a.groups_per_vol;
  const int row = r / a.groups_x;  // z of the plane (y pass) or y of the row (z pass)
  const int x0 = (r % a.groups_x) * COLS;

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    if constexpr (HAS_F) mbar_init(fbar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    auto load_signal = [&]() {
      const CUtensorMap *ms = a.maps ? a.maps + vol : &msrc;
      const int zoff = a.maps ? 0 : vol * N;
      if (a.maps) tensormap_acquire(ms);
      mbar_arrive_expect_tx(bar, TILE * 8u);
#pragma unroll
      for (int l = 0; l < NLOADS; ++l) {
        if (axis == 1)
          tma_load_3d(smem_u32(tile + l * NBOX * COLS), ms, x0, l * NBOX, zoff + row, bar);
        else
          tma_load_3d(smem_u32(tile + l * NBOX * COLS), ms, x0, row, zoff + l * NBOX, bar);
      }
    };
    auto load_filter = [&]() {
      const CUtensorMap *mf = a.fmaps ? a.fmaps + vol : &mfilt;
      const int fzoff = a.fmaps ? 0 : (a.filt_vol_elems ? vol : 0) * N;
      if (a.fmaps) tensormap_acquire(mf);
      mbar_arrive_expect_tx(fbar, TILE * 8u);
#pragma unroll
      for (int l = 0; l < NLOADS; ++l)
        tma_load_3d(smem_u32(ftile + l * NBOX * COLS), mf, x0, row, fzoff + l * NBOX, fbar);
    };
    if constexpr (OP == OP_CONV_FZ) load_filter();
    load_signal();
    if constexpr (OP == OP_CONV) load_filter();
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * (512 / N)];
  const int c = threadIdx.x % COLS;
  const int t = threadIdx.x / COLS;
  const ColSlot<COLS> sidx{c};
  // Each wait is a uniform decision (every thread takes the same branch, so no barrier is
  // left waiting); one that gives up lets the copies still in flight land before the CTA
  // exits.
  auto landed = [&](uint32_t b) {
    if (__syncthreads_and(mbar_wait_bounded(b, 0) ? 1 : 0)) return true;
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(bar, 0);
    if constexpr (HAS_F) mbar_wait_bounded(fbar, 0);
    return false;
  };
  if (!landed(OP == OP_CONV_FZ ? fbar : bar)) return;

  float2 v[E];
  if constexpr (OP == OP_CONV_FZ) {
    float2 f[E];
#pragma unroll
    for (int e = 0; e < E; ++e) f[e] = ftile[sidx(t + e * T)];
    __syncthreads();
    fft_forward<N, E>(f, t, tw, ftile, sidx, Plan{});
#pragma unroll
    for (int e = 0; e < E; ++e) ftile[sidx(t + e * T)] = f[e];  // own slots: read back by this thread only
    if (!landed(bar)) return;
  }
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = tile[sidx(t + e * T)];
  __syncthreads();

  if constexpr (OP == OP_FWD) {
    fft_forward<N, E>(v, t, tw, tile, sidx, Plan{});
  } else if constexpr (OP == OP_INV) {
    swap_all(v);
    fft_forward<N, E>(v, t, tw, tile, sidx, Plan{});
    swap_all(v);
  } else {
    fft_forward<N, E>(v, t, tw, tile, sidx, Plan{});
    if constexpr (OP == OP_CONV) {
      if (!landed(fbar)) return;
    }
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = cmul(v[e], ftile[sidx(t + e * T)]);
    swap_all(v);
    fft_forward<N, E>(v, t, tw, tile, sidx, Plan{});
    swap_all(v);
  }
  if (a.scale != 1.0f) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * a.scale, v[e].y * a.scale);
  }
  float2 *dst = (a.dsts ? a.dsts[vol] : a.dst + (long long)vol * a.vol_elems) + (long long)row * a.plane_pitch + x0 + c;
#pragma unroll
  for (int e = 0; e < E; ++e) dst[(long long)(t + e * T) * a.axis_stride] = v[e];
}

// x pass fed by TMA: thread 0 loads XC consecutive rows (XC*N*8 contiguous bytes) with
// one 2D bulk-tensor copy per 256-wide box; threads read their t + e*T elements
// (consecutive lanes, consecutive slots), run the Stockham stages through the padded
// exchange buffer and store straight to global memory.
template <int N, int E, int XC, int OP, class Plan>
__global__ void __launch_bounds__(XC *(N / E)) k_rows_tma(const __grid_constant__ CUtensorMap msrc, PassArgs a) {
  static_assert(OP == OP_FWD || OP == OP_INV, "x pass ops");
  constexpr int T = N / E;
  constexpr int NBOX = N > 256 ? 256 : N;
  constexpr int NLOADS = N / NBOX;
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tile = reinterpret_cast<float2 *>(smraw + 128);
  float2 *exch = tile + XC * N;
  float2 *tw = exch + XC * row_pitch<N>();
  const uint32_t bar = smem_u32(smraw);
  // Table mode: blockIdx -> (volume, row tile) and the volume's own map / destination.
  constexpr int TPV = N * N / XC;
  const int vol = a.maps ? (int)(blockIdx.x / TPV) : 0;
  const long long row0 = a.maps ? (long long)(blockIdx.x % TPV) * XC : (long long)blockIdx.x * XC;

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const CUtensorMap *ms = a.maps ? a.maps + vol : &msrc;
    if (a.maps) tensormap_acquire(ms);
    mbar_arrive_expect_tx(bar, (uint32_t)(XC * N * 8));
#pragma unroll
    for (int l = 0; l < NLOADS; ++l)
      tma_load_2d(smem_u32(tile + l * XC * NBOX), ms, l * NBOX, (int)row0, bar);
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * (512 / N)];
  const int t = threadIdx.x % T;
  const int c = threadIdx.x / T;
  const RowSlot<N> sidx{c * row_pitch<N>()};
  const int ok = __syncthreads_and(mbar_wait_bounded(bar, 0) ? 1 : 0);
  if (!ok) {
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(bar, 0);
    return;
  }
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = tile[rowtile_idx<N, XC>(c, t + e * T)];
  if constexpr (OP == OP_INV) swap_all(v);
  fft_forward<N, E>(v, t, tw, exch, sidx, Plan{});
  if constexpr (OP == OP_INV) swap_all(v);
  if (a.scale != 1.0f) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * a.scale, v[e].y * a.scale);
  }
  float2 *dst = (a.dsts ? a.dsts[vol] : a.dst) + (row0 + c) * N + t;
#pragma unroll
  for (int e = 0; e < E; ++e) dst[e * T] = v[e];
}

}  // namespace convgpu
