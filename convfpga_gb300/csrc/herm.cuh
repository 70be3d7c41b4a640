// Hermitian half spectra of real filters (CONVGPU_FILTER_REAL).
//
// The spectrum of a real cube satisfies F(kx, ky, kz) = conj(F(N-kx, N-ky, N-kz)) (indices
// mod N), so kx in [0, N/2] determines all of it. The filter's transform keeps the columns
// kx < Wp = N/2 + 16 only (a pitched "half" layout, idx = (z*N + y)*Wp + x; the 15 columns
// past N/2 are computed anyway and only round the width up to a multiple of every strided
// tile), and runs its y and z passes on that width: about half the bytes of the full
// transform, and half the workspace. The reference transforms full complex spectra of its
// real Gaussian filters (src/fft_conv3D.cpp:95-99, 222-231).
//
// k_zconv_half is the fused z pass against such a spectrum. One CTA serves two signal
// tiles of C columns along z:
//   A: columns x0 .. x0+C-1 of row y (x0 < N/2), filter H(x0 + c, y, kz);
//   B: columns N-x0-C .. N-x0-1 of row y' = (N - y) mod N, whose filter values are the
//      mirrors conj(H(x0 + C - c, y, (N - kz) mod N)) of the same half-spectrum columns.
// Tiles A over x0 = 0, C, ..., N/2 - C and every row cover the columns [0, N/2); tiles B
// cover [N/2, N): every pencil once. The filter tile is C + 2 columns wide (x0 .. x0+C+1,
// an even width so the box's inner bytes are a multiple of 16), so the half spectrum is
// read once for two signal tiles: a signal convolution reads (C+2)/(2C) of a full
// spectrum's bytes. Threads 0 .. C*T-1 transform tile A, the rest tile B, each tile being
// its own exchange buffer as in k_strided_tma.
#pragma once

#include "passes.cuh"

namespace convgpu {

// Half-spectrum row pitch (complex values) for size n, 0 where the half layout is not
// used (n < 64: a 64-wide pitch would not save bytes).
__host__ __device__ constexpr int half_pitch(int n) { return n >= 64 ? n / 2 + 16 : 0; }

template <int N, int COLS>
constexpr int zconv_half_smem_bytes() {
  return 128 + (2 * N * COLS + N * (COLS + 2)) * 8 + N * 8;
}

// CTAs per SM that shared memory allows (26 KB at N = 64, about 52 KB at 128 and 256,
// 111 KB at 512): registers are held to that occupancy too.
template <int N>
constexpr int zconv_half_min_blocks() {
  return N <= 64 ? 8 : (N <= 256 ? 4 : 2);
}

template <int N, int E, int COLS, class Plan>
__global__ void __launch_bounds__(2 * COLS *(N / E), zconv_half_min_blocks<N>())
    k_zconv_half(const __grid_constant__ CUtensorMap msig, const __grid_constant__ CUtensorMap mhalf, PassArgs a) {
  constexpr int T = N / E, TILE = N * COLS, FC = COLS + 2;
  constexpr int NBOX = N > 256 ? 256 : N, NLOADS = N / NBOX;
  constexpr int GROUPS = N / 2 / COLS;  // A tiles per row
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tiles = reinterpret_cast<float2 *>(smraw + 128);  // A, then B
  float2 *ftile = tiles + 2 * TILE;                          // [kz][C + 2]
  float2 *tw = ftile + N * FC;
  const uint32_t bar = smem_u32(smraw), fbar = bar + 8;  // the two signal tiles; the filter tile

  const int vol = blockIdx.x / (N * GROUPS);
  const int r = blockIdx.x % (N * GROUPS);
  const int y = r / GROUPS, x0 = (r % GROUPS) * COLS;
  const int yb = (N - y) & (N - 1), xb = N - x0 - COLS;

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_init(fbar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // the signal tiles first: the filter tile is needed only for the product, after their
    // transforms
    mbar_arrive_expect_tx(bar, (uint32_t)(2 * TILE * 8));
#pragma unroll
    for (int l = 0; l < NLOADS; ++l) {
      tma_load_3d(smem_u32(tiles + l * NBOX * COLS), &msig, x0, y, vol * N + l * NBOX, bar);
      tma_load_3d(smem_u32(tiles + TILE + l * NBOX * COLS), &msig, xb, yb, vol * N + l * NBOX, bar);
    }
    mbar_arrive_expect_tx(fbar, (uint32_t)(N * FC * 8));
    const int fz = (a.filt_vol_elems ? vol : 0) * N;
#pragma unroll
    for (int l = 0; l < NLOADS; ++l)
      tma_load_3d(smem_u32(ftile + l * NBOX * FC), &mhalf, x0, y, fz + l * NBOX, fbar);
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * (512 / N)];
  const int g = threadIdx.x / (COLS * T);  // 0: tile A, 1: tile B
  const int local = threadIdx.x % (COLS * T);
  const int c = local % COLS, t = local / COLS;
  float2 *tile = tiles + g * TILE;
  const ColSlot<COLS> sidx{c};
  // Each wait is a uniform decision; one that gives up lets the copies still in flight
  // land before the CTA exits.
  auto landed = [&](uint32_t b) {
    if (__syncthreads_and(mbar_wait_bounded(b, 0) ? 1 : 0)) return true;
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(bar, 0);
    mbar_wait_bounded(fbar, 0);
    return false;
  };
  if (!landed(bar)) return;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = tile[sidx(t + e * T)];
  __syncthreads();
  fft_forward<N, E>(v, t, tw, tile, sidx, Plan{});
  if (!landed(fbar)) return;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int kz = t + e * T;
    float2 f;
    if (g == 0) {
      f = ftile[kz * FC + c];
    } else {
      const float2 h = ftile[((N - kz) & (N - 1)) * FC + (COLS - c)];
      f = make_float2(h.x, -h.y);
    }
    v[e] = cmul(v[e], f);
  }
  swap_all(v);
  fft_forward<N, E>(v, t, tw, tile, sidx, Plan{});
  swap_all(v);
  if (a.scale != 1.0f) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * a.scale, v[e].y * a.scale);
  }
  float2 *dst = a.dst + (long long)vol * a.vol_elems + (long long)(g ? yb : y) * N + (g ? xb : x0) + c;
#pragma unroll
  for (int e = 0; e < E; ++e) dst[(long long)(t + e * T) * N * N] = v[e];
}

}  // namespace convgpu
