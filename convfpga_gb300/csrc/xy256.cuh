// Fused x + y pass for N = 256: one 256 x 256 plane per cluster of 8 CTAs.
//
// A plane (512 KiB) does not fit one CTA's shared memory, so an 8-CTA thread-block
// cluster shares it: CTA r holds rows 32r..32r+31, transforms them along x, then the
// cluster exchanges a 32 x 32 block between every pair of CTAs through distributed
// shared memory (an all-to-all transpose, 56 KiB pulled per CTA), after which CTA r holds
// all 256 rows of columns 32r..32r+31 and transforms them along y locally. Each plane
// crosses HBM once (read + write) instead of twice, which removes one full pass of
// every 2D (x, y) transform: the reference streams these two axes through an on-chip
// plane transpose (kernels/conv3D.cl:118-232, transpose + fft3db).
//
// The kernel is persistent: cluster c takes planes c, c + nclusters, ...; the next
// plane's rows are prefetched by TMA into a second buffer while the current one is
// transformed. Every CTA of a cluster runs the same number of iterations and reaches
// every cluster barrier; a TMA wait that gives up records kStatusTmaTimeout and the CTA
// carries on (its output is then wrong and the status word says so), so barriers never
// miss a participant.
#pragma once

#include <cooperative_groups.h>

#include "passes.cuh"

namespace convgpu {

constexpr int kXyCluster = 8;
constexpr int kXyRows = 256 / kXyCluster;                 // 32 rows per CTA
constexpr int kXyThreads = 256;
constexpr int kXyTile = kXyRows * 256;                    // complex values per row tile
// Dynamic shared memory: 2 barriers (128 B), two row tiles, the column tile, twiddles.
constexpr int kXySmem = 128 + 3 * kXyTile * 8 + 256 * 8;

template <bool INV>
__global__ void __cluster_dims__(kXyCluster, 1, 1) __launch_bounds__(kXyThreads, 1)
    k_xy256(const __grid_constant__ CUtensorMap mrows, float2 *__restrict__ dst, int nplanes, float scale,
            const float2 *__restrict__ tw512, unsigned int *status) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  constexpr int N = 256, E = 16, T = 16;
  using Plan = Radices<16, 16>;
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *xbuf0 = reinterpret_cast<float2 *>(smraw + 128);
  float2 *xbuf1 = xbuf0 + kXyTile;
  float2 *ybuf = xbuf1 + kXyTile;
  float2 *tw = ybuf + kXyTile;
  const uint32_t bar0 = smem_u32(smraw), bar1 = smem_u32(smraw + 8);
  const int rank = (int)cluster.block_rank();
  const int cid = blockIdx.x / kXyCluster;
  const int ncl = gridDim.x / kXyCluster;
  const int tid = threadIdx.x;

  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    mbar_fence_init();
  }
  for (int i = tid; i < N; i += kXyThreads) tw[i] = tw512[2 * i];
  __syncthreads();
  if (tid == 0 && cid < nplanes) {
    mbar_arrive_expect_tx(bar0, kXyTile * 8);
    tma_load_2d(smem_u32(xbuf0), &mrows, 0, cid * N + rank * kXyRows, bar0);
  }
  uint32_t parity0 = 0, parity1 = 0;
  int it = 0;
  for (int p = cid; p < nplanes; p += ncl, ++it) {
    const bool odd = it & 1;
    float2 *xb = odd ? xbuf1 : xbuf0;
    const int pn = p + ncl;
    if (tid == 0 && pn < nplanes) {  // prefetch the next plane into the other buffer
      const uint32_t bn = odd ? bar0 : bar1;
      mbar_arrive_expect_tx(bn, kXyTile * 8);
      tma_load_2d(smem_u32(odd ? xbuf0 : xbuf1), &mrows, 0, pn * N + rank * kXyRows, bn);
    }
    const int ok = __syncthreads_and(mbar_wait_bounded(odd ? bar1 : bar0, odd ? parity1 : parity0) ? 1 : 0);
    if (odd) parity1 ^= 1u;
    else parity0 ^= 1u;
    if (!ok && tid == 0 && status) atomicOr(status, kStatusTmaTimeout);

    // x transforms of the 32 rows, 16 rows per round, in place (swizzled exchange).
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
      const int row = 16 * q + tid / T, t = tid % T;
      float2 v[E];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const float2 a = xb[row * N + t + e * T];
        v[e] = INV ? cswap(a) : a;
      }
      __syncthreads();
      fft_forward<N, E>(v, t, tw, xb, SwzRow{row * N}, Plan{});
#pragma unroll
      for (int e = 0; e < E; ++e) xb[row * N + t + e * T] = v[e];  // natural order for the exchange
      __syncthreads();
    }
    cluster.sync();  // every CTA's row transforms are complete and visible

    // All-to-all: pull rows 32s..32s+31, columns 32r..32r+31 from every CTA s.
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const int i = tid + kXyThreads * k;
      const int x2 = i & 15, yl = (i >> 4) & 31, s = i >> 9;
      const float4 *src =
          reinterpret_cast<const float4 *>(cluster.map_shared_rank(xb, s) + yl * N + rank * kXyRows + 2 * x2);
      *reinterpret_cast<float4 *>(ybuf + (s * kXyRows + yl) * kXyRows + 2 * x2) = *src;
    }
    __syncthreads();
    cluster.sync();  // no CTA reads this plane's row tiles any more

    // y transforms of the 32 columns (256 rows each), 16 columns per round.
    float2 *plane = dst + (long long)p * N * N + rank * kXyRows;
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
      const int c = 16 * q + (tid & 15), t = tid >> 4;
      const ColSlot<kXyRows> sidx{c};
      float2 v[E];
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = ybuf[sidx(t + e * T)];
      __syncthreads();
      fft_forward<N, E>(v, t, tw, ybuf, sidx, Plan{});
#pragma unroll
      for (int e = 0; e < E; ++e) {
        float2 o = INV ? cswap(v[e]) : v[e];
        plane[(long long)(t + e * T) * N + c] = make_float2(o.x * scale, o.y * scale);
      }
      __syncthreads();
    }
  }
}

}  // namespace convgpu
