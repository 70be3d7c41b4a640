// Tensor-core split-precision path: the radix-16 stages of a 256-point transform
// (256 = 16 x 16, four-step) run as batches of 16-point DFTs written as real-form
// complex matmuls on the tensor cores, with split operands and FP32 accumulation:
//
//   [yr yi] = [xr xi] . [[ C  -S ]      C[n][k] = cos(2 pi n k / 16),
//                        [ S   C ]]     S[n][k] = sin(2 pi n k / 16)
//   x = xh + xl, M = Mh + Ml;  y ~= xh.Mh + xh.Ml + xl.Mh   (FP32 accumulate)
//
// Two split precisions (policies below): TF32x3 (default; ~1e-7 relative error per
// 256-point transform) and BF16x3 (~4e-6 per transform, above the 1e-5 end-to-end bound
// for a 256^3 convolution). One MMA group handles 16 DFT instances (one per A row)
// against four 8-column n-blocks (real / imaginary outputs 0-7 and 8-15). Twiddles
// between the two stages are applied in FP32 from the FP64-generated table. This is the
// reference's radix-4 butterfly engine (kernels/fft/fft_8.cl:275-351) replaced by dense
// DFT blocks on the matrix units.
#pragma once

#include <cuda_bf16.h>

#include "passes.cuh"

namespace convgpu {

// Fragment index kk (0..3) -> matrix index 2t, 2t+1, 2t+8, 2t+9 (C/D columns of
// m16n8k*, i.e. the DFT outputs a thread receives).
__device__ __forceinline__ int kk_idx(int t, int kk) { return 2 * t + (kk & 1) + ((kk >> 1) << 3); }

__device__ __forceinline__ uint32_t bf162_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

// (a, b) -> bf16x2 hi (rounded) and lo (rounded residual); a ~= hi.x + lo.x.
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  hi = bf162_bits(h);
  lo = bf162_bits(__floats2bfloat162_rn(a - hf.x, b - hf.y));
}

__device__ __forceinline__ uint32_t bneg(uint32_t v) { return v ^ 0x80008000u; }

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// TF32 round-to-nearest (ties away) of an FP32 value; the result is an FP32 bit pattern
// with the low 13 mantissa bits zero.
__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// x -> hi + lo, both TF32: hi = rna(x), lo = rna(x - hi) (x - hi is exact in FP32).
__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32_1688(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Scatters the four C/D n-blocks (re out 0-7, re out 8-15, im out 0-7, im out 8-15) into
// complex outputs y[r][kk] = output kk_idx(t,kk) of row g + 8r.
__device__ __forceinline__ void gather_outputs(const float (&d)[4][4], float2 (&y)[2][4]) {
  // d[j]: (row g, col 2t), (row g, col 2t+1), (row g+8, col 2t), (row g+8, col 2t+1)
  y[0][0] = make_float2(d[0][0], d[2][0]);
  y[0][1] = make_float2(d[0][1], d[2][1]);
  y[0][2] = make_float2(d[1][0], d[3][0]);
  y[0][3] = make_float2(d[1][1], d[3][1]);
  y[1][0] = make_float2(d[0][2], d[2][2]);
  y[1][1] = make_float2(d[0][3], d[2][3]);
  y[1][2] = make_float2(d[1][2], d[3][2]);
  y[1][3] = make_float2(d[1][3], d[3][3]);
}

// The real-form DFT-16 matrix M (rows: 16 real then 16 imaginary inputs; columns: 16
// real then 16 imaginary outputs) is [[C, -S], [S, C]]. Fragments are kept for the
// real-input rows only; the imaginary-input rows of n-block j are the real-input rows of
// n-block j ^ 2, negated for j < 2 (negation flips sign bits: exact for every split part).

// BF16x3: mma.sync m16n8k16, K = 16 per k-step (k-step 0: real inputs 0-15, 1: imaginary).
// A thread supplies inputs kk_idx(t,kk) of rows g, g+8. 24 MMAs per 16 DFTs.
struct PrecBf16x3 {
  struct Frags {
    uint32_t h[4][2];  // [n-block][register], real-input k-step
    uint32_t l[4][2];
  };
  __device__ __forceinline__ static int in_idx(int t, int kk) { return kk_idx(t, kk); }
  __device__ __forceinline__ static void make(Frags &f, const float2 *tw256, int g, int t) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int k2 = (j & 1) * 8 + g;
        float v[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int n2 = 2 * t + 8 * q + e;
          const float2 w = tw256[((k2 * n2) & 15) * 16];  // (cos, -sin)
          v[e] = (j < 2) ? w.x : w.y;                      // C for real outputs, -S for imaginary
        }
        split_bf16x2(v[0], v[1], f.h[j][q], f.l[j][q]);
      }
  }
  __device__ __forceinline__ static void dft16(const float2 (&x)[2][4], float2 (&y)[2][4], const Frags &f) {
    uint32_t ah[2][4], al[2][4];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const float x00 = s ? x[0][0].y : x[0][0].x, x01 = s ? x[0][1].y : x[0][1].x;
      const float x10 = s ? x[1][0].y : x[1][0].x, x11 = s ? x[1][1].y : x[1][1].x;
      const float x02 = s ? x[0][2].y : x[0][2].x, x03 = s ? x[0][3].y : x[0][3].x;
      const float x12 = s ? x[1][2].y : x[1][2].x, x13 = s ? x[1][3].y : x[1][3].x;
      split_bf16x2(x00, x01, ah[s][0], al[s][0]);  // row g,   k 2t, 2t+1
      split_bf16x2(x10, x11, ah[s][1], al[s][1]);  // row g+8, k 2t, 2t+1
      split_bf16x2(x02, x03, ah[s][2], al[s][2]);  // row g,   k 2t+8, 2t+9
      split_bf16x2(x12, x13, ah[s][3], al[s][3]);  // row g+8, k 2t+8, 2t+9
    }
    float d[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
      const int jj = j ^ 2;
      const uint32_t h0 = j < 2 ? bneg(f.h[jj][0]) : f.h[jj][0], h1 = j < 2 ? bneg(f.h[jj][1]) : f.h[jj][1];
      const uint32_t l0 = j < 2 ? bneg(f.l[jj][0]) : f.l[jj][0], l1 = j < 2 ? bneg(f.l[jj][1]) : f.l[jj][1];
      // (accumulating the small products first, as the TF32x3 paths do, measured no better
      // here: 1.50e-5 against 1.45e-5 rel-L2; 16 significant bits per value set the error)
      mma_bf16_16816(d[j], ah[0], f.h[j][0], f.h[j][1]);
      mma_bf16_16816(d[j], ah[0], f.l[j][0], f.l[j][1]);
      mma_bf16_16816(d[j], al[0], f.h[j][0], f.h[j][1]);
      mma_bf16_16816(d[j], ah[1], h0, h1);
      mma_bf16_16816(d[j], ah[1], l0, l1);
      mma_bf16_16816(d[j], al[1], h0, h1);
    }
    gather_outputs(d, y);
  }
};

// TF32x3: mma.sync m16n8k8, K = 8 per k-step (k-steps 0, 1: real inputs 0-7, 8-15;
// 2, 3: imaginary). A thread supplies inputs t + 4*kk of rows g, g+8. 48 MMAs per 16 DFTs.
struct PrecTf32x3 {
  struct Frags {
    uint32_t h[2][4][2];  // [real-input k-step][n-block][register]
    uint32_t l[2][4][2];
  };
  __device__ __forceinline__ static int in_idx(int t, int kk) { return t + 4 * kk; }
  __device__ __forceinline__ static void make(Frags &f, const float2 *tw256, int g, int t) {
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int k2 = (j & 1) * 8 + g;
          const int n2 = 8 * ks + t + 4 * q;
          const float2 w = tw256[((k2 * n2) & 15) * 16];
          split_tf32((j < 2) ? w.x : w.y, f.h[ks][j][q], f.l[ks][j][q]);
        }
  }
  __device__ __forceinline__ static uint32_t fneg(uint32_t v) { return v ^ 0x80000000u; }
  __device__ __forceinline__ static void dft16(const float2 (&x)[2][4], float2 (&y)[2][4], const Frags &f) {
    // A for k-step ks (0,1 real; 2,3 imaginary): a0 (row g, k t), a1 (row g+8, k t),
    // a2 (row g, k t+4), a3 (row g+8, k t+4); input index within the k-step is
    // 8*(ks&1) + t (+4) = t + 4*kk with kk = 2*(ks&1) (+1).
    uint32_t ah[4][4], al[4][4];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int kk0 = 2 * (ks & 1);
      const bool im = ks >= 2;
      split_tf32(im ? x[0][kk0].y : x[0][kk0].x, ah[ks][0], al[ks][0]);
      split_tf32(im ? x[1][kk0].y : x[1][kk0].x, ah[ks][1], al[ks][1]);
      split_tf32(im ? x[0][kk0 + 1].y : x[0][kk0 + 1].x, ah[ks][2], al[ks][2]);
      split_tf32(im ? x[1][kk0 + 1].y : x[1][kk0 + 1].x, ah[ks][3], al[ks][3]);
    }
    float d[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
      // pass 0: the small products of every k-step, so that they add up at their own
      // scale; pass 1: the large ones
#pragma unroll
      for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const int kr = ks & 1;
          uint32_t h0, h1, l0, l1;
          if (ks < 2) {
            h0 = f.h[kr][j][0], h1 = f.h[kr][j][1], l0 = f.l[kr][j][0], l1 = f.l[kr][j][1];
          } else {
            const int jj = j ^ 2;
            h0 = f.h[kr][jj][0], h1 = f.h[kr][jj][1], l0 = f.l[kr][jj][0], l1 = f.l[kr][jj][1];
            if (j < 2) h0 = fneg(h0), h1 = fneg(h1), l0 = fneg(l0), l1 = fneg(l1);
          }
          if (pass == 0) {
            mma_tf32_1688(d[j], ah[ks], l0, l1);
            mma_tf32_1688(d[j], al[ks], h0, h1);
          } else {
            mma_tf32_1688(d[j], ah[ks], h0, h1);
          }
        }
      }
    }
    gather_outputs(d, y);
  }
};

// Forward 256-point transforms of the 16 columns of `buf` (slot (p, c) = p*16 + c),
// natural order in, natural order out, with the result left in registers:
// X[q][r][kk] = output p = (warp + 8q) + 16*kk_idx(t,kk) of column c = g + 8r.
// buf is the exchange buffer between the two stages (its contents are consumed).
// With SWAP the inputs and outputs have re/im exchanged (unnormalised inverse).
template <class P, bool SWAP>
__device__ __forceinline__ void tc_fft256_cols(float2 *buf, float2 (&X)[2][2][4], const float2 *tw,
                                               const typename P::Frags &fr, int warp, int g, int t) {
  float2 Y[2][2][4];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int n1 = warp + 8 * q;
    float2 x[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float2 v = buf[(n1 + 16 * P::in_idx(t, kk)) * 16 + g + 8 * r];
        x[r][kk] = SWAP ? cswap(v) : v;
      }
    P::dft16(x, Y[q], fr);
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) Y[q][r][kk] = cmul(Y[q][r][kk], tw[(n1 * kk_idx(t, kk)) & 255]);
  }
  __syncthreads();  // every stage-1 read of buf is done
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) buf[(kk_idx(t, kk) + 16 * (warp + 8 * q)) * 16 + g + 8 * r] = Y[q][r][kk];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int k2 = warp + 8 * q;
    float2 x[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) x[r][kk] = buf[(k2 + 16 * P::in_idx(t, kk)) * 16 + g + 8 * r];
    P::dft16(x, X[q], fr);
    if constexpr (SWAP) {
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) X[q][r][kk] = cswap(X[q][r][kk]);
    }
  }
}

// Natural position of X[q][r][kk] (see tc_fft256_cols).
__device__ __forceinline__ int tc_pos(int warp, int q, int t, int kk) { return warp + 8 * q + 16 * kk_idx(t, kk); }

// y / z pass of N = 256 on the tensor cores (TMA-fed tile of 256 x 16 columns, 256
// threads). Same tiles, loads and stores as k_strided_tma<256, ..., COLS = 16>.
template <class P, int OP>
__global__ void __launch_bounds__(256) k_strided_tma_tc256(const __grid_constant__ CUtensorMap msrc,
                                                          const __grid_constant__ CUtensorMap mfilt, PassArgs a,
                                                          int axis) {
  constexpr int N = 256, COLS = 16, TILE = N * COLS;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tile = reinterpret_cast<float2 *>(smraw + 128);
  float2 *ftile = tile + TILE;
  float2 *tw = HAS_F ? ftile + TILE : tile + TILE;
  const uint32_t bar = smem_u32(smraw);
  const int vol = blockIdx.x / a.groups_per_vol;
  const int rr = blockIdx.x % a.groups_per_vol;
  const int row = rr / a.groups_x;
  const int x0 = (rr % a.groups_x) * COLS;

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, (HAS_F ? 2u : 1u) * TILE * 8u);
    if (axis == 1)
      tma_load_3d(smem_u32(tile), &msrc, x0, 0, vol * N + row, bar);
    else
      tma_load_3d(smem_u32(tile), &msrc, x0, row, vol * N, bar);
    if constexpr (HAS_F) {
      const int fv = a.filt_vol_elems ? vol : 0;
      tma_load_3d(smem_u32(ftile), &mfilt, x0, row, fv * N, bar);
    }
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * 2];
  const int ok = __syncthreads_and(mbar_wait_bounded(bar, 0) ? 1 : 0);
  if (!ok) {
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(bar, 0);
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  typename P::Frags fr;
  P::make(fr, tw, g, t);

  float2 X[2][2][4];
  if constexpr (OP == OP_FWD) {
    tc_fft256_cols<P, false>(tile, X, tw, fr, warp, g, t);
  } else if constexpr (OP == OP_INV) {
    tc_fft256_cols<P, true>(tile, X, tw, fr, warp, g, t);
  } else {
    if constexpr (OP == OP_CONV_FZ) {
      // Filter spectrum back into the filter tile, each thread into the slots it reads later.
      tc_fft256_cols<P, false>(ftile, X, tw, fr, warp, g, t);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) ftile[tc_pos(warp, q, t, kk) * 16 + g + 8 * r] = X[q][r][kk];
    }
    tc_fft256_cols<P, false>(tile, X, tw, fr, warp, g, t);
    __syncthreads();  // stage-2 reads of tile are done before it is refilled
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const int slot = tc_pos(warp, q, t, kk) * 16 + g + 8 * r;
          tile[slot] = cmul(X[q][r][kk], ftile[slot]);
        }
    __syncthreads();
    tc_fft256_cols<P, true>(tile, X, tw, fr, warp, g, t);
  }
  float2 *dst = a.dst + (long long)vol * a.vol_elems + (long long)row * a.plane_pitch + x0;
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        float2 v = X[q][r][kk];
        if (a.scale != 1.0f) v = make_float2(v.x * a.scale, v.y * a.scale);
        dst[(long long)tc_pos(warp, q, t, kk) * a.axis_stride + g + 8 * r] = v;
      }
}

// x pass of N = 256 on the tensor cores: 16 rows per CTA (one TMA box {256, 16}),
// warp w owns rows w and w + 8; stage 1 reads the unpadded TMA tile, stage 2 reads a
// padded exchange buffer (slot of position p in row c: c*272 + p + p/16).
template <class P, int OP>
__global__ void __launch_bounds__(256) k_rows_tma_tc256(const __grid_constant__ CUtensorMap msrc, PassArgs a) {
  static_assert(OP == OP_FWD || OP == OP_INV, "x pass ops");
  constexpr bool SWAP = OP == OP_INV;
  constexpr int N = 256, XC = 16, PITCH = 272;
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tile = reinterpret_cast<float2 *>(smraw + 128);
  float2 *exch = tile + XC * N;
  float2 *tw = exch + XC * PITCH;
  const uint32_t bar = smem_u32(smraw);
  const long long row0 = (long long)blockIdx.x * XC;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, (uint32_t)(XC * N * 8));
    tma_load_2d(smem_u32(tile), &msrc, 0, (int)row0, bar);
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw512[i * 2];
  const int ok = __syncthreads_and(mbar_wait_bounded(bar, 0) ? 1 : 0);
  if (!ok) {
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(bar, 0);
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  typename P::Frags fr;
  P::make(fr, tw, g, t);
  // Stage 1: group = row c, instance i = n1 (rows g, g+8), inputs at n1 + 16 n2.
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int c = warp + 8 * q;
    float2 x[2][4], y[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float2 v = tile[c * N + g + 8 * r + 16 * P::in_idx(t, kk)];
        x[r][kk] = SWAP ? cswap(v) : v;
      }
    P::dft16(x, y, fr);
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const int n1 = g + 8 * r, k2 = kk_idx(t, kk);
        exch[c * PITCH + k2 + 17 * n1] = cmul(y[r][kk], tw[(n1 * k2) & 255]);  // slot of p = k2 + 16 n1
      }
  }
  __syncthreads();
  float2 *dst = a.dst + row0 * N;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int c = warp + 8 * q;
    float2 x[2][4], y[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const int p = g + 8 * r + 16 * P::in_idx(t, kk);
        x[r][kk] = exch[c * PITCH + p + (p >> 4)];
      }
    P::dft16(x, y, fr);
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        float2 v = SWAP ? cswap(y[r][kk]) : y[r][kk];
        if (a.scale != 1.0f) v = make_float2(v.x * a.scale, v.y * a.scale);
        dst[(long long)c * N + g + 8 * r + 16 * kk_idx(t, kk)] = v;
      }
  }
}

}  // namespace convgpu
