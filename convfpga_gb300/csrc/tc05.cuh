// Tensor-core split-precision passes for N = 256 on the 5th-generation tensor cores
// (tcgen05): operands from shared-memory matrix descriptors, accumulators in tensor
// memory (TMEM), one thread issuing the MMAs, completion tracked on an mbarrier.
//
// A 256-point transform is 16 x 16 (four-step). A CTA holds 16 pencils, i.e. 256
// instances of each 16-point stage; thread m owns instance m and its A-operand row
//   [yr yi] = [xr xi] . [[C, -S], [S, C]]        (real form of the DFT-16 matrix)
// in split TF32x3: x = xh + xl, M = Mh + Ml, y ~= xh.Mh + xh.Ml + xl.Mh with FP32
// accumulation. One stage is 2 M-tiles (128 instances) x 4 K-steps (K = 8 TF32) x 3
// products = 24 MMAs (kind::tf32, M = 128, N = 32) into 64 TMEM columns; each thread
// reads its 32 results back with tcgen05.ld.32x32b, applies the FP32 twiddle
// W256^(n1 k2) and scatters them into the next stage's A rows.
//
// Operand layouts (K-major, TF32), SW = 0: canonical layout without swizzle (8-row x
// 16-byte core matrices, 128 bytes apart along K, 1024 bytes between 8-row groups);
// SW = 1: 128-byte swizzle (one 8 x 128-byte atom per 8-row group, 16-byte chunk c of
// row r stored at chunk c ^ r), which spreads the stage-2 scatter over more banks.
//
// Pencil mapping (instance (a, b) = thread 16 a + b; stage-1 input n2, stage-2 output k1):
//   strided tile (256 positions x 16 columns): a = n1 or k2, b = column;
//     stage-1 inputs at positions a + 16 n2, stage-2 outputs at positions a + 16 k1.
//   row tile (16 rows x 256): a = row, b = n1 or k2; the same positions along row a.
// The fused z ops keep the forward spectrum in registers: the thread that ends the
// forward transform with positions k2 + 16 k1 of column c owns the inverse's stage-1
// instance (n1 = k2, c), so multiply and inverse continue without a round trip.
//
// Shared memory (from a 1024-byte aligned base): A hi (aliases the TMA tile), A lo
// (aliases the filter tile), B hi, B lo, twiddles, barriers. The tiles are read into
// registers before the first A row is written.
//
// Ordering: a stage's MMAs are issued after a barrier that every thread reaches only
// after its previous tcgen05.ld completed (tcgen05.fence::before_thread_sync before it,
// ::after_thread_sync after it) and after its A writes were made visible to the async
// proxy (fence.proxy.async). A rows are rewritten only after the MMAs that read them
// signalled completion on the mbarrier.
#pragma once

#include "passes.cuh"

namespace convgpu {

constexpr unsigned kStatusMmaTimeout = 4u;  // a tcgen05 completion wait gave up
constexpr unsigned kStatusSmemAlign = 8u;   // dynamic shared memory not 1024-byte aligned

constexpr int kT5Threads = 256;
constexpr int kT5ABytes = 256 * 32 * 4;  // one A part (hi or lo): 256 rows x 32 TF32
constexpr int kT5BBytes = 32 * 32 * 4;   // one B part: 32 x 32 TF32
constexpr int kT5OffB = 2 * kT5ABytes;
constexpr int kT5OffTw = kT5OffB + 2 * kT5BBytes;
constexpr int kT5OffBar = kT5OffTw + 256 * 8;
constexpr int kT5Smem = kT5OffBar + 128;
constexpr uint32_t kT5Sbo = 1024;
// kind::tf32, D F32, A / B TF32 K-major, N = 32, M = 128
constexpr uint32_t kT5Idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

template <int SW>
__device__ __forceinline__ uint64_t t5_desc(uint32_t addr) {
  constexpr uint32_t lbo = SW ? 16u : 128u;
  constexpr uint64_t layout = SW ? 2ull : 0ull;  // 2 = 128-byte swizzle
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((kT5Sbo >> 4) & 0x3FFF) << 32) | (1ull << 46) | (layout << 61);
}

// Byte offset of the start of K-step s (8 TF32) inside an operand.
template <int SW>
__device__ __forceinline__ uint32_t t5_kstep(int s) {
  return SW ? (uint32_t)(32 * s) : (uint32_t)(256 * s);
}

// Byte offset of element (row m, k) of a K-major TF32 operand (32 K values per row).
template <int SW>
__device__ __forceinline__ uint32_t t5_off(int m, int k) {
  if (SW) return (uint32_t)((m >> 3) * 1024 + (m & 7) * 128 + ((((k >> 2) ^ (m & 7)) & 7) << 4) + (k & 3) * 4);
  return (uint32_t)((m >> 3) * 1024 + (k >> 2) * 128 + (m & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint32_t t5_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void t5_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void t5_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

struct T5Ctx {
  unsigned char *ah, *al;  // A operand parts (hi, lo)
  uint32_t bh, bl;         // B operand parts (shared-memory addresses)
  uint32_t tmem;           // TMEM base (64 columns)
  uint32_t bar;            // MMA-completion mbarrier
  uint32_t phase;
  int ok;  // 0 once a completion wait gave up
};

// Writes thread m's A row from 16 complex inputs (TF32 hi / lo split).
template <int SW>
__device__ __forceinline__ void t5_put_row(const T5Ctx &cx, int m, const float2 (&x)[16]) {
#pragma unroll
  for (int kg = 0; kg < 8; ++kg) {  // one 16-byte chunk = 4 K values
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = kg * 4 + j;
      const float v = k < 16 ? x[k].x : x[k - 16].y;
      h[j] = t5_rna(v);
      l[j] = t5_rna(v - __uint_as_float(h[j]));
    }
    const uint32_t off = t5_off<SW>(m, kg * 4);
    *reinterpret_cast<uint4 *>(cx.ah + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(cx.al + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

template <int SW>
__device__ __forceinline__ void t5_put(const T5Ctx &cx, int m, int k, float v) {
  const uint32_t h = t5_rna(v);
  const uint32_t off = t5_off<SW>(m, k);
  *reinterpret_cast<uint32_t *>(cx.ah + off) = h;
  *reinterpret_cast<uint32_t *>(cx.al + off) = t5_rna(v - __uint_as_float(h));
}

// Runs the 24 MMAs of one stage over the A rows all threads have written and returns
// this thread's row of D: y[k] = (re out k, im out k).
template <int SW>
__device__ __forceinline__ void t5_mma_stage(T5Ctx &cx, float2 (&y)[16]) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (threadIdx.x == 0) {
    const uint32_t ah = smem_u32(cx.ah), al = smem_u32(cx.al);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const uint32_t d = cx.tmem + (uint32_t)(32 * mt);
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const uint32_t ao = (uint32_t)(mt * 16 * 1024) + t5_kstep<SW>(s), bo = t5_kstep<SW>(s);
        const uint64_t ad[3] = {t5_desc<SW>(ah + ao), t5_desc<SW>(ah + ao), t5_desc<SW>(al + ao)};
        const uint64_t bd[3] = {t5_desc<SW>(cx.bh + bo), t5_desc<SW>(cx.bl + bo), t5_desc<SW>(cx.bh + bo)};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const uint32_t acc = (s == 0 && q == 0) ? 0u : 1u;
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
              "l"(ad[q]), "l"(bd[q]), "r"(kT5Idesc), "r"(acc));
        }
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(cx.bar)
                 : "memory");
  }
  if (!mbar_wait_bounded(cx.bar, cx.phase)) cx.ok = 0;
  cx.phase ^= 1u;
  t5_fence_after();
  const int w = threadIdx.x >> 5;
  const uint32_t taddr = cx.tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(32 * (w >> 2));
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) y[k] = make_float2(__uint_as_float(r[k]), __uint_as_float(r[16 + k]));
}

// Parks 16 complex values of this thread in TMEM columns 64.. (outside the MMA
// accumulators) and brings them back: frees 32 registers across a transform.
__device__ __forceinline__ uint32_t t5_stash_addr(const T5Ctx &cx) {
  const int w = threadIdx.x >> 5;
  return cx.tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(64 + 32 * (w >> 2));
}

__device__ __forceinline__ void t5_stash_st(const T5Ctx &cx, const float2 (&v)[16]) {
  uint32_t r[32];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    r[2 * k] = __float_as_uint(v[k].x);
    r[2 * k + 1] = __float_as_uint(v[k].y);
  }
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(t5_stash_addr(cx)),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
      "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),
      "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]),
      "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void t5_stash_ld(const T5Ctx &cx, float2 (&v)[16]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(t5_stash_addr(cx)));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(__uint_as_float(r[2 * k]), __uint_as_float(r[2 * k + 1]));
}

// 256-point forward transform of the CTA's 16 pencils. On entry x holds thread
// (a, b)'s stage-1 inputs; on exit its stage-2 outputs (see the mapping above).
template <int SW, bool ROWS>
__device__ __forceinline__ void t5_fft256(T5Ctx &cx, float2 (&x)[16], const float2 *tw) {
  const int m = threadIdx.x, a = m >> 4, b = m & 15;
  t5_put_row<SW>(cx, m, x);
  float2 y[16];
  t5_mma_stage<SW>(cx, y);
  const int n1 = ROWS ? b : a;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    const float2 v = cmul(y[k2], tw[(n1 * k2) & 255]);
    const int m2 = ROWS ? (16 * a + k2) : (16 * k2 + b);
    t5_put<SW>(cx, m2, n1, v.x);
    t5_put<SW>(cx, m2, 16 + n1, v.y);
  }
  t5_mma_stage<SW>(cx, x);
}

// y / z pass (axis 1 / 2, tile 256 positions x 16 columns) or x pass (ROWS, tile of
// 16 rows x 256) of 256^3 cubes on tcgen05, with the same tensor maps, grids and
// output addressing as the FP32 kernels k_strided_tma<256, 16, 16> / k_rows_tma.
template <int SW, int OP, bool ROWS>
__global__ void __launch_bounds__(kT5Threads, 3) k_tc05_256(const __grid_constant__ CUtensorMap msrc,
                                                         const __grid_constant__ CUtensorMap mfilt, PassArgs a,
                                                         int axis) {
  constexpr int N = 256, TILE = 4096;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  constexpr int kCols = HAS_F ? 128 : 64;  // accumulators (+ a park area for the fused ops)
  static_assert(!(ROWS && HAS_F), "fused ops are z passes");
  extern __shared__ __align__(1024) unsigned char smraw[];
  if (smem_u32(smraw) & 1023u) {  // the swizzle atoms and descriptors assume this
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusSmemAlign);
    return;
  }
  float2 *tile = reinterpret_cast<float2 *>(smraw);
  float2 *ftile = tile + TILE;
  float2 *tw = reinterpret_cast<float2 *>(smraw + kT5OffTw);
  unsigned char *bbuf = smraw + kT5OffB;
  const uint32_t tbar = smem_u32(smraw + kT5OffBar), mbar = tbar + 8;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smraw + kT5OffBar + 16);

  int vol = 0, row = 0, x0 = 0;
  long long row0 = 0;
  if (ROWS) {
    row0 = (long long)blockIdx.x * 16;
  } else {
    vol = blockIdx.x / a.groups_per_vol;
    const int rr = blockIdx.x % a.groups_per_vol;
    row = rr / a.groups_x;
    x0 = (rr % a.groups_x) * 16;
  }
  if (threadIdx.x == 0) {
    mbar_init(tbar, 1);
    mbar_init(mbar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(tbar, (HAS_F ? 2u : 1u) * TILE * 8u);
    if (ROWS) {
      tma_load_2d(smem_u32(tile), &msrc, 0, (int)row0, tbar);
    } else {
      if (axis == 1)
        tma_load_3d(smem_u32(tile), &msrc, x0, 0, vol * N + row, tbar);
      else
        tma_load_3d(smem_u32(tile), &msrc, x0, row, vol * N, tbar);
      if constexpr (HAS_F) tma_load_3d(smem_u32(ftile), &mfilt, x0, row, (a.filt_vol_elems ? vol : 0) * N, tbar);
    }
  }
  // Twiddles and the DFT-16 matrix while the tile loads. B[o][k]: o = output (re k2,
  // then im k2), k = input (re n2, then im n2); W16^(k2 n2) = (c, -s) gives
  // re = xr c + xi s, im = -xr s + xi c.
  for (int i = threadIdx.x; i < N; i += kT5Threads) tw[i] = a.tw512[2 * i];
  for (int i = threadIdx.x; i < 32 * 32; i += kT5Threads) {
    const int o = i >> 5, k = i & 31;
    const float2 w = a.tw512[32 * (((o & 15) * (k & 15)) & 15)];
    const float c = w.x, s = -w.y;
    const float v = o >= 16 ? (k >= 16 ? c : -s) : (k >= 16 ? s : c);
    const uint32_t h = t5_rna(v);
    const uint32_t off = t5_off<SW>(o, k);
    *reinterpret_cast<uint32_t *>(bbuf + off) = h;
    *reinterpret_cast<uint32_t *>(bbuf + kT5BBytes + off) = t5_rna(v - __uint_as_float(h));
  }
  const int loaded = __syncthreads_and(mbar_wait_bounded(tbar, 0) ? 1 : 0);
  if (!loaded) {  // no TMEM is held yet
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(tbar, 0);
    return;
  }

  T5Ctx cx;
  cx.ah = smraw;
  cx.al = smraw + kT5ABytes;
  cx.bh = smem_u32(bbuf);
  cx.bl = cx.bh + kT5BBytes;
  cx.bar = mbar;
  cx.phase = 0;
  cx.ok = 1;
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  t5_fence_before();
  __syncthreads();  // TMEM address published
  t5_fence_after();
  cx.tmem = *tslot;

  const int m = threadIdx.x, ia = m >> 4, ib = m & 15;
  auto gather = [&](const float2 *t, float2 (&x)[16], bool swap) {
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) {
      const float2 v = ROWS ? t[ia * N + ib + 16 * n2] : t[(ia + 16 * n2) * 16 + ib];
      x[n2] = swap ? cswap(v) : v;
    }
  };
  float2 x[16];
  if constexpr (OP == OP_FWD || OP == OP_INV) {
    gather(tile, x, OP == OP_INV);
    __syncthreads();  // tile consumed before A (which aliases it) is written
    t5_fft256<SW, ROWS>(cx, x, tw);
    if (OP == OP_INV) {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = cswap(x[k]);
    }
  } else {
    float2 f[16];
    if constexpr (OP == OP_CONV_FZ) {
      // signal parked in TMEM while the filter is transformed
      gather(tile, x, false);
      t5_stash_st(cx, x);
      gather(ftile, f, false);
      __syncthreads();
      t5_fft256<SW, false>(cx, f, tw);
      t5_stash_ld(cx, x);
      t5_stash_st(cx, f);
    } else {
      // filter spectrum (positions ia + 16 k1 of column ib) parked in TMEM
#pragma unroll
      for (int k1 = 0; k1 < 16; ++k1) f[k1] = ftile[(ia + 16 * k1) * 16 + ib];
      t5_stash_st(cx, f);
      gather(tile, x, false);
      __syncthreads();
    }
    t5_fft256<SW, false>(cx, x, tw);
    t5_stash_ld(cx, f);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) x[k1] = cswap(cmul(x[k1], f[k1]));
    t5_fft256<SW, false>(cx, x, tw);
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = cswap(x[k]);
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cx.tmem), "n"(kCols));
  if (!cx.ok && threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusMmaTimeout);

  if (ROWS) {
    float2 *dst = a.dst + (row0 + ia) * N + ib;
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
      float2 v = x[k1];
      if (a.scale != 1.0f) v = make_float2(v.x * a.scale, v.y * a.scale);
      dst[16 * k1] = v;
    }
  } else {
    float2 *dst = a.dst + (long long)vol * a.vol_elems + (long long)row * a.plane_pitch + x0 + ib;
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
      float2 v = x[k1];
      if (a.scale != 1.0f) v = make_float2(v.x * a.scale, v.y * a.scale);
      dst[(long long)(ia + 16 * k1) * a.axis_stride] = v;
    }
  }
}

}  // namespace convgpu
