// Tensor-core split-precision passes for N = 256 and 512 on the 5th-generation tensor
// cores (tcgen05): operands from shared-memory matrix descriptors, accumulators in tensor
// memory (TMEM), one thread issuing the MMAs, completion tracked on an mbarrier. (N = 512:
// a radix-2 step around two 256-point transforms, k_tc05_512 at the end of this file.)
//
// A 256-point transform is 16 x 16 (four-step). A CTA holds P pencils (P = 8 or 16),
// i.e. 16 P instances of each 16-point stage; thread m owns instance m and its A row
//   [yr yi] = [xr xi] . [[C, -S], [S, C]]        (real form of the DFT-16 matrix)
// in split TF32x3: x = xh + xl, M = Mh + Ml, y ~= xh.Ml + xl.Mh + xh.Mh with FP32
// accumulation, the two small products first so that they add up at their own scale.
// xh is x rounded to TF32 (nearest, ties away: add half an ulp to the bit pattern, clear
// the 13 low bits), xl = x - xh truncated to TF32; both are exact TF32 bit patterns
// made with integer operations only. One stage is P / 8 M-tiles (128 instances) x 4
// K-steps (K = 8 TF32) x 3 products = 12 MMAs per M-tile (kind::tf32, M = 128, N = 32) into 32 TMEM columns per
// M-tile; each thread reads its 32 results back with tcgen05.ld.32x32b, applies the
// FP32 twiddle W256^(n1 k2) and scatters them into the next stage's A rows.
//
// Operand layout (K-major, TF32, 128-byte swizzle): one 8-row x 128-byte atom per
// 8-row group (1024 bytes apart), 16-byte chunk c of row r stored at chunk c ^ (r & 7);
// the K-step s descriptor starts 32 s bytes into the atom.
//
// Pencil mapping (stage-1 input n2, stage-2 output k1):
//   strided tile (256 positions x P columns): thread m = P a + b, a = n1 or k2, b = column;
//     stage-1 inputs at positions a + 16 n2, stage-2 outputs at positions a + 16 k1;
//     stage-2 instance (k2, b) is row P k2 + b (the scatter is bank-conflict free for P = 8).
//   row tile (P rows x 256): thread m = 16 a + b, a = row, b = n1 or k2; the same
//     positions along row a; stage-2 instance (a, k2) is row 16 a + k2.
// The fused z ops continue from registers: the thread that ends the forward transform
// with positions k2 + 16 k1 of column c owns the inverse's stage-1 instance (n1 = k2, c).
// The operand that waits while another is transformed (the signal during the filter's
// transform, the filter spectrum during the signal's) is parked in spare TMEM columns.
//
// Shared memory (1024-byte aligned base): A hi (aliases the signal tile), A lo (aliases
// the filter tile), B hi, B lo, twiddles W256^j (one bulk copy of a constant block built
// once per device by k_tc05_consts), barriers. The tiles are read into registers before
// the first A row is written.
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

// Constant block (bytes): B hi | B lo | W256^j, j < 256. It sits in the twiddle buffer
// handed to the tensor-core path, right after the 512 twiddles W512^j.
constexpr int kT5BBytes = 32 * 32 * 4;  // one B part: 32 x 32 TF32
constexpr int kT5ConstBytes = 2 * kT5BBytes + 256 * 8;
constexpr int kT5ConstOffset = 512 * 8;

template <int P>
struct T5Geom {
  static_assert(P == 8 || P == 16, "8 or 16 pencils per CTA");
  static constexpr int kThreads = 16 * P;
  static constexpr int kMTiles = P / 8;
  static constexpr int kABytes = 16 * P * 128;  // one A part: 16 P rows x 32 TF32
  static constexpr int kOffB = 2 * kABytes;
  static constexpr int kOffTw = kOffB + 2 * kT5BBytes;
  static constexpr int kOffBar = kOffB + kT5ConstBytes;
  static constexpr int kSmem = kOffBar + 128;
  static constexpr int kMinBlocks = P == 8 ? 5 : 3;
};

// kind::tf32, D F32, A / B TF32 K-major, N = 32, M = 128
constexpr uint32_t kT5Idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

// Shared-memory descriptor: start address, LBO 16 (unused by swizzled K-major), SBO 1024,
// version 1 (bit 46), 128-byte swizzle (layout type 2, bits 61-63).
__device__ __forceinline__ uint64_t t5_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// Byte offset of element (row m, k) of a K-major TF32 operand (32 K values per row).
__device__ __forceinline__ uint32_t t5_off(int m, int k) {
  return (uint32_t)((m >> 3) * 1024 + (m & 7) * 128 + ((((k >> 2) ^ m) & 7) << 4) + (k & 3) * 4);
}

__device__ __forceinline__ uint32_t t5_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// Operand split of a data value: (TF32 nearest of v, TF32 truncation of the rest).
__device__ __forceinline__ uint2 t5_split(float v) {
  const uint32_t h = (__float_as_uint(v) + 0x1000u) & 0xFFFFE000u;
  return make_uint2(h, __float_as_uint(v - __uint_as_float(h)) & 0xFFFFE000u);
}

__device__ __forceinline__ void t5_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void t5_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// One-block kernel writing the constant block: B[o][k] with o = output (re k2, then im
// k2), k = input (re n2, then im n2); W16^(k2 n2) = (c, -s) gives re = xr c + xi s,
// im = -xr s + xi c. Split into TF32 hi and lo parts in the swizzled layout.
static __global__ void k_tc05_consts(unsigned char *blk, const float2 *tw512) {
  for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
    const int o = i >> 5, k = i & 31;
    const float2 w = tw512[32 * (((o & 15) * (k & 15)) & 15)];
    const float c = w.x, s = -w.y;
    const float v = o >= 16 ? (k >= 16 ? c : -s) : (k >= 16 ? s : c);
    const uint32_t h = t5_rna(v);
    const uint32_t off = t5_off(o, k);
    *reinterpret_cast<uint32_t *>(blk + off) = h;
    *reinterpret_cast<uint32_t *>(blk + kT5BBytes + off) = t5_rna(v - __uint_as_float(h));
  }
  float2 *tw = reinterpret_cast<float2 *>(blk + 2 * kT5BBytes);
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tw[i] = tw512[2 * i];
}

template <int P>
struct T5Ctx {
  unsigned char *ah, *al;  // A operand parts (hi, lo)
  uint32_t bh, bl;         // B operand parts (shared-memory addresses)
  uint32_t tmem;           // TMEM base: accumulators at 32 mt, park area after them
  uint32_t bar;            // MMA-completion mbarrier
  uint32_t phase;
  int ok;  // 0 once a completion wait gave up
};

// Writes thread m's A row from 16 complex inputs (TF32 hi / lo split).
template <int P>
__device__ __forceinline__ void t5_put_row(const T5Ctx<P> &cx, int m, const float2 (&x)[16]) {
#pragma unroll
  for (int kg = 0; kg < 8; ++kg) {  // one 16-byte chunk = 4 K values
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = kg * 4 + j;
      const uint2 hl = t5_split(k < 16 ? x[k].x : x[k - 16].y);
      h[j] = hl.x;
      l[j] = hl.y;
    }
    const uint32_t off = t5_off(m, kg * 4);
    *reinterpret_cast<uint4 *>(cx.ah + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(cx.al + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

template <int P>
__device__ __forceinline__ void t5_put(const T5Ctx<P> &cx, uint32_t off, float v) {
  const uint2 hl = t5_split(v);
  *reinterpret_cast<uint32_t *>(cx.ah + off) = hl.x;
  *reinterpret_cast<uint32_t *>(cx.al + off) = hl.y;
}

__device__ __forceinline__ void t5_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// TMEM address of this warp's 32 lanes in column block `col`.
__device__ __forceinline__ uint32_t t5_lane_addr(uint32_t tmem, int col) {
  const int w = threadIdx.x >> 5;
  return tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(col + 32 * (w >> 2));
}

// Parks 16 complex values of this thread in the TMEM columns after the accumulators and
// brings them back: frees 32 registers across a transform.
template <int P>
__device__ __forceinline__ void t5_stash_st(const T5Ctx<P> &cx, const float2 (&v)[16]) {
  uint32_t r[32];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    r[2 * k] = __float_as_uint(v[k].x);
    r[2 * k + 1] = __float_as_uint(v[k].y);
  }
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(t5_lane_addr(cx.tmem, 32 * (P / 8))),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
      "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),
      "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]),
      "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

template <int P>
__device__ __forceinline__ void t5_stash_ld(const T5Ctx<P> &cx, float2 (&v)[16]) {
  uint32_t r[32];
  t5_ld32(t5_lane_addr(cx.tmem, 32 * (P / 8)), r);
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(__uint_as_float(r[2 * k]), __uint_as_float(r[2 * k + 1]));
}

// Runs the MMAs of one stage over the A rows all threads have written and returns this
// thread's row of D: y[k] = (re out k, im out k).
template <int P>
__device__ __forceinline__ void t5_mma_stage(T5Ctx<P> &cx, float2 (&y)[16]) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (threadIdx.x == 0) {
    const uint32_t ah = smem_u32(cx.ah), al = smem_u32(cx.al);
#pragma unroll
    for (int mt = 0; mt < P / 8; ++mt) {
      const uint32_t d = cx.tmem + (uint32_t)(32 * mt);
      // products xh.Ml, xl.Mh (small) for all K-steps, then xh.Mh
#pragma unroll
      for (int q = 0; q < 3; ++q) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const uint32_t ao = (uint32_t)(mt * 16 * 1024 + 32 * s), bo = (uint32_t)(32 * s);
          const uint32_t aa = (q == 1 ? al : ah) + ao, bb = (q == 0 ? cx.bl : cx.bh) + bo;
          const uint32_t acc = (s == 0 && q == 0) ? 0u : 1u;
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
              "l"(t5_desc(aa)), "l"(t5_desc(bb)), "r"(kT5Idesc), "r"(acc));
        }
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(cx.bar)
                 : "memory");
  }
  if (!mbar_wait_bounded(cx.bar, cx.phase)) cx.ok = 0;
  cx.phase ^= 1u;
  t5_fence_after();
  uint32_t r[32];
  t5_ld32(t5_lane_addr(cx.tmem, 0), r);
#pragma unroll
  for (int k = 0; k < 16; ++k) y[k] = make_float2(__uint_as_float(r[k]), __uint_as_float(r[16 + k]));
}

// 256-point forward transform of the CTA's P pencils. On entry x holds this thread's
// stage-1 inputs; on exit its stage-2 outputs (see the mapping above).
template <int P, bool ROWS>
__device__ __forceinline__ void t5_fft256(T5Ctx<P> &cx, float2 (&x)[16], const float2 *tw) {
  const int m = threadIdx.x;
  const int a = ROWS ? (m >> 4) : (m / P), b = ROWS ? (m & 15) : (m % P);
  t5_put_row<P>(cx, m, x);
  float2 y[16];
  t5_mma_stage<P>(cx, y);
  const int n1 = ROWS ? b : a;
  // stage-2 row m2(k2) and its byte offsets for inputs n1 (re) and 16 + n1 (im)
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    const float2 v = cmul(y[k2], tw[(n1 * k2) & 255]);
    const int m2 = ROWS ? (16 * a + k2) : (P * k2 + b);
    t5_put<P>(cx, t5_off(m2, n1), v.x);
    t5_put<P>(cx, t5_off(m2, 16 + n1), v.y);
  }
  t5_mma_stage<P>(cx, x);
}

// y / z pass (axis 1 / 2, tile of 256 positions x P columns) or x pass (ROWS, tile of
// P rows x 256) of 256^3 cubes on tcgen05. a.tw512 carries the constant block at
// kT5ConstOffset bytes.
template <int P, int OP, bool ROWS>
__global__ void __launch_bounds__(T5Geom<P>::kThreads, T5Geom<P>::kMinBlocks)
    k_tc05_256(const __grid_constant__ CUtensorMap msrc, const __grid_constant__ CUtensorMap mfilt, PassArgs a,
               int axis) {
  using G = T5Geom<P>;
  constexpr int N = 256, TILE = 256 * P;
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  // accumulators (32 columns per M-tile) + a park area for the fused ops; power of 2 >= 32
  constexpr uint32_t kCols = HAS_F ? 64u * (P / 8) : 32u * (P / 8);
  static_assert(!(ROWS && HAS_F), "fused ops are z passes");
  extern __shared__ __align__(1024) unsigned char smraw[];
  if (smem_u32(smraw) & 1023u) {  // the swizzle atoms assume this
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusSmemAlign);
    return;
  }
  float2 *tile = reinterpret_cast<float2 *>(smraw);
  float2 *ftile = reinterpret_cast<float2 *>(smraw + G::kABytes);
  const float2 *tw = reinterpret_cast<const float2 *>(smraw + G::kOffTw);
  const uint32_t tbar = smem_u32(smraw + G::kOffBar), mbar = tbar + 8;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smraw + G::kOffBar + 16);

  int vol = 0, row = 0, x0 = 0;
  long long row0 = 0;
  if (ROWS) {
    row0 = (long long)blockIdx.x * P;
  } else {
    vol = blockIdx.x / a.groups_per_vol;
    const int rr = blockIdx.x % a.groups_per_vol;
    row = rr / a.groups_x;
    x0 = (rr % a.groups_x) * P;
  }
  if (threadIdx.x == 0) {
    mbar_init(tbar, 1);
    mbar_init(mbar, 1);
    mbar_fence_init();
    mbar_arrive_expect_tx(tbar, (HAS_F ? 2u : 1u) * TILE * 8u + (uint32_t)kT5ConstBytes);
    if (ROWS) {
      tma_load_2d(smem_u32(tile), &msrc, 0, (int)row0, tbar);
    } else {
      if (axis == 1)
        tma_load_3d(smem_u32(tile), &msrc, x0, 0, vol * N + row, tbar);
      else
        tma_load_3d(smem_u32(tile), &msrc, x0, row, vol * N, tbar);
      if constexpr (HAS_F) tma_load_3d(smem_u32(ftile), &mfilt, x0, row, (a.filt_vol_elems ? vol : 0) * N, tbar);
    }
    bulk_load(smem_u32(smraw + G::kOffB), reinterpret_cast<const unsigned char *>(a.tw512) + kT5ConstOffset,
              (uint32_t)kT5ConstBytes, tbar);
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  t5_fence_before();
  __syncthreads();  // barrier initialised, TMEM address published
  t5_fence_after();
  T5Ctx<P> cx;
  cx.ah = smraw;
  cx.al = smraw + G::kABytes;
  cx.bh = smem_u32(smraw + G::kOffB);
  cx.bl = cx.bh + kT5BBytes;
  cx.tmem = *tslot;
  cx.bar = mbar;
  cx.phase = 0;
  cx.ok = 1;

  const int loaded = __syncthreads_and(mbar_wait_bounded(tbar, 0) ? 1 : 0);
  if (!loaded) {
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(tbar, 0);  // copies still in flight land before the CTA exits
    t5_fence_before();
    __syncthreads();
    t5_fence_after();
    if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cx.tmem), "n"(kCols));
    return;
  }

  const int m = threadIdx.x;
  const int ia = ROWS ? (m >> 4) : (m / P), ib = ROWS ? (m & 15) : (m % P);
  auto gather = [&](const float2 *t, float2 (&x)[16], bool swap) {
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) {
      const float2 v = ROWS ? t[ia * N + ib + 16 * n2] : t[(ia + 16 * n2) * P + ib];
      x[n2] = swap ? cswap(v) : v;
    }
  };
  float2 x[16];
  if constexpr (OP == OP_FWD || OP == OP_INV) {
    gather(tile, x, OP == OP_INV);
    __syncthreads();  // tile consumed before A (which aliases it) is written
    t5_fft256<P, ROWS>(cx, x, tw);
    if (OP == OP_INV) {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = cswap(x[k]);
    }
  } else {
    float2 f[16];
    if constexpr (OP == OP_CONV_FZ) {
      gather(tile, x, false);
      t5_stash_st<P>(cx, x);  // signal parked while the filter is transformed
      gather(ftile, f, false);
      __syncthreads();
      t5_fft256<P, false>(cx, f, tw);
      t5_stash_ld<P>(cx, x);
      t5_stash_st<P>(cx, f);
    } else {
#pragma unroll
      for (int k1 = 0; k1 < 16; ++k1) f[k1] = ftile[(ia + 16 * k1) * P + ib];
      t5_stash_st<P>(cx, f);  // filter spectrum parked
      gather(tile, x, false);
      __syncthreads();
    }
    t5_fft256<P, false>(cx, x, tw);
    t5_stash_ld<P>(cx, f);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) x[k1] = cswap(cmul(x[k1], f[k1]));
    t5_fft256<P, false>(cx, x, tw);
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

// ------------------------------------------------------------------ N = 512
// A 512-point transform is one radix-2 step on the CUDA cores around two 256-point
// transforms on the tensor cores (t5_fft256 with P = 8 sub-pencils):
//   forward, decimation in frequency: u[p] = x[p] + x[p+256], w[p] = (x[p] - x[p+256]) W512^p
//     for p < 256; X[2k] = DFT256(u)[k], X[2k+1] = DFT256(w)[k];
//   inverse, decimation in time: E = IDFT256(X[2m]), O = IDFT256(X[2m+1]);
//     x[n] = E[n] + W512^-n O[n], x[n+256] = E[n] - W512^-n O[n] for n < 256.
// A CTA holds 4 pencils of 512 (4 columns of a y / z tile, or 4 rows of an x tile), i.e. 8
// sub-pencils of 256, so every tensor-core stage is one M = 128 tile, as for N = 256 with 8
// pencils. Sub-pencil j of pencil c (j = 0: u / even outputs, 1: w / odd outputs) is
// sub-column b = 4j + c of the strided mapping (thread m = 8a + b) or sub-row a = 2c + j
// of the row mapping (thread m = 16a + b); the threads that combine E and O are lanes m and
// m ^ 4 (strided) or m ^ 16 (rows) of one warp and exchange through a shuffle. The forward
// transform leaves X[2(q + 16k) + j] in the registers of thread (q, j, c); the fused z ops
// multiply both operands in that order and start the inverse from it, the plain forward
// pass stores it to positions 2(q + 16k) + j. Twiddles W512^p come from the engine's FP32
// table (generated in FP64), read through L1.
template <int OP, bool ROWS>
__global__ void __launch_bounds__(T5Geom<8>::kThreads, T5Geom<8>::kMinBlocks)
    k_tc05_512(const __grid_constant__ CUtensorMap msrc, const __grid_constant__ CUtensorMap mfilt, PassArgs a,
               int axis) {
  using G = T5Geom<8>;
  constexpr int N = 512, P = 4, TILE = N * P;  // 4 pencils: 16 KB, one A part
  static_assert(TILE * 8 == G::kABytes, "a tile is one A operand part");
  constexpr bool HAS_F = (OP == OP_CONV || OP == OP_CONV_FZ);
  constexpr uint32_t kCols = HAS_F ? 64u : 32u;
  static_assert(!(ROWS && HAS_F), "fused ops are z passes");
  extern __shared__ __align__(1024) unsigned char smraw[];
  if (smem_u32(smraw) & 1023u) {
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusSmemAlign);
    return;
  }
  float2 *tile = reinterpret_cast<float2 *>(smraw);
  float2 *ftile = reinterpret_cast<float2 *>(smraw + G::kABytes);
  const float2 *tw = reinterpret_cast<const float2 *>(smraw + G::kOffTw);
  const uint32_t tbar = smem_u32(smraw + G::kOffBar), mbar = tbar + 8;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smraw + G::kOffBar + 16);

  int vol = 0, row = 0, x0 = 0;
  long long row0 = 0;
  if (ROWS) {
    row0 = (long long)blockIdx.x * P;
  } else {
    vol = blockIdx.x / a.groups_per_vol;
    const int rr = blockIdx.x % a.groups_per_vol;
    row = rr / a.groups_x;
    x0 = (rr % a.groups_x) * P;
  }
  if (threadIdx.x == 0) {
    mbar_init(tbar, 1);
    mbar_init(mbar, 1);
    mbar_fence_init();
    mbar_arrive_expect_tx(tbar, (HAS_F ? 2u : 1u) * TILE * 8u + (uint32_t)kT5ConstBytes);
    if (ROWS) {
      tma_load_3d(smem_u32(tile), &msrc, 0, 0, (int)row0, tbar);  // rows viewed as (256, 2, rows)
    } else {
#pragma unroll
      for (int l = 0; l < 2; ++l) {  // a box is at most 256 long
        if (axis == 1)
          tma_load_3d(smem_u32(tile + l * 256 * P), &msrc, x0, 256 * l, vol * N + row, tbar);
        else
          tma_load_3d(smem_u32(tile + l * 256 * P), &msrc, x0, row, vol * N + 256 * l, tbar);
        if constexpr (HAS_F)
          tma_load_3d(smem_u32(ftile + l * 256 * P), &mfilt, x0, row, (a.filt_vol_elems ? vol : 0) * N + 256 * l,
                      tbar);
      }
    }
    bulk_load(smem_u32(smraw + G::kOffB), reinterpret_cast<const unsigned char *>(a.tw512) + kT5ConstOffset,
              (uint32_t)kT5ConstBytes, tbar);
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  T5Ctx<8> cx;
  cx.ah = smraw;
  cx.al = smraw + G::kABytes;
  cx.bh = smem_u32(smraw + G::kOffB);
  cx.bl = cx.bh + kT5BBytes;
  cx.tmem = *tslot;
  cx.bar = mbar;
  cx.phase = 0;
  cx.ok = 1;

  const int loaded = __syncthreads_and(mbar_wait_bounded(tbar, 0) ? 1 : 0);
  if (!loaded) {
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    mbar_wait_bounded(tbar, 0);
    t5_fence_before();
    __syncthreads();
    t5_fence_after();
    if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cx.tmem), "n"(kCols));
    return;
  }

  const int m = threadIdx.x;
  const int ia = ROWS ? (m >> 4) : (m >> 3), ib = ROWS ? (m & 15) : (m & 7);
  const int j = ROWS ? (ia & 1) : (ib >> 2);   // sub-pencil: even (0) or odd (1) outputs
  const int c = ROWS ? (ia >> 1) : (ib & 3);   // pencil of the tile
  const int q = ROWS ? ib : ia;                // this thread's 256-positions are q + 16 i
  const int partner = ROWS ? 16 : 4;           // lane of the other sub-pencil of the pencil
  const float sgn = j ? -1.f : 1.f;
  auto at = [&](const float2 *t, int p) -> float2 { return ROWS ? t[c * N + p] : t[p * P + c]; };
  // forward: stage-1 inputs of sub-pencil j, u or w at positions q + 16 n2 (the product
  // with (1, 0) for j = 0 is exact, so both sub-pencils take one branch-free path)
  auto gather_dif = [&](const float2 *t, float2 (&x)[16]) {
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) {
      const int p = q + 16 * n2;
      const float2 u = at(t, p), v = at(t, p + 256);
      const float2 d = make_float2(fmaf(sgn, v.x, u.x), fmaf(sgn, v.y, u.y));
      x[n2] = cmul(d, j ? __ldg(a.tw512 + p) : make_float2(1.f, 0.f));
    }
  };
  // inverse: stage-1 inputs of sub-pencil j from a natural-order spectrum, X[2(q + 16 n2) + j]
  auto gather_dit = [&](const float2 *t, float2 (&x)[16]) {
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) x[n2] = at(t, 2 * (q + 16 * n2) + j);
  };
  // after IDFT256 of both sub-pencils: x holds E (j = 0) or O (j = 1) at n = q + 16 k;
  // returns x[n] (j = 0) or x[n + 256] (j = 1)
  auto combine = [&](float2 (&x)[16]) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float2 w = __ldg(a.tw512 + q + 16 * k);
      const float2 t = cmul(x[k], j ? make_float2(w.x, -w.y) : make_float2(1.f, 0.f));
      const float rx = __shfl_xor_sync(0xffffffffu, t.x, partner);
      const float ry = __shfl_xor_sync(0xffffffffu, t.y, partner);
      x[k] = make_float2(fmaf(sgn, t.x, rx), fmaf(sgn, t.y, ry));
    }
  };

  float2 x[16];
  bool natural = true;  // outputs at n = q + 16 k + 256 j, else at 2(q + 16 k) + j
  if constexpr (OP == OP_FWD) {
    gather_dif(tile, x);
    __syncthreads();  // tile consumed before A (which aliases it) is written
    t5_fft256<8, ROWS>(cx, x, tw);
    natural = false;
  } else if constexpr (OP == OP_INV) {
    gather_dit(tile, x);
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = cswap(x[k]);
    __syncthreads();
    t5_fft256<8, ROWS>(cx, x, tw);
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = cswap(x[k]);
    combine(x);
  } else {
    float2 f[16];
    if constexpr (OP == OP_CONV_FZ) {
      gather_dif(tile, x);
      t5_stash_st<8>(cx, x);  // signal parked while the filter is transformed
      gather_dif(ftile, f);
      __syncthreads();
      t5_fft256<8, false>(cx, f, tw);
      t5_stash_ld<8>(cx, x);
      t5_stash_st<8>(cx, f);
    } else {
      gather_dit(ftile, f);  // the spectrum in the forward transform's register order
      t5_stash_st<8>(cx, f);
      gather_dif(tile, x);
      __syncthreads();
    }
    t5_fft256<8, false>(cx, x, tw);
    t5_stash_ld<8>(cx, f);
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = cswap(cmul(x[k], f[k]));
    t5_fft256<8, false>(cx, x, tw);
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = cswap(x[k]);
    combine(x);
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cx.tmem), "n"(kCols));
  if (!cx.ok && threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusMmaTimeout);

  float2 *dst = ROWS ? a.dst + (row0 + c) * N
                     : a.dst + (long long)vol * a.vol_elems + (long long)row * a.plane_pitch + x0 + c;
  const long long es = ROWS ? 1 : a.axis_stride;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    float2 v = x[k];
    if (a.scale != 1.0f) v = make_float2(v.x * a.scale, v.y * a.scale);
    const int pos = natural ? q + 16 * k + 256 * j : 2 * (q + 16 * k) + j;
    dst[(long long)pos * es] = v;
  }
}

}  // namespace convgpu
