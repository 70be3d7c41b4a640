// Fused x + y pass of the tensor-core split path for N = 256, staged through L2: the same
// schedule, scratch ring and dependency protocol as the FP32 pass k_xy_l2 (xyl2.cuh), with
// every 256-point transform run by t5_fft256 (tc05.cuh: two 16-point DFT stages as
// split-TF32 matmuls on tcgen05, FP32 twiddles on the CUDA cores).
//
// Items (8 pencils each, one M = 128 tile per tensor-core stage):
//   X(p, r): rows 8r..8r+7 of plane p (TMA box {256, 8}), row mapping of t5_fft256
//            (thread m = 16 a + b: row a, positions b + 16 i), stored to scratch slot p % R;
//   Y(p, c): columns 8c..8c+7 of the scratch slot (one 16 KB bulk copy of the slot's
//            column tile c), column mapping
//            (thread m = 8 a + b: column b, positions a + 16 i), stored to the output plane.
// Dependencies, signals, item claiming and the no-deadlock argument are those of k_xy_l2.
//
// Shared memory (1024-byte aligned): A hi (the TMA tile lands here and is read into
// registers before the first A row is written), A lo, B hi / lo and W256 (the constant
// block, one bulk copy at kernel start), barriers, the next item's index. TMEM: 32 columns
// for the whole kernel. Ordering inside an item follows k_tc05_256; between items, a proxy
// fence and a CTA barrier order the item's generic shared-memory writes and completed MMA
// reads before the next TMA write into the tile.
#pragma once

#include "tc05.cuh"
#include "xyl2.cuh"

namespace convgpu {

constexpr int kXyTcThreads = 128;
constexpr int kXyTcOffBar = T5Geom<8>::kOffBar;          // tile, A lo, B, W256 before it
constexpr int kXyTcSmem = kXyTcOffBar + 128 + 1024;      // + 1 KB so the base can be aligned
constexpr int kXyTcMinBlocks = 5;

template <bool INV>
__global__ void __launch_bounds__(kXyTcThreads, kXyTcMinBlocks)
    k_xy_l2_tc(const __grid_constant__ CUtensorMap msrc, float2 *scratch,
               float2 *dst, long long np, float scale, const float2 *tw512, unsigned *ctr, unsigned *status,
               int lag_planes) {
  constexpr int N = 256, C = 8, ITEMS = N / C, TILE = N * C, RING = XyL2Cfg<256>::RING;
  using G = T5Geom<8>;
  static_assert(TILE * 8 == G::kABytes, "a tile is one A operand part");
  constexpr uint32_t kCols = 32;
  extern __shared__ unsigned char smdyn[];
  // the swizzle atoms want a 1024-byte aligned base: align inside the allocation
  unsigned char *smraw = smdyn + ((1024u - (smem_u32(smdyn) & 1023u)) & 1023u);
  float2 *tile = reinterpret_cast<float2 *>(smraw);
  const float2 *tw = reinterpret_cast<const float2 *>(smraw + G::kOffTw);
  const uint32_t tbar = smem_u32(smraw + kXyTcOffBar), mbar = tbar + 8;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smraw + kXyTcOffBar + 16);
  long long *next = reinterpret_cast<long long *>(smraw + kXyTcOffBar + 32);
  unsigned *xdone = ctr, *yread = ctr + np;
  unsigned long long *work = reinterpret_cast<unsigned long long *>(ctr + 2 * np);
  const int lag = (int)(np < lag_planes ? np : lag_planes);
  const long long nitems = np * 2LL * ITEMS;
  const uint32_t spin = dep_wait_limit(status, kXyL2Spin);
  long long ahead = 0;

  if (threadIdx.x == 0) {
    mbar_init(tbar, 1);
    mbar_init(mbar, 1);
    mbar_fence_init();
    mbar_arrive_expect_tx(tbar, (uint32_t)kT5ConstBytes);
    bulk_load(smem_u32(smraw + G::kOffB), reinterpret_cast<const unsigned char *>(tw512) + kT5ConstOffset,
              (uint32_t)kT5ConstBytes, tbar);
    *next = (long long)atomicAdd(work, 1ull);
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
  bool ok = true;
  // the constant block; a CTA whose copy does not land does no items (its copy may still
  // be in flight, so it waits once more before leaving)
  const bool consts = __syncthreads_and(mbar_wait_bounded(tbar, 0) ? 1 : 0);
  uint32_t phase = 1;
  if (!consts) {
    mbar_wait_bounded(tbar, 0);
    ok = false;
  }

  const int m = threadIdx.x;
  while (consts) {
    const long long w = *next;
    if (w >= nitems) break;
    long long p;
    int tl;
    bool is_y;
    xyl2_item<ITEMS>(w, np, lag, p, tl, is_y);
    const int slot = (int)((unsigned)p % (unsigned)RING);  // p < np < 2^31
    if (threadIdx.x == 0) {
      if (is_y) {
        if (!wait_count(xdone + p, ITEMS, spin)) ok = false;
        asm volatile("fence.proxy.async.global;" ::: "memory");  // generic stores -> TMA reads
        mbar_arrive_expect_tx(tbar, (uint32_t)(TILE * 8));
        bulk_load(smem_u32(tile), scratch + (long long)slot * N * N + (long long)tl * N * C, (uint32_t)(TILE * 8),
                  tbar);  // column tile tl of the slot: one contiguous block
      } else {
        mbar_arrive_expect_tx(tbar, (uint32_t)(TILE * 8));
        tma_load_2d(smem_u32(tile), &msrc, 0, (int)(p * N + tl * C), tbar);
      }
    }
    const bool landed = __syncthreads_and(mbar_wait_bounded(tbar, phase) ? 1 : 0);
    phase ^= 1u;
    if (!landed) {  // the copy may still be in flight: let it land, then stop taking items
      if (threadIdx.x == 0) ok = false;
      mbar_wait_bounded(tbar, phase ^ 1u);
      break;
    }
    if (threadIdx.x == 0) {
      if (is_y) red_relaxed_add_u32(yread + p, 1u);  // slot read: it may be rewritten
      ahead = (long long)atomicAdd(work, 1ull);       // published at the end of this item
    }
    float2 v[16];
    const int ia = is_y ? (m >> 3) : (m >> 4), ib = is_y ? (m & 7) : (m & 15);
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) {
      const float2 e = is_y ? tile[(ia + 16 * n2) * C + ib] : tile[ia * N + ib + 16 * n2];
      v[n2] = INV ? cswap(e) : e;
    }
    __syncthreads();  // tile consumed before A (which aliases it) is written
    if (is_y)
      t5_fft256<8, false>(cx, v, tw);
    else
      t5_fft256<8, true>(cx, v, tw);
    if (INV) {
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = cswap(v[k]);
    }
    if (is_y) {
      float2 *o = dst + p * N * N + tl * C + ib;
      if (scale != 1.0f) {
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = make_float2(v[k].x * scale, v[k].y * scale);
      }
#pragma unroll
      for (int k = 0; k < 16; ++k) o[(long long)(ia + 16 * k) * N] = v[k];
    } else {
      if (p >= RING) {  // the slot's previous plane must have been read
        if (threadIdx.x == 0 && !wait_count(yread + (p - RING), ITEMS, spin)) ok = false;
        __syncthreads();
      }
      // the slot holds the plane as column tiles of C columns x N rows (as k_xy_l2)
      float2 *o = scratch + (long long)slot * N * N + (tl * C + ia) * C;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int x = ib + 16 * k;
        o[(x / C) * (N * C) + (x % C)] = v[k];
      }
      __syncthreads();  // every thread's stores issued
      if (threadIdx.x == 32) red_release_add_u32(xdone + p, 1u);
    }
    if (threadIdx.x == 0) *next = ahead;
    // this item's generic shared-memory writes before the next item's TMA write
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    t5_fence_before();
    __syncthreads();  // *next published, tile and TMEM free
    t5_fence_after();
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cx.tmem), "n"(kCols));
  if (threadIdx.x == 0 && status) {
    if (!ok) atomicOr(status, kStatusQueueWait);
    if (!cx.ok) atomicOr(status, kStatusMmaTimeout);
  }
}

}  // namespace convgpu
