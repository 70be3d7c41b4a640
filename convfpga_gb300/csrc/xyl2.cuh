// Fused x + y pass for N = 256 staged through L2: the x-transformed plane goes to a small
// ring of scratch planes instead of back to HBM, and the y transform reads it from there.
// A plane then crosses HBM once (read + write) instead of twice, as in the reference's
// on-chip plane transpose (kernels/conv3D.cl:118-232, transpose + fft3db).
//
// Work items (one persistent kernel, CTAs take items in order from an atomic counter):
//   X(p, r): x transform of rows 8r..8r+7 of plane p (TMA row load; the Stockham stages
//            exchange in the tile itself through XOR-swizzled slots), written to scratch
//            slot p % R;
//   Y(p, c): y transform of columns 8c..8c+7 of plane p (TMA box from the scratch slot;
//            the tile is its own exchange buffer), written to the destination plane.
// Order: X items of plane b and Y items of plane b - L, for b = 0, 1, ... (lag L planes).
// Dependencies:
//   Y(p, *) loads slot p % R only after all 32 X(p, *) items have stored (per-plane
//           counter, release add / acquire poll, then fence.proxy.async so the TMA read
//           sees the generic stores);
//   X(p, *) with p >= R stores only after all 32 Y(p - R, *) items have read the slot.
// Signals: an X item's "stored" signal is a release add posted by thread 32 as soon as a
// barrier has ordered every thread's stores before it (planes complete as early as
// possible: Y items wait on them); a Y item's "slot read" signal is a relaxed add
// right after its load landed (the data already sits in shared memory, so no later write
// to the slot can reach it). Thread 0 claims the next item's index when the current item's
// tile has landed and publishes it at the end of the item, so the atomic's latency hides
// behind the transform.
// A CTA holds its current item and the index of the next one; every item it waits on
// comes earlier in the order (R > L) and its signal is posted as soon as that item ends.
// So the oldest unfinished item is always some CTA's current item and its dependencies
// are done: no deadlock, whatever the number of resident CTAs. Every wait is bounded;
// one that gives up sets kStatusQueueWait in the device status word and the CTA carries
// on (the output is then wrong and the call reports an error).
//
// Scratch: R = 72 planes of 512 KiB (36 MiB), rewritten every R planes, so its lines stay in
// the 129 MB L2 between the X store and the Y load and are rarely written back to HBM. The
// lag (40 planes) and the ring were chosen by timing: a shorter lag or a smaller gap R - L
// makes items wait on their dependencies, a larger ring no longer stays in L2.
#pragma once

#include "passes.cuh"

namespace convgpu {

constexpr unsigned kStatusQueueWait = 16u;  // a dependency wait of the L2-staged pass gave up
constexpr int kXyL2Lag = 40;                // L: planes between a plane's X and Y items
constexpr int kXyL2Ring = 72;               // R: scratch planes (R > L)
constexpr int kXyL2Cols = 8;                // rows per X item, columns per Y item
constexpr int kXyL2Threads = kXyL2Cols * 16;
constexpr int kXyL2Items = 256 / kXyL2Cols;  // X (and Y) items per plane
constexpr uint32_t kXyL2Spin = 1u << 20;

// Dynamic shared memory: barrier (128 B), tile (TMA target and exchange buffer), 256
// twiddles, the next item index: about 18.5 KB, so registers (64 per thread) bound the
// CTAs per SM at 8.
constexpr int kXyL2Smem = 128 + kXyL2Cols * 256 * 8 + 256 * 8 + 16;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_relaxed_add_u32(unsigned *p, unsigned v) {
  asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Polls *p until it reaches `target` (bounded, with back-off). Thread 0 only.
__device__ __forceinline__ bool wait_count(const unsigned *p, unsigned target) {
  unsigned ns = 32;
  for (uint32_t i = 0; i < kXyL2Spin; ++i) {
    if (ld_acquire_u32(p) >= target) return true;
    __nanosleep(ns);
    if (ns < 512) ns <<= 1;
  }
  return false;
}

// Item w of the schedule for `np` planes with lag `lag`: plane, tile, and whether it is a
// Y item.
__device__ __forceinline__ void xyl2_item(long long w, long long np, int lag, long long &plane, int &tile,
                                          bool &is_y) {
  const long long head = (long long)lag * kXyL2Items;     // X only
  const long long body = (np - lag) * 2LL * kXyL2Items;  // X(b) then Y(b - lag)
  if (w < head) {
    plane = w / kXyL2Items;
    tile = (int)(w % kXyL2Items);
    is_y = false;
  } else if (w < head + body) {
    const long long v = w - head;
    const long long b = lag + v / (2 * kXyL2Items);
    const int r = (int)(v % (2 * kXyL2Items));
    is_y = r >= kXyL2Items;
    plane = is_y ? b - lag : b;
    tile = is_y ? r - kXyL2Items : r;
  } else {
    const long long v = w - head - body;
    plane = np - lag + v / kXyL2Items;
    tile = (int)(v % kXyL2Items);
    is_y = true;
  }
}

// Exchange slot of the Y items' in-place transform: ColSlot<8> with the position's lowest
// bit flipped in odd 16-blocks. A warp holds 4 pencil threads t (t = threadIdx.x / 8); the
// first stage's stores (positions 16t + r) then fill both halves of the banks instead of
// putting all four t in the same 16 banks (2 wavefronts per store instead of 4), and the
// second stage's reads (positions t + 16e) stay two wavefronts.
struct ColSwz8 {
  int c;
  __device__ __forceinline__ int operator()(int n) const { return (n ^ ((n >> 4) & 1)) * 8 + c; }
};

// msrc: 2D map over the source rows (box {256, 8}); mscr: 3D map over the `ring` scratch
// planes (box {8, 256, 1}). ctr: 2 * np counters (X stores done, Y reads done) and the
// work counter at ctr[2 * np], all zero at launch.
// Table mode (rmaps non-null): the planes belong to np / 256 cubes at unrelated
// addresses; plane p is plane p % 256 of cube p / 256, whose rows map is rmaps[p / 256]
// (in device memory) and whose output base is dsts[p / 256]; msrc and dst are unused.
template <bool INV>
__global__ void __launch_bounds__(kXyL2Threads, 8) k_xy_l2(const __grid_constant__ CUtensorMap msrc,
                                                           const __grid_constant__ CUtensorMap mscr, float2 *scratch,
                                                           float2 *dst, long long np, float scale,
                                                           const float2 *tw512, unsigned *ctr, unsigned *status,
                                                           int lag_planes, int ring, const CUtensorMap *rmaps,
                                                           float2 *const *dsts) {
  constexpr int N = 256, E = 16, T = N / E, C = kXyL2Cols;
  using Plan = Radices<16, 16>;
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tile = reinterpret_cast<float2 *>(smraw + 128);
  float2 *tw = tile + C * N;
  long long *next = reinterpret_cast<long long *>(tw + N);
  const uint32_t bar = smem_u32(smraw);
  unsigned *xdone = ctr, *yread = ctr + np;
  unsigned long long *work = reinterpret_cast<unsigned long long *>(ctr + 2 * np);
  const int lag = (int)(np < lag_planes ? np : lag_planes);
  const long long nitems = np * 2LL * kXyL2Items;
  long long ahead = 0;  // thread 0: the next item's index, claimed at this item's start
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
    *next = (long long)atomicAdd(work, 1ull);
  }
  // t[r*16 + k] = W_256^(r*k) = tw512[2*r*k] (r*k <= 225)
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = tw512[2 * ((i >> 4) * (i & 15))];
  const TwRT256 twr{tw};
  __syncthreads();
  uint32_t phase = 0;
  bool ok = true;
  for (;;) {
    const long long w = *next;
    if (w >= nitems) break;
    long long p;
    int tl;
    bool is_y;
    xyl2_item(w, np, lag, p, tl, is_y);
    const int slot = (int)(p % ring);
    if (threadIdx.x == 0) {
      if (is_y) {
        if (!wait_count(xdone + p, kXyL2Items)) ok = false;
        asm volatile("fence.proxy.async.global;" ::: "memory");  // generic stores -> TMA reads
        mbar_arrive_expect_tx(bar, (uint32_t)(C * N * 8));
        tma_load_3d(smem_u32(tile), &mscr, tl * C, 0, slot, bar);
      } else if (rmaps) {
        const CUtensorMap *m = rmaps + (p >> 8);
        tensormap_acquire(m);
        mbar_arrive_expect_tx(bar, (uint32_t)(C * N * 8));
        tma_load_2d(smem_u32(tile), m, 0, (int)((p & 255) * N + tl * C), bar);
      } else {
        mbar_arrive_expect_tx(bar, (uint32_t)(C * N * 8));
        tma_load_2d(smem_u32(tile), &msrc, 0, (int)(p * N + tl * C), bar);
      }
    }
    const bool landed = __syncthreads_and(mbar_wait_bounded(bar, phase) ? 1 : 0);
    phase ^= 1u;
    if (threadIdx.x == 0) {
      if (!landed) ok = false;
      if (is_y) red_relaxed_add_u32(yread + p, 1u);  // slot read: it may be rewritten
      ahead = (long long)atomicAdd(work, 1ull);       // published at the end of this item
    }
    float2 v[E];
    if (is_y) {
      const int c = threadIdx.x % C, t = threadIdx.x / C;
      const ColSlot<C> lidx{c};  // the TMA box's layout
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = tile[lidx(t + e * T)];
      __syncthreads();
      if (INV) swap_all(v);
      fft_forward<N, E>(v, t, twr, tile, ColSwz8{c}, Plan{});
      if (INV) swap_all(v);
    } else {
      const int t = threadIdx.x % T, c = threadIdx.x / T;
      const SwzRow sidx{c * N};
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = tile[c * N + t + e * T];
      __syncthreads();  // natural-order reads done before the swizzled exchange
      if (INV) swap_all(v);
      fft_forward<N, E>(v, t, twr, tile, sidx, Plan{});
      if (INV) swap_all(v);
    }
    if (is_y) {
      const int c = threadIdx.x % C, t = threadIdx.x / C;
      float2 *o = (rmaps ? dsts[p >> 8] + (p & 255) * N * N : dst + p * N * N) + tl * C + c;
#pragma unroll
      for (int e = 0; e < E; ++e) o[(long long)(t + e * T) * N] = make_float2(v[e].x * scale, v[e].y * scale);
    } else {
      const int t = threadIdx.x % T, c = threadIdx.x / T;
      if (p >= ring) {  // the slot's previous plane must have been read
        if (threadIdx.x == 0 && !wait_count(yread + (p - ring), kXyL2Items)) ok = false;
        __syncthreads();
      }
      float2 *o = scratch + (long long)slot * N * N + (long long)(tl * C + c) * N + t;
#pragma unroll
      for (int e = 0; e < E; ++e) o[e * T] = v[e];
      __syncthreads();  // every thread's stores issued
      // The barrier orders every thread's stores before this release (cumulativity); a
      // thread of another warp than the one issuing the loads signals it.
      if (threadIdx.x == 32) red_release_add_u32(xdone + p, 1u);
    }
    if (threadIdx.x == 0) *next = ahead;  // the atomic's latency hid behind the transform
    // this item's generic shared-memory writes before the next item's TMA write
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();  // *next published, tile free
  }
  if (threadIdx.x == 0 && !ok && status) atomicOr(status, kStatusQueueWait);
}

}  // namespace convgpu
