// Fused x + y pass for N = 128, 256 and 512 staged through L2: the x-transformed plane
// goes to a small ring of scratch planes instead of back to HBM, and the y transform reads
// it from there. (Written for N = 256 below; N = 128 uses 16-row / 16-column items and
// N = 512 4-row / 4-column items, see XyL2Cfg.)
// A plane then crosses HBM once (read + write) instead of twice, as in the reference's
// on-chip plane transpose (kernels/conv3D.cl:118-232, transpose + fft3db).
//
// Work items (one persistent kernel, CTAs take items in order from an atomic counter):
//   X(p, r): x transform of rows 8r..8r+7 of plane p (TMA row load; the Stockham stages
//            exchange in the tile itself through XOR-swizzled slots), written to scratch
//            slot p % R;
//   Y(p, c): y transform of columns 8c..8c+7 of plane p (one contiguous bulk copy from the
//            scratch slot, which holds a plane as N / 8 column tiles of 8 columns x N rows;
//            the tile is its own exchange buffer), written to the destination plane. (At
//            N = 512 the slot is row-major and the columns come as a TMA box.)
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
constexpr int kXyL2Threads = 128;
constexpr uint32_t kXyL2Spin = 1u << 20;

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

// Polls *p until it reaches `target`, at most `limit` probes with back-off. Thread 0 only.
__device__ __forceinline__ bool wait_count(const unsigned *p, unsigned target, uint32_t limit) {
  unsigned ns = 32;
  for (uint32_t i = 0; i < limit; ++i) {
    if (ld_acquire_u32(p) >= target) return true;
    __nanosleep(ns);
    if (ns < 512) ns <<= 1;
  }
  return false;
}

// Item w of the schedule for `np` planes with lag `lag` and `items` X (and Y) items per
// plane: plane, tile, and whether it is a Y item.
template <int ITEMS>
__device__ __forceinline__ void xyl2_item(long long w, long long np, int lag, long long &plane, int &tile,
                                          bool &is_y) {
  const long long head = (long long)lag * ITEMS;     // X only
  const long long body = (np - lag) * 2LL * ITEMS;  // X(b) then Y(b - lag)
  if (w < head) {
    plane = w / ITEMS;
    tile = (int)(w % ITEMS);
    is_y = false;
  } else if (w < head + body) {
    const long long v = w - head;
    const long long b = lag + v / (2 * ITEMS);
    const int r = (int)(v % (2 * ITEMS));
    is_y = r >= ITEMS;
    plane = is_y ? b - lag : b;
    tile = is_y ? r - ITEMS : r;
  } else {
    const long long v = w - head - body;
    plane = np - lag + v / ITEMS;
    tile = (int)(v % ITEMS);
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

// X items' exchange slot for N = 128 (16 rows of 128 per item): position n of row r at
// r*128 + (n ^ (((n >> 4) & 7) | ((r & 1) << 3))). A warp holds 4 rows x 8 threads; the
// first stage's stores (positions 16t + j) and the second stage's loads (t + 8i + 16j)
// then spread over all 32 banks (two wavefronts, the minimum for 256 bytes) instead of
// one bank pair.
struct SwzRow128 {
  int r;
  __device__ __forceinline__ int operator()(int n) const { return r * 128 + (n ^ (((n >> 4) & 7) | ((r & 1) << 3))); }
};

// Twiddles of the second stage of a 16 x 8 plan (N = 128, NS = 16, R = 8) from the table
// t[j*16 + k] = W_128^(j*k): a warp's threads read consecutive entries.
struct TwRT128 {
  const float2 *t;
};
template <int N, int NS, int R>
__device__ __forceinline__ float2 stage_tw(const TwRT128 &tw, int r, int k) {
  static_assert(N == 128 && NS == 16 && R == 8, "TwRT128 serves the second stage of a 16 x 8 plan");
  return tw.t[r * 16 + k];
}

// Y items' exchange slot for N = 512 (4 columns per item): ColSlot<4> with the position's
// low 2 bits XOR bits 4..5. A warp holds 8 consecutive pencil threads t x 4 columns; the
// first stage's stores (positions 16t + j), the later stages' loads (t + 32e) and the
// second stage's stores ((t/16)*256 + t%16 + 16j) then spread over all 32 banks (two
// wavefronts) instead of 8 lanes per bank pair.
struct ColSwz4 {
  int c;
  __device__ __forceinline__ int operator()(int n) const { return (n ^ ((n >> 4) & 3)) * 4 + c; }
};

// Twiddles of a 16 x 16 x 2 plan (N = 512): entries 0..255 hold W_512^(2*r*k) at r*16 + k
// (second stage, NS = 16, R = 16: a warp reads consecutive entries), entries 256..767 hold
// W_512^j (third stage, NS = 256, R = 2).
struct TwRT512 {
  const float2 *t;
};
template <int N, int NS, int R>
__device__ __forceinline__ float2 stage_tw(const TwRT512 &tw, int r, int k) {
  static_assert(N == 512 && ((NS == 16 && R == 16) || (NS == 256 && R == 2)), "TwRT512 serves a 16 x 16 x 2 plan");
  if constexpr (NS == 16)
    return tw.t[r * 16 + k];
  else
    return tw.t[256 + r * k];
}

// Per-size shape of the L2-staged pass. C: rows per X item = columns per Y item (each
// item is C*N = 2048 points for 128 threads of 16 points); LAG / RING: planes between a
// plane's X and Y items, and scratch planes (R > L; both chosen by timing: a shorter lag
// or gap R - L makes items wait on their dependencies, a larger ring leaves L2).
template <int N>
struct XyL2Cfg;
template <>
struct XyL2Cfg<256> {
  static constexpr int C = 8, LAG = 40, RING = 72, TWN = 256;
  static constexpr bool TILED = true;  // ring planes as column tiles (see k_xy_l2)
  using Plan = Radices<16, 16>;
  using Tw = TwRT256;
  // t[r*16 + k] = W_256^(r*k) = tw512[2*r*k] (r*k <= 225)
  static __device__ __forceinline__ float2 tw_entry(const float2 *tw512, int i) {
    return tw512[2 * ((i >> 4) * (i & 15))];
  }
  static __device__ __forceinline__ SwzRow xslot(int c) { return SwzRow{c * 256}; }
  static __device__ __forceinline__ ColSwz8 yslot(int c) { return ColSwz8{c}; }
  // C rows from the rows map, one box
  static __device__ __forceinline__ void load_x(uint32_t d, const CUtensorMap *m, int row0, uint32_t bar) {
    tma_load_2d(d, m, 0, row0, bar);
  }
};
template <>
struct XyL2Cfg<128> {
  // 16 items per plane, so the ~2,400 items the CTAs hold span ~150 planes; the ring is
  // 288 planes of 128 KiB (36 MiB), the same bytes as N = 256's. Lags of 96..192 planes
  // time the same within noise.
  static constexpr int C = 16, LAG = 160, RING = 288, TWN = 128;
  static constexpr bool TILED = true;
  using Plan = Radices<16, 8>;
  using Tw = TwRT128;
  // t[j*16 + k] = W_128^(j*k) = tw512[4*j*k] (j < 8, k < 16)
  static __device__ __forceinline__ float2 tw_entry(const float2 *tw512, int i) {
    return tw512[4 * ((i >> 4) * (i & 15))];
  }
  static __device__ __forceinline__ SwzRow128 xslot(int c) { return SwzRow128{c}; }
  static __device__ __forceinline__ ColSlot<16> yslot(int c) { return ColSlot<16>{c}; }
  static __device__ __forceinline__ void load_x(uint32_t d, const CUtensorMap *m, int row0, uint32_t bar) {
    tma_load_2d(d, m, 0, row0, bar);
  }
};
template <>
struct XyL2Cfg<512> {
  // 256 items per plane: the ~2,400 items the CTAs hold span ~10 planes. The ring is 18
  // planes of 2 MiB (36 MiB, as for the other sizes); lag / ring 8 / 16 and 14 / 24 time
  // no better.
  static constexpr int C = 4, LAG = 10, RING = 18, TWN = 768;
  // Row-major ring planes: with 4-column tiles a warp's stores of one row would touch 8
  // lines instead of 2 (measured 2% slower at 512^3).
  static constexpr bool TILED = false;
  using Plan = Radices<16, 16, 2>;
  using Tw = TwRT512;
  static __device__ __forceinline__ float2 tw_entry(const float2 *tw512, int i) {
    return i < 256 ? tw512[2 * ((i >> 4) * (i & 15))] : tw512[i - 256];
  }
  // a row's 512 slots: the low 4 bits XOR bits 4..7 (one row per warp, 32 threads)
  static __device__ __forceinline__ SwzRow xslot(int c) { return SwzRow{c * 512}; }
  static __device__ __forceinline__ ColSwz4 yslot(int c) { return ColSwz4{c}; }
  // rows map viewed as (256, 2, rows): one box lands C whole rows
  static __device__ __forceinline__ void load_x(uint32_t d, const CUtensorMap *m, int row0, uint32_t bar) {
    tma_load_3d(d, m, 0, 0, row0, bar);
  }
  // C columns of a row-major ring plane; a box is at most 256 long: rows 0..255 and
  // 256..511
  static __device__ __forceinline__ void load_y(uint32_t d, const CUtensorMap *m, int x0, int slot, uint32_t bar) {
    tma_load_3d(d, m, x0, 0, slot, bar);
    tma_load_3d(d + 256 * C * 8, m, x0, 256, slot, bar);
  }
};
// Dynamic shared memory: barrier (128 B), tile (TMA target and exchange buffer), the
// twiddle table, the next item index: 18-23 KB, so registers (64 per thread) bound the
// CTAs per SM at 8.
template <int N>
constexpr int xyl2_smem() {
  return 128 + XyL2Cfg<N>::C * N * 8 + XyL2Cfg<N>::TWN * 8 + 16;
}

// msrc: 2D map over the source rows (box {N, C}); scratch: Cfg::RING planes of N x N;
// mscr: 3D map over them (box {C, N, 1}), used where the ring planes are row-major.
// ctr: 2 * np counters (X stores done, Y reads done) and the work counter at ctr[2 * np],
// all zero at launch.
// TABLE: the planes belong to np / N cubes at unrelated addresses; plane p is plane p % N
// of cube p / N, whose rows map is rmaps[p / N] (in device memory) and whose output base
// is dsts[p / N]; msrc and dst are unused (and rmaps, dsts otherwise).
template <int N, bool INV, bool TABLE>
__global__ void __launch_bounds__(kXyL2Threads, 8) k_xy_l2(const __grid_constant__ CUtensorMap msrc,
                                                           const __grid_constant__ CUtensorMap mscr, float2 *scratch,
                                                           float2 *dst, long long np, float scale,
                                                           const float2 *tw512, unsigned *ctr, unsigned *status,
                                                           int lag_planes, const CUtensorMap *rmaps,
                                                           float2 *const *dsts) {
  using Cfg = XyL2Cfg<N>;
  constexpr int E = 16, T = N / E, C = Cfg::C, ITEMS = N / C, RING = Cfg::RING;
  static_assert(C * T == kXyL2Threads, "an item is one pencil tile per thread group");
  using Plan = typename Cfg::Plan;
  extern __shared__ __align__(128) unsigned char smraw[];
  float2 *tile = reinterpret_cast<float2 *>(smraw + 128);
  float2 *tw = tile + C * N;
  long long *next = reinterpret_cast<long long *>(tw + Cfg::TWN);
  const uint32_t bar = smem_u32(smraw);
  unsigned *xdone = ctr, *yread = ctr + np;
  unsigned long long *work = reinterpret_cast<unsigned long long *>(ctr + 2 * np);
  const int lag = (int)(np < lag_planes ? np : lag_planes);
  const long long nitems = np * 2LL * ITEMS;
  long long ahead = 0;  // thread 0: the next item's index, claimed at this item's start
  const uint32_t spin = dep_wait_limit(status, kXyL2Spin);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
    *next = (long long)atomicAdd(work, 1ull);
  }
  for (int i = threadIdx.x; i < Cfg::TWN; i += blockDim.x) tw[i] = Cfg::tw_entry(tw512, i);
  const typename Cfg::Tw twr{tw};
  __syncthreads();
  uint32_t phase = 0;
  bool ok = true;
  for (;;) {
    const long long w = *next;
    if (w >= nitems) break;
    long long p;
    int tl;
    bool is_y;
    xyl2_item<ITEMS>(w, np, lag, p, tl, is_y);
    const int slot = (int)((unsigned)p % (unsigned)RING);  // p < np < 2^31: a 32-bit remainder by a constant
    if (threadIdx.x == 0) {
      if (is_y) {
        if (!wait_count(xdone + p, ITEMS, spin)) ok = false;
        asm volatile("fence.proxy.async.global;" ::: "memory");  // generic stores -> TMA reads
        mbar_arrive_expect_tx(bar, (uint32_t)(C * N * 8));
        if constexpr (Cfg::TILED)  // the column tile is one contiguous block
          bulk_load(smem_u32(tile), scratch + (long long)slot * N * N + (long long)tl * N * C, (uint32_t)(C * N * 8),
                    bar);
        else
          Cfg::load_y(smem_u32(tile), &mscr, tl * C, slot, bar);
      } else if constexpr (TABLE) {
        const unsigned long long q = (unsigned long long)p;
        const CUtensorMap *m = rmaps + q / N;
        tensormap_acquire(m);
        mbar_arrive_expect_tx(bar, (uint32_t)(C * N * 8));
        Cfg::load_x(smem_u32(tile), m, (int)((q % N) * N + tl * C), bar);
      } else {
        mbar_arrive_expect_tx(bar, (uint32_t)(C * N * 8));
        Cfg::load_x(smem_u32(tile), &msrc, (int)(p * N + tl * C), bar);
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
      const ColSlot<C> lidx{c};  // the tile's layout: N rows of C values
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = tile[lidx(t + e * T)];
      __syncthreads();
      if (INV) swap_all(v);
      fft_forward<N, E>(v, t, twr, tile, Cfg::yslot(c), Plan{});
      if (INV) swap_all(v);
    } else {
      const int t = threadIdx.x % T, c = threadIdx.x / T;
      const auto sidx = Cfg::xslot(c);
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = tile[c * N + t + e * T];
      // A row's T threads are consecutive lanes of one warp (T divides 32) and its slots
      // are its own: the in-place exchange needs only warp barriers (timed the same as
      // CTA barriers).
      static_assert(32 % T == 0, "a row's threads must share a warp");
      __syncwarp();  // natural-order reads done before the swizzled exchange
      if (INV) swap_all(v);
      fft_forward<N, E, true>(v, t, twr, tile, sidx, Plan{});
      if (INV) swap_all(v);
    }
    if (is_y) {
      const int c = threadIdx.x % C, t = threadIdx.x / C;
      float2 *o;
      if constexpr (TABLE) {
        const unsigned long long q = (unsigned long long)p;
        o = dsts[q / N] + (long long)(q % N) * N * N + tl * C + c;
      } else {
        o = dst + p * N * N + tl * C + c;
      }
      if (scale != 1.0f) {  // the same value for every item: a uniform branch
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * scale, v[e].y * scale);
      }
#pragma unroll
      for (int e = 0; e < E; ++e) o[(long long)(t + e * T) * N] = v[e];
    } else {
      const int t = threadIdx.x % T, c = threadIdx.x / T;
      if (p >= RING) {  // the slot's previous plane must have been read
        if (threadIdx.x == 0 && !wait_count(yread + (p - RING), ITEMS, spin)) ok = false;
        __syncthreads();
      }
      if constexpr (Cfg::TILED) {
        // column tile x / C of the slot holds its C columns of every row contiguously
        float2 *o = scratch + (long long)slot * N * N + (tl * C + c) * C;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int x = t + e * T;
          o[(x / C) * (N * C) + (x % C)] = v[e];
        }
      } else {
        float2 *o = scratch + (long long)slot * N * N + (long long)(tl * C + c) * N + t;
#pragma unroll
        for (int e = 0; e < E; ++e) o[e * T] = v[e];
      }
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
