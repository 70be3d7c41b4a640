// Uneven batches in one persistent launch fed by a device work queue.
//
// A batch of convolutions of different power-of-two sizes (each with its own filter)
// becomes one list of work items (job, pass, tile). Per job the passes are
//   0 filter x-fwd (filter -> spectrum buffer)   1 signal x-fwd (signal -> out)
//   2 filter y-fwd                               3 signal y-fwd
//   4 z: filter z-fwd, signal z-fwd, (.), z-inv (CONV_FZ)
//   5 signal y-inv                               6 signal x-inv (with scale)
// and the queue lists every item of dependency level 0 (passes 0, 1) for all jobs,
// then level 1 (2, 3), then 2 (4), 3 (5), 4 (6). A fixed grid of CTAs dequeues items
// with an atomic counter; before a tile of pass p a CTA waits until every tile of the
// passes p depends on (for the same job) is counted done. Items are dequeued in level
// order and a CTA waits only on items dequeued before its own, by CTAs that are already
// running, so the launch cannot deadlock whatever number of CTAs is resident. Waits are
// bounded: after kSpinLimit probes (fewer when a test lowers the dependency-wait limit,
// tma.cuh: dep_wait_limit) the CTA records kStatusQueueTimeout in the device status word,
// skips the tile and counts it done, so the launch always terminates.
//
// Data written by one CTA is read by others in later passes, so every global load of
// cube data here uses ld.global.cg (L2, not the incoherent L1); a CTA publishes a finished
// item with a release add at device scope after a CTA barrier, and waiters poll with
// acquire loads. A work item covers several tiles (about 256 KiB of data) to spread the
// queue and dependency overhead.
//
// This replaces the reference's host-side orchestration of a batch
// (host/src/convfpga_svm_batch.c:302-662: a 2-deep software pipeline of OpenCL tasks for
// one fixed N) with device-side scheduling across sizes; the host captures the counter
// reset and the launch in a CUDA graph and replays it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "engine_internal.h"
#include "passes.cuh"

namespace convgpu {

constexpr unsigned kStatusQueueTimeout = 2u;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kPThreads = 256;
constexpr int kPasses = 7;
constexpr int kPTwOffset = 65536;                      // twiddles after two 32 KiB tiles
constexpr int kPSmemBytes = kPTwOffset + 512 * 8;      // + a 512-entry twiddle table
constexpr int kMaxJobs = 1 << 12;                      // item encoding: 12-bit job,
constexpr int kMaxTiles = 1 << 17;                     // 3-bit pass, 17-bit tile

struct UJob {
  const float2 *sig;
  const float2 *filt;
  float2 *out;
  float2 *spec;  // this job's filter spectrum workspace (N^3)
  int n;
  float scale;
};

// Elements per thread and radices per size (256 threads; COLS = 256 / (N / E) pencils
// or rows per tile).
template <int N>
struct PShape;
template <>
struct PShape<16> {
  static constexpr int E = 4;
  using Plan = Radices<4, 4>;
};
template <>
struct PShape<32> {
  static constexpr int E = 8;
  using Plan = Radices<8, 4>;
};
template <>
struct PShape<64> {
  static constexpr int E = 8;
  using Plan = Radices<8, 8>;
};
template <>
struct PShape<128> {
  static constexpr int E = 16;
  using Plan = Radices<16, 8>;
};
template <>
struct PShape<256> {
  static constexpr int E = 16;
  using Plan = Radices<16, 16>;
};
template <>
struct PShape<512> {
  static constexpr int E = 16;
  using Plan = Radices<16, 16, 2>;
};

__host__ __device__ inline int pshape_e(int n) { return n <= 16 ? 4 : (n <= 64 ? 8 : 16); }
// Tiles per pass of a cube of size n (N*N pencils per axis, COLS per tile).
__host__ __device__ inline int ptiles(int n) { return (n * n) / (kPThreads / (n / pshape_e(n))); }
// Tiles per work item: about 256 KiB of cube data, so the per-item queue and dependency
// overhead is spread over several tiles.
__host__ __device__ inline int pgroup(int n) {
  const int g = 128 / pshape_e(n);  // a tile is 256*E complex64 = 2 KiB * E
  const int t = ptiles(n);
  return g < t ? g : t;
}
// Work items per pass (completion counters count items).
__host__ __device__ inline int pitems(int n) { return ptiles(n) / pgroup(n); }

template <int N>
__device__ __forceinline__ void pencil_addr(int axis, int pid, long long &base, long long &stride) {
  if (axis == 0) {
    base = (long long)pid * N;
    stride = 1;
  } else if (axis == 1) {
    base = (long long)(pid / N) * N * N + (pid % N);
    stride = N;
  } else {
    base = pid;
    stride = (long long)N * N;
  }
}

// One tile of one pass of a cube of size N: the COLS pencils (rows for the x pass) are
// gathered through L2 into shared memory, transformed there, and stored.
template <int N>
__device__ __noinline__ void run_tile(const UJob &j, int pass, int tile, unsigned char *smraw, const float2 *tw512) {
  using S = PShape<N>;
  constexpr int E = S::E;
  constexpr int T = N / E;
  constexpr int COLS = kPThreads / T;
  float2 *buf = reinterpret_cast<float2 *>(smraw);
  float2 *fbuf = buf + COLS * N;
  float2 *tw = reinterpret_cast<float2 *>(smraw + kPTwOffset);
  int axis, op;
  const float2 *src;
  float2 *dst;
  float scale = 1.0f;
  switch (pass) {
    case 0: axis = 0, op = OP_FWD, src = j.filt, dst = j.spec; break;
    case 1: axis = 0, op = OP_FWD, src = j.sig, dst = j.out; break;
    case 2: axis = 1, op = OP_FWD, src = j.spec, dst = j.spec; break;
    case 3: axis = 1, op = OP_FWD, src = j.out, dst = j.out; break;
    case 4: axis = 2, op = OP_CONV_FZ, src = j.out, dst = j.out; break;
    case 5: axis = 1, op = OP_INV, src = j.out, dst = j.out; break;
    default: axis = 0, op = OP_INV, src = j.out, dst = j.out, scale = j.scale; break;
  }
  for (int i = threadIdx.x; i < N; i += kPThreads) tw[i] = __ldg(tw512 + i * (512 / N));

  float2 v[E];
  if (axis == 0) {
    // Rows [tile*COLS, +COLS): padded row slots c*(N + N/16) + n + n/16.
    constexpr int PITCH = row_pitch<N>();
    const long long row0 = (long long)tile * COLS;
    for (int i = threadIdx.x; i < COLS * N; i += kPThreads) {
      const int c = i / N, n = i % N;
      buf[c * PITCH + n + (n >> 4)] = __ldcg(src + (row0 + c) * N + n);
    }
    __syncthreads();
    const int t = threadIdx.x % T, c = threadIdx.x / T;
    const RowSlot<N> sidx{c * PITCH};
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = buf[sidx(t + e * T)];
    __syncthreads();
    if (op == OP_INV) swap_all(v);
    fft_forward<N, E>(v, t, tw, buf, sidx, typename S::Plan{});
    if (op == OP_INV) swap_all(v);
    if (scale != 1.0f) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * scale, v[e].y * scale);
    }
#pragma unroll
    for (int e = 0; e < E; ++e) dst[(row0 + c) * N + t + e * T] = v[e];
    return;
  }
  // Strided pencils pid = tile*COLS + c; slot (n, c) = n*COLS + c.
  for (int i = threadIdx.x; i < COLS * N; i += kPThreads) {
    const int c = i % COLS, n = i / COLS;
    long long base, stride;
    pencil_addr<N>(axis, tile * COLS + c, base, stride);
    buf[n * COLS + c] = __ldcg(src + base + n * stride);
    if (op == OP_CONV_FZ) fbuf[n * COLS + c] = __ldcg(j.spec + base + n * stride);
  }
  __syncthreads();
  const int c = threadIdx.x % COLS, t = threadIdx.x / COLS;
  const ColSlot<COLS> sidx{c};
  if (op == OP_CONV_FZ) {
    float2 f[E];
#pragma unroll
    for (int e = 0; e < E; ++e) f[e] = fbuf[sidx(t + e * T)];
    __syncthreads();
    fft_forward<N, E>(f, t, tw, fbuf, sidx, typename S::Plan{});
#pragma unroll
    for (int e = 0; e < E; ++e) fbuf[sidx(t + e * T)] = f[e];  // own slots
  }
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = buf[sidx(t + e * T)];
  __syncthreads();
  if (op == OP_INV) swap_all(v);
  fft_forward<N, E>(v, t, tw, buf, sidx, typename S::Plan{});
  if (op == OP_CONV_FZ) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = cswap(cmul(v[e], fbuf[sidx(t + e * T)]));
    __syncthreads();
    fft_forward<N, E>(v, t, tw, buf, sidx, typename S::Plan{});
  }
  if (op != OP_FWD) swap_all(v);
  long long base, stride;
  pencil_addr<N>(axis, tile * COLS + c, base, stride);
#pragma unroll
  for (int e = 0; e < E; ++e) dst[base + (long long)(t + e * T) * stride] = v[e];
}

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(int *p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int pass_dep(int pass, int k) {
  // passes each pass waits on (-1: none)
  switch (pass) {
    case 2: return k == 0 ? 0 : -1;
    case 3: return k == 0 ? 1 : -1;
    case 4: return k == 0 ? 2 : 3;
    case 5: return k == 0 ? 4 : -1;
    case 6: return k == 0 ? 5 : -1;
    default: return -1;
  }
}

__global__ void __launch_bounds__(kPThreads, 3) k_persistent_queue(const UJob *__restrict__ jobs,
                                                                const uint32_t *__restrict__ items, int nitems,
                                                                int *counters, int *head, const float2 *tw512,
                                                                unsigned *status) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int s_item, s_ok;
  const uint32_t spin = dep_wait_limit(status, kSpinLimit);
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) return;
    const uint32_t w = items[it];
    const int job = (int)(w >> 20), pass = (int)((w >> 17) & 7u), grp = (int)(w & 0x1FFFFu);
    const UJob jb = jobs[job];
    if (threadIdx.x == 0) {
      int ok = 1;
      const int target = pitems(jb.n);
      for (int k = 0; k < 2; ++k) {
        const int d = pass_dep(pass, k);
        if (d < 0) continue;
        const int *cnt = counters + job * kPasses + d;
        bool done = false;
        for (uint32_t i = 0; i < spin; ++i) {
          if (ld_acquire(cnt) >= target) {
            done = true;
            break;
          }
          __nanosleep(64);
        }
        if (!done) {
          ok = 0;
          atomicOr(status, kStatusQueueTimeout);
        }
      }
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) {
      const int g = pgroup(jb.n);
      for (int k = 0; k < g; ++k) {
        const int tile = grp * g + k;
        switch (jb.n) {
          case 16: run_tile<16>(jb, pass, tile, smraw, tw512); break;
          case 32: run_tile<32>(jb, pass, tile, smraw, tw512); break;
          case 64: run_tile<64>(jb, pass, tile, smraw, tw512); break;
          case 128: run_tile<128>(jb, pass, tile, smraw, tw512); break;
          case 256: run_tile<256>(jb, pass, tile, smraw, tw512); break;
          case 512: run_tile<512>(jb, pass, tile, smraw, tw512); break;
          default: break;
        }
        __syncthreads();  // shared buffers are reused by the next tile
      }
    }
    // Every thread's stores happen-before the barrier; thread 0's release add then
    // publishes them at device scope together with the completed count.
    __syncthreads();
    if (threadIdx.x == 0) red_release_add(counters + job * kPasses + pass, 1);
  }
}

// ------------------------------------------------------------------ small cubes, one launch
// One convolution of a small cube (N <= 64) as a single cooperative launch in three
// dependency levels: x+y of the filter's and the signal's planes (each block holds its
// planes in shared memory between the two transforms), the fused z pass, inverse y+x;
// each level's items spread over the grid, a grid barrier between levels. A 64^3 cube is 2 MiB and stays in L2, so separate launches are bound by
// launch gaps, not by HBM. The cooperative launch makes every block resident, so the
// barrier cannot wait on a block that never runs; each wait is still bounded and one that
// gives up sets kStatusQueueTimeout.
// Barrier k (k = 1, 2) of a launch waits until its counter reaches k * gridDim.x; every
// launch uses its own counter slot, zeroed before use.
// spin: the probe limit, read by the caller at kernel start (dep_wait_limit) so that the
// read stays off the barrier's critical path.
__device__ __forceinline__ bool small_grid_barrier(unsigned *slot, unsigned target, unsigned *status, uint32_t spin) {
  __shared__ int s_ok;
  __syncthreads();  // this block's stores for the level are done
  if (threadIdx.x == 0) {
    __threadfence();  // ... and visible device-wide before the arrival
    atomicAdd(slot, 1u);
    int ok = 0;
    for (uint32_t i = 0; i < spin; ++i) {
      if ((unsigned)ld_acquire(reinterpret_cast<const int *>(slot)) >= target) {
        ok = 1;
        break;
      }
      __nanosleep(32);
    }
    if (!ok && status) atomicOr(status, kStatusQueueTimeout);
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Column n-slots of plane-column x of plane q in P consecutive N x N planes (row-major).
struct PlaneCol {
  int base, n_stride;
  __device__ __forceinline__ int operator()(int n) const { return base + n * n_stride; }
};

// x then y transform of P consecutive N x N planes (P = 256 / (N * T) for N < 64, 1 for
// N = 64, so that every round keeps all 256 threads busy), src -> dst, the planes held in
// shared memory in between: x rows through a padded exchange buffer, y columns in place
// (a warp's lanes are consecutive columns). INV: unnormalised backward transforms and
// dst scaled by `scale`.
// REAL: src holds floats (a real filter), widened to (x, 0) as they land, so the result is
// bit-identical to that of the same values given as complex.
template <int N, bool INV, bool REAL = false>
__device__ __noinline__ void xy_planes_small(const float2 *src, float2 *dst, float scale, unsigned char *smraw,
                                             const float2 *tw512) {
  using S = PShape<N>;
  constexpr int E = S::E, T = N / E;
  constexpr int LINES = kPThreads / T;                 // rows (x) or columns (y) per round
  constexpr int P = LINES >= N ? LINES / N : 1;        // planes per call
  constexpr int ROUNDS = (P * N) / LINES;
  constexpr int PITCH = row_pitch<N>();
  static_assert(P * N % LINES == 0 && P * N * N * 8 + LINES * PITCH * 8 <= kPTwOffset, "plane buffers");
  float2 *pl = reinterpret_cast<float2 *>(smraw);
  float2 *ex = pl + P * N * N;
  float2 *tw = reinterpret_cast<float2 *>(smraw + kPTwOffset);
  for (int i = threadIdx.x; i < N; i += kPThreads) tw[i] = __ldg(tw512 + i * (512 / N));
  if constexpr (REAL) {
    const float *rsrc = reinterpret_cast<const float *>(src);
    for (int i = threadIdx.x; i < P * N * N; i += kPThreads) pl[i] = make_float2(__ldcg(rsrc + i), 0.f);
  } else {
    for (int i = threadIdx.x; i < P * N * N; i += kPThreads) pl[i] = __ldcg(src + i);
  }
  __syncthreads();
  float2 v[E];
#pragma unroll 1
  for (int rd = 0; rd < ROUNDS; ++rd) {  // x: row rr of the P planes
    const int t = threadIdx.x % T, rl = threadIdx.x / T, rr = rd * LINES + rl;
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = pl[rr * N + t + e * T];
    if (INV) swap_all(v);
    fft_forward<N, E>(v, t, tw, ex, RowSlot<N>{rl * PITCH}, typename S::Plan{});
    if (INV) swap_all(v);
#pragma unroll
    for (int e = 0; e < E; ++e) pl[rr * N + t + e * T] = v[e];
    __syncthreads();  // the exchange buffer is reused by the next round
  }
#pragma unroll 1
  for (int rd = 0; rd < ROUNDS; ++rd) {  // y: column x of plane q
    const int c = threadIdx.x % LINES, t = threadIdx.x / LINES, gc = rd * LINES + c;
    const int q = gc / N, x = gc % N;
    const PlaneCol sidx{q * N * N + x, N};
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = pl[sidx(t + e * T)];
    __syncthreads();  // every column's reads done before the in-place exchange
    if (INV) swap_all(v);
    fft_forward<N, E>(v, t, tw, pl, sidx, typename S::Plan{});
    if (INV) swap_all(v);
    if (scale != 1.0f) {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * scale, v[e].y * scale);
    }
#pragma unroll
    for (int e = 0; e < E; ++e) dst[sidx(t + e * T)] = v[e];
    __syncthreads();  // this round's columns read back before the next round's exchange
  }
}

template <int N>
constexpr int small_planes_per_item() {
  return (kPThreads / (N / PShape<N>::E)) >= N ? (kPThreads / (N / PShape<N>::E)) / N : 1;
}

// Levels: 0 x+y of the filter's and the signal's planes, 1 the fused z pass (the filter's
// z transform, product, inverse z), 2 inverse y+x of the output's planes.
// real: j.filt holds N^3 floats (CONVGPU_FILTER_REAL).
template <int N>
__global__ void __launch_bounds__(kPThreads, 3) k_small_conv(UJob j, unsigned *slot, const float2 *tw512,
                                                             unsigned *status, int real) {
  extern __shared__ __align__(128) unsigned char smraw[];
  constexpr int P = small_planes_per_item<N>(), NI = N / P;  // items per cube and level
  const long long PL = (long long)P * N * N;                 // elements per item
  const uint32_t spin = dep_wait_limit(status, kSpinLimit);
  for (int w = blockIdx.x; w < 2 * NI; w += gridDim.x) {
    if (w < NI && real)
      xy_planes_small<N, false, true>(
          reinterpret_cast<const float2 *>(reinterpret_cast<const float *>(j.filt) + w * PL), j.spec + w * PL, 1.f,
          smraw, tw512);
    else if (w < NI)
      xy_planes_small<N, false>(j.filt + w * PL, j.spec + w * PL, 1.f, smraw, tw512);
    else
      xy_planes_small<N, false>(j.sig + (w - NI) * PL, j.out + (w - NI) * PL, 1.f, smraw, tw512);
    __syncthreads();
  }
  if (!small_grid_barrier(slot, gridDim.x, status, spin)) return;
  for (int w = blockIdx.x; w < ptiles(N); w += gridDim.x) {
    run_tile<N>(j, 4, w, smraw, tw512);
    __syncthreads();
  }
  if (!small_grid_barrier(slot, 2u * gridDim.x, status, spin)) return;
  for (int w = blockIdx.x; w < NI; w += gridDim.x) {
    xy_planes_small<N, true>(j.out + w * PL, j.out + w * PL, j.scale, smraw, tw512);
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host side
namespace {

struct PPlan {
  std::vector<int> sizes;
  int nitems = 0;
  int grid = 0;
  size_t spec_elems = 0;
  std::vector<size_t> spec_off;
  UJob *d_jobs = nullptr;
  uint32_t *d_items = nullptr;
  int *d_counters = nullptr;  // njobs * kPasses counters + the queue head
  float2 *d_spec = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  ~PPlan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (d_jobs) cudaFree(d_jobs);
    if (d_items) cudaFree(d_items);
    if (d_counters) cudaFree(d_counters);
    if (d_spec) cudaFree(d_spec);
  }
};

std::mutex g_pmu;
std::map<std::vector<int>, std::unique_ptr<PPlan>> g_plans;
unsigned *g_small_slots = nullptr;  // barrier counters of the small-cube launches (a ring)
unsigned long long g_small_next = 0;
std::string g_perr;

cudaError_t build_plan(PPlan &p, const float2 *tw512, unsigned *status) {
  const int nj = (int)p.sizes.size();
  // work items, level by level
  static const int kLevelPasses[5][2] = {{0, 1}, {2, 3}, {4, -1}, {5, -1}, {6, -1}};
  std::vector<uint32_t> items;
  for (const auto &lv : kLevelPasses)
    for (int jb = 0; jb < nj; ++jb)
      for (int q = 0; q < 2; ++q) {
        const int pass = lv[q];
        if (pass < 0) continue;
        const int nitem = pitems(p.sizes[jb]);
        for (int t = 0; t < nitem; ++t) items.push_back(((uint32_t)jb << 20) | ((uint32_t)pass << 17) | (uint32_t)t);
      }
  p.nitems = (int)items.size();
  p.spec_off.resize(nj);
  p.spec_elems = 0;
  for (int jb = 0; jb < nj; ++jb) {
    p.spec_off[jb] = p.spec_elems;
    p.spec_elems += (size_t)p.sizes[jb] * p.sizes[jb] * p.sizes[jb];
  }
  cudaError_t e;
  if ((e = cudaMalloc(&p.d_jobs, sizeof(UJob) * nj)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&p.d_items, sizeof(uint32_t) * items.size())) != cudaSuccess) return e;
  if ((e = cudaMalloc(&p.d_counters, sizeof(int) * (nj * kPasses + 1))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&p.d_spec, sizeof(float2) * p.spec_elems)) != cudaSuccess) return e;
  if ((e = cudaMemcpy(p.d_items, items.data(), sizeof(uint32_t) * items.size(), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_persistent_queue, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes)) !=
      cudaSuccess)
    return e;
  // The occupancy query follows the kernel's carveout preference: ask for the largest
  // shared-memory share so that it counts the CTAs the launch can actually hold.
  if ((e = cudaFuncSetAttribute(k_persistent_queue, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared)) != cudaSuccess)
    return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent_queue, kPThreads, kPSmemBytes)) !=
      cudaSuccess)
    return e;
  p.grid = std::max(1, sms * std::max(1, per_sm));

  // Graph: reset counters and queue head, then the persistent launch.
  cudaStream_t cap;
  if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess) return e;
  e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemsetAsync(p.d_counters, 0, sizeof(int) * (nj * kPasses + 1), cap);
    k_persistent_queue<<<p.grid, kPThreads, kPSmemBytes, cap>>>(p.d_jobs, p.d_items, p.nitems, p.d_counters,
                                                                p.d_counters + nj * kPasses, tw512, status);
    e = cudaStreamEndCapture(cap, &p.graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p.exec, p.graph, 0);
  cudaStreamDestroy(cap);
  return e;
}

}  // namespace

int uneven_persistent(const UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt, void *d_out,
                      bool normalize, const float2 *tw512, unsigned *status, cudaStream_t stream, std::string &err) {
  if (njobs == 0) return 0;
  if (njobs > (unsigned)kMaxJobs) {
    err = "uneven batch: more than 4096 jobs";
    return -1;
  }
  std::vector<int> key(njobs);
  for (unsigned i = 0; i < njobs; ++i) {
    key[i] = (int)jobs[i].n;
    if (pitems(key[i]) > kMaxTiles) {
      err = "uneven batch: cube too large for the work-queue encoding";
      return -1;
    }
  }
  std::lock_guard<std::mutex> lk(g_pmu);
  auto it = g_plans.find(key);
  if (it == g_plans.end()) {
    auto p = std::make_unique<PPlan>();
    p->sizes = key;
    cudaError_t e = build_plan(*p, tw512, status);
    if (e != cudaSuccess) {
      err = std::string("uneven plan: ") + cudaGetErrorString(e);
      cudaGetLastError();
      return e == cudaErrorMemoryAllocation ? -4 : -3;
    }
    it = g_plans.emplace(key, std::move(p)).first;
  }
  PPlan &p = *it->second;
  std::vector<UJob> hj(njobs);
  for (unsigned i = 0; i < njobs; ++i) {
    const int n = (int)jobs[i].n;
    hj[i].sig = (const float2 *)d_sig + jobs[i].sig_off;
    hj[i].filt = (const float2 *)d_filt + jobs[i].filt_off;
    hj[i].out = (float2 *)d_out + jobs[i].out_off;
    hj[i].spec = p.d_spec + p.spec_off[i];
    hj[i].n = n;
    hj[i].scale = normalize ? (float)(1.0 / ((double)n * n * n)) : 1.0f;
  }
  // Pageable source: the call returns once the host array is staged, so hj may go away.
  cudaError_t e = cudaMemcpyAsync(p.d_jobs, hj.data(), sizeof(UJob) * njobs, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(p.exec, stream);
  if (e != cudaSuccess) {
    err = std::string("uneven launch: ") + cudaGetErrorString(e);
    return -3;
  }
  count_launches(1);
  return 0;
}

void release_uneven_plans() {
  std::lock_guard<std::mutex> lk(g_pmu);
  g_plans.clear();
  if (g_small_slots) cudaFree(g_small_slots);
  g_small_slots = nullptr;
  g_small_next = 0;
}

// One convolution of an N^3 cube (N = 16, 32 or 64) in one cooperative launch: sig and
// filt are N^3 complex64 each (filt N^3 floats with `real`), spec is N^3 of workspace for
// the filter spectrum.
// cudaErrorNotSupported for other N or when the grid cannot be co-resident.
cudaError_t launch_small_conv(int n, const float2 *sig, const float2 *filt, float2 *out, float2 *spec, float scale,
                              bool real, const float2 *tw512, unsigned *status, cudaStream_t s) {
  constexpr int kSlots = 1024;
  if (n != 16 && n != 32 && n != 64) return cudaErrorNotSupported;
  std::lock_guard<std::mutex> lk(g_pmu);
  cudaError_t e;
  if (!g_small_slots) {
    if ((e = cudaMalloc(&g_small_slots, kSlots * sizeof(unsigned))) != cudaSuccess) return e;
    g_small_next = 0;
  }
  if (g_small_next % kSlots == 0) {  // a fresh (or wrapped) ring: every slot back to zero
    if ((e = cudaMemsetAsync(g_small_slots, 0, kSlots * sizeof(unsigned), s)) != cudaSuccess) return e;
  }
  unsigned *slot = g_small_slots + (g_small_next++ % kSlots);
  void (*kern)(UJob, unsigned *, const float2 *, unsigned *, int) =
      n == 16 ? k_small_conv<16> : (n == 32 ? k_small_conv<32> : k_small_conv<64>);
  // attribute and grid per size, set once per device: the grid is the resident blocks, at
  // most the widest level
  static int grid_of[3] = {0, 0, 0}, grid_dev = -1;
  const int ai = n == 16 ? 0 : (n == 32 ? 1 : 2);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != grid_dev) {
    grid_of[0] = grid_of[1] = grid_of[2] = 0;
    grid_dev = dev;
  }
  // No carveout preference here (unlike the work queue): its grid of at most `widest`
  // blocks needs one per SM, and the rest of the SM's memory can stay L1 for its gathers.
  if (grid_of[ai] == 0 &&
      (e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes)) != cudaSuccess)
    return e;
  if (grid_of[ai] == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPThreads, kPSmemBytes)) != cudaSuccess)
      return e;
    if (per_sm <= 0) return cudaErrorNotSupported;
    const int widest = std::max(2 * n / (n == 64 ? 1 : (n == 32 ? 2 : 4)), ptiles(n));  // items of level 0 or 1
    grid_of[ai] = std::min(sms * per_sm, widest);
  }
  const int grid = grid_of[ai];
  UJob j;
  j.sig = sig;
  j.filt = filt;
  j.out = out;
  j.spec = spec;
  j.n = n;
  j.scale = scale;
  int real_i = real ? 1 : 0;
  void *args[] = {&j, &slot, (void *)&tw512, &status, &real_i};
  return cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kPThreads), args, kPSmemBytes, s);
}

}  // namespace convgpu
