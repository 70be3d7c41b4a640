// Runtime of the GB300 FFT convolution library: device selection, streams, workspace,
// the pass sequence of one convolution, and the pipelined host-buffer path.
//
// Reference behaviour mirrored here (host/src/*.c of pc2/ConvFPGA):
//  - fpga_initialize return codes 0 / -1..-5 (host/src/fpga_init.c:48-56, 57-121);
//  - conv entry points return fpga_t{valid=0} on NULL pointers or a non-power-of-two N
//    (host/src/convfpga.c:36-37) and never exit() on runtime errors (the reference's
//    checkError does: host/src/opencl_utils.c:421-439);
//  - outputs are unnormalised (x N^3) unless the caller asks for 1/N^3;
//  - fpga_t times in milliseconds, taken from device events like the reference's
//    OpenCL event profiling (host/src/convfpga.c:83-85, 169-172, 276-279, 360-375).
//
// Pass sequence of one convolution (per signal, 5 HBM passes; the reference streams
// 3 phases with a DDR transpose inside each 3D FFT, host/src/convfpga.c:74-363):
//   filter (shared):      x-fwd -> y-fwd -> z-fwd              (filter spectrum in workspace)
//   filter (per signal, or shared with one or two signals):
//                         x-fwd -> y-fwd                       (z done inside CONV_FZ)
//   signal:               x-fwd -> y-fwd -> z[fwd, (.)F, inv] -> y-inv -> x-inv(scale)
// With the fused pass in the plan (N = 128, 256, 512), x-fwd -> y-fwd and y-inv -> x-inv
// each run as one L2-staged launch. One cube of N <= 64 runs all of it in one cooperative
// launch (persistent.cu: launch_small_conv).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "abi_bridge.h"
#include "engine_internal.h"
#include "passes.cuh"

namespace convgpu {

// Flag bits shared with include/convgpu.h.
constexpr unsigned kFlagNormalize = 1u << 0;
constexpr unsigned kFlagPerSignalFilter = 1u << 1;
constexpr unsigned kFlagFilterIsSpectrum = 1u << 2;
constexpr unsigned kFlagTensorSplit = 1u << 3;
constexpr unsigned kFlagTensorBf16x3 = 1u << 4;
constexpr unsigned kFlagUnevenPerJob = 1u << 5;
constexpr unsigned kFlagUnevenQueue = 1u << 6;
constexpr unsigned kFlagHostSlabs = 1u << 7;
constexpr unsigned kFlagFilterCached = 1u << 8;
constexpr unsigned kFlagFilterReal = 1u << 9;

constexpr int kErrInval = -1;
constexpr int kErrNotInit = -2;
constexpr int kErrCuda = -3;
constexpr int kErrNoMem = -4;
constexpr int kErrUnsupported = -5;

static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};

void count_launches(unsigned long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

static void set_err(const std::string &s) { g_err = s; }
void record_error(const char *msg) { g_err = msg ? msg : ""; }
static int cuda_fail(cudaError_t e, const char *what) {
  set_err(std::string(what) + ": " + cudaGetErrorString(e));
  return (e == cudaErrorMemoryAllocation) ? kErrNoMem : kErrCuda;
}

static bool valid_n(unsigned n) { return n >= 16 && n <= 512 && (n & (n - 1)) == 0; }

// Allocations still to fail on purpose (testing hook, fail_next_allocations).
static std::atomic<unsigned> g_fail_allocs{0};

void fail_next_allocations(unsigned count) { g_fail_allocs.store(count); }

// Grow-only device buffer. Growing synchronises the device first, so work still in
// flight on the old block never sees it freed.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t b) {
    if (b <= bytes) return cudaSuccess;
    if (p) {
      cudaDeviceSynchronize();
      cudaFree(p);
      p = nullptr;
      bytes = 0;
    }
    for (unsigned f = g_fail_allocs.load(); f > 0;)
      if (g_fail_allocs.compare_exchange_weak(f, f - 1)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct Engine {
  std::recursive_mutex mu;
  bool init = false;
  int device = 0;
  bool use_svm = false;
  int pageable_access = 0;
  int sm_count = 0;
  cudaStream_t sc = nullptr, sh2d = nullptr, sd2h = nullptr;
  float2 *tw512 = nullptr;
  DevBuf ws;           // device API workspace (filter spectra)
  DevBuf hfilt;        // host API: filter input / spectrum
  DevBuf hreal[4];     // host API, real filters: float staging (3 chunk buffers + shared filter)
  // Key of the shared-filter spectrum held in hfilt (host API, CONVGPU_FILTER_CACHED):
  // the caller's filter pointer, N and path; valid only until hfilt is used otherwise.
  struct {
    const void *ptr = nullptr;
    unsigned n = 0;
    int tc = -1;
    bool valid = false;
  } hkey;
  DevBuf hio[3];       // host API: signal chunk buffers
  DevBuf hfio[3];      // host API: per-signal filter chunk buffers
  std::string plan_path;
  // End of the last call's work (CallOrder): the stream it was enqueued on and an event.
  cudaEvent_t last_done = nullptr;
  cudaStream_t last_stream = nullptr;
  bool last_valid = false;
};
static Engine g;

// ------------------------------------------------------------------ cross-stream order
// The workspace, the fused x+y pass's scratch ring and counters, and the uneven batch's
// cached plans are shared by every call, so calls enqueued on different streams are
// ordered on the GPU: every call records its end on its own stream (while that stream is
// certainly alive: a caller may destroy a stream after its last call), and a call on
// another stream than the previous one first makes that event a dependency of its stream.
// A stream that is being captured into a graph is left alone (the graph cannot wait on
// work outside it): a graph that contains a call must not run while another call is in
// flight.
static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return st != cudaStreamCaptureStatusNone;
}

struct CallOrder {
  cudaStream_t s;
  bool active;
  explicit CallOrder(cudaStream_t st) : s(st), active(!capturing(st)) {
    if (active && g.last_valid && g.last_stream != s) cudaStreamWaitEvent(s, g.last_done, 0);
  }
  // Records even when the call failed partway: the event then follows what was enqueued.
  ~CallOrder() {
    if (!active) return;
    if (!g.last_done && cudaEventCreateWithFlags(&g.last_done, cudaEventDisableTiming) != cudaSuccess) {
      g.last_done = nullptr;
      cudaGetLastError();
      return;
    }
    if (cudaEventRecord(g.last_done, s) == cudaSuccess) {
      g.last_stream = s;
      g.last_valid = true;
    } else {
      cudaGetLastError();
    }
  }
};

static void load_plan_cache(const std::string &path);

static cudaError_t upload_twiddles(float2 **dst) {
  std::vector<float2> h(512);
  const double two_pi = 6.283185307179586476925286766559;
  for (int j = 0; j < 512; ++j) {
    const double a = -two_pi * (double)j / 512.0;
    h[j] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  cudaError_t e = cudaMalloc(dst, kTwiddleBufBytes);
  if (e != cudaSuccess) return e;
  e = cudaMemcpy(*dst, h.data(), 512 * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  return tc05_init_consts(*dst, 0);
}

static void teardown_locked() {
  if (!g.init) return;
  cudaSetDevice(g.device);
  cudaDeviceSynchronize();
  release_uneven_plans();
  release_grouped_plans();
  release_xy_l2();
  g.ws.release();
  g.hfilt.release();
  for (auto &b : g.hreal) b.release();
  g.hkey.valid = false;
  for (auto &b : g.hio) b.release();
  for (auto &b : g.hfio) b.release();
  if (g.tw512) cudaFree(g.tw512);
  g.tw512 = nullptr;
  if (g.sc) cudaStreamDestroy(g.sc);
  if (g.sh2d) cudaStreamDestroy(g.sh2d);
  if (g.sd2h) cudaStreamDestroy(g.sd2h);
  g.sc = g.sh2d = g.sd2h = nullptr;
  if (g.last_done) cudaEventDestroy(g.last_done);
  g.last_done = nullptr;
  g.last_valid = false;
  g.init = false;
}

// Sets up the runtime on `dev`. Returns 0 or a negative fpga_initialize-style code.
static int setup_locked(int dev, bool use_svm) {
  if (g.init && g.device == dev) {
    g.use_svm = g.use_svm || use_svm;
    return 0;
  }
  teardown_locked();
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) {
    set_err(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return -3;
  }
  cudaDeviceGetAttribute(&g.pageable_access, cudaDevAttrPageableMemoryAccess, dev);
  cudaDeviceGetAttribute(&g.sm_count, cudaDevAttrMultiProcessorCount, dev);
  int can_map = 0;
  cudaDeviceGetAttribute(&can_map, cudaDevAttrCanMapHostMemory, dev);
  if (use_svm && !can_map && !g.pageable_access) {
    set_err("device cannot address host memory");
    return -5;
  }
  // The kernels are built for sm_103a only; a device they cannot load on is the
  // analogue of a bitstream that fails to load (-4).
  e = probe_kernel_image();
  if (e != cudaSuccess) {
    set_err(std::string("kernel image not loadable on this device: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return -4;
  }
  if ((e = cudaStreamCreateWithFlags(&g.sc, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&g.sh2d, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&g.sd2h, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = upload_twiddles(&g.tw512)) != cudaSuccess) {
    set_err(std::string("runtime setup: ") + cudaGetErrorString(e));
    g.init = true;  // let teardown release what was created
    teardown_locked();
    return -4;
  }
  const char *no_tma = std::getenv("CONVGPU_DISABLE_TMA");
  set_tma_enabled(!(no_tma && no_tma[0] == '1'));
  g.device = dev;
  g.use_svm = use_svm;
  g.init = true;
  return 0;
}

// Lazily initialises on the caller's current device (device / extension entry points).
static int ensure_init_locked() {
  if (g.init) return cudaSetDevice(g.device) == cudaSuccess ? 0 : kErrCuda;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    set_err("no CUDA device");
    return kErrNotInit;
  }
  return setup_locked(dev, false) == 0 ? 0 : kErrNotInit;
}

// ------------------------------------------------------------------ pass timing
// Optional per-pass timing: events around every pass on its own stream, summed per
// (axis, op) slot with the pass's algorithmic bytes (one read + one write of every
// cube, plus one read of the filter operand for the fused z pass).
constexpr int kSlots = 14;  // slot = axis * 4 + op; 12 / 13: fused x+y forward / inverse
static const char *const kSlotNames[kSlots] = {"x-fwd", "x-inv", "x-conv", "x-conv_fz", "y-fwd", "y-inv", "y-conv",
                                               "y-conv_fz", "z-fwd", "z-inv", "z-conv", "z-conv_fz", "xy-fwd", "xy-inv"};

// A named NVTX range on the calling thread around each pass's enqueue and each entry
// point, so that Nsight Systems / Compute group the launches by pass; without a tool
// attached each push / pop is a few nanoseconds.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

struct PassRec {
  int slot;
  double bytes;
  cudaEvent_t a, b;
};
static bool g_prof = false;
static std::vector<PassRec> g_prof_recs;

static cudaError_t pass(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                        long long filt_vol, int nvol, float scale, cudaStream_t s, int tc) {
  NvtxRange nv(kSlotNames[axis * 4 + op]);
  PassRec r{axis * 4 + op, 0.0, nullptr, nullptr};
  if (g_prof) {
    const double vol = (double)n * n * n * 8.0 * nvol;
    r.bytes = 2.0 * vol + ((op == OP_CONV || op == OP_CONV_FZ) ? vol : 0.0);
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, s);
  }
  cudaError_t e = tc ? launch_axis_pass_tc(n, axis, op, src, dst, filt, filt_vol, nvol, scale, g.tw512, s, tc - 1)
                     : launch_axis_pass(n, axis, op, src, dst, filt, filt_vol, nvol, scale, g.tw512, s);
  if (g_prof) {
    cudaEventRecord(r.b, s);
    g_prof_recs.push_back(r);
  }
  return e;
}

// True when the tensor-core path has kernels of its own for size n (N = 256; N = 512 in
// TF32x3); elsewhere it runs the FP32 kernels, the fused x+y pass included, and its
// results equal the FP32 path's.
static bool tc_kernels(int n, int tc) {
  return tc != 0 && (n == 256 || (n == 512 && tc - 1 == kTcTf32x3));
}

// Fused x + y pass: for the FP32 path plan kind kKindXy (1 L2-staged (N = 128, 256, 512),
// 2 8-CTA clusters (N = 256)); for the tensor-core path (tc != 0) the L2-staged pass on
// tcgen05 (N = 256). Returns cudaErrorNotSupported when it cannot run, in which case the
// caller runs the x and y passes separately.
static cudaError_t pass_xy(int n, const float2 *src, float2 *dst, int nvol, bool inverse, float scale,
                           cudaStream_t s, int tc = 0) {
  NvtxRange nv(kSlotNames[12 + (inverse ? 1 : 0)]);
  PassRec r{12 + (inverse ? 1 : 0), 0.0, nullptr, nullptr};
  if (g_prof) {
    r.bytes = 4.0 * (double)n * n * n * 8.0 * nvol;  // the x and y passes it replaces
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, s);
  }
  const bool tc_fused = tc_kernels(n, tc);  // else the FP32 pass, also for the tensor-core flag
  cudaError_t e = tc_fused ? launch_xy_l2_tc_pass(n, src, dst, nvol * n, inverse, scale, g.tw512, s)
                           : launch_xy_pass(n, src, dst, nvol * n, inverse, scale, g.tw512, s,
                                            get_pass_variant(n, kKindXy));
  if (g_prof) {
    cudaEventRecord(r.b, s);
    if (e == cudaSuccess) {
      g_prof_recs.push_back(r);
    } else {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
  }
  // the L2-staged pass is two launches: counter clear + pass
  if (e == cudaSuccess) count_launches((tc_fused || get_pass_variant(n, kKindXy) == 1) ? 2 : 1);
  return e;
}

static bool use_xy(int n, int tc) {
  if (tc_kernels(n, tc))  // the tcgen05 split-TF32 kernels of N = 256 have a fused form
    return n == 256 && tc - 1 == kTcTf32x3 && get_pass_variant(256, kKindTc) == 0 &&
           get_pass_variant(256, kKindTcXy) == 1;
  return (n == 128 || n == 256 || n == 512) && get_pass_variant(n, kKindXy) != 0;
}

// ------------------------------------------------------------------ pass sequences
#define CG_TRY(expr)                        \
  do {                                      \
    cudaError_t _e = (expr);                \
    if (_e != cudaSuccess) return _e;       \
    count_launches(1);                      \
  } while (0)

// x pass of real filter cubes (N^3 floats each) into complex spectra, profiled in the
// x-fwd slot with its own bytes (4 read + 8 written per point).
static cudaError_t pass_real(int n, const float *filt, float2 *spec, int count, cudaStream_t s) {
  NvtxRange nv("x-fwd real");
  PassRec r{0 * 4 + OP_FWD, 0.0, nullptr, nullptr};
  if (g_prof) {
    r.bytes = 12.0 * (double)n * n * n * count;
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, s);
  }
  const cudaError_t e = launch_axis_pass_real(n, filt, spec, count, g.tw512, s);
  if (g_prof) {
    cudaEventRecord(r.b, s);
    g_prof_recs.push_back(r);
  }
  return e;
}

// Hermitian half spectra of real filters (FP32 path, N >= 64, plan kind kKindHalf = 1).
static bool use_half(unsigned n, bool real, int tc) {
  return real && tc == 0 && half_spectrum_pitch((int)n) > 0 && get_pass_variant((int)n, kKindHalf) == 1;
}

// A pass over (or into, or against) a half spectrum, profiled in its axis/op slot with the
// bytes it moves: axis 0 reads N^3 floats and writes N^2 W values; axes 1 and 2 read and
// write N^2 W values; the paired fused z pass reads and writes the signal and reads a
// (C+2)/(2C) share of a full spectrum's bytes (C = 16 columns per tile below N = 256, 8 above).
static cudaError_t pass_half(int n, int axis, int op, const void *src, float2 *dst, const float2 *filt,
                             long long filt_vol, int nvol, float scale, cudaStream_t s) {
  NvtxRange nv(axis == 0 ? "x-fwd half" : (axis == 1 ? "y-fwd half" : (op == OP_CONV ? "z-conv half" : "z-fwd half")));
  PassRec r{axis * 4 + op, 0.0, nullptr, nullptr};
  if (g_prof) {
    const double v = (double)n * n * n, h = (double)n * n * half_spectrum_pitch(n);
    const double cols = n >= 256 ? 8.0 : 16.0;
    r.bytes = nvol * (axis == 0 ? 4.0 * v + 8.0 * h
                                : (op == OP_CONV ? 16.0 * v + 8.0 * v * (cols + 2.0) / (2.0 * cols) : 16.0 * h));
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, s);
  }
  const cudaError_t e = launch_axis_pass_half(n, axis, op, src, dst, filt, filt_vol, nvol, scale, g.tw512, s);
  if (g_prof) {
    cudaEventRecord(r.b, s);
    g_prof_recs.push_back(r);
  }
  return e;
}

// Half spectra of `count` real filters (N^3 floats each) into spec (N^2 W values each):
// x pass of the real rows, then y and z passes over the half width.
static cudaError_t enqueue_filter_half(int n, const float *filt, float2 *spec, int count, cudaStream_t s) {
  CG_TRY(pass_half(n, 0, OP_FWD, filt, spec, nullptr, 0, count, 1.f, s));
  CG_TRY(pass_half(n, 1, OP_FWD, spec, spec, nullptr, 0, count, 1.f, s));
  CG_TRY(pass_half(n, 2, OP_FWD, spec, spec, nullptr, 0, count, 1.f, s));
  return cudaSuccess;
}

// Filter spectra of `count` filters (x, y and, unless xy_only, z passes) into spec. With
// `real`, filt holds N^3 floats per filter (CONVGPU_FILTER_REAL); spec must not overlap it.
static cudaError_t enqueue_filter(int n, const float2 *filt, float2 *spec, int count, bool xy_only,
                                  cudaStream_t s, int tc = 0, bool real = false) {
  cudaError_t xe =
      (!real && use_xy(n, tc)) ? pass_xy(n, filt, spec, count, false, 1.f, s, tc) : cudaErrorNotSupported;
  if (xe != cudaSuccess && xe != cudaErrorNotSupported) return xe;
  if (xe == cudaErrorNotSupported) {
    if (real)
      CG_TRY(pass_real(n, reinterpret_cast<const float *>(filt), spec, count, s));
    else
      CG_TRY(pass(n, 0, OP_FWD, filt, spec, nullptr, 0, count, 1.f, s, tc));
    CG_TRY(pass(n, 1, OP_FWD, spec, spec, nullptr, 0, count, 1.f, s, tc));
  }
  if (!xy_only) CG_TRY(pass(n, 2, OP_FWD, spec, spec, nullptr, 0, count, 1.f, s, tc));
  return cudaSuccess;
}

// Signal passes. fop: OP_CONV (spec is a full spectrum, or with `half` a Hermitian half
// spectrum) or OP_CONV_FZ (xy only). mid (optional) is recorded after the fused z pass.
static cudaError_t enqueue_signals(int n, const float2 *sig, float2 *out, const float2 *spec,
                                   long long spec_vol, int fop, int nsig, float scale, cudaStream_t s,
                                   cudaEvent_t mid, int tc = 0, bool half = false) {
  cudaError_t xe = use_xy(n, tc) ? pass_xy(n, sig, out, nsig, false, 1.f, s, tc) : cudaErrorNotSupported;
  if (xe != cudaSuccess && xe != cudaErrorNotSupported) return xe;
  const bool fused = xe == cudaSuccess;
  if (!fused) {
    CG_TRY(pass(n, 0, OP_FWD, sig, out, nullptr, 0, nsig, 1.f, s, tc));
    CG_TRY(pass(n, 1, OP_FWD, out, out, nullptr, 0, nsig, 1.f, s, tc));
  }
  if (half)
    CG_TRY(pass_half(n, 2, OP_CONV, out, out, spec, spec_vol, nsig, 1.f, s));
  else
    CG_TRY(pass(n, 2, fop, out, out, spec, spec_vol, nsig, 1.f, s, tc));
  if (mid) cudaEventRecord(mid, s);
  if (fused) {
    const cudaError_t e = pass_xy(n, out, out, nsig, true, scale, s, tc);
    if (e == cudaSuccess) return cudaSuccess;
    if (e != cudaErrorNotSupported) return e;
  }
  CG_TRY(pass(n, 1, OP_INV, out, out, nullptr, 0, nsig, 1.f, s, tc));
  CG_TRY(pass(n, 0, OP_INV, out, out, nullptr, 0, nsig, scale, s, tc));
  return cudaSuccess;
}

static int tc_of(unsigned flags) {
  // 0: FP32 kernels; 1 + split precision for the tensor-core path.
  return (flags & (kFlagTensorSplit | kFlagTensorBf16x3)) ? 1 + ((flags & kFlagTensorBf16x3) ? kTcBf16x3 : kTcTf32x3)
                                                          : 0;
}

static size_t workspace_bytes_for(unsigned n, unsigned how_many, unsigned flags) {
  size_t vol = (size_t)n * n * n * sizeof(float2);
  if (flags & kFlagFilterIsSpectrum) return 0;
  if (use_half(n, (flags & kFlagFilterReal) != 0, tc_of(flags)))
    vol = (size_t)n * n * half_spectrum_pitch((int)n) * sizeof(float2);  // a half spectrum per filter
  if (flags & kFlagPerSignalFilter) return vol * how_many;
  return vol;
}

// Largest batch for which a shared filter's z transform runs inside the signals' fused z
// pass instead of as a pass of its own.
constexpr unsigned kSharedFilterFusedMax = 2;

// Whole convolution on device pointers, enqueued on stream s using workspace ws.
static cudaError_t enqueue_conv_device(unsigned n, const float2 *sig, const float2 *filt, float2 *out,
                                       unsigned how_many, unsigned flags, float2 *ws, cudaStream_t s) {
  const float scale = (flags & kFlagNormalize) ? (float)(1.0 / ((double)n * n * n)) : 1.0f;
  const long long V = (long long)n * n * n;
  const int tc = tc_of(flags);
  if (flags & kFlagFilterIsSpectrum) {
    const long long sv = (flags & kFlagPerSignalFilter) ? V : 0;
    return enqueue_signals(n, sig, out, filt, sv, OP_CONV, how_many, scale, s, nullptr, tc);
  }
  const bool real = (flags & kFlagFilterReal) != 0;
  // One small cube (N <= 64, 2 MiB, L2-resident): the whole convolution in one cooperative
  // launch instead of seven launches separated by launch gaps.
  if (how_many == 1 && tc == 0 && n <= 64) {
    const cudaError_t e =
        launch_small_conv((int)n, sig, filt, out, ws, scale, real, g.tw512, device_status_address(), s);
    if (e == cudaSuccess) {
      count_launches(1);
      return cudaSuccess;
    }
    cudaGetLastError();  // not applicable (size, residency): the per-pass launches below
  }
  if (use_half(n, real, tc)) {  // Hermitian half spectra, every signal through the paired z pass
    const bool per = (flags & kFlagPerSignalFilter) != 0;
    cudaError_t e = enqueue_filter_half((int)n, reinterpret_cast<const float *>(filt), ws, per ? (int)how_many : 1, s);
    if (e != cudaSuccess) return e;
    const long long hv = (long long)n * n * half_spectrum_pitch((int)n);
    return enqueue_signals(n, sig, out, ws, per ? hv : 0, OP_CONV, how_many, scale, s, nullptr, 0, true);
  }
  if (flags & kFlagPerSignalFilter) {
    cudaError_t e = enqueue_filter(n, filt, ws, how_many, true, s, tc, real);
    if (e != cudaSuccess) return e;
    return enqueue_signals(n, sig, out, ws, V, OP_CONV_FZ, how_many, scale, s, nullptr, tc);
  }
  // A shared filter's z transform is a pass of its own (read + write of one cube) when
  // its spectrum serves many signals; for one or two signals it is cheaper to redo it
  // inside each signal's fused z pass (about a quarter of a pass of extra arithmetic per
  // signal, no extra bytes).
  if (how_many <= kSharedFilterFusedMax) {
    cudaError_t e = enqueue_filter(n, filt, ws, 1, true, s, tc, real);
    if (e != cudaSuccess) return e;
    return enqueue_signals(n, sig, out, ws, 0, OP_CONV_FZ, how_many, scale, s, nullptr, tc);
  }
  cudaError_t e = enqueue_filter(n, filt, ws, 1, false, s, tc, real);
  if (e != cudaSuccess) return e;
  return enqueue_signals(n, sig, out, ws, 0, OP_CONV, how_many, scale, s, nullptr, tc);
}

// ------------------------------------------------------------------ bridge: setup
int bridge_initialize(const char *platform_name, const char *path, bool use_svm) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (path == nullptr || path[0] == '\0') {
    set_err("path missing");
    return -1;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    set_err("no CUDA devices");
    return -3;
  }
  int dev = 0;
  // "cuda:K" / "gpu:K" selects device K; any other name (the reference app passes the
  // Intel FPGA platform names) means the first device, as fpga_initialize picks
  // devices[0] (host/src/fpga_init.c:86).
  if (platform_name) {
    const char *p = nullptr;
    if (std::strncmp(platform_name, "cuda:", 5) == 0) p = platform_name + 5;
    if (std::strncmp(platform_name, "gpu:", 4) == 0) p = platform_name + 4;
    if (p) {
      char *end = nullptr;
      long k = std::strtol(p, &end, 10);
      if (end == p || *end != '\0' || k < 0 || k >= count) {
        set_err("no such CUDA device");
        return -2;
      }
      dev = (int)k;
    }
  }
  g.plan_path = path;
  const int rc = setup_locked(dev, use_svm);
  if (rc == 0) load_plan_cache(g.plan_path);  // anything that is not a plan cache is ignored
  return rc;
}

void bridge_final() {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  teardown_locked();
}

// ------------------------------------------------------------------ bridge: device API
int bridge_workspace_bytes(unsigned n, unsigned how_many, unsigned flags, size_t *bytes) {
  if (!bytes || !valid_n(n) || how_many == 0) return kErrInval;
  *bytes = workspace_bytes_for(n, how_many, flags);
  return 0;
}

int bridge_conv_device(unsigned n, const void *d_sig, const void *d_filt, void *d_out, unsigned how_many,
                       unsigned flags, void *stream) {
  if (!d_sig || !d_filt || !d_out || !valid_n(n)) {
    set_err("invalid arguments");
    return kErrInval;
  }
  if ((flags & kFlagFilterReal) && (flags & kFlagFilterIsSpectrum)) {
    set_err("CONVGPU_FILTER_REAL and CONVGPU_FILTER_IS_SPECTRUM exclude each other");
    return kErrInval;
  }
  if ((flags & kFlagFilterReal) && (reinterpret_cast<uintptr_t>(d_filt) & 3u)) {
    set_err("a real filter must be 4-byte aligned");
    return kErrInval;
  }
  if (how_many == 0) return 0;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_init_locked();
  if (rc) return rc;
  NvtxRange nv("convgpu_conv3d_device");
  cudaError_t e = g.ws.ensure(workspace_bytes_for(n, how_many, flags));
  if (e != cudaSuccess) return cuda_fail(e, "workspace");
  CallOrder order((cudaStream_t)stream);
  e = enqueue_conv_device(n, (const float2 *)d_sig, (const float2 *)d_filt, (float2 *)d_out, how_many, flags,
                          (float2 *)g.ws.p, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "launch");
  return 0;
}

int bridge_filter_spectrum_device(unsigned n, const void *d_filt, void *d_spec, unsigned count, void *stream) {
  if (!d_filt || !d_spec || !valid_n(n)) {
    set_err("invalid arguments");
    return kErrInval;
  }
  if (count == 0) return 0;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_init_locked();
  if (rc) return rc;
  NvtxRange nv("convgpu_filter_spectrum_device");
  CallOrder order((cudaStream_t)stream);
  cudaError_t e = enqueue_filter(n, (const float2 *)d_filt, (float2 *)d_spec, count, false, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "launch");
  return 0;
}

// Checks an uneven batch's descriptors before anything runs: every size supported; every
// cube's element range addressable from its base pointer (no wrap of the 64-bit address);
// a job's output either is its own signal (in place) or does not overlap it; and no two
// jobs' outputs overlap (their passes would overwrite each other's data). Returns "" or
// the reason.
static std::string check_jobs(const UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt,
                              const void *d_out) {
  const unsigned long long kMax = ~0ull;
  std::vector<std::pair<unsigned long long, unsigned>> outs(njobs);
  for (unsigned j = 0; j < njobs; ++j) {
    const UnevenJob &jb = jobs[j];
    if (!valid_n(jb.n)) return "job " + std::to_string(j) + ": size " + std::to_string(jb.n) + " not supported";
    const unsigned long long v = (unsigned long long)jb.n * jb.n * jb.n;
    const void *base[3] = {d_sig, d_filt, d_out};
    const unsigned long long off[3] = {jb.sig_off, jb.filt_off, jb.out_off};
    for (int k = 0; k < 3; ++k) {
      // byte end = base + (off + v) * 8 must not pass the end of the address space
      const unsigned long long b = (unsigned long long)reinterpret_cast<uintptr_t>(base[k]);
      if (off[k] > kMax / 8 - v || (off[k] + v) * 8 > kMax - b)
        return "job " + std::to_string(j) + ": offset " + std::to_string(off[k]) + " lies past the address space";
    }
    if (d_sig == d_out && jb.sig_off != jb.out_off && jb.sig_off < jb.out_off + v && jb.out_off < jb.sig_off + v)
      return "job " + std::to_string(j) + ": output partly overlaps its own signal";
    outs[j] = {jb.out_off, j};
  }
  std::sort(outs.begin(), outs.end());
  for (unsigned i = 1; i < njobs; ++i) {
    const UnevenJob &a = jobs[outs[i - 1].second];
    if (outs[i - 1].first + (unsigned long long)a.n * a.n * a.n > outs[i].first)
      return "outputs of jobs " + std::to_string(outs[i - 1].second) + " and " + std::to_string(outs[i].second) +
             " overlap";
  }
  return "";
}

int bridge_conv_uneven_device(const UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt,
                              void *d_out, unsigned flags, void *stream) {
  if (!jobs || !d_sig || !d_filt || !d_out) {
    set_err("invalid arguments");
    return kErrInval;
  }
  const std::string bad = check_jobs(jobs, njobs, d_sig, d_filt, d_out);
  if (!bad.empty()) {
    set_err(bad);
    return kErrInval;
  }
  const bool real = (flags & kFlagFilterReal) != 0;  // filter offsets then count floats
  if (real && !(flags & kFlagUnevenPerJob)) {
    set_err("CONVGPU_FILTER_REAL in an uneven batch needs CONVGPU_UNEVEN_PER_JOB");
    return kErrUnsupported;
  }
  if (real && (flags & kFlagFilterIsSpectrum)) {
    set_err("CONVGPU_FILTER_REAL and CONVGPU_FILTER_IS_SPECTRUM exclude each other");
    return kErrInval;
  }
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_init_locked();
  if (rc) return rc;
  NvtxRange nv("convgpu_conv3d_uneven_device");
  const bool normalize = (flags & kFlagNormalize) != 0;
  if (!(flags & (kFlagUnevenPerJob | kFlagTensorSplit | kFlagTensorBf16x3 | kFlagFilterIsSpectrum))) {
    std::string err;
    CallOrder order((cudaStream_t)stream);
    if (flags & kFlagUnevenQueue) {
      unsigned *status = device_status_address();
      if (!status) return cuda_fail(cudaErrorInvalidSymbol, "device status word");
      rc = uneven_persistent(jobs, njobs, d_sig, d_filt, d_out, normalize, g.tw512, status, (cudaStream_t)stream, err);
      if (rc) set_err(err);
      return rc;
    }
    rc = uneven_grouped(jobs, njobs, d_sig, d_filt, d_out, normalize, g.tw512, (cudaStream_t)stream, err);
    if (rc != kErrUnsupported) {
      if (rc) set_err(err);
      return rc;
    }
    // unaligned cubes: one job at a time below
  }
  // One job at a time (CONVGPU_UNEVEN_PER_JOB, the tensor-core path, or precomputed spectra).
  size_t need = 0;
  for (unsigned j = 0; j < njobs; ++j) need = std::max(need, workspace_bytes_for(jobs[j].n, 1, flags & ~kFlagPerSignalFilter));
  cudaError_t e = g.ws.ensure(need);
  if (e != cudaSuccess) return cuda_fail(e, "workspace");
  CallOrder order((cudaStream_t)stream);
  for (unsigned j = 0; j < njobs; ++j) {
    const float2 *s = (const float2 *)d_sig + jobs[j].sig_off;
    const float2 *f = real ? reinterpret_cast<const float2 *>((const float *)d_filt + jobs[j].filt_off)
                           : (const float2 *)d_filt + jobs[j].filt_off;
    if (real && (reinterpret_cast<uintptr_t>(f) & 3u)) {
      set_err("a real filter must be 4-byte aligned");
      return kErrInval;
    }
    float2 *o = (float2 *)d_out + jobs[j].out_off;
    e = enqueue_conv_device(jobs[j].n, s, f, o, 1, flags & ~kFlagPerSignalFilter, (float2 *)g.ws.p,
                            (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "launch");
  }
  return 0;
}

// ------------------------------------------------------------------ bridge: host API
namespace {
struct EvPool {
  std::vector<cudaEvent_t> ev;
  cudaEvent_t get() {
    cudaEvent_t e;
    cudaEventCreate(&e);
    ev.push_back(e);
    return e;
  }
  ~EvPool() {
    for (auto e : ev) cudaEventDestroy(e);
  }
};
float ms_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.f;
  return ms;
}
}  // namespace

// ------------------------------------------------------------------ host copies
// True for pageable host memory (malloc, fpgaf_complex_malloc, numpy arrays): a
// cudaMemcpyAsync to such memory returns only once the copy has completed (and one from it
// once the data is staged), so the host pipeline issues its downloads from a second thread.
static bool is_pageable(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeUnregistered;
}

// Shared-filter spectrum reuse for the host entry points (CONVGPU_FILTER_CACHED): true
// when hfilt still holds the spectrum of this filter pointer, N and path. Any other use
// of hfilt drops the key first; a flagged call that transforms the filter sets it again.
static bool filter_cache_hit(const void *filt, unsigned n, int tc, unsigned flags, bool per_signal) {
  const bool hit = (flags & kFlagFilterCached) && !per_signal && g.hkey.valid && g.hkey.ptr == filt &&
                   g.hkey.n == n && g.hkey.tc == tc;
  if (!hit) g.hkey.valid = false;
  return hit;
}
static void filter_cache_set(const void *filt, unsigned n, int tc, unsigned flags, bool per_signal) {
  if (!(flags & kFlagFilterCached) || per_signal) return;
  g.hkey.ptr = filt;
  g.hkey.n = n;
  g.hkey.tc = tc;
  g.hkey.valid = true;
}

// Host-buffer batch with slab-granular overlap (CONVGPU_HOST_SLABS, cubes of 32 MiB and
// more): each cube is copied in z-slabs; the x / y passes of a slab start as soon as it
// lands (planes are independent for those axes), the fused z pass runs once per cube,
// and the inverse y / x passes hand finished slabs to the device-to-host stream one by
// one, so pipeline fill and drain shrink from a cube to a slab. On GB300 the 16-32 MiB
// slab copies move fewer bytes per second than whole-cube copies, and the whole-cube
// pipeline measured faster end to end (599 vs 575 conv/s at 256^3 x 4), so it stays the
// default. Returns the error of the first failing call.
static cudaError_t conv_host_slabs(unsigned n, const float2 *sig, const float2 *filt, float2 *out, unsigned how_many,
                                   bool per_signal, float scale, int mode, unsigned flags, Timing &t) {
  const size_t V = (size_t)n * n * n;
  const size_t vbytes = V * sizeof(float2);
  const int slab = n >= 512 ? 16 : 32;  // planes per slab: 16 MiB at 256^3, 32 MiB at 512^3
  const int nslab = (int)n / slab;
  const size_t selems = (size_t)slab * n * n;
  const unsigned nbuf = std::min(3u, how_many);
  cudaError_t e = cudaSuccess;
  for (unsigned b = 0; b < nbuf && e == cudaSuccess; ++b) {
    e = g.hio[b].ensure(vbytes);
    if (e == cudaSuccess && per_signal) e = g.hfio[b].ensure(vbytes);
  }
  if (e == cudaSuccess && !per_signal) e = g.hfilt.ensure(vbytes);
  if (e != cudaSuccess) return e;
  EvPool pool;
  std::vector<cudaEvent_t> in((size_t)how_many * nslab), done((size_t)how_many * nslab), freed(nbuf);
  for (auto &v : in) v = pool.get();
  for (auto &v : done) v = pool.get();
  for (auto &v : freed) v = pool.get();
  std::vector<cudaEvent_t> h0(how_many), h1(how_many), c0(how_many), cm(how_many), c1(how_many), d0(how_many),
      d1(how_many);
  for (unsigned c = 0; c < how_many; ++c) {
    h0[c] = pool.get(), h1[c] = pool.get(), c0[c] = pool.get(), cm[c] = pool.get(), c1[c] = pool.get();
    d0[c] = pool.get(), d1[c] = pool.get();
  }
  cudaEvent_t f0 = pool.get(), f1 = pool.get(), f2 = pool.get();
  float2 *fspec = (float2 *)g.hfilt.p;
  const bool cached = filter_cache_hit(filt, n, 0, flags, per_signal);
  if (!per_signal && !cached) {
    cudaEventRecord(f0, g.sh2d);
    e = cudaMemcpyAsync(fspec, filt, vbytes, cudaMemcpyHostToDevice, g.sh2d);
    cudaEventRecord(f1, g.sh2d);
    cudaStreamWaitEvent(g.sc, f1, 0);
    if (e == cudaSuccess) e = enqueue_filter((int)n, fspec, fspec, 1, false, g.sc);
    cudaEventRecord(f2, g.sc);
    if (e == cudaSuccess) filter_cache_set(filt, n, 0, flags, per_signal);
  }
  auto planes = [&](int axis, int op, float2 *p, float sc) {
    if (e != cudaSuccess) return;
    e = launch_axis_pass_planes((int)n, axis, op, p, p, slab, sc, g.tw512, g.sc);
    if (e == cudaSuccess) count_launches(1);
  };
  // Downloads of cube c are enqueued after the uploads of cube c + 1 (see bridge_conv_host).
  auto out_cube = [&](unsigned c) {
    const unsigned b = c % nbuf;
    float2 *io = (float2 *)g.hio[b].p;
    cudaStreamWaitEvent(g.sd2h, done[c * nslab], 0);
    cudaEventRecord(d0[c], g.sd2h);
    for (int k = 0; k < nslab && e == cudaSuccess; ++k) {
      if (k) cudaStreamWaitEvent(g.sd2h, done[c * nslab + k], 0);
      e = cudaMemcpyAsync(out + c * V + k * selems, io + k * selems, selems * sizeof(float2), cudaMemcpyDeviceToHost,
                          g.sd2h);
    }
    cudaEventRecord(d1[c], g.sd2h);
    cudaEventRecord(freed[b], g.sd2h);
  };
  for (unsigned c = 0; c < how_many && e == cudaSuccess; ++c) {
    const unsigned b = c % nbuf;
    float2 *io = (float2 *)g.hio[b].p;
    float2 *fio = per_signal ? (float2 *)g.hfio[b].p : nullptr;
    if (c >= nbuf) cudaStreamWaitEvent(g.sh2d, freed[b], 0);
    cudaEventRecord(h0[c], g.sh2d);
    for (int k = 0; k < nslab && e == cudaSuccess; ++k) {
      e = cudaMemcpyAsync(io + k * selems, sig + c * V + k * selems, selems * sizeof(float2), cudaMemcpyHostToDevice,
                          g.sh2d);
      if (e == cudaSuccess && per_signal)
        e = cudaMemcpyAsync(fio + k * selems, filt + c * V + k * selems, selems * sizeof(float2),
                            cudaMemcpyHostToDevice, g.sh2d);
      cudaEventRecord(in[c * nslab + k], g.sh2d);
    }
    cudaEventRecord(h1[c], g.sh2d);
    if (c > 0) out_cube(c - 1);
    cudaStreamWaitEvent(g.sc, in[c * nslab], 0);
    cudaEventRecord(c0[c], g.sc);
    for (int k = 0; k < nslab && e == cudaSuccess; ++k) {
      if (k) cudaStreamWaitEvent(g.sc, in[c * nslab + k], 0);
      if (per_signal) {
        planes(0, OP_FWD, fio + k * selems, 1.f);
        planes(1, OP_FWD, fio + k * selems, 1.f);
      }
      planes(0, OP_FWD, io + k * selems, 1.f);
      planes(1, OP_FWD, io + k * selems, 1.f);
    }
    if (e == cudaSuccess)
      e = pass((int)n, 2, per_signal ? OP_CONV_FZ : OP_CONV, io, io, per_signal ? fio : fspec,
               per_signal ? (long long)V : 0, 1, 1.f, g.sc, 0);
    if (e == cudaSuccess) count_launches(1);
    cudaEventRecord(cm[c], g.sc);
    for (int k = 0; k < nslab && e == cudaSuccess; ++k) {
      planes(1, OP_INV, io + k * selems, 1.f);
      planes(0, OP_INV, io + k * selems, scale);
      cudaEventRecord(done[c * nslab + k], g.sc);
    }
    cudaEventRecord(c1[c], g.sc);
  }
  if (e == cudaSuccess) out_cube(how_many - 1);
  cudaError_t es = cudaStreamSynchronize(g.sd2h);
  cudaError_t es2 = cudaStreamSynchronize(g.sc);
  cudaError_t es3 = cudaStreamSynchronize(g.sh2d);
  if (e == cudaSuccess) e = es != cudaSuccess ? es : (es2 != cudaSuccess ? es2 : es3);
  if (e != cudaSuccess) return e;
  if (!per_signal && !cached) {
    t.filter_pcie_wr_t = ms_between(f0, f1);
    t.filter_exec_t = ms_between(f1, f2);
  }
  double inv = 0.0;
  for (unsigned c = 0; c < how_many; ++c) {
    t.sig_pcie_wr_t += ms_between(h0[c], h1[c]);
    t.sig_exec_t += ms_between(c0[c], cm[c]);
    inv += ms_between(cm[c], c1[c]);
    t.sig_pcie_rd_t += ms_between(d0[c], d1[c]);
  }
  if (mode == HOST_BATCH) {
    t.sig_exec_t += inv;
    t.siginv_exec_t = ms_between(c0[0], c1[how_many - 1]);
  } else {
    t.siginv_exec_t = inv;
  }
  return cudaSuccess;
}

Timing bridge_conv_host(unsigned n, const void *sig, const void *filt, void *out, unsigned how_many,
                        unsigned flags, int mode) {
  Timing t{0, 0, 0, 0, 0, 0, false};
  if (sig == nullptr || filt == nullptr || out == nullptr || !valid_n(n)) {
    set_err("invalid arguments");
    return t;
  }
  if (how_many == 0) {
    set_err("how_many is 0");
    return t;
  }
  if (flags & kFlagFilterIsSpectrum) {
    set_err("CONVGPU_FILTER_IS_SPECTRUM is not supported by the host-buffer entry points");
    return t;
  }
  const int tc = tc_of(flags);
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (ensure_init_locked() != 0) return t;
  (void)mode;
  NvtxRange nv("convgpu_conv3d_host");
  CallOrder order(g.sc);  // compute waits for device calls still in flight on other streams

  const bool per_signal = (flags & kFlagPerSignalFilter) != 0;
  const bool real = (flags & kFlagFilterReal) != 0;  // filt holds N^3 floats per filter
  const size_t V = (size_t)n * n * n;
  const size_t vbytes = V * sizeof(float2);
  const size_t fbytes = real ? V * sizeof(float) : vbytes;  // bytes of one filter on the host
  const float scale = (flags & kFlagNormalize) ? (float)(1.0 / ((double)V)) : 1.0f;
  if (!tc && !real && (flags & kFlagHostSlabs) && vbytes >= (size_t(32) << 20)) {
    cudaError_t e = conv_host_slabs(n, (const float2 *)sig, (const float2 *)filt, (float2 *)out, how_many, per_signal,
                                    scale, mode, flags, t);
    if (e != cudaSuccess) {
      cuda_fail(e, "host pipeline");
      return t;
    }
    if (const unsigned st = read_and_clear_device_status()) {
      set_err("device status " + std::to_string(st) + ": a kernel gave up a bounded wait (tile load, MMA or dependency)");
      return t;
    }
    t.valid = true;
    return t;
  }
  // Signals per chunk: at least one cube, about 64 MiB per chunk otherwise.
  const unsigned per_chunk = (unsigned)std::max<size_t>(1, std::min<size_t>(how_many, (64u << 20) / vbytes));
  const unsigned nchunks = (how_many + per_chunk - 1) / per_chunk;
  const unsigned nbuf = std::min(3u, nchunks);

  cudaError_t e = cudaSuccess;
  for (unsigned b = 0; b < nbuf && e == cudaSuccess; ++b) {
    e = g.hio[b].ensure(per_chunk * vbytes);
    if (e == cudaSuccess && per_signal) e = g.hfio[b].ensure(per_chunk * vbytes);
  }
  if (e == cudaSuccess) e = g.hfilt.ensure(vbytes * (per_signal ? per_chunk : 1));
  if (real) {  // real filters land in float staging buffers; the x pass widens them
    for (unsigned b = 0; b < nbuf && e == cudaSuccess && per_signal; ++b) e = g.hreal[b].ensure(per_chunk * fbytes);
    if (e == cudaSuccess && !per_signal) e = g.hreal[3].ensure(fbytes);
  }
  if (e != cudaSuccess) {
    cuda_fail(e, "device buffers");
    return t;
  }

  EvPool pool;
  cudaEvent_t f0 = pool.get(), f1 = pool.get(), f2 = pool.get();
  std::vector<cudaEvent_t> h0(nchunks), hf(nchunks), h1(nchunks), c0(nchunks), cf(nchunks), cs(nchunks),
      c1(nchunks), cm(nchunks), d0(nchunks), d1(nchunks), freed(nbuf);
  for (unsigned c = 0; c < nchunks; ++c) {
    h0[c] = pool.get();
    hf[c] = pool.get();
    h1[c] = pool.get();
    cf[c] = pool.get();
    cs[c] = pool.get();
    c0[c] = pool.get();
    c1[c] = pool.get();
    cm[c] = pool.get();
    d0[c] = pool.get();
    d1[c] = pool.get();
  }
  for (unsigned b = 0; b < nbuf; ++b) freed[b] = pool.get();

  float2 *fspec = (float2 *)g.hfilt.p;
  // Pageable output buffer: its downloads block the thread that issues them, so a second
  // thread issues them (below) while this one keeps uploading and launching.
  bool pageable_out = is_pageable(out);
  const bool half = use_half(n, real, tc);  // real filters as Hermitian half spectra
  const long long hv = half ? (long long)n * n * half_spectrum_pitch((int)n) : 0;
  const int key = tc + (real ? 8 : 0) + (half ? 16 : 0);  // path of the kept spectrum
  const bool cached = filter_cache_hit(filt, n, key, flags, per_signal);
  if (!per_signal && !cached) {
    float2 *fin = real ? (float2 *)g.hreal[3].p : fspec;
    cudaEventRecord(f0, g.sh2d);
    e = cudaMemcpyAsync(fin, filt, fbytes, cudaMemcpyHostToDevice, g.sh2d);
    cudaEventRecord(f1, g.sh2d);
    cudaStreamWaitEvent(g.sc, f1, 0);
    if (e == cudaSuccess)
      e = half ? enqueue_filter_half(n, (const float *)fin, fspec, 1, g.sc)
               : enqueue_filter(n, fin, fspec, 1, false, g.sc, tc, real);
    cudaEventRecord(f2, g.sc);
    if (e == cudaSuccess) filter_cache_set(filt, n, key, flags, per_signal);
  }

  // Downloads of chunk c are enqueued after the uploads of chunk c + 1, so a download
  // waiting for its compute never sits ahead of the next upload in a copy queue.
  auto out_chunk = [&](unsigned c) -> cudaError_t {
    const unsigned b = c % nbuf;
    const unsigned first = c * per_chunk;
    const unsigned cnt = std::min(per_chunk, how_many - first);
    cudaStreamWaitEvent(g.sd2h, c1[c], 0);
    cudaEventRecord(d0[c], g.sd2h);
    const cudaError_t r = cudaMemcpyAsync((float2 *)out + (size_t)first * V, g.hio[b].p, cnt * vbytes,
                                          cudaMemcpyDeviceToHost, g.sd2h);
    cudaEventRecord(d1[c], g.sd2h);
    cudaEventRecord(freed[b], g.sd2h);
    return r;
  };
  // Pageable output: a download thread takes chunk c once this thread has recorded its
  // compute end (c1[c]); chunk buffer b is reused once the download of chunk c - nbuf has
  // returned (which, for pageable memory, is when it has completed).
  std::mutex dl_mu;
  std::condition_variable dl_cv;
  int dl_ready = -1, dl_done = -1;
  bool dl_stop = false;
  cudaError_t dl_err = cudaSuccess;
  std::thread dl;
  auto download_loop = [&] {
    for (unsigned c = 0; c < nchunks; ++c) {
      {
        std::unique_lock<std::mutex> lk(dl_mu);
        dl_cv.wait(lk, [&] { return dl_stop || dl_ready >= (int)c; });
        if (dl_ready < (int)c) return;  // stopped before chunk c was launched
      }
      const cudaError_t r = out_chunk(c);
      std::lock_guard<std::mutex> lk(dl_mu);
      if (r != cudaSuccess && dl_err == cudaSuccess) dl_err = r;
      dl_done = (int)c;
      dl_cv.notify_all();
    }
  };
  if (pageable_out) {
    try {
      dl = std::thread(download_loop);
    } catch (...) {  // no thread to be had: downloads from this thread, as for pinned buffers
      pageable_out = false;
    }
  }
  for (unsigned c = 0; c < nchunks && e == cudaSuccess; ++c) {
    const unsigned b = c % nbuf;
    const unsigned first = c * per_chunk;
    const unsigned cnt = std::min(per_chunk, how_many - first);
    float2 *io = (float2 *)g.hio[b].p;
    if (c >= nbuf) {
      if (pageable_out) {
        std::unique_lock<std::mutex> lk(dl_mu);
        dl_cv.wait(lk, [&] { return dl_done >= (int)(c - nbuf) || dl_err != cudaSuccess; });
        if (dl_err != cudaSuccess) {
          e = dl_err;
          break;
        }
      } else {
        cudaStreamWaitEvent(g.sh2d, freed[b], 0);
      }
    }
    cudaEventRecord(h0[c], g.sh2d);
    // Per-signal filters go up first: their x+y pass then runs while the signals upload.
    void *fin = real ? g.hreal[b].p : g.hfio[b].p;
    if (per_signal)
      e = cudaMemcpyAsync(fin, (const char *)filt + (size_t)first * fbytes, cnt * fbytes, cudaMemcpyHostToDevice,
                          g.sh2d);
    cudaEventRecord(hf[c], g.sh2d);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(io, (const float2 *)sig + (size_t)first * V, cnt * vbytes, cudaMemcpyHostToDevice, g.sh2d);
    cudaEventRecord(h1[c], g.sh2d);
    if (e != cudaSuccess) break;
    if (c > 0 && !pageable_out) e = out_chunk(c - 1);
    if (e != cudaSuccess) break;
    cudaStreamWaitEvent(g.sc, per_signal ? hf[c] : h1[c], 0);
    cudaEventRecord(c0[c], g.sc);
    if (per_signal) {
      e = half ? enqueue_filter_half(n, (const float *)fin, (float2 *)g.hfio[b].p, (int)cnt, g.sc)
               : enqueue_filter(n, (const float2 *)fin, (float2 *)g.hfio[b].p, cnt, true, g.sc, tc, real);
      cudaEventRecord(cf[c], g.sc);
      cudaStreamWaitEvent(g.sc, h1[c], 0);
      cudaEventRecord(cs[c], g.sc);  // compute time excludes the wait for the signals' upload
      if (e == cudaSuccess)
        e = enqueue_signals(n, io, io, (const float2 *)g.hfio[b].p, half ? hv : (long long)V,
                            half ? OP_CONV : OP_CONV_FZ, cnt, scale, g.sc, cm[c], tc, half);
    } else {
      e = enqueue_signals(n, io, io, fspec, 0, OP_CONV, cnt, scale, g.sc, cm[c], tc, half);
    }
    cudaEventRecord(c1[c], g.sc);
    if (pageable_out) {
      std::lock_guard<std::mutex> lk(dl_mu);
      dl_ready = (int)c;
      dl_cv.notify_all();
    }
  }
  if (pageable_out) {
    {
      std::lock_guard<std::mutex> lk(dl_mu);
      if (e != cudaSuccess) dl_stop = true;  // chunks not launched are not downloaded
      dl_cv.notify_all();
    }
    dl.join();
    if (e == cudaSuccess) e = dl_err;
  } else if (e == cudaSuccess) {
    e = out_chunk(nchunks - 1);
  }
  cudaError_t es = cudaStreamSynchronize(g.sd2h);
  cudaError_t es2 = cudaStreamSynchronize(g.sc);
  cudaError_t es3 = cudaStreamSynchronize(g.sh2d);
  if (e == cudaSuccess) e = es != cudaSuccess ? es : (es2 != cudaSuccess ? es2 : es3);
  if (e != cudaSuccess) {
    cuda_fail(e, "host pipeline");
    return t;
  }
  if (const unsigned st = read_and_clear_device_status()) {
    set_err("device status " + std::to_string(st) + ": a kernel gave up a bounded wait (tile load, MMA or dependency)");
    return t;
  }
  if (!per_signal && !cached) {
    t.filter_pcie_wr_t = ms_between(f0, f1);
    t.filter_exec_t = ms_between(f1, f2);
  }
  double inv = 0.0;
  for (unsigned c = 0; c < nchunks; ++c) {
    t.sig_pcie_wr_t += ms_between(h0[c], h1[c]);
    t.sig_exec_t += per_signal ? ms_between(c0[c], cf[c]) + ms_between(cs[c], cm[c]) : ms_between(c0[c], cm[c]);
    inv += ms_between(cm[c], c1[c]);
    t.sig_pcie_rd_t += ms_between(d0[c], d1[c]);
  }
  // Single call: forward phase vs inverse phase. Batched call: like the reference,
  // sig_exec_t sums the per-signal compute phases and siginv_exec_t is the wall span
  // from the first compute to the last (host/src/convfpga_svm_batch.c:664-665).
  if (mode == HOST_BATCH) {
    t.sig_exec_t += inv;
    t.siginv_exec_t = ms_between(c0[0], c1[nchunks - 1]);
  } else {
    t.siginv_exec_t = inv;
  }
  t.valid = true;
  return t;
}

// ------------------------------------------------------------------ autotuner / plan cache
// The plan cache plays the role of the reference CPU path's FFTW wisdom file
// (src/fft_conv3D.cpp:85-112): one line per cube size with the shape variant chosen for
// each pass kind and the timings (microseconds per launch, variants 0 and 1) it was
// chosen from.
static const char *kKindNames[kPassKinds] = {"rows", "strided", "conv", "conv_fz", "xy", "tc", "tcxy", "herm"};

static void load_plan_cache(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char line[1024];
  while (std::fgets(line, sizeof(line), f)) {
    int n = 0;
    const char *q = std::strchr(line, '"');
    if (!q || std::sscanf(q, "\"%d\": {", &n) != 1 || !valid_n((unsigned)n)) continue;
    for (int k = 0; k < kPassKinds; ++k) {
      const std::string key = std::string("\"") + kKindNames[k] + "\": ";
      const char *p = std::strstr(line, key.c_str());
      int v = 0;
      if (p && std::sscanf(p + key.size(), "%d", &v) == 1) set_pass_variant(n, k, v);
    }
  }
  std::fclose(f);
}

struct TuneRow {
  int n;
  int choice[kPassKinds];
  double us[2][kPassKinds];
};
static std::vector<TuneRow> g_tuned;

static bool write_plan_cache(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, g.device);
  std::fprintf(f, "{\"convgpu_plan_cache\": 1, \"device\": \"%s\", \"sizes\": {\n", prop.name);
  for (size_t i = 0; i < g_tuned.size(); ++i) {
    const TuneRow &r = g_tuned[i];
    std::fprintf(f, "  \"%d\": {", r.n);
    for (int k = 0; k < kPassKinds; ++k) std::fprintf(f, "\"%s\": %d, ", kKindNames[k], r.choice[k]);
    for (int v = 0; v < 2; ++v) {
      std::fprintf(f, "\"us_v%d\": [", v);
      for (int k = 0; k < kPassKinds; ++k) std::fprintf(f, "%.2f%s", r.us[v][k], k + 1 < kPassKinds ? ", " : "");
      std::fprintf(f, "]%s", v == 0 ? ", " : "");
    }
    std::fprintf(f, "}%s\n", i + 1 < g_tuned.size() ? "," : "");
  }
  std::fprintf(f, "}}\n");
  std::fclose(f);
  return true;
}

// Times both shape variants of every pass kind for each size on a working set larger
// than L2 and keeps the faster; optionally writes the plan cache.
int bridge_autotune(const unsigned *sizes, unsigned count, int write_cache) {
  if (!sizes && count) return kErrInval;
  for (unsigned i = 0; i < count; ++i)
    if (!valid_n(sizes[i])) {
      set_err("autotune: unsupported size");
      return kErrInval;
    }
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_init_locked();
  if (rc) return rc;
  cudaStream_t s = g.sc;
  CallOrder order(s);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t err = cudaSuccess;
  for (unsigned i = 0; i < count && err == cudaSuccess; ++i) {
    const int n = (int)sizes[i];
    const size_t V = (size_t)n * n * n;
    const int nvol = (int)std::max<size_t>(1, (size_t(256) << 20) / (V * sizeof(float2)));
    err = g.ws.ensure(2 * nvol * V * sizeof(float2));
    if (err != cudaSuccess) break;
    float2 *data = (float2 *)g.ws.p;
    float2 *spec = data + nvol * V;
    cudaMemsetAsync(g.ws.p, 0, 2 * nvol * V * sizeof(float2), s);
    TuneRow row{};
    row.n = n;
    for (int k = 0; k < kPassKinds && err == cudaSuccess; ++k) {
      if (k == kKindXy) {
        // separate x and y passes (variant 0) against the L2-staged fused pass (variant 1);
        // the cluster pass (variant 2, N = 256) is not timed: it lost to both on every
        // measurement
        row.us[0][k] = row.us[row.choice[kKindRows]][kKindRows] + row.us[row.choice[kKindStrided]][kKindStrided];
        row.us[1][k] = 1e30;
        if (n == 128 || n == 256 || n == 512) {
          for (int w = 0; w < 2 && err == cudaSuccess; ++w) {
            err = launch_xy_pass(n, data, data, nvol * n, false, 1.f, g.tw512, s, 1);
            if (err == cudaErrorNotSupported) break;
          }
          if (err == cudaSuccess) {
            cudaEventRecord(e0, s);
            for (int t = 0; t < 5 && err == cudaSuccess; ++t)
              err = launch_xy_pass(n, data, data, nvol * n, false, 1.f, g.tw512, s, 1);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            row.us[1][k] = 1000.0 * ms / 5.0;
            count_launches(14);
          } else if (err == cudaErrorNotSupported) {
            err = cudaSuccess;
          }
        }
        row.choice[k] = row.us[1][k] < row.us[0][k] ? 1 : 0;
        set_pass_variant(n, k, row.choice[k]);
        continue;
      }
      if (k == kKindHalf) {
        // fused z pass of real filters: full spectrum (variant 0, the chosen conv shape)
        // against the paired pass over a Hermitian half spectrum (variant 1); a tie goes
        // to the half spectrum, whose filter transform also moves fewer bytes
        for (int v = 0; v < 2; ++v) row.us[v][k] = 0.0;
        if (half_spectrum_pitch(n) > 0) {
          for (int v = 0; v < 2 && err == cudaSuccess; ++v) {
            auto run = [&]() {
              return v ? launch_axis_pass_half(n, 2, OP_CONV, data, data, spec, 0, nvol, 1.f, g.tw512, s)
                       : launch_axis_pass(n, 2, OP_CONV, data, data, spec, 0, nvol, 1.f, g.tw512, s);
            };
            for (int w = 0; w < 2 && err == cudaSuccess; ++w) err = run();
            cudaEventRecord(e0, s);
            for (int t = 0; t < 5 && err == cudaSuccess; ++t) err = run();
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            row.us[v][k] = 1000.0 * ms / 5.0;
            count_launches(7);
          }
          if (err == cudaErrorNotSupported) {
            err = cudaSuccess;
            row.us[1][k] = 1e30;
          }
        }
        row.choice[k] = (half_spectrum_pitch(n) > 0 && row.us[1][k] <= 1.02 * row.us[0][k]) ? 1 : 0;
        set_pass_variant(n, k, row.choice[k]);
        continue;
      }
      if (k == kKindTcXy) {
        // x and y passes of the split-TF32 path (tcgen05, N = 256): separate passes
        // (variant 0) against the L2-staged fused pass (variant 1)
        for (int v = 0; v < 2; ++v) row.us[v][k] = 0.0;
        if (n == 256) {
          for (int v = 0; v < 2 && err == cudaSuccess; ++v) {
            auto run = [&]() {
              if (v == 1) return launch_xy_l2_tc_pass(n, data, data, nvol * n, false, 1.f, g.tw512, s);
              cudaError_t r = launch_axis_pass_tc(n, 0, OP_FWD, data, data, nullptr, 0, nvol, 1.f, g.tw512, s,
                                                  kTcTf32x3);
              if (r == cudaSuccess)
                r = launch_axis_pass_tc(n, 1, OP_FWD, data, data, nullptr, 0, nvol, 1.f, g.tw512, s, kTcTf32x3);
              return r;
            };
            const int keep = get_pass_variant(n, kKindTc);
            set_pass_variant(n, kKindTc, 0);
            for (int w = 0; w < 2 && err == cudaSuccess; ++w) err = run();
            cudaEventRecord(e0, s);
            for (int t = 0; t < 5 && err == cudaSuccess; ++t) err = run();
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            set_pass_variant(n, kKindTc, keep);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            row.us[v][k] = 1000.0 * ms / 5.0;
            count_launches(14);
          }
          if (err == cudaErrorNotSupported) {
            err = cudaSuccess;
            row.us[1][k] = 1e30;
          }
        }
        row.choice[k] = row.us[1][k] < row.us[0][k] ? 1 : 0;
        set_pass_variant(n, k, row.choice[k]);
        continue;
      }
      if (k == kKindTc) {
        // tensor-core kernel of the split-TF32 path, timed on its fused z pass
        for (int v = 0; v < 2; ++v) row.us[v][k] = 0.0;
        if (n == 256) {
          const int keep = get_pass_variant(n, k);
          for (int v = 0; v < 2 && err == cudaSuccess; ++v) {
            set_pass_variant(n, k, v);
            auto run = [&]() {
              return launch_axis_pass_tc(n, 2, OP_CONV_FZ, data, data, spec, (long long)V, nvol, 1.f, g.tw512, s,
                                         kTcTf32x3);
            };
            for (int w = 0; w < 2 && err == cudaSuccess; ++w) err = run();
            cudaEventRecord(e0, s);
            for (int t = 0; t < 5 && err == cudaSuccess; ++t) err = run();
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            row.us[v][k] = 1000.0 * ms / 5.0;
            count_launches(7);
          }
          set_pass_variant(n, k, keep);
        }
        row.choice[k] = row.us[1][k] < row.us[0][k] ? 1 : 0;
        set_pass_variant(n, k, row.choice[k]);
        continue;
      }
      const int axis = k == kKindRows ? 0 : (k == kKindStrided ? 1 : 2);
      const int op = k == kKindConv ? OP_CONV : (k == kKindConvFz ? OP_CONV_FZ : OP_FWD);
      const long long fv = k == kKindConvFz ? (long long)V : 0;
      for (int v = 0; v < 2 && err == cudaSuccess; ++v) {
        auto run = [&]() {
          return launch_axis_pass_variant(n, axis, op, data, data, spec, fv, nvol, 1.f, g.tw512, s, v);
        };
        for (int w = 0; w < 2 && err == cudaSuccess; ++w) err = run();
        cudaEventRecord(e0, s);
        for (int t = 0; t < 5 && err == cudaSuccess; ++t) err = run();
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        row.us[v][k] = 1000.0 * ms / 5.0;
        count_launches(7);
      }
      row.choice[k] = row.us[1][k] < row.us[0][k] ? 1 : 0;
      set_pass_variant(n, k, row.choice[k]);
    }
    g_tuned.erase(std::remove_if(g_tuned.begin(), g_tuned.end(), [&](const TuneRow &t) { return t.n == n; }),
                  g_tuned.end());
    g_tuned.push_back(row);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return cuda_fail(err, "autotune");
  if (const unsigned st = read_and_clear_device_status()) {
    set_err("autotune: device status " + std::to_string(st));
    return kErrCuda;
  }
  if (write_cache && !g.plan_path.empty() && !write_plan_cache(g.plan_path)) {
    set_err("autotune: cannot write the plan cache " + g.plan_path);
    return kErrInval;
  }
  return 0;
}

int bridge_plan_variant(unsigned n, int kind, int set_to) {
  if (!valid_n(n) || kind < 0 || kind >= kPassKinds) return kErrInval;
  if (set_to >= 0) set_pass_variant((int)n, kind, set_to);
  return get_pass_variant((int)n, kind);
}

// ------------------------------------------------------------------ bridge: misc
int bridge_device_info(int *device, int *pageable_access, int *sm_count) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_init_locked();
  if (rc) return rc;
  if (device) *device = g.device;
  if (pageable_access) *pageable_access = g.pageable_access;
  if (sm_count) *sm_count = g.sm_count;
  return 0;
}

unsigned long long bridge_launch_count() { return g_launches.load(); }

int bridge_pass_timing(int mode, double *ms, unsigned long long *launches, double *bytes) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  auto clear = [] {
    for (auto &r : g_prof_recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    g_prof_recs.clear();
  };
  if (mode == 0 || mode == 1) {
    if (g.init) cudaDeviceSynchronize();
    clear();
    g_prof = (mode == 1);
    return 0;
  }
  if (mode != 2 || !ms || !launches || !bytes) return kErrInval;
  for (int i = 0; i < kSlots; ++i) {
    ms[i] = 0.0;
    launches[i] = 0;
    bytes[i] = 0.0;
  }
  for (auto &r : g_prof_recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f;
    if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) return cuda_fail(cudaGetLastError(), "pass timing");
    ms[r.slot] += t;
    launches[r.slot] += 1;
    bytes[r.slot] += r.bytes;
  }
  return 0;
}

const char *bridge_last_error() { return g_err.c_str(); }

int bridge_host_alloc_pinned(size_t bytes, void **ptr) {
  if (!ptr) return kErrInval;
  *ptr = nullptr;
  if (bytes == 0) return 0;
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc");
  return 0;
}

int bridge_host_free_pinned(void *ptr) {
  if (!ptr) return 0;
  cudaError_t e = cudaFreeHost(ptr);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFreeHost");
  return 0;
}

int bridge_device_status(unsigned *status) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (!status) return kErrInval;
  int rc = ensure_init_locked();
  if (rc) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "synchronize");
  *status = read_and_clear_device_status();
  return 0;
}

int bridge_debug_wait_limit(int probes) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_init_locked();
  if (rc) return rc;
  const cudaError_t e = set_dependency_wait_limit(probes);
  if (e != cudaSuccess) return cuda_fail(e, "dependency wait limit");
  return 0;
}

int bridge_debug_fail_allocations(unsigned count) {
  fail_next_allocations(count);
  return 0;
}

int bridge_sync() {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "synchronize");
  return 0;
}

}  // namespace convgpu
