// convgpu_conv3d_device_noalloc: the device-pointer convolution for callers that must
// not allocate device memory.
//
// Who needs it: programs whose device memory belongs to another allocator (a framework's
// caching allocator or a memory pool sized once at start-up, where a foreign cudaMalloc
// can fail or fragment the pool), and steady-state loops that cannot afford the implicit
// device-wide synchronisation of cudaMalloc / cudaFree. The regular entry point,
// convgpu_conv3d_device, grows a workspace with cudaMalloc on first use of a size and
// creates streams and a twiddle table on first call; this one does neither.
//
// How: the only scratch the convolution needs is the filter spectrum. Here it lives in
// the file-scope array g_noalloc_scratch below, a fixed 16 MiB (kNoAllocScratchElems
// complex64 values) that every GPU which loads this library holds until the process
// exits. The twiddle table is a second file-scope array (4 KiB). On the first call on a
// device, with that device current, the host looks up both arrays' device addresses
// with cudaGetSymbolAddress and fills the twiddle table with cudaMemcpyToSymbol; that
// set-up runs once per device, so the first call should come before any stream capture.
// In host code the arrays' names are host-side stand-ins, not device addresses, so only
// the looked-up addresses are ever passed to kernels.
//
// Limits and sharing: a call needs how_many*N^3 scratch elements with
// CONVGPU_FILTER_PER_SIGNAL, N^3 for a shared filter and none with
// CONVGPU_FILTER_IS_SPECTRUM; larger requests return CONVGPU_EINVAL. Every call uses the
// same array, which keeps the previous call's contents; nothing in it has to start at
// zero, because each call's first filter pass writes every element that call later
// reads. Calls that overlap on the GPU (different streams, or host threads without
// ordering) race on the array.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "abi_bridge.h"
#include "engine_internal.h"
#include "passes.cuh"

namespace convgpu {

constexpr size_t kNoAllocScratchElems = size_t(1) << 21;  // 16 MiB of complex64
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocScratchElems];
static __device__ __align__(256) float2 g_noalloc_tw512[512];

namespace {
struct NoAllocDevice {
  bool ready = false;
  float2 *scratch = nullptr;  // device address of g_noalloc_scratch on this device
  float2 *tw512 = nullptr;    // device address of g_noalloc_tw512 on this device
};
NoAllocDevice g_dev[kNoAllocMaxDevices];
std::mutex g_setup_mu;
int fail(const std::string &msg, int code) {
  record_error(msg.c_str());
  return code;
}

// Once per device, with that device current: resolve the arrays' device addresses and
// fill the twiddle table (exp(-2*pi*i*j/512) in FP64, rounded to FP32).
int setup_device(int dev, NoAllocDevice **out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  NoAllocDevice &d = g_dev[dev];
  if (!d.ready) {
    cudaError_t e = cudaGetSymbolAddress((void **)&d.scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e), -3);
    e = cudaGetSymbolAddress((void **)&d.tw512, g_noalloc_tw512);
    if (e != cudaSuccess) return fail(std::string("cudaGetSymbolAddress(twiddles): ") + cudaGetErrorString(e), -3);
    float2 h[512];
    const double two_pi = 6.283185307179586476925286766559;
    for (int j = 0; j < 512; ++j) {
      const double a = -two_pi * (double)j / 512.0;
      h[j] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    e = cudaMemcpyToSymbol(g_noalloc_tw512, h, sizeof(h));
    if (e != cudaSuccess) return fail(std::string("cudaMemcpyToSymbol(twiddles): ") + cudaGetErrorString(e), -3);
    d.ready = true;
  }
  *out = &d;
  return 0;
}
}  // namespace

int conv_device_noalloc(unsigned n, const void *d_sig, const void *d_filt, void *d_out, unsigned how_many,
                        unsigned flags, void *stream) {
  constexpr unsigned kNormalize = 1u << 0, kPerSignal = 1u << 1, kIsSpectrum = 1u << 2, kTensor = 1u << 3,
                     kReal = 1u << 9;
  if (!d_sig || !d_filt || !d_out || n < 16 || n > 512 || (n & (n - 1)) != 0)
    return fail("invalid arguments: null pointer or N not a power of two in 16..512", -1);
  if (flags & kTensor) return fail("the no-allocation entry point runs the plain FP32 path only", -5);
  if (flags & kReal) return fail("CONVGPU_FILTER_REAL is not supported by the no-allocation entry point", -5);
  if (how_many == 0) return 0;
  const size_t V = (size_t)n * n * n;
  const size_t need = (flags & kIsSpectrum) ? 0 : ((flags & kPerSignal) ? V * how_many : V);
  if (need > kNoAllocScratchElems)
    return fail("filter spectra need " + std::to_string(need) + " complex values of scratch; this entry point has " +
                    std::to_string(kNoAllocScratchElems) + " (16 MiB)",
                -1);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(std::string("cudaGetDevice: ") + cudaGetErrorString(e), -3);
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail("device index out of range", -1);
  NoAllocDevice *d = nullptr;
  int rc = setup_device(dev, &d);
  if (rc) return rc;

  cudaStream_t s = (cudaStream_t)stream;
  const float2 *sig = (const float2 *)d_sig;
  const float2 *filt = (const float2 *)d_filt;
  float2 *out = (float2 *)d_out;
  const float scale = (flags & kNormalize) ? (float)(1.0 / (double)V) : 1.0f;
  const float2 *spec = filt;
  long long spec_vol = 0;
  int zop = OP_CONV;
  unsigned long long launches = 0;
  auto run = [&](int axis, int op, const float2 *src, float2 *dst, const float2 *f, long long fv, int nvol,
                 float sc) {
    if (e != cudaSuccess) return;
    e = launch_axis_pass((int)n, axis, op, src, dst, f, fv, nvol, sc, d->tw512, s);
    if (e == cudaSuccess) ++launches;
  };
  if (flags & kIsSpectrum) {
    spec_vol = (flags & kPerSignal) ? (long long)V : 0;
  } else if (flags & kPerSignal) {
    run(0, OP_FWD, filt, d->scratch, nullptr, 0, (int)how_many, 1.f);
    run(1, OP_FWD, d->scratch, d->scratch, nullptr, 0, (int)how_many, 1.f);
    spec = d->scratch;
    spec_vol = (long long)V;
    zop = OP_CONV_FZ;
  } else {
    run(0, OP_FWD, filt, d->scratch, nullptr, 0, 1, 1.f);
    run(1, OP_FWD, d->scratch, d->scratch, nullptr, 0, 1, 1.f);
    run(2, OP_FWD, d->scratch, d->scratch, nullptr, 0, 1, 1.f);
    spec = d->scratch;
  }
  run(0, OP_FWD, sig, out, nullptr, 0, (int)how_many, 1.f);
  run(1, OP_FWD, out, out, nullptr, 0, (int)how_many, 1.f);
  run(2, zop, out, out, spec, spec_vol, (int)how_many, 1.f);
  run(1, OP_INV, out, out, nullptr, 0, (int)how_many, 1.f);
  run(0, OP_INV, out, out, nullptr, 0, (int)how_many, scale);
  count_launches(launches);
  if (e != cudaSuccess) return fail(std::string("launch: ") + cudaGetErrorString(e), -3);
  return 0;
}

int bridge_conv_device_noalloc(unsigned n, const void *d_sig, const void *d_filt, void *d_out, unsigned how_many,
                               unsigned flags, void *stream) {
  return conv_device_noalloc(n, d_sig, d_filt, d_out, how_many, flags, stream);
}

}  // namespace convgpu
