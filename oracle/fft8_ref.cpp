/*
 * Test infrastructure only (part of the oracle, never linked into the product).
 *
 * Host driver around the reference's own FPGA FFT engine. The engine source
 * (kernels/fft/fft_8.cl, pc2/ConvFPGA) is compiled unchanged through fft8_shim.h;
 * this file only feeds it the way the reference kernels do and reads its outputs:
 *
 *  - input distribution: at step k (0 <= k < N/8) lane j carries
 *    x[bitrev3(j) * N/8 + k]                 (kernels/matrixTranspose/diagonal_bitrev.cl:17-26,
 *                                             used by fetch, kernels/conv3D.cl:24-69)
 *  - N/8 input steps followed by N/8 - 1 zero steps; outputs are valid from step
 *    N/8 - 1 on                              (kernels/conv3D.cl:85-112, fft3da)
 *  - the step index passed to fft_step is i mod N/8 (kernels/conv3D.cl:103)
 *  - outputs leave the engine in bit-reversed order (kernels/fft/fft_8.cl:28-30);
 *    fft8ref_1d_raw returns that raw order, the 3D helpers undo it.
 *  - the pointwise product uses the engine's comp_mult (kernels/fft/fft_8.cl:180-185),
 *    as the conv3D kernel does (kernels/conv3D.cl:517-570).
 *
 * Inverse transforms are the engine's unnormalised backward DFT
 * (kernels/fft/fft_8.cl:280-282, 346-348), so conv outputs carry a factor N^3,
 * exactly as the reference library returns them.
 *
 * Built by oracle/Makefile into oracle/_ref/libfft8ref.so, only where the reference
 * sources are present.
 */
#include "fft8_shim.h"
#include "fft/fft_8.cl"

#include <cstddef>
#include <cstring>
#include <vector>

namespace {

unsigned bitrev(unsigned v, int bits) {
  unsigned r = 0;
  for (int b = 0; b < bits; ++b) r |= ((v >> b) & 1u) << (bits - 1 - b);
  return r;
}

void set_lane(float2x8 &d, int j, float2 v) {
  switch (j) {
    case 0: d.i0 = v; break;
    case 1: d.i1 = v; break;
    case 2: d.i2 = v; break;
    case 3: d.i3 = v; break;
    case 4: d.i4 = v; break;
    case 5: d.i5 = v; break;
    case 6: d.i6 = v; break;
    default: d.i7 = v; break;
  }
}

float2 get_lane(const float2x8 &d, int j) {
  switch (j) {
    case 0: return d.i0;
    case 1: return d.i1;
    case 2: return d.i2;
    case 3: return d.i3;
    case 4: return d.i4;
    case 5: return d.i5;
    case 6: return d.i6;
    default: return d.i7;
  }
}

// One length-N transform through the engine; `out` receives the engine's raw
// (bit-reversed) output order.
void engine_1d(int logN, bool inverse, const float2 *in, float2 *out) {
  const int n = 1 << logN;
  const int steps = n / 8;
  std::vector<float2> delay(static_cast<size_t>(n + 8 * (logN - 2)), float2{0.f, 0.f});
  for (int i = 0; i < 2 * steps - 1; ++i) {
    float2x8 d;
    for (int j = 0; j < 8; ++j) {
      float2 v{0.f, 0.f};
      if (i < steps) v = in[bitrev(static_cast<unsigned>(j), 3) * steps + i];
      set_lane(d, j, v);
    }
    d = fft_step(d, i % steps, delay.data(), inverse, logN);
    if (i >= steps - 1) {
      const int m = i - (steps - 1);
      for (int j = 0; j < 8; ++j) out[8 * m + j] = get_lane(d, j);
    }
  }
}

// Natural-order transform of a strided pencil (in place).
void engine_pencil(int logN, bool inverse, float2 *base, size_t stride,
                   std::vector<float2> &tmp_in, std::vector<float2> &tmp_out) {
  const int n = 1 << logN;
  for (int i = 0; i < n; ++i) tmp_in[i] = base[static_cast<size_t>(i) * stride];
  engine_1d(logN, inverse, tmp_in.data(), tmp_out.data());
  for (int p = 0; p < n; ++p) base[static_cast<size_t>(bitrev(p, logN)) * stride] = tmp_out[p];
}

void engine_3d(int logN, bool inverse, float2 *vol) {
  const size_t n = static_cast<size_t>(1) << logN;
  std::vector<float2> a(n), b(n);
  for (size_t z = 0; z < n; ++z)            // x axis, contiguous
    for (size_t y = 0; y < n; ++y) engine_pencil(logN, inverse, vol + (z * n + y) * n, 1, a, b);
  for (size_t z = 0; z < n; ++z)            // y axis, stride N
    for (size_t x = 0; x < n; ++x) engine_pencil(logN, inverse, vol + z * n * n + x, n, a, b);
  for (size_t y = 0; y < n; ++y)            // z axis, stride N^2
    for (size_t x = 0; x < n; ++x) engine_pencil(logN, inverse, vol + y * n + x, n * n, a, b);
}

}  // namespace

extern "C" {

// Raw engine output order (bit-reversed) for one length-2^logN transform.
int fft8ref_1d_raw(int logN, int inverse, const float *in, float *out) {
  if (logN < 4 || logN > 12 || in == nullptr || out == nullptr) return -1;
  engine_1d(logN, inverse != 0, reinterpret_cast<const float2 *>(in), reinterpret_cast<float2 *>(out));
  return 0;
}

// In-place natural-order 3D transform of one N^3 cube (x fastest).
int fft8ref_fft3d(int logN, int inverse, float *vol) {
  if (logN < 4 || logN > 9 || vol == nullptr) return -1;
  engine_3d(logN, inverse != 0, reinterpret_cast<float2 *>(vol));
  return 0;
}

// out[b] = IFFT3(FFT3(sig[b]) (.) FFT3(filter[b or 0])), unnormalised; the same
// pipeline as fpgaf_conv3D / fpgaf_conv3D_svm_batch with the FPGA arithmetic.
int fft8ref_conv3d(int logN, unsigned batch, const float *sig, const float *filter, float *out,
                   int filter_per_signal) {
  if (logN < 4 || logN > 9 || sig == nullptr || filter == nullptr || out == nullptr) return -1;
  const size_t pts = static_cast<size_t>(1) << (3 * logN);
  const unsigned nfilt = filter_per_signal ? batch : 1u;
  std::vector<float2> fspec(pts * nfilt);
  std::memcpy(fspec.data(), filter, sizeof(float2) * pts * nfilt);
  for (unsigned f = 0; f < nfilt; ++f) engine_3d(logN, false, fspec.data() + f * pts);
  float2 *o = reinterpret_cast<float2 *>(out);
  std::memcpy(o, sig, sizeof(float2) * pts * batch);
  for (unsigned b = 0; b < batch; ++b) {
    float2 *v = o + b * pts;
    const float2 *f = fspec.data() + (filter_per_signal ? b : 0u) * pts;
    engine_3d(logN, false, v);
    for (size_t i = 0; i < pts; ++i) v[i] = comp_mult(v[i], f[i]);
    engine_3d(logN, true, v);
  }
  return 0;
}

}  // extern "C"
