// Device building blocks for the per-axis FFT passes (sm_103a).
//
// A length-N transform of one pencil is spread over T = N/E threads; thread t holds
// the E elements n = t + e*T (e = 0..E-1) in registers ("t + e*T order"). A plan is a
// list of radices R_0 * R_1 * ... = N, each dividing E. One radix-R stage is a
// Stockham autosort step: butterfly b (0 <= b < N/R, thread t owns b = t + i*T) reads
// elements b + r*N/R, multiplies input r by W_{Ns*R}^{r*(b mod Ns)} (Ns = product of the
// radices before it), runs an R-point DFT and writes output r' to position
// (b/Ns)*Ns*R + (b mod Ns) + r'*Ns. Stages exchange through shared memory; the last
// stage's outputs land back in the thread's own registers in t + e*T order, so
// natural-order results go straight to global memory. This replaces the reference's
// streaming radix-2^2 feed-forward engine with bit-reversed output
// (kernels/fft/fft_8.cl:275-351) and the bit-reversal / transpose buffers around it
// (kernels/matrixTranspose/diagonal_bitrev.cl:3-223): there is no reordering pass.
//
// Forward transforms use W = exp(-2*pi*i/N); the inverse is the unnormalised backward
// transform, computed as swap(re,im) -> forward -> swap(re,im), the same identity the
// reference engine uses (kernels/fft/fft_8.cl:280-282, 346-348).
#pragma once

#include <cuda_runtime.h>

namespace convgpu {

// Complex add / subtract as one packed two-lane FP32 instruction (add/sub.rn.f32x2,
// sm_100 and later): each lane rounds like a scalar add, half the instructions.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "add.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
// a * b; expression order of comp_mult (kernels/fft/fft_8.cl:180-185).
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cswap(float2 a) { return make_float2(a.y, a.x); }
// a * (-i)
__device__ __forceinline__ float2 cmul_negi(float2 a) { return make_float2(a.y, -a.x); }

// cos(2*pi*m/32) for m = 0..8 (quarter wave of the 32nd roots of unity).
__device__ __forceinline__ float cos32_q(int m) {
  switch (m) {
    case 0: return 1.0f;
    case 1: return 0.98078528040323044913f;
    case 2: return 0.92387953251128675613f;
    case 3: return 0.83146961230254523708f;
    case 4: return 0.70710678118654752440f;
    case 5: return 0.55557023301960222474f;
    case 6: return 0.38268343236508977173f;
    case 7: return 0.19509032201612826785f;
    default: return 0.0f;
  }
}
// cos(2*pi*m/32) and sin(2*pi*m/32) for m = 0..31 by quadrant symmetry.
__device__ __forceinline__ float cos32(int m) {
  m &= 31;
  if (m <= 8) return cos32_q(m);
  if (m <= 16) return -cos32_q(16 - m);
  if (m <= 24) return -cos32_q(m - 16);
  return cos32_q(32 - m);
}
__device__ __forceinline__ float sin32(int m) { return cos32(m - 8); }

// v * W_R^k with W_R = exp(-2*pi*i/R), R | 32. k is a compile-time constant after
// unrolling, so the special cases fold away.
template <int R>
__device__ __forceinline__ float2 mul_wconst(float2 v, int k) {
  const int m = (k * (32 / R)) & 31;
  if (m == 0) return v;
  if (m == 8) return cmul_negi(v);
  if (m == 16) return make_float2(-v.x, -v.y);
  if (m == 24) return make_float2(-v.y, v.x);
  const float c = cos32(m), s = sin32(m);
  if (m == 4 || m == 12 || m == 20 || m == 28) {
    // |c| == |s| == sqrt(2)/2: two multiplies instead of four.
    const float h = 0.70710678118654752440f;
    const float re = (c > 0.f ? v.x : -v.x) + (s > 0.f ? v.y : -v.y);
    const float im = (c > 0.f ? v.y : -v.y) - (s > 0.f ? v.x : -v.x);
    return make_float2(re * h, im * h);
  }
  // (v.x + i v.y) * (c - i s)
  return make_float2(v.x * c + v.y * s, v.y * c - v.x * s);
}

// In-register forward DFT of R points, natural order in and out.
template <int R>
__device__ __forceinline__ void dft(float2 (&x)[R]) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    const float2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  } else if constexpr (R == 4) {
    const float2 t0 = cadd(x[0], x[2]), t1 = csub(x[0], x[2]);
    const float2 t2 = cadd(x[1], x[3]), t3 = csub(x[1], x[3]);
    x[0] = cadd(t0, t2);
    x[2] = csub(t0, t2);
    x[1] = cadd(t1, cmul_negi(t3));
    x[3] = csub(t1, cmul_negi(t3));
  } else {
    // Radix-2 decimation in time over two R/2-point DFTs.
    constexpr int H = R / 2;
    float2 e[H], o[H];
#pragma unroll
    for (int k = 0; k < H; ++k) {
      e[k] = x[2 * k];
      o[k] = x[2 * k + 1];
    }
    dft<H>(e);
    dft<H>(o);
#pragma unroll
    for (int k = 0; k < H; ++k) {
      const float2 t = mul_wconst<R>(o[k], k);
      x[k] = cadd(e[k], t);
      x[k + H] = csub(e[k], t);
    }
  }
}

// Compile-time list of radices.
template <int... Rs>
struct Radices {};

template <int N, int E, class Plan>
struct PlanCheck;
template <int N, int E, int... Rs>
struct PlanCheck<N, E, Radices<Rs...>> {
  static constexpr int product = (Rs * ... * 1);
  static_assert(product == N, "radices must multiply to N");
  static_assert(((E % Rs == 0) && ...), "every radix must divide E");
  static constexpr int stages = sizeof...(Rs);
};

// Twiddle W_N^(r*k*N/(NS*R)) of input r of a butterfly with k = b mod NS, from a linear
// table tw[j] = W_N^j.
template <int N, int NS, int R>
__device__ __forceinline__ float2 stage_tw(const float2 *tw, int r, int k) {
  return tw[r * k * (N / (NS * R))];
}
// The same twiddles for the second stage of a 16 x 16 plan (N = 256) from a table laid out
// t[r*16 + k] = W_256^(r*k): threads with consecutive k read consecutive entries, where the
// linear table's r*k strides put up to 8 of a warp's reads in one bank.
struct TwRT256 {
  const float2 *t;
};
template <int N, int NS, int R>
__device__ __forceinline__ float2 stage_tw(const TwRT256 &tw, int r, int k) {
  static_assert(N == 256 && NS == 16 && R == 16, "TwRT256 serves the second stage of a 16 x 16 plan");
  return tw.t[r * 16 + k];
}

// One Stockham stage on registers v (t + e*T order on entry). When LAST is false the
// outputs are written to `sm` via `sidx` and read back in t + e*T order by the caller
// after a barrier. Twiddles come from `tw` through stage_tw.
//
//   SIdx: functor mapping a pencil position (0..N-1) to a shared-memory slot.
template <int N, int E, int R, int NS, bool LAST, class SIdx, class TW>
__device__ __forceinline__ void stockham_stage(float2 (&v)[E], int t, const TW &tw, float2 *sm, const SIdx &sidx) {
  constexpr int T = N / E;
  constexpr int B = E / R;  // butterflies per thread
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int b = t + i * T;
    const int k = b % NS;
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; ++r) x[r] = v[i + r * B];
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) x[r] = cmul(x[r], stage_tw<N, NS, R>(tw, r, k));
    }
    dft<R>(x);
    if constexpr (LAST) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[i + r * B] = x[r];
    } else {
      const int base = (b / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) sm[sidx(base + r * NS)] = x[r];
    }
  }
}

}  // namespace convgpu
