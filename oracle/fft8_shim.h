/*
 * Test infrastructure only (part of the oracle, never linked into the product).
 *
 * Compatibility shim that lets the reference FPGA FFT engine
 * (kernels/fft/fft_8.cl and kernels/fft/twid_radix4_8.cl of pc2/ConvFPGA) compile
 * as ordinary C++ on the host, unchanged, so that its arithmetic can pin the oracle.
 * It supplies the three OpenCL-C features those two files use:
 *   - the `float2` vector type with component-wise + and -,
 *   - the `constant` address-space qualifier (mapped to `static const`),
 *   - the `M_PI_F` constant.
 */
#ifndef CONVGPU_ORACLE_FFT8_SHIM_H
#define CONVGPU_ORACLE_FFT8_SHIM_H

#include <cmath>

struct float2 {
  float x;
  float y;
};

static inline float2 operator+(float2 a, float2 b) { return float2{a.x + b.x, a.y + b.y}; }
static inline float2 operator-(float2 a, float2 b) { return float2{a.x - b.x, a.y - b.y}; }

#define constant static const
#ifndef M_PI_F
#define M_PI_F 3.14159265358979323846f
#endif

#endif
