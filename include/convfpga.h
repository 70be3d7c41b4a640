/*
 * convfpga.h — drop-in C API of the GB300 FFT-based 3D convolution library.
 *
 * Same types and entry points as pc2/ConvFPGA's public header
 * (host/include/convfpga/convfpga.h:16-46), so a program written against that
 * library compiles and links against libconvgpu.so unchanged. Semantics kept:
 *
 *   out = IFFT3( FFT3(sig) (.) FFT3(filter) ), UNNORMALISED (a factor N^3 larger than a
 *   normalised circular convolution), complex64 cubes of N^3 points, x fastest
 *   (idx = z*N*N + y*N + x); all pointers are caller-owned HOST memory; the library
 *   copies in and out and keeps no pointer after the call returns.
 *
 * Differences from the FPGA library, all in the caller's favour:
 *   - N is a run-time argument: every power of two 16..512 works with one build
 *     (the FPGA bitstream fixes N at synthesis; a different N went undetected).
 *   - runtime errors return fpga_t{valid = false} instead of calling exit().
 *   - fpgaf_conv3D_svm_batch accepts any how_many, odd counts included, and distinct
 *     signals per batch slot.
 *   - calls made before fpga_initialize initialise the current CUDA device lazily.
 * Extensions (device pointers, streams, per-signal filters, 1/N^3 normalisation,
 * uneven batches) are declared in convgpu.h.
 */
#ifndef CONVGPU_CONVFPGA_H
#define CONVGPU_CONVFPGA_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Single-precision complex value, interleaved (real, imaginary).
 * Replaces: host/include/convfpga/convfpga.h:16-19. */
typedef struct {
  float x; /* real */
  float y; /* imaginary */
} float2;

/* Per-call timings in milliseconds, from device events.
 * Replaces: host/include/convfpga/convfpga.h:24-34.
 *   filter_pcie_wr_t  host->device copy of the filter
 *   filter_exec_t     filter 3D FFT
 *   sig_pcie_wr_t     host->device copy of the signal(s)
 *   sig_pcie_rd_t     device->host copy of the result(s)
 *   sig_exec_t        single call: forward passes + fused z (FFT, multiply, iFFT);
 *                     batch call: sum over signals of their compute time
 *   siginv_exec_t     single call: remaining inverse passes;
 *                     batch call: wall span from first to last signal compute
 *   valid             true when the call completed */
typedef struct fpga_timing {
  double filter_pcie_wr_t;
  double filter_exec_t;
  double sig_pcie_wr_t;
  double sig_pcie_rd_t;
  double sig_exec_t;
  double siginv_exec_t;
  bool valid;
} fpga_t;

/* Selects and prepares the GPU.
 * Replaces: host/include/convfpga/convfpga.h:36 (host/src/fpga_init.c:57-121).
 *   platform_name  "cuda:K" / "gpu:K" selects device K; any other string (including
 *                  the Intel FPGA platform names) or NULL selects device 0.
 *   path           must be non-empty, as for the bitstream path; names the plan-cache
 *                  file of the autotuner.
 *   use_svm        require that the device can address host memory.
 * Returns 0, or -1 path NULL/empty, -2 "cuda:K" names no device, -3 no CUDA device,
 * -4 this library's kernels cannot load on the device, -5 host memory not addressable. */
int fpga_initialize(const char *platform_name, const char *path, const bool use_svm);

/* Releases every device resource of the library.
 * Replaces: host/include/convfpga/convfpga.h:38 (host/src/fpga_init.c:127-137). */
void fpga_final(void);

/* 64-byte aligned host allocation for sz bytes; NULL when sz == 0; release with free().
 * Replaces: host/include/convfpga/convfpga.h:40 (host/src/fpga_init.c:37-43). */
void *fpgaf_complex_malloc(const size_t sz);

/* One convolution of N^3 points (sig, filter, out: N^3 float2 each).
 * Replaces: host/include/convfpga/convfpga.h:42 (host/src/convfpga.c:32-409).
 * valid = false for NULL pointers or N not a power of two in 16..512. */
fpga_t fpgaf_conv3D(const unsigned N, const float2 *sig, const float2 *filter, float2 *out);

/* As fpgaf_conv3D; the SVM variant of the reference streams host memory directly.
 * Replaces: host/include/convfpga/convfpga.h:44 (host/src/convfpga_svm.c:34-461). */
fpga_t fpgaf_conv3D_svm(const unsigned N, const float2 *sig, const float2 *filter, float2 *out);

/* how_many convolutions against one shared filter; sig and out hold how_many * N^3
 * float2, signal i at offset i * N^3. Host<->device copies overlap the compute.
 * Replaces: host/include/convfpga/convfpga.h:46 (host/src/convfpga_svm_batch.c:36-724). */
fpga_t fpgaf_conv3D_svm_batch(const unsigned N, const float2 *sig, const float2 *filter, float2 *out,
                              const unsigned how_many);

#ifdef __cplusplus
}
#endif

#endif /* CONVGPU_CONVFPGA_H */
