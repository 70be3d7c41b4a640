// Internal interface between the CUDA translation units (kernels + runtime).
// Uses CUDA's float2; never include the public convfpga.h next to this header
// (that header declares its own `float2`).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "abi_bridge.h"

namespace convgpu {

// Launches one per-axis pass over `nvol` cubes of size n (axis 0 = x, 1 = y, 2 = z).
// op: OP_FWD / OP_INV / OP_CONV / OP_CONV_FZ (passes.cuh). src may equal dst.
cudaError_t launch_axis_pass(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                             long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                             cudaStream_t s);

// x pass of `nvol` cubes of real data (N^3 floats each) into complex dst: the first pass of
// a real filter's transform (CONVGPU_FILTER_REAL).
cudaError_t launch_axis_pass_real(int n, const float *src, float2 *dst, int nvol, const float2 *tw512,
                                  cudaStream_t s);

// Hermitian half spectra of real filters (herm.cuh), N >= 64: axis 0 (OP_FWD) transforms
// real rows (src: N^3 floats per cube) into the half layout of pitch half_spectrum_pitch(n)
// (N * N * pitch values per cube); axis 1 / 2 (OP_FWD) transform that layout in place;
// axis 2 OP_CONV runs the signals' paired fused z pass against a half spectrum `filt`
// (filt_vol_elems: 0 shared, N*N*pitch per signal). cudaErrorNotSupported below N = 64
// or when tensor maps cannot describe the operands.
cudaError_t launch_axis_pass_half(int n, int axis, int op, const void *src, float2 *dst, const float2 *filt,
                                  long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                  cudaStream_t s);
int half_spectrum_pitch(int n);

// Split precision of the tensor-core path.
constexpr int kTcTf32x3 = 0;
constexpr int kTcBf16x3 = 1;

// As launch_axis_pass, with the radix-16 stages on the tensor cores (split operands,
// FP32 accumulate) where a tensor-core kernel exists (N = 256); FP32 kernels otherwise.
cudaError_t launch_axis_pass_tc(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                                long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                cudaStream_t s, int prec);

// Selects the TMA-fed y / z pass kernels (default) or the register-gather kernels.
void set_tma_enabled(bool on);

// Twiddle buffer of the engine: 512 twiddles W512^j followed by the constant block of
// the tcgen05 kernels (B operand hi / lo, W256^j), written by tc05_init_consts.
constexpr size_t kTwiddleBufBytes = 512 * 8 + 2 * 4096 + 256 * 8;
cudaError_t tc05_init_consts(float2 *tw, cudaStream_t s);

// Plan table: shape variant (0 / 1) per cube size and pass kind, chosen by the
// autotuner and recorded in the plan cache.
// kKindTc: tensor-core kernel of the split-TF32 path (0 tcgen05, 1 mma.sync), N = 256.
// kKindTcXy: x and y passes of the split-TF32 path on tcgen05, N = 256 (0 separate passes,
// 1 one pass staged through the L2 scratch ring).
// kKindHalf: spectra of real filters (CONVGPU_FILTER_REAL), N >= 64: 0 full, 1 Hermitian
// half spectra with the paired fused z pass (herm.cuh).
constexpr int kKindRows = 0, kKindStrided = 1, kKindConv = 2, kKindConvFz = 3, kKindXy = 4, kKindTc = 5,
              kKindTcXy = 6, kKindHalf = 7, kPassKinds = 8;
// Tensor-core form of the L2-staged x + y pass (tcgen05; xyl2.cu). It exists for N = 256
// only: any other n returns cudaErrorNotSupported without launching.
cudaError_t launch_xy_l2_tc_pass(int n, const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                                 const float2 *tw512, cudaStream_t s);
int pass_kind(int axis, int op);
void set_pass_variant(int n, int kind, int variant);
int get_pass_variant(int n, int kind);
// Fused x + y pass over `nplanes` planes (N = 128, 256, 512; cudaErrorNotSupported otherwise
// or when tensor maps cannot describe the operands). Plan kind kKindXy, N = 256: variant 1
// stages the x-transformed planes through an L2-resident scratch ring (one persistent
// kernel), variant 2 keeps each plane in the shared memory of an 8-CTA cluster; N = 128
// and 512: variant 1 is the L2-staged pass (16-row / 16-column and 4-row / 4-column items).
cudaError_t launch_xy_pass(int n, const float2 *src, float2 *dst, int nplanes, bool inverse, float scale,
                           const float2 *tw512, cudaStream_t s, int variant);
// x or y pass (FWD / INV) over `nplanes` consecutive N x N planes starting at src / dst
// (a slab of a cube; planes are independent for these axes).
cudaError_t launch_axis_pass_planes(int n, int axis, int op, const float2 *src, float2 *dst, int nplanes, float scale,
                                    const float2 *tw512, cudaStream_t s);
// launch_axis_pass with an explicit shape variant (the autotuner times both).
cudaError_t launch_axis_pass_variant(int n, int axis, int op, const float2 *src, float2 *dst, const float2 *filt,
                                     long long filt_vol_elems, int nvol, float scale, const float2 *tw512,
                                     cudaStream_t s, int variant);

// Table-mode launches (one launch over cubes at unrelated addresses): per-volume tensor
// maps of the source (and, for the fused z pass, of the filter spectrum) and per-volume
// destination bases, all in device memory. encode_table_map fills the map of one cube
// for kind 0 (rows, x pass), 1 (y pass) or 2 (z pass) with the box of that size's kernel.
#include <cuda.h>
bool encode_table_map(CUtensorMap *m, const void *cube, int n, int kind);
// Sets the kernel attributes the table-mode launches of size n need (call before a
// stream capture that contains them).
cudaError_t prepare_table_launches(int n);
cudaError_t launch_axis_pass_table(int n, int axis, int op, const CUtensorMap *maps, const CUtensorMap *fmaps,
                                   float2 *const *dsts, int nvol, float scale, const float2 *tw512,
                                   cudaStream_t s);
// Uneven batch as one CUDA graph of per-size table-mode launches (grouped.cu).
int uneven_grouped(const struct UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt,
                   void *d_out, bool normalize, const float2 *tw512, cudaStream_t stream, std::string &err);
void release_grouped_plans();
void release_xy_l2();
// L2-staged fused x + y pass (N = 256 or 128) over cubes at unrelated addresses (table
// mode): per-cube rows maps (encode_xy_table_map, in device memory), per-cube output bases
// and caller-owned dependency counters of xy_l2_counter_bytes(n, ncubes) bytes.
// prepare_xy_l2 allocates the size's scratch ring and sets the kernel attributes (call it
// before a capture).
cudaError_t prepare_xy_l2(int n);
size_t xy_l2_counter_bytes(int n, int ncubes);
bool encode_xy_table_map(CUtensorMap *m, const void *cube, int n);
cudaError_t launch_xy_l2_table(int n, const CUtensorMap *rmaps, float2 *const *dsts, int ncubes, bool inverse,
                               float scale, const float2 *tw512, unsigned *status, unsigned *ctr, cudaStream_t s);

// Device address of the status word (for kernels outside passes.cu).
unsigned int *device_status_address();

// Uneven batch through the persistent work-queue launch (persistent.cu). Plans (work
// items, counters, spectrum workspace, CUDA graph) are cached per sequence of sizes.
// Returns 0 or a CONVGPU_E* code with `err` set.
int uneven_persistent(const struct UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt,
                      void *d_out, bool normalize, const float2 *tw512, unsigned *status, cudaStream_t stream,
                      std::string &err);
void release_uneven_plans();
// One convolution of a small cube (N = 16, 32, 64) in one cooperative launch (persistent.cu);
// spec: N^3 of workspace. cudaErrorNotSupported when it does not apply.
cudaError_t launch_small_conv(int n, const float2 *sig, const float2 *filt, float2 *out, float2 *spec, float scale,
                              bool real, const float2 *tw512, unsigned *status, cudaStream_t s);

// Returns and clears the device status word (kStatus* bits; ~0 if it cannot be read).
unsigned int read_and_clear_device_status();
// Testing hook: every dependency wait (counters advanced by other CTAs) gives up after
// `probes` probes; probes < 0 restores each wait's own limit. Waits for the device first.
cudaError_t set_dependency_wait_limit(int probes);
// Testing hook: the next `count` allocations of the runtime's grow-only device buffers
// fail as out of memory.
void fail_next_allocations(unsigned count);

// Checks that this library's kernel image loads on the current device.
cudaError_t probe_kernel_image();

// Sets the calling thread's convgpu_last_error() text.
void record_error(const char *msg);

// Entry point without device allocations (noalloc.cu); returns 0 or a CONVGPU_E* code.
int conv_device_noalloc(unsigned n, const void *d_sig, const void *d_filt, void *d_out, unsigned how_many,
                        unsigned flags, void *stream);

// Counts kernel launches issued by this library (host-side, monotonic).
void count_launches(unsigned long long k);

}  // namespace convgpu
