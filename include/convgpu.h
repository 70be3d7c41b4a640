/*
 * convgpu.h — extensions of the GB300 FFT convolution library beyond convfpga.h.
 *
 * None of these has a counterpart in pc2/ConvFPGA; each extends one of its entry
 * points, named below. Device-pointer entry points are stream-ordered: they enqueue
 * work on `stream` (a cudaStream_t passed as void*, NULL = legacy default stream)
 * and return without waiting. They return 0 on success or a negative CONVGPU_E*
 * code; convgpu_last_error() describes the last failure of the calling thread.
 *
 * Data layout everywhere: complex64 (float2) cubes of N^3 points, x fastest
 * (idx = z*N*N + y*N + x), cube i of a batch at offset i*N^3.
 */
#ifndef CONVGPU_H
#define CONVGPU_H

#include "convfpga.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Flags */
#define CONVGPU_NORMALIZE (1u << 0)            /* scale outputs by 1/N^3 */
#define CONVGPU_FILTER_PER_SIGNAL (1u << 1)    /* filter holds how_many cubes, one per signal */
#define CONVGPU_FILTER_IS_SPECTRUM (1u << 2)   /* filter already holds FFT3(filter) */
#define CONVGPU_TENSOR_SPLIT (1u << 3)         /* tensor-core path, split TF32 (TF32x3) */
#define CONVGPU_TENSOR_BF16X3 (1u << 4)        /* tensor-core path, BF16x3 split (implies TENSOR_SPLIT) */
#define CONVGPU_UNEVEN_PER_JOB (1u << 5)       /* uneven batch: one job at a time */
#define CONVGPU_UNEVEN_QUEUE (1u << 6)         /* uneven batch: one persistent work-queue launch */
#define CONVGPU_HOST_SLABS (1u << 7)           /* host batch: stream cubes >= 32 MiB in z-slabs */
#define CONVGPU_FILTER_CACHED (1u << 8)        /* host batch: shared filter unchanged since the
                                                  last call with this flag, same pointer and N */
#define CONVGPU_FILTER_REAL (1u << 9)          /* filter is real: N^3 floats per filter cube */

/* Status codes */
#define CONVGPU_OK 0
#define CONVGPU_EINVAL (-1)
#define CONVGPU_ENOTINIT (-2)
#define CONVGPU_ECUDA (-3)
#define CONVGPU_ENOMEM (-4)
#define CONVGPU_EUNSUPPORTED (-5)

/* how_many convolutions on DEVICE pointers, enqueued on `stream`.
 * Extends fpgaf_conv3D_svm_batch (host/include/convfpga/convfpga.h:46) with device
 * buffers, per-signal filters (CONVGPU_FILTER_PER_SIGNAL), precomputed spectra
 * (CONVGPU_FILTER_IS_SPECTRUM), normalisation and the tensor-core path.
 * Tensor-core path: the radix-16 stages of N = 256 transforms run as 16-point DFT
 * matmuls on the tensor cores with split operands and FP32 accumulation (TF32x3:
 * ~1e-7 relative error per 256-point transform; BF16x3: ~4e-6, which exceeds 1e-5
 * relative L2 end to end on 256^3 convolutions). N = 512 with TF32x3 runs a radix-2
 * step on the CUDA cores around two such 256-point transforms. Other N, and BF16x3 at
 * N = 512, run the FP32 kernels.
 * Real filters (CONVGPU_FILTER_REAL): d_filter holds N^3 floats per filter cube (4-byte
 * aligned); the filter's first pass reads them directly, half the bytes of a complex
 * filter, and the result equals that of the same filter given as complex values with
 * zero imaginary parts. Not with CONVGPU_FILTER_IS_SPECTRUM. The reference takes complex
 * filters only; its real Gaussian filters are stored with zero imaginary parts.
 * d_sig may equal d_out (in place). The library's per-device workspace is shared by
 * all calls: calls on different streams must not overlap. */
int convgpu_conv3d_device(unsigned N, const float2 *d_sig, const float2 *d_filter, float2 *d_out,
                          unsigned how_many, unsigned flags, void *stream);

/* As convgpu_conv3d_device, but allocates no device memory: for callers that cannot
 * call cudaMalloc, such as programs whose device memory is owned by another allocator
 * (a framework's caching allocator, a pool sized at start-up) or steady-state loops that
 * cannot take cudaMalloc/cudaFree's device-wide synchronisation. It has no counterpart
 * in pc2/ConvFPGA.
 * Scratch is a fixed 16 MiB device array inside the library (CONVGPU_NOALLOC_SCRATCH_ELEMS
 * complex64 values), held by every GPU that loads the library until the process exits.
 * A call needs how_many*N^3 scratch values with CONVGPU_FILTER_PER_SIGNAL, N^3 for a
 * shared filter and none with CONVGPU_FILTER_IS_SPECTRUM; larger requests return
 * CONVGPU_EINVAL. CONVGPU_TENSOR_SPLIT returns CONVGPU_EUNSUPPORTED.
 * The first call on a device sets that device up (looks up the array's address and
 * fills a twiddle table), so make it before any stream capture. All calls share the
 * array: calls that overlap on the GPU race. Like convgpu_conv3d_device it returns once
 * the work is enqueued; a kernel that gives up a bounded wait reports it through
 * convgpu_device_status, not through this call's return code. */
#define CONVGPU_NOALLOC_SCRATCH_ELEMS (1u << 21)
int convgpu_conv3d_device_noalloc(unsigned N, const float2 *d_sig, const float2 *d_filter, float2 *d_out,
                                  unsigned how_many, unsigned flags, void *stream);

/* Host-buffer batch with the flags above (CONVGPU_FILTER_IS_SPECTRUM excluded). Copies
 * overlap compute on separate streams; pinned buffers (convgpu_host_alloc) copy fastest.
 * Filter-spectrum cache: with CONVGPU_FILTER_CACHED and a shared filter, the caller states
 * that the filter behind this host pointer has not changed since the last call that
 * passed the same pointer, N and tensor-core flags with CONVGPU_FILTER_CACHED; the library
 * then reuses the spectrum it kept on the device and neither copies nor transforms the
 * filter again (fpga_t reports 0 for both filter fields). Any call that does not hit the
 * cache, and fpga_final, drop the kept spectrum. The reference copies and transforms the
 * filter on every call (host/src/convfpga.c:74-172). With CONVGPU_FILTER_REAL the host
 * filter holds N^3 floats per cube and only those bytes are uploaded.
 * Extends fpgaf_conv3D_svm_batch (host/include/convfpga/convfpga.h:46). */
fpga_t convgpu_conv3d_host(unsigned N, const float2 *sig, const float2 *filter, float2 *out,
                           unsigned how_many, unsigned flags);

/* FFT3 of `count` filter cubes into d_spectrum (count*N^3 float2), for reuse with
 * CONVGPU_FILTER_IS_SPECTRUM: the reference transforms the filter on every call
 * (host/src/convfpga.c:74-172). */
int convgpu_filter_spectrum_device(unsigned N, const float2 *d_filter, float2 *d_spectrum, unsigned count,
                                   void *stream);

/* One entry of an uneven batch: cube size and element offsets from the base pointers. */
typedef struct {
  unsigned n;
  unsigned long long sig_offset;
  unsigned long long filter_offset;
  unsigned long long out_offset;
} convgpu_job;

/* Convolutions of different power-of-two sizes in one call (one filter per job),
 * on device pointers. Extends fpgaf_conv3D_svm_batch to uneven sizes.
 * Default: one CUDA graph, cached per sequence of job sizes, in which every size class is
 * a branch of seven launches (one per pass) over all jobs of that size; tensor maps are
 * rebuilt only when a job's buffers move. CONVGPU_UNEVEN_QUEUE runs the batch as one
 * persistent launch fed by a device work queue of (job, pass, tile) items (at most
 * 4096 jobs), also replayed from a cached graph. Graphs and filter-spectrum workspaces
 * stay allocated until fpga_final. With CONVGPU_UNEVEN_PER_JOB, CONVGPU_TENSOR_SPLIT,
 * CONVGPU_FILTER_IS_SPECTRUM, or cubes not 16-byte aligned, the jobs run one after
 * another through the per-size pass kernels. CONVGPU_FILTER_REAL (filters as N^3 floats,
 * filter offsets counted in floats) needs CONVGPU_UNEVEN_PER_JOB. */
int convgpu_conv3d_uneven_device(const convgpu_job *jobs, unsigned njobs, const float2 *d_sig_base,
                                 const float2 *d_filter_base, float2 *d_out_base, unsigned flags, void *stream);

/* Bytes of device workspace convgpu_conv3d_device uses for these arguments. */
int convgpu_workspace_bytes(unsigned N, unsigned how_many, unsigned flags, size_t *bytes);

/* Pinned (page-locked) host memory for fast copies; release with convgpu_host_free. */
int convgpu_host_alloc(size_t bytes, void **ptr);
int convgpu_host_free(void *ptr);

/* Device in use, whether it can read pageable host memory, and its SM count. */
int convgpu_device_info(int *device, int *pageable_access, int *sm_count);

/* Number of kernels this library has launched so far in the process. */
unsigned long long convgpu_launch_count(void);

/* Per-pass device timing, the analogue of the reference's per-phase OpenCL event
 * profiling (host/src/convfpga.c:83-85, 169-172, 276-279, 360-363).
 *   mode 1: clear and start recording (events around every pass on its stream)
 *   mode 0: clear and stop
 *   mode 2: wait for the recorded passes and fill the CONVGPU_PASS_SLOTS arrays:
 *           ms[slot] total milliseconds, launches[slot] count, bytes[slot] algorithmic
 *           bytes (one read + one write of every cube, plus the filter operand read of
 *           the fused z pass); slot = axis * 4 + op, axis 0/1/2 = x/y/z,
 *           op 0 forward, 1 inverse, 2 z fwd->multiply->inv, 3 same with the filter's
 *           z transform fused in; slots 12 / 13: fused x+y pass forward / inverse. */
#define CONVGPU_PASS_SLOTS 14
int convgpu_pass_timing(int mode, double *ms, unsigned long long *launches, double *bytes);

/* Waits for all work on the library's device. */
int convgpu_synchronize(void);

/* Autotuner: for each of `count` cube sizes, times both shape variants (radix split,
 * pencils per CTA, rows per CTA) of every pass kind on a working set larger than L2 and
 * keeps the faster. With write_cache, writes the choices and timings to the plan-cache
 * file named by fpga_initialize's `path`; fpga_initialize reads that file back. The
 * plan cache takes the role of the reference CPU path's FFTW wisdom file
 * (src/fft_conv3D.cpp:85-112). Not safe to call while other calls are in flight. */
int convgpu_autotune(const unsigned *sizes, unsigned count, int write_cache);

/* Plan-table entry of cube size N for pass kind (0 x pass, 1 y/z passes, 2 fused z pass,
 * 3 fused z pass with the filter's z transform, 4 x and y: 0 separate passes; N = 256:
 * 1 one pass staged through an L2-resident scratch ring, 2 one pass on 8-CTA clusters;
 * N = 128 and 512: 1 one pass staged through an L2-resident scratch ring;
 * 5 tensor-core kernels of CONVGPU_TENSOR_SPLIT, N = 256: 0 tcgen05 (TMEM accumulators),
 * 1 mma.sync; 6 x and y passes of the tcgen05 split path, N = 256: 0 separate passes, 1 one
 * pass staged through the L2-resident scratch ring; 7 spectra of real filters
 * (CONVGPU_FILTER_REAL, FP32 path, N >= 64): 0 full spectra, 1 Hermitian half spectra, kx up
 * to N/2 only, with a fused z pass that serves a column tile and its mirror from one read):
 * sets it to set_to (0 or 1; 0..2 for kind 4) when set_to >= 0, and returns the current
 * variant (or a negative CONVGPU_E* code). */
int convgpu_plan_variant(unsigned N, int kind, int set_to);

/* Waits for the device, then returns and clears the library's device status word in
 * *status: 0 when every kernel completed normally, otherwise the OR of
 *   1   a kernel gave up a bounded wait for its tile load (no output for that tile);
 *   2   the uneven work-queue launch gave up a bounded wait on a dependency;
 *   4   a tensor-core kernel gave up a bounded wait for its MMA completion;
 *   8   a tensor-core kernel found its shared memory misaligned and did nothing;
 *   16  the L2-staged x+y pass gave up a bounded wait on a plane dependency.
 * Any set bit means the affected outputs are wrong. Host-buffer calls, which wait for
 * their own kernels, read and clear the word themselves and then return an fpga_t with
 * valid == 0; stream-ordered device calls leave it for this function. */
int convgpu_device_status(unsigned *status);

/* Testing hooks for the failure contract (no counterpart in pc2/ConvFPGA, whose runtime
 * errors exit() the process: host/src/opencl_utils.c:421-439). Neither is meant for
 * production use; both leave every result path intact.
 *
 * convgpu_debug_dependency_wait_limit: every bounded wait of a kernel on a counter that
 * other CTAs advance (plane dependencies of the fused x+y pass, the uneven work queue, the
 * grid barriers of the one-launch small-cube path) gives up after `probes` probes
 * (0: at once); probes < 0 restores each wait's own limit. A wait that gives up sets its
 * status bit (2 or 16 above) and the kernel finishes without waiting, so the output is
 * wrong and the call reports it: host-buffer calls return valid == 0, device calls leave
 * the bit for convgpu_device_status. Waits for copies or MMAs in flight are not affected.
 * Waits for the device before it changes the limit; graphs captured earlier read the new
 * limit when they run.
 *
 * convgpu_debug_fail_allocations: the next `count` allocations of the library's
 * grow-only device buffers (workspace, host-pipeline staging) fail as out of memory; the
 * call that meets one returns CONVGPU_ENOMEM or an fpga_t with valid == 0, and later
 * calls allocate again. */
int convgpu_debug_dependency_wait_limit(int probes);
int convgpu_debug_fail_allocations(unsigned count);

/* Text of the calling thread's last error ("" if none). */
const char *convgpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CONVGPU_H */
