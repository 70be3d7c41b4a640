// The C ABI of libconvgpu.so: convfpga.h (the reference's entry points) and convgpu.h
// (extensions). This translation unit sees the public `float2` and no CUDA header;
// everything is forwarded to the runtime through abi_bridge.h.
#include <cstdlib>
#include <cstring>

#include "../../include/convgpu.h"
#include "abi_bridge.h"

static_assert(sizeof(float2) == 8, "float2 must be two packed floats");

namespace {
fpga_t to_fpga_t(const convgpu::Timing &t) {
  fpga_t r;
  r.filter_pcie_wr_t = t.filter_pcie_wr_t;
  r.filter_exec_t = t.filter_exec_t;
  r.sig_pcie_wr_t = t.sig_pcie_wr_t;
  r.sig_pcie_rd_t = t.sig_pcie_rd_t;
  r.sig_exec_t = t.sig_exec_t;
  r.siginv_exec_t = t.siginv_exec_t;
  r.valid = t.valid;
  return r;
}
}  // namespace

extern "C" {

int fpga_initialize(const char *platform_name, const char *path, const bool use_svm) {
  return convgpu::bridge_initialize(platform_name, path, use_svm);
}

void fpga_final(void) { convgpu::bridge_final(); }

void *fpgaf_complex_malloc(const size_t sz) {
  if (sz == 0) return nullptr;
  void *p = nullptr;
  if (posix_memalign(&p, 64, sz) != 0) return nullptr;
  return p;
}

fpga_t fpgaf_conv3D(const unsigned N, const float2 *sig, const float2 *filter, float2 *out) {
  return to_fpga_t(convgpu::bridge_conv_host(N, sig, filter, out, 1, 0, convgpu::HOST_PLAIN));
}

fpga_t fpgaf_conv3D_svm(const unsigned N, const float2 *sig, const float2 *filter, float2 *out) {
  return to_fpga_t(convgpu::bridge_conv_host(N, sig, filter, out, 1, 0, convgpu::HOST_SVM));
}

fpga_t fpgaf_conv3D_svm_batch(const unsigned N, const float2 *sig, const float2 *filter, float2 *out,
                              const unsigned how_many) {
  return to_fpga_t(convgpu::bridge_conv_host(N, sig, filter, out, how_many, 0, convgpu::HOST_BATCH));
}

int convgpu_conv3d_device(unsigned N, const float2 *d_sig, const float2 *d_filter, float2 *d_out,
                          unsigned how_many, unsigned flags, void *stream) {
  return convgpu::bridge_conv_device(N, d_sig, d_filter, d_out, how_many, flags, stream);
}

int convgpu_conv3d_device_noalloc(unsigned N, const float2 *d_sig, const float2 *d_filter, float2 *d_out,
                                  unsigned how_many, unsigned flags, void *stream) {
  return convgpu::bridge_conv_device_noalloc(N, d_sig, d_filter, d_out, how_many, flags, stream);
}

fpga_t convgpu_conv3d_host(unsigned N, const float2 *sig, const float2 *filter, float2 *out,
                           unsigned how_many, unsigned flags) {
  return to_fpga_t(convgpu::bridge_conv_host(N, sig, filter, out, how_many, flags, convgpu::HOST_BATCH));
}

int convgpu_filter_spectrum_device(unsigned N, const float2 *d_filter, float2 *d_spectrum, unsigned count,
                                   void *stream) {
  return convgpu::bridge_filter_spectrum_device(N, d_filter, d_spectrum, count, stream);
}

int convgpu_conv3d_uneven_device(const convgpu_job *jobs, unsigned njobs, const float2 *d_sig_base,
                                 const float2 *d_filter_base, float2 *d_out_base, unsigned flags, void *stream) {
  static_assert(sizeof(convgpu_job) == sizeof(convgpu::UnevenJob), "job layout");
  return convgpu::bridge_conv_uneven_device(reinterpret_cast<const convgpu::UnevenJob *>(jobs), njobs, d_sig_base,
                                            d_filter_base, d_out_base, flags, stream);
}

int convgpu_workspace_bytes(unsigned N, unsigned how_many, unsigned flags, size_t *bytes) {
  return convgpu::bridge_workspace_bytes(N, how_many, flags, bytes);
}

int convgpu_host_alloc(size_t bytes, void **ptr) { return convgpu::bridge_host_alloc_pinned(bytes, ptr); }

int convgpu_host_free(void *ptr) { return convgpu::bridge_host_free_pinned(ptr); }

int convgpu_device_info(int *device, int *pageable_access, int *sm_count) {
  return convgpu::bridge_device_info(device, pageable_access, sm_count);
}

unsigned long long convgpu_launch_count(void) { return convgpu::bridge_launch_count(); }

int convgpu_pass_timing(int mode, double *ms, unsigned long long *launches, double *bytes) {
  return convgpu::bridge_pass_timing(mode, ms, launches, bytes);
}

int convgpu_synchronize(void) { return convgpu::bridge_sync(); }

int convgpu_autotune(const unsigned *sizes, unsigned count, int write_cache) {
  return convgpu::bridge_autotune(sizes, count, write_cache);
}

int convgpu_plan_variant(unsigned N, int kind, int set_to) { return convgpu::bridge_plan_variant(N, kind, set_to); }

int convgpu_device_status(unsigned *status) { return convgpu::bridge_device_status(status); }

int convgpu_debug_dependency_wait_limit(int probes) { return convgpu::bridge_debug_wait_limit(probes); }

int convgpu_debug_fail_allocations(unsigned count) { return convgpu::bridge_debug_fail_allocations(count); }

const char *convgpu_last_error(void) { return convgpu::bridge_last_error(); }

}  // extern "C"
