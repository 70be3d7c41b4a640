// Bridge between the C ABI translation unit (api.cpp, which includes the public
// convfpga.h and therefore must not see CUDA's vector types) and the CUDA runtime
// translation unit (engine.cu). Only plain C++ types cross this boundary.
#pragma once

#include <cstddef>

namespace convgpu {

struct Timing {
  double filter_pcie_wr_t;
  double filter_exec_t;
  double sig_pcie_wr_t;
  double sig_pcie_rd_t;
  double sig_exec_t;
  double siginv_exec_t;
  bool valid;
};

// Host-buffer entry points: how the reference's three conv functions map.
enum HostMode : int { HOST_PLAIN = 0, HOST_SVM = 1, HOST_BATCH = 2 };

struct UnevenJob {  // layout of convgpu_job (include/convgpu.h)
  unsigned n;
  unsigned long long sig_off, filt_off, out_off;  // element offsets from the base pointers
};

int bridge_initialize(const char *platform_name, const char *path, bool use_svm);
void bridge_final();
Timing bridge_conv_host(unsigned n, const void *sig, const void *filt, void *out, unsigned how_many,
                        unsigned flags, int mode);
int bridge_conv_device(unsigned n, const void *d_sig, const void *d_filt, void *d_out, unsigned how_many,
                       unsigned flags, void *stream);
int bridge_filter_spectrum_device(unsigned n, const void *d_filt, void *d_spec, unsigned count, void *stream);
int bridge_conv_uneven_device(const UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt,
                              void *d_out, unsigned flags, void *stream);
int bridge_conv_device_noalloc(unsigned n, const void *d_sig, const void *d_filt, void *d_out, unsigned how_many,
                               unsigned flags, void *stream);
int bridge_workspace_bytes(unsigned n, unsigned how_many, unsigned flags, size_t *bytes);
int bridge_device_info(int *device, int *pageable_access, int *sm_count);
unsigned long long bridge_launch_count();
int bridge_pass_timing(int mode, double *ms, unsigned long long *launches, double *bytes);
const char *bridge_last_error();
int bridge_host_alloc_pinned(size_t bytes, void **ptr);
int bridge_host_free_pinned(void *ptr);
int bridge_sync();
int bridge_autotune(const unsigned *sizes, unsigned count, int write_cache);
int bridge_plan_variant(unsigned n, int kind, int set_to);
int bridge_device_status(unsigned *status);
int bridge_debug_wait_limit(int probes);
int bridge_debug_fail_allocations(unsigned count);

}  // namespace convgpu
