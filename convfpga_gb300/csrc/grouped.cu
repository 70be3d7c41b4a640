// Uneven batches as one CUDA graph of per-size launches.
//
// Jobs of the same cube size run together: each of the seven passes of a convolution
// (filter x, signal x, filter y, signal y, fused z, signal y-inv, signal x-inv) is one
// launch of the TMA-fed pass kernel over every job of that size, in table mode: each job
// brings its own tensor maps and destination base, so the jobs' cubes may sit anywhere.
// The size classes run as parallel branches of one CUDA graph, captured once per
// sequence of job sizes and replayed on every call; tensor maps are re-encoded and
// uploaded only when a job's buffers move. When the plan fuses the x and y passes of
// N = 256 or 128 (L2-staged pass), that class runs filter x+y, signal x+y, fused z and
// inverse y+x instead: three table-mode launches of the fused pass around the z launch.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "engine_internal.h"
#include "passes.cuh"

namespace convgpu {
namespace {

// rows(filter) rows(signal) rows(out) y(spec) y(out) z(out) z(spec), then the fused x+y
// pass's rows maps (N = 256 and 128): filter, signal, out
constexpr int kKinds = 10;

struct SizeGroup {
  int n = 0;
  std::vector<int> jobs;
  CUtensorMap *d_maps = nullptr;  // [kind][job in group]
  float2 **d_dsts = nullptr;      // [0][j] spectrum, [1][j] output
  std::vector<CUtensorMap> h_maps;
  std::vector<float2 *> h_dsts;
  unsigned *d_ctr = nullptr;  // dependency counters of the fused x+y launches
  bool xy = false;            // this class runs the fused x+y pass
};

struct GPlan {
  std::vector<int> sizes;
  std::vector<SizeGroup> groups;
  float2 *d_spec = nullptr;
  std::vector<size_t> spec_off;
  std::vector<const void *> ptr_key;  // buffers the uploaded maps describe
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  bool launched = false;
  ~GPlan() {
    if (done) cudaEventDestroy(done);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto &g : groups) {
      if (g.d_maps) cudaFree(g.d_maps);
      if (g.d_dsts) cudaFree(g.d_dsts);
      if (g.d_ctr) cudaFree(g.d_ctr);
    }
    if (d_spec) cudaFree(d_spec);
  }
};

std::mutex g_mu;
// key: job sizes, normalize + 2 * (fused x+y: bit 0 N = 256, bit 1 N = 128)
std::map<std::pair<std::vector<int>, int>, std::unique_ptr<GPlan>> g_plans;

cudaError_t enqueue_group(const SizeGroup &g, float scale, const float2 *tw512, cudaStream_t s) {
  const int k = (int)g.jobs.size();
  const CUtensorMap *m = g.d_maps;
  float2 *const *spec = g.d_dsts;
  float2 *const *out = g.d_dsts + k;
  cudaError_t e;
  if (g.xy) {
    unsigned *st = device_status_address();
    if ((e = launch_xy_l2_table(g.n, m + 7 * k, spec, k, false, 1.f, tw512, st, g.d_ctr, s)) != cudaSuccess)
      return e;
    if ((e = launch_xy_l2_table(g.n, m + 8 * k, out, k, false, 1.f, tw512, st, g.d_ctr, s)) != cudaSuccess)
      return e;
    if ((e = launch_axis_pass_table(g.n, 2, OP_CONV_FZ, m + 5 * k, m + 6 * k, out, k, 1.f, tw512, s)) != cudaSuccess)
      return e;
    return launch_xy_l2_table(g.n, m + 9 * k, out, k, true, scale, tw512, st, g.d_ctr, s);
  }
  if ((e = launch_axis_pass_table(g.n, 0, OP_FWD, m + 0 * k, nullptr, spec, k, 1.f, tw512, s)) != cudaSuccess) return e;
  if ((e = launch_axis_pass_table(g.n, 0, OP_FWD, m + 1 * k, nullptr, out, k, 1.f, tw512, s)) != cudaSuccess) return e;
  if ((e = launch_axis_pass_table(g.n, 1, OP_FWD, m + 3 * k, nullptr, spec, k, 1.f, tw512, s)) != cudaSuccess) return e;
  if ((e = launch_axis_pass_table(g.n, 1, OP_FWD, m + 4 * k, nullptr, out, k, 1.f, tw512, s)) != cudaSuccess) return e;
  if ((e = launch_axis_pass_table(g.n, 2, OP_CONV_FZ, m + 5 * k, m + 6 * k, out, k, 1.f, tw512, s)) != cudaSuccess)
    return e;
  if ((e = launch_axis_pass_table(g.n, 1, OP_INV, m + 4 * k, nullptr, out, k, 1.f, tw512, s)) != cudaSuccess) return e;
  return launch_axis_pass_table(g.n, 0, OP_INV, m + 2 * k, nullptr, out, k, scale, tw512, s);
}

// xy_mask: bit 0 fuses x and y for N = 256, bit 1 for N = 128.
cudaError_t build(GPlan &p, bool normalize, int xy_mask, const float2 *tw512) {
  std::map<int, int> idx;
  for (int j = 0; j < (int)p.sizes.size(); ++j) {
    const int n = p.sizes[j];
    if (!idx.count(n)) {
      idx[n] = (int)p.groups.size();
      p.groups.emplace_back();
      p.groups.back().n = n;
    }
    p.groups[idx[n]].jobs.push_back(j);
  }
  // largest cubes first: their launches are the long ones
  std::sort(p.groups.begin(), p.groups.end(), [](const SizeGroup &a, const SizeGroup &b) { return a.n > b.n; });
  size_t spec = 0;
  p.spec_off.resize(p.sizes.size());
  for (size_t j = 0; j < p.sizes.size(); ++j) {
    p.spec_off[j] = spec;
    spec += (size_t)p.sizes[j] * p.sizes[j] * p.sizes[j];
  }
  cudaError_t e;
  if ((e = cudaMalloc(&p.d_spec, spec * sizeof(float2))) != cudaSuccess) return e;
  for (auto &g : p.groups) {
    const size_t k = g.jobs.size();
    g.h_maps.resize(kKinds * k);
    g.h_dsts.resize(2 * k);
    if ((e = cudaMalloc(&g.d_maps, sizeof(CUtensorMap) * kKinds * k)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&g.d_dsts, sizeof(float2 *) * 2 * k)) != cudaSuccess) return e;
    g.xy = (g.n == 256 && (xy_mask & 1)) || (g.n == 128 && (xy_mask & 2));
    if (g.xy) {
      if ((e = prepare_xy_l2(g.n)) != cudaSuccess) return e;
      if ((e = cudaMalloc(&g.d_ctr, xy_l2_counter_bytes(g.n, (int)k))) != cudaSuccess) return e;
    }
  }
  if ((e = cudaEventCreateWithFlags(&p.done, cudaEventDisableTiming)) != cudaSuccess) return e;
  for (auto &g : p.groups)
    if ((e = prepare_table_launches(g.n)) != cudaSuccess) return e;
  // Capture: one branch per size class.
  cudaStream_t cap;
  if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess) return e;
  std::vector<cudaStream_t> br(p.groups.size(), nullptr);
  std::vector<cudaEvent_t> ev(p.groups.size() + 1, nullptr);
  for (auto &b : br)
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking);
  for (auto &v : ev)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaEventRecord(ev.back(), cap);
    for (size_t gi = 0; gi < p.groups.size() && e == cudaSuccess; ++gi) {
      const int n = p.groups[gi].n;
      const float scale = normalize ? (float)(1.0 / ((double)n * n * n)) : 1.0f;
      cudaStreamWaitEvent(br[gi], ev.back(), 0);
      e = enqueue_group(p.groups[gi], scale, tw512, br[gi]);
      cudaEventRecord(ev[gi], br[gi]);
      cudaStreamWaitEvent(cap, ev[gi], 0);
    }
    cudaError_t e2 = cudaStreamEndCapture(cap, &p.graph);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p.exec, p.graph, 0);
  for (auto b : br)
    if (b) cudaStreamDestroy(b);
  for (auto v : ev)
    if (v) cudaEventDestroy(v);
  cudaStreamDestroy(cap);
  return e;
}

}  // namespace

int uneven_grouped(const UnevenJob *jobs, unsigned njobs, const void *d_sig, const void *d_filt, void *d_out,
                   bool normalize, const float2 *tw512, cudaStream_t stream, std::string &err) {
  if (njobs == 0) return 0;
  std::vector<int> sizes(njobs);
  std::vector<const void *> ptrs(3 * njobs);
  for (unsigned j = 0; j < njobs; ++j) {
    sizes[j] = (int)jobs[j].n;
    ptrs[3 * j] = (const float2 *)d_sig + jobs[j].sig_off;
    ptrs[3 * j + 1] = (const float2 *)d_filt + jobs[j].filt_off;
    ptrs[3 * j + 2] = (const float2 *)d_out + jobs[j].out_off;
    for (int q = 0; q < 3; ++q)
      if ((reinterpret_cast<uintptr_t>(ptrs[3 * j + q]) & 15u) != 0) {
        err = "uneven batch: a cube is not 16-byte aligned";
        return -5;  // caller falls back to one job at a time
      }
  }
  std::lock_guard<std::mutex> lk(g_mu);
  // the L2-staged variant (1) has a table mode
  const int xy_mask = (get_pass_variant(256, kKindXy) == 1 ? 1 : 0) | (get_pass_variant(128, kKindXy) == 1 ? 2 : 0);
  auto key = std::make_pair(sizes, (normalize ? 1 : 0) + 2 * xy_mask);
  auto it = g_plans.find(key);
  if (it == g_plans.end()) {
    auto p = std::make_unique<GPlan>();
    p->sizes = sizes;
    cudaError_t e = build(*p, normalize, xy_mask, tw512);
    if (e != cudaSuccess) {
      err = std::string("uneven grouped plan: ") + cudaGetErrorString(e);
      cudaGetLastError();
      return e == cudaErrorMemoryAllocation ? -4 : -3;
    }
    it = g_plans.emplace(key, std::move(p)).first;
  }
  GPlan &p = *it->second;
  cudaError_t e = cudaSuccess;
  if (p.ptr_key != ptrs) {
    // The previous replay may still read the maps being replaced.
    if (p.launched) cudaEventSynchronize(p.done);
    for (auto &g : p.groups) {
      const size_t k = g.jobs.size();
      for (size_t v = 0; v < k; ++v) {
        const int j = g.jobs[v];
        const void *sg = ptrs[3 * j], *ft = ptrs[3 * j + 1], *ot = ptrs[3 * j + 2];
        float2 *sp = p.d_spec + p.spec_off[j];
        bool ok = encode_table_map(&g.h_maps[0 * k + v], ft, g.n, 0) && encode_table_map(&g.h_maps[1 * k + v], sg, g.n, 0) &&
                  encode_table_map(&g.h_maps[2 * k + v], ot, g.n, 0) && encode_table_map(&g.h_maps[3 * k + v], sp, g.n, 1) &&
                  encode_table_map(&g.h_maps[4 * k + v], ot, g.n, 1) && encode_table_map(&g.h_maps[5 * k + v], ot, g.n, 2) &&
                  encode_table_map(&g.h_maps[6 * k + v], sp, g.n, 2);
        if (ok && g.xy)
          ok = encode_xy_table_map(&g.h_maps[7 * k + v], ft, g.n) &&
               encode_xy_table_map(&g.h_maps[8 * k + v], sg, g.n) && encode_xy_table_map(&g.h_maps[9 * k + v], ot, g.n);
        if (!ok) {
          err = "uneven batch: tensor map encoding failed";
          return -5;
        }
        g.h_dsts[v] = sp;
        g.h_dsts[k + v] = (float2 *)ot;
      }
      // pageable sources: each call returns once the host data is staged
      e = cudaMemcpyAsync(g.d_maps, g.h_maps.data(), sizeof(CUtensorMap) * g.h_maps.size(), cudaMemcpyHostToDevice,
                          stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.d_dsts, g.h_dsts.data(), sizeof(float2 *) * g.h_dsts.size(), cudaMemcpyHostToDevice,
                            stream);
      if (e != cudaSuccess) break;
    }
    if (e == cudaSuccess) p.ptr_key = ptrs;
  }
  if (e == cudaSuccess) e = cudaGraphLaunch(p.exec, stream);
  if (e == cudaSuccess) e = cudaEventRecord(p.done, stream);
  if (e != cudaSuccess) {
    err = std::string("uneven grouped launch: ") + cudaGetErrorString(e);
    return -3;
  }
  p.launched = true;
  count_launches(7 * p.groups.size());
  return 0;
}

void release_grouped_plans() {
  std::lock_guard<std::mutex> lk(g_mu);
  g_plans.clear();
}

}  // namespace convgpu
