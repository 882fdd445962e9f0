// timing.cu — optional per-kernel CUDA-event timing (profiling aid).
//
// When enabled, every launch wrapper records an event pair on the launch
// stream around its kernel.  Pairs are kept until dmgs_timing_collect, which
// waits for them, accumulates elapsed times per kernel and recycles the
// events.  Disabled (the default) it costs one branch per launch.
#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace dmgs_host {

static const char *kKernelNames[K_COUNT] = {
    "preprocess", "bin_compact", "bin_depth_sort", "bin_tile_count", "bin_scan", "bin_emit",
    "blend_fwd",
    "blend_bwd", "preprocess_bwd", "mark_visible", "bind_fwd", "bind_bwd", "bind3_fwd",
    "bind3_bwd", "debug", "batch_preprocess", "batch_binning", "batch_blend_fwd",
    "batch_blend_bwd", "batch_preprocess_bwd", "l1_ssim", "face_cull", "fc_fwd", "fc_bwd", "tex_fwd", "tex_bwd", "sh_colors", "bin_row_emit", "tex_scatter"};

namespace {
struct Pending { int kid; cudaEvent_t a, b; };
std::mutex g_mu;
bool g_on = false;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
cudaEvent_t g_open[K_COUNT];
double g_ms[K_COUNT];
long long g_n[K_COUNT];

cudaEvent_t take() {
  if (!g_free.empty()) { cudaEvent_t e = g_free.back(); g_free.pop_back(); return e; }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

void timing_begin(int kid, cudaStream_t s) {
  if (!g_on) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t a = take();
  cudaEventRecord(a, s);
  g_open[kid] = a;
}

void timing_end(int kid, cudaStream_t s) {
  if (!g_on) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t b = take();
  cudaEventRecord(b, s);
  g_pending.push_back({kid, g_open[kid], b});
}

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

}  // namespace dmgs_host

using namespace dmgs_host;

extern "C" int64_t dmgs_kernel_launches(void) { return g_launches.load(); }

extern "C" int dmgs_timing_enable(int32_t on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_on = on != 0;
  return DMGS_OK;
}

extern "C" int dmgs_timing_collect(int32_t *n, const char **names, double *total_ms,
                                   int64_t *launches) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto &p : g_pending) {
    cudaEventSynchronize(p.b);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      g_ms[p.kid] += ms;
      g_n[p.kid] += 1;
    }
    g_free.push_back(p.a);
    g_free.push_back(p.b);
  }
  g_pending.clear();
  int cap = n ? *n : 0, w = 0;
  for (int k = 0; k < K_COUNT && w < cap; ++k) {
    if (g_n[k] == 0) continue;
    if (names) names[w] = kKernelNames[k];
    if (total_ms) total_ms[w] = g_ms[k];
    if (launches) launches[w] = g_n[k];
    ++w;
  }
  if (n) *n = w;
  for (int k = 0; k < K_COUNT; ++k) { g_ms[k] = 0.0; g_n[k] = 0; }
  return DMGS_OK;
}
