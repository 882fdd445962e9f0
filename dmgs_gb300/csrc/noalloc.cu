// noalloc.cu — a backward entry point that allocates nothing.
//
// dmgs_raster_bwd needs a caller-provided scratch buffer (the per-Gaussian
// gradient accumulators of the blend adjoint, 48 bytes per Gaussian).  Some
// callers cannot provide one: a plugin running inside a host application
// that owns the device's memory pool and forbids cudaMalloc, or a real-time
// loop that must not call cudaMalloc/cudaFree (they synchronise the device)
// between frames.  dmgs_raster_bwd_noalloc serves them: its scratch is the
// file-scope device array below, sized for DMGS_NOALLOC_MAX_GAUSSIANS
// Gaussians (12 MiB).  Every GPU that loads this library holds that array
// until the process exits.
//
// The array's name is only a host-side stand-in in host code, so the first
// call on each device (with that device current) looks up its device address
// with cudaGetSymbolAddress and caches it; that first call should come before
// any stream capture begins.  The cached address outlives a cudaDeviceReset
// (after which the array may live elsewhere), so the entry point must not be
// used on a device after that device was reset.  All calls share the one
// array and it keeps the previous call's contents: the adjoint clears the
// accumulators it needs at the start of every call, and calls whose work
// overlaps on the GPU (two streams, or two host threads) race on the array.
#include <mutex>

#include "kernels.cuh"

namespace {

constexpr size_t kFloatsPerGaussian = 12;  // 48-byte accumulator record
static __device__ __align__(256) float g_noalloc_bwd_scratch[(size_t)DMGS_NOALLOC_MAX_GAUSSIANS *
                                                             kFloatsPerGaussian];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

int scratch_address(void **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return dmgs_host::cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    dmgs_host::set_error("raster_bwd_noalloc: device ordinal %d exceeds %d", dev, kMaxDevices);
    return DMGS_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_scratch_addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_bwd_scratch);
    if (e != cudaSuccess) return dmgs_host::cuda_fail(e, "cudaGetSymbolAddress");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return DMGS_OK;
}

}  // namespace

extern "C" int dmgs_raster_bwd(const DmgsView *view, const DmgsGaussians *g,
                               const float *dL_dout_color, const void *geom_state,
                               size_t geom_bytes, const void *binning_state, size_t binning_bytes,
                               int64_t num_rendered, const void *image_state, size_t image_bytes,
                               void *bwd_scratch, size_t bwd_scratch_bytes,
                               const DmgsGrads *grads, dmgs_stream_t stream);

extern "C" int dmgs_raster_bwd_noalloc(const DmgsView *view, const DmgsGaussians *g,
                                       const float *dL_dout_color, const void *geom_state,
                                       size_t geom_bytes, const void *binning_state,
                                       size_t binning_bytes, int64_t num_rendered,
                                       const void *image_state, size_t image_bytes,
                                       const DmgsGrads *grads, dmgs_stream_t stream) {
  if (!g) {
    dmgs_host::set_error("raster_bwd_noalloc: gaussians is NULL");
    return DMGS_ERR_ARG;
  }
  if (g->P > DMGS_NOALLOC_MAX_GAUSSIANS) {
    dmgs_host::set_error(
        "raster_bwd_noalloc: %d Gaussians exceed the static scratch limit of %d; "
        "use dmgs_raster_bwd with a caller-provided scratch buffer",
        g->P, DMGS_NOALLOC_MAX_GAUSSIANS);
    return DMGS_ERR_ARG;
  }
  void *scratch = nullptr;
  const int r = scratch_address(&scratch);
  if (r != DMGS_OK) return r;
  return dmgs_raster_bwd(view, g, dL_dout_color, geom_state, geom_bytes, binning_state,
                         binning_bytes, num_rendered, image_state, image_bytes, scratch,
                         sizeof(g_noalloc_bwd_scratch), grads, stream);
}
