// capi.cu — the extern "C" entry points of include/dmgs.h.
//
// Host-side argument validation mirrors the reference wrapper's checks
// (exactly one colour source, exactly one covariance source); shapes are the
// caller's responsibility beyond what the sizes given here can check.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "kernels.cuh"

namespace dmgs_host {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what) {
  set_error("CUDA error in %s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return DMGS_ERR_CUDA;
}

int raise_smem_limit(const void *func, size_t bytes) {
  if (bytes <= 48 * 1024) return DMGS_OK;  // the default limit
  int dev = 0;
  DMGS_CUDA(cudaGetDevice(&dev));
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[{dev, func}];
  if (bytes > cur) {
    DMGS_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
  }
  return DMGS_OK;
}

}  // namespace dmgs_host

using namespace dmgs;
using dmgs_host::set_error;

namespace {

int check_view(const DmgsView *v) {
  if (!v) { set_error("view is NULL"); return DMGS_ERR_ARG; }
  if (v->width <= 0 || v->height <= 0 || v->width > 65535 * TILE || v->height > 65535 * TILE) {
    set_error("invalid image size %d x %d", v->width, v->height);
    return DMGS_ERR_ARG;
  }
  if (v->sh_degree < 0 || v->sh_degree > 3) {
    set_error("sh_degree must be in 0..3, got %d", v->sh_degree);
    return DMGS_ERR_ARG;
  }
  if (!v->bg || !v->viewmatrix || !v->projmatrix || !v->campos) {
    set_error("view pointers (bg, viewmatrix, projmatrix, campos) must be non-NULL");
    return DMGS_ERR_ARG;
  }
  if (!(v->tanfovx > 0.f) || !(v->tanfovy > 0.f)) {
    set_error("tanfovx/tanfovy must be positive");
    return DMGS_ERR_ARG;
  }
  return DMGS_OK;
}

int check_gaussians(const DmgsGaussians *g, int D) {
  if (!g) { set_error("gaussians is NULL"); return DMGS_ERR_ARG; }
  if (g->P < 0) { set_error("P must be >= 0"); return DMGS_ERR_ARG; }
  if (g->P == 0) return DMGS_OK;
  if (!g->means3D || !g->opacities) { set_error("means3D and opacities are required"); return DMGS_ERR_ARG; }
  if ((g->shs == nullptr) == (g->colors_precomp == nullptr)) {
    set_error("Please provide exactly one of either SHs or precomputed colors!");
    return DMGS_ERR_ARG;
  }
  const bool sr = g->scales != nullptr || g->rotations != nullptr;
  const bool sr_full = g->scales != nullptr && g->rotations != nullptr;
  if ((!sr_full && g->cov3D_precomp == nullptr) || (sr && g->cov3D_precomp != nullptr)) {
    set_error("Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!");
    return DMGS_ERR_ARG;
  }
  if (g->shs && g->M < (D + 1) * (D + 1)) {
    set_error("shs has %d coefficients per Gaussian, degree %d needs %d", g->M, D, (D + 1) * (D + 1));
    return DMGS_ERR_ARG;
  }
  if (g->rotations && (reinterpret_cast<uintptr_t>(g->rotations) & 15)) {
    set_error("rotations must be 16-byte aligned");
    return DMGS_ERR_ARG;
  }
  return DMGS_OK;
}

ViewParams make_params(const DmgsView *v) {
  ViewParams p;
  p.W = v->width;
  p.H = v->height;
  p.gx = (v->width + TILE - 1) / TILE;
  p.gy = (v->height + TILE - 1) / TILE;
  // focal = size / (2 tan(fov/2)), single precision (the CPU oracle's focal())
  volatile float two_tx = 2.0f * v->tanfovx;
  volatile float two_ty = 2.0f * v->tanfovy;
  volatile float fx = (float)v->width / two_tx;
  volatile float fy = (float)v->height / two_ty;
  p.fx = fx;
  p.fy = fy;
  p.tanfovx = v->tanfovx;
  p.tanfovy = v->tanfovy;
  p.scale_modifier = v->scale_modifier;
  p.D = v->sh_degree;
  p.prefiltered = v->prefiltered;
  return p;
}

GaussianPtrs make_gptrs(const DmgsGaussians *g) {
  GaussianPtrs p;
  p.P = g->P;
  p.M = g->M;
  p.means3D = g->means3D;
  p.opacities = g->opacities;
  p.shs = g->shs;
  p.colors = g->colors_precomp;
  p.scales = g->cov3D_precomp ? nullptr : g->scales;
  p.rotations = g->cov3D_precomp ? nullptr : g->rotations;
  p.cov3D = g->cov3D_precomp;
  return p;
}

// Reads the kernel status word; returns a DMGS error for set bits.
int check_status(const char *geom, const GeomLayout &L, cudaStream_t s, uint32_t *host4) {
  uint32_t h[CI_WORDS] = {};
  cudaError_t e = cudaMemcpyAsync(h, geom + L.counters, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return dmgs_host::cuda_fail(e, "status copy");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return dmgs_host::cuda_fail(e, "cudaStreamSynchronize");
  if (host4) memcpy(host4, h, sizeof(h));
  if (h[0] & ST_PREFILTER) {
    set_error("a point failed the frustum test although prefiltered is set");
    return DMGS_ERR_PREFILTER;
  }
  if (h[0] & ST_OVERFLOW) { set_error("instance buffer overflow"); return DMGS_ERR_OVERFLOW; }
  if (h[0] & ST_BOUNDS) { set_error("a kernel index left its buffer"); return DMGS_ERR_DEVICE; }
  return DMGS_OK;
}

int debug_sync(const DmgsView *v, cudaStream_t s, const char *what) {
  if (!v->debug) return DMGS_OK;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return dmgs_host::cuda_fail(e, what);
  e = cudaGetLastError();
  if (e != cudaSuccess) return dmgs_host::cuda_fail(e, what);
  return DMGS_OK;
}

#define RET_IF(x)          \
  do {                     \
    int r_ = (x);          \
    if (r_ != DMGS_OK) return r_; \
  } while (0)

}  // namespace

extern "C" {

const char *dmgs_last_error(void) { return dmgs_host::g_err; }
int32_t dmgs_abi_version(void) { return DMGS_ABI_VERSION; }

size_t dmgs_geom_state_bytes(int32_t P, int32_t width, int32_t height) {
  return geom_layout(P, width, height).total;
}
size_t dmgs_binning_state_bytes(int64_t num_rendered, int32_t width, int32_t height) {
  return bin_layout(num_rendered, width, height).total;
}
size_t dmgs_image_state_bytes(int32_t width, int32_t height) { return img_layout(width, height).total; }
size_t dmgs_bwd_scratch_bytes(int32_t P) { return bwd_scratch_bytes(P); }

int dmgs_raster_fwd_geometry(const DmgsView *view, const DmgsGaussians *g, void *geom_state,
                             size_t geom_bytes, int32_t *radii, int64_t *num_rendered,
                             dmgs_stream_t stream) {
  RET_IF(check_view(view));
  RET_IF(check_gaussians(g, view->sh_degree));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const GeomLayout L = geom_layout(g->P, view->width, view->height);
  if (!geom_state || geom_bytes < L.total) {
    set_error("geometry state too small: %zu < %zu bytes", geom_bytes, L.total);
    return DMGS_ERR_STATE;
  }
  if (g->P > 0 && !radii) { set_error("radii is NULL"); return DMGS_ERR_ARG; }
  char *geom = static_cast<char *>(geom_state);
  const ViewParams vp = make_params(view);
  RET_IF(launch_preprocess(vp, view->viewmatrix, view->projmatrix, view->campos, make_gptrs(g),
                           radii, L, geom, s));
  RET_IF(debug_sync(view, s, "preprocess"));
  BinViews bv;
  bv.n = 1;
  RET_IF(make_bin_view(L, geom, 0xffffffffu, nullptr, 0u, bv.v[0]));
  RET_IF(launch_binning_geometry(bv, s));
  uint32_t h[CI_WORDS];
  RET_IF(check_status(geom, L, s, h));
  if (num_rendered) *num_rendered = (int64_t)h[CI_K];
  return DMGS_OK;
}

int dmgs_raster_fwd_render(const DmgsView *view, const DmgsGaussians *g, void *geom_state,
                           size_t geom_bytes, void *binning_state, size_t binning_bytes,
                           int64_t num_rendered, void *image_state, size_t image_bytes,
                           float *out_color, dmgs_stream_t stream) {
  RET_IF(check_view(view));
  if (!g || g->P < 0) { set_error("gaussians invalid"); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const GeomLayout L = geom_layout(g->P, view->width, view->height);
  const BinLayout B = bin_layout(num_rendered, view->width, view->height);
  const ImgLayout I = img_layout(view->width, view->height);
  if (!geom_state || geom_bytes < L.total) { set_error("geometry state too small"); return DMGS_ERR_STATE; }
  if (!binning_state || binning_bytes < B.total) { set_error("binning state too small: %zu < %zu", binning_bytes, B.total); return DMGS_ERR_STATE; }
  if (!image_state || image_bytes < I.total) { set_error("image state too small"); return DMGS_ERR_STATE; }
  if (!out_color) { set_error("out_color is NULL"); return DMGS_ERR_ARG; }
  if (num_rendered < 0 || num_rendered > 0xffffffffll) { set_error("num_rendered out of range"); return DMGS_ERR_ARG; }
  char *geom = static_cast<char *>(geom_state);
  char *bin = static_cast<char *>(binning_state);
  char *img = static_cast<char *>(image_state);
  const ViewParams vp = make_params(view);
  BinViews bv;
  bv.n = 1;
  RET_IF(make_bin_view(L, geom, 0xffffffffu, bin + B.point_list, (uint32_t)num_rendered, bv.v[0]));
  RET_IF(launch_emit(bv, s));
  RET_IF(debug_sync(view, s, "emit"));
  RET_IF(launch_blend_fwd(vp, L, geom, B, bin, I, img, view->bg, out_color, s));
  RET_IF(debug_sync(view, s, "blend_fwd"));
  if (view->debug) RET_IF(check_status(geom, L, s, nullptr));
  return DMGS_OK;
}

int dmgs_raster_fwd(const DmgsView *view, const DmgsGaussians *g, dmgs_alloc_fn alloc,
                    void *alloc_ctx, int32_t *radii, float *out_color, int64_t *num_rendered,
                    dmgs_stream_t stream) {
  RET_IF(check_view(view));
  RET_IF(check_gaussians(g, view->sh_degree));
  if (!alloc) { set_error("alloc callback is NULL"); return DMGS_ERR_ARG; }
  const size_t gb = dmgs_geom_state_bytes(g->P, view->width, view->height);
  void *geom = alloc(alloc_ctx, 0, gb);
  if (!geom) { set_error("geometry allocation of %zu bytes failed", gb); return DMGS_ERR_STATE; }
  int64_t K = 0;
  RET_IF(dmgs_raster_fwd_geometry(view, g, geom, gb, radii, &K, stream));
  const size_t bb = dmgs_binning_state_bytes(K, view->width, view->height);
  void *bin = alloc(alloc_ctx, 1, bb);
  if (!bin) { set_error("binning allocation of %zu bytes failed", bb); return DMGS_ERR_STATE; }
  const size_t ib = dmgs_image_state_bytes(view->width, view->height);
  void *img = alloc(alloc_ctx, 2, ib);
  if (!img) { set_error("image allocation of %zu bytes failed", ib); return DMGS_ERR_STATE; }
  if (num_rendered) *num_rendered = K;
  return dmgs_raster_fwd_render(view, g, geom, gb, bin, bb, K, img, ib, out_color, stream);
}

}  // extern "C"

namespace {

// Both backward entry points: f64 selects the FP64-sum mode, whose scratch
// holds the [P][12] double accumulators after the float records.
int raster_bwd_impl(const DmgsView *view, const DmgsGaussians *g, const float *dL_dout_color,
                    const void *geom_state, size_t geom_bytes, const void *binning_state,
                    size_t binning_bytes, int64_t num_rendered, const void *image_state,
                    size_t image_bytes, void *bwd_scratch, size_t bwd_scratch_bytes_,
                    const DmgsGrads *grads, dmgs_stream_t stream, bool f64) {
  RET_IF(check_view(view));
  RET_IF(check_gaussians(g, view->sh_degree));
  if (!grads || !dL_dout_color) { set_error("grads / dL_dout_color is NULL"); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const GeomLayout L = geom_layout(g->P, view->width, view->height);
  const BinLayout B = bin_layout(num_rendered, view->width, view->height);
  const ImgLayout I = img_layout(view->width, view->height);
  if (!geom_state || geom_bytes < L.total) { set_error("geometry state too small"); return DMGS_ERR_STATE; }
  if (!binning_state || binning_bytes < B.total) { set_error("binning state too small"); return DMGS_ERR_STATE; }
  if (!image_state || image_bytes < I.total) { set_error("image state too small"); return DMGS_ERR_STATE; }
  const size_t need = f64 ? bwd_scratch_bytes(g->P) + align_up((size_t)g->P * 96, 256)
                          : bwd_scratch_bytes(g->P);
  if (!bwd_scratch || bwd_scratch_bytes_ < need) { set_error("backward scratch too small: %zu < %zu bytes", bwd_scratch_bytes_, need); return DMGS_ERR_STATE; }
  if (grads->dL_drotations && (reinterpret_cast<uintptr_t>(grads->dL_drotations) & 15)) {
    set_error("dL_drotations must be 16-byte aligned");
    return DMGS_ERR_ARG;
  }
  const char *geom = static_cast<const char *>(geom_state);
  const char *bin = static_cast<const char *>(binning_state);
  const char *img = static_cast<const char *>(image_state);
  float *gacc = static_cast<float *>(bwd_scratch);
  double *gacc64 = f64 ? reinterpret_cast<double *>(static_cast<char *>(bwd_scratch) +
                                                    bwd_scratch_bytes(g->P))
                       : nullptr;
  const ViewParams vp = make_params(view);
  RET_IF(launch_blend_bwd(vp, L, geom, B, bin, I, img, view->bg, dL_dout_color, gacc, gacc64, s));
  RET_IF(debug_sync(view, s, "blend_bwd"));
  DmgsGrads out = *grads;
  RET_IF(launch_preprocess_bwd(vp, view->viewmatrix, view->projmatrix, view->campos,
                               make_gptrs(g), L, geom, gacc, out, s));
  RET_IF(debug_sync(view, s, "preprocess_bwd"));
  return DMGS_OK;
}

}  // namespace

extern "C" {

size_t dmgs_bwd_scratch_f64_bytes(int32_t P) {
  return P < 0 ? 0 : bwd_scratch_bytes(P) + align_up((size_t)P * 96, 256);
}

int dmgs_raster_bwd(const DmgsView *view, const DmgsGaussians *g, const float *dL_dout_color,
                    const void *geom_state, size_t geom_bytes, const void *binning_state,
                    size_t binning_bytes, int64_t num_rendered, const void *image_state,
                    size_t image_bytes, void *bwd_scratch, size_t bwd_scratch_bytes_,
                    const DmgsGrads *grads, dmgs_stream_t stream) {
  return raster_bwd_impl(view, g, dL_dout_color, geom_state, geom_bytes, binning_state,
                         binning_bytes, num_rendered, image_state, image_bytes, bwd_scratch,
                         bwd_scratch_bytes_, grads, stream, false);
}

int dmgs_raster_bwd_f64sum(const DmgsView *view, const DmgsGaussians *g,
                           const float *dL_dout_color, const void *geom_state, size_t geom_bytes,
                           const void *binning_state, size_t binning_bytes, int64_t num_rendered,
                           const void *image_state, size_t image_bytes, void *bwd_scratch,
                           size_t bwd_scratch_bytes_, const DmgsGrads *grads,
                           dmgs_stream_t stream) {
  return raster_bwd_impl(view, g, dL_dout_color, geom_state, geom_bytes, binning_state,
                         binning_bytes, num_rendered, image_state, image_bytes, bwd_scratch,
                         bwd_scratch_bytes_, grads, stream, true);
}

int dmgs_mark_visible(int32_t P, const float *means3D, const float *viewmatrix,
                      const float *projmatrix, uint8_t *present, dmgs_stream_t stream) {
  (void)projmatrix;
  if (P < 0 || (P > 0 && (!means3D || !viewmatrix || !present))) {
    set_error("mark_visible: invalid arguments");
    return DMGS_ERR_ARG;
  }
  return launch_mark_visible(P, means3D, viewmatrix, present, reinterpret_cast<cudaStream_t>(stream));
}

int dmgs_debug_geometry(int32_t P, int32_t width, int32_t height, const void *geom_state,
                        size_t geom_bytes, int32_t *rect, uint32_t *tiles_touched, float *depth,
                        float *xy, float *conic_opacity, float *rgb, dmgs_stream_t stream) {
  const GeomLayout L = geom_layout(P, width, height);
  if (!geom_state || geom_bytes < L.total) { set_error("geometry state too small"); return DMGS_ERR_STATE; }
  return launch_debug_geometry(L, static_cast<const char *>(geom_state), rect, tiles_touched, depth,
                               xy, conic_opacity, rgb, reinterpret_cast<cudaStream_t>(stream));
}

int dmgs_debug_binning(int32_t P, int32_t width, int32_t height, int64_t num_rendered,
                       const void *geom_state, size_t geom_bytes, const void *binning_state,
                       size_t binning_bytes, uint64_t *keys, uint32_t *values, uint32_t *ranges,
                       dmgs_stream_t stream) {
  const GeomLayout L = geom_layout(P, width, height);
  const BinLayout B = bin_layout(num_rendered, width, height);
  if (!geom_state || geom_bytes < L.total) { set_error("geometry state too small"); return DMGS_ERR_STATE; }
  if (!binning_state || binning_bytes < B.total) { set_error("binning state too small"); return DMGS_ERR_STATE; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const char *bin = static_cast<const char *>(binning_state);
  if (ranges) DMGS_CUDA(cudaMemcpyAsync(ranges, static_cast<const char *>(geom_state) + L.ranges, (size_t)L.T() * 8, cudaMemcpyDeviceToDevice, s));
  if ((keys || values) && num_rendered > 0)
    return launch_debug_keys(L, static_cast<const char *>(geom_state), B, bin, keys, values, s);
  return DMGS_OK;
}

int dmgs_debug_image(int32_t width, int32_t height, const void *image_state, size_t image_bytes,
                     float *final_T, uint32_t *n_contrib, dmgs_stream_t stream) {
  const ImgLayout I = img_layout(width, height);
  if (!image_state || image_bytes < I.total) { set_error("image state too small"); return DMGS_ERR_STATE; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const char *img = static_cast<const char *>(image_state);
  const size_t n = (size_t)width * height;
  if (final_T) DMGS_CUDA(cudaMemcpyAsync(final_T, img + I.final_T, n * 4, cudaMemcpyDeviceToDevice, s));
  if (n_contrib) DMGS_CUDA(cudaMemcpyAsync(n_contrib, img + I.n_contrib, n * 4, cudaMemcpyDeviceToDevice, s));
  return DMGS_OK;
}

int dmgs_bind_fwd(const DmgsFaceBinding *b, float *xyz, float *cov, float *rot_t2w,
                  float *cov3D_L, dmgs_stream_t stream) {
  if (!b || b->F < 0 || b->G <= 0 || (b->F > 0 && (!b->verts || !b->faces || !b->bc))) {
    set_error("bind_fwd: invalid arguments");
    return DMGS_ERR_ARG;
  }
  return launch_bind_fwd(*b, xyz, cov, rot_t2w, cov3D_L, reinterpret_cast<cudaStream_t>(stream));
}

int dmgs_bind_bwd(const DmgsFaceBinding *b, const float *dL_dxyz, const float *dL_dcov,
                  float *dL_dverts, float *dL_dscale_factor, dmgs_stream_t stream) {
  if (!b || b->F < 0 || b->G <= 0 || !dL_dverts ||
      (b->F > 0 && (!b->verts || !b->faces || !b->bc))) {
    set_error("bind_bwd: invalid arguments");
    return DMGS_ERR_ARG;
  }
  return launch_bind_bwd(*b, dL_dxyz, dL_dcov, dL_dverts, dL_dscale_factor,
                         reinterpret_cast<cudaStream_t>(stream));
}

int dmgs_bind3_fwd(const DmgsFaceBinding3 *b, float *xyz, float *scales, float *rotations,
                   dmgs_stream_t stream) {
  if (!b || b->F < 0 || b->G <= 0 ||
      (b->F > 0 && (!b->verts || !b->faces || !b->bc || !b->scaling2d || !b->rotation2d))) {
    set_error("bind3_fwd: invalid arguments");
    return DMGS_ERR_ARG;
  }
  return launch_bind3_fwd(*b, xyz, scales, rotations, reinterpret_cast<cudaStream_t>(stream));
}

int dmgs_bind3_bwd(const DmgsFaceBinding3 *b, const float *dL_dxyz, const float *dL_dscales,
                   const float *dL_drotations, float *dL_dverts, float *dL_dscaling2d,
                   float *dL_drotation2d, dmgs_stream_t stream) {
  if (!b || b->F < 0 || b->G <= 0 || !dL_dverts ||
      (b->F > 0 && (!b->verts || !b->faces || !b->bc || !b->scaling2d || !b->rotation2d))) {
    set_error("bind3_bwd: invalid arguments");
    return DMGS_ERR_ARG;
  }
  return launch_bind3_bwd(*b, dL_dxyz, dL_dscales, dL_drotations, dL_dverts, dL_dscaling2d,
                          dL_drotation2d, reinterpret_cast<cudaStream_t>(stream));
}

int dmgs_vertex_frustum_mask(const float *verts, int32_t N, const float *full_proj,
                             float cube_len, int32_t piece_id, int32_t n_piece,
                             const uint8_t *and_mask, uint8_t *mask, dmgs_stream_t stream) {
  if (N < 0 || (N > 0 && (!verts || !full_proj || !mask))) {
    set_error("vertex_frustum_mask: invalid arguments");
    return DMGS_ERR_ARG;
  }
  const bool ok = piece_id < 0 || (n_piece == 2 && piece_id < 2) || (n_piece == 4 && piece_id < 4);
  if (!ok) {
    set_error("vertex_frustum_mask: piece %d of %d is not a screen half or quarter", piece_id, n_piece);
    return DMGS_ERR_ARG;
  }
  return launch_vertex_frustum(verts, N, full_proj, cube_len, piece_id, n_piece, and_mask, mask,
                               reinterpret_cast<cudaStream_t>(stream));
}

size_t dmgs_face_cull_scratch_bytes(int32_t F) { return F < 0 ? 0 : face_cull_scratch_bytes(F); }

int dmgs_face_cull(const float *verts, int32_t V, const int64_t *faces, int32_t F,
                   const float *full_proj, uint8_t *face_mask, int32_t *kept_faces,
                   int32_t *num_kept, void *scratch, size_t scratch_bytes, dmgs_stream_t stream) {
  if (F < 0 || V < 0 || !num_kept || (F > 0 && (!verts || !faces || !full_proj || !kept_faces))) {
    set_error("face_cull: invalid arguments");
    return DMGS_ERR_ARG;
  }
  if (F > 0 && (!scratch || scratch_bytes < face_cull_scratch_bytes(F))) {
    set_error("face_cull: scratch too small");
    return DMGS_ERR_STATE;
  }
  return launch_face_cull(verts, V, faces, F, full_proj, face_mask, kept_faces, num_kept,
                          static_cast<char *>(scratch), reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"
