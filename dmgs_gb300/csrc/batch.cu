// batch.cu — the multi-view batched form (C ABI in include/dmgs.h).
//
// State buffer (one caller allocation): for every view its geometry state,
// instance list (capacity-bounded), image state, 2D-gradient accumulators
// and radii scratch, then two work-queue counters for the persistent blend
// launches.  Nothing here synchronises with the host, so a forward +
// backward step can be captured in a CUDA graph and replayed; the only
// host-visible result besides the outputs is the per-view status word read
// by dmgs_batch_status.
#include <cstring>

#include "kernels.cuh"

using namespace dmgs;
using dmgs_host::set_error;

namespace {

struct ViewLayout {
  size_t geom, bin, img, gacc, radii;
  GeomLayout G;
  BinLayout B;
  ImgLayout I;
};

struct BatchLayout {
  int n;
  ViewLayout v[MAX_BATCH_VIEWS];
  size_t queue, total;
};

// Layout of one view's state starting at offset o; returns the end offset.
size_t view_layout(const DmgsView &view, int P, int64_t cap, bool with_adjoint, size_t o,
                   ViewLayout &V) {
  V.G = geom_layout(P, view.width, view.height);
  V.B = bin_layout(cap, view.width, view.height, P);
  V.I = img_layout(view.width, view.height);
  V.geom = o;  o = align_up(o + V.G.total, 256);
  V.bin = o;   o = align_up(o + V.B.total, 256);
  V.img = o;   o = align_up(o + V.I.total, 256);
  V.gacc = o;  o = align_up(o + (with_adjoint ? bwd_scratch_bytes(P) : 0), 256);
  V.radii = o; o = align_up(o + (size_t)P * 4 + 4, 256);
  return o;
}

// Pv: the Gaussian count of every view (nullptr: P for all); with_adjoint:
// reserve the 2D-gradient accumulators of the backward.
int make_layout(const DmgsBatch *b, int P, BatchLayout &L, const int32_t *Pv = nullptr,
                bool with_adjoint = true) {
  if (!b || b->nviews < 1 || b->nviews > MAX_BATCH_VIEWS || !b->views || !b->capacity) {
    set_error("batch: nviews must be 1..%d with views and capacity arrays", MAX_BATCH_VIEWS);
    return DMGS_ERR_ARG;
  }
  L.n = b->nviews;
  size_t o = 0;
  for (int v = 0; v < L.n; ++v) {
    if (Pv) P = Pv[v];
    if (P < 0) {
      set_error("batch: view %d has a negative Gaussian count", v);
      return DMGS_ERR_ARG;
    }
    const DmgsView &view = b->views[v];
    if (view.width <= 0 || view.height <= 0) {
      set_error("batch: view %d has an invalid size", v);
      return DMGS_ERR_ARG;
    }
    const int64_t cap = b->capacity[v];
    if (cap < 0 || cap > 0xfffffffell) {
      set_error("batch: view %d capacity out of range", v);
      return DMGS_ERR_ARG;
    }
    o = view_layout(view, P, cap, with_adjoint, o, L.v[v]);
  }
  L.queue = o;
  o = align_up(o + 64, 256);
  L.total = o;
  return DMGS_OK;
}

ViewParams params_of(const DmgsView *v) {
  ViewParams p;
  p.W = v->width;
  p.H = v->height;
  p.gx = (v->width + TILE - 1) / TILE;
  p.gy = (v->height + TILE - 1) / TILE;
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

GaussianPtrs gptrs_of(const DmgsGaussians *g) {
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

#define RET_IF(x)                 \
  do {                            \
    int r_ = (x);                 \
    if (r_ != DMGS_OK) return r_; \
  } while (0)

int check_view(const DmgsView &w, int v) {
  if (!w.bg || !w.viewmatrix || !w.projmatrix || !w.campos || w.sh_degree < 0 ||
      w.sh_degree > 3 || !(w.tanfovx > 0.f) || !(w.tanfovy > 0.f)) {
    set_error("batch: view %d is invalid", v);
    return DMGS_ERR_ARG;
  }
  return DMGS_OK;
}

// The Gaussian set rendered by view v (input-mode rules of the drop-in).
int check_gaussians(const DmgsGaussians *g, const DmgsView &w, int v) {
  if (!g || g->P < 0) { set_error("batch: invalid Gaussians for view %d", v); return DMGS_ERR_ARG; }
  if (g->P == 0) return DMGS_OK;
  if (!g->means3D || !g->opacities || (g->shs == nullptr) == (g->colors_precomp == nullptr) ||
      ((g->scales == nullptr || g->rotations == nullptr) && g->cov3D_precomp == nullptr) ||
      ((g->scales != nullptr || g->rotations != nullptr) && g->cov3D_precomp != nullptr)) {
    set_error("batch: give exactly one colour source and one covariance source");
    return DMGS_ERR_ARG;
  }
  if (g->shs && g->M < (w.sh_degree + 1) * (w.sh_degree + 1)) {
    set_error("batch: too few SH coefficients for view %d", v);
    return DMGS_ERR_ARG;
  }
  if (g->rotations && (reinterpret_cast<uintptr_t>(g->rotations) & 15)) {
    set_error("rotations must be 16-byte aligned");
    return DMGS_ERR_ARG;
  }
  return DMGS_OK;
}

int check_common(const DmgsBatch *b, const DmgsGaussians *g, void *state, size_t bytes,
                 BatchLayout &L) {
  if (!g || g->P < 0) { set_error("batch: invalid Gaussians"); return DMGS_ERR_ARG; }
  int r = make_layout(b, g->P, L);
  if (r != DMGS_OK) return r;
  if (!state || bytes < L.total) {
    set_error("batch: state too small: %zu < %zu bytes", bytes, L.total);
    return DMGS_ERR_STATE;
  }
  for (int v = 0; v < b->nviews; ++v) RET_IF(check_view(b->views[v], v));
  for (int v = 0; v < b->nviews; ++v) RET_IF(check_gaussians(g, b->views[v], v));
  const int ppt = b->pixels_per_thread ? b->pixels_per_thread : 4;
  const int gpb = b->gaussians_per_batch ? b->gaussians_per_batch : 128;
  const bool pair = b->tile_shape == 1 || b->tile_shape == 2;
  if ((ppt != 1 && ppt != 2 && ppt != 4) || (gpb != 128 && gpb != 256 && gpb != 512) ||
      b->tile_shape < 0 || b->tile_shape > 2 || (pair && (ppt == 1 || gpb == 512))) {
    set_error("batch: unsupported blend tuning: %d pixels/thread, batch %d, tile shape %d", ppt,
              gpb, b->tile_shape);
    return DMGS_ERR_ARG;
  }
  return DMGS_OK;
}

BlendCfg cfg_of(const DmgsBatch *b) {
  BlendCfg c = default_blend_cfg();
  if (b->pixels_per_thread) c.ppt = b->pixels_per_thread;
  if (b->gaussians_per_batch) c.batch = b->gaussians_per_batch;
  if (b->tile_shape == 1) c.sx = 2;
  if (b->tile_shape == 2) c.sy = 2;
  return c;
}

struct SameBase {
  char *p[MAX_BATCH_VIEWS];
  operator char *const *() const { return p; }
};
SameBase same_base(char *st) {
  SameBase b;
  for (int v = 0; v < MAX_BATCH_VIEWS; ++v) b.p[v] = st;
  return b;
}

// base[v]: the buffer view v's layout offsets are relative to.
void fill_views(const DmgsBatch *b, const BatchLayout &L, char *const *base, BatchViews &bv) {
  bv.nviews = b->nviews;
  for (int v = 0; v < b->nviews; ++v) {
    const ViewLayout &V = L.v[v];
    char *st = base[v];
    char *geom = st + V.geom;
    BatchView &o = bv.v[v];
    o.vp = params_of(&b->views[v]);
    o.viewm = b->views[v].viewmatrix;
    o.projm = b->views[v].projmatrix;
    o.campos = b->views[v].campos;
    o.radii = (b->radii && b->radii[v]) ? b->radii[v] : reinterpret_cast<int32_t *>(st + V.radii);
    o.feat = reinterpret_cast<float4 *>(geom + V.G.feat);
    o.flags = reinterpret_cast<uint8_t *>(geom + V.G.flags);
    o.blkcnt = reinterpret_cast<uint32_t *>(geom + V.G.blkcnt);
    o.counters = reinterpret_cast<uint32_t *>(geom + V.G.counters);
    o.gacc = reinterpret_cast<const float *>(st + V.gacc);
    o.dL_dmeans2D = nullptr;
  }
}

void fill_blend(const DmgsBatch *b, const BatchLayout &L, char *const *bases, BlendBatch &bb) {
  bb.nviews = b->nviews;
  int base = 0;
  for (int v = 0; v < b->nviews; ++v) {
    const ViewLayout &V = L.v[v];
    char *st = bases[v];
    char *geom = st + V.geom, *bin = st + V.bin, *img = st + V.img;
    BlendView &o = bb.v[v];
    o.W = b->views[v].width;
    o.H = b->views[v].height;
    o.gx = V.G.gx;
    o.T = V.G.T();
    o.P = (uint32_t)V.G.P;
    o.tile_base = base;
    base += o.T;
    o.ranges = reinterpret_cast<const uint2 *>(geom + V.G.ranges);
    o.point_list = reinterpret_cast<const uint32_t *>(bin + V.B.point_list);
    o.feat = reinterpret_cast<const float4 *>(geom + V.G.feat);
    o.bg = b->views[v].bg;
    o.out_color = b->out_color ? b->out_color[v] : nullptr;
    o.final_T = reinterpret_cast<float *>(img + V.I.final_T);
    o.n_contrib = reinterpret_cast<uint32_t *>(img + V.I.n_contrib);
    o.dL_dout = nullptr;
    o.gacc = reinterpret_cast<float *>(st + V.gacc);
    o.gacc64 = nullptr;
  }
  bb.total = base;
}

}  // namespace

extern "C" size_t dmgs_batch_state_bytes(const DmgsBatch *b, int32_t P) {
  BatchLayout L;
  if (P < 0 || make_layout(b, P, L) != DMGS_OK) return 0;
  return L.total;
}

extern "C" int dmgs_raster_fwd_batched(const DmgsBatch *b, const DmgsGaussians *g, void *state,
                                       size_t state_bytes, dmgs_stream_t stream) {
  BatchLayout L;
  RET_IF(check_common(b, g, state, state_bytes, L));
  if (!b->out_color) { set_error("batch: out_color is NULL"); return DMGS_ERR_ARG; }
  for (int v = 0; v < b->nviews; ++v)
    if (!b->out_color[v]) { set_error("batch: out_color[%d] is NULL", v); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char *st = static_cast<char *>(state);
  BatchViews bv;
  fill_views(b, L, same_base(st), bv);
  RET_IF(launch_preprocess_batched(bv, gptrs_of(g), s));
  BinViews bins;
  bins.n = b->nviews;
  for (int v = 0; v < b->nviews; ++v) {
    const ViewLayout &V = L.v[v];
    RET_IF(make_bin_view(V.G, st + V.geom, (uint32_t)b->capacity[v], st + V.bin + V.B.point_list,
                         (uint32_t)b->capacity[v], bins.v[v]));
  }
  RET_IF(launch_binning_geometry(bins, s));
  RET_IF(launch_emit(bins, s));
  BlendBatch bb;
  fill_blend(b, L, same_base(st), bb);
  uint32_t *queue = reinterpret_cast<uint32_t *>(st + L.queue);
  DMGS_CUDA(cudaMemsetAsync(queue, 0, 4, s));
  RET_IF(launch_blend_batch_fwd(bb, cfg_of(b), queue, s));
  return DMGS_OK;
}

extern "C" int dmgs_raster_bwd_batched(const DmgsBatch *b, const DmgsGaussians *g,
                                       const float *const *dL_dout_color, void *state,
                                       size_t state_bytes, const DmgsGrads *grads,
                                       float *const *dL_dmeans2D, float *densify_accum,
                                       float *densify_count, dmgs_stream_t stream) {
  BatchLayout L;
  RET_IF(check_common(b, g, state, state_bytes, L));
  if (!dL_dout_color || !grads) { set_error("batch: dL_dout_color / grads is NULL"); return DMGS_ERR_ARG; }
  if ((densify_accum == nullptr) != (densify_count == nullptr)) {
    set_error("batch: densify_accum and densify_count must both be given or both be NULL");
    return DMGS_ERR_ARG;
  }
  for (int v = 0; v < b->nviews; ++v)
    if (!dL_dout_color[v]) { set_error("batch: dL_dout_color[%d] is NULL", v); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char *st = static_cast<char *>(state);
  BlendBatch bb;
  fill_blend(b, L, same_base(st), bb);
  for (int v = 0; v < b->nviews; ++v) {
    bb.v[v].dL_dout = dL_dout_color[v];
    DMGS_CUDA(cudaMemsetAsync(bb.v[v].gacc, 0, (size_t)g->P * 48, s));
  }
  uint32_t *queue = reinterpret_cast<uint32_t *>(st + L.queue) + 1;
  DMGS_CUDA(cudaMemsetAsync(queue, 0, 4, s));
  RET_IF(launch_blend_batch_bwd(bb, cfg_of(b), queue, s));
  BatchViews bv;
  fill_views(b, L, same_base(st), bv);
  for (int v = 0; v < b->nviews; ++v) bv.v[v].dL_dmeans2D = dL_dmeans2D ? dL_dmeans2D[v] : nullptr;
  RET_IF(launch_preprocess_bwd_batched(bv, gptrs_of(g), *grads, densify_accum, densify_count, s));
  return DMGS_OK;
}

extern "C" int dmgs_batch_status(const DmgsBatch *b, int32_t P, const void *state,
                                 size_t state_bytes, int64_t *num_rendered, dmgs_stream_t stream) {
  BatchLayout L;
  RET_IF(make_layout(b, P, L));
  if (!state || state_bytes < L.total) { set_error("batch: state too small"); return DMGS_ERR_STATE; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const char *st = static_cast<const char *>(state);
  uint32_t h[MAX_BATCH_VIEWS][CI_WORDS];
  for (int v = 0; v < b->nviews; ++v)
    DMGS_CUDA(cudaMemcpyAsync(h[v], st + L.v[v].geom + L.v[v].G.counters, CI_WORDS * 4,
                              cudaMemcpyDeviceToHost, s));
  DMGS_CUDA(cudaStreamSynchronize(s));
  int rc = DMGS_OK;
  for (int v = 0; v < b->nviews; ++v) {
    if (num_rendered) num_rendered[v] = (int64_t)h[v][CI_K];
    if (h[v][CI_STATUS] & ST_OVERFLOW) {
      set_error("batch: view %d needs %u instances, capacity %lld", v, h[v][CI_K],
                (long long)b->capacity[v]);
      rc = DMGS_ERR_OVERFLOW;
    } else if ((h[v][CI_STATUS] & ST_PREFILTER) && rc == DMGS_OK) {
      set_error("batch: view %d: a point failed the frustum test although prefiltered is set", v);
      rc = DMGS_ERR_PREFILTER;
    } else if ((h[v][CI_STATUS] & ST_BOUNDS) && rc == DMGS_OK) {
      set_error("batch: view %d: a kernel index left its buffer", v);
      rc = DMGS_ERR_DEVICE;
    }
  }
  return rc;
}

extern "C" int dmgs_batch_counters(const DmgsBatch *b, int32_t P, const void *state,
                                   size_t state_bytes, uint32_t *words, dmgs_stream_t stream) {
  BatchLayout L;
  RET_IF(make_layout(b, P, L));
  if (!state || state_bytes < L.total) { set_error("batch: state too small"); return DMGS_ERR_STATE; }
  if (!words) { set_error("batch: words is NULL"); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const char *st = static_cast<const char *>(state);
  for (int v = 0; v < b->nviews; ++v)
    DMGS_CUDA(cudaMemcpyAsync(words + 16 * v, st + L.v[v].geom + L.v[v].G.counters, CI_WORDS * 4,
                              cudaMemcpyDeviceToHost, s));
  DMGS_CUDA(cudaStreamSynchronize(s));
  return DMGS_OK;
}

// ---------------------------------------------------------------------------
// Serving form: every view renders its own Gaussian set (requests for
// several resident scenes in one launch sequence), forward only, each view
// in its own state buffer (requests are placed independently in an arena).
// ---------------------------------------------------------------------------

namespace {

int multi_check(const DmgsBatch *b, const DmgsGaussians *g, void *const *state,
                const size_t *state_bytes, BatchLayout &L) {
  if (!g || !state || !state_bytes) {
    set_error("multi: gaussians, state or state_bytes is NULL");
    return DMGS_ERR_ARG;
  }
  if (!b || b->nviews < 1 || b->nviews > MAX_BATCH_VIEWS || !b->views || !b->capacity) {
    set_error("multi: nviews must be 1..%d with views and capacity arrays", MAX_BATCH_VIEWS);
    return DMGS_ERR_ARG;
  }
  L.n = b->nviews;
  for (int v = 0; v < b->nviews; ++v) {
    RET_IF(check_view(b->views[v], v));
    RET_IF(check_gaussians(&g[v], b->views[v], v));
    const int64_t cap = b->capacity[v];
    if (cap < 0 || cap > 0xfffffffell || b->views[v].width <= 0 || b->views[v].height <= 0) {
      set_error("multi: view %d has an invalid size or capacity", v);
      return DMGS_ERR_ARG;
    }
    const size_t need = view_layout(b->views[v], g[v].P, cap, false, 0, L.v[v]);
    if (!state[v] || state_bytes[v] < need) {
      set_error("multi: state of view %d too small: %zu < %zu bytes", v, state_bytes[v], need);
      return DMGS_ERR_STATE;
    }
  }
  return DMGS_OK;
}

}  // namespace

extern "C" size_t dmgs_multi_view_state_bytes(const DmgsView *view, const DmgsGaussians *g,
                                              int64_t capacity) {
  if (!view || !g || g->P < 0 || capacity < 0 || view->width <= 0 || view->height <= 0) return 0;
  ViewLayout V;
  return view_layout(*view, g->P, capacity, false, 0, V);
}

extern "C" int dmgs_render_multi(const DmgsBatch *b, const DmgsGaussians *g, void *const *state,
                                 const size_t *state_bytes, uint32_t *queue,
                                 dmgs_stream_t stream) {
  BatchLayout L;
  RET_IF(multi_check(b, g, state, state_bytes, L));
  if (!b->out_color || !queue) { set_error("multi: out_color or queue is NULL"); return DMGS_ERR_ARG; }
  for (int v = 0; v < b->nviews; ++v)
    if (!b->out_color[v]) { set_error("multi: out_color[%d] is NULL", v); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char *const *base = reinterpret_cast<char *const *>(state);
  BatchViews bv;
  fill_views(b, L, base, bv);
  BinViews bins;
  bins.n = b->nviews;
  for (int v = 0; v < b->nviews; ++v) {
    const ViewLayout &V = L.v[v];
    const BatchView &o = bv.v[v];
    RET_IF(launch_preprocess(o.vp, o.viewm, o.projm, o.campos, gptrs_of(&g[v]), o.radii, V.G,
                             base[v] + V.geom, s));
    RET_IF(make_bin_view(V.G, base[v] + V.geom, (uint32_t)b->capacity[v],
                         base[v] + V.bin + V.B.point_list, (uint32_t)b->capacity[v], bins.v[v]));
  }
  RET_IF(launch_binning_geometry(bins, s));
  RET_IF(launch_emit(bins, s));
  BlendBatch bb;
  fill_blend(b, L, base, bb);
  DMGS_CUDA(cudaMemsetAsync(queue, 0, 4, s));
  RET_IF(launch_blend_batch_fwd(bb, cfg_of(b), queue, s));
  return DMGS_OK;
}

extern "C" int dmgs_multi_status_async(const DmgsBatch *b, const DmgsGaussians *g,
                                       void *const *state, const size_t *state_bytes,
                                       uint32_t *host_words, dmgs_stream_t stream) {
  BatchLayout L;
  RET_IF(multi_check(b, g, state, state_bytes, L));
  if (!host_words) { set_error("multi: host_words is NULL"); return DMGS_ERR_ARG; }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  for (int v = 0; v < b->nviews; ++v)  // words CI_STATUS, CI_K
    DMGS_CUDA(cudaMemcpyAsync(host_words + 2 * v,
                              static_cast<const char *>(state[v]) + L.v[v].geom + L.v[v].G.counters,
                              8, cudaMemcpyDeviceToHost, s));
  return DMGS_OK;
}
