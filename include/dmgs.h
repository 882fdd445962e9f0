/*
 * dmgs.h — C ABI of the GB300 (sm_103a) Gaussian-splatting rasteriser and
 * mesh->Gaussian face binding.
 *
 * Plain pointers and sizes only.  Every pointer argument documented as
 * "device" is a CUDA device address; every call is asynchronous on the given
 * stream unless documented otherwise.  Functions return DMGS_OK (0) or a
 * negative DMGS_ERR_* code; dmgs_last_error() then holds a message for the
 * calling thread.  No exception crosses this boundary.
 *
 * The reference calls its rasteriser through the pybind module
 * `diff_gaussian_rasterization._C` of the un-vendored submodule
 * submodules/diff-gaussian-rasterization (.gitmodules:4-6): entry points
 * `rasterize_gaussians`, `rasterize_gaussians_backward` and `mark_visible`,
 * reached from `GaussianRasterizer.forward` / `markVisible`, which the
 * reference tree calls at gaussian_renderer/__init__.py:51,86-94 and
 * :144,178-186.  The binding entry points replace the torch-op chains of
 * scene/gaussian_geo_model_mlp_flex.py:267-316,370-385 and
 * scene/gaussian_geo_model_finetune.py:414-421,446-483.
 */
#ifndef DMGS_H
#define DMGS_H

#include <stddef.h>
#include <stdint.h>

/* Version of the structs and entry points below; dmgs_abi_version() returns
 * the value the library was built with.  Raised whenever a struct layout or
 * a signature changes. */
#define DMGS_ABI_VERSION 8

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *dmgs_stream_t; /* identical to cudaStream_t */

enum {
  DMGS_OK = 0,
  DMGS_ERR_ARG = -1,       /* invalid argument: size, null pointer, input mode */
  DMGS_ERR_CUDA = -2,      /* a CUDA runtime call failed */
  DMGS_ERR_STATE = -3,     /* a state buffer is smaller than required */
  DMGS_ERR_PREFILTER = -4, /* prefiltered=1 but a point failed the frustum test */
  DMGS_ERR_OVERFLOW = -5,  /* a capacity-bounded buffer ran out of instance slots */
  DMGS_ERR_DEVICE = -6     /* a kernel reported a bounds or wait-limit failure */
};

#define DMGS_TILE 16 /* tile edge in pixels (16 x 16 tiles) */

/* Per-view constants: the fields of GaussianRasterizationSettings
 * (built at gaussian_renderer/__init__.py:36-49). */
typedef struct DmgsView {
  int32_t width, height;   /* image size in pixels */
  float tanfovx, tanfovy;  /* tan(FoV/2) */
  float scale_modifier;    /* multiplies `scales` (scale/rotation mode) */
  int32_t sh_degree;       /* active SH degree D, 0..3 */
  int32_t prefiltered;     /* 1: caller guarantees every point is in front of z=0.2 */
  int32_t debug;           /* 1: synchronise and check after every kernel */
  const float *bg;         /* [3] device, background colour */
  const float *viewmatrix; /* [16] device, world->view, column-major
                              (scene/cameras.py:54 storage) */
  const float *projmatrix; /* [16] device, world->clip (scene/cameras.py:56) */
  const float *campos;     /* [3] device, camera centre (scene/cameras.py:57) */
} DmgsView;

/* Gaussian inputs.  Exactly one of {shs, colors_precomp} and exactly one of
 * {scales+rotations, cov3D_precomp} must be non-NULL (the reference raises
 * otherwise).  All arrays are device, fp32, contiguous. */
typedef struct DmgsGaussians {
  int32_t P;                   /* number of Gaussians */
  int32_t M;                   /* SH coefficients per Gaussian in `shs` */
  const float *means3D;        /* [P,3] */
  const float *opacities;      /* [P] (activated) */
  const float *shs;            /* [P,M,3] coefficient-major, or NULL */
  const float *colors_precomp; /* [P,3] or NULL */
  const float *scales;         /* [P,3] or NULL */
  const float *rotations;      /* [P,4] quaternion (r,x,y,z), used as given */
  const float *cov3D_precomp;  /* [P,6] (xx,xy,xz,yy,yz,zz) or NULL */
} DmgsGaussians;

/* Gradient outputs of the backward pass (all device, fp32).  Every array
 * given is fully written (zeros for culled Gaussians); NULL entries are
 * skipped.  dL_dmeans2D is w.r.t. NDC (x, y); its third column is zero. */
typedef struct DmgsGrads {
  float *dL_dmeans2D;   /* [P,3] */
  float *dL_dcolors;    /* [P,3] */
  float *dL_dopacity;   /* [P]   */
  float *dL_dmeans3D;   /* [P,3] */
  float *dL_dcov3D;     /* [P,6] */
  float *dL_dsh;        /* [P,M,3] */
  float *dL_dscales;    /* [P,3] */
  float *dL_drotations; /* [P,4] */
} DmgsGrads;

/* ---------------------------------------------------------------------- *
 * State buffers.  The forward pass keeps three caller-owned device buffers
 * (the reference's geomBuffer / binningBuffer / imgBuffer) that the
 * backward pass reads again.  Sizes in bytes; every buffer 256-B aligned.
 * ---------------------------------------------------------------------- */
size_t dmgs_geom_state_bytes(int32_t P, int32_t width, int32_t height);
size_t dmgs_binning_state_bytes(int64_t num_rendered, int32_t width, int32_t height);
size_t dmgs_image_state_bytes(int32_t width, int32_t height);
size_t dmgs_bwd_scratch_bytes(int32_t P);

/* Forward, phase 1 (replaces the preprocess + tile-count half of
 * `rasterize_gaussians`): per-Gaussian projection, covariance, conic, radius,
 * SH colour and tile rectangle; per-tile instance counts and offsets.
 * Writes radii [P] (device, int32).  Synchronises the stream once and
 * returns the number of (tile, Gaussian) instances in *num_rendered (host). */
int dmgs_raster_fwd_geometry(const DmgsView *view, const DmgsGaussians *g,
                             void *geom_state, size_t geom_bytes, int32_t *radii,
                             int64_t *num_rendered, dmgs_stream_t stream);

/* Forward, phase 2 (replaces the binning + blend half of
 * `rasterize_gaussians`): emits the instances, sorts every tile's list by
 * (depth, index), writes tile ranges and blends out_color [3,H,W] (device). */
int dmgs_raster_fwd_render(const DmgsView *view, const DmgsGaussians *g,
                           void *geom_state, size_t geom_bytes,
                           void *binning_state, size_t binning_bytes,
                           int64_t num_rendered, void *image_state,
                           size_t image_bytes, float *out_color,
                           dmgs_stream_t stream);

/* One-call forward with caller allocation callbacks (the reference's
 * resize-functor design): alloc(ctx, which, bytes) returns a device buffer
 * of at least `bytes` for which = 0 (geometry), 1 (binning), 2 (image), or
 * NULL on failure.  Returns num_rendered in *num_rendered. */
typedef void *(*dmgs_alloc_fn)(void *ctx, int32_t which, size_t bytes);
int dmgs_raster_fwd(const DmgsView *view, const DmgsGaussians *g,
                    dmgs_alloc_fn alloc, void *alloc_ctx, int32_t *radii,
                    float *out_color, int64_t *num_rendered,
                    dmgs_stream_t stream);

/* Backward (replaces `rasterize_gaussians_backward`): blend adjoint then
 * preprocess adjoint.  dL_dout_color [3,H,W] device.  `bwd_scratch` holds
 * dmgs_bwd_scratch_bytes(P) bytes. */
int dmgs_raster_bwd(const DmgsView *view, const DmgsGaussians *g,
                    const float *dL_dout_color, const void *geom_state,
                    size_t geom_bytes, const void *binning_state,
                    size_t binning_bytes, int64_t num_rendered,
                    const void *image_state, size_t image_bytes,
                    void *bwd_scratch, size_t bwd_scratch_bytes,
                    const DmgsGrads *grads, dmgs_stream_t stream);

/* Backward with FP64 gradient sums (no counterpart in the reference): the
 * same arguments and results as dmgs_raster_bwd, but the blend adjoint adds
 * every Gaussian's per-pixel gradient terms into double-precision
 * accumulators, so the gradients do not depend on the order in which tiles
 * and warps finish (to well below float32 resolution).  dmgs_raster_bwd adds
 * them with float atomics, whose order changes from run to run.  A
 * verification mode, slower than dmgs_raster_bwd; `bwd_scratch` holds
 * dmgs_bwd_scratch_f64_bytes(P) bytes (144 per Gaussian). */
size_t dmgs_bwd_scratch_f64_bytes(int32_t P);
int dmgs_raster_bwd_f64sum(const DmgsView *view, const DmgsGaussians *g,
                           const float *dL_dout_color, const void *geom_state,
                           size_t geom_bytes, const void *binning_state,
                           size_t binning_bytes, int64_t num_rendered,
                           const void *image_state, size_t image_bytes,
                           void *bwd_scratch, size_t bwd_scratch_bytes,
                           const DmgsGrads *grads, dmgs_stream_t stream);

/* Backward for callers that cannot allocate device memory (this entry point
 * has no counterpart in the reference).  A plugin inside a host application
 * that owns the device's memory pool, or a real-time loop that must not call
 * cudaMalloc/cudaFree between frames, cannot hand dmgs_raster_bwd its
 * scratch buffer; this variant keeps that scratch in a static device array
 * of the library instead (DMGS_NOALLOC_MAX_GAUSSIANS x 48 bytes = 12 MiB,
 * held by every GPU that loads the library until exit) and allocates
 * nothing.  Arguments and results are those of dmgs_raster_bwd without the
 * scratch pair; g->P above the limit returns DMGS_ERR_ARG.  The first call on
 * a device looks up the array's address (cudaGetSymbolAddress), so make it
 * before any stream capture begins.  All calls share the array: calls whose
 * work overlaps on the GPU race.  The looked-up address is kept for the life
 * of the process: after a cudaDeviceReset on a device, do not call this entry
 * point on that device again (the array may then live at another address). */
#define DMGS_NOALLOC_MAX_GAUSSIANS 262144
int dmgs_raster_bwd_noalloc(const DmgsView *view, const DmgsGaussians *g,
                            const float *dL_dout_color, const void *geom_state,
                            size_t geom_bytes, const void *binning_state,
                            size_t binning_bytes, int64_t num_rendered,
                            const void *image_state, size_t image_bytes,
                            const DmgsGrads *grads, dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Multi-view batched form (no counterpart in the reference, which renders
 * one view per call: render_and_eval.py:42-44, train_geo_stage2.py:101).
 * A batch of views of one Gaussian set: one preprocess pass for all views,
 * per-view binning into capacity-bounded instance lists (no host
 * synchronisation, so the calls can be captured in a CUDA graph), blending
 * of every view's tiles by one persistent launch, and an adjoint that sums
 * the views' gradients and writes them once.  A view whose instances exceed
 * its capacity renders background and is reported by dmgs_batch_status.
 * ---------------------------------------------------------------------- */
#define DMGS_MAX_BATCH_VIEWS 16
typedef struct DmgsBatch {
  int32_t nviews;                  /* 1..DMGS_MAX_BATCH_VIEWS */
  const DmgsView *views;           /* [nviews] host array */
  float *const *out_color;         /* [nviews] device pointers, [3,H,W] each */
  int32_t *const *radii;           /* [nviews] device pointers to [P], or NULL */
  const int64_t *capacity;         /* [nviews] instance-list capacity per view */
  int32_t pixels_per_thread;       /* blend tuning: 1, 2 or 4 (0: 4) */
  int32_t gaussians_per_batch;     /* blend tuning: 128, 256 or 512 (0: 128) */
  int32_t tile_shape;              /* blend tuning, pixels per CTA: 0 = 16x16 (one binning
                                      tile), 1 = 32x16, 2 = 16x32 (two adjacent tiles, each
                                      blended from its own list; pixels per thread 2 or 4,
                                      batch 128 or 256) */
} DmgsBatch;

size_t dmgs_batch_state_bytes(const DmgsBatch *b, int32_t P);
/* Forward of every view; asynchronous, no host synchronisation. */
int dmgs_raster_fwd_batched(const DmgsBatch *b, const DmgsGaussians *g,
                            void *state, size_t state_bytes,
                            dmgs_stream_t stream);
/* Adjoint of the batch: dL_dout_color[v] [3,H,W] per view; `grads` receive
 * the sum over views (its dL_dmeans2D is unused); dL_dmeans2D[v] (may be
 * NULL, or have NULL entries) receives view v's NDC-mean gradient [P,3].
 * densify_accum / densify_count ([P] each, both or neither, may be NULL):
 * the reference's densification statistics fused over the batch
 * (scene/gaussian_model.py:405-407, called once per view by train.py:116):
 * for every view v in which Gaussian i is visible, densify_accum[i] +=
 * |(dL_dmeans2D[v][i][0], dL_dmeans2D[v][i][1])| and densify_count[i] += 1.
 * They accumulate across calls; the caller zeroes them. */
int dmgs_raster_bwd_batched(const DmgsBatch *b, const DmgsGaussians *g,
                            const float *const *dL_dout_color, void *state,
                            size_t state_bytes, const DmgsGrads *grads,
                            float *const *dL_dmeans2D, float *densify_accum,
                            float *densify_count, dmgs_stream_t stream);
/* Synchronises the stream, writes each view's instance count to
 * num_rendered[v] and returns DMGS_ERR_OVERFLOW when a view exceeded its
 * capacity (or another DMGS_ERR_* from a view's status word). */
int dmgs_batch_status(const DmgsBatch *b, int32_t P, const void *state,
                      size_t state_bytes, int64_t *num_rendered,
                      dmgs_stream_t stream);

/* Diagnostics (no counterpart in the reference): synchronises the stream and
 * copies each view's 16 binning counter words into words[16v .. 16v+15]
 * (host): 0 status bits, 1 instances K, 2 row-list entries (visible Gaussian
 * x tile row it covers), 3 longest tile list, 4 visible Gaussians, 8 binning
 * chunks; the other words are internal. */
int dmgs_batch_counters(const DmgsBatch *b, int32_t P, const void *state,
                        size_t state_bytes, uint32_t *words, dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Serving form (no counterpart in the reference): a batch whose views each
 * render their own Gaussian set — render requests for several resident
 * scenes — forward only, in one launch sequence: per-view preprocess and
 * capacity-bounded binning, then one persistent blend over every view's
 * tiles.  `g` points to nviews Gaussian sets (g[v] is rendered by view v);
 * each view has its own state buffer state[v] of state_bytes[v] >=
 * dmgs_multi_view_state_bytes(view, g, capacity) bytes (so requests can be
 * placed independently in a device arena); `queue` is 4 bytes of device
 * memory for the blend's work counter.  b->radii may be NULL (the state
 * holds a radii scratch).  No host synchronisation, no adjoint scratch.
 * ---------------------------------------------------------------------- */
size_t dmgs_multi_view_state_bytes(const DmgsView *view, const DmgsGaussians *g,
                                   int64_t capacity);
int dmgs_render_multi(const DmgsBatch *b, const DmgsGaussians *g, void *const *state,
                      const size_t *state_bytes, uint32_t *queue,
                      dmgs_stream_t stream);
/* Enqueues on `stream` the copy of view v's status word and instance count
 * into host_words[2v] and host_words[2v+1] (host memory, pinned for the copy
 * to stay asynchronous); read them once the stream has passed this point.
 * Status bits: 1 prefiltered point culled, 2 capacity overflow (the view
 * rendered background; the count is the capacity it needs), 4 index out of
 * its buffer. */
int dmgs_multi_status_async(const DmgsBatch *b, const DmgsGaussians *g,
                            void *const *state, const size_t *state_bytes,
                            uint32_t *host_words, dmgs_stream_t stream);

/* Frustum face culling of the stage-3 binding (replaces in_frustum and the
 * face selection of scene/gaussian_geo_model_finetune.py:33-48,404-409):
 * face f is kept when its centroid, taken through full_proj (the camera's
 * full_proj_transform as stored, 16 floats, device), has |x/w|, |y/w|, |z/w|
 * < 1.05 with w = p.w + 1e-6 > 0.  face_mask[F] (may be NULL) receives
 * 1/0 per face; kept_faces receives the kept face indices in order and
 * *num_kept (device int32) their number.  verts: [V,3], faces: [F,3] int64
 * (device); a face with a vertex index outside [0, V) is not kept. */
size_t dmgs_face_cull_scratch_bytes(int32_t F);
/* Vertex frustum mask of the real-scene stage 2 (replaces in_frustum,
 * scene/gaussian_geo_model_mlp_flex_colmap.py:31-76, as getMesh_in_frustum
 * calls it at :299-302 and :319-322): vertex i of verts [N,3] (device) is
 * moved by cube_len / 2 on every axis, taken through full_proj (16 floats,
 * device, stored row-vector convention) and kept (mask[i] = 1) when
 * w = p.w + 1e-6 > 0 and p.xyz / w lies in the screen piece widened by
 * 0.05: the whole screen for piece_id < 0, else half piece_id of n_piece = 2
 * (left, right) or quarter piece_id of n_piece = 4 (bit 0: right, bit 1:
 * top); z always within +-1.05.  and_mask ([N] bytes, may be NULL) is
 * ANDed in (the background grid's vertex mask). */
int dmgs_vertex_frustum_mask(const float *verts, int32_t N, const float *full_proj,
                             float cube_len, int32_t piece_id, int32_t n_piece,
                             const uint8_t *and_mask, uint8_t *mask, dmgs_stream_t stream);
int dmgs_face_cull(const float *verts, int32_t V, const int64_t *faces, int32_t F,
                   const float *full_proj, uint8_t *face_mask, int32_t *kept_faces,
                   int32_t *num_kept, void *scratch, size_t scratch_bytes,
                   dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * FlexiCubes isosurface extraction on a regular grid (replaces the
 * triangle path of `FlexiCubes.__call__`, geo/flexicubes.py:180-260, with
 * grad_func=None and output_tetmesh=False, as stage 2 calls it:
 * scene/gaussian_geo_model_mlp_flex.py:250-251).  The grid is the one of
 * `construct_voxel_grid_v2` (geo/flexicubes.py:133-157): vertices in
 * (i, j, k) lexicographic order, N = (rx+1)(ry+1)(rz+1), cubes likewise,
 * C = rx ry rz.  Weights are the RAW per-cube parameters (normalised inside
 * as beta = tanh(b) 0.99 + 1, alpha = tanh(a) 0.99 + 1,
 * gamma = sigmoid(g) 0.99 + 0.005); NULL means all ones after
 * normalisation, as in the reference.
 *
 * Three calls: dmgs_fc_count runs the classification and the scans and
 * returns (after synchronising the stream) counts[8] = {surface cubes, dual
 * vertices, L_dev entries, surface edges, quads, flipped quads, 0, 0};
 * the caller sizes the outputs from them:
 *   vertices [n_vd + n_quads (training) | n_vd, 3] f32,
 *   faces    [4 n_quads (training) | 2 n_quads, 3] int64,
 *   L_dev    [n_entries] f32, surf_edges [n_edges, 2] int64,
 *   work     dmgs_fc_work_bytes(counts) bytes (kept for the adjoint);
 * dmgs_fc_emit writes them in the reference's order; dmgs_fc_bwd takes
 * dL/dvertices (MODIFIED: the quad centres' gradients are added to the dual
 * vertices' rows) and dL/dL_dev and writes dense gradients w.r.t. x [N,3],
 * s [N] and the raw weights [C,12], [C,8], [C] (each optional when its
 * weight is NULL).
 * ---------------------------------------------------------------------- */
typedef struct DmgsFcGrid {
  const float *x;     /* [N,3] vertex positions (deformed grid) */
  const float *s;     /* [N] scalar field, s < 0 inside */
  const float *beta;  /* [C,12] raw edge weights or NULL */
  const float *alpha; /* [C,8] raw corner weights or NULL */
  const float *gamma; /* [C] raw quad-split weights or NULL */
  int32_t rx, ry, rz; /* cubes per axis */
  int32_t training;   /* 1: four triangles per quad around a centre vertex */
  /* row strides in floats of beta / alpha / gamma (0: dense, 12 / 8 / 1);
   * the gradient arrays of dmgs_fc_bwd use the same strides.  The reference
   * passes column slices of one [C,21] tensor (strides 21, 21, 21). */
  int32_t beta_stride, alpha_stride, gamma_stride;
  /* Cube subset of the per-view extraction of the real-scene stage 2
   * (construct_cubes of geo/flexicubes_no_adjacent.py:129-145, fed by the
   * vertex frustum mask of scene/gaussian_geo_model_mlp_flex_colmap.py:
   * 299-303): [N] bytes, cube (i,j,k) takes part iff the mask of its corner
   * (i,j,k) is non-zero; NULL: every cube.  With a subset, a surface edge is
   * listed when a participating cube holds it and becomes a quad only when
   * all four cubes around it participate (the reference's edge counts), and
   * the weights must be NULL. */
  const uint8_t *vert_mask;
  /* 1: no C16/C19 re-check (geo/flexicubes_no_adjacent.py:300-340 with
   * de_ambiguity=False, as that variant is called); 0: the re-check of
   * geo/flexicubes.py (required to be 1 with a cube subset). */
  int32_t no_ambiguity_check;
} DmgsFcGrid;

/* Dual Marching Cubes tables the library derives: groups[256*4] edge masks of
 * the dual vertices, num_vd[256], check[256*5] (flag, di, dj, dk, complement
 * case) — the meaning of geo/tables.py's dmc_table / num_vd_table /
 * check_table.  Host only. */
int dmgs_fc_tables(uint16_t *groups, uint8_t *num_vd, int8_t *check);
size_t dmgs_fc_state_bytes(int32_t rx, int32_t ry, int32_t rz);
size_t dmgs_fc_work_bytes(const uint32_t *counts);
int dmgs_fc_count(const DmgsFcGrid *g, void *state, size_t state_bytes, uint32_t *counts,
                  dmgs_stream_t stream);
int dmgs_fc_emit(const DmgsFcGrid *g, const uint32_t *counts, void *state,
                 size_t state_bytes, void *work, size_t work_bytes, float *vertices,
                 int64_t *faces, float *L_dev, int64_t *surf_edges, dmgs_stream_t stream);
int dmgs_fc_bwd(const DmgsFcGrid *g, const uint32_t *counts, const void *state,
                size_t state_bytes, const void *work, size_t work_bytes,
                const float *vertices, float *dL_dvertices, const float *dL_dL_dev,
                float *dx, float *ds, float *dbeta, float *dalpha, float *dgamma,
                dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Hash-grid texture (replaces MLPTexture3D.sample_noact, geo/texture.py:
 * 101-112, whose encoding is tiny-cuda-nn's HashGrid): positions -> features
 *   t = clamp((xyz - lo) / (hi - lo), 0, 1); enc = 16-level x 2-feature
 *   hash encoding (base resolution 16, 2^19 entries per level, the given
 *   per-level scale); out = W3 relu(W2 relu(W1 enc)), no biases.
 * table: [entries, 2] f32 (dmgs_tex_table_entries); W1, W2: [32,32];
 * W3: [channels, 32] (torch Linear layout); channels in {3, 12, 27, 48}.
 * dmgs_tex_bwd writes (overwrites) dW1..dW3, the table gradient (optional)
 * scaled by 128 and the position gradient (optional) unscaled, as the
 * reference's two backward hooks (geo/texture.py:72-73) leave them.
 * ---------------------------------------------------------------------- */
typedef struct DmgsTexture {
  const float *table;    /* [entries, 2] */
  const float *W1, *W2, *W3;
  int32_t channels;
  float aabb[6];         /* lo x, y, z, hi x, y, z */
  float per_level_scale; /* exp(ln(4096 / 16) / 15) in the reference */
} DmgsTexture;

int64_t dmgs_tex_table_entries(float per_level_scale);
int dmgs_tex_fwd(const DmgsTexture *t, int64_t n, const float *xyz, float *out,
                 dmgs_stream_t stream);
size_t dmgs_tex_bwd_scratch_bytes(int64_t n);  /* 128 B per point, 16-byte aligned */
int dmgs_tex_bwd(const DmgsTexture *t, int64_t n, const float *xyz, const float *dout,
                 float *dxyz, float *dtable, float *dW1, float *dW2, float *dW3,
                 void *scratch, size_t scratch_bytes, dmgs_stream_t stream);
/* The same pair keeping the encoding: dmgs_tex_fwd_enc also writes each
 * point's 32 encoding values to enc ([n, 32] f32, 128 B per point, 16-byte
 * aligned), and dmgs_tex_bwd_enc reads them instead of recomputing the 128
 * table gathers per point (the reference's autograd likewise keeps the
 * MLP's input for its backward).  The values are those the forward used,
 * so the gradients equal dmgs_tex_bwd's. */
int dmgs_tex_fwd_enc(const DmgsTexture *t, int64_t n, const float *xyz, float *out, float *enc,
                     dmgs_stream_t stream);
int dmgs_tex_bwd_enc(const DmgsTexture *t, int64_t n, const float *xyz, const float *enc,
                     const float *dout, float *dxyz, float *dtable, float *dW1, float *dW2,
                     float *dW3, void *scratch, size_t scratch_bytes, dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * The renderer's Python colour path (gaussian_renderer/__init__.py:165-170:
 * eval_sh of utils/sh_utils.py:25-110 on the normalised direction from the
 * camera centre, then sigmoid) fused:
 *   colors[p][c] = sigmoid(sum_k b_k(dir_p) sh[p][c][k]),
 *   dir_p = (xyz[p] - campos) / |xyz[p] - campos|.
 * sh: [P,3,K] fp32 device (channel-major, K >= (deg+1)^2, deg 0..3); xyz
 * [P,3]; campos [3] device; colors [P,3].  The adjoint writes dL/dsh
 * [P,3,K] (zeros above the active degree) and, when dL_dxyz is not NULL,
 * dL/dxyz [P,3] through the normalisation.
 * ---------------------------------------------------------------------- */
int dmgs_sh_colors_fwd(int32_t P, int32_t deg, int32_t K, const float *sh, const float *xyz,
                       const float *campos, float *colors, dmgs_stream_t stream);
int dmgs_sh_colors_bwd(int32_t P, int32_t deg, int32_t K, const float *sh, const float *xyz,
                       const float *campos, const float *dL_dcolors, float *dL_dsh,
                       float *dL_dxyz, dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Fused photometric loss (no counterpart kernel in the reference, which
 * composes it from torch ops: l1_loss and ssim of utils/loss_utils.py as
 * used by train_geo_stage2.py:114-116):
 *   loss = (1 - lambda) mean|image - target| + lambda (1 - mean SSIM),
 * SSIM with an 11 x 11 Gaussian window (sigma 1.5), zero padding, C1 = 0.01^2,
 * C2 = 0.03^2, per channel.  image / target: [C,H,W] fp32 device arrays;
 * writes *loss (device scalar, may be NULL) and grad = dloss/dimage [C,H,W].
 * ---------------------------------------------------------------------- */
size_t dmgs_l1_ssim_scratch_bytes(int32_t C, int32_t H, int32_t W);
int dmgs_l1_ssim(const float *image, const float *target, int32_t C, int32_t H,
                 int32_t W, float lambda_dssim, float *loss, float *grad,
                 void *scratch, size_t scratch_bytes, dmgs_stream_t stream);

/* Frustum test (replaces `mark_visible`): present[i] = 1 iff point i lies in
 * front of view-space z = 0.2.  present: [P] uint8 device. */
int dmgs_mark_visible(int32_t P, const float *means3D, const float *viewmatrix,
                      const float *projmatrix, uint8_t *present,
                      dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Debug views of the forward state (tests): copy the integer binning
 * outputs to device arrays.  rect: [P,4] int32 (xmin,ymin,xmax,ymax) tile
 * rectangle (zeros when culled); tiles_touched [P] uint32; depth [P] f32;
 * keys [K] uint64 ((tile<<32)|depth_bits), values [K] uint32, ranges [T,2]
 * uint32.  Any output may be NULL.
 * ---------------------------------------------------------------------- */
int dmgs_debug_geometry(int32_t P, int32_t width, int32_t height,
                        const void *geom_state, size_t geom_bytes,
                        int32_t *rect, uint32_t *tiles_touched, float *depth,
                        float *xy, float *conic_opacity, float *rgb,
                        dmgs_stream_t stream);
int dmgs_debug_binning(int32_t P, int32_t width, int32_t height,
                       int64_t num_rendered, const void *geom_state,
                       size_t geom_bytes, const void *binning_state,
                       size_t binning_bytes, uint64_t *keys, uint32_t *values,
                       uint32_t *ranges, dmgs_stream_t stream);
int dmgs_debug_image(int32_t width, int32_t height, const void *image_state,
                     size_t image_bytes, float *final_T, uint32_t *n_contrib,
                     dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Mesh -> Gaussian face binding, stage-2 form
 * (scene/gaussian_geo_model_mlp_flex.py:258-335 renew_gaussian,
 *  :370-385 get_covariance_dyn; geo/mesh_utils.py:16-57).
 * Per face f with vertices v0,v1,v2: frame R = [x, y, n] (x = unit(v1-v0),
 * n = unit((v1-v0) x (v2-v0)), y = unit(n x x)); Gaussian g of the face sits
 * at bc[g] . (v0,v1,v2); the face covariance is (R L k)(R L k)^T packed to 6
 * floats with L = [[s, m01 s, 0], [0, m11 s, 0], [0, 0, z_scale]],
 * s = |v1-v0| rad_base, (m01, m11) the affine map of the equilateral
 * triangle onto the face (identity when adaptive_cov = 0), and
 * k = tanh(scale_factor) * max_scale, or k = 1 when scale_factor is NULL
 * (the real-scene variant, scene/gaussian_geo_model_mlp_flex_colmap.py:
 * 494-512, which has no learnable scale).  Gradients flow to the vertices
 * through the means and through R only (L is a constant, as in the reference).
 * ---------------------------------------------------------------------- */
typedef struct DmgsFaceBinding {
  int32_t F;             /* faces */
  int32_t V;             /* vertices */
  int32_t G;             /* Gaussians per face */
  int32_t bc_per_gaussian; /* 1: bc is [F*G,3]; 0: bc is a shared [G,3] table */
  int32_t adaptive_cov;  /* 1: affine covariance (reference default) */
  float rad_base;        /* generate_barycentric_v2 radius for G */
  float z_scale;         /* spatial_lr_scale * 1e-6 */
  float max_scale;       /* 2.0 in the reference */
  const float *verts;    /* [V,3] device */
  const int64_t *faces;  /* [F,3] device */
  const float *bc;       /* barycentric weights, device */
  const float *scale_factor; /* [1] device (pre-tanh), or NULL: k = 1 */
} DmgsFaceBinding;

/* Forward: xyz [F*G,3], cov [F*G,6] (device); rot_t2w [F,9] (row-major 3x3,
 * may be NULL) and cov3D_L [F,9] (may be NULL). */
int dmgs_bind_fwd(const DmgsFaceBinding *b, float *xyz, float *cov,
                  float *rot_t2w, float *cov3D_L, dmgs_stream_t stream);

/* Adjoint: from dL_dxyz [F*G,3] and dL_dcov [F*G,6] (either may be NULL)
 * accumulate dL_dverts [V,3] (zeroed here) and dL_dscale_factor [1]
 * (zeroed here, may be NULL). */
int dmgs_bind_bwd(const DmgsFaceBinding *b, const float *dL_dxyz,
                  const float *dL_dcov, float *dL_dverts,
                  float *dL_dscale_factor, dmgs_stream_t stream);

/* Stage-3 form (scene/gaussian_geo_model_finetune.py:396-421 renew_gaussian,
 * :446-483 get_scaling / get_rotation / get_rot_matrix): per Gaussian
 * xyz = bc . tri, scales = (exp(s0), exp(s1), thin_z), rotation = the unit
 * quaternion of R_t2w * [[a,-b,0],[b,a,0],[0,0,1]] with (a,b) = unit(rot2d).
 * The quaternion's sign is fixed so that its real part is >= 0. */
typedef struct DmgsFaceBinding3 {
  int32_t F, V, G;
  float thin_z;             /* thin_z_scale */
  const float *verts;       /* [V,3] */
  const int64_t *faces;     /* [F,3] */
  const float *bc;          /* [G,3] shared table */
  const float *scaling2d;   /* [F*G,2] pre-activation */
  const float *rotation2d;  /* [F*G,2] */
} DmgsFaceBinding3;

int dmgs_bind3_fwd(const DmgsFaceBinding3 *b, float *xyz, float *scales,
                   float *rotations, dmgs_stream_t stream);
/* Adjoint: dL_dverts [V,3], dL_dscaling2d [F*G,2], dL_drotation2d [F*G,2]
 * (all zeroed/written here; any may be NULL except dL_dverts). */
int dmgs_bind3_bwd(const DmgsFaceBinding3 *b, const float *dL_dxyz,
                   const float *dL_dscales, const float *dL_drotations,
                   float *dL_dverts, float *dL_dscaling2d,
                   float *dL_drotation2d, dmgs_stream_t stream);

/* ---------------------------------------------------------------------- *
 * Kernel timing (a profiling aid with no counterpart in the reference).
 * While enabled, every kernel this library launches is bracketed by CUDA
 * events on its own stream.  dmgs_timing_collect synchronises on the
 * recorded events, returns per-kernel totals (at most *n entries; *n is set
 * to the number written) and resets them.  Names stay valid until unload.
 * ---------------------------------------------------------------------- */
int dmgs_timing_enable(int32_t on);
/* Kernels this library has launched (enqueued) since it was loaded. */
int64_t dmgs_kernel_launches(void);
int dmgs_timing_collect(int32_t *n, const char **names, double *total_ms,
                        int64_t *launches);

/* Library information. */
const char *dmgs_last_error(void);
int32_t dmgs_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DMGS_H */
