// kernels.cuh — internal launch wrappers (one per kernel family).  Each
// returns DMGS_OK or a DMGS_ERR_* code; they enqueue work on `stream` only.
#pragma once
#include "common.cuh"

namespace dmgs {

struct GaussianPtrs {
  int P, M;
  const float *means3D, *opacities, *shs, *colors, *scales, *rotations, *cov3D;
};

// One view of a multi-view batch, as the per-Gaussian kernels see it.
struct BatchView {
  ViewParams vp;
  const float *viewm, *projm, *campos;  // device
  int32_t *radii;                       // [P] or a [P] scratch when the caller passes none
  float4 *feat;                         // geometry state of this view
  uint8_t *flags;
  uint32_t *blkcnt;
  uint32_t *counters;
  const float *gacc;                    // adjoint: this view's 2D gradient records
  float *dL_dmeans2D;                   // adjoint: optional per-view output [P,3]
};

struct BatchViews {
  int nviews;
  BatchView v[16];
};

// preprocess.cu
int launch_preprocess_batched(const BatchViews &bv, const GaussianPtrs &g, cudaStream_t s);
int launch_preprocess(const ViewParams &vp, const float *viewm, const float *projm,
                      const float *campos, const GaussianPtrs &g, int32_t *radii,
                      const GeomLayout &L, char *geom, cudaStream_t s);
int launch_mark_visible(int P, const float *means3D, const float *viewm, uint8_t *present,
                        cudaStream_t s);

// loss.cu
size_t l1_ssim_scratch_bytes(int C, int H, int W);
int launch_l1_ssim(const float *x, const float *y, int C, int H, int W, float lambda,
                   float *loss, float *grad, char *scratch, cudaStream_t s);

// binning.cu — every stage bins a set of views in one launch per stage.
constexpr int MAX_BIN_VIEWS = 16;

// One view's binning: its geometry-state arrays and sizes.
struct BinView {
  int P, nb_pre, nb_radix;
  int gx, gy;            // tile grid
  int R, nb;             // segment counting: tile rows per band, bands
  int nxs;               // row pieces of at most XSEG tiles
  uint32_t n_rhist_max, n_rcnt_max;
  const uint8_t *flags;
  const float4 *feat;
  uint32_t *blkcnt, *counters, *part, *k0, *k1, *v0, *v1, *rhist, *cstart, *rcnt, *cnt2;
  uint2 *srect;          // packed tile rectangle per depth-sorted position
  uint2 *ranges;
  uint32_t *point_list;  // emission target (K_alloc entries)
  uint2 *rowlist;        // row lists (K_alloc entries)
  uint32_t K_cap;        // list capacity checked by the ranges (0xffffffff: sized afterwards)
  uint32_t K_alloc;      // entries of point_list
  uint32_t rows_alloc;   // entries of rowlist
  uint32_t cmax;         // chunk bound
};

struct BinViews {
  int n;
  BinView v[MAX_BIN_VIEWS];
};

// One array per view for the generic scan.
struct ScanView {
  uint32_t *data;
  const uint32_t *n_dev;  // device length (nullptr: n_max)
  uint32_t n_max;
  uint32_t *part;
  uint32_t *total_out;
  uint32_t *status;
};

struct ScanViews {
  int n;
  ScanView v[MAX_BIN_VIEWS];
};

// Fill one view's binning record from its geometry state; point_list /
// K_alloc may be set later (after the instance count is known).
// bin: the binning state (point list, then row lists: bin_layout(K_alloc)),
// or nullptr until the instance count is known.
int make_bin_view(const GeomLayout &L, char *geom, uint32_t K_cap, char *bin, uint32_t K_alloc,
                  BinView &B);
int launch_binning_geometry(const BinViews &bv, cudaStream_t s);
// Exclusive scan of one u32 array of n entries in place (part: scan_part_words(n)
// words of scratch; total to *total_out, overflow bit into *status when given).
int launch_scan1(uint32_t *data, uint32_t n, uint32_t *part, uint32_t *total_out,
                 uint32_t *status, cudaStream_t s);
size_t scan_part_words(uint32_t n);
int launch_emit(const BinViews &bv, cudaStream_t s);
int launch_debug_keys(const GeomLayout &L, const char *geom, const BinLayout &B, const char *bin,
                      uint64_t *keys, uint32_t *values, cudaStream_t s);
int launch_debug_geometry(const GeomLayout &L, const char *geom, int32_t *rect,
                          uint32_t *tiles_touched, float *depth, float *xy, float *conic_opacity,
                          float *rgb, cudaStream_t s);

// blend.cu
constexpr int MAX_BATCH_VIEWS = 16;

// One view of a blend launch: its tile grid and the buffers of its tiles.
struct BlendView {
  int W, H, gx, T;     // image size, tile-grid width, tiles
  uint32_t P;          // Gaussians (records of feat): list entries >= P are skipped
  int tile_base;       // first work item of this view
  const uint2 *ranges;
  const uint32_t *point_list;
  const float4 *feat;
  const float *bg;
  float *out_color;     // forward outputs
  float *final_T;
  uint32_t *n_contrib;
  const float *dL_dout; // adjoint inputs/outputs
  float *gacc;
  double *gacc64;       // adjoint in FP64-sum mode: [P][12] double accumulators (else null)
};

struct BlendBatch {
  int nviews, total;    // views, work items (sum of tiles, or of CTA cells)
  int sx = 1, sy = 1;   // tiles per CTA along x and y (set by the launchers)
  BlendView v[MAX_BATCH_VIEWS];
};

// Tuning parameters of the blend kernels: pixels per thread (1, 2, 4),
// Gaussians staged per batch (128, 256, 512) and the CTA shape in 16x16
// tiles, sx x sy: 1x1, or 2x1 / 1x2 (32x16 / 16x32 pixels: two binning
// tiles per CTA; pixels per thread 2 or 4, batch 128 or 256).
struct BlendCfg {
  int ppt, batch;
  int sx = 1, sy = 1;
};
inline BlendCfg default_blend_cfg() { return BlendCfg{4, 128, 1, 1}; }  // autotuned on GB300

// queue == nullptr: one CTA per work item; else a persistent grid pulling
// items from *queue (which must be zero at launch).
int launch_blend_batch_fwd(const BlendBatch &bb, const BlendCfg &cfg, uint32_t *queue,
                           cudaStream_t s);
int launch_blend_batch_bwd(const BlendBatch &bb, const BlendCfg &cfg, uint32_t *queue,
                           cudaStream_t s);
int launch_blend_fwd(const ViewParams &vp, const GeomLayout &L, const char *geom,
                     const BinLayout &B, const char *bin, const ImgLayout &I, char *img,
                     const float *bg, float *out_color, cudaStream_t s);
// gacc64 != nullptr: the FP64-sum mode (gradient terms added into [P][12]
// doubles, then rounded into gacc for the preprocess adjoint).
int launch_blend_bwd(const ViewParams &vp, const GeomLayout &L, const char *geom,
                     const BinLayout &B, const char *bin, const ImgLayout &I, const char *img,
                     const float *bg, const float *dL_dout, float *gacc, double *gacc64,
                     cudaStream_t s);

// preprocess_bwd.cu
int launch_preprocess_bwd_batched(const BatchViews &bv, const GaussianPtrs &g, const DmgsGrads &out,
                                  float *densify_accum, float *densify_count, cudaStream_t s);
int launch_preprocess_bwd(const ViewParams &vp, const float *viewm, const float *projm,
                          const float *campos, const GaussianPtrs &g, const GeomLayout &L,
                          const char *geom, const float *gacc, const DmgsGrads &out,
                          cudaStream_t s);

// binding.cu
int launch_bind_fwd(const DmgsFaceBinding &b, float *xyz, float *cov, float *rot, float *covL,
                    cudaStream_t s);
int launch_bind_bwd(const DmgsFaceBinding &b, const float *dxyz, const float *dcov,
                    float *dverts, float *dsf, cudaStream_t s);
// Frustum face culling (binding.cu): scratch bytes and launcher.
size_t face_cull_scratch_bytes(int F);
int launch_face_cull(const float *verts, int V, const int64_t *faces, int F,
                     const float *full_proj, uint8_t *face_mask, int32_t *kept, int32_t *num_kept,
                     char *scratch, cudaStream_t s);
// Vertex frustum mask of the real-scene stage 2 (binding.cu).
int launch_vertex_frustum(const float *verts, int N, const float *full_proj, float cube_len,
                          int piece_id, int n_piece, const uint8_t *and_mask, uint8_t *out,
                          cudaStream_t s);
int launch_bind3_fwd(const DmgsFaceBinding3 &b, float *xyz, float *scales, float *rots,
                     cudaStream_t s);
int launch_bind3_bwd(const DmgsFaceBinding3 &b, const float *dxyz, const float *dscales,
                     const float *drots, float *dverts, float *dscaling, float *drot2d,
                     cudaStream_t s);

}  // namespace dmgs
