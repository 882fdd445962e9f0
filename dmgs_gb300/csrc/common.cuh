// common.cuh — shared device helpers, state layout and launch checking for
// the sm_103a rasteriser.  Everything here is internal to libdmgs_gb300.so;
// the public surface is include/dmgs.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/dmgs.h"

namespace dmgs {

constexpr int TILE = DMGS_TILE;               // 16 x 16 pixel tiles
constexpr int TILE_PIX = TILE * TILE;         // 256 pixels, one thread each
constexpr int NUM_SMS_HINT = 152;             // GB300: 2 dies x 76 SMs

// Status word bits written by kernels (never a trap or assert).
constexpr uint32_t ST_PREFILTER = 1u;   // prefiltered point failed the z test
constexpr uint32_t ST_OVERFLOW = 2u;    // instance slots exhausted
constexpr uint32_t ST_BOUNDS = 4u;      // an index left its buffer

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// IEEE single-precision ops with explicit rounding: the integer-determining
// part of preprocess must not be contracted into FMAs so that the CPU oracle
// (numpy float32) reproduces radii, rectangles and depth keys bit for bit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }

// Per-view constants after host-side preparation.
struct ViewParams {
  int W, H;
  int gx, gy;            // tile grid
  float fx, fy;          // focal lengths (host float32, see focal())
  float tanfovx, tanfovy;
  float scale_modifier;
  int D;                 // active SH degree
  int prefiltered;
};

// ---------------------------------------------------------------------------
// Geometry state.  Per Gaussian, a 48-byte record = 3 x float4:
//   f0 = (x, y, conic_a, conic_b)    pixel-space mean, conic (a b; b c)
//   f1 = (conic_c, opacity, r, g)
//   f2 = (b, depth, rect_lo, rect_hi) rect packed as 2 x (u16 | u16 << 16)
// A culled Gaussian has rect_lo == rect_hi == 0 and radius 0.
// Per Gaussian also one flags byte: FLAG_VISIBLE | SH clamp bits (r, g, b).
// Then the binning working set: per-block visible counts, the visible
// Gaussians' depth keys / indices (two ping-pong copies for the radix sort),
// the radix block histograms, the per-(tile, chunk) count matrix, scan
// partials, per-tile ranges and the counters word block.
// ---------------------------------------------------------------------------
constexpr uint8_t FLAG_VISIBLE = 8;      // flags byte: radius > 0, tile rectangle non-empty
constexpr int PRE_BLOCK = 256;           // preprocess / compaction block
constexpr int RADIX_BLOCK = 256;         // radix sort block (8 warps)
constexpr int RADIX_ITEMS = 8;           // keys per thread
constexpr int RADIX_TILE = RADIX_BLOCK * RADIX_ITEMS;  // 2048 keys per block
constexpr int CHUNK_MIN_GAUSS = 64;     // visible Gaussians per binning chunk (mean, minimum)
constexpr int CHUNK_COUNT_MAX = 2048;    // binning chunks per view (maximum)
constexpr int CHUNK_W_GAUSS = 2;         // chunk weight of a Gaussian: this + ceil(rows / 16)
constexpr int SEG_MAX = 32;              // row segments (groups of chunks) per view, maximum
constexpr int XSEG = 512;                // tiles of one row handled by a tile-emission block
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096 elements per block

// counters[] indices
constexpr int CI_STATUS = 0;   // ST_* bits
constexpr int CI_K = 1;        // instances (u32; K < 2^32 enforced)
constexpr int CI_K1 = 2;       // row-list entries (visible Gaussian x tile row it covers)
constexpr int CI_MAXLIST = 3;  // longest tile list
constexpr int CI_V = 4;        // visible Gaussians
constexpr int CI_NBR = 5;      // radix blocks in use = ceil(V / RADIX_TILE)
constexpr int CI_NRH = 6;      // radix histogram entries = 256 * NBR
constexpr int CI_W = 7;        // total chunk weight of the visible Gaussians
constexpr int CI_C = 8;        // chunks
constexpr int CI_NRC = 9;      // row-count entries = gy * C
constexpr int CI_WORDS = 16;

// Geometry state of one view.  Binning arrays: per-block visible counts;
// (depth bits, index) ping-pong pairs of the radix sort; radix histograms;
// per depth-sorted position the packed tile rectangle (srect, 8 B); chunk
// starts; the row counts [gy][C] (Gaussians of chunk c covering tile row r,
// scanned in place into row-list offsets); the segment counts [T][S]
// (instances of tile t from row segment s, scanned in place into list
// offsets); scan partials; tile ranges; counters.
struct GeomLayout {
  size_t feat, flags, blkcnt, dkey0, dkey1, dval0, dval1, rhist, srect, cstart, rcnt, cnt2,
      scanpart, ranges, counters, total;
  int P, gx, gy;
  int nb_pre, nb_radix;
  size_t n_rhist_max, n_rcnt_max, n_cnt2_max, n_part_max;
  __host__ __device__ int T() const { return gx * gy; }
};

__host__ __device__ inline GeomLayout geom_layout(int P, int W, int H) {
  GeomLayout L;
  L.P = P;
  L.gx = (W + TILE - 1) / TILE;
  L.gy = (H + TILE - 1) / TILE;
  const size_t T = (size_t)L.gx * L.gy;
  L.nb_pre = (P + PRE_BLOCK - 1) / PRE_BLOCK;
  L.nb_radix = (P + RADIX_TILE - 1) / RADIX_TILE;
  L.n_rhist_max = (size_t)256 * L.nb_radix;
  L.n_rcnt_max = (size_t)L.gy * CHUNK_COUNT_MAX;
  L.n_cnt2_max = T * SEG_MAX;
  size_t nmax = L.n_rcnt_max > L.n_rhist_max ? L.n_rcnt_max : L.n_rhist_max;
  if (L.n_cnt2_max > nmax) nmax = L.n_cnt2_max;
  if ((size_t)L.nb_pre > nmax) nmax = L.nb_pre;
  if ((size_t)P > nmax) nmax = P;
  L.n_part_max = (nmax + SCAN_TILE - 1) / SCAN_TILE + 1;
  size_t o = 0;
  L.feat = o;      o = align_up(o + (size_t)P * 48, 256);
  L.flags = o;     o = align_up(o + (size_t)P, 256);
  L.blkcnt = o;    o = align_up(o + (size_t)L.nb_pre * 4 + 4, 256);
  L.dkey0 = o;     o = align_up(o + (size_t)P * 4, 256);
  L.dkey1 = o;     o = align_up(o + (size_t)P * 4, 256);
  L.dval0 = o;     o = align_up(o + (size_t)P * 4, 256);
  L.dval1 = o;     o = align_up(o + (size_t)P * 4, 256);
  L.rhist = o;     o = align_up(o + L.n_rhist_max * 4 + 4, 256);
  L.srect = o;     o = align_up(o + (size_t)P * 8, 256);
  L.cstart = o;    o = align_up(o + (CHUNK_COUNT_MAX + 1) * 4, 256);
  L.rcnt = o;      o = align_up(o + L.n_rcnt_max * 4 + 4, 256);
  L.cnt2 = o;      o = align_up(o + L.n_cnt2_max * 4 + 4, 256);
  L.scanpart = o;  o = align_up(o + L.n_part_max * 4, 256);
  L.ranges = o;    o = align_up(o + T * 8, 256);
  L.counters = o;  o = align_up(o + CI_WORDS * 4, 256);
  L.total = o;
  return L;
}

// Binning state: the per-tile Gaussian index lists, concatenated in tile
// order (K entries, 4 B each), then the row lists they are split from (one
// 8-byte entry {Gaussian index, x0 | x1 << 16} per visible Gaussian and tile
// row it covers).  Row entries are at most K (every entry yields at least
// one instance) and at most P x (tile rows); P < 0: bound by K alone.
struct BinLayout {
  size_t point_list, rowlist, rows, total;
};

__host__ __device__ inline size_t row_entries_max(int64_t K, int H, int64_t P) {
  const size_t k = (size_t)(K > 0 ? K : 0);
  if (P < 0) return k;
  const size_t pr = (size_t)P * (size_t)((H + TILE - 1) / TILE);
  return pr < k ? pr : k;
}

__host__ __device__ inline BinLayout bin_layout(int64_t K, int W, int H, int64_t P = -1) {
  (void)W;
  BinLayout L;
  const size_t k = (size_t)(K > 0 ? K : 0);
  L.point_list = 0;
  L.rowlist = align_up(k * 4, 256);
  L.rows = row_entries_max(K, H, P);
  L.total = L.rowlist + align_up(L.rows * 8, 256) + 256;
  return L;
}

struct ImgLayout {
  size_t final_T, n_contrib, total;
};

__host__ __device__ inline ImgLayout img_layout(int W, int H) {
  ImgLayout L;
  size_t n = (size_t)W * H;
  size_t o = 0;
  L.final_T = o;   o = align_up(o + n * 4, 256);
  L.n_contrib = o; o = align_up(o + n * 4, 256);
  L.total = o;
  return L;
}

// Backward scratch: per-Gaussian 2D gradient accumulators, 48 B record:
//   g0 = (dL/dndc_x, dL/dndc_y, dL/dconic_a, dL/dconic_b)
//   g1 = (dL/dconic_c, dL/dopacity, dL/dr, dL/dg)
//   g2 = (dL/db, 0, 0, 0)
inline size_t bwd_scratch_bytes(int P) { return align_up((size_t)P * 48, 256); }

__device__ __forceinline__ uint32_t pack_u16x2(int lo, int hi) {
  return (uint32_t)lo | ((uint32_t)hi << 16);
}

__device__ __forceinline__ void red_add_v4(float *addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};"
               :: "l"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// SH constants of the real spherical-harmonics basis up to degree 3
// (the same polynomial as utils/sh_utils.py:41-99).
__constant__ static const float kSH_C0 = 0.28209479177387814f;
__constant__ static const float kSH_C1 = 0.4886025119029199f;
__constant__ static const float kSH_C2[5] = {1.0925484305920792f, -1.0925484305920792f,
                                             0.31539156525252005f, -1.0925484305920792f,
                                             0.5462742152960396f};
__constant__ static const float kSH_C3[7] = {-0.5900435899266435f, 2.890611442640554f,
                                             -0.4570457994644658f, 0.3731763325901154f,
                                             -0.4570457994644658f, 1.445305721320277f,
                                             -0.5900435899266435f};

}  // namespace dmgs

// Host-side error plumbing shared by the C-ABI translation units.
namespace dmgs_host {
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

// Kernel timing registry (timing.cu).  Kernel ids index kKernelNames.
enum KernelId {
  K_PREPROCESS = 0, K_BIN_COMPACT, K_BIN_SORT, K_BIN_COUNT, K_BIN_SCAN, K_BIN_EMIT, K_BLEND_FWD,
  K_BLEND_BWD, K_PREPROCESS_BWD, K_MARK_VISIBLE, K_BIND_FWD, K_BIND_BWD, K_BIND3_FWD,
  K_BIND3_BWD, K_DEBUG, K_BATCH_PREPROCESS, K_BATCH_BINNING, K_BATCH_BLEND_FWD,
  K_BATCH_BLEND_BWD, K_BATCH_PREPROCESS_BWD, K_LOSS, K_FACE_CULL, K_FC_FWD, K_FC_BWD, K_TEX_FWD, K_TEX_BWD, K_SH_COLORS, K_BIN_ROWS, K_TEX_SCATTER, K_COUNT
};
void timing_begin(int kid, cudaStream_t s);
void timing_end(int kid, cudaStream_t s);
void note_launch();  // counts every kernel launch (dmgs_kernel_launches)
// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes` (never lowers it: the attribute is per device and shared by
// every host thread, so concurrent callers with different sizes cannot undo
// each other).  One lock for every kernel of the library.
int raise_smem_limit(const void *func, size_t bytes);
}  // namespace dmgs_host

// Bracket one kernel launch with the timing registry (no-op when disabled).
#define DMGS_TIMED(kid, stream, ...)               \
  do {                                             \
    dmgs_host::timing_begin(dmgs_host::kid, stream); \
    __VA_ARGS__;                                   \
    dmgs_host::timing_end(dmgs_host::kid, stream);   \
  } while (0)

#define DMGS_CUDA(call)                                                  \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) return dmgs_host::cuda_fail(e_, #call);       \
  } while (0)

#define DMGS_LAUNCH_CHECK(name)                                          \
  do {                                                                   \
    cudaError_t e_ = cudaGetLastError();                                 \
    if (e_ != cudaSuccess) return dmgs_host::cuda_fail(e_, name);        \
  } while (0)
