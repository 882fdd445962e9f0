// blend.cu — per-tile front-to-back alpha blending (forward) and its adjoint.
//
// Semantics (3DGS tile renderer, reached from gaussian_renderer/__init__.py:86-94):
//   power = -1/2 (a dx^2 + c dy^2) - b dx dy, d = mean2D - pixel
//   skip if power > 0; alpha = min(0.99, o e^power); skip if alpha < 1/255
//   stop before the Gaussian that would bring T below 1e-4
//   C += alpha T rgb; T *= 1 - alpha; out = C + T bg
// final_T and n_contrib (1-based list position of the last blended Gaussian)
// are kept for the adjoint, which walks the list back to front, recomputes
// T by division and accumulates per-Gaussian gradients.
//
// Design (both kernels are instruction-issue bound: the visible Gaussians'
// records and the tile lists are L2-resident):
// * a CTA blends one 16x16 tile at a time with 256/PPT threads; warp w owns
//   the 2 PPT consecutive rows from 2 PPT w, lane l the PPT pixels of column
//   l%16 in rows band + l/16 + 2k, which share dx and every shared-memory
//   load (PPT = 1, 2 or 4, a tuning parameter);
// * CTA shape (a tuning parameter): 16x16 (one binning tile), or 32x16 /
//   16x32 pixels — a union of two adjacent 16x16 binning tiles, each half of
//   the CTA blending one of them from its own list (so every pixel still sees
//   exactly its tile's Gaussians in the same order); the halves synchronise
//   on their own named barriers and meet only between work items, and the
//   pair's records, mostly the same Gaussians, share the SM's L1;
// * work items are the (view, tile) pairs of one or several views (the
//   multi-view batched form renders many views in one launch); CTAs either
//   take one item each or, persistent, pull items from an atomic counter;
// * Gaussians are staged in shared memory in batches of BATCH (128, 256 or
//   512, a tuning parameter); in the forward the next batch's global loads
//   are in flight while the current batch is blended (double buffer);
// * at staging, the conic is scaled by -log2(e)/2 (so the falloff is one
//   ex2 instruction) and a per-Gaussian exponent threshold
//   log2(1/(255 o)) is precomputed: a pair below it cannot reach alpha 1/255
//   and is rejected before the exponential (the alpha test itself is still
//   applied afterwards);
// * each staged Gaussian carries a mask of the warps' row bands its
//   alpha >= 1/255 ellipse can reach (a superset, from the exponent's
//   maximum over each band's rectangle): a warp whose band it misses never
//   visits it (per-warp visit lists, one ballot per 32 staged Gaussians) —
//   only pairs the exact test would reject are skipped;
// * the forward and the adjoint evaluate the exponent with the same
//   explicitly rounded operations, so their skip/stop decisions agree;
// * the adjoint sums a Gaussian's nine gradient terms over the thread's
//   pixels, then over the warp with a transposed reduce-scatter (12
//   shuffles); nine lanes then issue one scalar reduction each.
#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr float ALPHA_MIN = 1.0f / 255.0f;
constexpr float ALPHA_MAX = 0.99f;
constexpr float T_EPS = 0.0001f;
constexpr float LOG2E = 1.4426950408889634f;
constexpr float LOG2_255 = 7.994353436858858f;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Staged Gaussian (forward): s0 = (x, y, A, B), s1 = (C, o, thr, r),
// s2 = (g, b, footprint rows, 0) with exponent2 = A dx^2 + B dx dy + C dy^2
// (A = -a log2e / 2, B = -b log2e, C = -c log2e / 2) and thr = log2(1 / (255 o)).
// The footprint rows (bits 0-15) cover the tile rows where alpha can reach
// 1/255 (a superset of the rows the exact test accepts): with warp bands
// of 4 or more rows, whole bands (band_rows); with bands of 2 rows, the
// ellipse (a dx^2 + 2 b dx dy + c dy^2) <= 2 ln(255 o)'s vertical extent,
// sqrt(R^2 a / det) inflated by 0.1% + 0.01 px (footprint), refined per row
// (exact_rows).
struct Staged {
  float4 s0, s1, s2;
};

__device__ __forceinline__ uint32_t span_mask(float centre, float ext) {
  const float lo = fmaxf(ceilf(centre - ext), 0.f);
  const float hi = fminf(floorf(centre + ext), 15.f);
  if (!(lo <= hi)) return 0u;
  const int l = (int)lo, h = (int)hi;
  return (0xffffu >> (15 - h)) & (0xffffu << l);
}

__device__ __forceinline__ uint32_t footprint(float a, float b, float c, float o, float cx, float cy) {
  if (!(o >= ALPHA_MIN)) return 0u;                  // alpha <= o < 1/255 everywhere
  const float det = a * c - b * b;
  if (!(det > 0.f) || !(a > 0.f) || !(c > 0.f)) return 0xffffu;  // not an ellipse
  const float R2 = 2.f * (__logf(o) + 5.541263545158426f);  // 2 ln(255 o)
  if (!(R2 >= 0.f)) return 0u;
  const float ey = sqrtf(R2 * a / det) * 1.001f + 0.01f;
  return span_mask(cy, ey);
}

// Row mask refined per row: for pixel row r (dy = cy - r fixed) the exponent
// A dx^2 + B dx dy + C dy^2 (A < 0) is largest at dx = -B dy / (2A), clamped
// to the tile's columns (dx in [cx - 15, cx], widened by 0.01); the row is kept
// when that maximum reaches thr less a margin of 0.01 + 1e-5 x a bound on the
// terms' magnitudes over the tile (|A| X^2 + |B| X Y + |C| Y^2 with X, Y the
// largest |dx|, |dy|), far above the rounding of either evaluation.  Rows the
// bounding-box mask keeps but no pixel of which reaches alpha 1/255 — the
// ellipse passing the tile's corner — are dropped, so warps skip them.
__device__ __forceinline__ uint32_t exact_rows(uint32_t m, float A, float B, float C, float thr,
                                               float cx, float cy) {
  if (!(A < 0.f) || m == 0u) return m;
  const float k = -B / (2.f * A);
  const float lo = cx - 15.01f, hi = cx + 0.01f;
  const float X = fmaxf(fabsf(lo), fabsf(hi)), Y = fmaxf(fabsf(cy), fabsf(cy - 15.f));
  const float mag = fabsf(A) * X * X + fabsf(B) * X * Y + fabsf(C) * Y * Y;
  const float lim = thr - (0.01f + 1e-5f * mag);
  uint32_t rows = 0u;
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const float dy = cy - (float)r;
    const float dxs = fminf(fmaxf(k * dy, lo), hi);
    const float e = fmaf(fmaf(C, dy, B * dxs), dy, A * dxs * dxs);
    if (e >= lim) rows |= 1u << r;
  }
  return m & rows;
}

// Row mask at the granularity of the warps' bands of RB consecutive tile
// rows (RB >= 4): a band's RB bits are set when the exponent can reach thr
// somewhere in the rectangle dx in [cx - 15, cx], dy in [cy - r1, cy - r0]
// (rows r0..r1 of the band, both ranges widened by 0.01): a continuous
// superset of the band's pixels.  The exponent is concave (A < 0, the conic
// positive definite), so its maximum over the rectangle is 0 when the
// centre lies inside, else the largest of the four edges' maxima, each the
// 1D maximum clamped to its edge (dx = kx dy on a horizontal edge, dy = ky dx
// on a vertical one).  The margin is that of exact_rows.  Half the cost of
// the per-row refinement at RB = 8, and the masks only select which warps
// visit a staged Gaussian.
template <int RB>
__device__ __forceinline__ uint32_t band_rows(float a, float b, float c, float o, float A, float B,
                                              float C, float thr, float cx, float cy) {
  if (!(o >= ALPHA_MIN)) return 0u;  // alpha <= o < 1/255 everywhere
  if (!(a * c - b * b > 0.f) || !(a > 0.f) || !(c > 0.f) || !(A < 0.f) || !(C < 0.f))
    return 0xffffu;  // not an ellipse: every band
  const float lo = cx - 15.01f, hi = cx + 0.01f;
  const float X = fmaxf(fabsf(lo), fabsf(hi)), Y = fmaxf(fabsf(cy), fabsf(cy - 15.f));
  const float mag = fabsf(A) * X * X + fabsf(B) * X * Y + fabsf(C) * Y * Y;
  const float lim = thr - (0.01f + 1e-5f * mag);
  const float kx = -B / (2.f * A), ky = -B / (2.f * C);
  const float yl = ky * lo, yh = ky * hi;  // unclamped optimum dy on the two vertical edges
  const bool x_in = lo <= 0.f && hi >= 0.f;
  auto ev = [&](float dx, float dy) { return fmaf(fmaf(C, dy, B * dx), dy, A * dx * dx); };
  uint32_t rows = 0u;
#pragma unroll
  for (int r0 = 0; r0 < 16; r0 += RB) {
    const float ylo = cy - (float)(r0 + RB - 1) - 0.01f, yhi = cy - (float)r0 + 0.01f;
    float e = fmaxf(ev(fminf(fmaxf(kx * ylo, lo), hi), ylo), ev(fminf(fmaxf(kx * yhi, lo), hi), yhi));
    e = fmaxf(e, ev(lo, fminf(fmaxf(yl, ylo), yhi)));
    e = fmaxf(e, ev(hi, fminf(fmaxf(yh, ylo), yhi)));
    const bool keep = e >= lim || (x_in && ylo <= 0.f && yhi >= 0.f);
    if (keep) rows |= ((1u << RB) - 1u) << r0;
  }
  return rows;
}

// (ox, oy): pixel origin of the tile being blended; RB: rows per warp band
// (the mask's granularity: per row below 4).
template <int RB>
__device__ __forceinline__ Staged stage(const float4 f0, const float4 f1, const float4 f2,
                                        float ox, float oy) {
  Staged S;
  const float A = __fmul_rn(-0.5f * LOG2E, f0.z);
  const float B = __fmul_rn(-LOG2E, f0.w);
  const float C = __fmul_rn(-0.5f * LOG2E, f1.x);
  const float thr = -LOG2_255 - __log2f(f1.y);
  const float cx = f0.x - ox, cy = f0.y - oy;
  const uint32_t m =
      RB >= 4 ? band_rows<RB>(f0.z, f0.w, f1.x, f1.y, A, B, C, thr, cx, cy)
              : exact_rows(footprint(f0.z, f0.w, f1.x, f1.y, cx, cy), A, B, C, thr, cx, cy);
  S.s0 = make_float4(f0.x, f0.y, A, B);
  S.s1 = make_float4(C, f1.y, thr, f1.z);
  S.s2 = make_float4(f1.w, f2.x, __uint_as_float(m), 0.f);
  return S;
}

// Exponent (base 2) of the Gaussian at (dx, dy).  Explicit intrinsics: the
// adjoint evaluates the identical sequence.
__device__ __forceinline__ float exponent2(float A, float B, float C, float dx, float dy) {
  const float ax2 = __fmul_rn(__fmul_rn(A, dx), dx);
  const float q = __fmul_rn(B, dx);
  return __fmaf_rn(__fmaf_rn(C, dy, q), dy, ax2);
}

// The 48-byte record of list entry id; an entry outside the Gaussians (which
// a correct list never holds) reads as a zero-opacity record, whose
// footprint is empty, so no read leaves the geometry state.
__device__ __forceinline__ void load_record(const BlendView &V, uint32_t id, float4 &f0, float4 &f1,
                                            float4 &f2) {
  if (id < V.P) {
    f0 = V.feat[3 * id]; f1 = V.feat[3 * id + 1]; f2 = V.feat[3 * id + 2];
  } else {
    f0 = f1 = f2 = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Work item -> (view, tile).
__device__ __forceinline__ int find_view(const BlendBatch &bb, int item) {
  int v = 0;
  while (v + 1 < bb.nviews && item >= bb.v[v + 1].tile_base) ++v;
  return v;
}

// Tile of half h of a CTA covering NT tiles for the view-local work item q:
// NT = 1, one tile per item; NT = 2, the item is a cell of the grid of
// (sx x sy)-tile cells, sx * sy = 2.  Returns false when that tile lies
// outside the grid (an odd tile count along the pair's axis).
template <int NT>
__device__ __forceinline__ bool item_tile(const BlendBatch &bb, const BlendView &V, int q, int h,
                                          int &tx, int &ty) {
  if constexpr (NT == 1) {
    tx = q % V.gx;
    ty = q / V.gx;
    return true;
  } else {
    const int gxs = (V.gx + bb.sx - 1) / bb.sx;
    const int qx = q % gxs, qy = q / gxs;
    tx = qx * bb.sx + (bb.sx == 2 ? h : 0);
    ty = qy * bb.sy + (bb.sy == 2 ? h : 0);
    return tx < V.gx && ty < V.T / V.gx;
  }
}

// Barrier of the ht threads of half h (NT = 2: named barrier 1 + h; barrier
// 0 stays the whole CTA's), and its popc-reduction form.
template <int NT>
__device__ __forceinline__ void half_sync(int h, int ht) {
  if constexpr (NT == 1) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + h), "r"(ht) : "memory");
  }
}

template <int NT>
__device__ __forceinline__ int half_count(int h, int ht, bool p) {
  if constexpr (NT == 1) {
    return __syncthreads_count(p);
  } else {
    int r;
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.popc.u32 %0, %2, %3, q;\n\t}"
                 : "=r"(r)
                 : "r"((int)p), "r"(1 + h), "r"(ht)
                 : "memory");
    return r;
  }
}

// Next work item of this CTA (all threads receive the same value).
__device__ __forceinline__ int next_item(uint32_t *queue, int &slot, int *s_item) {
  if (queue == nullptr) return slot++ == 0 ? (int)blockIdx.x : INT_MAX;
  __syncthreads();
  if (threadIdx.x == 0) *s_item = (int)atomicAdd(queue, 1u);
  __syncthreads();
  return *s_item;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// The staged Gaussians (of cnt) whose footprint rows meet this warp's rows,
// in staging order, written to this warp's list; returns their number.  One
// ballot per 32 staged Gaussians replaces a per-Gaussian test in the loop.
__device__ __forceinline__ int visit_list(const uint32_t *masks, int cnt, uint32_t warp_rows,
                                          uint16_t *list, int lane) {
  int nv = 0;
  for (int j0 = 0; j0 < cnt; j0 += 32) {
    const int j = j0 + lane;
    const bool hit = j < cnt && (masks[j] & warp_rows);
    const unsigned bal = __ballot_sync(FULL, hit);
    if (hit) list[nv + __popc(bal & lanemask_lt())] = (uint16_t)j;
    nv += __popc(bal);
  }
  __syncwarp();
  return nv;
}

// Warp w owns the band of 2 PPT consecutive tile rows starting at 2 PPT w;
// lane l the column l % 16 and the rows band + l / 16 + 2k (k < PPT).  A
// Gaussian whose footprint misses a band is never visited by its warp.
template <int PPT>
struct PixelLayout {
  int col, r0;
  uint32_t warp_rows;
  __device__ __forceinline__ explicit PixelLayout(int tid) {  // tid: thread index in the tile's half
    const int w = tid >> 5;
    col = tid & 15;
    r0 = 2 * PPT * w + ((tid >> 4) & 1);
    warp_rows = ((1u << (2 * PPT)) - 1u) << (2 * PPT * w);
  }
  __device__ __forceinline__ int row(int k) const { return r0 + 2 * k; }
};

// NT: tiles per CTA (1, or 2 for the 32x16 / 16x32 shapes); THREADS per tile.
template <int PPT, int BATCH, int NT = 1>
__global__ void __launch_bounds__(NT * 256 / PPT)
blend_fwd_kernel(const BlendBatch bb, uint32_t *queue) {
  constexpr int THREADS = 256 / PPT;
  constexpr int LOADS = (BATCH + THREADS - 1) / THREADS;
  __shared__ float4 S0[NT][2][BATCH];
  __shared__ float4 S1[NT][2][BATCH];
  __shared__ float4 S2[NT][2][BATCH];
  __shared__ uint32_t SM[NT][2][BATCH];               // footprint rows
  __shared__ uint16_t VL[NT * THREADS / 32][BATCH];   // per-warp visit lists
  __shared__ int s_item;
  const int h = NT == 1 ? 0 : (int)threadIdx.x / THREADS;  // the CTA half (tile) of this thread
  const int tid = (int)threadIdx.x - h * THREADS;
  const int lane = tid & 31;
  const PixelLayout<PPT> lay(tid);
  int slot = 0;
  for (int item = next_item(queue, slot, &s_item); item < bb.total;
       item = next_item(queue, slot, &s_item)) {
    const BlendView &V = bb.v[find_view(bb, item)];
    int tx, ty;
    const bool tv = item_tile<NT>(bb, V, item - V.tile_base, h, tx, ty);
    const int tile = ty * V.gx + tx;
    const int px = tx * TILE + lay.col;
    const float pxf = (float)px;
    const float ox = (float)(tx * TILE), oy = (float)(ty * TILE);
    const uint2 range = tv ? V.ranges[tile] : make_uint2(0u, 0u);
    const int n = (int)(range.y - range.x);
    bool done[PPT], inside[PPT];
    float T[PPT], cr[PPT], cg[PPT], cb[PPT], pyf[PPT];
    uint32_t last[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      const int py = ty * TILE + lay.row(k);
      inside[k] = tv && px < V.W && py < V.H;
      done[k] = !inside[k];
      pyf[k] = (float)py;
      T[k] = 1.f; cr[k] = cg[k] = cb[k] = 0.f; last[k] = 0;
    }
    auto all_done = [&]() {
      bool d = true;
#pragma unroll
      for (int k = 0; k < PPT; ++k) d = d && done[k];
      return d;
    };
    float4 pf0[LOADS], pf1[LOADS], pf2[LOADS];
#pragma unroll
    for (int l = 0; l < LOADS; ++l) {
      const int i = l * THREADS + tid;
      if (i < n && i < BATCH) {
        load_record(V, V.point_list[range.x + i], pf0[l], pf1[l], pf2[l]);
      }
    }
    int buf = 0;
    for (int base = 0; base < n; base += BATCH) {
#pragma unroll
      for (int l = 0; l < LOADS; ++l) {
        const int sl = l * THREADS + tid;
        if (sl < BATCH && base + sl < n) {
          const Staged st = stage<2 * PPT>(pf0[l], pf1[l], pf2[l], ox, oy);
          S0[h][buf][sl] = st.s0; S1[h][buf][sl] = st.s1; S2[h][buf][sl] = st.s2;
          SM[h][buf][sl] = __float_as_uint(st.s2.z);
        }
      }
      if (half_count<NT>(h, THREADS, all_done()) == THREADS) break;
      const int nbase = base + BATCH;
#pragma unroll
      for (int l = 0; l < LOADS; ++l) {
        const int sl = l * THREADS + tid;
        if (sl < BATCH && nbase + sl < n) {
          load_record(V, V.point_list[range.x + nbase + sl], pf0[l], pf1[l], pf2[l]);
        }
      }
      const int cnt = min(BATCH, n - base);
      bool warp_done = __all_sync(FULL, all_done());
      uint16_t *vl = VL[threadIdx.x >> 5];
      const int nvis = warp_done ? 0 : visit_list(SM[h][buf], cnt, lay.warp_rows, vl, lane);
      for (int i = 0; i < nvis && !warp_done; ++i) {
        const int j = vl[i];
        const float4 s0 = S0[h][buf][j];
        const float4 s1 = S1[h][buf][j];
        const float4 s2 = S2[h][buf][j];
        const float dx = __fsub_rn(s0.x, pxf);
        // pass 1: exponent and range test of every pixel (no branches); the
        // footprint rows, a superset of what this test accepts, only
        // select the warps that visit
        float e2[PPT];
        bool ok[PPT];
        bool any = false;
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          e2[k] = exponent2(s0.z, s0.w, s1.x, dx, __fsub_rn(s0.y, pyf[k]));
          ok[k] = !done[k] && !(e2[k] > 0.f) && !(e2[k] < s1.z);
          any |= ok[k];
        }
        if (!__any_sync(FULL, any)) continue;  // warp-uniform
        // pass 2: alpha, stop test and accumulation, predicated
        const uint32_t pos = (uint32_t)(base + j + 1);
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          const float alpha = fminf(ALPHA_MAX, __fmul_rn(s1.y, ex2_approx(e2[k])));
          const bool take = ok[k] && !(alpha < ALPHA_MIN);
          const float test_T = T[k] * (1.f - alpha);
          const bool stop = take && test_T < T_EPS;
          const bool blend = take && !stop;
          const float w = blend ? alpha * T[k] : 0.f;
          cr[k] = fmaf(s1.w, w, cr[k]); cg[k] = fmaf(s2.x, w, cg[k]); cb[k] = fmaf(s2.y, w, cb[k]);
          T[k] = blend ? test_T : T[k];
          last[k] = blend ? pos : last[k];
          done[k] = done[k] || stop;
        }
        warp_done = __all_sync(FULL, all_done());
      }
      buf ^= 1;
    }
    const size_t HW = (size_t)V.H * V.W;
    const float bgr = __ldg(V.bg), bgg = __ldg(V.bg + 1), bgb = __ldg(V.bg + 2);
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      if (!inside[k]) continue;
      const int pix = (int)pyf[k] * V.W + px;
      V.final_T[pix] = T[k];
      V.n_contrib[pix] = last[k];
      V.out_color[pix] = cr[k] + T[k] * bgr;
      V.out_color[HW + pix] = cg[k] + T[k] * bgg;
      V.out_color[2 * HW + pix] = cb[k] + T[k] * bgb;
    }
    __syncthreads();  // shared buffers are reused by the next item
  }
}

// ------------------------------- adjoint -----------------------------------

// Staged Gaussian (adjoint): s0 = (x, y, A, B), s1 = (C, o, thr, r),
// s2 = (g, b, ka, kb), s3 = (kc, kd, id bits, footprint rows) with ka = -a W/2,
// kb = -b W/2, kc = -c H/2, kd = -b H/2 (the NDC-mean gradient factors).
struct StagedB {
  float4 s0, s1, s2, s3;
};

template <int RB>
__device__ __forceinline__ StagedB stage_b(const float4 f0, const float4 f1, const float4 f2,
                                           uint32_t id, float hw, float hh, float ox, float oy) {
  const Staged s = stage<RB>(f0, f1, f2, ox, oy);
  StagedB S;
  S.s0 = s.s0;
  S.s1 = s.s1;
  S.s2 = make_float4(s.s2.x, s.s2.y, -f0.z * hw, -f0.w * hw);
  S.s3 = make_float4(-f1.x * hh, -f0.w * hh, __uint_as_float(id), s.s2.z);
  return S;
}

// Adjoint state of one pixel.  acc = colour accumulated behind the Gaussian
// being visited (excluding it); after a blended Gaussian with alpha a and
// colour c it becomes acc + a (c - acc), the reference's one-step-delayed
// update (last_alpha * last_color + (1 - last_alpha) * accum) done at once.
// acc enters the gradients only through (c - acc) . dL/dpixel, so the state
// keeps the scalar ag = acc . dL/dpixel, updated by ag + a (c . dL/dpixel - ag).
struct PixelState {
  float T, Tfb, g0, g1, g2;  // transmittance, T_final * (bg . dL/dpixel), dL/dpixel
  float ag;
  uint32_t last_contrib;
};

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void init_pixel(PixelState &ps, bool inside, int pix, size_t HW,
                                           const float *__restrict__ final_Ts,
                                           const uint32_t *__restrict__ n_contrib,
                                           const float *__restrict__ dL_dout, float bg0,
                                           float bg1, float bg2) {
  const float T_final = inside ? final_Ts[pix] : 0.f;
  ps.last_contrib = inside ? n_contrib[pix] : 0u;
  ps.g0 = inside ? dL_dout[pix] : 0.f;
  ps.g1 = inside ? dL_dout[HW + pix] : 0.f;
  ps.g2 = inside ? dL_dout[2 * HW + pix] : 0.f;
  ps.T = T_final;
  ps.Tfb = T_final * (bg0 * ps.g0 + bg1 * ps.g1 + bg2 * ps.g2);
  ps.ag = 0.f;
}

// One (pixel, Gaussian) term of the adjoint, accumulated into e[0..2] and
// e[6..8] when `take` (the pair was blended in the forward); otherwise the
// state and e[] are left as they are.  Evaluated without branches: the state
// updates are selects or scaled by a factor selected to 0, so a warp whose
// lanes differ in `take` runs one straight-line path.  T is recovered by
// dividing by (1 - alpha) with the hardware reciprocal (alpha <= 0.99).
__device__ __forceinline__ void adjoint_pair(PixelState &ps, bool take, float alpha, float G,
                                             const float4 &s1, const float4 &s2, float dy,
                                             float *e) {
  const float inv = rcp_approx(1.f - alpha);
  const float Tn = ps.T * inv;
  const float cg = fmaf(s2.y, ps.g2, fmaf(s2.x, ps.g1, s1.w * ps.g0));  // c . dL/dpixel
  const float S = cg - ps.ag;                    // (c - acc) . dL/dpixel
  const float dL_dalpha = S * Tn - ps.Tfb * inv;
  const float Gd = take ? G * dL_dalpha : 0.f;  // dL/dopacity term
  const float at = take ? alpha : 0.f;
  const float wt = at * Tn;                      // dL/drgb weight
  const float gy = Gd * dy;
  // dL/dpower = o G dL/dalpha and the thread's pixels share dx: the mean and
  // conic terms need only sum Gd, sum Gd dy and sum Gd dy^2 (combined with
  // o and dx once per Gaussian)
  e[0] += Gd;
  e[1] += gy;
  e[2] += gy * dy;
  e[6] += wt * ps.g0;             // dL/drgb
  e[7] += wt * ps.g1;
  e[8] += wt * ps.g2;
  ps.T = take ? Tn : ps.T;
  ps.ag = fmaf(at, S, ps.ag);
}

// From the thread's sums (e[0] = sum Gd, e[1] = sum Gd dy, e[2] = sum Gd dy^2
// over its pixels; u = o Gd = dL/dpower) to the gradient terms: e0 =
// dL/dndc_x, e1 = dL/dndc_y, e2..e4 = (sum u dx^2, sum u dx dy, sum u dy^2)
// for the conic (scaled by -1/2, -1, -1/2 at the atomics), e5 = dL/dopacity.
__device__ __forceinline__ void adjoint_finish(float dx, float o, const float4 &s2,
                                               const float4 &s3, float *e) {
  e[5] = e[0];
  const float su = o * e[0], suy = o * e[1], suy2 = o * e[2];
  const float sux = dx * su;
  e[0] = sux * s2.z + suy * s2.w;
  e[1] = suy * s3.x + sux * s3.y;
  e[2] = sux * dx;
  e[3] = suy * dx;
  e[4] = suy2;
}

// Transposed reduce-scatter of the 9 gradient slots over the warp, 12
// shuffles: each level halves the slots a lane keeps (5 | 4, 3 | 2, 2 | 1,
// 1 | 1) and adds its partner's copy of them; afterwards the even lane 2q
// holds the warp sum of slot slot9(q) (q = lane bits 4..1), none when that
// is >= 9.
__device__ __forceinline__ float warp_reduce_scatter9(const float (&v)[9], int lane) {
  float a[5], b[3], c[2];
  {
    const bool hi = lane & 16;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const float up = i < 4 ? v[5 + i] : 0.f;
      a[i] = (hi ? up : v[i]) + __shfl_xor_sync(FULL, hi ? v[i] : up, 16);
    }
  }
  {
    const bool hi = lane & 8;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float up = i < 2 ? a[3 + i] : 0.f;
      b[i] = (hi ? up : a[i]) + __shfl_xor_sync(FULL, hi ? a[i] : up, 8);
    }
  }
  {
    const bool hi = lane & 4;
    c[0] = (hi ? b[2] : b[0]) + __shfl_xor_sync(FULL, hi ? b[0] : b[2], 4);
    c[1] = (hi ? 0.f : b[1]) + __shfl_xor_sync(FULL, hi ? b[1] : 0.f, 4);
  }
  const bool hi = lane & 2;
  const float d = (hi ? c[1] : c[0]) + __shfl_xor_sync(FULL, hi ? c[0] : c[1], 2);
  return d + __shfl_xor_sync(FULL, d, 1);
}

// slot of the even lane 2q after warp_reduce_scatter9 (15: none)
__device__ __forceinline__ int slot9(int q) {
  return (int)((0xFFF8F765FF43F210ull >> (4 * q)) & 15u);
}


// F64: the FP64-sum mode — the warp sums are added into double accumulators
// (V.gacc64), so the result does not depend on the order in which warps and
// tiles finish to well below float32 resolution.
template <int PPT, int BATCH, bool F64 = false, int NT = 1>
__global__ void __launch_bounds__(NT * 256 / PPT, (PPT == 4 ? 10 : (PPT == 2 ? 6 : 4)) / NT)
blend_bwd_kernel(const BlendBatch bb, uint32_t *queue) {
  constexpr int THREADS = 256 / PPT;
  __shared__ float4 S0[NT][BATCH], S1[NT][BATCH], S2[NT][BATCH], S3[NT][BATCH];
  __shared__ uint32_t SM[NT][BATCH];                 // footprint rows
  __shared__ uint16_t VL[NT * THREADS / 32][BATCH];  // per-warp visit lists
  __shared__ uint32_t sMaxLast[NT];
  __shared__ int s_item;
  const int h = NT == 1 ? 0 : (int)threadIdx.x / THREADS;  // the CTA half (tile) of this thread
  const int tid = (int)threadIdx.x - h * THREADS;
  const int lane = tid & 31;
  const PixelLayout<PPT> lay(tid);
  int slot_ = 0;
  for (int item = next_item(queue, slot_, &s_item); item < bb.total;
       item = next_item(queue, slot_, &s_item)) {
    const BlendView &V = bb.v[find_view(bb, item)];
    int tx, ty;
    const bool tv = item_tile<NT>(bb, V, item - V.tile_base, h, tx, ty);
    const int tile = ty * V.gx + tx;
    const int px = tx * TILE + lay.col;
    const float pxf = (float)px;
    const float ox = (float)(tx * TILE), oy = (float)(ty * TILE);
    const uint2 range = tv ? V.ranges[tile] : make_uint2(0u, 0u);
    const int n = (int)(range.y - range.x);
    if (n == 0) continue;  // uniform over the tile's half
    const size_t HW = (size_t)V.H * V.W;
    const float bg0 = __ldg(V.bg), bg1 = __ldg(V.bg + 1), bg2 = __ldg(V.bg + 2);
    PixelState ps[PPT];
    float pyf[PPT];
    uint32_t mylast = 0;
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      const int py = ty * TILE + lay.row(k);
      pyf[k] = (float)py;
      const bool in = tv && px < V.W && py < V.H;
      init_pixel(ps[k], in, py * V.W + px, HW, V.final_T, V.n_contrib, V.dL_dout, bg0, bg1, bg2);
      mylast = max(mylast, ps[k].last_contrib);
    }
    if (tid == 0) sMaxLast[h] = 0;
    half_sync<NT>(h, THREADS);
    atomicMax(&sMaxLast[h], mylast);
    half_sync<NT>(h, THREADS);
    const int max_last = (int)sMaxLast[h];  // list positions >= max_last are never blended
    const float hw = 0.5f * (float)V.W, hh = 0.5f * (float)V.H;
    for (int top = max_last; top > 0; top -= BATCH) {
      const int cnt = min(BATCH, top);
      half_sync<NT>(h, THREADS);
      for (int sl = tid; sl < cnt; sl += THREADS) {
        const uint32_t id = V.point_list[range.x + top - 1 - sl];  // back to front
        float4 f0, f1, f2;
        load_record(V, id, f0, f1, f2);
        const StagedB st = stage_b<2 * PPT>(f0, f1, f2, id, hw, hh, ox, oy);
        S0[h][sl] = st.s0; S1[h][sl] = st.s1; S2[h][sl] = st.s2; S3[h][sl] = st.s3;
        SM[h][sl] = __float_as_uint(st.s3.w);
      }
      half_sync<NT>(h, THREADS);
      uint16_t *vl = VL[threadIdx.x >> 5];
      const int nvis = visit_list(SM[h], cnt, lay.warp_rows, vl, lane);
      for (int i = 0; i < nvis; ++i) {
        const int j = vl[i];
        const int li = top - 1 - j;
        const float4 s0 = S0[h][j], s1 = S1[h][j];
        const float dx = __fsub_rn(s0.x, pxf);
        float e2[PPT];
        bool ok[PPT];
        bool cand = false;
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          e2[k] = exponent2(s0.z, s0.w, s1.x, dx, __fsub_rn(s0.y, pyf[k]));
          ok[k] = li < (int)ps[k].last_contrib && !(e2[k] > 0.f) && !(e2[k] < s1.z);
          cand |= ok[k];
        }
        if (!__any_sync(FULL, cand)) continue;  // warp-uniform
        const float4 s2 = S2[h][j], s3 = S3[h][j];
        float e[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) e[i] = 0.f;  // e[3..5] are set by adjoint_finish
        bool any = false;
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          const float G = ex2_approx(e2[k]);
          const float alpha = fminf(ALPHA_MAX, __fmul_rn(s1.y, G));
          const bool take = ok[k] && !(alpha < ALPHA_MIN);
          adjoint_pair(ps[k], take, alpha, G, s1, s2, __fsub_rn(s0.y, pyf[k]), e);
          any |= take;
        }
        if (__ballot_sync(FULL, any)) {
          adjoint_finish(dx, s1.y, s2, s3, e);
          const float sum = warp_reduce_scatter9(e, lane);
          const int slot = slot9((lane >> 1) & 15);
          if (!(lane & 1) && slot < 9) {
            const float scale = (slot == 2 || slot == 4) ? -0.5f : (slot == 3 ? -1.f : 1.f);
            if constexpr (F64)
              atomicAdd(V.gacc64 + (size_t)__float_as_uint(s3.z) * 12 + slot, (double)(sum * scale));
            else
              atomicAdd(V.gacc + (size_t)__float_as_uint(s3.z) * 12 + slot, sum * scale);
          }
        }
      }
    }
  }
}

// Persistent grid = resident CTAs (SMs x blocks per SM), looked up once per
// kernel and device (no runtime queries while a graph is being captured
// after the first call).
template <typename K>
int grid_for(K kernel, int threads, int total, bool persistent, int &grid, int &cached_dev,
             int &cached_slots) {
  if (!persistent) { grid = total; return DMGS_OK; }
  int dev = 0;
  DMGS_CUDA(cudaGetDevice(&dev));
  if (dev != cached_dev) {
    int sms = 0, per = 0;
    DMGS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DMGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0));
    cached_slots = sms * max(per, 1);
    cached_dev = dev;
  }
  grid = max(1, min(total, cached_slots));
  return DMGS_OK;
}

template <int PPT, int BATCH, int NT = 1>
int run_fwd(const BlendBatch &bb, uint32_t *queue, cudaStream_t s) {
  thread_local int cdev = -1, cslots = 0;  // per kernel instantiation and host thread
  int grid;
  const int r = grid_for(blend_fwd_kernel<PPT, BATCH, NT>, NT * 256 / PPT, bb.total,
                         queue != nullptr, grid, cdev, cslots);
  if (r != DMGS_OK) return r;
  dmgs_host::note_launch(), blend_fwd_kernel<PPT, BATCH, NT><<<grid, NT * 256 / PPT, 0, s>>>(bb, queue);
  return DMGS_OK;
}

template <int PPT, int BATCH, bool F64 = false, int NT = 1>
int run_bwd(const BlendBatch &bb, uint32_t *queue, cudaStream_t s) {
  thread_local int cdev = -1, cslots = 0;  // per kernel instantiation and host thread
  int grid;
  const int r = grid_for(blend_bwd_kernel<PPT, BATCH, F64, NT>, NT * 256 / PPT, bb.total,
                         queue != nullptr, grid, cdev, cslots);
  if (r != DMGS_OK) return r;
  dmgs_host::note_launch(), blend_bwd_kernel<PPT, BATCH, F64, NT><<<grid, NT * 256 / PPT, 0, s>>>(bb, queue);
  return DMGS_OK;
}

// Rounds the FP64 accumulators into the float records the preprocess
// adjoint reads.
__global__ void gacc_round_kernel(const double *__restrict__ g64, float *__restrict__ g, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) g[i] = (float)g64[i];
}

template <bool FWD>
int dispatch(const BlendBatch &bb, const BlendCfg &cfg, uint32_t *queue, cudaStream_t s) {
  const bool pair = cfg.sx * cfg.sy == 2;
  if (cfg.sx * cfg.sy > 2 || cfg.sx < 1 || cfg.sy < 1) {
    dmgs_host::set_error("unsupported blend CTA shape: %d x %d tiles", cfg.sx, cfg.sy);
    return DMGS_ERR_ARG;
  }
#define DMGS_BLEND_CASE(P_, B_)                                                     \
  if (!pair && cfg.ppt == P_ && cfg.batch == B_)                                    \
    return FWD ? run_fwd<P_, B_>(bb, queue, s) : run_bwd<P_, B_>(bb, queue, s);
  DMGS_BLEND_CASE(1, 128) DMGS_BLEND_CASE(1, 256) DMGS_BLEND_CASE(1, 512)
  DMGS_BLEND_CASE(2, 128) DMGS_BLEND_CASE(2, 256) DMGS_BLEND_CASE(2, 512)
  DMGS_BLEND_CASE(4, 128) DMGS_BLEND_CASE(4, 256) DMGS_BLEND_CASE(4, 512)
#undef DMGS_BLEND_CASE
#define DMGS_BLEND_PAIR(P_, B_)                                                     \
  if (pair && cfg.ppt == P_ && cfg.batch == B_)                                     \
    return FWD ? run_fwd<P_, B_, 2>(bb, queue, s) : run_bwd<P_, B_, false, 2>(bb, queue, s);
  DMGS_BLEND_PAIR(2, 128) DMGS_BLEND_PAIR(2, 256)
  DMGS_BLEND_PAIR(4, 128) DMGS_BLEND_PAIR(4, 256)
#undef DMGS_BLEND_PAIR
  dmgs_host::set_error("unsupported blend configuration: %d pixels/thread, batch %d, %dx%d tiles",
                       cfg.ppt, cfg.batch, cfg.sx, cfg.sy);
  return DMGS_ERR_ARG;
}

// The batch with its work items counted in CTA cells of sx x sy tiles.
BlendBatch with_shape(const BlendBatch &bb, const BlendCfg &cfg) {
  BlendBatch b = bb;
  b.sx = cfg.sx;
  b.sy = cfg.sy;
  if (cfg.sx * cfg.sy == 1) return b;
  int base = 0;
  for (int v = 0; v < b.nviews; ++v) {
    BlendView &o = b.v[v];
    const int gy = o.gx > 0 ? o.T / o.gx : 0;
    o.tile_base = base;
    base += ((o.gx + cfg.sx - 1) / cfg.sx) * ((gy + cfg.sy - 1) / cfg.sy);
  }
  b.total = base;
  return b;
}

}  // namespace

int launch_blend_batch_fwd(const BlendBatch &bb, const BlendCfg &cfg, uint32_t *queue,
                           cudaStream_t s) {
  if (bb.total <= 0) return DMGS_OK;
  int r = DMGS_OK;
  const BlendBatch b = with_shape(bb, cfg);
  DMGS_TIMED(K_BLEND_FWD, s, r = dispatch<true>(b, cfg, queue, s));
  if (r != DMGS_OK) return r;
  DMGS_LAUNCH_CHECK("blend_fwd_kernel");
  return DMGS_OK;
}

int launch_blend_batch_bwd(const BlendBatch &bb, const BlendCfg &cfg, uint32_t *queue,
                           cudaStream_t s) {
  if (bb.total <= 0) return DMGS_OK;
  int r = DMGS_OK;
  const BlendBatch b = with_shape(bb, cfg);
  DMGS_TIMED(K_BLEND_BWD, s, r = dispatch<false>(b, cfg, queue, s));
  if (r != DMGS_OK) return r;
  DMGS_LAUNCH_CHECK("blend_bwd_kernel");
  return DMGS_OK;
}

BlendView make_blend_view(const ViewParams &vp, const GeomLayout &L, const char *geom,
                          const BinLayout &B, const char *bin, const ImgLayout &I, char *img,
                          const float *bg) {
  BlendView v;
  v.W = vp.W; v.H = vp.H; v.gx = L.gx; v.T = L.T(); v.tile_base = 0;
  v.P = (uint32_t)L.P;
  v.ranges = reinterpret_cast<const uint2 *>(geom + L.ranges);
  v.point_list = reinterpret_cast<const uint32_t *>(bin + B.point_list);
  v.feat = reinterpret_cast<const float4 *>(geom + L.feat);
  v.bg = bg;
  v.out_color = nullptr;
  v.final_T = reinterpret_cast<float *>(img + I.final_T);
  v.n_contrib = reinterpret_cast<uint32_t *>(img + I.n_contrib);
  v.dL_dout = nullptr;
  v.gacc = nullptr;
  v.gacc64 = nullptr;
  return v;
}

int launch_blend_fwd(const ViewParams &vp, const GeomLayout &L, const char *geom,
                     const BinLayout &B, const char *bin, const ImgLayout &I, char *img,
                     const float *bg, float *out_color, cudaStream_t s) {
  BlendBatch bb;
  bb.nviews = 1;
  bb.v[0] = make_blend_view(vp, L, geom, B, bin, I, img, bg);
  bb.v[0].out_color = out_color;
  bb.total = bb.v[0].T;
  return launch_blend_batch_fwd(bb, default_blend_cfg(), nullptr, s);
}

int launch_blend_bwd(const ViewParams &vp, const GeomLayout &L, const char *geom,
                     const BinLayout &B, const char *bin, const ImgLayout &I, const char *img,
                     const float *bg, const float *dL_dout, float *gacc, double *gacc64,
                     cudaStream_t s) {
  DMGS_CUDA(cudaMemsetAsync(gacc, 0, (size_t)L.P * 48, s));
  BlendBatch bb;
  bb.nviews = 1;
  bb.v[0] = make_blend_view(vp, L, geom, B, bin, I, const_cast<char *>(img), bg);
  bb.v[0].dL_dout = dL_dout;
  bb.v[0].gacc = gacc;
  bb.v[0].gacc64 = gacc64;
  bb.total = bb.v[0].T;
  if (gacc64 == nullptr) return launch_blend_batch_bwd(bb, default_blend_cfg(), nullptr, s);
  const size_t n = (size_t)L.P * 12;
  DMGS_CUDA(cudaMemsetAsync(gacc64, 0, n * sizeof(double), s));
  if (bb.total > 0) {
    int r = DMGS_OK;
    DMGS_TIMED(K_BLEND_BWD, s, r = (run_bwd<4, 128, true>(bb, nullptr, s)));
    if (r != DMGS_OK) return r;
    DMGS_LAUNCH_CHECK("blend_bwd_kernel (FP64 sums)");
  }
  if (n > 0) {
    dmgs_host::note_launch(), gacc_round_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(gacc64, gacc, n);
    DMGS_LAUNCH_CHECK("gacc_round_kernel");
  }
  return DMGS_OK;
}

}  // namespace dmgs
