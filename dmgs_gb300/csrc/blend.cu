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
// * one 128-thread CTA per 16x16 tile; thread t owns pixels (t%16, t/16)
//   and (t%16, t/16 + 8), which share dx and every shared-memory load;
// * Gaussians are staged in shared memory in batches of 256; in the forward
//   the next batch's global loads are in flight while the current batch is
//   blended (double buffer);
// * at staging, the conic is scaled by -log2(e)/2 (so the falloff is one
//   ex2 instruction) and a per-Gaussian exponent threshold
//   log2(1/(255 o)) is precomputed: a pair below it cannot reach alpha 1/255
//   and is rejected before the exponential (the alpha test itself is still
//   applied afterwards);
// * each staged Gaussian carries row/column masks of the tile pixels its
//   alpha >= 1/255 ellipse can reach (a superset): a warp skips it with one
//   uniform test when it misses the warp's rows, a lane when it misses the
//   lane's column — only pairs the exact test would reject are skipped;
// * the forward and the adjoint evaluate the exponent with the same
//   explicitly rounded operations, so their skip/stop decisions agree;
// * the adjoint sums a Gaussian's nine gradient terms over the thread's two
//   pixels, then over the warp with a transposed reduce-scatter (16
//   shuffles); nine lanes then issue one scalar reduction each.
#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int BLEND_THREADS = 128;
constexpr int BATCH = 256;
constexpr int PER_THREAD = BATCH / BLEND_THREADS;  // Gaussians staged per thread
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
// s2 = (g, b, footprint masks, 0) with exponent2 = A dx^2 + B dx dy + C dy^2
// (A = -a log2e / 2, B = -b log2e, C = -c log2e / 2) and thr = log2(1 / (255 o)).
// The footprint masks (bits 0-15: tile rows, 16-31: tile columns) cover the
// pixels of this tile where alpha can reach 1/255: the ellipse
// (a dx^2 + 2 b dx dy + c dy^2) <= 2 ln(255 o), whose half-extents are
// sqrt(R^2 c / det) and sqrt(R^2 a / det), inflated by 0.1% + 0.01 px so that
// the masks are a superset of the pixels the exact test accepts.
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
  if (!(det > 0.f) || !(a > 0.f) || !(c > 0.f)) return 0xffffffffu;  // not an ellipse
  const float R2 = 2.f * (__logf(o) + 5.541263545158426f);  // 2 ln(255 o)
  if (!(R2 >= 0.f)) return 0u;
  const float ex = sqrtf(R2 * c / det) * 1.001f + 0.01f;
  const float ey = sqrtf(R2 * a / det) * 1.001f + 0.01f;
  return span_mask(cy, ey) | (span_mask(cx, ex) << 16);
}

// (ox, oy): pixel origin of the tile being blended.
__device__ __forceinline__ Staged stage(const float4 f0, const float4 f1, const float4 f2,
                                        float ox, float oy) {
  Staged S;
  const float A = __fmul_rn(-0.5f * LOG2E, f0.z);
  const float B = __fmul_rn(-LOG2E, f0.w);
  const float C = __fmul_rn(-0.5f * LOG2E, f1.x);
  const float thr = -LOG2_255 - __log2f(f1.y);
  const uint32_t m = footprint(f0.z, f0.w, f1.x, f1.y, f0.x - ox, f0.y - oy);
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

// Returns alpha (>= 1/255) or 0 when the pair is skipped; G = e^power.
__device__ __forceinline__ float pair_alpha(float e2, float o, float thr, float &G) {
  if (e2 > 0.f || e2 < thr) return 0.f;
  G = ex2_approx(e2);
  const float alpha = fminf(ALPHA_MAX, __fmul_rn(o, G));
  return alpha < ALPHA_MIN ? 0.f : alpha;
}

__global__ void __launch_bounds__(BLEND_THREADS, 6)
blend_fwd_kernel(int W, int H, int gx, const uint2 *__restrict__ ranges,
                 const uint32_t *__restrict__ point_list, const float4 *__restrict__ feat,
                 const float *__restrict__ bg, float *__restrict__ out_color,
                 float *__restrict__ final_T, uint32_t *__restrict__ n_contrib) {
  __shared__ float4 S0[2][BATCH];
  __shared__ float4 S1[2][BATCH];
  __shared__ float4 S2[2][BATCH];
  const int tile = blockIdx.x;
  const int tx = tile % gx, ty = tile / gx;
  const int tid = threadIdx.x;
  const int px = tx * TILE + (tid & (TILE - 1));
  const int py0 = ty * TILE + (tid >> 4);
  const int py1 = py0 + 8;
  const bool in0 = px < W && py0 < H, in1 = px < W && py1 < H;
  const float pxf = (float)px, py0f = (float)py0, py1f = (float)py1;
  const float ox = (float)(tx * TILE), oy = (float)(ty * TILE);
  const uint2 range = ranges[tile];
  const int n = (int)(range.y - range.x);
  // footprint-mask bits of this thread's pixels and of its warp's rows
  const int r0 = tid >> 4;
  const uint32_t colbit = 1u << (16 + (tid & 15));
  const uint32_t row0bit = 1u << r0, row1bit = 1u << (r0 + 8);
  const uint32_t warp_rows = (3u << ((r0 >> 1) << 1)) | (3u << (((r0 >> 1) << 1) + 8));

  bool done0 = !in0, done1 = !in1;
  float T0 = 1.f, T1 = 1.f;
  float r0c = 0.f, g0 = 0.f, b0 = 0.f, r1 = 0.f, g1 = 0.f, b1 = 0.f;
  uint32_t last0 = 0, last1 = 0;

  // prefetch batch 0 into registers
  float4 pf0[PER_THREAD], pf1[PER_THREAD], pf2[PER_THREAD];
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int i = k * BLEND_THREADS + tid;
    if (i < n) {
      const uint32_t id = point_list[range.x + i];
      pf0[k] = feat[3 * id]; pf1[k] = feat[3 * id + 1]; pf2[k] = feat[3 * id + 2];
    }
  }
  int buf = 0;
  for (int base = 0; base < n; base += BATCH) {
    // stage the prefetched batch (buffer `buf` was last read two batches ago,
    // before the barrier below of the previous iteration)
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
      const int i = base + k * BLEND_THREADS + tid;
      if (i < n) {
        const Staged s = stage(pf0[k], pf1[k], pf2[k], ox, oy);
        const int slot = k * BLEND_THREADS + tid;
        S0[buf][slot] = s.s0; S1[buf][slot] = s.s1; S2[buf][slot] = s.s2;
      }
    }
    if (__syncthreads_count(done0 && done1) == BLEND_THREADS) break;
    // prefetch the next batch while this one is blended
    const int nbase = base + BATCH;
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
      const int i = nbase + k * BLEND_THREADS + tid;
      if (i < n) {
        const uint32_t id = point_list[range.x + i];
        pf0[k] = feat[3 * id]; pf1[k] = feat[3 * id + 1]; pf2[k] = feat[3 * id + 2];
      }
    }
    const int cnt = min(BATCH, n - base);
    for (int j = 0; j < cnt && !(done0 && done1); ++j) {
      const float4 s2 = S2[buf][j];
      const uint32_t m = __float_as_uint(s2.z);
      if (!(m & warp_rows)) continue;  // warp-uniform: the footprint misses the warp's rows
      if (!(m & colbit)) continue;
      const float4 s0 = S0[buf][j];
      const float4 s1 = S1[buf][j];
      const float dx = __fsub_rn(s0.x, pxf);
      if (!done0 && (m & row0bit)) {
        float G;
        const float e2 = exponent2(s0.z, s0.w, s1.x, dx, __fsub_rn(s0.y, py0f));
        const float alpha = pair_alpha(e2, s1.y, s1.z, G);
        if (alpha > 0.f) {
          const float test_T = T0 * (1.f - alpha);
          if (test_T < T_EPS) {
            done0 = true;
          } else {
            const float w = alpha * T0;
            r0c = fmaf(s1.w, w, r0c); g0 = fmaf(s2.x, w, g0); b0 = fmaf(s2.y, w, b0);
            T0 = test_T;
            last0 = base + j + 1;
          }
        }
      }
      if (!done1 && (m & row1bit)) {
        float G;
        const float e2 = exponent2(s0.z, s0.w, s1.x, dx, __fsub_rn(s0.y, py1f));
        const float alpha = pair_alpha(e2, s1.y, s1.z, G);
        if (alpha > 0.f) {
          const float test_T = T1 * (1.f - alpha);
          if (test_T < T_EPS) {
            done1 = true;
          } else {
            const float w = alpha * T1;
            r1 = fmaf(s1.w, w, r1); g1 = fmaf(s2.x, w, g1); b1 = fmaf(s2.y, w, b1);
            T1 = test_T;
            last1 = base + j + 1;
          }
        }
      }
    }
    buf ^= 1;
  }
  const size_t HW = (size_t)H * W;
  const float bgr = __ldg(bg), bgg = __ldg(bg + 1), bgb = __ldg(bg + 2);
  if (in0) {
    const int pix = py0 * W + px;
    final_T[pix] = T0;
    n_contrib[pix] = last0;
    out_color[pix] = r0c + T0 * bgr;
    out_color[HW + pix] = g0 + T0 * bgg;
    out_color[2 * HW + pix] = b0 + T0 * bgb;
  }
  if (in1) {
    const int pix = py1 * W + px;
    final_T[pix] = T1;
    n_contrib[pix] = last1;
    out_color[pix] = r1 + T1 * bgr;
    out_color[HW + pix] = g1 + T1 * bgg;
    out_color[2 * HW + pix] = b1 + T1 * bgb;
  }
}

// ------------------------------- adjoint -----------------------------------

// Staged Gaussian (adjoint): s0 = (x, y, A, B), s1 = (C, o, thr, r),
// s2 = (g, b, ka, kb), s3 = (kc, kd, id bits, footprint masks) with ka = -a W/2,
// kb = -b W/2, kc = -c H/2, kd = -b H/2 (the NDC-mean gradient factors).
struct StagedB {
  float4 s0, s1, s2, s3;
};

__device__ __forceinline__ StagedB stage_b(const float4 f0, const float4 f1, const float4 f2,
                                           uint32_t id, float hw, float hh, float ox, float oy) {
  const Staged s = stage(f0, f1, f2, ox, oy);
  StagedB S;
  S.s0 = s.s0;
  S.s1 = s.s1;
  S.s2 = make_float4(s.s2.x, s.s2.y, -f0.z * hw, -f0.w * hw);
  S.s3 = make_float4(-f1.x * hh, -f0.w * hh, __uint_as_float(id), s.s2.z);
  return S;
}

struct PixelState {
  float T, T_final, g0, g1, g2, bg_dot;
  float acc_r, acc_g, acc_b, last_alpha, last_r, last_g, last_b;
  uint32_t last_contrib;
};

__device__ __forceinline__ void init_pixel(PixelState &ps, bool inside, int pix, size_t HW,
                                           const float *__restrict__ final_Ts,
                                           const uint32_t *__restrict__ n_contrib,
                                           const float *__restrict__ dL_dout, float bg0,
                                           float bg1, float bg2) {
  ps.T_final = inside ? final_Ts[pix] : 0.f;
  ps.last_contrib = inside ? n_contrib[pix] : 0u;
  ps.g0 = inside ? dL_dout[pix] : 0.f;
  ps.g1 = inside ? dL_dout[HW + pix] : 0.f;
  ps.g2 = inside ? dL_dout[2 * HW + pix] : 0.f;
  ps.T = ps.T_final;
  ps.bg_dot = bg0 * ps.g0 + bg1 * ps.g1 + bg2 * ps.g2;
  ps.acc_r = ps.acc_g = ps.acc_b = 0.f;
  ps.last_alpha = ps.last_r = ps.last_g = ps.last_b = 0.f;
}

// One (pixel, Gaussian) term of the adjoint, accumulated into e[0..8];
// returns whether the pair contributed.
__device__ __forceinline__ bool adjoint_pair(PixelState &ps, const float4 &s0, const float4 &s1,
                                             const float4 &s2, const float4 &s3, float dx,
                                             float dy, float *e) {
  float G;
  const float e2 = exponent2(s0.z, s0.w, s1.x, dx, dy);
  const float alpha = pair_alpha(e2, s1.y, s1.z, G);
  if (alpha == 0.f) return false;
  const float inv = __frcp_rn(1.f - alpha);
  ps.T = ps.T * inv;
  const float w = alpha * ps.T;
  ps.acc_r = ps.last_alpha * ps.last_r + (1.f - ps.last_alpha) * ps.acc_r;
  ps.acc_g = ps.last_alpha * ps.last_g + (1.f - ps.last_alpha) * ps.acc_g;
  ps.acc_b = ps.last_alpha * ps.last_b + (1.f - ps.last_alpha) * ps.acc_b;
  const float cr = s1.w, cg = s2.x, cb = s2.y;
  ps.last_r = cr; ps.last_g = cg; ps.last_b = cb;
  ps.last_alpha = alpha;
  float dL_dalpha =
      ((cr - ps.acc_r) * ps.g0 + (cg - ps.acc_g) * ps.g1 + (cb - ps.acc_b) * ps.g2) * ps.T;
  dL_dalpha -= ps.T_final * inv * ps.bg_dot;
  const float Gd = G * dL_dalpha;  // dL/dopacity term
  const float u = s1.y * Gd;       // dL/dpower = o G dL/dalpha
  const float ux = u * dx, uy = u * dy;
  e[0] += ux * s2.z + uy * s2.w;   // dL/dndc_x
  e[1] += uy * s3.x + ux * s3.y;   // dL/dndc_y
  e[2] += ux * dx;                 // x -1/2 -> dL/dconic_a
  e[3] += ux * dy;                 // x -1   -> dL/dconic_b
  e[4] += uy * dy;                 // x -1/2 -> dL/dconic_c
  e[5] += Gd;                      // dL/dopacity
  e[6] += w * ps.g0;               // dL/drgb
  e[7] += w * ps.g1;
  e[8] += w * ps.g2;
  return true;
}

// Transposed reduce-scatter of 16 slots over the warp: afterwards the lane
// whose bits (4,3,2,1) equal s holds the warp sum of slot s.
__device__ __forceinline__ float warp_reduce_scatter16(float v[16], int lane) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const bool hi = lane & 16;
    const float keep = hi ? v[i + 8] : v[i];
    const float send = hi ? v[i] : v[i + 8];
    v[i] = keep + __shfl_xor_sync(FULL, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool hi = lane & 8;
    const float keep = hi ? v[i + 4] : v[i];
    const float send = hi ? v[i] : v[i + 4];
    v[i] = keep + __shfl_xor_sync(FULL, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool hi = lane & 4;
    const float keep = hi ? v[i + 2] : v[i];
    const float send = hi ? v[i] : v[i + 2];
    v[i] = keep + __shfl_xor_sync(FULL, send, 4);
  }
  {
    const bool hi = lane & 2;
    const float keep = hi ? v[1] : v[0];
    const float send = hi ? v[0] : v[1];
    v[0] = keep + __shfl_xor_sync(FULL, send, 2);
  }
  return v[0] + __shfl_xor_sync(FULL, v[0], 1);
}

__global__ void __launch_bounds__(BLEND_THREADS)
blend_bwd_kernel(int W, int H, int gx, const uint2 *__restrict__ ranges,
                 const uint32_t *__restrict__ point_list, const float4 *__restrict__ feat,
                 const float *__restrict__ bg, const float *__restrict__ final_Ts,
                 const uint32_t *__restrict__ n_contrib, const float *__restrict__ dL_dout,
                 float *__restrict__ gacc) {
  __shared__ float4 S0[BATCH], S1[BATCH], S2[BATCH], S3[BATCH];
  __shared__ uint32_t sMaxLast;
  const int tile = blockIdx.x;
  const int tx = tile % gx, ty = tile / gx;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int px = tx * TILE + (tid & (TILE - 1));
  const int py0 = ty * TILE + (tid >> 4);
  const int py1 = py0 + 8;
  const bool in0 = px < W && py0 < H, in1 = px < W && py1 < H;
  const float pxf = (float)px, py0f = (float)py0, py1f = (float)py1;
  const float ox = (float)(tx * TILE), oy = (float)(ty * TILE);
  const uint2 range = ranges[tile];
  const int n = (int)(range.y - range.x);
  if (n == 0) return;
  const int r0 = tid >> 4;
  const uint32_t colbit = 1u << (16 + (tid & 15));
  const uint32_t row0bit = 1u << r0, row1bit = 1u << (r0 + 8);
  const uint32_t warp_rows = (3u << ((r0 >> 1) << 1)) | (3u << (((r0 >> 1) << 1) + 8));

  const size_t HW = (size_t)H * W;
  const float bg0 = __ldg(bg), bg1 = __ldg(bg + 1), bg2 = __ldg(bg + 2);
  PixelState P0, P1;
  init_pixel(P0, in0, py0 * W + px, HW, final_Ts, n_contrib, dL_dout, bg0, bg1, bg2);
  init_pixel(P1, in1, py1 * W + px, HW, final_Ts, n_contrib, dL_dout, bg0, bg1, bg2);
  if (tid == 0) sMaxLast = 0;
  __syncthreads();
  atomicMax(&sMaxLast, max(P0.last_contrib, P1.last_contrib));
  __syncthreads();
  const int max_last = (int)sMaxLast;  // list positions >= max_last are never blended
  const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;

  // Walk list positions max_last-1 down to 0 in batches of BATCH.
  for (int top = max_last; top > 0; top -= BATCH) {
    const int cnt = min(BATCH, top);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
      const int slot = k * BLEND_THREADS + tid;
      if (slot < cnt) {
        const uint32_t id = point_list[range.x + top - 1 - slot];  // back to front
        const StagedB s =
            stage_b(feat[3 * id], feat[3 * id + 1], feat[3 * id + 2], id, hw, hh, ox, oy);
        S0[slot] = s.s0; S1[slot] = s.s1; S2[slot] = s.s2; S3[slot] = s.s3;
      }
    }
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      const int li = top - 1 - j;
      const float4 s3 = S3[j];
      const uint32_t m = __float_as_uint(s3.w);
      if (!(m & warp_rows)) continue;  // warp-uniform: the footprint misses the warp's rows
      const float4 s0 = S0[j], s1 = S1[j], s2 = S2[j];
      float e[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) e[i] = 0.f;
      const float dx = __fsub_rn(s0.x, pxf);
      bool any = false;
      if ((m & colbit) && (m & row0bit) && li < (int)P0.last_contrib)
        any |= adjoint_pair(P0, s0, s1, s2, s3, dx, __fsub_rn(s0.y, py0f), e);
      if ((m & colbit) && (m & row1bit) && li < (int)P1.last_contrib)
        any |= adjoint_pair(P1, s0, s1, s2, s3, dx, __fsub_rn(s0.y, py1f), e);
      if (__ballot_sync(FULL, any)) {
        const float sum = warp_reduce_scatter16(e, lane);
        const int slot = (lane >> 1) & 15;  // lane bits (4,3,2,1)
        if (!(lane & 1) && slot < 9) {
          const float scale = (slot == 2 || slot == 4) ? -0.5f : (slot == 3 ? -1.f : 1.f);
          atomicAdd(gacc + (size_t)__float_as_uint(s3.z) * 12 + slot, sum * scale);
        }
      }
    }
  }
}

}  // namespace

int launch_blend_fwd(const ViewParams &vp, const GeomLayout &L, const char *geom,
                     const BinLayout &B, const char *bin, const ImgLayout &I, char *img,
                     const float *bg, float *out_color, cudaStream_t s) {
  const int T = L.T();
  if (T == 0) return DMGS_OK;
  DMGS_TIMED(K_BLEND_FWD, s, blend_fwd_kernel<<<T, BLEND_THREADS, 0, s>>>(
      vp.W, vp.H, L.gx, reinterpret_cast<const uint2 *>(geom + L.ranges),
      reinterpret_cast<const uint32_t *>(bin + B.point_list),
      reinterpret_cast<const float4 *>(geom + L.feat), bg, out_color,
      reinterpret_cast<float *>(img + I.final_T), reinterpret_cast<uint32_t *>(img + I.n_contrib)));
  DMGS_LAUNCH_CHECK("blend_fwd_kernel");
  return DMGS_OK;
}

int launch_blend_bwd(const ViewParams &vp, const GeomLayout &L, const char *geom,
                     const BinLayout &B, const char *bin, const ImgLayout &I, const char *img,
                     const float *bg, const float *dL_dout, float *gacc, cudaStream_t s) {
  const int T = L.T();
  DMGS_CUDA(cudaMemsetAsync(gacc, 0, (size_t)L.P * 48, s));
  if (T == 0) return DMGS_OK;
  DMGS_TIMED(K_BLEND_BWD, s, blend_bwd_kernel<<<T, BLEND_THREADS, 0, s>>>(
      vp.W, vp.H, L.gx, reinterpret_cast<const uint2 *>(geom + L.ranges),
      reinterpret_cast<const uint32_t *>(bin + B.point_list),
      reinterpret_cast<const float4 *>(geom + L.feat), bg,
      reinterpret_cast<const float *>(img + I.final_T),
      reinterpret_cast<const uint32_t *>(img + I.n_contrib), dL_dout, gacc));
  DMGS_LAUNCH_CHECK("blend_bwd_kernel");
  return DMGS_OK;
}

}  // namespace dmgs
