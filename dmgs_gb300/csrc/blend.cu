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
// Design: one 256-thread CTA per 16x16 tile, one pixel per thread.  Gaussian
// records (48 B: mean, conic, opacity, rgb) are staged in shared memory in
// batches of 256; a batch loop stops once every pixel of the tile is done
// (__syncthreads_count).  The adjoint reduces each Gaussian's nine gradient
// terms across the warp (32 pixels) with shuffles before one lane issues
// three 16-byte vector atomics (red.global.add.v4.f32).
#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int BATCH = 256;
constexpr float ALPHA_MIN = 1.0f / 255.0f;
constexpr float ALPHA_MAX = 0.99f;
constexpr float T_EPS = 0.0001f;

// Exponent of the 2D Gaussian, written with explicit intrinsics so the
// forward and the adjoint kernels evaluate it identically (their skip and
// stop decisions must agree).
__device__ __forceinline__ float gauss_power(float a, float b, float c, float dx, float dy) {
  const float q = __fmaf_rn(__fmul_rn(a, dx), dx, __fmul_rn(__fmul_rn(c, dy), dy));
  return __fmaf_rn(-0.5f, q, -__fmul_rn(__fmul_rn(b, dx), dy));
}

__global__ void __launch_bounds__(TILE_PIX)
blend_fwd_kernel(int W, int H, int gx, const uint2 *__restrict__ ranges,
                 const uint32_t *__restrict__ point_list, const float4 *__restrict__ feat,
                 const float *__restrict__ bg, float *__restrict__ out_color,
                 float *__restrict__ final_T, uint32_t *__restrict__ n_contrib) {
  __shared__ float4 sA[BATCH];
  __shared__ float4 sB[BATCH];
  __shared__ float sC[BATCH];
  const int tile = blockIdx.x;
  const int tx = tile % gx, ty = tile / gx;
  const int tid = threadIdx.x;
  const int px = tx * TILE + (tid & (TILE - 1));
  const int py = ty * TILE + (tid / TILE);
  const bool inside = px < W && py < H;
  const float pxf = (float)px, pyf = (float)py;
  const uint2 range = ranges[tile];
  const int n = (int)(range.y - range.x);

  bool done = !inside;
  float T = 1.f, Cr = 0.f, Cg = 0.f, Cb = 0.f;
  uint32_t contributor = 0, last = 0;

  for (int base = 0; base < n; base += BATCH) {
    if (__syncthreads_count(done) == TILE_PIX) break;
    const int i = base + tid;
    if (i < n) {
      const uint32_t id = point_list[range.x + i];
      sA[tid] = feat[3 * id + 0];
      sB[tid] = feat[3 * id + 1];
      sC[tid] = feat[3 * id + 2].x;
    }
    __syncthreads();
    const int cnt = min(BATCH, n - base);
    for (int j = 0; !done && j < cnt; ++j) {
      ++contributor;
      const float4 A = sA[j];
      const float4 B = sB[j];
      const float dx = __fsub_rn(A.x, pxf), dy = __fsub_rn(A.y, pyf);
      const float power = gauss_power(A.z, A.w, B.x, dx, dy);
      if (power > 0.f) continue;
      const float alpha = fminf(ALPHA_MAX, __fmul_rn(B.y, __expf(power)));
      if (alpha < ALPHA_MIN) continue;
      const float test_T = T * (1.f - alpha);
      if (test_T < T_EPS) { done = true; continue; }
      const float w = alpha * T;
      Cr += B.z * w;
      Cg += B.w * w;
      Cb += sC[j] * w;
      T = test_T;
      last = contributor;
    }
  }
  if (inside) {
    const int pix = py * W + px;
    final_T[pix] = T;
    n_contrib[pix] = last;
    const size_t HW = (size_t)H * W;
    out_color[pix] = Cr + T * __ldg(bg);
    out_color[HW + pix] = Cg + T * __ldg(bg + 1);
    out_color[2 * HW + pix] = Cb + T * __ldg(bg + 2);
  }
}

__global__ void __launch_bounds__(TILE_PIX)
blend_bwd_kernel(int W, int H, int gx, const uint2 *__restrict__ ranges,
                 const uint32_t *__restrict__ point_list, const float4 *__restrict__ feat,
                 const float *__restrict__ bg, const float *__restrict__ final_Ts,
                 const uint32_t *__restrict__ n_contrib, const float *__restrict__ dL_dout,
                 float *__restrict__ gacc) {
  __shared__ float4 sA[BATCH];
  __shared__ float4 sB[BATCH];
  __shared__ float sC[BATCH];
  __shared__ uint32_t sId[BATCH];
  __shared__ uint32_t sMaxLast;
  const int tile = blockIdx.x;
  const int tx = tile % gx, ty = tile / gx;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int px = tx * TILE + (tid & (TILE - 1));
  const int py = ty * TILE + (tid / TILE);
  const bool inside = px < W && py < H;
  const float pxf = (float)px, pyf = (float)py;
  const uint2 range = ranges[tile];
  const int n = (int)(range.y - range.x);
  if (n == 0) return;

  const int pix = py * W + px;
  const size_t HW = (size_t)H * W;
  const float T_final = inside ? final_Ts[pix] : 0.f;
  float T = T_final;
  const uint32_t last_contrib = inside ? n_contrib[pix] : 0u;
  const float g0 = inside ? dL_dout[pix] : 0.f;
  const float g1 = inside ? dL_dout[HW + pix] : 0.f;
  const float g2 = inside ? dL_dout[2 * HW + pix] : 0.f;
  const float bg0 = __ldg(bg), bg1 = __ldg(bg + 1), bg2 = __ldg(bg + 2);
  const float bg_dot = bg0 * g0 + bg1 * g1 + bg2 * g2;
  const float ddelx_dx = 0.5f * (float)W, ddely_dy = 0.5f * (float)H;

  if (tid == 0) sMaxLast = 0;
  __syncthreads();
  atomicMax(&sMaxLast, last_contrib);
  __syncthreads();
  const int max_last = (int)sMaxLast;  // list positions >= max_last are never blended

  float acc_r = 0.f, acc_g = 0.f, acc_b = 0.f;
  float last_alpha = 0.f, last_r = 0.f, last_g = 0.f, last_b = 0.f;

  // Walk list positions max_last-1 down to 0 in batches of BATCH.
  for (int top = max_last; top > 0; top -= BATCH) {
    const int cnt = min(BATCH, top);
    __syncthreads();
    if (tid < cnt) {
      const int li = top - 1 - tid;  // list index, back to front
      const uint32_t id = point_list[range.x + li];
      sId[tid] = id;
      sA[tid] = feat[3 * id + 0];
      sB[tid] = feat[3 * id + 1];
      sC[tid] = feat[3 * id + 2].x;
    }
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      const int li = top - 1 - j;
      float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f, v4 = 0.f, v5 = 0.f, v6 = 0.f, v7 = 0.f,
            v8 = 0.f;
      bool contrib = false;
      if (li < (int)last_contrib) {
        const float4 A = sA[j];
        const float4 B = sB[j];
        const float dx = __fsub_rn(A.x, pxf), dy = __fsub_rn(A.y, pyf);
        const float power = gauss_power(A.z, A.w, B.x, dx, dy);
        if (power <= 0.f) {
          const float G = __expf(power);
          const float alpha = fminf(ALPHA_MAX, __fmul_rn(B.y, G));
          if (alpha >= ALPHA_MIN) {
            contrib = true;
            T = T / (1.f - alpha);
            const float dchannel_dcolor = alpha * T;
            const float cr = B.z, cg = B.w, cbl = sC[j];
            acc_r = last_alpha * last_r + (1.f - last_alpha) * acc_r;
            acc_g = last_alpha * last_g + (1.f - last_alpha) * acc_g;
            acc_b = last_alpha * last_b + (1.f - last_alpha) * acc_b;
            last_r = cr; last_g = cg; last_b = cbl;
            float dL_dalpha = (cr - acc_r) * g0 + (cg - acc_g) * g1 + (cbl - acc_b) * g2;
            dL_dalpha *= T;
            last_alpha = alpha;
            dL_dalpha += (-T_final / (1.f - alpha)) * bg_dot;
            const float dL_dG = B.y * dL_dalpha;
            const float gdx = G * dx, gdy = G * dy;
            const float dG_ddelx = -gdx * A.z - gdy * A.w;
            const float dG_ddely = -gdy * B.x - gdx * A.w;
            v0 = dL_dG * dG_ddelx * ddelx_dx;      // dL/dndc_x
            v1 = dL_dG * dG_ddely * ddely_dy;      // dL/dndc_y
            v2 = -0.5f * gdx * dx * dL_dG;         // dL/dconic_a
            v3 = -gdx * dy * dL_dG;                // dL/dconic_b
            v4 = -0.5f * gdy * dy * dL_dG;         // dL/dconic_c
            v5 = G * dL_dalpha;                    // dL/dopacity
            v6 = dchannel_dcolor * g0;             // dL/drgb
            v7 = dchannel_dcolor * g1;
            v8 = dchannel_dcolor * g2;
          }
        }
      }
      if (__ballot_sync(0xffffffffu, contrib)) {
        v0 = warp_sum(v0); v1 = warp_sum(v1); v2 = warp_sum(v2);
        v3 = warp_sum(v3); v4 = warp_sum(v4); v5 = warp_sum(v5);
        v6 = warp_sum(v6); v7 = warp_sum(v7); v8 = warp_sum(v8);
        if (lane == 0) {
          float *g = gacc + (size_t)sId[j] * 12;
          red_add_v4(g, v0, v1, v2, v3);
          red_add_v4(g + 4, v4, v5, v6, v7);
          red_add_v4(g + 8, v8, 0.f, 0.f, 0.f);
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
  DMGS_TIMED(K_BLEND_FWD, s, blend_fwd_kernel<<<T, TILE_PIX, 0, s>>>(
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
  DMGS_TIMED(K_BLEND_BWD, s, blend_bwd_kernel<<<T, TILE_PIX, 0, s>>>(
      vp.W, vp.H, L.gx, reinterpret_cast<const uint2 *>(geom + L.ranges),
      reinterpret_cast<const uint32_t *>(bin + B.point_list),
      reinterpret_cast<const float4 *>(geom + L.feat), bg,
      reinterpret_cast<const float *>(img + I.final_T),
      reinterpret_cast<const uint32_t *>(img + I.n_contrib), dL_dout, gacc));
  DMGS_LAUNCH_CHECK("blend_bwd_kernel");
  return DMGS_OK;
}

}  // namespace dmgs
