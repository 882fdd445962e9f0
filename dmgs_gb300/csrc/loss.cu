// loss.cu — fused L1 + SSIM photometric loss and its gradient.
//
// The reference's training loss (train_geo_stage2.py:114-116 with
// utils/loss_utils.py): (1 - lambda) mean |x - y| + lambda (1 - mean SSIM),
// SSIM with an 11 x 11 Gaussian window (sigma 1.5, normalised), zero padding
// of 5, C1 = 0.01^2, C2 = 0.03^2, per channel, averaged over channels and
// pixels (Wang et al. 2004).  In torch that is five depthwise convolutions
// forward and their adjoints.  Here two kernels:
//
//   1. moments: each 16 x 16 tile of every channel loads x, y with a 5-pixel
//      halo into shared memory, blurs the five moments (x, y, xx, yy, xy)
//      separably, and per pixel forms S and the partial derivatives of S
//      w.r.t. mu_x (A), E[x^2] (B) and E[xy] (D); the block's sums of S and
//      |x - y| go to per-block partials;
//   2. gradient: each tile blurs A, B, D (the window is symmetric, so the
//      adjoint of the blur is the same blur) and forms
//      dL/dx = (1 - lambda)/N sign(x - y) - lambda/N (wA + 2 x wB + y wD);
//      the first block also reduces the partials into the loss.
//
// With s11 = E[x^2] - mu_x^2, s22 = E[y^2] - mu_y^2, s12 = E[xy] - mu_x mu_y,
// N1 = 2 mu_x mu_y + C1, N2 = 2 s12 + C2, D1 = mu_x^2 + mu_y^2 + C1,
// D2 = s11 + s22 + C2, S = N1 N2 / (D1 D2):
//   dS/dE[x^2] = -S / D2,  dS/dE[xy] = 2 N1 / (D1 D2),
//   dS/dmu_x   = 2 mu_y (N2 - N1) / (D1 D2) - 2 mu_x S / D1 + 2 mu_x S / D2.
#include <cmath>

#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int LT = 16;        // output tile
constexpr int LR = 5;         // window radius
constexpr int LH = LT + 2 * LR;  // tile with halo (26)

struct Window {
  float w[2 * LR + 1];
};

// Separable blur of NQ quantities held in shared memory as [NQ][LH][LH]
// (halo included): horizontal pass into hs [NQ][LH][LT], vertical pass to
// the tile's pixel (ty, tx) -> out[NQ].
template <int NQ>
__device__ __forceinline__ void blur_tile(const float (*in)[LH][LH], float (*hs)[LH][LT],
                                          const Window &W, float *out) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < LH; r += LT) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      float a = 0.f;
#pragma unroll
      for (int k = 0; k <= 2 * LR; ++k) a = fmaf(W.w[k], in[q][r][tx + k], a);
      hs[q][r][tx] = a;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    float a = 0.f;
#pragma unroll
    for (int k = 0; k <= 2 * LR; ++k) a = fmaf(W.w[k], hs[q][ty + k][tx], a);
    out[q] = a;
  }
}

__device__ __forceinline__ float block_sum(float v, float *red) {
  const int t = threadIdx.y * LT + threadIdx.x;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((t & 31) == 0) red[t >> 5] = v;
  __syncthreads();
  float s = 0.f;
  if (t < LT * LT / 32) s = red[t];
  if (t < 32) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// Grid: (tiles x, tiles y, channels).  ABD: [3][C][H][W] scratch;
// part: 2 floats per block (sum S, sum |x - y|).
__global__ void __launch_bounds__(LT * LT)
ssim_moments_kernel(const float *__restrict__ x, const float *__restrict__ y, int H, int Wd,
                    Window W, float *__restrict__ ABD, float *__restrict__ part) {
  __shared__ float in[5][LH][LH];
  __shared__ float hs[5][LH][LT];
  __shared__ float red[LT * LT / 32];
  const int c = blockIdx.z;
  const size_t plane = (size_t)H * Wd;
  const float *xc = x + c * plane, *yc = y + c * plane;
  const int ox = blockIdx.x * LT - LR, oy = blockIdx.y * LT - LR;
  for (int i = threadIdx.y * LT + threadIdx.x; i < LH * LH; i += LT * LT) {
    const int r = i / LH, q = i - r * LH;
    const int gy = oy + r, gx = ox + q;
    float a = 0.f, b = 0.f;
    if (gy >= 0 && gy < H && gx >= 0 && gx < Wd) {
      a = xc[(size_t)gy * Wd + gx];
      b = yc[(size_t)gy * Wd + gx];
    }
    in[0][r][q] = a; in[1][r][q] = b;
    in[2][r][q] = a * a; in[3][r][q] = b * b; in[4][r][q] = a * b;
  }
  __syncthreads();
  float m[5];
  blur_tile<5>(in, hs, W, m);
  const int px = blockIdx.x * LT + threadIdx.x, py = blockIdx.y * LT + threadIdx.y;
  const bool inside = px < Wd && py < H;
  float S = 0.f, l1 = 0.f;
  if (inside) {
    constexpr float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
    const float mx = m[0], my = m[1];
    const float s11 = m[2] - mx * mx, s22 = m[3] - my * my, s12 = m[4] - mx * my;
    const float N1 = 2.f * mx * my + C1, N2 = 2.f * s12 + C2;
    const float D1 = mx * mx + my * my + C1, D2 = s11 + s22 + C2;
    const float inv = 1.f / (D1 * D2);
    S = N1 * N2 * inv;
    const float A = 2.f * my * (N2 - N1) * inv - 2.f * mx * S / D1 + 2.f * mx * S / D2;
    const float B = -S / D2;
    const float Dd = 2.f * N1 * inv;
    const size_t o = c * plane + (size_t)py * Wd + px;
    const size_t all = (size_t)gridDim.z * plane;
    ABD[o] = A;
    ABD[all + o] = B;
    ABD[2 * all + o] = Dd;
    l1 = fabsf(in[0][threadIdx.y + LR][threadIdx.x + LR] - in[1][threadIdx.y + LR][threadIdx.x + LR]);
  }
  const float sS = block_sum(S, red);
  __syncthreads();
  const float sL = block_sum(l1, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const size_t b = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    part[2 * b] = sS;
    part[2 * b + 1] = sL;
  }
}

__global__ void __launch_bounds__(LT * LT)
ssim_grad_kernel(const float *__restrict__ x, const float *__restrict__ y, int H, int Wd,
                 Window W, const float *__restrict__ ABD, float lambda, float inv_n,
                 float *__restrict__ grad, const float *__restrict__ part, int nparts,
                 float *__restrict__ loss) {
  __shared__ float in[3][LH][LH];
  __shared__ float hs[3][LH][LT];
  __shared__ float red[LT * LT / 32];
  const int c = blockIdx.z;
  const size_t plane = (size_t)H * Wd;
  const size_t all = (size_t)gridDim.z * plane;
  const int ox = blockIdx.x * LT - LR, oy = blockIdx.y * LT - LR;
  for (int i = threadIdx.y * LT + threadIdx.x; i < LH * LH; i += LT * LT) {
    const int r = i / LH, q = i - r * LH;
    const int gy = oy + r, gx = ox + q;
    const bool ok = gy >= 0 && gy < H && gx >= 0 && gx < Wd;
    const size_t o = c * plane + (size_t)gy * Wd + gx;
    in[0][r][q] = ok ? ABD[o] : 0.f;
    in[1][r][q] = ok ? ABD[all + o] : 0.f;
    in[2][r][q] = ok ? ABD[2 * all + o] : 0.f;
  }
  __syncthreads();
  float b[3];
  blur_tile<3>(in, hs, W, b);
  const int px = blockIdx.x * LT + threadIdx.x, py = blockIdx.y * LT + threadIdx.y;
  if (px < Wd && py < H) {
    const size_t o = c * plane + (size_t)py * Wd + px;
    const float xv = x[o], yv = y[o], d = xv - yv;
    const float sgn = (d > 0.f) ? 1.f : (d < 0.f ? -1.f : 0.f);
    const float dS = b[0] + 2.f * xv * b[1] + yv * b[2];
    grad[o] = (1.f - lambda) * inv_n * sgn - lambda * inv_n * dS;
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && loss) {
    // the partials of all blocks of the moments kernel (launched before)
    float sS = 0.f, sL = 0.f;
    for (int i = threadIdx.y * LT + threadIdx.x; i < nparts; i += LT * LT) {
      sS += part[2 * i];
      sL += part[2 * i + 1];
    }
    __syncthreads();
    sS = block_sum(sS, red);
    __syncthreads();
    sL = block_sum(sL, red);
    if (threadIdx.x == 0 && threadIdx.y == 0)
      *loss = (1.f - lambda) * sL * inv_n + lambda * (1.f - sS * inv_n);
  }
}

Window gaussian_window() {
  Window W;
  double g[2 * LR + 1], sum = 0.0;
  for (int k = -LR; k <= LR; ++k) {
    g[k + LR] = std::exp(-(double)(k * k) / (2.0 * 1.5 * 1.5));
    sum += g[k + LR];
  }
  for (int k = 0; k <= 2 * LR; ++k) W.w[k] = (float)(g[k] / sum);
  return W;
}

size_t nblocks(int C, int H, int W) {
  return (size_t)C * ((H + LT - 1) / LT) * ((W + LT - 1) / LT);
}

}  // namespace

}  // namespace dmgs

using namespace dmgs;

extern "C" size_t dmgs_l1_ssim_scratch_bytes(int32_t C, int32_t H, int32_t W) {
  if (C <= 0 || H <= 0 || W <= 0) return 0;
  return l1_ssim_scratch_bytes(C, H, W);
}

extern "C" int dmgs_l1_ssim(const float *image, const float *target, int32_t C, int32_t H,
                            int32_t W, float lambda_dssim, float *loss, float *grad, void *scratch,
                            size_t scratch_bytes, dmgs_stream_t stream) {
  if (C <= 0 || H <= 0 || W <= 0 || !image || !target || !grad) {
    dmgs_host::set_error("l1_ssim: invalid arguments");
    return DMGS_ERR_ARG;
  }
  if (!scratch || scratch_bytes < l1_ssim_scratch_bytes(C, H, W)) {
    dmgs_host::set_error("l1_ssim: scratch too small");
    return DMGS_ERR_STATE;
  }
  return launch_l1_ssim(image, target, C, H, W, lambda_dssim, loss, grad,
                        static_cast<char *>(scratch), reinterpret_cast<cudaStream_t>(stream));
}

namespace dmgs {

size_t l1_ssim_scratch_bytes(int C, int H, int W) {
  return align_up((size_t)3 * C * H * W * 4, 256) + nblocks(C, H, W) * 8;
}

int launch_l1_ssim(const float *x, const float *y, int C, int H, int W, float lambda,
                   float *loss, float *grad, char *scratch, cudaStream_t s) {
  const Window win = gaussian_window();
  float *ABD = reinterpret_cast<float *>(scratch);
  float *part = reinterpret_cast<float *>(scratch + align_up((size_t)3 * C * H * W * 4, 256));
  const dim3 grid((W + LT - 1) / LT, (H + LT - 1) / LT, C), block(LT, LT);
  const float inv_n = 1.f / ((float)C * (float)H * (float)W);
  DMGS_TIMED(K_LOSS, s, {
    dmgs_host::note_launch(), ssim_moments_kernel<<<grid, block, 0, s>>>(x, y, H, W, win, ABD, part);
    dmgs_host::note_launch(), ssim_grad_kernel<<<grid, block, 0, s>>>(
        x, y, H, W, win, ABD, lambda, inv_n, grad, part, (int)nblocks(C, H, W), loss);
  });
  DMGS_LAUNCH_CHECK("ssim kernels");
  return DMGS_OK;
}

}  // namespace dmgs
