// shcolor.cu — the renderer's Python-side colour path fused into one kernel
// and its adjoint (gaussian_renderer/__init__.py:165-170, used by render_dyn
// in stage 2 and by render when convert_SHs_python is set):
//
//   dir = (xyz - campos) / |xyz - campos|
//   colour_c = sigmoid( sum_k b_k(dir) sh[c][k] ),  c = 0..2
//
// b_k is the real SH basis of degree <= 3 with the constants (kSH_C*,
// common.cuh) and signs of utils/sh_utils.py:25-110 (eval_sh); sh is the [P, 3, K] channel-major view
// of the features (K >= (deg + 1)^2 coefficients per channel).  In torch the
// path is ~30 kernels over [P, 3, K] tensors; here one thread per Gaussian
// reads its 12 B position and 3 (deg + 1)^2 coefficients once and writes
// 12 B.  The adjoint recomputes the basis, writes dL/dsh (zero for the
// coefficients above the active degree) and, optionally, dL/dxyz through the
// direction's normalisation.
#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int SHC_THREADS = 256;

// Basis values b[0..15] at unit direction (x, y, z) and, when G is given,
// their partial derivatives G[k][0..2] w.r.t. (x, y, z).
template <bool GRAD>
__device__ __forceinline__ void sh_basis(float x, float y, float z, int deg, float (&b)[16],
                                         float (&G)[16][3]) {
  b[0] = kSH_C0;
  if (GRAD) G[0][0] = G[0][1] = G[0][2] = 0.f;
  if (deg < 1) return;
  b[1] = -kSH_C1 * y;
  b[2] = kSH_C1 * z;
  b[3] = -kSH_C1 * x;
  if (GRAD) {
    G[1][0] = 0.f;   G[1][1] = -kSH_C1; G[1][2] = 0.f;
    G[2][0] = 0.f;   G[2][1] = 0.f;  G[2][2] = kSH_C1;
    G[3][0] = -kSH_C1;  G[3][1] = 0.f;  G[3][2] = 0.f;
  }
  if (deg < 2) return;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  b[4] = kSH_C2[0] * xy;
  b[5] = kSH_C2[1] * yz;
  b[6] = kSH_C2[2] * (2.f * zz - xx - yy);
  b[7] = kSH_C2[3] * xz;
  b[8] = kSH_C2[4] * (xx - yy);
  if (GRAD) {
    G[4][0] = kSH_C2[0] * y;         G[4][1] = kSH_C2[0] * x;         G[4][2] = 0.f;
    G[5][0] = 0.f;                G[5][1] = kSH_C2[1] * z;         G[5][2] = kSH_C2[1] * y;
    G[6][0] = -2.f * kSH_C2[2] * x;  G[6][1] = -2.f * kSH_C2[2] * y;  G[6][2] = 4.f * kSH_C2[2] * z;
    G[7][0] = kSH_C2[3] * z;         G[7][1] = 0.f;                G[7][2] = kSH_C2[3] * x;
    G[8][0] = 2.f * kSH_C2[4] * x;   G[8][1] = -2.f * kSH_C2[4] * y;  G[8][2] = 0.f;
  }
  if (deg < 3) return;
  b[9] = kSH_C3[0] * y * (3.f * xx - yy);
  b[10] = kSH_C3[1] * xy * z;
  b[11] = kSH_C3[2] * y * (4.f * zz - xx - yy);
  b[12] = kSH_C3[3] * z * (2.f * zz - 3.f * xx - 3.f * yy);
  b[13] = kSH_C3[4] * x * (4.f * zz - xx - yy);
  b[14] = kSH_C3[5] * z * (xx - yy);
  b[15] = kSH_C3[6] * x * (xx - 3.f * yy);
  if (GRAD) {
    G[9][0] = 6.f * kSH_C3[0] * xy;              G[9][1] = 3.f * kSH_C3[0] * (xx - yy);
    G[9][2] = 0.f;
    G[10][0] = kSH_C3[1] * yz;                   G[10][1] = kSH_C3[1] * xz;
    G[10][2] = kSH_C3[1] * xy;
    G[11][0] = -2.f * kSH_C3[2] * xy;            G[11][1] = kSH_C3[2] * (4.f * zz - xx - 3.f * yy);
    G[11][2] = 8.f * kSH_C3[2] * yz;
    G[12][0] = -6.f * kSH_C3[3] * xz;            G[12][1] = -6.f * kSH_C3[3] * yz;
    G[12][2] = kSH_C3[3] * (6.f * zz - 3.f * xx - 3.f * yy);
    G[13][0] = kSH_C3[4] * (4.f * zz - 3.f * xx - yy);  G[13][1] = -2.f * kSH_C3[4] * xy;
    G[13][2] = 8.f * kSH_C3[4] * xz;
    G[14][0] = 2.f * kSH_C3[5] * xz;             G[14][1] = -2.f * kSH_C3[5] * yz;
    G[14][2] = kSH_C3[5] * (xx - yy);
    G[15][0] = 3.f * kSH_C3[6] * (xx - yy);      G[15][1] = -6.f * kSH_C3[6] * xy;
    G[15][2] = 0.f;
  }
}

// The first 16 coefficients of one channel row: four 16-byte loads when the
// row is 16-byte aligned (K a multiple of 4 and an aligned base), else scalar.
__device__ __forceinline__ void load_row16(const float *s, bool vec, int nb, float (&v)[16]) {
  if (vec) {
    const float4 *s4 = reinterpret_cast<const float4 *>(s);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 f = q * 4 < nb ? __ldg(s4 + q) : make_float4(0.f, 0.f, 0.f, 0.f);
      v[4 * q] = f.x; v[4 * q + 1] = f.y; v[4 * q + 2] = f.z; v[4 * q + 3] = f.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = k < nb ? __ldg(s + k) : 0.f;
  }
}

__device__ __forceinline__ void unit_dir(const float *xyz, const float *campos, int p, float (&d)[3],
                                         float &len) {
  const float dx = xyz[3 * (size_t)p] - __ldg(campos), dy = xyz[3 * (size_t)p + 1] - __ldg(campos + 1),
              dz = xyz[3 * (size_t)p + 2] - __ldg(campos + 2);
  len = sqrtf(dx * dx + dy * dy + dz * dz);
  d[0] = dx / len;
  d[1] = dy / len;
  d[2] = dz / len;
}

__global__ void __launch_bounds__(SHC_THREADS)
sh_colors_fwd_kernel(int P, int deg, int K, const float *__restrict__ sh, const float *__restrict__ xyz,
                     const float *__restrict__ campos, float *__restrict__ colors) {
  const int p = blockIdx.x * SHC_THREADS + threadIdx.x;
  if (p >= P) return;
  float d[3], len;
  unit_dir(xyz, campos, p, d, len);
  float b[16], G[16][3];
  sh_basis<false>(d[0], d[1], d[2], deg, b, G);
  const int nb = (deg + 1) * (deg + 1);
  const bool vec = (K & 3) == 0 && (reinterpret_cast<uintptr_t>(sh) & 15) == 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[16];
    load_row16(sh + ((size_t)p * 3 + c) * K, vec, nb, v);
    float r = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < nb) r = fmaf(b[k], v[k], r);
    colors[3 * (size_t)p + c] = 1.f / (1.f + expf(-r));
  }
}

__global__ void __launch_bounds__(SHC_THREADS)
sh_colors_bwd_kernel(int P, int deg, int K, const float *__restrict__ sh, const float *__restrict__ xyz,
                     const float *__restrict__ campos, const float *__restrict__ dcolors,
                     float *__restrict__ dsh, float *__restrict__ dxyz) {
  const int p = blockIdx.x * SHC_THREADS + threadIdx.x;
  if (p >= P) return;
  float d[3], len;
  unit_dir(xyz, campos, p, d, len);
  float b[16], G[16][3];
  sh_basis<true>(d[0], d[1], d[2], deg, b, G);
  const int nb = (deg + 1) * (deg + 1);
  const bool vec = (K & 3) == 0 && (reinterpret_cast<uintptr_t>(sh) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(dsh) & 15) == 0;
  float gd[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[16];
    load_row16(sh + ((size_t)p * 3 + c) * K, vec, nb, v);
    float r = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < nb) r = fmaf(b[k], v[k], r);
    const float sg = 1.f / (1.f + expf(-r));
    const float dr = dcolors[3 * (size_t)p + c] * sg * (1.f - sg);
    float o[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      o[k] = k < nb ? dr * b[k] : 0.f;
      if (k < nb)
#pragma unroll
        for (int a = 0; a < 3; ++a) gd[a] = fmaf(dr * v[k], G[k][a], gd[a]);
    }
    float *out = dsh + ((size_t)p * 3 + c) * K;
    if (vec) {
      float4 *o4 = reinterpret_cast<float4 *>(out);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q * 4 < K) o4[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (k < K) out[k] = o[k];
    }
    for (int k = 16; k < K; ++k) out[k] = 0.f;
  }
  if (dxyz) {
    // through dir = D / |D|: dL/dD = (g - dir (dir . g)) / |D|
    const float dot = gd[0] * d[0] + gd[1] * d[1] + gd[2] * d[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) dxyz[3 * (size_t)p + a] = (gd[a] - d[a] * dot) / len;
  }
}

}  // namespace

}  // namespace dmgs

using namespace dmgs;
using dmgs_host::set_error;

extern "C" {

int dmgs_sh_colors_fwd(int32_t P, int32_t deg, int32_t K, const float *sh, const float *xyz,
                       const float *campos, float *colors, dmgs_stream_t stream) {
  if (P < 0 || deg < 0 || deg > 3 || K < (deg + 1) * (deg + 1) ||
      (P > 0 && (!sh || !xyz || !campos || !colors))) {
    set_error("sh_colors_fwd: invalid arguments (degree 0..3, K >= (deg+1)^2)");
    return DMGS_ERR_ARG;
  }
  if (P == 0) return DMGS_OK;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  DMGS_TIMED(K_SH_COLORS, s,
             dmgs_host::note_launch(), sh_colors_fwd_kernel<<<(P + SHC_THREADS - 1) / SHC_THREADS, SHC_THREADS, 0, s>>>(
                 P, deg, K, sh, xyz, campos, colors));
  DMGS_LAUNCH_CHECK("sh_colors_fwd");
  return DMGS_OK;
}

int dmgs_sh_colors_bwd(int32_t P, int32_t deg, int32_t K, const float *sh, const float *xyz,
                       const float *campos, const float *dL_dcolors, float *dL_dsh,
                       float *dL_dxyz, dmgs_stream_t stream) {
  if (P < 0 || deg < 0 || deg > 3 || K < (deg + 1) * (deg + 1) ||
      (P > 0 && (!sh || !xyz || !campos || !dL_dcolors || !dL_dsh))) {
    set_error("sh_colors_bwd: invalid arguments (degree 0..3, K >= (deg+1)^2)");
    return DMGS_ERR_ARG;
  }
  if (P == 0) return DMGS_OK;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  DMGS_TIMED(K_SH_COLORS, s,
             dmgs_host::note_launch(), sh_colors_bwd_kernel<<<(P + SHC_THREADS - 1) / SHC_THREADS, SHC_THREADS, 0, s>>>(
                 P, deg, K, sh, xyz, campos, dL_dcolors, dL_dsh, dL_dxyz));
  DMGS_LAUNCH_CHECK("sh_colors_bwd");
  return DMGS_OK;
}

}  // extern "C"
