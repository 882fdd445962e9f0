// preprocess_bwd.cu — per-Gaussian adjoint of the forward geometry.
//
// Input: the per-Gaussian 2D gradients the blend adjoint accumulated
// (dL/d NDC mean, dL/d conic (a, b, c) with b the off-diagonal scalar,
// dL/d opacity, dL/d rgb).  Output: gradients w.r.t. every forward input.
//
// Chain (derived here, conventions of the reference adjoint):
//   conic = inverse(cov2D)           -> dL/dA, dL/dB, dL/dC (cov2D = [[A,B],[B,C]])
//   cov2D = T Sigma T^T, T = J W     -> dL/dSigma = T^T Gs T, dL/dT = 2 Gs T Sigma
//   J(t), t = W m + t0               -> dL/dt with the 1.3 tan(fov) clamp: zero
//                                        gradient through a clamped coordinate,
//                                        the clamped value held constant
//   ndc = hom.xy / (hom.w + 1e-7)    -> dL/dm
//   rgb = max(0, SH(dir) + 0.5)      -> dL/dsh, dL/dm through dir = unit(m - campos)
//   Sigma = (R S)(R S)^T             -> dL/dscale, dL/dquaternion (unnormalised)
// Culled Gaussians (radius 0, empty rectangle in the geometry state) get
// zeros in every output.  Results are staged in shared memory and each
// block stores its contiguous slice of every output array with coalesced
// writes (most Gaussians are culled: their outputs are zero-filled at full
// bandwidth instead of by strided per-thread stores).
#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int BWD_BLOCK = 128;
constexpr int SP = BWD_BLOCK + 1;  // shared-memory row pitch of the output slots

// Shared-memory output slots of one block: element k of Gaussian g of a
// field lives at field[k * SP + g].  Lanes writing element k of different
// Gaussians hit consecutive banks, and the pitch of BWD_BLOCK + 1 keeps the
// Gaussian-major reads of the stores (consecutive k of one g) conflict-free.
struct Slots {
  float *m2, *col, *op, *m3, *cov, *sc, *rot, *sh;
};

__host__ __device__ constexpr size_t slot_floats(int M) { return (size_t)(23 + 3 * M) * SP; }

__device__ __forceinline__ Slots make_slots(float *sm) {
  Slots S;
  S.m2 = sm;
  S.col = S.m2 + 3 * SP;
  S.op = S.col + 3 * SP;
  S.m3 = S.op + SP;
  S.cov = S.m3 + 3 * SP;
  S.sc = S.cov + 6 * SP;
  S.rot = S.sc + 3 * SP;
  S.sh = S.rot + 4 * SP;
  return S;
}

// Calls term(k, b_k, db_k/dx, db_k/dy, db_k/dz) for every SH basis function
// of degree <= D at the unit direction (x, y, z) (the real SH basis with the
// PlenOctree constants of utils/sh_utils.py:25-110), k in coefficient order.
template <typename F>
__device__ __forceinline__ void for_each_sh_term(int D, float x, float y, float z, F &&term) {
  term(0, kSH_C0, 0.f, 0.f, 0.f);
  if (D > 0) {
    term(1, -kSH_C1 * y, 0.f, -kSH_C1, 0.f);
    term(2, kSH_C1 * z, 0.f, 0.f, kSH_C1);
    term(3, -kSH_C1 * x, -kSH_C1, 0.f, 0.f);
    if (D > 1) {
      const float xx = x * x, yy = y * y, zz = z * z;
      term(4, kSH_C2[0] * x * y, kSH_C2[0] * y, kSH_C2[0] * x, 0.f);
      term(5, kSH_C2[1] * y * z, 0.f, kSH_C2[1] * z, kSH_C2[1] * y);
      term(6, kSH_C2[2] * (2.f * zz - xx - yy), -2.f * kSH_C2[2] * x, -2.f * kSH_C2[2] * y, 4.f * kSH_C2[2] * z);
      term(7, kSH_C2[3] * x * z, kSH_C2[3] * z, 0.f, kSH_C2[3] * x);
      term(8, kSH_C2[4] * (xx - yy), 2.f * kSH_C2[4] * x, -2.f * kSH_C2[4] * y, 0.f);
      if (D > 2) {
        term(9, kSH_C3[0] * y * (3.f * xx - yy), 6.f * kSH_C3[0] * x * y, kSH_C3[0] * (3.f * xx - 3.f * yy), 0.f);
        term(10, kSH_C3[1] * x * y * z, kSH_C3[1] * y * z, kSH_C3[1] * x * z, kSH_C3[1] * x * y);
        term(11, kSH_C3[2] * y * (4.f * zz - xx - yy), -2.f * kSH_C3[2] * x * y,
             kSH_C3[2] * (4.f * zz - xx - 3.f * yy), 8.f * kSH_C3[2] * y * z);
        term(12, kSH_C3[3] * z * (2.f * zz - 3.f * xx - 3.f * yy), -6.f * kSH_C3[3] * x * z,
             -6.f * kSH_C3[3] * y * z, kSH_C3[3] * (6.f * zz - 3.f * xx - 3.f * yy));
        term(13, kSH_C3[4] * x * (4.f * zz - xx - yy), kSH_C3[4] * (4.f * zz - 3.f * xx - yy),
             -2.f * kSH_C3[4] * x * y, 8.f * kSH_C3[4] * x * z);
        term(14, kSH_C3[5] * z * (xx - yy), 2.f * kSH_C3[5] * x * z, -2.f * kSH_C3[5] * y * z,
             kSH_C3[5] * (xx - yy));
        term(15, kSH_C3[6] * x * (xx - 3.f * yy), kSH_C3[6] * (3.f * xx - 3.f * yy),
             -6.f * kSH_C3[6] * x * y, 0.f);
      }
    }
  }
}

// ACC: add into the slots (several views of one Gaussian, possibly from
// several threads at once: a shared-memory atomic add); else assign.
template <bool ACC>
__device__ __forceinline__ void put(float &slot, float v) {
  if (ACC) atomicAdd(&slot, v);
  else slot = v;
}

// SH: also the SH adjoint (dL/dsh and the direction term of dL/dmean);
// without it the caller handles the SH colour's adjoint.
template <bool ACC, bool SH = true>
__device__ __forceinline__ void
preprocess_bwd_one(int idx, int t, const ViewParams &vp, const float *__restrict__ viewm_g,
                   const float *__restrict__ projm_g, const float *__restrict__ campos_g, int M,
                   const float *__restrict__ means, const float *__restrict__ shs,
                   const float *__restrict__ scales, const float *__restrict__ rots,
                   const float *__restrict__ cov3D, const uint8_t *__restrict__ flags,
                   const float *__restrict__ gacc, const DmgsGrads &out, const Slots &S_) {
  const int nsh = (vp.D + 1) * (vp.D + 1);
  const float4 ga = reinterpret_cast<const float4 *>(gacc)[3 * idx];
  const float4 gb = reinterpret_cast<const float4 *>(gacc)[3 * idx + 1];
  const float gblue = gacc[12 * idx + 8];
  const float dndc_x = ga.x, dndc_y = ga.y;
  const float dca = ga.z, dcb = ga.w, dcc = gb.x;
  const float dop = gb.y;
  float drgb[3] = {gb.z, gb.w, gblue};

  if (out.dL_dmeans2D && !ACC) { S_.m2[t] = dndc_x; S_.m2[SP + t] = dndc_y; S_.m2[2 * SP + t] = 0.f; }
  if (out.dL_dopacity) put<ACC>(S_.op[t], dop);
  if (out.dL_dcolors) { put<ACC>(S_.col[t], drgb[0]); put<ACC>(S_.col[SP + t], drgb[1]); put<ACC>(S_.col[2 * SP + t], drgb[2]); }

  float V[16], Pm[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) { V[i] = viewm_g[i]; Pm[i] = projm_g[i]; }  // global or shared
  const float mx = means[3 * idx], my = means[3 * idx + 1], mz = means[3 * idx + 2];

  // --- recompute the forward quantities ---------------------------------
  const float tx0 = V[0] * mx + V[4] * my + V[8] * mz + V[12];
  const float ty0 = V[1] * mx + V[5] * my + V[9] * mz + V[13];
  const float tz = V[2] * mx + V[6] * my + V[10] * mz + V[14];

  float S[6];
  float R[9], sc[3];
  const bool from_sr = (cov3D == nullptr);
  float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!from_sr) {
#pragma unroll
    for (int i = 0; i < 6; ++i) S[i] = cov3D[6 * idx + i];
  } else {
    q = reinterpret_cast<const float4 *>(rots)[idx];
    const float r = q.x, x = q.y, y = q.z, z = q.w;
    R[0] = 1.f - 2.f * (y * y + z * z); R[1] = 2.f * (x * y - r * z); R[2] = 2.f * (x * z + r * y);
    R[3] = 2.f * (x * y + r * z); R[4] = 1.f - 2.f * (x * x + z * z); R[5] = 2.f * (y * z - r * x);
    R[6] = 2.f * (x * z - r * y); R[7] = 2.f * (y * z + r * x); R[8] = 1.f - 2.f * (x * x + y * y);
    sc[0] = vp.scale_modifier * scales[3 * idx];
    sc[1] = vp.scale_modifier * scales[3 * idx + 1];
    sc[2] = vp.scale_modifier * scales[3 * idx + 2];
    float Mm[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Mm[i * 3 + j] = R[i * 3 + j] * sc[j];
    auto sig = [&](int i, int k) {
      return Mm[i * 3] * Mm[k * 3] + Mm[i * 3 + 1] * Mm[k * 3 + 1] + Mm[i * 3 + 2] * Mm[k * 3 + 2];
    };
    S[0] = sig(0, 0); S[1] = sig(0, 1); S[2] = sig(0, 2); S[3] = sig(1, 1); S[4] = sig(1, 2); S[5] = sig(2, 2);
  }
  const float Sg[9] = {S[0], S[1], S[2], S[1], S[3], S[4], S[2], S[4], S[5]};

  const float limx = 1.3f * vp.tanfovx, limy = 1.3f * vp.tanfovy;
  const float txtz = tx0 / tz, tytz = ty0 / tz;
  const float tx = fminf(limx, fmaxf(-limx, txtz)) * tz;
  const float ty = fminf(limy, fmaxf(-limy, tytz)) * tz;
  const float xmul = (txtz < -limx || txtz > limx) ? 0.f : 1.f;
  const float ymul = (tytz < -limy || tytz > limy) ? 0.f : 1.f;
  const float inv = 1.f / tz, inv2 = inv * inv, inv3 = inv2 * inv;
  const float J00 = vp.fx * inv, J02 = -vp.fx * tx * inv2;
  const float J11 = vp.fy * inv, J12 = -vp.fy * ty * inv2;
  // W_ij = V[i + 4j]
  float T[2][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T[0][j] = J00 * V[4 * j + 0] + J02 * V[4 * j + 2];
    T[1][j] = J11 * V[4 * j + 1] + J12 * V[4 * j + 2];
  }
  float TS[2][3];  // T Sigma
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      TS[a][j] = T[a][0] * Sg[j] + T[a][1] * Sg[3 + j] + T[a][2] * Sg[6 + j];
  const float A = TS[0][0] * T[0][0] + TS[0][1] * T[0][1] + TS[0][2] * T[0][2] + 0.3f;
  const float Bc = TS[0][0] * T[1][0] + TS[0][1] * T[1][1] + TS[0][2] * T[1][2];
  const float C = TS[1][0] * T[1][0] + TS[1][1] * T[1][1] + TS[1][2] * T[1][2] + 0.3f;

  // --- conic -> cov2D ----------------------------------------------------
  const float det = A * C - Bc * Bc;
  const float det2 = det * det;
  float dA = 0.f, dB = 0.f, dC = 0.f;
  if (det2 != 0.f) {
    const float id2 = 1.f / det2;
    dA = id2 * (-C * C * dca + Bc * C * dcb - Bc * Bc * dcc);
    dB = id2 * (2.f * Bc * C * dca - (A * C + Bc * Bc) * dcb + 2.f * A * Bc * dcc);
    dC = id2 * (-Bc * Bc * dca + A * Bc * dcb - A * A * dcc);
  }
  // Gs = [[dA, dB/2], [dB/2, dC]]
  const float Gs00 = dA, Gs01 = 0.5f * dB, Gs11 = dC;

  // dL/dSigma_sym = T^T Gs T
  float GT[2][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    GT[0][j] = Gs00 * T[0][j] + Gs01 * T[1][j];
    GT[1][j] = Gs01 * T[0][j] + Gs11 * T[1][j];
  }
  float dS[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dS[i * 3 + j] = T[0][i] * GT[0][j] + T[1][i] * GT[1][j];
  if (out.dL_dcov3D) {
    float *o = S_.cov + t;
    put<ACC>(o[0], dS[0]); put<ACC>(o[SP], 2.f * dS[1]); put<ACC>(o[2 * SP], 2.f * dS[2]);
    put<ACC>(o[3 * SP], dS[4]); put<ACC>(o[4 * SP], 2.f * dS[5]); put<ACC>(o[5 * SP], dS[8]);
  }

  // dL/dT = 2 Gs T Sigma
  float dT[2][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    dT[0][j] = 2.f * (Gs00 * TS[0][j] + Gs01 * TS[1][j]);
    dT[1][j] = 2.f * (Gs01 * TS[0][j] + Gs11 * TS[1][j]);
  }
  // dL/dJ = dL/dT W^T  (W_bk = V[b + 4k])
  float dJ00 = 0.f, dJ02 = 0.f, dJ11 = 0.f, dJ12 = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dJ00 += dT[0][k] * V[4 * k + 0];
    dJ02 += dT[0][k] * V[4 * k + 2];
    dJ11 += dT[1][k] * V[4 * k + 1];
    dJ12 += dT[1][k] * V[4 * k + 2];
  }
  const float dtx = xmul * (-vp.fx * inv2) * dJ02;
  const float dty = ymul * (-vp.fy * inv2) * dJ12;
  const float dtz = -vp.fx * inv2 * dJ00 - vp.fy * inv2 * dJ11 +
                    2.f * vp.fx * tx * inv3 * dJ02 + 2.f * vp.fy * ty * inv3 * dJ12;
  float dm[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) dm[k] = V[4 * k] * dtx + V[4 * k + 1] * dty + V[4 * k + 2] * dtz;

  // --- projected mean ----------------------------------------------------
  {
    const float hx = Pm[0] * mx + Pm[4] * my + Pm[8] * mz + Pm[12];
    const float hy = Pm[1] * mx + Pm[5] * my + Pm[9] * mz + Pm[13];
    const float hw = Pm[3] * mx + Pm[7] * my + Pm[11] * mz + Pm[15];
    const float mw = 1.f / (hw + 1e-7f);
    const float mw2 = mw * mw;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float jx = Pm[4 * k] * mw - hx * mw2 * Pm[4 * k + 3];
      const float jy = Pm[4 * k + 1] * mw - hy * mw2 * Pm[4 * k + 3];
      dm[k] += dndc_x * jx + dndc_y * jy;
    }
  }

  // --- SH colour ---------------------------------------------------------
  if (SH && shs != nullptr) {
    const uint8_t cl = flags[idx];
    if (cl & 1) drgb[0] = 0.f;
    if (cl & 2) drgb[1] = 0.f;
    if (cl & 4) drgb[2] = 0.f;
    const float vx_ = mx - campos_g[0], vy_ = my - campos_g[1], vz_ = mz - campos_g[2];
    const float len = sqrtf(vx_ * vx_ + vy_ * vy_ + vz_ * vz_);
    const float il = 1.f / len;
    const float x = vx_ * il, y = vy_ * il, z = vz_ * il;
    const float *sh = shs + (size_t)idx * M * 3;
    float *dsh = out.dL_dsh ? S_.sh + t : nullptr;
    // basis value b_k and its partial derivatives (bx, by, bz) w.r.t. the
    // unnormalised-direction components x, y, z
    float gdx = 0.f, gdy = 0.f, gdz = 0.f;
    auto term = [&](int k, float b, float bx, float by, float bz) {
      const float s0 = sh[3 * k], s1 = sh[3 * k + 1], s2 = sh[3 * k + 2];
      if (dsh) { put<ACC>(dsh[3 * k * SP], b * drgb[0]); put<ACC>(dsh[(3 * k + 1) * SP], b * drgb[1]); put<ACC>(dsh[(3 * k + 2) * SP], b * drgb[2]); }
      const float dot = s0 * drgb[0] + s1 * drgb[1] + s2 * drgb[2];
      gdx += bx * dot; gdy += by * dot; gdz += bz * dot;
    };
    for_each_sh_term(vp.D, x, y, z, term);
    if (dsh)
      if (!ACC) for (int i = 3 * nsh; i < 3 * M; ++i) dsh[i * SP] = 0.f;
    // d unit(v)/dv . g = (g - u (u . g)) / |v|
    const float ug = x * gdx + y * gdy + z * gdz;
    dm[0] += (gdx - x * ug) * il;
    dm[1] += (gdy - y * ug) * il;
    dm[2] += (gdz - z * ug) * il;
  }

  if (out.dL_dmeans3D) {
    put<ACC>(S_.m3[t], dm[0]);
    put<ACC>(S_.m3[SP + t], dm[1]);
    put<ACC>(S_.m3[2 * SP + t], dm[2]);
  }

  // --- scale / rotation --------------------------------------------------
  if (from_sr && (out.dL_dscales || out.dL_drotations)) {
    // dL/dM = 2 dS M,  M = R diag(sc)
    float Mm[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Mm[i * 3 + j] = R[i * 3 + j] * sc[j];
    float dM[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        dM[i * 3 + j] = 2.f * (dS[i * 3] * Mm[j] + dS[i * 3 + 1] * Mm[3 + j] + dS[i * 3 + 2] * Mm[6 + j]);
    if (out.dL_dscales) {
#pragma unroll
      for (int j = 0; j < 3; ++j)
        put<ACC>(S_.sc[j * SP + t],
                 vp.scale_modifier * (dM[j] * R[j] + dM[3 + j] * R[3 + j] + dM[6 + j] * R[6 + j]));
    }
    if (out.dL_drotations) {
      float G[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) G[i * 3 + j] = dM[i * 3 + j] * sc[j];
      const float r = q.x, x = q.y, y = q.z, z = q.w;
      const float dr = 2.f * (-z * G[1] + y * G[2] + z * G[3] - x * G[5] - y * G[6] + x * G[7]);
      const float dx = 2.f * (y * G[1] + z * G[2] + y * G[3] - 2.f * x * G[4] - r * G[5] + z * G[6] +
                              r * G[7] - 2.f * x * G[8]);
      const float dy = 2.f * (-2.f * y * G[0] + x * G[1] + r * G[2] + x * G[3] + z * G[5] - r * G[6] +
                              z * G[7] - 2.f * y * G[8]);
      const float dz = 2.f * (-2.f * z * G[0] - r * G[1] + x * G[2] + r * G[3] - 2.f * z * G[4] +
                              y * G[5] + x * G[6] + y * G[7]);
      { put<ACC>(S_.rot[t], dr); put<ACC>(S_.rot[SP + t], dx); put<ACC>(S_.rot[2 * SP + t], dy); put<ACC>(S_.rot[3 * SP + t], dz); }
    }
  }
}


// Stores the block's contiguous slice of one output array (n elements per
// Gaussian): element i of the slice is element i % n of Gaussian i / n;
// Gaussians culled in every view get zeros (their slots are never written).
__device__ __forceinline__ void store_slice(float *dst, const float *src, int n, int start,
                                            int nvalid, const uint32_t *vmask) {
  if (!dst) return;
  float *d = dst + (size_t)start * n;
  const int cnt = nvalid * n;
  // ceil(2^32 / n) for n >= 2; i / n = umulhi(i, magic) exactly for i, n < 2^16
  const uint32_t magic = n > 1 ? (uint32_t)(0xffffffffull / (uint32_t)n) + 1u : 0u;
  auto gauss = [&](int i) { return n > 1 ? (int)__umulhi((uint32_t)i, magic) : i; };
  auto vis = [&](int g) { return (vmask[g >> 5] >> (g & 31)) & 1u; };
  if ((n & 3) == 0 && (cnt & 3) == 0 && (reinterpret_cast<uintptr_t>(d) & 15) == 0) {
    // whole float4s never straddle two Gaussians when n % 4 == 0
    float4 *d4 = reinterpret_cast<float4 *>(d);
    for (int i = threadIdx.x; i < (cnt >> 2); i += BWD_BLOCK) {
      const int g = gauss(i << 2), k = (i << 2) - g * n;
      const float *s = src + k * SP + g;
      d4[i] = vis(g) ? make_float4(s[0], s[SP], s[2 * SP], s[3 * SP]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  } else {
    for (int i = threadIdx.x; i < cnt; i += BWD_BLOCK) {
      const int g = gauss(i), k = i - g * n;
      d[i] = vis(g) ? src[k * SP + g] : 0.f;
    }
  }
}

__global__ void __launch_bounds__(BWD_BLOCK)
preprocess_bwd_kernel(ViewParams vp, const float *__restrict__ viewm_g,
                      const float *__restrict__ projm_g, const float *__restrict__ campos_g,
                      int P, int M, const float *__restrict__ means,
                      const float *__restrict__ shs, const float *__restrict__ scales,
                      const float *__restrict__ rots, const float *__restrict__ cov3D,
                      const uint8_t *__restrict__ flags, const float *__restrict__ gacc,
                      DmgsGrads out) {
  extern __shared__ float sm[];
  __shared__ uint32_t vmask[BWD_BLOCK / 32];
  const int B = BWD_BLOCK;
  const int t = threadIdx.x;
  const int start = blockIdx.x * B;
  const int idx = start + t;
  const Slots S_ = make_slots(sm);
  const bool vis = idx < P && (flags[idx] & FLAG_VISIBLE);
  const uint32_t bal = __ballot_sync(0xffffffffu, vis);
  if ((t & 31) == 0) vmask[t >> 5] = bal;
  if (vis)
    preprocess_bwd_one<false>(idx, t, vp, viewm_g, projm_g, campos_g, M, means, shs, scales, rots,
                              cov3D, flags, gacc, out, S_);
  __syncthreads();
  const int nvalid = min(B, P - start);
  store_slice(out.dL_dmeans2D, S_.m2, 3, start, nvalid, vmask);
  store_slice(out.dL_dcolors, S_.col, 3, start, nvalid, vmask);
  store_slice(out.dL_dopacity, S_.op, 1, start, nvalid, vmask);
  store_slice(out.dL_dmeans3D, S_.m3, 3, start, nvalid, vmask);
  store_slice(out.dL_dcov3D, S_.cov, 6, start, nvalid, vmask);
  store_slice(out.dL_dscales, S_.sc, 3, start, nvalid, vmask);
  store_slice(out.dL_drotations, S_.rot, 4, start, nvalid, vmask);
  store_slice(out.dL_dsh, S_.sh, 3 * M, start, nvalid, vmask);
}

// Multi-view adjoint: the gradients of all views of a batch, summed.  A
// Gaussian is visible in few of the views, so a thread per Gaussian looping
// over the views would leave most lanes idle for the geometric part (the
// longest).  Instead the block lists its (Gaussian, view) pairs — thread t's
// Gaussian contributes one pair per view it is visible in, placed by a
// block-wide scan — and the threads take the pairs in turn, adding each
// view's geometric gradients (mean through the projection and the EWA
// Jacobian, scale and rotation or covariance, opacity, colour: 14 values)
// into the Gaussian's shared-memory sums with atomic adds.  The SH part is
// linear in each view's colour gradient: the Gaussian's own thread then runs
// it over its views with the 3M SH-gradient sums in registers, adds each
// view's direction term to the mean gradient and writes every output of its
// Gaussian (zeros when it is culled in every view).  The per-view
// screen-space gradient and the densification statistics (optional
// outputs) are handled by the same thread: all views' visibility bytes and
// 2D gradients are loaded at once (independent loads), then written out,
// zero where the Gaussian is not visible.
constexpr int ACC_SLOTS = 14;  // colour 3, opacity 1, mean 3, scale 3 + rotation 4 (or covariance 6)

__global__ void __launch_bounds__(BWD_BLOCK)
preprocess_bwd_batched_kernel(const BatchViews bv, int P, int M, const float *__restrict__ means,
                              const float *__restrict__ shs, const float *__restrict__ scales,
                              const float *__restrict__ rots, const float *__restrict__ cov3D,
                              DmgsGrads out, int want_xy, float *__restrict__ densify_accum,
                              float *__restrict__ densify_count) {
  __shared__ float acc[ACC_SLOTS * SP];
  __shared__ uint32_t wsum[BWD_BLOCK / 32];
  __shared__ uint16_t pairs[BWD_BLOCK * MAX_BATCH_VIEWS];
  const int B = BWD_BLOCK;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int start = blockIdx.x * B;
  const int idx = start + t;
  Slots S_;
  S_.m2 = nullptr;
  S_.col = acc;
  S_.op = acc + 3 * SP;
  S_.m3 = acc + 4 * SP;
  S_.sc = acc + 7 * SP;
  S_.rot = acc + 10 * SP;
  S_.cov = acc + 7 * SP;  // covariance mode has no scale/rotation
  S_.sh = nullptr;
  for (int i = t; i < ACC_SLOTS * SP; i += B) acc[i] = 0.f;
  // per-view constants in shared memory: the pair loop below reads them
  // with a different view per lane, which from the kernel parameters would
  // be serialised constant-bank loads
  __shared__ ViewParams s_vp[MAX_BATCH_VIEWS];
  __shared__ float s_mat[MAX_BATCH_VIEWS][36];  // view matrix, projection matrix, camera centre
  __shared__ const float *s_gacc[MAX_BATCH_VIEWS];
  __shared__ const uint8_t *s_flags[MAX_BATCH_VIEWS];
  if (t < bv.nviews) {
    s_vp[t] = bv.v[t].vp;
    s_gacc[t] = bv.v[t].gacc;
    s_flags[t] = bv.v[t].flags;
  }
  for (int i = t; i < bv.nviews * 35; i += B) {
    const int v = i / 35, k = i - v * 35;
    const BatchView &W = bv.v[v];
    s_mat[v][k] = k < 16 ? __ldg(W.viewm + k) : (k < 32 ? __ldg(W.projm + k - 16) : __ldg(W.campos + k - 32));
  }
  uint32_t vm = 0u;
  uint8_t fl[MAX_BATCH_VIEWS];
  if (idx < P) {
#pragma unroll
    for (int v = 0; v < MAX_BATCH_VIEWS; ++v) fl[v] = v < bv.nviews ? bv.v[v].flags[idx] : 0u;
#pragma unroll
    for (int v = 0; v < MAX_BATCH_VIEWS; ++v) vm |= ((fl[v] & FLAG_VISIBLE) ? 1u : 0u) << v;
    if (want_xy) {
      float2 g2[MAX_BATCH_VIEWS];
#pragma unroll
      for (int v = 0; v < MAX_BATCH_VIEWS; ++v)
        g2[v] = ((vm >> v) & 1u) ? *reinterpret_cast<const float2 *>(bv.v[v].gacc + 12 * (size_t)idx)
                                 : make_float2(0.f, 0.f);
      float nsum = 0.f;
#pragma unroll
      for (int v = 0; v < MAX_BATCH_VIEWS; ++v) {
        if (v >= bv.nviews) break;
        float *d2 = bv.v[v].dL_dmeans2D;
        if (d2) {
          d2[3 * (size_t)idx] = g2[v].x;
          d2[3 * (size_t)idx + 1] = g2[v].y;
          d2[3 * (size_t)idx + 2] = 0.f;
        }
        if ((vm >> v) & 1u) nsum += sqrtf(g2[v].x * g2[v].x + g2[v].y * g2[v].y);
      }
      if (densify_accum && vm) {
        densify_accum[idx] += nsum;
        densify_count[idx] += (float)__popc(vm);
      }
    }
  }
  // block-wide exclusive scan of the pair counts
  const uint32_t cnt = __popc(vm);
  uint32_t inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  uint32_t off = inc - cnt, total = 0;
#pragma unroll
  for (int w = 0; w < BWD_BLOCK / 32; ++w) {
    off += w < wid ? wsum[w] : 0u;
    total += wsum[w];
  }
  for (uint32_t m = vm; m; m &= m - 1) pairs[off++] = (uint16_t)((t << 4) | (__ffs(m) - 1));
  __syncthreads();
  for (uint32_t i = t; i < total; i += B) {
    const uint32_t pr = pairs[i];
    const int gl = (int)(pr >> 4), v = (int)(pr & 15u);
    const ViewParams vp = s_vp[v];
    preprocess_bwd_one<true, false>(start + gl, gl, vp, s_mat[v], s_mat[v] + 16, s_mat[v] + 32, M,
                                    means, shs, scales, rots, cov3D, s_flags[v], s_gacc[v], out, S_);
  }
  __syncthreads();
  if (idx >= P) return;

  // --- the Gaussian's own thread: SH over its views, then every output ---
  float dm[3] = {S_.m3[t], S_.m3[SP + t], S_.m3[2 * SP + t]};
  const bool want_sh = shs != nullptr && (out.dL_dsh != nullptr || out.dL_dmeans3D != nullptr);
  float dsh[48];
#pragma unroll
  for (int i = 0; i < 48; ++i) dsh[i] = 0.f;
  if (want_sh && vm) {
    const float mx = means[3 * (size_t)idx], my = means[3 * (size_t)idx + 1],
                mz = means[3 * (size_t)idx + 2];
    const float *sh = shs + (size_t)idx * M * 3;
    for (uint32_t m = vm; m; m &= m - 1) {
      const int v = __ffs(m) - 1;
      const float *gv = s_gacc[v] + 12 * (size_t)idx;
      float drgb[3] = {gv[6], gv[7], gv[8]};
      const uint32_t clamp = s_flags[v][idx];
      if (clamp & 1) drgb[0] = 0.f;
      if (clamp & 2) drgb[1] = 0.f;
      if (clamp & 4) drgb[2] = 0.f;
      const float *cp = s_mat[v] + 32;
      const float vx_ = mx - cp[0], vy_ = my - cp[1], vz_ = mz - cp[2];
      const float len = sqrtf(vx_ * vx_ + vy_ * vy_ + vz_ * vz_);
      const float il = 1.f / len;
      const float x = vx_ * il, y = vy_ * il, z = vz_ * il;
      float gdx = 0.f, gdy = 0.f, gdz = 0.f;
      for_each_sh_term(s_vp[v].D, x, y, z, [&](int k, float b, float bx, float by, float bz) {
        dsh[3 * k] += b * drgb[0];
        dsh[3 * k + 1] += b * drgb[1];
        dsh[3 * k + 2] += b * drgb[2];
        const float dot = sh[3 * k] * drgb[0] + sh[3 * k + 1] * drgb[1] + sh[3 * k + 2] * drgb[2];
        gdx += bx * dot; gdy += by * dot; gdz += bz * dot;
      });
      const float ug = x * gdx + y * gdy + z * gdz;
      dm[0] += (gdx - x * ug) * il;
      dm[1] += (gdy - y * ug) * il;
      dm[2] += (gdz - z * ug) * il;
    }
  }
  const size_t i3 = 3 * (size_t)idx;
  if (out.dL_dcolors) {
    out.dL_dcolors[i3] = S_.col[t]; out.dL_dcolors[i3 + 1] = S_.col[SP + t]; out.dL_dcolors[i3 + 2] = S_.col[2 * SP + t];
  }
  if (out.dL_dopacity) out.dL_dopacity[idx] = S_.op[t];
  if (out.dL_dmeans3D) {
    out.dL_dmeans3D[i3] = dm[0]; out.dL_dmeans3D[i3 + 1] = dm[1]; out.dL_dmeans3D[i3 + 2] = dm[2];
  }
  if (out.dL_dcov3D) {
#pragma unroll
    for (int k = 0; k < 6; ++k) out.dL_dcov3D[6 * (size_t)idx + k] = S_.cov[k * SP + t];
  }
  if (out.dL_dscales) {
    out.dL_dscales[i3] = S_.sc[t]; out.dL_dscales[i3 + 1] = S_.sc[SP + t]; out.dL_dscales[i3 + 2] = S_.sc[2 * SP + t];
  }
  if (out.dL_drotations)
    reinterpret_cast<float4 *>(out.dL_drotations)[idx] =
        make_float4(S_.rot[t], S_.rot[SP + t], S_.rot[2 * SP + t], S_.rot[3 * SP + t]);
  if (out.dL_dsh) {
    // the Gaussian's 3M contiguous floats: coefficients above degree 3 (or
    // the active degree) stay zero
    float *d = out.dL_dsh + (size_t)idx * M * 3;
    const int n = 3 * M;
    if (n >= 48 && (n & 3) == 0 && (reinterpret_cast<uintptr_t>(d) & 15) == 0) {
      float4 *d4 = reinterpret_cast<float4 *>(d);
#pragma unroll
      for (int i = 0; i < 12; ++i) d4[i] = make_float4(dsh[4 * i], dsh[4 * i + 1], dsh[4 * i + 2], dsh[4 * i + 3]);
      for (int i = 12; i < (n >> 2); ++i) d4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
#pragma unroll
      for (int i = 0; i < 48; ++i)
        if (i < n) d[i] = dsh[i];
      for (int i = 48; i < n; ++i) d[i] = 0.f;
    }
  }
}

}  // namespace

int launch_preprocess_bwd(const ViewParams &vp, const float *viewm, const float *projm,
                          const float *campos, const GaussianPtrs &g, const GeomLayout &L,
                          const char *geom, const float *gacc, const DmgsGrads &out,
                          cudaStream_t s) {
  if (g.P <= 0) return DMGS_OK;
  const size_t smem = slot_floats(g.M) * 4;
  if (smem > 200 * 1024) {
    dmgs_host::set_error("preprocess_bwd: %d SH coefficients per Gaussian exceed shared memory", g.M);
    return DMGS_ERR_ARG;
  }
  if (int r = dmgs_host::raise_smem_limit((const void *)preprocess_bwd_kernel, smem)) return r;
  DMGS_TIMED(K_PREPROCESS_BWD, s, dmgs_host::note_launch(), preprocess_bwd_kernel<<<(g.P + BWD_BLOCK - 1) / BWD_BLOCK, BWD_BLOCK, smem, s>>>(
      vp, viewm, projm, campos, g.P, g.M, g.means3D, g.shs, g.scales, g.rotations, g.cov3D,
      reinterpret_cast<const uint8_t *>(geom + L.flags), gacc, out));
  DMGS_LAUNCH_CHECK("preprocess_bwd_kernel");
  return DMGS_OK;
}

}  // namespace dmgs

namespace dmgs {

int launch_preprocess_bwd_batched(const BatchViews &bv, const GaussianPtrs &g, const DmgsGrads &out,
                                  float *densify_accum, float *densify_count, cudaStream_t s) {
  if (g.P <= 0) return DMGS_OK;
  int want_xy = densify_accum != nullptr;
  for (int v = 0; v < bv.nviews; ++v) want_xy |= bv.v[v].dL_dmeans2D != nullptr;
  DMGS_TIMED(K_BATCH_PREPROCESS_BWD, s,
             dmgs_host::note_launch(), preprocess_bwd_batched_kernel<<<(g.P + BWD_BLOCK - 1) / BWD_BLOCK, BWD_BLOCK, 0, s>>>(
                 bv, g.P, g.M, g.means3D, g.shs, g.scales, g.rotations, g.cov3D, out, want_xy,
                 densify_accum, densify_count));
  DMGS_LAUNCH_CHECK("preprocess_bwd_batched_kernel");
  return DMGS_OK;
}

}  // namespace dmgs
