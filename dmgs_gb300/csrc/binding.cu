// binding.cu — mesh -> Gaussian face binding and its adjoint.
//
// Stage-2 form: scene/gaussian_geo_model_mlp_flex.py:258-335 (renew_gaussian)
// and :370-385 (get_covariance_dyn), with the frame of geo/mesh_utils.py:43-57.
// The reference evaluates it as ~40 separate torch ops per step; here one
// thread handles one face (frame, affine triangle-space covariance, the G
// Gaussian means) and one thread one face in the adjoint.
//
// Stage-3 form: scene/gaussian_geo_model_finetune.py:396-421 (renew_gaussian)
// and :446-483 (get_scaling / get_rotation / get_rot_matrix).  The rotation
// matrix -> quaternion step uses Shepperd's method (pick the largest of
// trace, R00, R11, R22 to divide by), made sign-unique by a non-negative real
// part, then normalised — the same function the reference obtains from
// pytorch3d's matrix_to_quaternion followed by F.normalize.
#include "kernels.cuh"

namespace dmgs {

namespace {

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float norm(f3 a) { return sqrtf(dot(a, a)); }

constexpr float NRM_EPS = 1e-12f;  // torch.nn.functional.normalize default eps

// Faces whose vertex indices leave [0, V) are skipped (their outputs are
// left as written by the caller; no gradient is scattered).
__device__ __forceinline__ bool face_ok(int64_t i0, int64_t i1, int64_t i2, int V) {
  return i0 >= 0 && i1 >= 0 && i2 >= 0 && i0 < V && i1 < V && i2 < V;
}

__device__ __forceinline__ f3 load_v(const float *verts, int64_t i) {
  return mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
}

// unit(v) = v / max(|v|, eps) and its adjoint.
__device__ __forceinline__ f3 unit(f3 v, float &len) {
  len = norm(v);
  return (1.f / fmaxf(len, NRM_EPS)) * v;
}
__device__ __forceinline__ f3 unit_adj(f3 u, float len, f3 g) {
  if (len > NRM_EPS) return (1.f / len) * (g - dot(u, g) * u);
  return (1.f / NRM_EPS) * g;
}

struct Frame {
  f3 e01, e02, x, y, n, nraw, u;
  float len, nlen, ulen;
};

__device__ __forceinline__ Frame face_frame(f3 v0, f3 v1, f3 v2) {
  Frame F;
  F.e01 = v1 - v0;
  F.e02 = v2 - v0;
  F.x = unit(F.e01, F.len);
  F.nraw = cross(F.e01, F.e02);
  F.n = unit(F.nraw, F.nlen);
  F.u = cross(F.n, F.x);
  F.y = unit(F.u, F.ulen);
  return F;
}

// Adjoint of the frame: gradients w.r.t. x, y, n -> w.r.t. v0, v1, v2.
__device__ __forceinline__ void face_frame_adj(const Frame &F, f3 gx, f3 gy, f3 gn, f3 &g0,
                                               f3 &g1, f3 &g2) {
  const f3 gu = unit_adj(F.y, F.ulen, gy);
  gn = gn + cross(F.x, gu);       // u = n x x
  gx = gx + cross(gu, F.n);
  const f3 gnr = unit_adj(F.n, F.nlen, gn);
  f3 ge01 = cross(F.e02, gnr);    // nraw = e01 x e02
  f3 ge02 = cross(gnr, F.e01);
  ge01 = ge01 + unit_adj(F.x, F.len, gx);
  g1 = ge01;
  g2 = ge02;
  g0 = mk(0.f, 0.f, 0.f) - ge01 - ge02;
}

// Triangle-space factor L (3x3 row-major) of the stage-2 covariance.
__device__ __forceinline__ void tri_L(const Frame &F, float rad_base, float z_scale, int adaptive,
                                      float *L) {
  const float len = fmaxf(F.len, NRM_EPS);
  float m01 = 0.f, m11 = 1.f;
  if (adaptive) {
    const float Ax = dot(F.e02, F.x), Ay = dot(F.e02, F.y);
    const float Ex = len * 0.5f, Ey = len * 0.8660254037844386f;  // sqrt(3)/2
    m01 = (Ax - Ex) / Ey;
    m11 = Ay / Ey;
  }
  const float s = len * rad_base;
  L[0] = s;   L[1] = m01 * s; L[2] = 0.f;
  L[3] = 0.f; L[4] = m11 * s; L[5] = 0.f;
  L[6] = 0.f; L[7] = 0.f;     L[8] = z_scale;
}

__device__ __forceinline__ float bc_at(const DmgsFaceBinding &b, int f, int g, int k) {
  return b.bc_per_gaussian ? b.bc[((size_t)f * b.G + g) * 3 + k] : b.bc[g * 3 + k];
}

__global__ void bind_fwd_kernel(DmgsFaceBinding b, float *__restrict__ xyz,
                                float *__restrict__ cov, float *__restrict__ rot,
                                float *__restrict__ covL) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= b.F) return;
  const int64_t i0 = b.faces[3 * (size_t)f], i1 = b.faces[3 * (size_t)f + 1],
                i2 = b.faces[3 * (size_t)f + 2];
  if (!face_ok(i0, i1, i2, b.V)) return;
  const f3 v0 = load_v(b.verts, i0), v1 = load_v(b.verts, i1), v2 = load_v(b.verts, i2);
  const Frame F = face_frame(v0, v1, v2);
  float L[9];
  tri_L(F, b.rad_base, b.z_scale, b.adaptive_cov, L);
  // no scale factor: the real-scene variant's covariance, L unscaled
  // (scene/gaussian_geo_model_mlp_flex_colmap.py:494-512)
  const float k = b.scale_factor ? tanhf(b.scale_factor[0]) * b.max_scale : 1.f;
  const float R[9] = {F.x.x, F.y.x, F.n.x, F.x.y, F.y.y, F.n.y, F.x.z, F.y.z, F.n.z};
  float Mf[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Mf[i * 3 + j] = k * (R[i * 3] * L[j] + R[i * 3 + 1] * L[3 + j] + R[i * 3 + 2] * L[6 + j]);
  auto sig = [&](int i, int j) {
    return Mf[i * 3] * Mf[j * 3] + Mf[i * 3 + 1] * Mf[j * 3 + 1] + Mf[i * 3 + 2] * Mf[j * 3 + 2];
  };
  const float c[6] = {sig(0, 0), sig(0, 1), sig(0, 2), sig(1, 1), sig(1, 2), sig(2, 2)};
  if (rot)
    for (int i = 0; i < 9; ++i) rot[(size_t)f * 9 + i] = R[i];
  if (covL)
    for (int i = 0; i < 9; ++i) covL[(size_t)f * 9 + i] = L[i];
  for (int g = 0; g < b.G; ++g) {
    const float w0 = bc_at(b, f, g, 0), w1 = bc_at(b, f, g, 1), w2 = bc_at(b, f, g, 2);
    const size_t o = (size_t)f * b.G + g;
    if (xyz) {
      xyz[3 * o] = w0 * v0.x + w1 * v1.x + w2 * v2.x;
      xyz[3 * o + 1] = w0 * v0.y + w1 * v1.y + w2 * v2.y;
      xyz[3 * o + 2] = w0 * v0.z + w1 * v1.z + w2 * v2.z;
    }
    if (cov)
      for (int i = 0; i < 6; ++i) cov[6 * o + i] = c[i];
  }
}

__global__ void bind_bwd_kernel(DmgsFaceBinding b, const float *__restrict__ dxyz,
                                const float *__restrict__ dcov, float *__restrict__ dverts,
                                float *__restrict__ dsf) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  float dk_local = 0.f;
  if (f < b.F) {
    const int64_t i0 = b.faces[3 * (size_t)f], i1 = b.faces[3 * (size_t)f + 1],
                  i2 = b.faces[3 * (size_t)f + 2];
    if (face_ok(i0, i1, i2, b.V)) {
    const f3 v0 = load_v(b.verts, i0), v1 = load_v(b.verts, i1), v2 = load_v(b.verts, i2);
    f3 g0 = mk(0.f, 0.f, 0.f), g1 = g0, g2 = g0;
    float gc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int g = 0; g < b.G; ++g) {
      const size_t o = (size_t)f * b.G + g;
      if (dxyz) {
        const f3 d = mk(dxyz[3 * o], dxyz[3 * o + 1], dxyz[3 * o + 2]);
        g0 = g0 + bc_at(b, f, g, 0) * d;
        g1 = g1 + bc_at(b, f, g, 1) * d;
        g2 = g2 + bc_at(b, f, g, 2) * d;
      }
      if (dcov)
        for (int i = 0; i < 6; ++i) gc[i] += dcov[6 * o + i];
    }
    if (dcov) {
      const Frame F = face_frame(v0, v1, v2);
      float L[9];
      tri_L(F, b.rad_base, b.z_scale, b.adaptive_cov, L);
      const float th = b.scale_factor ? tanhf(b.scale_factor[0]) : 0.f;
      const float k = b.scale_factor ? th * b.max_scale : 1.f;
      const float R[9] = {F.x.x, F.y.x, F.n.x, F.x.y, F.y.y, F.n.y, F.x.z, F.y.z, F.n.z};
      float RL[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          RL[i * 3 + j] = R[i * 3] * L[j] + R[i * 3 + 1] * L[3 + j] + R[i * 3 + 2] * L[6 + j];
      // symmetric gradient of the packed covariance
      const float Gs[9] = {gc[0], 0.5f * gc[1], 0.5f * gc[2], 0.5f * gc[1], gc[3],
                           0.5f * gc[4], 0.5f * gc[2], 0.5f * gc[4], gc[5]};
      // dMf = 2 Gs Mf, Mf = k RL
      float dMf[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          dMf[i * 3 + j] = 2.f * k * (Gs[i * 3] * RL[j] + Gs[i * 3 + 1] * RL[3 + j] + Gs[i * 3 + 2] * RL[6 + j]);
      float dk = 0.f;
#pragma unroll
      for (int i = 0; i < 9; ++i) dk += dMf[i] * RL[i];
      if (b.scale_factor) dk_local = dk * b.max_scale * (1.f - th * th);
      // dR = dMf (k L)^T
      float dR[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          dR[i * 3 + j] = k * (dMf[i * 3] * L[j * 3] + dMf[i * 3 + 1] * L[j * 3 + 1] + dMf[i * 3 + 2] * L[j * 3 + 2]);
      const f3 gxv = mk(dR[0], dR[3], dR[6]);
      const f3 gyv = mk(dR[1], dR[4], dR[7]);
      const f3 gnv = mk(dR[2], dR[5], dR[8]);
      f3 h0, h1, h2;
      face_frame_adj(F, gxv, gyv, gnv, h0, h1, h2);
      g0 = g0 + h0; g1 = g1 + h1; g2 = g2 + h2;
    }
    atomicAdd(dverts + 3 * i0, g0.x); atomicAdd(dverts + 3 * i0 + 1, g0.y); atomicAdd(dverts + 3 * i0 + 2, g0.z);
    atomicAdd(dverts + 3 * i1, g1.x); atomicAdd(dverts + 3 * i1 + 1, g1.y); atomicAdd(dverts + 3 * i1 + 2, g1.z);
    atomicAdd(dverts + 3 * i2, g2.x); atomicAdd(dverts + 3 * i2 + 1, g2.y); atomicAdd(dverts + 3 * i2 + 2, g2.z);
    }
  }
  if (dsf) {
    const float s = warp_sum(dk_local);
    if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(dsf, s);
  }
}

// ----------------------------- stage 3 -----------------------------------

// Unit quaternion (w, x, y, z), w >= 0, of a rotation matrix (row-major),
// Shepperd's method, plus the unnormalised value and branch for the adjoint.
struct QuatOut { float q[4]; float raw[4]; int branch; };

__device__ __forceinline__ QuatOut mat_to_quat(const float *R) {
  QuatOut o;
  const float tr = R[0] + R[4] + R[8];
  float w, x, y, z;
  int br;
  if (tr >= R[0] && tr >= R[4] && tr >= R[8]) {
    br = 0;
    w = 0.5f * sqrtf(fmaxf(1.f + tr, 0.f));
    const float d = 0.25f / fmaxf(w, 0.05f);
    x = (R[7] - R[5]) * d; y = (R[2] - R[6]) * d; z = (R[3] - R[1]) * d;
  } else if (R[0] >= R[4] && R[0] >= R[8]) {
    br = 1;
    x = 0.5f * sqrtf(fmaxf(1.f + R[0] - R[4] - R[8], 0.f));
    const float d = 0.25f / fmaxf(x, 0.05f);
    w = (R[7] - R[5]) * d; y = (R[1] + R[3]) * d; z = (R[2] + R[6]) * d;
  } else if (R[4] >= R[8]) {
    br = 2;
    y = 0.5f * sqrtf(fmaxf(1.f - R[0] + R[4] - R[8], 0.f));
    const float d = 0.25f / fmaxf(y, 0.05f);
    w = (R[2] - R[6]) * d; x = (R[1] + R[3]) * d; z = (R[5] + R[7]) * d;
  } else {
    br = 3;
    z = 0.5f * sqrtf(fmaxf(1.f - R[0] - R[4] + R[8], 0.f));
    const float d = 0.25f / fmaxf(z, 0.05f);
    w = (R[3] - R[1]) * d; x = (R[2] + R[6]) * d; y = (R[5] + R[7]) * d;
  }
  const float sgn = w < 0.f ? -1.f : 1.f;
  o.raw[0] = sgn * w; o.raw[1] = sgn * x; o.raw[2] = sgn * y; o.raw[3] = sgn * z;
  const float n = sqrtf(o.raw[0] * o.raw[0] + o.raw[1] * o.raw[1] + o.raw[2] * o.raw[2] + o.raw[3] * o.raw[3]);
  const float inv = 1.f / fmaxf(n, NRM_EPS);
  for (int i = 0; i < 4; ++i) o.q[i] = o.raw[i] * inv;
  o.branch = br | (sgn < 0.f ? 4 : 0);
  return o;
}

// Adjoint of mat_to_quat: dq (w.r.t. the normalised output) -> dR.
__device__ __forceinline__ void mat_to_quat_adj(const float *R, const QuatOut &o, const float *dq,
                                                float *dR) {
  const float n = sqrtf(o.raw[0] * o.raw[0] + o.raw[1] * o.raw[1] + o.raw[2] * o.raw[2] + o.raw[3] * o.raw[3]);
  float dr[4];
  const float qd = o.q[0] * dq[0] + o.q[1] * dq[1] + o.q[2] * dq[2] + o.q[3] * dq[3];
  for (int i = 0; i < 4; ++i) dr[i] = n > NRM_EPS ? (dq[i] - o.q[i] * qd) / n : dq[i] / NRM_EPS;
  const float sgn = (o.branch & 4) ? -1.f : 1.f;
  for (int i = 0; i < 4; ++i) dr[i] *= sgn;  // gradient w.r.t. the pre-sign (w, x, y, z)
  for (int i = 0; i < 9; ++i) dR[i] = 0.f;
  const int br = o.branch & 3;
  // big = 0.5 sqrt(arg); the other three = (R[a] +/- R[b]) * 0.25 / max(big, 0.05)
  float big;
  int bi;
  float arg;
  float sgnd[9];
  for (int i = 0; i < 9; ++i) sgnd[i] = 0.f;
  if (br == 0) { arg = 1.f + R[0] + R[4] + R[8]; sgnd[0] = sgnd[4] = sgnd[8] = 1.f; bi = 0; }
  else if (br == 1) { arg = 1.f + R[0] - R[4] - R[8]; sgnd[0] = 1.f; sgnd[4] = sgnd[8] = -1.f; bi = 1; }
  else if (br == 2) { arg = 1.f - R[0] + R[4] - R[8]; sgnd[4] = 1.f; sgnd[0] = sgnd[8] = -1.f; bi = 2; }
  else { arg = 1.f - R[0] - R[4] + R[8]; sgnd[8] = 1.f; sgnd[0] = sgnd[4] = -1.f; bi = 3; }
  big = 0.5f * sqrtf(fmaxf(arg, 0.f));
  const bool clampd = big < 0.05f;
  const float den = fmaxf(big, 0.05f);
  const float d = 0.25f / den;
  // the three linear components: value_c = lin_c * d, lin_c = R[a] +/- R[b]
  int ia[3], ib[3], oc[3];
  float sb[3];
  if (br == 0) { oc[0] = 1; ia[0] = 7; ib[0] = 5; sb[0] = -1.f; oc[1] = 2; ia[1] = 2; ib[1] = 6; sb[1] = -1.f; oc[2] = 3; ia[2] = 3; ib[2] = 1; sb[2] = -1.f; }
  else if (br == 1) { oc[0] = 0; ia[0] = 7; ib[0] = 5; sb[0] = -1.f; oc[1] = 2; ia[1] = 1; ib[1] = 3; sb[1] = 1.f; oc[2] = 3; ia[2] = 2; ib[2] = 6; sb[2] = 1.f; }
  else if (br == 2) { oc[0] = 0; ia[0] = 2; ib[0] = 6; sb[0] = -1.f; oc[1] = 1; ia[1] = 1; ib[1] = 3; sb[1] = 1.f; oc[2] = 3; ia[2] = 5; ib[2] = 7; sb[2] = 1.f; }
  else { oc[0] = 0; ia[0] = 3; ib[0] = 1; sb[0] = -1.f; oc[1] = 1; ia[1] = 2; ib[1] = 6; sb[1] = 1.f; oc[2] = 2; ia[2] = 5; ib[2] = 7; sb[2] = 1.f; }
  float dd = 0.f;  // gradient w.r.t. d
  for (int c = 0; c < 3; ++c) {
    const float lin = R[ia[c]] + sb[c] * R[ib[c]];
    dR[ia[c]] += dr[oc[c]] * d;
    dR[ib[c]] += dr[oc[c]] * d * sb[c];
    dd += dr[oc[c]] * lin;
  }
  float dbig = dr[bi];
  if (!clampd) dbig += dd * (-0.25f / (den * den));
  // big = 0.5 sqrt(arg)  ->  dbig/darg = 0.25 / sqrt(arg) = 0.125 / big
  if (big > 0.f) {
    const float darg = dbig * 0.125f / big;
    for (int i = 0; i < 9; ++i) dR[i] += darg * sgnd[i];
  }
}

__global__ void bind3_fwd_kernel(DmgsFaceBinding3 b, float *__restrict__ xyz,
                                 float *__restrict__ scales, float *__restrict__ rots) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= b.F) return;
  const int64_t i0 = b.faces[3 * (size_t)f], i1 = b.faces[3 * (size_t)f + 1],
                i2 = b.faces[3 * (size_t)f + 2];
  if (!face_ok(i0, i1, i2, b.V)) return;
  const f3 v0 = load_v(b.verts, i0), v1 = load_v(b.verts, i1), v2 = load_v(b.verts, i2);
  const Frame F = face_frame(v0, v1, v2);
  const float Rw[9] = {F.x.x, F.y.x, F.n.x, F.x.y, F.y.y, F.n.y, F.x.z, F.y.z, F.n.z};
  for (int g = 0; g < b.G; ++g) {
    const size_t o = (size_t)f * b.G + g;
    const float w0 = b.bc[g * 3], w1 = b.bc[g * 3 + 1], w2 = b.bc[g * 3 + 2];
    if (xyz) {
      xyz[3 * o] = w0 * v0.x + w1 * v1.x + w2 * v2.x;
      xyz[3 * o + 1] = w0 * v0.y + w1 * v1.y + w2 * v2.y;
      xyz[3 * o + 2] = w0 * v0.z + w1 * v1.z + w2 * v2.z;
    }
    if (scales) {
      scales[3 * o] = expf(b.scaling2d[2 * o]);
      scales[3 * o + 1] = expf(b.scaling2d[2 * o + 1]);
      scales[3 * o + 2] = b.thin_z;
    }
    if (rots) {
      const float ra = b.rotation2d[2 * o], rb = b.rotation2d[2 * o + 1];
      const float cn = 1.f / fmaxf(sqrtf(ra * ra + rb * rb), NRM_EPS);
      const float a = ra * cn, s = rb * cn;
      // R = Rw * [[a,-s,0],[s,a,0],[0,0,1]]
      float R[9];
      for (int i = 0; i < 3; ++i) {
        R[i * 3 + 0] = Rw[i * 3] * a + Rw[i * 3 + 1] * s;
        R[i * 3 + 1] = -Rw[i * 3] * s + Rw[i * 3 + 1] * a;
        R[i * 3 + 2] = Rw[i * 3 + 2];
      }
      const QuatOut q = mat_to_quat(R);
      for (int i = 0; i < 4; ++i) rots[4 * o + i] = q.q[i];
    }
  }
}

__global__ void bind3_bwd_kernel(DmgsFaceBinding3 b, const float *__restrict__ dxyz,
                                 const float *__restrict__ dscales,
                                 const float *__restrict__ drots, float *__restrict__ dverts,
                                 float *__restrict__ dscaling, float *__restrict__ drot2d) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= b.F) return;
  const int64_t i0 = b.faces[3 * (size_t)f], i1 = b.faces[3 * (size_t)f + 1],
                i2 = b.faces[3 * (size_t)f + 2];
  if (!face_ok(i0, i1, i2, b.V)) return;
  const f3 v0 = load_v(b.verts, i0), v1 = load_v(b.verts, i1), v2 = load_v(b.verts, i2);
  const Frame F = face_frame(v0, v1, v2);
  const float Rw[9] = {F.x.x, F.y.x, F.n.x, F.x.y, F.y.y, F.n.y, F.x.z, F.y.z, F.n.z};
  f3 g0 = mk(0.f, 0.f, 0.f), g1 = g0, g2 = g0;
  float dRw[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int g = 0; g < b.G; ++g) {
    const size_t o = (size_t)f * b.G + g;
    if (dxyz) {
      const f3 d = mk(dxyz[3 * o], dxyz[3 * o + 1], dxyz[3 * o + 2]);
      g0 = g0 + b.bc[g * 3] * d;
      g1 = g1 + b.bc[g * 3 + 1] * d;
      g2 = g2 + b.bc[g * 3 + 2] * d;
    }
    if (dscaling) {
      dscaling[2 * o] = dscales ? dscales[3 * o] * expf(b.scaling2d[2 * o]) : 0.f;
      dscaling[2 * o + 1] = dscales ? dscales[3 * o + 1] * expf(b.scaling2d[2 * o + 1]) : 0.f;
    }
    float dra = 0.f, drb = 0.f;
    if (drots) {
      const float ra = b.rotation2d[2 * o], rb = b.rotation2d[2 * o + 1];
      const float clen = sqrtf(ra * ra + rb * rb);
      const float cn = 1.f / fmaxf(clen, NRM_EPS);
      const float a = ra * cn, s = rb * cn;
      float R[9];
      for (int i = 0; i < 3; ++i) {
        R[i * 3 + 0] = Rw[i * 3] * a + Rw[i * 3 + 1] * s;
        R[i * 3 + 1] = -Rw[i * 3] * s + Rw[i * 3 + 1] * a;
        R[i * 3 + 2] = Rw[i * 3 + 2];
      }
      const QuatOut q = mat_to_quat(R);
      const float dq[4] = {drots[4 * o], drots[4 * o + 1], drots[4 * o + 2], drots[4 * o + 3]};
      float dR[9];
      mat_to_quat_adj(R, q, dq, dR);
      float da = 0.f, ds = 0.f;
      for (int i = 0; i < 3; ++i) {
        dRw[i * 3] += dR[i * 3] * a - dR[i * 3 + 1] * s;
        dRw[i * 3 + 1] += dR[i * 3] * s + dR[i * 3 + 1] * a;
        dRw[i * 3 + 2] += dR[i * 3 + 2];
        da += dR[i * 3] * Rw[i * 3] + dR[i * 3 + 1] * Rw[i * 3 + 1];
        ds += dR[i * 3] * Rw[i * 3 + 1] - dR[i * 3 + 1] * Rw[i * 3];
      }
      // (a, s) = unit(ra, rb)
      if (clen > NRM_EPS) {
        const float dot_ = a * da + s * ds;
        dra = (da - a * dot_) / clen;
        drb = (ds - s * dot_) / clen;
      } else {
        dra = da / NRM_EPS;
        drb = ds / NRM_EPS;
      }
    }
    if (drot2d) { drot2d[2 * o] = dra; drot2d[2 * o + 1] = drb; }
  }
  if (drots) {
    f3 h0, h1, h2;
    face_frame_adj(F, mk(dRw[0], dRw[3], dRw[6]), mk(dRw[1], dRw[4], dRw[7]),
                   mk(dRw[2], dRw[5], dRw[8]), h0, h1, h2);
    g0 = g0 + h0; g1 = g1 + h1; g2 = g2 + h2;
  }
  atomicAdd(dverts + 3 * i0, g0.x); atomicAdd(dverts + 3 * i0 + 1, g0.y); atomicAdd(dverts + 3 * i0 + 2, g0.z);
  atomicAdd(dverts + 3 * i1, g1.x); atomicAdd(dverts + 3 * i1 + 1, g1.y); atomicAdd(dverts + 3 * i1 + 2, g1.z);
  atomicAdd(dverts + 3 * i2, g2.x); atomicAdd(dverts + 3 * i2 + 1, g2.y); atomicAdd(dverts + 3 * i2 + 2, g2.z);
}

}  // namespace

int launch_bind_fwd(const DmgsFaceBinding &b, float *xyz, float *cov, float *rot, float *covL,
                    cudaStream_t s) {
  if (b.F <= 0) return DMGS_OK;
  DMGS_TIMED(K_BIND_FWD, s, dmgs_host::note_launch(), bind_fwd_kernel<<<(b.F + 255) / 256, 256, 0, s>>>(b, xyz, cov, rot, covL));
  DMGS_LAUNCH_CHECK("bind_fwd_kernel");
  return DMGS_OK;
}

int launch_bind_bwd(const DmgsFaceBinding &b, const float *dxyz, const float *dcov,
                    float *dverts, float *dsf, cudaStream_t s) {
  DMGS_CUDA(cudaMemsetAsync(dverts, 0, (size_t)b.V * 3 * 4, s));
  if (dsf) DMGS_CUDA(cudaMemsetAsync(dsf, 0, 4, s));
  if (b.F <= 0) return DMGS_OK;
  DMGS_TIMED(K_BIND_BWD, s, dmgs_host::note_launch(), bind_bwd_kernel<<<(b.F + 255) / 256, 256, 0, s>>>(b, dxyz, dcov, dverts, dsf));
  DMGS_LAUNCH_CHECK("bind_bwd_kernel");
  return DMGS_OK;
}

int launch_bind3_fwd(const DmgsFaceBinding3 &b, float *xyz, float *scales, float *rots,
                     cudaStream_t s) {
  if (b.F <= 0) return DMGS_OK;
  DMGS_TIMED(K_BIND3_FWD, s, dmgs_host::note_launch(), bind3_fwd_kernel<<<(b.F + 255) / 256, 256, 0, s>>>(b, xyz, scales, rots));
  DMGS_LAUNCH_CHECK("bind3_fwd_kernel");
  return DMGS_OK;
}

int launch_bind3_bwd(const DmgsFaceBinding3 &b, const float *dxyz, const float *dscales,
                     const float *drots, float *dverts, float *dscaling, float *drot2d,
                     cudaStream_t s) {
  DMGS_CUDA(cudaMemsetAsync(dverts, 0, (size_t)b.V * 3 * 4, s));
  if (b.F <= 0) return DMGS_OK;
  DMGS_TIMED(K_BIND3_BWD, s, dmgs_host::note_launch(), bind3_bwd_kernel<<<(b.F + 255) / 256, 256, 0, s>>>(b, dxyz, dscales, drots, dverts, dscaling,
                                                     drot2d));
  DMGS_LAUNCH_CHECK("bind3_bwd_kernel");
  return DMGS_OK;
}

namespace {

constexpr int CULL_BLOCK = 256;

// Face f is in the frustum when its centroid (the mean of its vertices),
// taken through the full projection (row-vector convention of the stored
// matrix: p_j = sum_i c_i M[i][j] + M[3][j]), has |x/w|, |y/w|, |z/w| < 1.05
// with w = p_3 + 1e-6 > 0 — the stage-3 test of
// scene/gaussian_geo_model_finetune.py:33-48.  A face with a vertex index
// outside [0, V) is not kept.
__device__ __forceinline__ bool face_in_frustum(const float *__restrict__ verts, int V,
                                                const int64_t *__restrict__ faces, int f,
                                                const float *__restrict__ M) {
  int64_t vi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vi[k] = faces[3 * (size_t)f + k];
    if (vi[k] < 0 || vi[k] >= V) return false;
  }
  float c[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int a = 0; a < 3; ++a) c[a] += verts[3 * vi[k] + a];
#pragma unroll
  for (int a = 0; a < 3; ++a) c[a] = c[a] / 3.f;
  float p[4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
    p[j] = c[0] * __ldg(M + j) + c[1] * __ldg(M + 4 + j) + c[2] * __ldg(M + 8 + j) + __ldg(M + 12 + j);
  const float w = p[3] + 1e-6f;
  return w > 0.f && fabsf(p[0] / w) < 1.05f && fabsf(p[1] / w) < 1.05f && fabsf(p[2] / w) < 1.05f;
}

// The test per face, the per-block count of kept faces (for the
// order-preserving compaction).
__global__ void __launch_bounds__(CULL_BLOCK)
face_cull_test_kernel(const float *__restrict__ verts, int V, const int64_t *__restrict__ faces,
                      int F, const float *__restrict__ M, uint8_t *__restrict__ mask,
                      uint32_t *__restrict__ blkcnt) {
  const int f = blockIdx.x * CULL_BLOCK + threadIdx.x;
  const bool keep = f < F && face_in_frustum(verts, V, faces, f, M);
  if (f < F && mask) mask[f] = keep ? 1 : 0;
  const int n = __syncthreads_count(keep);
  if (threadIdx.x == 0) blkcnt[blockIdx.x] = (uint32_t)n;
}

// Kept face indices at their block's scanned offset, in face order (the
// test is recomputed: cheaper than a round trip of a flag through memory).
__global__ void __launch_bounds__(CULL_BLOCK)
face_cull_compact_kernel(const float *__restrict__ verts, int V, const int64_t *__restrict__ faces,
                         int F, const float *__restrict__ M, const uint32_t *__restrict__ blkoff,
                         int32_t *__restrict__ kept) {
  __shared__ uint32_t wcount[CULL_BLOCK / 32];
  const int f = blockIdx.x * CULL_BLOCK + threadIdx.x;
  const bool keep = f < F && face_in_frustum(verts, V, faces, f, M);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(0xffffffffu, keep);
  if (lane == 0) wcount[wid] = __popc(b);
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < wid; ++w) before += wcount[w];
  if (keep) {
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    kept[blkoff[blockIdx.x] + before + __popc(b & lt)] = f;
  }
}

// Vertex frustum mask of the real-scene stage 2 (in_frustum,
// scene/gaussian_geo_model_mlp_flex_colmap.py:31-76): the grid vertex
// shifted by half a cube edge (the shift folded into the matrix's last row,
// as the reference does) taken through full_proj (row-vector convention,
// stored [4,4]); kept when w = p.w + 1e-6 > 0 and p.xyz / w lies inside the
// view's screen piece widened by 0.05 (the whole screen, a half or a
// quarter).  Optional and_mask ([N] bytes) is ANDed in.
__global__ void __launch_bounds__(256)
vertex_frustum_kernel(const float *__restrict__ verts, int N, const float *__restrict__ M, float half,
                      int piece_id, int n_piece, const uint8_t *__restrict__ and_mask,
                      uint8_t *__restrict__ out) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= N) return;
  const float x = verts[3 * (size_t)i], y = verts[3 * (size_t)i + 1], z = verts[3 * (size_t)i + 2];
  float p[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float m0 = __ldg(M + j), m1 = __ldg(M + 4 + j), m2 = __ldg(M + 8 + j);
    const float c = __fadd_rn(__ldg(M + 12 + j),
                              __fadd_rn(__fadd_rn(__fmul_rn(m0, half), __fmul_rn(m1, half)),
                                        __fmul_rn(m2, half)));
    p[j] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, m0), __fmul_rn(y, m1)), __fmul_rn(z, m2)), c);
  }
  const float w = __fadd_rn(p[3], 1e-6f);
  const float q[3] = {__fdiv_rn(p[0], w), __fdiv_rn(p[1], w), __fdiv_rn(p[2], w)};
  bool keep;
  if (piece_id < 0) {
    keep = fabsf(q[0]) < 1.05f && fabsf(q[1]) < 1.05f && fabsf(q[2]) < 1.05f;
  } else {
    // screen piece [lo, hi] in x and y (z spans [-1, 1]), widened by 0.05
    float lx = -1.f, hx = 1.f, ly = -1.f, hy = 1.f;
    if (n_piece == 2) {
      if (piece_id == 0) hx = 0.f; else lx = 0.f;
    } else {
      if (piece_id & 1) lx = 0.f; else hx = 0.f;
      if (piece_id & 2) ly = 0.f; else hy = 0.f;
    }
    keep = q[0] > __fsub_rn(lx, 0.05f) && q[1] > __fsub_rn(ly, 0.05f) && q[2] > -1.05f &&
           q[0] < __fadd_rn(hx, 0.05f) && q[1] < __fadd_rn(hy, 0.05f) && q[2] < 1.05f;
  }
  keep = keep && w > 0.f;
  if (and_mask) keep = keep && and_mask[i] != 0;
  out[i] = keep ? 1 : 0;
}

}  // namespace

int launch_vertex_frustum(const float *verts, int N, const float *full_proj, float cube_len,
                          int piece_id, int n_piece, const uint8_t *and_mask, uint8_t *out,
                          cudaStream_t s) {
  if (N <= 0) return DMGS_OK;
  DMGS_TIMED(K_FACE_CULL, s, dmgs_host::note_launch(), vertex_frustum_kernel<<<(N + 255) / 256, 256, 0, s>>>(
      verts, N, full_proj, 0.5f * cube_len, piece_id, n_piece, and_mask, out));
  DMGS_LAUNCH_CHECK("vertex_frustum_kernel");
  return DMGS_OK;
}

size_t face_cull_scratch_bytes(int F) {
  const uint32_t nb = (uint32_t)((F + CULL_BLOCK - 1) / CULL_BLOCK);
  return align_up((size_t)nb * 4 + 4, 256) + scan_part_words(nb) * 4;
}

int launch_face_cull(const float *verts, int V, const int64_t *faces, int F,
                     const float *full_proj, uint8_t *face_mask, int32_t *kept, int32_t *num_kept,
                     char *scratch, cudaStream_t s) {
  if (F <= 0) {
    DMGS_CUDA(cudaMemsetAsync(num_kept, 0, 4, s));
    return DMGS_OK;
  }
  const uint32_t nb = (uint32_t)((F + CULL_BLOCK - 1) / CULL_BLOCK);
  uint32_t *blkcnt = reinterpret_cast<uint32_t *>(scratch);
  uint32_t *part = reinterpret_cast<uint32_t *>(scratch + align_up((size_t)nb * 4 + 4, 256));
  DMGS_TIMED(K_FACE_CULL, s, {
    dmgs_host::note_launch(), face_cull_test_kernel<<<nb, CULL_BLOCK, 0, s>>>(verts, V, faces, F, full_proj, face_mask, blkcnt);
    int r = launch_scan1(blkcnt, nb, part, reinterpret_cast<uint32_t *>(num_kept), nullptr, s);
    if (r != DMGS_OK) return r;
    dmgs_host::note_launch(), face_cull_compact_kernel<<<nb, CULL_BLOCK, 0, s>>>(verts, V, faces, F, full_proj, blkcnt, kept);
  });
  DMGS_LAUNCH_CHECK("face_cull");
  return DMGS_OK;
}

}  // namespace dmgs
