// preprocess.cu — per-Gaussian forward geometry (EWA projection, conic,
// radius, tile rectangle, SH colour) and the per-tile instance counts.
//
// Semantics follow the 3DGS preprocess the reference calls through
// GaussianRasterizer (gaussian_renderer/__init__.py:86-94); the rotation and
// covariance packing conventions are those of utils/general_utils.py:64-110
// and the SH polynomial that of utils/sh_utils.py:75-99.
//
// Design: one thread per Gaussian.  The integer-determining chain (view z,
// NDC position, 2D covariance, radius, rectangle) uses explicitly rounded
// IEEE ops so that it is reproducible on the CPU.  Each block also records
// how many of its Gaussians are visible, for the order-preserving
// compaction that starts the binning (binning.cu).
#include "kernels.cuh"

namespace dmgs {

namespace {

__device__ __forceinline__ void load_mat(const float *__restrict__ p, float *m) {
#pragma unroll
  for (int i = 0; i < 16; ++i) m[i] = __ldg(p + i);
}

// Sigma = R diag(s)^2 R^T in the fixed op order of the CPU oracle.
__device__ __forceinline__ void cov3d_scale_rot(float sx, float sy, float sz, float4 q,
                                                float *cov) {
  const float r = q.x, x = q.y, y = q.z, z = q.w;
  float R[9];
  R[0] = sub(1.f, mul(2.f, add(mul(y, y), mul(z, z))));
  R[1] = mul(2.f, sub(mul(x, y), mul(r, z)));
  R[2] = mul(2.f, add(mul(x, z), mul(r, y)));
  R[3] = mul(2.f, add(mul(x, y), mul(r, z)));
  R[4] = sub(1.f, mul(2.f, add(mul(x, x), mul(z, z))));
  R[5] = mul(2.f, sub(mul(y, z), mul(r, x)));
  R[6] = mul(2.f, sub(mul(x, z), mul(r, y)));
  R[7] = mul(2.f, add(mul(y, z), mul(r, x)));
  R[8] = sub(1.f, mul(2.f, add(mul(x, x), mul(y, y))));
  float Mm[9];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Mm[i * 3 + 0] = mul(R[i * 3 + 0], sx);
    Mm[i * 3 + 1] = mul(R[i * 3 + 1], sy);
    Mm[i * 3 + 2] = mul(R[i * 3 + 2], sz);
  }
  auto sig = [&](int i, int k) {
    return add(add(mul(Mm[i * 3], Mm[k * 3]), mul(Mm[i * 3 + 1], Mm[k * 3 + 1])),
               mul(Mm[i * 3 + 2], Mm[k * 3 + 2]));
  };
  cov[0] = sig(0, 0); cov[1] = sig(0, 1); cov[2] = sig(0, 2);
  cov[3] = sig(1, 1); cov[4] = sig(1, 2); cov[5] = sig(2, 2);
}

__device__ __forceinline__ int trunc_sat(float v) { return __float2int_rz(v); }

// One Gaussian; returns true when it is visible (radius > 0, non-empty
// tile rectangle).
__device__ __forceinline__ bool
preprocess_one(int idx, const ViewParams &vp, const float *__restrict__ viewm_g,
               const float *__restrict__ projm_g, const float *__restrict__ campos_g, int M,
               const float *__restrict__ means, const float *__restrict__ opac,
               const float *__restrict__ shs, const float *__restrict__ colors,
               const float *__restrict__ scales, const float *__restrict__ rots,
               const float *__restrict__ cov3D, int32_t *__restrict__ radii,
               float4 *__restrict__ feat, uint8_t *__restrict__ flags,
               uint32_t *__restrict__ counters) {

  float V[16], Pm[16];
  load_mat(viewm_g, V);
  load_mat(projm_g, Pm);

  const float x = __ldg(means + 3 * idx), y = __ldg(means + 3 * idx + 1),
              z = __ldg(means + 3 * idx + 2);
  const float vx = add(add(add(mul(V[0], x), mul(V[4], y)), mul(V[8], z)), V[12]);
  const float vy = add(add(add(mul(V[1], x), mul(V[5], y)), mul(V[9], z)), V[13]);
  const float vz = add(add(add(mul(V[2], x), mul(V[6], y)), mul(V[10], z)), V[14]);

  auto cull = [&]() {
    radii[idx] = 0;
    flags[idx] = 0;
    feat[3 * idx + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
  };
  if (!(vz > 0.2f)) {
    if (vp.prefiltered) atomicOr(counters, ST_PREFILTER);
    cull();
    return false;
  }
  const float hx = add(add(add(mul(Pm[0], x), mul(Pm[4], y)), mul(Pm[8], z)), Pm[12]);
  const float hy = add(add(add(mul(Pm[1], x), mul(Pm[5], y)), mul(Pm[9], z)), Pm[13]);
  const float hw = add(add(add(mul(Pm[3], x), mul(Pm[7], y)), mul(Pm[11], z)), Pm[15]);
  const float pw = dvd(1.f, add(hw, 1e-7f));
  const float ndcx = mul(hx, pw), ndcy = mul(hy, pw);
  const float Wf = (float)vp.W, Hf = (float)vp.H;
  const float px = mul(sub(mul(add(ndcx, 1.f), Wf), 1.f), 0.5f);
  const float py = mul(sub(mul(add(ndcy, 1.f), Hf), 1.f), 0.5f);

  float S[6];
  if (cov3D != nullptr) {
#pragma unroll
    for (int i = 0; i < 6; ++i) S[i] = __ldg(cov3D + 6 * idx + i);
  } else {
    const float mod = vp.scale_modifier;
    const float sx = mul(__ldg(scales + 3 * idx), mod);
    const float sy = mul(__ldg(scales + 3 * idx + 1), mod);
    const float sz = mul(__ldg(scales + 3 * idx + 2), mod);
    const float4 q = __ldg(reinterpret_cast<const float4 *>(rots) + idx);
    cov3d_scale_rot(sx, sy, sz, q, S);
  }

  // EWA: cov2D = (J W) Sigma (J W)^T with the Jacobian evaluated at the
  // position clamped to 1.3x the field of view.
  const float limx = mul(1.3f, vp.tanfovx), limy = mul(1.3f, vp.tanfovy);
  const float txtz = dvd(vx, vz), tytz = dvd(vy, vz);
  const float tx = mul(fminf(limx, fmaxf(-limx, txtz)), vz);
  const float ty = mul(fminf(limy, fmaxf(-limy, tytz)), vz);
  const float vz2 = mul(vz, vz);
  const float J00 = dvd(vp.fx, vz);
  const float J02 = dvd(-mul(vp.fx, tx), vz2);
  const float J11 = dvd(vp.fy, vz);
  const float J12 = dvd(-mul(vp.fy, ty), vz2);
  float T0[3], T1[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T0[j] = add(mul(J00, V[4 * j + 0]), mul(J02, V[4 * j + 2]));
    T1[j] = add(mul(J11, V[4 * j + 1]), mul(J12, V[4 * j + 2]));
  }
  const float Sg[9] = {S[0], S[1], S[2], S[1], S[3], S[4], S[2], S[4], S[5]};
  float U0[3], U1[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    U0[j] = add(add(mul(T0[0], Sg[j]), mul(T0[1], Sg[3 + j])), mul(T0[2], Sg[6 + j]));
    U1[j] = add(add(mul(T1[0], Sg[j]), mul(T1[1], Sg[3 + j])), mul(T1[2], Sg[6 + j]));
  }
  float c00 = add(add(mul(U0[0], T0[0]), mul(U0[1], T0[1])), mul(U0[2], T0[2]));
  const float c01 = add(add(mul(U0[0], T1[0]), mul(U0[1], T1[1])), mul(U0[2], T1[2]));
  float c11 = add(add(mul(U1[0], T1[0]), mul(U1[1], T1[1])), mul(U1[2], T1[2]));
  c00 = add(c00, 0.3f);
  c11 = add(c11, 0.3f);
  const float det = sub(mul(c00, c11), mul(c01, c01));
  if (det == 0.f) { cull(); return false; }
  const float det_inv = dvd(1.f, det);
  const float ca = mul(c11, det_inv), cb = mul(-c01, det_inv), cc = mul(c00, det_inv);
  const float mid = mul(0.5f, add(c00, c11));
  const float disc = fmaxf(0.1f, sub(mul(mid, mid), det));
  const float sq = __fsqrt_rn(disc);
  const float l1 = add(mid, sq), l2 = sub(mid, sq);
  const int rad = trunc_sat(ceilf(mul(3.f, __fsqrt_rn(fmaxf(l1, l2)))));
  if (rad <= 0) { cull(); return false; }
  const float r = (float)rad;
  const int x0 = min(vp.gx, max(0, trunc_sat(dvd(sub(px, r), (float)TILE))));
  const int y0 = min(vp.gy, max(0, trunc_sat(dvd(sub(py, r), (float)TILE))));
  const int x1 = min(vp.gx, max(0, trunc_sat(dvd(add(add(px, r), (float)(TILE - 1)), (float)TILE))));
  const int y1 = min(vp.gy, max(0, trunc_sat(dvd(add(add(py, r), (float)(TILE - 1)), (float)TILE))));
  if ((x1 - x0) * (y1 - y0) == 0) { cull(); return false; }

  // Colour: precomputed, or SH (degree <= 3) at the view direction, +0.5,
  // clamped at 0 with the clamp recorded for the adjoint.
  float cr, cg, cbl;
  uint8_t clampbits = 0;
  if (colors != nullptr) {
    cr = __ldg(colors + 3 * idx); cg = __ldg(colors + 3 * idx + 1); cbl = __ldg(colors + 3 * idx + 2);
  } else {
    const float *sh = shs + (size_t)idx * M * 3;
    float dx = x - __ldg(campos_g), dy = y - __ldg(campos_g + 1), dz = z - __ldg(campos_g + 2);
    const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
    dx *= inv; dy *= inv; dz *= inv;
    float b[16];
    b[0] = kSH_C0;
    int nb = 1;
    if (vp.D > 0) {
      b[1] = -kSH_C1 * dy; b[2] = kSH_C1 * dz; b[3] = -kSH_C1 * dx;
      nb = 4;
      if (vp.D > 1) {
        const float xx = dx * dx, yy = dy * dy, zz = dz * dz;
        b[4] = kSH_C2[0] * dx * dy;
        b[5] = kSH_C2[1] * dy * dz;
        b[6] = kSH_C2[2] * (2.f * zz - xx - yy);
        b[7] = kSH_C2[3] * dx * dz;
        b[8] = kSH_C2[4] * (xx - yy);
        nb = 9;
        if (vp.D > 2) {
          b[9] = kSH_C3[0] * dy * (3.f * xx - yy);
          b[10] = kSH_C3[1] * dx * dy * dz;
          b[11] = kSH_C3[2] * dy * (4.f * zz - xx - yy);
          b[12] = kSH_C3[3] * dz * (2.f * zz - 3.f * xx - 3.f * yy);
          b[13] = kSH_C3[4] * dx * (4.f * zz - xx - yy);
          b[14] = kSH_C3[5] * dz * (xx - yy);
          b[15] = kSH_C3[6] * dx * (xx - 3.f * yy);
          nb = 16;
        }
      }
    }
    float rr = 0.f, gg = 0.f, bb = 0.f;
    for (int k = 0; k < nb; ++k) {
      rr += b[k] * __ldg(sh + 3 * k);
      gg += b[k] * __ldg(sh + 3 * k + 1);
      bb += b[k] * __ldg(sh + 3 * k + 2);
    }
    rr += 0.5f; gg += 0.5f; bb += 0.5f;
    clampbits = (rr < 0.f ? 1 : 0) | (gg < 0.f ? 2 : 0) | (bb < 0.f ? 4 : 0);
    cr = fmaxf(rr, 0.f); cg = fmaxf(gg, 0.f); cbl = fmaxf(bb, 0.f);
  }
  flags[idx] = FLAG_VISIBLE | clampbits;

  const float o = __ldg(opac + idx);
  radii[idx] = rad;
  feat[3 * idx + 0] = make_float4(px, py, ca, cb);
  feat[3 * idx + 1] = make_float4(cc, o, cr, cg);
  feat[3 * idx + 2] = make_float4(cbl, vz, __uint_as_float(pack_u16x2(x0, y0)),
                                  __uint_as_float(pack_u16x2(x1, y1)));

  return true;
}

__global__ void __launch_bounds__(PRE_BLOCK)
preprocess_kernel(ViewParams vp, const float *__restrict__ viewm_g,
                  const float *__restrict__ projm_g, const float *__restrict__ campos_g,
                  int P, int M, const float *__restrict__ means,
                  const float *__restrict__ opac, const float *__restrict__ shs,
                  const float *__restrict__ colors, const float *__restrict__ scales,
                  const float *__restrict__ rots, const float *__restrict__ cov3D,
                  int32_t *__restrict__ radii, float4 *__restrict__ feat,
                  uint8_t *__restrict__ flags, uint32_t *__restrict__ blkcnt,
                  uint32_t *__restrict__ counters) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const bool vis = idx < P &&
                   preprocess_one(idx, vp, viewm_g, projm_g, campos_g, M, means, opac, shs, colors,
                                  scales, rots, cov3D, radii, feat, flags, counters);
  const int nvis = __syncthreads_count(vis);
  if (threadIdx.x == 0) blkcnt[blockIdx.x] = (uint32_t)nvis;
}


// Multi-view preprocess: one thread per Gaussian computes its geometry for
// every view of the batch (the inputs are read from DRAM once; the repeated
// per-view reads hit L1), writing each view's records and per-block visible
// counts.
__global__ void __launch_bounds__(PRE_BLOCK)
preprocess_batched_kernel(const BatchViews bv, int P, int M, const float *__restrict__ means,
                          const float *__restrict__ opac, const float *__restrict__ shs,
                          const float *__restrict__ colors, const float *__restrict__ scales,
                          const float *__restrict__ rots, const float *__restrict__ cov3D) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  for (int v = 0; v < bv.nviews; ++v) {
    const BatchView &V = bv.v[v];
    const bool vis = idx < P &&
                     preprocess_one(idx, V.vp, V.viewm, V.projm, V.campos, M, means, opac, shs,
                                    colors, scales, rots, cov3D, V.radii, V.feat, V.flags,
                                    V.counters);
    const int nvis = __syncthreads_count(vis);
    if (threadIdx.x == 0) V.blkcnt[blockIdx.x] = (uint32_t)nvis;
  }
}

__global__ void mark_visible_kernel(int P, const float *__restrict__ means,
                                    const float *__restrict__ viewm_g,
                                    uint8_t *__restrict__ present) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= P) return;
  const float x = means[3 * idx], y = means[3 * idx + 1], z = means[3 * idx + 2];
  const float vz = add(add(add(mul(__ldg(viewm_g + 2), x), mul(__ldg(viewm_g + 6), y)),
                           mul(__ldg(viewm_g + 10), z)), __ldg(viewm_g + 14));
  present[idx] = vz > 0.2f ? 1 : 0;
}

}  // namespace

int launch_preprocess(const ViewParams &vp, const float *viewm, const float *projm,
                      const float *campos, const GaussianPtrs &g, int32_t *radii,
                      const GeomLayout &L, char *geom, cudaStream_t s) {
  float4 *feat = reinterpret_cast<float4 *>(geom + L.feat);
  uint8_t *flags = reinterpret_cast<uint8_t *>(geom + L.flags);
  uint32_t *blkcnt = reinterpret_cast<uint32_t *>(geom + L.blkcnt);
  uint32_t *counters = reinterpret_cast<uint32_t *>(geom + L.counters);
  DMGS_CUDA(cudaMemsetAsync(counters, 0, CI_WORDS * 4, s));
  if (g.P > 0) {
    const int blocks = L.nb_pre;
    DMGS_TIMED(K_PREPROCESS, s, dmgs_host::note_launch(), preprocess_kernel<<<blocks, PRE_BLOCK, 0, s>>>(vp, viewm, projm, campos, g.P, g.M, g.means3D,
                                                 g.opacities, g.shs, g.colors, g.scales,
                                                 g.rotations, g.cov3D, radii, feat, flags, blkcnt,
                                                 counters));
    DMGS_LAUNCH_CHECK("preprocess_kernel");
  }
  return DMGS_OK;
}

int launch_mark_visible(int P, const float *means3D, const float *viewm, uint8_t *present,
                        cudaStream_t s) {
  if (P <= 0) return DMGS_OK;
  DMGS_TIMED(K_MARK_VISIBLE, s, dmgs_host::note_launch(), mark_visible_kernel<<<(P + 255) / 256, 256, 0, s>>>(P, means3D, viewm, present));
  DMGS_LAUNCH_CHECK("mark_visible_kernel");
  return DMGS_OK;
}

}  // namespace dmgs

namespace dmgs {
namespace {
__global__ void debug_geometry_kernel(int P, int gx, const float4 *__restrict__ feat,
                                      int32_t *rect, uint32_t *tiles_touched, float *depth,
                                      float *xy, float *conic_opacity, float *rgb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= P) return;
  const float4 f0 = feat[3 * idx], f1 = feat[3 * idx + 1], f2 = feat[3 * idx + 2];
  const uint32_t lo = __float_as_uint(f2.z), hi = __float_as_uint(f2.w);
  const int x0 = lo & 0xffff, y0 = lo >> 16, x1 = hi & 0xffff, y1 = hi >> 16;
  const bool vis = (lo | hi) != 0u;
  if (rect) { rect[4 * idx] = x0; rect[4 * idx + 1] = y0; rect[4 * idx + 2] = x1; rect[4 * idx + 3] = y1; }
  if (tiles_touched) tiles_touched[idx] = vis ? (uint32_t)((x1 - x0) * (y1 - y0)) : 0u;
  if (depth) depth[idx] = vis ? f2.y : 0.f;
  if (xy) { xy[2 * idx] = vis ? f0.x : 0.f; xy[2 * idx + 1] = vis ? f0.y : 0.f; }
  if (conic_opacity) {
    conic_opacity[4 * idx] = vis ? f0.z : 0.f; conic_opacity[4 * idx + 1] = vis ? f0.w : 0.f;
    conic_opacity[4 * idx + 2] = vis ? f1.x : 0.f; conic_opacity[4 * idx + 3] = vis ? f1.y : 0.f;
  }
  if (rgb) { rgb[3 * idx] = vis ? f1.z : 0.f; rgb[3 * idx + 1] = vis ? f1.w : 0.f; rgb[3 * idx + 2] = vis ? f2.x : 0.f; }
  (void)gx;
}
}  // namespace

int launch_debug_geometry(const GeomLayout &L, const char *geom, int32_t *rect,
                          uint32_t *tiles_touched, float *depth, float *xy, float *conic_opacity,
                          float *rgb, cudaStream_t s) {
  if (L.P <= 0) return DMGS_OK;
  DMGS_TIMED(K_DEBUG, s, dmgs_host::note_launch(), debug_geometry_kernel<<<(L.P + 255) / 256, 256, 0, s>>>(
      L.P, L.gx, reinterpret_cast<const float4 *>(geom + L.feat), rect, tiles_touched, depth, xy,
      conic_opacity, rgb));
  DMGS_LAUNCH_CHECK("debug_geometry_kernel");
  return DMGS_OK;
}
}  // namespace dmgs

namespace dmgs {

int launch_preprocess_batched(const BatchViews &bv, const GaussianPtrs &g, cudaStream_t s) {
  for (int v = 0; v < bv.nviews; ++v)
    DMGS_CUDA(cudaMemsetAsync(bv.v[v].counters, 0, CI_WORDS * 4, s));
  if (g.P <= 0) return DMGS_OK;
  DMGS_TIMED(K_BATCH_PREPROCESS, s,
             dmgs_host::note_launch(), preprocess_batched_kernel<<<(g.P + PRE_BLOCK - 1) / PRE_BLOCK, PRE_BLOCK, 0, s>>>(
                 bv, g.P, g.M, g.means3D, g.opacities, g.shs, g.colors, g.scales, g.rotations,
                 g.cov3D));
  DMGS_LAUNCH_CHECK("preprocess_batched_kernel");
  return DMGS_OK;
}

}  // namespace dmgs
