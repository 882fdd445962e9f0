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

// View-space z of a mean (column-major view matrix), in the op order the
// CPU oracle uses.
__device__ __forceinline__ float view_z(const float *V, float x, float y, float z) {
  return add(add(add(mul(V[2], x), mul(V[6], y)), mul(V[10], z)), V[14]);
}

// Pixel-space position of a mean: homogeneous projection, perspective
// divide, NDC -> pixel.
__device__ __forceinline__ float2 pixel_of(const ViewParams &vp, const float *Pm, float x,
                                           float y, float z) {
  const float hx = add(add(add(mul(Pm[0], x), mul(Pm[4], y)), mul(Pm[8], z)), Pm[12]);
  const float hy = add(add(add(mul(Pm[1], x), mul(Pm[5], y)), mul(Pm[9], z)), Pm[13]);
  const float hw = add(add(add(mul(Pm[3], x), mul(Pm[7], y)), mul(Pm[11], z)), Pm[15]);
  const float pw = dvd(1.f, add(hw, 1e-7f));
  const float ndcx = mul(hx, pw), ndcy = mul(hy, pw);
  const float Wf = (float)vp.W, Hf = (float)vp.H;
  return make_float2(mul(sub(mul(add(ndcx, 1.f), Wf), 1.f), 0.5f),
                     mul(sub(mul(add(ndcy, 1.f), Hf), 1.f), 0.5f));
}

// Geometry of one Gaussian in one view (position, 3D covariance S and
// opacity o given): projection, EWA 2D covariance, conic, radius and tile
// rectangle.  Writes radii[idx] and, when visible, every field of the record
// but the colour (feat[1].zw, feat[2].x), which color_one adds; a culled
// Gaussian gets radius 0 and flags 0.  Returns whether it is visible (radius
// > 0, non-empty tile rectangle).
__device__ __forceinline__ bool
geometry_one(int idx, const ViewParams &vp, const float *V, const float *Pm, float x, float y,
             float z, const float *S, float o, int32_t *__restrict__ radii,
             float4 *__restrict__ feat, uint8_t *__restrict__ flags,
             uint32_t *__restrict__ counters) {
  const float vx = add(add(add(mul(V[0], x), mul(V[4], y)), mul(V[8], z)), V[12]);
  const float vy = add(add(add(mul(V[1], x), mul(V[5], y)), mul(V[9], z)), V[13]);
  const float vz = view_z(V, x, y, z);

  auto cull = [&]() {
    radii[idx] = 0;
    flags[idx] = 0;
  };
  if (!(vz > 0.2f)) {
    if (vp.prefiltered) atomicOr(counters, ST_PREFILTER);
    cull();
    return false;
  }
  const float2 pix = pixel_of(vp, Pm, x, y, z);
  const float px = pix.x, py = pix.y;

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
  // x / 16 as x * (1/16): both round the same exact value, so the results
  // are identical (the IEEE division costs a dozen instructions)
  constexpr float INV_TILE = 1.f / (float)TILE;
  static_assert((TILE & (TILE - 1)) == 0, "the tile size is a power of two");
  const int x0 = min(vp.gx, max(0, trunc_sat(mul(sub(px, r), INV_TILE))));
  const int y0 = min(vp.gy, max(0, trunc_sat(mul(sub(py, r), INV_TILE))));
  const int x1 = min(vp.gx, max(0, trunc_sat(mul(add(add(px, r), (float)(TILE - 1)), INV_TILE))));
  const int y1 = min(vp.gy, max(0, trunc_sat(mul(add(add(py, r), (float)(TILE - 1)), INV_TILE))));
  if ((x1 - x0) * (y1 - y0) == 0) { cull(); return false; }

  radii[idx] = rad;
  float *f = reinterpret_cast<float *>(feat + 3 * idx);
  *reinterpret_cast<float4 *>(f) = make_float4(px, py, ca, cb);
  *reinterpret_cast<float2 *>(f + 4) = make_float2(cc, o);
  f[9] = vz;
  *reinterpret_cast<float2 *>(f + 10) =
      make_float2(__uint_as_float(pack_u16x2(x0, y0)), __uint_as_float(pack_u16x2(x1, y1)));
  return true;
}

// Colour of a visible Gaussian in one view: precomputed, or SH (degree <= 3)
// at the view direction, +0.5, clamped at 0 with the clamp recorded in the
// flags for the adjoint.  Completes the record written by geometry_one.
__device__ __forceinline__ void color_one(int idx, const ViewParams &vp,
                                          const float *__restrict__ campos_g, int M, float x,
                                          float y, float z, const float *__restrict__ shs,
                                          const float *__restrict__ colors,
                                          float4 *__restrict__ feat, uint8_t *__restrict__ flags) {
  float cr, cg, cbl;
  uint8_t clampbits = 0;
  if (colors != nullptr) {
    cr = __ldg(colors + 3 * idx); cg = __ldg(colors + 3 * idx + 1); cbl = __ldg(colors + 3 * idx + 2);
  } else {
    const float *sh = shs + (size_t)idx * M * 3;
    float dx = x - campos_g[0], dy = y - campos_g[1], dz = z - campos_g[2];  // global or shared
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
#pragma unroll
    for (int k = 0; k < 16; ++k) {  // unrolled: b[] stays in registers
      if (k < nb) {
        rr += b[k] * __ldg(sh + 3 * k);
        gg += b[k] * __ldg(sh + 3 * k + 1);
        bb += b[k] * __ldg(sh + 3 * k + 2);
      }
    }
    rr += 0.5f; gg += 0.5f; bb += 0.5f;
    clampbits = (rr < 0.f ? 1 : 0) | (gg < 0.f ? 2 : 0) | (bb < 0.f ? 4 : 0);
    cr = fmaxf(rr, 0.f); cg = fmaxf(gg, 0.f); cbl = fmaxf(bb, 0.f);
  }
  flags[idx] = FLAG_VISIBLE | clampbits;
  float *f = reinterpret_cast<float *>(feat + 3 * idx);
  *reinterpret_cast<float2 *>(f + 6) = make_float2(cr, cg);
  f[8] = cbl;
}

// View-independent inputs of one Gaussian: position, 3D covariance (given,
// or from scale and rotation), opacity.
__device__ __forceinline__ void load_gaussian(int idx, float scale_modifier,
                                              const float *__restrict__ means,
                                              const float *__restrict__ opac,
                                              const float *__restrict__ scales,
                                              const float *__restrict__ rots,
                                              const float *__restrict__ cov3D, float &x, float &y,
                                              float &z, float *S, float &o) {
  x = __ldg(means + 3 * idx); y = __ldg(means + 3 * idx + 1); z = __ldg(means + 3 * idx + 2);
  if (cov3D != nullptr) {
#pragma unroll
    for (int i = 0; i < 6; ++i) S[i] = __ldg(cov3D + 6 * idx + i);
  } else {
    const float sx = mul(__ldg(scales + 3 * idx), scale_modifier);
    const float sy = mul(__ldg(scales + 3 * idx + 1), scale_modifier);
    const float sz = mul(__ldg(scales + 3 * idx + 2), scale_modifier);
    const float4 q = __ldg(reinterpret_cast<const float4 *>(rots) + idx);
    cov3d_scale_rot(sx, sy, sz, q, S);
  }
  o = __ldg(opac + idx);
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
  bool vis = false;
  if (idx < P) {
    float V[16], Pm[16], S[6], x, y, z, o;
    load_mat(viewm_g, V);
    load_mat(projm_g, Pm);
    load_gaussian(idx, vp.scale_modifier, means, opac, scales, rots, cov3D, x, y, z, S, o);
    vis = geometry_one(idx, vp, V, Pm, x, y, z, S, o, radii, feat, flags, counters);
    if (vis) color_one(idx, vp, campos_g, M, x, y, z, shs, colors, feat, flags);
  }
  const int nvis = __syncthreads_count(vis);
  if (threadIdx.x == 0) blkcnt[blockIdx.x] = (uint32_t)nvis;
}

// Lists the block's (Gaussian, view) pairs whose bits are set in the
// per-thread view masks m into pairs[] as (thread << 4) | view, thread-major;
// returns how many there are.  Every thread of the block calls it.
template <int NW>
__device__ __forceinline__ uint32_t list_pairs(uint32_t m, uint16_t *pairs, uint32_t *wsum) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t cnt = __popc(m);
  uint32_t inc = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += u;
  }
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  uint32_t off = inc - cnt, total = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    off += w < wid ? wsum[w] : 0u;
    total += wsum[w];
  }
  for (uint32_t mm = m; mm; mm &= mm - 1) pairs[off++] = (uint16_t)((t << 4) | (__ffs(mm) - 1));
  __syncthreads();
  return total;
}

// Multi-view preprocess, one block of PRE_BLOCK Gaussians and every view.
//
// Phase 1, a thread per Gaussian: the view-independent inputs are loaded and
// the 3D covariance formed once; then, per view, a test of the view depth
// (the full chain's own value and test) and of the projected centre against
// a conservative radius bound decides whether the pair can be visible at
// all.  The bound: the EWA chain's larger eigenvalue is at most
// tr(J W Sigma W^T J^T) + 0.62 <= |J|_F^2 |W|_F^2 |Sigma|_F + 0.62, with
// |J|_F^2 <= (fx^2 (1 + limx^2) + fy^2 (1 + limy^2)) / z^2 for the Jacobian
// at the clamped position; widened by 0.1% and 2 pixels for rounding, and
// the centre compared with a margin of 2 + 1e-4 |x| pixels, it never culls a
// pair the full chain keeps.  With cameras inside the scene about 40% of
// the pairs lie in front of the camera but only ~7% pass the test.
// Phase 2 runs the full geometry on the block's candidate pairs, listed
// compactly so that every lane does useful work (a per-lane early exit
// would leave the warps running the chain for their slowest lane).
// Phase 3 takes the visible pairs, listed the same way, through the colour
// (SH evaluation, 48 coefficient loads).  Each view's per-block visible
// count feeds its compaction.
__global__ void __launch_bounds__(PRE_BLOCK)
preprocess_batched_kernel(const BatchViews bv, int P, int M, const float *__restrict__ means,
                          const float *__restrict__ opac, const float *__restrict__ shs,
                          const float *__restrict__ colors, const float *__restrict__ scales,
                          const float *__restrict__ rots, const float *__restrict__ cov3D) {
  constexpr int NW = PRE_BLOCK / 32;
  __shared__ uint32_t wcnt[NW][MAX_BATCH_VIEWS];
  __shared__ uint32_t wsum[NW];
  __shared__ uint16_t pairs[PRE_BLOCK * MAX_BATCH_VIEWS];
  __shared__ uint32_t s_vm[PRE_BLOCK];
  // the block's Gaussians (position, covariance, opacity) for the per-pair
  // passes, one array per field
  __shared__ float s_g[10][PRE_BLOCK];
  // per-view constants of the per-pair passes (a different view per lane:
  // from the kernel parameters those would be serialised constant-bank
  // loads); the matrices padded to 17 words so different views fall in
  // different banks
  __shared__ ViewParams s_vp[MAX_BATCH_VIEWS];
  __shared__ float s_V[MAX_BATCH_VIEWS][17], s_P[MAX_BATCH_VIEWS][17];
  // pre-test constants per view, read as 16-byte broadcasts: the view
  // matrix's z row; the projection's x, y and w rows; (W, H, TILE gx + 2,
  // TILE gy + 2); (bound factor, prefiltered, no bound, -)
  __shared__ float4 s_pre[MAX_BATCH_VIEWS][6];
  __shared__ float s_cam[MAX_BATCH_VIEWS][3];
  __shared__ float4 *s_feat[MAX_BATCH_VIEWS];
  __shared__ uint8_t *s_flags[MAX_BATCH_VIEWS];
  __shared__ int32_t *s_radii[MAX_BATCH_VIEWS];
  __shared__ uint32_t *s_counters[MAX_BATCH_VIEWS];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int nv = bv.nviews;
  if (t < nv) {
    const BatchView &V = bv.v[t];
    s_vp[t] = V.vp;
    s_cam[t][0] = __ldg(V.campos);
    s_cam[t][1] = __ldg(V.campos + 1);
    s_cam[t][2] = __ldg(V.campos + 2);
    s_feat[t] = V.feat;
    s_flags[t] = V.flags;
    s_radii[t] = V.radii;
    s_counters[t] = V.counters;
    // |J|_F^2 z^2 |W|_F^2 bound factor of the pre-test
    float w2 = 0.f;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float w = __ldg(V.viewm + 4 * j + i);
        w2 += w * w;
      }
    const float limx = mul(1.3f, V.vp.tanfovx), limy = mul(1.3f, V.vp.tanfovy);
    const float kv = (V.vp.fx * V.vp.fx * (1.f + limx * limx) + V.vp.fy * V.vp.fy * (1.f + limy * limy)) * w2;
    const float *vm = V.viewm, *pm = V.projm;
    s_pre[t][0] = make_float4(__ldg(vm + 2), __ldg(vm + 6), __ldg(vm + 10), __ldg(vm + 14));
    s_pre[t][1] = make_float4(__ldg(pm + 0), __ldg(pm + 4), __ldg(pm + 8), __ldg(pm + 12));
    s_pre[t][2] = make_float4(__ldg(pm + 1), __ldg(pm + 5), __ldg(pm + 9), __ldg(pm + 13));
    s_pre[t][3] = make_float4(__ldg(pm + 3), __ldg(pm + 7), __ldg(pm + 11), __ldg(pm + 15));
    s_pre[t][4] = make_float4((float)V.vp.W, (float)V.vp.H, (float)(TILE * V.vp.gx) + 2.f,
                              (float)(TILE * V.vp.gy) + 2.f);
    // another scale modifier than the first view's (uncommon): no bound
    const bool nobound = cov3D == nullptr && V.vp.scale_modifier != bv.v[0].vp.scale_modifier;
    s_pre[t][5] = make_float4(kv, V.vp.prefiltered ? 1.f : 0.f, nobound ? 1.f : 0.f, 0.f);
  }
  for (int i = t; i < nv * 32; i += PRE_BLOCK) {
    const int v = i >> 5, k = i & 31;
    if (k < 16) s_V[v][k] = __ldg(bv.v[v].viewm + k);
    else s_P[v][k - 16] = __ldg(bv.v[v].projm + k - 16);
  }
  s_vm[t] = 0u;
  __syncthreads();

  const int base = blockIdx.x * PRE_BLOCK;
  const int idx = base + t;
  const float mod0 = s_vp[0].scale_modifier;
  uint32_t cm = 0u;  // candidate views of this thread's Gaussian
  if (idx < P) {
    float S[6], x, y, z, o;
    load_gaussian(idx, mod0, means, opac, scales, rots, cov3D, x, y, z, S, o);
    s_g[0][t] = x; s_g[1][t] = y; s_g[2][t] = z;
#pragma unroll
    for (int i = 0; i < 6; ++i) s_g[3 + i][t] = S[i];
    s_g[9][t] = o;
    const float sfro =
        sqrtf(S[0] * S[0] + S[3] * S[3] + S[5] * S[5] + 2.f * (S[1] * S[1] + S[2] * S[2] + S[4] * S[4]));
    for (int v = 0; v < nv; ++v) {
      // the full chain's view depth, same ops and operands
      const float4 zr = s_pre[v][0];
      const float vz = add(add(add(mul(zr.x, x), mul(zr.y, y)), mul(zr.z, z)), zr.w);
      const float4 fl = s_pre[v][5];
      // Branch-free: every lane evaluates the bound (a warp holds Gaussians
      // on both sides of the camera in nearly every view), then selects.
      // The approximate reciprocal and reciprocal square root (2 ulp) move
      // the centre by ~1e-6 of its value and the bound by far less than its
      // 0.1% widening; beyond z = 1e18 (z^2 near the end of the approximate
      // division's range) and for views without a bound the pair is a
      // candidate.
      const float4 a = s_pre[v][1], b = s_pre[v][2], c = s_pre[v][3], im = s_pre[v][4];
      const float hx = add(add(add(mul(a.x, x), mul(a.y, y)), mul(a.z, z)), a.w);
      const float hy = add(add(add(mul(b.x, x), mul(b.y, y)), mul(b.z, z)), b.w);
      const float hw = add(add(add(mul(c.x, x), mul(c.y, y)), mul(c.z, z)), c.w);
      const float pw = __fdividef(1.f, add(hw, 1e-7f));
      const float px = mul(sub(mul(add(mul(hx, pw), 1.f), im.x), 1.f), 0.5f);
      const float py = mul(sub(mul(add(mul(hy, pw), 1.f), im.y), 1.f), 0.5f);
      const float q = __fdividef(fl.x * sfro, vz * vz) + 0.62f;
      const float rb = 3.0116f * (q * rsqrtf(q)) + 2.f;  // 3.01 sqrt(1.001 q) + 2
      const float ax = 1e-4f * fabsf(px), ay = 1e-4f * fabsf(py);
      // NaN anywhere leaves every comparison false: the pair stays a candidate
      const bool outside = px + rb + ax < -1.f || px - rb - ax > im.z || py + rb + ay < -1.f ||
                           py - rb - ay > im.w;
      const bool front = vz > 0.2f;  // the full chain's first test, on the same value
      if (!front && fl.y != 0.f) atomicOr(s_counters[v], ST_PREFILTER);
      const bool cand = front && (fl.z != 0.f || !(vz < 1e18f) || !outside);
      if (cand) {
        cm |= 1u << v;
      } else {
        s_radii[v][idx] = 0;
        s_flags[v][idx] = 0;
      }
    }
  }

  // Phase 2: full geometry of the candidate pairs.
  const uint32_t ncand = list_pairs<NW>(cm, pairs, wsum);
  for (uint32_t i = t; i < ncand; i += PRE_BLOCK) {
    const uint32_t pr = pairs[i];
    const int gl = (int)(pr >> 4), v = (int)(pr & 15u);
    float S[6], x = s_g[0][gl], y = s_g[1][gl], z = s_g[2][gl], o = s_g[9][gl];
#pragma unroll
    for (int k = 0; k < 6; ++k) S[k] = s_g[3 + k][gl];
    if (cov3D == nullptr && s_vp[v].scale_modifier != mod0)
      load_gaussian(base + gl, s_vp[v].scale_modifier, means, opac, scales, rots, cov3D, x, y, z, S, o);
    if (geometry_one(base + gl, s_vp[v], s_V[v], s_P[v], x, y, z, S, o, s_radii[v], s_feat[v],
                     s_flags[v], s_counters[v]))
      atomicOr(&s_vm[gl], 1u << v);
  }
  __syncthreads();

  // Phase 3: colour of the visible pairs, and the per-view block counts.
  const uint32_t vm = s_vm[t];
  for (int v = 0; v < nv; ++v) {
    const uint32_t b = __ballot_sync(0xffffffffu, (vm >> v) & 1u);
    if (lane == 0) wcnt[wid][v] = __popc(b);
  }
  const uint32_t total = list_pairs<NW>(vm, pairs, wsum);
  if (t < nv) {
    uint32_t n = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) n += wcnt[w][t];
    bv.v[t].blkcnt[blockIdx.x] = n;
  }
  for (uint32_t i = t; i < total; i += PRE_BLOCK) {
    const uint32_t pr = pairs[i];
    const int gl = (int)(pr >> 4), v = (int)(pr & 15u);
    const ViewParams vp = s_vp[v];
    color_one(base + gl, vp, s_cam[v], M, s_g[0][gl], s_g[1][gl], s_g[2][gl], shs, colors,
              s_feat[v], s_flags[v]);
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
                                      const uint8_t *__restrict__ flags, int32_t *rect,
                                      uint32_t *tiles_touched, float *depth, float *xy,
                                      float *conic_opacity, float *rgb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= P) return;
  // the record of a culled Gaussian is not written: read it only when visible
  const bool vis = flags[idx] & FLAG_VISIBLE;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 f0 = vis ? feat[3 * idx] : zero, f1 = vis ? feat[3 * idx + 1] : zero;
  const float4 f2 = vis ? feat[3 * idx + 2] : zero;
  const uint32_t lo = __float_as_uint(f2.z), hi = __float_as_uint(f2.w);
  const int x0 = lo & 0xffff, y0 = lo >> 16, x1 = hi & 0xffff, y1 = hi >> 16;
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
      L.P, L.gx, reinterpret_cast<const float4 *>(geom + L.feat),
      reinterpret_cast<const uint8_t *>(geom + L.flags), rect, tiles_touched, depth, xy,
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
