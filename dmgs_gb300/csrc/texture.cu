// texture.cu — the stage-2 hash-grid texture: positions -> SH features
// (MLPTexture3D.sample_noact, geo/texture.py:101-112, called at
// scene/gaussian_geo_model_mlp_flex.py:313), forward and adjoint.
//
//   t   = clamp((xyz - lo) / (hi - lo), 0, 1)
//   enc = multiresolution hash encoding of t: 16 levels x 2 features
//         (tiny-cuda-nn HashGrid as configured at geo/texture.py:57-69:
//         base resolution 16, per-level scale 256^(1/15), 2^19 entries per
//         level, trilinear interpolation)
//   out = W3 relu(W2 relu(W1 enc))   (bias-free, geo/texture.py:18-40)
//
// Encoding conventions (Mueller et al. 2022, with tiny-cuda-nn's grid
// rules): level l has scale s_l = 2^(l log2 b) 16 - 1 and resolution
// ceil(s_l) + 1; p = t s_l + 1/2 splits into cell floor(p) and fraction;
// a corner's entry is x + y r + z r^2 while the level's dense grid fits its
// table (size r^3 rounded up to 8, capped at 2^19), else the spatial hash
// x * 1 ^ y * 2654435761 ^ z * 805459861 (32-bit), modulo the table size.
//
// Two kernels, one thread per point, persistent grids:
//   forward   hash gathers (the 50 MB table is L2-resident), the 32-32-32-C
//             MLP from shared-memory weights (warp-broadcast reads), outputs
//             staged per warp in shared memory for coalesced row stores;
//   adjoint   recomputes the forward, runs the MLP adjoint, accumulates the
//             three weight gradients as 128-point outer-product GEMMs staged
//             in shared memory (each thread owns a fixed 3x4 / 2x4 sub-block
//             in registers across all its tiles; one atomic per entry per
//             block at the end) and writes each point's dL/denc; then a
//             light full-occupancy kernel scatters the table gradient with
//             float2 atomics and forms the position gradient from the
//             interpolation weights' derivatives.
// The reference's gradient hooks (geo/texture.py:72-73 with _MLP's
// loss_scale): the table receives 128x its true gradient, the positions
// their true gradient.
#include <cmath>

#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int TEX_LEVELS = 16;
constexpr int TEX_FEAT = TEX_LEVELS * 2;  // encoding width
constexpr int TEX_MAXC = 48;              // channels (SH degree 3: 3 x 16)
constexpr int TEX_THREADS = 128;
constexpr uint32_t TEX_LOG2_HASHMAP = 19;
constexpr uint32_t TEX_BASE_RES = 16;
constexpr float TEX_GRAD_SCALE = 128.f;

struct TexLevels {
  float scale[TEX_LEVELS];
  uint32_t res[TEX_LEVELS];
  uint32_t offset[TEX_LEVELS];
  uint32_t size[TEX_LEVELS];
  uint32_t hashed;  // bit l: level l is hashed
  uint32_t entries;
};

TexLevels make_levels(float per_level_scale) {
  TexLevels L{};
  // 2^(l log2 b) 16 - 1 in double from the float log2 b, rounded once
  const double log2b = (double)(float)std::log2((double)per_level_scale);
  uint32_t off = 0;
  for (int l = 0; l < TEX_LEVELS; ++l) {
    const float scale = (float)(std::exp2((double)l * log2b) * (double)TEX_BASE_RES - 1.0);
    const uint32_t res = (uint32_t)ceilf(scale) + 1u;
    const uint64_t dense = (uint64_t)res * res * res;
    const uint64_t cap = 1ull << TEX_LOG2_HASHMAP;
    const uint64_t size = std::min<uint64_t>((dense + 7) / 8 * 8, cap);
    L.scale[l] = scale;
    L.res[l] = res;
    L.offset[l] = off;
    L.size[l] = (uint32_t)size;
    if (dense > size) L.hashed |= 1u << l;
    off += (uint32_t)size;
  }
  L.entries = off;
  return L;
}

struct TexArgs {
  const float2 *table;
  const float *W1, *W2, *W3;
  float lo[3], ext[3];
  int64_t n;
};

__device__ __forceinline__ uint32_t corner_index(const TexLevels &L, int l, uint32_t cx, uint32_t cy,
                                                 uint32_t cz) {
  uint32_t idx;
  if ((L.hashed >> l) & 1u) {
    idx = cx ^ (cy * 2654435761u) ^ (cz * 805459861u);
  } else {
    const uint32_t r = L.res[l];
    idx = cx + cy * r + cz * r * r;
  }
  return L.offset[l] + idx % L.size[l];
}

// Normalised, clamped texture coordinate (and whether the clamp passes the
// gradient: inside [0, 1] inclusive, as torch.clamp's adjoint).
__device__ __forceinline__ void tex_coord(const TexArgs &A, const float *xyz, int64_t p, float (&t)[3],
                                          bool (&pass)[3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float v = __fdiv_rn(__fsub_rn(__ldg(xyz + 3 * p + d), A.lo[d]), A.ext[d]);
    pass[d] = v >= 0.f && v <= 1.f;
    t[d] = fminf(fmaxf(v, 0.f), 1.f);
  }
}

struct LevelPos {
  uint32_t c[3];
  float f[3];
};

__device__ __forceinline__ LevelPos level_pos(const TexLevels &L, int l, const float (&t)[3]) {
  LevelPos q;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float p = __fadd_rn(__fmul_rn(t[d], L.scale[l]), 0.5f);
    const float c = floorf(p);
    q.c[d] = (uint32_t)(int)c;
    q.f[d] = __fsub_rn(p, c);
  }
  return q;
}

__device__ __forceinline__ float corner_weight(const LevelPos &q, int corner) {
  const float w0 = (corner & 1) ? q.f[0] : __fsub_rn(1.f, q.f[0]);
  const float w1 = (corner & 2) ? q.f[1] : __fsub_rn(1.f, q.f[1]);
  const float w2 = (corner & 4) ? q.f[2] : __fsub_rn(1.f, q.f[2]);
  return __fmul_rn(__fmul_rn(w0, w1), w2);
}

__device__ __forceinline__ void encode(const TexArgs &A, const TexLevels &L, const float (&t)[3],
                                       float (&enc)[TEX_FEAT]) {
#pragma unroll
  for (int l = 0; l < TEX_LEVELS; ++l) {
    const LevelPos q = level_pos(L, l, t);
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      const float w = corner_weight(q, corner);
      const float2 v = __ldg(A.table + corner_index(L, l, q.c[0] + (corner & 1), q.c[1] + ((corner >> 1) & 1),
                                                    q.c[2] + ((corner >> 2) & 1)));
      a0 = __fadd_rn(a0, __fmul_rn(w, v.x));
      a1 = __fadd_rn(a1, __fmul_rn(w, v.y));
    }
    enc[2 * l] = a0;
    enc[2 * l + 1] = a1;
  }
}

// y = W x for a row-major [R][32] weight matrix in shared memory (rows read
// as float4, the same address across the warp: broadcasts).
template <int R>
__device__ __forceinline__ void matvec(const float *__restrict__ W, const float (&x)[32], float (&y)[R]) {
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const float4 *w = reinterpret_cast<const float4 *>(W + j * 32);
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float4 v = w[k];
      acc = fmaf(v.x, x[4 * k], acc);
      acc = fmaf(v.y, x[4 * k + 1], acc);
      acc = fmaf(v.z, x[4 * k + 2], acc);
      acc = fmaf(v.w, x[4 * k + 3], acc);
    }
    y[j] = acc;
  }
}

// x = W^T y for a row-major [R][32] matrix.
template <int R>
__device__ __forceinline__ void matvec_t(const float *__restrict__ W, const float (&y)[R], float (&x)[32]) {
#pragma unroll
  for (int k = 0; k < 32; ++k) x[k] = 0.f;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const float4 *w = reinterpret_cast<const float4 *>(W + j * 32);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float4 v = w[k];
      x[4 * k] = fmaf(v.x, y[j], x[4 * k]);
      x[4 * k + 1] = fmaf(v.y, y[j], x[4 * k + 1]);
      x[4 * k + 2] = fmaf(v.z, y[j], x[4 * k + 2]);
      x[4 * k + 3] = fmaf(v.w, y[j], x[4 * k + 3]);
    }
  }
}

template <int C>
__device__ __forceinline__ void load_weights(const TexArgs &A, float *sW1, float *sW2, float *sW3) {
  for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
    sW1[i] = A.W1[i];
    sW2[i] = A.W2[i];
  }
  for (int i = threadIdx.x; i < C * 32; i += blockDim.x) sW3[i] = A.W3[i];
  __syncthreads();
}

template <int C>
__global__ void __launch_bounds__(TEX_THREADS)
tex_fwd_kernel(const TexArgs A, const TexLevels L, const float *__restrict__ xyz, float *__restrict__ out,
               float *__restrict__ enc_out) {
  __shared__ __align__(16) float sW1[32 * 32], sW2[32 * 32], sW3[C * 32];
  constexpr int SC = C | 1;  // odd row stride: conflict-free per-lane row writes
  __shared__ float stage[TEX_THREADS / 32][32 * SC];
  load_weights<C>(A, sW1, sW2, sW3);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t ntiles = (A.n + TEX_THREADS - 1) / TEX_THREADS;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t p = tile * TEX_THREADS + threadIdx.x;
    float o[C];
    if (p < A.n) {
      float t[3];
      bool pass[3];
      tex_coord(A, xyz, p, t, pass);
      float enc[TEX_FEAT], h[32], g[32];
      encode(A, L, t, enc);
      if (enc_out) {  // kept for the adjoint: [n][32] rows, 16-byte aligned
        float4 *row = reinterpret_cast<float4 *>(enc_out + 32 * p);
#pragma unroll
        for (int k = 0; k < 8; ++k) row[k] = make_float4(enc[4 * k], enc[4 * k + 1], enc[4 * k + 2], enc[4 * k + 3]);
      }
      matvec<32>(sW1, enc, h);
#pragma unroll
      for (int k = 0; k < 32; ++k) h[k] = fmaxf(h[k], 0.f);
      matvec<32>(sW2, h, g);
#pragma unroll
      for (int k = 0; k < 32; ++k) g[k] = fmaxf(g[k], 0.f);
      matvec<C>(sW3, g, o);
    }
    // rows of the warp's 32 points are contiguous in out: stage and store
    float *st = stage[wid];
    if (p < A.n)
#pragma unroll
      for (int j = 0; j < C; ++j) st[lane * SC + j] = o[j];
    __syncwarp();
    const int64_t p0 = tile * TEX_THREADS + wid * 32;
    const int64_t nrow = A.n - p0 < 32 ? A.n - p0 : 32;
    for (int i = lane; i < nrow * C; i += 32) out[p0 * C + i] = st[(i / C) * SC + i % C];
    __syncwarp();
  }
}

// Adjoint.  Shared memory per block (rows = the block's 128 points): the
// weights; R0 [128][SA] (dL/dout, then dh2, then dh1: the left operands of
// the outer-product GEMMs); R1 [128][SB] (h2, then each thread's dL/denc);
// H1 and E [128][SB] (h1 and enc, kept from the recomputation: right
// operands of the layer-2 and layer-1 GEMMs and the ReLU masks).
constexpr int SA = TEX_MAXC + 1, SB = 33;

// acc[r][c] += sum over the block's points q of a[q][row r] b[q][col c]
template <int R, int SAx>
__device__ __forceinline__ void outer_gemm(const float *__restrict__ a, int row0, int nrows,
                                           const float *__restrict__ b, int col0, float (&acc)[R][4]) {
  for (int q = 0; q < TEX_THREADS; ++q) {
    float bv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) bv[c] = b[q * SB + col0 + c];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float av = row0 + r < nrows ? a[q * SAx + row0 + r] : 0.f;
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(av, bv[c], acc[r][c]);
    }
  }
}

template <int C>
__global__ void __launch_bounds__(TEX_THREADS)
tex_bwd_kernel(const TexArgs A, const TexLevels L, const float *__restrict__ xyz,
               const float *__restrict__ enc_in, const float *__restrict__ dout, float *__restrict__ denc,
               float *__restrict__ dW1, float *__restrict__ dW2, float *__restrict__ dW3) {
  extern __shared__ __align__(16) float smem[];
  float *sW1 = smem, *sW2 = sW1 + 32 * 32, *sW3 = sW2 + 32 * 32;
  float *R0 = sW3 + TEX_MAXC * 32;
  float *R1 = R0 + TEX_THREADS * SA;
  float *H1 = R1 + TEX_THREADS * SB;
  float *E = H1 + TEX_THREADS * SB;
  load_weights<C>(A, sW1, sW2, sW3);
  const int tid = threadIdx.x;
  // owned sub-blocks: dW3 rows R3 (t/8) .., cols 4 (t%8) .. +3; dW2 / dW1
  // rows 2 (t/8) .. +1
  const int cg = (tid & 7) * 4, rg = tid >> 3;
  constexpr int R3 = (C + 15) / 16;
  float acc3[R3][4], acc2[2][4], acc1[2][4];
#pragma unroll
  for (int r = 0; r < R3; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc3[r][c] = 0.f;
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc2[r][c] = acc1[r][c] = 0.f;
  float *e_row = E + tid * SB, *h1_row = H1 + tid * SB;

  const int64_t ntiles = (A.n + TEX_THREADS - 1) / TEX_THREADS;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t p = tile * TEX_THREADS + tid;
    const bool valid = p < A.n;
    float t[3] = {0.f, 0.f, 0.f};
    bool pass[3] = {false, false, false};
    float h2[32];
    {
      float enc[TEX_FEAT], h1[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) enc[k] = h1[k] = h2[k] = 0.f;
      if (valid) {
        if (enc_in) {  // the forward's encoding (the same arithmetic, so the same values)
          const float4 *row = reinterpret_cast<const float4 *>(enc_in + 32 * p);
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const float4 v = __ldg(row + k);
            enc[4 * k] = v.x; enc[4 * k + 1] = v.y; enc[4 * k + 2] = v.z; enc[4 * k + 3] = v.w;
          }
        } else {
          tex_coord(A, xyz, p, t, pass);
          encode(A, L, t, enc);
        }
        matvec<32>(sW1, enc, h1);
#pragma unroll
        for (int k = 0; k < 32; ++k) h1[k] = fmaxf(h1[k], 0.f);
        matvec<32>(sW2, h1, h2);
#pragma unroll
        for (int k = 0; k < 32; ++k) h2[k] = fmaxf(h2[k], 0.f);
      }
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        e_row[k] = enc[k];
        h1_row[k] = h1[k];
        R1[tid * SB + k] = h2[k];
      }
    }
    // dL/dout rows of the block into R0 (coalesced); invalid rows zero
    {
      const int64_t p0 = tile * TEX_THREADS;
      const int nrow = (int)(A.n - p0 < TEX_THREADS ? A.n - p0 : TEX_THREADS);
      for (int i = tid; i < nrow * C; i += TEX_THREADS) R0[(i / C) * SA + i % C] = dout[p0 * C + i];
      if (!valid)
#pragma unroll
        for (int j = 0; j < C; ++j) R0[tid * SA + j] = 0.f;
    }
    __syncthreads();
    // layer 3: dW3 += dy h2^T;  dh2 = relu'(h2) (W3^T dy)
    outer_gemm<R3, SA>(R0, R3 * rg, C, R1, cg, acc3);
    float d[32];
    {
      float dy[C];
#pragma unroll
      for (int j = 0; j < C; ++j) dy[j] = R0[tid * SA + j];
      matvec_t<C>(sW3, dy, d);
    }
#pragma unroll
    for (int k = 0; k < 32; ++k) d[k] = h2[k] > 0.f ? d[k] : 0.f;
    __syncthreads();
    // layer 2: dW2 += dh2 h1^T;  dh1 = relu'(h1) (W2^T dh2)
#pragma unroll
    for (int k = 0; k < 32; ++k) R0[tid * SA + k] = d[k];
    __syncthreads();
    outer_gemm<2, SA>(R0, 2 * rg, 32, H1, cg, acc2);
    float g[32];
    matvec_t<32>(sW2, d, g);
#pragma unroll
    for (int k = 0; k < 32; ++k) g[k] = h1_row[k] > 0.f ? g[k] : 0.f;
    __syncthreads();
    // layer 1: dW1 += dh1 enc^T;  dL/denc = W1^T dh1
#pragma unroll
    for (int k = 0; k < 32; ++k) R0[tid * SA + k] = g[k];
    __syncthreads();
    outer_gemm<2, SA>(R0, 2 * rg, 32, E, cg, acc1);
    matvec_t<32>(sW1, g, d);
    __syncthreads();  // every GEMM read done before the next tile's staging
    if (!valid) continue;
    float4 *row = reinterpret_cast<float4 *>(denc + 32 * p);
#pragma unroll
    for (int k = 0; k < 8; ++k) row[k] = make_float4(d[4 * k], d[4 * k + 1], d[4 * k + 2], d[4 * k + 3]);
  }
  // block partials of the weight gradients
#pragma unroll
  for (int r = 0; r < R3; ++r) {
    const int row = R3 * rg + r;
    if (row < C)
#pragma unroll
      for (int c = 0; c < 4; ++c) atomicAdd(dW3 + row * 32 + cg + c, acc3[r][c]);
  }
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      atomicAdd(dW2 + (2 * rg + r) * 32 + cg + c, acc2[r][c]);
      atomicAdd(dW1 + (2 * rg + r) * 32 + cg + c, acc1[r][c]);
    }
}

// Table (128 x the true gradient) and position gradients from each point's
// dL/denc row: a light kernel (few registers, full occupancy) so that the
// latency of the gathers and atomics is hidden by many warps.  The level
// loop stays rolled and reads the level table from shared memory.
__global__ void __launch_bounds__(256)
tex_scatter_kernel(const TexArgs A, const TexLevels L, const float *__restrict__ xyz,
                   const float *__restrict__ denc, float *__restrict__ dxyz, float2 *__restrict__ dtable) {
  __shared__ TexLevels sL;
  if (threadIdx.x == 0) sL = L;
  __syncthreads();
  const int64_t p = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (p >= A.n) return;
  float t[3];
  bool pass[3];
  tex_coord(A, xyz, p, t, pass);
  const float *dr = denc + 32 * p;
  float gt[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
  for (int l = 0; l < TEX_LEVELS; ++l) {
    const LevelPos q = level_pos(sL, l, t);
    const float2 g = *reinterpret_cast<const float2 *>(dr + 2 * l);
    float dl[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      const uint32_t idx = corner_index(sL, l, q.c[0] + (corner & 1), q.c[1] + ((corner >> 1) & 1),
                                        q.c[2] + ((corner >> 2) & 1));
      const float w = corner_weight(q, corner);
      if (dtable) atomicAdd(dtable + idx, make_float2(TEX_GRAD_SCALE * w * g.x, TEX_GRAD_SCALE * w * g.y));
      if (dxyz) {
        const float2 v = __ldg(A.table + idx);
        const float gv = g.x * v.x + g.y * v.y;
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
          // d w / d f_dd: the other two factors, signed by the corner's bit
          float o = 1.f;
#pragma unroll
          for (int e2 = 0; e2 < 3; ++e2)
            if (e2 != dd) o *= ((corner >> e2) & 1) ? q.f[e2] : 1.f - q.f[e2];
          dl[dd] += (((corner >> dd) & 1) ? o : -o) * gv;
        }
      }
    }
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) gt[dd] += dl[dd] * sL.scale[l];
  }
  if (dxyz)
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) dxyz[3 * p + dd] = pass[dd] ? gt[dd] / A.ext[dd] : 0.f;
}

constexpr size_t tex_bwd_smem() {
  return (size_t)(32 * 32 * 2 + TEX_MAXC * 32 + TEX_THREADS * (SA + 3 * SB)) * sizeof(float);
}

bool tex_ok(const DmgsTexture *tx) {
  if (!tx || !tx->table || !tx->W1 || !tx->W2 || !tx->W3) return false;
  if (tx->channels != 3 && tx->channels != 12 && tx->channels != 27 && tx->channels != 48) return false;
  if (!(tx->per_level_scale > 1.f)) return false;
  for (int d = 0; d < 3; ++d)
    if (!(tx->aabb[3 + d] > tx->aabb[d])) return false;
  return true;
}

TexArgs make_args(const DmgsTexture *tx, int64_t n) {
  TexArgs A;
  A.table = reinterpret_cast<const float2 *>(tx->table);
  A.W1 = tx->W1;
  A.W2 = tx->W2;
  A.W3 = tx->W3;
  for (int d = 0; d < 3; ++d) {
    A.lo[d] = tx->aabb[d];
    A.ext[d] = tx->aabb[3 + d] - tx->aabb[d];
  }
  A.n = n;
  return A;
}

template <typename K>
int persistent_grid(K kernel, size_t smem, int64_t n, int &grid) {
  thread_local int cached_dev = -1, cached_slots = 0;  // per kernel instantiation and host thread
  int dev = 0;
  DMGS_CUDA(cudaGetDevice(&dev));
  if (dev != cached_dev) {
    int sms = 0, per = 0;
    DMGS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DMGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, TEX_THREADS, smem));
    cached_slots = sms * std::max(per, 1);
    cached_dev = dev;
  }
  const int64_t tiles = (n + TEX_THREADS - 1) / TEX_THREADS;
  grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, cached_slots));
  return DMGS_OK;
}

template <int C>
int run_fwd(const TexArgs &A, const TexLevels &L, const float *xyz, float *out, float *enc,
            cudaStream_t s) {
  int grid;
  if (int r = persistent_grid(tex_fwd_kernel<C>, 0, A.n, grid)) return r;
  dmgs_host::note_launch(), tex_fwd_kernel<C><<<grid, TEX_THREADS, 0, s>>>(A, L, xyz, out, enc);
  return DMGS_OK;
}

template <int C>
int run_bwd(const TexArgs &A, const TexLevels &L, const float *xyz, const float *enc,
            const float *dout, float *dxyz, float *dtable, float *dW1, float *dW2, float *dW3,
            float *denc, cudaStream_t s) {
  if (int r = dmgs_host::raise_smem_limit((const void *)tex_bwd_kernel<C>, tex_bwd_smem())) return r;
  int grid;
  if (int r = persistent_grid(tex_bwd_kernel<C>, tex_bwd_smem(), A.n, grid)) return r;
  // timed apart: the MLP adjoint (weight-gradient GEMMs) and the scatter of
  // the encoding gradients into the table and the positions
  DMGS_TIMED(K_TEX_BWD, s, dmgs_host::note_launch(), tex_bwd_kernel<C><<<grid, TEX_THREADS, tex_bwd_smem(), s>>>(
      A, L, xyz, enc, dout, denc, dW1, dW2, dW3));
  if (dxyz || dtable)
    DMGS_TIMED(K_TEX_SCATTER, s, dmgs_host::note_launch(), tex_scatter_kernel<<<(unsigned)((A.n + 255) / 256), 256, 0, s>>>(
        A, L, xyz, denc, dxyz, reinterpret_cast<float2 *>(dtable)));
  return DMGS_OK;
}

}  // namespace

namespace {

int tex_fwd_impl(const DmgsTexture *tx, int64_t n, const float *xyz, float *out, float *enc,
                 dmgs_stream_t stream) {
  if (!tex_ok(tx) || n < 0 || (n > 0 && (!xyz || !out)) ||
      (enc && (reinterpret_cast<uintptr_t>(enc) & 15))) {
    dmgs_host::set_error("tex_fwd: invalid arguments");
    return DMGS_ERR_ARG;
  }
  if (n == 0) return DMGS_OK;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const TexArgs A = make_args(tx, n);
  const TexLevels L = make_levels(tx->per_level_scale);
  int r = DMGS_OK;
  DMGS_TIMED(K_TEX_FWD, s, {
    switch (tx->channels) {
      case 3: r = run_fwd<3>(A, L, xyz, out, enc, s); break;
      case 12: r = run_fwd<12>(A, L, xyz, out, enc, s); break;
      case 27: r = run_fwd<27>(A, L, xyz, out, enc, s); break;
      default: r = run_fwd<48>(A, L, xyz, out, enc, s); break;
    }
  });
  if (r != DMGS_OK) return r;
  DMGS_LAUNCH_CHECK("tex_fwd");
  return DMGS_OK;
}

int tex_bwd_impl(const DmgsTexture *tx, int64_t n, const float *xyz, const float *enc,
                 const float *dout, float *dxyz, float *dtable, float *dW1, float *dW2, float *dW3,
                 void *scratch, size_t scratch_bytes, dmgs_stream_t stream) {
  if (!tex_ok(tx) || n < 0 || !dW1 || !dW2 || !dW3 || (n > 0 && (!xyz || !dout)) ||
      (enc && (reinterpret_cast<uintptr_t>(enc) & 15))) {
    dmgs_host::set_error("tex_bwd: invalid arguments");
    return DMGS_ERR_ARG;
  }
  if (n > 0 && (!scratch || scratch_bytes < dmgs_tex_bwd_scratch_bytes(n) ||
                (reinterpret_cast<uintptr_t>(scratch) & 15))) {
    dmgs_host::set_error("tex_bwd: scratch must hold dmgs_tex_bwd_scratch_bytes(n) bytes, 16-byte aligned");
    return DMGS_ERR_STATE;
  }
  float *denc = static_cast<float *>(scratch);
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const TexLevels L = make_levels(tx->per_level_scale);
  DMGS_CUDA(cudaMemsetAsync(dW1, 0, 32 * 32 * 4, s));
  DMGS_CUDA(cudaMemsetAsync(dW2, 0, 32 * 32 * 4, s));
  DMGS_CUDA(cudaMemsetAsync(dW3, 0, (size_t)tx->channels * 32 * 4, s));
  if (dtable) DMGS_CUDA(cudaMemsetAsync(dtable, 0, (size_t)L.entries * 8, s));
  if (n == 0) return DMGS_OK;
  const TexArgs A = make_args(tx, n);
  int r = DMGS_OK;
  switch (tx->channels) {
    case 3: r = run_bwd<3>(A, L, xyz, enc, dout, dxyz, dtable, dW1, dW2, dW3, denc, s); break;
    case 12: r = run_bwd<12>(A, L, xyz, enc, dout, dxyz, dtable, dW1, dW2, dW3, denc, s); break;
    case 27: r = run_bwd<27>(A, L, xyz, enc, dout, dxyz, dtable, dW1, dW2, dW3, denc, s); break;
    default: r = run_bwd<48>(A, L, xyz, enc, dout, dxyz, dtable, dW1, dW2, dW3, denc, s); break;
  }
  if (r != DMGS_OK) return r;
  DMGS_LAUNCH_CHECK("tex_bwd");
  return DMGS_OK;
}

}  // namespace

}  // namespace dmgs

using namespace dmgs;
using dmgs_host::set_error;

extern "C" {

int64_t dmgs_tex_table_entries(float per_level_scale) {
  if (!(per_level_scale > 1.f)) return -1;
  return (int64_t)make_levels(per_level_scale).entries;
}


int dmgs_tex_fwd(const DmgsTexture *tx, int64_t n, const float *xyz, float *out, dmgs_stream_t stream) {
  return tex_fwd_impl(tx, n, xyz, out, nullptr, stream);
}

int dmgs_tex_fwd_enc(const DmgsTexture *tx, int64_t n, const float *xyz, float *out, float *enc,
                     dmgs_stream_t stream) {
  if (n > 0 && !enc) {
    set_error("tex_fwd_enc: the encoding buffer is required");
    return DMGS_ERR_ARG;
  }
  return tex_fwd_impl(tx, n, xyz, out, enc, stream);
}

size_t dmgs_tex_bwd_scratch_bytes(int64_t n) { return n > 0 ? (size_t)n * 32 * sizeof(float) : 0; }

int dmgs_tex_bwd(const DmgsTexture *tx, int64_t n, const float *xyz, const float *dout, float *dxyz,
                 float *dtable, float *dW1, float *dW2, float *dW3, void *scratch,
                 size_t scratch_bytes, dmgs_stream_t stream) {
  return tex_bwd_impl(tx, n, xyz, nullptr, dout, dxyz, dtable, dW1, dW2, dW3, scratch,
                      scratch_bytes, stream);
}

int dmgs_tex_bwd_enc(const DmgsTexture *tx, int64_t n, const float *xyz, const float *enc,
                     const float *dout, float *dxyz, float *dtable, float *dW1, float *dW2,
                     float *dW3, void *scratch, size_t scratch_bytes, dmgs_stream_t stream) {
  if (n > 0 && !enc) {
    set_error("tex_bwd_enc: the encoding buffer is required");
    return DMGS_ERR_ARG;
  }
  return tex_bwd_impl(tx, n, xyz, enc, dout, dxyz, dtable, dW1, dW2, dW3, scratch, scratch_bytes,
                      stream);
}

}  // extern "C"
