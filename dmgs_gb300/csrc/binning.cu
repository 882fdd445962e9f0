// binning.cu — (tile, Gaussian) lists ordered by depth, without sorting the
// instance list.
//
// The reference pipeline (duplicateWithKeys -> radix sort of the 64-bit
// (tile << 32 | depth_bits) instance keys -> identifyTileRanges) yields, per
// tile, the covering Gaussians in depth order, ties in Gaussian-index order.
// The same lists are produced here with work linear in the number of visible
// Gaussians V plus the instances K:
//
//   1. compact   the visible Gaussians in index order: (depth_bits, index)
//   2. sort      them by depth bits with a stable LSD radix sort (4 x 8-bit
//                digits) -> depth order, ties in index order;
//   3. chunk     the sorted list is cut into C contiguous chunks of equal
//                work (weight of a Gaussian: CHUNK_W_GAUSS + ceil(tiles/32),
//                the warp iterations it costs below) -> chunk starts;
//   4. count     each chunk counts its instances per tile -> count matrix
//                [T][C];
//   5. scan      the matrix in (tile, chunk) order -> the first slot of every
//                (tile, chunk) pair, the tile ranges and K;
//   6. emit      one warp per chunk walks its Gaussians in depth order and
//                appends each Gaussian index to the lists of the tiles it
//                covers, its running slots in shared memory.
//
// Because every chunk appends in depth order and chunks are laid out in
// depth order within every tile, each tile's list is exactly the reference's
// sorted list.  Nothing of size K is read back or sorted; K is written once.
// Near Gaussians cover thousands of tiles and sort together, so chunks of
// equal Gaussian count would differ in work by an order of magnitude; equal
// weight keeps one warp per chunk balanced.  The count matrix (T x C x 4 B,
// 33 MB at 4056 tiles and 2048 chunks) stays in L2.
#include <algorithm>

#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Block-wide exclusive scan of one value per thread (u64 accumulation).
template <int THREADS>
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v,
                                                                   unsigned long long *total) {
  __shared__ unsigned long long warp_sums[THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long u = __shfl_up_sync(FULL, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    unsigned long long s = lane < THREADS / 32 ? warp_sums[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long u = __shfl_up_sync(FULL, s, o);
      if (lane >= o) s += u;
    }
    if (lane < THREADS / 32) warp_sums[lane] = s;  // inclusive
  }
  __syncthreads();
  const unsigned long long before = (wid > 0 ? warp_sums[wid - 1] : 0ull) + inc - v;
  if (total) *total = warp_sums[THREADS / 32 - 1];
  __syncthreads();
  return before;
}

__device__ __forceinline__ uint32_t scan_len(const uint32_t *n_dev, uint32_t n_max) {
  return n_dev ? min(*n_dev, n_max) : n_max;
}

// ---- generic exclusive scan (u32, in place), three phases ----------------

__global__ void __launch_bounds__(SCAN_THREADS)
scan_reduce_kernel(const uint32_t *__restrict__ data, const uint32_t *__restrict__ n_dev,
                   uint32_t n_max, uint32_t *__restrict__ part) {
  const uint32_t n = scan_len(n_dev, n_max);
  const uint32_t base = blockIdx.x * SCAN_TILE;
  if (base >= n) return;
  unsigned long long s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    const uint32_t k = base + i * SCAN_THREADS + threadIdx.x;
    if (k < n) s += data[k];
  }
  unsigned long long tot;
  block_exclusive_scan<SCAN_THREADS>(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = (uint32_t)tot;
}

// One block: exclusive scan of the per-block partials (or of the whole
// array when it fits one block); total to *total_out, overflow flagged.
__global__ void __launch_bounds__(SCAN_THREADS)
scan_single_kernel(uint32_t *__restrict__ data, const uint32_t *__restrict__ n_dev, uint32_t n_max,
                   int partials_of_tiles, uint32_t *__restrict__ total_out,
                   uint32_t *__restrict__ status) {
  uint32_t n = scan_len(n_dev, n_max);
  if (partials_of_tiles) n = (n + SCAN_TILE - 1) / SCAN_TILE;
  const uint32_t per = (n + SCAN_THREADS - 1) / SCAN_THREADS;
  const uint32_t beg = min(n, threadIdx.x * per), end = min(n, beg + per);
  unsigned long long s = 0;
  for (uint32_t k = beg; k < end; ++k) s += data[k];
  unsigned long long tot;
  unsigned long long run = block_exclusive_scan<SCAN_THREADS>(s, &tot);
  for (uint32_t k = beg; k < end; ++k) {
    const uint32_t v = data[k];
    data[k] = (uint32_t)run;
    run += v;
  }
  if (threadIdx.x == 0) {
    if (total_out) *total_out = (uint32_t)tot;
    if (tot > 0xffffffffull && status) atomicOr(status, ST_OVERFLOW);
  }
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_down_kernel(uint32_t *__restrict__ data, const uint32_t *__restrict__ n_dev, uint32_t n_max,
                 const uint32_t *__restrict__ part) {
  const uint32_t n = scan_len(n_dev, n_max);
  const uint32_t base = blockIdx.x * SCAN_TILE;
  if (base >= n) return;
  // blocked: thread i owns elements base + i*ITEMS .. +ITEMS-1
  uint32_t v[SCAN_ITEMS];
  unsigned long long s = 0;
  const uint32_t k0 = base + threadIdx.x * SCAN_ITEMS;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = (k0 + i < n) ? data[k0 + i] : 0u;
    s += v[i];
  }
  unsigned long long run = block_exclusive_scan<SCAN_THREADS>(s, nullptr) + part[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (k0 + i < n) data[k0 + i] = (uint32_t)run;
    run += v[i];
  }
}

// ---- compaction of visible Gaussians (index order) ----------------------

__global__ void __launch_bounds__(PRE_BLOCK)
compact_kernel(int P, const uint8_t *__restrict__ flags, const float4 *__restrict__ feat,
               const uint32_t *__restrict__ blkoff, uint32_t *__restrict__ dkey,
               uint32_t *__restrict__ dval) {
  const int idx = blockIdx.x * PRE_BLOCK + threadIdx.x;
  const bool v = idx < P && (flags[idx] & FLAG_VISIBLE);
  __shared__ uint32_t wcount[PRE_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(FULL, v);
  if (lane == 0) wcount[wid] = __popc(b);
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < wid; ++w) before += wcount[w];
  if (v) {
    const uint32_t pos = blkoff[blockIdx.x] + before + __popc(b & lanemask_lt());
    dkey[pos] = __float_as_uint(feat[3 * idx + 2].y);
    dval[pos] = (uint32_t)idx;
  }
}

// One thread: derived sizes from V.
__global__ void params_kernel(int T, uint32_t cmax, uint32_t *__restrict__ counters) {
  const uint32_t V = counters[CI_V];
  const uint32_t nbr = (V + RADIX_TILE - 1) / RADIX_TILE;
  const uint32_t C = min((V + CHUNK_MIN_GAUSS - 1) / CHUNK_MIN_GAUSS, cmax);
  counters[CI_NBR] = nbr;
  counters[CI_NRH] = 256u * nbr;
  counters[CI_C] = C;
  counters[CI_NCM] = (uint32_t)T * C;
}

// ---- stable LSD radix sort of (depth_bits, index), 8 bits per pass -------

__global__ void __launch_bounds__(RADIX_BLOCK)
radix_hist_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ counters,
                  int shift, uint32_t *__restrict__ rhist) {
  const uint32_t V = counters[CI_V], nbr = counters[CI_NBR];
  const uint32_t b = blockIdx.x;
  if (b >= nbr) return;
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
#pragma unroll
  for (int i = 0; i < RADIX_ITEMS; ++i) {
    const uint32_t k = b * RADIX_TILE + i * RADIX_BLOCK + threadIdx.x;
    if (k < V) atomicAdd(&h[(keys[k] >> shift) & 255u], 1u);
  }
  __syncthreads();
  rhist[threadIdx.x * nbr + b] = h[threadIdx.x];  // digit-major
}

// Lanes whose 8-bit digit equals this lane's (invalid lanes, digit 256, group
// together): nine ballots instead of match.any.
__device__ __forceinline__ unsigned digit_peers(int d) {
  unsigned peers = FULL;
#pragma unroll
  for (int b = 0; b < 9; ++b) {
    const bool bit = (d >> b) & 1;
    const unsigned m = __ballot_sync(FULL, bit);
    peers &= bit ? m : ~m;
  }
  return peers;
}

// Warp w of block b owns keys [b*2048 + w*256, +256), visited in 8 rounds
// of 32 (round-major, then lane) — the input order, so the pass is stable.
__global__ void __launch_bounds__(RADIX_BLOCK)
radix_scatter_kernel(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                     uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                     const uint32_t *__restrict__ counters, int shift,
                     const uint32_t *__restrict__ rhist_scanned) {
  const uint32_t V = counters[CI_V], nbr = counters[CI_NBR];
  const uint32_t b = blockIdx.x;
  if (b >= nbr) return;
  __shared__ uint32_t wh[RADIX_BLOCK / 32][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < (RADIX_BLOCK / 32) * 256; i += RADIX_BLOCK) (&wh[0][0])[i] = 0u;
  __syncthreads();
  uint32_t key[RADIX_ITEMS], val[RADIX_ITEMS];
  int dig[RADIX_ITEMS];
  const uint32_t base = b * RADIX_TILE + w * (32 * RADIX_ITEMS);
#pragma unroll
  for (int r = 0; r < RADIX_ITEMS; ++r) {
    const uint32_t k = base + r * 32 + lane;
    const bool ok = k < V;
    key[r] = ok ? kin[k] : 0u;
    val[r] = ok ? vin[k] : 0u;
    dig[r] = ok ? (int)((key[r] >> shift) & 255u) : 256;
    const unsigned peers = digit_peers(dig[r]);
    if (dig[r] < 256 && lane == __ffs(peers) - 1) wh[w][dig[r]] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const int d = threadIdx.x;  // RADIX_BLOCK == 256 digits
    uint32_t run = rhist_scanned[d * nbr + b];
#pragma unroll
    for (int w2 = 0; w2 < RADIX_BLOCK / 32; ++w2) {
      const uint32_t c = wh[w2][d];
      wh[w2][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RADIX_ITEMS; ++r) {
    const unsigned peers = digit_peers(dig[r]);
    uint32_t pos = 0;
    if (dig[r] < 256) pos = wh[w][dig[r]] + __popc(peers & lanemask_lt());
    __syncwarp();
    if (dig[r] < 256) {
      kout[pos] = key[r];
      vout[pos] = val[r];
      if (lane == __ffs(peers) - 1) wh[w][dig[r]] += __popc(peers);
    }
    __syncwarp();
  }
}

// ---- per-(tile, chunk) counts --------------------------------------------

__device__ __forceinline__ void unpack_rect(float4 f2, int &x0, int &y0, int &x1, int &y1) {
  const uint32_t lo = __float_as_uint(f2.z), hi = __float_as_uint(f2.w);
  x0 = lo & 0xffff; y0 = lo >> 16; x1 = hi & 0xffff; y1 = hi >> 16;
}

// L2 eviction-priority hints: the instance list is written 4 bytes at a time
// by many warps, so its lines should stay in L2 until complete (evict_last);
// the count-matrix reads of the emission are used once (evict_first).
__device__ __forceinline__ uint64_t l2_policy_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_hint(uint32_t *ptr, uint32_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(ptr), "r"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ uint32_t ld_hint(const uint32_t *ptr, uint64_t pol) {
  uint32_t v;
  asm volatile("ld.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(ptr), "l"(pol));
  return v;
}

// Lane `lane` visits tiles lane, lane+32, ... of a rw-wide rectangle in
// row-major order; row/column advance incrementally.  The divisions by rw
// (numerators <= 32) use a per-rectangle multiplier M = floor(2^16 / rw) + 1
// for rw <= 32, exact for numerators below 2^16 / rw (>= 2048), and M = 0
// for wider rectangles (every quotient is 0).
__device__ __forceinline__ uint32_t walk_magic(int rw) {
  return rw <= 32 ? 65536u / (uint32_t)rw + 1u : 0u;
}

struct RectWalk {
  int row, col, dr, dc, rw;
  __device__ __forceinline__ RectWalk(int lane, int rw_, uint32_t M) : rw(rw_) {
    row = (int)(((uint32_t)lane * M) >> 16);
    col = lane - row * rw;
    dr = (int)((32u * M) >> 16);
    dc = 32 - dr * rw;
  }
  __device__ __forceinline__ void next() {
    row += dr; col += dc;
    if (col >= rw) { col -= rw; ++row; }
  }
};

// ---- equal-work chunks of the depth-sorted list ---------------------------

// Weight of sorted position s: the warp iterations its Gaussian costs the
// count and emit kernels (a fixed part plus one per 32 covered tiles).
__global__ void __launch_bounds__(256)
chunk_weight_kernel(const float4 *__restrict__ feat, const uint32_t *__restrict__ order,
                    const uint32_t *__restrict__ counters, uint32_t *__restrict__ weight) {
  const uint32_t V = counters[CI_V];
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  int x0, y0, x1, y1;
  unpack_rect(feat[3 * order[s] + 2], x0, y0, x1, y1);
  const uint32_t area = (uint32_t)((x1 - x0) * (y1 - y0));
  weight[s] = CHUNK_W_GAUSS + (area + 31u) / 32u;
}

// From the exclusive prefix of the weights: chunk c = the positions whose
// prefix lies in [c W / C, (c + 1) W / C).  Prefixes strictly increase (each
// weight >= 1), so the chunk of a position never decreases; position s opens
// the chunks between its predecessor's and its own.  cstart[C] = V.
__global__ void __launch_bounds__(256)
chunk_bounds_kernel(const uint32_t *__restrict__ prefix, const uint32_t *__restrict__ counters,
                    uint32_t *__restrict__ cstart) {
  const uint32_t V = counters[CI_V], C = counters[CI_C];
  const unsigned long long W = counters[CI_W];
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V || W == 0) return;
  const uint32_t cs = (uint32_t)((unsigned long long)prefix[s] * C / W);
  const uint32_t cp = s > 0 ? (uint32_t)((unsigned long long)prefix[s - 1] * C / W) : 0u;
  for (uint32_t c = (s > 0 ? cp + 1 : 0u); c <= cs; ++c) cstart[c] = s;
  if (s == V - 1)
    for (uint32_t c = cs + 1; c <= C; ++c) cstart[c] = V;
}

// ---- counting and emission: one warp per (chunk, band of tile rows) -------
// A band is R consecutive rows of tiles; its running slots live in shared
// memory (R * gx words).  The warp walks its chunk's Gaussians in depth order,
// 32 at a time (lane i holds Gaussian g0 + i), selects by ballot the ones
// whose rectangle meets the band and visits each one's tiles within the band,
// its lanes spread over them.  One Gaussian covers each tile once, so within
// a Gaussian the lanes touch distinct slots and a plain read/modify/write
// suffices; __syncwarp orders consecutive Gaussians.  COUNT: slots start at
// 0 and end as this chunk's per-tile counts (written to the count matrix).
// EMIT: slots start at the scanned counts (first list position of each
// (tile, chunk)) and each visit appends the Gaussian index.  Indices and
// rectangles are loaded two and one groups ahead.
struct Bands {
  int gx, gy, R, nb;  // grid, rows per band, bands
};

template <bool EMIT>
__global__ void __launch_bounds__(32)
band_kernel(Bands bd, const float4 *__restrict__ feat, const uint32_t *__restrict__ order,
            uint32_t *__restrict__ counters, const uint32_t *__restrict__ cstart,
            uint32_t *__restrict__ cmat, uint32_t *__restrict__ point_list, uint32_t K_alloc) {
  extern __shared__ uint32_t slot[];
  const uint32_t C = counters[CI_C];
  const uint32_t c = blockIdx.x / (uint32_t)bd.nb;
  const int b = (int)(blockIdx.x - c * (uint32_t)bd.nb);
  if (c >= C) return;
  const int lane = threadIdx.x;
  const int ys = b * bd.R, ye = min(bd.gy, ys + bd.R);
  const int t0 = ys * bd.gx, nt = (ye - ys) * bd.gx;
  const uint32_t s0 = cstart[c], s1 = cstart[c + 1];
  const uint64_t keep = l2_policy_last();
  if (EMIT) {
    // an overflowed view (instances above the list capacity) emits nothing
    if (s0 >= s1 || (counters[CI_STATUS] & ST_OVERFLOW)) return;
    const uint64_t once = l2_policy_first();
    int i = lane;
    for (; i + 96 < nt; i += 128) {
      const uint32_t a = ld_hint(cmat + (size_t)(t0 + i) * C + c, once);
      const uint32_t e = ld_hint(cmat + (size_t)(t0 + i + 32) * C + c, once);
      const uint32_t f = ld_hint(cmat + (size_t)(t0 + i + 64) * C + c, once);
      const uint32_t g = ld_hint(cmat + (size_t)(t0 + i + 96) * C + c, once);
      slot[i] = a; slot[i + 32] = e; slot[i + 64] = f; slot[i + 96] = g;
    }
    for (; i < nt; i += 32) slot[i] = ld_hint(cmat + (size_t)(t0 + i) * C + c, once);
  } else {
    for (int i = lane; i < nt; i += 32) slot[i] = 0u;
  }
  __syncwarp();
  bool bad = false;
  const float4 none = make_float4(0.f, 0.f, 0.f, 0.f);
  bool vA = s0 + lane < s1, vB = s0 + 32 + lane < s1;
  uint32_t idA = vA ? order[s0 + lane] : 0u;
  uint32_t idB = vB ? order[s0 + 32 + lane] : 0u;
  float4 rA = vA ? feat[3 * idA + 2] : none;
  for (uint32_t g0 = s0; g0 < s1; g0 += 32) {
    const uint32_t id = idA;
    const float4 r = rA;
    const bool v = vA;
    idA = idB; vA = vB;
    rA = vA ? feat[3 * idA + 2] : none;
    vB = g0 + 64 + lane < s1;
    idB = vB ? order[g0 + 64 + lane] : 0u;
    int x0, y0, x1, y1;
    unpack_rect(r, x0, y0, x1, y1);
    const int cy0 = max(y0, ys), cy1 = min(y1, ye);
    const bool hit = v && cy0 < cy1 && x0 < x1;
    unsigned m = __ballot_sync(FULL, hit);
    const uint32_t xy = hit ? ((uint32_t)x0 | ((uint32_t)(cy0 - ys) << 16)) : 0u;
    const uint32_t wa = hit ? ((uint32_t)(x1 - x0) | ((uint32_t)((x1 - x0) * (cy1 - cy0)) << 16)) : 1u;
    const uint32_t mg = walk_magic(hit ? x1 - x0 : 1);  // lane-parallel, once per group
    while (m) {
      const int i = __ffs(m) - 1;
      m &= m - 1;
      const uint32_t xyi = __shfl_sync(FULL, xy, i), wai = __shfl_sync(FULL, wa, i);
      const uint32_t mgi = __shfl_sync(FULL, mg, i);
      const uint32_t idi = EMIT ? __shfl_sync(FULL, id, i) : 0u;
      const int bx = (int)(xyi & 0xffffu), by = (int)(xyi >> 16);
      const int rw = (int)(wai & 0xffffu), area = (int)(wai >> 16);
      RectWalk it(lane, rw, mgi);
      const int o = by * bd.gx + bx;
      int j = lane;
      // two tiles per step (distinct slots: independent read/modify/writes)
      for (; j + 32 < area; j += 64) {
        const int a0 = o + it.row * bd.gx + it.col;
        it.next();
        const int a1 = o + it.row * bd.gx + it.col;
        it.next();
        const uint32_t p0 = slot[a0], p1 = slot[a1];
        slot[a0] = p0 + 1u;
        slot[a1] = p1 + 1u;
        if (EMIT) {
          if (p0 < K_alloc) st_hint(point_list + p0, idi, keep); else bad = true;
          if (p1 < K_alloc) st_hint(point_list + p1, idi, keep); else bad = true;
        }
      }
      if (j < area) {
        const int a0 = o + it.row * bd.gx + it.col;
        const uint32_t p0 = slot[a0];
        slot[a0] = p0 + 1u;
        if (EMIT) {
          if (p0 < K_alloc) st_hint(point_list + p0, idi, keep); else bad = true;
        }
      }
      __syncwarp();
    }
  }
  if (EMIT) {
    if (bad) atomicOr(&counters[CI_STATUS], ST_BOUNDS);
  } else {
    for (int i = lane; i < nt; i += 32) cmat[(size_t)(t0 + i) * C + c] = slot[i];
  }
}

// Tile ranges from the scanned count matrix.  When the instances exceed the
// list capacity (capacity-bounded callers), every range is left empty and
// the overflow bit is set, so no kernel reads past the list buffer.
__global__ void ranges_kernel(int T, const uint32_t *__restrict__ cmat_scanned,
                              uint32_t *__restrict__ counters, uint2 *__restrict__ ranges,
                              uint32_t K_cap) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const uint32_t C = counters[CI_C], K = counters[CI_K];
  const bool over = K > K_cap || (counters[CI_STATUS] & ST_OVERFLOW);
  if (over && t == 0) atomicOr(&counters[CI_STATUS], ST_OVERFLOW);
  uint2 r = make_uint2(0u, 0u);
  if (C > 0 && !over) {
    const uint32_t a = cmat_scanned[(size_t)t * C];
    const uint32_t e = (t + 1 < T) ? cmat_scanned[(size_t)(t + 1) * C] : K;
    if (e > a) r = make_uint2(a, e);
    atomicMax(&counters[CI_MAXLIST], e - a);
  }
  ranges[t] = r;
}

// Debug view: sorted keys in the reference's form (tile << 32 | depth_bits).
__global__ void debug_keys_kernel(int T, const uint2 *__restrict__ ranges,
                                  const uint32_t *__restrict__ point_list,
                                  const float4 *__restrict__ feat, uint64_t *__restrict__ keys_out,
                                  uint32_t *__restrict__ values_out) {
  const int t = blockIdx.x;
  const uint2 r = ranges[t];
  for (uint32_t i = r.x + threadIdx.x; i < r.y; i += blockDim.x) {
    const uint32_t id = point_list[i];
    if (keys_out) keys_out[i] = ((uint64_t)t << 32) | __float_as_uint(feat[3 * id + 2].y);
    if (values_out) values_out[i] = id;
  }
}


}  // namespace

namespace {

constexpr int BAND_TILES = 1024;  // target slots per band (4 KB of shared memory)

// Bands of tile rows and the chunk count for a gx x gy grid: enough
// (chunk, band) warps to fill the GPU in one wave, each band's slots small
// enough for many resident warps per SM.
struct BandPlan {
  Bands bd;
  uint32_t cmax;
  size_t smem;
};

int band_plan(int gx, int gy, BandPlan &pl) {
  pl.bd.gx = gx;
  pl.bd.gy = gy;
  pl.bd.R = std::max(1, std::min(gy, BAND_TILES / std::max(gx, 1)));
  pl.bd.nb = (gy + pl.bd.R - 1) / pl.bd.R;
  pl.smem = (size_t)pl.bd.R * gx * 4;
  if (pl.smem > 220 * 1024) {
    dmgs_host::set_error("image too large: a row of %d tiles exceeds the binning kernels' shared memory", gx);
    return DMGS_ERR_ARG;
  }
  int dev = 0;
  DMGS_CUDA(cudaGetDevice(&dev));
  thread_local int cached_dev = -1;
  thread_local size_t cached_smem = 0;
  thread_local int cached_resident = 0;
  if (dev != cached_dev || pl.smem != cached_smem) {
    if (pl.smem > 48 * 1024) {
      DMGS_CUDA(cudaFuncSetAttribute(band_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pl.smem));
      DMGS_CUDA(cudaFuncSetAttribute(band_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pl.smem));
    }
    int sms = 0, a = 0, b = 0;
    DMGS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DMGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, band_kernel<false>, 32, pl.smem));
    DMGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, band_kernel<true>, 32, pl.smem));
    cached_dev = dev;
    cached_smem = pl.smem;
    cached_resident = std::max(1, std::min(a, b)) * sms;
  }
  pl.cmax = (uint32_t)std::max(1, std::min(CHUNK_COUNT_MAX, cached_resident / pl.bd.nb));
  return DMGS_OK;
}

}  // namespace

int launch_scan(uint32_t *data, const uint32_t *n_dev, uint32_t n_max, uint32_t *part,
                uint32_t *total_out, uint32_t *status, cudaStream_t s) {
  if (n_max <= (uint32_t)SCAN_TILE * 4) {
    dmgs_host::note_launch(), scan_single_kernel<<<1, SCAN_THREADS, 0, s>>>(data, n_dev, n_max, 0, total_out, status);
    DMGS_LAUNCH_CHECK("scan_single_kernel");
    return DMGS_OK;
  }
  const uint32_t nb = (n_max + SCAN_TILE - 1) / SCAN_TILE;
  dmgs_host::note_launch(), scan_reduce_kernel<<<nb, SCAN_THREADS, 0, s>>>(data, n_dev, n_max, part);
  DMGS_LAUNCH_CHECK("scan_reduce_kernel");
  dmgs_host::note_launch(), scan_single_kernel<<<1, SCAN_THREADS, 0, s>>>(part, n_dev, n_max, 1, total_out, status);
  DMGS_LAUNCH_CHECK("scan_single_kernel");
  dmgs_host::note_launch(), scan_down_kernel<<<nb, SCAN_THREADS, 0, s>>>(data, n_dev, n_max, part);
  DMGS_LAUNCH_CHECK("scan_down_kernel");
  return DMGS_OK;
}

int launch_binning_geometry(const GeomLayout &L, char *geom, uint32_t K_cap, cudaStream_t s) {
  uint32_t *counters = reinterpret_cast<uint32_t *>(geom + L.counters);
  uint32_t *blkcnt = reinterpret_cast<uint32_t *>(geom + L.blkcnt);
  uint32_t *part = reinterpret_cast<uint32_t *>(geom + L.scanpart);
  uint32_t *k0 = reinterpret_cast<uint32_t *>(geom + L.dkey0);
  uint32_t *k1 = reinterpret_cast<uint32_t *>(geom + L.dkey1);
  uint32_t *v0 = reinterpret_cast<uint32_t *>(geom + L.dval0);
  uint32_t *v1 = reinterpret_cast<uint32_t *>(geom + L.dval1);
  uint32_t *rhist = reinterpret_cast<uint32_t *>(geom + L.rhist);
  uint32_t *cmat = reinterpret_cast<uint32_t *>(geom + L.cmat);
  const float4 *feat = reinterpret_cast<const float4 *>(geom + L.feat);
  const int T = L.T();
  BandPlan pl;
  if (int r = band_plan(L.gx, L.gy, pl)) return r;
  if (L.P > 0) {
    DMGS_TIMED(K_BIN_COMPACT, s, {
      int r = launch_scan(blkcnt, nullptr, (uint32_t)L.nb_pre, part, counters + CI_V, counters, s);
      if (r != DMGS_OK) return r;
      dmgs_host::note_launch(), compact_kernel<<<L.nb_pre, PRE_BLOCK, 0, s>>>(L.P, reinterpret_cast<const uint8_t *>(geom + L.flags), feat, blkcnt, k0, v0);
    });
    DMGS_LAUNCH_CHECK("compact_kernel");
  }
  dmgs_host::note_launch(), params_kernel<<<1, 1, 0, s>>>(T, pl.cmax, counters);
  DMGS_LAUNCH_CHECK("params_kernel");
  if (L.P > 0) {
    DMGS_TIMED(K_BIN_SORT, s, {
      uint32_t *ki = k0, *vi = v0, *ko = k1, *vo = v1;
      for (int pass = 0; pass < 4; ++pass) {
        const int shift = 8 * pass;
        dmgs_host::note_launch(), radix_hist_kernel<<<L.nb_radix, RADIX_BLOCK, 0, s>>>(ki, counters, shift, rhist);
        int r = launch_scan(rhist, counters + CI_NRH, (uint32_t)L.n_rhist_max, part, nullptr,
                            nullptr, s);
        if (r != DMGS_OK) return r;
        dmgs_host::note_launch(), radix_scatter_kernel<<<L.nb_radix, RADIX_BLOCK, 0, s>>>(ki, vi, ko, vo, counters, shift,
                                                                 rhist);
        uint32_t *t1 = ki; ki = ko; ko = t1;
        uint32_t *t2 = vi; vi = vo; vo = t2;
      }
    });  // four passes: the sorted order ends in (k0, v0)
    DMGS_LAUNCH_CHECK("radix_sort");
  }
  if (L.P > 0) {
    uint32_t *cstart = reinterpret_cast<uint32_t *>(geom + L.cstart);
    DMGS_TIMED(K_BIN_COUNT, s, {
      // the sorted keys end in k0, so k1 is free for the chunk weights
      dmgs_host::note_launch(), chunk_weight_kernel<<<L.nb_pre, 256, 0, s>>>(feat, v0, counters, k1);
      int r = launch_scan(k1, counters + CI_V, (uint32_t)L.P, part, counters + CI_W, counters, s);
      if (r != DMGS_OK) return r;
      dmgs_host::note_launch(), chunk_bounds_kernel<<<L.nb_pre, 256, 0, s>>>(k1, counters, cstart);
      dmgs_host::note_launch(), band_kernel<false><<<pl.cmax * pl.bd.nb, 32, pl.smem, s>>>(
          pl.bd, feat, v0, counters, cstart, cmat, nullptr, 0u);
    });
    DMGS_LAUNCH_CHECK("tile_count");
  }
  DMGS_TIMED(K_BIN_SCAN, s, {
    if (L.P > 0) {
      int r = launch_scan(cmat, counters + CI_NCM, (uint32_t)L.n_cmat_max, part, counters + CI_K,
                          counters, s);
      if (r != DMGS_OK) return r;
    }
    dmgs_host::note_launch(), ranges_kernel<<<(T + 255) / 256, 256, 0, s>>>(T, cmat, counters,
                                                  reinterpret_cast<uint2 *>(geom + L.ranges), K_cap);
  });
  DMGS_LAUNCH_CHECK("ranges_kernel");
  return DMGS_OK;
}

int launch_emit(const GeomLayout &L, char *geom, const BinLayout &B, char *bin, int64_t K,
                cudaStream_t s) {
  if (L.P <= 0 || K <= 0) return DMGS_OK;
  BandPlan pl;
  if (int r = band_plan(L.gx, L.gy, pl)) return r;
  DMGS_TIMED(K_BIN_EMIT, s,
             dmgs_host::note_launch(), band_kernel<true><<<pl.cmax * pl.bd.nb, 32, pl.smem, s>>>(
                 pl.bd, reinterpret_cast<const float4 *>(geom + L.feat),
                 reinterpret_cast<const uint32_t *>(geom + L.dval0),
                 reinterpret_cast<uint32_t *>(geom + L.counters),
                 reinterpret_cast<const uint32_t *>(geom + L.cstart),
                 reinterpret_cast<uint32_t *>(geom + L.cmat),
                 reinterpret_cast<uint32_t *>(bin + B.point_list), (uint32_t)K));
  DMGS_LAUNCH_CHECK("emit_kernel");
  return DMGS_OK;
}

int launch_debug_keys(const GeomLayout &L, const char *geom, const BinLayout &B, const char *bin,
                      uint64_t *keys, uint32_t *values, cudaStream_t s) {
  DMGS_TIMED(K_DEBUG, s, dmgs_host::note_launch(), debug_keys_kernel<<<L.T(), 256, 0, s>>>(
      L.T(), reinterpret_cast<const uint2 *>(geom + L.ranges),
      reinterpret_cast<const uint32_t *>(bin + B.point_list),
      reinterpret_cast<const float4 *>(geom + L.feat), keys, values));
  DMGS_LAUNCH_CHECK("debug_keys_kernel");
  return DMGS_OK;
}

}  // namespace dmgs
