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
//   4. count     each chunk counts its instances per tile -> count matrix,
//                stored chunk-major [C][T] (coalesced in every kernel);
//   5. scan      per tile over the chunks (the within-tile offset of every
//                (tile, chunk) pair and the tile's total), then over the
//                tile totals -> tile bases, the tile ranges and K;
//   6. emit      one warp per chunk walks its Gaussians in depth order and
//                appends each Gaussian index to the lists of the tiles it
//                covers, its running slots in shared memory.
//
// Because every chunk appends in depth order and chunks are laid out in
// depth order within every tile, each tile's list is exactly the reference's
// sorted list.  Nothing of size K is read back or sorted; K is written once.
// Near Gaussians cover thousands of tiles and sort together, so chunks of
// equal Gaussian count would differ in work by an order of magnitude; equal
// weight keeps one warp per chunk balanced.  The count matrix (C x T x 4 B,
// 20 MB at 4056 tiles and 1216 chunks) stays in L2.
//
// Every kernel bins several views at once (blockIdx.y = view, each view with
// its own geometry state and sizes): a batch of views fills the GPU with one
// launch per stage instead of one small launch per stage and view.
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

// ---- generic exclusive scan (u32, in place), three phases, per view -----

__device__ __forceinline__ uint32_t scan_len(const ScanView &v) {
  return v.n_dev ? min(*v.n_dev, v.n_max) : v.n_max;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_reduce_kernel(const ScanViews sv) {
  const ScanView &v = sv.v[blockIdx.y];
  const uint32_t n = scan_len(v);
  const uint32_t base = blockIdx.x * SCAN_TILE;
  if (base >= n) return;
  unsigned long long s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    const uint32_t k = base + i * SCAN_THREADS + threadIdx.x;
    if (k < n) s += v.data[k];
  }
  unsigned long long tot;
  block_exclusive_scan<SCAN_THREADS>(s, &tot);
  if (threadIdx.x == 0) v.part[blockIdx.x] = (uint32_t)tot;
}

// One block per view: exclusive scan of the per-block partials (or of the
// whole array when it fits one block); total to *total_out, overflow flagged.
__global__ void __launch_bounds__(SCAN_THREADS)
scan_single_kernel(const ScanViews sv, int partials_of_tiles) {
  const ScanView &v = sv.v[blockIdx.y];
  uint32_t n = scan_len(v);
  uint32_t *data = v.data;
  if (partials_of_tiles) {
    n = (n + SCAN_TILE - 1) / SCAN_TILE;
    data = v.part;
  }
  const uint32_t per = (n + SCAN_THREADS - 1) / SCAN_THREADS;
  const uint32_t beg = min(n, threadIdx.x * per), end = min(n, beg + per);
  unsigned long long s = 0;
  for (uint32_t k = beg; k < end; ++k) s += data[k];
  unsigned long long tot;
  unsigned long long run = block_exclusive_scan<SCAN_THREADS>(s, &tot);
  for (uint32_t k = beg; k < end; ++k) {
    const uint32_t x = data[k];
    data[k] = (uint32_t)run;
    run += x;
  }
  if (threadIdx.x == 0) {
    if (v.total_out) *v.total_out = (uint32_t)tot;
    if (tot > 0xffffffffull && v.status) atomicOr(v.status, ST_OVERFLOW);
  }
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_down_kernel(const ScanViews sv) {
  const ScanView &v = sv.v[blockIdx.y];
  const uint32_t n = scan_len(v);
  const uint32_t base = blockIdx.x * SCAN_TILE;
  if (base >= n) return;
  // blocked: thread i owns elements base + i*ITEMS .. +ITEMS-1
  uint32_t x[SCAN_ITEMS];
  unsigned long long s = 0;
  const uint32_t k0 = base + threadIdx.x * SCAN_ITEMS;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    x[i] = (k0 + i < n) ? v.data[k0 + i] : 0u;
    s += x[i];
  }
  unsigned long long run = block_exclusive_scan<SCAN_THREADS>(s, nullptr) + v.part[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (k0 + i < n) v.data[k0 + i] = (uint32_t)run;
    run += x[i];
  }
}

// ---- compaction of visible Gaussians (index order) ----------------------

__global__ void __launch_bounds__(PRE_BLOCK)
compact_kernel(const BinViews bv) {
  const BinView &B = bv.v[blockIdx.y];
  if ((int)blockIdx.x >= B.nb_pre) return;
  const int idx = blockIdx.x * PRE_BLOCK + threadIdx.x;
  const bool v = idx < B.P && (B.flags[idx] & FLAG_VISIBLE);
  __shared__ uint32_t wcount[PRE_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(FULL, v);
  if (lane == 0) wcount[wid] = __popc(b);
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < wid; ++w) before += wcount[w];
  if (v) {
    const uint32_t pos = B.blkcnt[blockIdx.x] + before + __popc(b & lanemask_lt());
    B.k0[pos] = __float_as_uint(B.feat[3 * idx + 2].y);
    B.v0[pos] = (uint32_t)idx;
  }
}

// One thread per view: derived sizes from V.
__global__ void params_kernel(const BinViews bv) {
  const int vi = threadIdx.x;
  if (vi >= bv.n) return;
  const BinView &B = bv.v[vi];
  uint32_t *counters = B.counters;
  const uint32_t V = counters[CI_V];
  const uint32_t nbr = (V + RADIX_TILE - 1) / RADIX_TILE;
  const uint32_t C = min((V + CHUNK_MIN_GAUSS - 1) / CHUNK_MIN_GAUSS, B.cmax);
  counters[CI_NBR] = nbr;
  counters[CI_NRH] = 256u * nbr;
  counters[CI_C] = C;
  counters[CI_NCM] = (uint32_t)(B.bd.gx * B.bd.gy) * C;
}

// ---- stable LSD radix sort of (depth_bits, index), 8 bits per pass -------

__global__ void __launch_bounds__(RADIX_BLOCK)
radix_hist_kernel(const BinViews bv, int pass) {
  const BinView &B = bv.v[blockIdx.y];
  const uint32_t *keys = (pass & 1) ? B.k1 : B.k0;
  const int shift = 8 * pass;
  const uint32_t V = B.counters[CI_V], nbr = B.counters[CI_NBR];
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
  B.rhist[threadIdx.x * nbr + b] = h[threadIdx.x];  // digit-major
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
radix_scatter_kernel(const BinViews bv, int pass) {
  const BinView &B = bv.v[blockIdx.y];
  // pass p reads (k0, v0) when p is even and writes (k1, v1), and back
  const uint32_t *kin = (pass & 1) ? B.k1 : B.k0, *vin = (pass & 1) ? B.v1 : B.v0;
  uint32_t *kout = (pass & 1) ? B.k0 : B.k1, *vout = (pass & 1) ? B.v0 : B.v1;
  const int shift = 8 * pass;
  const uint32_t *rhist_scanned = B.rhist;
  const uint32_t V = B.counters[CI_V], nbr = B.counters[CI_NBR];
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

// Chunk segments of the per-tile offset scan: segment s = chunks
// [s L, (s + 1) L), L = ceil(C / segs).
__device__ __forceinline__ uint32_t seg_len(uint32_t C, uint32_t segs) { return (C + segs - 1) / segs; }

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
chunk_weight_kernel(const BinViews bv) {
  const BinView &B = bv.v[blockIdx.y];
  const uint32_t V = B.counters[CI_V];
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  int x0, y0, x1, y1;
  unpack_rect(B.feat[3 * B.v0[s] + 2], x0, y0, x1, y1);
  const uint32_t area = (uint32_t)((x1 - x0) * (y1 - y0));
  B.k1[s] = CHUNK_W_GAUSS + (area + 31u) / 32u;  // the sorted keys end in k0: k1 is free
}

// From the exclusive prefix of the weights: chunk c = the positions whose
// prefix lies in [c W / C, (c + 1) W / C).  Prefixes strictly increase (each
// weight >= 1), so the chunk of a position never decreases; position s opens
// the chunks between its predecessor's and its own.  cstart[C] = V.
__global__ void __launch_bounds__(256)
chunk_bounds_kernel(const BinViews bv) {
  const BinView &B = bv.v[blockIdx.y];
  const uint32_t *prefix = B.k1;
  uint32_t *cstart = B.cstart;
  const uint32_t V = B.counters[CI_V], C = B.counters[CI_C];
  const unsigned long long W = B.counters[CI_W];
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V || W == 0) return;
  const uint32_t cs = (uint32_t)((unsigned long long)prefix[s] * C / W);
  const uint32_t cp = s > 0 ? (uint32_t)((unsigned long long)prefix[s - 1] * C / W) : 0u;
  for (uint32_t c = (s > 0 ? cp + 1 : 0u); c <= cs; ++c) cstart[c] = s;
  if (s == V - 1)
    for (uint32_t c = cs + 1; c <= C; ++c) cstart[c] = V;
}

// ---- counting and emission: one warp per (chunk, band of tile rows) -------
// A band is R consecutive rows of tiles (R * gx <= ~1024 tiles).

// Per-(tile, chunk) counts of one (chunk, band of tile rows) without walking
// the instances: every Gaussian whose rectangle meets the band adds +1 / -1
// at the four corners of its rectangle clipped to the band, in a 2D
// difference grid of (R + 1) x (gx + 1) cells (shared-memory atomics, the 32
// Gaussians of a group in parallel); inclusive prefix sums along the rows and
// then the columns turn it into the counts of the band's tiles.  Work per
// warp: 4 updates per Gaussian plus 2 passes over the band's tiles, instead
// of one visit per instance.  Indices and rectangles are loaded one group
// ahead.
__global__ void __launch_bounds__(32)
count_kernel(const BinViews bv) {
  extern __shared__ int dgrid[];
  const BinView &Bv = bv.v[blockIdx.y];
  const Bands bd = Bv.bd;
  const uint32_t C = Bv.counters[CI_C];
  const uint32_t c = blockIdx.x / (uint32_t)bd.nb;
  const int b = (int)(blockIdx.x - c * (uint32_t)bd.nb);
  if (c >= C) return;
  const int lane = threadIdx.x;
  const int ys = b * bd.R, ye = min(bd.gy, ys + bd.R), R = ye - ys;
  const int W = bd.gx + 1;
  for (int i = lane; i < (R + 1) * W; i += 32) dgrid[i] = 0;
  __syncwarp();
  const uint32_t s0 = Bv.cstart[c], s1 = Bv.cstart[c + 1];
  const float4 none = make_float4(0.f, 0.f, 0.f, 0.f);
  bool vA = s0 + lane < s1;
  float4 rA = vA ? Bv.feat[3 * Bv.v0[s0 + lane] + 2] : none;
  for (uint32_t g0 = s0; g0 < s1; g0 += 32) {
    const float4 r = rA;
    const bool v = vA;
    vA = g0 + 32 + lane < s1;
    rA = vA ? Bv.feat[3 * Bv.v0[g0 + 32 + lane] + 2] : none;
    int x0, y0, x1, y1;
    unpack_rect(r, x0, y0, x1, y1);
    const int cy0 = max(y0, ys) - ys, cy1 = min(y1, ye) - ys;
    if (v && cy0 < cy1 && x0 < x1) {
      atomicAdd(&dgrid[cy0 * W + x0], 1);
      atomicAdd(&dgrid[cy0 * W + x1], -1);
      atomicAdd(&dgrid[cy1 * W + x0], -1);
      atomicAdd(&dgrid[cy1 * W + x1], 1);
    }
  }
  __syncwarp();
  for (int row = 0; row < R; ++row) {  // inclusive prefix along each row, 32 columns at a time
    int carry = 0;
    for (int xb = 0; xb < bd.gx; xb += 32) {
      const int x = xb + lane;
      int val = x < bd.gx ? dgrid[row * W + x] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(FULL, val, o);
        if (lane >= o) val += u;
      }
      val += carry;
      if (x < bd.gx) dgrid[row * W + x] = val;
      carry = __shfl_sync(FULL, val, 31);
    }
  }
  __syncwarp();
  for (int x = lane; x < bd.gx; x += 32) {  // inclusive prefix along each column -> counts
    int run = 0;
    for (int row = 0; row < R; ++row) {
      run += dgrid[row * W + x];
      Bv.cmat[(size_t)c * (bd.gx * bd.gy) + (ys + row) * bd.gx + x] = (uint32_t)run;
    }
  }
}

// Emission.  The band's running slots live in shared memory (R * gx words),
// starting at the first list position of each (tile, this chunk): tile base
// + the counts of the earlier chunk segments + the offset within this
// chunk's segment.  The warp walks its chunk's Gaussians in depth order, 32
// at a time (lane i holds Gaussian g0 + i; indices and rectangles loaded two
// and one groups ahead), selects by ballot the ones whose rectangle meets the
// band and visits each one's tiles within the band, its lanes spread over
// them, appending the Gaussian index.  One Gaussian covers each tile once, so
// within a Gaussian the lanes touch distinct slots and a plain
// read/modify/write suffices; __syncwarp orders consecutive Gaussians.
__global__ void __launch_bounds__(32)
emit_kernel(const BinViews bv) {
  extern __shared__ uint32_t slot[];
  const BinView &Bv = bv.v[blockIdx.y];
  const Bands bd = Bv.bd;
  const float4 *__restrict__ feat = Bv.feat;
  const uint32_t *__restrict__ order = Bv.v0;
  uint32_t *__restrict__ counters = Bv.counters;
  uint32_t *__restrict__ cmat = Bv.cmat;
  uint32_t *__restrict__ point_list = Bv.point_list;
  const uint32_t K_alloc = Bv.K_alloc;
  const uint32_t C = counters[CI_C];
  const uint32_t c = blockIdx.x / (uint32_t)bd.nb;
  const int b = (int)(blockIdx.x - c * (uint32_t)bd.nb);
  if (c >= C) return;
  const int lane = threadIdx.x;
  const int ys = b * bd.R, ye = min(bd.gy, ys + bd.R);
  const int t0 = ys * bd.gx, nt = (ye - ys) * bd.gx;
  const uint32_t s0 = Bv.cstart[c], s1 = Bv.cstart[c + 1];
  const uint64_t keep = l2_policy_last();
  // an overflowed view (instances above the list capacity) emits nothing
  if (s0 >= s1 || (counters[CI_STATUS] & ST_OVERFLOW)) return;
  {
    const uint64_t once = l2_policy_first();
    const int T = bd.gx * bd.gy;
    const uint32_t *off = cmat + (size_t)c * T + t0;
    const uint32_t *tb = Bv.tbase + t0;
    const uint32_t *sp = Bv.segpre + (size_t)(c / seg_len(C, CHUNK_SEGS)) * T + t0;
    int i = lane;
    for (; i + 96 < nt; i += 128) {
      uint32_t a[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        a[u] = ld_hint(off + i + 32 * u, once) + tb[i + 32 * u] + sp[i + 32 * u];
#pragma unroll
      for (int u = 0; u < 4; ++u) slot[i + 32 * u] = a[u];
    }
    for (; i < nt; i += 32) slot[i] = ld_hint(off + i, once) + tb[i] + sp[i];
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
      const uint32_t idi = __shfl_sync(FULL, id, i);
      const int bx = (int)(xyi & 0xffffu), by = (int)(xyi >> 16);
      const int rw = (int)(wai & 0xffffu), area = (int)(wai >> 16);
      RectWalk it(lane, rw, mgi);
      const int o = by * bd.gx + bx;
      int j = lane;
      // four, then two tiles per step (distinct slots: independent read/modify/writes)
      for (; j + 96 < area; j += 128) {
        int a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          a[u] = o + it.row * bd.gx + it.col;
          it.next();
        }
        uint32_t p[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) p[u] = slot[a[u]];
#pragma unroll
        for (int u = 0; u < 4; ++u) slot[a[u]] = p[u] + 1u;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (p[u] < K_alloc) st_hint(point_list + p[u], idi, keep); else bad = true;
        }
      }
      for (; j + 32 < area; j += 64) {
        const int a0 = o + it.row * bd.gx + it.col;
        it.next();
        const int a1 = o + it.row * bd.gx + it.col;
        it.next();
        const uint32_t p0 = slot[a0], p1 = slot[a1];
        slot[a0] = p0 + 1u;
        slot[a1] = p1 + 1u;
        if (p0 < K_alloc) st_hint(point_list + p0, idi, keep); else bad = true;
        if (p1 < K_alloc) st_hint(point_list + p1, idi, keep); else bad = true;
      }
      if (j < area) {
        const int a0 = o + it.row * bd.gx + it.col;
        const uint32_t p0 = slot[a0];
        slot[a0] = p0 + 1u;
        if (p0 < K_alloc) st_hint(point_list + p0, idi, keep); else bad = true;
      }
      __syncwarp();
    }
  }
  if (bad) atomicOr(&counters[CI_STATUS], ST_BOUNDS);
}

// Within-tile offsets of every (tile, chunk).  A block takes 32 tiles (the
// lanes: chunk-major storage makes each step a coalesced 128-byte row
// segment) and CHUNK_SEGS contiguous chunk segments (the warps), so a view
// of 4,056 tiles keeps ~4,000 warps busy.  Each thread writes the exclusive
// prefix of its segment in place; the segment totals give, per tile,
// segpre[s][t] (the counts of the earlier segments) and the tile total
// tbase[t].  Offset of (t, c) = scanned tbase[t] + segpre[seg(c)][t] +
// cmat[c][t].
__global__ void __launch_bounds__(32 * CHUNK_SEGS)
tile_scan_kernel(const BinViews bv) {
  __shared__ uint32_t segsum[CHUNK_SEGS][32];
  const BinView &B = bv.v[blockIdx.y];
  const int T = B.bd.gx * B.bd.gy;
  if ((int)blockIdx.x * 32 >= T) return;  // block-uniform
  const int lane = threadIdx.x & 31, seg = threadIdx.x >> 5;
  const int t = blockIdx.x * 32 + lane;
  const uint32_t C = B.counters[CI_C], L = seg_len(C, CHUNK_SEGS);
  const uint32_t c0 = min(C, seg * L), c1 = min(C, c0 + L);
  uint32_t *col = B.cmat + t;
  uint32_t run = 0;
  if (t < T) {
    uint32_t c = c0;
    for (; c + 16 <= c1; c += 16) {
      uint32_t x[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) x[u] = col[(size_t)(c + u) * T];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        col[(size_t)(c + u) * T] = run;
        run += x[u];
      }
    }
    for (; c < c1; ++c) {
      const uint32_t x = col[(size_t)c * T];
      col[(size_t)c * T] = run;
      run += x;
    }
  }
  segsum[seg][lane] = run;
  __syncthreads();
  if (t < T) {
    uint32_t pre = 0;
    for (int q = 0; q < seg; ++q) pre += segsum[q][lane];
    B.segpre[(size_t)seg * T + t] = pre;
    if (seg == CHUNK_SEGS - 1) B.tbase[t] = pre + run;
  }
}

// Tile ranges from the scanned tile bases.  When the instances exceed the
// list capacity (capacity-bounded callers), every range is left empty and
// the overflow bit is set, so no kernel reads past the list buffer.
__global__ void ranges_kernel(const BinViews bv) {
  const BinView &B = bv.v[blockIdx.y];
  const int T = B.bd.gx * B.bd.gy;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  uint32_t *counters = B.counters;
  const uint32_t K = counters[CI_K];
  const bool over = K > B.K_cap || (counters[CI_STATUS] & ST_OVERFLOW);
  if (over && t == 0) atomicOr(&counters[CI_STATUS], ST_OVERFLOW);
  uint2 r = make_uint2(0u, 0u);
  if (B.P > 0 && !over) {
    const uint32_t a = B.tbase[t];
    const uint32_t e = (t + 1 < T) ? B.tbase[t + 1] : K;
    if (e > a) r = make_uint2(a, e);
    atomicMax(&counters[CI_MAXLIST], e - a);
  }
  B.ranges[t] = r;
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

uint32_t count_grid_bytes(const Bands &bd) { return (uint32_t)((bd.R + 1) * (bd.gx + 1) * 4); }

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
  if (pl.smem > 220 * 1024 || count_grid_bytes(pl.bd) > 220 * 1024) {
    dmgs_host::set_error("image too large: a row of %d tiles exceeds the binning kernels' shared memory", gx);
    return DMGS_ERR_ARG;
  }
  int dev = 0;
  DMGS_CUDA(cudaGetDevice(&dev));
  thread_local int cached_dev = -1;
  thread_local size_t cached_smem = 0;
  thread_local int cached_resident = 0;
  if (dev != cached_dev || pl.smem != cached_smem) {
    const size_t csm = count_grid_bytes(pl.bd);
    // raised only (a launch uses its largest view), shared by every host thread
    const size_t need = std::max(pl.smem, csm);
    if (int r = dmgs_host::raise_smem_limit((const void *)count_kernel, need)) return r;
    if (int r = dmgs_host::raise_smem_limit((const void *)emit_kernel, need)) return r;
    int sms = 0, a = 0, b = 0;
    DMGS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DMGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, count_kernel, 32, csm));
    DMGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, emit_kernel, 32, pl.smem));
    cached_dev = dev;
    cached_smem = pl.smem;
    cached_resident = std::max(1, std::min(a, b)) * sms;
  }
  pl.cmax = (uint32_t)std::max(1, std::min(CHUNK_COUNT_MAX, cached_resident / pl.bd.nb));
  return DMGS_OK;
}

}  // namespace

namespace {

// Scan of one array per view: host bound n_max (the launch size), device
// length *n_dev when given.
int launch_scan_views(const ScanViews &sv, cudaStream_t s) {
  uint32_t n_max = 0;
  for (int v = 0; v < sv.n; ++v) n_max = std::max(n_max, sv.v[v].n_max);
  const dim3 one(1, sv.n);
  if (n_max <= (uint32_t)SCAN_TILE * 4) {
    dmgs_host::note_launch(), scan_single_kernel<<<one, SCAN_THREADS, 0, s>>>(sv, 0);
    DMGS_LAUNCH_CHECK("scan_single_kernel");
    return DMGS_OK;
  }
  const dim3 grid((n_max + SCAN_TILE - 1) / SCAN_TILE, sv.n);
  dmgs_host::note_launch(), scan_reduce_kernel<<<grid, SCAN_THREADS, 0, s>>>(sv);
  DMGS_LAUNCH_CHECK("scan_reduce_kernel");
  dmgs_host::note_launch(), scan_single_kernel<<<one, SCAN_THREADS, 0, s>>>(sv, 1);
  DMGS_LAUNCH_CHECK("scan_single_kernel");
  dmgs_host::note_launch(), scan_down_kernel<<<grid, SCAN_THREADS, 0, s>>>(sv);
  DMGS_LAUNCH_CHECK("scan_down_kernel");
  return DMGS_OK;
}

template <typename F>
ScanViews scan_views(const BinViews &bv, F &&f) {
  ScanViews sv;
  sv.n = bv.n;
  for (int v = 0; v < bv.n; ++v) sv.v[v] = f(bv.v[v]);
  return sv;
}

}  // namespace

int launch_scan1(uint32_t *data, uint32_t n, uint32_t *part, uint32_t *total_out,
                 uint32_t *status, cudaStream_t s) {
  ScanViews sv;
  sv.n = 1;
  sv.v[0] = ScanView{data, nullptr, n, part, total_out, status};
  return launch_scan_views(sv, s);
}

size_t scan_part_words(uint32_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

int make_bin_view(const GeomLayout &L, char *geom, uint32_t K_cap, char *point_list,
                  uint32_t K_alloc, BinView &B) {
  BandPlan pl;
  if (int r = band_plan(L.gx, L.gy, pl)) return r;
  B.P = L.P;
  B.nb_pre = L.nb_pre;
  B.nb_radix = L.nb_radix;
  B.n_rhist_max = (uint32_t)L.n_rhist_max;
  B.n_cmat_max = (uint32_t)L.n_cmat_max;
  B.flags = reinterpret_cast<const uint8_t *>(geom + L.flags);
  B.feat = reinterpret_cast<const float4 *>(geom + L.feat);
  B.blkcnt = reinterpret_cast<uint32_t *>(geom + L.blkcnt);
  B.counters = reinterpret_cast<uint32_t *>(geom + L.counters);
  B.part = reinterpret_cast<uint32_t *>(geom + L.scanpart);
  B.k0 = reinterpret_cast<uint32_t *>(geom + L.dkey0);
  B.k1 = reinterpret_cast<uint32_t *>(geom + L.dkey1);
  B.v0 = reinterpret_cast<uint32_t *>(geom + L.dval0);
  B.v1 = reinterpret_cast<uint32_t *>(geom + L.dval1);
  B.rhist = reinterpret_cast<uint32_t *>(geom + L.rhist);
  B.cmat = reinterpret_cast<uint32_t *>(geom + L.cmat);
  B.cstart = reinterpret_cast<uint32_t *>(geom + L.cstart);
  B.tbase = reinterpret_cast<uint32_t *>(geom + L.tbase);
  B.segpre = reinterpret_cast<uint32_t *>(geom + L.segpre);
  B.ranges = reinterpret_cast<uint2 *>(geom + L.ranges);
  B.point_list = reinterpret_cast<uint32_t *>(point_list);
  B.K_cap = K_cap;
  B.K_alloc = K_alloc;
  B.bd = pl.bd;
  B.cmax = pl.cmax;
  B.smem = (uint32_t)pl.smem;
  return DMGS_OK;
}

int launch_binning_geometry(const BinViews &bv, cudaStream_t s) {
  if (bv.n < 1) return DMGS_OK;
  int nb_pre = 0, nb_radix = 0, P = 0, T = 0;
  uint32_t smem = 0, count_smem = 0, band_blocks = 0;
  for (int v = 0; v < bv.n; ++v) {
    const BinView &B = bv.v[v];
    nb_pre = std::max(nb_pre, B.nb_pre);
    nb_radix = std::max(nb_radix, B.nb_radix);
    P = std::max(P, B.P);
    T = std::max(T, B.bd.gx * B.bd.gy);
    smem = std::max(smem, B.smem);
    count_smem = std::max(count_smem, count_grid_bytes(B.bd));
    band_blocks = std::max(band_blocks, B.cmax * (uint32_t)B.bd.nb);
  }
  const int nv = bv.n;
  if (P > 0) {
    DMGS_TIMED(K_BIN_COMPACT, s, {
      int r = launch_scan_views(scan_views(bv, [](const BinView &B) {
        return ScanView{B.blkcnt, nullptr, (uint32_t)B.nb_pre, B.part, B.counters + CI_V, B.counters};
      }), s);
      if (r != DMGS_OK) return r;
      dmgs_host::note_launch(), compact_kernel<<<dim3(nb_pre, nv), PRE_BLOCK, 0, s>>>(bv);
    });
    DMGS_LAUNCH_CHECK("compact_kernel");
  }
  dmgs_host::note_launch(), params_kernel<<<1, 32, 0, s>>>(bv);
  DMGS_LAUNCH_CHECK("params_kernel");
  if (P > 0) {
    DMGS_TIMED(K_BIN_SORT, s, {
      const ScanViews hs = scan_views(bv, [](const BinView &B) {
        return ScanView{B.rhist, B.counters + CI_NRH, B.n_rhist_max, B.part, nullptr, nullptr};
      });
      for (int pass = 0; pass < 4; ++pass) {
        dmgs_host::note_launch(), radix_hist_kernel<<<dim3(nb_radix, nv), RADIX_BLOCK, 0, s>>>(bv, pass);
        int r = launch_scan_views(hs, s);
        if (r != DMGS_OK) return r;
        dmgs_host::note_launch(), radix_scatter_kernel<<<dim3(nb_radix, nv), RADIX_BLOCK, 0, s>>>(bv, pass);
      }
    });  // four passes: the sorted order ends in (k0, v0)
    DMGS_LAUNCH_CHECK("radix_sort");
    DMGS_TIMED(K_BIN_COUNT, s, {
      dmgs_host::note_launch(), chunk_weight_kernel<<<dim3(nb_pre, nv), 256, 0, s>>>(bv);
      int r = launch_scan_views(scan_views(bv, [](const BinView &B) {
        return ScanView{B.k1, B.counters + CI_V, (uint32_t)B.P, B.part, B.counters + CI_W, B.counters};
      }), s);
      if (r != DMGS_OK) return r;
      dmgs_host::note_launch(), chunk_bounds_kernel<<<dim3(nb_pre, nv), 256, 0, s>>>(bv);
      dmgs_host::note_launch(), count_kernel<<<dim3(band_blocks, nv), 32, count_smem, s>>>(bv);
    });
    DMGS_LAUNCH_CHECK("tile_count");
  }
  DMGS_TIMED(K_BIN_SCAN, s, {
    if (P > 0) {
      dmgs_host::note_launch(), tile_scan_kernel<<<dim3((T + 31) / 32, nv), 32 * CHUNK_SEGS, 0, s>>>(bv);
      int r = launch_scan_views(scan_views(bv, [](const BinView &B) {
        return ScanView{B.tbase, nullptr, (uint32_t)(B.bd.gx * B.bd.gy), B.part, B.counters + CI_K,
                        B.counters};
      }), s);
      if (r != DMGS_OK) return r;
    }
    dmgs_host::note_launch(), ranges_kernel<<<dim3((T + 255) / 256, nv), 256, 0, s>>>(bv);
  });
  DMGS_LAUNCH_CHECK("ranges_kernel");
  return DMGS_OK;
}

int launch_emit(const BinViews &bv, cudaStream_t s) {
  uint32_t smem = 0, band_blocks = 0;
  bool any = false;
  for (int v = 0; v < bv.n; ++v) {
    const BinView &B = bv.v[v];
    if (B.P <= 0 || B.K_alloc == 0) continue;
    any = true;
    smem = std::max(smem, B.smem);
    band_blocks = std::max(band_blocks, B.cmax * (uint32_t)B.bd.nb);
  }
  if (!any) return DMGS_OK;
  DMGS_TIMED(K_BIN_EMIT, s,
             dmgs_host::note_launch(), emit_kernel<<<dim3(band_blocks, bv.n), 32, smem, s>>>(bv));
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
