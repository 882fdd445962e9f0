// binning.cu — (tile, Gaussian) lists ordered by depth, without sorting the
// instance list.
//
// The reference pipeline (duplicateWithKeys -> radix sort of the 64-bit
// (tile << 32 | depth_bits) instance keys -> identifyTileRanges) yields, per
// tile, the covering Gaussians in depth order, ties in Gaussian-index order.
// The same lists are produced here with work linear in the visible Gaussians
// V, their (Gaussian, tile row) pairs K1 and the instances K:
//
//   1. compact   the visible Gaussians in index order: (depth_bits, index);
//   2. sort      them by depth bits with a stable LSD radix sort (4 x 8-bit
//                digits) -> depth order, ties in index order;
//   3. chunk     the sorted list is cut into C contiguous chunks of equal
//                work (weight of a Gaussian: CHUNK_W_GAUSS + its tile rows
//                / 16 + its tiles / 64) -> chunk starts; the packed tile rectangles are laid
//                out in sorted order on the way (srect);
//   4. rows      each chunk counts its Gaussians per tile row (a 1D
//                difference array) -> row counts [gy][C], scanned flat into
//                the offsets of the ROW LISTS: per tile row, the Gaussians
//                covering it in depth order, each entry {index, x0 | x1 << 16};
//   5. segments  groups of C / S consecutive chunks (row segments) count
//                their instances per tile (a 2D difference grid over a band
//                of tile rows) -> segment counts [T][S], scanned flat into
//                every (tile, segment)'s list offset, K and the tile ranges;
//   6. emit      one warp per chunk appends its Gaussians to the row lists
//                (the rows of its Gaussians spread over the lanes, ranks of
//                equal rows by bitwise ballots); then one block per (tile row,
//                segment) splits that segment of the row list into its
//                tiles' lists through a shared-memory staging buffer (counts,
//                offsets and ranks per sub-pass) and copies each tile's run
//                out contiguously.
//
// Every step keeps depth order within a tile: chunks and segments are depth
// ranges laid out in depth order, and within a warp the instances are ranked
// in Gaussian order.  Nothing of size K is sorted or read back; the K-sized
// list is written once, in runs, and the row lists (K1 8-byte entries) are
// written once and read once.  The row and segment offsets are small (gy x C
// and T x S words).
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
  for (uint32_t tile = blockIdx.x; tile * (uint32_t)SCAN_TILE < n; tile += gridDim.x) {
    const uint32_t base = tile * SCAN_TILE;
    unsigned long long s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const uint32_t k = base + i * SCAN_THREADS + threadIdx.x;
      if (k < n) s += v.data[k];
    }
    unsigned long long tot;
    block_exclusive_scan<SCAN_THREADS>(s, &tot);
    if (threadIdx.x == 0) v.part[tile] = (uint32_t)tot;
  }
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
  for (uint32_t tile = blockIdx.x; tile * (uint32_t)SCAN_TILE < n; tile += gridDim.x) {
    // blocked: thread i owns elements base + i*ITEMS .. +ITEMS-1
    uint32_t x[SCAN_ITEMS];
    unsigned long long s = 0;
    const uint32_t k0 = tile * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      x[i] = (k0 + i < n) ? v.data[k0 + i] : 0u;
      s += x[i];
    }
    unsigned long long run = block_exclusive_scan<SCAN_THREADS>(s, nullptr) + v.part[tile];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      if (k0 + i < n) v.data[k0 + i] = (uint32_t)run;
      run += x[i];
    }
  }
}

// ---- compaction of visible Gaussians (index order) ----------------------

// Each block compacts CPT preprocess blocks (PRE_BLOCK x CPT Gaussians, CPT
// consecutive per thread, their flag bytes read as one word); the scanned
// per-preprocess-block counts give the block's first output position.
constexpr int CPT = 4;

__global__ void __launch_bounds__(PRE_BLOCK)
compact_kernel(const BinViews bv) {
  const BinView &B = bv.v[blockIdx.y];
  const int base = blockIdx.x * PRE_BLOCK * CPT;
  if (base >= B.P) return;  // block-uniform
  const int i0 = base + threadIdx.x * CPT;
  uint32_t f4 = 0u;
  if (i0 + CPT <= B.P) {
    f4 = *reinterpret_cast<const uint32_t *>(B.flags + i0);  // i0 % 4 == 0, the array 256-B aligned
  } else {
#pragma unroll
    for (int k = 0; k < CPT; ++k)
      if (i0 + k < B.P) f4 |= (uint32_t)B.flags[i0 + k] << (8 * k);
  }
  uint32_t vis = 0u;
#pragma unroll
  for (int k = 0; k < CPT; ++k) vis |= ((f4 >> (8 * k)) & FLAG_VISIBLE) ? 1u << k : 0u;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int c = __popc(vis);
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += u;
  }
  __shared__ int wsum[PRE_BLOCK / 32];
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  uint32_t pos = B.blkcnt[blockIdx.x * CPT] + (uint32_t)(incl - c);
  for (int w = 0; w < wid; ++w) pos += (uint32_t)wsum[w];
  const float *feat = reinterpret_cast<const float *>(B.feat);
  for (uint32_t m = vis; m; m &= m - 1) {
    const int idx = i0 + __ffs(m) - 1;
    B.k0[pos] = __float_as_uint(feat[12 * (size_t)idx + 9]);  // depth: record float 9
    B.v0[pos] = (uint32_t)idx;
    ++pos;
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
  counters[CI_NRC] = (uint32_t)B.gy * C;
}

// ---- stable LSD radix sort of (depth_bits, index), 8 bits per pass -------

__global__ void __launch_bounds__(RADIX_BLOCK)
radix_hist_kernel(const BinViews bv, int pass) {
  const BinView &B = bv.v[blockIdx.y];
  const uint32_t *keys = (pass & 1) ? B.k1 : B.k0;
  const int shift = 8 * pass;
  const uint32_t V = B.counters[CI_V], nbr = B.counters[CI_NBR];
  __shared__ uint32_t h[256];
  for (uint32_t b = blockIdx.x; b < nbr; b += gridDim.x) {  // key tiles of RADIX_TILE
    h[threadIdx.x] = 0;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RADIX_ITEMS; ++i) {
      const uint32_t k = b * RADIX_TILE + i * RADIX_BLOCK + threadIdx.x;
      if (k < V) atomicAdd(&h[(keys[k] >> shift) & 255u], 1u);
    }
    __syncthreads();
    B.rhist[threadIdx.x * nbr + b] = h[threadIdx.x];  // digit-major
    __syncthreads();
  }
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
  __shared__ uint32_t wh[RADIX_BLOCK / 32][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint32_t b = blockIdx.x; b < nbr; b += gridDim.x) {  // key tiles of RADIX_TILE
    for (int i = threadIdx.x; i < (RADIX_BLOCK / 32) * 256; i += RADIX_BLOCK) (&wh[0][0])[i] = 0u;
    __syncthreads();
    uint32_t key[RADIX_ITEMS], val[RADIX_ITEMS];
    int dig[RADIX_ITEMS];
    unsigned peers[RADIX_ITEMS];
    const uint32_t base = b * RADIX_TILE + w * (32 * RADIX_ITEMS);
#pragma unroll
    for (int r = 0; r < RADIX_ITEMS; ++r) {
      const uint32_t k = base + r * 32 + lane;
      const bool ok = k < V;
      key[r] = ok ? kin[k] : 0u;
      val[r] = ok ? vin[k] : 0u;
      dig[r] = ok ? (int)((key[r] >> shift) & 255u) : 256;
      peers[r] = digit_peers(dig[r]);
      if (dig[r] < 256 && lane == __ffs(peers[r]) - 1) wh[w][dig[r]] += __popc(peers[r]);
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
      uint32_t pos = 0;
      if (dig[r] < 256) pos = wh[w][dig[r]] + __popc(peers[r] & lanemask_lt());
      __syncwarp();
      if (dig[r] < 256) {
        kout[pos] = key[r];
        vout[pos] = val[r];
        if (lane == __ffs(peers[r]) - 1) wh[w][dig[r]] += __popc(peers[r]);
      }
      __syncwarp();
    }
    __syncthreads();  // wh is cleared for the next tile
  }
}

// ---- packed rectangles and shared helpers ---------------------------------

// rect = (x0 | y0 << 16, x1 | y1 << 16): tiles [x0, x1) x [y0, y1)
__device__ __forceinline__ void unpack_rect(uint2 r, int &x0, int &y0, int &x1, int &y1) {
  x0 = (int)(r.x & 0xffffu); y0 = (int)(r.x >> 16); x1 = (int)(r.y & 0xffffu); y1 = (int)(r.y >> 16);
}

// Inclusive warp prefix sum.
__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Balanced expansion: lane i holds an item with n_i instances (exclusive
// prefix excl_i over the lanes); instance q of the group (item-major order)
// belongs to the largest lane o with excl_o <= q.  Five shuffles.
__device__ __forceinline__ int expansion_owner(int excl, int q) {
  int o = 0;
#pragma unroll
  for (int st = 16; st > 0; st >>= 1) {
    const int e = __shfl_sync(FULL, excl, o + st);
    if (e <= q) o += st;
  }
  return o;
}

// Lanes of `act` whose value v (< 2^nbits) equals this lane's: one ballot
// per bit.
__device__ __forceinline__ unsigned value_peers(int v, int nbits, unsigned act) {
  unsigned m = act;
  for (int b = 0; b < nbits; ++b) {
    const bool bit = (v >> b) & 1;
    const unsigned bb = __ballot_sync(FULL, bit);
    m &= bit ? bb : ~bb;
  }
  return m;
}

__device__ __forceinline__ int bits_for(int n) { return n > 1 ? 32 - __clz(n - 1) : 1; }

// First chunk of row segment sg (of S) when the view has C chunks.
__device__ __forceinline__ uint32_t seg_chunk(int sg, uint32_t C, int S) {
  return (uint32_t)((unsigned long long)sg * C / (unsigned)S);
}

// ---- step 3: equal-work chunks of the depth-sorted list --------------------

// Weight of sorted position s: the work its Gaussian costs the binning
// kernels (a fixed part, one per 16 covered tile rows for the row lists and
// one per 64 covered tiles for the tile lists), so that chunks and the row
// segments built from them carry similar numbers of instances; the packed
// rectangle is stored in sorted order for every later pass.
__global__ void __launch_bounds__(256)
chunk_weight_kernel(const BinViews bv) {
  const BinView &B = bv.v[blockIdx.y];
  const uint32_t V = B.counters[CI_V];
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < V; s += gridDim.x * blockDim.x) {
    const float4 f2 = B.feat[3 * B.v0[s] + 2];
    const uint2 r = make_uint2(__float_as_uint(f2.z), __float_as_uint(f2.w));
    B.srect[s] = r;
    int x0, y0, x1, y1;
    unpack_rect(r, x0, y0, x1, y1);
    const uint32_t rows = (uint32_t)(y1 - y0), area = rows * (uint32_t)(x1 - x0);
    B.k1[s] = CHUNK_W_GAUSS + (rows + 15u) / 16u + (area + 63u) / 64u;  // k1 is free: the sorted keys end in k0
  }
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
  if (W == 0) return;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < V; s += gridDim.x * blockDim.x) {
    const uint32_t cs = (uint32_t)((unsigned long long)prefix[s] * C / W);
    const uint32_t cp = s > 0 ? (uint32_t)((unsigned long long)prefix[s - 1] * C / W) : 0u;
    for (uint32_t c = (s > 0 ? cp + 1 : 0u); c <= cs; ++c) cstart[c] = s;
    if (s == V - 1)
      for (uint32_t c = cs + 1; c <= C; ++c) cstart[c] = V;
  }
}

// ---- step 4: row counts, one warp per chunk ---------------------------------

// Gaussians of chunk c per tile row: +1 at the first row and -1 after the
// last of every rectangle in a difference array over the rows, then a
// prefix sum.  Written row-major [gy][C] so that one flat exclusive scan
// gives every (row, chunk)'s offset in the concatenated row lists.
__global__ void __launch_bounds__(32)
row_count_kernel(const BinViews bv) {
  extern __shared__ int rdiff[];  // gy + 1
  const BinView &B = bv.v[blockIdx.y];
  const uint32_t C = B.counters[CI_C];
  const uint32_t c = blockIdx.x;
  if (c >= C) return;
  const int lane = threadIdx.x, gy = B.gy;
  for (int i = lane; i <= gy; i += 32) rdiff[i] = 0;
  __syncwarp();
  const uint32_t s0 = B.cstart[c], s1 = B.cstart[c + 1];
  for (uint32_t s = s0 + lane; s < s1; s += 32) {
    int x0, y0, x1, y1;
    unpack_rect(B.srect[s], x0, y0, x1, y1);
    if (x0 < x1 && y0 < y1) {
      atomicAdd(&rdiff[y0], 1);
      atomicAdd(&rdiff[y1], -1);
    }
  }
  __syncwarp();
  int carry = 0;
  for (int rb = 0; rb < gy; rb += 32) {
    const int r = rb + lane;
    const int v = warp_incl_scan(r < gy ? rdiff[r] : 0, lane) + carry;
    if (r < gy) B.rcnt[(size_t)r * C + c] = (uint32_t)v;
    carry = __shfl_sync(FULL, v, 31);
  }
}

// ---- step 5: segment counts per tile ---------------------------------------

// Instances of every tile of a band of tile rows from row segment sg (the
// Gaussians of chunks [sg C / S, (sg + 1) C / S)): every rectangle clipped to
// the band adds +1 / -1 at its four corners in a 2D difference grid of
// (R + 1) x (gx + 1) cells (shared-memory atomics from every warp of the
// block); prefix sums along the rows, then the columns, give the counts,
// written to cnt2[t * S + sg] — tile-major, so one flat exclusive scan gives
// every (tile, segment)'s list offset.
__global__ void __launch_bounds__(256)
seg_count_kernel(const BinViews bv, int S) {
  extern __shared__ int dg[];
  const BinView &B = bv.v[blockIdx.y];
  if ((int)blockIdx.x >= S * B.nb) return;  // block-uniform
  const int sg = blockIdx.x / B.nb, b = blockIdx.x - sg * B.nb;
  const int gx = B.gx, ys = b * B.R, ye = min(B.gy, ys + B.R), R = ye - ys, Wd = gx + 1;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int i = tid; i < (R + 1) * Wd; i += 256) dg[i] = 0;
  __syncthreads();
  const uint32_t C = B.counters[CI_C];
  uint32_t s0 = 0, s1 = 0;
  if (C > 0) {
    s0 = B.cstart[seg_chunk(sg, C, S)];
    s1 = B.cstart[seg_chunk(sg + 1, C, S)];
  }
  for (uint32_t s = s0 + tid; s < s1; s += 256) {
    int x0, y0, x1, y1;
    unpack_rect(B.srect[s], x0, y0, x1, y1);
    const int cy0 = max(y0, ys) - ys, cy1 = min(y1, ye) - ys;
    if (cy0 < cy1 && x0 < x1) {
      atomicAdd(&dg[cy0 * Wd + x0], 1);
      atomicAdd(&dg[cy0 * Wd + x1], -1);
      atomicAdd(&dg[cy1 * Wd + x0], -1);
      atomicAdd(&dg[cy1 * Wd + x1], 1);
    }
  }
  __syncthreads();
  for (int row = w; row < R; row += 8) {  // inclusive prefix along each row
    int carry = 0;
    for (int xb = 0; xb < gx; xb += 32) {
      const int x = xb + lane;
      const int v = warp_incl_scan(x < gx ? dg[row * Wd + x] : 0, lane) + carry;
      if (x < gx) dg[row * Wd + x] = v;
      carry = __shfl_sync(FULL, v, 31);
    }
  }
  __syncthreads();
  for (int x = tid; x < gx; x += 256) {  // inclusive prefix along each column -> counts
    int run = 0;
    for (int row = 0; row < R; ++row) {
      run += dg[row * Wd + x];
      B.cnt2[((size_t)(ys + row) * gx + x) * S + sg] = (uint32_t)run;
    }
  }
}

// Tile ranges from the scanned segment counts: tile t starts at its first
// segment's offset.  When the instances exceed the list capacity
// (capacity-bounded callers), every range is left empty and the overflow bit
// is set, so no kernel reads past the list buffer.
__global__ void ranges_kernel(const BinViews bv, int S) {
  const BinView &B = bv.v[blockIdx.y];
  const int T = B.gx * B.gy;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  uint32_t *counters = B.counters;
  const uint32_t K = counters[CI_K];
  const bool over = K > B.K_cap || (counters[CI_STATUS] & ST_OVERFLOW);
  if (over && t == 0) atomicOr(&counters[CI_STATUS], ST_OVERFLOW);
  uint2 r = make_uint2(0u, 0u);
  if (B.P > 0 && !over) {
    const uint32_t a = B.cnt2[(size_t)t * S];
    const uint32_t e = (t + 1 < T) ? B.cnt2[(size_t)(t + 1) * S] : K;
    if (e > a) r = make_uint2(a, e);
    atomicMax(&counters[CI_MAXLIST], e - a);
  }
  B.ranges[t] = r;
}

// ---- step 6a: row lists, one warp per chunk --------------------------------

// The chunk's Gaussians are taken 32 at a time (depth order); the (Gaussian,
// row) pairs of the group are spread over the lanes in Gaussian-major order
// (balanced expansion), so pairs of one row rank by their Gaussian's depth
// order: rank = lanes of lower index in the same row (a ballot per bit), then the row's
// running slot (shared memory) advances by the row's pairs.
__global__ void __launch_bounds__(32)
row_emit_kernel(const BinViews bv) {
  extern __shared__ uint32_t rcur[];  // gy running slots
  const BinView &B = bv.v[blockIdx.y];
  uint32_t *counters = B.counters;
  const uint32_t C = counters[CI_C];
  const uint32_t c = blockIdx.x;
  if (c >= C || (counters[CI_STATUS] & ST_OVERFLOW)) return;
  const int lane = threadIdx.x, gy = B.gy, nbits = bits_for(gy);
  for (int r = lane; r < gy; r += 32) rcur[r] = B.rcnt[(size_t)r * C + c];
  __syncwarp();
  const uint32_t s0 = B.cstart[c], s1 = B.cstart[c + 1];
  const uint32_t cap = B.rows_alloc;
  const uint2 *__restrict__ srect = B.srect;
  const uint32_t *__restrict__ order = B.v0;
  uint2 *__restrict__ rowlist = B.rowlist;
  const unsigned lt = lanemask_lt();
  bool bad = false;
  for (uint32_t g0 = s0; g0 < s1; g0 += 32) {
    const uint32_t s = g0 + lane;
    const bool v = s < s1;
    const uint2 rr = v ? srect[s] : make_uint2(0u, 0u);
    const uint32_t id = v ? order[s] : 0u;
    int x0, y0, x1, y1;
    unpack_rect(rr, x0, y0, x1, y1);
    const int n = (x0 < x1 && y0 < y1) ? y1 - y0 : 0;
    const int incl = warp_incl_scan(n, lane);
    const int total = __shfl_sync(FULL, incl, 31);
    const int excl = incl - n;
    const uint32_t xr = (rr.x & 0xffffu) | (rr.y << 16);
    for (int base = 0; base < total; base += 32) {
      const int q = base + lane;
      const bool act = q < total;
      const int o = expansion_owner(excl, q);
      const int row = __shfl_sync(FULL, y0, o) + (q - __shfl_sync(FULL, excl, o));
      const uint32_t ido = __shfl_sync(FULL, id, o);
      const uint32_t xro = __shfl_sync(FULL, xr, o);
      const unsigned amask = total - base >= 32 ? FULL : (1u << (total - base)) - 1u;
      const unsigned peers = value_peers(act ? row : 0, nbits, amask);
      const uint32_t p = act ? rcur[row] + __popc(peers & lt) : 0u;
      __syncwarp();
      if (act) {
        if (p < cap) rowlist[p] = make_uint2(ido, xro); else bad = true;
        if ((peers & lt) == 0u) rcur[row] += __popc(peers);
      }
      __syncwarp();
    }
  }
  if (bad) atomicOr(&counters[CI_STATUS], ST_BOUNDS);
}

// ---- step 6b: tile lists, one block per (tile row, row piece, segment) -----

constexpr int TE_WARPS = 8;
constexpr int TE_THREADS = 32 * TE_WARPS;
constexpr int STAGE_CAP = 8192;    // staged instances per sub-pass
constexpr int TE_PER = 4;          // row-list entries per thread considered for a sub-pass
constexpr int TE_ENTRIES = TE_THREADS * TE_PER;

__host__ __device__ inline size_t tile_emit_smem_words(int nx) {
  return (size_t)nx + (nx + 1) + (size_t)TE_WARPS * (nx + 1) + STAGE_CAP + TE_WARPS +
         (TE_WARPS + 1) + (size_t)TE_WARPS * (2 * (size_t)nx + 32);
}

__device__ __forceinline__ int block_sum_te(int v, int *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  int t = 0;
#pragma unroll
  for (int i = 0; i < TE_WARPS; ++i) t += red[i];
  return t;
}

// The block's entries (one segment of one row list, depth order) are split
// into sub-passes whose instances fit the staging buffer; per sub-pass, each
// warp takes a contiguous slice of entries (about equal instance counts):
// (A) per-warp counts per tile (1D difference array); (B) per tile the
// exclusive prefix over the warps and the tiles' staging offsets, giving
// every warp an absolute staging cursor per tile; (C) the slice's entries in
// order, one at a time, each writing its Gaussian index at the cursor of
// every tile it covers (tile x always by lane x % 32, so no two lanes share
// a cursor and no ranks are needed); (D) each tile's staged run copied to
// the tile's list at its running position (coalesced).
__global__ void __launch_bounds__(TE_THREADS)
tile_emit_kernel(const BinViews bv, int S) {
  extern __shared__ uint32_t te[];
  const BinView &B = bv.v[blockIdx.y];
  const int sg = blockIdx.x % S, rest = blockIdx.x / S;
  const int xs = rest % B.nxs, r = rest / B.nxs;
  if (r >= B.gy) return;  // block-uniform
  uint32_t *counters = B.counters;
  const uint32_t C = counters[CI_C];
  if (C == 0 || (counters[CI_STATUS] & ST_OVERFLOW)) return;
  const uint32_t f0 = seg_chunk(sg, C, S), f1 = seg_chunk(sg + 1, C, S);
  if (f0 >= f1) return;
  const uint32_t e0 = B.rcnt[(size_t)r * C + f0];
  const uint32_t e1 = f1 < C ? B.rcnt[(size_t)r * C + f1]
                             : (r + 1 < B.gy ? B.rcnt[(size_t)(r + 1) * C] : counters[CI_K1]);
  if (e0 >= e1) return;
  const int xa = xs * XSEG, nx = min(B.gx - xa, XSEG), nbits = bits_for(nx);
  uint32_t *tcur = te;                                   // [nx] running list positions
  uint32_t *soff = tcur + nx;                            // [nx + 1] staging offsets
  int *wc = reinterpret_cast<int *>(soff + nx + 1);      // [TE_WARPS][nx + 1] counts / cursors
  uint32_t *stage = reinterpret_cast<uint32_t *>(wc + TE_WARPS * (nx + 1));  // [STAGE_CAP]
  int *red = reinterpret_cast<int *>(stage + STAGE_CAP);  // [TE_WARPS]
  uint32_t *bnd = reinterpret_cast<uint32_t *>(red + TE_WARPS);  // [TE_WARPS + 1] slice starts
  // per warp: start / end bit masks per tile [nx] each (zero between
  // groups) and the Gaussian indices of the current group of 32 entries
  uint32_t *smask = bnd + TE_WARPS + 1;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  uint32_t *sbeg = smask + (size_t)w * (2 * nx + 32), *send = sbeg + nx, *gids = send + nx;
  for (int i = tid; i < TE_WARPS * (2 * nx + 32); i += TE_THREADS) smask[i] = 0u;
  const unsigned lt = lanemask_lt();
  const uint2 *__restrict__ rl = B.rowlist;
  uint32_t *__restrict__ out = B.point_list;
  const uint32_t cap = B.K_alloc;
  for (int x = tid; x < nx; x += TE_THREADS)
    tcur[x] = B.cnt2[((size_t)r * B.gx + xa + x) * S + sg];
  int *wcw = wc + w * (nx + 1);
  bool bad = false;
  auto clip = [&](uint2 en, int &a, int &b) {
    a = max((int)(en.y & 0xffffu), xa) - xa;
    b = min((int)(en.y >> 16), xa + nx) - xa;
  };
  for (uint32_t e = e0; e < e1;) {
    // sub-pass: the longest run of entries whose instances fit the staging
    // buffer (block scan of the clipped widths of up to TE_ENTRIES entries),
    // cut into one contiguous slice per warp at equal instance counts
    const uint32_t navail = min(e1 - e, (uint32_t)TE_ENTRIES);
    int wd[TE_PER];
    int tsum = 0;
#pragma unroll
    for (int k = 0; k < TE_PER; ++k) {
      const uint32_t i = (uint32_t)tid * TE_PER + k;
      int a = 0, b = 0;
      if (i < navail) clip(rl[e + i], a, b);
      wd[k] = max(b - a, 0);
      tsum += wd[k];
    }
    const int tin = warp_incl_scan(tsum, lane);
    __syncthreads();  // red[] and bnd[] of the previous sub-pass are no longer read
    if (lane == 31) red[w] = tin;
    if (tid <= TE_WARPS) bnd[tid] = 0xffffffffu;
    __syncthreads();
    int wbase = 0, itot = 0;
#pragma unroll
    for (int i = 0; i < TE_WARPS; ++i) {
      wbase += i < w ? red[i] : 0;
      itot += red[i];
    }
    int run = wbase + tin - tsum;  // instances before this thread's entries
    int fit = 0;
#pragma unroll
    for (int k = 0; k < TE_PER; ++k) {
      run += wd[k];
      fit += (run <= STAGE_CAP && (uint32_t)tid * TE_PER + k < navail) ? 1 : 0;
    }
    const uint32_t En = max(1u, (uint32_t)block_sum_te(fit, red));
    const int I = min(itot, STAGE_CAP);  // instances of the first En entries (all of them when they fit)
    {
      int ex = wbase + tin - tsum;
#pragma unroll
      for (int k = 0; k < TE_PER; ++k) {
        const uint32_t i = (uint32_t)tid * TE_PER + k;
        if (i < En && I > 0) {
          const int wi = (int)((long long)ex * TE_WARPS / I);
          atomicMin(&bnd[min(wi, TE_WARPS - 1)], i);
        }
        ex += wd[k];
      }
    }
    __syncthreads();
    if (tid == 0) {  // slice starts: first entry whose instances begin in the warp's share
      uint32_t m = En;
      bnd[TE_WARPS] = En;
      for (int i = TE_WARPS - 1; i >= 1; --i) {
        m = min(m, bnd[i]);
        bnd[i] = m;
      }
      bnd[0] = 0;
    }
    __syncthreads();
    const uint32_t sa = e + bnd[w], sb = e + bnd[w + 1];
    // (A) this warp's counts per tile
    for (int i = lane; i <= nx; i += 32) wcw[i] = 0;
    __syncwarp();
    for (uint32_t i = sa + lane; i < sb; i += 32) {
      int a, b;
      clip(rl[i], a, b);
      if (a < b) {
        atomicAdd(&wcw[a], 1);
        atomicAdd(&wcw[b], -1);
      }
    }
    __syncwarp();
    {
      int carry = 0;
      for (int xb = 0; xb < nx; xb += 32) {
        const int x = xb + lane;
        const int v = warp_incl_scan(x < nx ? wcw[x] : 0, lane) + carry;
        if (x < nx) wcw[x] = v;
        carry = __shfl_sync(FULL, v, 31);
      }
    }
    __syncthreads();
    // (B) per tile: prefix over the warps, tile totals, staging offsets
    for (int x = tid; x < nx; x += TE_THREADS) {
      int run = 0;
#pragma unroll
      for (int w2 = 0; w2 < TE_WARPS; ++w2) {
        const int cw = wc[w2 * (nx + 1) + x];
        wc[w2 * (nx + 1) + x] = run;
        run += cw;
      }
      soff[x] = (uint32_t)run;
    }
    __syncthreads();
    if (w == 0) {  // exclusive scan of the tile totals (nx <= XSEG)
      uint32_t carry = 0;
      for (int xb = 0; xb < nx; xb += 32) {
        const int x = xb + lane;
        const int t = x < nx ? (int)soff[x] : 0;
        const int incl = warp_incl_scan(t, lane);
        if (x < nx) soff[x] = carry + (uint32_t)(incl - t);
        carry += (uint32_t)__shfl_sync(FULL, incl, 31);
      }
      if (lane == 0) soff[nx] = carry;
    }
    __syncthreads();
    for (int x = tid; x < nx; x += TE_THREADS) {  // absolute staging cursors of every warp
      const int o = (int)soff[x];
#pragma unroll
      for (int w2 = 0; w2 < TE_WARPS; ++w2) wc[w2 * (nx + 1) + x] += o;
    }
    __syncthreads();
    // (C) stage the slice's instances, 32 entries (depth order) at a time:
    // lane j sets bit j at its entry's first tile a_j in sbeg and at its end
    // b_j in send; inclusive OR-prefixes over the tiles give the entries
    // begun at or before tile x and those ended at or before it, so tile x
    // is covered by M_x = begun & ~ended, which the lane owning x (x % 32)
    // appends in bit (entry) order at its cursor — so a tile's cursor is
    // only ever touched by one lane and entries land in the order they come.
    for (uint32_t g0 = sa; g0 < sb; g0 += 32) {
      const uint32_t i = g0 + lane;
      const uint2 en = i < sb ? rl[i] : make_uint2(0u, 0u);
      int a = 0, b = 0;
      if (i < sb) clip(en, a, b);
      const bool has = a < b;
      gids[lane] = en.x;
      if (has) {
        atomicOr(&sbeg[a], 1u << lane);
        if (b < nx) atomicOr(&send[b], 1u << lane);  // an end at nx is never read
      }
      const int lo = (int)__reduce_min_sync(FULL, has ? (unsigned)a : 0xffffffffu);
      const int hi = (int)__reduce_max_sync(FULL, has ? (unsigned)b : 0u);
      __syncwarp();
      if (lo < hi) {  // warp-uniform; chunks up to the one holding hi (clears send[hi])
        uint32_t cb = 0u, ce = 0u;  // carries of the two OR-prefixes
        for (int xb = lo & ~31; xb <= hi && xb < nx; xb += 32) {
          const int x = xb + lane;
          uint32_t vb = x < nx ? sbeg[x] : 0u, ve = x < nx ? send[x] : 0u;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ub = __shfl_up_sync(FULL, vb, o), ue = __shfl_up_sync(FULL, ve, o);
            if (lane >= o) { vb |= ub; ve |= ue; }
          }
          vb |= cb;
          ve |= ce;
          cb = __shfl_sync(FULL, vb, 31);
          ce = __shfl_sync(FULL, ve, 31);
          if (x < nx) {
            sbeg[x] = 0u;
            send[x] = 0u;
            uint32_t mm = vb & ~ve;
            if (mm) {
              uint32_t p = (uint32_t)wcw[x];
              do {
                const int j = __ffs(mm) - 1;
                mm &= mm - 1;
                if (p < STAGE_CAP) stage[p] = gids[j]; else bad = true;
                ++p;
              } while (mm);
              wcw[x] = (int)p;
            }
          }
        }
      }
      __syncwarp();
    }
    __syncthreads();
    // (D) copy each tile's staged run to its list
    for (int x = w; x < nx; x += TE_WARPS) {
      const uint32_t a = soff[x], n = soff[x + 1] - a, dst = tcur[x];
      for (uint32_t j = lane; j < n; j += 32) {
        if (dst + j < cap) out[dst + j] = stage[a + j]; else bad = true;
      }
      __syncwarp();
      if (lane == 0) tcur[x] = dst + n;
    }
    __syncthreads();
    e += En;
  }
  if (bad) atomicOr(&counters[CI_STATUS], ST_BOUNDS);
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

// Bands of tile rows for the segment counts: about 1024 tiles per band (a
// 4 KB difference grid).
void band_plan(int gx, int gy, int &R, int &nb) {
  R = std::max(1, std::min(gy, 1024 / std::max(gx, 1)));
  nb = (gy + R - 1) / R;
}

size_t seg_grid_bytes(int R, int gx) { return (size_t)(R + 1) * (gx + 1) * 4; }

int device_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return NUM_SMS_HINT;
  thread_local int cached_dev = -1, cached_sms = NUM_SMS_HINT;
  if (dev != cached_dev) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
      cached_sms = sms;
    cached_dev = dev;
  }
  return cached_sms;
}

// Row segments per view for a launch: enough (row, piece, segment) blocks
// for about five waves of the tile emission (short blocks balance uneven
// rows).  A pure function of the views'
// grids and the device, so the geometry and the emission launches of one
// set of views agree.
int seg_plan(const BinViews &bv) {
  long rows = 0;
  for (int v = 0; v < bv.n; ++v) rows += (long)bv.v[v].gy * bv.v[v].nxs;
  const long target = 32L * device_sms();
  const long S = rows > 0 ? (target + rows - 1) / rows : 1;
  return (int)std::max(1L, std::min((long)SEG_MAX, S));
}

// Scan of one array per view: host bound n_max (the launch size), device
// length *n_dev when given.
// Blocks per view for a grid-stride launch over at most `units` work units
// whose actual count is only known on the device: about two resident waves
// of `per_sm` blocks per SM shared by the views, so that a launch sized for
// the worst case does not schedule thousands of blocks that find no work.
int bounded_blocks(size_t units, int nviews, int per_sm) {
  const size_t cap = std::max<size_t>(1, (size_t)2 * device_sms() * per_sm / std::max(nviews, 1));
  return (int)std::max<size_t>(1, std::min(units, cap));
}

int launch_scan_views(const ScanViews &sv, cudaStream_t s) {
  uint32_t n_max = 0;
  for (int v = 0; v < sv.n; ++v) n_max = std::max(n_max, sv.v[v].n_max);
  const dim3 one(1, sv.n);
  if (n_max <= (uint32_t)SCAN_TILE * 4) {
    dmgs_host::note_launch(), scan_single_kernel<<<one, SCAN_THREADS, 0, s>>>(sv, 0);
    DMGS_LAUNCH_CHECK("scan_single_kernel");
    return DMGS_OK;
  }
  const dim3 grid(bounded_blocks((n_max + SCAN_TILE - 1) / SCAN_TILE, sv.n, 2), sv.n);
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

constexpr size_t SMEM_LIMIT = 220 * 1024;

}  // namespace

int launch_scan1(uint32_t *data, uint32_t n, uint32_t *part, uint32_t *total_out,
                 uint32_t *status, cudaStream_t s) {
  ScanViews sv;
  sv.n = 1;
  sv.v[0] = ScanView{data, nullptr, n, part, total_out, status};
  return launch_scan_views(sv, s);
}

size_t scan_part_words(uint32_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

int make_bin_view(const GeomLayout &L, char *geom, uint32_t K_cap, char *bin, uint32_t K_alloc,
                  BinView &B) {
  B.P = L.P;
  B.nb_pre = L.nb_pre;
  B.nb_radix = L.nb_radix;
  B.gx = L.gx;
  B.gy = L.gy;
  band_plan(L.gx, L.gy, B.R, B.nb);
  B.nxs = (L.gx + XSEG - 1) / XSEG;
  const size_t rows_smem = (size_t)(L.gy + 1) * 4;
  if (seg_grid_bytes(B.R, L.gx) > SMEM_LIMIT || rows_smem > SMEM_LIMIT) {
    dmgs_host::set_error("image too large for the binning kernels' shared memory (%d x %d tiles)",
                         L.gx, L.gy);
    return DMGS_ERR_ARG;
  }
  B.n_rhist_max = (uint32_t)L.n_rhist_max;
  B.n_rcnt_max = (uint32_t)L.n_rcnt_max;
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
  B.srect = reinterpret_cast<uint2 *>(geom + L.srect);
  B.cstart = reinterpret_cast<uint32_t *>(geom + L.cstart);
  B.rcnt = reinterpret_cast<uint32_t *>(geom + L.rcnt);
  B.cnt2 = reinterpret_cast<uint32_t *>(geom + L.cnt2);
  B.ranges = reinterpret_cast<uint2 *>(geom + L.ranges);
  // the caller sized the state with bin_layout(K_alloc, ...) (plain form: K
  // row entries) or bin_layout(K_alloc, ..., P) (capacity-bounded forms:
  // fewer); the smaller bound is always inside the buffer
  const BinLayout BL = bin_layout(K_alloc, L.gx * TILE, L.gy * TILE, L.P);
  B.point_list = bin ? reinterpret_cast<uint32_t *>(bin + BL.point_list) : nullptr;
  B.rowlist = bin ? reinterpret_cast<uint2 *>(bin + BL.rowlist) : nullptr;
  B.K_cap = K_cap;
  B.K_alloc = bin ? K_alloc : 0u;
  B.rows_alloc = bin ? (uint32_t)BL.rows : 0u;
  B.cmax = CHUNK_COUNT_MAX;
  return DMGS_OK;
}

int launch_binning_geometry(const BinViews &bv, cudaStream_t s) {
  if (bv.n < 1) return DMGS_OK;
  int nb_pre = 0, nb_radix = 0, P = 0, T = 0, gy = 0, nb = 0;
  uint32_t cmax = 0;
  size_t seg_smem = 0;
  for (int v = 0; v < bv.n; ++v) {
    const BinView &B = bv.v[v];
    nb_pre = std::max(nb_pre, B.nb_pre);
    nb_radix = std::max(nb_radix, B.nb_radix);
    P = std::max(P, B.P);
    T = std::max(T, B.gx * B.gy);
    gy = std::max(gy, B.gy);
    nb = std::max(nb, B.nb);
    cmax = std::max(cmax, B.cmax);
    seg_smem = std::max(seg_smem, seg_grid_bytes(B.R, B.gx));
  }
  const int S = seg_plan(bv);
  const int nv = bv.n;
  // grid-stride kernels over the visible Gaussians (counted on the device)
  const int rgrid = bounded_blocks((size_t)nb_radix, nv, 8);  // key tiles
  const int pgrid = bounded_blocks((size_t)nb_pre, nv, 8);    // blocks of 256 positions
  const size_t rows_smem = (size_t)(gy + 1) * 4;
  if (int r = dmgs_host::raise_smem_limit((const void *)row_count_kernel, rows_smem)) return r;
  if (int r = dmgs_host::raise_smem_limit((const void *)seg_count_kernel, seg_smem)) return r;
  if (P > 0) {
    DMGS_TIMED(K_BIN_COMPACT, s, {
      int r = launch_scan_views(scan_views(bv, [](const BinView &B) {
        return ScanView{B.blkcnt, nullptr, (uint32_t)B.nb_pre, B.part, B.counters + CI_V, B.counters};
      }), s);
      if (r != DMGS_OK) return r;
      dmgs_host::note_launch(), compact_kernel<<<dim3((nb_pre + CPT - 1) / CPT, nv), PRE_BLOCK, 0, s>>>(bv);
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
        dmgs_host::note_launch(), radix_hist_kernel<<<dim3(rgrid, nv), RADIX_BLOCK, 0, s>>>(bv, pass);
        int r = launch_scan_views(hs, s);
        if (r != DMGS_OK) return r;
        dmgs_host::note_launch(), radix_scatter_kernel<<<dim3(rgrid, nv), RADIX_BLOCK, 0, s>>>(bv, pass);
      }
    });  // four passes: the sorted order ends in (k0, v0)
    DMGS_LAUNCH_CHECK("radix_sort");
    DMGS_TIMED(K_BIN_COUNT, s, {
      dmgs_host::note_launch(), chunk_weight_kernel<<<dim3(pgrid, nv), 256, 0, s>>>(bv);
      int r = launch_scan_views(scan_views(bv, [](const BinView &B) {
        return ScanView{B.k1, B.counters + CI_V, (uint32_t)B.P, B.part, B.counters + CI_W, B.counters};
      }), s);
      if (r != DMGS_OK) return r;
      dmgs_host::note_launch(), chunk_bounds_kernel<<<dim3(pgrid, nv), 256, 0, s>>>(bv);
      dmgs_host::note_launch(), row_count_kernel<<<dim3(cmax, nv), 32, rows_smem, s>>>(bv);
      dmgs_host::note_launch(), seg_count_kernel<<<dim3(S * nb, nv), 256, seg_smem, s>>>(bv, S);
    });
    DMGS_LAUNCH_CHECK("tile_count");
    DMGS_TIMED(K_BIN_SCAN, s, {
      int r = launch_scan_views(scan_views(bv, [](const BinView &B) {
        return ScanView{B.rcnt, B.counters + CI_NRC, B.n_rcnt_max, B.part, B.counters + CI_K1,
                        B.counters};
      }), s);
      if (r != DMGS_OK) return r;
      r = launch_scan_views(scan_views(bv, [S](const BinView &B) {
        return ScanView{B.cnt2, nullptr, (uint32_t)(B.gx * B.gy) * (uint32_t)S, B.part,
                        B.counters + CI_K, B.counters};
      }), s);
      if (r != DMGS_OK) return r;
    });
    DMGS_LAUNCH_CHECK("binning scans");
  }
  dmgs_host::note_launch(), ranges_kernel<<<dim3((T + 255) / 256, nv), 256, 0, s>>>(bv, S);
  DMGS_LAUNCH_CHECK("ranges_kernel");
  return DMGS_OK;
}

int launch_emit(const BinViews &bv, cudaStream_t s) {
  int gy = 0, nxs = 0, gxm = 0;
  uint32_t cmax = 0;
  bool any = false;
  for (int v = 0; v < bv.n; ++v) {
    const BinView &B = bv.v[v];
    if (B.P <= 0 || B.K_alloc == 0) continue;
    any = true;
    gy = std::max(gy, B.gy);
    nxs = std::max(nxs, B.nxs);
    gxm = std::max(gxm, std::min(B.gx, XSEG));
    cmax = std::max(cmax, B.cmax);
  }
  if (!any) return DMGS_OK;
  const int S = seg_plan(bv);
  const size_t rows_smem = (size_t)gy * 4;
  const size_t te_smem = tile_emit_smem_words(gxm) * 4;
  if (int r = dmgs_host::raise_smem_limit((const void *)row_emit_kernel, rows_smem)) return r;
  if (int r = dmgs_host::raise_smem_limit((const void *)tile_emit_kernel, te_smem)) return r;
  DMGS_TIMED(K_BIN_ROWS, s,
             dmgs_host::note_launch(), row_emit_kernel<<<dim3(cmax, bv.n), 32, rows_smem, s>>>(bv));
  DMGS_LAUNCH_CHECK("row_emit_kernel");
  DMGS_TIMED(K_BIN_EMIT, s,
             dmgs_host::note_launch(), tile_emit_kernel<<<dim3(gy * nxs * S, bv.n), TE_THREADS, te_smem, s>>>(bv, S));
  DMGS_LAUNCH_CHECK("tile_emit_kernel");
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
