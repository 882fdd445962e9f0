// binning.cu — (tile, Gaussian) instance emission and per-tile depth sort.
//
// The reference pipeline (duplicateWithKeys -> radix sort of 64-bit
// (tile << 32 | depth_bits) keys -> identifyTileRanges) produces, for each
// tile, the list of covering Gaussians ordered by depth with ties in
// Gaussian-index order.  Here the tile boundaries are known before any
// instance is written (tile_start from the difference-grid counts), so:
//   1. scatter: every visible Gaussian claims one slot per covered tile
//      inside that tile's segment (atomic cursor per tile) and writes the
//      unique sort key (depth_bits << 32 | index);
//   2. segment sort: one CTA per tile sorts its segment in shared memory
//      (bitonic network; segments longer than the shared capacity are
//      sorted in chunks and merged through global memory) and writes the
//      Gaussian indices (point_list) and the tile range.
// The result equals the reference's sorted value list and ranges exactly:
// within a tile the key (depth_bits, index) is unique, so the order does
// not depend on which slot an instance claimed.
#include "kernels.cuh"

namespace dmgs {

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SORT_CAP = 4096;  // keys sorted in shared memory at once (32 KB)

__global__ void __launch_bounds__(256)
scatter_kernel(int P, int gx, const float4 *__restrict__ feat,
               uint32_t *__restrict__ cursor, uint64_t *__restrict__ keys, uint32_t K,
               uint32_t *__restrict__ counters) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= P) return;
  const float4 f2 = feat[3 * idx + 2];
  const uint32_t lo = __float_as_uint(f2.z), hi = __float_as_uint(f2.w);
  const int x0 = lo & 0xffff, y0 = lo >> 16, x1 = hi & 0xffff, y1 = hi >> 16;
  if (x1 <= x0 || y1 <= y0) return;
  const uint64_t key = ((uint64_t)__float_as_uint(f2.y) << 32) | (uint32_t)idx;
  for (int y = y0; y < y1; ++y)
    for (int x = x0; x < x1; ++x) {
      const uint32_t pos = atomicAdd(cursor + y * gx + x, 1u);
      if (pos < K) keys[pos] = key;
      else atomicOr(counters, ST_BOUNDS);
    }
}

__global__ void init_cursor_kernel(int T, const uint32_t *__restrict__ tile_start,
                                   uint32_t *__restrict__ cursor) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < T) cursor[t] = tile_start[t];
}

// Ascending bitonic sort of n2 (power of two) keys in shared memory.
__device__ __forceinline__ void bitonic_smem(uint64_t *s, int n2) {
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int p = threadIdx.x; p < (n2 >> 1); p += blockDim.x) {
        const int i = 2 * p - (p & (j - 1));
        const int l = i + j;
        const uint64_t a = s[i], b = s[l];
        const bool up = (i & k) == 0;
        if ((a > b) == up) { s[i] = b; s[l] = a; }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ int lower_bound_u64(const uint64_t *a, int n, uint64_t v) {
  int lo = 0, hi = n;
  while (lo < hi) { const int m = (lo + hi) >> 1; if (a[m] < v) lo = m + 1; else hi = m; }
  return lo;
}
__device__ __forceinline__ int upper_bound_u64(const uint64_t *a, int n, uint64_t v) {
  int lo = 0, hi = n;
  while (lo < hi) { const int m = (lo + hi) >> 1; if (a[m] <= v) lo = m + 1; else hi = m; }
  return lo;
}

__global__ void __launch_bounds__(SORT_THREADS)
segment_sort_kernel(int T, const uint32_t *__restrict__ tile_start, uint64_t *__restrict__ keys,
                    uint64_t *__restrict__ keys_alt, uint32_t *__restrict__ point_list,
                    uint2 *__restrict__ ranges) {
  __shared__ uint64_t s[SORT_CAP];
  const int t = blockIdx.x;
  if (t >= T) return;
  const uint32_t beg = tile_start[t], end = tile_start[t + 1];
  const int n = (int)(end - beg);
  if (threadIdx.x == 0) ranges[t] = n > 0 ? make_uint2(beg, end) : make_uint2(0u, 0u);
  if (n == 0) return;
  uint64_t *seg = keys + beg;
  if (n <= SORT_CAP) {
    int n2 = 2;
    while (n2 < n) n2 <<= 1;
    for (int i = threadIdx.x; i < n2; i += blockDim.x) s[i] = i < n ? seg[i] : ~0ull;
    __syncthreads();
    bitonic_smem(s, n2);
    for (int i = threadIdx.x; i < n; i += blockDim.x) point_list[beg + i] = (uint32_t)s[i];
    return;
  }
  // Long segment: sort SORT_CAP chunks in place, then merge runs pairwise.
  for (int c0 = 0; c0 < n; c0 += SORT_CAP) {
    const int m = min(SORT_CAP, n - c0);
    int n2 = 2;
    while (n2 < m) n2 <<= 1;
    for (int i = threadIdx.x; i < n2; i += blockDim.x) s[i] = i < m ? seg[c0 + i] : ~0ull;
    __syncthreads();
    bitonic_smem(s, n2);
    for (int i = threadIdx.x; i < m; i += blockDim.x) seg[c0 + i] = s[i];
    __syncthreads();
  }
  uint64_t *src = seg, *dst = keys_alt + beg;
  for (int w = SORT_CAP; w < n; w <<= 1) {
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      const int a0 = (e / (2 * w)) * (2 * w);
      const int b0 = a0 + w;
      const int na = min(w, n - a0);
      const int nb = max(0, min(w, n - b0));
      const uint64_t v = src[e];
      int pos;
      if (e < b0) pos = (e - a0) + lower_bound_u64(src + b0, nb, v);
      else pos = (e - b0) + upper_bound_u64(src + a0, na, v);
      dst[a0 + pos] = v;
    }
    __syncthreads();
    uint64_t *tmp = src; src = dst; dst = tmp;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) point_list[beg + i] = (uint32_t)src[i];
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

int launch_scatter(const GeomLayout &L, const char *geom, const BinLayout &B, char *bin,
                   int64_t K, cudaStream_t s) {
  const int T = L.T();
  uint32_t *cursor = reinterpret_cast<uint32_t *>(bin + B.cursor);
  DMGS_TIMED(K_INIT_CURSOR, s, init_cursor_kernel<<<(T + 255) / 256, 256, 0, s>>>(
      T, reinterpret_cast<const uint32_t *>(geom + L.tile_start), cursor));
  DMGS_LAUNCH_CHECK("init_cursor_kernel");
  if (L.P > 0 && K > 0) {
    DMGS_TIMED(K_SCATTER, s, scatter_kernel<<<(L.P + 255) / 256, 256, 0, s>>>(
        L.P, L.gx, reinterpret_cast<const float4 *>(geom + L.feat), cursor,
        reinterpret_cast<uint64_t *>(bin + B.keys), (uint32_t)K,
        reinterpret_cast<uint32_t *>(const_cast<char *>(geom) + L.counters)));
    DMGS_LAUNCH_CHECK("scatter_kernel");
  }
  return DMGS_OK;
}

int launch_segment_sort(const GeomLayout &L, const char *geom, const BinLayout &B, char *bin,
                        int64_t K, cudaStream_t s) {
  (void)K;
  const int T = L.T();
  DMGS_TIMED(K_SEGMENT_SORT, s, segment_sort_kernel<<<T, SORT_THREADS, 0, s>>>(
      T, reinterpret_cast<const uint32_t *>(geom + L.tile_start),
      reinterpret_cast<uint64_t *>(bin + B.keys), reinterpret_cast<uint64_t *>(bin + B.keys_alt),
      reinterpret_cast<uint32_t *>(bin + B.point_list), reinterpret_cast<uint2 *>(bin + B.ranges)));
  DMGS_LAUNCH_CHECK("segment_sort_kernel");
  return DMGS_OK;
}

int launch_debug_keys(const GeomLayout &L, const char *geom, const BinLayout &B, const char *bin,
                      uint64_t *keys, uint32_t *values, cudaStream_t s) {
  DMGS_TIMED(K_DEBUG, s, debug_keys_kernel<<<L.T(), 256, 0, s>>>(
      L.T(), reinterpret_cast<const uint2 *>(bin + B.ranges),
      reinterpret_cast<const uint32_t *>(bin + B.point_list),
      reinterpret_cast<const float4 *>(geom + L.feat), keys, values));
  DMGS_LAUNCH_CHECK("debug_keys_kernel");
  return DMGS_OK;
}

}  // namespace dmgs
