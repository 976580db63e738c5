// primitives.cu -- scan, reductions, histograms and sorts used by convert.cu.
#include <climits>

#include "primitives.cuh"

namespace mgb {
namespace prim {
namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// exclusive scan of one int64 per thread across the block; returns the
// exclusive prefix, *total = block sum
__device__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t s_warp[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t u = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += u;
  }
  if (lane == 31) s_warp[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    int64_t x = lane < nw ? s_warp[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int64_t u = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += u;
    }
    if (lane < nw) s_warp[lane] = x;  // inclusive warp prefix
  }
  __syncthreads();
  const int64_t warp_excl = w ? s_warp[w - 1] : 0;
  *total = s_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_excl + inc - v;
}

template <typename Tin>
__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_sums(const Tin* __restrict__ in, int64_t n,
                                                               int64_t* __restrict__ sums) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t v = 0;
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const int64_t i = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
    if (i < n) v += (int64_t)in[i];
  }
  int64_t total;
  block_exclusive_scan(v, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// exclusive scan of sums[0..nb) in place by one block; total -> *d_total
__global__ void __launch_bounds__(1024) scan_sums(int64_t* sums, int64_t nb, int64_t* d_total) {
  const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
  const int64_t b0 = (int64_t)threadIdx.x * per;
  int64_t local = 0;
  for (int64_t i = b0; i < b0 + per && i < nb; i++) local += sums[i];
  int64_t total;
  int64_t run = block_exclusive_scan(local, &total);
  for (int64_t i = b0; i < b0 + per && i < nb; i++) {
    const int64_t v = sums[i];
    sums[i] = run;
    run += v;
  }
  if (threadIdx.x == 0 && d_total) *d_total = total;
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply(const Tin* __restrict__ in, Tout* __restrict__ out,
                                                           int64_t n, const int64_t* __restrict__ sums) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  int64_t v[SCAN_ITEMS];
  int64_t local = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const int64_t i = base + k;
    v[k] = i < n ? (int64_t)in[i] : 0;
    local += v[k];
  }
  int64_t total;
  int64_t run = block_exclusive_scan(local, &total) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const int64_t i = base + k;
    if (i < n) out[i] = (Tout)run;
    run += v[k];
  }
}

__global__ void fill_i32(int32_t* p, int32_t v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void max_i32_kernel(const int32_t* __restrict__ in, int64_t n, int32_t* out) {
  int32_t m = INT_MIN;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, in[i]);
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void sum_i32_kernel(const int32_t* __restrict__ in, int64_t n, unsigned long long* out) {
  int64_t sacc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    sacc += in[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, (unsigned long long)sacc);
}

// counts[k] += 1 for every key in [0, nbins); few hot keys per CTA are
// counted in shared memory first (CtaHist)
__global__ void histogram_kernel(const int32_t* __restrict__ keys, int64_t n, int32_t* counts, int64_t nbins) {
  MGB_CTA_HIST(h);
  hist_init(h);
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = keys[i];
    if (k >= 0 && k < nbins) hist_add(h, counts, (unsigned long long)k);
  }
  __syncthreads();
  hist_flush(h, counts);
}

__global__ void sorted_flags_kernel(const int32_t* __restrict__ r, const int32_t* __restrict__ c, int64_t n,
                                    int32_t* flag, int32_t* dup) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i + 1 < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r0 = r[i], r1 = r[i + 1];
    if (c == nullptr) {
      if (r0 > r1) *flag = 0;
    } else {
      const int32_t c0 = c[i], c1 = c[i + 1];
      if (r0 > r1 || (r0 == r1 && c0 > c1)) *flag = 0;
      if (dup && r0 == r1 && c0 == c1) *dup = 1;
    }
  }
}

// ---- segmented sort ------------------------------------------------------

constexpr int SEG_SMALL = 32;
constexpr int SEG_MED = 4096;
constexpr int SEG_MED_THREADS = 512;

__global__ void classify_segments(const int32_t* __restrict__ seg, int64_t nseg, int32_t* lists, int64_t cap,
                                  int32_t* counters) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nseg; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t len = seg[i + 1] - seg[i];
    if (len <= 1) continue;
    const int cls = len <= SEG_SMALL ? 0 : (len <= SEG_MED ? 1 : 2);
    const int32_t slot = atomicAdd(counters + cls, 1);
    lists[cls * cap + slot] = (int32_t)i;
  }
}

__global__ void sort_small_segments(uint64_t* keys, const int32_t* __restrict__ seg, const int32_t* __restrict__ list,
                                    const int32_t* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < *count; w += nw) {
    const int32_t s = list[w];
    const int32_t b = seg[s], len = seg[s + 1] - b;
    uint64_t v = lane < len ? keys[b + lane] : ~0ull;
    // bitonic sort across the 32 lanes
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        const uint64_t o = __shfl_xor_sync(0xffffffffu, v, j);
        const bool up = ((lane & k) == 0);
        const bool lower = ((lane & j) == 0);
        const uint64_t mn = v < o ? v : o, mx = v < o ? o : v;
        v = (lower == up) ? mn : mx;
      }
    }
    if (lane < len) keys[b + lane] = v;
  }
}

// bitonic sort of m (power of two, <= SEG_MED) keys in shared memory
__device__ void bitonic_smem(uint64_t* sk, int m) {
  for (int k = 2; k <= m; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const uint64_t a = sk[i], b = sk[p];
          const bool up = ((i & k) == 0);
          if ((a > b) == up) { sk[i] = b; sk[p] = a; }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(SEG_MED_THREADS) sort_medium_segments(uint64_t* keys, const int32_t* __restrict__ seg,
                                                                        const int32_t* __restrict__ list,
                                                                        const int32_t* __restrict__ count) {
  __shared__ uint64_t sk[SEG_MED];
  for (int64_t w = blockIdx.x; w < *count; w += gridDim.x) {
    const int32_t s = list[w];
    const int32_t b = seg[s], len = seg[s + 1] - b;
    int m = 64;
    while (m < len) m <<= 1;
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) sk[i] = i < len ? keys[b + i] : ~0ull;
    __syncthreads();
    bitonic_smem(sk, m);
    for (int i = threadIdx.x; i < len; i += blockDim.x) keys[b + i] = sk[i];
  }
}

// large segments: sort 4096-chunks in shared memory, then merge runs pairwise
// (merge path: each thread emits a contiguous slice of the output)
__device__ int64_t merge_corank(const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb, int64_t k) {
  // number of elements taken from a among the first k outputs (stable: a first on ties)
  int64_t lo = k > nb ? k - nb : 0, hi = k < na ? k : na;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid] <= b[k - mid - 1]) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(SEG_MED_THREADS) sort_large_segments(uint64_t* keys, uint64_t* tmp,
                                                                       const int32_t* __restrict__ seg,
                                                                       const int32_t* __restrict__ list,
                                                                       const int32_t* __restrict__ count) {
  __shared__ uint64_t sk[SEG_MED];
  for (int64_t w = blockIdx.x; w < *count; w += gridDim.x) {
    const int32_t s = list[w];
    const int64_t b = seg[s], len = seg[s + 1] - b;
    uint64_t* src = keys + b;
    uint64_t* dst = tmp + b;
    for (int64_t c0 = 0; c0 < len; c0 += SEG_MED) {
      const int cl = (int)min((int64_t)SEG_MED, len - c0);
      __syncthreads();
      for (int i = threadIdx.x; i < SEG_MED; i += blockDim.x) sk[i] = i < cl ? src[c0 + i] : ~0ull;
      __syncthreads();
      bitonic_smem(sk, SEG_MED);
      for (int i = threadIdx.x; i < cl; i += blockDim.x) src[c0 + i] = sk[i];
    }
    __syncthreads();
    bool in_src = true;
    for (int64_t width = SEG_MED; width < len; width <<= 1) {
      const uint64_t* from = in_src ? src : dst;
      uint64_t* to = in_src ? dst : src;
      for (int64_t a0 = 0; a0 < len; a0 += 2 * width) {
        const int64_t na = min(width, len - a0);
        const int64_t nb = max((int64_t)0, min(width, len - a0 - width));
        const int64_t tot = na + nb;
        const int64_t per = (tot + blockDim.x - 1) / blockDim.x;
        const int64_t k0 = min(tot, (int64_t)threadIdx.x * per), k1 = min(tot, k0 + per);
        const uint64_t* A = from + a0;
        const uint64_t* B = from + a0 + na;
        int64_t ia = merge_corank(A, na, B, nb, k0);
        int64_t ib = k0 - ia;
        for (int64_t k = k0; k < k1; k++) {
          if (ib >= nb || (ia < na && A[ia] <= B[ib])) to[a0 + k] = A[ia++];
          else to[a0 + k] = B[ib++];
        }
      }
      __syncthreads();
      in_src = !in_src;
    }
    if (!in_src)
      for (int64_t i = threadIdx.x; i < len; i += blockDim.x) src[i] = dst[i];
    __syncthreads();
  }
}

__global__ void scatter_row_keys(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols, int64_t n,
                                 int32_t* cursor, uint64_t* keys) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t slot = atomicAdd(cursor + rows[i], 1);
    keys[slot] = ((uint64_t)(uint32_t)cols[i] << 32) | (uint64_t)(uint32_t)i;
  }
}

__global__ void gather_sorted(const uint64_t* __restrict__ keys, const int32_t* __restrict__ rows, int64_t n,
                              int32_t* out_rows, int32_t* out_cols, int32_t* perm) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t key = keys[k];
    const int32_t p = (int32_t)(uint32_t)(key & 0xffffffffull);
    perm[k] = p;
    out_cols[k] = (int32_t)(uint32_t)(key >> 32);
    out_rows[k] = rows[p];
  }
}

}  // namespace

template <typename Tin, typename Tout>
int exclusive_scan(const Tin* in, Tout* out, int64_t n, cudaStream_t s, int64_t* d_total) {
  if (n <= 0) {
    if (d_total) MGB_CUDA_CHECK(cudaMemsetAsync(d_total, 0, sizeof(int64_t), s));
    return MGB_SUCCESS;
  }
  Scratch sc(s);
  const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  int64_t* sums;
  MGB_SCRATCH(sc, sums, nb);
  scan_tile_sums<Tin><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums);
  MGB_LAUNCH_CHECK();
  scan_sums<<<1, 1024, 0, s>>>(sums, nb, d_total);
  MGB_LAUNCH_CHECK();
  scan_apply<Tin, Tout><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template int exclusive_scan<int32_t, int32_t>(const int32_t*, int32_t*, int64_t, cudaStream_t, int64_t*);
template int exclusive_scan<int32_t, int64_t>(const int32_t*, int64_t*, int64_t, cudaStream_t, int64_t*);
template int exclusive_scan<uint8_t, int64_t>(const uint8_t*, int64_t*, int64_t, cudaStream_t, int64_t*);
template int exclusive_scan<uint8_t, int32_t>(const uint8_t*, int32_t*, int64_t, cudaStream_t, int64_t*);

int reduce_max_i32(const int32_t* in, int64_t n, int32_t* d_out, cudaStream_t s) {
  fill_i32<<<1, 32, 0, s>>>(d_out, INT_MIN, 1);
  MGB_LAUNCH_CHECK();
  if (n <= 0) return MGB_SUCCESS;
  max_i32_kernel<<<blocks_for(n, 256, (int64_t)num_sms() * 8), 256, 0, s>>>(in, n, d_out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int reduce_sum_i32(const int32_t* in, int64_t n, int64_t* d_out, cudaStream_t s) {
  MGB_CUDA_CHECK(cudaMemsetAsync(d_out, 0, sizeof(int64_t), s));
  if (n <= 0) return MGB_SUCCESS;
  sum_i32_kernel<<<blocks_for(n, 256, (int64_t)num_sms() * 8), 256, 0, s>>>(
      in, n, reinterpret_cast<unsigned long long*>(d_out));
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int histogram(const int32_t* keys, int64_t n, int32_t* counts, int64_t nbins, cudaStream_t s) {
  MGB_CUDA_CHECK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * (nbins > 0 ? nbins : 0), s));
  if (n <= 0 || nbins <= 0) return MGB_SUCCESS;
  histogram_kernel<<<blocks_for(n, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(keys, n, counts, nbins);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int coo_sorted_flags(const int32_t* rows, const int32_t* cols, int64_t n, int32_t* d_flag, int32_t* d_dup,
                     cudaStream_t s) {
  fill_i32<<<1, 32, 0, s>>>(d_flag, 1, 1);
  MGB_LAUNCH_CHECK();
  if (d_dup) MGB_CUDA_CHECK(cudaMemsetAsync(d_dup, 0, sizeof(int32_t), s));
  if (n <= 1) return MGB_SUCCESS;
  sorted_flags_kernel<<<blocks_for(n, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(rows, cols, n, d_flag, d_dup);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int rows_sorted_flag(const int32_t* rows, int64_t n, int32_t* d_flag, cudaStream_t s) {
  return coo_sorted_flags(rows, nullptr, n, d_flag, nullptr, s);
}

int segmented_sort_u64(uint64_t* keys, const int32_t* seg, int64_t nseg, int64_t nkeys, cudaStream_t s) {
  if (nseg <= 0 || nkeys <= 1) return MGB_SUCCESS;
  Scratch sc(s);
  int32_t* lists;
  int32_t* counters;
  MGB_SCRATCH(sc, lists, 3 * nseg);
  MGB_SCRATCH(sc, counters, 4);
  MGB_CUDA_CHECK(cudaMemsetAsync(counters, 0, 4 * sizeof(int32_t), s));
  classify_segments<<<blocks_for(nseg, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(seg, nseg, lists, nseg, counters);
  MGB_LAUNCH_CHECK();
  int32_t h[4];
  MGB_CUDA_CHECK(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));
  if (h[0] > 0) {
    sort_small_segments<<<blocks_for((int64_t)h[0] * 32, 256, (int64_t)num_sms() * 32), 256, 0, s>>>(
        keys, seg, lists, counters);
    MGB_LAUNCH_CHECK();
  }
  if (h[1] > 0) {
    sort_medium_segments<<<(unsigned)min((int64_t)h[1], (int64_t)num_sms() * 8), SEG_MED_THREADS, 0, s>>>(
        keys, seg, lists + nseg, counters + 1);
    MGB_LAUNCH_CHECK();
  }
  if (h[2] > 0) {
    uint64_t* tmp;
    MGB_SCRATCH(sc, tmp, nkeys);
    sort_large_segments<<<(unsigned)min((int64_t)h[2], (int64_t)num_sms() * 4), SEG_MED_THREADS, 0, s>>>(
        keys, tmp, seg, lists + 2 * nseg, counters + 2);
    MGB_LAUNCH_CHECK();
  }
  return MGB_SUCCESS;
}

int stable_sort_rows_cols(const int32_t* rows, const int32_t* cols, int64_t n, int64_t nrows, int32_t* out_rows,
                          int32_t* out_cols, int32_t* perm, cudaStream_t s) {
  if (n <= 0) return MGB_SUCCESS;
  Scratch sc(s);
  int32_t *counts, *starts, *cursor;
  uint64_t* keys;
  MGB_SCRATCH(sc, counts, nrows + 1);
  MGB_SCRATCH(sc, starts, nrows + 1);
  MGB_SCRATCH(sc, cursor, nrows + 1);
  MGB_SCRATCH(sc, keys, n);
  int st = histogram(rows, n, counts, nrows, s);
  if (st) return st;
  MGB_CUDA_CHECK(cudaMemsetAsync(counts + nrows, 0, sizeof(int32_t), s));
  st = exclusive_scan<int32_t, int32_t>(counts, starts, nrows + 1, s);
  if (st) return st;
  MGB_CUDA_CHECK(cudaMemcpyAsync(cursor, starts, sizeof(int32_t) * (nrows + 1), cudaMemcpyDeviceToDevice, s));
  scatter_row_keys<<<blocks_for(n, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(rows, cols, n, cursor, keys);
  MGB_LAUNCH_CHECK();
  st = segmented_sort_u64(keys, starts, nrows, n, s);
  if (st) return st;
  gather_sorted<<<blocks_for(n, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(keys, rows, n, out_rows, out_cols, perm);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

}  // namespace prim
}  // namespace mgb
