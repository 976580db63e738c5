// primitives.cuh -- device-wide building blocks for the GPU conversions:
// exclusive scan, reductions, stable (row, col) sort of COO entries and
// per-row segmented sort.  All scratch is stream-ordered (cudaMallocAsync).
#pragma once

#include "mgb_internal.cuh"

namespace mgb {
namespace prim {

// RAII stream-ordered scratch; freed with cudaFreeAsync on the same stream.
class Scratch {
 public:
  explicit Scratch(cudaStream_t s) : s_(s) {}
  ~Scratch() {
    for (int i = 0; i < n_; i++) cudaFreeAsync(p_[i], s_);
  }
  template <typename T>
  cudaError_t get(T** out, size_t count) {
    *out = nullptr;
    if (n_ >= 32) return cudaErrorMemoryAllocation;
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, count ? count * sizeof(T) : 16, s_);
    if (e == cudaSuccess) {
      p_[n_++] = p;
      *out = static_cast<T*>(p);
    }
    return e;
  }

 private:
  cudaStream_t s_;
  void* p_[32];
  int n_ = 0;
};

#define MGB_SCRATCH(sc, ptr, count) MGB_CUDA_CHECK((sc).get(&(ptr), (size_t)(count)))

// Exclusive scan of n values (any integer type in, any integer type out,
// 64-bit accumulation).  Optionally writes the total to *d_total (device).
template <typename Tin, typename Tout>
int exclusive_scan(const Tin* in, Tout* out, int64_t n, cudaStream_t s, int64_t* d_total = nullptr);

// Max over n int32 values into *d_out (device); n == 0 writes INT32_MIN.
int reduce_max_i32(const int32_t* in, int64_t n, int32_t* d_out, cudaStream_t s);
// Sum over n int32 values into *d_out (device, 64-bit).
int reduce_sum_i32(const int32_t* in, int64_t n, int64_t* d_out, cudaStream_t s);

// Counts of keys in [0, nbins) (out of range keys are ignored).
int histogram(const int32_t* keys, int64_t n, int32_t* counts, int64_t nbins, cudaStream_t s);

// 1 if (row, col) pairs are sorted lexicographically (duplicates allowed),
// else 0, written to *d_flag (device).  Also *d_dup = 1 if an adjacent
// duplicate (row, col) exists (only meaningful when sorted).
int coo_sorted_flags(const int32_t* rows, const int32_t* cols, int64_t n, int32_t* d_flag,
                     int32_t* d_dup, cudaStream_t s);
// 1 if rows are non-decreasing.
int rows_sorted_flag(const int32_t* rows, int64_t n, int32_t* d_flag, cudaStream_t s);

// Sort the keys of each segment [seg[i], seg[i+1]) ascending (keys unique
// within a segment, so any sort is stable).  nseg segments, seg has nseg+1
// entries (int32 offsets into keys).
int segmented_sort_u64(uint64_t* keys, const int32_t* seg, int64_t nseg, int64_t nkeys, cudaStream_t s);

// Stable sort of COO entries by (row, col): writes the permutation (source
// index per output slot) to perm[n] and the sorted rows/cols to
// out_rows/out_cols.  Rows must lie in [0, nrows).  Equivalent to the
// reference's two stable counting sorts (by column, then by row).
int stable_sort_rows_cols(const int32_t* rows, const int32_t* cols, int64_t n, int64_t nrows,
                          int32_t* out_rows, int32_t* out_cols, int32_t* perm, cudaStream_t s);

// Copy a device scalar to the host (synchronises the stream).
template <typename T>
int to_host(const T* d, T* h, cudaStream_t s) {
  MGB_CUDA_CHECK(cudaMemcpyAsync(h, d, sizeof(T), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));
  return MGB_SUCCESS;
}

inline unsigned blocks_for(int64_t n, int threads, int64_t cap = 1 << 20) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

}  // namespace prim
}  // namespace mgb
