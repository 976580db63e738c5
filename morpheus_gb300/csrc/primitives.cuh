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

// ---- counting into few hot bins --------------------------------------------
// A histogram whose entries fall into few distinct bins per CTA (the
// diagonals of a banded or stencil matrix: 27 bins for a 27-point stencil,
// however many entries) serialises on global atomics.  CtaHist counts in
// shared memory first: lanes of a warp holding the same key are merged
// (__match_any_sync), the warp's leader for that key adds into an
// open-addressing table of HIST_SLOTS (key, count) pairs, and the CTA
// flushes the table with one global atomic per occupied slot.  A key that
// finds no free slot within HIST_PROBES probes marks the table full and,
// like every key after it, goes straight to the global counter, so the
// counts are exact in every case and scattered keys pay little for the try.
constexpr int HIST_SLOTS = 2048;
constexpr int HIST_PROBES = 8;
constexpr unsigned long long HIST_EMPTY = ~0ull;

struct CtaHist {
  unsigned long long* keys;  // HIST_SLOTS keys, HIST_EMPTY where free
  int32_t* counts;           // HIST_SLOTS counts
  int* full;                 // set once a key found no slot
};

// every thread of the CTA, followed by __syncthreads()
__device__ __forceinline__ void hist_init(CtaHist h) {
  for (int i = threadIdx.x; i < HIST_SLOTS; i += blockDim.x) {
    h.keys[i] = HIST_EMPTY;
    h.counts[i] = 0;
  }
  if (threadIdx.x == 0) *h.full = 0;
}

// counts one occurrence of key (global[key] += 1, in the end)
__device__ __forceinline__ void hist_add(CtaHist h, int32_t* global, unsigned long long key) {
  const unsigned same = __match_any_sync(__activemask(), key);
  if ((int)(threadIdx.x & 31) != __ffs(same) - 1) return;  // one lane per distinct key adds
  const int inc = __popc(same);
  if (!*reinterpret_cast<volatile int*>(h.full)) {
    unsigned slot = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 53) & (HIST_SLOTS - 1);
    for (int p = 0; p < HIST_PROBES; p++) {
      const unsigned long long prev = atomicCAS(h.keys + slot, HIST_EMPTY, key);
      if (prev == HIST_EMPTY || prev == key) {
        atomicAdd(h.counts + slot, inc);
        return;
      }
      slot = (slot + 1) & (HIST_SLOTS - 1);
    }
    *reinterpret_cast<volatile int*>(h.full) = 1;
  }
  atomicAdd(global + key, inc);
}

// every thread of the CTA, after a __syncthreads() that follows the last hist_add
__device__ __forceinline__ void hist_flush(CtaHist h, int32_t* global) {
  for (int i = threadIdx.x; i < HIST_SLOTS; i += blockDim.x) {
    const unsigned long long k = h.keys[i];
    if (k != HIST_EMPTY && h.counts[i]) atomicAdd(global + k, h.counts[i]);
  }
}

// global[key] += 1 with the lanes of a warp holding the same key merged
// (row counts of row-sorted entries: consecutive lanes share a row)
__device__ __forceinline__ void warp_merged_add(int32_t* global, int64_t key) {
  const unsigned same = __match_any_sync(__activemask(), (unsigned long long)key);
  if ((int)(threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(global + key, __popc(same));
}

#define MGB_CTA_HIST(name)                                  \
  __shared__ unsigned long long name##_keys[::mgb::prim::HIST_SLOTS]; \
  __shared__ int32_t name##_counts[::mgb::prim::HIST_SLOTS];          \
  __shared__ int name##_full;                                         \
  const ::mgb::prim::CtaHist name{name##_keys, name##_counts, &name##_full}

inline unsigned blocks_for(int64_t n, int threads, int64_t cap = 1 << 20) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

}  // namespace prim
}  // namespace mgb
