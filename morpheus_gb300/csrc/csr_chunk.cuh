// csr_chunk.cuh -- one warp chunk of the lane-segment CSR SpMV, shared by the
// single-matrix kernel (spmv_csr.cu) and the batched kernel (spmv_batched.cu).
// The algorithm is described at the top of spmv_csr.cu.
#pragma once

#include "mgb_internal.cuh"

namespace mgb {
namespace csr {

constexpr int CSR_WARPS = 8;          // warps per CTA
constexpr int CSR_SEG = 8;            // default entries per lane per staging step
constexpr int64_t CSR_CHUNK = 2048;   // default nominal nonzeros per warp
constexpr int CSR_RO_STAGE = 512;     // row offsets staged per warp

// first index i in [lo, hi] with ro[i] >= key (hi if none), 32 lanes cooperating
__device__ __forceinline__ int64_t warp_lower_bound(const int32_t* __restrict__ ro, int64_t lo,
                                                    int64_t hi, int64_t key, int lane) {
  // invariant: ro[i] < key for i < lo; ro[i] >= key for i >= hi (virtually)
  while (hi - lo > 32) {
    const int64_t span = hi - lo;
    const int64_t p = lo + (span * (lane + 1)) / 33;  // 32 interior pivots
    const bool less = (int64_t)__ldg(ro + p) < key;
    const unsigned m = __ballot_sync(0xffffffffu, less);
    // pivots are increasing, so 'less' holds on a prefix of the lanes
    const int cnt = __popc(m);
    const int64_t new_lo = cnt ? __shfl_sync(0xffffffffu, p, cnt - 1) + 1 : lo;
    const int64_t new_hi = __shfl_sync(0xffffffffu, p, cnt < 32 ? cnt : 31);
    lo = new_lo;
    hi = cnt < 32 ? new_hi : hi;
  }
  // at most 32 candidates left: [lo, hi)
  const int64_t q = lo + lane;
  const bool less = q < hi && (int64_t)__ldg(ro + q) < key;
  return lo + __popc(__ballot_sync(0xffffffffu, less));
}

// Shared-memory staging of one warp.
template <typename T, int SEG>
struct WarpStage {
  T val[32 * (SEG + 1)];
  int32_t col[32 * (SEG + 1)];
  int32_t ro[CSR_RO_STAGE];
};

// Rows [begin, end) of one warp chunk.
struct RowRange {
  int64_t begin, end;
};

// x read through the read-only global path
template <typename T>
struct XGlobal {
  const T* __restrict__ p;
  __device__ __forceinline__ T operator()(int32_t c) const { return __ldg(p + c); }
};
// x staged in shared memory (p points into the kernel's shared array)
template <typename T>
struct XShared {
  const T* p;
  __device__ __forceinline__ T operator()(int32_t c) const { return p[c]; }
};

// Processes warp chunk `wc` of one CSR matrix: the rows whose first entry lies
// in [wc*chunk, (wc+1)*chunk).  Chunks are whole rows, so every y entry is
// written by exactly one warp.  Returns the chunk's rows (their y entries are
// visible to the whole warp after a __syncwarp()).  xl(c) reads x[c].
template <typename T, int SEG, typename XL>
__device__ __forceinline__ RowRange csr_chunk_x(int64_t wc, int64_t chunk, int64_t nrows, int64_t ncols,
                                                const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                                                const T* __restrict__ va, XL xl, T* __restrict__ y, int init,
                                                WarpStage<T, SEG>& stg, int lane) {
  constexpr int CSR_PAD = SEG + 1;
  T* sv = stg.val;
  int32_t* sc = stg.col;
  int32_t* sro = stg.ro;
  // rows starting in [s0, s1)
  const int64_t s0 = wc * chunk, s1 = s0 + chunk;
  int64_t r_begin = warp_lower_bound(ro, 0, nrows + 1, s0, lane);
  int64_t r_end = warp_lower_bound(ro, r_begin, nrows + 1, s1, lane);
  if (r_begin > nrows) r_begin = nrows;
  if (r_end > nrows) r_end = nrows;
  if (r_begin >= r_end) return RowRange{r_begin, r_begin};
  const int64_t nr = r_end - r_begin;
  const bool staged = nr < CSR_RO_STAGE;  // offsets r_begin..r_end in smem
  __syncwarp();
  if (staged)
    for (int64_t i = lane; i <= nr; i += 32) sro[i] = __ldg(ro + r_begin + i);
  __syncwarp();
  auto ro_at = [&](int64_t i) -> int64_t {
    return staged ? (int64_t)sro[i - r_begin] : (int64_t)__ldg(ro + i);
  };
  const int64_t E0 = ro_at(r_begin), E1 = ro_at(r_end);
  if (E0 >= E1) {  // only empty rows
    if (init)
      for (int64_t r = r_begin + lane; r < r_end; r += 32) y[r] = T(0);
    return RowRange{r_begin, r_end};
  }
  const int64_t A0 = E0 & ~(int64_t)7;  // 32-byte aligned column segments
  int64_t KW = (E1 - A0 + 31) / 32;
  KW = (KW + SEG - 1) / SEG * SEG;
  const int64_t la = A0 + lane * KW;
  const int64_t lb = min(la + KW, E1);
  const int64_t e_lo = max(la, E0);
  const bool active = e_lo < lb;

  // lane's first row: lane 0 starts at r_begin (so leading empty rows are
  // flushed); others at the row containing e_lo (empty rows sitting at a
  // lane boundary are flushed by the previous lane's tail loop).
  int64_t r = r_end;
  if (active) {
    if (lane == 0) {
      r = r_begin;
    } else {
      int64_t lo = r_begin, hi = r_end;  // first i in [lo, hi] with ro[i] > e_lo
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (ro_at(mid) <= e_lo) lo = mid + 1; else hi = mid;
      }
      r = lo - 1;
    }
  }
  int64_t rs = active ? ro_at(r) : 0;
  int64_t re = active ? ro_at(r + 1) : 0;
  T acc = (active && rs >= e_lo && !init) ? y[r] : T(0);
  int64_t hrow = -1;
  T hval = T(0);

  for (int64_t s = 0; s < KW; s += SEG) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < SEG; q++) {
      const int f = q * 32 + lane;
      const int L = f / SEG, j = f % SEG;
      const int64_t e = A0 + L * KW + s + j;
      const bool in = e >= E0 && e < E1;
      sv[L * CSR_PAD + j] = in ? ldg_stream(va + e) : T(0);
      sc[L * CSR_PAD + j] = in ? ldg_stream(ci + e) : 0;
    }
    __syncwarp();
    T v[SEG], xv[SEG];
#pragma unroll
    for (int k = 0; k < SEG; k++) {
      const int64_t e = la + s + k;
      const bool valid = e >= e_lo && e < lb;
      const int32_t c = sc[lane * CSR_PAD + k];
      v[k] = valid ? sv[lane * CSR_PAD + k] : T(0);
      xv[k] = (valid && (uint64_t)(int64_t)c < (uint64_t)ncols) ? xl(c) : T(0);
    }
#pragma unroll
    for (int k = 0; k < SEG; k++) {
      const int64_t e = la + s + k;
      const bool valid = e >= e_lo && e < lb;
      while (valid && e >= re) {
        if (rs >= e_lo) { y[r] = acc; } else { hrow = r; hval = acc; }
        r++;
        rs = re;
        re = ro_at(r + 1);
        acc = init ? T(0) : y[r];
      }
      acc = fmadd(v[k], xv[k], acc);
    }
  }
  // rows ending exactly at the lane end (and empty rows sitting there)
  if (active) {
    while (r < r_end && re <= lb) {
      if (rs >= e_lo) { y[r] = acc; } else { hrow = r; hval = acc; }
      r++;
      if (r < r_end) {
        rs = re;
        re = ro_at(r + 1);
        acc = init ? T(0) : y[r];  // empty rows at lb are flushed here
      }
    }
  }
  // tail partial (a row that started in this lane's range and continues into
  // the next lane; a row starting exactly at lb belongs to the next lane)
  // and segmented scan
  const bool has_tail = active && r < r_end && rs < lb;
  const int64_t key = has_tail ? r : -1 - (int64_t)lane;
  T cv = has_tail ? acc : T(0);
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T u = __shfl_up_sync(0xffffffffu, cv, d);
    const int64_t k2 = __shfl_up_sync(0xffffffffu, key, d);
    if (lane >= d && k2 == key) cv += u;
  }
  const T vprev = __shfl_up_sync(0xffffffffu, cv, 1);
  const int64_t kprev = __shfl_up_sync(0xffffffffu, key, 1);
  if (hrow >= 0) y[hrow] = (lane > 0 && kprev == hrow) ? hval + vprev : hval;
  return RowRange{r_begin, r_end};
}

template <typename T, int64_t CHUNK, int SEG>
__device__ __forceinline__ RowRange csr_chunk(int64_t wc, int64_t nrows, int64_t ncols,
                                              const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                                              const T* __restrict__ va, const T* __restrict__ x,
                                              T* __restrict__ y, int init, WarpStage<T, SEG>& stg, int lane) {
  return csr_chunk_x<T, SEG>(wc, CHUNK, nrows, ncols, ro, ci, va, XGlobal<T>{x}, y, init, stg, lane);
}

}  // namespace csr
}  // namespace mgb
