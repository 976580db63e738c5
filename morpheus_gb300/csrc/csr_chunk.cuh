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

// Shared-memory staging of one warp (RO: row offsets staged per chunk).
template <typename T, int SEG, int RO = CSR_RO_STAGE>
struct WarpStage {
  T val[32 * (SEG + 1)];
  int32_t col[32 * (SEG + 1)];
  int32_t ro[RO];
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

// Rows of warp chunk `wc`: those whose first entry lies in [wc*chunk,
// (wc+1)*chunk), found by two 32-ary searches over the row offsets.
__device__ __forceinline__ RowRange chunk_rows(int64_t wc, int64_t chunk, int64_t nrows,
                                               const int32_t* __restrict__ ro, int lane) {
  const int64_t s0 = wc * chunk, s1 = s0 + chunk;
  int64_t r_begin = warp_lower_bound(ro, 0, nrows + 1, s0, lane);
  int64_t r_end = warp_lower_bound(ro, r_begin, nrows + 1, s1, lane);
  if (r_begin > nrows) r_begin = nrows;
  if (r_end > nrows) r_end = nrows;
  return RowRange{r_begin, r_end};
}

// Rows of warp chunk `wc` read from a chunk plan: plan[k] = the first row
// whose first entry is at or after k*chunk (nrows if none), k = 0..nchunks.
// Values are clamped, so a plan made for another structure gives wrong
// sums but no access outside the matrix.
__device__ __forceinline__ RowRange planned_rows(int64_t wc, int64_t nrows, const int32_t* __restrict__ plan) {
  int64_t r_begin = __ldg(plan + wc), r_end = __ldg(plan + wc + 1);
  r_begin = r_begin < 0 ? 0 : (r_begin > nrows ? nrows : r_begin);
  r_end = r_end < r_begin ? r_begin : (r_end > nrows ? nrows : r_end);
  return RowRange{r_begin, r_end};
}

// Processes the rows [rows.begin, rows.end) of one warp chunk of a CSR
// matrix.  Chunks are whole rows, so every y entry is written by exactly one
// warp.  Returns the chunk's rows (their y entries are visible to the whole
// warp after a __syncwarp()).  xl(c) reads x[c].  BOUNDED: the row walk also
// stops at the chunk's last row, which only matters for row offsets that are
// not non-decreasing (then sums are wrong but nothing outside the chunk's
// rows is touched); the batched chunk-queue kernel, whose speed drops 12 %
// with the extra bound (measured), walks unbounded and relies on valid
// offsets, as the reference's kernels do.
// IDX: the type of entry and row indices inside the routine (int32_t is
// exact when nnz < 2^31 - 4096, as the launchers require, and nrows < 2^31 -
// 32); RO: row offsets staged per chunk.
template <typename T, int SEG, typename XL, bool BOUNDED = true, typename IDX = int64_t, int RO = CSR_RO_STAGE>
__device__ __forceinline__ RowRange csr_rows_x(RowRange rows, int64_t nrows, int64_t ncols,
                                               const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                                               const T* __restrict__ va, XL xl, T* __restrict__ y, int init,
                                               WarpStage<T, SEG, RO>& stg, int lane) {
  constexpr int CSR_PAD = SEG + 1;
  T* sv = stg.val;
  int32_t* sc = stg.col;
  int32_t* sro = stg.ro;
  const IDX r_begin = (IDX)rows.begin, r_end = (IDX)rows.end;
  if (r_begin >= r_end) return RowRange{r_begin, r_begin};
  const IDX nr = r_end - r_begin;
  const bool staged = nr < RO;  // offsets r_begin..r_end in smem
  __syncwarp();
  if (staged)
    for (IDX i = lane; i <= nr; i += 32) sro[i] = __ldg(ro + r_begin + i);
  __syncwarp();
  auto ro_at = [&](IDX i) -> IDX {
    return staged ? (IDX)sro[i - r_begin] : (IDX)__ldg(ro + i);
  };
  const IDX E0 = ro_at(r_begin), E1 = ro_at(r_end);
  if (E0 >= E1) {  // only empty rows
    if (init)
      for (IDX r = r_begin + lane; r < r_end; r += 32) y[r] = T(0);
    return RowRange{r_begin, r_end};
  }
  const IDX A0 = E0 & ~(IDX)7;  // 32-byte aligned column segments
  IDX KW = (E1 - A0 + 31) / 32;
  KW = (KW + SEG - 1) / SEG * SEG;
  const IDX la = A0 + lane * KW;
  const IDX lb = min(la + KW, E1);
  const IDX e_lo = max(la, E0);
  const bool active = e_lo < lb;

  // lane's first row: lane 0 starts at r_begin (so leading empty rows are
  // flushed); others at the row containing e_lo (empty rows sitting at a
  // lane boundary are flushed by the previous lane's tail loop).
  IDX r = r_end;
  if (active) {
    if (lane == 0) {
      r = r_begin;
    } else {
      IDX lo = r_begin, hi = r_end;  // first i in [lo, hi] with ro[i] > e_lo
      while (lo < hi) {
        const IDX mid = (lo + hi) >> 1;
        if (ro_at(mid) <= e_lo) lo = mid + 1; else hi = mid;
      }
      r = lo - 1;
    }
  }
  IDX rs = active ? ro_at(r) : 0;
  IDX re = active ? ro_at(r + 1) : 0;
  T acc = (active && rs >= e_lo && !init) ? y[r] : T(0);
  IDX hrow = -1;
  T hval = T(0);

  for (IDX s = 0; s < KW; s += SEG) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < SEG; q++) {
      const int f = q * 32 + lane;
      const int L = f / SEG, j = f % SEG;
      const IDX e = A0 + L * KW + s + j;
      const bool in = e >= E0 && e < E1;
      sv[L * CSR_PAD + j] = in ? ldg_stream(va + e) : T(0);
      sc[L * CSR_PAD + j] = in ? ldg_stream(ci + e) : 0;
    }
    __syncwarp();
    T v[SEG], xv[SEG];
#pragma unroll
    for (int k = 0; k < SEG; k++) {
      const IDX e = la + s + k;
      const bool valid = e >= e_lo && e < lb;
      const int32_t c = sc[lane * CSR_PAD + k];
      v[k] = valid ? sv[lane * CSR_PAD + k] : T(0);
      xv[k] = (valid && (uint64_t)(int64_t)c < (uint64_t)ncols) ? xl(c) : T(0);
    }
#pragma unroll
    for (int k = 0; k < SEG; k++) {
      const IDX e = la + s + k;
      const bool valid = e >= e_lo && e < lb;
      while (valid && e >= re && (!BOUNDED || r + 1 < r_end)) {
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
  const IDX key = has_tail ? r : -1 - (IDX)lane;
  T cv = has_tail ? acc : T(0);
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T u = __shfl_up_sync(0xffffffffu, cv, d);
    const IDX k2 = __shfl_up_sync(0xffffffffu, key, d);
    if (lane >= d && k2 == key) cv += u;
  }
  const T vprev = __shfl_up_sync(0xffffffffu, cv, 1);
  const IDX kprev = __shfl_up_sync(0xffffffffu, key, 1);
  if (hrow >= 0) y[hrow] = (lane > 0 && kprev == hrow) ? hval + vprev : hval;
  return RowRange{r_begin, r_end};
}

// Processes warp chunk `wc` of one CSR matrix: the rows whose first entry
// lies in [wc*chunk, (wc+1)*chunk).
template <typename T, int SEG, typename XL>
__device__ __forceinline__ RowRange csr_chunk_x(int64_t wc, int64_t chunk, int64_t nrows, int64_t ncols,
                                                const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                                                const T* __restrict__ va, XL xl, T* __restrict__ y, int init,
                                                WarpStage<T, SEG>& stg, int lane) {
  return csr_rows_x<T, SEG>(chunk_rows(wc, chunk, nrows, ro, lane), nrows, ncols, ro, ci, va, xl, y, init, stg,
                            lane);
}

// the batched chunk-queue form: fixed chunk size, unbounded row walk, 32-bit
// indices (the caller skips matrices with nnz >= 2^31 - 4096 or nrows >=
// 2^31 - 32; measured on the 4,096-matrix batch: 0.785 -> 0.753 ms)
template <typename T, int64_t CHUNK, int SEG>
__device__ __forceinline__ RowRange csr_chunk(int64_t wc, int64_t nrows, int64_t ncols,
                                              const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                                              const T* __restrict__ va, const T* __restrict__ x,
                                              T* __restrict__ y, int init, WarpStage<T, SEG>& stg, int lane) {
  return csr_rows_x<T, SEG, XGlobal<T>, false, int32_t>(chunk_rows(wc, CHUNK, nrows, ro, lane), nrows, ncols, ro,
                                                        ci, va, XGlobal<T>{x}, y, init, stg, lane);
}

}  // namespace csr
}  // namespace mgb

namespace mgb {
namespace csr {

// Split chunk k of a CSR matrix: exactly the entries [k*chunk, min((k+1)*chunk,
// nnz)), whatever rows they belong to (rows longer than a chunk are spread
// over several warps).  Rows that start and end inside the chunk are written
// to y; the row continuing from the previous chunk (started before E0) and
// the row continuing into the next one (ends after E1) leave their partial
// sums as carries: carry slot 2k for the row entering the chunk, 2k+1 for
// the row leaving it, (-1, 0) when there is none (a row spanning the whole
// chunk fills both slots, so each row's carries stay consecutive).  A carry
// fix-up adds them in chunk order.  Empty rows are zero-filled (init) by the
// chunk whose range holds their start offset; trailing empty rows (start ==
// nnz) by the last chunk's last lane.
template <typename T, int SEG>
__device__ __forceinline__ void csr_split_chunk(int64_t k, int64_t chunk, int64_t nchunks, int64_t nrows,
                                                int64_t ncols, int64_t nnz, const int32_t* __restrict__ ro,
                                                const int32_t* __restrict__ ci, const T* __restrict__ va,
                                                const T* __restrict__ x, T* __restrict__ y, int init,
                                                int32_t* __restrict__ carry_row, T* __restrict__ carry_val,
                                                WarpStage<T, SEG>& stg, int lane) {
  constexpr int CSR_PAD = SEG + 1;
  T* sv = stg.val;
  int32_t* sc = stg.col;
  int32_t* sro = stg.ro;
  const int64_t E0 = k * chunk;
  const int64_t E1 = min(E0 + chunk, nnz);
  const bool last = k == nchunks - 1;
  // rows starting in [E0, E1) (all remaining rows for the last chunk)
  const int64_t r_a = warp_lower_bound(ro, 0, nrows + 1, E0, lane);
  const int64_t r_end = last ? nrows : min(warp_lower_bound(ro, r_a, nrows + 1, E1, lane), nrows);
  // the row entering the chunk: started before E0, still has entries at E0
  const bool has_in = E0 < E1 && r_a > 0 && (r_a > nrows || (int64_t)__ldg(ro + r_a) > E0);
  const int64_t r_lo = has_in ? r_a - 1 : r_a;  // first row the lanes walk
  const int64_t r_hi = r_end;                   // rows [r_lo, r_hi)
  if (lane == 0) {
    carry_row[2 * k] = -1;
    carry_val[2 * k] = T(0);
    carry_row[2 * k + 1] = -1;
    carry_val[2 * k + 1] = T(0);
  }
  if (r_lo >= r_hi) return;
  const int64_t nr = r_hi - r_lo;
  const bool staged = nr < CSR_RO_STAGE;
  __syncwarp();
  if (staged)
    for (int64_t i = lane; i <= nr; i += 32) sro[i] = __ldg(ro + r_lo + i);
  __syncwarp();
  auto ro_at = [&](int64_t i) -> int64_t { return staged ? (int64_t)sro[i - r_lo] : (int64_t)__ldg(ro + i); };
  // the row leaving the chunk: ends after E1 (only the last row can)
  const int64_t r_out = (r_hi > r_lo && ro_at(r_hi) > E1) ? r_hi - 1 : -1;
  auto put = [&](int64_t r, T v) {  // a finished sum of row r over this chunk
    if (has_in && r == r_lo) {
      carry_row[2 * k] = (int32_t)r;
      carry_val[2 * k] = v;
      if (r == r_out) carry_row[2 * k + 1] = (int32_t)r;  // spans the chunk: keep its carries consecutive
    } else if (r == r_out) {
      carry_row[2 * k + 1] = (int32_t)r;
      carry_val[2 * k + 1] = v;
    } else {
      y[r] = v;
    }
  };
  if (E0 >= E1) {  // no entries (nnz == 0 handled by the launcher; only empty rows here)
    if (init)
      for (int64_t r = r_lo + lane; r < r_hi; r += 32) y[r] = T(0);
    return;
  }
  const int64_t A0 = E0 & ~(int64_t)7;
  int64_t KW = (E1 - A0 + 31) / 32;
  KW = (KW + SEG - 1) / SEG * SEG;
  const int64_t la = A0 + lane * KW;
  const int64_t lb = min(la + KW, E1);
  const int64_t e_lo = max(la, E0);
  const bool active = e_lo < lb;
  int64_t r = r_hi;
  if (active) {
    if (lane == 0) {
      r = r_lo;
    } else {
      int64_t lo = r_lo, hi = r_hi;  // first i in [lo, hi] with ro[i] > e_lo
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (ro_at(mid) <= e_lo) lo = mid + 1; else hi = mid;
      }
      r = lo - 1;
    }
  }
  int64_t rs = active ? ro_at(r) : 0;
  int64_t re = active ? ro_at(r + 1) : 0;
  // seed with y only rows that start in this lane and end in this chunk
  auto seed = [&](int64_t rr, int64_t s, int64_t e) -> T {
    return (!init && s >= e_lo && e <= E1 && !(has_in && rr == r_lo)) ? y[rr] : T(0);
  };
  T acc = active ? seed(r, rs, re) : T(0);
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
    for (int q = 0; q < SEG; q++) {
      const int64_t e = la + s + q;
      const bool valid = e >= e_lo && e < lb;
      const int32_t c = sc[lane * CSR_PAD + q];
      v[q] = valid ? sv[lane * CSR_PAD + q] : T(0);
      xv[q] = (valid && (uint64_t)(int64_t)c < (uint64_t)ncols) ? __ldg(x + c) : T(0);
    }
#pragma unroll
    for (int q = 0; q < SEG; q++) {
      const int64_t e = la + s + q;
      const bool valid = e >= e_lo && e < lb;
      while (valid && e >= re && r + 1 < r_hi) {  // (the bound only matters for invalid offsets)
        if (rs >= e_lo) { put(r, acc); } else { hrow = r; hval = acc; }
        r++;
        rs = re;
        re = ro_at(r + 1);
        acc = seed(r, rs, re);
      }
      acc = fmadd(v[q], xv[q], acc);
    }
  }
  // rows ending exactly at the lane end (and empty rows sitting there)
  if (active) {
    while (r < r_hi && re <= lb) {
      if (rs >= e_lo) { put(r, acc); } else { hrow = r; hval = acc; }
      r++;
      if (r < r_hi) {
        rs = re;
        re = ro_at(r + 1);
        acc = seed(r, rs, re);
      }
    }
  }
  // tail partials and the segmented scan, as in csr_chunk_x; the row leaving
  // the chunk ends in no lane: the last lane holding it writes its carry
  const bool has_tail = active && r < r_hi && rs < lb;
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
  const int64_t knext = __shfl_down_sync(0xffffffffu, key, 1);
  if (hrow >= 0) put(hrow, (lane > 0 && kprev == hrow) ? hval + vprev : hval);
  if (has_tail && r == r_out && (lane == 31 || knext != key)) put(r, cv);
}

}  // namespace csr
}  // namespace mgb
