// convert.cu -- format conversions on the GPU, bit-exact with the reference's
// Serial convert (the reference's CUDA convert throws NotImplementedException
// for every pair: impl/<Fmt>/Cuda/Morpheus_Convert_Impl.hpp).
//
// Every X -> COO builds the reference's pre-sort array in the reference's
// order (including the (0,0,0) tail entries left when exact zeros are dropped)
// and, only if that array is not sorted, applies a stable (row, col) sort
// (equal to the reference's two stable counting sorts,
// impl/Coo/Serial/Morpheus_Sort_Impl.hpp:109-164).  Every COO -> Y follows the
// reference's placement loop: slot numbers restart whenever the row changes,
// later entries overwrite earlier ones at the same slot, remainders keep COO
// order.  Output sizes come from *_plan calls, which also apply the
// reference's fill-tolerance test (impl/Morpheus_Utils.hpp:91-105, in FP32).
#include <algorithm>
#include <climits>
#include <vector>

#include "primitives.cuh"

namespace mgb {
namespace {

using prim::blocks_for;
using prim::Scratch;

inline unsigned grid_for(int64_t n) { return blocks_for(n, 256, (int64_t)num_sms() * 16); }

// core/src/impl/Morpheus_Utils.hpp:91-105 (single-precision arithmetic)
bool exceeds_tolerance(int64_t num_rows, int64_t num_entries, int64_t num_columns) {
  const float max_fill = 10.0f;
  const float threshold = 100e6f;
  const float size = float(num_columns) * float(num_rows);
  const float fill_ratio = size / std::max(1.0f, float(num_entries));
  return fill_ratio > max_fill && size > threshold;
}

template <typename T>
__global__ void fill_kernel(T* p, T v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

template <typename T>
int fill(T* p, T v, int64_t n, cudaStream_t s) {
  if (n <= 0) return MGB_SUCCESS;
  fill_kernel<T><<<grid_for(n), 256, 0, s>>>(p, v, n);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

// min index whose row is out of [0, nrows) (or n), via atomicMin
__global__ void first_bad_row(const int32_t* __restrict__ r, int64_t n, int64_t nrows, unsigned long long* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (r[i] < 0 || r[i] >= nrows) atomicMin(out, (unsigned long long)i);
}
__global__ void first_bad_col(const int32_t* __restrict__ c, int64_t n, int64_t ncols, unsigned long long* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (c[i] < 0 || c[i] >= ncols) atomicMin(out, (unsigned long long)i);
}

// Device words an entry point reads back with one copy and one stream
// synchronisation: the validation result, the plan's sizes and the
// sortedness flags, computed by kernels queued one after another.
struct Words {
  unsigned long long bad_row, bad_col;  // first index out of range (~0: none)
  int64_t total, total2;                // plan sizes
  int32_t sorted, dup, maxv, pad;
};

int words_alloc(Scratch& sc, Words** d, cudaStream_t s) {
  MGB_SCRATCH(sc, *d, 1);
  MGB_CUDA_CHECK(cudaMemsetAsync(*d, 0xff, 2 * sizeof(unsigned long long), s));
  MGB_CUDA_CHECK(cudaMemsetAsync(&(*d)->total, 0, sizeof(Words) - 2 * sizeof(unsigned long long), s));
  return MGB_SUCCESS;
}

int words_read(const Words* d, Words* h, cudaStream_t s) {
  MGB_CUDA_CHECK(cudaMemcpyAsync(h, d, sizeof(Words), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));
  return MGB_SUCCESS;
}

// MGB_ERR_INVALID_INPUT (read by the caller with its other words) if any row
// is outside [0, nrows) or column outside [0, ncols): the reference has no
// check and indexes out of bounds there.  Queued without a synchronisation.
int validate_async(const int32_t* rows, const int32_t* cols, int64_t n, int64_t nrows, int64_t ncols, Words* d,
                   cudaStream_t s) {
  if (n <= 0) return MGB_SUCCESS;
  first_bad_row<<<grid_for(n), 256, 0, s>>>(rows, n, nrows, &d->bad_row);
  MGB_LAUNCH_CHECK();
  first_bad_col<<<grid_for(n), 256, 0, s>>>(cols, n, ncols, &d->bad_col);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

inline bool words_valid(const Words& h) { return h.bad_row == ~0ull && h.bad_col == ~0ull; }

int sorted_and_dup(const int32_t* r, const int32_t* c, int64_t n, bool* sorted, bool* dup, cudaStream_t s) {
  Scratch sc(s);
  int32_t* d;
  MGB_SCRATCH(sc, d, 2);
  int st = prim::coo_sorted_flags(r, c, n, d, d + 1, s);
  if (st) return st;
  int32_t h[2];
  MGB_CUDA_CHECK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));
  *sorted = h[0] != 0;
  if (dup) *dup = h[1] != 0;
  return MGB_SUCCESS;
}

template <typename T>
__global__ void gather_values(const T* __restrict__ src, const int32_t* __restrict__ perm, T* dst, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = src[perm[k]];
}

// In-place stable (row, col) sort of a COO array with rows in [0, nbins).
template <typename T>
int sort_coo_inplace(int32_t* rows, int32_t* cols, T* vals, int64_t n, int64_t nbins, cudaStream_t s) {
  if (n <= 1) return MGB_SUCCESS;
  Scratch sc(s);
  int32_t *r2, *c2, *perm;
  T* v2;
  MGB_SCRATCH(sc, r2, n);
  MGB_SCRATCH(sc, c2, n);
  MGB_SCRATCH(sc, perm, n);
  MGB_SCRATCH(sc, v2, n);
  int st = prim::stable_sort_rows_cols(rows, cols, n, nbins, r2, c2, perm, s);
  if (st) return st;
  gather_values<T><<<grid_for(n), 256, 0, s>>>(vals, perm, v2, n);
  MGB_LAUNCH_CHECK();
  MGB_CUDA_CHECK(cudaMemcpyAsync(rows, r2, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
  MGB_CUDA_CHECK(cudaMemcpyAsync(cols, c2, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
  MGB_CUDA_CHECK(cudaMemcpyAsync(vals, v2, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
  return MGB_SUCCESS;
}

// The reference's "if (!is_sorted(dst)) sort_by_row_and_column(dst)" on a
// freshly built COO; rows of the pre-sort array are in [0, nrows).
template <typename T>
int sort_if_unsorted(mgb_coo* dst, cudaStream_t s) {
  if (dst->nnz <= 1) return MGB_SUCCESS;
  bool sorted = false;
  int st = sorted_and_dup(dst->row_indices, dst->column_indices, dst->nnz, &sorted, nullptr, s);
  if (st || sorted) return st;
  return sort_coo_inplace<T>(dst->row_indices, dst->column_indices, static_cast<T*>(dst->values), dst->nnz,
                             dst->nrows, s);
}

int check_coo_dst(const mgb_coo* d, int64_t nrows, int64_t ncols, int64_t nnz) {
  MGB_REQUIRE(d != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(d->nrows == nrows && d->ncols == ncols && d->nnz == nnz, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(nnz == 0 || (d->row_indices && d->column_indices && d->values), MGB_ERR_BAD_ARGUMENT);
  return MGB_SUCCESS;
}

template <typename T>
int zero_coo(mgb_coo* d, cudaStream_t s) {
  if (d->nnz <= 0) return MGB_SUCCESS;
  MGB_CUDA_CHECK(cudaMemsetAsync(d->row_indices, 0, sizeof(int32_t) * d->nnz, s));
  MGB_CUDA_CHECK(cudaMemsetAsync(d->column_indices, 0, sizeof(int32_t) * d->nnz, s));
  MGB_CUDA_CHECK(cudaMemsetAsync(d->values, 0, sizeof(T) * d->nnz, s));
  return MGB_SUCCESS;
}

// ---------------------------------------------------------------- CSR <-> COO
// impl/Csr/Serial/Morpheus_Convert_Impl.hpp:70-97
__global__ void expand_rows(const int32_t* __restrict__ ro, int64_t nrows, int64_t nnz, int32_t* rows,
                            int64_t shift) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = max((int64_t)ro[r], (int64_t)0), b = min((int64_t)ro[r + 1], nnz);
    for (int64_t j = a; j < b; j++) rows[j + shift] = (int32_t)r;
  }
}

template <typename T>
int csr_to_coo(const mgb_csr* src, mgb_coo* dst, cudaStream_t s) {
  MGB_REQUIRE(src != nullptr, MGB_ERR_BAD_ARGUMENT);
  int st = check_coo_dst(dst, src->nrows, src->ncols, src->nnz);
  if (st) return st;
  if (src->nnz == 0) return MGB_SUCCESS;
  expand_rows<<<grid_for(src->nrows), 256, 0, s>>>(src->row_offsets, src->nrows, src->nnz, dst->row_indices, 0);
  MGB_LAUNCH_CHECK();
  MGB_CUDA_CHECK(cudaMemcpyAsync(dst->column_indices, src->column_indices, sizeof(int32_t) * src->nnz,
                                 cudaMemcpyDeviceToDevice, s));
  MGB_CUDA_CHECK(cudaMemcpyAsync(dst->values, src->values, sizeof(T) * src->nnz, cudaMemcpyDeviceToDevice, s));
  return MGB_SUCCESS;
}

// impl/Csr/Serial/Morpheus_Convert_Impl.hpp:99-151: counting scatter, COO order within a row
template <typename T>
int coo_to_csr(const mgb_coo* src, mgb_csr* dst, cudaStream_t s) {
  MGB_REQUIRE(src != nullptr && dst != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(dst->nrows == src->nrows && dst->ncols == src->ncols && dst->nnz == src->nnz, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(dst->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  const int64_t n = src->nnz, N = src->nrows;
  Scratch sc(s);
  Words* dw;
  int st = words_alloc(sc, &dw, s);
  if (st) return st;
  st = validate_async(src->row_indices, src->column_indices, n, N, src->ncols, dw, s);
  if (st) return st;
  if (n > 0) {
    st = prim::rows_sorted_flag(src->row_indices, n, &dw->sorted, s);
    if (st) return st;
  }
  Words hw;
  st = words_read(dw, &hw, s);
  if (st) return st;
  if (!words_valid(hw)) return MGB_ERR_INVALID_INPUT;
  int32_t* counts;
  MGB_SCRATCH(sc, counts, N + 1);
  st = prim::histogram(src->row_indices, n, counts, N, s);
  if (st) return st;
  MGB_CUDA_CHECK(cudaMemsetAsync(counts + N, 0, sizeof(int32_t), s));
  st = prim::exclusive_scan<int32_t, int32_t>(counts, dst->row_offsets, N + 1, s);
  if (st || n == 0) return st;
  if (hw.sorted) {
    MGB_CUDA_CHECK(cudaMemcpyAsync(dst->column_indices, src->column_indices, sizeof(int32_t) * n,
                                   cudaMemcpyDeviceToDevice, s));
    MGB_CUDA_CHECK(cudaMemcpyAsync(dst->values, src->values, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
    return MGB_SUCCESS;
  }
  // unsorted rows: stable partition by row (keys = COO position only)
  int32_t *zeros, *r2, *c2, *perm;
  MGB_SCRATCH(sc, zeros, n);
  MGB_SCRATCH(sc, r2, n);
  MGB_SCRATCH(sc, c2, n);
  MGB_SCRATCH(sc, perm, n);
  MGB_CUDA_CHECK(cudaMemsetAsync(zeros, 0, sizeof(int32_t) * n, s));
  st = prim::stable_sort_rows_cols(src->row_indices, zeros, n, N, r2, c2, perm, s);
  if (st) return st;
  gather_values<int32_t><<<grid_for(n), 256, 0, s>>>(src->column_indices, perm, dst->column_indices, n);
  MGB_LAUNCH_CHECK();
  gather_values<T><<<grid_for(n), 256, 0, s>>>(static_cast<const T*>(src->values), perm,
                                                static_cast<T*>(dst->values), n);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

// ---------------------------------------------------------------- DIA -> COO
// impl/Dia/Serial/Morpheus_Convert_Impl.hpp:72-118 (slab order = diagonal-major)
template <typename T>
__global__ void dia_flags(const int32_t* __restrict__ offs, const T* __restrict__ vals, int64_t nrows,
                          int64_t ncols, int64_t pitch, int64_t total, uint8_t* flags) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / pitch, row = t - i * pitch;
    const int64_t col = row + offs[i];
    flags[t] = (row < nrows && col >= 0 && col < ncols && vals[t] != T(0)) ? 1 : 0;
  }
}

template <typename T>
__global__ void dia_scatter(const int32_t* __restrict__ offs, const T* __restrict__ vals, int64_t pitch,
                            int64_t total, const uint8_t* __restrict__ flags, const int64_t* __restrict__ pos,
                            int64_t limit, int32_t* rows, int32_t* cols, T* out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    if (!flags[t]) continue;
    const int64_t p = pos[t];
    if (p >= limit) continue;
    const int64_t i = t / pitch, row = t - i * pitch;
    rows[p] = (int32_t)row;
    cols[p] = (int32_t)(row + offs[i]);
    out[p] = vals[t];
  }
}

// writes the DIA entries (nonzero, in range) into dst at [0, found); returns found
template <typename T>
int dia_part_to_coo(const mgb_dia* src, mgb_coo* dst, int64_t limit, int64_t* found, cudaStream_t s) {
  *found = 0;
  const int64_t total = src->pitch * src->ndiags;
  if (total == 0) return MGB_SUCCESS;
  Scratch sc(s);
  uint8_t* flags;
  int64_t *pos, *d_total;
  MGB_SCRATCH(sc, flags, total);
  MGB_SCRATCH(sc, pos, total);
  MGB_SCRATCH(sc, d_total, 1);
  dia_flags<T><<<grid_for(total), 256, 0, s>>>(src->diagonal_offsets, static_cast<const T*>(src->values),
                                               src->nrows, src->ncols, src->pitch, total, flags);
  MGB_LAUNCH_CHECK();
  int st = prim::exclusive_scan<uint8_t, int64_t>(flags, pos, total, s, d_total);
  if (st) return st;
  dia_scatter<T><<<grid_for(total), 256, 0, s>>>(src->diagonal_offsets, static_cast<const T*>(src->values),
                                                 src->pitch, total, flags, pos, limit, dst->row_indices,
                                                 dst->column_indices, static_cast<T*>(dst->values));
  MGB_LAUNCH_CHECK();
  return prim::to_host(d_total, found, s);
}

int check_dia(const mgb_dia* d) {
  MGB_REQUIRE(d != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(d->nrows >= 0 && d->ncols >= 0 && d->nnz >= 0 && d->ndiags >= 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(d->ndiags == 0 || (d->pitch >= d->nrows && d->diagonal_offsets && d->values), MGB_ERR_BAD_ARGUMENT);
  return MGB_SUCCESS;
}

template <typename T>
int dia_to_coo(const mgb_dia* src, mgb_coo* dst, cudaStream_t s) {
  int st = check_dia(src);
  if (st) return st;
  st = check_coo_dst(dst, src->nrows, src->ncols, src->nnz);
  if (st || src->nnz == 0) return st;
  st = zero_coo<T>(dst, s);
  if (st) return st;
  int64_t found = 0;
  st = dia_part_to_coo<T>(src, dst, dst->nnz, &found, s);
  if (st) return st;
  MGB_REQUIRE(found <= src->nnz, MGB_ERR_RUNTIME);  // the reference would write past dst
  return sort_if_unsorted<T>(dst, s);
}

// ---------------------------------------------------------------- COO -> DIA
// impl/Dia/Serial/Morpheus_Convert_Impl.hpp:120-169
__global__ void diag_bins(const int32_t* __restrict__ r, const int32_t* __restrict__ c, int64_t n, int64_t nrows,
                          int32_t* bins) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bins[i] = (int32_t)((int64_t)c[i] - r[i] + nrows - 1);
}
__global__ void nonzero_flags(const int32_t* __restrict__ a, int64_t n, uint8_t* f) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = a[i] != 0;
}
__global__ void bins_to_offsets(const uint8_t* __restrict__ f, const int32_t* __restrict__ slot, int64_t nb,
                                int64_t nrows, int32_t* offs) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x)
    if (f[b]) offs[slot[b]] = (int32_t)(b - nrows + 1);
}

// place values(row, slot) = v; owner != nullptr resolves collisions to the
// highest COO position (the reference's loop order: last write wins)
template <typename T>
__global__ void dia_place(const int32_t* __restrict__ r, const int32_t* __restrict__ bins, const T* __restrict__ v,
                          int64_t n, const int32_t* __restrict__ slot, int64_t pitch, T* vals, int32_t* owner,
                          int pass) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t at = r[i] + pitch * (int64_t)slot[bins[i]];
    if (owner == nullptr) vals[at] = v[i];
    else if (pass == 0) atomicMax(owner + at, (int32_t)i);
    else if (owner[at] == (int32_t)i) vals[at] = v[i];
  }
}

int diag_histogram(const mgb_coo* src, int32_t** bins, int32_t** counts, Scratch& sc, cudaStream_t s) {
  const int64_t nb = src->nrows + src->ncols - 1;
  MGB_SCRATCH(sc, *bins, src->nnz);
  MGB_SCRATCH(sc, *counts, nb > 0 ? nb : 1);
  if (src->nnz) {
    diag_bins<<<grid_for(src->nnz), 256, 0, s>>>(src->row_indices, src->column_indices, src->nnz, src->nrows, *bins);
    MGB_LAUNCH_CHECK();
  }
  return prim::histogram(*bins, src->nnz, *counts, nb, s);
}

// Argument checks of a COO source (the index range checks are queued with
// validate_async and read with the caller's other words).
int check_coo_args(const mgb_coo* src) {
  MGB_REQUIRE(src != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(src->nrows >= 0 && src->ncols >= 0 && src->nnz >= 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(src->nnz == 0 || (src->row_indices && src->column_indices && src->values), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(src->nrows + src->ncols < INT32_MAX, MGB_ERR_INVALID_INPUT);
  return MGB_SUCCESS;
}

// COO -> DIA sizes: the diagonal histogram, its occupied bins and their
// exclusive scan (slot of every occupied diagonal), queued with the
// validation and, when `flags`, the sortedness flags; one host read.
struct DiaPlan {
  int32_t *bins = nullptr, *counts = nullptr, *slot = nullptr;
  uint8_t* f = nullptr;
  Words h{};
};
int dia_plan(const mgb_coo* src, bool flags, DiaPlan* p, Scratch& sc, cudaStream_t s) {
  int st = check_coo_args(src);
  if (st) return st;
  Words* dw;
  st = words_alloc(sc, &dw, s);
  if (st) return st;
  st = validate_async(src->row_indices, src->column_indices, src->nnz, src->nrows, src->ncols, dw, s);
  if (st) return st;
  if (src->nnz > 0) {
    const int64_t nb = src->nrows + src->ncols - 1;
    st = diag_histogram(src, &p->bins, &p->counts, sc, s);
    if (st) return st;
    MGB_SCRATCH(sc, p->f, nb);
    MGB_SCRATCH(sc, p->slot, nb);
    nonzero_flags<<<grid_for(nb), 256, 0, s>>>(p->counts, nb, p->f);
    MGB_LAUNCH_CHECK();
    st = prim::exclusive_scan<uint8_t, int32_t>(p->f, p->slot, nb, s, &dw->total);
    if (st) return st;
    if (flags) {
      st = prim::coo_sorted_flags(src->row_indices, src->column_indices, src->nnz, &dw->sorted, &dw->dup, s);
      if (st) return st;
    }
  }
  st = words_read(dw, &p->h, s);
  if (st) return st;
  if (!words_valid(p->h)) return MGB_ERR_INVALID_INPUT;
  if (exceeds_tolerance(src->nrows, src->nnz, p->h.total)) return MGB_ERR_FORMAT_CONVERSION;
  return MGB_SUCCESS;
}

int coo_to_dia_plan(const mgb_coo* src, int64_t* ndiags, cudaStream_t s) {
  MGB_REQUIRE(ndiags != nullptr, MGB_ERR_BAD_ARGUMENT);
  *ndiags = 0;
  Scratch sc(s);
  DiaPlan p;
  const int st = dia_plan(src, false, &p, sc, s);
  if (st == MGB_SUCCESS || st == MGB_ERR_FORMAT_CONVERSION) *ndiags = p.h.total;
  return st;
}

template <typename T>
int coo_to_dia(const mgb_coo* src, mgb_dia* dst, cudaStream_t s) {
  Scratch sc(s);
  DiaPlan p;
  int st = dia_plan(src, true, &p, sc, s);
  if (st) return st;
  const int64_t nd = p.h.total;
  MGB_REQUIRE(dst != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(dst->nrows == src->nrows && dst->ncols == src->ncols && dst->nnz == src->nnz && dst->ndiags == nd &&
                  dst->pitch >= src->nrows,
              MGB_ERR_INVALID_INPUT);
  if (nd == 0) return MGB_SUCCESS;
  MGB_REQUIRE(dst->diagonal_offsets && dst->values, MGB_ERR_BAD_ARGUMENT);
  const int64_t n = src->nnz, nb = src->nrows + src->ncols - 1;
  int32_t *bins = p.bins, *slot = p.slot;
  bins_to_offsets<<<grid_for(nb), 256, 0, s>>>(p.f, slot, nb, src->nrows, dst->diagonal_offsets);
  MGB_LAUNCH_CHECK();
  MGB_CUDA_CHECK(cudaMemsetAsync(dst->values, 0, sizeof(T) * dst->pitch * nd, s));
  const bool sorted = p.h.sorted != 0, dup = p.h.dup != 0;
  const T* v = static_cast<const T*>(src->values);
  T* out = static_cast<T*>(dst->values);
  if (sorted && !dup) {
    dia_place<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, bins, v, n, slot, dst->pitch, out, nullptr, 0);
    MGB_LAUNCH_CHECK();
  } else {
    int32_t* owner;
    MGB_SCRATCH(sc, owner, dst->pitch * nd);
    st = fill<int32_t>(owner, -1, dst->pitch * nd, s);
    if (st) return st;
    for (int pass = 0; pass < 2; pass++) {
      dia_place<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, bins, v, n, slot, dst->pitch, out, owner, pass);
      MGB_LAUNCH_CHECK();
    }
  }
  return MGB_SUCCESS;
}

// ---------------------------------------------------------------- ELL -> COO
// impl/Ell/Serial/Morpheus_Convert_Impl.hpp:68-109
__global__ void ell_row_counts(const int32_t* __restrict__ ci, int64_t nrows, int64_t width, int64_t pitch,
                               int32_t* counts) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = 0;
    for (int64_t k = 0; k < width; k++) c += ci[r + pitch * k] != MGB_INVALID_INDEX;
    counts[r] = c;
  }
}

// per row: ELL slots in order, then (HYB) the row's COO-prefix entries
template <typename T>
__global__ void ell_rows_to_coo(const int32_t* __restrict__ ci, const T* __restrict__ ev, int64_t nrows,
                                int64_t width, int64_t pitch, const int32_t* __restrict__ pos, int64_t limit,
                                const int32_t* __restrict__ coo_start, const int32_t* __restrict__ coo_count,
                                const int32_t* __restrict__ cc, const T* __restrict__ cv, int32_t* rows,
                                int32_t* cols, T* out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = pos[r];
    for (int64_t k = 0; k < width; k++) {
      const int32_t c = ci[r + pitch * k];
      if (c != MGB_INVALID_INDEX) {
        if (p < limit) { rows[p] = (int32_t)r; cols[p] = c; out[p] = ev[r + pitch * k]; }
        p++;
      }
    }
    if (coo_count) {
      const int64_t a = coo_start[r], cnt = coo_count[r];
      for (int64_t j = a; j < a + cnt; j++) {
        if (p < limit) { rows[p] = (int32_t)r; cols[p] = cc[j]; out[p] = cv[j]; }
        p++;
      }
    }
  }
}

int check_ell(const mgb_ell* e) {
  MGB_REQUIRE(e != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(e->nrows >= 0 && e->ncols >= 0 && e->nnz >= 0 && e->width >= 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(e->width == 0 || (e->pitch >= e->nrows && e->column_indices && e->values), MGB_ERR_BAD_ARGUMENT);
  return MGB_SUCCESS;
}

__global__ void add_i32(int32_t* a, const int32_t* __restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] += b[i];
}

// ELL (+ optional HYB COO-prefix) -> pre-sort COO in row-major order;
// *found = entries produced (entries beyond dst->nnz are counted, not written)
template <typename T>
int ell_like_to_coo(const mgb_ell* e, const mgb_coo* cpart, int64_t coo_prefix, mgb_coo* dst, int64_t* found,
                    cudaStream_t s) {
  const int64_t N = e->nrows;
  *found = 0;
  if (N == 0) return MGB_SUCCESS;
  Scratch sc(s);
  int32_t *counts, *pos, *coo_counts = nullptr, *coo_start = nullptr;
  int64_t* d_total;
  MGB_SCRATCH(sc, counts, N + 1);
  MGB_SCRATCH(sc, pos, N + 1);
  MGB_SCRATCH(sc, d_total, 1);
  if (e->width > 0) {
    ell_row_counts<<<grid_for(N), 256, 0, s>>>(e->column_indices, N, e->width, e->pitch, counts);
    MGB_LAUNCH_CHECK();
  } else {
    MGB_CUDA_CHECK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * N, s));
  }
  MGB_CUDA_CHECK(cudaMemsetAsync(counts + N, 0, sizeof(int32_t), s));
  int st;
  if (cpart && coo_prefix > 0) {
    MGB_SCRATCH(sc, coo_counts, N + 1);
    MGB_SCRATCH(sc, coo_start, N + 1);
    st = prim::histogram(cpart->row_indices, coo_prefix, coo_counts, N, s);
    if (st) return st;
    MGB_CUDA_CHECK(cudaMemsetAsync(coo_counts + N, 0, sizeof(int32_t), s));
    st = prim::exclusive_scan<int32_t, int32_t>(coo_counts, coo_start, N + 1, s);
    if (st) return st;
    add_i32<<<grid_for(N), 256, 0, s>>>(counts, coo_counts, N);
    MGB_LAUNCH_CHECK();
  }
  st = prim::exclusive_scan<int32_t, int32_t>(counts, pos, N + 1, s, d_total);
  if (st) return st;
  ell_rows_to_coo<T><<<grid_for(N), 256, 0, s>>>(
      e->column_indices, static_cast<const T*>(e->values), N, e->width, e->pitch, pos, dst->nnz, coo_start,
      coo_counts, cpart ? cpart->column_indices : nullptr, cpart ? static_cast<const T*>(cpart->values) : nullptr,
      dst->row_indices, dst->column_indices, static_cast<T*>(dst->values));
  MGB_LAUNCH_CHECK();
  return prim::to_host(d_total, found, s);
}

template <typename T>
int ell_to_coo(const mgb_ell* src, mgb_coo* dst, cudaStream_t s) {
  int st = check_ell(src);
  if (st) return st;
  st = check_coo_dst(dst, src->nrows, src->ncols, src->nnz);
  if (st || src->nnz == 0) return st;
  st = zero_coo<T>(dst, s);
  if (st) return st;
  int64_t found = 0;
  st = ell_like_to_coo<T>(src, nullptr, 0, dst, &found, s);
  if (st) return st;
  MGB_REQUIRE(found <= src->nnz, MGB_ERR_RUNTIME);
  return sort_if_unsorted<T>(dst, s);
}

// ---------------------------------------------------------------- HYB -> COO
// impl/Hyb/Serial/Morpheus_Convert_Impl.hpp:62-108.  The COO part is consumed
// row by row while its row index equals the current row: exactly its longest
// prefix with non-decreasing in-range rows.
__global__ void first_consume_break(const int32_t* __restrict__ r, int64_t n, int64_t nrows,
                                    unsigned long long* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = r[i];
    if (v < 0 || v >= nrows || (i > 0 && v < r[i - 1])) atomicMin(out, (unsigned long long)i);
  }
}

template <typename T>
int hyb_to_coo(const mgb_hyb* src, mgb_coo* dst, cudaStream_t s) {
  MGB_REQUIRE(src != nullptr, MGB_ERR_BAD_ARGUMENT);
  int st = check_ell(&src->ell);
  if (st) return st;
  const mgb_coo* c = &src->coo;
  MGB_REQUIRE(c->nnz >= 0 && (c->nnz == 0 || (c->row_indices && c->column_indices && c->values)),
              MGB_ERR_BAD_ARGUMENT);
  const int64_t nnz = src->ell.nnz + c->nnz;
  st = check_coo_dst(dst, src->ell.nrows, src->ell.ncols, nnz);
  if (st || nnz == 0) return st;
  st = zero_coo<T>(dst, s);
  if (st) return st;
  int64_t prefix = c->nnz;
  if (c->nnz > 0) {
    Scratch sc(s);
    unsigned long long* d;
    MGB_SCRATCH(sc, d, 1);
    const unsigned long long big = ~0ull;
    MGB_CUDA_CHECK(cudaMemcpyAsync(d, &big, sizeof(big), cudaMemcpyHostToDevice, s));
    first_consume_break<<<grid_for(c->nnz), 256, 0, s>>>(c->row_indices, c->nnz, src->ell.nrows, d);
    MGB_LAUNCH_CHECK();
    unsigned long long h;
    st = prim::to_host(d, &h, s);
    if (st) return st;
    if (h != big) prefix = (int64_t)h;
  }
  int64_t found = 0;
  st = ell_like_to_coo<T>(&src->ell, c, prefix, dst, &found, s);
  if (st) return st;
  MGB_REQUIRE(found <= nnz, MGB_ERR_RUNTIME);
  return sort_if_unsorted<T>(dst, s);
}

// ------------------------------------------------------- COO -> ELL / HYB
// slot of entry i = i - (start of its run of equal row indices): the
// reference's loop restarts n whenever the row index changes
// (impl/Ell/Serial/Morpheus_Convert_Impl.hpp:160-172, Hyb :174-195).
__global__ void run_flags(const int32_t* __restrict__ r, int64_t n, uint8_t* f) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = (i == 0 || r[i] != r[i - 1]) ? 1 : 0;
}
__global__ void run_starts(const uint8_t* __restrict__ f, const int32_t* __restrict__ excl, int64_t n,
                           int32_t* starts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (f[i]) starts[excl[i]] = (int32_t)i;
}
__global__ void run_slots(const uint8_t* __restrict__ f, const int32_t* __restrict__ excl,
                          const int32_t* __restrict__ starts, int64_t n, int32_t* slot) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    slot[i] = (int32_t)(i - starts[excl[i] + f[i] - 1]);
}
__global__ void sorted_slots(const int32_t* __restrict__ r, const int32_t* __restrict__ row_start, int64_t n,
                             int32_t* slot) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    slot[i] = (int32_t)(i - row_start[r[i]]);
}

// Slot of every entry in its row (the reference's placement counter, which
// restarts whenever the row changes).  rows_sorted: the rows are
// non-decreasing (read by the caller); counts: the row histogram (N + 1
// entries, the last one zero).
int compute_slots(const mgb_coo* src, bool rows_sorted_flag, int32_t* counts, int32_t* slot, bool* collisions,
                  Scratch& sc, cudaStream_t s) {
  const int64_t n = src->nnz, N = src->nrows;
  *collisions = false;
  if (n == 0) return MGB_SUCCESS;
  int st = MGB_SUCCESS;
  if (rows_sorted_flag) {
    int32_t* start;
    MGB_SCRATCH(sc, start, N + 1);
    st = prim::exclusive_scan<int32_t, int32_t>(counts, start, N + 1, s);
    if (st) return st;
    sorted_slots<<<grid_for(n), 256, 0, s>>>(src->row_indices, start, n, slot);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
  *collisions = true;
  uint8_t* f;
  int32_t *excl, *starts;
  MGB_SCRATCH(sc, f, n);
  MGB_SCRATCH(sc, excl, n);
  MGB_SCRATCH(sc, starts, n);
  run_flags<<<grid_for(n), 256, 0, s>>>(src->row_indices, n, f);
  MGB_LAUNCH_CHECK();
  st = prim::exclusive_scan<uint8_t, int32_t>(f, excl, n, s);
  if (st) return st;
  run_starts<<<grid_for(n), 256, 0, s>>>(f, excl, n, starts);
  MGB_LAUNCH_CHECK();
  run_slots<<<grid_for(n), 256, 0, s>>>(f, excl, starts, n, slot);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

// ELL placement of entries with slot < W; owner resolves collisions to the
// highest position.  Entries with slot >= W are marked for the COO part.
template <typename T>
__global__ void ell_place(const int32_t* __restrict__ r, const int32_t* __restrict__ c, const T* __restrict__ v,
                          const int32_t* __restrict__ slot, int64_t n, int64_t W, int64_t pitch, int32_t* eci,
                          T* ev, int32_t* owner, int pass, uint8_t* to_coo) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = slot[i];
    if (k >= W) {
      if (to_coo && pass == 0) to_coo[i] = 1;
      continue;
    }
    if (to_coo && pass == 0) to_coo[i] = 0;
    const int64_t at = r[i] + pitch * k;
    if (owner == nullptr) {
      eci[at] = c[i];
      ev[at] = v[i];
    } else if (pass == 0) {
      atomicMax(owner + at, (int32_t)i);
    } else if (owner[at] == (int32_t)i) {
      eci[at] = c[i];
      ev[at] = v[i];
    }
  }
}

template <typename T>
__global__ void coo_part_scatter(const int32_t* __restrict__ r, const int32_t* __restrict__ c,
                                 const T* __restrict__ v, const uint8_t* __restrict__ f,
                                 const int64_t* __restrict__ pos, int64_t n, int64_t limit, int32_t* orow,
                                 int32_t* ocol, T* oval) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (f[i] && pos[i] < limit) {
      orow[pos[i]] = r[i];
      ocol[pos[i]] = c[i];
      oval[pos[i]] = v[i];
    }
}

template <typename T>
int place_ell(const mgb_coo* src, mgb_ell* e, int64_t W, const int32_t* slot, bool collisions, uint8_t* to_coo,
              Scratch& sc, cudaStream_t s) {
  const int64_t n = src->nnz;
  const int64_t slab = e->pitch * e->width;
  int st = fill<int32_t>(e->column_indices, MGB_INVALID_INDEX, slab, s);
  if (st) return st;
  if (slab) MGB_CUDA_CHECK(cudaMemsetAsync(e->values, 0, sizeof(T) * slab, s));
  if (n == 0) return MGB_SUCCESS;
  const T* v = static_cast<const T*>(src->values);
  T* ev = static_cast<T*>(e->values);
  if (!collisions) {
    ell_place<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, src->column_indices, v, slot, n, W, e->pitch,
                                             e->column_indices, ev, nullptr, 0, to_coo);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
  int32_t* owner;
  MGB_SCRATCH(sc, owner, slab > 0 ? slab : 1);
  st = fill<int32_t>(owner, -1, slab, s);
  if (st) return st;
  for (int pass = 0; pass < 2; pass++) {
    ell_place<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, src->column_indices, v, slot, n, W, e->pitch,
                                             e->column_indices, ev, owner, pass, to_coo);
    MGB_LAUNCH_CHECK();
  }
  return MGB_SUCCESS;
}

// The row histogram of a COO source (N + 1 entries, the last one zero),
// queued with the validation, the rows-sorted flag and (width > 0) the
// number of entries a width-W ELL part holds, or (width == 0) the longest
// row; one host read.
struct RowPlan {
  int32_t* counts = nullptr;
  Words h{};
};
int row_plan(const mgb_coo* src, int64_t width, RowPlan* p, Scratch& sc, cudaStream_t s);

int coo_to_ell_plan(const mgb_coo* src, int64_t* epr, cudaStream_t s) {
  MGB_REQUIRE(epr != nullptr, MGB_ERR_BAD_ARGUMENT);
  *epr = 0;
  int st = check_coo_args(src);
  if (st) return st;
  if (src->nrows == 0) return src->nnz > 0 ? MGB_ERR_INVALID_INPUT : MGB_SUCCESS;  // every row out of range
  Scratch sc(s);
  RowPlan p;
  st = row_plan(src, 0, &p, sc, s);
  if (st) return st;
  *epr = p.h.maxv > 0 ? p.h.maxv : 0;
  if (exceeds_tolerance(src->nrows, src->nnz, *epr)) return MGB_ERR_FORMAT_CONVERSION;
  return MGB_SUCCESS;
}

template <typename T>
int coo_to_ell(const mgb_coo* src, mgb_ell* dst, cudaStream_t s) {
  int st = check_coo_args(src);
  if (st) return st;
  if (src->nrows == 0 && src->nnz > 0) return MGB_ERR_INVALID_INPUT;  // every row out of range
  Scratch sc(s);
  RowPlan p;
  int64_t W = 0;
  if (src->nrows > 0) {
    st = row_plan(src, 0, &p, sc, s);
    if (st) return st;
    W = p.h.maxv > 0 ? p.h.maxv : 0;
    if (exceeds_tolerance(src->nrows, src->nnz, W)) return MGB_ERR_FORMAT_CONVERSION;
  }
  MGB_REQUIRE(dst != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(dst->nrows == src->nrows && dst->ncols == src->ncols && dst->nnz == src->nnz &&
                  dst->entries_per_row == W && dst->width >= W && dst->pitch >= src->nrows,
              MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(dst->width * dst->pitch == 0 || (dst->column_indices && dst->values), MGB_ERR_BAD_ARGUMENT);
  int32_t* slot;
  MGB_SCRATCH(sc, slot, src->nnz);
  bool coll = false;
  st = compute_slots(src, p.h.sorted != 0, p.counts, slot, &coll, sc, s);
  if (st) return st;
  return place_ell<T>(src, dst, W, slot, coll, nullptr, sc, s);
}

__global__ void sum_min_kernel(const int32_t* __restrict__ counts, int64_t n, int64_t W, unsigned long long* out) {
  int64_t acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += min((int64_t)counts[i], W);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, (unsigned long long)acc);
}

// impl/Hyb/Serial/Morpheus_Convert_Impl.hpp:110-151 (width = max(1, nnz/nrows)
// unless the caller passes one)
int row_plan(const mgb_coo* src, int64_t width, RowPlan* p, Scratch& sc, cudaStream_t s) {
  const int64_t N = src->nrows;
  Words* dw;
  int st = words_alloc(sc, &dw, s);
  if (st) return st;
  st = validate_async(src->row_indices, src->column_indices, src->nnz, N, src->ncols, dw, s);
  if (st) return st;
  MGB_SCRATCH(sc, p->counts, N + 1);
  st = prim::histogram(src->row_indices, src->nnz, p->counts, N, s);
  if (st) return st;
  MGB_CUDA_CHECK(cudaMemsetAsync(p->counts + N, 0, sizeof(int32_t), s));
  if (width > 0) {
    sum_min_kernel<<<grid_for(N), 256, 0, s>>>(p->counts, N, width, reinterpret_cast<unsigned long long*>(&dw->total));
    MGB_LAUNCH_CHECK();
  } else {
    st = prim::reduce_max_i32(p->counts, N, &dw->maxv, s);
    if (st) return st;
  }
  st = prim::rows_sorted_flag(src->row_indices, src->nnz, &dw->sorted, s);
  if (st) return st;
  st = words_read(dw, &p->h, s);
  if (st) return st;
  return words_valid(p->h) ? MGB_SUCCESS : MGB_ERR_INVALID_INPUT;
}

int coo_to_hyb_plan(const mgb_coo* src, int64_t width, int64_t* epr, int64_t* ell_nnz, int64_t* coo_nnz,
                    cudaStream_t s) {
  MGB_REQUIRE(epr && ell_nnz && coo_nnz && width >= 0, MGB_ERR_BAD_ARGUMENT);
  int st = check_coo_args(src);
  if (st) return st;
  MGB_REQUIRE(src->nrows > 0, MGB_ERR_INVALID_INPUT);  // the reference divides by nrows
  const int64_t W = width > 0 ? width : std::max<int64_t>(1, src->nnz / src->nrows);
  Scratch sc(s);
  RowPlan p;
  st = row_plan(src, W, &p, sc, s);
  if (st) return st;
  *epr = W;
  *ell_nnz = p.h.total;
  *coo_nnz = src->nnz - p.h.total;
  if (exceeds_tolerance(src->nrows, *ell_nnz, W)) return MGB_ERR_FORMAT_CONVERSION;
  return MGB_SUCCESS;
}

template <typename T>
int coo_to_hyb(const mgb_coo* src, mgb_hyb* dst, cudaStream_t s) {
  MGB_REQUIRE(dst != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(dst->ell.entries_per_row >= 0, MGB_ERR_BAD_ARGUMENT);
  int st = check_coo_args(src);
  if (st) return st;
  MGB_REQUIRE(src->nrows > 0, MGB_ERR_INVALID_INPUT);  // the reference divides by nrows
  const int64_t W = dst->ell.entries_per_row > 0 ? dst->ell.entries_per_row
                                                 : std::max<int64_t>(1, src->nnz / src->nrows);
  Scratch sc(s);
  RowPlan p;
  st = row_plan(src, W, &p, sc, s);
  if (st) return st;
  const int64_t en = p.h.total, cn = src->nnz - p.h.total;
  if (exceeds_tolerance(src->nrows, en, W)) return MGB_ERR_FORMAT_CONVERSION;
  mgb_ell* e = &dst->ell;
  mgb_coo* c = &dst->coo;
  MGB_REQUIRE(e->nrows == src->nrows && e->ncols == src->ncols && e->nnz == en && e->entries_per_row == W &&
                  e->width >= W && e->pitch >= src->nrows,
              MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(c->nrows == src->nrows && c->ncols == src->ncols && c->nnz == cn, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(e->width * e->pitch == 0 || (e->column_indices && e->values), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(cn == 0 || (c->row_indices && c->column_indices && c->values), MGB_ERR_BAD_ARGUMENT);
  const int64_t n = src->nnz;
  st = zero_coo<T>(c, s);
  if (st) return st;
  int32_t* slot;
  uint8_t* to_coo;
  MGB_SCRATCH(sc, slot, n);
  MGB_SCRATCH(sc, to_coo, n);
  bool coll = false;
  st = compute_slots(src, p.h.sorted != 0, p.counts, slot, &coll, sc, s);
  if (st) return st;
  st = place_ell<T>(src, e, W, slot, coll, to_coo, sc, s);
  if (st || n == 0) return st;
  int64_t* pos;
  MGB_SCRATCH(sc, pos, n);
  st = prim::exclusive_scan<uint8_t, int64_t>(to_coo, pos, n, s);
  if (st) return st;
  coo_part_scatter<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, src->column_indices,
                                                  static_cast<const T*>(src->values), to_coo, pos, n, cn,
                                                  c->row_indices, c->column_indices, static_cast<T*>(c->values));
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

// ---------------------------------------------------------------- HDC -> COO
// impl/Hdc/Serial/Morpheus_Convert_Impl.hpp:64-130
template <typename T>
int hdc_to_coo(const mgb_hdc* src, mgb_coo* dst, cudaStream_t s) {
  MGB_REQUIRE(src != nullptr, MGB_ERR_BAD_ARGUMENT);
  int st = check_dia(&src->dia);
  if (st) return st;
  const mgb_csr* c = &src->csr;
  MGB_REQUIRE(c->nnz >= 0 && c->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(c->nnz == 0 || (c->column_indices && c->values), MGB_ERR_BAD_ARGUMENT);
  const int64_t nnz = src->dia.nnz + c->nnz;
  st = check_coo_dst(dst, src->dia.nrows, src->dia.ncols, nnz);
  if (st || nnz == 0) return st;
  st = zero_coo<T>(dst, s);
  if (st) return st;
  int64_t found = 0;
  st = dia_part_to_coo<T>(&src->dia, dst, nnz, &found, s);
  if (st) return st;
  MGB_REQUIRE(found + c->nnz <= nnz, MGB_ERR_RUNTIME);
  if (c->nnz > 0) {
    expand_rows<<<grid_for(c->nrows), 256, 0, s>>>(c->row_offsets, c->nrows, c->nnz, dst->row_indices, found);
    MGB_LAUNCH_CHECK();
    MGB_CUDA_CHECK(cudaMemcpyAsync(dst->column_indices + found, c->column_indices, sizeof(int32_t) * c->nnz,
                                   cudaMemcpyDeviceToDevice, s));
    MGB_CUDA_CHECK(cudaMemcpyAsync(static_cast<T*>(dst->values) + found, c->values, sizeof(T) * c->nnz,
                                   cudaMemcpyDeviceToDevice, s));
  }
  return sort_if_unsorted<T>(dst, s);
}

// ---------------------------------------------------------------- COO -> HDC
// impl/Hdc/Serial/Morpheus_Convert_Impl.hpp:132-226
__global__ void true_diag_flags(const int32_t* __restrict__ counts, int64_t nb, int32_t min_elem, uint8_t* f,
                                int32_t* dia_counts) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
    const bool t = counts[b] >= min_elem;
    f[b] = t;
    dia_counts[b] = t ? counts[b] : 0;
  }
}
// midpoint bin recorded as offset 0 (exact only for square matrices)
__global__ void hdc_offsets(const uint8_t* __restrict__ f, const int32_t* __restrict__ slot, int64_t nb,
                            int64_t nrows, int32_t* offs) {
  const int64_t mid = nb / 2;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x)
    if (f[b]) offs[slot[b]] = (b == mid) ? 0 : (int32_t)(b - nrows + 1);
}

// first matching stored offset (the reference's break on the first match)
__global__ void hdc_classify(const int32_t* __restrict__ r, const int32_t* __restrict__ c, int64_t n,
                             const int32_t* __restrict__ offs, int64_t nd, int32_t* dslot, uint8_t* is_csr) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = c[i] - r[i];
    int64_t lo = 0, hi = nd;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (offs[mid] < d) lo = mid + 1; else hi = mid;
    }
    const bool hit = lo < nd && offs[lo] == d;
    dslot[i] = hit ? (int32_t)lo : -1;
    is_csr[i] = hit ? 0 : 1;
  }
}

template <typename T>
__global__ void hdc_dia_place(const int32_t* __restrict__ r, const T* __restrict__ v, const int32_t* __restrict__ dslot,
                              int64_t n, int64_t pitch, T* vals, int32_t* owner, int pass) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (dslot[i] < 0) continue;
    const int64_t at = r[i] + pitch * (int64_t)dslot[i];
    if (owner == nullptr) vals[at] = v[i];
    else if (pass == 0) atomicMax(owner + at, (int32_t)i);
    else if (owner[at] == (int32_t)i) vals[at] = v[i];
  }
}

// COO -> HDC sizes: the diagonal histogram, the true diagonals (>= floor(0.2
// N) entries), their slots and entry count, queued with the validation and
// (when `flags`) the sortedness flags; one host read.
struct HdcPlan {
  int32_t *bins = nullptr, *counts = nullptr, *slot = nullptr;
  uint8_t* f = nullptr;
  Words h{};
};
int hdc_plan(const mgb_coo* src, bool flags, HdcPlan* p, Scratch& sc, cudaStream_t s) {
  int st = check_coo_args(src);
  if (st) return st;
  MGB_REQUIRE(src->nrows > 0 && src->ncols > 0, MGB_ERR_INVALID_INPUT);
  const int64_t nb = src->nrows + src->ncols - 1;
  const int32_t min_elem = (int32_t)((double)src->nrows * 0.2);  // HdcMatrix::true_diagonal_ratio
  Words* dw;
  st = words_alloc(sc, &dw, s);
  if (st) return st;
  st = validate_async(src->row_indices, src->column_indices, src->nnz, src->nrows, src->ncols, dw, s);
  if (st) return st;
  st = diag_histogram(src, &p->bins, &p->counts, sc, s);
  if (st) return st;
  int32_t* dcounts;
  MGB_SCRATCH(sc, p->f, nb);
  MGB_SCRATCH(sc, dcounts, nb);
  MGB_SCRATCH(sc, p->slot, nb);
  true_diag_flags<<<grid_for(nb), 256, 0, s>>>(p->counts, nb, min_elem, p->f, dcounts);
  MGB_LAUNCH_CHECK();
  st = prim::exclusive_scan<uint8_t, int32_t>(p->f, p->slot, nb, s, &dw->total);
  if (st) return st;
  st = prim::reduce_sum_i32(dcounts, nb, &dw->total2, s);
  if (st) return st;
  if (flags && src->nnz > 0) {
    st = prim::coo_sorted_flags(src->row_indices, src->column_indices, src->nnz, &dw->sorted, &dw->dup, s);
    if (st) return st;
  }
  st = words_read(dw, &p->h, s);
  if (st) return st;
  if (!words_valid(p->h)) return MGB_ERR_INVALID_INPUT;
  if (exceeds_tolerance(src->nrows, p->h.total2, p->h.total)) return MGB_ERR_FORMAT_CONVERSION;
  return MGB_SUCCESS;
}

int coo_to_hdc_plan(const mgb_coo* src, int64_t* ndiags, int64_t* dia_nnz, int64_t* csr_nnz, cudaStream_t s) {
  MGB_REQUIRE(ndiags && dia_nnz && csr_nnz, MGB_ERR_BAD_ARGUMENT);
  Scratch sc(s);
  HdcPlan p;
  const int st = hdc_plan(src, false, &p, sc, s);
  if (st == MGB_SUCCESS || st == MGB_ERR_FORMAT_CONVERSION) {
    *ndiags = p.h.total;
    *dia_nnz = p.h.total2;
    *csr_nnz = src->nnz - p.h.total2;
  }
  return st;
}

template <typename T>
int coo_to_hdc(const mgb_coo* src, mgb_hdc* dst, cudaStream_t s) {
  MGB_REQUIRE(dst != nullptr, MGB_ERR_BAD_ARGUMENT);
  Scratch sc(s);
  HdcPlan p;
  int st = hdc_plan(src, true, &p, sc, s);
  if (st) return st;
  const int64_t nd = p.h.total, dn = p.h.total2, cn = src->nnz - p.h.total2;
  mgb_dia* D = &dst->dia;
  mgb_csr* C = &dst->csr;
  MGB_REQUIRE(D->nrows == src->nrows && D->ncols == src->ncols && D->nnz == dn && D->ndiags == nd &&
                  D->pitch >= src->nrows,
              MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(C->nrows == src->nrows && C->ncols == src->ncols && C->nnz == cn, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(C->row_offsets && (nd == 0 || (D->diagonal_offsets && D->values)), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(cn == 0 || (C->column_indices && C->values), MGB_ERR_BAD_ARGUMENT);
  const int64_t n = src->nnz, N = src->nrows, nb = src->nrows + src->ncols - 1;
  uint8_t* f = p.f;
  int32_t* slot = p.slot;
  if (nd > 0) {
    hdc_offsets<<<grid_for(nb), 256, 0, s>>>(f, slot, nb, N, D->diagonal_offsets);
    MGB_LAUNCH_CHECK();
    // std::sort of the stored offsets (impl/Hdc/Serial/Morpheus_Convert_Impl.hpp:193-195)
    std::vector<int32_t> h((size_t)nd);
    MGB_CUDA_CHECK(cudaMemcpyAsync(h.data(), D->diagonal_offsets, sizeof(int32_t) * nd, cudaMemcpyDeviceToHost, s));
    MGB_CUDA_CHECK(cudaStreamSynchronize(s));
    std::sort(h.begin(), h.end());
    MGB_CUDA_CHECK(cudaMemcpyAsync(D->diagonal_offsets, h.data(), sizeof(int32_t) * nd, cudaMemcpyHostToDevice, s));
    MGB_CUDA_CHECK(cudaMemsetAsync(D->values, 0, sizeof(T) * D->pitch * nd, s));
  }
  if (n == 0) {
    MGB_CUDA_CHECK(cudaMemsetAsync(C->row_offsets, 0, sizeof(int32_t) * (N + 1), s));
    return MGB_SUCCESS;
  }
  int32_t* dslot;
  uint8_t* is_csr;
  int64_t *cpos, *d_csr;
  MGB_SCRATCH(sc, dslot, n);
  MGB_SCRATCH(sc, is_csr, n);
  MGB_SCRATCH(sc, cpos, n);
  MGB_SCRATCH(sc, d_csr, 1);
  hdc_classify<<<grid_for(n), 256, 0, s>>>(src->row_indices, src->column_indices, n, D->diagonal_offsets, nd, dslot,
                                           is_csr);
  MGB_LAUNCH_CHECK();
  st = prim::exclusive_scan<uint8_t, int64_t>(is_csr, cpos, n, s, d_csr);
  if (st) return st;
  // a non-square matrix with a true diagonal in the midpoint bin sends more
  // entries to CSR than were counted (the reference writes out of bounds):
  // the scatter below stops at cn, and the count is checked at the end
  const T* v = static_cast<const T*>(src->values);
  const bool sorted = p.h.sorted != 0, dup = p.h.dup != 0;
  if (nd > 0) {
    if (sorted && !dup) {
      hdc_dia_place<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, v, dslot, n, D->pitch, static_cast<T*>(D->values),
                                                    nullptr, 0);
      MGB_LAUNCH_CHECK();
    } else {
      int32_t* owner;
      MGB_SCRATCH(sc, owner, D->pitch * nd);
      st = fill<int32_t>(owner, -1, D->pitch * nd, s);
      if (st) return st;
      for (int pass = 0; pass < 2; pass++) {
        hdc_dia_place<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, v, dslot, n, D->pitch,
                                                      static_cast<T*>(D->values), owner, pass);
        MGB_LAUNCH_CHECK();
      }
    }
  }
  // CSR part: entries in COO order (csr_entries counter of the reference),
  // row_offsets = exclusive scan of per-row counts, last = csr_nnz
  int32_t *rows_c, *counts_c;
  MGB_SCRATCH(sc, rows_c, cn > 0 ? cn : 1);
  MGB_SCRATCH(sc, counts_c, N + 1);
  if (cn > 0) {
    MGB_CUDA_CHECK(cudaMemsetAsync(C->column_indices, 0, sizeof(int32_t) * cn, s));
    MGB_CUDA_CHECK(cudaMemsetAsync(C->values, 0, sizeof(T) * cn, s));
    // slots the scatter leaves empty hold row N, which the histogram ignores
    st = fill<int32_t>(rows_c, (int32_t)N, cn, s);
    if (st) return st;
    coo_part_scatter<T><<<grid_for(n), 256, 0, s>>>(src->row_indices, src->column_indices, v, is_csr, cpos, n, cn,
                                                    rows_c, C->column_indices, static_cast<T*>(C->values));
    MGB_LAUNCH_CHECK();
  }
  st = prim::histogram(rows_c, cn, counts_c, N, s);
  if (st) return st;
  MGB_CUDA_CHECK(cudaMemsetAsync(counts_c + N, 0, sizeof(int32_t), s));
  st = prim::exclusive_scan<int32_t, int32_t>(counts_c, C->row_offsets, N + 1, s);
  if (st) return st;
  const int32_t last = (int32_t)cn;
  int64_t ncsr = 0;
  MGB_CUDA_CHECK(cudaMemcpyAsync(C->row_offsets + N, &last, sizeof(int32_t), cudaMemcpyHostToDevice, s));
  MGB_CUDA_CHECK(cudaMemcpyAsync(&ncsr, d_csr, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));  // 'last' and 'ncsr' live on this stack frame
  MGB_REQUIRE(ncsr <= cn, MGB_ERR_RUNTIME);
  return MGB_SUCCESS;
}

// ---------------------------------------------------------------- sort API
template <typename T>
int coo_sort(mgb_coo* A, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && A->nnz >= 0, MGB_ERR_BAD_ARGUMENT);
  if (A->nnz <= 1) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_indices && A->column_indices && A->values, MGB_ERR_BAD_ARGUMENT);
  Scratch sc(s);
  Words* dw;
  int st = words_alloc(sc, &dw, s);
  if (st) return st;
  st = prim::reduce_max_i32(A->row_indices, A->nnz, &dw->maxv, s);
  if (st) return st;
  // rows and columns must be >= 0 (the counting sort indexes by them)
  st = validate_async(A->row_indices, A->column_indices, A->nnz, INT32_MAX, INT32_MAX, dw, s);
  if (st) return st;
  Words hw;
  st = words_read(dw, &hw, s);
  if (st) return st;
  if (!words_valid(hw)) return MGB_ERR_INVALID_INPUT;
  return sort_coo_inplace<T>(A->row_indices, A->column_indices, static_cast<T*>(A->values), A->nnz,
                             (int64_t)hw.maxv + 1, s);
}

int coo_is_sorted(const mgb_coo* A, int* out, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && out != nullptr && A->nnz >= 0, MGB_ERR_BAD_ARGUMENT);
  *out = 1;
  if (A->nnz <= 1) return MGB_SUCCESS;
  bool sorted = false;
  int st = sorted_and_dup(A->row_indices, A->column_indices, A->nnz, &sorted, nullptr, s);
  if (st) return st;
  *out = sorted ? 1 : 0;
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

#define MGB_CONV_PAIR(NAME, SRC, DST)                                                            \
  int mgb_convert_##NAME##_f64(const SRC* src, DST* dst, void* stream) {                         \
    return mgb::NAME<double>(src, dst, mgb::as_stream(stream));                                  \
  }                                                                                              \
  int mgb_convert_##NAME##_f32(const SRC* src, DST* dst, void* stream) {                         \
    return mgb::NAME<float>(src, dst, mgb::as_stream(stream));                                   \
  }

extern "C" {

MGB_CONV_PAIR(csr_to_coo, mgb_csr, mgb_coo)
MGB_CONV_PAIR(coo_to_csr, mgb_coo, mgb_csr)
MGB_CONV_PAIR(dia_to_coo, mgb_dia, mgb_coo)
MGB_CONV_PAIR(coo_to_dia, mgb_coo, mgb_dia)
MGB_CONV_PAIR(ell_to_coo, mgb_ell, mgb_coo)
MGB_CONV_PAIR(coo_to_ell, mgb_coo, mgb_ell)
MGB_CONV_PAIR(hyb_to_coo, mgb_hyb, mgb_coo)
MGB_CONV_PAIR(coo_to_hyb, mgb_coo, mgb_hyb)
MGB_CONV_PAIR(hdc_to_coo, mgb_hdc, mgb_coo)
MGB_CONV_PAIR(coo_to_hdc, mgb_coo, mgb_hdc)

int mgb_convert_coo_to_dia_plan(const mgb_coo* src, int64_t* ndiags, void* stream) {
  return mgb::coo_to_dia_plan(src, ndiags, mgb::as_stream(stream));
}
int mgb_convert_coo_to_ell_plan(const mgb_coo* src, int64_t* entries_per_row, void* stream) {
  return mgb::coo_to_ell_plan(src, entries_per_row, mgb::as_stream(stream));
}
int mgb_convert_coo_to_hyb_plan(const mgb_coo* src, int64_t width, int64_t* entries_per_row, int64_t* ell_nnz,
                                int64_t* coo_nnz, void* stream) {
  return mgb::coo_to_hyb_plan(src, width, entries_per_row, ell_nnz, coo_nnz, mgb::as_stream(stream));
}
int mgb_convert_coo_to_hdc_plan(const mgb_coo* src, int64_t* ndiags, int64_t* dia_nnz, int64_t* csr_nnz,
                                void* stream) {
  return mgb::coo_to_hdc_plan(src, ndiags, dia_nnz, csr_nnz, mgb::as_stream(stream));
}
int mgb_coo_sort_by_row_and_column_f64(mgb_coo* A, void* stream) {
  return mgb::coo_sort<double>(A, mgb::as_stream(stream));
}
int mgb_coo_sort_by_row_and_column_f32(mgb_coo* A, void* stream) {
  return mgb::coo_sort<float>(A, mgb::as_stream(stream));
}
int mgb_coo_is_sorted(const mgb_coo* A, int* sorted, void* stream) {
  return mgb::coo_is_sorted(A, sorted, mgb::as_stream(stream));
}

}  // extern "C"
