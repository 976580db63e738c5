// analytics_counts.cu -- the reference's per-row / per-diagonal nonzero counts
// and its thresholded vector count, on the device:
//
//   count_nnz_per_row       core/src/Morpheus_MatrixAnalytics.hpp:112-124
//                           (Serial CSR: impl/Csr/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:57-62)
//   count_nnz_per_diagonal  core/src/Morpheus_MatrixAnalytics.hpp:206-218
//                           (index = column - row + nrows - 1, vector of nrows + ncols - 1;
//                           impl/Csr/Kokkos/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:59-76)
//   count_nnz(vec, thr)     core/src/Morpheus_VectorAnalytics.hpp:124 (entries > thr and != 0;
//                           impl/DenseVector/Kokkos/Morpheus_VectorAnalytics_Impl.hpp:122-145)
//
// Per format, with the reference's semantics (which differ between formats):
//   CSR / COO  every stored entry, per row and per diagonal
//   DIA        per row: diagonal slots whose column lies inside the matrix,
//              values not inspected (impl/Dia/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:40-72);
//              per diagonal: slots holding a nonzero value, over all pitch
//              rows of the slab (impl/Dia/Kokkos/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:37-78)
//   ELL        per row: slots with a valid column (impl/Ell/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:40-74);
//              per diagonal: with k = the row's slots holding a valid column
//              and a nonzero value, the first k slots of the row are
//              inspected and those that are valid and nonzero counted
//              (impl/Ell/Kokkos/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:36-124;
//              a row whose entries do not come first loses some)
//   HYB / HDC  the ELL / DIA part (with init) plus the COO / CSR part
//              (impl/Hyb/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:42-58,
//              impl/Hyb/Serial/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:43-59,
//              impl/Hdc/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:42-58,
//              impl/Hdc/Serial/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:42-58)
//
// With init != 0 the output is zeroed first, else counts are added to it.
// Entries whose row or column lies outside the matrix are skipped (the
// reference indexes out of bounds there).  All counts are int32 like the
// reference's index vectors; the calls are asynchronous except
// mgb_count_nnz_vector, which returns its count to the host.
#include "primitives.cuh"

namespace mgb {
namespace {

inline unsigned grid_for(int64_t n) { return prim::blocks_for(n, 256, (int64_t)num_sms() * 16); }

__global__ void csr_row_counts(const int32_t* __restrict__ ro, int64_t nrows, int32_t* __restrict__ out, int init) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x)
    out[r] = (init ? 0 : out[r]) + (ro[r + 1] - ro[r]);
}

__global__ void coo_row_counts(const int32_t* __restrict__ ri, int64_t nnz, int64_t nrows, int32_t* out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = ri[k];
    if (r >= 0 && r < nrows) prim::warp_merged_add(out, r);
  }
}

__global__ void csr_diag_counts(const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, int64_t nrows,
                                int64_t ncols, int32_t* out) {
  // one warp per row: coalesced column reads for long rows; few hot
  // diagonals per CTA are counted in shared memory first
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrows; r += warps) {
    for (int32_t j = ro[r] + lane; j < ro[r + 1]; j += 32) {
      const int64_t c = ci[j];
      if (c >= 0 && c < ncols) prim::hist_add(h, out, (unsigned long long)(c - r + nrows - 1));
    }
  }
  __syncthreads();
  prim::hist_flush(h, out);
}

__global__ void coo_diag_counts(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci, int64_t nnz,
                                int64_t nrows, int64_t ncols, int32_t* out) {
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = ri[k], c = ci[k];
    if (r >= 0 && r < nrows && c >= 0 && c < ncols)
      prim::hist_add(h, out, (unsigned long long)(c - r + nrows - 1));
  }
  __syncthreads();
  prim::hist_flush(h, out);
}

__global__ void count_above(const int32_t* __restrict__ v, int64_t n, int32_t thr, unsigned long long* cnt) {
  unsigned long long a = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = v[i];
    a += (e > thr && e != 0) ? 1ull : 0ull;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0 && a) atomicAdd(cnt, a);
}

int zero_if(int32_t* out, int64_t n, int init, cudaStream_t s) {
  if (init && n > 0) MGB_CUDA_CHECK(cudaMemsetAsync(out, 0, sizeof(int32_t) * (size_t)n, s));
  return MGB_SUCCESS;
}

// DIA per row: in-range diagonal slots (thread per row; the offsets are read
// by every thread of a warp at once, one broadcast each)
__global__ void dia_row_counts(const int32_t* __restrict__ off, int64_t nd, int64_t nrows, int64_t ncols,
                               int32_t* __restrict__ out, int init) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = init ? 0 : out[r];
    for (int64_t n = 0; n < nd; n++) {
      const int64_t col = r + __ldg(off + n);
      c += (col >= 0 && col < ncols) ? 1 : 0;
    }
    out[r] = c;
  }
}

// DIA per diagonal: nonzero slots over the whole slab column (pitch rows),
// summed per CTA in shared memory (one global atomic per CTA and diagonal)
constexpr int DIAG_SMEM = 1024;
template <typename T>
__global__ void dia_diag_counts(const int32_t* __restrict__ off, int64_t nd, int64_t pitch, const T* __restrict__ v,
                                int64_t nrows, int64_t nbins, int32_t* __restrict__ out) {
  for (int64_t d0 = (int64_t)blockIdx.y * DIAG_SMEM; d0 < nd; d0 += (int64_t)gridDim.y * DIAG_SMEM) {
    const int64_t dn = nd - d0 < DIAG_SMEM ? nd - d0 : DIAG_SMEM;
    __shared__ int32_t s_cnt[DIAG_SMEM];
    for (int i = threadIdx.x; i < dn; i += blockDim.x) s_cnt[i] = 0;
    __syncthreads();
    for (int64_t n = 0; n < dn; n++) {
      const T* col = v + pitch * (d0 + n);
      int32_t c = 0;
      for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < pitch;
           j += (int64_t)gridDim.x * blockDim.x)
        c += col[j] != T(0) ? 1 : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if ((threadIdx.x & 31) == 0 && c) atomicAdd(s_cnt + n, c);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < dn; i += blockDim.x) {
      const int64_t bin = (int64_t)__ldg(off + d0 + i) + nrows - 1;
      if (s_cnt[i] && bin >= 0 && bin < nbins) atomicAdd(out + bin, s_cnt[i]);
    }
    __syncthreads();
  }
}

// ELL per row: slots with a valid column (column-major slab: coalesced)
__global__ void ell_row_counts(const int32_t* __restrict__ ci, int64_t width, int64_t pitch, int64_t nrows,
                               int32_t* __restrict__ out, int init) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = init ? 0 : out[r];
    for (int64_t n = 0; n < width; n++) c += __ldg(ci + r + pitch * n) != MGB_INVALID_INDEX ? 1 : 0;
    out[r] = c;
  }
}

// ELL per diagonal: k = valid nonzero slots of the row, then the first k
// slots are inspected (the reference's counting and scan, restated)
template <typename T>
__global__ void ell_diag_counts(const int32_t* __restrict__ ci, const T* __restrict__ v, int64_t width,
                                int64_t pitch, int64_t nrows, int64_t ncols, int32_t* __restrict__ out) {
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t k = 0;
    for (int64_t n = 0; n < width; n++) {
      const int32_t c = __ldg(ci + r + pitch * n);
      k += (c != MGB_INVALID_INDEX && __ldg(v + r + pitch * n) != T(0)) ? 1 : 0;
    }
    for (int64_t n = 0; n < k; n++) {
      const int64_t c = __ldg(ci + r + pitch * n);
      if (c != MGB_INVALID_INDEX && __ldg(v + r + pitch * n) != T(0) && c >= 0 && c < ncols)
        prim::hist_add(h, out, (unsigned long long)(c - r + nrows - 1));
    }
  }
  __syncthreads();
  prim::hist_flush(h, out);
}

// ---- per-format launchers (descriptor checks, then the kernels) ----------

int row_counts_csr(const mgb_csr* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr && out != nullptr, MGB_ERR_BAD_ARGUMENT);
  csr_row_counts<<<grid_for(A->nrows), 256, 0, s>>>(A->row_offsets, A->nrows, out, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int row_counts_coo(const mgb_coo* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && (A->nnz == 0 || A->row_indices != nullptr), MGB_ERR_BAD_ARGUMENT);
  if (int st = zero_if(out, A->nrows, init, s)) return st;
  if (A->nnz == 0) return MGB_SUCCESS;
  coo_row_counts<<<grid_for(A->nnz), 256, 0, s>>>(A->row_indices, A->nnz, A->nrows, out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int row_counts_dia(const mgb_dia* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz) && A->ndiags >= 0, MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && (A->ndiags == 0 || A->diagonal_offsets != nullptr), MGB_ERR_BAD_ARGUMENT);
  dia_row_counts<<<grid_for(A->nrows), 256, 0, s>>>(A->diagonal_offsets, A->ndiags, A->nrows, A->ncols, out, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int row_counts_ell(const mgb_ell* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz) && A->width >= 0, MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && A->pitch >= A->nrows && (A->width == 0 || A->column_indices != nullptr),
              MGB_ERR_BAD_ARGUMENT);
  ell_row_counts<<<grid_for(A->nrows), 256, 0, s>>>(A->column_indices, A->width, A->pitch, A->nrows, out, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int diag_counts_csr(const mgb_csr* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0 || A->ncols == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && A->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz == 0 || A->column_indices != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = zero_if(out, A->nrows + A->ncols - 1, init, s)) return st;
  if (A->nnz == 0) return MGB_SUCCESS;
  csr_diag_counts<<<grid_for(A->nrows * 32), 256, 0, s>>>(A->row_offsets, A->column_indices, A->nrows, A->ncols,
                                                          out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int diag_counts_coo(const mgb_coo* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0 || A->ncols == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && (A->nnz == 0 || (A->row_indices && A->column_indices)), MGB_ERR_BAD_ARGUMENT);
  if (int st = zero_if(out, A->nrows + A->ncols - 1, init, s)) return st;
  if (A->nnz == 0) return MGB_SUCCESS;
  coo_diag_counts<<<grid_for(A->nnz), 256, 0, s>>>(A->row_indices, A->column_indices, A->nnz, A->nrows, A->ncols,
                                                   out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int diag_counts_dia(const mgb_dia* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz) && A->ndiags >= 0, MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0 || A->ncols == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && A->pitch >= A->nrows, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->ndiags == 0 || (A->diagonal_offsets && A->values), MGB_ERR_BAD_ARGUMENT);
  const int64_t nbins = A->nrows + A->ncols - 1;
  if (int st = zero_if(out, nbins, init, s)) return st;
  if (A->ndiags == 0) return MGB_SUCCESS;
  int64_t gx = (A->pitch + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 4;
  if (gx > cap) gx = cap;
  int64_t gy = (A->ndiags + DIAG_SMEM - 1) / DIAG_SMEM;
  if (gy > 65535) gy = 65535;
  dia_diag_counts<T><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(
      A->diagonal_offsets, A->ndiags, A->pitch, static_cast<const T*>(A->values), A->nrows, nbins, out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int diag_counts_ell(const mgb_ell* A, int32_t* out, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz) && A->width >= 0, MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0 || A->ncols == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && A->pitch >= A->nrows, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->width == 0 || (A->column_indices && A->values), MGB_ERR_BAD_ARGUMENT);
  if (int st = zero_if(out, A->nrows + A->ncols - 1, init, s)) return st;
  if (A->width == 0) return MGB_SUCCESS;
  ell_diag_counts<T><<<grid_for(A->nrows), 256, 0, s>>>(A->column_indices, static_cast<const T*>(A->values),
                                                        A->width, A->pitch, A->nrows, A->ncols, out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_count_nnz_per_row_csr(const mgb_csr* A, int32_t* out, int init, void* stream) {
  return row_counts_csr(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_row_coo(const mgb_coo* A, int32_t* out, int init, void* stream) {
  return row_counts_coo(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_row_dia(const mgb_dia* A, int32_t* out, int init, void* stream) {
  return row_counts_dia(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_row_ell(const mgb_ell* A, int32_t* out, int init, void* stream) {
  return row_counts_ell(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_row_hyb(const mgb_hyb* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = row_counts_ell(&A->ell, out, init, as_stream(stream))) return st;
  return row_counts_coo(&A->coo, out, 0, as_stream(stream));
}
int mgb_count_nnz_per_row_hdc(const mgb_hdc* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = row_counts_dia(&A->dia, out, init, as_stream(stream))) return st;
  return row_counts_csr(&A->csr, out, 0, as_stream(stream));
}

int mgb_count_nnz_per_diagonal_csr(const mgb_csr* A, int32_t* out, int init, void* stream) {
  return diag_counts_csr(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_coo(const mgb_coo* A, int32_t* out, int init, void* stream) {
  return diag_counts_coo(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_dia_f64(const mgb_dia* A, int32_t* out, int init, void* stream) {
  return diag_counts_dia<double>(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_dia_f32(const mgb_dia* A, int32_t* out, int init, void* stream) {
  return diag_counts_dia<float>(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_ell_f64(const mgb_ell* A, int32_t* out, int init, void* stream) {
  return diag_counts_ell<double>(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_ell_f32(const mgb_ell* A, int32_t* out, int init, void* stream) {
  return diag_counts_ell<float>(A, out, init, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_hyb_f64(const mgb_hyb* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = diag_counts_ell<double>(&A->ell, out, init, as_stream(stream))) return st;
  return diag_counts_coo(&A->coo, out, 0, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_hyb_f32(const mgb_hyb* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = diag_counts_ell<float>(&A->ell, out, init, as_stream(stream))) return st;
  return diag_counts_coo(&A->coo, out, 0, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_hdc_f64(const mgb_hdc* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = diag_counts_dia<double>(&A->dia, out, init, as_stream(stream))) return st;
  return diag_counts_csr(&A->csr, out, 0, as_stream(stream));
}
int mgb_count_nnz_per_diagonal_hdc_f32(const mgb_hdc* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (int st = diag_counts_dia<float>(&A->dia, out, init, as_stream(stream))) return st;
  return diag_counts_csr(&A->csr, out, 0, as_stream(stream));
}

int mgb_count_nnz_vector(const int32_t* v, int64_t n, int32_t threshold, int64_t* count, void* stream) {
  MGB_REQUIRE(count != nullptr && n >= 0 && (n == 0 || v != nullptr), MGB_ERR_BAD_ARGUMENT);
  *count = 0;
  if (n == 0) return MGB_SUCCESS;
  const cudaStream_t s = as_stream(stream);
  prim::Scratch sc(s);
  unsigned long long* d;
  MGB_SCRATCH(sc, d, 1);
  MGB_CUDA_CHECK(cudaMemsetAsync(d, 0, sizeof(unsigned long long), s));
  count_above<<<grid_for(n), 256, 0, s>>>(v, n, threshold, d);
  MGB_LAUNCH_CHECK();
  unsigned long long h = 0;
  MGB_CUDA_CHECK(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));
  *count = (int64_t)h;
  return MGB_SUCCESS;
}

}  // extern "C"
