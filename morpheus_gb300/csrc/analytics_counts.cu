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
    if (r >= 0 && r < nrows) atomicAdd(out + r, 1);
  }
}

__global__ void csr_diag_counts(const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, int64_t nrows,
                                int64_t ncols, int32_t* out) {
  // one warp per row: coalesced column reads for long rows
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrows; r += warps) {
    for (int32_t j = ro[r] + lane; j < ro[r + 1]; j += 32) {
      const int64_t c = ci[j];
      if (c >= 0 && c < ncols) atomicAdd(out + (c - r + nrows - 1), 1);
    }
  }
}

__global__ void coo_diag_counts(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci, int64_t nnz,
                                int64_t nrows, int64_t ncols, int32_t* out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = ri[k], c = ci[k];
    if (r >= 0 && r < nrows && c >= 0 && c < ncols) atomicAdd(out + (c - r + nrows - 1), 1);
  }
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

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_count_nnz_per_row_csr(const mgb_csr* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr && out != nullptr, MGB_ERR_BAD_ARGUMENT);
  csr_row_counts<<<grid_for(A->nrows), 256, 0, as_stream(stream)>>>(A->row_offsets, A->nrows, out, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int mgb_count_nnz_per_row_coo(const mgb_coo* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && (A->nnz == 0 || A->row_indices != nullptr), MGB_ERR_BAD_ARGUMENT);
  const cudaStream_t s = as_stream(stream);
  if (int st = zero_if(out, A->nrows, init, s)) return st;
  if (A->nnz == 0) return MGB_SUCCESS;
  coo_row_counts<<<grid_for(A->nnz), 256, 0, s>>>(A->row_indices, A->nnz, A->nrows, out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int mgb_count_nnz_per_diagonal_csr(const mgb_csr* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0 || A->ncols == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && A->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz == 0 || A->column_indices != nullptr, MGB_ERR_BAD_ARGUMENT);
  const cudaStream_t s = as_stream(stream);
  if (int st = zero_if(out, A->nrows + A->ncols - 1, init, s)) return st;
  if (A->nnz == 0) return MGB_SUCCESS;
  csr_diag_counts<<<grid_for(A->nrows * 32), 256, 0, s>>>(A->row_offsets, A->column_indices, A->nrows, A->ncols,
                                                          out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int mgb_count_nnz_per_diagonal_coo(const mgb_coo* A, int32_t* out, int init, void* stream) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0 || A->ncols == 0) return MGB_SUCCESS;
  MGB_REQUIRE(out != nullptr && (A->nnz == 0 || (A->row_indices && A->column_indices)), MGB_ERR_BAD_ARGUMENT);
  const cudaStream_t s = as_stream(stream);
  if (int st = zero_if(out, A->nrows + A->ncols - 1, init, s)) return st;
  if (A->nnz == 0) return MGB_SUCCESS;
  coo_diag_counts<<<grid_for(A->nnz), 256, 0, s>>>(A->row_indices, A->column_indices, A->nnz, A->nrows, A->ncols,
                                                   out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
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
