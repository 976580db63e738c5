// spmv_csr_rows.cu -- CSR SpMV for rows of (nearly) equal, short length, and
// the per-matrix choice between the two CSR kernels.
//
// The reference chooses its scalar (thread-per-row) CSR kernel only when the
// user sets MATOPT_SHORT_ROWS (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:59-92).
// Here the choice is measured: mgb_csr_choose_kernel reads the row lengths
// once and picks
//   MGB_CSR_ROWS     when 32 rows of the longest length fit one staged tile
//                    (longest row <= 28) and the longest row is <= 1.5 x
//                    mean + 2 (stencils, banded matrices, FEM meshes), else
//   MGB_CSR_SPLIT    when some row is longer than 8192 entries or rows
//                    average >= 512 (split nonzero chunks with carries,
//                    spmv_csr.cu), else
//   MGB_CSR_SEGMENTS the lane-segment kernel of spmv_csr.cu (any structure).
//
// Row-tile kernel: one warp owns 32 consecutive rows.  The tile's entries are
// one contiguous range of the CSR arrays; up to ROWS_TILE_MAX of them are
// staged into shared memory with coalesced loads, then every lane walks its
// own row from shared memory in lockstep with the others (equal lengths keep
// every FP64 FMA full-warp), and neighbouring rows read neighbouring x
// entries, so the x loads of a warp are (nearly) coalesced instead of 32
// separate gathers.  Tiles whose range is longer are processed in pieces.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int ROWS_WARPS = 4;
constexpr int ROWS_TILE_MAX = 896;  // 32 rows x 28 entries

// DOT: also x[0..nrows) . y, one partial per warp in
// partials[blockIdx.x * ROWS_WARPS + warp].
template <typename T, bool DOT>
__global__ void __launch_bounds__(ROWS_WARPS * 32, 5)
spmv_csr_rowtile(int64_t nrows, int64_t ncols, const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                 const T* __restrict__ va, const T* __restrict__ x, T* __restrict__ y, int init,
                 T* __restrict__ partials) {
  __shared__ T s_val[ROWS_WARPS][ROWS_TILE_MAX];
  __shared__ int32_t s_col[ROWS_WARPS][ROWS_TILE_MAX];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  T* sv = s_val[w];
  int32_t* sc = s_col[w];
  const int64_t ntiles = (nrows + 31) >> 5;
  T part = T(0);
  for (int64_t tile = (int64_t)blockIdx.x * ROWS_WARPS + w; tile < ntiles;
       tile += (int64_t)gridDim.x * ROWS_WARPS) {
    const int64_t r = (tile << 5) + lane;
    const bool valid = r < nrows;
    const int32_t rs = __ldg(ro + (valid ? r : nrows));
    const int32_t re = valid ? __ldg(ro + r + 1) : rs;
    const int32_t tb = __shfl_sync(0xffffffffu, rs, 0);
    const int32_t te = (int32_t)__reduce_max_sync(0xffffffffu, (unsigned)re);
    T acc = (valid && !init) ? y[r] : T(0);
    for (int32_t c = tb; c < te; c += ROWS_TILE_MAX) {
      const int32_t cend = (te - c < ROWS_TILE_MAX) ? te : c + ROWS_TILE_MAX;
      __syncwarp();
      for (int32_t i = c + lane; i < cend; i += 32) {
        sv[i - c] = ldg_stream(va + i);
        sc[i - c] = ldg_stream(ci + i);
      }
      __syncwarp();
      const int32_t lo = max(rs, c), hi = min(re, cend);
      // lockstep over the longest intersection in the warp
      const int32_t n = (int32_t)__reduce_max_sync(0xffffffffu, (unsigned)max(hi - lo, 0));
#pragma unroll 4
      for (int32_t j = 0; j < n; j++) {
        const int32_t e = lo + j;
        if (e < hi) {
          const int32_t col = sc[e - c];
          const T xv = ((unsigned)col < (uint64_t)ncols) ? __ldg(x + col) : T(0);
          acc = fmadd(sv[e - c], xv, acc);
        }
      }
    }
    if (valid) {
      y[r] = acc;
      if (DOT) part = fmadd(x[r], acc, part);
    }
  }
  if (DOT) {
    part = warp_sum(part);
    if (lane == 0) partials[(int64_t)blockIdx.x * ROWS_WARPS + w] = part;
  }
}

__global__ void row_shape_kernel(const int32_t* __restrict__ ro, int64_t nrows, int* mx) {
  int m = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x)
    m = max(m, ro[r + 1] - ro[r]);
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

template <typename T>
int launch_rows(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, int64_t* npartials) {
  const int64_t ntiles = (A->nrows + 31) / 32;
  int64_t blocks = (ntiles + ROWS_WARPS - 1) / ROWS_WARPS;
  if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
  if (npartials) *npartials = blocks * ROWS_WARPS;
  if (npartials && !partials) return MGB_SUCCESS;
  if (partials)
    spmv_csr_rowtile<T, true><<<(unsigned)blocks, ROWS_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->row_offsets, A->column_indices, static_cast<const T*>(A->values), x, y, init,
        partials);
  else
    spmv_csr_rowtile<T, false><<<(unsigned)blocks, ROWS_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->row_offsets, A->column_indices, static_cast<const T*>(A->values), x, y, init,
        nullptr);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int choose(const mgb_csr* A, int* variant, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && variant != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  *variant = MGB_CSR_SEGMENTS;
  if (A->nrows == 0 || A->nnz == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  int* d = nullptr;
  MGB_CUDA_CHECK(cudaMallocAsync((void**)&d, sizeof(int), s));
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(int), s);
  if (e == cudaSuccess) {
    int64_t blocks = (A->nrows + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (blocks > cap) blocks = cap;
    row_shape_kernel<<<(unsigned)blocks, 256, 0, s>>>(A->row_offsets, A->nrows, d);
    e = cudaGetLastError();
  }
  int mx = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&mx, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(d, s);
  if (e != cudaSuccess) return record_cuda_error(e);
  const double mean = (double)A->nnz / (double)A->nrows;
  if (32 * mx <= ROWS_TILE_MAX && (double)mx <= 1.5 * mean + 2.0) *variant = MGB_CSR_ROWS;
  // rows longer than a few chunks: one warp per row would be the critical
  // path (measured: a 150,000-entry row 746 -> 56 us; rows of 1,000-6,000
  // entries 66 -> 46 us; the power-law matrix, mean 15, stays faster whole)
  if (mx > 8192 || mean >= 512.0) *variant = MGB_CSR_SPLIT;
  return MGB_SUCCESS;
}

}  // namespace

// CSR SpMV entry with an explicit kernel choice (used by spmv_csr.cu too)
template <typename T>
int launch_csr_rows(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, int64_t* npartials) {
  return launch_rows<T>(A, x, y, init, s, partials, npartials);
}
template int launch_csr_rows<double>(const mgb_csr*, const double*, double*, int, cudaStream_t, double*, int64_t*);
template int launch_csr_rows<float>(const mgb_csr*, const float*, float*, int, cudaStream_t, float*, int64_t*);

}  // namespace mgb

extern "C" int mgb_csr_choose_kernel(const mgb_csr* A, int* variant, void* stream) {
  return mgb::choose(A, variant, mgb::as_stream(stream));
}
