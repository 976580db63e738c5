// spmv_coo.cu -- COO SpMV for sm_103a (segmented reduction over row-sorted keys).
//
// Replaces the reference's CUDA COO path (impl/Coo/Cuda/Morpheus_Multiply_Impl.hpp:50-176:
// flat kernel impl/Coo/Kernels/Morpheus_Multiply_Impl.hpp:121-208, carry pass
// impl/DenseVector/Kernels/Morpheus_Segmented_Reduction_Impl.hpp:40-162 and a
// serial <<<1,1>>> tail).  Like that path the matrix must be sorted by row;
// columns may be in any order and duplicates are allowed.  Semantics are the
// Serial multiply (impl/Coo/Serial/Morpheus_Multiply_Impl.hpp:38-59):
// y = 0 if init, then y[I[n]] += V[n] * x[J[n]].
//
// Design: one warp per chunk of COO_CH consecutive entries, staged through
// shared memory with coalesced loads.  Row runs inside the chunk are found
// with a ballot; each lane sums whole runs with one FMA per entry (runs longer
// than COO_LONG are summed by the whole warp).  Interior runs are complete
// rows and are stored directly.  The first and last run of every chunk may
// continue in a neighbouring chunk, so they are written as carries and a
// second, tiny kernel adds the carries of each row in chunk order:
// deterministic, no atomics.  With init, rows without entries are zero-filled
// by the chunk that sees the gap, so y is written exactly once and never read.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int COO_WARPS = 8;
constexpr int COO_CH = 256;
constexpr int COO_LONG = 64;

template <typename T>
__device__ __forceinline__ T gather_x(const T* __restrict__ x, int32_t c, int64_t ncols) {
  return ((uint64_t)(int64_t)c < (uint64_t)ncols) ? __ldg(x + c) : T(0);
}

// zero-fill rows (a, b) exclusive on both ends, cooperatively by the warp
__device__ __forceinline__ void zero_gap_warp(int64_t a, int64_t b, int lane, double* y) {
  for (int64_t r = a + 1 + lane; r < b; r += 32) y[r] = 0.0;
}
__device__ __forceinline__ void zero_gap_warp(int64_t a, int64_t b, int lane, float* y) {
  for (int64_t r = a + 1 + lane; r < b; r += 32) y[r] = 0.0f;
}

template <typename T>
__global__ void __launch_bounds__(COO_WARPS * 32, 4)
spmv_coo_chunks(int64_t nrows, int64_t ncols, int64_t nnz,
                const int32_t* __restrict__ ri, const int32_t* __restrict__ ci,
                const T* __restrict__ va, const T* __restrict__ x,
                T* __restrict__ y, int init, int32_t* __restrict__ carry_row,
                T* __restrict__ carry_val) {
  __shared__ int32_t s_row[COO_WARPS][COO_CH];
  __shared__ int32_t s_col[COO_WARPS][COO_CH];
  __shared__ T s_val[COO_WARPS][COO_CH];
  __shared__ int16_t s_start[COO_WARPS][COO_CH + 1];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  int32_t* sr = s_row[w];
  int32_t* sc = s_col[w];
  T* sv = s_val[w];
  int16_t* ss = s_start[w];
  const unsigned lt_mask = (1u << lane) - 1u;

  const int64_t nchunks = (nnz + COO_CH - 1) / COO_CH;
  for (int64_t k = (int64_t)blockIdx.x * COO_WARPS + w; k < nchunks;
       k += (int64_t)gridDim.x * COO_WARPS) {
    const int64_t base = k * COO_CH;
    const int cnt = (int)min((int64_t)COO_CH, nnz - base);
    const int64_t prev_row = base > 0 ? (int64_t)ri[base - 1] : -1;
#pragma unroll
    for (int j = 0; j < COO_CH / 32; j++) {
      const int idx = j * 32 + lane;
      if (idx < cnt) {
        sr[idx] = ldg_stream(ri + base + idx);
        sc[idx] = ldg_stream(ci + base + idx);
        sv[idx] = ldg_stream(va + base + idx);
      }
    }
    __syncwarp();
    // run starts
    int nruns = 0;
#pragma unroll
    for (int g = 0; g < COO_CH / 32; g++) {
      const int idx = g * 32 + lane;
      const bool flag = idx < cnt && (idx == 0 || sr[idx] != sr[idx - 1]);
      const unsigned bal = __ballot_sync(0xffffffffu, flag);
      if (flag) ss[nruns + __popc(bal & lt_mask)] = (int16_t)idx;
      nruns += __popc(bal);
    }
    if (lane == 0) ss[nruns] = (int16_t)cnt;
    __syncwarp();

    const bool last_chunk = (k == nchunks - 1);
    // short runs: one lane per run
    for (int j = lane; j < nruns; j += 32) {
      const int a = ss[j], b = ss[j + 1];
      const int64_t row = sr[a];
      if (init) {
        const int64_t before = (j == 0) ? prev_row : (int64_t)sr[ss[j - 1]];
        if (row - before > 1 && row - before <= 33)
          for (int64_t r = before + 1; r < row; r++)
            if (r >= 0 && r < nrows) y[r] = T(0);
        if (last_chunk && j == nruns - 1 && nrows - row > 1 && nrows - row <= 33)
          for (int64_t r = row + 1; r < nrows; r++) y[r] = T(0);
      }
      if (b - a > COO_LONG) continue;
      T s = T(0);
      for (int e = a; e < b; e++) s = fmadd(sv[e], gather_x(x, sc[e], ncols), s);
      if (j == 0) {
        carry_row[2 * k] = (int32_t)row;
        carry_val[2 * k] = s;
        if (nruns == 1) { carry_row[2 * k + 1] = (int32_t)row; carry_val[2 * k + 1] = T(0); }
      } else if (j == nruns - 1) {
        carry_row[2 * k + 1] = (int32_t)row;
        carry_val[2 * k + 1] = s;
      } else if (row >= 0 && row < nrows) {
        y[row] = init ? s : y[row] + s;
      }
    }
    // long gaps (init only): whole warp fills
    if (init) {
      for (int j0 = 0; j0 < nruns; j0 += 32) {
        const int j = j0 + lane;
        bool big = false;
        int64_t lo_gap = 0, hi_gap = 0;
        if (j < nruns) {
          const int64_t row = sr[ss[j]];
          const int64_t before = (j == 0) ? prev_row : (int64_t)sr[ss[j - 1]];
          if (row - before > 33) { big = true; lo_gap = max(before, (int64_t)-1); hi_gap = min(row, nrows); }
        }
        unsigned m = __ballot_sync(0xffffffffu, big);
        while (m) {
          const int l = __ffs(m) - 1;
          m &= m - 1;
          zero_gap_warp(__shfl_sync(0xffffffffu, lo_gap, l), __shfl_sync(0xffffffffu, hi_gap, l), lane, y);
        }
      }
      if (last_chunk) {
        const int64_t row = sr[ss[nruns - 1]];
        if (nrows - row > 33) zero_gap_warp(max(row, (int64_t)-1), nrows, lane, y);
      }
    }
    // long runs: whole warp per run
    for (int j0 = 0; j0 < nruns; j0 += 32) {
      const int jj = j0 + lane;
      const bool lng = jj < nruns && (ss[jj + 1] - ss[jj]) > COO_LONG;
      unsigned m = __ballot_sync(0xffffffffu, lng);
      while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const int j = j0 + l;
        const int a = ss[j], b = ss[j + 1];
        T s = T(0);
        for (int e = a + lane; e < b; e += 32) s = fmadd(sv[e], gather_x(x, sc[e], ncols), s);
        s = warp_sum(s);
        if (lane == 0) {
          const int64_t row = sr[a];
          if (j == 0) {
            carry_row[2 * k] = (int32_t)row;
            carry_val[2 * k] = s;
            if (nruns == 1) { carry_row[2 * k + 1] = (int32_t)row; carry_val[2 * k + 1] = T(0); }
          } else if (j == nruns - 1) {
            carry_row[2 * k + 1] = (int32_t)row;
            carry_val[2 * k + 1] = s;
          } else if (row >= 0 && row < nrows) {
            y[row] = init ? s : y[row] + s;
          }
        }
      }
    }
    __syncwarp();
  }
}

// Adds the carries of each row in chunk order.  carry_row is non-decreasing.
template <typename T>
__global__ void coo_carry_fixup(int64_t ncarry, int64_t nrows,
                                const int32_t* __restrict__ cr,
                                const T* __restrict__ cv, T* __restrict__ y,
                                int init) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncarry) return;
  const int32_t r = cr[i];
  if (i > 0 && cr[i - 1] == r) return;
  T s = T(0);
  for (int64_t j = i; j < ncarry && cr[j] == r; j++) s += cv[j];
  if (r >= 0 && r < nrows) y[r] = init ? s : y[r] + s;
}

}  // namespace

template <typename T>
int launch_coo(const mgb_coo* A, const T* x, T* y, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nrows < ((int64_t)1 << 31), MGB_ERR_INVALID_INPUT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(y != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (A->nnz == 0) {
    if (init) MGB_CUDA_CHECK(cudaMemsetAsync(y, 0, sizeof(T) * A->nrows, s));
    return MGB_SUCCESS;
  }
  MGB_REQUIRE(A->row_indices && A->column_indices && A->values && x, MGB_ERR_BAD_ARGUMENT);
  const int64_t nchunks = (A->nnz + COO_CH - 1) / COO_CH;
  const int64_t ncarry = 2 * nchunks;
  void* scratch = nullptr;
  const size_t rows_bytes = ((sizeof(int32_t) * ncarry + 255) / 256) * 256;
  MGB_CUDA_CHECK(cudaMallocAsync(&scratch, rows_bytes + sizeof(T) * ncarry, s));
  int32_t* cr = static_cast<int32_t*>(scratch);
  T* cv = reinterpret_cast<T*>(static_cast<char*>(scratch) + rows_bytes);
  const int64_t blocks = (nchunks + COO_WARPS - 1) / COO_WARPS;
  spmv_coo_chunks<T><<<(unsigned)blocks, COO_WARPS * 32, 0, s>>>(
      A->nrows, A->ncols, A->nnz, A->row_indices, A->column_indices,
      static_cast<const T*>(A->values), x, y, init, cr, cv);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    coo_carry_fixup<T><<<(unsigned)((ncarry + 255) / 256), 256, 0, s>>>(ncarry, A->nrows, cr, cv, y, init);
    e = cudaGetLastError();
  }
  cudaError_t ef = cudaFreeAsync(scratch, s);
  if (e != cudaSuccess) return record_cuda_error(e);
  if (ef != cudaSuccess) return record_cuda_error(ef);
  return MGB_SUCCESS;
}

template int launch_coo<double>(const mgb_coo*, const double*, double*, int, cudaStream_t);
template int launch_coo<float>(const mgb_coo*, const float*, float*, int, cudaStream_t);

}  // namespace mgb

extern "C" {

int mgb_spmv_coo_f64(const mgb_coo* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_coo<double>(A, x, y, init, mgb::as_stream(stream));
}

int mgb_spmv_coo_f32(const mgb_coo* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_coo<float>(A, x, y, init, mgb::as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free COO SpMV.
//
// For callers that cannot allocate device memory while they run: code inside
// a CUDA-graph-captured region of a host application that forbids
// allocations, real-time or embedded hosts that reserve all memory up front,
// and plugins whose host process owns the allocator.  mgb_spmv_coo_f64 takes
// its carry buffer from cudaMallocAsync; this variant takes it from a fixed
// file-scope device array instead, so it never calls cudaMalloc, cudaFree or
// any allocating routine.
//
// Limits and rules:
//  * The array is COO_NOALLOC_BYTES (4 MiB) of device memory that every GPU
//    which loads this library holds until the process exits.  It holds two
//    carries (int32 row + double value) per 256-entry chunk, so A->nnz may be
//    at most 44,736,512; larger matrices get MGB_ERR_INVALID_INPUT before any
//    work is queued.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current) and
//    caches it; make that first call before any stream capture.
//  * Every call uses the same array and leaves the previous call's carries
//    in it.  Nothing in it needs to start at zero: each call writes every
//    carry slot it reads.  Calls that overlap on the GPU (other streams, other
//    host threads) race on the array; serialise them.
// ---------------------------------------------------------------------------
#include <mutex>

namespace mgb {
namespace {
constexpr size_t COO_NOALLOC_BYTES = size_t(4) << 20;
}  // namespace
}  // namespace mgb

static __device__ __align__(256) unsigned char g_coo_noalloc_scratch[mgb::COO_NOALLOC_BYTES];

namespace mgb {
namespace {

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[128] = {};

// Device address of the scratch array for the current device (set-up on the
// first call per device).
int noalloc_scratch(void** out) {
  int dev = 0;
  MGB_CUDA_CHECK(cudaGetDevice(&dev));
  MGB_REQUIRE(dev >= 0 && dev < 128, MGB_ERR_RUNTIME);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_coo_noalloc_scratch);
    if (e != cudaSuccess) return record_cuda_error(e);
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return MGB_SUCCESS;
}

int launch_coo_noalloc_f64(const mgb_coo* A, const double* x, double* y, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  const int64_t nchunks = (A->nnz + COO_CH - 1) / COO_CH;
  const int64_t ncarry = 2 * nchunks;
  const size_t rows_bytes = ((sizeof(int32_t) * (size_t)ncarry + 255) / 256) * 256;
  MGB_REQUIRE(rows_bytes + sizeof(double) * (size_t)ncarry <= COO_NOALLOC_BYTES, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(A->nrows < ((int64_t)1 << 31), MGB_ERR_INVALID_INPUT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(y != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (A->nnz == 0) {
    if (init) MGB_CUDA_CHECK(cudaMemsetAsync(y, 0, sizeof(double) * A->nrows, s));
    return MGB_SUCCESS;
  }
  MGB_REQUIRE(A->row_indices && A->column_indices && A->values && x, MGB_ERR_BAD_ARGUMENT);
  void* scratch = nullptr;
  int st = noalloc_scratch(&scratch);
  if (st != MGB_SUCCESS) return st;
  int32_t* cr = static_cast<int32_t*>(scratch);
  double* cv = reinterpret_cast<double*>(static_cast<char*>(scratch) + rows_bytes);
  const int64_t blocks = (nchunks + COO_WARPS - 1) / COO_WARPS;
  spmv_coo_chunks<double><<<(unsigned)blocks, COO_WARPS * 32, 0, s>>>(
      A->nrows, A->ncols, A->nnz, A->row_indices, A->column_indices,
      static_cast<const double*>(A->values), x, y, init, cr, cv);
  MGB_LAUNCH_CHECK();
  coo_carry_fixup<double><<<(unsigned)((ncarry + 255) / 256), 256, 0, s>>>(ncarry, A->nrows, cr, cv, y, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" int mgb_spmv_coo_f64_noalloc(const mgb_coo* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_coo_noalloc_f64(A, x, y, init, mgb::as_stream(stream));
}
