// spmv_csr.cu -- CSR SpMV for sm_103a.
//
// Replaces the reference's CUDA CSR path (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:50-157,
// kernels impl/Csr/Kernels/Morpheus_Multiply_Impl.hpp:36-168), which picks one
// threads-per-row value from the global mean row length and reduces through
// volatile shared memory.  Semantics follow the Serial multiply
// (impl/Csr/Serial/Morpheus_Multiply_Impl.hpp:38-58): per row,
// sum = init ? 0 : y[i]; sum += A(i,j) * x[j] over the row; y[i] = sum.
//
// GB300 constraint that shapes this kernel: the FP64 pipe retires about one
// warp-wide DFMA per 16 SM cycles and charges that slot whether 1 or 32 lanes
// are active.  A kernel whose lanes walk rows of different lengths, or that
// reduces every row with a shuffle tree, spends most FP64 slots on idle lanes.
// So the work is split by NONZEROS, not rows:
//
//  * Warp chunks.  Warp w takes the rows whose first entry lies in the nominal
//    range [w*CHUNK, (w+1)*CHUNK) (two 32-ary searches over row_offsets, or
//    two entries of a chunk plan made once per matrix structure;
//    CHUNK = 2048, smaller for matrices too small to fill the GPU), so
//    every chunk is a whole number of rows and no row crosses warps: no
//    atomics, no scratch, deterministic.  The plan removes the searches'
//    ~10 dependent loads per warp (measured on GB300: 5 % on a 2e6-row
//    power-law matrix, 17 % on a 65,536-row Laplacian), with the same y.
//  * Lane segments.  The chunk's nonzeros [E0, E1) are cut into 32 contiguous
//    lane ranges of KW entries.  Lane l walks its range accumulating with one
//    FMA per entry into the current row and flushing at row ends; every FMA
//    instruction is issued by all 32 lanes together.
//  * Staging.  Each step the warp loads 8 entries of every lane range
//    (4 x 64-byte pieces per load instruction) into padded shared memory, so
//    HBM reads stay sector-complete and shared-memory reads conflict-free.
//    Row offsets of the chunk are staged too, so row-end tests never wait on
//    global memory.
//  * Rows crossing lanes.  A row that continues into the next lane leaves a
//    tail partial; one 5-step segmented shuffle scan per chunk (keyed by row)
//    forwards the partials, and the lane where the row ends adds them: 6
//    extra FP64 warp instructions per ~2048 nonzeros.
// With init == 0 a row's accumulator starts from y[i] (a load, no extra add).
#include <type_traits>

#include "csr_chunk.cuh"
#include "primitives.cuh"

namespace mgb {
namespace {

constexpr int CSR_WARPS = 8;  // warps per CTA

// DOT: also x[0..nrows) . y of the finished rows, one partial per CTA in
// partials[blockIdx.x] (the fused step of an iterative solver; the matrix is
// square there; the launcher caps the grid at the resident CTAs).  With a chunk plan the warps read
// their rows from it instead of searching the row offsets.  SMALL: 32-bit
// indices in the chunk routine, 256 staged row offsets and 4 CTAs per SM
// (64 registers) -- measured on GB300 faster for FP32 (power-law 183 ->
// 164 us) and slower for FP64 (195 -> 206 us), so FP32 only.
template <typename T, bool DOT, bool SMALL = false>
__global__ void __launch_bounds__(CSR_WARPS * 32, SMALL ? 4 : 3)
spmv_csr_segments(int64_t nrows, int64_t ncols, int64_t nnz, int64_t nchunks, int64_t chunk,
                  const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                  const T* __restrict__ va, const T* __restrict__ x,
                  T* __restrict__ y, int init, T* __restrict__ partials, const int32_t* __restrict__ plan) {
  constexpr int RO = SMALL ? 256 : csr::CSR_RO_STAGE;
  using IDX = typename std::conditional<SMALL, int32_t, int64_t>::type;
  __shared__ csr::WarpStage<T, csr::CSR_SEG, RO> stage[CSR_WARPS];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  T part = T(0);
  for (int64_t wc = (int64_t)blockIdx.x * CSR_WARPS + w; wc < nchunks;
       wc += (int64_t)gridDim.x * CSR_WARPS) {
    const csr::RowRange rows = plan ? csr::planned_rows(wc, nrows, plan) : csr::chunk_rows(wc, chunk, nrows, ro, lane);
    const csr::RowRange rr = csr::csr_rows_x<T, csr::CSR_SEG, csr::XGlobal<T>, true, IDX>(
        rows, nrows, ncols, ro, ci, va, csr::XGlobal<T>{x}, y, init, stage[w], lane);
    if (DOT) {
      __syncwarp();  // the chunk's y entries, written by any lane, are visible to the warp
      for (int64_t r = rr.begin + lane; r < rr.end; r += 32) part = fmadd(x[r], y[r], part);
    }
  }
  if (DOT) {
    __shared__ T s_part[CSR_WARPS];
    part = warp_sum(part);
    if (lane == 0) s_part[w] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      T t = T(0);
#pragma unroll
      for (int i = 0; i < CSR_WARPS; i++) t += s_part[i];
      partials[blockIdx.x] = t;
    }
  }
}

// Chunk plan: plan[k] = first row r with ro[r] >= k*chunk, nrows if none
// (k = 0..nchunks).  One thread per row r in [0, nrows] writes the keys in
// (ro[r-1], ro[r]]; row nrows also writes every key past nnz.  For valid
// offsets every entry is written exactly once.
__global__ void csr_chunk_plan(int64_t nrows, int64_t nchunks, int64_t chunk, const int32_t* __restrict__ ro,
                               int32_t* __restrict__ plan) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k_lo = r == 0 ? 0 : (int64_t)__ldg(ro + r - 1) / chunk + 1;
    int64_t k_hi = r == nrows ? nchunks : (int64_t)__ldg(ro + r) / chunk;
    if (k_hi > nchunks) k_hi = nchunks;
    for (int64_t k = k_lo < 0 ? 0 : k_lo; k <= k_hi; k++) plan[k] = (int32_t)r;
  }
}

// Split variant: fixed nonzero chunks (rows of any length spread over
// warps), carries for the rows crossing chunk ends, fixed-order fix-up.
template <typename T>
__global__ void __launch_bounds__(CSR_WARPS * 32, 3)
spmv_csr_split(int64_t nrows, int64_t ncols, int64_t nnz, int64_t nchunks, int64_t chunk,
               const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, const T* __restrict__ va,
               const T* __restrict__ x, T* __restrict__ y, int init, int32_t* __restrict__ carry_row,
               T* __restrict__ carry_val) {
  __shared__ csr::WarpStage<T, csr::CSR_SEG> stage[CSR_WARPS];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  for (int64_t k = (int64_t)blockIdx.x * CSR_WARPS + w; k < nchunks; k += (int64_t)gridDim.x * CSR_WARPS)
    csr::csr_split_chunk<T, csr::CSR_SEG>(k, chunk, nchunks, nrows, ncols, nnz, ro, ci, va, x, y, init, carry_row,
                                          carry_val, stage[w], lane);
}

// y[r] = (init ? 0 : y[r]) + the carries of row r, added in chunk order; a
// row's carries are consecutive (rows < 0 mark empty slots)
template <typename T>
__global__ void split_carry_fixup(int64_t ncarry, int64_t nrows, const int32_t* __restrict__ cr,
                                  const T* __restrict__ cv, T* __restrict__ y, int init) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncarry) return;
  const int32_t r = cr[i];
  if (r < 0 || r >= nrows || (i > 0 && cr[i - 1] == r)) return;
  T s = init ? T(0) : y[r];
  for (int64_t j = i; j < ncarry && cr[j] == r; j++) s += cv[j];
  y[r] = s;
}

// x[0..n) . y[0..n) into per-block partials (the split variant's fused dot,
// after its fix-up)
template <typename T>
__global__ void __launch_bounds__(256) rows_dot_partials(const T* __restrict__ x, const T* __restrict__ y, int64_t n,
                                                         T* __restrict__ partials) {
  __shared__ T s[8];
  T a = T(0);
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
    a = fmadd(x[i], y[i], a);
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x < 32) {
    T t = threadIdx.x < 8 ? s[threadIdx.x] : T(0);
    t = warp_sum(t);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
  }
}

template <typename T>
int launch_split(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, int64_t* npartials) {
  const int64_t dot_blocks = (int64_t)num_sms() * 4;
  if (npartials) *npartials = dot_blocks;
  if (npartials && !partials) return take_device_query_error();
  if (A->nnz == 0) {
    if (init) MGB_CUDA_CHECK(cudaMemsetAsync(y, 0, sizeof(T) * A->nrows, s));
  } else {
    const int64_t chunk = csr::CSR_CHUNK;
    const int64_t nchunks = (A->nnz + chunk - 1) / chunk;
    const int64_t ncarry = 2 * nchunks;
    void* scratch = nullptr;
    const size_t rows_bytes = ((sizeof(int32_t) * (size_t)ncarry + 255) / 256) * 256;
    MGB_CUDA_CHECK(cudaMallocAsync(&scratch, rows_bytes + sizeof(T) * (size_t)ncarry, s));
    int32_t* cr = static_cast<int32_t*>(scratch);
    T* cv = reinterpret_cast<T*>(static_cast<char*>(scratch) + rows_bytes);
    int64_t blocks = (nchunks + CSR_WARPS - 1) / CSR_WARPS;
    if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
    spmv_csr_split<T><<<(unsigned)blocks, CSR_WARPS * 32, 0, s>>>(A->nrows, A->ncols, A->nnz, nchunks, chunk,
                                                                  A->row_offsets, A->column_indices,
                                                                  static_cast<const T*>(A->values), x, y, init, cr,
                                                                  cv);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
      split_carry_fixup<T><<<(unsigned)((ncarry + 255) / 256), 256, 0, s>>>(ncarry, A->nrows, cr, cv, y, init);
      e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(scratch, s);
    if (e != cudaSuccess) return record_cuda_error(e);
    if (ef != cudaSuccess) return record_cuda_error(ef);
  }
  if (partials) {
    rows_dot_partials<T><<<(unsigned)dot_blocks, 256, 0, s>>>(x, y, A->nrows, partials);
    MGB_LAUNCH_CHECK();
  }
  return MGB_SUCCESS;
}

template <typename T>
int launch_csr(const mgb_csr* A, const T* x, T* y, int init, void* stream, int variant = MGB_CSR_SEGMENTS) {
  return launch_csr_dot<T>(A, x, y, init, stream, variant, nullptr, nullptr);
}

}  // namespace

// Chunk size of the lane-segment kernel: 2048 nonzeros, halved (down to
// 256) while the matrix would give fewer chunks than the GPU holds resident
// warps and a chunk still spans at least 8 mean rows, so that small matrices
// spread over every SM (chunks hold whole rows, so splitting matrices of long
// rows finer only adds empty chunks).  The kernel runs nnz / chunk + 1
// chunks, so rows whose first entry is at nnz (trailing empty rows) always
// belong to some chunk.
int64_t segments_chunk(const mgb_csr* A) {
  int64_t chunk = csr::CSR_CHUNK;
  const int64_t resident = (int64_t)num_sms() * CSR_WARPS * 3;
  const int64_t mean_row = A->nnz / (A->nrows > 0 ? A->nrows : 1);
  while (chunk > 256 && A->nnz / chunk < resident && chunk / 2 >= 8 * mean_row) chunk >>= 1;
  return chunk;
}

int make_plan(const mgb_csr* A, int32_t* plan, int64_t entries, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && plan != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz < ((int64_t)1 << 31) - 4096, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(A->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  const int64_t chunk = segments_chunk(A);
  const int64_t nchunks = A->nnz / chunk + 1;
  MGB_REQUIRE(entries == nchunks + 1, MGB_ERR_BAD_ARGUMENT);
  csr_chunk_plan<<<prim::blocks_for(A->nrows + 1, 256), 256, 0, s>>>(A->nrows, nchunks, chunk, A->row_offsets,
                                                                      plan);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int launch_csr_dot(const mgb_csr* A, const T* x, T* y, int init, void* stream, int variant, T* partials,
                   int64_t* npartials, const int32_t* plan, int64_t plan_entries) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz < ((int64_t)1 << 31) - 4096, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(valid_csr_variant(variant),
              MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr && y != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz == 0 || (A->column_indices && A->values && x), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(plan == nullptr || variant == MGB_CSR_SEGMENTS, MGB_ERR_BAD_ARGUMENT);
  if (variant == MGB_CSR_ROWS || variant == MGB_CSR_ROWS_GATHER)
    return launch_csr_rows<T>(A, x, y, init, as_stream(stream), partials, npartials, variant == MGB_CSR_ROWS_GATHER);
  if (variant == MGB_CSR_SPLIT) return launch_split<T>(A, x, y, init, as_stream(stream), partials, npartials);
  const int64_t chunk = segments_chunk(A);
  const int64_t nchunks = A->nnz / chunk + 1;
  MGB_REQUIRE(plan == nullptr || plan_entries == nchunks + 1, MGB_ERR_BAD_ARGUMENT);
  int64_t blocks = (nchunks + CSR_WARPS - 1) / CSR_WARPS;
  if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
  const bool small = sizeof(T) == 4 && A->nrows < 0x7fffff00LL;
  if (npartials || partials) {  // the fused dot: one partial per CTA, grid capped at the resident CTAs
    const int64_t resident = (int64_t)num_sms() * (small ? 4 : 3);
    if (blocks > resident) blocks = resident;
    if (npartials) *npartials = blocks;
  }
  if (npartials && !partials) return take_device_query_error();
  const T* va = static_cast<const T*>(A->values);
  const cudaStream_t s = as_stream(stream);
  if (small && partials)
    spmv_csr_segments<T, true, true><<<(unsigned)blocks, CSR_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->nnz, nchunks, chunk, A->row_offsets, A->column_indices, va, x, y, init, partials,
        plan);
  else if (small)
    spmv_csr_segments<T, false, true><<<(unsigned)blocks, CSR_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->nnz, nchunks, chunk, A->row_offsets, A->column_indices, va, x, y, init, nullptr,
        plan);
  else if (partials)
    spmv_csr_segments<T, true><<<(unsigned)blocks, CSR_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->nnz, nchunks, chunk, A->row_offsets, A->column_indices, va, x, y, init, partials,
        plan);
  else
    spmv_csr_segments<T, false><<<(unsigned)blocks, CSR_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->nnz, nchunks, chunk, A->row_offsets, A->column_indices, va, x, y, init, nullptr,
        plan);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}
template int launch_csr_dot<double>(const mgb_csr*, const double*, double*, int, void*, int, double*, int64_t*,
                                    const int32_t*, int64_t);
template int launch_csr_dot<float>(const mgb_csr*, const float*, float*, int, void*, int, float*, int64_t*,
                                   const int32_t*, int64_t);

}  // namespace mgb

extern "C" {

int mgb_spmv_csr_f64(const mgb_csr* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_csr<double>(A, x, y, init, stream);
}

int mgb_spmv_csr_f32(const mgb_csr* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_csr<float>(A, x, y, init, stream);
}

int mgb_spmv_csr_variant_f64(const mgb_csr* A, const double* x, double* y, int init, int variant, void* stream) {
  return mgb::launch_csr<double>(A, x, y, init, stream, variant);
}

int mgb_spmv_csr_variant_f32(const mgb_csr* A, const float* x, float* y, int init, int variant, void* stream) {
  return mgb::launch_csr<float>(A, x, y, init, stream, variant);
}

int mgb_csr_plan_entries(const mgb_csr* A, int64_t* entries) {
  if (A == nullptr || entries == nullptr || mgb::bad_sizes(A->nrows, A->ncols, A->nnz)) return MGB_ERR_BAD_ARGUMENT;
  *entries = A->nnz / mgb::segments_chunk(A) + 2;
  return mgb::take_device_query_error();
}

int mgb_csr_plan(const mgb_csr* A, int32_t* plan, int64_t entries, void* stream) {
  return mgb::make_plan(A, plan, entries, mgb::as_stream(stream));
}

int mgb_spmv_csr_planned_f64(const mgb_csr* A, const int32_t* plan, int64_t entries, const double* x, double* y,
                             int init, void* stream) {
  if (plan == nullptr) return MGB_ERR_BAD_ARGUMENT;
  return mgb::launch_csr_dot<double>(A, x, y, init, stream, MGB_CSR_SEGMENTS, nullptr, nullptr, plan, entries);
}

int mgb_spmv_csr_planned_f32(const mgb_csr* A, const int32_t* plan, int64_t entries, const float* x, float* y,
                             int init, void* stream) {
  if (plan == nullptr) return MGB_ERR_BAD_ARGUMENT;
  return mgb::launch_csr_dot<float>(A, x, y, init, stream, MGB_CSR_SEGMENTS, nullptr, nullptr, plan, entries);
}

}  // extern "C"
