// spmv_coo.cu -- COO SpMV for sm_103a (row-sorted keys).
//
// Replaces the reference's CUDA COO path (impl/Coo/Cuda/Morpheus_Multiply_Impl.hpp:50-176:
// flat kernel impl/Coo/Kernels/Morpheus_Multiply_Impl.hpp:121-208, carry pass
// impl/DenseVector/Kernels/Morpheus_Segmented_Reduction_Impl.hpp:40-162 and a
// serial <<<1,1>>> tail).  Like that path the matrix must be sorted by row;
// columns may be in any order and duplicates are allowed.  Semantics are the
// Serial multiply (impl/Coo/Serial/Morpheus_Multiply_Impl.hpp:38-59):
// y = 0 if init, then y[I[n]] += V[n] * x[J[n]].
//
// Design: fixed chunks of COO_CHUNK consecutive entries, one warp each, cut
// into 32 contiguous lane ranges (the lane-segment scheme of spmv_csr.cu, so
// every FP64 FMA is issued by all 32 lanes).  Row indices, columns and values
// are staged through padded shared memory with coalesced loads; a lane
// detects row ends by comparing consecutive row indices.  Rows that cross
// lanes are combined by one segmented shuffle scan per chunk.  The first and
// last row of a chunk may continue in a neighbouring chunk, so their sums are
// written as carries and a small second kernel adds each row's carries in
// chunk order; interior rows are stored directly: deterministic, no atomics,
// no searches.  With init, rows without entries are zero-filled by the lane
// that sees the gap, so y is written once per row.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int COO_WARPS = 8;
constexpr int COO_SEG = 8;                  // entries per lane per staging step
constexpr int COO_PAD = COO_SEG + 1;        // padded lane stride in shared memory
constexpr int64_t COO_CHUNK = 2048;         // entries per warp chunk (largest)

// 2048 entries per chunk, halved (down to 256) while the matrix would give
// fewer chunks than the GPU holds resident warps, so small matrices still
// spread over every SM.
inline int64_t coo_chunk_size(int64_t nnz) {
  int64_t chunk = COO_CHUNK;
  const int64_t resident = (int64_t)num_sms() * COO_WARPS * 3;
  while (chunk > 256 && nnz / chunk < resident) chunk >>= 1;
  return chunk;
}

template <typename T>
__device__ __forceinline__ T gather_x(const T* __restrict__ x, int32_t c, int64_t ncols) {
  return ((uint64_t)(int64_t)c < (uint64_t)ncols) ? __ldg(x + c) : T(0);
}

// IDX: entry and row index type inside the kernel (int32_t when nnz < 2^31 -
// 4096: measured on GB300, power-law COO 252 -> 221 us, same arithmetic).
template <typename T, typename IDX>
__global__ void __launch_bounds__(COO_WARPS * 32, 3)
spmv_coo_segments(int64_t nrows, int64_t ncols, int64_t nnz, int64_t chunk, const int32_t* __restrict__ ri,
                  const int32_t* __restrict__ ci, const T* __restrict__ va, const T* __restrict__ x,
                  T* __restrict__ y, int init, int32_t* __restrict__ carry_row, T* __restrict__ carry_val) {
  __shared__ T s_val[COO_WARPS][32 * COO_PAD];
  __shared__ int32_t s_col[COO_WARPS][32 * COO_PAD];
  __shared__ int32_t s_row[COO_WARPS][32 * COO_PAD];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  T* sv = s_val[w];
  int32_t* sc = s_col[w];
  int32_t* sr = s_row[w];

  const IDX nchunks = (nnz + chunk - 1) / chunk;
  const IDX KW = chunk / 32;  // entries per lane, a multiple of COO_SEG
  for (IDX k = (IDX)blockIdx.x * COO_WARPS + w; k < nchunks; k += (IDX)gridDim.x * COO_WARPS) {
    const IDX base = k * chunk;
    const IDX cend = min(base + chunk, nnz);
    const IDX la = base + (IDX)lane * KW;
    const IDX lb = min(la + KW, cend);
    const bool active = la < lb;
    const IDX first_row = __ldg(ri + base);
    const IDX last_row = __ldg(ri + cend - 1);
    // row of the entry before this lane's range, and of the entry after it
    const IDX prev = (active && la > 0) ? (IDX)__ldg(ri + la - 1) : -1;
    const IDX next = (active && lb < cend) ? (IDX)__ldg(ri + lb) : -2;

    auto finalize = [&](IDX row, T total) {
      if (row == first_row) {
        carry_row[2 * k] = (int32_t)row;
        carry_val[2 * k] = total;
        if (first_row == last_row) {
          carry_row[2 * k + 1] = (int32_t)row;
          carry_val[2 * k + 1] = T(0);
        }
      } else if (row == last_row) {
        carry_row[2 * k + 1] = (int32_t)row;
        carry_val[2 * k + 1] = total;
      } else if (row >= 0 && row < nrows) {
        y[row] = total;
      }
    };
    auto zero_gap = [&](IDX from, IDX to) {  // rows (from, to), init only
      for (IDX g = max(from + 1, (IDX)0); g < min(to, (IDX)nrows); g++) y[g] = T(0);
    };

    IDX cur = -1;          // row being accumulated
    bool cur_here = false;     // it started inside this lane's range
    IDX hrow = -1;
    T hval = T(0), acc = T(0);

    for (IDX st = 0; st < KW; st += COO_SEG) {
      __syncwarp();
#pragma unroll
      for (int q = 0; q < COO_SEG; q++) {
        const int f = q * 32 + lane;
        const int L = f / COO_SEG, j = f % COO_SEG;
        const IDX e = base + (IDX)L * KW + st + j;
        const bool in = e < cend;
        sr[L * COO_PAD + j] = in ? ldg_stream(ri + e) : -1;
        sc[L * COO_PAD + j] = in ? ldg_stream(ci + e) : 0;
        sv[L * COO_PAD + j] = in ? ldg_stream(va + e) : T(0);
      }
      __syncwarp();
      T v[COO_SEG], xv[COO_SEG];
      int32_t rw[COO_SEG];
#pragma unroll
      for (int kk = 0; kk < COO_SEG; kk++) {
        const bool valid = la + st + kk < lb;
        rw[kk] = sr[lane * COO_PAD + kk];
        v[kk] = valid ? sv[lane * COO_PAD + kk] : T(0);
        xv[kk] = valid ? gather_x(x, sc[lane * COO_PAD + kk], ncols) : T(0);
      }
#pragma unroll
      for (int kk = 0; kk < COO_SEG; kk++) {
        const IDX e = la + st + kk;
        if (e < lb && rw[kk] != cur) {  // a new row starts at e (or the lane's first row)
          if (cur >= 0) {
            if (cur_here) finalize(cur, acc); else { hrow = cur; hval = acc; }
          }
          const IDX before = (cur >= 0) ? cur : prev;
          if (init && rw[kk] - before > 1) zero_gap(before, rw[kk]);
          cur = rw[kk];
          cur_here = (e > la) || (prev != cur);
          const bool carried = (cur == first_row) || (cur == last_row);
          acc = (init || carried || !cur_here || cur < 0 || cur >= nrows) ? T(0) : y[cur];
        }
        acc = fmadd(v[kk], xv[kk], acc);
      }
    }
    // the lane's last row: continues into the next lane, or ends here
    bool has_tail = false;
    if (active) {
      if (next == cur) {
        has_tail = true;
      } else {
        if (cur_here) finalize(cur, acc); else { hrow = cur; hval = acc; }
      }
    }
    const IDX key = has_tail ? cur : -1 - (IDX)lane;
    T cv = has_tail ? acc : T(0);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, cv, d);
      const IDX k2 = __shfl_up_sync(0xffffffffu, key, d);
      if (lane >= d && k2 == key) cv += u;
    }
    const T vprev = __shfl_up_sync(0xffffffffu, cv, 1);
    const IDX kprev = __shfl_up_sync(0xffffffffu, key, 1);
    if (hrow >= 0) finalize(hrow, (lane > 0 && kprev == hrow) ? hval + vprev : hval);
    // rows after the last entry of the matrix (init): whole warp fills
    if (init && k == nchunks - 1)
      for (IDX g = max(last_row + 1, (IDX)0) + lane; g < nrows; g += 32) y[g] = T(0);
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
  const int64_t chunk = coo_chunk_size(A->nnz);
  const int64_t nchunks = (A->nnz + chunk - 1) / chunk;
  const int64_t ncarry = 2 * nchunks;
  void* scratch = nullptr;
  const size_t rows_bytes = ((sizeof(int32_t) * ncarry + 255) / 256) * 256;
  MGB_CUDA_CHECK(cudaMallocAsync(&scratch, rows_bytes + sizeof(T) * ncarry, s));
  int32_t* cr = static_cast<int32_t*>(scratch);
  T* cv = reinterpret_cast<T*>(static_cast<char*>(scratch) + rows_bytes);
  const int64_t blocks = (nchunks + COO_WARPS - 1) / COO_WARPS;
  if (A->nnz < ((int64_t)1 << 31) - 4096)
    spmv_coo_segments<T, int32_t><<<(unsigned)blocks, COO_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->nnz, chunk, A->row_indices, A->column_indices,
        static_cast<const T*>(A->values), x, y, init, cr, cv);
  else
    spmv_coo_segments<T, int64_t><<<(unsigned)blocks, COO_WARPS * 32, 0, s>>>(
        A->nrows, A->ncols, A->nnz, chunk, A->row_indices, A->column_indices,
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
// For callers that cannot allocate device memory while they run: real-time
// loops of a host application that forbids allocation once it is running,
// embedded hosts that reserve all device memory up front, and plugins whose
// host process owns the allocator.  mgb_spmv_coo_f64 takes
// its carry buffer from cudaMallocAsync; this variant takes it from a fixed
// file-scope device array instead, so it never calls cudaMalloc, cudaFree or
// any allocating routine.
//
// Limits and rules:
//  * The array is COO_NOALLOC_BYTES (4 MiB) of device memory that every GPU
//    which loads this library holds until the process exits.  It holds two
//    carries (int32 row + double value) per 2048-entry chunk, so A->nnz may be
//    at most 357,892,096; larger matrices get MGB_ERR_INVALID_INPUT before any
//    work is queued.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current) and
//    caches it with the unique ID of the current CUDA context; make that
//    first call before any stream capture.  A later call that finds another
//    context current (after cudaDeviceReset, or a context the caller made
//    current through the driver API) looks the address up again, so the
//    first call in each new context is a set-up call too.  Where the driver
//    gives no context ID, every call looks the address up.
//  * Every call uses the same array and leaves the previous call's carries
//    in it.  Nothing in it needs to start at zero: each call writes every
//    carry slot it reads.  Calls that overlap on the GPU (other streams, other
//    host threads) race on the array; serialise them.
// ---------------------------------------------------------------------------
#include <cuda.h>  // CUcontext / CUresult types only: the driver calls are resolved at run time

#include <mutex>

namespace mgb {
namespace {
constexpr size_t COO_NOALLOC_BYTES = size_t(4) << 20;
}  // namespace
}  // namespace mgb

static __device__ __align__(256) unsigned char g_coo_noalloc_scratch[mgb::COO_NOALLOC_BYTES];

namespace mgb {
namespace {

struct NoallocSlot {
  unsigned long long ctx_id;  // unique ID of the context the address belongs to (0: none)
  void* ptr;
};
std::mutex g_noalloc_mutex;
NoallocSlot g_noalloc[128] = {};

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (no
// link against the driver library).  Context IDs are unique for the life of
// the process, unlike context handles, which a new context may reuse.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current == nullptr || get_id == nullptr || get_current(&c) != CUDA_SUCCESS || c == nullptr ||
      get_id(c, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the scratch array in the current context: looked up on
// the first call per device and again whenever the current context changed.
int noalloc_scratch(void** out) {
  int dev = 0;
  MGB_CUDA_CHECK(cudaGetDevice(&dev));
  MGB_REQUIRE(dev >= 0 && dev < 128, MGB_ERR_RUNTIME);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoallocSlot& slot = g_noalloc[dev];
  const unsigned long long id = current_ctx_id();
  if (slot.ptr == nullptr || id == 0 || slot.ctx_id != id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_coo_noalloc_scratch);
    if (e != cudaSuccess) return record_cuda_error(e);
    slot.ptr = p;
    slot.ctx_id = id != 0 ? id : current_ctx_id();  // the look-up may have created the context
  }
  *out = slot.ptr;
  return MGB_SUCCESS;
}

int launch_coo_noalloc_f64(const mgb_coo* A, const double* x, double* y, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  const int64_t chunk = coo_chunk_size(A->nnz);
  const int64_t nchunks = (A->nnz + chunk - 1) / chunk;
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
  spmv_coo_segments<double, int32_t><<<(unsigned)blocks, COO_WARPS * 32, 0, s>>>(  // nnz is far below 2^31 here
      A->nrows, A->ncols, A->nnz, chunk, A->row_indices, A->column_indices,
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
