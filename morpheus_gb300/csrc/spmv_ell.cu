// spmv_ell.cu -- ELL and HYB SpMV for sm_103a.
//
// ELL replaces impl/Ell/Cuda/Morpheus_Multiply_Impl.hpp:41-80 (kernel
// impl/Ell/Kernels/Morpheus_Multiply_Impl.hpp:37-65).  Semantics are the
// Serial multiply (impl/Ell/Serial/Morpheus_Multiply_Impl.hpp:38-67): y = 0 if
// init, then for each row and each of the `width` padded slots whose column
// is not the invalid index (-1), y[i] += values(i, n) * x[col].
//
// HYB replaces impl/Hyb/Cuda/Morpheus_Multiply_Impl.hpp:42-53: the ELL part
// with init, then the COO part accumulating into y.
//
// Layout: slot (i, n) at [i + pitch * n], pitch = nrows (column-major, the
// reference's CUDA LayoutLeft).  A thread owns RPT = 4 consecutive rows and
// reads each slot column with one 16-byte load of their column indices
// (int4) and, only where one of the 4 slots holds an entry, 16-byte loads of
// the values (two double2 / one float4): padding values are never read, and
// a warp whose 128 rows are all padding at slot n skips the value sectors.
// Pitches or pointers that do not allow 16-byte loads take 2 or 1 rows per
// thread.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int ELL_THREADS = 256;

template <typename T, int RPT> struct EllVec;
template <> struct EllVec<double, 4> {
  static __device__ __forceinline__ void load(const double* p, double* o) {
    const double2 a = __ldcs(reinterpret_cast<const double2*>(p));
    const double2 b = __ldcs(reinterpret_cast<const double2*>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  }
};
template <> struct EllVec<float, 4> {
  static __device__ __forceinline__ void load(const float* p, float* o) {
    const float4 v = __ldcs(reinterpret_cast<const float4*>(p)); o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
};
template <> struct EllVec<double, 2> {
  static __device__ __forceinline__ void load(const double* p, double* o) {
    const double2 v = __ldcs(reinterpret_cast<const double2*>(p)); o[0] = v.x; o[1] = v.y;
  }
};
template <> struct EllVec<float, 2> {
  static __device__ __forceinline__ void load(const float* p, float* o) {
    const float2 v = __ldcs(reinterpret_cast<const float2*>(p)); o[0] = v.x; o[1] = v.y;
  }
};
template <typename T> struct EllVec<T, 1> {
  static __device__ __forceinline__ void load(const T* p, T* o) { o[0] = __ldcs(p); }
};

template <int RPT> struct IdxVec;
template <> struct IdxVec<4> {
  static __device__ __forceinline__ void load(const int32_t* p, int32_t* o) {
    const int4 v = __ldcs(reinterpret_cast<const int4*>(p)); o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
};
template <> struct IdxVec<2> {
  static __device__ __forceinline__ void load(const int32_t* p, int32_t* o) {
    const int2 v = __ldcs(reinterpret_cast<const int2*>(p)); o[0] = v.x; o[1] = v.y;
  }
};
template <> struct IdxVec<1> {
  static __device__ __forceinline__ void load(const int32_t* p, int32_t* o) { o[0] = __ldcs(p); }
};

// MINB: resident CTAs of 256 threads per SM the kernel is compiled for (0:
// no register cap); the launcher picks it.
template <typename T, int RPT, int MINB>
__global__ void __launch_bounds__(ELL_THREADS, MINB)
spmv_ell_rows(int64_t nrows, int64_t ncols, int64_t width, int64_t pitch,
              const int32_t* __restrict__ ci, const T* __restrict__ va,
              const T* __restrict__ x, T* __restrict__ y, int init) {
  const int64_t ngroups = (nrows + RPT - 1) / RPT;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row0 = g * RPT;
    const bool full = row0 + RPT <= nrows;
    T acc[RPT];
#pragma unroll
    for (int i = 0; i < RPT; i++) acc[i] = (row0 + i < nrows && !init) ? y[row0 + i] : T(0);
    for (int64_t n = 0; n < width; n++) {
      const int64_t base = row0 + pitch * n;
      int32_t c[RPT];
      if (full) {
        IdxVec<RPT>::load(ci + base, c);
      } else {
#pragma unroll
        for (int i = 0; i < RPT; i++) c[i] = (row0 + i < nrows) ? __ldcs(ci + base + i) : -1;
      }
      bool any = false;
#pragma unroll
      for (int i = 0; i < RPT; i++) any |= ((uint64_t)(int64_t)c[i] < (uint64_t)ncols);
      if (any) {
        T v[RPT];
        if (full) {
          EllVec<T, RPT>::load(va + base, v);
        } else {
#pragma unroll
          for (int i = 0; i < RPT; i++) v[i] = (row0 + i < nrows) ? __ldcs(va + base + i) : T(0);
        }
#pragma unroll
        for (int i = 0; i < RPT; i++)
          if ((uint64_t)(int64_t)c[i] < (uint64_t)ncols) acc[i] = fmadd(v[i], __ldg(x + c[i]), acc[i]);
      }
    }
#pragma unroll
    for (int i = 0; i < RPT; i++)
      if (row0 + i < nrows) y[row0 + i] = acc[i];
  }
}

}  // namespace

template <typename T, int MINB>
int launch_ell_rows(const mgb_ell* A, const T* x, T* y, int init, cudaStream_t s, int64_t blocks, int rpt) {
  const T* va = static_cast<const T*>(A->values);
  if (rpt == 4)
    spmv_ell_rows<T, 4, MINB><<<(unsigned)blocks, ELL_THREADS, 0, s>>>(
        A->nrows, A->ncols, A->width, A->pitch, A->column_indices, va, x, y, init);
  else if (rpt == 2)
    spmv_ell_rows<T, 2, MINB><<<(unsigned)blocks, ELL_THREADS, 0, s>>>(
        A->nrows, A->ncols, A->width, A->pitch, A->column_indices, va, x, y, init);
  else
    spmv_ell_rows<T, 1, MINB><<<(unsigned)blocks, ELL_THREADS, 0, s>>>(
        A->nrows, A->ncols, A->width, A->pitch, A->column_indices, va, x, y, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int launch_ell(const mgb_ell* A, const T* x, T* y, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz) && A->width >= 0, MGB_ERR_BAD_ARGUMENT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(y != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->width == 0 || (A->pitch >= A->nrows && A->column_indices && A->values && x),
              MGB_ERR_BAD_ARGUMENT);
  // 16-byte loads need every slot column (row0 + pitch * n, row0 a multiple
  // of RPT) 16-byte aligned: pitch a multiple of 4 and 16-byte base pointers
  const uintptr_t ap = reinterpret_cast<uintptr_t>(A->values), ai = reinterpret_cast<uintptr_t>(A->column_indices);
  const bool vec4 = (A->pitch % 4 == 0) && (ap % 16 == 0) && (ai % 16 == 0);
  const bool vec2 = (A->pitch % 2 == 0) && (ap % (2 * sizeof(T)) == 0) && (ai % 8 == 0);
  const int rpt = vec4 ? 4 : (vec2 ? 2 : 1);
  const int64_t groups = (A->nrows + rpt - 1) / rpt;
  int64_t blocks = (groups + ELL_THREADS - 1) / ELL_THREADS;
  const int64_t cap = (int64_t)num_sms() * 64;
  if (blocks > cap) blocks = cap;
  // Register caps (measured, 27-point stencil in ELL / power-law HYB at the
  // p90 width): FP32 at 8 CTAs per SM, 178 -> 173 us / 252 -> 240 us.  FP64
  // at 6 CTAs per SM where at least half the slots hold entries (FMA-heavy:
  // stencil 258 -> 241 us), uncapped for mostly-padding slabs (HYB p90: 277
  // us uncapped, 297 us at 6 CTAs).
  if constexpr (sizeof(T) == 4) {
    return launch_ell_rows<T, 8>(A, x, y, init, s, blocks, rpt);
  } else {
    const bool dense = 2 * A->nnz >= A->nrows * A->width;
    if (dense) return launch_ell_rows<T, 6>(A, x, y, init, s, blocks, rpt);
    return launch_ell_rows<T, 0>(A, x, y, init, s, blocks, rpt);
  }
}

template int launch_ell<double>(const mgb_ell*, const double*, double*, int, cudaStream_t);
template int launch_ell<float>(const mgb_ell*, const float*, float*, int, cudaStream_t);

template <typename T>
int launch_hyb(const mgb_hyb* A, const T* x, T* y, int init, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->ell.nrows == A->coo.nrows, MGB_ERR_INVALID_INPUT);
  int st = launch_ell<T>(&A->ell, x, y, init, s);
  if (st != MGB_SUCCESS) return st;
  if (A->coo.nnz == 0) return MGB_SUCCESS;
  return launch_coo<T>(&A->coo, x, y, 0, s);
}

}  // namespace mgb

extern "C" {

int mgb_spmv_ell_f64(const mgb_ell* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_ell<double>(A, x, y, init, mgb::as_stream(stream));
}
int mgb_spmv_ell_f32(const mgb_ell* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_ell<float>(A, x, y, init, mgb::as_stream(stream));
}
int mgb_spmv_hyb_f64(const mgb_hyb* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_hyb<double>(A, x, y, init, mgb::as_stream(stream));
}
int mgb_spmv_hyb_f32(const mgb_hyb* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_hyb<float>(A, x, y, init, mgb::as_stream(stream));
}

}  // extern "C"
