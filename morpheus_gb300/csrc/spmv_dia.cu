// spmv_dia.cu -- DIA and HDC SpMV for sm_103a.
//
// DIA replaces impl/Dia/Cuda/Morpheus_Multiply_Impl.hpp:41-85 (kernel
// impl/Dia/Kernels/Morpheus_Multiply_Impl.hpp:37-84).  Semantics are the
// Serial multiply (impl/Dia/Serial/Morpheus_Multiply_Impl.hpp:38-64): per row,
// sum = init ? 0 : y[row]; for each stored diagonal n in order, if the column
// row + offset[n] is inside [0, ncols), sum += values(row, n) * x[col].
//
// HDC replaces impl/Hdc/Cuda/Morpheus_Multiply_Impl.hpp:42-53, which runs the
// DIA kernel (init) and then the CSR kernel (accumulate).  Here both parts are
// fused: each thread finishes the DIA sum of its rows and then adds the row's
// CSR-remainder entries, in that order, and writes y once.
//
// Layout: values(i, n) at values[i + pitch * n], pitch a multiple of 32, so a
// thread owning RPT consecutive rows reads its slab entries with one 16-byte
// (FP64, RPT = 2) or 16-byte (FP32, RPT = 4) vector load per diagonal; the
// warp covers 32 * RPT consecutive rows, fully coalesced.  Offsets live in
// shared memory (chunks of DIA_OFF_CHUNK diagonals).  x is read through the
// read-only path: neighbouring diagonals hit the same lines in L1/L2.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int DIA_THREADS = 256;
constexpr int DIA_OFF_CHUNK = 512;
// FP64: pairs of diagonals whose slab and x loads are issued together
// (measured 204 -> 197 us on the 27-point stencil at 160^3).  FP32: the plain
// diagonal loop, which the compiler unrolls itself at 40 registers; explicit
// groups of 2 or 4 raise the register count and lower occupancy (87 us
// plain, 93-97 us grouped).
template <typename T> constexpr int kDiaUnroll = sizeof(T) == 4 ? 1 : 2;
// Resident CTAs of 256 threads per SM the kernel is compiled for (0: no
// register cap).  FP64: 8 (32 registers, a few bytes of spills), the FP64
// pipe fed by 64 warps: 27-point stencil DIA 197 -> 195 us, HDC 220 -> 209 us
// (5 / 6 CTAs: 199 / 196 us).  FP32 is fastest uncapped (40 registers:
// 87 us; capped at 5-8 CTAs: 88.5-95.6 us).
template <typename T> constexpr int kDiaMinBlocks = sizeof(T) == 4 ? 0 : 8;

template <typename T> struct Vec;
template <> struct Vec<double> { using type = double2; static constexpr int n = 2; };
template <> struct Vec<float> { using type = float4; static constexpr int n = 4; };

template <typename T>
__device__ __forceinline__ void load_vec(const T* p, T* out);
template <>
__device__ __forceinline__ void load_vec<double>(const double* p, double* out) {
  const double2 v = __ldcs(reinterpret_cast<const double2*>(p));
  out[0] = v.x; out[1] = v.y;
}
template <>
__device__ __forceinline__ void load_vec<float>(const float* p, float* out) {
  const float4 v = __ldcs(reinterpret_cast<const float4*>(p));
  out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
}

// The RPT slab entries of rows row0.. of one diagonal: one 16-byte load when
// all RPT rows exist, else element loads (rows past nrows read as 0).
template <typename T, int RPT>
__device__ __forceinline__ void dia_load(const T* vp, int64_t row0, int64_t nrows, T* v) {
  if (RPT > 1 && row0 + RPT <= nrows) {
    load_vec<T>(vp, v);
  } else {
#pragma unroll
    for (int i = 0; i < RPT; i++) v[i] = (row0 + i < nrows) ? __ldcs(vp + i) : T(0);
  }
}

// One thread = RPT consecutive rows (vector path, requires pitch % RPT == 0
// and an aligned values pointer) or RPT = 1 (scalar path).
template <typename T, int RPT, bool HDC>
__global__ void __launch_bounds__(DIA_THREADS, kDiaMinBlocks<T>)
spmv_dia_rows(int64_t nrows, int64_t ncols, int ndiags, int64_t pitch,
              const int32_t* __restrict__ offs, const T* __restrict__ vals,
              const int32_t* __restrict__ cro, const int32_t* __restrict__ cci,
              const T* __restrict__ cva, int64_t csr_nnz,
              const T* __restrict__ x, T* __restrict__ y, int init) {
  constexpr int DU = kDiaUnroll<T>;
  __shared__ int32_t s_off[DIA_OFF_CHUNK];
  const int64_t ngroups = (nrows + RPT - 1) / RPT;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // grid-stride over row groups; every thread of the CTA runs the same number
  // of iterations so the __syncthreads around offset staging are uniform.
  const int64_t first = (int64_t)blockIdx.x * blockDim.x;
  for (int64_t g0 = first; g0 < ngroups; g0 += stride) {
    const int64_t g = g0 + threadIdx.x;
    const int64_t row0 = g * RPT;
    T acc[RPT];
#pragma unroll
    for (int i = 0; i < RPT; i++) {
      const int64_t r = row0 + i;
      acc[i] = (r < nrows && !init) ? y[r] : T(0);
    }
    for (int d0 = 0; d0 < ndiags; d0 += DIA_OFF_CHUNK) {
      const int dn = min(DIA_OFF_CHUNK, ndiags - d0);
      __syncthreads();
      for (int t = threadIdx.x; t < dn; t += blockDim.x) s_off[t] = offs[d0 + t];
      __syncthreads();
      if (g < ngroups) {
        // DU diagonals at a time: every slab and x load of the group
        // is issued before the first FMA, then the FMAs run in diagonal order
        // (the Serial summation order is kept).
        int d = 0;
        if constexpr (DU > 1) for (; d + DU <= dn; d += DU) {
          T v[DU][RPT], xv[DU][RPT];
          int64_t off[DU];
#pragma unroll
          for (int u = 0; u < DU; u++) {
            off[u] = s_off[d + u];
            dia_load<T, RPT>(vals + row0 + pitch * (int64_t)(d0 + d + u), row0, nrows, v[u]);
#pragma unroll
            for (int i = 0; i < RPT; i++) {
              const int64_t col = row0 + i + off[u];
              xv[u][i] = (row0 + i < nrows && col >= 0 && col < ncols) ? __ldg(x + col) : T(0);
            }
          }
#pragma unroll
          for (int u = 0; u < DU; u++)
#pragma unroll
            for (int i = 0; i < RPT; i++) {
              const int64_t col = row0 + i + off[u];
              if (row0 + i < nrows && col >= 0 && col < ncols) acc[i] = fmadd(v[u][i], xv[u][i], acc[i]);
            }
        }
        for (; d < dn; d++) {
          const int64_t off = s_off[d];
          T v[RPT];
          dia_load<T, RPT>(vals + row0 + pitch * (int64_t)(d0 + d), row0, nrows, v);
#pragma unroll
          for (int i = 0; i < RPT; i++) {
            const int64_t col = row0 + i + off;
            if (row0 + i < nrows && col >= 0 && col < ncols)
              acc[i] = fmadd(v[i], __ldg(x + col), acc[i]);
          }
        }
      }
    }
    if (g < ngroups) {
#pragma unroll
      for (int i = 0; i < RPT; i++) {
        const int64_t r = row0 + i;
        if (r < nrows) {
          T a = acc[i];
          if (HDC) {
            int32_t rs = cro[r], re = cro[r + 1];
            rs = max(rs, 0);
            re = (int32_t)min((int64_t)re, csr_nnz);
            for (int32_t j = rs; j < re; j++) {
              const int32_t c = cci[j];
              if ((uint64_t)(int64_t)c < (uint64_t)ncols) a = fmadd(cva[j], __ldg(x + c), a);
            }
          }
          y[r] = a;
        }
      }
    }
  }
}

template <typename T, bool HDC>
int launch_dia_rows(const mgb_dia* D, const mgb_csr* C, const T* x, T* y, int init,
                    cudaStream_t s) {
  constexpr int V = Vec<T>::n;
  const bool vec_ok = (D->pitch % V == 0) &&
                      (reinterpret_cast<uintptr_t>(D->values) % 16 == 0);
  const int64_t rpt = vec_ok ? V : 1;
  const int64_t groups = (D->nrows + rpt - 1) / rpt;
  int64_t blocks = (groups + DIA_THREADS - 1) / DIA_THREADS;
  const int64_t cap = (int64_t)num_sms() * 64;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  const int32_t* cro = HDC ? C->row_offsets : nullptr;
  const int32_t* cci = HDC ? C->column_indices : nullptr;
  const T* cva = HDC ? static_cast<const T*>(C->values) : nullptr;
  const int64_t cnnz = HDC ? C->nnz : 0;
  const T* vals = static_cast<const T*>(D->values);
  if (vec_ok)
    spmv_dia_rows<T, V, HDC><<<(unsigned)blocks, DIA_THREADS, 0, s>>>(
        D->nrows, D->ncols, (int)D->ndiags, D->pitch, D->diagonal_offsets, vals,
        cro, cci, cva, cnnz, x, y, init);
  else
    spmv_dia_rows<T, 1, HDC><<<(unsigned)blocks, DIA_THREADS, 0, s>>>(
        D->nrows, D->ncols, (int)D->ndiags, D->pitch, D->diagonal_offsets, vals,
        cro, cci, cva, cnnz, x, y, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int check_dia(const mgb_dia* D) {
  MGB_REQUIRE(D != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(D->nrows, D->ncols, D->nnz) && D->ndiags >= 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(D->ndiags == 0 || (D->pitch >= D->nrows && D->diagonal_offsets && D->values),
              MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(D->ndiags < ((int64_t)1 << 31), MGB_ERR_INVALID_INPUT);
  return MGB_SUCCESS;
}

template <typename T>
int launch_dia(const mgb_dia* D, const T* x, T* y, int init, cudaStream_t s) {
  int st = check_dia(D);
  if (st != MGB_SUCCESS) return st;
  if (D->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(y != nullptr && (D->ndiags == 0 || x != nullptr), MGB_ERR_BAD_ARGUMENT);
  return launch_dia_rows<T, false>(D, nullptr, x, y, init, s);
}

template <typename T>
int launch_hdc(const mgb_hdc* H, const T* x, T* y, int init, cudaStream_t s) {
  MGB_REQUIRE(H != nullptr, MGB_ERR_BAD_ARGUMENT);
  int st = check_dia(&H->dia);
  if (st != MGB_SUCCESS) return st;
  const mgb_csr* C = &H->csr;
  MGB_REQUIRE(!bad_sizes(C->nrows, C->ncols, C->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(C->nrows == H->dia.nrows, MGB_ERR_INVALID_INPUT);
  if (H->dia.nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(y != nullptr && x != nullptr && C->row_offsets != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(C->nnz == 0 || (C->column_indices && C->values), MGB_ERR_BAD_ARGUMENT);
  return launch_dia_rows<T, true>(&H->dia, C, x, y, init, s);
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_spmv_dia_f64(const mgb_dia* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_dia<double>(A, x, y, init, mgb::as_stream(stream));
}
int mgb_spmv_dia_f32(const mgb_dia* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_dia<float>(A, x, y, init, mgb::as_stream(stream));
}
int mgb_spmv_hdc_f64(const mgb_hdc* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_hdc<double>(A, x, y, init, mgb::as_stream(stream));
}
int mgb_spmv_hdc_f32(const mgb_hdc* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_hdc<float>(A, x, y, init, mgb::as_stream(stream));
}

}  // extern "C"
