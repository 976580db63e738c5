// vector_ops.cu -- dot / reduce / waxpby for sm_103a.
//
// dot replaces impl/DenseVector/Cuda/Morpheus_Dot_Impl.hpp:59-144 (cuBLAS
// cublasDdot when enabled -- with the float overload wrongly calling Ddot --
// else two kernels plus a synchronous copy).  Semantics: Serial dot
// (impl/DenseVector/Serial/Morpheus_Dot_Impl.hpp:38-59), sum of x[i]*y[i].
// reduce replaces impl/DenseVector/Cuda/Morpheus_Reduction_Impl.hpp:175-234
// (multi-pass kernels and a host Kahan finish).  Semantics: the Serial Kahan
// sum of in[0..size) (impl/DenseVector/Serial/Morpheus_Reduction_Impl.hpp:40-61);
// here a fixed-shape pairwise tree, deterministic for a given size and GPU.
// waxpby replaces impl/DenseVector/Cuda/Morpheus_WAXPBY_Impl.hpp:40-70:
// w = alpha*x + beta*y with the alpha == 1 / beta == 1 special cases of
// impl/DenseVector/Serial/Morpheus_WAXPBY_Impl.hpp:59-65.
//
// Reductions: a grid of at most 4 CTAs per SM accumulates with one FMA (dot)
// or add (reduce) per element and 16-byte loads, reduces in-CTA with
// shuffles, and a one-CTA kernel sums the per-CTA partials.  The partials live
// in stream-ordered scratch (cudaMallocAsync), so no global state is shared
// between calls or streams.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int RED_THREADS = 256;

template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T s_part[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) s_part[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? s_part[threadIdx.x] : T(0);
  if (w == 0) v = warp_sum(v);
  return v;  // valid in thread 0
}

// 16-byte streaming load / store of V = 16 / sizeof(T) elements at vector index i
template <typename T>
__device__ __forceinline__ void ld16(const T* p, int64_t i, T* a) {
  if constexpr (sizeof(T) == 8) {
    const double2 v = __ldcs(reinterpret_cast<const double2*>(p) + i);
    a[0] = v.x; a[1] = v.y;
  } else {
    const float4 v = __ldcs(reinterpret_cast<const float4*>(p) + i);
    a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
  }
}

template <typename T>
__device__ __forceinline__ void st16(T* p, int64_t i, const T* a) {
  if constexpr (sizeof(T) == 8) __stcs(reinterpret_cast<double2*>(p) + i, make_double2(a[0], a[1]));
  else __stcs(reinterpret_cast<float4*>(p) + i, make_float4(a[0], a[1], a[2], a[3]));
}

// Exact fixed-point accumulation of doubles on the integer pipe.  On this GPU
// the FP64 add rate (5.3e11 per second measured, the same as the FMA rate)
// bounds a pure FP64 sum at 8 bytes per add, 4.2 TB/s, below HBM.  The sum
// kernel therefore adds 7 of every 16 elements here instead: the two pipes
// run side by side (2^26 doubles: 90 us, against 138 us all-FP64 and 160 us
// all-integer).
//
// The accumulator is a signed 128-bit integer whose unit is
// 2^(S - 1150 + EXACT_HEADROOM) for the largest biased exponent S seen so far;
// each element's 53-bit significand is placed 10 bits below the top of a
// 64-bit word and shifted into place, so an element of exponent S occupies
// bits [64 - EXACT_HEADROOM .. 126 - EXACT_HEADROOM] and up to 2^20 of them
// sum without overflow.  A larger exponent shifts the accumulator right
// first (dropped bits are below 2^-100 of the largest element).  Inf and NaN
// are added in FP64 so they propagate as in the Serial sum.
constexpr int EXACT_HEADROOM = 20;

struct ExactSum {
  __int128 acc = 0;
  int S = 0;

  __device__ __forceinline__ void add(double v, double& fp_fallback) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const int e = (int)(b >> 52) & 0x7ff;
    if (e == 0x7ff) {
      fp_fallback += v;
      return;
    }
    // subnormals: exponent 1 without the implicit bit
    const int64_t m = (int64_t)(((b & 0xfffffffffffffull) | (e ? (1ull << 52) : 0ull)) << 10);
    const int64_t ms = (b >> 63) ? -m : m;
    const int s = max(e, 1);
    if (s > S) {
      acc >>= min(s - S, 127);
      S = s;
    }
    // ms * 2^64 (the bit pattern shifted as unsigned: no signed left shift)
    const __int128 t = (__int128)((unsigned __int128)(uint64_t)ms << 64);
    acc += t >> min(S - s + EXACT_HEADROOM, 127);
  }

  // the accumulated value as a double (at most two roundings)
  __device__ __forceinline__ double value() const {
    if (acc == 0) return 0.0;
    const double d = fma((double)(long long)(acc >> 64), 0x1p64, (double)(unsigned long long)acc);
    return ldexp(d, S - 1149 + EXACT_HEADROOM);
  }
};

// MODE 0: dot(x, y); MODE 1: dot(x, x); MODE 2: sum(x)
// Each grid-stride step of the vector body issues eight 16-byte loads per
// thread before it accumulates (U vectors of x, and of y for MODE 0), so an
// SM with 1,024 threads keeps 128 KB of loads in flight.  Four accumulators
// per thread.  Measured on x.y over 2^26 doubles: 7.0 TB/s of reads with
// U = 4 at 4 CTAs per SM, against 6.4-6.9 TB/s with 1-2 and 5.6-6.2 TB/s
// at 2 or 8 CTAs per SM.
template <typename T, int MODE>
__global__ void __launch_bounds__(RED_THREADS, 4)
reduce_partial(int64_t n, const T* __restrict__ x, const T* __restrict__ y,
               T* __restrict__ partial) {
  T acc[4] = {T(0), T(0), T(0), T(0)};
  constexpr bool EXACT = (MODE == 2) && sizeof(T) == 8;  // FP64 sum: split with the integer pipe
  ExactSum ex;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  // 16-byte vector body when both pointers are 16-byte aligned
  constexpr int V = 16 / sizeof(T);
  constexpr int U = (MODE == 0) ? 4 : 8;
  const bool vec = (reinterpret_cast<uintptr_t>(x) % 16 == 0) &&
                   (MODE != 0 || reinterpret_cast<uintptr_t>(y) % 16 == 0);
  int64_t done = 0;
  if (vec) {
    const int64_t nv = n / V;
    int64_t i = tid;
#pragma unroll 1
    for (; i + (U - 1) * nth < nv; i += U * nth) {
      T a[U][V], b[U][V];
#pragma unroll
      for (int u = 0; u < U; u++) {
        ld16(x, i + u * nth, a[u]);
        if constexpr (MODE == 0) ld16(y, i + u * nth, b[u]);
      }
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int k = 0; k < V; k++) {
          T& s = acc[(u * V + k) & 3];
          if constexpr (MODE == 0) s = fmadd(a[u][k], b[u][k], s);
          else if constexpr (MODE == 1) s = fmadd(a[u][k], a[u][k], s);
          else if constexpr (EXACT) {
            // 7 of the 16 elements of the step (spread over the step)
            if ((u * V + k) * 7 % 16 < 7) ex.add(a[u][k], s);
            else s += a[u][k];
          } else s += a[u][k];
        }
    }
    for (; i < nv; i += nth) {
      T a[V], b[V];
      ld16(x, i, a);
      if constexpr (MODE == 0) ld16(y, i, b);
#pragma unroll
      for (int k = 0; k < V; k++) {
        T& s = acc[k & 3];
        if constexpr (MODE == 0) s = fmadd(a[k], b[k], s);
        else if constexpr (MODE == 1) s = fmadd(a[k], a[k], s);
        else s += a[k];
      }
    }
    done = nv * V;
  }
  for (int64_t i = done + tid; i < n; i += nth) {
    const T a = __ldcs(x + i);
    if (MODE == 0) acc[0] = fmadd(a, __ldcs(y + i), acc[0]);
    else if (MODE == 1) acc[0] = fmadd(a, a, acc[0]);
    else acc[0] += a;
  }
  T total = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  if constexpr (EXACT) total += ex.value();
  const T s = block_sum(total);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(1024) sum_partials(int n, const T* __restrict__ p, T* __restrict__ out) {
  T acc = T(0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += p[i];
  const T s = block_sum(acc);
  if (threadIdx.x == 0) *out = s;
}

template <typename T, int MODE>
int launch_reduce(int64_t n, const T* x, const T* y, T* d_result, cudaStream_t s) {
  MGB_REQUIRE(n >= 0 && d_result != nullptr, MGB_ERR_BAD_ARGUMENT);
  if (n == 0) {
    MGB_CUDA_CHECK(cudaMemsetAsync(d_result, 0, sizeof(T), s));
    return MGB_SUCCESS;
  }
  MGB_REQUIRE(x != nullptr && (MODE != 0 || y != nullptr), MGB_ERR_BAD_ARGUMENT);
  int64_t blocks = (n + RED_THREADS * 8 - 1) / (RED_THREADS * 8);
  const int64_t cap = (int64_t)num_sms() * 4;
  if (blocks > cap) blocks = cap;
  T* partial = nullptr;
  MGB_CUDA_CHECK(cudaMallocAsync((void**)&partial, sizeof(T) * blocks, s));
  reduce_partial<T, MODE><<<(unsigned)blocks, RED_THREADS, 0, s>>>(n, x, y, partial);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    sum_partials<T><<<1, 1024, 0, s>>>((int)blocks, partial, d_result);
    e = cudaGetLastError();
  }
  cudaError_t ef = cudaFreeAsync(partial, s);
  if (e != cudaSuccess) return record_cuda_error(e);
  if (ef != cudaSuccess) return record_cuda_error(ef);
  return MGB_SUCCESS;
}

template <typename T, int MODE>
int reduce_to_host(int64_t n, const T* x, const T* y, T* result, cudaStream_t s) {
  MGB_REQUIRE(result != nullptr, MGB_ERR_BAD_ARGUMENT);
  T* d = nullptr;
  MGB_CUDA_CHECK(cudaMallocAsync((void**)&d, sizeof(T), s));
  int st = launch_reduce<T, MODE>(n, x, y, d, s);
  if (st == MGB_SUCCESS) {
    cudaError_t e = cudaMemcpyAsync(result, d, sizeof(T), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = record_cuda_error(e);
  }
  cudaError_t ef = cudaFreeAsync(d, s);
  if (st == MGB_SUCCESS && ef != cudaSuccess) st = record_cuda_error(ef);
  return st;
}

template <typename T>
int dot_any(int64_t n, const T* x, const T* y, T* out, cudaStream_t s, bool host) {
  if (x == y) return host ? reduce_to_host<T, 1>(n, x, x, out, s) : launch_reduce<T, 1>(n, x, x, out, s);
  return host ? reduce_to_host<T, 0>(n, x, y, out, s) : launch_reduce<T, 0>(n, x, y, out, s);
}

// MODE 0: alpha*x + beta*y, 1: x + beta*y, 2: alpha*x + y
template <typename T, int MODE>
__device__ __forceinline__ T wax(T alpha, T a, T beta, T b) {
  if constexpr (MODE == 1) return fmadd(beta, b, a);
  else if constexpr (MODE == 2) return fmadd(alpha, a, b);
  else return fmadd(alpha, a, beta * b);
}

// w may be x or y (in-place updates): each element is read and written by
// the same thread at the same index, so the pointers carry no __restrict__.
// 16-byte loads and stores when all three are 16-byte aligned.
template <typename T, int MODE>
__global__ void waxpby_kernel(int64_t n, T alpha, const T* x, T beta, const T* y, T* w) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  constexpr int V = 16 / sizeof(T);
  const bool vec = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y) |
                     reinterpret_cast<uintptr_t>(w)) % 16) == 0;
  int64_t done = 0;
  if (vec) {
    const int64_t nv = n / V;
    for (int64_t i = tid; i < nv; i += nth) {
      T a[V], b[V], r[V];
      ld16(x, i, a);
      ld16(y, i, b);
#pragma unroll
      for (int k = 0; k < V; k++) r[k] = wax<T, MODE>(alpha, a[k], beta, b[k]);
      st16(w, i, r);
    }
    done = nv * V;
  }
  for (int64_t i = done + tid; i < n; i += nth)
    __stcs(w + i, wax<T, MODE>(alpha, __ldcs(x + i), beta, __ldcs(y + i)));
}

template <typename T>
int launch_waxpby(int64_t n, T alpha, const T* x, T beta, const T* y, T* w, cudaStream_t s) {
  MGB_REQUIRE(n >= 0, MGB_ERR_BAD_ARGUMENT);
  if (n == 0) return MGB_SUCCESS;
  MGB_REQUIRE(x && y && w, MGB_ERR_BAD_ARGUMENT);
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;  // one resident wave of 2,048 threads per SM
  if (blocks > cap) blocks = cap;
  if (alpha == T(1))
    waxpby_kernel<T, 1><<<(unsigned)blocks, 256, 0, s>>>(n, alpha, x, beta, y, w);
  else if (beta == T(1))
    waxpby_kernel<T, 2><<<(unsigned)blocks, 256, 0, s>>>(n, alpha, x, beta, y, w);
  else
    waxpby_kernel<T, 0><<<(unsigned)blocks, 256, 0, s>>>(n, alpha, x, beta, y, w);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_dot_f64(int64_t n, const double* x, const double* y, double* result, void* stream) {
  return mgb::dot_any<double>(n, x, y, result, mgb::as_stream(stream), true);
}
int mgb_dot_f32(int64_t n, const float* x, const float* y, float* result, void* stream) {
  return mgb::dot_any<float>(n, x, y, result, mgb::as_stream(stream), true);
}
int mgb_dot_f64_async(int64_t n, const double* x, const double* y, double* d_result, void* stream) {
  return mgb::dot_any<double>(n, x, y, d_result, mgb::as_stream(stream), false);
}
int mgb_dot_f32_async(int64_t n, const float* x, const float* y, float* d_result, void* stream) {
  return mgb::dot_any<float>(n, x, y, d_result, mgb::as_stream(stream), false);
}
int mgb_reduce_f64(const double* in, int64_t size, double* result, void* stream) {
  return mgb::reduce_to_host<double, 2>(size, in, nullptr, result, mgb::as_stream(stream));
}
int mgb_reduce_f32(const float* in, int64_t size, float* result, void* stream) {
  return mgb::reduce_to_host<float, 2>(size, in, nullptr, result, mgb::as_stream(stream));
}
int mgb_reduce_f64_async(const double* in, int64_t size, double* d_result, void* stream) {
  return mgb::launch_reduce<double, 2>(size, in, nullptr, d_result, mgb::as_stream(stream));
}
int mgb_reduce_f32_async(const float* in, int64_t size, float* d_result, void* stream) {
  return mgb::launch_reduce<float, 2>(size, in, nullptr, d_result, mgb::as_stream(stream));
}
int mgb_waxpby_f64(int64_t n, double alpha, const double* x, double beta, const double* y, double* w, void* stream) {
  return mgb::launch_waxpby<double>(n, alpha, x, beta, y, w, mgb::as_stream(stream));
}
int mgb_waxpby_f32(int64_t n, float alpha, const float* x, float beta, const float* y, float* w, void* stream) {
  return mgb::launch_waxpby<float>(n, alpha, x, beta, y, w, mgb::as_stream(stream));
}

}  // extern "C"
