// mgb_internal.cuh -- shared helpers of the morpheus-gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mgb.h"

namespace mgb {

// Records the CUDA error text for mgb_last_cuda_error_string() and returns
// MGB_ERR_CUDA (or MGB_ERR_ALLOC for an out-of-memory error).
int record_cuda_error(cudaError_t e);

// Number of SMs of the current device (queried once per device and cached,
// unlike the reference which queries device properties on every launch,
// impl/Morpheus_CudaUtils.hpp:77-90).  If the query fails it records the CUDA
// error, returns 1 (a grid that is still valid) and flags the failure for
// take_device_query_error(), which MGB_LAUNCH_CHECK consults: the entry point
// then returns MGB_ERR_CUDA instead of running on a guessed SM count.
int num_sms();
// MGB_ERR_CUDA once after a failed num_sms() query on this thread, else MGB_SUCCESS.
int take_device_query_error();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace mgb

#define MGB_CUDA_CHECK(call)                                  \
  do {                                                        \
    cudaError_t mgb_e_ = (call);                              \
    if (mgb_e_ != cudaSuccess) return ::mgb::record_cuda_error(mgb_e_); \
  } while (0)

#define MGB_LAUNCH_CHECK()                                          \
  do {                                                              \
    MGB_CUDA_CHECK(cudaGetLastError());                             \
    const int mgb_q_ = ::mgb::take_device_query_error();            \
    if (mgb_q_ != MGB_SUCCESS) return mgb_q_;                       \
  } while (0)

#define MGB_REQUIRE(cond, status) \
  do {                            \
    if (!(cond)) return (status); \
  } while (0)

namespace mgb {

constexpr int WARP = 32;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// fused multiply-add in the value type (one DFMA / FFMA per nonzero)
__device__ __forceinline__ double fmadd(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmadd(float a, float b, float c) { return fmaf(a, b, c); }

// Read-only, no-L1-allocate streaming loads for matrix data that is used once.
template <typename T>
__device__ __forceinline__ T ldg_stream(const T* p) { return __ldcs(p); }

// Launchers shared between translation units (HYB = ELL + COO).
template <typename T>
int launch_ell(const mgb_ell* A, const T* x, T* y, int init, cudaStream_t s);
template <typename T>
int launch_coo(const mgb_coo* A, const T* x, T* y, int init, cudaStream_t s);
// CSR SpMV with an explicit kernel (MGB_CSR_SEGMENTS / MGB_CSR_ROWS /
// MGB_CSR_SPLIT / MGB_CSR_ROWS_GATHER).  With partials != nullptr the kernel also forms
// x[0..nrows) . y, one partial per warp, *npartials of them; partials ==
// nullptr with npartials != nullptr only reports that count.  plan: an
// optional chunk plan of plan_entries entries (lane-segment kernel only).
template <typename T>
int launch_csr_dot(const mgb_csr* A, const T* x, T* y, int init, void* stream, int variant, T* partials,
                   int64_t* npartials, const int32_t* plan = nullptr, int64_t plan_entries = 0);
template <typename T>
int launch_csr_rows(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials = nullptr,
                    int64_t* npartials = nullptr, bool gather = false);

// Validation helpers for descriptors.
inline bool bad_sizes(int64_t a, int64_t b, int64_t c) { return a < 0 || b < 0 || c < 0; }
inline bool valid_csr_variant(int v) {
  return v == MGB_CSR_SEGMENTS || v == MGB_CSR_ROWS || v == MGB_CSR_SPLIT || v == MGB_CSR_ROWS_GATHER;
}

}  // namespace mgb
