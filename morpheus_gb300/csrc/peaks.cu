// peaks.cu -- measurement kernels for the ceilings of the SpMV kernels' two
// non-HBM binding units on this GPU.  They have no counterpart in the
// reference; bench.py times them with CUDA events in the same run as the
// SpMV kernels, so every roofline names a ceiling measured on the same GPU
// and clock.
//
//  * FP64 FMA issue rate.  SpMV performs one FMA per stored entry; on this
//    part the FP64 pipe, not HBM, bounds the DIA and stencil CSR kernels.
//    Every lane of every warp runs 8 independent FMA chains, so the count
//    of FMA lane-operations per second is the pipe's throughput.
//  * Random 8-byte gathers from an L2-resident table.  CSR / COO SpMV on a
//    matrix with scattered columns reads one x entry per stored entry, each
//    in its own 32-byte sector; the L1TEX sector rate bounds those kernels.
//    Each thread hashes (thread, step) to a table index (a 32-bit
//    multiply-xorshift mix) and keeps 8 gathers in flight.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int PEAK_THREADS = 256;

__global__ void __launch_bounds__(PEAK_THREADS) peak_dfma(int64_t iters, double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double m = 1.0 - 1.0 / 1048576.0, c = 1.0 / 4096.0;
  double a0 = 1.0 + threadIdx.x, a1 = a0 + 0.5, a2 = a0 + 0.25, a3 = a0 + 0.125;
  double a4 = a0 - 0.5, a5 = a0 - 0.25, a6 = a0 - 0.125, a7 = a0 + 0.0625;
  for (int64_t i = 0; i < iters; i++) {
    a0 = fma(a0, m, c);
    a1 = fma(a1, m, c);
    a2 = fma(a2, m, c);
    a3 = fma(a3, m, c);
    a4 = fma(a4, m, c);
    a5 = fma(a5, m, c);
    a6 = fma(a6, m, c);
    a7 = fma(a7, m, c);
  }
  out[t] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}

__device__ __forceinline__ uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}

__global__ void __launch_bounds__(PEAK_THREADS) peak_gather(const double* __restrict__ table, uint32_t mask,
                                                            int64_t steps, double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t h = mix32((uint32_t)t * 2654435761u + 0x9e3779b9u);
  double s = 0.0;
  for (int64_t i = 0; i < steps; i++) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      h = mix32(h + (uint32_t)k);
      v[k] = __ldg(table + (h & mask));
    }
    s += ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
  }
  out[t] = s;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_peak_dfma_f64(int64_t blocks, int64_t iters, double* out, void* stream) {
  if (blocks <= 0 || blocks > 0x7fffffffLL || iters <= 0 || out == nullptr) return MGB_ERR_BAD_ARGUMENT;
  mgb::peak_dfma<<<(unsigned)blocks, mgb::PEAK_THREADS, 0, mgb::as_stream(stream)>>>(iters, out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int mgb_peak_gather_f64(const double* table, int64_t table_len, int64_t blocks, int64_t steps, double* out,
                        void* stream) {
  if (table == nullptr || out == nullptr || blocks <= 0 || blocks > 0x7fffffffLL || steps <= 0)
    return MGB_ERR_BAD_ARGUMENT;
  if (table_len <= 0 || table_len > ((int64_t)1 << 32) || (table_len & (table_len - 1)) != 0)
    return MGB_ERR_BAD_ARGUMENT;  // a power of two, so the index is a mask
  mgb::peak_gather<<<(unsigned)blocks, mgb::PEAK_THREADS, 0, mgb::as_stream(stream)>>>(
      table, (uint32_t)(table_len - 1), steps, out);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int mgb_peak_threads_per_block(void) { return mgb::PEAK_THREADS; }

}  // extern "C"
