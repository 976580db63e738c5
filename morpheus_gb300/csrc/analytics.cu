// analytics.cu -- matrix analytics and the format selector's feature vector.
//
// Reference analytics (core/src/Morpheus_MatrixAnalytics.hpp:85-261):
// average_nnnz, density, max/min/std_nnnz, count_nnz_per_row,
// count_nnz_per_diagonal, count_diagonals, count_true_diagonals.  The
// reference computes each with its own pass (and returns std_nnnz as an
// integer, truncating it, :177-193); here one pass over the row offsets and
// one over the column indices produce every statistic, in FP64.
#include <climits>
#include <cmath>

#include "primitives.cuh"

namespace mgb {
namespace {

using prim::blocks_for;
using prim::Scratch;

inline unsigned grid_for(int64_t n) { return blocks_for(n, 256, (int64_t)num_sms() * 16); }

// row-length moments: sum, sum of squares, max, min
struct RowStats {
  unsigned long long sum;
  double sumsq;
  int max;
  int min;
};

__global__ void row_stats_kernel(const int32_t* __restrict__ ro, int64_t nrows, int64_t hyb_w,
                                 unsigned long long* sum, double* sumsq, int* mx, int* mn,
                                 unsigned long long* hyb_excess) {
  unsigned long long s = 0, ex = 0;
  double q = 0.0;
  int a = 0, b = INT_MAX;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int len = ro[r + 1] - ro[r];
    s += (unsigned long long)len;
    q += (double)len * (double)len;
    a = max(a, len);
    b = min(b, len);
    if (len > hyb_w) ex += (unsigned long long)(len - hyb_w);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    ex += __shfl_xor_sync(0xffffffffu, ex, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
    a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sum, s);
    atomicAdd(hyb_excess, ex);
    atomicAdd(sumsq, q);
    atomicMax(mx, a);
    atomicMin(mn, b);
  }
}

// per-entry diagonal bin (c - r + nrows - 1) and max |c - r|
__global__ void csr_diag_kernel(const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, int64_t nrows,
                                int64_t ncols, int32_t* counts, int* bw) {
  int local = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    for (int32_t j = ro[r]; j < ro[r + 1]; j++) {
      const int64_t c = ci[j];
      if (c < 0 || c >= ncols) continue;
      const int64_t d = c - r;
      atomicAdd(counts + (d + nrows - 1), 1);
      local = max(local, (int)(d < 0 ? -d : d));
    }
  }
  local = __reduce_max_sync(0xffffffffu, local);
  if ((threadIdx.x & 31) == 0) atomicMax(bw, local);
}

__global__ void diag_summary_kernel(const int32_t* __restrict__ counts, int64_t nb, int32_t min_elem,
                                    unsigned long long* ndiag, unsigned long long* ntrue,
                                    unsigned long long* true_nnz) {
  unsigned long long a = 0, b = 0, c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = counts[i];
    a += k > 0;
    if (k >= min_elem && k > 0) {
      b += 1;
      c += (unsigned long long)k;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(ndiag, a);
    atomicAdd(ntrue, b);
    atomicAdd(true_nnz, c);
  }
}

__global__ void init_stats(unsigned long long* u, double* d, int* i) {
  u[0] = 0; u[1] = 0; u[2] = 0; u[3] = 0; u[4] = 0;
  d[0] = 0.0;
  i[0] = 0;        // max len
  i[1] = INT_MAX;  // min len
  i[2] = 0;        // bandwidth
}

bool exceeds_tolerance(double num_rows, double num_entries, double num_columns) {
  const float size = float(num_columns) * float(num_rows);  // impl/Morpheus_Utils.hpp:91-105
  const float fill = size / std::max(1.0f, float(num_entries));
  return fill > 10.0f && size > 100e6f;
}

int analyze(const mgb_csr* A, double* out, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && out != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nrows > 0 && A->ncols > 0 && A->nnz >= 0 && A->row_offsets, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz == 0 || A->column_indices, MGB_ERR_BAD_ARGUMENT);
  const int64_t N = A->nrows, M = A->ncols, nb = N + M - 1;
  const int64_t hyb_w = std::max<int64_t>(1, A->nnz / N);
  Scratch sc(s);
  unsigned long long* u;
  double* d;
  int* iv;
  int32_t* counts;
  MGB_SCRATCH(sc, u, 5);
  MGB_SCRATCH(sc, d, 1);
  MGB_SCRATCH(sc, iv, 3);
  MGB_SCRATCH(sc, counts, nb);
  init_stats<<<1, 1, 0, s>>>(u, d, iv);
  MGB_LAUNCH_CHECK();
  MGB_CUDA_CHECK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * nb, s));
  row_stats_kernel<<<grid_for(N), 256, 0, s>>>(A->row_offsets, N, hyb_w, u, d, iv, iv + 1, u + 4);
  MGB_LAUNCH_CHECK();
  if (A->nnz > 0) {
    csr_diag_kernel<<<grid_for(N), 256, 0, s>>>(A->row_offsets, A->column_indices, N, M, counts, iv + 2);
    MGB_LAUNCH_CHECK();
  }
  const int32_t min_elem = (int32_t)((double)N * 0.2);  // HdcMatrix::true_diagonal_ratio
  diag_summary_kernel<<<grid_for(nb), 256, 0, s>>>(counts, nb, min_elem, u + 1, u + 2, u + 3);
  MGB_LAUNCH_CHECK();
  unsigned long long hu[5];
  double hd;
  int hi[3];
  MGB_CUDA_CHECK(cudaMemcpyAsync(hu, u, sizeof(hu), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaMemcpyAsync(&hd, d, sizeof(hd), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaMemcpyAsync(hi, iv, sizeof(hi), cudaMemcpyDeviceToHost, s));
  MGB_CUDA_CHECK(cudaStreamSynchronize(s));
  const double nnz = (double)hu[0];
  const double mean = nnz / (double)N;
  const double var = std::max(0.0, hd / (double)N - mean * mean);
  const double ndiag = (double)hu[1];
  // analytics (MGB_ANALYTICS_* indices in mgb.h)
  out[0] = mean;                         // average_nnnz
  out[1] = nnz / ((double)N * (double)M);  // density
  out[2] = (double)hi[0];                // max_nnnz
  out[3] = (double)hi[1];                // min_nnnz
  out[4] = std::sqrt(var);               // std_nnnz (not truncated)
  out[5] = ndiag;                        // count_diagonals
  out[6] = (double)hu[2];                // count_true_diagonals (>= floor(0.2 N) entries)
  out[7] = (double)hu[3];                // entries on true diagonals
  out[8] = (double)hi[2];                // bandwidth max |c - r|
  out[9] = (double)hu[4];                // entries beyond the mean ELL width (HYB COO part)
  // feasibility under the reference's fill-tolerance rule
  out[10] = exceeds_tolerance((double)N, nnz, ndiag) ? 0.0 : 1.0;                      // DIA
  out[11] = exceeds_tolerance((double)N, nnz, (double)hi[0]) ? 0.0 : 1.0;              // ELL
  const double hyb_ell = nnz - (double)hu[4];
  out[12] = exceeds_tolerance((double)N, hyb_ell, (double)hyb_w) ? 0.0 : 1.0;          // HYB
  out[13] = exceeds_tolerance((double)N, (double)hu[3], (double)hu[2]) ? 0.0 : 1.0;    // HDC
  return MGB_SUCCESS;
}

// Selector features (MGB_FEATURES = 12) from the analytics.
int features(const mgb_csr* A, float* f, uint8_t* feasible, cudaStream_t s) {
  double a[14];
  int st = analyze(A, a, s);
  if (st) return st;
  const double N = (double)A->nrows, nnz = std::max(1.0, a[0] * N);
  const double mean = a[0];
  auto l2 = [](double v) { return std::log2(std::max(1.0, v)); };
  f[0] = (float)l2(N);
  f[1] = (float)l2(nnz);
  f[2] = (float)mean;
  f[3] = (float)(a[4] / std::max(mean, 1e-9));        // coefficient of variation of row lengths
  f[4] = (float)l2(a[2]);                              // longest row
  f[5] = (float)a[3];                                  // shortest row
  f[6] = (float)l2(a[5]);                              // occupied diagonals
  f[7] = (float)l2(a[5] * N / nnz);                    // DIA fill ratio
  f[8] = (float)(a[7] / nnz);                          // share of entries on true diagonals
  f[9] = (float)l2(a[2] * N / nnz);                    // ELL fill ratio
  f[10] = (float)(a[9] / nnz);                         // HYB COO share
  f[11] = (float)(a[8] / std::max(1.0, N));            // relative bandwidth
  if (feasible) {
    feasible[0] = 1;                  // COO
    feasible[1] = 1;                  // CSR
    feasible[2] = a[10] > 0.5;        // DIA
    feasible[3] = a[11] > 0.5;        // ELL
    feasible[4] = a[12] > 0.5;        // HYB
    feasible[5] = a[13] > 0.5;        // HDC
  }
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_analytics_csr(const mgb_csr* A, double* out14, void* stream) {
  return mgb::analyze(A, out14, mgb::as_stream(stream));
}

int mgb_features_csr(const mgb_csr* A, float* features12, uint8_t* feasible6, void* stream) {
  MGB_REQUIRE(features12 != nullptr, MGB_ERR_BAD_ARGUMENT);
  return mgb::features(A, features12, feasible6, mgb::as_stream(stream));
}

}  // extern "C"
