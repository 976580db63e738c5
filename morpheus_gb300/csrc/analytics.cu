// analytics.cu -- matrix analytics and the format selector's feature vector.
//
// Reference analytics (core/src/Morpheus_MatrixAnalytics.hpp:85-261):
// average_nnnz, density, max/min/std_nnnz, count_nnz_per_row,
// count_nnz_per_diagonal, count_diagonals, count_true_diagonals.  The
// reference computes each with its own pass (and returns std_nnnz as an
// integer, truncating it, :177-193); here one pass over the row offsets and
// one over the column indices produce every statistic, in FP64.
//
// Every format is analysed in place, without a conversion: one pass over
// its arrays gives the row lengths and the diagonal histogram of the entries
// its COO form would hold (what convert-to-COO keeps: every COO / CSR entry,
// DIA slots inside the matrix holding a nonzero value, ELL slots with a
// valid column), so a matrix has the same statistics and selector features
// whichever format is active.
#include <climits>
#include <cmath>

#include "primitives.cuh"

namespace mgb {
namespace {

using prim::blocks_for;
using prim::Scratch;

inline unsigned grid_for(int64_t n) { return blocks_for(n, 256, (int64_t)num_sms() * 16); }

// Row lengths: from CSR row offsets, or from a per-row count array.
struct LensFromOffsets {
  const int32_t* ro;
  __device__ int operator()(int64_t r) const { return ro[r + 1] - ro[r]; }
};
struct LensFromCounts {
  const int32_t* len;
  __device__ int operator()(int64_t r) const { return len[r]; }
};

// row-length moments: sum, sum of squares, max, min, and the entries beyond
// the mean ELL width
template <typename LEN>
__global__ void row_stats_kernel(LEN lens, int64_t nrows, int64_t hyb_w,
                                 unsigned long long* sum, double* sumsq, int* mx, int* mn,
                                 unsigned long long* hyb_excess) {
  unsigned long long s = 0, ex = 0;
  double q = 0.0;
  int a = 0, b = INT_MAX;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int len = lens(r);
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

// per-entry diagonal bin (c - r + nrows - 1)
__global__ void csr_diag_kernel(const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, int64_t nrows,
                                int64_t ncols, int32_t* counts) {
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    for (int32_t j = ro[r]; j < ro[r + 1]; j++) {
      const int64_t c = ci[j];
      if (c < 0 || c >= ncols) continue;
      prim::hist_add(h, counts, (unsigned long long)(c - r + nrows - 1));
    }
  }
  __syncthreads();
  prim::hist_flush(h, counts);
}

// Diagonal summary: occupied diagonals, true diagonals and their entries,
// and the bandwidth max |c - r| over the occupied bins (bin = c - r + nrows - 1).
__global__ void diag_summary_kernel(const int32_t* __restrict__ counts, int64_t nb, int64_t nrows, int32_t min_elem,
                                    unsigned long long* ndiag, unsigned long long* ntrue,
                                    unsigned long long* true_nnz, int* bw) {
  unsigned long long a = 0, b = 0, c = 0;
  int w = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = counts[i];
    a += k > 0;
    if (k > 0) {
      const int64_t d = i - (nrows - 1);
      w = max(w, (int)(d < 0 ? -d : d));
    }
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
    w = max(w, __shfl_xor_sync(0xffffffffu, w, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(ndiag, a);
    atomicAdd(ntrue, b);
    atomicAdd(true_nnz, c);
    atomicMax(bw, w);
  }
}

// ---- COO-form row lengths and diagonal histogram of each format ---------

__global__ void coo_form_coo(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci, int64_t nnz,
                             int64_t nrows, int64_t ncols, int32_t* lens, int32_t* diag) {
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = ri[k], c = ci[k];
    if (r < 0 || r >= nrows || c < 0 || c >= ncols) continue;
    prim::warp_merged_add(lens, r);
    prim::hist_add(h, diag, (unsigned long long)(c - r + nrows - 1));
  }
  __syncthreads();
  prim::hist_flush(h, diag);
}

// CSR entries added to existing lengths (the CSR part of HDC)
__global__ void coo_form_csr(const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, int64_t nrows,
                             int64_t ncols, int32_t* lens, int32_t* diag) {
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t n = 0;
    for (int32_t j = ro[r]; j < ro[r + 1]; j++) {
      const int64_t c = ci[j];
      if (c < 0 || c >= ncols) continue;
      n++;
      prim::hist_add(h, diag, (unsigned long long)(c - r + nrows - 1));
    }
    lens[r] += n;
  }
  __syncthreads();
  prim::hist_flush(h, diag);
}

// DIA: thread per row over the diagonals; per-diagonal counts are summed per
// warp (ballot) and per CTA in shared memory when the CTA's diagonals fit.
constexpr int FORM_DIAG_SMEM = 1024;
template <typename T>
__global__ void coo_form_dia(const int32_t* __restrict__ off, int64_t nd, int64_t pitch, const T* __restrict__ v,
                             int64_t nrows, int64_t ncols, int32_t* lens, int32_t* diag) {
  __shared__ int32_t s_cnt[FORM_DIAG_SMEM];
  const bool in_smem = nd <= FORM_DIAG_SMEM;
  if (in_smem) {
    for (int i = threadIdx.x; i < nd; i += blockDim.x) s_cnt[i] = 0;
    __syncthreads();
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t rows_padded = (nrows + blockDim.x - 1) / blockDim.x * blockDim.x;  // whole warps iterate
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows_padded; r += stride) {
    const bool row_ok = r < nrows;
    int32_t n = 0;
    for (int64_t k = 0; k < nd; k++) {
      const int64_t c = r + __ldg(off + k);
      const bool hit = row_ok && c >= 0 && c < ncols && __ldg(v + r + pitch * k) != T(0);
      n += hit ? 1 : 0;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if ((threadIdx.x & 31) == 0 && m) {
        if (in_smem) atomicAdd(s_cnt + k, __popc(m));
        else atomicAdd(diag + (__ldg(off + k) + nrows - 1), __popc(m));
      }
    }
    if (row_ok) lens[r] += n;
  }
  if (in_smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < nd; i += blockDim.x)
      if (s_cnt[i]) atomicAdd(diag + (__ldg(off + i) + nrows - 1), s_cnt[i]);
  }
}

// ELL: every slot with a valid column (explicit zeros included, as the
// conversion to COO keeps them)
__global__ void coo_form_ell(const int32_t* __restrict__ ci, int64_t width, int64_t pitch, int64_t nrows,
                             int64_t ncols, int32_t* lens, int32_t* diag) {
  MGB_CTA_HIST(h);
  prim::hist_init(h);
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t n = 0;
    for (int64_t k = 0; k < width; k++) {
      const int64_t c = __ldg(ci + r + pitch * k);
      if (c == MGB_INVALID_INDEX || c < 0 || c >= ncols) continue;
      n++;
      prim::hist_add(h, diag, (unsigned long long)(c - r + nrows - 1));
    }
    lens[r] += n;
  }
  __syncthreads();
  prim::hist_flush(h, diag);
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

// The format-specific pass: row lengths (lens, zeroed, unless the format
// has row offsets) and the diagonal histogram (counts, zeroed).
struct FormPass {
  virtual ~FormPass() = default;
  virtual int run(int32_t* lens, int32_t* counts, cudaStream_t s) const = 0;
  virtual const int32_t* row_offsets() const { return nullptr; }  // lengths straight from CSR offsets
};

int analyze_pass(int64_t N, int64_t M, int64_t nnz_meta, const FormPass& pass, double* out, cudaStream_t s) {
  MGB_REQUIRE(out != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(N > 0 && M > 0 && nnz_meta >= 0, MGB_ERR_BAD_ARGUMENT);
  const int64_t nb = N + M - 1;
  const int64_t hyb_w = std::max<int64_t>(1, nnz_meta / N);
  Scratch sc(s);
  unsigned long long* u;
  double* d;
  int* iv;
  int32_t* counts;
  int32_t* lens = nullptr;
  MGB_SCRATCH(sc, u, 5);
  MGB_SCRATCH(sc, d, 1);
  MGB_SCRATCH(sc, iv, 3);
  MGB_SCRATCH(sc, counts, nb);
  const int32_t* ro = pass.row_offsets();
  if (ro == nullptr) {
    MGB_SCRATCH(sc, lens, N);
    MGB_CUDA_CHECK(cudaMemsetAsync(lens, 0, sizeof(int32_t) * N, s));
  }
  init_stats<<<1, 1, 0, s>>>(u, d, iv);
  MGB_LAUNCH_CHECK();
  MGB_CUDA_CHECK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * nb, s));
  if (int st = pass.run(lens, counts, s)) return st;
  if (ro != nullptr)
    row_stats_kernel<<<grid_for(N), 256, 0, s>>>(LensFromOffsets{ro}, N, hyb_w, u, d, iv, iv + 1, u + 4);
  else
    row_stats_kernel<<<grid_for(N), 256, 0, s>>>(LensFromCounts{lens}, N, hyb_w, u, d, iv, iv + 1, u + 4);
  MGB_LAUNCH_CHECK();
  const int32_t min_elem = (int32_t)((double)N * 0.2);  // HdcMatrix::true_diagonal_ratio
  diag_summary_kernel<<<grid_for(nb), 256, 0, s>>>(counts, nb, N, min_elem, u + 1, u + 2, u + 3, iv + 2);
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

// ---- the pass of each format --------------------------------------------

struct CsrPass : FormPass {
  const mgb_csr* A;
  explicit CsrPass(const mgb_csr* a) : A(a) {}
  const int32_t* row_offsets() const override { return A->row_offsets; }
  int run(int32_t*, int32_t* counts, cudaStream_t s) const override {
    if (A->nnz == 0) return MGB_SUCCESS;
    csr_diag_kernel<<<grid_for(A->nrows), 256, 0, s>>>(A->row_offsets, A->column_indices, A->nrows, A->ncols,
                                                       counts);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
};

struct CooPass : FormPass {
  const mgb_coo* A;
  explicit CooPass(const mgb_coo* a) : A(a) {}
  int run(int32_t* lens, int32_t* counts, cudaStream_t s) const override {
    if (A->nnz == 0) return MGB_SUCCESS;
    coo_form_coo<<<grid_for(A->nnz), 256, 0, s>>>(A->row_indices, A->column_indices, A->nnz, A->nrows, A->ncols,
                                                  lens, counts);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
};

template <typename T>
struct DiaPass : FormPass {
  const mgb_dia* A;
  explicit DiaPass(const mgb_dia* a) : A(a) {}
  int run(int32_t* lens, int32_t* counts, cudaStream_t s) const override {
    if (A->ndiags == 0) return MGB_SUCCESS;
    coo_form_dia<T><<<grid_for(A->nrows), 256, 0, s>>>(A->diagonal_offsets, A->ndiags, A->pitch,
                                                       static_cast<const T*>(A->values), A->nrows, A->ncols, lens,
                                                       counts);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
};

struct EllPass : FormPass {
  const mgb_ell* A;
  explicit EllPass(const mgb_ell* a) : A(a) {}
  int run(int32_t* lens, int32_t* counts, cudaStream_t s) const override {
    if (A->width == 0) return MGB_SUCCESS;
    coo_form_ell<<<grid_for(A->nrows), 256, 0, s>>>(A->column_indices, A->width, A->pitch, A->nrows, A->ncols, lens,
                                                    counts);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
};

struct HybPass : FormPass {
  EllPass ell;
  CooPass coo;
  explicit HybPass(const mgb_hyb* a) : ell(&a->ell), coo(&a->coo) {}
  int run(int32_t* lens, int32_t* counts, cudaStream_t s) const override {
    if (int st = ell.run(lens, counts, s)) return st;
    return coo.run(lens, counts, s);
  }
};

template <typename T>
struct HdcPass : FormPass {
  DiaPass<T> dia;
  const mgb_csr* csr;
  explicit HdcPass(const mgb_hdc* a) : dia(&a->dia), csr(&a->csr) {}
  int run(int32_t* lens, int32_t* counts, cudaStream_t s) const override {
    if (int st = dia.run(lens, counts, s)) return st;
    if (csr->nnz == 0) return MGB_SUCCESS;
    coo_form_csr<<<grid_for(csr->nrows), 256, 0, s>>>(csr->row_offsets, csr->column_indices, csr->nrows, csr->ncols,
                                                      lens, counts);
    MGB_LAUNCH_CHECK();
    return MGB_SUCCESS;
  }
};

// Descriptor checks of each format (sizes, pointers the pass reads).
bool csr_ok(const mgb_csr* A) {
  return A && A->nrows > 0 && A->ncols > 0 && A->nnz >= 0 && A->row_offsets && (A->nnz == 0 || A->column_indices);
}
bool coo_ok(const mgb_coo* A) {
  return A && A->nrows > 0 && A->ncols > 0 && A->nnz >= 0 && (A->nnz == 0 || (A->row_indices && A->column_indices));
}
bool dia_ok(const mgb_dia* A) {
  return A && A->nrows > 0 && A->ncols > 0 && A->nnz >= 0 && A->ndiags >= 0 && A->pitch >= A->nrows &&
         (A->ndiags == 0 || (A->diagonal_offsets && A->values));
}
bool ell_ok(const mgb_ell* A) {
  return A && A->nrows > 0 && A->ncols > 0 && A->nnz >= 0 && A->width >= 0 && A->pitch >= A->nrows &&
         (A->width == 0 || A->column_indices);
}
bool hyb_ok(const mgb_hyb* A) {
  return A && ell_ok(&A->ell) && A->coo.nnz >= 0 && A->coo.nrows == A->ell.nrows && A->coo.ncols == A->ell.ncols &&
         (A->coo.nnz == 0 || (A->coo.row_indices && A->coo.column_indices));
}
bool hdc_ok(const mgb_hdc* A) {
  return A && dia_ok(&A->dia) && A->csr.nrows == A->dia.nrows && A->csr.ncols == A->dia.ncols && A->csr.nnz >= 0 &&
         A->csr.row_offsets && (A->csr.nnz == 0 || A->csr.column_indices);
}

int analyze(const mgb_csr* A, double* out, cudaStream_t s) {
  MGB_REQUIRE(csr_ok(A), MGB_ERR_BAD_ARGUMENT);
  return analyze_pass(A->nrows, A->ncols, A->nnz, CsrPass(A), out, s);
}

// Selector features (MGB_FEATURES = 12) from the analytics.
int features_from(const double* a, double N, float* f, uint8_t* feasible) {
  const double nnz = std::max(1.0, a[0] * N);
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

int features(const mgb_csr* A, float* f, uint8_t* feasible, cudaStream_t s) {
  double a[14];
  if (int st = analyze(A, a, s)) return st;
  return features_from(a, (double)A->nrows, f, feasible);
}

// Analytics and features of any format (its COO form, analysed in place).
template <typename Pass, typename D>
int analyze_any(const D* A, int64_t N, int64_t M, int64_t nnz, double* out, cudaStream_t s) {
  return analyze_pass(N, M, nnz, Pass(A), out, s);
}
template <typename Pass, typename D>
int features_any(const D* A, int64_t N, int64_t M, int64_t nnz, float* f, uint8_t* feasible, cudaStream_t s) {
  MGB_REQUIRE(f != nullptr, MGB_ERR_BAD_ARGUMENT);
  double a[14];
  if (int st = analyze_pass(N, M, nnz, Pass(A), a, s)) return st;
  return features_from(a, (double)N, f, feasible);
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

namespace {
// row / column counts and metadata nnz of every descriptor
inline int64_t rows_of(const mgb_coo* A) { return A->nrows; }
inline int64_t rows_of(const mgb_dia* A) { return A->nrows; }
inline int64_t rows_of(const mgb_ell* A) { return A->nrows; }
inline int64_t rows_of(const mgb_hyb* A) { return A->ell.nrows; }
inline int64_t rows_of(const mgb_hdc* A) { return A->dia.nrows; }
inline int64_t cols_of(const mgb_coo* A) { return A->ncols; }
inline int64_t cols_of(const mgb_dia* A) { return A->ncols; }
inline int64_t cols_of(const mgb_ell* A) { return A->ncols; }
inline int64_t cols_of(const mgb_hyb* A) { return A->ell.ncols; }
inline int64_t cols_of(const mgb_hdc* A) { return A->dia.ncols; }
inline int64_t nnz_of(const mgb_coo* A) { return A->nnz; }
inline int64_t nnz_of(const mgb_dia* A) { return A->nnz; }
inline int64_t nnz_of(const mgb_ell* A) { return A->nnz; }
inline int64_t nnz_of(const mgb_hyb* A) { return A->ell.nnz + A->coo.nnz; }
inline int64_t nnz_of(const mgb_hdc* A) { return A->dia.nnz + A->csr.nnz; }

template <typename Pass, typename D>
int analytics_entry(bool ok, const D* A, double* out, void* stream) {
  if (!ok) return MGB_ERR_BAD_ARGUMENT;
  return mgb::analyze_any<Pass>(A, rows_of(A), cols_of(A), nnz_of(A), out, mgb::as_stream(stream));
}
template <typename Pass, typename D>
int features_entry(bool ok, const D* A, float* f, uint8_t* feasible, void* stream) {
  if (!ok) return MGB_ERR_BAD_ARGUMENT;
  return mgb::features_any<Pass>(A, rows_of(A), cols_of(A), nnz_of(A), f, feasible, mgb::as_stream(stream));
}
}  // namespace

extern "C" {

int mgb_analytics_coo(const mgb_coo* A, double* out14, void* stream) {
  return analytics_entry<mgb::CooPass>(mgb::coo_ok(A), A, out14, stream);
}
int mgb_analytics_dia_f64(const mgb_dia* A, double* out14, void* stream) {
  return analytics_entry<mgb::DiaPass<double>>(mgb::dia_ok(A), A, out14, stream);
}
int mgb_analytics_dia_f32(const mgb_dia* A, double* out14, void* stream) {
  return analytics_entry<mgb::DiaPass<float>>(mgb::dia_ok(A), A, out14, stream);
}
int mgb_analytics_ell(const mgb_ell* A, double* out14, void* stream) {
  return analytics_entry<mgb::EllPass>(mgb::ell_ok(A), A, out14, stream);
}
int mgb_analytics_hyb(const mgb_hyb* A, double* out14, void* stream) {
  return analytics_entry<mgb::HybPass>(mgb::hyb_ok(A), A, out14, stream);
}
int mgb_analytics_hdc_f64(const mgb_hdc* A, double* out14, void* stream) {
  return analytics_entry<mgb::HdcPass<double>>(mgb::hdc_ok(A), A, out14, stream);
}
int mgb_analytics_hdc_f32(const mgb_hdc* A, double* out14, void* stream) {
  return analytics_entry<mgb::HdcPass<float>>(mgb::hdc_ok(A), A, out14, stream);
}

int mgb_features_coo(const mgb_coo* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::CooPass>(mgb::coo_ok(A), A, features12, feasible6, stream);
}
int mgb_features_dia_f64(const mgb_dia* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::DiaPass<double>>(mgb::dia_ok(A), A, features12, feasible6, stream);
}
int mgb_features_dia_f32(const mgb_dia* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::DiaPass<float>>(mgb::dia_ok(A), A, features12, feasible6, stream);
}
int mgb_features_ell(const mgb_ell* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::EllPass>(mgb::ell_ok(A), A, features12, feasible6, stream);
}
int mgb_features_hyb(const mgb_hyb* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::HybPass>(mgb::hyb_ok(A), A, features12, feasible6, stream);
}
int mgb_features_hdc_f64(const mgb_hdc* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::HdcPass<double>>(mgb::hdc_ok(A), A, features12, feasible6, stream);
}
int mgb_features_hdc_f32(const mgb_hdc* A, float* features12, uint8_t* feasible6, void* stream) {
  return features_entry<mgb::HdcPass<float>>(mgb::hdc_ok(A), A, features12, feasible6, stream);
}

}  // extern "C"
