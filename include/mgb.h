/*
 * mgb.h -- C ABI of morpheus-gb300, a GB300 (sm_103a) implementation of the
 * Morpheus sparse matrix-vector hot path.
 *
 * Every entry point takes non-owning DEVICE pointers plus sizes and a CUDA
 * stream (NULL = the legacy default stream), returns an mgb_status, never
 * exits and never throws.  SpMV and waxpby are asynchronous on the stream;
 * the scalar-returning dot/reduce synchronise the stream before returning,
 * like the reference's CUDA dot/reduce (which copy the scalar back).
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the Morpheus project root).  The reference is a C++ template library, so
 * "replaces" means: the body of the Cuda-space overload that
 * Morpheus::multiply / convert / dot / reduce / waxpby dispatch to for that
 * container.  The C++ front end in Morpheus_GB300.hpp keeps the reference's
 * template signatures and calls these functions.
 */
#ifndef MGB_H
#define MGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: one per reference exception class
 * (core/src/Morpheus_Exceptions.hpp:32-73) plus CUDA / timeout / argument. */
typedef enum mgb_status {
  MGB_SUCCESS                 = 0,
  MGB_ERR_NOT_IMPLEMENTED     = 1, /* NotImplementedException   */
  MGB_ERR_FORMAT_CONVERSION   = 2, /* FormatConversionException */
  MGB_ERR_INVALID_INPUT       = 3, /* InvalidInputException     */
  MGB_ERR_RUNTIME             = 4, /* RuntimeException          */
  MGB_ERR_IO                  = 5, /* IOException               */
  MGB_ERR_CUDA                = 6, /* a CUDA runtime call failed */
  MGB_ERR_TIMEOUT             = 7, /* a bounded device wait ran out */
  MGB_ERR_BAD_ARGUMENT        = 8, /* null pointer / negative size / bad enum */
  MGB_ERR_ALLOC               = 9  /* device allocation failed  */
} mgb_status;

/* Format enum, same order as Morpheus::formats_e
 * (core/src/Morpheus_FormatsRegistry.hpp:56-64). */
typedef enum mgb_format {
  MGB_COO_FORMAT = 0,
  MGB_CSR_FORMAT = 1,
  MGB_DIA_FORMAT = 2,
  MGB_ELL_FORMAT = 3,
  MGB_HYB_FORMAT = 4,
  MGB_HDC_FORMAT = 5,
  MGB_NFORMATS   = 6
} mgb_format;

/* ELL padding marker (core/src/Morpheus_EllMatrix.hpp:563). */
#define MGB_INVALID_INDEX (-1)

/* ---- container descriptors (device pointers, column-major slabs) -------- */

/* core/src/Morpheus_CooMatrix.hpp: row_indices/column_indices/values[nnz] */
typedef struct mgb_coo {
  int64_t nrows, ncols, nnz;
  int32_t* row_indices;
  int32_t* column_indices;
  void* values; /* double* or float* per the entry point's suffix */
} mgb_coo;

/* core/src/Morpheus_CsrMatrix.hpp:533-537 */
typedef struct mgb_csr {
  int64_t nrows, ncols, nnz;
  int32_t* row_offsets; /* nrows + 1 */
  int32_t* column_indices;
  void* values;
} mgb_csr;

/* core/src/Morpheus_DiaMatrix.hpp:192-201.  values(i, n) is at
 * values[i + pitch * n]; pitch = pad(nrows, 32) (the reference's
 * get_pad_size, core/src/impl/Dia/Morpheus_Utils_Impl.hpp:33-36). */
typedef struct mgb_dia {
  int64_t nrows, ncols, nnz, ndiags, pitch;
  int32_t* diagonal_offsets; /* ndiags, ascending */
  void* values;              /* pitch * ndiags */
} mgb_dia;

/* core/src/Morpheus_EllMatrix.hpp:189-202.  Slot (i, n) is at
 * [i + pitch * n] for n < width; width = pad(entries_per_row, 32);
 * pitch = nrows.  Padding slots hold (MGB_INVALID_INDEX, 0). */
typedef struct mgb_ell {
  int64_t nrows, ncols, nnz, entries_per_row, width, pitch;
  int32_t* column_indices;
  void* values;
} mgb_ell;

/* core/src/Morpheus_HybMatrix.hpp:473-476: ELL part + COO remainder. */
typedef struct mgb_hyb {
  mgb_ell ell;
  mgb_coo coo;
} mgb_hyb;

/* core/src/Morpheus_HdcMatrix.hpp:464-467: DIA part + CSR remainder. */
typedef struct mgb_hdc {
  mgb_dia dia;
  mgb_csr csr;
} mgb_hdc;

/* ---- library ----------------------------------------------------------- */

/* Human-readable name of a status code (static storage). */
const char* mgb_status_string(int status);

/* Library version as major*10000 + minor*100 + patch. */
int mgb_version(void);

/* Text of the last CUDA error seen by this thread (static storage). */
const char* mgb_last_cuda_error_string(void);

/* ---- SpMV: y = A*x (init != 0) or y += A*x (init == 0) ------------------
 * Morpheus::multiply<ExecSpace>(A, x, y[, init])
 * (core/src/Morpheus_Multiply.hpp:57-78).  x has ncols entries, y nrows. */

/* replaces impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:50-157 */
int mgb_spmv_csr_f64(const mgb_csr* A, const double* x, double* y, int init, void* stream);
int mgb_spmv_csr_f32(const mgb_csr* A, const float* x, float* y, int init, void* stream);

/* CSR kernel choice.  The reference runs its thread-per-row kernel only when
 * the user sets MATOPT_SHORT_ROWS (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:59-92);
 * here mgb_csr_choose_kernel measures the row lengths and the columns of a
 * sample of neighbouring rows (one pass, synchronises) and returns
 * MGB_CSR_ROWS for short rows of nearly equal length whose neighbouring rows
 * read neighbouring columns (stencils, banded and mesh matrices: the row-tile
 * kernel, coalesced x reads), MGB_CSR_ROWS_GATHER for short rows of nearly
 * equal length with scattered columns (the row-tile kernel with a smaller
 * shared-memory carve-out, leaving L1 to the x reads), MGB_CSR_SPLIT when some row is
 * longer than 8192 entries or rows average >= 512 (a row is then spread over
 * several warps instead of one: the reference's vector kernel gives a whole
 * row to one vector, impl/Csr/Kernels/Morpheus_Multiply_Impl.hpp), or
 * MGB_CSR_SEGMENTS otherwise (the lane-segment kernel that mgb_spmv_csr_*
 * always uses).  Every kernel gives the Serial result on every structure;
 * the choice is speed only.  Callers cache the choice per matrix. */
#define MGB_CSR_SEGMENTS 1
#define MGB_CSR_ROWS 2
#define MGB_CSR_SPLIT 3 /* fixed nonzero chunks + carries: very long rows */
#define MGB_CSR_ROWS_GATHER 4 /* row tiles, more L1: short rows, scattered columns */
int mgb_csr_choose_kernel(const mgb_csr* A, int* variant, void* stream);
int mgb_spmv_csr_variant_f64(const mgb_csr* A, const double* x, double* y, int init, int variant, void* stream);
int mgb_spmv_csr_variant_f32(const mgb_csr* A, const float* x, float* y, int init, int variant, void* stream);

/* Chunk plan of the lane-segment kernel (MGB_CSR_SEGMENTS).  The reference
 * has no plan: its CSR kernels map rows to threads directly
 * (impl/Csr/Kernels/Morpheus_Multiply_Impl.hpp:36-168).  Each warp of the
 * lane-segment kernel otherwise finds its rows with two searches over
 * row_offsets on every call; the plan stores the first row of every warp
 * chunk, int32 entries = mgb_csr_plan_entries, so that a multiply reads two
 * integers instead.  It depends on nrows, nnz, row_offsets and the GPU it was
 * made on, not on values or x: make it once per matrix structure (one light
 * kernel, asynchronous) and pass it to every planned multiply with that
 * structure.  Same y, bit for bit, as mgb_spmv_csr_variant_* with
 * MGB_CSR_SEGMENTS.  A plan of the wrong size is MGB_ERR_BAD_ARGUMENT; a plan
 * made for another structure of the same size gives wrong sums but reads
 * nothing outside the matrix. */
int mgb_csr_plan_entries(const mgb_csr* A, int64_t* entries);
int mgb_csr_plan(const mgb_csr* A, int32_t* plan, int64_t entries, void* stream);
int mgb_spmv_csr_planned_f64(const mgb_csr* A, const int32_t* plan, int64_t entries, const double* x, double* y,
                             int init, void* stream);
int mgb_spmv_csr_planned_f32(const mgb_csr* A, const int32_t* plan, int64_t entries, const float* x, float* y,
                             int init, void* stream);

/* replaces impl/Coo/Cuda/Morpheus_Multiply_Impl.hpp:50-176.  Like the
 * reference's CUDA path, A must be sorted by row (columns in any order). */
int mgb_spmv_coo_f64(const mgb_coo* A, const double* x, double* y, int init, void* stream);
int mgb_spmv_coo_f32(const mgb_coo* A, const float* x, float* y, int init, void* stream);

/* Allocation-free variant of mgb_spmv_coo_f64; it has no counterpart in the
 * reference.  For callers that may not allocate device memory while they run
 * (real-time loops that forbid allocation once running, hosts that reserve all
 * device memory up front, plugins whose host owns the allocator): the carry
 * buffer is a fixed 4 MiB file-scope device array instead of cudaMallocAsync,
 * and no allocating call is made.  Limits: A->nnz <= 357,892,096, otherwise
 * MGB_ERR_INVALID_INPUT before any work is queued; every GPU that loads the
 * library holds the 4 MiB until exit; the first call on a device looks up the
 * array's address (make it before any stream capture), and so does the first
 * call after the current CUDA context changed (cudaDeviceReset, or another
 * context made current through the driver API); all calls share the
 * array, so calls overlapping on the GPU race -- serialise them.  Same result
 * as mgb_spmv_coo_f64. */
int mgb_spmv_coo_f64_noalloc(const mgb_coo* A, const double* x, double* y, int init, void* stream);

/* replaces impl/Dia/Cuda/Morpheus_Multiply_Impl.hpp:41-85 */
int mgb_spmv_dia_f64(const mgb_dia* A, const double* x, double* y, int init, void* stream);
int mgb_spmv_dia_f32(const mgb_dia* A, const float* x, float* y, int init, void* stream);

/* replaces impl/Ell/Cuda/Morpheus_Multiply_Impl.hpp:41-80 */
int mgb_spmv_ell_f64(const mgb_ell* A, const double* x, double* y, int init, void* stream);
int mgb_spmv_ell_f32(const mgb_ell* A, const float* x, float* y, int init, void* stream);

/* replaces impl/Hyb/Cuda/Morpheus_Multiply_Impl.hpp:42-53 (ELL init, then COO
 * accumulate); the COO part must be sorted by row. */
int mgb_spmv_hyb_f64(const mgb_hyb* A, const double* x, double* y, int init, void* stream);
int mgb_spmv_hyb_f32(const mgb_hyb* A, const float* x, float* y, int init, void* stream);

/* replaces impl/Hdc/Cuda/Morpheus_Multiply_Impl.hpp:42-53 (DIA init, then CSR
 * accumulate), fused into one pass over the rows. */
int mgb_spmv_hdc_f64(const mgb_hdc* A, const double* x, double* y, int init, void* stream);
int mgb_spmv_hdc_f32(const mgb_hdc* A, const float* x, float* y, int init, void* stream);

/* ---- dense vector ops ---------------------------------------------------- */

/* Morpheus::dot<ExecSpace>(n, x, y) (core/src/Morpheus_Dot.hpp:50-58);
 * replaces impl/DenseVector/Cuda/Morpheus_Dot_Impl.hpp:59-144.
 * Writes the scalar to *result (host) and synchronises the stream. */
int mgb_dot_f64(int64_t n, const double* x, const double* y, double* result, void* stream);
int mgb_dot_f32(int64_t n, const float* x, const float* y, float* result, void* stream);

/* Asynchronous dot: the scalar is written to device memory d_result. */
int mgb_dot_f64_async(int64_t n, const double* x, const double* y, double* d_result, void* stream);
int mgb_dot_f32_async(int64_t n, const float* x, const float* y, float* d_result, void* stream);

/* Morpheus::reduce<ExecSpace>(in, size) (core/src/Morpheus_Reduction.hpp:46-52);
 * replaces impl/DenseVector/Cuda/Morpheus_Reduction_Impl.hpp:175-234.  The
 * sum is deterministic for a given size and GPU.  In FP64, vectors of a few
 * million elements or more have 7 of every 16 elements added exactly in
 * 128-bit fixed point on the integer pipe and the rest in FP64 (the FP64
 * add rate of this GPU would otherwise bound the sum below HBM bandwidth);
 * the error is within that of an FP64 tree sum, and Inf / NaN propagate as
 * in the Serial sum.  A sum whose FP64 partial sums would overflow can come
 * out finite when the exact part carries it. */
int mgb_reduce_f64(const double* in, int64_t size, double* result, void* stream);
int mgb_reduce_f32(const float* in, int64_t size, float* result, void* stream);
int mgb_reduce_f64_async(const double* in, int64_t size, double* d_result, void* stream);
int mgb_reduce_f32_async(const float* in, int64_t size, float* d_result, void* stream);

/* Morpheus::waxpby<ExecSpace>(n, alpha, x, beta, y, w): w = alpha*x + beta*y
 * (core/src/Morpheus_WAXPBY.hpp:52-64); replaces
 * impl/DenseVector/Cuda/Morpheus_WAXPBY_Impl.hpp:40-70. */
int mgb_waxpby_f64(int64_t n, double alpha, const double* x, double beta, const double* y, double* w, void* stream);
int mgb_waxpby_f32(int64_t n, float alpha, const float* x, float beta, const float* y, float* w, void* stream);

/* ---- analytics and format selection ---------------------------------------
 * Morpheus analytics (core/src/Morpheus_MatrixAnalytics.hpp:85-261) from one
 * pass over a CSR matrix, written to out14 (host):
 *   [0] average_nnnz  [1] density  [2] max_nnnz  [3] min_nnnz
 *   [4] std_nnnz (FP64; the reference truncates it to an integer)
 *   [5] count_diagonals  [6] count_true_diagonals (>= floor(0.2 N) entries)
 *   [7] entries on true diagonals  [8] bandwidth max|c - r|
 *   [9] entries beyond the mean ELL width (size of a reference HYB's COO part)
 *   [10..13] 1 if DIA / ELL / HYB / HDC pass the reference fill-tolerance test
 * Synchronises the stream. */
int mgb_analytics_csr(const mgb_csr* A, double* out14, void* stream);
/* The same statistics for the other formats, read in place (no conversion):
 * they describe the entries the matrix's COO form would hold -- every COO
 * entry, DIA slots inside the matrix holding a nonzero value, ELL slots with
 * a valid column -- so a matrix gives the same values whichever format is
 * active.  The reference computes its analytics through count_nnz_per_row /
 * count_nnz_per_diagonal of each format (core/src/Morpheus_MatrixAnalytics.hpp:85-261).
 * DIA and HDC read values and come in both value types. */
int mgb_analytics_coo(const mgb_coo* A, double* out14, void* stream);
int mgb_analytics_dia_f64(const mgb_dia* A, double* out14, void* stream);
int mgb_analytics_dia_f32(const mgb_dia* A, double* out14, void* stream);
int mgb_analytics_ell(const mgb_ell* A, double* out14, void* stream);
int mgb_analytics_hyb(const mgb_hyb* A, double* out14, void* stream);
int mgb_analytics_hdc_f64(const mgb_hdc* A, double* out14, void* stream);
int mgb_analytics_hdc_f32(const mgb_hdc* A, double* out14, void* stream);

/* Per-row and per-diagonal nonzero counts into device int32 vectors
 * (count_nnz_per_row / count_nnz_per_diagonal,
 * core/src/Morpheus_MatrixAnalytics.hpp:112-124,206-218): out has nrows
 * entries, resp. nrows + ncols - 1 with diagonal d = column - row at
 * index d + nrows - 1.  init != 0 zeroes out first, else counts are added.
 * Asynchronous. */
int mgb_count_nnz_per_row_csr(const mgb_csr* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_row_coo(const mgb_coo* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_csr(const mgb_csr* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_coo(const mgb_coo* A, int32_t* out, int init, void* stream);
/* The other formats, with the reference's per-format semantics:
 *   DIA per row: diagonal slots whose column lies inside the matrix, values
 *     not inspected (impl/Dia/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:40-72);
 *     per diagonal: slots holding a nonzero value over all pitch rows
 *     (impl/Dia/Kokkos/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:37-78).
 *   ELL per row: slots with a valid column (impl/Ell/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp:40-74);
 *     per diagonal: with k = the row's valid nonzero slots, the valid nonzero
 *     slots among its first k slots
 *     (impl/Ell/Kokkos/Morpheus_NonZeros_Per_Diagonal_Impl.hpp:36-124).
 *   HYB / HDC: the ELL / DIA part (init as given) plus the COO / CSR part
 *     (impl/{Hyb,Hdc}/Serial/Morpheus_NonZeros_Per_{Row,Diagonal}_Impl.hpp). */
int mgb_count_nnz_per_row_dia(const mgb_dia* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_row_ell(const mgb_ell* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_row_hyb(const mgb_hyb* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_row_hdc(const mgb_hdc* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_dia_f64(const mgb_dia* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_dia_f32(const mgb_dia* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_ell_f64(const mgb_ell* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_ell_f32(const mgb_ell* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_hyb_f64(const mgb_hyb* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_hyb_f32(const mgb_hyb* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_hdc_f64(const mgb_hdc* A, int32_t* out, int init, void* stream);
int mgb_count_nnz_per_diagonal_hdc_f32(const mgb_hdc* A, int32_t* out, int init, void* stream);
/* Number of entries of a device int32 vector that are > threshold and != 0
 * (count_nnz, core/src/Morpheus_VectorAnalytics.hpp:124); with the
 * per-diagonal counts it gives count_diagonals (threshold 0) and
 * count_true_diagonals(A, threshold).  Synchronises the stream. */
int mgb_count_nnz_vector(const int32_t* v, int64_t n, int32_t threshold, int64_t* count, void* stream);

/* The format selector's 12 input features (host floats) and the feasibility
 * mask of the six formats (host bytes, may be NULL); no reference counterpart
 * (the reference's format choice is the --morpheus-format flag,
 * impl/Morpheus_Core.cpp:101-125). */
int mgb_features_csr(const mgb_csr* A, float* features12, uint8_t* feasible6, void* stream);
/* The same features of the other formats, computed in place (see
 * mgb_analytics_coo): a matrix gets the same features in every format. */
int mgb_features_coo(const mgb_coo* A, float* features12, uint8_t* feasible6, void* stream);
int mgb_features_dia_f64(const mgb_dia* A, float* features12, uint8_t* feasible6, void* stream);
int mgb_features_dia_f32(const mgb_dia* A, float* features12, uint8_t* feasible6, void* stream);
int mgb_features_ell(const mgb_ell* A, float* features12, uint8_t* feasible6, void* stream);
int mgb_features_hyb(const mgb_hyb* A, float* features12, uint8_t* feasible6, void* stream);
int mgb_features_hdc_f64(const mgb_hdc* A, float* features12, uint8_t* feasible6, void* stream);
int mgb_features_hdc_f32(const mgb_hdc* A, float* features12, uint8_t* feasible6, void* stream);

/* Selector network 12 -> 64 -> 64 -> 6 (ReLU, softmax over feasible formats),
 * FP32 device buffers.  params: mgb_mlp_num_params() floats; mu/sigma: the
 * 12 standardisation constants; X: n x 12; feasible: n x 6 bytes (or NULL).
 * forward writes log-probabilities (n x 6); grad writes the mean gradient of
 * the cross-entropy loss over n samples and the mean loss (device scalar,
 * may be NULL); adam applies one Adam step (step counts from 1). */
int mgb_mlp_num_params(void);
int mgb_mlp_forward_f32(const float* params, const float* mu, const float* sigma, const float* X,
                        const uint8_t* feasible, int64_t n, float* logp, void* stream);
int mgb_mlp_grad_f32(const float* params, const float* mu, const float* sigma, const float* X,
                     const int32_t* labels, const uint8_t* feasible, int64_t n, float* grads, float* loss,
                     void* stream);
int mgb_mlp_adam_f32(float* params, const float* grads, float* m, float* v, int64_t nparams, float lr, float beta1,
                     float beta2, float eps, int step, void* stream);

/* ---- batched CSR SpMV ----------------------------------------------------
 * No counterpart in the reference, whose equivalent is one
 * Morpheus::multiply call per matrix (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:94-157).
 * y_i = A_i * x_i (init) or y_i += A_i * x_i for every item, in one persistent
 * launch: warps take lane-segment chunks of any matrix from an atomic work
 * counter.  Usage: allocate mgb_spmv_batched_csr_workspace_bytes() of device
 * memory, plan once per (batch, config) -- the plan reads the device item
 * array and needs no host synchronisation -- then launch as often as needed.
 * A launch is two memsets (work counter, error flag) plus one kernel, so it
 * can be captured in a CUDA graph.  Workspace word 3 reports the last launch:
 * 0 when it ran, 1 when its config differs from the planned one (it did
 * nothing).  Items must not share y, and each item must have nnz < 2^31 - 4096
 * and nrows < 2^31 - 32 (an item beyond that is skipped by the chunk-queue
 * configs, which set word 3 to 3).  A chunk-queue plan whose chunk total
 * exceeds 2^31 - 1 is recorded for no config (word 3 = 4 after the plan),
 * so every later launch does nothing and sets word 3 to 1. */
typedef struct mgb_csr_batch_item {
  int64_t nrows, ncols, nnz;
  int32_t* row_offsets;
  int32_t* column_indices;
  void* values;
  void* x;
  void* y;
} mgb_csr_batch_item;

int mgb_spmv_batched_csr_num_configs(void);
/* chunk = nonzeros per warp chunk, seg = entries staged per lane per step */
int mgb_spmv_batched_csr_config_info(int config, int64_t* chunk, int* seg);
int mgb_spmv_batched_csr_workspace_bytes(int64_t nitems, int64_t* bytes);
int mgb_spmv_batched_csr_plan(const mgb_csr_batch_item* d_items, int64_t nitems, int config, void* workspace,
                              int64_t workspace_bytes, void* stream);
int mgb_spmv_batched_csr_f64(const mgb_csr_batch_item* d_items, int64_t nitems, int config, void* workspace,
                             int init, void* stream);
int mgb_spmv_batched_csr_f32(const mgb_csr_batch_item* d_items, int64_t nitems, int config, void* workspace,
                             int init, void* stream);
/* Autotuner: plans and times every config (`reps` launches each, CUDA
 * events), writes the fastest to *best_config and the per-config ms to
 * ms_per_config[num_configs] (may be NULL), and leaves the workspace planned
 * for the best.  Overwrites every y. Synchronises the stream. */
int mgb_spmv_batched_csr_autotune_f64(const mgb_csr_batch_item* d_items, int64_t nitems, void* workspace,
                                      int64_t workspace_bytes, int reps, int* best_config, float* ms_per_config,
                                      void* stream);
int mgb_spmv_batched_csr_autotune_f32(const mgb_csr_batch_item* d_items, int64_t nitems, void* workspace,
                                      int64_t workspace_bytes, int reps, int* best_config, float* ms_per_config,
                                      void* stream);

/* ---- format conversion on the device ------------------------------------
 * Morpheus::convert<ExecSpace>(src, dst) (core/src/Morpheus_Convert.hpp:53-57)
 * for every pair through COO (impl/Morpheus_Convert_Impl.hpp:82-104); the
 * reference's CUDA space throws NotImplementedException for all of them
 * (impl/<Fmt>/Cuda/Morpheus_Convert_Impl.hpp), so each entry point below
 * replaces the Serial routine named beside it and returns bit-identical
 * structures (indices, padding, order, tie-breaks).
 *
 * Destinations are caller-allocated: set every size field of *dst and point
 * its arrays at device buffers of those sizes.  Sizes that depend on the data
 * come from the matching *_plan call, which also applies the reference's
 * fill-tolerance test (impl/Morpheus_Utils.hpp:91-105) and returns
 * MGB_ERR_FORMAT_CONVERSION where the reference throws
 * FormatConversionException.  Rows/columns outside the matrix are rejected
 * with MGB_ERR_INVALID_INPUT (the reference indexes out of bounds there).
 * Conversions synchronise the stream (they read sizes back to the host). */

/* impl/Csr/Serial/Morpheus_Convert_Impl.hpp:70-97; dst: nnz entries */
int mgb_convert_csr_to_coo_f64(const mgb_csr* src, mgb_coo* dst, void* stream);
int mgb_convert_csr_to_coo_f32(const mgb_csr* src, mgb_coo* dst, void* stream);
/* impl/Csr/Serial/Morpheus_Convert_Impl.hpp:99-151; dst: nrows+1 offsets, nnz entries */
int mgb_convert_coo_to_csr_f64(const mgb_coo* src, mgb_csr* dst, void* stream);
int mgb_convert_coo_to_csr_f32(const mgb_coo* src, mgb_csr* dst, void* stream);
/* impl/Dia/Serial/Morpheus_Convert_Impl.hpp:72-118; dst: src->nnz entries */
int mgb_convert_dia_to_coo_f64(const mgb_dia* src, mgb_coo* dst, void* stream);
int mgb_convert_dia_to_coo_f32(const mgb_dia* src, mgb_coo* dst, void* stream);
/* impl/Dia/Serial/Morpheus_Convert_Impl.hpp:120-169 */
int mgb_convert_coo_to_dia_plan(const mgb_coo* src, int64_t* ndiags, void* stream);
int mgb_convert_coo_to_dia_f64(const mgb_coo* src, mgb_dia* dst, void* stream);
int mgb_convert_coo_to_dia_f32(const mgb_coo* src, mgb_dia* dst, void* stream);
/* impl/Ell/Serial/Morpheus_Convert_Impl.hpp:68-109 */
int mgb_convert_ell_to_coo_f64(const mgb_ell* src, mgb_coo* dst, void* stream);
int mgb_convert_ell_to_coo_f32(const mgb_ell* src, mgb_coo* dst, void* stream);
/* impl/Ell/Serial/Morpheus_Convert_Impl.hpp:111-173 (width = longest row) */
int mgb_convert_coo_to_ell_plan(const mgb_coo* src, int64_t* entries_per_row, void* stream);
int mgb_convert_coo_to_ell_f64(const mgb_coo* src, mgb_ell* dst, void* stream);
int mgb_convert_coo_to_ell_f32(const mgb_coo* src, mgb_ell* dst, void* stream);
/* impl/Hyb/Serial/Morpheus_Convert_Impl.hpp:62-108 */
int mgb_convert_hyb_to_coo_f64(const mgb_hyb* src, mgb_coo* dst, void* stream);
int mgb_convert_hyb_to_coo_f32(const mgb_hyb* src, mgb_coo* dst, void* stream);
/* impl/Hyb/Serial/Morpheus_Convert_Impl.hpp:110-196.  width = 0 selects the
 * reference rule max(1, nnz / nrows); the fill call reads the width from
 * dst->ell.entries_per_row. */
int mgb_convert_coo_to_hyb_plan(const mgb_coo* src, int64_t width, int64_t* entries_per_row, int64_t* ell_nnz,
                                int64_t* coo_nnz, void* stream);
int mgb_convert_coo_to_hyb_f64(const mgb_coo* src, mgb_hyb* dst, void* stream);
int mgb_convert_coo_to_hyb_f32(const mgb_coo* src, mgb_hyb* dst, void* stream);
/* impl/Hdc/Serial/Morpheus_Convert_Impl.hpp:64-130 */
int mgb_convert_hdc_to_coo_f64(const mgb_hdc* src, mgb_coo* dst, void* stream);
int mgb_convert_hdc_to_coo_f32(const mgb_hdc* src, mgb_coo* dst, void* stream);
/* impl/Hdc/Serial/Morpheus_Convert_Impl.hpp:132-226 (true diagonals hold at
 * least floor(0.2 * nrows) entries) */
int mgb_convert_coo_to_hdc_plan(const mgb_coo* src, int64_t* ndiags, int64_t* dia_nnz, int64_t* csr_nnz,
                                void* stream);
int mgb_convert_coo_to_hdc_f64(const mgb_coo* src, mgb_hdc* dst, void* stream);
int mgb_convert_coo_to_hdc_f32(const mgb_coo* src, mgb_hdc* dst, void* stream);

/* In-place stable sort by (row, column): impl/Coo/Serial/Morpheus_Sort_Impl.hpp:109-164 */
int mgb_coo_sort_by_row_and_column_f64(mgb_coo* A, void* stream);
int mgb_coo_sort_by_row_and_column_f32(mgb_coo* A, void* stream);
/* impl/Coo/Serial/Morpheus_Sort_Impl.hpp:166-186; *sorted = 1 or 0 */
int mgb_coo_is_sorted(const mgb_coo* A, int* sorted, void* stream);

/* ---- CSR SpMV from host memory --------------------------------------------
 * y = A*x (init) or y += A*x where the descriptor's arrays, x and y are HOST
 * pointers (pinned memory for overlap): the matrix is copied in nblocks
 * nnz-balanced row blocks (at most 64; nblocks <= 0: three blocks of 47 / 47 /
 * 6 % of the nonzeros, so that little work is left after the last copy) and
 * block b is multiplied while block b+1 is in flight, y coming back per block.
 * The host-space counterpart of the reference's Serial / OpenMP multiply on
 * host containers (impl/Csr/Serial/Morpheus_Multiply_Impl.hpp:38-58).
 * `variant` as for mgb_spmv_csr_variant_*; `workspace` a device buffer of
 * mgb_spmv_csr_host_workspace_bytes (or NULL).  Synchronises the stream. */
int mgb_spmv_csr_host_f64(const mgb_csr* A, const double* x, double* y, int init, int variant, int64_t nblocks,
                          void* workspace, int64_t workspace_bytes, void* stream);
int mgb_spmv_csr_host_f32(const mgb_csr* A, const float* x, float* y, int init, int variant, int64_t nblocks,
                          void* workspace, int64_t workspace_bytes, void* stream);
/* Device workspace for the host-data SpMV (256-byte aligned; NULL workspace:
 * the call takes stream-ordered scratch instead).  value_bytes 8 or 4. */
int mgb_spmv_csr_host_workspace_bytes(const mgb_csr* A, int value_bytes, int64_t* bytes);

/* ---- fused solver steps (no reference counterpart) -----------------------
 * The steps either side of SpMV in an iterative solver, fused into the pass
 * that produces their input; a CG written on the reference's multiply / dot /
 * waxpby (core/src/Morpheus_{Multiply,Dot,WAXPBY}.hpp) reads those vectors
 * again.  Results are deterministic (fixed-order partial sums).
 *
 * y = A*x (init) or y += A*x, and *dot = x[0..nrows) . y, with the CSR kernel
 * `variant` (mgb_csr_choose_kernel); dot is a DEVICE pointer; needs
 * nrows <= ncols.  Asynchronous. */
int mgb_spmv_dot_csr_f64(const mgb_csr* A, const double* x, double* y, int init, int variant, double* dot,
                         void* stream);
int mgb_spmv_dot_csr_f32(const mgb_csr* A, const float* x, float* y, int init, int variant, float* dot,
                         void* stream);
/* w = alpha*x + beta*y and *dot = w . w (device pointer).  Asynchronous. */
int mgb_waxpby_dot_f64(int64_t n, double alpha, const double* x, double beta, const double* y, double* w,
                       double* dot, void* stream);
int mgb_waxpby_dot_f32(int64_t n, float alpha, const float* x, float beta, const float* y, float* w, float* dot,
                       void* stream);
/* Conjugate gradients for a symmetric positive definite CSR matrix: x (device,
 * initial guess in, solution out) until ||r|| <= rtol * ||b|| or max_iters
 * iterations.  alpha, beta and r.r stay on the device (five kernels per
 * iteration: SpMV + p.Ap, alpha, x/r update + r.r, beta, p update), blocks
 * of 16 iterations are one CUDA graph, and the host reads the state once per
 * block.  *iters and *rel_residual (= sqrt(r.r / b.b) of the recurrence)
 * are host pointers (may be NULL).  MGB_ERR_RUNTIME if p.Ap <= 0 (the matrix
 * is not SPD).  Synchronises the stream. */
int mgb_cg_csr_f64(const mgb_csr* A, int variant, const double* b, double* x, int64_t max_iters, double rtol,
                   int64_t* iters, double* rel_residual, void* stream);
int mgb_cg_csr_f32(const mgb_csr* A, int variant, const float* b, float* x, int64_t max_iters, double rtol,
                   int64_t* iters, double* rel_residual, void* stream);

/* ---- measurement (no reference counterpart) --------------------------------
 * Ceilings of the SpMV kernels' non-HBM binding units on the current GPU,
 * for roofline reports; the caller times the launch (CUDA events on the same
 * stream).  Blocks of mgb_peak_threads_per_block() threads; `out` receives
 * one double per thread (blocks * threads entries; keeps the work live).
 *
 * FP64 FMA throughput: every thread runs iters x 8 independent fma chains,
 * so one launch performs blocks * threads * iters * 8 FMA lane-operations. */
int mgb_peak_dfma_f64(int64_t blocks, int64_t iters, double* out, void* stream);
/* Random 8-byte gathers from table[table_len] (table_len a power of two; a
 * table that fits in L2 measures the L2 -> SM sector path the x reads of
 * scattered SpMV take): blocks * threads * steps * 8 gathers per launch. */
int mgb_peak_gather_f64(const double* table, int64_t table_len, int64_t blocks, int64_t steps, double* out,
                        void* stream);
int mgb_peak_threads_per_block(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* MGB_H */
