// spmv_host.cu -- CSR SpMV on a matrix and vectors that live in HOST memory.
//
// The reference runs multiply on host-space containers with its Serial or
// OpenMP backends (impl/Csr/Serial/Morpheus_Multiply_Impl.hpp:38-58,
// impl/Csr/OpenMP/Morpheus_Multiply_Impl.hpp:37-58); a GPU caller with host
// data would copy the whole matrix, then multiply, then copy y back.  Here the
// copy and the multiply are pipelined: the matrix is cut into nnz-balanced
// row blocks; block b+1 is copied host->device on the caller's stream while
// block b is multiplied on a second stream, and y of each block is copied
// back as soon as it is final.  Transfers then hide the kernel time, and the
// call costs about the transfer time of the bytes at the host link's rate.
//
// Row offsets of each block are rebased on the device so the ordinary CSR
// kernels run unchanged on the block.  Host arrays should be pinned (page-
// locked) for asynchronous copies; the call synchronises the caller's
// stream before it returns, so host buffers may be reused immediately.  The
// device copies live in a caller-provided workspace (keep it across calls:
// no allocation per call) or, without one, in stream-ordered scratch; the
// second stream and its events are created once per thread and device.
#include "primitives.cuh"

namespace mgb {
namespace {

__global__ void rebase_offsets(int32_t* __restrict__ ro, int64_t n, int32_t base) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    ro[i] -= base;
}

// first row r in [0, nrows] with ro[r] >= key
int64_t host_lower_bound(const int32_t* ro, int64_t nrows, int64_t key) {
  int64_t lo = 0, hi = nrows;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((int64_t)ro[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

constexpr int64_t MAX_BLOCKS = 64;

inline int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }

// device workspace: ro (nrows + MAX_BLOCKS) | ci (nnz) | va (nnz) | x (ncols) | y (nrows)
int64_t host_workspace_bytes(const mgb_csr* A, int64_t vbytes) {
  return align256(4 * (A->nrows + MAX_BLOCKS)) + align256(4 * A->nnz) + align256(vbytes * A->nnz) +
         align256(vbytes * A->ncols) + align256(vbytes * A->nrows);
}

// per-thread copy/compute pipeline objects, created once per device
struct HostPipe {
  int dev = -1;
  cudaStream_t k = nullptr;
  cudaEvent_t ev[MAX_BLOCKS + 2] = {};
  void release() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e), e = nullptr;
    if (k) cudaStreamDestroy(k), k = nullptr;
    dev = -1;
  }
  cudaError_t ensure() {
    int d = 0;
    cudaError_t ce = cudaGetDevice(&d);
    if (ce != cudaSuccess) return ce;
    if (d == dev) return cudaSuccess;
    release();
    ce = cudaStreamCreateWithFlags(&k, cudaStreamNonBlocking);
    for (auto& e : ev)
      if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (ce == cudaSuccess) dev = d;
    else release();
    return ce;
  }
  ~HostPipe() { release(); }
};
thread_local HostPipe t_pipe;

template <typename T>
int spmv_csr_host(const mgb_csr* A, const T* xh, T* yh, int init, int variant, int64_t nblocks, void* workspace,
                  int64_t workspace_bytes, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(valid_csr_variant(variant),
              MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz < ((int64_t)1 << 31) - 4096, MGB_ERR_INVALID_INPUT);
  const int64_t N = A->nrows, M = A->ncols, nnz = A->nnz;
  if (N == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr && yh != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(nnz == 0 || (A->column_indices && A->values && xh), MGB_ERR_BAD_ARGUMENT);
  const int32_t* ro_h = A->row_offsets;
  MGB_REQUIRE(ro_h[0] == 0 && (int64_t)ro_h[N] == nnz, MGB_ERR_INVALID_INPUT);
  const int32_t* ci_h = A->column_indices;
  const T* va_h = static_cast<const T*>(A->values);
  // Only the last block's kernel and y copy are not hidden behind the
  // host link, so by default the matrix goes in three blocks of 47 / 47 / 6 %
  // of the nonzeros.  Measured on GB300 with a 405 MB power-law matrix:
  // 1 / 2 / 4 / 8 / 16 equal blocks take 2.20 / 2.17 / 2.18 / 2.26 / 2.33 ms
  // (more, smaller copies cost more); the tapered split: see the design notes.
  // An explicit nblocks gives equal blocks.
  const bool tapered = nblocks <= 0;
  if (tapered) nblocks = 3;
  if (nblocks > N) nblocks = N;
  MGB_REQUIRE(nblocks <= MAX_BLOCKS, MGB_ERR_BAD_ARGUMENT);
  // nnz-balanced row boundaries
  int64_t rb[MAX_BLOCKS + 1];
  rb[0] = 0;
  for (int64_t b = 1; b < nblocks; b++) {
    const int64_t target = (tapered && nblocks == 3) ? (b == 1 ? nnz * 47 / 100 : nnz * 94 / 100) : nnz * b / nblocks;
    int64_t r = host_lower_bound(ro_h, N, target);
    rb[b] = r < rb[b - 1] ? rb[b - 1] : r;
  }
  rb[nblocks] = N;

  const int64_t need = host_workspace_bytes(A, sizeof(T));
  prim::Scratch sc(s);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (ws == nullptr) {
    MGB_SCRATCH(sc, ws, need);
  } else {
    MGB_REQUIRE(workspace_bytes >= need && (reinterpret_cast<uintptr_t>(ws) & 255u) == 0, MGB_ERR_BAD_ARGUMENT);
  }
  int32_t* d_ro = reinterpret_cast<int32_t*>(ws);
  ws += align256(4 * (N + MAX_BLOCKS));
  int32_t* d_ci = nnz > 0 ? reinterpret_cast<int32_t*>(ws) : nullptr;
  ws += align256(4 * nnz);
  T* d_va = nnz > 0 ? reinterpret_cast<T*>(ws) : nullptr;
  ws += align256((int64_t)sizeof(T) * nnz);
  T* d_x = (M > 0 && xh) ? reinterpret_cast<T*>(ws) : nullptr;
  ws += align256((int64_t)sizeof(T) * M);
  T* d_y = reinterpret_cast<T*>(ws);

  int status = MGB_SUCCESS;
  cudaError_t ce = t_pipe.ensure();
  const cudaStream_t k = t_pipe.k;
  cudaEvent_t* ev = t_pipe.ev;
  // ev[0]: x on the device; ev[1 + b]: block b on the device; ev[nblocks + 1]: all done
  if (ce == cudaSuccess && d_x) ce = cudaMemcpyAsync(d_x, xh, sizeof(T) * M, cudaMemcpyHostToDevice, s);
  if (ce == cudaSuccess) ce = cudaEventRecord(ev[0], s);
  if (ce == cudaSuccess) ce = cudaStreamWaitEvent(k, ev[0], 0);
  for (int64_t b = 0; b < nblocks && ce == cudaSuccess && status == MGB_SUCCESS; b++) {
    const int64_t r0 = rb[b], r1 = rb[b + 1], nr = r1 - r0;
    const int64_t e0 = ro_h[r0], e1 = ro_h[r1];
    int32_t* ro_b = d_ro + r0 + b;  // each block keeps its own nr + 1 offsets
    ce = cudaMemcpyAsync(ro_b, ro_h + r0, sizeof(int32_t) * (nr + 1), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && e1 > e0)
      ce = cudaMemcpyAsync(d_ci + e0, ci_h + e0, sizeof(int32_t) * (e1 - e0), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && e1 > e0)
      ce = cudaMemcpyAsync(d_va + e0, va_h + e0, sizeof(T) * (e1 - e0), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && !init && nr > 0)
      ce = cudaMemcpyAsync(d_y + r0, yh + r0, sizeof(T) * nr, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && e0 != 0 && nr > 0) {
      rebase_offsets<<<prim::blocks_for(nr + 1, 256), 256, 0, s>>>(ro_b, nr + 1, (int32_t)e0);
      ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaEventRecord(ev[1 + b], s);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(k, ev[1 + b], 0);
    if (ce == cudaSuccess && nr > 0) {
      const mgb_csr blk{nr, M, e1 - e0, ro_b, d_ci ? d_ci + e0 : nullptr, d_va ? d_va + e0 : nullptr};
      status = launch_csr_dot<T>(&blk, d_x, d_y + r0, init, k, variant, nullptr, nullptr);
      if (status == MGB_SUCCESS)
        ce = cudaMemcpyAsync(yh + r0, d_y + r0, sizeof(T) * nr, cudaMemcpyDeviceToHost, k);
    }
  }
  if (ce == cudaSuccess && status == MGB_SUCCESS) ce = cudaEventRecord(ev[nblocks + 1], k);
  if (ce == cudaSuccess && status == MGB_SUCCESS) ce = cudaStreamWaitEvent(s, ev[nblocks + 1], 0);
  // the caller's stream now orders after every copy and kernel; wait for
  // the host-visible y (and for k, so scratch is released in stream order).
  // Both streams are drained on every path, errors included: copies queued
  // on s read the caller's host buffers, which it may reuse once we return.
  const cudaError_t ce_sync = k ? cudaStreamSynchronize(k) : cudaSuccess;
  const cudaError_t ce_sync_s = cudaStreamSynchronize(s);
  if (status != MGB_SUCCESS) return status;
  if (ce != cudaSuccess) return record_cuda_error(ce);
  if (ce_sync != cudaSuccess) return record_cuda_error(ce_sync);
  if (ce_sync_s != cudaSuccess) return record_cuda_error(ce_sync_s);
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_spmv_csr_host_workspace_bytes(const mgb_csr* A, int value_bytes, int64_t* bytes) {
  if (A == nullptr || bytes == nullptr || (value_bytes != 4 && value_bytes != 8) ||
      mgb::bad_sizes(A->nrows, A->ncols, A->nnz))
    return MGB_ERR_BAD_ARGUMENT;
  *bytes = mgb::host_workspace_bytes(A, value_bytes);
  return MGB_SUCCESS;
}

int mgb_spmv_csr_host_f64(const mgb_csr* A, const double* x, double* y, int init, int variant, int64_t nblocks,
                          void* workspace, int64_t workspace_bytes, void* stream) {
  return mgb::spmv_csr_host<double>(A, x, y, init, variant, nblocks, workspace, workspace_bytes,
                                    mgb::as_stream(stream));
}

int mgb_spmv_csr_host_f32(const mgb_csr* A, const float* x, float* y, int init, int variant, int64_t nblocks,
                          void* workspace, int64_t workspace_bytes, void* stream) {
  return mgb::spmv_csr_host<float>(A, x, y, init, variant, nblocks, workspace, workspace_bytes,
                                   mgb::as_stream(stream));
}

}  // extern "C"
