// solver.cu -- the steps either side of SpMV in an iterative solver, fused,
// and a conjugate-gradient driver built from them.
//
// No reference counterpart: Morpheus stops at multiply / dot / waxpby
// (core/src/Morpheus_Multiply.hpp, Morpheus_Dot.hpp, Morpheus_WAXPBY.hpp), and
// a CG written on top of them reads p and Ap again for p.Ap and r again for
// r.r.  Here
//   mgb_spmv_dot_csr_*   y = A*x and x.y in one pass (the SpMV kernel adds
//                        x[i]*y[i] of every finished row to a per-warp
//                        partial; p.Ap of CG),
//   mgb_waxpby_dot_*     w = alpha*x + beta*y and w.w in one pass (r.r),
//   mgb_cg_csr_*         CG with every scalar (alpha, beta, r.r) kept on the
//                        device: five kernels per iteration and no host
//                        synchronisation inside a block of iterations, which
//                        is captured once as a CUDA graph and replayed.
// Partials are summed in a fixed order by one CTA, so results are
// deterministic for a given matrix and kernel choice.
#include <cmath>

#include "primitives.cuh"

namespace mgb {
namespace {

constexpr int FIN_THREADS = 1024;
constexpr int VEC_THREADS = 256;

inline int vec_blocks(int64_t n) { return (int)prim::blocks_for(n, VEC_THREADS, (int64_t)num_sms() * 8); }

// one CTA: the sum of p[0..n) in a fixed order
template <typename T>
__device__ __forceinline__ T block_sum_fixed(const T* __restrict__ p, int64_t n) {
  __shared__ T s[FIN_THREADS / 32];
  T a = T(0);
  for (int64_t i = threadIdx.x; i < n; i += FIN_THREADS) a += p[i];
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
  __syncthreads();
  T t = T(0);
  if (threadIdx.x < 32) {
    t = s[threadIdx.x];
    t = warp_sum(t);
  }
  return t;  // valid in thread 0
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) sum_partials(const T* __restrict__ p, int64_t n, T* out) {
  const T t = block_sum_fixed(p, n);
  if (threadIdx.x == 0) *out = t;
}

// w = alpha*x + beta*y, partials[block] = sum of w^2 over the block's entries
template <typename T>
__global__ void __launch_bounds__(VEC_THREADS) waxpby_dot_kernel(int64_t n, T alpha, const T* __restrict__ x, T beta,
                                                                 const T* __restrict__ y, T* __restrict__ w,
                                                                 T* __restrict__ partials) {
  __shared__ T s[VEC_THREADS / 32];
  T a = T(0);
  for (int64_t i = (int64_t)blockIdx.x * VEC_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * VEC_THREADS) {
    const T v = fmadd(alpha, x[i], beta * y[i]);
    w[i] = v;
    a = fmadd(v, v, a);
  }
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x < 32) {
    T t = threadIdx.x < VEC_THREADS / 32 ? s[threadIdx.x] : T(0);
    t = warp_sum(t);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------- CG state
template <typename T>
struct CgState {
  T rr;      // r.r of the current residual
  T bb;      // b.b
  T tol2;    // (rtol^2) * b.b
  T alpha, beta;
  long long iters;
  long long max_iters;
  int done;  // converged, broke down or reached max_iters: further steps change nothing
  int breakdown;
};

// alpha = rr / pAp (pAp summed from the SpMV partials)
template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) cg_alpha(const T* __restrict__ partials, int64_t n, CgState<T>* st) {
  const T pap = block_sum_fixed(partials, n);
  if (threadIdx.x == 0) {
    if (st->done) {
      st->alpha = T(0);
    } else if (!(pap > T(0))) {  // not SPD along p (or NaN): stop
      st->alpha = T(0);
      st->done = 1;
      st->breakdown = 1;
    } else {
      st->alpha = st->rr / pap;
    }
  }
}

// x += alpha p; r -= alpha Ap; partials[block] = sum r^2
template <typename T>
__global__ void __launch_bounds__(VEC_THREADS) cg_update(int64_t n, const CgState<T>* __restrict__ st,
                                                         const T* __restrict__ p, const T* __restrict__ ap,
                                                         T* __restrict__ x, T* __restrict__ r,
                                                         T* __restrict__ partials) {
  __shared__ T s[VEC_THREADS / 32];
  const T alpha = st->alpha;
  T a = T(0);
  for (int64_t i = (int64_t)blockIdx.x * VEC_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * VEC_THREADS) {
    x[i] = fmadd(alpha, p[i], x[i]);
    const T v = fmadd(-alpha, ap[i], r[i]);
    r[i] = v;
    a = fmadd(v, v, a);
  }
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x < 32) {
    T t = threadIdx.x < VEC_THREADS / 32 ? s[threadIdx.x] : T(0);
    t = warp_sum(t);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
  }
}

// beta = rr_new / rr; convergence and iteration count
template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) cg_beta(const T* __restrict__ partials, int64_t n, CgState<T>* st) {
  const T rr_new = block_sum_fixed(partials, n);
  if (threadIdx.x == 0) {
    if (st->done) {
      st->beta = T(0);
    } else {
      st->beta = rr_new / st->rr;
      st->rr = rr_new;
      st->iters += 1;
      if (rr_new <= st->tol2 || st->iters >= st->max_iters) st->done = 1;
    }
  }
}

// p = r + beta p
template <typename T>
__global__ void __launch_bounds__(VEC_THREADS) cg_direction(int64_t n, const CgState<T>* __restrict__ st,
                                                            const T* __restrict__ r, T* __restrict__ p) {
  const T beta = st->beta;
  if (st->done && beta == T(0) && st->alpha == T(0)) return;  // frozen: p no longer used
  for (int64_t i = (int64_t)blockIdx.x * VEC_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * VEC_THREADS)
    p[i] = fmadd(beta, p[i], r[i]);
}

// r = b - r (r holds A x), p = r, partials[block] = r^2, partials_b[block] = b^2
template <typename T>
__global__ void __launch_bounds__(VEC_THREADS) cg_start(int64_t n, const T* __restrict__ b, T* __restrict__ r,
                                                        T* __restrict__ p, T* __restrict__ partials,
                                                        T* __restrict__ partials_b) {
  __shared__ T s[2][VEC_THREADS / 32];
  T a = T(0), c = T(0);
  for (int64_t i = (int64_t)blockIdx.x * VEC_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * VEC_THREADS) {
    const T bi = b[i];
    const T v = bi - r[i];
    r[i] = v;
    p[i] = v;
    a = fmadd(v, v, a);
    c = fmadd(bi, bi, c);
  }
  a = warp_sum(a);
  c = warp_sum(c);
  if ((threadIdx.x & 31) == 0) {
    s[0][threadIdx.x >> 5] = a;
    s[1][threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    T t = threadIdx.x < VEC_THREADS / 32 ? s[0][threadIdx.x] : T(0);
    T u = threadIdx.x < VEC_THREADS / 32 ? s[1][threadIdx.x] : T(0);
    t = warp_sum(t);
    u = warp_sum(u);
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = t;
      partials_b[blockIdx.x] = u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) cg_init_state(const T* __restrict__ pr, const T* __restrict__ pb,
                                                             int64_t n, T rtol, long long max_iters,
                                                             CgState<T>* st) {
  const T rr = block_sum_fixed(pr, n);
  __syncthreads();
  const T bb = block_sum_fixed(pb, n);
  if (threadIdx.x == 0) {
    st->rr = rr;
    st->bb = bb;
    st->tol2 = rtol * rtol * bb;
    st->alpha = T(0);
    st->beta = T(0);
    st->iters = 0;
    st->max_iters = max_iters;
    st->breakdown = 0;
    st->done = (rr <= st->tol2 || max_iters <= 0) ? 1 : 0;
  }
}

template <typename T>
int check_csr(const mgb_csr* A, int variant) {
  MGB_REQUIRE(A != nullptr && !bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(valid_csr_variant(variant),
              MGB_ERR_BAD_ARGUMENT);
  return MGB_SUCCESS;
}

template <typename T>
int spmv_dot(const mgb_csr* A, const T* x, T* y, int init, int variant, T* dot, void* stream) {
  if (int st = check_csr<T>(A, variant)) return st;
  MGB_REQUIRE(A->nrows <= A->ncols, MGB_ERR_INVALID_INPUT);  // x . y needs x over the rows
  MGB_REQUIRE(dot != nullptr, MGB_ERR_BAD_ARGUMENT);
  const cudaStream_t s = as_stream(stream);
  if (A->nrows == 0) {
    MGB_CUDA_CHECK(cudaMemsetAsync(dot, 0, sizeof(T), s));
    return MGB_SUCCESS;
  }
  int64_t np = 0;
  if (int st = launch_csr_dot<T>(A, x, y, init, stream, variant, nullptr, &np)) return st;
  prim::Scratch sc(s);
  T* part;
  MGB_SCRATCH(sc, part, np);
  if (int st = launch_csr_dot<T>(A, x, y, init, stream, variant, part, &np)) return st;
  sum_partials<T><<<1, FIN_THREADS, 0, s>>>(part, np, dot);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int waxpby_dot(int64_t n, T alpha, const T* x, T beta, const T* y, T* w, T* dot, void* stream) {
  MGB_REQUIRE(n >= 0 && dot != nullptr, MGB_ERR_BAD_ARGUMENT);
  const cudaStream_t s = as_stream(stream);
  if (n == 0) {
    MGB_CUDA_CHECK(cudaMemsetAsync(dot, 0, sizeof(T), s));
    return MGB_SUCCESS;
  }
  MGB_REQUIRE(x && y && w, MGB_ERR_BAD_ARGUMENT);
  const int nb = vec_blocks(n);
  prim::Scratch sc(s);
  T* part;
  MGB_SCRATCH(sc, part, nb);
  waxpby_dot_kernel<T><<<nb, VEC_THREADS, 0, s>>>(n, alpha, x, beta, y, w, part);
  MGB_LAUNCH_CHECK();
  sum_partials<T><<<1, FIN_THREADS, 0, s>>>(part, nb, dot);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

// Iterations per captured graph between host convergence checks.
constexpr int CG_BLOCK = 16;

template <typename T>
int cg_iterations(const mgb_csr* A, int variant, int64_t n, T* x, T* r, T* p, T* ap, T* part_spmv, T* part_vec,
                  int64_t np_spmv, int nb, CgState<T>* st, cudaStream_t s) {
  for (int k = 0; k < CG_BLOCK; k++) {
    if (int e = launch_csr_dot<T>(A, p, ap, 1, s, variant, part_spmv, &np_spmv)) return e;
    cg_alpha<T><<<1, FIN_THREADS, 0, s>>>(part_spmv, np_spmv, st);
    cg_update<T><<<nb, VEC_THREADS, 0, s>>>(n, st, p, ap, x, r, part_vec);
    cg_beta<T><<<1, FIN_THREADS, 0, s>>>(part_vec, nb, st);
    cg_direction<T><<<nb, VEC_THREADS, 0, s>>>(n, st, r, p);
    MGB_LAUNCH_CHECK();
  }
  return MGB_SUCCESS;
}

template <typename T>
int cg(const mgb_csr* A, int variant, const T* b, T* x, int64_t max_iters, double rtol, int64_t* iters,
       double* rel_residual, void* stream) {
  if (int st = check_csr<T>(A, variant)) return st;
  MGB_REQUIRE(A->nrows == A->ncols, MGB_ERR_INVALID_INPUT);
  MGB_REQUIRE(rtol >= 0.0 && max_iters >= 0, MGB_ERR_BAD_ARGUMENT);
  const int64_t n = A->nrows;
  if (iters) *iters = 0;
  if (rel_residual) *rel_residual = 0.0;
  if (n == 0) return MGB_SUCCESS;
  MGB_REQUIRE(b != nullptr && x != nullptr, MGB_ERR_BAD_ARGUMENT);
  const cudaStream_t s = as_stream(stream);
  int64_t np_spmv = 0;
  if (int e = launch_csr_dot<T>(A, x, x, 1, stream, variant, nullptr, &np_spmv)) return e;
  const int nb = vec_blocks(n);
  prim::Scratch sc(s);
  T *r, *p, *ap, *part_spmv, *part_vec, *part_b;
  CgState<T>* st;
  MGB_SCRATCH(sc, r, n);
  MGB_SCRATCH(sc, p, n);
  MGB_SCRATCH(sc, ap, n);
  MGB_SCRATCH(sc, part_spmv, np_spmv);
  MGB_SCRATCH(sc, part_vec, nb);
  MGB_SCRATCH(sc, part_b, nb);
  MGB_SCRATCH(sc, st, 1);
  // r = b - A x, p = r
  if (int e = launch_csr_dot<T>(A, x, r, 1, stream, variant, nullptr, nullptr)) return e;
  cg_start<T><<<nb, VEC_THREADS, 0, s>>>(n, b, r, p, part_vec, part_b);
  cg_init_state<T><<<1, FIN_THREADS, 0, s>>>(part_vec, part_b, nb, (T)rtol, (long long)max_iters, st);
  MGB_LAUNCH_CHECK();

  // one block of CG_BLOCK iterations, captured on a private stream and
  // replayed on the caller's stream until the device state says done
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int status = MGB_SUCCESS;
  cudaError_t ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (ce == cudaSuccess) {
    status = cg_iterations<T>(A, variant, n, x, r, p, ap, part_spmv, part_vec, np_spmv, nb, st, cs);
    cudaError_t ce2 = cudaStreamEndCapture(cs, &graph);
    if (status == MGB_SUCCESS && ce2 != cudaSuccess) ce = ce2;
  }
  if (status == MGB_SUCCESS && ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
  CgState<T> h{};
  if (status == MGB_SUCCESS && ce == cudaSuccess) {
    for (int64_t done = 0; done < max_iters + CG_BLOCK; done += CG_BLOCK) {
      ce = cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
      if (ce != cudaSuccess || h.done) break;
      ce = cudaGraphLaunch(exec, s);
      if (ce != cudaSuccess) break;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  if (status != MGB_SUCCESS) return status;
  if (ce != cudaSuccess) return record_cuda_error(ce);
  if (iters) *iters = (int64_t)h.iters;
  if (rel_residual) *rel_residual = h.bb > T(0) ? std::sqrt((double)h.rr / (double)h.bb) : std::sqrt((double)h.rr);
  if (h.breakdown) return MGB_ERR_RUNTIME;
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_spmv_dot_csr_f64(const mgb_csr* A, const double* x, double* y, int init, int variant, double* dot,
                         void* stream) {
  return mgb::spmv_dot<double>(A, x, y, init, variant, dot, stream);
}
int mgb_spmv_dot_csr_f32(const mgb_csr* A, const float* x, float* y, int init, int variant, float* dot,
                         void* stream) {
  return mgb::spmv_dot<float>(A, x, y, init, variant, dot, stream);
}
int mgb_waxpby_dot_f64(int64_t n, double alpha, const double* x, double beta, const double* y, double* w,
                       double* dot, void* stream) {
  return mgb::waxpby_dot<double>(n, alpha, x, beta, y, w, dot, stream);
}
int mgb_waxpby_dot_f32(int64_t n, float alpha, const float* x, float beta, const float* y, float* w, float* dot,
                       void* stream) {
  return mgb::waxpby_dot<float>(n, alpha, x, beta, y, w, dot, stream);
}
int mgb_cg_csr_f64(const mgb_csr* A, int variant, const double* b, double* x, int64_t max_iters, double rtol,
                   int64_t* iters, double* rel_residual, void* stream) {
  return mgb::cg<double>(A, variant, b, x, max_iters, rtol, iters, rel_residual, stream);
}
int mgb_cg_csr_f32(const mgb_csr* A, int variant, const float* b, float* x, int64_t max_iters, double rtol,
                   int64_t* iters, double* rel_residual, void* stream) {
  return mgb::cg<float>(A, variant, b, x, max_iters, rtol, iters, rel_residual, stream);
}

}  // extern "C"
