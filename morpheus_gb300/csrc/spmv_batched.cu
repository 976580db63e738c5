// spmv_batched.cu -- many independent CSR SpMVs in one persistent launch.
//
// No counterpart in the reference: its baseline is one Morpheus::multiply
// call (one kernel launch, plus a device-property query) per matrix
// (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:94-157).
//
// Layout: a device array of mgb_csr_batch_item descriptors (matrix arrays, x,
// y).  A plan kernel splits every matrix into lane-segment warp chunks
// (nnz / CHUNK + 1 each, the same chunking as spmv_csr.cu) and writes the
// chunk prefix over the batch into the workspace.  The batched kernel is
// persistent (a few CTAs per SM): each warp takes the next chunk from an
// atomic work counter, finds its matrix by binary search in the prefix and
// runs csr::csr_chunk on it.  Warps never wait on each other, so there is no
// spin-wait to bound; the counter is reset by a memset before each launch, so
// memset + kernel capture into a CUDA graph.
//
// Tunables (CHUNK nonzeros per warp = 32 x lane range, SEG = entries staged
// per lane per step, the "vector width" of the staging loads) form six
// chunk-queue configurations.  Two more configurations give each CTA a whole
// matrix at a time (largest first): the CTA copies the matrix's x into
// shared memory (up to 64 KB) with cp.async and its warps split the matrix
// into nnz-balanced chunks, so the random x reads become shared-memory reads
// instead of one L1TEX sector per nonzero (the unit that binds the
// chunk-queue kernel); with two buffers the next matrix's x is copied while
// the CTA works on the current one.  Two last configurations also give each
// CTA a whole matrix but read x through L1.  mgb_spmv_batched_csr_autotune_*
// times every configuration on the actual batch with CUDA events and returns
// the fastest.
#include <atomic>

#include "csr_chunk.cuh"
#include "primitives.cuh"

namespace mgb {
namespace {

constexpr int BAT_WARPS = 8;
constexpr int BAT_NCONFIGS = 11;
constexpr int BAT_FIRST_XS = 6;  // configurations >= 6 are matrix per CTA (largest first)
// configurations 6, 7 and 10 keep x in shared memory, 8 and 9 read it through L1
constexpr bool bat_is_xl1(int c) { return c == 8 || c == 9; }
// chunk-queue configs: nonzeros per chunk; matrix-per-CTA configs: 0 (each
// matrix is cut into WARPS x BAT_XS_CPW chunks of at least 256 nonzeros)
constexpr int64_t BAT_CHUNK[BAT_NCONFIGS] = {512, 1024, 2048, 4096, 1024, 2048, 0, 0, 0, 0, 0};
constexpr int BAT_SEG[BAT_NCONFIGS] = {8, 8, 8, 8, 4, 4, 8, 8, 8, 8, 8};
constexpr int BAT_XS_CPW[BAT_NCONFIGS] = {0, 0, 0, 0, 0, 0, 1, 2, 1, 2, 2};  // chunks per warp
// x-in-shared-memory configs: x buffers and warps per CTA (6: two CTAs of 8
// warps per SM; 7: one CTA of 16 warps, the next matrix's x copied during
// this one; 10: one CTA of 24 warps, 32-bit chunk indices)
constexpr int bat_xs_nbuf(int c) { return c == 7 ? 2 : 1; }
constexpr int bat_xs_warps(int c) { return c == 6 ? 8 : (c == 7 ? 16 : 24); }
constexpr int bat_xs_ctas(int c) { return bat_xs_warps(c) >= 16 ? 1 : 16 / bat_xs_warps(c); }
constexpr int BAT_XS_BYTES = 64 * 1024;  // per x buffer (larger x: read from global)
// workspace: int32 header[4] = {work counter, total work items, planned
// config, error flag}, then int32[nitems + 1]: the chunk prefix (chunk-queue
// configs) or the matrix order, largest nnz first (matrix-per-CTA configs)
constexpr int BAT_HEADER = 4;

__global__ void batch_chunk_counts(const mgb_csr_batch_item* __restrict__ items, int64_t n, int64_t chunk,
                                   int32_t* counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    counts[i] = (int32_t)(items[i].nnz / chunk + 1);
}

// A chunk total beyond int32 cannot be indexed by the chunk queue: the plan
// is then recorded for no configuration (-1), so every launch sets the error
// flag and does nothing.
__global__ void batch_finish_plan(int32_t* ws, const int64_t* total, int config) {
  const bool fits = *total <= (int64_t)0x7fffffff;
  ws[0] = 0;
  ws[1] = fits ? (int32_t)*total : 0;
  ws[2] = fits ? config : -1;
  ws[3] = fits ? 0 : 4;
}

template <typename T, int CFG>
__global__ void __launch_bounds__(BAT_WARPS * 32, 3)
spmv_batched_csr(const mgb_csr_batch_item* __restrict__ items, int64_t nitems, int32_t* ws, int init) {
  constexpr int64_t CHUNK = BAT_CHUNK[CFG];
  constexpr int SEG = BAT_SEG[CFG];
  __shared__ csr::WarpStage<T, SEG> stage[BAT_WARPS];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  if (ws[2] != CFG) {  // planned for another configuration
    if (threadIdx.x == 0) ws[3] = 1;
    return;
  }
  const int32_t total = ws[1];
  const int32_t* __restrict__ prefix = ws + BAT_HEADER;
  while (true) {
    int g = 0;
    if (lane == 0) g = atomicAdd(ws, 1);
    g = __shfl_sync(0xffffffffu, g, 0);
    if (g >= total) break;
    // matrix owning chunk g: last i with prefix[i] <= g (a 32-ary search:
    // the first i with prefix[i] > g, minus one; prefix[nitems] = total > g)
    int64_t lo = csr::warp_lower_bound(prefix, 0, nitems, (int64_t)g + 1, lane) - 1;
    lo = lo < 0 ? 0 : lo;
    const mgb_csr_batch_item it = items[lo];
    if (it.nnz >= ((int64_t)1 << 31) - 4096 || it.nrows >= ((int64_t)1 << 31) - 32) {  // beyond 32-bit indices
      if (lane == 0) ws[3] = 3;
      continue;
    }
    csr::csr_chunk<T, CHUNK, SEG>(g - __ldg(prefix + lo), it.nrows, it.ncols, it.row_offsets, it.column_indices,
                                  static_cast<const T*>(it.values), static_cast<const T*>(it.x),
                                  static_cast<T*>(it.y), init, stage[w], lane);
  }
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Starts the copy of x[0, n) into shared memory at xs with cp.async (no
// registers held, every copy of the CTA in flight at once): 16-byte pieces
// when x is 16-byte aligned, otherwise one element per copy.
template <typename T>
__device__ __forceinline__ void copy_x_async(T* xs, const T* __restrict__ xg, int64_t n) {
  int64_t done = 0;
  if ((reinterpret_cast<uintptr_t>(xg) & 15u) == 0) {
    constexpr int64_t V = 16 / sizeof(T);
    const int64_t nv = n / V;
    for (int64_t i = threadIdx.x; i < nv; i += blockDim.x)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(xs + i * V)), "l"(xg + i * V)
                   : "memory");
    done = nv * V;
  }
  for (int64_t i = done + threadIdx.x; i < n; i += blockDim.x)
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(smem_u32(xs + i)), "l"(xg + i),
                 "n"((int)sizeof(T))
                 : "memory");
}

// One CTA per matrix at a time, x in shared memory (configs 6, 7, 10).
// Each CTA takes the next matrix (largest first), copies its x (up to
// BAT_XS_BYTES) into shared memory with cp.async, and its warps split the
// matrix into nnz-balanced chunks whose random x reads are shared-memory
// reads.  With NBUF = 2 the copy of the next matrix's x is in flight while
// the CTA works on the current one (one CTA of 16 warps per SM); with NBUF =
// 1 and 8 warps two CTAs share an SM, and one computes while the other
// copies; with 24 warps one CTA holds as many warps as the chunk queue (its
// chunks then use 32-bit indices and skip items beyond them, as the chunk
// queue does).  A wider x is read from global memory.  No thread waits on
// another CTA, so there is no spin-wait.
template <typename T, int CFG, int NBUF, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, bat_xs_ctas(CFG))
spmv_batched_csr_xs(const mgb_csr_batch_item* __restrict__ items, int64_t nitems, int32_t* ws, int init) {
  constexpr bool I32 = WARPS >= 24;  // 32-bit chunk routine (register budget of 768 threads)
  constexpr int SEG = BAT_SEG[CFG];
  constexpr int64_t CPW = BAT_XS_CPW[CFG];
  constexpr int64_t XCAP = BAT_XS_BYTES / sizeof(T);  // entries per x buffer
  extern __shared__ __align__(16) unsigned char bat_smem[];
  csr::WarpStage<T, SEG>* stage = reinterpret_cast<csr::WarpStage<T, SEG>*>(bat_smem + NBUF * BAT_XS_BYTES);
  __shared__ int s_q[2];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  if (ws[2] != CFG) {
    if (threadIdx.x == 0) ws[3] = 1;
    return;
  }
  const int32_t* __restrict__ order = ws + BAT_HEADER;
  // takes the next matrix into slot b and starts the copy of its x into
  // buffer b (one cp.async group per call, possibly empty)
  auto fetch = [&](int b) {
    if (threadIdx.x == 0) s_q[b] = atomicAdd(ws, 1);
    __syncthreads();
    const int q = s_q[b];
    if (q < nitems) {
      const mgb_csr_batch_item& it = items[__ldg(order + q)];
      if (it.ncols <= XCAP)
        copy_x_async(reinterpret_cast<T*>(bat_smem + b * BAT_XS_BYTES), static_cast<const T*>(it.x), it.ncols);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  int cur = 0;
  fetch(0);
  while (true) {
    const int q = s_q[cur];
    if (q >= nitems) break;
    if constexpr (NBUF == 2) {
      fetch(cur ^ 1);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();  // x of matrix q is in shared memory
    const mgb_csr_batch_item it = items[__ldg(order + q)];
    const T* xs = reinterpret_cast<const T*>(bat_smem + cur * BAT_XS_BYTES);
    const T* xg = static_cast<const T*>(it.x);
    const bool xin = it.ncols <= XCAP;
    int64_t chunk = (it.nnz + WARPS * CPW - 1) / (WARPS * CPW);
    chunk = chunk < 256 ? 256 : (chunk > 4096 ? 4096 : chunk);
    const int64_t nch = it.nnz / chunk + 1;
    const T* va = static_cast<const T*>(it.values);
    T* y = static_cast<T*>(it.y);
    const bool too_big = it.nnz >= ((int64_t)1 << 31) - 4096 || it.nrows >= ((int64_t)1 << 31) - 32;
    if (I32 && too_big) {
      if (threadIdx.x == 0) ws[3] = 3;
    } else {
      for (int64_t c = w; c < nch; c += WARPS) {
        if constexpr (I32) {
          const csr::RowRange rows = csr::chunk_rows(c, chunk, it.nrows, it.row_offsets, lane);
          if (xin)
            csr::csr_rows_x<T, SEG, csr::XShared<T>, false, int32_t>(rows, it.nrows, it.ncols, it.row_offsets,
                                                                     it.column_indices, va, csr::XShared<T>{xs}, y,
                                                                     init, stage[w], lane);
          else
            csr::csr_rows_x<T, SEG, csr::XGlobal<T>, false, int32_t>(rows, it.nrows, it.ncols, it.row_offsets,
                                                                     it.column_indices, va, csr::XGlobal<T>{xg}, y,
                                                                     init, stage[w], lane);
        } else {
          if (xin)
            csr::csr_chunk_x<T, SEG>(c, chunk, it.nrows, it.ncols, it.row_offsets, it.column_indices, va,
                                     csr::XShared<T>{xs}, y, init, stage[w], lane);
          else
            csr::csr_chunk_x<T, SEG>(c, chunk, it.nrows, it.ncols, it.row_offsets, it.column_indices, va,
                                     csr::XGlobal<T>{xg}, y, init, stage[w], lane);
        }
      }
    }
    __syncthreads();  // buffer `cur` and s_q[cur] are reused by the next fetch
    if constexpr (NBUF == 2) {
      cur ^= 1;
    } else {
      fetch(0);
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// One CTA per matrix at a time with x read through L1 (configs >= BAT_FIRST_XL1):
// the CTA's warps share one matrix, so its x (up to a few tens of KB) stays
// in L1 while they work on it; no staging, no wait.
template <typename T, int CFG>
__global__ void __launch_bounds__(BAT_WARPS * 32, 3)
spmv_batched_csr_xl1(const mgb_csr_batch_item* __restrict__ items, int64_t nitems, int32_t* ws, int init) {
  constexpr int SEG = BAT_SEG[CFG];
  constexpr int64_t CPW = BAT_XS_CPW[CFG];
  __shared__ csr::WarpStage<T, SEG> stage[BAT_WARPS];
  __shared__ int s_q;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  if (ws[2] != CFG) {
    if (threadIdx.x == 0) ws[3] = 1;
    return;
  }
  const int32_t* __restrict__ order = ws + BAT_HEADER;
  while (true) {
    if (threadIdx.x == 0) s_q = atomicAdd(ws, 1);
    __syncthreads();
    const int q = s_q;
    __syncthreads();
    if (q >= nitems) break;
    const mgb_csr_batch_item it = items[__ldg(order + q)];
    int64_t chunk = (it.nnz + BAT_WARPS * CPW - 1) / (BAT_WARPS * CPW);
    chunk = chunk < 256 ? 256 : (chunk > 4096 ? 4096 : chunk);
    const int64_t nch = it.nnz / chunk + 1;
    for (int64_t c = w; c < nch; c += BAT_WARPS)
      csr::csr_chunk_x<T, SEG>(c, chunk, it.nrows, it.ncols, it.row_offsets, it.column_indices,
                               static_cast<const T*>(it.values), csr::XGlobal<T>{static_cast<const T*>(it.x)},
                               static_cast<T*>(it.y), init, stage[w], lane);
  }
}

// order keys: (INT32_MAX - nnz) << 32 | index, so an ascending sort puts the
// largest matrices first (longest-processing-time-first scheduling)
__global__ void batch_order_keys(const mgb_csr_batch_item* __restrict__ items, int64_t n, uint64_t* keys) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t z = items[i].nnz;
    z = z < 0 ? 0 : (z > 0x7fffffffLL ? 0x7fffffffLL : z);
    keys[i] = ((uint64_t)(0x7fffffffLL - z) << 32) | (uint64_t)i;
  }
}

__global__ void batch_order_finish(const uint64_t* __restrict__ keys, int64_t n, int32_t* ws, int config) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    ws[BAT_HEADER + i] = (int32_t)(keys[i] & 0xffffffffu);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ws[0] = 0;
    ws[1] = (int32_t)n;
    ws[2] = config;
    ws[3] = 0;
  }
}

int64_t workspace_bytes(int64_t nitems) { return sizeof(int32_t) * (BAT_HEADER + nitems + 1); }

int plan(const mgb_csr_batch_item* items, int64_t nitems, int config, void* workspace, int64_t ws_bytes,
         cudaStream_t s) {
  MGB_REQUIRE(items != nullptr && workspace != nullptr && nitems > 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(config >= 0 && config < BAT_NCONFIGS, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(ws_bytes >= workspace_bytes(nitems), MGB_ERR_BAD_ARGUMENT);
  int32_t* ws = static_cast<int32_t*>(workspace);
  MGB_REQUIRE(nitems < 0x7fffffffLL, MGB_ERR_INVALID_INPUT);
  if (config >= BAT_FIRST_XS) {
    prim::Scratch sc(s);
    uint64_t* keys;
    int32_t* seg;
    MGB_SCRATCH(sc, keys, nitems);
    MGB_SCRATCH(sc, seg, 2);
    const int32_t hseg[2] = {0, (int32_t)nitems};
    MGB_CUDA_CHECK(cudaMemcpyAsync(seg, hseg, sizeof(hseg), cudaMemcpyHostToDevice, s));
    batch_order_keys<<<prim::blocks_for(nitems, 256), 256, 0, s>>>(items, nitems, keys);
    MGB_LAUNCH_CHECK();
    int st = prim::segmented_sort_u64(keys, seg, 1, nitems, s);
    if (st) return st;
    batch_order_finish<<<prim::blocks_for(nitems, 256), 256, 0, s>>>(keys, nitems, ws, config);
    MGB_LAUNCH_CHECK();
    // hseg is read by the copy before this function returns
    MGB_CUDA_CHECK(cudaStreamSynchronize(s));
    return MGB_SUCCESS;
  }
  int32_t* counts;
  int64_t* d_total;
  prim::Scratch sc(s);
  MGB_SCRATCH(sc, counts, nitems + 1);
  MGB_SCRATCH(sc, d_total, 1);
  batch_chunk_counts<<<prim::blocks_for(nitems, 256), 256, 0, s>>>(items, nitems, BAT_CHUNK[config], counts);
  MGB_LAUNCH_CHECK();
  MGB_CUDA_CHECK(cudaMemsetAsync(counts + nitems, 0, sizeof(int32_t), s));
  int st = prim::exclusive_scan<int32_t, int32_t>(counts, ws + BAT_HEADER, nitems + 1, s, d_total);
  if (st) return st;
  batch_finish_plan<<<1, 1, 0, s>>>(ws, d_total, config);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T, int CFG>
int launch_cfg(const mgb_csr_batch_item* items, int64_t nitems, int32_t* ws, int init, cudaStream_t s) {
  if constexpr (bat_is_xl1(CFG)) {
    spmv_batched_csr_xl1<T, CFG><<<num_sms() * 3, BAT_WARPS * 32, 0, s>>>(items, nitems, ws, init);
  } else if constexpr (CFG >= BAT_FIRST_XS) {
    constexpr int NBUF = bat_xs_nbuf(CFG);
    constexpr int WARPS = bat_xs_warps(CFG);
    constexpr size_t smem = NBUF * BAT_XS_BYTES + WARPS * sizeof(csr::WarpStage<T, BAT_SEG[CFG]>);
    // set once per device (a function attribute, not a stream operation)
    static std::atomic<bool> attr_set[64];
    int dev = 0;
    MGB_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !attr_set[dev].load(std::memory_order_acquire)) {
      MGB_CUDA_CHECK(cudaFuncSetAttribute(spmv_batched_csr_xs<T, CFG, NBUF, WARPS>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      if (dev >= 0 && dev < 64) attr_set[dev].store(true, std::memory_order_release);
    }
    spmv_batched_csr_xs<T, CFG, NBUF, WARPS>
        <<<num_sms() * bat_xs_ctas(CFG), WARPS * 32, smem, s>>>(items, nitems, ws, init);
  } else {
    spmv_batched_csr<T, CFG><<<num_sms() * 3, BAT_WARPS * 32, 0, s>>>(items, nitems, ws, init);
  }
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int launch(const mgb_csr_batch_item* items, int64_t nitems, int config, void* workspace, int init,
           cudaStream_t s) {
  MGB_REQUIRE(items != nullptr && workspace != nullptr && nitems > 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(config >= 0 && config < BAT_NCONFIGS, MGB_ERR_BAD_ARGUMENT);
  int32_t* ws = static_cast<int32_t*>(workspace);
  MGB_CUDA_CHECK(cudaMemsetAsync(ws, 0, sizeof(int32_t), s));      // work counter
  MGB_CUDA_CHECK(cudaMemsetAsync(ws + 3, 0, sizeof(int32_t), s));  // error flag: reports this launch only
  switch (config) {
    case 0: return launch_cfg<T, 0>(items, nitems, ws, init, s);
    case 1: return launch_cfg<T, 1>(items, nitems, ws, init, s);
    case 2: return launch_cfg<T, 2>(items, nitems, ws, init, s);
    case 3: return launch_cfg<T, 3>(items, nitems, ws, init, s);
    case 4: return launch_cfg<T, 4>(items, nitems, ws, init, s);
    case 5: return launch_cfg<T, 5>(items, nitems, ws, init, s);
    case 6: return launch_cfg<T, 6>(items, nitems, ws, init, s);
    case 7: return launch_cfg<T, 7>(items, nitems, ws, init, s);
    case 8: return launch_cfg<T, 8>(items, nitems, ws, init, s);
    case 9: return launch_cfg<T, 9>(items, nitems, ws, init, s);
    default: return launch_cfg<T, 10>(items, nitems, ws, init, s);
  }
}

// Times every configuration (plan + `reps` launches after one warm-up) and
// leaves the workspace planned for the fastest.  y is overwritten.
template <typename T>
int autotune(const mgb_csr_batch_item* items, int64_t nitems, void* workspace, int64_t ws_bytes, int reps,
             int* best, float* ms_out, cudaStream_t s) {
  MGB_REQUIRE(best != nullptr && reps > 0, MGB_ERR_BAD_ARGUMENT);
  cudaEvent_t e0, e1;
  MGB_CUDA_CHECK(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return record_cuda_error(ce);
  }
  int st = MGB_SUCCESS;
  float best_ms = 0.0f;
  *best = -1;
  for (int c = 0; c < BAT_NCONFIGS && st == MGB_SUCCESS; c++) {
    st = plan(items, nitems, c, workspace, ws_bytes, s);
    if (st == MGB_SUCCESS) st = launch<T>(items, nitems, c, workspace, 1, s);
    if (st != MGB_SUCCESS) break;
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps && st == MGB_SUCCESS; r++) st = launch<T>(items, nitems, c, workspace, 1, s);
    cudaEventRecord(e1, s);
    ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) {
      st = record_cuda_error(ce);
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)reps;
    if (ms_out) ms_out[c] = ms;
    if (*best < 0 || ms < best_ms) {
      best_ms = ms;
      *best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == MGB_SUCCESS) st = plan(items, nitems, *best, workspace, ws_bytes, s);
  return st;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_spmv_batched_csr_num_configs(void) { return mgb::BAT_NCONFIGS; }

int mgb_spmv_batched_csr_config_info(int config, int64_t* chunk, int* seg) {
  if (config < 0 || config >= mgb::BAT_NCONFIGS || !chunk || !seg) return MGB_ERR_BAD_ARGUMENT;
  *chunk = mgb::BAT_CHUNK[config];
  *seg = mgb::BAT_SEG[config];
  return MGB_SUCCESS;
}

int mgb_spmv_batched_csr_workspace_bytes(int64_t nitems, int64_t* bytes) {
  if (nitems <= 0 || !bytes) return MGB_ERR_BAD_ARGUMENT;
  *bytes = mgb::workspace_bytes(nitems);
  return MGB_SUCCESS;
}

int mgb_spmv_batched_csr_plan(const mgb_csr_batch_item* d_items, int64_t nitems, int config, void* workspace,
                              int64_t workspace_bytes, void* stream) {
  return mgb::plan(d_items, nitems, config, workspace, workspace_bytes, mgb::as_stream(stream));
}

int mgb_spmv_batched_csr_f64(const mgb_csr_batch_item* d_items, int64_t nitems, int config, void* workspace,
                             int init, void* stream) {
  return mgb::launch<double>(d_items, nitems, config, workspace, init, mgb::as_stream(stream));
}

int mgb_spmv_batched_csr_f32(const mgb_csr_batch_item* d_items, int64_t nitems, int config, void* workspace,
                             int init, void* stream) {
  return mgb::launch<float>(d_items, nitems, config, workspace, init, mgb::as_stream(stream));
}

int mgb_spmv_batched_csr_autotune_f64(const mgb_csr_batch_item* d_items, int64_t nitems, void* workspace,
                                      int64_t workspace_bytes, int reps, int* best_config, float* ms_per_config,
                                      void* stream) {
  return mgb::autotune<double>(d_items, nitems, workspace, workspace_bytes, reps, best_config, ms_per_config,
                               mgb::as_stream(stream));
}

int mgb_spmv_batched_csr_autotune_f32(const mgb_csr_batch_item* d_items, int64_t nitems, void* workspace,
                                      int64_t workspace_bytes, int reps, int* best_config, float* ms_per_config,
                                      void* stream) {
  return mgb::autotune<float>(d_items, nitems, workspace, workspace_bytes, reps, best_config, ms_per_config,
                              mgb::as_stream(stream));
}

}  // extern "C"
