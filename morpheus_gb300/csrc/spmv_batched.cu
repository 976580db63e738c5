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
// configurations; mgb_spmv_batched_csr_autotune_* times each on the actual
// batch with CUDA events and returns the fastest.
#include "csr_chunk.cuh"
#include "primitives.cuh"

namespace mgb {
namespace {

constexpr int BAT_WARPS = 8;
constexpr int BAT_NCONFIGS = 6;
constexpr int64_t BAT_CHUNK[BAT_NCONFIGS] = {512, 1024, 2048, 4096, 1024, 2048};
constexpr int BAT_SEG[BAT_NCONFIGS] = {8, 8, 8, 8, 4, 4};
// workspace: int32 header[4] = {work counter, total chunks, planned config,
// error flag}, then int32 prefix[nitems + 1]
constexpr int BAT_HEADER = 4;

__global__ void batch_chunk_counts(const mgb_csr_batch_item* __restrict__ items, int64_t n, int64_t chunk,
                                   int32_t* counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    counts[i] = (int32_t)(items[i].nnz / chunk + 1);
}

__global__ void batch_finish_plan(int32_t* ws, const int64_t* total, int config) {
  ws[0] = 0;
  ws[1] = (int32_t)*total;
  ws[2] = config;
  ws[3] = 0;
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
    // matrix owning chunk g: last i with prefix[i] <= g
    int64_t lo = 0, hi = nitems - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (__ldg(prefix + mid) <= g) lo = mid; else hi = mid - 1;
    }
    const mgb_csr_batch_item it = items[lo];
    csr::csr_chunk<T, CHUNK, SEG>(g - __ldg(prefix + lo), it.nrows, it.ncols, it.row_offsets, it.column_indices,
                                  static_cast<const T*>(it.values), static_cast<const T*>(it.x),
                                  static_cast<T*>(it.y), init, stage[w], lane);
  }
}

int64_t workspace_bytes(int64_t nitems) { return sizeof(int32_t) * (BAT_HEADER + nitems + 1); }

int plan(const mgb_csr_batch_item* items, int64_t nitems, int config, void* workspace, int64_t ws_bytes,
         cudaStream_t s) {
  MGB_REQUIRE(items != nullptr && workspace != nullptr && nitems > 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(config >= 0 && config < BAT_NCONFIGS, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(ws_bytes >= workspace_bytes(nitems), MGB_ERR_BAD_ARGUMENT);
  int32_t* ws = static_cast<int32_t*>(workspace);
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
  const int blocks = num_sms() * 3;
  spmv_batched_csr<T, CFG><<<blocks, BAT_WARPS * 32, 0, s>>>(items, nitems, ws, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

template <typename T>
int launch(const mgb_csr_batch_item* items, int64_t nitems, int config, void* workspace, int init,
           cudaStream_t s) {
  MGB_REQUIRE(items != nullptr && workspace != nullptr && nitems > 0, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(config >= 0 && config < BAT_NCONFIGS, MGB_ERR_BAD_ARGUMENT);
  int32_t* ws = static_cast<int32_t*>(workspace);
  MGB_CUDA_CHECK(cudaMemsetAsync(ws, 0, sizeof(int32_t), s));  // work counter
  switch (config) {
    case 0: return launch_cfg<T, 0>(items, nitems, ws, init, s);
    case 1: return launch_cfg<T, 1>(items, nitems, ws, init, s);
    case 2: return launch_cfg<T, 2>(items, nitems, ws, init, s);
    case 3: return launch_cfg<T, 3>(items, nitems, ws, init, s);
    case 4: return launch_cfg<T, 4>(items, nitems, ws, init, s);
    default: return launch_cfg<T, 5>(items, nitems, ws, init, s);
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
