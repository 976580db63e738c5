// spmv_csr_rows.cu -- CSR SpMV for rows of (nearly) equal, short length, and
// the per-matrix choice between the CSR kernels.
//
// The reference chooses its scalar (thread-per-row) CSR kernel only when the
// user sets MATOPT_SHORT_ROWS (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:59-92).
// Here the choice is measured: mgb_csr_choose_kernel reads the row lengths
// and the columns of a sample of neighbouring rows once and picks
//   MGB_CSR_SPLIT       when some row is longer than 8192 entries or rows
//                       average >= 512 (split nonzero chunks with carries,
//                       spmv_csr.cu), else, for short rows of nearly equal
//                       length (longest row <= 28 and <= 1.5 x mean + 2):
//   MGB_CSR_ROWS        when neighbouring rows read neighbouring columns
//                       (stencils, banded matrices, FEM meshes), or
//   MGB_CSR_ROWS_GATHER when their columns are scattered, else
//   MGB_CSR_SEGMENTS    the lane-segment kernel of spmv_csr.cu (any structure).
//
// Row-tile kernel: one warp owns 32 consecutive rows.  The tile's entries are
// one contiguous range of the CSR arrays; up to TILE of them at a time are
// staged into shared memory with cp.async (all in flight at once), then every
// lane walks its own row from shared memory in lockstep with the others
// (equal lengths keep every FP64 FMA full-warp), issuing its x reads 8, 4,
// 2, 1 at a time so that FMA slots match the row length exactly.  TILE holds
// a whole tile (224 / 448 / 896 entries for 32 rows of the mean length), and
// the two variants differ in CTAs per SM, i.e. in the shared-memory carve-out
// and the L1 left beside it: neighbouring columns touch few x sectors and
// want resident warps (about 172 KB of shared memory), scattered columns
// need L1 lines for their misses in flight (about 129 KB; with 233 KB the
// same kernel ran at half speed).  The measurements are at rows_config.
#include <atomic>

#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int ROWS_WARPS = 4;
constexpr int ROWS_TILE_MAX = 896;  // 32 rows x 28 entries: the longest rows a tile is chosen for

__device__ __forceinline__ unsigned rows_smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
// one element global -> shared with cp.async (no register round trip)
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(rows_smem_u32(dst)), "l"(src), "n"(BYTES)
               : "memory");
}

// x reads of U consecutive entries of every lane's row, then their FMAs
// (staged entry e sits at sv[e - cv] and sc[e - cc])
template <int U, typename T>
__device__ __forceinline__ void rows_step(int32_t j, int32_t lo, int32_t hi, int32_t cv, int32_t cc, int64_t ncols,
                                          const T* sv, const int32_t* sc, const T* __restrict__ x, T& acc) {
  T xv[U], vv[U];
#pragma unroll
  for (int q = 0; q < U; q++) {
    const int32_t e = lo + j + q;
    const bool ok = e < hi;
    const int32_t col = ok ? sc[e - cc] : 0;
    vv[q] = ok ? sv[e - cv] : T(0);
    xv[q] = (ok && (unsigned)col < (uint64_t)ncols) ? __ldg(x + col) : T(0);
  }
#pragma unroll
  for (int q = 0; q < U; q++)
    if (lo + j + q < hi) acc = fmadd(vv[q], xv[q], acc);
}

// Stages entries [c, cend) of the values and columns into shared memory.
// VEC: 16-byte cp.async pieces from the 16-byte boundaries at or below c
// (the arrays must be 16-byte aligned), the ragged end element by element,
// never past cend; returns the first staged entry of each array (*cv, *cc).
// Otherwise one element per copy, staged from c.  Measured on the 27-point
// stencil (160^3): FP32 202 -> 184 us with 16-byte pieces, FP64 320 -> 346 us
// (FP64 keeps element copies).
template <typename T, bool VEC>
__device__ __forceinline__ void stage_tile(int32_t c, int32_t cend, const int32_t* __restrict__ ci,
                                           const T* __restrict__ va, T* sv, int32_t* sc, int lane, int32_t* cv,
                                           int32_t* cc) {
  if constexpr (VEC) {
    constexpr int VV = 16 / sizeof(T);
    const int32_t av = c & ~(VV - 1), ac = c & ~3;
    const int32_t ev = cend & ~(VV - 1), ec = cend & ~3;
    for (int32_t i = av + lane * VV; i < ev; i += 32 * VV)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(rows_smem_u32(sv + (i - av))), "l"(va + i)
                   : "memory");
    for (int32_t i = max(ev, av) + lane; i < cend; i += 32) cp_async_elem<sizeof(T)>(sv + (i - av), va + i);
    for (int32_t i = ac + lane * 4; i < ec; i += 128)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(rows_smem_u32(sc + (i - ac))), "l"(ci + i)
                   : "memory");
    for (int32_t i = max(ec, ac) + lane; i < cend; i += 32) cp_async_elem<4>(sc + (i - ac), ci + i);
    *cv = av;
    *cc = ac;
  } else {
    for (int32_t i = c + lane; i < cend; i += 32) {
      cp_async_elem<sizeof(T)>(sv + (i - c), va + i);
      cp_async_elem<4>(sc + (i - c), ci + i);
    }
    *cv = c;
    *cc = c;
  }
}

// DOT: also x[0..nrows) . y, one partial per CTA in partials[blockIdx.x]
// (the launcher then caps the grid at the resident CTAs, so a solver sums a
// few thousand partials, not one per tile).
template <typename T, bool DOT, int TILE, int MINB, bool VEC>
__global__ void __launch_bounds__(ROWS_WARPS * 32, MINB)
spmv_csr_rowtile(int64_t nrows, int64_t ncols, const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                 const T* __restrict__ va, const T* __restrict__ x, T* __restrict__ y, int init,
                 T* __restrict__ partials) {
  // VEC stages from up to 16 bytes before the tile: room for the extra entries
  constexpr int PADV = VEC ? 16 / (int)sizeof(T) : 0, PADC = VEC ? 4 : 0;
  __shared__ __align__(16) T s_val[ROWS_WARPS][TILE + PADV];
  __shared__ __align__(16) int32_t s_col[ROWS_WARPS][TILE + PADC];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  T* sv = s_val[w];
  int32_t* sc = s_col[w];
  const int64_t ntiles = (nrows + 31) >> 5;
  T part = T(0);
  for (int64_t tile = (int64_t)blockIdx.x * ROWS_WARPS + w; tile < ntiles;
       tile += (int64_t)gridDim.x * ROWS_WARPS) {
    const int64_t r = (tile << 5) + lane;
    const bool valid = r < nrows;
    const int32_t rs = __ldg(ro + (valid ? r : nrows));
    const int32_t re = valid ? __ldg(ro + r + 1) : rs;
    const int32_t tb = __shfl_sync(0xffffffffu, rs, 0);
    const int32_t te = (int32_t)__reduce_max_sync(0xffffffffu, (unsigned)re);
    T acc = (valid && !init) ? y[r] : T(0);
    for (int32_t c = tb; c < te; c += TILE) {
      const int32_t cend = (te - c < TILE) ? te : c + TILE;
      __syncwarp();  // the previous piece's shared-memory reads are done
      int32_t cv = c, cc = c;
      stage_tile<T, VEC>(c, cend, ci, va, sv, sc, lane, &cv, &cc);
      asm volatile("cp.async.wait_all;\n" ::: "memory");
      __syncwarp();
      const int32_t lo = max(rs, c), hi = min(re, cend);
      // lockstep over the longest intersection in the warp (n is warp-uniform)
      const int32_t n = (int32_t)__reduce_max_sync(0xffffffffu, (unsigned)max(hi - lo, 0));
      int32_t j = 0;
      // rows of up to 28 entries (896-entry tiles): rounds of 16 first
      // (27-point stencil: 318 -> 311 us FP64; with shorter rows the extra
      // round only costs registers: 2-D Laplacian FP32 62 -> 70 us)
      if constexpr (TILE >= 896)
        for (; j + 16 <= n; j += 16) rows_step<16>(j, lo, hi, cv, cc, ncols, sv, sc, x, acc);
      for (; j + 8 <= n; j += 8) rows_step<8>(j, lo, hi, cv, cc, ncols, sv, sc, x, acc);
      if (j + 4 <= n) {
        rows_step<4>(j, lo, hi, cv, cc, ncols, sv, sc, x, acc);
        j += 4;
      }
      if (j + 2 <= n) {
        rows_step<2>(j, lo, hi, cv, cc, ncols, sv, sc, x, acc);
        j += 2;
      }
      if (j < n) rows_step<1>(j, lo, hi, cv, cc, ncols, sv, sc, x, acc);
    }
    if (valid) {
      y[r] = acc;
      if (DOT) part = fmadd(x[r], acc, part);
    }
  }
  if (DOT) {
    __shared__ T s_part[ROWS_WARPS];
    part = warp_sum(part);
    if (lane == 0) s_part[w] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      T t = T(0);
#pragma unroll
      for (int i = 0; i < ROWS_WARPS; i++) t += s_part[i];
      partials[blockIdx.x] = t;
    }
  }
}

// Row shape of a CSR matrix: shape[0] = longest row; over every 16th row r
// (and row r + 1), shape[1] = entries k of the shorter of the two rows with
// |col(r+1, k) - col(r, k) - 1| <= 2 (neighbouring rows reading neighbouring
// columns), shape[2] = entries compared.
__global__ void row_shape_kernel(const int32_t* __restrict__ ro, const int32_t* __restrict__ ci, int64_t nrows,
                                 unsigned long long* shape) {
  int m = 0;
  unsigned long long near = 0, cmp = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = ro[r], b = ro[r + 1];
    m = max(m, b - a);
    if ((r & 15) == 0 && r + 1 < nrows) {
      const int32_t b2 = ro[r + 2];
      const int32_t len = min(min(b - a, b2 - b), 64);
      for (int32_t k = 0; k < len; k++) {
        const int64_t d = (int64_t)ci[b + k] - (int64_t)ci[a + k] - 1;
        near += (d >= -2 && d <= 2) ? 1u : 0u;
      }
      cmp += (unsigned long long)(len > 0 ? len : 0);
    }
  }
  m = __reduce_max_sync(0xffffffffu, m);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    near += __shfl_xor_sync(0xffffffffu, near, o);
    cmp += __shfl_xor_sync(0xffffffffu, cmp, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(shape, (unsigned long long)m);
    atomicAdd(shape + 1, near);
    atomicAdd(shape + 2, cmp);
  }
}

// Launches one staging configuration.  The shared-memory carve-out is set
// to what MINB CTAs need (once per device): the driver would otherwise take
// the largest carve-out that the CTAs fit, and the L1 left beside it is what
// the x reads' misses in flight live in (measured: 12 scattered entries per
// row, 448-entry staging, 10 CTAs: 213 us with a 233 KB carve-out, 110 us at
// 6 CTAs in 129 KB).
template <typename T, bool DOT, int TILE, int MINB, bool VEC>
int launch_rows_vec(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, unsigned blocks) {
  static std::atomic<bool> carve_set[64];
  int dev = 0;
  MGB_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || !carve_set[dev].load(std::memory_order_acquire)) {
    constexpr int padv = VEC ? 16 / (int)sizeof(T) : 0, padc = VEC ? 4 : 0;
    constexpr int per_cta =
        ROWS_WARPS * ((TILE + padv) * (int)sizeof(T) + (TILE + padc) * (int)sizeof(int32_t)) + 1024;
    constexpr int pct = (MINB * per_cta * 100 + 228 * 1024 - 1) / (228 * 1024);
    MGB_CUDA_CHECK(cudaFuncSetAttribute(spmv_csr_rowtile<T, DOT, TILE, MINB, VEC>,
                                        cudaFuncAttributePreferredSharedMemoryCarveout, pct > 100 ? 100 : pct));
    if (dev >= 0 && dev < 64) carve_set[dev].store(true, std::memory_order_release);
  }
  spmv_csr_rowtile<T, DOT, TILE, MINB, VEC><<<blocks, ROWS_WARPS * 32, 0, s>>>(
      A->nrows, A->ncols, A->row_offsets, A->column_indices, static_cast<const T*>(A->values), x, y, init,
      partials);
  return MGB_SUCCESS;
}

// FP32 with 16-byte aligned values and columns stages 16-byte pieces
template <typename T, bool DOT, int TILE, int MINB>
int launch_rows_cfg(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, unsigned blocks) {
  const bool aligned = (reinterpret_cast<uintptr_t>(A->values) % 16 == 0) &&
                       (reinterpret_cast<uintptr_t>(A->column_indices) % 16 == 0);
  if (sizeof(T) == 4 && aligned)
    return launch_rows_vec<T, DOT, TILE, MINB, sizeof(T) == 4>(A, x, y, init, s, partials, blocks);
  return launch_rows_vec<T, DOT, TILE, MINB, false>(A, x, y, init, s, partials, blocks);
}

// CTAs per SM of a staging configuration: as many as fit a shared-memory
// budget (neighbouring columns: resident warps for the latency-bound tiles,
// 180 KB in FP64, 215 KB in FP32 -- the 27-point stencil in FP32, 896 x 6:
// 185.0 us, 896 x 7: 172.5 us; 135 KB for scattered columns: L1 for the
// misses in flight), at most 12.  Measured on GB300 (us per SpMV, FP64, TILE x CTAs):
//   5-point Laplacian 2048^2:      224 x 12  69.6
//   band of 13, N = 2M:            448 x 10  78.5   448 x 8  71.7
//   27-point stencil 160^3:        896 x 5  342.8   896 x 4  319.7   896 x 3  388.7
//   scattered, 12 per row, N = 2M: 448 x 10 213.4   224 x 10 108.6   448 x 6 109.7
//   scattered, 20 per row:         896 x 5  263.3   224 x 10 160.2   896 x 3 147.5
//   scattered, 27 per row, N = 1M: 896 x 5  237.4   896 x 3  133.1   (lane segments 162)
template <typename T>
constexpr int rows_ctas(int tile, bool gather) {
  const int per_cta = ROWS_WARPS * tile * (int)(sizeof(T) + sizeof(int32_t)) + 1024;
  const int n = (gather ? 135 * 1024 : (sizeof(T) == 4 ? 215 : 180) * 1024) / per_cta;
  return n > 12 ? 12 : (n < 1 ? 1 : n);
}

// Staging size: the smallest of 224 / 448 / 896 entries that holds a tile of
// 32 rows of the mean length (longer tiles are processed in pieces, so this
// is a performance choice only).  Returns the CTAs per SM of the choice.
template <typename T>
int rows_config(const mgb_csr* A, bool gather, int* tile) {
  const int64_t tile_entries = 32 * (A->nnz / (A->nrows > 0 ? A->nrows : 1)) + 8;
  *tile = tile_entries <= 224 ? 224 : (tile_entries <= 448 ? 448 : 896);
  return rows_ctas<T>(*tile, gather);
}

template <typename T, bool DOT>
int launch_rows_variant(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials,
                        unsigned blocks, bool gather) {
  int tile = 0;
  rows_config<T>(A, gather, &tile);
  if (gather) {
    if (tile == 224) return launch_rows_cfg<T, DOT, 224, rows_ctas<T>(224, true)>(A, x, y, init, s, partials, blocks);
    if (tile == 448) return launch_rows_cfg<T, DOT, 448, rows_ctas<T>(448, true)>(A, x, y, init, s, partials, blocks);
    return launch_rows_cfg<T, DOT, 896, rows_ctas<T>(896, true)>(A, x, y, init, s, partials, blocks);
  }
  if (tile == 224) return launch_rows_cfg<T, DOT, 224, rows_ctas<T>(224, false)>(A, x, y, init, s, partials, blocks);
  if (tile == 448) return launch_rows_cfg<T, DOT, 448, rows_ctas<T>(448, false)>(A, x, y, init, s, partials, blocks);
  return launch_rows_cfg<T, DOT, 896, rows_ctas<T>(896, false)>(A, x, y, init, s, partials, blocks);
}

template <typename T>
int launch_rows(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, int64_t* npartials,
                bool gather) {
  const int64_t ntiles = (A->nrows + 31) / 32;
  int64_t blocks = (ntiles + ROWS_WARPS - 1) / ROWS_WARPS;
  if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
  if (npartials || partials) {
    // the fused dot: one partial per CTA, grid capped at the resident CTAs
    int tile = 0;
    const int64_t resident = (int64_t)num_sms() * rows_config<T>(A, gather, &tile);
    if (blocks > resident) blocks = resident;
    if (npartials) *npartials = blocks;
  }
  if (npartials && !partials) return take_device_query_error();
  const int st = partials ? launch_rows_variant<T, true>(A, x, y, init, s, partials, (unsigned)blocks, gather)
                         : launch_rows_variant<T, false>(A, x, y, init, s, nullptr, (unsigned)blocks, gather);
  if (st != MGB_SUCCESS) return st;
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int choose(const mgb_csr* A, int* variant, cudaStream_t s) {
  MGB_REQUIRE(A != nullptr && variant != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  *variant = MGB_CSR_SEGMENTS;
  if (A->nrows == 0 || A->nnz == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr && A->column_indices != nullptr, MGB_ERR_BAD_ARGUMENT);
  unsigned long long* d = nullptr;
  MGB_CUDA_CHECK(cudaMallocAsync((void**)&d, 3 * sizeof(unsigned long long), s));
  cudaError_t e = cudaMemsetAsync(d, 0, 3 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) {
    int64_t blocks = (A->nrows + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (blocks > cap) blocks = cap;
    row_shape_kernel<<<(unsigned)blocks, 256, 0, s>>>(A->row_offsets, A->column_indices, A->nrows, d);
    e = cudaGetLastError();
  }
  unsigned long long shape[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(shape, d, sizeof(shape), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(d, s);
  if (e != cudaSuccess) return record_cuda_error(e);
  const double mx = (double)shape[0];
  const double mean = (double)A->nnz / (double)A->nrows;
  const bool neighbouring = shape[2] == 0 || 2 * shape[1] >= shape[2];
  if (32 * mx <= ROWS_TILE_MAX && mx <= 1.5 * mean + 2.0) {
    *variant = neighbouring ? MGB_CSR_ROWS : MGB_CSR_ROWS_GATHER;
  }
  // rows longer than a few chunks: one warp per row would be the critical
  // path (measured: a 150,000-entry row 746 -> 56 us; rows of 1,000-6,000
  // entries 66 -> 46 us; the power-law matrix, mean 15, stays faster whole)
  if (mx > 8192 || mean >= 512.0) *variant = MGB_CSR_SPLIT;
  return MGB_SUCCESS;
}

}  // namespace

// CSR SpMV entry with an explicit kernel choice (used by spmv_csr.cu too)
template <typename T>
int launch_csr_rows(const mgb_csr* A, const T* x, T* y, int init, cudaStream_t s, T* partials, int64_t* npartials,
                    bool gather) {
  return launch_rows<T>(A, x, y, init, s, partials, npartials, gather);
}
template int launch_csr_rows<double>(const mgb_csr*, const double*, double*, int, cudaStream_t, double*, int64_t*,
                                     bool);
template int launch_csr_rows<float>(const mgb_csr*, const float*, float*, int, cudaStream_t, float*, int64_t*,
                                    bool);

}  // namespace mgb

extern "C" int mgb_csr_choose_kernel(const mgb_csr* A, int* variant, void* stream) {
  return mgb::choose(A, variant, mgb::as_stream(stream));
}
