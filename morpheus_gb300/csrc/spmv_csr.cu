// spmv_csr.cu -- CSR SpMV for sm_103a.
//
// Replaces the reference's CUDA CSR path (impl/Csr/Cuda/Morpheus_Multiply_Impl.hpp:50-157,
// kernels impl/Csr/Kernels/Morpheus_Multiply_Impl.hpp:36-168), which picks one
// threads-per-row value from the global mean row length and reduces through
// volatile shared memory.  Semantics follow the Serial multiply
// (impl/Csr/Serial/Morpheus_Multiply_Impl.hpp:38-58): per row,
// sum = init ? 0 : y[i]; sum += A(i,j) * x[j] over the row; y[i] = sum.
//
// GB300 constraint that shapes this kernel: the FP64 pipe retires about one
// warp-wide DFMA per 16 SM cycles and charges that slot whether 1 or 32 lanes
// are active.  A kernel whose lanes walk rows of different lengths, or that
// reduces every row with a shuffle tree, spends most FP64 slots on idle lanes.
// So the work is split by NONZEROS, not rows:
//
//  * Warp chunks.  Warp w takes the rows whose first entry lies in the nominal
//    range [w*CHUNK, (w+1)*CHUNK) (two 32-ary searches over row_offsets), so
//    every chunk is a whole number of rows and no row crosses warps: no
//    atomics, no scratch, deterministic.
//  * Lane segments.  The chunk's nonzeros [E0, E1) are cut into 32 contiguous
//    lane ranges of KW entries.  Lane l walks its range accumulating with one
//    FMA per entry into the current row and flushing at row ends; every FMA
//    instruction is issued by all 32 lanes together.
//  * Staging.  Each step the warp loads 8 entries of every lane range
//    (4 x 64-byte pieces per load instruction) into padded shared memory, so
//    HBM reads stay sector-complete and shared-memory reads conflict-free.
//    Row offsets of the chunk are staged too, so row-end tests never wait on
//    global memory.
//  * Rows crossing lanes.  A row that continues into the next lane leaves a
//    tail partial; one 5-step segmented shuffle scan per chunk (keyed by row)
//    forwards the partials, and the lane where the row ends adds them: 6
//    extra FP64 warp instructions per ~2048 nonzeros.
// With init == 0 a row's accumulator starts from y[i] (a load, no extra add).
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int CSR_WARPS = 8;          // warps per CTA
constexpr int CSR_SEG = 8;            // entries per lane per staging step
constexpr int CSR_PAD = CSR_SEG + 1;  // padded lane stride in shared memory
constexpr int64_t CSR_CHUNK = 2048;   // nominal nonzeros per warp
constexpr int CSR_RO_STAGE = 512;     // row offsets staged per warp

// first index i in [lo, hi] with ro[i] >= key (hi if none), 32 lanes cooperating
__device__ __forceinline__ int64_t warp_lower_bound(const int32_t* __restrict__ ro, int64_t lo,
                                                    int64_t hi, int64_t key, int lane) {
  // invariant: ro[i] < key for i < lo; ro[i] >= key for i >= hi (virtually)
  while (hi - lo > 32) {
    const int64_t span = hi - lo;
    const int64_t p = lo + (span * (lane + 1)) / 33;  // 32 interior pivots
    const bool less = (int64_t)__ldg(ro + p) < key;
    const unsigned m = __ballot_sync(0xffffffffu, less);
    // pivots are increasing, so 'less' holds on a prefix of the lanes
    const int cnt = __popc(m);
    const int64_t new_lo = cnt ? __shfl_sync(0xffffffffu, p, cnt - 1) + 1 : lo;
    const int64_t new_hi = __shfl_sync(0xffffffffu, p, cnt < 32 ? cnt : 31);
    lo = new_lo;
    hi = cnt < 32 ? new_hi : hi;
  }
  // at most 32 candidates left: [lo, hi)
  const int64_t q = lo + lane;
  const bool less = q < hi && (int64_t)__ldg(ro + q) < key;
  return lo + __popc(__ballot_sync(0xffffffffu, less));
}

template <typename T>
__global__ void __launch_bounds__(CSR_WARPS * 32, 3)
spmv_csr_segments(int64_t nrows, int64_t ncols, int64_t nnz, int64_t nchunks,
                  const int32_t* __restrict__ ro, const int32_t* __restrict__ ci,
                  const T* __restrict__ va, const T* __restrict__ x,
                  T* __restrict__ y, int init) {
  __shared__ T s_val[CSR_WARPS][32 * CSR_PAD];
  __shared__ int32_t s_col[CSR_WARPS][32 * CSR_PAD];
  __shared__ int32_t s_ro[CSR_WARPS][CSR_RO_STAGE];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  T* sv = s_val[w];
  int32_t* sc = s_col[w];
  int32_t* sro = s_ro[w];

  for (int64_t wc = (int64_t)blockIdx.x * CSR_WARPS + w; wc < nchunks;
       wc += (int64_t)gridDim.x * CSR_WARPS) {
    // rows starting in [s0, s1)
    const int64_t s0 = wc * CSR_CHUNK, s1 = s0 + CSR_CHUNK;
    int64_t r_begin = warp_lower_bound(ro, 0, nrows + 1, s0, lane);
    int64_t r_end = warp_lower_bound(ro, r_begin, nrows + 1, s1, lane);
    if (r_begin > nrows) r_begin = nrows;
    if (r_end > nrows) r_end = nrows;
    if (r_begin >= r_end) continue;
    const int64_t nr = r_end - r_begin;
    const bool staged = nr < CSR_RO_STAGE;  // offsets r_begin..r_end in smem
    __syncwarp();
    if (staged)
      for (int64_t i = lane; i <= nr; i += 32) sro[i] = __ldg(ro + r_begin + i);
    __syncwarp();
    auto ro_at = [&](int64_t i) -> int64_t {
      return staged ? (int64_t)sro[i - r_begin] : (int64_t)__ldg(ro + i);
    };
    const int64_t E0 = ro_at(r_begin), E1 = ro_at(r_end);
    if (E0 >= E1) {  // only empty rows
      if (init)
        for (int64_t r = r_begin + lane; r < r_end; r += 32) y[r] = T(0);
      continue;
    }
    const int64_t A0 = E0 & ~(int64_t)7;  // 32-byte aligned column segments
    int64_t KW = (E1 - A0 + 31) / 32;
    KW = (KW + CSR_SEG - 1) / CSR_SEG * CSR_SEG;
    const int64_t la = A0 + lane * KW;
    const int64_t lb = min(la + KW, E1);
    const int64_t e_lo = max(la, E0);
    const bool active = e_lo < lb;

    // lane's first row: lane 0 starts at r_begin (so leading empty rows are
    // flushed); others at the row containing e_lo (empty rows sitting at a
    // lane boundary are flushed by the previous lane's tail loop).
    int64_t r = r_end;
    if (active) {
      if (lane == 0) {
        r = r_begin;
      } else {
        int64_t lo = r_begin, hi = r_end;  // first i in [lo, hi] with ro[i] > e_lo
        while (lo < hi) {
          const int64_t mid = (lo + hi) >> 1;
          if (ro_at(mid) <= e_lo) lo = mid + 1; else hi = mid;
        }
        r = lo - 1;
      }
    }
    int64_t rs = active ? ro_at(r) : 0;
    int64_t re = active ? ro_at(r + 1) : 0;
    T acc = (active && rs >= e_lo && !init) ? y[r] : T(0);
    int64_t hrow = -1;
    T hval = T(0);

    for (int64_t s = 0; s < KW; s += CSR_SEG) {
      __syncwarp();
#pragma unroll
      for (int q = 0; q < CSR_SEG; q++) {
        const int f = q * 32 + lane;
        const int L = f / CSR_SEG, j = f % CSR_SEG;
        const int64_t e = A0 + L * KW + s + j;
        const bool in = e >= E0 && e < E1;
        sv[L * CSR_PAD + j] = in ? ldg_stream(va + e) : T(0);
        sc[L * CSR_PAD + j] = in ? ldg_stream(ci + e) : 0;
      }
      __syncwarp();
      T v[CSR_SEG], xv[CSR_SEG];
#pragma unroll
      for (int k = 0; k < CSR_SEG; k++) {
        const int64_t e = la + s + k;
        const bool valid = e >= e_lo && e < lb;
        const int32_t c = sc[lane * CSR_PAD + k];
        v[k] = valid ? sv[lane * CSR_PAD + k] : T(0);
        xv[k] = (valid && (uint64_t)(int64_t)c < (uint64_t)ncols) ? __ldg(x + c) : T(0);
      }
#pragma unroll
      for (int k = 0; k < CSR_SEG; k++) {
        const int64_t e = la + s + k;
        const bool valid = e >= e_lo && e < lb;
        while (valid && e >= re) {
          if (rs >= e_lo) { y[r] = acc; } else { hrow = r; hval = acc; }
          r++;
          rs = re;
          re = ro_at(r + 1);
          acc = init ? T(0) : y[r];
        }
        acc = fmadd(v[k], xv[k], acc);
      }
    }
    // rows ending exactly at the lane end (and empty rows sitting there)
    if (active) {
      while (r < r_end && re <= lb) {
        if (rs >= e_lo) { y[r] = acc; } else { hrow = r; hval = acc; }
        r++;
        if (r < r_end) {
          rs = re;
          re = ro_at(r + 1);
          acc = init ? T(0) : y[r];  // empty rows at lb are flushed here
        }
      }
    }
    // tail partial (a row that started in this lane's range and continues into
    // the next lane; a row starting exactly at lb belongs to the next lane)
    // and segmented scan
    const bool has_tail = active && r < r_end && rs < lb;
    const int64_t key = has_tail ? r : -1 - (int64_t)lane;
    T cv = has_tail ? acc : T(0);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, cv, d);
      const int64_t k2 = __shfl_up_sync(0xffffffffu, key, d);
      if (lane >= d && k2 == key) cv += u;
    }
    const T vprev = __shfl_up_sync(0xffffffffu, cv, 1);
    const int64_t kprev = __shfl_up_sync(0xffffffffu, key, 1);
    if (hrow >= 0) y[hrow] = (lane > 0 && kprev == hrow) ? hval + vprev : hval;
  }
}

template <typename T>
int launch_csr(const mgb_csr* A, const T* x, T* y, int init, void* stream) {
  MGB_REQUIRE(A != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(!bad_sizes(A->nrows, A->ncols, A->nnz), MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz < ((int64_t)1 << 31) - 4096, MGB_ERR_INVALID_INPUT);
  if (A->nrows == 0) return MGB_SUCCESS;
  MGB_REQUIRE(A->row_offsets != nullptr && y != nullptr, MGB_ERR_BAD_ARGUMENT);
  MGB_REQUIRE(A->nnz == 0 || (A->column_indices && A->values && x), MGB_ERR_BAD_ARGUMENT);
  // one extra chunk so rows whose first entry is at nnz (trailing empty rows)
  // always belong to some chunk
  const int64_t nchunks = A->nnz / CSR_CHUNK + 1;
  int64_t blocks = (nchunks + CSR_WARPS - 1) / CSR_WARPS;
  if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
  spmv_csr_segments<T><<<(unsigned)blocks, CSR_WARPS * 32, 0, as_stream(stream)>>>(
      A->nrows, A->ncols, A->nnz, nchunks, A->row_offsets, A->column_indices,
      static_cast<const T*>(A->values), x, y, init);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_spmv_csr_f64(const mgb_csr* A, const double* x, double* y, int init, void* stream) {
  return mgb::launch_csr<double>(A, x, y, init, stream);
}

int mgb_spmv_csr_f32(const mgb_csr* A, const float* x, float* y, int init, void* stream) {
  return mgb::launch_csr<float>(A, x, y, init, stream);
}

}  // extern "C"
