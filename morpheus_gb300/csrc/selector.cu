// selector.cu -- the learned format selector's network: forward, backward and
// Adam kernels for a 12 -> 64 -> 64 -> 6 MLP (ReLU, masked softmax), FP32.
//
// No counterpart in the reference, whose only format choice is the
// user-supplied --morpheus-format flag (impl/Morpheus_Core.cpp:101-125).
// The six outputs follow formats_e (COO, CSR, DIA, ELL, HYB, HDC).
//
// Parameter blob (MGB_MLP_NPARAMS floats): W1[64][12], b1[64], W2[64][64],
// b2[64], W3[6][64], b3[6].  Inputs are standardised as (x - mu) / sigma.
// Formats whose conversion the reference would refuse (fill tolerance) are
// masked out of the softmax.
//
// Gradients are deterministic: each warp accumulates its samples into its own
// shared-memory slice, slices are summed in a fixed order per CTA, and CTA
// partials are summed in a fixed order by a final kernel.
#include "mgb_internal.cuh"

namespace mgb {
namespace {

constexpr int NF = 12, H = 64, NO = 6;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * NF, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + NO * H, NPARAMS = OFF_B3 + NO;
static_assert(NPARAMS == 5382, "parameter count");
constexpr int G_WARPS = 4;        // warps per CTA in the gradient kernel
constexpr int G_SAMPLES = 64;     // samples per CTA
constexpr float NEG = -1e30f;

struct Act {
  float z1[2], h1[2], z2[2], h2[2];  // this lane's hidden units l and l + 32
  float p[NO];                       // softmax (masked), identical in every lane
  float loss;
};

// forward pass of one sample by one warp; P = parameters (shared memory)
__device__ __forceinline__ void forward_warp(const float* P, const float* xn, const uint8_t* mask, float* sh,
                                             int lane, Act& a) {
  // layer 1
#pragma unroll
  for (int t = 0; t < 2; t++) {
    const int u = lane + 32 * t;
    float z = P[OFF_B1 + u];
#pragma unroll
    for (int i = 0; i < NF; i++) z = fmaf(P[OFF_W1 + u * NF + i], xn[i], z);
    a.z1[t] = z;
    a.h1[t] = fmaxf(z, 0.0f);
    sh[u] = a.h1[t];
  }
  __syncwarp();
  // layer 2
#pragma unroll
  for (int t = 0; t < 2; t++) {
    const int u = lane + 32 * t;
    float z = P[OFF_B2 + u];
    for (int i = 0; i < H; i++) z = fmaf(P[OFF_W2 + u * H + i], sh[i], z);
    a.z2[t] = z;
    a.h2[t] = fmaxf(z, 0.0f);
  }
  __syncwarp();
  sh[lane] = a.h2[0];
  sh[lane + 32] = a.h2[1];
  __syncwarp();
  // output layer: logits in every lane (6 dot products of length 64)
  float z3[NO];
  float mx = NEG;
#pragma unroll
  for (int o = 0; o < NO; o++) {
    float part = P[OFF_W3 + o * H + lane] * sh[lane] + P[OFF_W3 + o * H + lane + 32] * sh[lane + 32];
    part = warp_sum(part);
    z3[o] = part + P[OFF_B3 + o];
    if (mask && !mask[o]) z3[o] = NEG;
    mx = fmaxf(mx, z3[o]);
  }
  float s = 0.0f;
#pragma unroll
  for (int o = 0; o < NO; o++) {
    a.p[o] = (z3[o] <= NEG * 0.5f) ? 0.0f : __expf(z3[o] - mx);
    s += a.p[o];
  }
#pragma unroll
  for (int o = 0; o < NO; o++) a.p[o] /= s;
  __syncwarp();
}

__device__ __forceinline__ void standardise(const float* x, const float* mu, const float* sigma, float* xn) {
#pragma unroll
  for (int i = 0; i < NF; i++) xn[i] = (x[i] - mu[i]) / sigma[i];
}

__global__ void mlp_forward_kernel(const float* __restrict__ params, const float* __restrict__ mu,
                                   const float* __restrict__ sigma, const float* __restrict__ X,
                                   const uint8_t* __restrict__ mask, int64_t n, float* __restrict__ logits) {
  __shared__ float P[NPARAMS];
  __shared__ float sh[8][H];
  for (int i = threadIdx.x; i < NPARAMS; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t s = (int64_t)blockIdx.x * 8 + w; s < n; s += (int64_t)gridDim.x * 8) {
    float xn[NF];
    standardise(X + s * NF, mu, sigma, xn);
    Act a;
    forward_warp(P, xn, mask ? mask + s * NO : nullptr, sh[w], lane, a);
    // report log-probabilities (masked formats get a very negative value)
    if (lane < NO) logits[s * NO + lane] = a.p[lane] > 0.0f ? __logf(a.p[lane]) : NEG;
  }
}

// forward + backward for up to G_SAMPLES samples per CTA; writes the CTA's
// gradient sum and loss sum to partial[blockIdx.x]
__global__ void __launch_bounds__(G_WARPS * 32)
mlp_grad_kernel(const float* __restrict__ params, const float* __restrict__ mu, const float* __restrict__ sigma,
                const float* __restrict__ X, const int32_t* __restrict__ labels, const uint8_t* __restrict__ mask,
                int64_t n, float* __restrict__ partial, float* __restrict__ loss_partial) {
  extern __shared__ float smem[];
  float* P = smem;                            // NPARAMS
  float* G = P + NPARAMS;                     // G_WARPS * NPARAMS gradient slices
  float* SH = G + G_WARPS * NPARAMS;          // G_WARPS * H
  float* LS = SH + G_WARPS * H;               // G_WARPS losses
  for (int i = threadIdx.x; i < NPARAMS; i += blockDim.x) P[i] = params[i];
  for (int i = threadIdx.x; i < G_WARPS * NPARAMS; i += blockDim.x) G[i] = 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* g = G + w * NPARAMS;
  float* sh = SH + w * H;
  float loss = 0.0f;
  const int64_t s_begin = (int64_t)blockIdx.x * G_SAMPLES;
  const int64_t s_end = min(n, s_begin + G_SAMPLES);
  for (int64_t s = s_begin + w; s < s_end; s += G_WARPS) {
    float xn[NF];
    standardise(X + s * NF, mu, sigma, xn);
    const uint8_t* mk = mask ? mask + s * NO : nullptr;
    Act a;
    forward_warp(P, xn, mk, sh, lane, a);
    const int y = labels[s];
    loss += -__logf(fmaxf(a.p[y], 1e-30f));
    float dz3[NO];
#pragma unroll
    for (int o = 0; o < NO; o++) dz3[o] = a.p[o] - (o == y ? 1.0f : 0.0f);
    // h2 is in sh (from forward_warp); dW3, db3
#pragma unroll
    for (int o = 0; o < NO; o++) {
      g[OFF_W3 + o * H + lane] += dz3[o] * sh[lane];
      g[OFF_W3 + o * H + lane + 32] += dz3[o] * sh[lane + 32];
    }
    if (lane < NO) g[OFF_B3 + lane] += dz3[lane];
    // dh2 = W3^T dz3, dz2 = dh2 * relu'(z2)
    float dz2[2];
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const int u = lane + 32 * t;
      float d = 0.0f;
#pragma unroll
      for (int o = 0; o < NO; o++) d = fmaf(P[OFF_W3 + o * H + u], dz3[o], d);
      dz2[t] = a.z2[t] > 0.0f ? d : 0.0f;
    }
    __syncwarp();
    // restore h1 into sh for dW2
    sh[lane] = a.h1[0];
    sh[lane + 32] = a.h1[1];
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const int u = lane + 32 * t;
      for (int i = 0; i < H; i++) g[OFF_W2 + u * H + i] += dz2[t] * sh[i];
      g[OFF_B2 + u] += dz2[t];
    }
    __syncwarp();
    // dh1 = W2^T dz2 (needs every lane's dz2): share dz2 through sh
    sh[lane] = dz2[0];
    sh[lane + 32] = dz2[1];
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const int u = lane + 32 * t;  // hidden unit of layer 1
      float d = 0.0f;
      for (int k = 0; k < H; k++) d = fmaf(P[OFF_W2 + k * H + u], sh[k], d);
      const float dz1 = a.z1[t] > 0.0f ? d : 0.0f;
#pragma unroll
      for (int i = 0; i < NF; i++) g[OFF_W1 + u * NF + i] += dz1 * xn[i];
      g[OFF_B1 + u] += dz1;
    }
    __syncwarp();
  }
  if (lane == 0) LS[w] = loss;
  __syncthreads();
  // fixed-order sum of the warp slices
  for (int i = threadIdx.x; i < NPARAMS; i += blockDim.x) {
    float t = 0.0f;
    for (int k = 0; k < G_WARPS; k++) t += G[k * NPARAMS + i];
    partial[(int64_t)blockIdx.x * NPARAMS + i] = t;
  }
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int k = 0; k < G_WARPS; k++) t += LS[k];
    loss_partial[blockIdx.x] = t;
  }
}

__global__ void mlp_sum_partials(const float* __restrict__ partial, const float* __restrict__ loss_partial,
                                 int nblocks, float inv_n, float* __restrict__ grads, float* __restrict__ loss) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAMS; i += gridDim.x * blockDim.x) {
    float t = 0.0f;
    for (int b = 0; b < nblocks; b++) t += partial[(int64_t)b * NPARAMS + i];
    grads[i] = t * inv_n;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && loss) {
    float t = 0.0f;
    for (int b = 0; b < nblocks; b++) t += loss_partial[b];
    *loss = t * inv_n;
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

size_t grad_smem() { return sizeof(float) * (NPARAMS + G_WARPS * NPARAMS + G_WARPS * H + G_WARPS); }

int grad(const float* params, const float* mu, const float* sigma, const float* X, const int32_t* labels,
         const uint8_t* mask, int64_t n, float* grads, float* loss, cudaStream_t s) {
  MGB_REQUIRE(params && mu && sigma && X && labels && grads && n > 0, MGB_ERR_BAD_ARGUMENT);
  static bool attr_set[64] = {false};
  int dev = 0;
  MGB_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    MGB_CUDA_CHECK(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)grad_smem()));
    attr_set[dev] = true;
  }
  const int64_t nblocks = (n + G_SAMPLES - 1) / G_SAMPLES;
  float* scratch = nullptr;
  MGB_CUDA_CHECK(cudaMallocAsync((void**)&scratch, sizeof(float) * nblocks * (NPARAMS + 1), s));
  float* partial = scratch;
  float* lpart = scratch + nblocks * NPARAMS;
  mlp_grad_kernel<<<(unsigned)nblocks, G_WARPS * 32, grad_smem(), s>>>(params, mu, sigma, X, labels, mask, n,
                                                                        partial, lpart);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    mlp_sum_partials<<<(NPARAMS + 255) / 256, 256, 0, s>>>(partial, lpart, (int)nblocks, 1.0f / (float)n, grads,
                                                          loss);
    e = cudaGetLastError();
  }
  cudaError_t ef = cudaFreeAsync(scratch, s);
  if (e != cudaSuccess) return record_cuda_error(e);
  if (ef != cudaSuccess) return record_cuda_error(ef);
  return MGB_SUCCESS;
}

}  // namespace
}  // namespace mgb

extern "C" {

int mgb_mlp_num_params(void) { return mgb::NPARAMS; }

int mgb_mlp_forward_f32(const float* params, const float* mu, const float* sigma, const float* X,
                        const uint8_t* feasible, int64_t n, float* logp, void* stream) {
  MGB_REQUIRE(params && mu && sigma && X && logp && n >= 0, MGB_ERR_BAD_ARGUMENT);
  if (n == 0) return MGB_SUCCESS;
  const int64_t blocks = (n + 7) / 8;
  mgb::mlp_forward_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, mgb::as_stream(stream)>>>(
      params, mu, sigma, X, feasible, n, logp);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

int mgb_mlp_grad_f32(const float* params, const float* mu, const float* sigma, const float* X,
                     const int32_t* labels, const uint8_t* feasible, int64_t n, float* grads, float* loss,
                     void* stream) {
  return mgb::grad(params, mu, sigma, X, labels, feasible, n, grads, loss, mgb::as_stream(stream));
}

int mgb_mlp_adam_f32(float* params, const float* grads, float* m, float* v, int64_t nparams, float lr, float beta1,
                     float beta2, float eps, int step, void* stream) {
  MGB_REQUIRE(params && grads && m && v && nparams > 0 && step > 0, MGB_ERR_BAD_ARGUMENT);
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  mgb::adam_kernel<<<(unsigned)((nparams + 255) / 256), 256, 0, mgb::as_stream(stream)>>>(
      params, grads, m, v, nparams, lr, beta1, beta2, eps, c1, c2);
  MGB_LAUNCH_CHECK();
  return MGB_SUCCESS;
}

}  // extern "C"
