// Rank-predictor MLP (5 -> 64 -> 64 -> 64 -> 1, ReLU, sigmoid output), FP32,
// with hand-written inference, backward and Adam kernels (sm_103a).
//
// Parameters are one flat fp32 buffer (AGB_MLP_NPARAM floats):
//   W1[64][5] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4
// Forward:  h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), h3 = relu(W3 h2 + b3),
//           y = sigmoid(W4 h3 + b4).
// Loss (training): L = mean_b (y_b - t_b)^2.
// One thread per sample; the parameters are staged in shared memory.  The
// backward kernel accumulates each block's gradient in shared memory and adds
// it to the global gradient with one atomic per parameter per block.
#include "common.cuh"

namespace {

constexpr int IN = 5, H = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + H,
              NPARAM = OFF_B4 + 1;
static_assert(NPARAM == AGB_MLP_NPARAM, "parameter layout");

AGB_DEV void load_params(const float* __restrict__ p, float* sp) {
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sp[i] = p[i];
  __syncthreads();
}

// hidden activations of one sample; returns the output pre-activation
AGB_DEV float forward_one(const float* sp, const float* x, float* h1, float* h2, float* h3) {
#pragma unroll 4
  for (int o = 0; o < H; ++o) {
    float a = sp[OFF_B1 + o];
#pragma unroll
    for (int i = 0; i < IN; ++i) a = fmaf(sp[OFF_W1 + o * IN + i], x[i], a);
    h1[o] = fmaxf(a, 0.f);
  }
#pragma unroll 4
  for (int o = 0; o < H; ++o) {
    float a = sp[OFF_B2 + o];
    for (int i = 0; i < H; ++i) a = fmaf(sp[OFF_W2 + o * H + i], h1[i], a);
    h2[o] = fmaxf(a, 0.f);
  }
#pragma unroll 4
  for (int o = 0; o < H; ++o) {
    float a = sp[OFF_B3 + o];
    for (int i = 0; i < H; ++i) a = fmaf(sp[OFF_W3 + o * H + i], h2[i], a);
    h3[o] = fmaxf(a, 0.f);
  }
  float z = sp[OFF_B4];
  for (int i = 0; i < H; ++i) z = fmaf(sp[OFF_W4 + i], h3[i], z);
  return z;
}

AGB_DEV float sigmoid(float z) { return 1.f / (1.f + __expf(-z)); }

__global__ void __launch_bounds__(128) mlp_forward_kernel(const float* __restrict__ params, const float* __restrict__ X,
                                                          int B, float* __restrict__ Y) {
  __shared__ float sp[NPARAM];
  load_params(params, sp);
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float x[IN], h1[H], h2[H], h3[H];
#pragma unroll
  for (int i = 0; i < IN; ++i) x[i] = X[(int64_t)b * IN + i];
  Y[b] = sigmoid(forward_one(sp, x, h1, h2, h3));
}

// Forward + backward of the MSE loss for a batch, deterministic: every warp
// accumulates its lanes' contributions (warp shuffles, a fixed tree) into its
// own slice of shared memory, the block adds its four slices in warp order and
// writes one partial gradient row (and partial loss) per block to `part`;
// mlp_reduce_kernel then adds the rows in block order.  No float atomics, so a
// training run is reproducible bit for bit.
constexpr int BW = 128, NWARP = BW / 32;
__global__ void __launch_bounds__(BW) mlp_backward_kernel(const float* __restrict__ params, const float* __restrict__ X,
                                                          const float* __restrict__ T, int B, float inv_batch,
                                                          float* __restrict__ part, float* __restrict__ part_loss) {
  extern __shared__ float smem_f[];
  float* sp = smem_f;                              // [NPARAM]
  const int wid = threadIdx.x >> 5;
  float* sgw = smem_f + NPARAM * (1 + wid);       // this warp's gradient slice [NPARAM]
  for (int i = threadIdx.x; i < NWARP * NPARAM; i += blockDim.x) smem_f[NPARAM + i] = 0.f;
  load_params(params, sp);
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const bool lane0 = (threadIdx.x & 31) == 0;
  const bool live = b < B;
  float x[IN], h1[H], h2[H], h3[H];
#pragma unroll
  for (int i = 0; i < IN; ++i) x[i] = live ? X[(int64_t)b * IN + i] : 0.f;
  const float y = sigmoid(forward_one(sp, x, h1, h2, h3));
  const float t = live ? T[b] : y;
  const float err2 = (y - t) * (y - t);
  const float dz = 2.f * (y - t) * inv_batch * y * (1.f - y);
  // layer 4: z = W4 h3 + b4
  {
    const float r = warp_sum(dz);
    if (lane0) sgw[OFF_B4] += r;
  }
  float d3[H];
  for (int i = 0; i < H; ++i) {
    const float r = warp_sum(dz * h3[i]);
    if (lane0) sgw[OFF_W4 + i] += r;
    d3[i] = (h3[i] > 0.f) ? dz * sp[OFF_W4 + i] : 0.f;
  }
  // layer 3: h3 = relu(W3 h2 + b3)
  float d2[H];
  for (int i = 0; i < H; ++i) d2[i] = 0.f;
  for (int o = 0; o < H; ++o) {
    const float g = d3[o];
    const float rb = warp_sum(g);
    if (lane0) sgw[OFF_B3 + o] += rb;
    for (int i = 0; i < H; ++i) {
      const float r = warp_sum(g * h2[i]);
      if (lane0) sgw[OFF_W3 + o * H + i] += r;
      d2[i] = fmaf(g, sp[OFF_W3 + o * H + i], d2[i]);
    }
  }
  for (int i = 0; i < H; ++i)
    if (h2[i] <= 0.f) d2[i] = 0.f;
  // layer 2: h2 = relu(W2 h1 + b2)
  float d1[H];
  for (int i = 0; i < H; ++i) d1[i] = 0.f;
  for (int o = 0; o < H; ++o) {
    const float g = d2[o];
    const float rb = warp_sum(g);
    if (lane0) sgw[OFF_B2 + o] += rb;
    for (int i = 0; i < H; ++i) {
      const float r = warp_sum(g * h1[i]);
      if (lane0) sgw[OFF_W2 + o * H + i] += r;
      d1[i] = fmaf(g, sp[OFF_W2 + o * H + i], d1[i]);
    }
  }
  // layer 1: h1 = relu(W1 x + b1)
  for (int o = 0; o < H; ++o) {
    const float g = (h1[o] > 0.f) ? d1[o] : 0.f;
    const float rb = warp_sum(g);
    if (lane0) sgw[OFF_B1 + o] += rb;
#pragma unroll
    for (int i = 0; i < IN; ++i) {
      const float r = warp_sum(g * x[i]);
      if (lane0) sgw[OFF_W1 + o * IN + i] += r;
    }
  }
  __shared__ float red[32];
  const float tot = block_sum(live ? err2 : 0.f, red);  // fixed tree (ends with a barrier)
  float* row = part + (int64_t)blockIdx.x * NPARAM;
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) {
    float acc = 0.f;
#pragma unroll
    for (int w = 0; w < NWARP; ++w) acc += smem_f[NPARAM * (1 + w) + i];
    row[i] = acc;
  }
  if (threadIdx.x == 0) part_loss[blockIdx.x] = tot;
}

// grads[i] = sum over blocks (in block order) of part[block][i]; loss likewise.
__global__ void mlp_reduce_kernel(const float* __restrict__ part, const float* __restrict__ part_loss, int nblocks,
                                  float* __restrict__ grads, float* __restrict__ loss_sum) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NPARAM) {
    float acc = 0.f;
    for (int b = 0; b < nblocks; ++b) acc += part[(int64_t)b * NPARAM + i];
    grads[i] = acc;
  }
  if (i == 0 && loss_sum) {
    float l = 0.f;
    for (int b = 0; b < nblocks; ++b) l += part_loss[b];
    *loss_sum = l;
  }
}

// Adam with decoupled weight decay (AdamW): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
// p -= lr * (mhat / (sqrt(vhat) + eps) + wd * p).
__global__ void mlp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float wd,
                                float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / c1, vh = vi / c2;
  p[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * p[i]);
}

}  // namespace

extern "C" int agb_mlp_forward(const float* params, const float* X, int B, float* Y, void* stream) {
  if (!params || !X || !Y || B < 0) return AGB_ERR_ARG;
  if (B == 0) return AGB_OK;
  mlp_forward_kernel<<<(B + 127) / 128, 128, 0, (cudaStream_t)stream>>>(params, X, B, Y);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

extern "C" size_t agb_mlp_backward_workspace(int B) {
  const size_t nb = B > 0 ? (size_t)(B + BW - 1) / BW : 0;
  return agb_align(nb * NPARAM * sizeof(float)) + agb_align(nb * sizeof(float));
}

extern "C" int agb_mlp_backward(const float* params, const float* X, const float* T, int B, float* grads,
                                float* loss_sum, void* ws, size_t ws_bytes, void* stream) {
  if (!params || !X || !T || !grads || B <= 0 || !ws) return AGB_ERR_ARG;
  if (ws_bytes < agb_mlp_backward_workspace(B)) return AGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = (B + BW - 1) / BW;
  float* part = (float*)ws;
  float* part_loss = (float*)((char*)ws + agb_align((size_t)nb * NPARAM * sizeof(float)));
  const size_t smem = (size_t)(1 + NWARP) * NPARAM * sizeof(float);
  const cudaError_t oe = agb_smem_optin(mlp_backward_kernel, smem);
  if (oe != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, oe);
    return AGB_ERR_CUDA;
  }
  mlp_backward_kernel<<<nb, BW, smem, s>>>(params, X, T, B, 1.f / (float)B, part, part_loss);
  AGB_CHECK_LAUNCH();
  mlp_reduce_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(part, part_loss, nb, grads, loss_sum);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

extern "C" int agb_mlp_adam(float* params, const float* grads, float* m, float* v, int step, float lr, float beta1,
                            float beta2, float eps, float weight_decay, void* stream) {
  if (!params || !grads || !m || !v || step <= 0) return AGB_ERR_ARG;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  mlp_adam_kernel<<<(NPARAM + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, NPARAM, lr, beta1,
                                                                         beta2, eps, weight_decay, c1, c2);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
