// The warm-start network: a 3-layer MLP (BF16 weights and activations, FP32 accumulation)
// trained on the device with hand-written forward, backward and Adam kernels.
//
//   h1 = relu(x W1^T + b1),  h2 = relu(h1 W2^T + b2),  y = h2 W3^T + b3
//   loss = mean((y - t)^2)
//
// FP32 master weights and Adam moments; BF16 copies of the weights feed the GEMMs, and the
// activations are stored in BF16 (the GEMM inputs of the next layer and of the backward
// pass).  One GEMM kernel covers every product of the forward and backward passes through
// element strides: C[M][N] (+)= sum_k A(m, k) B(k, n), A and B in BF16, FP32 accumulation.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cpals_internal.cuh"

namespace cpals {
namespace {

constexpr int GM = 64, GN = 64, GK = 32;  // block tile
constexpr int GTHREADS = 256;             // 16 x 16 threads, 4 x 4 outputs each

// C[m][n] = alpha * sum_k A[m*sam + k*sak] * B[k*sbk + n*sbn] (+ beta * C), row-major C (ldc)
__global__ void __launch_bounds__(GTHREADS) k_gemm_bf16(const __nv_bfloat16* __restrict__ A, int64_t sam,
                                                        int64_t sak, const __nv_bfloat16* __restrict__ B, int64_t sbk,
                                                        int64_t sbn, float* __restrict__ C, int64_t ldc, int M, int N,
                                                        int K, float beta) {
  __shared__ float As[GK][GM + 4];
  __shared__ float Bs[GK][GN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * GM, n0 = blockIdx.x * GN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += GK) {
    for (int e = threadIdx.x; e < GK * GM; e += GTHREADS) {
      const int kk = e / GM, mm = e % GM;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? __bfloat162float(A[(int64_t)m * sam + (int64_t)k * sak]) : 0.f;
    }
    for (int e = threadIdx.x; e < GK * GN; e += GTHREADS) {
      const int kk = e / GN, nn = e % GN;
      const int n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = (n < N && k < K) ? __bfloat162float(B[(int64_t)k * sbk + (int64_t)n * sbn]) : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < M && n < N) {
        float* c = &C[(int64_t)m * ldc + n];
        *c = (beta != 0.f ? beta * *c : 0.f) + acc[i][j];
      }
    }
}

// Y (FP32 [B][N]) += bias; optional ReLU; BF16 copy for the next GEMM.
__global__ void k_bias_act(float* __restrict__ Y, const float* __restrict__ bias, int B, int N, int relu,
                           __nv_bfloat16* __restrict__ Yb) {
  const int64_t n = (int64_t)B * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    float v = Y[e] + bias[e % N];
    if (relu) v = fmaxf(v, 0.f);
    Y[e] = v;
    if (Yb) Yb[e] = __float2bfloat16_rn(v);
  }
}

// dY = 2 (Y - T) / (B N) (mean squared error), loss partial sums per block
__global__ void k_mse_grad(const float* __restrict__ Y, const float* __restrict__ T, int64_t n, float scale,
                           __nv_bfloat16* __restrict__ dYb, float* __restrict__ dY, double* __restrict__ loss) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[e] - T[e];
    s += (double)d * d;
    const float g = 2.f * d * scale;
    dY[e] = g;
    dYb[e] = __float2bfloat16_rn(g);
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (threadIdx.x == 0) loss[blockIdx.x] = t;
  }
}

// dH (FP32 [B][N], the product dY W) *= (H > 0); BF16 copy
__global__ void k_relu_back(float* __restrict__ dH, const __nv_bfloat16* __restrict__ H, int64_t n,
                            __nv_bfloat16* __restrict__ dHb) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float g = (__bfloat162float(H[e]) > 0.f) ? dH[e] : 0.f;
    dH[e] = g;
    dHb[e] = __float2bfloat16_rn(g);
  }
}

// db[n] = sum_b dY[b][n] (fixed order over the batch)
__global__ void k_bias_grad(const float* __restrict__ dY, int B, int N, float* __restrict__ db) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += dY[(int64_t)b * N + n];
    db[n] = s;
  }
}

// Adam (Kingma and Ba 2015) on the FP32 master parameters; BF16 copy of the weights
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int64_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ pb) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float a = b1 * m1[e] + (1.f - b1) * gg;
    const float b = b2 * m2[e] + (1.f - b2) * gg * gg;
    m1[e] = a;
    m2[e] = b;
    const float v = p[e] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    p[e] = v;
    if (pb) pb[e] = __float2bfloat16_rn(v);
  }
}

__global__ void k_to_bf16(const float* __restrict__ x, int64_t n, __nv_bfloat16* __restrict__ y) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    y[e] = __float2bfloat16_rn(x[e]);
}

// gather rows idx[b] of a device dataset (FP32 [N][W]) into X (FP32 and BF16 [B][W])
__global__ void k_gather_rows(const float* __restrict__ D, int W, const int* __restrict__ idx, int B,
                              float* __restrict__ X, __nv_bfloat16* __restrict__ Xb) {
  const int64_t n = (int64_t)B * W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / W), w = (int)(e % W);
    const float v = D[(int64_t)idx[b] * W + w];
    if (X) X[e] = v;
    if (Xb) Xb[e] = __float2bfloat16_rn(v);
  }
}

int grid1(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

}  // namespace
}  // namespace cpals

using namespace cpals;

struct cpals_mlp {
  int device = 0;
  int w[4] = {};  // in, h1, h2, out
  int64_t np = 0;
  int64_t off[6] = {};  // W1 b1 W2 b2 W3 b3 offsets into the parameter vector
  float* p = nullptr;   // FP32 master parameters
  float* g = nullptr;   // gradients
  float* m1 = nullptr;
  float* m2 = nullptr;
  __nv_bfloat16* pb = nullptr;  // BF16 copy (weights used by the GEMMs)
  int bcap = 0;
  float *x = nullptr, *t = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr, *dy = nullptr, *dh2 = nullptr,
        *dh1 = nullptr;
  __nv_bfloat16 *xb = nullptr, *h1b = nullptr, *h2b = nullptr, *dyb = nullptr, *dh2b = nullptr, *dh1b = nullptr;
  double* loss = nullptr;
  int* idx = nullptr;
  float* dx = nullptr;  // device dataset inputs [N][in]
  float* dt = nullptr;  // device dataset targets [N][out]
  int64_t dn = 0;
  int64_t step = 0;
  cudaStream_t st = nullptr;
};

namespace {

void gemm(cpals_mlp* m, const __nv_bfloat16* A, int64_t sam, int64_t sak, const __nv_bfloat16* B, int64_t sbk,
          int64_t sbn, float* C, int64_t ldc, int M, int N, int K) {
  dim3 grid((N + GN - 1) / GN, (M + GM - 1) / GM);
  k_gemm_bf16<<<grid, GTHREADS, 0, m->st>>>(A, sam, sak, B, sbk, sbn, C, ldc, M, N, K, 0.f);
}

int ensure_batch(cpals_mlp* m, int B) {
  if (B <= m->bcap) return CPALS_OK;
  cudaFree(m->x);
  cudaFree(m->t);
  cudaFree(m->h1);
  cudaFree(m->h2);
  cudaFree(m->y);
  cudaFree(m->dy);
  cudaFree(m->dh2);
  cudaFree(m->dh1);
  cudaFree(m->xb);
  cudaFree(m->h1b);
  cudaFree(m->h2b);
  cudaFree(m->dyb);
  cudaFree(m->dh2b);
  cudaFree(m->dh1b);
  cudaFree(m->loss);
  cudaFree(m->idx);
  const int64_t in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  bool ok = cudaMalloc(&m->x, 4 * B * in) == cudaSuccess && cudaMalloc(&m->t, 4 * B * o) == cudaSuccess &&
            cudaMalloc(&m->h1, 4 * B * a) == cudaSuccess && cudaMalloc(&m->h2, 4 * B * b) == cudaSuccess &&
            cudaMalloc(&m->y, 4 * B * o) == cudaSuccess && cudaMalloc(&m->dy, 4 * B * o) == cudaSuccess &&
            cudaMalloc(&m->dh2, 4 * B * b) == cudaSuccess && cudaMalloc(&m->dh1, 4 * B * a) == cudaSuccess &&
            cudaMalloc(&m->xb, 2 * B * in) == cudaSuccess && cudaMalloc(&m->h1b, 2 * B * a) == cudaSuccess &&
            cudaMalloc(&m->h2b, 2 * B * b) == cudaSuccess && cudaMalloc(&m->dyb, 2 * B * o) == cudaSuccess &&
            cudaMalloc(&m->dh2b, 2 * B * b) == cudaSuccess && cudaMalloc(&m->dh1b, 2 * B * a) == cudaSuccess &&
            cudaMalloc(&m->loss, sizeof(double) * 4096) == cudaSuccess &&
            cudaMalloc(&m->idx, sizeof(int) * B) == cudaSuccess;
  if (!ok) return CPALS_E_CUDA;
  m->bcap = B;
  return CPALS_OK;
}

// forward pass on m->xb (BF16 [B][in]); y, h1, h2 (FP32) and BF16 copies
void forward(cpals_mlp* m, int B) {
  const int in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  const __nv_bfloat16* W1 = m->pb + m->off[0];
  const __nv_bfloat16* W2 = m->pb + m->off[2];
  const __nv_bfloat16* W3 = m->pb + m->off[4];
  // h1[b][j] = sum_k x[b][k] W1[j][k]
  gemm(m, m->xb, in, 1, W1, 1, in, m->h1, a, B, a, in);
  k_bias_act<<<grid1((int64_t)B * a), 256, 0, m->st>>>(m->h1, m->p + m->off[1], B, a, 1, m->h1b);
  gemm(m, m->h1b, a, 1, W2, 1, a, m->h2, b, B, b, a);
  k_bias_act<<<grid1((int64_t)B * b), 256, 0, m->st>>>(m->h2, m->p + m->off[3], B, b, 1, m->h2b);
  gemm(m, m->h2b, b, 1, W3, 1, b, m->y, o, B, o, b);
  k_bias_act<<<grid1((int64_t)B * o), 256, 0, m->st>>>(m->y, m->p + m->off[5], B, o, 0, nullptr);
}

// backward pass (targets in m->t), gradients into m->g; returns the block loss partials count
int backward(cpals_mlp* m, int B) {
  const int in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  const __nv_bfloat16* W2 = m->pb + m->off[2];
  const __nv_bfloat16* W3 = m->pb + m->off[4];
  const int64_t ny = (int64_t)B * o;
  const int lb = grid1(ny);
  k_mse_grad<<<lb, 256, 0, m->st>>>(m->y, m->t, ny, 1.f / (float)ny, m->dyb, m->dy, m->loss);
  // dW3[i][j] = sum_b dy[b][i] h2[b][j];  db3 = sum_b dy
  gemm(m, m->dyb, 1, o, m->h2b, b, 1, m->g + m->off[4], b, o, b, B);
  k_bias_grad<<<(o + 255) / 256, 256, 0, m->st>>>(m->dy, B, o, m->g + m->off[5]);
  // dh2[b][j] = sum_i dy[b][i] W3[i][j], masked
  gemm(m, m->dyb, o, 1, W3, b, 1, m->dh2, b, B, b, o);
  k_relu_back<<<grid1((int64_t)B * b), 256, 0, m->st>>>(m->dh2, m->h2b, (int64_t)B * b, m->dh2b);
  gemm(m, m->dh2b, 1, b, m->h1b, a, 1, m->g + m->off[2], a, b, a, B);
  k_bias_grad<<<(b + 255) / 256, 256, 0, m->st>>>(m->dh2, B, b, m->g + m->off[3]);
  gemm(m, m->dh2b, b, 1, W2, a, 1, m->dh1, a, B, a, b);
  k_relu_back<<<grid1((int64_t)B * a), 256, 0, m->st>>>(m->dh1, m->h1b, (int64_t)B * a, m->dh1b);
  gemm(m, m->dh1b, 1, a, m->xb, in, 1, m->g + m->off[0], in, a, in, B);
  k_bias_grad<<<(a + 255) / 256, 256, 0, m->st>>>(m->dh1, B, a, m->g + m->off[1]);
  return lb;
}

double read_loss(cpals_mlp* m, int nblocks) {
  std::vector<double> h(nblocks);
  cudaMemcpyAsync(h.data(), m->loss, sizeof(double) * nblocks, cudaMemcpyDeviceToHost, m->st);
  cudaStreamSynchronize(m->st);
  double s = 0.0;
  for (double v : h) s += v;
  return s;
}

void adam(cpals_mlp* m, float lr) {
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
  k_adam<<<grid1(m->np), 256, 0, m->st>>>(m->p, m->g, m->m1, m->m2, m->np, lr, b1, b2, 1e-8f, c1, c2, m->pb);
}

}  // namespace

extern "C" {

int cpals_mlp_create(cpals_mlp** out, int device, const int* widths) {
  if (!out || !widths) return CPALS_E_ARG;
  for (int i = 0; i < 4; ++i)
    if (widths[i] < 1 || widths[i] > 65536) return CPALS_E_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPALS_E_CUDA;
  DeviceGuard guard(device);
  cpals_mlp* m = new cpals_mlp();
  m->device = device;
  for (int i = 0; i < 4; ++i) m->w[i] = widths[i];
  int64_t o = 0;
  for (int l = 0; l < 3; ++l) {
    m->off[2 * l] = o;
    o += (int64_t)m->w[l + 1] * m->w[l];
    m->off[2 * l + 1] = o;
    o += m->w[l + 1];
  }
  m->np = o;
  bool ok = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&m->p, 4 * o) == cudaSuccess && cudaMalloc(&m->g, 4 * o) == cudaSuccess &&
            cudaMalloc(&m->m1, 4 * o) == cudaSuccess && cudaMalloc(&m->m2, 4 * o) == cudaSuccess &&
            cudaMalloc(&m->pb, 2 * o) == cudaSuccess;
  if (!ok) {
    cpals_mlp_destroy(m);
    return CPALS_E_CUDA;
  }
  cudaMemset(m->p, 0, 4 * o);
  cudaMemset(m->g, 0, 4 * o);
  cudaMemset(m->m1, 0, 4 * o);
  cudaMemset(m->m2, 0, 4 * o);
  cudaMemset(m->pb, 0, 2 * o);
  *out = m;
  return CPALS_OK;
}

int cpals_mlp_destroy(cpals_mlp* m) {
  if (!m) return CPALS_OK;
  DeviceGuard guard(m->device);
  for (void* q : {(void*)m->p, (void*)m->g, (void*)m->m1, (void*)m->m2, (void*)m->pb, (void*)m->x, (void*)m->t,
                  (void*)m->h1, (void*)m->h2, (void*)m->y, (void*)m->dy, (void*)m->dh2, (void*)m->dh1,
                  (void*)m->xb, (void*)m->h1b, (void*)m->h2b, (void*)m->dyb, (void*)m->dh2b, (void*)m->dh1b,
                  (void*)m->loss, (void*)m->idx, (void*)m->dx, (void*)m->dt})
    cudaFree(q);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return CPALS_OK;
}

int64_t cpals_mlp_num_params(cpals_mlp* m) { return m ? m->np : -1; }

// FP32 parameters: W1 [h1][in], b1, W2 [h2][h1], b2, W3 [out][h2], b3; resets Adam.
int cpals_mlp_set_params(cpals_mlp* m, const float* host_params) {
  if (!m || !host_params) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->p, host_params, 4 * m->np, cudaMemcpyHostToDevice, m->st));
  CPALS_CUDA_TRY(cudaMemsetAsync(m->m1, 0, 4 * m->np, m->st));
  CPALS_CUDA_TRY(cudaMemsetAsync(m->m2, 0, 4 * m->np, m->st));
  k_to_bf16<<<grid1(m->np), 256, 0, m->st>>>(m->p, m->np, m->pb);
  m->step = 0;
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));
  return CPALS_OK;
}

int cpals_mlp_get_params(cpals_mlp* m, float* host_params) {
  if (!m || !host_params) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_params, m->p, 4 * m->np, cudaMemcpyDeviceToHost, m->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));
  return CPALS_OK;
}

// Forward pass of B host inputs (FP32 [B][in]) into host outputs (FP32 [B][out]).
int cpals_mlp_forward(cpals_mlp* m, const float* host_x, int B, float* host_y) {
  if (!m || !host_x || !host_y || B < 1) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  if (ensure_batch(m, B) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->x, host_x, 4LL * B * m->w[0], cudaMemcpyHostToDevice, m->st));
  k_to_bf16<<<grid1((int64_t)B * m->w[0]), 256, 0, m->st>>>(m->x, (int64_t)B * m->w[0], m->xb);
  forward(m, B);
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_y, m->y, 4LL * B * m->w[3], cudaMemcpyDeviceToHost, m->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));
  return CPALS_OK;
}

// Loss and gradients (FP32, same layout as the parameters) of one host batch, no update.
int cpals_mlp_gradients(cpals_mlp* m, const float* host_x, const float* host_t, int B, float* host_grads,
                        double* loss_out) {
  if (!m || !host_x || !host_t || !host_grads || B < 1) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  if (ensure_batch(m, B) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->x, host_x, 4LL * B * m->w[0], cudaMemcpyHostToDevice, m->st));
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->t, host_t, 4LL * B * m->w[3], cudaMemcpyHostToDevice, m->st));
  k_to_bf16<<<grid1((int64_t)B * m->w[0]), 256, 0, m->st>>>(m->x, (int64_t)B * m->w[0], m->xb);
  forward(m, B);
  const int lb = backward(m, B);
  const double l = read_loss(m, lb);
  if (loss_out) *loss_out = l / ((double)B * m->w[3]);
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_grads, m->g, 4 * m->np, cudaMemcpyDeviceToHost, m->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));
  return CPALS_OK;
}

// Device copy of a training set (FP32 inputs [N][in], targets [N][out]).
int cpals_mlp_set_dataset(cpals_mlp* m, const float* host_x, const float* host_t, int64_t N) {
  if (!m || !host_x || !host_t || N < 1) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  cudaFree(m->dx);
  cudaFree(m->dt);
  m->dx = m->dt = nullptr;
  if (cudaMalloc(&m->dx, 4 * N * m->w[0]) != cudaSuccess || cudaMalloc(&m->dt, 4 * N * m->w[3]) != cudaSuccess)
    return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->dx, host_x, 4 * N * m->w[0], cudaMemcpyHostToDevice, m->st));
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->dt, host_t, 4 * N * m->w[3], cudaMemcpyHostToDevice, m->st));
  m->dn = N;
  return CPALS_OK;
}

// `steps` Adam steps on batches of B rows of the device dataset; batch s uses rows
// idx[s*B .. s*B+B-1].  losses (may be null) receives each step's mean loss.
int cpals_mlp_train(cpals_mlp* m, const int* host_idx, int steps, int B, float lr, double* losses) {
  if (!m || !host_idx || steps < 1 || B < 1 || !m->dx) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  if (ensure_batch(m, B) != CPALS_OK) return CPALS_E_CUDA;
  for (int64_t i = 0; i < (int64_t)steps * B; ++i)
    if (host_idx[i] < 0 || host_idx[i] >= m->dn) return CPALS_E_ARG;
  for (int s = 0; s < steps; ++s) {
    CPALS_CUDA_TRY(cudaMemcpyAsync(m->idx, host_idx + (int64_t)s * B, sizeof(int) * B, cudaMemcpyHostToDevice, m->st));
    k_gather_rows<<<grid1((int64_t)B * m->w[0]), 256, 0, m->st>>>(m->dx, m->w[0], m->idx, B, nullptr, m->xb);
    k_gather_rows<<<grid1((int64_t)B * m->w[3]), 256, 0, m->st>>>(m->dt, m->w[3], m->idx, B, m->t, nullptr);
    forward(m, B);
    const int lb = backward(m, B);
    adam(m, lr);
    if (losses) losses[s] = read_loss(m, lb) / ((double)B * m->w[3]);
  }
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));
  return CPALS_OK;
}

}  // extern "C"
