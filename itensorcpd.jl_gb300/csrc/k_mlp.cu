// The warm-start network: a 3-layer MLP (BF16 weights and activations, FP32 accumulation)
// trained on the device with hand-written forward, backward and Adam kernels.
//
//   h1 = relu(x W1^T + b1),  h2 = relu(h1 W2^T + b2),  y = h2 W3^T + b3
//   loss = mean((y - t)^2)
//
// FP32 master weights and Adam moments.  Every product of the forward and backward passes
// runs on the tensor cores (k_gemm_tc.cu: tcgen05.mma.kind::f16, BF16 operands, FP32
// accumulation in TMEM), over split-K slices that the epilogue kernel sums in a fixed order
// while it adds the bias, applies the activation or the ReLU mask and writes the BF16
// panels the next GEMMs read: activations and gradients both as they are and transposed
// (the weight gradients reduce over the batch), weights as W and W^T.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cpals_internal.cuh"
#include "gemm_tc.cuh"

namespace cpals {
namespace {

// dY = 2 (Y - T) / (B N) (mean squared error), loss partial sums per block
__global__ void k_mse_grad(const float* __restrict__ Y, const float* __restrict__ T, int64_t n, float scale,
                           float* __restrict__ dY, double* __restrict__ loss) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[e] - T[e];
    s += (double)d * d;
    const float g = 2.f * d * scale;
    dY[e] = g;
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

// db[n] = sum_b dY[b][n] (fixed order over the batch)
__global__ void k_bias_grad(const float* __restrict__ dY, int B, int N, float* __restrict__ db) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += dY[(int64_t)b * N + n];
    db[n] = s;
  }
}

// The training step's position, on the device so that one captured step serves every step:
// k = step within the current cpals_mlp_train call (index offset and loss slot), t = Adam's
// step count before this step.
struct MlpStep {
  long long k;
  long long t;
};

constexpr int kLossSlots = 64;  // steps whose loss partials are kept before a read-back

// gather rows idx[k * B + b] of a device dataset (FP32 [N][W]) into X (FP32 [B][W])
__global__ void k_gather_step(const float* __restrict__ D, int W, const int* __restrict__ idx, int B,
                              float* __restrict__ X, const MlpStep* __restrict__ st) {
  const int* ix = idx + st->k * B;
  const int64_t n = (int64_t)B * W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / W), w = (int)(e % W);
    X[e] = D[(int64_t)ix[b] * W + w];
  }
}

// Adam (Kingma and Ba 2015) on the FP32 master parameters, with the bias corrections of step
// t + 1 formed on the device
__global__ void k_adam_step(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, int64_t n, float lr, float b1, float b2, float eps,
                            const MlpStep* __restrict__ st) {
  const float t = (float)(st->t + 1);
  const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float a = b1 * m1[e] + (1.f - b1) * gg;
    const float b = b2 * m2[e] + (1.f - b2) * gg * gg;
    m1[e] = a;
    m2[e] = b;
    const float v = p[e] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    p[e] = v;
  }
}

__global__ void k_step_end(MlpStep* st) {
  st->k += 1;
  st->t += 1;
}

// the loss partials of step k go to slot k % kLossSlots
__global__ void k_mse_grad_step(const float* __restrict__ Y, const float* __restrict__ T, int64_t n, float scale,
                                float* __restrict__ dY, double* __restrict__ loss, int lb, const MlpStep* __restrict__ st) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[e] - T[e];
    s += (double)d * d;
    const float g = 2.f * d * scale;
    dY[e] = g;
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (threadIdx.x == 0) loss[(st->k % kLossSlots) * lb + blockIdx.x] = t;
  }
}

int grid1(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

}  // namespace
}  // namespace cpals

using namespace cpals;

struct cpals_mlp {
  int device = 0;
  int sms = 1;
  int w[4] = {};  // in, h1, h2, out
  int64_t np = 0;
  int64_t off[6] = {};  // W1 b1 W2 b2 W3 b3 offsets into the parameter vector
  float* p = nullptr;   // FP32 master parameters
  float* g = nullptr;   // gradients
  float* m1 = nullptr;
  float* m2 = nullptr;
  // weight panels: W_l as [out][in] (forward) and W_l^T (backward; layers 2 and 3)
  __nv_bfloat16 *W1p = nullptr, *W2p = nullptr, *W2t = nullptr, *W3p = nullptr, *W3t = nullptr;
  int bcap = 0;
  float *x = nullptr, *t = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr, *dy = nullptr, *dh2 = nullptr,
        *dh1 = nullptr;
  // activation / gradient panels: p = as stored ([batch][features]), t = transposed
  __nv_bfloat16 *Xp = nullptr, *Xt = nullptr, *H1p = nullptr, *H1t = nullptr, *H2p = nullptr, *H2t = nullptr,
                *DYp = nullptr, *DYt = nullptr, *DH2p = nullptr, *DH2t = nullptr, *DH1t = nullptr;
  float* part = nullptr;  // split-K partial sums
  double* loss = nullptr;  // per-block loss partials
  int* err = nullptr;      // the GEMM's error word (2 ints)
  int* idx = nullptr;
  int64_t idx_cap = 0;
  float* dx = nullptr;  // device dataset inputs [N][in]
  float* dt = nullptr;  // device dataset targets [N][out]
  int64_t dn = 0;
  int64_t step = 0;
  double train_ms = 0.0;  // device time of the last cpals_mlp_train call (its launches only)
  MlpStep* dstep = nullptr;             // the device step state
  cudaGraphExec_t step_graph = nullptr;  // one captured training step
  int graph_B = 0;
  float graph_lr = 0.f;
  const int* graph_idx = nullptr;
  const float* graph_dx = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t st = nullptr;
};

namespace {

// C = A B^T on the tensor cores (A: M x K panel, B: N x K panel), then the epilogue
cudaError_t gemm(cpals_mlp* m, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const float* bias,
                 int mode, const float* mask, float* out32, __nv_bfloat16* prm, __nv_bfloat16* ptr) {
  const int sp = gemm_tc_splits(M, N, K, m->sms);
  cudaError_t e = gemm_tc_launch(A, B, M, N, K, sp, m->part, m->err, m->st);
  if (e != cudaSuccess) return e;
  return gemm_tc_epilogue(m->part, sp, M, N, bias, mode, mask, out32, prm, ptr, m->st);
}

// pack a row-major FP32 matrix [M][N] into its panels
cudaError_t pack(cpals_mlp* m, const float* src, int M, int N, __nv_bfloat16* prm, __nv_bfloat16* ptr) {
  return gemm_tc_epilogue(src, 1, M, N, nullptr, 0, nullptr, nullptr, prm, ptr, m->st);
}

// split-K partial floats the 8 products of a batch of B need
int64_t part_floats(const cpals_mlp* m, int B) {
  const int in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  const int shapes[8][3] = {{B, a, in}, {B, b, a}, {B, o, b}, {o, b, B}, {B, b, o}, {b, a, B}, {B, a, b}, {a, in, B}};
  int64_t need = 0;
  for (const auto& sh : shapes)
    need = std::max(need, (int64_t)gemm_tc_splits(sh[0], sh[1], sh[2], m->sms) * sh[0] * sh[1]);
  return need;
}

template <typename T>
bool alloc0(T** q, int64_t elems) {
  *q = nullptr;
  if (cudaMalloc(q, sizeof(T) * (size_t)std::max<int64_t>(elems, 1)) != cudaSuccess) return false;
  return cudaMemset(*q, 0, sizeof(T) * (size_t)std::max<int64_t>(elems, 1)) == cudaSuccess;
}

void free_batch(cpals_mlp* m) {
  for (void* q : {(void*)m->x, (void*)m->t, (void*)m->h1, (void*)m->h2, (void*)m->y, (void*)m->dy, (void*)m->dh2,
                  (void*)m->dh1, (void*)m->Xp, (void*)m->Xt, (void*)m->H1p, (void*)m->H1t, (void*)m->H2p,
                  (void*)m->H2t, (void*)m->DYp, (void*)m->DYt, (void*)m->DH2p, (void*)m->DH2t, (void*)m->DH1t,
                  (void*)m->part, (void*)m->loss})
    cudaFree(q);
  m->x = m->t = m->h1 = m->h2 = m->y = m->dy = m->dh2 = m->dh1 = m->part = nullptr;
  m->Xp = m->Xt = m->H1p = m->H1t = m->H2p = m->H2t = m->DYp = m->DYt = m->DH2p = m->DH2t = m->DH1t = nullptr;
  m->loss = nullptr;
  m->bcap = 0;
}

void drop_step_graph(cpals_mlp* m);

int ensure_batch(cpals_mlp* m, int B) {
  if (B <= m->bcap) return CPALS_OK;
  drop_step_graph(m);  // it holds the old buffers
  free_batch(m);
  const int64_t in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  bool ok = alloc0(&m->x, B * in) && alloc0(&m->t, B * o) && alloc0(&m->h1, B * a) && alloc0(&m->h2, B * b) &&
            alloc0(&m->y, B * o) && alloc0(&m->dy, B * o) && alloc0(&m->dh2, B * b) && alloc0(&m->dh1, B * a) &&
            alloc0(&m->Xp, panel_elems(B, in)) && alloc0(&m->Xt, panel_elems(in, B)) &&
            alloc0(&m->H1p, panel_elems(B, a)) && alloc0(&m->H1t, panel_elems(a, B)) &&
            alloc0(&m->H2p, panel_elems(B, b)) && alloc0(&m->H2t, panel_elems(b, B)) &&
            alloc0(&m->DYp, panel_elems(B, o)) && alloc0(&m->DYt, panel_elems(o, B)) &&
            alloc0(&m->DH2p, panel_elems(B, b)) && alloc0(&m->DH2t, panel_elems(b, B)) &&
            alloc0(&m->DH1t, panel_elems(a, B)) && alloc0(&m->part, part_floats(m, B)) &&
            alloc0(&m->loss, 4096);
  if (!ok) {
    free_batch(m);
    return CPALS_E_CUDA;
  }
  m->bcap = B;
  return CPALS_OK;
}

// the BF16 weight panels from the FP32 master parameters
cudaError_t refresh_weights(cpals_mlp* m) {
  const int in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  cudaError_t e = pack(m, m->p + m->off[0], a, in, m->W1p, nullptr);
  if (e == cudaSuccess) e = pack(m, m->p + m->off[2], b, a, m->W2p, m->W2t);
  if (e == cudaSuccess) e = pack(m, m->p + m->off[4], o, b, m->W3p, m->W3t);
  return e;
}

// forward pass on the input panels (from m->x); y, h1, h2 (FP32) and their panels
cudaError_t forward(cpals_mlp* m, int B) {
  const int in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  cudaError_t e = pack(m, m->x, B, in, m->Xp, m->Xt);
  if (e == cudaSuccess) e = gemm(m, m->Xp, m->W1p, B, a, in, m->p + m->off[1], 1, nullptr, m->h1, m->H1p, m->H1t);
  if (e == cudaSuccess) e = gemm(m, m->H1p, m->W2p, B, b, a, m->p + m->off[3], 1, nullptr, m->h2, m->H2p, m->H2t);
  if (e == cudaSuccess) e = gemm(m, m->H2p, m->W3p, B, o, b, m->p + m->off[5], 0, nullptr, m->y, nullptr, nullptr);
  return e;
}

// backward pass (targets in m->t), gradients into m->g, loss partials of this step into
// m->loss[slot * lb ..]; returns the number of loss partials (lb)
int backward(cpals_mlp* m, int B, int slot, cudaError_t* err, const MlpStep* dstep = nullptr) {
  const int in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  const int64_t ny = (int64_t)B * o;
  const int lb = std::min(grid1(ny), 64);
  if (dstep)
    k_mse_grad_step<<<lb, 256, 0, m->st>>>(m->y, m->t, ny, 1.f / (float)ny, m->dy, m->loss, lb, dstep);
  else
    k_mse_grad<<<lb, 256, 0, m->st>>>(m->y, m->t, ny, 1.f / (float)ny, m->dy, m->loss + (int64_t)slot * lb);
  cudaError_t e = pack(m, m->dy, B, o, m->DYp, m->DYt);
  // dW3 = dy^T h2, db3 = sum_b dy
  if (e == cudaSuccess) e = gemm(m, m->DYt, m->H2t, o, b, B, nullptr, 0, nullptr, m->g + m->off[4], nullptr, nullptr);
  k_bias_grad<<<(o + 255) / 256, 256, 0, m->st>>>(m->dy, B, o, m->g + m->off[5]);
  // dh2 = (dy W3) masked by h2 > 0
  if (e == cudaSuccess) e = gemm(m, m->DYp, m->W3t, B, b, o, nullptr, 2, m->h2, m->dh2, m->DH2p, m->DH2t);
  if (e == cudaSuccess) e = gemm(m, m->DH2t, m->H1t, b, a, B, nullptr, 0, nullptr, m->g + m->off[2], nullptr, nullptr);
  k_bias_grad<<<(b + 255) / 256, 256, 0, m->st>>>(m->dh2, B, b, m->g + m->off[3]);
  // dh1 = (dh2 W2) masked by h1 > 0
  if (e == cudaSuccess) e = gemm(m, m->DH2p, m->W2t, B, a, b, nullptr, 2, m->h1, m->dh1, nullptr, m->DH1t);
  if (e == cudaSuccess) e = gemm(m, m->DH1t, m->Xt, a, in, B, nullptr, 0, nullptr, m->g + m->off[0], nullptr, nullptr);
  k_bias_grad<<<(a + 255) / 256, 256, 0, m->st>>>(m->dh1, B, a, m->g + m->off[1]);
  if (e == cudaSuccess) e = cudaGetLastError();
  *err = e;
  return lb;
}

// one training step on the device state: the batch's rows, forward, backward, Adam, the
// weight panels, the state advanced; the same launches every step, so it is captured once
cudaError_t train_step(cpals_mlp* m, int B, float lr) {
  k_gather_step<<<grid1((int64_t)B * m->w[0]), 256, 0, m->st>>>(m->dx, m->w[0], m->idx, B, m->x, m->dstep);
  k_gather_step<<<grid1((int64_t)B * m->w[3]), 256, 0, m->st>>>(m->dt, m->w[3], m->idx, B, m->t, m->dstep);
  cudaError_t e = forward(m, B);
  if (e != cudaSuccess) return e;
  (void)backward(m, B, 0, &e, m->dstep);
  if (e != cudaSuccess) return e;
  k_adam_step<<<grid1(m->np), 256, 0, m->st>>>(m->p, m->g, m->m1, m->m2, m->np, lr, 0.9f, 0.999f, 1e-8f, m->dstep);
  e = refresh_weights(m);
  if (e != cudaSuccess) return e;
  k_step_end<<<1, 1, 0, m->st>>>(m->dstep);
  return cudaGetLastError();
}

void drop_step_graph(cpals_mlp* m) {
  if (m->step_graph) cudaGraphExecDestroy(m->step_graph);
  m->step_graph = nullptr;
}

// captures train_step for (B, lr) and the current buffers; on failure the steps run eagerly
void build_step_graph(cpals_mlp* m, int B, float lr) {
  drop_step_graph(m);
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    (void)cudaGetLastError();
    return;
  }
  const cudaError_t e = train_step(m, B, lr);
  const cudaError_t ec = cudaStreamEndCapture(m->st, &g);
  if (e == cudaSuccess && ec == cudaSuccess && g && cudaGraphInstantiate(&m->step_graph, g, 0) == cudaSuccess) {
    m->graph_B = B;
    m->graph_lr = lr;
    m->graph_idx = m->idx;
    m->graph_dx = m->dx;
  } else {
    m->step_graph = nullptr;
    (void)cudaGetLastError();
  }
  if (g) cudaGraphDestroy(g);
}

// synchronise; CPALS_E_DEVICE (and the word cleared) if a GEMM's bounded wait expired
int finish(cpals_mlp* m) {
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));
  int h = 0;
  CPALS_CUDA_TRY(cudaMemcpy(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    CPALS_CUDA_TRY(cudaMemset(m->err, 0, 2 * sizeof(int)));
    return CPALS_E_DEVICE;
  }
  return CPALS_OK;
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
  cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
  m->sms = std::max(m->sms, 1);
  for (int i = 0; i < 4; ++i) m->w[i] = widths[i];
  int64_t o = 0;
  for (int l = 0; l < 3; ++l) {
    m->off[2 * l] = o;
    o += (int64_t)m->w[l + 1] * m->w[l];
    m->off[2 * l + 1] = o;
    o += m->w[l + 1];
  }
  m->np = o;
  const int64_t in = m->w[0], a = m->w[1], b = m->w[2], y = m->w[3];
  bool ok = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&m->ev0) == cudaSuccess && cudaEventCreate(&m->ev1) == cudaSuccess && alloc0(&m->p, o) &&
            alloc0(&m->g, o) && alloc0(&m->m1, o) && alloc0(&m->m2, o) && alloc0(&m->err, 2) &&
            alloc0(&m->W1p, panel_elems(a, in)) && alloc0(&m->W2p, panel_elems(b, a)) &&
            alloc0(&m->W2t, panel_elems(a, b)) && alloc0(&m->W3p, panel_elems(y, b)) &&
            alloc0(&m->W3t, panel_elems(b, y)) && alloc0(&m->dstep, 1) && gemm_tc_prepare() == cudaSuccess;
  if (!ok) {
    cpals_mlp_destroy(m);
    return CPALS_E_CUDA;
  }
  *out = m;
  return CPALS_OK;
}

int cpals_mlp_destroy(cpals_mlp* m) {
  if (!m) return CPALS_OK;
  DeviceGuard guard(m->device);
  drop_step_graph(m);
  free_batch(m);
  for (void* q : {(void*)m->dstep, (void*)m->p, (void*)m->g, (void*)m->m1, (void*)m->m2, (void*)m->err, (void*)m->W1p, (void*)m->W2p,
                  (void*)m->W2t, (void*)m->W3p, (void*)m->W3t, (void*)m->idx, (void*)m->dx, (void*)m->dt})
    cudaFree(q);
  if (m->ev0) cudaEventDestroy(m->ev0);
  if (m->ev1) cudaEventDestroy(m->ev1);
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
  CPALS_CUDA_TRY(refresh_weights(m));
  m->step = 0;
  return finish(m);
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
  CPALS_CUDA_TRY(forward(m, B));
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_y, m->y, 4LL * B * m->w[3], cudaMemcpyDeviceToHost, m->st));
  return finish(m);
}

// Loss and gradients (FP32, same layout as the parameters) of one host batch, no update.
int cpals_mlp_gradients(cpals_mlp* m, const float* host_x, const float* host_t, int B, float* host_grads,
                        double* loss_out) {
  if (!m || !host_x || !host_t || !host_grads || B < 1) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  if (ensure_batch(m, B) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->x, host_x, 4LL * B * m->w[0], cudaMemcpyHostToDevice, m->st));
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->t, host_t, 4LL * B * m->w[3], cudaMemcpyHostToDevice, m->st));
  CPALS_CUDA_TRY(forward(m, B));
  cudaError_t e = cudaSuccess;
  const int lb = backward(m, B, 0, &e);
  CPALS_CUDA_TRY(e);
  std::vector<double> h(lb);
  CPALS_CUDA_TRY(cudaMemcpyAsync(h.data(), m->loss, sizeof(double) * lb, cudaMemcpyDeviceToHost, m->st));
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_grads, m->g, 4 * m->np, cudaMemcpyDeviceToHost, m->st));
  const int rc = finish(m);
  if (rc != CPALS_OK) return rc;
  double l = 0.0;
  for (double v : h) l += v;
  if (loss_out) *loss_out = l / ((double)B * m->w[3]);
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
// idx[s*B .. s*B+B-1].  losses (may be null) receives each step's mean loss.  The indices
// go to the device once; the losses come back once per 64 steps.
int cpals_mlp_train(cpals_mlp* m, const int* host_idx, int steps, int B, float lr, double* losses) {
  if (!m || !host_idx || steps < 1 || B < 1 || !m->dx) return CPALS_E_ARG;
  DeviceGuard guard(m->device);
  if (ensure_batch(m, B) != CPALS_OK) return CPALS_E_CUDA;
  const int64_t nidx = (int64_t)steps * B;
  for (int64_t i = 0; i < nidx; ++i)
    if (host_idx[i] < 0 || host_idx[i] >= m->dn) return CPALS_E_ARG;
  if (nidx > m->idx_cap) {
    cudaFree(m->idx);
    m->idx = nullptr;
    m->idx_cap = 0;
    if (cudaMalloc(&m->idx, sizeof(int) * nidx) != cudaSuccess) return CPALS_E_CUDA;
    m->idx_cap = nidx;
  }
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->idx, host_idx, sizeof(int) * nidx, cudaMemcpyHostToDevice, m->st));
  const MlpStep h0{0, (long long)m->step};
  CPALS_CUDA_TRY(cudaMemcpyAsync(m->dstep, &h0, sizeof(MlpStep), cudaMemcpyHostToDevice, m->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(m->st));  // h0 is a stack value
  if (!m->step_graph || m->graph_B != B || m->graph_lr != lr || m->graph_idx != m->idx || m->graph_dx != m->dx)
    build_step_graph(m, B, lr);
  const int lb = std::min(grid1((int64_t)B * m->w[3]), 64);
  std::vector<double> h;
  m->train_ms = 0.0;
  for (int s0 = 0; s0 < steps; s0 += kLossSlots) {
    const int ns = std::min(kLossSlots, steps - s0);
    CPALS_CUDA_TRY(cudaEventRecord(m->ev0, m->st));
    for (int j = 0; j < ns; ++j) {
      if (m->step_graph)
        CPALS_CUDA_TRY(cudaGraphLaunch(m->step_graph, m->st));
      else
        CPALS_CUDA_TRY(train_step(m, B, lr));
    }
    CPALS_CUDA_TRY(cudaEventRecord(m->ev1, m->st));
    h.assign((size_t)ns * lb, 0.0);
    CPALS_CUDA_TRY(cudaMemcpyAsync(h.data(), m->loss, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, m->st));
    const int rc = finish(m);
    if (rc != CPALS_OK) return rc;
    float ms = 0.f;
    CPALS_CUDA_TRY(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    m->train_ms += ms;
    if (losses)
      for (int j = 0; j < ns; ++j) {  // step s0 + j wrote slot j (s0 is a multiple of the slot count)
        double l = 0.0;
        for (int q = 0; q < lb; ++q) l += h[(size_t)j * lb + q];
        losses[s0 + j] = l / ((double)B * m->w[3]);
      }
  }
  m->step += steps;
  return CPALS_OK;
}

// Device time (CUDA events on the network's stream) of the last cpals_mlp_train call, in ms,
// and the tensor-core flops of one training step of B rows (the eight GEMMs).
int cpals_mlp_train_stats(cpals_mlp* m, int B, double* ms, double* flops_per_step) {
  if (!m || B < 1) return CPALS_E_ARG;
  const double in = m->w[0], a = m->w[1], b = m->w[2], o = m->w[3];
  if (ms) *ms = m->train_ms;
  // forward: x W1^T, h1 W2^T, h2 W3^T; backward: three weight gradients, two input gradients
  if (flops_per_step) *flops_per_step = 2.0 * B * (2.0 * in * a + 3.0 * a * b + 3.0 * b * o);
  return CPALS_OK;
}

}  // extern "C"
