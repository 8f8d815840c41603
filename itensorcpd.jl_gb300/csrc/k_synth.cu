// Seeded synthetic tensors generated on the device: T = sum_r w_r F_0(:,r) o F_1(:,r) o ...
// plus Gaussian noise, written column-major in FP32.  This is the generator of the
// benchmark workloads (low rank plus noise at a given SNR) moved next to the data, so that
// training sets of thousands of large tensors never cross the host link.
//
// The noise is counter-based: element e draws its normal deviate from SplitMix64 (Steele,
// Lea and Flood 2014) of (seed, e), turned into two uniforms and one Box-Muller deviate.
// Its scale sigma is chosen so that the expected noise norm sigma * sqrt(numel) equals
// ||signal|| / 10^(snr_db / 20), with ||signal||^2 = w^T (G_0 .* G_1 .* ...) w computed on
// the host from the factor Grams.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cpals_internal.cuh"

namespace cpals {
namespace {

struct SynthGeom {
  int64_t dims[kMaxOrder];
  int64_t foff[kMaxOrder];  // offset of factor m in the concatenated factors
  int64_t numel;
};

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_synth(const float* __restrict__ F, int order, SynthGeom g, int R, const float* __restrict__ w,
                        float sigma, uint64_t seed, float* __restrict__ T) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < g.numel; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rest = e;
    int64_t idx[kMaxOrder];
    for (int m = 0; m < order; ++m) {
      idx[m] = rest % g.dims[m];
      rest /= g.dims[m];
    }
    float acc = 0.f;
    for (int r = 0; r < R; ++r) {
      float p = w[r];
      for (int m = 0; m < order; ++m) p *= __ldg(&F[g.foff[m] + idx[m] + g.dims[m] * (int64_t)r]);
      acc += p;
    }
    if (sigma > 0.f) {
      const uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)e));
      const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);  // (0, 1)
      const float u2 = (float)((h >> 16) & 0xFFFFFFull) * (1.0f / 16777216.0f);
      acc += sigma * sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
    }
    T[e] = acc;
  }
}

}  // namespace
}  // namespace cpals

using namespace cpals;

extern "C" {

// host_factors: F_0, F_1, ... (I_m x R column-major, FP64) concatenated; d_out: device FP32
// buffer of prod(dims) elements (column-major).  snr_db <= -1000 (or a non-finite value)
// means no noise.  Runs on the legacy default stream and returns when the tensor is written.
int cpals_synth_lowrank(int device, int order, const int64_t* dims, int64_t rank, const double* host_factors,
                        const double* host_weights, double snr_db, uint64_t seed, float* d_out) {
  if (order < 1 || order > kMaxOrder || !dims || rank < 1 || !host_factors || !host_weights || !d_out)
    return CPALS_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPALS_E_CUDA;
  DeviceGuard guard(device);
  SynthGeom g{};
  int64_t off = 0;
  g.numel = 1;
  for (int m = 0; m < order; ++m) {
    if (dims[m] < 1) return CPALS_E_ARG;
    g.dims[m] = dims[m];
    g.foff[m] = off;
    off += dims[m] * rank;
    g.numel *= dims[m];
  }
  // ||signal||^2 = w^T (G_0 .* ... .* G_{N-1}) w
  const int R = (int)rank;
  std::vector<double> H((size_t)R * R, 1.0);
  for (int m = 0; m < order; ++m) {
    const double* Fm = host_factors + g.foff[m];
    for (int a = 0; a < R; ++a)
      for (int b = 0; b < R; ++b) {
        double s = 0.0;
        for (int64_t i = 0; i < dims[m]; ++i) s += Fm[i + dims[m] * a] * Fm[i + dims[m] * b];
        H[(size_t)a * R + b] *= s;
      }
  }
  double sig2 = 0.0;
  for (int a = 0; a < R; ++a)
    for (int b = 0; b < R; ++b) sig2 += host_weights[a] * H[(size_t)a * R + b] * host_weights[b];
  float sigma = 0.f;
  if (std::isfinite(snr_db) && snr_db > -1000.0)
    sigma = (float)(std::sqrt(std::max(sig2, 0.0) / (double)g.numel) / std::pow(10.0, snr_db / 20.0));
  std::vector<float> f32(off), w32(R);
  for (int64_t i = 0; i < off; ++i) f32[i] = (float)host_factors[i];
  for (int r = 0; r < R; ++r) w32[r] = (float)host_weights[r];
  float *dF = nullptr, *dw = nullptr;
  if (cudaMalloc(&dF, sizeof(float) * off) != cudaSuccess || cudaMalloc(&dw, sizeof(float) * R) != cudaSuccess) {
    cudaFree(dF);
    return CPALS_E_CUDA;
  }
  cudaMemcpy(dF, f32.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  cudaMemcpy(dw, w32.data(), sizeof(float) * R, cudaMemcpyHostToDevice);
  const int blocks = (int)std::min<int64_t>((g.numel + 255) / 256, 65536);
  k_synth<<<blocks, 256>>>(dF, order, g, R, dw, sigma, seed, d_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);  // the tensor is complete on return
  cudaFree(dF);
  cudaFree(dw);
  return e == cudaSuccess ? CPALS_OK : CPALS_E_CUDA;
}

}  // extern "C"
