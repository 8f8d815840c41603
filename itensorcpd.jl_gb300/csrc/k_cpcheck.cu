// Convergence checks that compare consecutive iterates instead of the target:
// CPDiffCheck (src/converge_checks/cp_diff_check.jl:20-68) and CPAngleCheck
// (src/converge_checks/cp_angle_check.jl:20-68).  Both need
//
//   <T_prev, T_curr> = lam_prev^T (P_0^T F_0 .* P_1^T F_1 .* ...) lam        (cp_cp_contract,
//                                                           src/algebra/cp_contract.jl:32-52)
//   ||T_curr||^2     = lam^T (G_0 .* G_1 .* ...) lam      (norm_factors, converge_checks.jl:5-11)
//
// with P_m the previous iterate's factors and G_m = F_m^T F_m the Grams the sweep keeps.
// The cross Grams are I_m x R by I_m x R FP64 products.  FP64 issue is the limit here, so
// k_cross_gram cuts every cross Gram into 64 x 64 output tiles and S row splits, giving
// about two blocks per SM, and writes the split partials; k_cp_check sums them in split
// order, forms both quadratic forms, reduces them over its blocks in block order (the last
// block to finish does this) and runs the check's update on one thread.
//
// FP64 throughout: the fit between consecutive iterates, 1 - sqrt(|a + b - 2c|) / sqrt(a),
// cancels to the size of the change, so lower precision would hide changes below 1e-4.
#include "cpals_internal.cuh"

namespace cpals {
namespace {

constexpr int XT = 64;  // output tile edge
constexpr int XK = 16;  // rows staged per step

__device__ double warp_block_sum(double v, double* sv) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) sv[w] = v;
  __syncthreads();
  double t = (lane < nw) ? sv[lane] : 0.0;
  for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  __syncthreads();
  return t;
}

// grid (S, nt*nt, order), 256 threads.  Block (s, tile, m) computes rows [r0, r1) of
// P_m^T F_m for the 64 x 64 tile (ti, tj); the tile-0 blocks also copy those rows of F_m
// (and block (0, 0, 0) lambda) into the buffer that becomes PrevCP.
__global__ void __launch_bounds__(256) k_cross_gram(CrossArgs a) {
  const DevCheck* chk = a.chk;
  if (chk->done) return;
  __shared__ double ps[XK][XT];
  __shared__ double fs[XK][XT];
  const int s = blockIdx.x, tile = blockIdx.y, m = blockIdx.z;
  const int R = a.R;
  const int nt = (R + XT - 1) / XT;
  const int ti = tile / nt, tj = tile - ti * nt;
  const int64_t In = a.dims[m];
  const int64_t rows = (In + a.S - 1) / a.S;
  const int64_t r0 = min(In, (int64_t)s * rows), r1 = min(In, r0 + rows);
  const int sel = chk->psel;
  const double* __restrict__ Fm = a.F[m];
  if (tile == 0) {
    double* __restrict__ dst = a.prevF[sel ^ 1] + a.off[m];
    for (int64_t e = r0 * R + threadIdx.x; e < r1 * R; e += blockDim.x) dst[e] = Fm[e];
    if (m == 0 && s == 0)
      for (int r = threadIdx.x; r < R; r += blockDim.x) a.prevLam[sel ^ 1][r] = a.lam[r];
  }
  if (!chk->has_prev) return;
  const double* __restrict__ Pm = a.prevF[sel] + a.off[m];
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int64_t kk = r0; kk < r1; kk += XK) {
#pragma unroll
    for (int q = 0; q < (XK * XT) / 256; ++q) {
      const int e = threadIdx.x + 256 * q;
      const int k = e >> 6, c = e & (XT - 1);
      const int64_t row = kk + k;
      const int ca = ti * XT + c, cb = tj * XT + c;
      ps[k][c] = (row < r1 && ca < R) ? Pm[row * R + ca] : 0.0;
      fs[k][c] = (row < r1 && cb < R) ? Fm[row * R + cb] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < XK; ++k) {
      double pa[4], fb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) pa[i] = ps[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) fb[j] = fs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(pa[i], fb[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* __restrict__ out = a.xpart + ((int64_t)m * a.S + s) * (int64_t)R * R;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ti * XT + ty + 16 * i;
    if (r >= R) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tj * XT + tx + 16 * j;
      if (c < R) out[(int64_t)r * R + c] = acc[i][j];
    }
  }
}

// The check's update (cp_diff_check.jl:20-68 / cp_angle_check.jl:20-68) on one thread.
__device__ void cp_check_update(DevCheck& k, double inner, double self, double* traj, int64_t traj_cap) {
  const bool angle = (k.kind == CPALS_CHECK_ANGLE);
  k.iter += 1;
  if (!k.has_prev) {  // PrevCP === nothing: store this iterate and its norm
    k.has_prev = 1;
    k.norm_prev = angle ? sqrt(self) : self;
    k.psel ^= 1;
    if (k.sweeps < traj_cap) traj[k.sweeps] = NAN;
    k.sweeps += 1;
    return;
  }
  double cur, norm_now;
  if (angle) {
    norm_now = sqrt(self);
    double theta = inner / (norm_now * k.norm_prev);
    theta = theta > 1.0 ? 1.0 : theta;  // NaN passes through, as in the reference
    cur = acos(theta);
  } else {
    norm_now = self;
    const double nres = sqrt(fabs(k.norm_prev + self - 2.0 * fabs(inner)));
    cur = 1.0 - nres / sqrt(fabs(k.norm_prev));
  }
  const double delta = fabs(k.lastfit - cur);
  k.lastfit = cur;
  k.psel ^= 1;
  k.norm_prev = norm_now;
  if (k.sweeps < traj_cap) traj[k.sweeps] = cur;
  k.sweeps += 1;
  if (delta < k.tol) {
    k.counter += 1;
    if (k.counter >= 2) {
      k.total_iter = k.iter;
      k.iter = 0;
      k.counter = 0;
      k.final_fit = k.lastfit;
      k.lastfit = 0.0;
      k.has_prev = 0;
      k.done = 1;
      return;
    }
  } else {
    k.counter = 0;
  }
  if (k.iter >= k.max_counter) {
    k.total_iter = k.iter;
    k.iter = 0;
    k.counter = 0;
    k.final_fit = k.lastfit;
    k.lastfit = 0.0;
    k.has_prev = 0;
  }
}

// grid ceil(R*R / 256), 256 threads.  Thread e = (r, c) forms
// lam_prev[r] lam[c] prod_m sum_s xpart[m][s][r][c] and lam[r] lam[c] prod_m G_m[r][c].
__global__ void __launch_bounds__(256) k_cp_check(CrossArgs a) {
  DevCheck* chk = a.chk;
  if (chk->done) return;
  __shared__ double sv[8];
  __shared__ int s_last;
  const int R = a.R;
  const int64_t RR = (int64_t)R * R;
  const int sel = chk->psel;
  const int has_prev = chk->has_prev;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double inner = 0.0, self = 0.0;
  if (e < RR) {
    const int r = (int)(e / R), c = (int)(e - (int64_t)r * R);
    double g = a.lam[r] * a.lam[c];
    for (int m = 0; m < a.order; ++m) g *= a.G[m][e];
    self = g;
    if (has_prev) {
      double h = a.prevLam[sel][r] * a.lam[c];
      for (int m = 0; m < a.order; ++m) {
        const double* __restrict__ xp = a.xpart + (int64_t)m * a.S * RR + e;
        double x = 0.0;
        for (int s = 0; s < a.S; ++s) x += xp[(int64_t)s * RR];
        h *= x;
      }
      inner = h;
    }
  }
  inner = warp_block_sum(inner, sv);
  self = warp_block_sum(self, sv);
  if (threadIdx.x == 0) {
    a.red[2 * blockIdx.x] = inner;
    a.red[2 * blockIdx.x + 1] = self;
    __threadfence();
    s_last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double ti = 0.0, ts = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    ti += __ldcg(&a.red[2 * b]);
    ts += __ldcg(&a.red[2 * b + 1]);
  }
  ti = warp_block_sum(ti, sv);
  ts = warp_block_sum(ts, sv);
  if (threadIdx.x != 0) return;
  *a.counter = 0u;
  cp_check_update(*chk, ti, ts, a.traj, a.traj_cap);
}

}  // namespace

int cross_splits(int order, int R, int num_sms) {
  const int nt = (R + XT - 1) / XT;
  const int per = order * nt * nt;
  const int s = (2 * num_sms + per - 1) / per;
  return s < 1 ? 1 : (s > 64 ? 64 : s);
}

cudaError_t launch_cp_check(const CrossArgs& a, cudaStream_t st) {
  const int nt = (a.R + XT - 1) / XT;
  k_cross_gram<<<dim3(a.S, nt * nt, a.order), 256, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t RR = (int64_t)a.R * a.R;
  k_cp_check<<<(unsigned)((RR + 255) / 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace cpals
